#!/usr/bin/env python3
"""Benchmark of the CellFlow simulation step on GB300.

One bench step is one simulation step (cell list + force/density/integrator)
of the configured workload, default the README-scale plain step: N=100,000
particles, T=8 types, positions uniform in [-1,1]^3 (shifted to [0,2)^3),
force table ~ N(0, 0.5), interaction radius 0.0920 (mean neighbour count
about 40), dt 0.01.  Inputs are seeded synthetic data of that shape.

Timing: W warm-up steps, then K steps each bracketed by CUDA events recorded
on the library's stream around the step's phases (cf_profile_enable); a
256 MiB write flushes L2 between timed steps, outside the timed intervals.
value = N * K / (sum of step times), particle-steps/s.  e2e repeats the step
through the public C ABI with host buffers: per step the AoS particle state
(44 B per particle) goes host->device from pinned memory, the step runs, and
the state comes back device->host; value = N * steps / host wall time.

--impl reference times the reference's own step (its kernel body compiled on
the host from its sources, oracle/_ref, with OpenMP on every core; the oracle
restatement where that is absent) on a bounded sample of particles per step.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FLUSH_BYTES = 256 << 20
REFERENCE_BUDGET_S = 240.0  # whole reference steps when the run fits in this


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default=None,
                    help="one workload alone (default: the 100k headline with the 1M, batched and rollout "
                         "workloads as nested records)")
    ap.add_argument("--no-nested", action="store_true", help="the headline workload alone")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--prox-calls", type=int, default=50, help="proximity-graph calls timed (workloads with a distance)")
    ap.add_argument("--profile-steps", type=int, default=None, metavar="S",
                    help="no timing: step the workload's world S times with --variant and exit (a short, "
                         "fixed launch sequence for ncu captures)")
    ap.add_argument("--variant", type=int, default=None, help="force-kernel variant for --profile-steps "
                    "(default: the autotuner's pick)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = [r.split(",") for r in Path(self.path).read_text().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


FORCE_PROFILE = "profiles/step_force_kernel_plain_n100k_blobs_n1m.md"


def profile_figure(key: str, workload: str):
    """A figure of the committed ncu summary of the force kernel: its `KEY WORKLOAD VALUE` line, or None."""
    f = ROOT / FORCE_PROFILE
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] == key and parts[1] == workload:
            return float(parts[2])
    return None


def profiled_traffic(workload: str):
    """DRAM bytes (read + write) of one force-kernel launch on this workload from the committed
    ncu summary (a `traffic_bytes_per_launch WORKLOAD BYTES` line), or None."""
    v = profile_figure("traffic_bytes_per_launch", workload)
    if v is None:
        return None
    return {"bytes_per_launch": int(v), "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, " + FORCE_PROFILE}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float) -> float:
    """The largest value over the ranks of the process group (x itself without one).  Replicas
    only: this timing reduction is the one collective of a multi-GPU run."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, ms_max: float, world: int) -> float:
    """Whole-job units/s of `world` replicas that each processed units_per_rank, the slowest in ms_max."""
    return units_per_rank * world / (ms_max * 1e-3)


def cpu_reference_sample(w, params, pos, types, table, radio, budget_s: float):
    """Times the reference step on the host over a strided sample of rows.
    Returns (particle-steps/s, kind, cores, sample description)."""
    import numpy as np

    import oracle

    try:
        oracle.build_ref(gpu=False)
    except Exception:
        pass
    kind = "reference" if oracle.ref_available() else "port"
    cores = os.cpu_count() or 1
    vel = np.zeros_like(pos)
    counts = np.zeros(w.n, np.int32)
    rec = oracle.to_records(pos, vel, types)

    def run(rows):
        b, e, s = rows
        t0 = time.perf_counter()
        if kind == "reference":
            oracle.ref_step(rec, table, radio, counts, params, rows=rows)
        else:
            oracle.step_f32(pos, vel, types, counts, table, radio, params, rows=rows)
        return time.perf_counter() - t0, len(range(b, e, s))

    # calibrate on a small sample, then size the sample to the budget
    stride = max(1, w.n // (8 * cores))
    dt, r = run((0, w.n, stride))
    rate = r / max(dt, 1e-9)
    rows_target = int(max(cores, min(w.n, rate * budget_s)))
    stride = max(1, w.n // rows_target)
    dt, r = run((0, w.n, stride))
    desc = (f"{r} of {w.n} particles (every {stride}th), each against all {w.n}, one step from the initial "
            f"state; {cores} OpenMP threads; {dt:.2f} s"
            + ("" if stride == 1 else "; rate extrapolated from the strided sample (each sampled row costs a full row)"))
    return r / dt, kind, cores, desc


def host_cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            key, _, val = line.partition(":")
            if key.strip() == "Model name" and val.strip():
                return val.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            key, _, val = line.partition(":")
            if key.strip().lower() in ("model name", "cpu model", "processor name") and val.strip():
                return val.strip()
        import platform

        return platform.processor() or platform.machine()
    except OSError:
        return "unknown"


def run_reference_arm(args, rank, world):
    """--impl reference: the reference's own step on the host cores."""
    if rank != 0:
        return
    import numpy as np

    from cellflow_gb300 import inputs

    import oracle

    try:
        oracle.build_ref(gpu=False)
    except Exception:
        pass
    kind = "reference" if oracle.ref_available() else "port"
    cores = os.cpu_count() or 1

    if args.workload in inputs.BATCHED:
        # the reference steps one world at a time: step s samples world (37 s) mod worlds
        bw = inputs.BATCHED[args.workload]
        params = bw.params()
        sizes = bw.sizes()
        total_n = int(sizes.sum())
        config = {"workload": bw.name, "worlds": bw.worlds, "total_particles": total_n, "types": bw.num_types,
                  "radius": bw.radius, "seed": bw.seed}
        worlds_in = {}

        def world_inputs(s):
            k = (37 * s) % bw.worlds
            if k not in worlds_in:
                p, t, tab = bw.world(k, int(sizes[k]))
                worlds_in[k] = (p, t, tab, oracle.to_records(p, np.zeros_like(p), t))
            return worlds_in[k]
        radio = np.zeros(bw.num_types, np.float32)
        full_n = total_n
    else:
        if args.workload in ROLLOUT:
            # the reference has no adjoint: its step on the rollout's configuration
            cfg = ROLLOUT[args.workload]
            w = inputs.Workload(args.workload, n=cfg["n"], num_types=cfg["types"], radius=cfg["radius"],
                                steps=cfg["steps"], seed=cfg["seed"])
        else:
            w = inputs.WORKLOADS[args.workload]
        params = w.params()
        p0, t0_, tab0 = w.positions(), w.types(), w.table()
        fixed = (p0, t0_, tab0, oracle.to_records(p0, np.zeros_like(p0), t0_))
        config = workload_config(w)

        def world_inputs(s):
            return fixed
        radio = np.zeros(w.num_types, np.float32)
        full_n = w.n

    # each step: a strided sample of rows of one world, sized to about one second
    def one(s, frac):
        pos, types, table, rec = world_inputs(s)
        n = len(pos)
        stride_ = max(1, int(round(1.0 / frac)))
        rows = (0, n, stride_)
        counts = np.zeros(n, np.int32)
        t0 = time.perf_counter()
        if kind == "reference":
            oracle.ref_step(rec, table, radio, counts, params, rows=rows)
        else:
            oracle.step_f32(pos, np.zeros_like(pos), types, counts, table, radio, params, rows=rows)
        return time.perf_counter() - t0, len(range(*rows)), n

    # calibrate on a small strided sample; run whole steps when the whole run (warm-up and
    # timed steps) fits in REFERENCE_BUDGET_S seconds, else strided samples of about one
    # second per step, whose per-step time is then an extrapolation (labelled as such)
    frac = min(1.0, 8.0 * cores / max(len(world_inputs(0)[0]), 1))
    dt, r, _ = one(0, frac)
    full_step_s = dt / frac if frac > 0 else dt
    if full_step_s * (args.warmup + args.steps) <= REFERENCE_BUDGET_S:
        frac = 1.0
    elif dt > 0:
        frac = min(1.0, frac / dt)
    for s in range(args.warmup):
        one(s, frac)
    total_t, total_rows = 0.0, 0
    for s in range(args.steps):
        dt, r, _ = one(s, frac)
        total_t += dt
        total_rows += r
    value = total_rows / total_t
    whole = frac >= 1.0
    sample = (f"per step about {total_rows // max(args.steps, 1)} particles "
              + ("(every particle of the world: whole steps)" if whole else
                 f"(a {frac:.3g} strided fraction of one world; ms_per_step extrapolated from it)")
              + f", each against all particles of its world; {cores} OpenMP threads")
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * full_n / value, "ms_per_step_measured": whole,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Philox), see config",
        "config": config,
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": kind,
                         "cpu_model": host_cpu_model(),
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(w) -> dict:
    return {"workload": w.name, "n": w.n, "types": w.num_types, "radius": w.radius, "dt": w.delta_t,
            "box": "[-1,1]^3 shifted to [0,2)^3", "positions": "uniform" if not w.blobs else
            f"{w.blobs} gaussian blobs sigma {w.blob_sigma}", "force_table": f"N({w.table_mean},{w.table_sigma})",
            "l2": "flushed between timed steps (256 MiB write)", "seed": w.seed}


def run_gb300(args, rank, world, local, name, steps, warmup, cpu_seconds, extras=True):
    """One plain-step workload: the timed steps, the force-kernel and cell-list rooflines, the CPU
    baseline, end to end through the C ABI, and (extras) the reference kernel built for this GPU and
    the proximity graph.  Returns rank 0's record (None on other ranks)."""
    import numpy as np
    import torch

    import cellflow_gb300 as cf
    from cellflow_gb300 import _lib, inputs
    from cellflow_gb300.world import PARTICLE_DTYPE, ParticleSimulation

    lib = _lib.load()
    w = inputs.WORKLOADS[name]
    params = w.params()
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    stream = torch.cuda.Stream()
    sim = ParticleSimulation(w.n, w.num_types, w.extent, w.extent, w.extent)
    sim.set_stream(stream.cuda_stream)
    sim.set_particles(pos, types)
    sim.setForceTable(table)
    sim.setRadioByType(radio)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(warmup):
        sim.simulate(params, 1)
    # picks the force-kernel variant on the state the timed steps start from; restores the state
    force_variant = sim.autotune(params, 5)
    sim.sync()
    state0 = sim.get_state()

    # ---- timed region: K steps, per-phase CUDA events, L2 flushed between steps
    _lib.check(lib.cf_profile_enable(sim.handle, 1), "cf_profile_enable")
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
                          if os.environ.get("CUDA_VISIBLE_DEVICES", "").isdigit() else local)
    clocks.start()
    barrier()
    tally0 = lib.cf_kernel_launches()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.zero_()
            sim.simulate(params, 1)
    barrier()
    wall = time.perf_counter() - wall0
    launches = lib.cf_kernel_launches() - tally0
    clk = clocks.stop()
    prof = _lib.PhaseTimes()
    _lib.check(lib.cf_profile_read(sim.handle, C.byref(prof)), "cf_profile_read")
    _lib.check(lib.cf_profile_enable(sim.handle, 0), "cf_profile_enable")
    step_ms_total = prof.cell_list_ms + prof.force_ms
    t_max = max_over_ranks(step_ms_total)
    value = replica_throughput(w.n * steps, t_max, world)

    # ---- work counters: replay the same K steps from the same state, untimed
    sim.set_state(*state0)
    c27_total, inter_total, tested_total = 0, 0, 0
    for _ in range(steps):
        c27, _ = sim.work_counters(params)
        tested_total += sim.force_work(params)[1]
        sim.simulate(params, 1)
        _, inter = sim.work_counters(params)
        c27_total += c27
        inter_total += inter
    flops = 9 * c27_total + 17 * inter_total + 25 * w.n * steps
    force_s = prof.force_ms * 1e-3
    achieved_tflops = flops / force_s / 1e12
    peak_fp32 = C.c_double()
    _lib.check(lib.cf_measure_fp32_peak(C.byref(peak_fp32)), "cf_measure_fp32_peak")
    cells = 1
    g = sim.grid(params)
    for a in range(3):
        cells *= g.cells[a]
    cell_bytes = (112 * w.n + 8 * cells) * steps
    cell_gbs = cell_bytes / (prof.cell_list_ms * 1e-3) / 1e9
    peaks = measured_peaks()

    # ---- end to end through the C ABI with host buffers
    e2e_steps = args.e2e_steps or max(10, steps // 2)
    host = torch.empty(w.n * PARTICLE_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    host_np = host.numpy().view(PARTICLE_DTYPE)
    sim.set_state(*state0)
    host_np[:] = sim.getParticleData()
    hp = C.c_void_p(host.data_ptr())
    pc = params.to_c()

    def e2e_run(one_call: bool) -> float:
        """Host wall time of e2e_steps steps, each uploading the pinned AoS records, stepping and
        reading them back; L2 flushed before each step, outside the timed span."""
        def step():
            if one_call:
                _lib.check(lib.cf_step_host(sim.handle, C.byref(pc), hp, hp, w.n), "cf_step_host")
            else:
                _lib.check(lib.cf_set_particles(sim.handle, hp, w.n), "cf_set_particles")
                sim.simulate(params, 1)
                _lib.check(lib.cf_get_particles(sim.handle, hp, w.n), "cf_get_particles")

        for _ in range(3):
            step()
        barrier()
        total = 0.0
        for _ in range(e2e_steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step()
            total += time.perf_counter() - t0
        return total

    sim.set_state(*state0)
    host_np[:] = sim.getParticleData()
    e2e_three_wall = e2e_run(False)
    sim.set_state(*state0)
    host_np[:] = sim.getParticleData()
    e2e_wall = e2e_run(True)
    e2e_value = w.n * e2e_steps * world / e2e_wall

    # ---- reference kernel on this GPU (its O(N^2) kernel built for sm_103a), a few steps
    ref_gpu = reference_gpu_kernel(w, params, pos, types, table, radio, stream) if rank == 0 and extras else None

    # ---- proximity graph (edges/s) on the state the timed steps left
    prox = proximity_timing(sim, w, stream, args.prox_calls) if w.prox_distance is not None and extras else None

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, kind, cores, desc = cpu_reference_sample(w, params, pos, types, table, radio, cpu_seconds)
            cpu = {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": kind, "sample": desc,
                   "cpu_model": host_cpu_model()}
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": t_max / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox4x32-10), shapes and distributions of the workload",
            "config": workload_config(w),
            "force_variant": force_variant,
            "roofline": {
                "kernel": "step_force_kernel (force + density + integrator)", "bound": "fp32",
                "achieved": achieved_tflops, "peak": peak_fp32.value, "unit": "TFLOP/s",
                "frac": achieved_tflops / peak_fp32.value,
                "peak_source": "FP32 FMA chains on every SM, measured in this run (cf_measure_fp32_peak); "
                               "MEASURED_PEAKS.json has no FP32 figure",
                "work_model": "9*C27 + 17*I + 25*N flops per step",
                "c27_per_particle_step": c27_total / (w.n * steps),
                "interacting_per_particle_step": inter_total / (w.n * steps),
                "tested_per_particle_step": tested_total / (w.n * steps),
                "tested_note": "candidate tests of the force kernel's filter per particle (cf_force_work): the "
                               "union of each 32-particle item's stencils, against the canonical C27",
                "traffic": (profiled_traffic(w.name) or {}).get("bytes_per_launch"),
                "traffic_unit": "bytes per launch (one ncu capture of this workload's force kernel)",
                "traffic_source": (profiled_traffic(w.name) or {}).get("source"),
                "ncu_fma_pipe_pct": profile_figure("fma_pipe_inst_pct", w.name),
                "ncu_issue_active_pct": profile_figure("issue_active_pct", w.name),
            },
            "roofline_cell_list": {
                "bound": "hbm", "achieved": cell_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": cell_gbs / peaks.get("hbm_gbs", 6800.0),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if not peaks.get("fallback") else "fallback",
                "work_model": "112 B/particle + 8 B/cell per step",
            },
            "phase_ms_per_step": {"cell_list": prof.cell_list_ms / steps, "force": prof.force_ms / steps},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": w.n * 44,
                    "d2h_bytes_per_step": w.n * 44, "steps": e2e_steps,
                    "path": "cf_step_host: pinned 44-B AoS records up, one step, records back (one CUDA graph)",
                    "three_calls": {"value": w.n * e2e_steps * world / e2e_three_wall, "unit": "particle-steps/s",
                                    "path": "cf_set_particles + cf_step + cf_get_particles"}},
            "gpu_launches": int(launches),
            "gpu_launches_expected": int(prof.launches),
            "clocks": clk,
            "wall_s_timed_region": wall,
            "cpu_baseline": cpu,
            "reference_gpu_kernel": ref_gpu,
            "proximity": prox,
            "library": cf.__name__ + ": " + _lib.load().cf_version().decode(),
        }
        if not extras:
            for k in ("reference_gpu_kernel", "proximity", "library"):
                line.pop(k)
    sim.close()
    return line


def run_batched(args, rank, world, local, name="batched_256w", steps=100, warmup=100, cpu_seconds=12.0):
    """batched_256w: 256 independent worlds stepped together (cf_batch_*), a 100-step loop
    captured in one CUDA graph and replayed; the same worlds stepped one by one through the
    plain API (each world's step its own CUDA graph) are timed beside it.  One bench step is
    one simulation step of every world; K is rounded up to whole replays of the 100-step
    graph.  The force-kernel roofline comes from profiled steps of the batch (per-phase
    events) and the work counters of the same steps.  Returns rank 0's record."""
    import numpy as np
    import torch

    from cellflow_gb300 import _lib, inputs
    from cellflow_gb300.world import Batch, ParticleSimulation

    bw = inputs.BATCHED[name]
    params = bw.params()
    sizes = bw.sizes()
    parts = [bw.world(k, int(n)) for k, n in enumerate(sizes)]
    pos = np.concatenate([p[0] for p in parts])
    types = np.concatenate([p[1] for p in parts])
    tables = np.stack([p[2] for p in parts])
    total = int(sizes.sum())
    stream = torch.cuda.Stream()
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    lib = _lib.load()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    batch = Batch(sizes, bw.num_types, bw.extent, bw.extent, bw.extent, seed=bw.seed)
    batch.set_stream(stream.cuda_stream)
    batch.set_particles(pos, types)
    batch.set_force_tables(tables)
    variant = batch.autotune(params, 5)
    batch.capture(params, bw.graph_steps)
    _, graph_kernels = batch.graph_info()
    replays = max(1, -(-steps // bw.graph_steps))
    warm = max(1, -(-warmup // bw.graph_steps))
    for _ in range(warm):
        batch.replay()
    batch.sync()
    batch.set_particles(pos, types)  # timed replays start from the initial state
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(replays)]
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    tally0 = lib.cf_kernel_launches()
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            batch.replay()
            e1.record(stream)
    barrier()
    launches = lib.cf_kernel_launches() - tally0
    clk = clocks.stop()
    batch_ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    t_max = max_over_ranks(batch_ms)
    steps_timed = replays * bw.graph_steps
    value = replica_throughput(total * steps_timed, t_max, world)

    # ---- force-kernel roofline: profiled steps of the batch from the initial state (phase
    # events), then the work counters of the same steps replayed untimed
    wh = batch.world_handle()
    prof_steps = min(20, bw.graph_steps)
    batch.set_particles(pos, types)
    _lib.check(lib.cf_profile_enable(wh, 1), "cf_profile_enable")
    with torch.cuda.stream(stream):
        for _ in range(prof_steps):
            flush.zero_()
            batch.simulate(params, 1)
    prof = _lib.PhaseTimes()
    _lib.check(lib.cf_profile_read(wh, C.byref(prof)), "cf_profile_read")
    _lib.check(lib.cf_profile_enable(wh, 0), "cf_profile_enable")
    batch.set_particles(pos, types)
    c27_total, inter_total = 0, 0
    pc = params.to_c()
    for _ in range(prof_steps):
        c27, inter = C.c_uint64(), C.c_uint64()
        _lib.check(lib.cf_work_counters(wh, C.byref(pc), C.byref(c27), None), "cf_work_counters")
        batch.simulate(params, 1)
        _lib.check(lib.cf_work_counters(wh, C.byref(pc), None, C.byref(inter)), "cf_work_counters")
        c27_total += c27.value
        inter_total += inter.value
    flops = 9 * c27_total + 17 * inter_total + 25 * total * prof_steps
    achieved = flops / (prof.force_ms * 1e-3) / 1e12
    peak_fp32 = C.c_double()
    _lib.check(lib.cf_measure_fp32_peak(C.byref(peak_fp32)), "cf_measure_fp32_peak")

    # ---- end to end: host state in (pinned), one replay, host state out
    pin = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory()  # noqa: E731
    hpos, hvel, hcnt = pin((total, 4), torch.float32), pin((total, 4), torch.float32), pin((total,), torch.int32)
    batch.set_particles(pos, types)
    ptrs = [C.c_void_p(x.data_ptr()) for x in (hpos, hvel, hcnt)]
    _lib.check(lib.cf_batch_get_state(batch.handle, *ptrs), "cf_batch_get_state")
    e2e_reps = max(1, replays)
    barrier()
    e2e_wall = 0.0
    for _ in range(e2e_reps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(lib.cf_batch_set_state(batch.handle, *ptrs), "cf_batch_set_state")
        batch.replay()
        _lib.check(lib.cf_batch_get_state(batch.handle, *ptrs), "cf_batch_get_state")
        e2e_wall += time.perf_counter() - t0
    e2e_value = total * bw.graph_steps * e2e_reps * world / e2e_wall
    batch.close()

    # ---- the same worlds stepped one by one through the plain step, same stream
    sims = []
    for k, n in enumerate(sizes):
        s = ParticleSimulation(int(n), bw.num_types, bw.extent, bw.extent, bw.extent)
        s.set_stream(stream.cuda_stream)
        s.set_particles(parts[k][0], parts[k][1])
        s.setForceTable(parts[k][2])
        s.setRadioByType(np.zeros(bw.num_types, np.float32))
        s.set_force_variant(variant)
        sims.append(s)
    for s in sims:
        s.simulate(params, 2)
    torch.cuda.synchronize()
    for k, s in enumerate(sims):
        s.set_particles(parts[k][0], parts[k][1])
    wbw_steps = bw.graph_steps
    with torch.cuda.stream(stream):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in sims:
            s.simulate(params, wbw_steps)
        e1.record(stream)
    e1.synchronize()
    wbw_ms = e0.elapsed_time(e1)
    wbw_value = total * wbw_steps / (wbw_ms * 1e-3)
    for s in sims:
        s.close()

    if rank != 0:
        return None
    cpu = None
    if not args.no_cpu_baseline:
        cpu = batched_cpu_sample(bw, params, sizes, parts, cpu_seconds)
    return {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": steps_timed, "warmup": warm * bw.graph_steps, "ms_per_step": t_max / steps_timed,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Philox4x32-10): per world uniform positions, uniform types, N(0,0.5) table",
        "config": {"workload": bw.name, "worlds": bw.worlds, "n_per_world": f"log-uniform [{bw.n_min}, "
                   f"{bw.n_max}]", "total_particles": total, "n_min": int(sizes.min()),
                   "n_max": int(sizes.max()), "types": bw.num_types, "radius": bw.radius, "dt": bw.delta_t,
                   "graph_steps": bw.graph_steps, "replays": replays,
                   "l2": "flushed between replays (256 MiB write); state larger than L2", "seed": bw.seed},
        "force_variant": variant,
        "world_by_world": {"value": wbw_value, "unit": "particle-steps/s", "steps": wbw_steps,
                           "path": "256 ParticleSimulation objects on one stream, one step graph each"},
        "batched_over_world_by_world": value / wbw_value,
        "roofline": {
            "kernel": "step_force_kernel (force + density + integrator), all 256 worlds in one launch",
            "bound": "fp32", "achieved": achieved, "peak": peak_fp32.value, "unit": "TFLOP/s",
            "frac": achieved / peak_fp32.value,
            "peak_source": "FP32 FMA chains on every SM, measured in this run (cf_measure_fp32_peak)",
            "work_model": "9*C27 + 17*I + 25*N flops per step",
            "steps": prof_steps, "force_ms_per_step": prof.force_ms / max(prof.steps, 1),
            "cell_list_ms_per_step": prof.cell_list_ms / max(prof.steps, 1),
            "c27_per_particle_step": c27_total / (total * prof_steps),
            "interacting_per_particle_step": inter_total / (total * prof_steps),
        },
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": total * 36 //
                bw.graph_steps, "d2h_bytes_per_step": total * 36 // bw.graph_steps,
                "path": "cf_batch_set_state (pinned) + 100-step graph replay + cf_batch_get_state",
                "replays": e2e_reps},
        "gpu_launches": int(launches), "gpu_launches_expected": graph_kernels * replays,
        "clocks": clk,
        "cpu_baseline": cpu,
    }


def batched_cpu_sample(bw, params, sizes, parts, budget_s: float):
    """The reference step on the host, world by world (it has no batching): strided rows of
    worlds taken in a fixed order until the time budget is spent.  Returns the cpu_baseline
    record in particle-steps/s over all the particles the sample covered."""
    import numpy as np

    import oracle

    try:
        oracle.build_ref(gpu=False)
    except Exception:
        pass
    kind = "reference" if oracle.ref_available() else "port"
    cores = os.cpu_count() or 1
    radio = np.zeros(bw.num_types, np.float32)
    rows_done, t_total, worlds_done = 0, 0.0, 0
    for s in range(bw.worlds):
        k = (37 * s) % bw.worlds
        pos, types, table = parts[k]
        n = len(pos)
        stride = max(1, n // (64 * cores))
        rows = (0, n, stride)
        counts = np.zeros(n, np.int32)
        t0 = time.perf_counter()
        if kind == "reference":
            oracle.ref_step(oracle.to_records(pos, np.zeros_like(pos), types), table, radio, counts, params, rows=rows)
        else:
            oracle.step_f32(pos, np.zeros_like(pos), types, counts, table, radio, params, rows=rows)
        t_total += time.perf_counter() - t0
        rows_done += len(range(*rows))
        worlds_done += 1
        if t_total > budget_s:
            break
    return {"value": rows_done / t_total, "unit": "particle-steps/s", "cores": cores, "kind": kind,
            "cpu_model": host_cpu_model(),
            "sample": f"{rows_done} particles of {worlds_done} worlds (strided rows, each against all particles "
                      f"of its world), one step from the initial state, world by world; {cores} OpenMP threads; "
                      f"{t_total:.2f} s"}


ROLLOUT = {"rollout_n16k_k64": dict(n=16384, types=6, radius=0.1, steps=64, every=16, bins=32, r_max=0.2,
                                    seed=0x5EED0005)}


def run_rollout(args, rank, world, local, name="rollout_n16k_k64", steps=5, warmup=3, cpu_seconds=12.0):
    """rollout_n16k_k64: the differentiable rollout.  One bench step is one forward + backward
    pass of the K-step rollout with the soft radial distribution loss (cf_rollout_forward,
    cf_rdf, cf_rdf_backward, cf_rollout_backward); the plain step (cf_step, K steps) is timed
    beside it for the adjoint / forward cost ratio, and the adjoint kernels of a profiled
    backward (per-step events, no graph) against the adjoint work model for their roofline.
    Returns rank 0's record."""
    import numpy as np
    import torch

    from cellflow_gb300 import _lib, inputs
    from cellflow_gb300.world import ParticleSimulation

    cfg = ROLLOUT[name]
    n, T, K = cfg["n"], cfg["types"], cfg["steps"]
    w = inputs.Workload(name, n=n, num_types=T, radius=cfg["radius"], steps=K, seed=cfg["seed"])
    params = w.params()
    pos, types, table = w.positions(), w.types(), w.table()
    target_table = inputs.gaussian_table(T, 0.0, 0.5, cfg["seed"] + 1)
    stream = torch.cuda.Stream()
    sim = ParticleSimulation(n, T, w.extent, w.extent, w.extent)
    sim.set_stream(stream.cuda_stream)
    sim.set_particles(pos, types)
    sim.setRadioByType(np.zeros(T, np.float32))
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    lib = _lib.load()
    bins, r_max = cfg["bins"], cfg["r_max"]
    with torch.cuda.stream(stream):
        hist = torch.empty((T, T, bins), dtype=torch.float32, device="cuda")
        target = torch.empty_like(hist)
        ghist = torch.empty_like(hist)
        pos4 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        pos4[:, :3] = torch.from_numpy(pos).cuda()
        vel4 = torch.zeros_like(pos4)
        xk, vk, gx, g0, gv0 = (torch.empty_like(pos4) for _ in range(5))
    stream.synchronize()
    # target: the radial distribution after K steps under the hidden table
    sim.setForceTable(target_table)
    sim.rollout_forward(params, K, cfg["every"], pos4.data_ptr(), vel4.data_ptr(), xk.data_ptr(), None)
    sim.rdf(bins, r_max, target.data_ptr(), xk.data_ptr())
    sim.sync()
    sim.setForceTable(table)
    s0 = sim.get_state()

    def train_step():
        sim.rollout_forward(params, K, cfg["every"], pos4.data_ptr(), vel4.data_ptr(), xk.data_ptr(), None)
        sim.rdf(bins, r_max, hist.data_ptr(), xk.data_ptr())
        with torch.cuda.stream(stream):
            torch.sub(hist, target, out=ghist).mul_(2.0 / hist.numel())
        sim.rdf_backward(bins, r_max, ghist.data_ptr(), gx.data_ptr(), xk.data_ptr())
        return sim.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), gv0.data_ptr())

    def timed(fn, reps):
        ms = []
        for _ in range(reps):
            sim.set_state(*s0)
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    for _ in range(max(warmup, 3)):
        sim.set_state(*s0)
        train_step()
    sim.sync()
    reps = max(1, steps // 10) if steps >= 10 else steps
    clocks = ClockSampler(local)
    clocks.start()
    fwd_plain = timed(lambda: sim.simulate(params, K), reps)
    fwd_roll = timed(lambda: sim.rollout_forward(params, K, cfg["every"], None, None, None, None), reps)
    bwd = timed(lambda: sim.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), gv0.data_ptr()), reps)
    tally0 = lib.cf_kernel_launches()
    train = timed(train_step, reps)
    launches = lib.cf_kernel_launches() - tally0
    clk = clocks.stop()
    med = statistics.median
    step_fwd = med(fwd_plain) / K
    step_bwd = med(bwd) / K
    value = n * K / (med(train) * 1e-3)
    # end to end: host positions in, gradients out (pinned), one training pass
    hpos = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    hpos[:, :3] = torch.from_numpy(pos)
    hgrad = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    e2e = []
    for _ in range(reps):
        sim.set_state(*s0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            pos4.copy_(hpos, non_blocking=True)
        gF, gp = train_step()  # reads the table and parameter gradients back (synchronises)
        with torch.cuda.stream(stream):
            hgrad.copy_(g0, non_blocking=True)
        stream.synchronize()
        e2e.append(time.perf_counter() - t0)
    # ---- adjoint roofline: a profiled backward (events around each adjoint step's kernels),
    # and the work counters of the K forward states it differentiates
    sim.set_state(*s0)
    sim.rollout_forward(params, K, cfg["every"], None, None, None, None)
    _lib.check(lib.cf_profile_enable(sim.handle, 1), "cf_profile_enable")
    sim.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), gv0.data_ptr())
    prof = _lib.PhaseTimes()
    _lib.check(lib.cf_profile_read(sim.handle, C.byref(prof)), "cf_profile_read")
    _lib.check(lib.cf_profile_enable(sim.handle, 0), "cf_profile_enable")
    sim.set_state(*s0)
    c27_total, inter_total = 0, 0
    for _ in range(K):
        c27, _ = sim.work_counters(params)
        sim.simulate(params, 1)
        _, inter = sim.work_counters(params)
        c27_total += c27
        inter_total += inter
    adj_flops = 9 * c27_total + 70 * inter_total + 41 * n * K
    adj_tflops = adj_flops / (prof.adjoint_ms * 1e-3) / 1e12 if prof.adjoint_ms > 0 else None
    peak_fp32 = C.c_double()
    _lib.check(lib.cf_measure_fp32_peak(C.byref(peak_fp32)), "cf_measure_fp32_peak")
    line = None
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": reps, "warmup": max(warmup, 3), "ms_per_step": med(train),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox4x32-10): uniform positions, N(0,0.5) table, hidden N(0,0.5) target "
                    "table",
            "config": {"workload": name, "n": n, "types": T, "radius": cfg["radius"], "rollout_steps": K,
                       "checkpoint_every": cfg["every"], "loss": f"MSE of the soft radial distribution "
                       f"({bins} bins, r <= {r_max})", "l2": "state smaller than L2; 256 MiB flush before each "
                       "timed pass"},
            "unit_of_step": "one forward + backward pass of the K-step rollout and its loss",
            "forward_step_ms": step_fwd, "rollout_forward_step_ms": med(fwd_roll) / K,
            "adjoint_step_ms": step_bwd, "adjoint_over_forward": step_bwd / step_fwd,
            "roofline": {
                "kernel": "adj_prep_kernel + adj_pair_kernel (one backward step), timed alone in a profiled "
                          "backward",
                "bound": "fp32", "achieved": adj_tflops, "peak": peak_fp32.value, "unit": "TFLOP/s",
                "frac": adj_tflops / peak_fp32.value if adj_tflops else None,
                "peak_source": "FP32 FMA chains on every SM, measured in this run (cf_measure_fp32_peak)",
                "work_model": "9*C27 + 70*I + 41*N flops per adjoint step (include/cellflow/work_model.h)",
                "adjoint_kernels_ms_per_step": prof.adjoint_ms / max(prof.adjoint_steps, 1),
                "steps": int(prof.adjoint_steps),
                "c27_per_particle_step": c27_total / (n * K),
                "interacting_per_particle_step": inter_total / (n * K),
            },
            "e2e": {"value": n * K / med(e2e), "unit": "particle-steps/s", "h2d_bytes_per_step": n * 16,
                    "d2h_bytes_per_step": n * 16 + 4 * (T * T + 6),
                    "path": "pinned positions in, rollout + loss + adjoint, pinned position gradients out"},
            "gpu_launches": int(launches), "clocks": clk,
        }
        if not args.no_cpu_baseline:
            # the reference has no adjoint: its forward step on the rollout's world, for scale
            v, kind, cores, desc = cpu_reference_sample(w, params, pos, types, table,
                                                        np.zeros(T, np.float32), cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": kind,
                                    "sample": desc + " (forward step only: the reference has no adjoint)",
                                    "cpu_model": host_cpu_model()}
    sim.close()
    return line


def proximity_timing(sim, w, stream, calls):
    """Proximity-graph edges/s at the workload's distance and connection limit, in the
    reference's call shape (generateProximityGraph, ParticleSimulation.cu:625-687): line
    vertices written into a device buffer standing in for the GL VBO, the vertex count read
    back, one synchronising call per frame.  Also the host edge list (cf_proximity_edges)
    and the reference's own kernel built for sm_103a on the same particles."""
    import numpy as np
    import torch

    import oracle

    n, mc, dist = w.n, w.prox_max_conn, w.prox_distance
    cap_v = 2 * n * mc
    verts = torch.empty(cap_v * 6, dtype=torch.float32, device="cuda")
    colors = [((t * 37 % 11) / 10.0, (t * 53 % 7) / 6.0, (t * 17 % 5) / 4.0) for t in range(w.num_types)]
    torch.cuda.synchronize()
    for _ in range(3):
        sim.proximity_vertices_device(dist, mc, colors, verts.data_ptr(), cap_v)
    t0 = time.perf_counter()
    for _ in range(calls):
        nv = sim.proximity_vertices_device(dist, mc, colors, verts.data_ptr(), cap_v)
    dev_s = (time.perf_counter() - t0) / calls
    edges = nv // 2
    sim.proximity_edges(dist, mc)
    t0 = time.perf_counter()
    for _ in range(calls):
        host_edges = sim.proximity_edges(dist, mc)
    host_s = (time.perf_counter() - t0) / calls
    peaks = measured_peaks()
    prox_bytes = 16 * n + 8 * int(edges)
    out = {
        "distance": dist, "max_conn": mc, "edges": int(edges), "calls": calls,
        "value": edges / dev_s, "unit": "edges/s", "ms_per_call": dev_s * 1e3,
        "roofline": {"bound": "hbm", "achieved": prox_bytes / dev_s / 1e9, "peak": peaks.get("hbm_gbs"),
                     "unit": "GB/s", "frac": prox_bytes / dev_s / 1e9 / peaks.get("hbm_gbs", 6800.0),
                     "work_model": "16 B/particle + 8 B/edge per call (the call is latency-bound: the proximity "
                                   "grid's cell list, a selection pass that writes the vertices, a count "
                                   "read-back)"},
        "path": "cf_proximity_vertices_device (device VBO written by the selection pass in arbitrary edge order, as the reference's atomicAdd append; count read back; synchronising, as the reference)",
        "host_edges": {"value": len(host_edges) / host_s, "unit": "edges/s", "ms_per_call": host_s * 1e3,
                       "path": "cf_proximity_edges (int32 pairs into host memory)"},
    }
    try:
        lib = oracle.ref_gpu_lib()
    except (FileNotFoundError, OSError) as exc:
        out["reference_gpu_kernel"] = {"unavailable": str(exc)}
        return out
    rec = sim.getParticleData()
    parts = torch.from_numpy(np.ascontiguousarray(rec).view(np.uint8).copy()).cuda()
    cols = torch.tensor(np.asarray(colors, np.float32).ravel(), device="cuda")
    ref_verts = torch.empty(n * 2 * min(mc, 32) * 6, dtype=torch.float32, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref_calls = 3
    times = []
    with torch.cuda.stream(stream):
        for k in range(ref_calls + 1):
            count.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = lib.cfref_gpu_proximity(C.c_void_p(parts.data_ptr()), n, dist, mc, C.c_void_p(cols.data_ptr()),
                                         w.num_types, C.c_void_p(ref_verts.data_ptr()),
                                         C.c_void_p(count.data_ptr()), C.c_void_p(stream.cuda_stream))
            if rc:
                raise RuntimeError(f"reference proximity kernel launch failed: {rc}")
            e1.record(stream)
            e1.synchronize()
            if k:
                times.append(e0.elapsed_time(e1))
    ref_edges = int(count.item()) // 2
    ms = sum(times) / len(times)
    out["reference_gpu_kernel"] = {
        "value": ref_edges / (ms * 1e-3), "unit": "edges/s", "ms_per_call": ms, "edges": ref_edges,
        "same_edge_count": ref_edges == edges,
        "calls": ref_calls, "note": "reference O(N^2) kernel <<<ceil(N/256),256>>>, kernel time only (CUDA events)"}
    return out


def reference_gpu_kernel(w, params, pos, types, table, radio, stream):
    """The reference step kernel (sm_103a build of ParticleSimulation.cu:69-166) on the same
    inputs, launched as ParticleSimulation::simulate does; a few steps, CUDA events."""
    import numpy as np
    import torch

    import oracle

    try:
        lib = oracle.ref_gpu_lib()
    except (FileNotFoundError, OSError) as exc:
        return {"unavailable": str(exc)}
    rec = oracle.to_records(pos, np.zeros_like(pos), types)
    d_part = torch.from_numpy(rec.view(np.uint8).copy()).cuda()
    d_table = torch.from_numpy(np.ascontiguousarray(table, np.float32).ravel()).cuda()
    d_radio = torch.from_numpy(radio).cuda()
    cnt = [torch.zeros(w.n, dtype=torch.int32, device="cuda") for _ in range(2)]
    p = params
    steps = 3 if w.n <= 200_000 else 1

    def launch(k):
        rc = lib.cfref_gpu_step(C.c_void_p(d_part.data_ptr()), C.c_void_p(d_table.data_ptr()),
                                C.c_void_p(d_radio.data_ptr()), C.c_void_p(cnt[k % 2].data_ptr()),
                                C.c_void_p(cnt[(k + 1) % 2].data_ptr()), w.n, p.radius, p.delta_t, p.friction,
                                p.repulsion, p.attraction, p.k, p.balance, p.canvas_width, p.canvas_height,
                                p.canvas_depth, p.num_particle_types, p.ratio_with_lfo, p.force_multiplier,
                                p.max_expected_neighbors, C.c_void_p(stream.cuda_stream))
        if rc:
            raise RuntimeError(f"reference kernel launch failed: {rc}")

    with torch.cuda.stream(stream):
        launch(0)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            launch(k + 1)
        e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": w.n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms, "steps": steps,
            "note": "reference O(N^2) kernel, in place (racy as in the reference), <<<ceil(N/256),256>>>"}


def profile_steps(args) -> None:
    """--profile-steps S: S plain steps of the workload from its initial state under one force-kernel
    variant, nothing timed, for an ncu capture of step k with `-k regex:step_force_kernel -s k-1 -c 1`;
    then, where the workload has a proximity distance, one proximity-graph call (device vertices,
    the reference's call shape).  For a rollout workload: one forward + loss + backward pass of an
    S-step rollout instead (zero loss target), the launch sequence of one training pass."""
    import numpy as np

    from cellflow_gb300 import inputs
    from cellflow_gb300.world import ParticleSimulation

    if args.workload in ROLLOUT:
        profile_rollout(args)
        return
    w = inputs.WORKLOADS[args.workload]
    params = w.params()
    sim = ParticleSimulation(w.n, w.num_types, w.extent, w.extent, w.extent)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(w.num_types, np.float32))
    if args.variant is not None:
        sim.set_force_variant(args.variant)
    sim.simulate(params, args.profile_steps)
    sim.sync()
    edges = None
    if w.prox_distance is not None:
        import torch

        cap_v = 2 * w.n * w.prox_max_conn
        verts = torch.empty(cap_v * 6, dtype=torch.float32, device="cuda")
        colors = [(1.0, 1.0, 1.0)] * w.num_types
        edges = sim.proximity_vertices_device(w.prox_distance, w.prox_max_conn, colors, verts.data_ptr(), cap_v) // 2
    sim.close()
    print(json.dumps({"profile_steps": args.profile_steps, "workload": w.name, "variant": args.variant,
                      "proximity_edges": edges}))


def profile_rollout(args) -> None:
    """--profile-steps S on a rollout workload: one S-step training pass (cf_rollout_forward,
    cf_rdf, cf_rdf_backward, cf_rollout_backward) on the workload's world, nothing timed."""
    import numpy as np
    import torch

    from cellflow_gb300 import inputs
    from cellflow_gb300.world import ParticleSimulation

    cfg = ROLLOUT[args.workload]
    n, T, K = cfg["n"], cfg["types"], args.profile_steps
    w = inputs.Workload(args.workload, n=n, num_types=T, radius=cfg["radius"], steps=K, seed=cfg["seed"])
    params = w.params()
    stream = torch.cuda.Stream()
    sim = ParticleSimulation(n, T, w.extent, w.extent, w.extent)
    sim.set_stream(stream.cuda_stream)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(T, np.float32))
    bins, r_max = cfg["bins"], cfg["r_max"]
    with torch.cuda.stream(stream):
        hist = torch.empty((T, T, bins), dtype=torch.float32, device="cuda")
        ghist = torch.empty_like(hist)
        xk, gx, g0, gv0 = (torch.empty((n, 4), dtype=torch.float32, device="cuda") for _ in range(4))
    stream.synchronize()
    sim.rollout_forward(params, K, min(cfg["every"], K), None, None, xk.data_ptr(), None)
    sim.rdf(bins, r_max, hist.data_ptr(), xk.data_ptr())
    with torch.cuda.stream(stream):
        torch.mul(hist, 2.0 / hist.numel(), out=ghist)
    sim.rdf_backward(bins, r_max, ghist.data_ptr(), gx.data_ptr(), xk.data_ptr())
    sim.rollout_backward(gx.data_ptr(), None, g0.data_ptr(), gv0.data_ptr())
    sim.sync()
    sim.close()
    print(json.dumps({"profile_steps": K, "workload": args.workload}))


HEADLINE = "plain_n100k_t8"
# the nested records of the default run: (workload, steps, warm-up steps)
NESTED = (("blobs_n1m_t12", 20, 3), ("batched_256w", 100, 100), ("rollout_n16k_k64", 5, 3))


def run_workload(args, rank, world, local, name, steps, warmup, cpu_seconds, extras=True):
    from cellflow_gb300 import inputs

    if name in inputs.BATCHED:
        return run_batched(args, rank, world, local, name, steps, warmup, cpu_seconds)
    if name in ROLLOUT:
        return run_rollout(args, rank, world, local, name, steps, warmup, cpu_seconds)
    return run_gb300(args, rank, world, local, name, steps, warmup, cpu_seconds, extras)


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.workload is None:
        args.workload = HEADLINE
        nested = not args.no_nested
    else:
        nested = False
    if args.profile_steps is not None:
        profile_steps(args)
        return
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    line = run_workload(args, rank, world, local, args.workload, args.steps, args.warmup, args.cpu_seconds)
    if nested:
        # the other configurations, each with its own timing, roofline, CPU baseline and e2e
        records = {}
        for name, steps, warmup in NESTED:
            records[name] = run_workload(args, rank, world, local, name, steps, warmup, args.cpu_seconds / 2,
                                         extras=False)
        if line is not None:
            line["workloads"] = records
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
