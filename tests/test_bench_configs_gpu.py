"""Parity on the benchmarked configurations themselves, at their full sizes.

* the cell list of plain_n100k_t8 (21^3 grid) and blobs_n1m_t12 (115^3 grid),
  after a few steps have made the blob cells dense: cell ids, sorted order and
  cell bounds bit-exact against the oracle's stable sort;
* one step of plain_n100k_t8 and blobs_n1m_t12 from an evolved state (non-zero
  velocities and previous counts): a strided sample of particles against the
  oracle (each sampled particle computed against all N), counts bit-exact and
  acceleration, velocity and position under the per-particle tolerances of
  tests/parity.py; the errors of the GPU and of the FP32 oracle against the
  FP64 oracle are printed;
* the batched_256w batch (256 worlds, 4.1M particles) after one step: sampled
  worlds, the smallest and the largest among them, bit-identical to the same
  world stepped alone, and their counts equal to the oracle on sampled rows.
"""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300.world import Batch, ParticleSimulation
from tests.parity import REL, acc_error, check_step, min_image

pytestmark = pytest.mark.gpu

EVOLVE = {"plain_n100k_t8": 5, "blobs_n1m_t12": 3}
SAMPLE_ROWS = {"plain_n100k_t8": 2000, "blobs_n1m_t12": 400}


def evolved_world(name):
    w = inputs.WORKLOADS[name]
    params = w.params()
    table = w.table()
    sim = ParticleSimulation(w.n, w.num_types, w.extent, w.extent, w.extent)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(table)
    sim.setRadioByType(np.zeros(w.num_types, np.float32))
    sim.simulate(params, EVOLVE[name])
    return w, params, table, sim


@pytest.mark.parametrize("name", ["plain_n100k_t8", "blobs_n1m_t12"])
def test_benchmark_cell_list_bit_exact(cflib, name):
    w, params, _, sim = evolved_world(name)
    pos4, _, _ = sim.get_state()
    g, cell_of, order, start, end = sim.cell_list(params)
    sim.close()
    # the step's grid: the largest cells per axis whose side exceeds the geometric cutoff
    # sqrt(radius^2 - 1e-4) (21^3 at 100k, 115^3 at 1M)
    assert min(g.cells) >= 5 and not g.generic_wrap
    o_cell, o_order, o_start, o_end = oracle.cell_list(pos4[:, :3], list(g.cells), list(g.inv_cell))
    assert np.array_equal(cell_of, o_cell)
    assert np.array_equal(order, o_order)
    assert np.array_equal(start, o_start)
    assert np.array_equal(end, o_end)
    pop = (end - start).astype(np.int64)
    if name == "blobs_n1m_t12":
        assert pop.max() >= 100  # dense blob cells are part of what was compared
    print(f"\n{name}: {len(cell_of)} particles, {len(start)} cells, largest cell {pop.max()}")


@pytest.mark.parametrize("name", ["plain_n100k_t8", "blobs_n1m_t12"])
def test_benchmark_step_sampled_rows(cflib, name):
    w, params, table, sim = evolved_world(name)
    pos4, vel4, cnt = sim.get_state()
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    sim.close()
    pos, vel = pos4[:, :3].copy(), vel4[:, :3].copy()
    types = pos4[:, 3].view(np.uint32).copy()
    radio = np.zeros(w.num_types, np.float32)
    assert np.abs(vel).max() > 0 and cnt.max() > 0  # an evolved state
    stride = max(1, w.n // SAMPLE_ROWS[name])
    rows = (0, w.n, stride)
    sel = np.arange(0, w.n, stride)
    po, vo, ao, co = oracle.step_f32(pos, vel, types, cnt, table, radio, params, rows=rows)
    p64, v64, a64, c64, mag = oracle.step_f64(pos, vel, types, cnt, table, radio, params, rows=rows)
    assert np.array_equal(counts[sel], co[sel])
    errs = check_step(rec[sel], po[sel], vo[sel], ao[sel], mag[sel], params.delta_t, w.extent, name)
    # errors against FP64, in the units of the tolerance: the GPU and the FP32 oracle side by side
    gpu64 = {"acc": acc_error(rec["acc"][sel], a64[sel], mag[sel]),
             "vel": float(np.abs(rec["vel"][sel] - v64[sel]).max()),
             "pos": float(np.abs(min_image(rec["pos"][sel] - p64[sel], w.extent)).max())}
    ref64 = {"acc": acc_error(ao[sel], a64[sel], mag[sel]),
             "vel": float(np.abs(vo[sel] - v64[sel]).max()),
             "pos": float(np.abs(min_image(po[sel] - p64[sel], w.extent)).max())}
    print(f"\n{name}: {len(sel)} rows, counts exact ({co[sel].mean():.1f} mean); vs FP32 oracle {errs}; "
          f"vs FP64 oracle: GPU {gpu64}, FP32 oracle {ref64} (acc in units of the term size, vel/pos absolute)")
    assert gpu64["acc"] <= 10 * max(ref64["acc"], REL)


def test_batched_256w_worlds_equal_worlds_alone(cflib):
    bw = inputs.BATCHED["batched_256w"]
    params = bw.params()
    sizes = bw.sizes()
    parts = [bw.world(k, int(n)) for k, n in enumerate(sizes)]
    batch = Batch(sizes, bw.num_types, bw.extent, bw.extent, bw.extent, seed=bw.seed)
    batch.set_particles(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]))
    batch.set_force_tables(np.stack([p[2] for p in parts]))
    batch.simulate(params, 1)
    bpos, bvel, bcnt = batch.get_state()
    off = batch.offsets
    batch.close()
    assert off[-1] == int(sizes.sum()) > 4_000_000
    rng = np.random.default_rng(256)
    pick = sorted({int(np.argmin(sizes)), int(np.argmax(sizes)), *rng.choice(bw.worlds, 8, replace=False).tolist()})
    radio = np.zeros(bw.num_types, np.float32)
    for k in pick:
        pos, types, table = parts[k]
        n = len(pos)
        sim = ParticleSimulation(n, bw.num_types, bw.extent, bw.extent, bw.extent)
        sim.set_particles(pos, types)
        sim.setForceTable(table)
        sim.setRadioByType(radio)
        sim.simulate(params, 1)
        apos, avel, acnt = sim.get_state()
        sim.close()
        a, b = off[k], off[k + 1]
        assert np.array_equal(bpos[a:b, :3], apos[:, :3]), f"world {k}: positions differ from the world alone"
        assert np.array_equal(bvel[a:b, :3], avel[:, :3]), f"world {k}: velocities differ from the world alone"
        assert np.array_equal(bcnt[a:b], acnt), f"world {k}: counts differ from the world alone"
        stride = max(1, n // 200)
        _, _, _, co = oracle.step_f32(pos, np.zeros_like(pos), types, np.zeros(n, np.int32), table, radio, params,
                                      rows=(0, n, stride))
        sel = np.arange(0, n, stride)
        assert np.array_equal(bcnt[a:b][sel], co[sel]), f"world {k}: counts differ from the oracle"
    print(f"\nbatched_256w: worlds {pick} (sizes {[int(sizes[k]) for k in pick]}) equal the worlds alone")
