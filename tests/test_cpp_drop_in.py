"""The C++ drop-in (include/cellflow/ParticleSimulation.hpp): a caller written against the
reference's class compiles against it (CPU) and computes what the Python binding computes
(GPU, same seeds, same calls)."""

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "drop_in.cpp"
LIB_DIR = ROOT / "cellflow_gb300"
CUDA = Path("/usr/local/cuda")


def compile_drop_in(out: Path) -> Path:
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = out / "drop_in"
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off", f"-I{ROOT / 'include'}",
           f"-I{CUDA / 'include'}", str(SRC), "-o", str(exe), f"-L{LIB_DIR}", "-lcellflow", f"-L{CUDA / 'lib64'}",
           "-lcudart", f"-Wl,-rpath,{LIB_DIR}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_drop_in_compiles(cflib, tmp_path):
    assert compile_drop_in(tmp_path).exists()


@pytest.mark.gpu
def test_drop_in_matches_python_binding(cflib, tmp_path):
    """The C++ frame loop and the same calls through the Python binding give the same
    particles, proximity graph and triangle mesh."""
    from cellflow_gb300.world import ParticleSimulation, SimulationParams, lfo_ratio

    exe = compile_drop_in(tmp_path)
    n, steps = 4096, 5
    r = subprocess.run([str(exe), str(n), str(steps)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    fields = dict(kv.split("=") for kv in r.stdout.split()[3:])

    T = 6
    sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0, seed=1)
    sim.updateCanvasDimensions(2.0, 2.0)
    sim.initializeParticles(seed=2, spawn_region=2000.0)
    for i in range(T):
        sim.setRadioByTypeValue(i, float(np.float32(0.05) * np.float32(i)))
    sim.regenerateForceTable(seed=3)
    raw = sim.getRawForceTableValues().copy()
    raw.reshape(-1)[0] = 0.5
    raw.reshape(-1)[T + 1] = -0.25
    sim.setRawForceTableValues(raw)
    sim.updateForceTable(0.28, -0.20, 1.0)
    params = SimulationParams(radius=0.1, delta_t=0.01, canvas_width=2.0, canvas_height=2.0, canvas_depth=2.0,
                              num_particle_types=T)

    def frame(f):
        params.ratio_with_lfo = lfo_ratio(0.1, 0.05, 0.5, float(np.float32(f) / np.float32(60.0)))
        sim.simulate(params, 1)

    for f in range(steps):
        frame(f)
    sim.moveUniverse(-0.125, 0.0)
    sim.moveUniverse(0.0, 0.125)
    frame(steps)
    sim.rotateRadioByType()
    frame(steps + 1)
    rec = sim.getParticleData()
    edges = sim.proximity_edges(0.05, 5)
    tris = sim.triangle_mesh(0.05, 5)
    sim.close()
    assert int(fields["frames"]) == steps + 2 and int(fields["mapped"]) == 0
    assert int(fields["line_vertices"]) == 2 * len(edges)
    assert int(fields["triangle_vertices"]) == 3 * len(tris)
    first = np.array([float(v) for v in r.stdout.split()[0][len("first=("):-1].split(",")], np.float32)
    assert np.array_equal(first, rec["pos"][0])  # printed with 9 digits: exact for float32
    pos_sum = float(np.sum(rec["pos"].astype(np.float64)))
    assert abs(float(fields["pos_sum"]) - pos_sum) <= 1e-9 * max(1.0, abs(pos_sum))
    assert int(float(fields["type_sum"])) == int(rec["ptype"].sum())


@pytest.mark.gpu
def test_move_universe_matches_reference_arithmetic(cflib):
    """moveUniverse (ParticleSimulation.cu:169-185): every coordinate becomes
    fmodf((p + d) + W, W) in float32, with the world's own box (the reference
    used a default 8000-unit canvas there whatever the world's box)."""
    from cellflow_gb300.world import ParticleSimulation

    n, W, H = 5000, 3.0, 2.0
    rng = np.random.default_rng(3)
    ext = np.array([W, H, H], np.float32)
    pos = (rng.random((n, 3), dtype=np.float32) * ext).astype(np.float32)
    types = rng.integers(0, 4, n).astype(np.uint32)
    sim = ParticleSimulation(n, 4, W, H, H)
    sim.set_particles(pos, types)
    want = pos.copy()
    for d in ((-0.7, 0.0, 0.0), (0.0, 1.9, 0.0), (2.5, -1.25, 0.3), (-2.9, 0.0, -1.999)):
        sim.moveUniverse(*d)
        dd = np.array(d, np.float32)
        want = np.fmod((want + dd) + ext, ext).astype(np.float32)
    got = sim.get_state()[0]
    assert np.array_equal(got[:, :3], want)
    assert np.array_equal(got[:, 3].view(np.uint32), types)
    sim.updateCanvasDimensions(4.0, 4.0)  # the depth follows the height
    sim.moveUniverse(0.5, 0.5)
    want = np.fmod((want + np.float32(0.5) * np.array([1, 1, 0], np.float32)) + np.float32(4.0), np.float32(4.0))
    assert np.array_equal(sim.get_state()[0][:, :3], want.astype(np.float32))
    sim.close()
