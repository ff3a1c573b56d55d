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
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}",
           str(SRC), "-o", str(exe), f"-L{LIB_DIR}", "-lcellflow", f"-L{CUDA / 'lib64'}", "-lcudart",
           f"-Wl,-rpath,{LIB_DIR}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_drop_in_compiles(cflib, tmp_path):
    assert compile_drop_in(tmp_path).exists()


@pytest.mark.gpu
def test_drop_in_matches_python_binding(cflib, tmp_path):
    from cellflow_gb300.world import ParticleSimulation, SimulationParams

    exe = compile_drop_in(tmp_path)
    n, steps = 4096, 5
    r = subprocess.run([str(exe), str(n), str(steps)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    fields = dict(kv.split("=") for kv in r.stdout.split()[2:])

    sim = ParticleSimulation(n, 6, 2.0, 2.0, 2.0, seed=7)
    sim.initializeParticles(seed=8, spawn_region=2000.0)
    sim.updateForceTable(0.28, -0.20, 1.0)
    params = SimulationParams(radius=0.1, delta_t=0.01, canvas_width=2.0, canvas_height=2.0, canvas_depth=2.0,
                              num_particle_types=6)
    sim.simulate(params, steps)
    rec = sim.getParticleData()
    edges = sim.proximity_edges(0.05, 5)
    tris = sim.triangle_mesh(0.05, 5)
    sim.close()
    assert int(fields["line_vertices"]) == 2 * len(edges)
    assert int(fields["triangle_vertices"]) == 3 * len(tris)
    pos_sum = float(np.sum(rec["pos"].astype(np.float64)))
    assert abs(float(fields["pos_sum"]) - pos_sum) <= 1e-6 * max(1.0, abs(pos_sum))
