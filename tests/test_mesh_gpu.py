"""Triangle mesh on the GPU (cf_triangle_mesh / cf_triangle_mesh_device) against the oracle,
which reproduces the reference kernel body (ParticleSimulation.cu:280-424) bit for bit:
triangles in i order then pair order, vertices bit-exact (positions, flat normals, colours)."""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300._lib import CellFlowError
from cellflow_gb300.world import ParticleSimulation
from tests.test_oracle import GOLDEN, mesh_case

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def world(pos, types, T, extent=2.0):
    sim = ParticleSimulation(len(pos), T, extent, extent, extent)
    sim.set_particles(pos, types)
    return sim


def device_vertices(sim, dist, mc, cols):
    tris = sim.triangle_mesh(dist, mc)
    buf = torch.zeros((max(3 * len(tris), 1), 9), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    count = sim.triangle_mesh_device(dist, mc, cols.tolist(), buf.data_ptr(), 3 * len(tris))
    torch.cuda.synchronize()
    return tris, buf[:count].cpu().numpy()


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_mesh_matches_reference_golden(cflib, tag):
    g = np.load(GOLDEN / "mesh_n1024.npz")
    pos, types, dist, mc, cols, T = mesh_case(g, tag)
    sim = world(pos, types, T)
    tris, verts = device_vertices(sim, dist, mc, cols)
    sim.close()
    o_tris, _ = oracle.triangle_mesh(pos, types, dist, mc, cols, T)
    assert np.array_equal(tris, o_tris)
    assert np.array_equal(verts.view(np.uint32), g[f"{tag}_vertices"].view(np.uint32))


@pytest.mark.parametrize("n,T,dist,mc", [(6000, 6, 0.06, 8), (3000, 1, 0.08, 32), (2000, 3, 0.5, 12)])
def test_mesh_matches_oracle(cflib, n, T, dist, mc):
    pos = inputs.uniform_positions(n, 41 + n)
    types = inputs.uniform_types(n, T, 41 + n)
    cols = np.random.default_rng(n).random((T, 3)).astype(np.float32)
    sim = world(pos, types, T)
    tris, verts = device_vertices(sim, dist, mc, cols)
    sim.close()
    o_tris, o_verts = oracle.triangle_mesh(pos, types, dist, mc, cols, T)
    assert np.array_equal(tris, o_tris)
    assert np.array_equal(verts.view(np.uint32), o_verts.view(np.uint32))


def test_mesh_edge_cases(cflib):
    pos = inputs.uniform_positions(500, 3)
    types = inputs.uniform_types(500, 2, 3)
    sim = world(pos, types, 2)
    assert len(sim.triangle_mesh(0.3, 0)) == 0          # max_conn 0: no neighbours kept
    assert len(sim.triangle_mesh(0.0, 8)) == 0          # distance 0: nothing within it
    with pytest.raises(CellFlowError):
        sim.triangle_mesh(-1.0, 4)
    tris = sim.triangle_mesh(0.3, 8)
    import ctypes as C

    count = C.c_int()
    small = np.zeros((1, 3), np.int32)
    rc = sim._lib.cf_triangle_mesh(sim.handle, 0.3, 8, small.ctypes.data, 1, C.byref(count))
    assert rc != 0 and count.value == len(tris)       # capacity error, count still reported
    assert np.array_equal(small[0], tris[0])
    sim.close()
