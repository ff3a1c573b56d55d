"""Proximity-graph edges (ParticleSimulation.cu:188-277) on the GPU against the oracle
and the reference's own kernel body: the edge sets must be identical."""

import ctypes

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300._lib import CellFlowError
from cellflow_gb300.world import ParticleSimulation
from tests.parity import edge_set

pytestmark = pytest.mark.gpu


def world(n, T, seed, extent=2.0, pos=None):
    w = inputs.Workload("prox", n=n, num_types=T, radius=0.1, steps=1, seed=seed, extent=extent)
    pos = w.positions() if pos is None else pos
    types = w.types()
    sim = ParticleSimulation(n, T, extent, extent, extent)
    sim.set_particles(pos, types)
    return sim, pos, types


@pytest.mark.parametrize("n,T,dist,mc", [(4096, 6, 0.05, 5), (20000, 3, 0.08, 5), (6000, 2, 0.3, 3),
                                          (3000, 1, 0.5, 16), (3000, 4, 0.2, 1), (3000, 4, 0.2, 0)])
def test_edges_match_oracle(cflib, n, T, dist, mc):
    sim, pos, types = world(n, T, seed=n + mc)
    got = sim.proximity_edges(dist, mc)
    sim.close()
    ref = oracle.proximity_edges(pos, types, dist, mc)
    assert np.array_equal(got, ref)  # same set and the same i-then-distance order


def test_edges_match_reference_kernel_body(cflib):
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built here")
    n, T = 5000, 3
    sim, pos, types = world(n, T, seed=3)
    got = sim.proximity_edges(0.2, 5)
    sim.close()
    cols = np.random.default_rng(0).random((T, 3)).astype(np.float32)
    verts = oracle.ref_proximity_vertices(oracle.to_records(pos, np.zeros_like(pos), types), 0.2, 5, cols, T)
    key = {pos[i].tobytes(): i for i in range(n)}
    ref = [(key[verts[2 * k, :3].tobytes()], key[verts[2 * k + 1, :3].tobytes()]) for k in range(len(verts) // 2)]
    assert edge_set(got) == set(ref)


def test_truncation_keeps_lowest_indices(cflib):
    """Many in-range candidates: only the first 2*maxConn by index are sorted (:215)."""
    n = 2000
    rng = np.random.default_rng(4)
    pos = (np.float32(1.0) + rng.normal(0, 0.01, (n, 3))).astype(np.float32)
    sim, _, types = world(n, 1, seed=5, pos=pos)
    got = sim.proximity_edges(0.05, 4)
    sim.close()
    ref = oracle.proximity_edges(pos, types, 0.05, 4)
    assert np.array_equal(got, ref)


def test_capacity_error(cflib):
    from cellflow_gb300._lib import CF_ERR_CAPACITY, CellFlowError

    sim, pos, types = world(3000, 2, seed=6)
    with pytest.raises(CellFlowError) as e:
        sim.proximity_edges(0.3, 5, cap=10)
    assert e.value.code == CF_ERR_CAPACITY
    sim.close()


def test_vertices_layout(cflib):
    """Vertex buffer in the reference's format: (x, y, z, r, g, b) for i then j, colour of i's type.
    The edges' order in the buffer is arbitrary (as the reference's atomicAdd append), so the
    vertex pairs are compared with the edge list's as sorted rows."""
    import torch

    n, T = 4000, 3
    sim, pos, types = world(n, T, seed=8)
    edges = sim.proximity_edges(0.1, 5)
    colors = [(0.9, 0.1, 0.2), (0.1, 0.8, 0.3), (0.2, 0.3, 0.9)]
    cap = 2 * len(edges) + 4
    buf = torch.zeros((cap, 6), dtype=torch.float32, device="cuda")
    count = sim.proximity_vertices_device(0.1, 5, colors, buf.data_ptr(), cap)
    v = buf.cpu().numpy()[:count]
    sim.close()
    assert count == 2 * len(edges)
    cols = np.asarray(colors, np.float32)
    want = np.concatenate([pos[edges[:, 0]], cols[types[edges[:, 0]] % T], pos[edges[:, 1]],
                           cols[types[edges[:, 0]] % T]], axis=1)
    got = np.concatenate([v[0::2], v[1::2]], axis=1)
    order = lambda a: a[np.lexsort(a.T[::-1])]
    assert np.array_equal(order(got), order(want))


def test_vertices_capacity(cflib):
    """A vertex buffer too small for the edges gets CF_ERR_CAPACITY (the vertices that fit
    are written, none past the buffer)."""
    import torch

    from cellflow_gb300._lib import CF_ERR_CAPACITY

    n, T = 4000, 3
    sim, pos, types = world(n, T, seed=8)
    edges = sim.proximity_edges(0.1, 5)
    colors = [(0.9, 0.1, 0.2), (0.1, 0.8, 0.3), (0.2, 0.3, 0.9)]
    buf = torch.zeros((8, 6), dtype=torch.float32, device="cuda")
    with pytest.raises(CellFlowError) as e:
        sim.proximity_vertices_device(0.1, 5, colors, buf.data_ptr(), 8)
    assert e.value.code == CF_ERR_CAPACITY
    sim.close()


def test_full_size_edges(cflib):
    """The README-scale configuration (100k, T=8, 0.05, maxConn 5): identical edge list."""
    w = inputs.README_SCALE
    sim, pos, types = world(w.n, w.num_types, seed=w.seed)
    types = w.types()
    pos = w.positions()
    sim.set_particles(pos, types)
    got = sim.proximity_edges(w.prox_distance, w.prox_max_conn)
    sim.close()
    ref = oracle.proximity_edges(pos, types, w.prox_distance, w.prox_max_conn)
    assert np.array_equal(got, ref)


def test_selection_graphs_follow_parameters_and_positions(cflib):
    """The proximity and triangle-mesh passes run as cached graphs: alternating distances and
    connection limits re-capture them, and after steps the cached graphs see the new
    positions.  Every call is checked against the oracle."""
    n, T = 6000, 3
    w = inputs.Workload("prox_cache", n=n, num_types=T, radius=0.1, steps=1, seed=41)
    sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(T, np.float32))
    cols = np.full((T, 3), 0.5, np.float32)
    for step, (dist, mc) in enumerate([(0.05, 5), (0.1, 3), (0.05, 5), (0.05, 2), (0.1, 3)]):
        rec = sim.getParticleData()
        got = sim.proximity_edges(dist, mc)
        assert np.array_equal(got, oracle.proximity_edges(rec["pos"], rec["ptype"], dist, mc)), (step, dist, mc)
        tris = sim.triangle_mesh(dist, mc + 1)
        ref_tris, _ = oracle.triangle_mesh(rec["pos"], rec["ptype"], dist, mc + 1, cols, T)
        assert np.array_equal(tris, ref_tris), (step, dist, mc)
        sim.simulate(w.params(), 2)
    sim.close()
