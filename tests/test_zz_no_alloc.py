"""cf_proximity_edges_noalloc: proximity edges for callers that may not allocate device
memory while they run (a renderer's per-frame loop, or an application whose device
memory belongs to its own pool).  It keeps all scratch in one fixed device array, so
this test checks, through the C ABI, that two calls in a row give exactly the edges
of cf_proximity_edges and of the oracle's restatement of the reference kernel
(edges are integer pairs: the tolerance is equality), and that sizes beyond its
fixed capacity are refused.  This file is collected last."""

import ctypes as C

import numpy as np
import pytest

import oracle
from cellflow_gb300 import _lib, inputs
from cellflow_gb300.world import ParticleSimulation

pytestmark = pytest.mark.gpu


def edges_without_allocating(lib, sim, extent, distance, max_conn, cap):
    import torch

    view = sim.device_buffers()
    out = torch.full((max(cap, 1), 2), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    count = C.c_int(-1)
    rc = lib.cf_proximity_edges_noalloc(C.c_void_p(view.pos4), view.n, extent, extent, extent, distance, max_conn,
                                        C.c_void_p(out.data_ptr()), cap, C.byref(count), None)
    _lib.check(rc, "cf_proximity_edges_noalloc")
    return out[: count.value].cpu().numpy()


def oracle_edges(sim, distance, max_conn):
    pos4 = sim.get_state()[0]
    return oracle.proximity_edges(pos4[:, :3], pos4[:, 3].view(np.uint32), distance, max_conn)


def test_noalloc_edges_match_twice_in_a_row(cflib):
    w = inputs.Workload("noalloc", n=20000, num_types=4, radius=0.1, steps=1, seed=21)
    sim = ParticleSimulation(w.n, w.num_types, w.extent, w.extent, w.extent)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.sync()

    cap = w.n * 5
    first = edges_without_allocating(cflib, sim, w.extent, 0.08, 5, cap)
    expect_first = sim.proximity_edges(0.08, 5)
    assert len(first) > 1000
    assert np.array_equal(first, expect_first)
    assert np.array_equal(first, oracle_edges(sim, 0.08, 5))

    # second call: moved particles and other parameters, over the previous call's scratch contents
    sim.simulate(w.params(), 2)
    sim.sync()
    second = edges_without_allocating(cflib, sim, w.extent, 0.12, 3, cap)
    expect_second = sim.proximity_edges(0.12, 3)
    assert np.array_equal(second, expect_second)
    assert np.array_equal(second, oracle_edges(sim, 0.12, 3))
    assert not np.array_equal(first[: len(second)], second)
    sim.close()


def test_noalloc_refuses_sizes_beyond_capacity(cflib):
    count = C.c_int(0)
    rc = cflib.cf_proximity_edges_noalloc(C.c_void_p(0), 65537, 2.0, 2.0, 2.0, 0.1, 5, C.c_void_p(0), 0,
                                          C.byref(count), None)
    assert rc == _lib.CF_ERR_INVALID
    assert b"65536" in cflib.cf_last_error()
