"""cf_step_host (one step from and to host records) equals cf_set_particles + cf_step +
cf_get_particles bit for bit, with page-locked buffers (one CUDA graph; aligned and not)
and pageable ones (the three calls), and reports a position outside the box like the
separate calls."""

import numpy as np
import pytest

from cellflow_gb300 import inputs
from cellflow_gb300._lib import CF_ERR_DOMAIN, CellFlowError
from cellflow_gb300.world import PARTICLE_DTYPE, ParticleSimulation

pytestmark = pytest.mark.gpu


def world(w):
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(w.num_types, np.float32))
    return sim


def pinned_records(n, offset=0):
    """Page-locked 44-B records starting `offset` bytes into a page-locked allocation."""
    import torch

    buf = torch.empty(n * PARTICLE_DTYPE.itemsize + 16, dtype=torch.uint8).pin_memory()
    return buf, buf.numpy()[offset:offset + n * PARTICLE_DTYPE.itemsize].view(PARTICLE_DTYPE)


# page-locked records are read and written in place word by word, at any 4-B aligned
# start (offset 4) and any count; pageable ones go through the three calls
@pytest.mark.parametrize("n,pinned,offset", [(20000, True, 0), (10240, True, 0), (20000, True, 4),
                                             (20000, False, 0)])
def test_step_host_equals_the_three_calls(cflib, n, pinned, offset):
    w = inputs.Workload("host", n=n, num_types=5, radius=0.1, steps=1, seed=31)
    params = w.params()
    a, b = world(w), world(w)
    rec = a.getParticleData()
    keep = None
    if pinned:
        keep, io = pinned_records(w.n, offset)
        io[:] = rec
    else:
        io = rec.copy()
    for step in range(4):
        ref_in = io.copy()
        b.setParticleData(ref_in)
        b.simulate(params, 1)
        ref = b.getParticleData()
        a.step_host(params, io, io)
        for f in ("pos", "vel", "acc", "ptype"):
            assert np.array_equal(io[f], ref[f]), (step, f)
        assert np.array_equal(a.getNeighborCounts(), b.getNeighborCounts())
    a.close()
    b.close()
    del keep


def test_step_host_reports_domain_errors(cflib):
    w = inputs.Workload("host_err", n=1000, num_types=3, radius=0.1, steps=1, seed=32)
    params = w.params()
    sim = world(w)
    keep, io = pinned_records(w.n)
    io[:] = sim.getParticleData()
    sim.step_host(params, io, io)
    io["pos"][7] = (2.5, 0.5, 0.5)
    with pytest.raises(CellFlowError) as e:
        sim.step_host(params, io, io)
    assert e.value.code == CF_ERR_DOMAIN
    io["pos"][7] = (0.5, 0.5, 0.5)
    sim.step_host(params, io, io)  # the error word was cleared
    sim.close()
    del keep
