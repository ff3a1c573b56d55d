"""Host-side fault injection: a cap on the library's device memory and a one-shot
injected CUDA error at a named call site.  Every failure is made on the host (the
call that would fail is not made), so no GPU faults: the tests check that the
error comes back as the status code and message the library documents, that no
half-built object is left behind, and that the world works again afterwards."""

import ctypes as C

import numpy as np
import pytest

from cellflow_gb300 import inputs
from cellflow_gb300._lib import CF_ERR_ALLOC, CF_ERR_CUDA, CF_ERR_INVALID, CellFlowError

CUDA_ERROR_MEMORY_ALLOCATION = 2
CUDA_ERROR_LAUNCH_FAILURE = 719
CUDA_ERROR_NOT_READY = 600


def test_injection_arguments(cflib):
    assert cflib.cf_inject_cuda_error(b"cudaMalloc", 0, 0) == CF_ERR_INVALID
    assert cflib.cf_inject_cuda_error(b"cudaMalloc", 2, -1) == CF_ERR_INVALID
    assert cflib.cf_injection_pending() == 0
    assert cflib.cf_inject_cuda_error(b"no such site", 2, 0) == 0
    assert cflib.cf_injection_pending() == 1
    assert cflib.cf_inject_cuda_error(None, 0, 0) == 0
    assert cflib.cf_injection_pending() == 0
    assert cflib.cf_device_memory_in_use(None) == CF_ERR_INVALID


@pytest.fixture
def no_limits(cflib):
    yield
    cflib.cf_set_device_memory_limit(0)
    cflib.cf_inject_cuda_error(None, 0, 0)


def in_use(lib):
    v = C.c_size_t()
    assert lib.cf_device_memory_in_use(C.byref(v)) == 0
    return v.value


def world(n=3000, T=4, seed=5):
    from cellflow_gb300.world import ParticleSimulation

    w = inputs.Workload("fault", n=n, num_types=T, radius=0.15, steps=1, seed=seed)
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(T, np.float32))
    return sim, w.params()


@pytest.mark.gpu
def test_memory_limit_fails_cleanly_and_recovers(cflib, no_limits):
    from cellflow_gb300.world import ParticleSimulation

    base = in_use(cflib)
    cflib.cf_set_device_memory_limit(base + 4096)
    with pytest.raises(CellFlowError) as e:
        ParticleSimulation(100_000, 6, 2.0, 2.0, 2.0)
    assert e.value.code == CF_ERR_ALLOC and "limit" in str(e.value)
    assert in_use(cflib) == base  # nothing of the failed world is held
    cflib.cf_set_device_memory_limit(0)

    sim, params = world()
    ref, _ = world()
    held = in_use(cflib)
    cflib.cf_set_device_memory_limit(held + 4096)
    with pytest.raises(CellFlowError) as e:
        sim.setParticleCount(500_000)
    assert e.value.code == CF_ERR_ALLOC
    # no half-allocated world: every call reports it, none launches work
    with pytest.raises(CellFlowError) as e:
        sim.simulate(params, 1)
    assert e.value.code == CF_ERR_INVALID and "reallocation" in str(e.value)
    cflib.cf_set_device_memory_limit(0)
    sim.setParticleCount(3000, seed=5)
    sim.simulate(params, 1)
    sim.close()
    ref.close()


@pytest.mark.gpu
def test_lazy_scratch_allocation_failure_leaves_no_half_pair(cflib, no_limits):
    """The proximity buffers are allocated on first use as a pair: the second of the
    two failing must not leave the first in place as if both existed."""
    sim, params = world()
    want = sim.proximity_edges(0.05, 4)
    sim2, _ = world()
    assert cflib.cf_inject_cuda_error(b"cudaMalloc", CUDA_ERROR_MEMORY_ALLOCATION, 1) == 0  # the second allocation
    with pytest.raises(CellFlowError) as e:
        sim2.proximity_edges(0.05, 4)
    assert e.value.code == CF_ERR_ALLOC
    assert cflib.cf_injection_pending() == 0
    assert np.array_equal(sim2.proximity_edges(0.05, 4), want)
    sim.close()
    sim2.close()


@pytest.mark.gpu
@pytest.mark.parametrize("site", ["launch_step_force", "cudaStreamSynchronize", "cudaGraphLaunch"])
def test_injected_cuda_error_is_reported_and_the_world_recovers(cflib, no_limits, site):
    sim, params = world()
    ref, _ = world()
    assert cflib.cf_inject_cuda_error(site.encode(), CUDA_ERROR_LAUNCH_FAILURE, 0) == 0
    with pytest.raises(CellFlowError) as e:
        sim.simulate(params, 1)
        sim.sync()
    assert e.value.code == CF_ERR_CUDA
    assert site in str(e.value) and "launch failure" in str(e.value)
    assert cflib.cf_injection_pending() == 0
    # the next calls redo the whole step: the state equals a world that never failed
    sim.set_state(*ref.get_state())
    sim.simulate(params, 3)
    ref.simulate(params, 3)
    for a, b in zip(sim.get_state(), ref.get_state()):
        assert np.array_equal(a, b)
    sim.close()
    ref.close()


@pytest.mark.gpu
def test_injection_skips_the_named_number_of_calls(cflib, no_limits):
    sim, params = world()
    sim.simulate(params, 1)  # the step's graph is captured: from here one graph launch per step
    assert cflib.cf_inject_cuda_error(b"cudaGraphLaunch", CUDA_ERROR_NOT_READY, 2) == 0
    sim.simulate(params, 2)
    assert cflib.cf_injection_pending() == 1
    with pytest.raises(CellFlowError):
        sim.simulate(params, 1)
    assert cflib.cf_injection_pending() == 0
    sim.simulate(params, 1)
    sim.close()
