"""cf_kernel_launches counts every kernel the library puts on a stream: a step replayed
from its CUDA graph on the world's own stream or on a caller's stream adds the same number,
which is also the step's launch count in the profile record; a batch replay adds its
graph's kernel nodes; a rollout adds one step's kernels per step; the radial distribution,
launched directly, adds its own kernels."""

import ctypes as C

import numpy as np
import pytest

from cellflow_gb300 import _lib, inputs
from cellflow_gb300.world import Batch, ParticleSimulation

pytestmark = pytest.mark.gpu


def world(w):
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    sim.set_particles(w.positions(), w.types())
    sim.setForceTable(w.table())
    sim.setRadioByType(np.zeros(w.num_types, np.float32))
    return sim


def delta(lib, fn):
    t0 = lib.cf_kernel_launches()
    fn()
    return lib.cf_kernel_launches() - t0


def test_step_launches_direct_graph_and_profile_agree(cflib):
    import torch

    lib = _lib.load()
    w = inputs.Workload("tally", n=30000, num_types=5, radius=0.1, steps=1, seed=41)
    params = w.params()
    sim = world(w)
    # the world's own stream
    direct = delta(lib, lambda: (sim.simulate(params, 3), sim.sync()))
    assert direct > 0 and direct % 3 == 0
    # own stream: one captured graph per step, replayed
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.simulate(params, 1)
    sim.sync()
    graph = delta(lib, lambda: (sim.simulate(params, 3), sim.sync()))
    assert graph == direct
    # the profile record's per-step count (a formula over the grid) says the same
    _lib.check(lib.cf_profile_enable(sim.handle, 1), "cf_profile_enable")
    profiled = delta(lib, lambda: (sim.simulate(params, 3), sim.sync()))
    prof = _lib.PhaseTimes()
    _lib.check(lib.cf_profile_read(sim.handle, C.byref(prof)), "cf_profile_read")
    _lib.check(lib.cf_profile_enable(sim.handle, 0), "cf_profile_enable")
    assert profiled == direct == prof.launches
    sim.close()


def test_batch_replay_adds_its_graph_kernels(cflib):
    import torch

    lib = _lib.load()
    bw = inputs.BatchedWorkload("tally_batch", worlds=4, n_min=2048, n_max=4096, num_types=4, radius=0.1,
                                graph_steps=5, seed=43)
    sizes = bw.sizes()
    parts = [bw.world(k, int(n)) for k, n in enumerate(sizes)]
    batch = Batch(sizes, bw.num_types, seed=bw.seed)
    stream = torch.cuda.Stream()
    batch.set_stream(stream.cuda_stream)
    batch.set_particles(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]))
    batch.set_force_tables(np.stack([p[2] for p in parts]))
    batch.capture(bw.params(), bw.graph_steps)
    steps, kernels = batch.graph_info()
    assert steps == bw.graph_steps and kernels > 0
    assert delta(lib, lambda: (batch.replay(), batch.sync())) == kernels
    batch.close()


def test_rollout_forward_counts_each_step(cflib):
    import torch

    lib = _lib.load()
    w = inputs.Workload("tally_roll", n=8192, num_types=4, radius=0.1, steps=1, seed=47)
    params = w.params()
    sim = world(w)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.simulate(params, 1)
    sim.sync()
    per_step = delta(lib, lambda: (sim.simulate(params, 1), sim.sync()))
    K = 6
    rolled = delta(lib, lambda: (sim.rollout_forward(params, K, 3, None, None, None, None), sim.sync()))
    assert rolled == K * per_step
    sim.close()


def test_direct_launches_are_counted(cflib):
    """cf_rdf launches its kernels directly: the position pack, the five cell-list kernels
    of its grid, the histogram and its normalisation."""
    import torch

    lib = _lib.load()
    w = inputs.Workload("tally_rdf", n=8192, num_types=4, radius=0.1, steps=1, seed=53)
    sim = world(w)
    T, bins = w.num_types, 16
    hist = torch.empty((T, T, bins), dtype=torch.float32, device="cuda")
    pos4 = torch.zeros((w.n, 4), dtype=torch.float32, device="cuda")
    pos4[:, :3] = torch.from_numpy(w.positions()).cuda()
    torch.cuda.synchronize()
    n = delta(lib, lambda: (sim.rdf(bins, 0.2, hist.data_ptr(), pos4.data_ptr()), sim.sync()))
    assert n == 1 + 5 + 2
    sim.close()
