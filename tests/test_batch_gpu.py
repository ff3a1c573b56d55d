"""Batched ensembles: every world of a batch steps exactly (bit for bit) like the same
world run alone through the plain step, which itself matches the oracle."""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300.world import Batch, ParticleSimulation

pytestmark = pytest.mark.gpu


def world_inputs(k, n, T, seed):
    pos = inputs.uniform_positions(n, seed + k)
    types = inputs.uniform_types(n, T, seed + k)
    table = inputs.gaussian_table(T, 0.0, 0.5, seed + k)
    return pos, types, table


@pytest.mark.parametrize("sizes,radius", [([3000, 17, 9000, 1, 0, 5000], 0.1), ([2048, 4096, 65536 // 8], 0.3)])
def test_batch_equals_worlds_run_alone(cflib, sizes, radius):
    T, seed = 6, 77
    w = inputs.Workload("b", n=1, num_types=T, radius=radius, steps=1, seed=seed)
    params = w.params()
    batch = Batch(sizes, T, 2.0, 2.0, 2.0, seed=seed)
    parts = [world_inputs(k, n, T, seed) for k, n in enumerate(sizes)]
    batch.set_particles(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]))
    batch.set_force_tables(np.stack([p[2] for p in parts]))
    batch.simulate(params, 3)
    bpos, bvel, bcnt = batch.get_state()
    off = batch.offsets
    batch.close()
    for k, n in enumerate(sizes):
        if n == 0:
            continue
        sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0)
        sim.set_particles(parts[k][0], parts[k][1])
        sim.setForceTable(parts[k][2])
        sim.setRadioByType(np.zeros(T, np.float32))
        sim.simulate(params, 3)
        pos4, vel4, cnt = sim.get_state()
        sim.close()
        s = slice(off[k], off[k + 1])
        assert np.array_equal(bpos[s], pos4), f"world {k} positions"
        assert np.array_equal(bvel[s], vel4), f"world {k} velocities"
        assert np.array_equal(bcnt[s], cnt), f"world {k} counts"


def test_batch_first_step_matches_oracle(cflib):
    sizes, T, seed = [2500, 4000], 5, 91
    w = inputs.Workload("b", n=1, num_types=T, radius=0.12, steps=1, seed=seed)
    params = w.params()
    batch = Batch(sizes, T, seed=seed)
    parts = [world_inputs(k, n, T, seed) for k, n in enumerate(sizes)]
    batch.set_particles(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]))
    batch.set_force_tables(np.stack([p[2] for p in parts]))
    batch.simulate(params, 1)
    _, _, cnt = batch.get_state()
    off = batch.offsets
    batch.close()
    for k, n in enumerate(sizes):
        pos, types, table = parts[k]
        _, _, _, co = oracle.step_f32(pos, np.zeros_like(pos), types, np.zeros(n, np.int32), table,
                                      np.zeros(T, np.float32), params)
        assert np.array_equal(cnt[off[k]:off[k + 1]], co)


def test_batch_graph_replay_equals_steps(cflib):
    sizes, T = [5000, 3000, 7000], 6
    w = inputs.Workload("b", n=1, num_types=T, radius=0.1, steps=1, seed=5)
    params = w.params()
    a = Batch(sizes, T, seed=5)
    b = Batch(sizes, T, seed=5)
    a.simulate(params, 6)
    b.capture(params, 3)
    b.replay()
    b.replay()
    sa = a.get_state()
    sb = b.get_state()
    a.close()
    b.close()
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y)


def test_batch_types_out_of_range_reported(cflib):
    from cellflow_gb300._lib import CellFlowError

    batch = Batch([100, 100], 3)
    pos = inputs.uniform_positions(200, 1)
    types = np.zeros(200, np.uint32)
    types[150] = 7
    batch.set_particles(pos, types)
    batch.simulate(inputs.Workload("b", n=1, num_types=3, radius=0.1, steps=1).params(), 1)
    with pytest.raises(CellFlowError):
        batch.sync()
    batch.close()
