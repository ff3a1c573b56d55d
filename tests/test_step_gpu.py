"""Parity of the GPU step (cell list + force + integrator) with the oracle.

Every test calls the sm_103a library through its C ABI (ctypes) and checks
against the CPU restatement in oracle/ (and, where built, the reference's
own kernel body compiled on the host), per the tolerances in parity.py.
"""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300._lib import CF_ERR_DOMAIN, CF_ERR_INVALID, CellFlowError
from cellflow_gb300.world import ParticleSimulation, SimulationParams
from tests.parity import check_step

pytestmark = pytest.mark.gpu


def make_world(w: inputs.Workload, pos=None, types=None, table=None, radio=None):
    pos = w.positions() if pos is None else pos
    types = w.types() if types is None else types
    table = w.table() if table is None else table
    radio = np.zeros(w.num_types, np.float32) if radio is None else radio
    sim = ParticleSimulation(w.n, w.num_types, w.extent, w.extent, w.extent)
    sim.set_particles(pos, types)
    sim.setForceTable(table)
    sim.setRadioByType(radio)
    return sim, pos, types, table, radio


def one_step_parity(w, params, pos, types, table, radio, vel=None, counts=None, label=""):
    n = len(pos)
    vel = np.zeros_like(pos) if vel is None else vel
    counts = np.zeros(n, np.int32) if counts is None else counts
    sim = ParticleSimulation(n, w.num_types, params.canvas_width, params.canvas_height, params.canvas_depth)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = types.astype(np.uint32).view(np.float32)
    vel4 = np.zeros((n, 4), np.float32)
    vel4[:, :3] = vel
    sim.set_state(pos4, vel4, counts)
    sim.setForceTable(table)
    sim.setRadioByType(radio)
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    got_counts = sim.getNeighborCounts()
    sim.close()
    po, vo, ao, co = oracle.step_f32(pos, vel, types, counts, table, radio, params)
    _, _, _, c64, mag = oracle.step_f64(pos, vel, types, counts, table, radio, params)
    assert np.array_equal(got_counts, co), f"{label}: neighbour counts differ in {np.sum(got_counts != co)} particles"
    errs = check_step(rec, po, vo, ao, mag, params.delta_t, params.canvas_width, label)
    return rec, got_counts, errs


def test_plain_small_one_step(cflib):
    w = inputs.PLAIN_SMALL
    pos, types, table = w.positions(), w.types(), w.table()
    rec, counts, errs = one_step_parity(w, w.params(), pos, types, table, np.zeros(w.num_types, np.float32),
                                        label="n4096")
    assert 1.5 < counts.mean() < 3.0


def test_plain_small_matches_reference_kernel_body(cflib):
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built here")
    w = inputs.PLAIN_SMALL
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    params = w.params()
    sim, *_ = make_world(w, pos, types, table, radio)
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    sim.close()
    ref, ref_counts = oracle.ref_step(oracle.to_records(pos, np.zeros_like(pos), types), table, radio,
                                      np.zeros(w.n, np.int32), params)
    assert np.array_equal(counts, ref_counts)
    _, _, _, _, mag = oracle.step_f64(pos, np.zeros_like(pos), types, np.zeros(w.n, np.int32), table, radio, params)
    check_step(rec, ref["pos"], ref["vel"], ref["acc"], mag, params.delta_t, 2.0, "vs reference body")


def test_dense_random_velocities_and_prev_counts(cflib):
    w = inputs.Workload("dense", n=3000, num_types=5, radius=0.25, steps=1, seed=11)
    rng = np.random.default_rng(5)
    vel = rng.normal(0, 0.5, (w.n, 3)).astype(np.float32)
    counts = rng.integers(0, 200, w.n).astype(np.int32)
    one_step_parity(w, w.params(), w.positions(), w.types(), w.table(), np.zeros(w.num_types, np.float32),
                    vel=vel, counts=counts, label="dense")


def test_per_type_radius(cflib):
    """ratio != 0: a distinct effective radius per type pair (ParticleSimulation.cu:108-110)."""
    w = inputs.Workload("ratio", n=4000, num_types=7, radius=0.12, steps=1, seed=12)
    params = w.params()
    params.ratio_with_lfo = 0.6
    radio = np.linspace(-0.9, 0.8, w.num_types).astype(np.float32)
    one_step_parity(w, params, w.positions(), w.types(), w.table(), radio, label="per-type radius")


def test_generic_wrap_small_grid(cflib):
    """Radius above a fifth of the box: fewer than 5 cells, per-candidate reference wrap."""
    w = inputs.Workload("coarse", n=1500, num_types=4, radius=0.55, steps=1, seed=13)
    sim, pos, types, table, radio = make_world(w)
    g = sim.grid(w.params())
    sim.close()
    assert g.generic_wrap == 1
    one_step_parity(w, w.params(), pos, types, table, radio, label="generic")


def test_non_cubic_box(cflib):
    w = inputs.Workload("box", n=3000, num_types=3, radius=0.1, steps=1, seed=14)
    params = w.params()
    params.canvas_width, params.canvas_height, params.canvas_depth = 2.0, 1.0, 0.7
    pos = w.positions() * np.array([1.0, 0.5, 0.35], np.float32)
    pos = pos.astype(np.float32)
    pos[:, 1] = np.minimum(pos[:, 1], np.nextafter(np.float32(1.0), np.float32(0)))
    pos[:, 2] = np.minimum(pos[:, 2], np.nextafter(np.float32(0.7), np.float32(0)))
    one_step_parity(w, params, pos, w.types(), w.table(), np.zeros(w.num_types, np.float32), label="box")


def test_app_scale_preset_parameters(cflib):
    """Parameters of the reference's settings.json preset (T=8, radius 285, canvas 8000) with
    particles spawned in its 2000-wide central cube, force table from its transform."""
    n, T = 4096, 8
    params = SimulationParams(radius=285.0, delta_t=0.34, friction=0.5, repulsion=50.0, attraction=0.93, k=21.02,
                              balance=0.3, canvas_width=8000.0, canvas_height=8000.0, canvas_depth=8000.0,
                              num_particle_types=T, ratio_with_lfo=1.0, force_multiplier=1.38,
                              max_expected_neighbors=400)
    u = inputs.unit24(inputs._words(3 * n, 1, 99)).reshape(n, 3)
    pos = (np.float32(3000.0) + u * np.float32(2000.0)).astype(np.float32)
    types = inputs.uniform_types(n, T, 99)
    raw = (inputs.unit24(inputs._words(T * T, 6, 99)) * np.float32(2) - np.float32(1)).astype(np.float32)
    table = oracle.force_table(raw, 0.28, -0.16, -0.32)
    w = inputs.Workload("preset", n=n, num_types=T, radius=285.0, steps=1)
    rec, counts, _ = one_step_parity(w, params, pos, types, table, np.zeros(T, np.float32), label="preset")
    assert counts.mean() > 10


def test_rollout_short(cflib):
    """Ten steps: counts stay bit-exact over the first steps; positions stay close."""
    w = inputs.PLAIN_SMALL
    params = w.params()
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    sim, *_ = make_world(w, pos, types, table, radio)
    p, v, c = pos.copy(), np.zeros_like(pos), np.zeros(w.n, np.int32)
    exact_steps = 0
    for step in range(10):
        sim.simulate(params, 1)
        p, v, _, c = oracle.step_f32(p, v, types, c, table, radio, params)
        got = sim.getNeighborCounts()
        if np.array_equal(got, c) and exact_steps == step:
            exact_steps += 1
    rec = sim.getParticleData()
    sim.close()
    assert exact_steps >= 3, f"counts diverged after {exact_steps} steps"
    d = np.abs(((rec["pos"] - p) + 1.0) % 2.0 - 1.0).max()
    assert d < 1e-3, f"10-step position drift {d}"


def test_autotune_keeps_state_and_results(cflib):
    """Force-kernel stagings give bit-identical steps; splitting an item over 2 or 4 warps,
    and pairing lanes in the drain (staging 2: a home's pairs summed in two parts), change
    only the summation order (same counts, forces within rounding); autotuning restores
    the state."""
    w = inputs.Workload("tune", n=30000, num_types=5, radius=0.12, steps=1, seed=19)
    params = w.params()
    sim, pos, types, table, radio = make_world(w)
    before = sim.get_state()
    chosen = sim.autotune(params, 2)
    assert chosen in range(15)
    after = sim.get_state()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    sim.close()
    results, counts = {}, {}
    for variant in range(15):
        s, *_ = make_world(w, pos, types, table, radio)
        s.set_force_variant(variant)
        s.simulate(params, 1)
        results[variant] = s.getParticleData()
        counts[variant] = s.getNeighborCounts()
        s.close()
    for variant in range(15):
        # the unpaired stagings 0, 1, 3 of one split give identical results; the paired (2) and
        # balanced (12-14) drains add partial sums in their own fixed order
        same_split = variant if variant >= 12 else variant - variant % 4 + (2 if variant % 4 == 2 else 0)
        for f in ("pos", "vel", "acc"):
            assert np.array_equal(results[same_split][f], results[variant][f]), (variant, f)
        assert np.array_equal(counts[0], counts[variant]), variant
        scale = np.abs(results[0]["acc"]).max()
        assert np.abs(results[0]["acc"] - results[variant]["acc"]).max() <= 1e-6 * scale, variant
    s, *_ = make_world(w, pos, types, table, radio)
    with pytest.raises(CellFlowError):
        s.set_force_variant(15)
    s.close()


def test_zero_table_is_pure_friction(cflib):
    w = inputs.Workload("friction", n=2000, num_types=3, radius=0.1, steps=1, seed=15)
    rng = np.random.default_rng(1)
    vel = rng.normal(0, 1, (w.n, 3)).astype(np.float32)
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    sim.set_particles(w.positions(), w.types(), vel)
    sim.setForceTable(np.zeros(9, np.float32))
    params = w.params()
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    sim.close()
    expect = (vel * np.float32(params.friction)).astype(np.float32)
    assert np.array_equal(rec["vel"], expect)
    assert not np.any(rec["acc"])


def test_translation_invariance_counts(cflib):
    """Shifting every particle by a whole number of cells changes no neighbour count."""
    w = inputs.Workload("shift", n=3000, num_types=4, radius=0.1, steps=1, seed=16)
    pos, types, table = w.positions(), w.types(), w.table()
    sim, *_ = make_world(w, pos, types, table)
    sim.simulate(w.params(), 1)
    c0 = sim.getNeighborCounts()
    shifted = ((pos.astype(np.float64) + 0.5) % 2.0).astype(np.float32)
    sim.set_particles(shifted, types)
    sim.simulate(w.params(), 1)
    c1 = sim.getNeighborCounts()
    sim.close()
    _, _, _, o1 = oracle.step_f32(shifted, np.zeros_like(pos), types, np.zeros(w.n, np.int32), table,
                                  np.zeros(w.num_types, np.float32), w.params())
    assert np.array_equal(c1, o1)
    assert abs(int(c0.sum()) - int(c1.sum())) <= 0.01 * c0.sum() + 4


def test_aos_round_trip(cflib):
    w = inputs.PLAIN_SMALL
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    rec = oracle.to_records(w.positions(), np.random.default_rng(0).normal(size=(w.n, 3)), w.types(),
                            acc=np.random.default_rng(1).normal(size=(w.n, 3)))
    sim.setParticleData(rec)
    back = sim.getParticleData()
    sim.close()
    for f in ("pos", "vel", "acc", "ptype"):
        assert np.array_equal(back[f], rec[f]), f


def test_spawn_matches_host_generator(cflib):
    """cf_initialize_particles draws Philox4x32-10 with counter (i,0,0,0) and the seed as key."""
    n, T, seed = 5000, 6, 0x1234_5678_9ABC
    sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0)
    sim.initializeParticles(seed, 2000.0)
    rec = sim.getParticleData()
    sim.close()
    words = inputs.philox4x32(np.arange(n, dtype=np.uint64), 0, seed)
    u = inputs.unit24(words[:, :3])
    expect = (np.float32(0.0) + u * np.float32(2.0)).astype(np.float32)
    assert np.array_equal(rec["pos"], expect)
    assert np.array_equal(rec["ptype"], ((words[:, 3].astype(np.uint64) * T) >> 32).astype(np.uint32))
    assert not np.any(rec["vel"])


def test_domain_error_reported(cflib):
    w = inputs.Workload("bad", n=100, num_types=2, radius=0.1, steps=1, seed=17)
    pos = w.positions()
    pos[3, 0] = 2.5
    sim = ParticleSimulation(w.n, w.num_types, 2.0, 2.0, 2.0)
    sim.set_particles(pos, w.types())
    sim.simulate(w.params(), 1)
    with pytest.raises(CellFlowError) as e:
        sim.sync()
    assert e.value.code == CF_ERR_DOMAIN
    sim.sync()  # the error word was cleared
    sim.close()


def test_invalid_arguments(cflib):
    with pytest.raises(CellFlowError) as e:
        ParticleSimulation(10, 0, 2.0, 2.0, 2.0)
    assert e.value.code == CF_ERR_INVALID
    sim = ParticleSimulation(10, 3, 2.0, 2.0, 2.0)
    params = SimulationParams(num_particle_types=4, canvas_width=2, canvas_height=2, canvas_depth=2)
    with pytest.raises(CellFlowError):
        sim.simulate(params, 1)
    with pytest.raises(CellFlowError):
        sim.proximity_edges(0.1, 17)
    sim.close()


@pytest.mark.parametrize("name", ["plain_n4096_t6", "blobs_small"])
def test_cell_list_bit_exact(cflib, name):
    if name == "blobs_small":
        w = inputs.Workload("blobs_small", n=50_000, num_types=12, radius=0.02, steps=1, blobs=16,
                            blob_sigma=0.02, seed=18)
    else:
        w = inputs.WORKLOADS[name]
    sim, pos, *_ = make_world(w)
    g, cell_of, order, start, end = sim.cell_list(w.params())
    sim.close()
    o_cell, o_order, o_start, o_end = oracle.cell_list(pos, list(g.cells), list(g.inv_cell))
    assert np.array_equal(cell_of, o_cell)
    assert np.array_equal(order, o_order)
    assert np.array_equal(start, o_start)
    assert np.array_equal(end, o_end)


def test_work_counters(cflib):
    w = inputs.PLAIN_SMALL
    sim, pos, types, table, radio = make_world(w)
    params = w.params()
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    c27, inter = sim.work_counters(params)
    g = sim.grid(params)
    sim.close()
    m = [int(np.floor(2.0 / np.float64(np.float32(0.1))))] * 3
    inv = [np.float32(m[0] / 2.0)] * 3
    assert inter == int(counts.sum())
    assert c27 == int(round(oracle.c27(rec["pos"], m, inv)))


def test_force_work_bounds(cflib):
    """cf_force_work: every particle is staged by its own item, every interacting pair is
    among the candidates tested, and no item tests more than 32 particles' worth."""
    w = inputs.Workload("fw", n=20000, num_types=4, radius=0.1, steps=1, seed=23)
    sim, pos, types, table, radio = make_world(w)
    params = w.params()
    staged, tested = sim.force_work(params)
    before = sim.get_state()
    sim.simulate(params, 1)
    counts = sim.getNeighborCounts()
    c27, _ = sim.work_counters(params)
    sim.close()
    assert staged >= w.n and int(counts.sum()) <= tested <= 32 * staged
    assert tested >= int(counts.sum()) + w.n  # every particle also tests itself (masked out)
    print(f"\nfilter tests per particle {tested / w.n:.1f}, staged per particle {staged / w.n:.2f}")
    assert before[0].shape[0] == w.n


@pytest.mark.parametrize("wl", ["plain_n100k_t8", "blobs_n1m_t12"])
def test_full_size_sampled_rows(cflib, wl):
    """Full-size configurations: a strided sample of particles against the oracle, which
    computes those rows over all N particles; plus the symmetric-count property."""
    w = inputs.WORKLOADS[wl]
    params = w.params()
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    sim, *_ = make_world(w, pos, types, table, radio)
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    sim.close()
    assert int(counts.sum()) % 2 == 0  # uniform radius: the interaction relation is symmetric
    stride = max(1, w.n // 400)
    rows = (0, w.n, stride)
    po, vo, ao, co = oracle.step_f32(pos, np.zeros_like(pos), types, np.zeros(w.n, np.int32), table, radio, params,
                                     rows=rows)
    sel = np.arange(0, w.n, stride)
    assert np.array_equal(counts[sel], co[sel])
    scale = np.abs(ao[sel]).max()
    err = np.abs(rec["acc"][sel] - ao[sel]).max() / scale
    assert err < 1e-5, err
