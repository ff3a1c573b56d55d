"""Edge cases of the GPU step against the oracle: empty and single-particle worlds,
particles on the box faces and pairs across the periodic boundary at the interaction
threshold, every particle in one cell, rows of 4096 cells (one row per tile of the cell
list), items split over several warps when a world has a single item, and dense blobs
under the lane-paired drain."""

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300.world import ParticleSimulation, SimulationParams
from tests.parity import check_step

pytestmark = pytest.mark.gpu


def params_for(T, radius, W=2.0, H=2.0, D=2.0):
    return SimulationParams(radius=radius, delta_t=0.01, friction=0.51, repulsion=64.83, attraction=3.06, k=29.45,
                            balance=0.79, canvas_width=W, canvas_height=H, canvas_depth=D, num_particle_types=T,
                            ratio_with_lfo=0.0, force_multiplier=2.33, max_expected_neighbors=400)


def step_vs_oracle(pos, types, table, params, vel=None, variant=None, label=""):
    n = len(pos)
    T = params.num_particle_types
    vel = np.zeros_like(pos) if vel is None else vel
    radio = np.zeros(T, np.float32)
    sim = ParticleSimulation(n, T, params.canvas_width, params.canvas_height, params.canvas_depth)
    sim.set_particles(pos, types, vel)
    sim.setForceTable(table)
    sim.setRadioByType(radio)
    if variant is not None:
        sim.set_force_variant(variant)
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    sim.close()
    zeros = np.zeros(n, np.int32)
    po, vo, ao, co = oracle.step_f32(pos, vel, types, zeros, table, radio, params)
    assert np.array_equal(counts, co), f"{label}: counts differ in {np.sum(counts != co)} particles"
    if n:
        _, _, _, _, mag = oracle.step_f64(pos, vel, types, zeros, table, radio, params)
        check_step(rec, po, vo, ao, mag, params.delta_t, params.canvas_width, label)
    return rec, counts


def test_empty_world(cflib):
    params = params_for(3, 0.1)
    sim = ParticleSimulation(0, 3, 2.0, 2.0, 2.0)
    sim.simulate(params, 3)
    sim.sync()
    assert len(sim.getParticleData()) == 0
    assert len(sim.getNeighborCounts()) == 0
    assert len(sim.proximity_edges(0.05, 5)) == 0
    assert len(sim.triangle_mesh(0.05, 6)) == 0
    sim.close()


def test_single_particle_is_pure_friction(cflib):
    params = params_for(2, 0.1)
    pos = np.array([[1.9999, 0.0, 1.0]], np.float32)
    vel = np.array([[0.5, -0.25, 1.0]], np.float32)
    rec, counts = step_vs_oracle(pos, np.array([1], np.uint32), np.ones((2, 2), np.float32), params, vel=vel,
                                 label="single")
    assert counts[0] == 0
    assert np.array_equal(rec["vel"][0], (vel[0] * np.float32(params.friction)).astype(np.float32))


def test_faces_corners_and_threshold_pairs_across_the_boundary(cflib):
    """Particles on x/y/z = 0 and the largest float below W, and pairs straddling each periodic
    face with squared distance + 1e-4 just below, at and above the reference's threshold."""
    W = np.float32(2.0)
    top = np.nextafter(W, np.float32(0))
    params = params_for(3, 0.1)
    rng = np.random.default_rng(3)
    pts = []
    for x in (0.0, top):
        for y in (0.0, top):
            for z in (0.0, top):
                pts.append((x, y, z))
    # pairs across each face: one particle near 0, its partner near W, separated by about the radius
    eff = np.float32(0.1)
    d_star = float(np.sqrt(np.float64(eff) ** 2 - 1e-4))
    for axis in range(3):
        for frac in (0.999999, 1.0, 1.000001, 0.5, 0.25):
            d = d_star * frac
            a = rng.uniform(0.3, 1.7, 3)
            b = a.copy()
            a[axis] = d * 0.4
            b[axis] = 2.0 - d * 0.6
            pts += [tuple(a), tuple(b)]
    pos = np.array(pts, np.float32)
    pos = np.minimum(pos, top)
    types = rng.integers(0, 3, len(pos)).astype(np.uint32)
    table = rng.normal(0, 0.5, (3, 3)).astype(np.float32)
    step_vs_oracle(pos, types, table, params, label="faces")


def test_every_particle_in_one_cell(cflib):
    """3000 particles inside one cell: one row of cells holds them all, so every item stages
    thousands of candidates in many batches."""
    rng = np.random.default_rng(4)
    n, T = 3000, 4
    params = params_for(T, 0.1)
    pos = (np.float32(1.0) + rng.uniform(0, 0.03, (n, 3))).astype(np.float32)
    types = rng.integers(0, T, n).astype(np.uint32)
    table = rng.normal(0, 0.5, (T, T)).astype(np.float32)
    rec, counts = step_vs_oracle(pos, types, table, params, label="one cell")
    assert counts.min() == n - 1
    for variant in (2, 5, 11, 12, 14):
        step_vs_oracle(pos, types, table, params, variant=variant, label=f"one cell, variant {variant}")


def test_rows_of_4096_cells(cflib):
    """A long thin box: 4096 cells along x (the widest row a cell-list tile holds, one row per
    tile), 10 along y and z.  Radius 0.012: with the reference's +1e-4 softening the geometric
    cutoff is sqrt(0.012^2 - 1e-4) = 0.0066 (no pair interacts below radius 0.01).  A strided
    sample of particles is checked against the oracle, each row over all N."""
    rng = np.random.default_rng(5)
    n, T = 120_000, 3
    W, H = 27.5, 0.07
    params = params_for(T, 0.012, W=W, H=H, D=H)
    pos = np.stack([rng.uniform(0, W, n), rng.uniform(0, H, n), rng.uniform(0, H, n)], 1).astype(np.float32)
    pos[:, 0] = np.minimum(pos[:, 0], np.nextafter(np.float32(W), np.float32(0)))
    pos[:, 1:] = np.minimum(pos[:, 1:], np.nextafter(np.float32(H), np.float32(0)))
    types = rng.integers(0, T, n).astype(np.uint32)
    table = rng.normal(0, 0.5, (T, T)).astype(np.float32)
    radio = np.zeros(T, np.float32)
    sim = ParticleSimulation(n, T, W, H, H)
    g = sim.grid(params)
    assert list(g.cells) == [4096, 10, 10], list(g.cells)
    sim.set_particles(pos, types)
    sim.setForceTable(table)
    sim.setRadioByType(radio)
    sim.simulate(params, 1)
    rec = sim.getParticleData()
    counts = sim.getNeighborCounts()
    sim.close()
    stride = 97
    zeros = np.zeros(n, np.int32)
    po, vo, ao, co = oracle.step_f32(pos, np.zeros_like(pos), types, zeros, table, radio, params, rows=(0, n, stride))
    sel = np.arange(0, n, stride)
    assert np.array_equal(counts[sel], co[sel])
    assert counts[sel].sum() > 500
    scale = np.abs(ao[sel]).max()
    assert np.abs(rec["acc"][sel] - ao[sel]).max() <= 1e-5 * scale


@pytest.mark.parametrize("variant", range(15))
def test_single_item_world_under_every_variant(cflib, variant):
    """20 particles in one cell of a 6-cell grid: one item, so with 2 or 4 warps per item some
    warps have few or no candidates."""
    w = inputs.Workload("tiny", n=20, num_types=3, radius=0.3, steps=1, seed=21)
    pos = (np.float32(1.05) + np.float32(0.05) * w.positions()).astype(np.float32)
    rec, counts = step_vs_oracle(pos, w.types(), w.table(), params_for(3, 0.3), variant=variant,
                                 label=f"tiny, variant {variant}")
    assert counts.min() == 19


@pytest.mark.parametrize("variant", [1, 2, 6, 10, 12, 13, 14])
def test_skewed_occupancy_under_lane_pairing(cflib, variant):
    """Dense Gaussian blobs (hundreds of neighbours next to a few): the lanes of an item have
    very uneven hit counts, so the lane-paired drain (stagings 2: variants 2, 6, 10) hands
    large parts of busy lanes' hits to idle ones, and the balanced drain (variants 12-14)
    splits every batch's hits evenly over the lanes; counts stay bit-exact and forces within
    the step tolerance, as with the unpaired staging (variant 1)."""
    n, T = 12000, 5
    pos = inputs.blob_positions(n, 6, 0.04, 0x5EED0031)
    types = inputs.uniform_types(n, T, 0x5EED0031)
    table = inputs.gaussian_table(T, 0.1, 0.6, 0x5EED0031)
    rec, counts = step_vs_oracle(pos, types, table, params_for(T, 0.05), variant=variant,
                                 label=f"blobs, variant {variant}")
    med = np.median(counts)
    assert counts.max() > 2 * med and counts.min() < med / 4


@pytest.mark.parametrize("variant", [1, 2, 12])
def test_lattice_at_the_threshold_overflows_the_band_list(cflib, variant):
    """A cubic lattice whose spacing puts every nearest-neighbour pair within rounding of
    the interaction threshold: each of an item's homes has six such band pairs, far more
    per batch than the drain lists (64), so the batch's band pairs are found again by
    re-walking every home's hits; the neighbour counts stay bit-exact against the oracle,
    pairs across the periodic boundary included."""
    m, T, r = 10, 3, 0.1
    a = np.float32(np.sqrt(np.float32(r) * np.float32(r) - np.float32(1e-4)))
    W = float(np.float32(m) * a)
    k = np.arange(m, dtype=np.float32)
    g = np.stack(np.meshgrid(k, k, k, indexing="ij"), axis=-1).reshape(-1, 3)
    pos = ((g + np.float32(0.5)) * a).astype(np.float32)
    # a jitter of a few ulp of the spacing puts the pairs on both sides of the threshold
    pos = (pos + np.random.default_rng(8).uniform(-3e-7, 3e-7, pos.shape)).astype(np.float32)
    types = (np.arange(len(pos)) % T).astype(np.uint32)
    table = np.random.default_rng(9).normal(0, 0.5, (T, T)).astype(np.float32)
    params = params_for(T, r, W, W, W)
    rec, counts = step_vs_oracle(pos, types, table, params, variant=variant, label=f"lattice, variant {variant}")
    assert 0 < counts.mean() < 6.0
