"""The oracle is pinned: it reproduces the golden vectors (made by the reference's own
kernel bodies and table transform) bit for bit, and agrees with the reference pieces
on fresh random cases when they are built here.  CPU only."""

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from cellflow_gb300 import inputs
from cellflow_gb300.world import SimulationParams

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLDEN / name)


def test_golden_plain_one_and_five_steps():
    g = load("step_plain_n4096_t6.npz")
    w = inputs.PLAIN_SMALL
    pos, types = w.positions(), w.types()
    assert np.array_equal(g["table"], w.table())
    radio = np.zeros(w.num_types, np.float32)
    p, v, c = pos, np.zeros_like(pos), np.zeros(w.n, np.int32)
    for step in range(1, 6):
        p, v, a, c = oracle.step_f32(p, v, types, c, g["table"], radio, w.params())
        if step == 1:
            assert np.array_equal(p, g["pos1"]) and np.array_equal(v, g["vel1"]) and np.array_equal(a, g["acc1"])
            assert np.array_equal(c, g["cnt1"])
    assert np.array_equal(p, g["pos5"]) and np.array_equal(v, g["vel5"]) and np.array_equal(c, g["cnt5"])


def test_golden_preset_step():
    g = load("step_preset_settings_n2048.npz")
    fields = json.loads((GOLDEN / "manifest.json").read_text())["fixtures"]["step_preset_settings_n2048.npz"]
    params = SimulationParams(**{k: (int(v) if k in ("num_particle_types", "max_expected_neighbors") else float(v))
                                 for k, v in zip(fields["params_order"], g["params"])})
    p, v, a, c = oracle.step_f32(g["pos"], np.zeros_like(g["pos"]), g["types"], np.zeros(len(g["pos"]), np.int32),
                                 g["table"], g["radio"], params)
    assert np.array_equal(c, g["cnt1"]) and c.mean() > 5
    assert np.array_equal(p, g["pos1"]) and np.array_equal(v, g["vel1"]) and np.array_equal(a, g["acc1"])


def test_golden_force_tables():
    g = load("force_tables_presets.npz")
    for key in ("settings", "eater", "littlecells", "pulser"):
        rng, bias, off = (float(x) for x in g[f"{key}_args"])
        assert np.array_equal(oracle.force_table(g[f"{key}_raw"], rng, bias, off), g[f"{key}_table"]), key


def test_golden_proximity():
    g = load("proximity_n4096.npz")
    pos = inputs.uniform_positions(4096, 0x5EED0020)
    for tag in ("a", "b", "c"):
        dist, mc, T = g[f"{tag}_args"]
        types = inputs.uniform_types(4096, int(T), 0x5EED0020)
        edges = oracle.proximity_edges(pos, types, float(dist), int(mc))
        assert np.array_equal(edges, g[f"{tag}_edges"]), tag


def mesh_case(g, tag, n=1024, seed=0x5EED0030):
    dist, mc, T = g[f"{tag}_args"]
    T = int(T)
    pos = inputs.uniform_positions(n, seed)
    types = inputs.uniform_types(n, T, seed)
    cols = (np.arange(3 * T, dtype=np.float32).reshape(T, 3) + 1.0) / np.float32(3 * T)
    return pos, types, float(dist), int(mc), cols, T


def test_golden_triangle_mesh():
    """The restated mesh reproduces the reference kernel body's vertices bit for bit, including the
    64-triangle cap (case b) and max_conn above 32 (case c)."""
    g = load("mesh_n1024.npz")
    for tag in ("a", "b", "c"):
        pos, types, dist, mc, cols, T = mesh_case(g, tag)
        tris, verts = oracle.triangle_mesh(pos, types, dist, mc, cols, T)
        assert np.array_equal(verts.view(np.uint32), g[f"{tag}_vertices"].view(np.uint32)), tag
        assert np.all(tris[:, 0] < tris[:, 1]) and np.all(tris[:, 1] < tris[:, 2])
    per = np.bincount(oracle.triangle_mesh(*mesh_case(g, "b"))[0][:, 0])
    assert per.max() == 64


def test_fp64_oracle_close_to_fp32():
    w = inputs.PLAIN_SMALL
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    z = np.zeros(w.n, np.int32)
    p32, v32, a32, c32 = oracle.step_f32(pos, np.zeros_like(pos), types, z, table, radio, w.params())
    p64, v64, a64, c64, mag = oracle.step_f64(pos, np.zeros_like(pos), types, z, table, radio, w.params())
    assert np.array_equal(c32, c64)
    err = (np.abs(a32 - a64).max(axis=1) / np.maximum(mag, 1e-30)).max()
    assert err < 2e-5  # the float displacement itself carries ~1e-6 relative rounding


def test_rotate_and_lfo():
    v = np.arange(5, dtype=np.float32)
    assert np.array_equal(oracle.rotate(v), np.array([4, 0, 1, 2, 3], np.float32))
    assert oracle.lfo(0.25, 0.0, 1.0, 2.0) == np.float32(0.25)


def test_cell_list_is_a_stable_sort():
    pos = inputs.uniform_positions(5000, 3)
    m = [7, 5, 9]
    inv = [np.float32(mm / 2.0) for mm in m]
    cell_of, order, start, end = oracle.cell_list(pos, m, inv)
    assert np.array_equal(order, np.argsort(cell_of, kind="stable"))
    cells = np.arange(np.prod(m))
    pop = np.bincount(cell_of, minlength=len(cells))
    assert np.array_equal(end - start, pop)


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_equals_reference_body(seed):
    rng = np.random.default_rng(seed)
    n, T = 1500, int(rng.integers(1, 10))
    ext = float(rng.choice([2.0, 8000.0, 37.5]))
    pos = (rng.random((n, 3)) * ext).astype(np.float32)
    vel = rng.normal(0, ext * 1e-3, (n, 3)).astype(np.float32)
    types = rng.integers(0, T, n).astype(np.uint32)
    table = rng.normal(0, 0.5, T * T).astype(np.float32)
    radio = rng.uniform(-1, 1, T).astype(np.float32)
    counts = rng.integers(0, 100, n).astype(np.int32)
    params = SimulationParams(radius=ext * float(rng.uniform(0.03, 0.3)), delta_t=0.05, friction=0.6,
                              repulsion=40.0, attraction=2.0, k=20.0, balance=0.5, canvas_width=ext,
                              canvas_height=ext, canvas_depth=ext, num_particle_types=T,
                              ratio_with_lfo=float(rng.uniform(-1, 1)), force_multiplier=1.7,
                              max_expected_neighbors=int(rng.integers(5, 500)))
    p, v, a, c = oracle.step_f32(pos, vel, types, counts, table, radio, params)
    rec, rc = oracle.ref_step(oracle.to_records(pos, vel, types), table, radio, counts, params)
    assert np.array_equal(c, rc)
    assert np.array_equal(p, rec["pos"]) and np.array_equal(v, rec["vel"]) and np.array_equal(a, rec["acc"])
