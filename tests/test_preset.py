"""Preset files (CellFlowWidget::loadPreset / savePreset, CellFlowWidget.cpp:1070-1259).

CPU tests check the library's JSON reader against Python's json module (on
synthetic presets with every key, on the reference's own preset files when
the reference tree is present, and on malformed text).  GPU tests apply
presets to a world: the force table must equal, bit for bit, the golden
tables that the reference's own transform produced from the four preset
files (tests/golden/force_tables_presets.npz), and save -> load must round-trip.
"""

import json
import os
from pathlib import Path

import numpy as np
import pytest

import oracle

from cellflow_gb300._lib import PRESET_BITS, CellFlowError
from cellflow_gb300.world import SimulationParams, parse_preset

GOLDEN = Path(__file__).resolve().parent / "golden"
REFERENCE = oracle.reference_root() / "cuda-native"
PRESETS = ["settings.json", "eater.json", "littlecells.json", "pulser.json"]

F32 = np.float32

FULL = {
    "PARTICLE_COUNT": 1234, "numParticleTypes": 3, "radius": 285.5, "delta_t": 0.34, "friction": 0.5,
    "repulsion": 50.0, "attraction": 0.93, "k": 21.02, "balance": 0.3, "forceMultiplier": 1.38,
    "forceRange": 0.28, "forceBias": -0.16, "forceOffset": -0.32, "ratio": 0.5, "lfoA": 0.25, "lfoS": 5.15,
    "canvasWidth": 8000, "canvasHeight": 6000, "canvasDepth": 4000, "spawnRegionSize": 2000,
    "pointSize": 10, "depthFadeStart": 0.1, "enableDOF": True, "invertPan": False, "effectType": 2,
    "metaball": 0, "label": "café \"quoted\"\n",
    "particleColors": [{"r": 0.9, "g": 0.18, "b": 0.18}, {"b": 0.5, "g": 0.25, "r": 0.125}],
    "radioByType": [0.1, -0.25, 0.75],
    "rawForceTable": [0.5, -0.25, 1e-3, -1e-7, 0.0, -0.0, 0.75, 1.0, -1.0],
}


def check_against_json(pre, obj):
    """Every interpreted key as float32 / int; uninterpreted keys preserved as JSON text."""
    fmap = {"radius": "radius", "delta_t": "delta_t", "friction": "friction", "repulsion": "repulsion",
            "attraction": "attraction", "k": "k", "balance": "balance", "forceMultiplier": "force_multiplier",
            "canvasWidth": "canvas_width", "canvasHeight": "canvas_height", "canvasDepth": "canvas_depth"}
    for key, field in fmap.items():
        if key in obj:
            assert getattr(pre.params, field) == F32(obj[key]), key
    for key, field in (("forceRange", "force_range"), ("forceBias", "force_bias"), ("forceOffset", "force_offset"),
                       ("ratio", "ratio"), ("lfoA", "lfo_a"), ("lfoS", "lfo_s"), ("spawnRegionSize", "spawn_region")):
        if key in obj:
            assert getattr(pre, field) == F32(obj[key]), key
    if "numParticleTypes" in obj:
        assert pre.params.num_particle_types == obj["numParticleTypes"]
        assert pre.present & PRESET_BITS["numParticleTypes"]
    if "PARTICLE_COUNT" in obj:
        assert pre.particle_count == obj["PARTICLE_COUNT"]
    if "radioByType" in obj:
        assert pre.n_radio == len(obj["radioByType"])
        assert np.array_equal(np.array(pre.radio[:pre.n_radio], F32), np.array(obj["radioByType"], F32))
    if "rawForceTable" in obj:
        assert pre.n_raw == len(obj["rawForceTable"])
        got = np.array(pre.raw[:pre.n_raw], F32)
        want = np.array(obj["rawForceTable"], F32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))  # signed zeros too
    if "particleColors" in obj:
        assert pre.n_colors == len(obj["particleColors"])
        for c, d in zip(pre.colors[:pre.n_colors], obj["particleColors"]):
            assert (c.r, c.g, c.b) == (F32(d["r"]), F32(d["g"]), F32(d["b"]))
    known = {"PARTICLE_COUNT", "numParticleTypes", "radioByType", "rawForceTable", "particleColors",
             "forceRange", "forceBias", "forceOffset", "ratio", "lfoA", "lfoS", "spawnRegionSize", *fmap}
    extra = {k: v for k, v in obj.items() if k not in known}
    got_extra = json.loads("{" + pre.extra.decode() + "}") if pre.extra else {}
    assert got_extra == extra


def test_parse_every_key(cflib):
    pre = parse_preset(json.dumps(FULL, indent=4))
    check_against_json(pre, FULL)
    for bit in ("PARTICLE_COUNT", "radius", "canvas", "forceTransform", "lfo", "radioByType", "rawForceTable",
                "particleColors", "spawnRegionSize"):
        assert pre.present & PRESET_BITS[bit], bit


def test_absent_keys_take_the_reference_defaults(cflib):
    pre = parse_preset('{"radius": 3}')
    assert pre.present == PRESET_BITS["radius"]
    assert pre.params.friction == F32(0.51) and pre.params.force_multiplier == F32(2.33)
    assert (pre.force_range, pre.force_bias, pre.force_offset, pre.lfo_s) == (F32(0.28), F32(-0.2), F32(1.0),
                                                                             F32(0.1))
    assert pre.n_raw == 0 and pre.n_radio == 0 and pre.extra == b""


def test_numbers_and_escapes(cflib):
    obj = {"radius": -0.0, "k": 1.5e-3, "delta_t": 12e2, "friction": 0.30000001192092896, "note": "€é\t/",
           "nested": {"a": [1, {"b": None}], "c": True}}
    text = json.dumps(obj).replace("/", "\\/")  # an escaped solidus reads as "/"
    pre = parse_preset(text)
    check_against_json(pre, obj)
    assert np.float32(pre.params.radius).view(np.uint32) == np.float32(-0.0).view(np.uint32)


@pytest.mark.parametrize("bad", ['{"radius": }', '[1, 2]', '{"a": 1,}', '{"a": "unterminated}', '{"a": "\\x"}',
                                 '{"a": 01}', '{"a": 1} trailing', '{"a": tru}', "", '{"a": 1e}',
                                 "[" * 100 + "]" * 100, '{"a": "\\ud800"}'])
def test_malformed_text_is_rejected(cflib, bad):
    with pytest.raises(CellFlowError, match="preset JSON"):
        parse_preset(bad)


@pytest.mark.skipif(not REFERENCE.exists(), reason="the reference tree is not present")
@pytest.mark.parametrize("name", PRESETS)
def test_reference_preset_files(cflib, name):
    text = (REFERENCE / name).read_bytes()
    check_against_json(parse_preset(text), json.loads(text))


# ---- on a world (GPU) ------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("key", ["settings", "eater", "littlecells", "pulser"])
def test_apply_gives_the_reference_force_table(cflib, key):
    from cellflow_gb300.world import ParticleSimulation

    g = np.load(GOLDEN / "force_tables_presets.npz")
    raw, args, table = g[f"{key}_raw"], g[f"{key}_args"], g[f"{key}_table"]
    T = int(round(np.sqrt(raw.size)))
    text = json.dumps({"numParticleTypes": T, "PARTICLE_COUNT": 777, "forceRange": float(args[0]),
                       "forceBias": float(args[1]), "forceOffset": float(args[2]),
                       "rawForceTable": [float(x) for x in raw], "radius": 42.0, "radioByType": [0.5] * T})
    sim = ParticleSimulation(100, 4, 8000.0, 8000.0, 8000.0)
    params, pre = sim.loadPreset(text, seed=3)
    assert sim.getParticleCount() == 777 and sim.getNumParticleTypes() == T
    assert np.array_equal(np.asarray(sim.getRawForceTableValues(), F32).ravel(), raw.astype(F32))
    assert np.array_equal(np.asarray(sim.getForceTable(), F32).ravel().view(np.uint32),
                          table.astype(F32).view(np.uint32))
    assert np.array_equal(np.asarray(sim.getRadioByType(), F32), np.full(T, 0.5, F32))
    assert params.radius == 42.0 and params.num_particle_types == T
    sim.close()


@pytest.mark.gpu
def test_save_load_round_trip(cflib):
    from cellflow_gb300.world import ParticleSimulation

    a = ParticleSimulation(500, 3, 8000.0, 8000.0, 8000.0)
    params, pre = a.loadPreset(json.dumps(FULL))
    text = a.savePreset(params, pre)
    obj = json.loads(text)
    assert obj["PARTICLE_COUNT"] == FULL["PARTICLE_COUNT"] and obj["numParticleTypes"] == 3
    for k in ("pointSize", "depthFadeStart", "enableDOF", "invertPan", "effectType", "metaball", "label"):
        assert obj[k] == FULL[k], k
    b = ParticleSimulation(10, 2, 8000.0, 8000.0, 8000.0)
    params_b, _ = b.loadPreset(text)
    assert params_b == params
    for getter in ("getRawForceTableValues", "getForceTable", "getRadioByType"):
        assert np.array_equal(np.asarray(getattr(a, getter)()), np.asarray(getattr(b, getter)())), getter
    a.close()
    b.close()


@pytest.mark.gpu
def test_partial_tables_keep_the_rest(cflib):
    """loadPreset copies only min(len, T*T) raw entries and min(len, T) radius values (:1160-1175)."""
    from cellflow_gb300.world import ParticleSimulation

    sim = ParticleSimulation(100, 3, 8000.0, 8000.0, 8000.0)
    raw0 = np.asarray(sim.getRawForceTableValues(), F32).ravel().copy()
    radio0 = np.asarray(sim.getRadioByType(), F32).copy()
    sim.loadPreset(json.dumps({"rawForceTable": [0.5, 0.25], "radioByType": [0.125]}))
    raw1 = np.asarray(sim.getRawForceTableValues(), F32).ravel()
    radio1 = np.asarray(sim.getRadioByType(), F32)
    assert raw1[0] == F32(0.5) and raw1[1] == F32(0.25) and np.array_equal(raw1[2:], raw0[2:])
    assert radio1[0] == F32(0.125) and np.array_equal(radio1[1:], radio0[1:])
    sim.close()
