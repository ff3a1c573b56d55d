"""Generates the golden vectors in tests/golden/ from the reference's own code.

Run where the reference tree is present (it reads its sources through
oracle/build_ref.sh and its preset JSONs):

    python tests/golden/make_golden.py [reference_root]

Inputs are regenerated from seeds by cellflow_gb300.inputs (integer Philox,
identical on every machine), so only outputs, tables and preset parameters
are stored.  Outputs come from the reference kernel bodies
(cuda-native/src/ParticleSimulation.cu:69-166 and :188-277) and its table
transform (:521-531) compiled on the host by oracle/ref_host_shim.cu; the
step runs with Jacobi meaning (every particle sees the start-of-step state).
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from cellflow_gb300 import inputs  # noqa: E402
from cellflow_gb300.world import SimulationParams  # noqa: E402

PRESETS = ["settings.json", "eater.json", "littlecells.json", "pulser.json"]


def sha256(path: Path) -> str:
    return hashlib.sha256(path.read_bytes()).hexdigest()


def preset_params(obj: dict, canvas: float) -> SimulationParams:
    T = int(obj["numParticleTypes"])
    return SimulationParams(
        radius=float(obj["radius"]), delta_t=float(obj["delta_t"]), friction=float(obj["friction"]),
        repulsion=float(obj["repulsion"]), attraction=float(obj["attraction"]), k=float(obj["k"]),
        balance=float(obj["balance"]), canvas_width=canvas, canvas_height=canvas, canvas_depth=canvas,
        num_particle_types=T, ratio_with_lfo=float(obj.get("ratio", 0.0)),
        force_multiplier=float(obj["forceMultiplier"]), max_expected_neighbors=400,
    )


def ref_rollout(pos, types, table, radio, params, steps):
    rec = oracle.to_records(pos, np.zeros_like(pos), types)
    counts = np.zeros(len(pos), np.int32)
    snaps = []
    for _ in range(steps):
        rec, counts = oracle.ref_step(rec, table, radio, counts, params)
        snaps.append((rec.copy(), counts.copy()))
    return snaps


def main(ref_root: str | None = None) -> None:
    import os

    ref_root = ref_root or str(oracle.reference_root())
    os.environ["CELLFLOW_REFERENCE"] = ref_root
    if not oracle.build_ref(gpu=False):
        raise SystemExit("reference pieces not found")
    src = Path(ref_root) / "cuda-native/src/ParticleSimulation.cu"
    manifest = {"reference_sha256": {"cuda-native/src/ParticleSimulation.cu": sha256(src)}, "fixtures": {}}

    # 1. the small plain configuration: 1 and 5 Jacobi steps
    w = inputs.PLAIN_SMALL
    pos, types, table = w.positions(), w.types(), w.table()
    radio = np.zeros(w.num_types, np.float32)
    snaps = ref_rollout(pos, types, table, radio, w.params(), 5)
    np.savez_compressed(
        HERE / "step_plain_n4096_t6.npz", table=table,
        pos1=snaps[0][0]["pos"], vel1=snaps[0][0]["vel"], acc1=snaps[0][0]["acc"], cnt1=snaps[0][1].astype(np.int16),
        pos5=snaps[4][0]["pos"], vel5=snaps[4][0]["vel"], cnt5=snaps[4][1].astype(np.int16),
    )
    manifest["fixtures"]["step_plain_n4096_t6.npz"] = {
        "workload": w.name, "n": w.n, "types": w.num_types, "radius": w.radius, "seed": w.seed,
        "steps": [1, 5], "source": "reference step kernel body, host build, Jacobi",
    }

    # 2. force tables of the four presets (ParticleSimulation.cu:521-531)
    tables = {}
    for name in PRESETS:
        obj = json.loads((Path(ref_root) / "cuda-native" / name).read_text())
        T = int(obj["numParticleTypes"])
        raw = np.asarray(obj["rawForceTable"][: T * T], np.float32)
        key = name.replace(".json", "")
        tables[f"{key}_raw"] = raw
        tables[f"{key}_args"] = np.asarray([obj["forceRange"], obj["forceBias"], obj["forceOffset"]], np.float32)
        tables[f"{key}_table"] = oracle.ref_force_table(raw, T, float(np.float32(obj["forceRange"])),
                                                        float(np.float32(obj["forceBias"])),
                                                        float(np.float32(obj["forceOffset"])))
    np.savez_compressed(HERE / "force_tables_presets.npz", **tables)
    manifest["fixtures"]["force_tables_presets.npz"] = {"presets": PRESETS, "source": "reference updateForceTable"}

    # 3. app-scale step with the settings.json preset: canvas 8000, spawn cube 2000
    obj = json.loads((Path(ref_root) / "cuda-native/settings.json").read_text())
    params = preset_params(obj, 8000.0)
    T, n, seed = params.num_particle_types, 2048, 0x5EED0010
    u = inputs.unit24(inputs._words(3 * n, 1, seed)).reshape(n, 3)
    ppos = (np.float32(3000.0) + u * np.float32(2000.0)).astype(np.float32)
    ptypes = inputs.uniform_types(n, T, seed)
    ptable = tables["settings_table"]
    pradio = np.asarray(obj["radioByType"][:T], np.float32)
    psnaps = ref_rollout(ppos, ptypes, ptable, pradio, params, 1)
    np.savez_compressed(HERE / "step_preset_settings_n2048.npz", pos=ppos, types=ptypes, table=ptable, radio=pradio,
                        params=np.asarray([getattr(params, f) for f in params.__dataclass_fields__], np.float64),
                        pos1=psnaps[0][0]["pos"], vel1=psnaps[0][0]["vel"], acc1=psnaps[0][0]["acc"],
                        cnt1=psnaps[0][1].astype(np.int16))
    manifest["fixtures"]["step_preset_settings_n2048.npz"] = {
        "preset": "settings.json", "n": n, "spawn": "3000 + 2000*u", "seed": seed,
        "params_order": list(params.__dataclass_fields__), "source": "reference step kernel body",
    }

    # 4. proximity edges (reference kernel body, i order)
    prox = {}
    for tag, (dist, mc, T2) in {"a": (0.05, 5, 6), "b": (0.2, 3, 2), "c": (0.12, 16, 1)}.items():
        n2 = 4096
        pos2 = inputs.uniform_positions(n2, 0x5EED0020)
        types2 = inputs.uniform_types(n2, T2, 0x5EED0020)
        cols = np.full((T2, 3), 0.5, np.float32)
        verts = oracle.ref_proximity_vertices(oracle.to_records(pos2, np.zeros_like(pos2), types2), dist, mc, cols, T2)
        key = {pos2[i].tobytes(): i for i in range(n2)}
        edges = np.asarray([(key[verts[2 * k, :3].tobytes()], key[verts[2 * k + 1, :3].tobytes()])
                            for k in range(len(verts) // 2)], np.int32).reshape(-1, 2)
        prox[f"{tag}_edges"] = edges
        prox[f"{tag}_args"] = np.asarray([dist, mc, T2], np.float64)
    np.savez_compressed(HERE / "proximity_n4096.npz", **prox)
    manifest["fixtures"]["proximity_n4096.npz"] = {"n": 4096, "seed": 0x5EED0020,
                                                    "source": "reference proximity kernel body, i order"}
    mesh_golden(manifest)
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    print("golden vectors written to", HERE)


# 5. triangle mesh (reference kernel body, host wrapper's distance, i order)
MESH_CASES = {"a": (0.15, 5, 3), "b": (0.25, 32, 2), "c": (0.31, 40, 4)}  # b and c reach 64 triangles


def mesh_golden(manifest: dict) -> None:
    mesh = {}
    n = 1024
    for tag, (dist, mc, T) in MESH_CASES.items():
        pos = inputs.uniform_positions(n, 0x5EED0030)
        types = inputs.uniform_types(n, T, 0x5EED0030)
        cols = (np.arange(3 * T, dtype=np.float32).reshape(T, 3) + 1.0) / np.float32(3 * T)
        verts = oracle.ref_triangle_mesh(oracle.to_records(pos, np.zeros_like(pos), types), dist, mc, cols, T)
        mesh[f"{tag}_vertices"] = verts
        mesh[f"{tag}_args"] = np.asarray([dist, mc, T], np.float64)
    np.savez_compressed(HERE / "mesh_n1024.npz", **mesh)
    manifest["fixtures"].pop("mesh_n2048.npz", None)
    manifest["fixtures"]["mesh_n1024.npz"] = {"n": n, "seed": 0x5EED0030, "colors": "(arange(3T) + 1) / 3T",
                                              "source": "reference triangle-mesh kernel body, i order"}


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[-1] == "--mesh-only":
        # add the mesh fixture to an existing manifest without rewriting the others
        import os

        os.environ["CELLFLOW_REFERENCE"] = sys.argv[1] if len(sys.argv) > 2 else str(oracle.reference_root())
        if not oracle.build_ref(gpu=False):
            raise SystemExit("reference pieces not found")
        m = json.loads((HERE / "manifest.json").read_text())
        mesh_golden(m)
        (HERE / "manifest.json").write_text(json.dumps(m, indent=1) + "\n")
    else:
        main(*sys.argv[1:])
