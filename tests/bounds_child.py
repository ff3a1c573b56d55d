"""Child process of tests/test_bounds_build_gpu.py: runs a fixed sequence of
library calls (steps on a uniform and a clustered world, the proximity graph,
the triangle mesh) and prints their results' digests and the bounds report as
one JSON line.  Run once with the normal library and once with
CELLFLOW_LIBRARY=bounds (the bounds-checked build); with the checked build it
also plants an out-of-range item through cf_debug_force_bad_item."""

import ctypes as C
import hashlib
import json

import numpy as np

from cellflow_gb300 import _lib, inputs
from cellflow_gb300.world import ParticleSimulation, SimulationParams


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def report(lib) -> dict:
    checked, found = C.c_int(), C.c_int()
    where = C.create_string_buffer(64)
    index, limit = C.c_longlong(), C.c_longlong()
    _lib.check(lib.cf_debug_bounds(C.byref(checked), C.byref(found), where, 64, C.byref(index), C.byref(limit)),
               "cf_debug_bounds")
    return {"checked": checked.value, "found": found.value, "where": where.value.decode(), "index": index.value,
            "limit": limit.value}


def params_for(T: int, radius: float) -> SimulationParams:
    return SimulationParams(radius=radius, delta_t=0.01, friction=0.51, repulsion=64.83, attraction=3.06, k=29.45,
                            balance=0.79, canvas_width=2.0, canvas_height=2.0, canvas_depth=2.0, num_particle_types=T,
                            ratio_with_lfo=0.0, force_multiplier=2.33, max_expected_neighbors=400)


def main() -> None:
    lib = _lib.load()
    out = {"results": {}}
    cases = {
        "uniform": (20000, 6, 0.1, inputs.Workload("bounds_u", n=20000, num_types=6, radius=0.1, steps=1,
                                                   seed=71).positions()),
        "blobs": (30000, 5, 0.05, inputs.blob_positions(30000, 8, 0.03, 72)),
    }
    for name, (n, T, radius, pos) in cases.items():
        types = inputs.uniform_types(n, T, 73)
        table = inputs.gaussian_table(T, 0.1, 0.6, 74)
        params = params_for(T, radius)
        sim = ParticleSimulation(n, T, 2.0, 2.0, 2.0)
        sim.set_particles(pos, types)
        sim.setForceTable(table)
        sim.setRadioByType(np.zeros(T, np.float32))
        sim.simulate(params, 5)
        state = sim.get_state()
        edges = sim.proximity_edges(0.05, 5)
        tris = sim.triangle_mesh(0.04, 6)
        out["results"][name] = {"state": digest(*state), "edges": digest(edges), "n_edges": len(edges),
                                "triangles": digest(tris), "n_triangles": len(tris)}
        if name == "uniform":
            keep = (sim, params, n)
        else:
            sim.close()
    out["after_runs"] = report(lib)
    sim, params, n = keep
    if out["after_runs"]["checked"]:
        p = params.to_c()
        _lib.check(lib.cf_debug_force_bad_item(sim._h, C.byref(p), n + 2), "cf_debug_force_bad_item")
        out["planted"] = report(lib)
        sim.simulate(params, 1)
        out["after_planted"] = report(lib)
    else:
        p = params.to_c()
        out["plant_rc"] = lib.cf_debug_force_bad_item(sim._h, C.byref(p), n + 2)
    out["n"] = n
    sim.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
