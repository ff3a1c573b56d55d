"""The C ABI library loads and exports every function include/*.h declares (no GPU needed)."""

import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> set[str]:
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = header.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(cf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_core_entry_points():
    names = declared_functions()
    for must in ("cf_create", "cf_destroy", "cf_step", "cf_get_particles", "cf_set_particles",
                 "cf_update_force_table", "cf_proximity_edges", "cf_sync", "cf_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(cflib):
    from cellflow_gb300 import _lib

    exported = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True,
                              check=True).stdout
    symbols = {line.split()[-1] for line in exported.splitlines() if line.strip()}
    missing = declared_functions() - symbols
    assert not missing, f"declared but not exported: {sorted(missing)}"
    for name in declared_functions():
        assert hasattr(cflib, name)


def test_bounds_build_exports_the_same_symbols():
    """The bounds-checked library (-DCF_DEBUG_BOUNDS) builds and exports every declared function."""
    from cellflow_gb300 import build

    lib = build.build(bounds=True)
    exported = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True,
                              check=True).stdout
    symbols = {line.split()[-1] for line in exported.splitlines() if line.strip()}
    missing = declared_functions() - symbols
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_binding_covers_header(cflib):
    from cellflow_gb300 import _lib

    assert declared_functions() <= set(_lib.declared_symbols())


def test_host_only_calls_without_gpu(cflib):
    """Entry points that touch no device memory work on a CPU-only host."""
    from cellflow_gb300._lib import StepParams

    p = StepParams()
    cflib.cf_default_params(p)
    assert abs(p.radius - 42.07) < 1e-5 and p.num_particle_types == 6 and p.max_expected_neighbors == 400
    assert cflib.cf_version().startswith(b"cellflow-gb300")
    assert cflib.cf_lfo_ratio(0.5, 0.0, 0.1, 3.0) == pytest.approx(0.5)
    # the normal library reports itself unchecked, with nothing recorded
    import ctypes as C

    checked, found = C.c_int(7), C.c_int(7)
    where = C.create_string_buffer(b"x" * 16)
    assert cflib.cf_debug_bounds(C.byref(checked), C.byref(found), where, 16, None, None) == 0
    assert checked.value == 0 and found.value == 0 and where.value == b""


def test_lfo_matches_oracle(cflib):
    import oracle

    for ratio, a, s, t in [(0.0, 0.2, 0.1, 1.3), (1.0, 0.5, 5.15, 17.0), (-0.3, 1.0, 0.7, 0.25)]:
        assert cflib.cf_lfo_ratio(ratio, a, s, t) == oracle.lfo(ratio, a, s, t)
