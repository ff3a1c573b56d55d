"""The bounds-checked library (libcellflow_bounds.so, -DCF_DEBUG_BOUNDS): it gives
the same results as the normal library bit for bit, records no violation on
valid inputs, and an out-of-range item planted through cf_debug_force_bad_item
is recorded (file, line, index, limit) and skipped instead of faulting.  The
checked build pads every device buffer, so the planted index stays inside its
allocation even where a check were missing.  Each library runs in a child
process (tests/bounds_child.py)."""

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

from cellflow_gb300 import _lib, build

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def run_child(bounds: bool) -> dict:
    env = dict(os.environ)
    env.pop("CELLFLOW_LIBRARY", None)
    if bounds:
        env["CELLFLOW_LIBRARY"] = "bounds"
    res = subprocess.run([sys.executable, "-m", "tests.bounds_child"], cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    return json.loads(res.stdout.strip().splitlines()[-1])


def test_bounds_build_matches_and_reports(cflib):
    build.build(bounds=True)
    normal = run_child(False)
    checked = run_child(True)
    assert normal["after_runs"]["checked"] == 0 and checked["after_runs"]["checked"] == 1
    assert normal["results"] == checked["results"]  # bit-identical steps, edges and triangles
    for name, r in checked["results"].items():
        assert r["n_edges"] > 0, name
    assert checked["results"]["blobs"]["n_triangles"] > 0
    assert normal["after_runs"]["found"] == 0 and checked["after_runs"]["found"] == 0
    assert normal["plant_rc"] == _lib.CF_ERR_INVALID  # the normal library has no planting hook
    n = checked["n"]
    planted = checked["planted"]
    assert planted["found"] == 1, planted
    assert planted["where"].startswith("step.cu:"), planted
    assert planted["index"] == n + 2 and planted["limit"] == n, planted
    assert checked["after_planted"]["found"] == 0  # the record was cleared and the next step is clean
