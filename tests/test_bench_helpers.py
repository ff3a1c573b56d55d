"""bench.py helpers that need no GPU: the figures it reads from the committed ncu summary
(traffic, FMA-pipe and issue figures per workload), the host CPU record of the CPU baseline,
and the defaults of its command line (100k workload, the contract's K and W)."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


@pytest.mark.parametrize("workload", ["plain_n100k_t8", "blobs_n1m_t12"])
def test_profile_figures_present(workload):
    t = bench.profiled_traffic(workload)
    assert t is not None and t["bytes_per_launch"] > 1_000_000
    assert "dram__bytes_read.sum" in t["source"]
    for key in ("fma_pipe_inst_pct", "issue_active_pct"):
        v = bench.profile_figure(key, workload)
        assert v is not None and 0.0 < v <= 100.0


def test_profile_figure_absent_workload():
    assert bench.profile_figure("traffic_bytes_per_launch", "no_such_workload") is None
    assert bench.profiled_traffic("no_such_workload") is None


def test_host_cpu_model_is_recorded():
    m = bench.host_cpu_model()
    assert isinstance(m, str) and m


def test_default_command_line(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse_args()
    # no workload named: the 100k headline with the other configurations nested in its record
    assert a.gpus == 1 and a.impl == "gb300" and a.workload is None and not a.no_nested
    assert bench.HEADLINE == "plain_n100k_t8"
    assert [name for name, _, _ in bench.NESTED] == ["blobs_n1m_t12", "batched_256w", "rollout_n16k_k64"]
    assert a.warmup >= 3 and a.steps >= 1 and all(w >= 3 for _, _, w in bench.NESTED)
    assert a.profile_steps is None and a.variant is None
