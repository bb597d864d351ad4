"""The bench's roofline inputs: the per-launch figures it reads from the
committed ncu summary of the query kernel, and the CUDA-core issue bound it
derives from them (CPU only)."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_profile_figures_parse():
    b = _bench()
    traffic = b.load_traffic()
    inst = b.load_profile_figure("inst_executed_per_launch")
    assert traffic is not None and inst is not None
    # DRAM bytes of one 1080p launch: at least the 116 MB of records read once
    assert b.Q * b.EVAL_BYTES <= traffic < b.Q * (b.EVAL_BYTES + b.OUT_BYTES) * 1.1
    assert inst > 0 and b.load_profile_figure("no_such_figure") is None


def test_issue_bound_arithmetic():
    b = _bench()
    clocks = {"sm_mhz": 2000.0}
    r = b.issue_bound(4.0 * 152 * 2000e6 * 1e-4, 152, clocks, 2e-4)  # 100 us of issue at 4/cycle/SM
    assert r["bound_us"] == pytest.approx(100.0)
    assert r["frac"] == pytest.approx(0.5)
    assert b.issue_bound(None, 152, clocks, 1e-4) is None
    assert b.issue_bound(1e6, 152, {}, 1e-4) is None
