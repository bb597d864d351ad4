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
    inst = b.load_profile_figure("inst_executed_per_launch")
    raw = b.load_profile_figure("traffic_bytes_per_launch")
    assert raw is not None and inst is not None
    # DRAM bytes of one 1080p launch: at least the records read once
    assert b.Q * 20 <= raw < b.Q * (b.EVAL_BYTES + b.OUT_BYTES) * 1.1
    assert inst > 0 and b.load_profile_figure("no_such_figure") is None


def test_traffic_reported_only_for_the_profiled_sources():
    b = _bench()
    traffic, src = b.load_traffic()
    with open(os.path.join(ROOT, "profiles", "infer_kernel_1080p.md")) as fh:
        recorded = [ln.split(":", 1)[1].strip() for ln in fh if ln.startswith("kernel_source_sha256_16:")]
    if recorded and recorded[0] == b.kernel_source_hash():
        assert traffic == b.load_profile_figure("traffic_bytes_per_launch") and "ncu" in src
    else:
        assert traffic is None and "changed" in src


def test_issue_bound_arithmetic():
    b = _bench()
    clocks = {"sm_mhz": 2000.0}
    r = b.issue_bound(4.0 * 152 * 2000e6 * 1e-4, 152, clocks, 2e-4)  # 100 us of issue at 4/cycle/SM
    assert r["bound_us"] == pytest.approx(100.0)
    assert r["frac"] == pytest.approx(0.5)
    assert b.issue_bound(None, 152, clocks, 1e-4) is None
    assert b.issue_bound(1e6, 152, {}, 1e-4) is None
