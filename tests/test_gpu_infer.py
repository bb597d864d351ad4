"""nrc_infer / nrc_infer_encoded on the GPU against the reference's Evaluate()
(golden vectors), the oracle's fp32-accumulating forward and the FP64 oracle."""
import numpy as np
import pytest

from gpu_util import count, dev, f16, host

pytestmark = pytest.mark.gpu

# Tolerance of the fused path against the oracle's fp16-activation / fp32-sum
# forward: the tensor core sums in a different order, which can flip the fp16
# rounding of an activation; outputs stay within 1e-2 absolute at unit scale
# and 5e-4 on average.
TOL_MAX = 1e-2
TOL_MEAN = 5e-4


def run_infer(c, rec, n=None, cap=None, weight_set=0, encoded=False, sentinel=np.nan):
    import torch

    cap = rec.shape[0] if cap is None else cap
    n = cap if n is None else n
    out = torch.full((max(cap, 1), 3), float(sentinel), dtype=torch.float32, device="cuda")
    if encoded:
        c.infer_encoded(dev(rec), count(n), out, capacity=cap, weight_set=weight_set)
    else:
        c.infer(dev(rec), count(n), out, capacity=cap, weight_set=weight_set)
    return host(out)


@pytest.mark.parametrize("key", ["uniform", "he"])
def test_infer_encoded_vs_reference_evaluate(cuda, oracle, golden, key):
    """Same weights, same pre-encoded inputs as test/main.cpp's Evaluate()."""
    from vknrc_gb300 import Cache

    ev = golden["evaluate"]
    w, x, y = ev[f"w_{key}"], ev[f"x_{key}"], f16(ev[f"y_{key}"])
    with Cache() as c:
        c.set_weights(w)
        got = run_infer(c, x.view(np.int16), encoded=True).astype(np.float64)
    o64 = oracle.forward_f64(w, x)
    o32 = oracle.forward_f32(w, x).astype(np.float64)
    scale = max(1e-3, np.abs(o64).max())
    ref_err = np.abs(y - o64)
    gpu_err = np.abs(got - o64)
    print(f"\n[{key}] max|gpu-ref|={np.abs(got - y).max():.3e} gpu-vs-fp64 mean={gpu_err.mean():.3e} "
          f"max={gpu_err.max():.3e}; ref-vs-fp64 mean={ref_err.mean():.3e} max={ref_err.max():.3e}")
    assert np.max(np.abs(got - y)) <= 2 * ref_err.max() + 4e-3 * scale
    assert gpu_err.mean() <= ref_err.mean()
    assert np.abs(got - o32).max() <= TOL_MAX * scale


@pytest.mark.parametrize("n", [1, 2, 3, 127, 128, 129, 511, 1000, 4097, 65536])
def test_infer_records_vs_oracle(cuda, oracle, n):
    from vknrc_gb300 import Cache, synthetic as S

    rec = S.inputs(S.rng_for(11, n), n)
    with Cache(seed=99) as c:
        w = c.get_weights(0)
        got = run_infer(c, rec)
    ref = np.maximum(oracle.forward_f32(w, oracle.encode(rec)), 0)
    scale = max(1.0, np.abs(ref).max())
    err = np.abs(got - ref)
    assert err.max() <= TOL_MAX * scale, err.max()
    assert err.mean() <= TOL_MEAN * scale, err.mean()
    assert np.all(got >= 0)


@pytest.mark.parametrize("n,cap", [(0, 300), (300, 200), (200, 300), (5, 1)])
def test_infer_count_clamped_to_capacity(cuda, oracle, n, cap):
    from vknrc_gb300 import Cache, synthetic as S

    rec = S.inputs(S.rng_for(12), cap)
    with Cache(seed=5) as c:
        w = c.get_weights(0)
        got = run_infer(c, rec, n=n, cap=cap, sentinel=-7.0)
    m = min(n, cap)
    ref = np.maximum(oracle.forward_f32(w, oracle.encode(rec[:m])), 0)
    assert np.abs(got[:m] - ref).max(initial=0) <= TOL_MAX * max(1.0, np.abs(ref).max(initial=0))
    assert np.all(got[m:] == -7.0)


def test_infer_full_frame_properties(cuda, oracle):
    """1920x1080 queries: sampled rows vs the oracle, run-to-run identical."""
    from vknrc_gb300 import Cache, synthetic as S

    n = 1920 * 1080
    rec = S.inputs(S.rng_for(13), n)
    with Cache(seed=21) as c:
        w = c.get_weights(0)
        a = run_infer(c, rec)
        b = run_infer(c, rec)
    assert np.array_equal(a, b)
    idx = np.random.default_rng(0).choice(n, 20000, replace=False)
    idx.sort()
    ref = np.maximum(oracle.forward_f32(w, oracle.encode(rec[idx])), 0)
    assert np.abs(a[idx] - ref).max() <= TOL_MAX * max(1.0, np.abs(ref).max())


def test_weight_sets_select_vectors(cuda):
    from vknrc_gb300 import Cache, synthetic as S

    rec = S.inputs(S.rng_for(14), 256)
    with Cache(seed=1) as c:
        w = c.get_weights(0)
        w2 = (w.view(np.float16) * np.float16(0.5)).view(np.uint16)
        c.set_weights(w2)
        use = run_infer(c, rec, weight_set=0)
        trn = run_infer(c, rec, weight_set=1)
        assert np.array_equal(use, trn)
    assert c.h is None
