"""FP8 (E4M3) precision form of the cache query: per-layer absmax scales, an
E4M3 copy of use_weights refreshed after every training call and rescaled
once per 16 steps, kind::f8f6f4 MMAs with fp32 accumulation.

Checks: the E4M3 weights and scales the GPU keeps equal the oracle's
quantization of the same rendering weights bit for bit (fresh cache: scales
from the weight bounds; after training: the GPU's scales, with the weights
re-quantized every call); the FP8 query against the oracle's FP8 forward on
the same weights and scales (an activation that lands on an E4M3 rounding
boundary may round the other way after a different fp32 summation order,
which moves an output by up to a few E4M3 steps, so the bound is on the median
and the 99th percentile); and the FP8 query's error against the FP64 oracle,
reported beside the fp16 query's."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def _f32(x):
    return np.float32(x)


def test_fp8_quantization_matches_oracle(cuda, oracle):
    from vknrc_gb300 import Cache, synthetic as S

    with Cache(seed=90, fp8_inference=1, learning_rate=1e-3) as c:
        w8, sc = c.get_fp8()
        ref_w8, st = oracle.fp8_quantize(c.get_weights(0))  # fresh: no activations seen yet
        assert np.array_equal(w8, ref_w8)
        assert np.array_equal(sc["scale_w"], st[0:6]) and np.array_equal(sc["scale_x"], st[6:12])
        assert np.array_equal(sc["c"], st[12:18]) and sc["inv_sx0"] == st[18]
        # 20 training steps: the scales are recomputed when the step count reaches 16;
        # the E4M3 weights follow every step
        for k in range(20):
            c.train(dev(S.train_records(S.rng_for(91, k), 4096, target="field", sigma=1.0)), count(4096),
                    write_use=True)
        w8, sc = c.get_fp8()
        use = c.get_weights(0)
        assert not np.array_equal(sc["scale_x"], st[6:12])  # activations were observed
        f16 = use.view(np.float16).astype(np.float32)
        for l in range(6):
            lo, hi = l * 4096, (l * 4096 + 4096 if l < 5 else 20672)
            assert np.array_equal(w8[lo:hi], oracle.e4m3(f16[lo:hi] * sc["inv_w"][l])), l
            if l < 5:
                assert sc["c"][l] == _f32(_f32(sc["scale_w"][l] * sc["scale_x"][l]) / sc["scale_x"][l + 1])
        assert sc["c"][5] == _f32(sc["scale_w"][5] * sc["scale_x"][5])
        assert c.error() == 0


def test_fp8_query_vs_oracle_and_fp64(cuda, oracle):
    import torch

    from vknrc_gb300 import Cache, synthetic as S

    n = 32768
    rec = S.inputs(S.rng_for(92), n)
    with Cache(seed=93, fp8_inference=1, learning_rate=1e-3) as c:
        for k in range(32):
            c.train(dev(S.train_records(S.rng_for(94, k), 4096, target="field", sigma=1.0)), count(4096),
                    write_use=True)
        out8 = torch.full((n + 5, 3), -1.0, dtype=torch.float32, device="cuda")
        out16 = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        c.infer_fp8(dev(np.concatenate([rec, np.zeros((5, 14), np.float32)])), count(n), out8)
        c.infer(dev(rec), count(n), out16)
        got8, got16 = host(out8), host(out16)
        w8, sc = c.get_fp8()
        use = c.get_weights(0)
        assert c.error() == 0
    assert np.all(got8[n:] == -1.0)
    got8 = got8[:n]
    ref8 = np.maximum(oracle.forward_fp8(w8, sc["c"], sc["inv_sx0"], oracle.encode_f32(rec), nthreads=8), 0)
    d = np.abs(got8 - ref8)
    scale = float(np.abs(ref8).mean())
    assert np.median(d) <= 1e-3 * max(scale, 1e-3), (np.median(d), scale)
    assert np.quantile(d, 0.99) <= 0.1 * max(scale, 1e-3), (np.quantile(d, 0.99), scale)
    f64 = np.maximum(oracle.forward_f64(use, oracle.encode(rec), nthreads=8), 0)
    e8 = float(np.mean(np.abs(got8 - f64)) / np.mean(np.abs(f64)))
    e16 = float(np.mean(np.abs(got16 - f64)) / np.mean(np.abs(f64)))
    print(f"mean relative query error vs FP64: fp16 {e16:.3e}, fp8 {e8:.3e}")
    assert e16 < e8 < 0.2


def test_fp8_needs_the_form_enabled(cuda):
    import torch

    from vknrc_gb300 import Cache, NRCError

    with Cache(seed=95) as c:
        out = torch.empty((8, 3), dtype=torch.float32, device="cuda")
        with pytest.raises(NRCError):
            c.infer_fp8(torch.zeros((8, 14), dtype=torch.float32, device="cuda"), count(8), out)
        with pytest.raises(NRCError):
            c.get_fp8()
