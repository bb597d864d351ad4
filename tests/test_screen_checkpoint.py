"""Screen pass (shader/src/screen.frag:10-31) and cache checkpoints.

CPU: the oracle's screen pass against an independent float64 restatement of
the shader's formulas, and its fixed points (black, the white point).
GPU: nrc_screen against the oracle (accumulation image bit for bit; the
tone-mapped values within the error of pow, UNORM8 within one step), and a
checkpoint that restores a cache exactly: training continued from a loaded
checkpoint equals training continued in the saved cache, bit for bit."""
import numpy as np
import pytest

from gpu_util import count, dev, host


def _hejl64(x):
    va = 1.425 * x + 0.05
    return (x * va + 0.004) / (x * (va + 0.55) + 0.0491) - 0.0821


def _colors(seed, h, w):
    rng = np.random.default_rng(seed)
    c = np.zeros((h, w, 4), np.float32)
    c[..., :3] = rng.lognormal(-0.5, 1.5, (h, w, 3)).astype(np.float32)
    c[0, 0, :3] = 0.0  # black
    c[0, 1, :3] = 3.2  # the white point
    return c


def test_oracle_screen_matches_float64_formula(oracle):
    c = _colors(1, 17, 23)
    o8, of = oracle.screen(c)
    ref = np.maximum(_hejl64(c[..., :3].astype(np.float64)) / _hejl64(3.2), 0.0) ** (1 / 2.2)
    assert np.allclose(of[..., :3], ref, rtol=2e-6, atol=2e-6)
    assert np.all(of[..., 3] == 1.0) and np.all(o8[..., 3] == 255)
    assert np.all(o8[0, 0, :3] == 0) and np.all(of[0, 0, :3] == 0.0)  # tone curve < 0 at black -> 0
    assert np.all(o8[0, 1, :3] == 255) and np.allclose(of[0, 1, :3], 1.0, atol=1e-6)
    assert np.all(np.abs(o8[..., :3].astype(int) - np.round(np.clip(ref, 0, 1) * 255)) <= 1)


def test_oracle_screen_accumulates_running_average(oracle):
    frames = [_colors(s, 5, 7) for s in range(4)]
    acc = np.zeros((5, 7, 4), np.float32)
    for k, f in enumerate(frames):
        oracle.screen(f, acc, k)
    mean = np.mean([f[..., :3].astype(np.float64) for f in frames], axis=0)
    assert np.allclose(acc[..., :3], mean, rtol=1e-5)
    assert np.all(acc[..., 3] == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("acc_count", [None, 0, 1, 7])
def test_gpu_screen_vs_oracle(cuda, oracle, acc_count):
    import torch

    from vknrc_gb300 import nrc

    h, w = 181, 333
    c = _colors(5, h, w)
    acc0 = _colors(6, h, w)
    acc0[..., 3] = 0.0
    acc_h = acc0.copy() if acc_count is not None else None
    o8_ref, of_ref = oracle.screen(c, acc_h, acc_count or 0)
    acc_d = dev(acc0) if acc_count is not None else None
    o8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    of = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    nrc.screen(dev(c), acc_d, acc_count or 0, o8, of)
    if acc_count is not None:
        assert np.array_equal(host(acc_d), acc_h)
    got_f, got_8 = host(of), host(o8)
    assert np.allclose(got_f, of_ref, rtol=4e-7, atol=1e-7)  # powf: a few ulp
    d = np.abs(got_8.astype(int) - o8_ref.astype(int))
    assert d.max() <= 1 and np.mean(d > 0) < 1e-3


@pytest.mark.gpu
def test_checkpoint_restores_training_exactly(cuda):
    from vknrc_gb300 import Cache, NRCError, synthetic as S

    recs = [dev(S.train_records(S.rng_for(70, k), 4096, target="field", sigma=0.5)) for k in range(5)]
    with Cache(seed=71, learning_rate=1e-3, beta2=0.99) as a, Cache(seed=72) as b:
        for k in range(3):
            a.train(recs[k], count(4096), write_use=True)
        blob = a.save_checkpoint()
        for k in range(3, 5):
            a.train(recs[k], count(4096), write_use=True)
        b.load_checkpoint(blob)  # b had other weights and the reference hyper-parameters
        for k in range(3, 5):
            b.train(recs[k], count(4096), write_use=True)
        sa, ea = a.get_optimizer()
        sb, eb = b.get_optimizer()
        assert sa == sb and sa[0] == 5
        assert np.array_equal(ea, eb)
        assert np.array_equal(a.get_weights(0), b.get_weights(0))
        assert np.array_equal(a.get_weights(1), b.get_weights(1))
        bad = bytearray(blob)
        bad[1000] ^= 1
        for wrong in (bytes(bad), blob[:-1], b"x" * len(blob)):
            with pytest.raises(NRCError) as e:
                b.load_checkpoint(wrong)
            assert e.value.status == 9
        assert np.array_equal(b.get_optimizer()[1], eb)  # a rejected blob changes nothing
