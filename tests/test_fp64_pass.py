"""The torch FP64 training pass (tests/fp64_pass.py) equals the C oracle's FP64
mode on the same weights and records (CPU, float64)."""
import numpy as np
import torch

import fp64_pass as F


def test_fp64_pass_matches_oracle(oracle):
    from vknrc_gb300 import synthetic as S

    rng = S.rng_for(77)
    w = rng.normal(0.0, np.sqrt(2.0 / 64.0), F.P)
    rec = S.train_records(rng, 700, target="field", sigma=1.0)
    enc = oracle.encode(rec[:, 6:])
    g_ref, loss_ref = oracle.train_grad_w64(w, enc, rec[:, :3], nthreads=4)
    x = torch.from_numpy(enc.view(np.float16).astype(np.float64))
    t = torch.from_numpy(rec[:, :3].astype(np.float64))
    g, loss = F.grad_and_loss(torch.from_numpy(w), x, t)
    np.testing.assert_allclose(g.numpy(), g_ref, rtol=1e-9, atol=1e-12 * np.abs(g_ref).max())
    assert abs(float(loss) - loss_ref) <= 1e-10 * loss_ref


def test_fp64_adam_first_step_moves_by_lr():
    w = np.random.default_rng(1).normal(0, 0.2, F.P)
    opt = F.Fp64Adam(w, 1e-3, 0.9, 0.99, 1e-8, "cpu")
    x = torch.rand(300, 64, dtype=torch.float64)
    t = torch.rand(300, 3, dtype=torch.float64)
    opt.step(x, t)
    # the first bias-corrected step is lr * g / (|g| + eps): lr wherever |g| >> eps
    g, _ = F.grad_and_loss(torch.from_numpy(w), x, t)
    big = (g / 300).abs() > 1e-4
    moved = (opt.w - torch.from_numpy(w)).abs()
    assert big.sum() > F.P // 2
    assert torch.allclose(moved[big], torch.full_like(moved[big], 1e-3), rtol=1e-3)
