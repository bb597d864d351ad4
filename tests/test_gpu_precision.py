"""Precision forms: the BF16 path (bf16 weights, features, activations and
gradients; fp32 master weights and Adam moments) against the oracle run in the
same format, and both precision forms against the FP64 oracle.

Tolerances: the query as the fp16 query test (the GPU accumulates each layer in
fp32 in MMA order, the oracle in input order; a 16-bit rounding boundary can
fall between them, so single outputs may differ by a few bf16 steps);
gradients by the median / p99 of the error relative to the sum of absolute
terms; the loss after 1000 online steps within 5% of the FP64 oracle's (bf16
carries 8 mantissa bits against fp16's 11; the fp16 path is held to 2%)."""
import os

import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu

BF16 = 1


def test_bf16_query_vs_oracle_and_fp64(cuda, oracle):
    import torch

    from vknrc_gb300 import Cache, synthetic as S

    n = 65536
    rec = S.inputs(S.rng_for(80), n)
    errs = {}
    for fmt in (0, BF16):
        with Cache(seed=81, precision=fmt) as c:
            w = c.get_weights(0)
            out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            c.infer(dev(rec), count(n), out)
            got = host(out)
        enc = oracle.encode(rec, fmt=fmt)
        ref = np.maximum(oracle.forward_f32(w, enc, nthreads=8, fmt=fmt), 0)
        f64 = np.maximum(oracle.forward_f64(w, enc, nthreads=8, fmt=fmt), 0)
        scale = max(1.0, float(np.abs(ref).max()))
        tol = 2e-2 if fmt else 1e-2
        assert np.max(np.abs(got - ref)) <= tol * scale, (fmt, np.max(np.abs(got - ref)))
        errs[fmt] = float(np.mean(np.abs(got - f64)) / np.mean(np.abs(f64)))
    print(f"mean relative query error vs FP64: fp16 {errs[0]:.3e}, bf16 {errs[BF16]:.3e}")
    assert errs[BF16] < 3e-2 and errs[0] < 5e-3


def test_bf16_gradient_vs_oracle(cuda, oracle):
    from vknrc_gb300 import Cache, synthetic as S

    n = 16384
    recs = S.train_records(S.rng_for(82), n, target="field", sigma=0.5)
    with Cache(seed=83, precision=BF16) as c:
        w = c.get_weights(1)
        g = cuda.zeros(20672, dtype=cuda.float32, device="cuda")
        c.gradient(dev(recs), count(n), g)
        got = host(g).astype(np.float64)
    enc = oracle.encode(recs[:, 6:], fmt=BF16)
    ref, absum, _ = oracle.train_grad(w, enc, recs[:, :3], mode=0, want_abs=True, nthreads=8, fmt=BF16)
    rel = np.abs(got - ref) / (absum + 1e-30)
    assert np.median(rel) < 1e-4, np.median(rel)
    assert np.quantile(rel, 0.99) < 5e-3, np.quantile(rel, 0.99)
    f64, _, _ = oracle.train_grad(w, enc, recs[:, :3], mode=1, want_abs=True, nthreads=8, fmt=BF16)
    print(f"bf16 gradient: median rel err vs same-format oracle {np.median(rel):.2e}, vs FP64 "
          f"{np.median(np.abs(got - f64) / (absum + 1e-30)):.2e}")


def test_bf16_training_step_and_storage(cuda, oracle):
    """One BF16 step: Adam from the fp32 master weights writes bf16 weight
    vectors that equal the oracle's Adam on the GPU's own gradient."""
    from vknrc_gb300 import Cache, synthetic as S

    n = 4096
    recs = S.train_records(S.rng_for(84), n, target="field", sigma=0.5)
    with Cache(seed=85, precision=BF16, learning_rate=1e-3) as a, Cache(seed=85, precision=BF16,
                                                                       learning_rate=1e-3) as b:
        _, ent0 = a.get_optimizer()
        u = ent0[:, 2].copy().view(np.uint32).astype(np.uint64)
        bf = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)  # round to nearest even
        assert np.array_equal(a.get_weights(1), bf)  # the He weights stored as bf16
        g = cuda.zeros(20672, dtype=cuda.float32, device="cuda")
        b.gradient(dev(recs), count(n), g)
        a.train(dev(recs), count(n), write_use=True)
        hp = oracle.HParams(1e-3, 0.9, 0.999, 1e-8, 0.99, 1.0, 16384)
        opt = oracle.Optimizer(ent0[:, 2].copy(), hp)
        opt.entries[:] = ent0
        opt.prepare(n)
        w16, use16 = opt.adam(host(g), n, write_use=True, fmt=BF16)
        st, ent = a.get_optimizer()
        assert st[0] == 1
        assert np.array_equal(ent, opt.entries)
        assert np.array_equal(a.get_weights(1), w16) and np.array_equal(a.get_weights(0), use16)


def test_bf16_loss_curve_vs_fp64_oracle(cuda, oracle):
    from vknrc_gb300 import Cache, synthetic as S

    steps, records, lr, b1, b2, eps = 1000, 1024, 1e-3, 0.9, 0.99, 1e-8
    threads = os.cpu_count() or 1
    gpu_loss, ref_loss = [], []
    with Cache(seed=2024, learning_rate=lr, beta1=b1, beta2=b2, epsilon=eps, track_loss=1, precision=BF16) as c:
        _, entries = c.get_optimizer()
        w = entries[:, 2].astype(np.float64)
        m = np.zeros_like(w)
        v = np.zeros_like(w)
        b1t = b2t = 1.0
        n = count(records)
        c.get_loss()
        for step in range(steps):
            rec = S.train_records(S.rng_for(555, step), records, target="field", sigma=1.0)
            c.train(dev(rec), n)
            s, k = c.get_loss()
            gpu_loss.append(s / k)
            g, loss = oracle.train_grad_w64(w, oracle.encode(rec[:, 6:]), rec[:, :3], nthreads=threads)
            ref_loss.append(loss / records)
            g = g / records
            m = b1 * m + (1 - b1) * g
            v = b2 * v + (1 - b2) * g * g
            b1t *= b1
            b2t *= b2
            w = w - lr * (m / (1 - b1t)) / (np.sqrt(v / (1 - b2t)) + eps)
        assert c.error() == 0
    gpu_loss, ref_loss = np.asarray(gpu_loss), np.asarray(ref_loss)
    assert np.all(np.isfinite(gpu_loss))
    assert gpu_loss[-100:].mean() < 0.5 * gpu_loss[:10].mean()
    rel = abs(gpu_loss[-100:].mean() - ref_loss[-100:].mean()) / ref_loss[-100:].mean()
    print(f"bf16 loss: last-100 mean {gpu_loss[-100:].mean():.4g} (fp64 {ref_loss[-100:].mean():.4g}); "
          f"rel diff {rel:.4f}")
    assert rel <= 0.05


def test_mixed_precision_batches_and_checkpoint_format(cuda):
    from vknrc_gb300 import Cache, NRCError, nrc, synthetic as S

    recs = [dev(S.train_records(S.rng_for(86, b), 2048, target="field", sigma=0.5)) for b in range(4)]
    mk = lambda p: Cache(seed=87, precision=p, train_batch_size=2048)
    a16, abf, s16, sbf = mk(0), mk(BF16), mk(0), mk(BF16)
    try:
        jobs = lambda cs: [nrc.train_job(c, recs, [count(2048) for _ in range(4)]) for c in cs]
        nrc.train_many(jobs([a16, abf]), ctas=[20, 20])  # two launches, one per format
        nrc.train_many(jobs([s16]), ctas=[20])
        nrc.train_many(jobs([sbf]), ctas=[20])
        assert np.array_equal(a16.get_optimizer()[1], s16.get_optimizer()[1])
        assert np.array_equal(abf.get_optimizer()[1], sbf.get_optimizer()[1])
        assert not np.array_equal(a16.get_weights(0), abf.get_weights(0))
        blob = abf.save_checkpoint()
        with pytest.raises(NRCError):
            s16.load_checkpoint(blob)  # bf16 vectors into an fp16 cache
        sbf.load_checkpoint(blob)
        assert np.array_equal(sbf.get_weights(0), abf.get_weights(0))
        with pytest.raises(NRCError):
            abf.encode(dev(S.inputs(S.rng_for(88), 16)), count(16), cuda.empty((16, 64), dtype=cuda.int16,
                                                                               device="cuda"))
    finally:
        for c in (a16, abf, s16, sbf):
            c.close()
