"""The GPU's prepare, optimizer and loss-gradient arithmetic against the
reference's own shader code (tests/golden/train_golden.npz, made by compiling
nrc_train_prepare.comp, nrc_optimize.comp and NN_nv.glsl's
NNLoadDA3_RelativeL2LuminanceLoss from the reference tree; see
tests/test_train_golden.py for the tolerances and their reason), and the fused
trainer tied to those passes: one fused step equals nrc_gradient followed by
nrc_optimize bit for bit."""
import numpy as np
import pytest

import test_train_golden as TG
from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def ref_cache(tg, **extra):
    from vknrc_gb300 import Cache

    lr, b1, b2, eps, a, s = (float(x) for x in tg["hparams"])
    return Cache(seed=1, learning_rate=lr, beta1=b1, beta2=b2, epsilon=eps, ema_alpha=a, loss_scale=s,
                 train_batch_size=int(tg["batch_cap"]), **extra)


def state_tuple(t):
    return (int(t[0]), *(float(np.float32(x)) for x in t[1:]))


def test_optimize_first_step_vs_reference(cuda):
    tg = dict(np.load(TG.GOLDEN))
    e_in = np.zeros((20672, 4), np.float32)
    e_in[:, 2] = tg["he_w32"]
    e_in[:, 3] = tg["he_w32"]
    with ref_cache(tg) as c:
        c.set_weights(tg["he_w32"].astype(np.float16).view(np.uint16))
        c.set_optimizer((0, 1.0, 1.0, 1.0, 0.0), e_in)
        cnt = count(int(tg["he_count"]))
        c.optimize(dev(tg["he_grad"]), cnt, write_use=True)
        st, ent = c.get_optimizer()
        w16, use16 = c.get_weights(1), c.get_weights(0)
        assert c.error() == 0
    assert st == state_tuple(tg["he_state"])
    st_o = TG.state(tg["he_state"])
    hp = TG.hparams(tg)
    TG.check_entries(ent, tg["he_entries_out"], TG.train_tolerance(e_in, tg["he_grad"], int(tg["he_count"]), st_o, hp))
    assert TG.f16_ulp_diff(w16, tg["he_w16"]).max() <= 1
    assert TG.f16_ulp_diff(use16, tg["he_use16"]).max() <= 1
    bad = ~np.isfinite(tg["he_grad"])
    assert bad.any() and (ent[bad, 0] == 0).all() and (ent[bad, 2] == e_in[bad, 2]).all()


def test_optimize_mid_run_vs_reference(cuda):
    tg = dict(np.load(TG.GOLDEN))
    with ref_cache(tg, use_ema_weights=1) as c:
        c.set_optimizer(state_tuple(tg["mid_state_in"]), tg["mid_entries_in"])
        c.optimize(dev(tg["mid_grad"]), count(int(tg["mid_count"])), write_use=True)
        st, ent = c.get_optimizer()
        w16, use16 = c.get_weights(1), c.get_weights(0)
    assert st == state_tuple(tg["mid_state"])
    tol = TG.train_tolerance(tg["mid_entries_in"], tg["mid_grad"], int(tg["mid_count"]), TG.state(tg["mid_state"]),
                             TG.hparams(tg))
    TG.check_entries(ent, tg["mid_entries_out"], tol)
    assert TG.f16_ulp_diff(w16, tg["mid_w16"]).max() <= 1
    assert TG.f16_ulp_diff(use16, tg["mid_use16"]).max() <= 1


@pytest.mark.parametrize("k", range(10))
def test_prepare_vs_reference(cuda, k):
    """Every golden count from both golden states: clamped count written back,
    state advanced exactly as the compiled nrc_train_prepare.comp does, and for
    a zero count nothing of the parameters written."""
    tg = dict(np.load(TG.GOLDEN))
    assert len(tg["prep_counts"]) == 20
    for j in (k, k + 10):
        with ref_cache(tg) as c:
            c.set_optimizer(state_tuple(tg["prep_state_in"][j]), None)
            _, ent0 = c.get_optimizer()
            w0 = c.get_weights(1)
            cnt = count(int(tg["prep_counts"][j:j + 1].view(np.int32)[0]))  # the count's bits as int32
            c.optimize(dev(np.zeros(20672, np.float32)), cnt, write_use=True)
            st, ent = c.get_optimizer()
            assert int(host(cnt)[0]) & 0xFFFFFFFF == int(tg["prep_n"][j])
            assert st == state_tuple(tg["prep_state_out"][j])
            if tg["prep_n"][j] == 0:
                np.testing.assert_array_equal(ent, ent0)
                np.testing.assert_array_equal(c.get_weights(1), w0)


@pytest.mark.parametrize("part", ["records", "edges"])
def test_loss_rows_vs_reference(cuda, part):
    import torch
    from vknrc_gb300 import nrc

    tg = dict(np.load(TG.GOLDEN))
    sl = slice(0, 16384) if part == "records" else slice(16384, None)
    p, t = tg["loss_pred"][sl], tg["loss_target"][sl]
    rows = torch.zeros((p.shape[0], 2), dtype=torch.int32, device="cuda")
    nrc.loss_gradient(dev(p), dev(t), count(p.shape[0]), rows)
    got = host(rows).view(np.uint32)
    TG.check_loss_rows(got, tg["loss_rows"][sl])
    if part == "records":
        assert np.isinf(TG.f16_words(got)).any()  # the lognormal(0, 1.5) tail overflows as in the reference


def test_loss_rows_bf16_vs_oracle(cuda, oracle):
    import torch
    from vknrc_gb300 import nrc

    tg = dict(np.load(TG.GOLDEN))
    p, t = tg["loss_pred"], tg["loss_target"]
    rows = torch.zeros((p.shape[0], 2), dtype=torch.int32, device="cuda")
    nrc.loss_gradient(dev(p), dev(t), count(p.shape[0]), rows, precision=1)
    np.testing.assert_array_equal(host(rows).view(np.uint32), oracle.loss_rows(p, t, 1.0, fmt=1))


def test_fused_step_equals_gradient_then_optimize(cuda):
    """nrc_train (one fused launch) gives exactly what nrc_gradient followed by
    nrc_optimize gives on the same records (16,384 records with lognormal(0, 1.5)
    targets, whose fp16 overflow the optimizer scrubs)."""
    import torch
    from vknrc_gb300 import Cache, synthetic as S

    recs = dev(S.train_records(S.rng_for(31, 1), 16384, sigma=1.5))
    kw = dict(seed=11, learning_rate=1e-3, beta2=0.99)
    with Cache(**kw) as a, Cache(**kw) as b:
        a.train(recs, count(16384), write_use=True)
        g = torch.zeros(20672, dtype=torch.float32, device="cuda")
        b.gradient(recs, count(16384), g)
        b.optimize(g, count(16384), write_use=True)
        sa, ea = a.get_optimizer()
        sb, eb = b.get_optimizer()
        assert sa == sb
        np.testing.assert_array_equal(ea, eb)
        np.testing.assert_array_equal(a.get_weights(1), b.get_weights(1))
        np.testing.assert_array_equal(a.get_weights(0), b.get_weights(0))
        assert a.error() == 0 and b.error() == 0
