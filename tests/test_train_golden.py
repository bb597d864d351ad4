"""The oracle's training arithmetic against the reference's own shader code.

tests/golden/train_golden.npz holds the outputs of nrc_train_prepare.comp,
nrc_optimize.comp and NN_nv.glsl's NNLoadDA3_RelativeL2LuminanceLoss compiled
from the reference tree as C++ (oracle/ref/ref_train.cpp, made by
tests/golden/make_golden.py) on the single-step training case's records (16,384
records, lognormal(0, 1.5) targets, He weights) and on edge cases.

Tolerances. GLSL lets a compiler contract a*b + c into one fused multiply-add;
the reference's code compiled here keeps every product rounded, while the oracle
and the GPU fuse the moment, EMA and luminance multiply-adds. The two differ by
at most about one rounding of the larger term, so each fp32 field is compared
within 8 ulp of the magnitude of the terms that form it (train_tolerance), fp16
outputs within one fp16 ulp, and everything that involves no multiply-add
(the prepare pass, the NaN/Inf scrub, which gradient rows overflow) exactly.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "train_golden.npz")


@pytest.fixture(scope="module")
def tg():
    return dict(np.load(GOLDEN))


def hparams(tg):
    lr, b1, b2, eps, a, s = (float(x) for x in tg["hparams"])
    return O.HParams(lr, b1, b2, eps, a, s, int(tg["batch_cap"]))


def state(t):
    return O.OptState(int(t[0]), float(t[1]), float(t[2]), float(t[3]), float(t[4]))


def f16_words(rows):
    """(n, 2) row words -> (n, 3) float32 of the three fp16 gradient values."""
    h = np.stack([rows[:, 0] & 0xFFFF, rows[:, 0] >> 16, rows[:, 1] & 0xFFFF], -1).astype(np.uint16)
    return h.view(np.float16).astype(np.float32)


def f16_ulp_diff(a, b):
    """Distance in fp16 steps between two arrays of fp16 bit patterns (sign-magnitude order)."""
    def key(x):
        x = x.astype(np.int64)
        return np.where(x & 0x8000, -(x & 0x7FFF), x)
    return np.abs(key(a) - key(b))


def check_loss_rows(got, want):
    """Rows within one fp16 step per value, with the same values infinite."""
    gh, wh = f16_words(got), f16_words(want)
    assert np.array_equal(np.isinf(gh), np.isinf(wh)), "the rows that overflow to inf differ"
    assert np.array_equal(np.signbit(gh[np.isinf(gh)]), np.signbit(wh[np.isinf(wh)]))
    fin = np.isfinite(wh)
    bits_g = np.stack([got[:, 0] & 0xFFFF, got[:, 0] >> 16, got[:, 1] & 0xFFFF], -1)
    bits_w = np.stack([want[:, 0] & 0xFFFF, want[:, 0] >> 16, want[:, 1] & 0xFFFF], -1)
    d = f16_ulp_diff(bits_g[fin], bits_w[fin])
    assert d.max(initial=0) <= 1, f"loss rows differ by {d.max()} fp16 steps"
    assert (got[:, 1] >> 16 == 0).all()  # the padding half is zero
    return float((d == 0).mean())


def train_tolerance(entries_in, grad, count, st, hp, use_ema=False):
    """Per-field bound (m, v, w, ema) on |oracle - reference|: 8 ulp of each
    field's term magnitudes, from a float64 evaluation of the update."""
    e = entries_in.astype(np.float64)
    g = grad.astype(np.float64) / count / hp.loss_scale
    g[~np.isfinite(g)] = 0.0
    b1, b2 = float(np.float32(hp.beta1)), float(np.float32(hp.beta2))
    m = b1 * e[:, 0] + (1 - b1) * g
    v = b2 * e[:, 1] + (1 - b2) * g * g
    sm = np.abs(b1 * e[:, 0]) + np.abs((1 - b1) * g)
    sv = b2 * e[:, 1] + (1 - b2) * g * g
    hm, hv = m / (1 - st.beta1_t), v / (1 - st.beta2_t)
    den = np.sqrt(hv) + hp.epsilon
    upd = hp.learning_rate * np.abs(hm) / den
    # w carries the rounding of m and v through the update
    sw = np.abs(e[:, 2]) + upd + hp.learning_rate * (sm / (1 - st.beta1_t)) / den
    eta, eta1 = 1 - st.alpha_t, 1 - st.alpha_t_1
    ea, eb = (1 - hp.ema_alpha) / eta, hp.ema_alpha * eta1
    se = np.abs(ea) * (np.abs(e[:, 2]) + upd) + np.abs(eb * e[:, 3]) + np.abs(ea) * sw
    return 8 * 2.0 ** -23 * np.stack([sm, sv, sw, se], -1) + 1e-45


def check_entries(got, want, tol):
    d = np.abs(got.astype(np.float64) - want.astype(np.float64))
    bad = d > tol
    assert not bad.any(), f"{bad.sum()} entry fields beyond tolerance; worst field {np.argmax((d / tol).max(0))}"


def test_prepare_bit_exact(tg):
    hp = hparams(tg)
    for c, s_in, s_out, n in zip(tg["prep_counts"], tg["prep_state_in"], tg["prep_state_out"], tg["prep_n"]):
        st = state(s_in)
        got = O.lib().oracle_prepare(int(c), ctypes.byref(hp), ctypes.byref(st))
        assert got == int(n)
        assert (st.t, np.float32(st.beta1_t), np.float32(st.beta2_t), np.float32(st.alpha_t),
                np.float32(st.alpha_t_1)) == (int(s_out[0]), *np.float32(s_out[1:]))


def test_prepare_dispatch_size(tg):
    # the indirect dispatch covers the clamped count in work groups of 128
    assert np.array_equal(tg["prep_groups"], (tg["prep_n"].astype(np.int64) + 127) // 128)


def test_loss_rows_single_step(tg):
    n = 16384
    got = O.loss_rows(tg["loss_pred"][:n], tg["loss_target"][:n], 1.0)
    same = check_loss_rows(got, tg["loss_rows"][:n])
    assert same > 0.999
    # the lognormal(0, 1.5) tail overflows fp16 in the reference
    assert np.isinf(f16_words(tg["loss_rows"][:n])).any()


def test_loss_rows_edges(tg):
    check_loss_rows(O.loss_rows(tg["loss_pred"][16384:], tg["loss_target"][16384:], 1.0), tg["loss_rows"][16384:])


def _optimizer(tg, entries_in, st):
    opt = O.Optimizer(np.zeros(O.P, np.float32), hparams(tg))
    opt.entries[:] = entries_in
    opt.state = state(st)
    return opt


def test_optimize_first_step(tg):
    e_in = np.zeros((O.P, 4), np.float32)
    e_in[:, 2] = tg["he_w32"]
    e_in[:, 3] = tg["he_w32"]
    opt = _optimizer(tg, e_in, tg["he_state"])
    w16, use16 = opt.adam(tg["he_grad"], int(tg["he_count"]), write_use=True, use_ema=False)
    tol = train_tolerance(e_in, tg["he_grad"], int(tg["he_count"]), opt.state, opt.hp)
    check_entries(opt.entries, tg["he_entries_out"], tol)
    assert f16_ulp_diff(w16, tg["he_w16"]).max() <= 1
    assert f16_ulp_diff(use16, tg["he_use16"]).max() <= 1
    # the gradient entries the overflowed rows poisoned are scrubbed: no update to m
    bad = ~np.isfinite(tg["he_grad"])
    assert bad.any() and (tg["he_entries_out"][bad, 0] == 0).all()
    assert (opt.entries[bad, 0] == 0).all()


def test_optimize_mid_run_with_nonfinite_gradients(tg):
    opt = _optimizer(tg, tg["mid_entries_in"], tg["mid_state"])
    w16, use16 = opt.adam(tg["mid_grad"], int(tg["mid_count"]), write_use=True, use_ema=True)
    tol = train_tolerance(tg["mid_entries_in"], tg["mid_grad"], int(tg["mid_count"]), opt.state, opt.hp)
    check_entries(opt.entries, tg["mid_entries_out"], tol)
    assert f16_ulp_diff(w16, tg["mid_w16"]).max() <= 1
    assert f16_ulp_diff(use16, tg["mid_use16"]).max() <= 1
    bad = ~np.isfinite(tg["mid_grad"])
    # scrubbed parameters: m decays, v decays (gradient taken as 0)
    b1 = np.float32(tg["hparams"][1])
    np.testing.assert_array_equal(opt.entries[bad, 0], (b1 * tg["mid_entries_in"][bad, 0]).astype(np.float32))


def test_optimize_count_zero_writes_nothing(tg):
    opt = _optimizer(tg, tg["mid_entries_in"], tg["mid_state"])
    before = opt.entries.copy()
    opt.adam(tg["mid_grad"], 0, write_use=True)
    np.testing.assert_array_equal(opt.entries, before)


@pytest.mark.skipif(O.ref_lib() is None or not hasattr(O.ref_lib(), "ref_optimize"),
                    reason="reference library not built here")
def test_golden_reproduces_from_reference(tg):
    """The committed vectors are what the reference's compiled shaders give now."""
    st = state(tg["mid_state"])
    e = tg["mid_entries_in"].copy()
    w16, use16 = np.zeros(O.P, np.uint16), np.zeros(O.P, np.uint16)
    O.ref_optimize(e, tg["mid_grad"], int(tg["mid_count"]), st, True, w16, use16)
    np.testing.assert_array_equal(e, tg["mid_entries_out"])
    np.testing.assert_array_equal(use16, tg["mid_use16"])
    np.testing.assert_array_equal(O.ref_loss_rows(tg["loss_pred"], tg["loss_target"]), tg["loss_rows"])
