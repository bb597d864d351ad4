"""The CPU oracle pinned against the reference's own code (golden vectors) and
checked for internal consistency (finite differences, optimizer algebra)."""
import numpy as np
import pytest

F16_ULP_1 = 2.0 ** -11  # one fp16 ulp just below 1.0


def test_encode_matches_reference_glsl(oracle, golden):
    """oracle_encode vs shader/src/NRCRecord.glsl:78-95 compiled as C++ (golden)."""
    g = golden["encode"]
    enc = oracle.encode(g["records"])
    ref = g["encoded"]
    exact = np.r_[0:36, 56:64]
    assert np.array_equal(enc[:, exact], ref[:, exact]), "frequency / albedo / constant features must be bit-exact"
    # one-blob features: the restatement evaluates the quartic in fused Horner
    # form; the reference source leaves contraction to the compiler.
    ob = np.r_[36:56]
    a = enc[:, ob].view(np.float16).astype(np.float64)
    b = ref[:, ob].view(np.float16).astype(np.float64)
    assert np.max(np.abs(a - b)) <= F16_ULP_1
    assert np.mean(enc[:, ob] != ref[:, ob]) < 0.03


def test_sph_encode_matches_reference_glsl(oracle, golden):
    g = golden["encode"]
    s = oracle.sph_encode(g["dirs"])
    assert np.max(np.abs(s - g["sph"])) <= 2e-7
    assert s[0, 0] == 0.5 and s[1, 0] == 0.5  # x = y = 0 branch


def test_expf_within_one_ulp(oracle):
    xs = np.linspace(-87.0, 0.0, 5001, dtype=np.float32)
    xs = np.concatenate([xs, -np.random.default_rng(0).random(2000).astype(np.float32)])
    mine = np.array([oracle.expf(float(x)) for x in xs], np.float64)
    exact = np.exp(xs.astype(np.float64))
    ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(mine - exact) / ulp) <= 1.0


def test_forward_matches_reference_evaluate(oracle, golden):
    """fp32-accumulating forward vs test/main.cpp Evaluate() (fp16 accumulation)."""
    ev = golden["evaluate"]
    for key in ("uniform", "he"):
        w, x, y = ev[f"w_{key}"], ev[f"x_{key}"], ev[f"y_{key}"].view(np.float16).astype(np.float64)
        o32 = oracle.forward_f32(w, x).astype(np.float64)
        o64 = oracle.forward_f64(w, x)
        scale = max(1e-3, np.abs(o64).max())
        ref_err = np.abs(y - o64)
        our_err = np.abs(o32 - o64)
        # the restatement agrees with the reference within the reference's own fp16 error
        assert np.max(np.abs(o32 - y)) <= 2 * ref_err.max() + 4e-3 * scale, key
        # and is at least as close to FP64 as the reference is
        assert our_err.mean() <= ref_err.mean() + 1e-6, key


def test_encoded_golden_inputs_consistent(oracle, golden):
    ev = golden["evaluate"]
    enc = oracle.encode(ev["records_he"])
    assert np.mean(enc != ev["x_he"]) < 0.01


def _np_forward_f64(w, x):
    """Plain numpy float64 forward; w float64[P], x float64[n, 64]; returns out, acts."""
    acts = [x]
    a = x
    for l in range(5):
        W = w[l * 4096:(l + 1) * 4096].reshape(64, 64)
        a = np.maximum(a @ W.T, 0.0)
        acts.append(a)
    W5 = w[5 * 4096:5 * 4096 + 192].reshape(3, 64)
    return a @ W5.T, acts


def test_gradient_restatement_finite_difference(oracle):
    """FP64 gradient of the relative-L2 loss (denominator held constant, as in
    NN_nv.glsl:178-196) against central differences of a numpy forward."""
    rng = np.random.default_rng(5)
    n = 24
    w16 = rng.normal(0, np.sqrt(2 / 64), 20672).astype(np.float16)
    x16 = rng.random((n, 64)).astype(np.float16)
    t = rng.lognormal(0, 0.5, (n, 3)).astype(np.float32)
    g, _, loss = oracle.train_grad(w16.view(np.uint16), x16.view(np.uint16), t, mode=1)
    w = w16.astype(np.float64)
    x = x16.astype(np.float64)
    out, _ = _np_forward_f64(w, x)
    lum = np.maximum(out, 0) @ np.array([0.299, 0.587, 0.114])
    den = lum * lum + 0.01

    def L(wv):
        o, _ = _np_forward_f64(wv, x)
        return np.sum((o - t) ** 2 / den[:, None])

    assert abs(L(w) - loss) <= 1e-9 * max(1.0, abs(loss))
    idx = np.concatenate([rng.integers(0, 5 * 4096, 40), 5 * 4096 + rng.integers(0, 192, 10)])
    h = 1e-5
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (L(wp) - L(wm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[i])


def test_gradient_gpu_semantics_close_to_fp64(oracle):
    rng = np.random.default_rng(6)
    n = 256
    w16 = rng.normal(0, np.sqrt(2 / 64), 20672).astype(np.float16).view(np.uint16)
    x16 = rng.random((n, 64)).astype(np.float16).view(np.uint16)
    t = rng.lognormal(0, 0.5, (n, 3)).astype(np.float32)
    g0, a0, _ = oracle.train_grad(w16, x16, t, mode=0, want_abs=True)
    g1, _, _ = oracle.train_grad(w16, x16, t, mode=1)
    rel = np.abs(g0 - g1) / (a0 + 1e-12)
    # fp16 activations and fp16 dA (as the reference stores them) cost about 1e-3 typical
    assert np.median(rel) < 5e-3
    assert np.quantile(rel, 0.99) < 5e-2


def test_optimizer_step_semantics(oracle):
    """nrc_train_prepare.comp + nrc_optimize.comp restated: count clamp, state
    advance only for n > 0, NaN/Inf scrub, bias correction, EMA formula."""
    hp = oracle.HParams(0.002, 0.9, 0.999, 1e-8, 0.99, 1.0, 16384)
    rng = np.random.default_rng(7)
    w0 = rng.normal(0, 0.1, oracle.P).astype(np.float32)
    opt = oracle.Optimizer(w0, hp)
    assert opt.prepare(0) == 0 and opt.state.t == 0
    assert opt.prepare(50000) == 16384
    assert opt.state.t == 1 and abs(opt.state.beta1_t - 0.9) < 1e-7 and abs(opt.state.alpha_t - 0.99) < 1e-7
    assert opt.state.alpha_t_1 == 1.0
    grad = rng.normal(0, 1, oracle.P).astype(np.float32) * 100
    grad[5] = np.nan
    grad[6] = np.inf
    w16, use16 = opt.adam(grad, 100, write_use=True)
    g = grad.astype(np.float64) / 100
    g[5] = g[6] = 0
    m = 0.1 * g
    v = 0.001 * g * g
    w = w0 - 0.002 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    assert np.allclose(opt.entries[:, 2], w, rtol=1e-5, atol=1e-7)
    assert opt.entries[5, 2] == w0[5] and opt.entries[6, 2] == w0[6]
    eta_t, eta_t1 = 1 - 0.99, 1 - 1.0
    ema = (1 - 0.99) / eta_t * w + 0.99 * eta_t1 * w0
    assert np.allclose(opt.entries[:, 3], ema, rtol=1e-5, atol=1e-6)
    assert np.array_equal(w16, opt.entries[:, 2].astype(np.float16).view(np.uint16))
    assert np.array_equal(use16, w16)
    before = opt.entries.copy()
    opt.adam(grad, 0)
    assert np.array_equal(before, opt.entries)


def test_e4m3_conversion_follows_the_format(oracle):
    """oracle_f32_to_e4m3 / oracle_e4m3_to_f32 (the FP8 query's conversions)
    against the E4M3 definition: bias 7, 3 mantissa bits, subnormals at
    2^-9, no infinities, max 448, NaN codes 0x7F/0xFF; round to nearest even,
    saturated to +-448."""
    codes = np.arange(256, dtype=np.uint8)
    vals = oracle.e4m3_decode(codes)
    finite = ~np.isnan(vals)
    assert set(codes[~finite].tolist()) == {0x7F, 0xFF}
    s, e, m = codes >> 7, (codes >> 3) & 15, (codes & 7).astype(np.float64)
    mag = np.where(e == 0, m * 2.0 ** -9, (1.0 + m / 8.0) * 2.0 ** (e.astype(np.int64) - 7))
    ref = np.where(s == 1, -mag, mag).astype(np.float32)
    assert np.array_equal(vals[finite], ref[finite])
    assert np.array_equal(oracle.e4m3(vals[finite]), codes[finite])  # every finite code round-trips
    assert oracle.e4m3([448.0, 449.0, 1000.0, 1e30, -1e30]).tolist() == [0x7E, 0x7E, 0x7E, 0x7E, 0xFE]
    assert oracle.e4m3([float("nan")]).tolist() == [0x7F]
    # midpoints between neighbours (and between 0 and the smallest subnormal)
    # go to the even code; a hair either side goes to the nearer neighbour
    pos = np.concatenate([[0.0], np.sort(vals[finite & (vals > 0)]).astype(np.float64)])
    lo, hi = pos[:-1], pos[1:]
    mid = ((lo + hi) / 2).astype(np.float32)
    c_lo, c_hi = oracle.e4m3(lo.astype(np.float32)), oracle.e4m3(hi.astype(np.float32))
    want = np.where(c_lo % 2 == 0, c_lo, c_hi)
    assert np.array_equal(oracle.e4m3(mid), want)
    below = np.nextafter(mid, np.float32(0))
    above = np.nextafter(mid, np.float32(np.inf))
    assert np.array_equal(oracle.e4m3(below), c_lo)
    assert np.array_equal(oracle.e4m3(above), c_hi)
    assert np.array_equal(oracle.e4m3(-mid), want | 0x80)


def test_fp8_quantize_scales_and_weights(oracle):
    """oracle_fp8_quantize: per-layer weight scale max|W_l| / 448, its inverse,
    and each weight e4m3(w * 448 / max|W_l|); with no observed activations the
    input scales follow the bound max|x_l| <= max|x_{l-1}| * max row sum |W|
    from max|x_0| = 1, and c[l] = s_w[l] s_x[l] / s_x[l+1]."""
    rng = np.random.default_rng(5)
    w = (rng.standard_normal(20672) * np.sqrt(2 / 64)).astype(np.float16)
    w8, st = oracle.fp8_quantize(w.view(np.uint16))
    s_w, s_x, c, inv_sx0, inv_w = st[0:6], st[6:12], st[12:18], st[18], st[19:25]
    layer = np.minimum(np.arange(20672) // 4096, 5)
    wf = w.astype(np.float32)
    amax = np.array([np.abs(wf[layer == l]).max() for l in range(6)], np.float32)
    assert np.array_equal(s_w, amax / np.float32(448))
    assert np.array_equal(inv_w, np.float32(448) / amax)
    assert np.array_equal(w8, oracle.e4m3(wf * inv_w[layer]))
    rowsum = [np.abs(wf[layer == l].reshape(-1, 64)).sum(1).max() for l in range(6)]
    ax = [1.0]
    for l in range(1, 6):
        ax.append(ax[-1] * rowsum[l - 1])
    assert np.allclose(s_x, np.array(ax) / 448, rtol=1e-5)
    assert np.allclose(c[:5], s_w[:5] * s_x[:5] / s_x[1:], rtol=1e-6)
    assert np.isclose(c[5], s_w[5] * s_x[5], rtol=1e-6) and np.isclose(inv_sx0, 1 / s_x[0], rtol=1e-6)


def test_encode_f32_rounds_to_the_16_bit_encodings(oracle):
    """oracle_encode_f32 (the FP8 query's unrounded features) rounded to fp16
    (numpy's round to nearest even) and to bf16 (round to nearest even on the
    bit pattern) gives oracle_encode's fp16 and bf16 features bit for bit."""
    from vknrc_gb300 import synthetic as S

    rec = S.inputs(S.rng_for(91), 4096)
    rec[:7, 0] = [0.0, -0.0, 1e-30, 3.75, -2.5e6, 1e38, 0.5]  # edge positions (large, tiny, exact)
    f = oracle.encode_f32(rec)
    assert np.array_equal(f.astype(np.float16).view(np.uint16), oracle.encode(rec, 0))
    u = f.view(np.uint32).astype(np.uint64)
    bf = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    assert np.array_equal(bf, oracle.encode(rec, 1))
