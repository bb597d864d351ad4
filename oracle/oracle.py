"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so) — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only to check the GPU path against. The product library never uses it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libnrcref.so")

P = 20672

_lib = None
_ref = None


def build() -> None:
    subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        vp, i64, i32, f32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float
        _lib.oracle_encode.argtypes = [vp, i64, vp]
        _lib.oracle_encode_fmt.argtypes = [vp, i64, vp, i32]
        _lib.oracle_forward_f32_fmt.argtypes = [vp, vp, i64, vp, i32, i32]
        _lib.oracle_forward_f64_fmt.argtypes = [vp, vp, i64, vp, i32, i32]
        _lib.oracle_train_grad_fmt.argtypes = [vp, vp, vp, i64, f32, i32, vp, vp, vp, i32, i32]
        _lib.oracle_adam_fmt.argtypes = [vp, vp, ctypes.c_uint32, vp, vp, vp, vp, i32, i32]
        _lib.oracle_sph_encode.argtypes = [vp, i64, vp]
        _lib.oracle_forward_f32.argtypes = [vp, vp, i64, vp, i32]
        _lib.oracle_forward_f64.argtypes = [vp, vp, i64, vp, i32]
        _lib.oracle_train_grad.argtypes = [vp, vp, vp, i64, f32, i32, vp, vp, vp, i32]
        _lib.oracle_train_grad_w64.argtypes = [vp, vp, vp, i64, f32, vp, vp, i32]
        _lib.oracle_scatter.argtypes = [vp, vp, i64, vp, vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp]
        _lib.oracle_prepare.argtypes = [ctypes.c_uint32, vp, vp]
        _lib.oracle_prepare.restype = ctypes.c_uint32
        _lib.oracle_adam.argtypes = [vp, vp, ctypes.c_uint32, vp, vp, vp, vp, i32]
        _lib.oracle_screen.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, i32, ctypes.c_uint32, vp, vp]
        _lib.oracle_unpack.argtypes = [vp, vp, i64, i64, vp, i64]
        _lib.oracle_path_trace.argtypes = [vp, vp, vp, vp]
        _lib.oracle_f32_to_e4m3.argtypes = [f32]
        _lib.oracle_f32_to_e4m3.restype = ctypes.c_uint8
        _lib.oracle_e4m3_to_f32.argtypes = [ctypes.c_uint8]
        _lib.oracle_e4m3_to_f32.restype = f32
        _lib.oracle_encode_f32.argtypes = [vp, i64, vp]
        _lib.oracle_fp8_quantize.argtypes = [vp, i32, vp, vp, vp]
        _lib.oracle_forward_fp8.argtypes = [vp, vp, f32, vp, i64, vp, i32]
        _lib.oracle_loss_rows.argtypes = [vp, vp, i64, f32, i32, vp]
        _lib.oracle_expf.argtypes = [f32]
        _lib.oracle_expf.restype = f32
    return _lib


def ref_lib():
    """The reference's own CPU code (built from the reference tree), or None."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB_PATH):
        _ref = ctypes.CDLL(REF_LIB_PATH)
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        _ref.ref_encode.argtypes = [vp, i64, vp]
        _ref.ref_sph_encode.argtypes = [vp, i64, vp]
        _ref.ref_evaluate.argtypes = [vp, vp, i64, vp]
        _ref.ref_train.argtypes = [vp, vp, vp, i64, vp]
        if hasattr(_ref, "ref_prepare"):
            _ref.ref_prepare.argtypes = [ctypes.c_uint32, vp, vp]
            _ref.ref_prepare.restype = ctypes.c_uint32
            _ref.ref_optimize.argtypes = [vp, vp, i64, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp]
            _ref.ref_loss_rows.argtypes = [vp, vp, i64, ctypes.c_float, vp]
    return _ref


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def encode(records: np.ndarray, fmt: int = 0) -> np.ndarray:
    """records (n, 14) float32 -> (n, 64) uint16 bit patterns: fp16 (fmt 0) or bf16 (fmt 1)."""
    r = _c(records, np.float32).reshape(-1, 14)
    out = np.empty((r.shape[0], 64), np.uint16)
    lib().oracle_encode_fmt(_p(r), r.shape[0], _p(out), fmt)
    return out


def sph_encode(dirs: np.ndarray) -> np.ndarray:
    d = _c(dirs, np.float32).reshape(-1, 3)
    out = np.empty((d.shape[0], 2), np.float32)
    lib().oracle_sph_encode(_p(d), d.shape[0], _p(out))
    return out


def expf(x: float) -> float:
    return lib().oracle_expf(x)


def forward_f32(weights: np.ndarray, enc: np.ndarray, nthreads: int = 1, fmt: int = 0) -> np.ndarray:
    w = _c(weights, np.uint16)
    e = _c(enc, np.uint16).reshape(-1, 64)
    out = np.empty((e.shape[0], 3), np.float32)
    lib().oracle_forward_f32_fmt(_p(w), _p(e), e.shape[0], _p(out), nthreads, fmt)
    return out


def forward_f64(weights: np.ndarray, enc: np.ndarray, nthreads: int = 1, fmt: int = 0) -> np.ndarray:
    w = _c(weights, np.uint16)
    e = _c(enc, np.uint16).reshape(-1, 64)
    out = np.empty((e.shape[0], 3), np.float64)
    lib().oracle_forward_f64_fmt(_p(w), _p(e), e.shape[0], _p(out), nthreads, fmt)
    return out


def train_grad(weights, enc, target, loss_scale=1.0, mode=0, nthreads=1, want_abs=False, fmt=0):
    """Returns (grad[P] float64 sum over records, grad_abs or None, loss_sum).
    fmt: 16-bit format of weights, features and stored activations (0 fp16, 1 bf16)."""
    w = _c(weights, np.uint16)
    e = _c(enc, np.uint16).reshape(-1, 64)
    t = _c(target, np.float32).reshape(-1, 3)
    g = np.zeros(P, np.float64)
    a = np.zeros(P, np.float64) if want_abs else None
    loss = ctypes.c_double(0.0)
    lib().oracle_train_grad_fmt(_p(w), _p(e), _p(t), e.shape[0], loss_scale, mode, _p(g),
                                _p(a) if a is not None else None, ctypes.byref(loss), nthreads, fmt)
    return g, a, loss.value


def train_grad_w64(weights64, enc, target, loss_scale=1.0, nthreads=1):
    """FP64 gradient sums and loss with FP64 weights (the FP64 oracle's training
    loop). Returns (grad[P] float64, loss_sum)."""
    w = _c(weights64, np.float64)
    assert w.size == P
    e = _c(enc, np.uint16).reshape(-1, 64)
    t = _c(target, np.float32).reshape(-1, 3)
    g = np.zeros(P, np.float64)
    loss = ctypes.c_double(0.0)
    lib().oracle_train_grad_w64(_p(w), _p(e), _p(t), e.shape[0], loss_scale, _p(g), ctypes.byref(loss), nthreads)
    return g, loss.value


def scatter(pred, dst, bias_factor_r, factor_gb, train_records):
    """Destination epilogue (nrc_inference.comp:50-73) on host copies: updates
    bias_factor_r ([H][W][4] float32) and the train record arrays ((cap, 20)
    float32 each, or None) in place, in query order."""
    pred = _c(pred, np.float32).reshape(-1, 3)
    dst = _c(dst, np.uint32).reshape(-1)
    assert pred.shape[0] == dst.shape[0]
    assert bias_factor_r.dtype == np.float32 and bias_factor_r.flags.c_contiguous
    gb = _c(factor_gb, np.float32)
    h, w = bias_factor_r.shape[0], bias_factor_r.shape[1]
    ptrs = (ctypes.c_void_p * 4)()
    caps = (ctypes.c_uint32 * 4)()
    for b in range(4):
        t = train_records[b] if b < len(train_records) else None
        if t is not None:
            assert t.dtype == np.float32 and t.flags.c_contiguous and t.shape[1] == 20
            ptrs[b] = t.ctypes.data
            caps[b] = t.shape[0]
    lib().oracle_scatter(_p(pred), _p(dst), dst.shape[0], _p(bias_factor_r), _p(gb), w, h, ptrs, caps)


def screen(color, accumulate=None, accumulate_count=0):
    """Screen pass (screen.frag:10-31) on host arrays: color (H, W, 4) float32;
    accumulate (H, W, 4) float32 updated in place when given. Returns
    (rgba8 (H, W, 4) uint8, rgba (H, W, 4) float32)."""
    c = _c(color, np.float32)
    h, w = c.shape[0], c.shape[1]
    o8 = np.empty((h, w, 4), np.uint8)
    of = np.empty((h, w, 4), np.float32)
    if accumulate is not None:
        assert accumulate.dtype == np.float32 and accumulate.flags.c_contiguous
    lib().oracle_screen(_p(c), _p(accumulate) if accumulate is not None else None, w, h, int(accumulate is not None),
                        accumulate_count, _p(o8), _p(of))
    return o8, of


class _Scene(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("vertex_indices", ctypes.c_void_p), ("texcoords", ctypes.c_void_p),
                ("texcoord_indices", ctypes.c_void_p), ("materials", ctypes.c_void_p),
                ("material_ids", ctypes.c_void_p), ("transforms", ctypes.c_void_p), ("textures", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("texcoord_count", ctypes.c_uint32),
                ("material_count", ctypes.c_uint32), ("primitive_count", ctypes.c_uint32),
                ("instance_count", ctypes.c_uint32), ("texture_count", ctypes.c_uint32)]


class _Texture(ctypes.Structure):
    _fields_ = [("texels", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


def _scene_struct(sc: dict):
    """(oracle_scene, keep-alive list) for a scene dict of numpy arrays."""
    arrs = {k: np.ascontiguousarray(v) for k, v in sc.items() if k not in ("textures", "instance_ranges")}
    texs = [np.ascontiguousarray(t) for t in sc["textures"]]
    ttab = (_Texture * max(1, len(texs)))()
    for i, t in enumerate(texs):
        ttab[i] = _Texture(t.ctypes.data, t.shape[1], t.shape[0])
    S = _Scene(_p(arrs["vertices"]), _p(arrs["vertex_indices"]), _p(arrs["texcoords"]), _p(arrs["texcoord_indices"]),
               _p(arrs["materials"]), _p(arrs["material_ids"]), _p(arrs["transforms"]),
               ctypes.cast(ttab, ctypes.c_void_p), arrs["vertices"].shape[0], arrs["texcoords"].shape[0],
               arrs["materials"].shape[0], arrs["vertex_indices"].shape[0], arrs["transforms"].shape[0], len(texs))
    return S, (arrs, texs, ttab)


class TraceParams(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("look", ctypes.c_float * 3), ("side", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("left_method", ctypes.c_uint32), ("right_method", ctypes.c_uint32),
                ("train_probability", ctypes.c_float)]


class _TraceOut(ctypes.Structure):
    _fields_ = [("eval_records", ctypes.c_void_p), ("eval_count", ctypes.c_uint32),
                ("eval_capacity", ctypes.c_uint32), ("train_records", ctypes.c_void_p * 4),
                ("train_counts", ctypes.c_uint32 * 4), ("bias_factor_r", ctypes.c_void_p),
                ("factor_gb", ctypes.c_void_p)]


def path_trace(sc: dict, params: TraceParams, eval_capacity: int) -> dict:
    """The path tracer on host (nrc_trace_oracle.c): returns eval records (k, 5)
    uint32, train records [4 x (count, 10)] uint32 words, train counts,
    bias_factor_r (H, W, 4) and factor_gb (H, W, 2)."""
    S, keep = _scene_struct(sc)
    ranges = np.ascontiguousarray(sc["instance_ranges"], np.uint32)
    h, w = params.height, params.width
    ev = np.zeros((eval_capacity, 5), np.uint32)
    tr = [np.zeros((16384, 10), np.uint32) for _ in range(4)]
    bf = np.zeros((h, w, 4), np.float32)
    gb = np.zeros((h, w, 2), np.float32)
    o = _TraceOut()
    o.eval_records = ev.ctypes.data
    o.eval_capacity = eval_capacity
    for b in range(4):
        o.train_records[b] = tr[b].ctypes.data
    o.bias_factor_r = bf.ctypes.data
    o.factor_gb = gb.ctypes.data
    lib().oracle_path_trace(ctypes.byref(S), _p(ranges), ctypes.byref(params), ctypes.byref(o))
    counts = [int(o.train_counts[b]) for b in range(4)]
    return {"eval": ev[: min(o.eval_count, eval_capacity)], "eval_count": int(o.eval_count),
            "train": [tr[b][: min(counts[b], 16384)] for b in range(4)], "train_counts": counts,
            "bias_factor_r": bf, "factor_gb": gb}


def unpack(sc: dict, packed_words: np.ndarray, first_word: int = 0) -> np.ndarray:
    """UnpackNRCInput (NRCRecord.glsl:97-125) on host: packed_words (n, k)
    uint32 records whose packed input starts at column first_word. Returns
    (n, 14) float32 nrc_input records."""
    S, keep = _scene_struct(sc)
    w = np.ascontiguousarray(packed_words, np.uint32)
    n = w.shape[0]
    out = np.empty((n, 14), np.float32)
    base = w[:, first_word:]
    lib().oracle_unpack(ctypes.byref(S), _p(np.ascontiguousarray(base)) if first_word else _p(w), n,
                        base.shape[1] if first_word else w.shape[1], _p(out), 14)
    return out


def encode_f32(records: np.ndarray) -> np.ndarray:
    """records (n, 14) -> (n, 64) float32 features before any rounding."""
    r = _c(records, np.float32).reshape(-1, 14)
    out = np.empty((r.shape[0], 64), np.float32)
    lib().oracle_encode_f32(_p(r), r.shape[0], _p(out))
    return out


def e4m3(x) -> np.ndarray:
    """float32 array -> E4M3 bytes (round to nearest even, saturated)."""
    x = np.asarray(x, np.float32).ravel()
    return np.array([lib().oracle_f32_to_e4m3(float(v)) for v in x], np.uint8)


def e4m3_decode(b) -> np.ndarray:
    b = np.asarray(b, np.uint8).ravel()
    return np.array([lib().oracle_e4m3_to_f32(int(v)) for v in b], np.float32)


def fp8_quantize(w16: np.ndarray, fmt: int = 0, seen=None):
    """The FP8 refresh: returns (w8 (P,) uint8, state (25,) float32: s_w[6],
    s_x[6], c[6], 1/s_x[0], 448/max|W|[6])."""
    w = _c(w16, np.uint16)
    sn = _c(np.zeros(6) if seen is None else seen, np.float32)
    st = np.empty(25, np.float32)
    w8 = np.empty(P, np.uint8)
    lib().oracle_fp8_quantize(_p(w), fmt, _p(sn), _p(st), _p(w8))
    return w8, st


def forward_fp8(w8: np.ndarray, c, inv_sx0: float, feats: np.ndarray, nthreads: int = 1) -> np.ndarray:
    f = _c(feats, np.float32).reshape(-1, 64)
    cc = _c(c, np.float32)
    out = np.empty((f.shape[0], 3), np.float32)
    lib().oracle_forward_fp8(_p(_c(w8, np.uint8)), _p(cc), float(inv_sx0), _p(f), f.shape[0], _p(out), nthreads)
    return out


class OptState(ctypes.Structure):
    _fields_ = [("t", ctypes.c_uint32), ("beta1_t", ctypes.c_float), ("beta2_t", ctypes.c_float),
                ("alpha_t", ctypes.c_float), ("alpha_t_1", ctypes.c_float)]


class HParams(ctypes.Structure):
    _fields_ = [("learning_rate", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("epsilon", ctypes.c_float), ("ema_alpha", ctypes.c_float), ("loss_scale", ctypes.c_float),
                ("batch_cap", ctypes.c_uint32)]


class Optimizer:
    """Host mirror of the reference's optimizer state (nrc_train_prepare + nrc_optimize)."""

    def __init__(self, weights_f32: np.ndarray, hp: HParams):
        self.hp = hp
        self.state = OptState(0, 1.0, 1.0, 1.0, 0.0)
        self.entries = np.zeros((P, 4), np.float32)
        self.entries[:, 2] = weights_f32
        self.entries[:, 3] = weights_f32

    def prepare(self, count: int) -> int:
        return lib().oracle_prepare(count, ctypes.byref(self.hp), ctypes.byref(self.state))

    def adam(self, grad32: np.ndarray, count: int, write_use: bool = True, use_ema: bool = False, fmt: int = 0):
        g = _c(grad32, np.float32)
        w16 = np.zeros(P, np.uint16)
        use16 = np.zeros(P, np.uint16) if write_use else None
        lib().oracle_adam_fmt(_p(self.entries), _p(g), count, ctypes.byref(self.state), ctypes.byref(self.hp),
                              _p(w16), _p(use16) if use16 is not None else None, int(use_ema), fmt)
        return w16, use16


def loss_rows(pred: np.ndarray, target: np.ndarray, loss_scale: float = 1.0, fmt: int = 0) -> np.ndarray:
    """(n, 2) uint32: the relative-L2 gradient row words of each (prediction, target) pair."""
    p = _c(pred, np.float32).reshape(-1, 3)
    t = _c(target, np.float32).reshape(-1, 3)
    out = np.empty((p.shape[0], 2), np.uint32)
    lib().oracle_loss_rows(_p(p), _p(t), p.shape[0], float(loss_scale), fmt, _p(out))
    return out


def ref_prepare(count: int, state: OptState):
    """nrc_train_prepare.comp compiled from the reference: (clamped count, work groups); advances state."""
    r = ref_lib()
    groups = ctypes.c_uint32(0)
    n = r.ref_prepare(count, ctypes.byref(state), ctypes.byref(groups))
    return n, groups.value


def ref_optimize(entries: np.ndarray, grad: np.ndarray, count: int, state: OptState, use_ema: bool,
                 w16: np.ndarray, use16: np.ndarray) -> None:
    """nrc_optimize.comp compiled from the reference, in place on entries / w16 / use16."""
    assert entries.dtype == np.float32 and entries.flags.c_contiguous and entries.shape == (P, 4)
    assert w16.dtype == np.uint16 and use16.dtype == np.uint16
    g = _c(grad, np.float32)
    ref_lib().ref_optimize(_p(entries), _p(g), P, count, ctypes.byref(state), int(use_ema), _p(w16), _p(use16))


def ref_loss_rows(pred: np.ndarray, target: np.ndarray, loss_scale: float = 1.0) -> np.ndarray:
    """NNLoadDA3_RelativeL2LuminanceLoss compiled from the reference: (n, 2) uint32 row words."""
    p = _c(pred, np.float32).reshape(-1, 3)
    t = _c(target, np.float32).reshape(-1, 3)
    out = np.empty((p.shape[0], 2), np.uint32)
    ref_lib().ref_loss_rows(_p(p), _p(t), p.shape[0], float(loss_scale), _p(out))
    return out


def ref_encode(records: np.ndarray):
    r = ref_lib()
    if r is None:
        return None
    rec = _c(records, np.float32).reshape(-1, 14)
    out = np.empty((rec.shape[0], 64), np.uint16)
    r.ref_encode(_p(rec), rec.shape[0], _p(out))
    return out


def ref_sph_encode(dirs: np.ndarray):
    r = ref_lib()
    if r is None:
        return None
    d = _c(dirs, np.float32).reshape(-1, 3)
    out = np.empty((d.shape[0], 2), np.float32)
    r.ref_sph_encode(_p(d), d.shape[0], _p(out))
    return out


def ref_evaluate(weights: np.ndarray, enc: np.ndarray):
    r = ref_lib()
    if r is None:
        return None
    w = _c(weights, np.uint16)
    e = _c(enc, np.uint16).reshape(-1, 64)
    out = np.empty((e.shape[0], 3), np.uint16)
    r.ref_evaluate(_p(w), _p(e), e.shape[0], _p(out))
    return out
