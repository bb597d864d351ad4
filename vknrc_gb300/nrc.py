"""Python binding of libnrc.so (include/nrc.h) over ctypes.

Thin glue for tests and benchmarks: device memory and streams come from
PyTorch tensors, every call goes through the C ABI. There is no fallback: if
libnrc.so is missing the import of a Cache fails loudly.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

P = 20672
IN_FLOATS = 14
TRAIN_FLOATS = 20
TRAIN_BATCH_SIZE = 16384
TRAIN_BATCH_COUNT = 4
WEIGHTS_USE, WEIGHTS_TRAIN = 0, 1

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "no CUDA device", 4: "unsupported device",
          5: "out of device memory", 6: "device timeout", 7: "misaligned buffer", 8: "too large",
          9: "bad checkpoint"}

EXPORTS = [
    "nrc_status_string", "nrc_default_config", "nrc_create", "nrc_destroy", "nrc_reset", "nrc_he_init_host",
    "nrc_encode", "nrc_sph_encode", "nrc_infer", "nrc_infer_encoded", "nrc_train", "nrc_gradient", "nrc_frame",
    "nrc_get_weights", "nrc_set_weights", "nrc_get_optimizer", "nrc_set_optimizer", "nrc_get_loss",
    "nrc_get_error", "nrc_get_device_buffers", "nrc_train_noalloc", "nrc_train_batches", "nrc_infer_scatter",
    "nrc_frame_scatter", "nrc_infer_many", "nrc_train_many", "nrc_plan_query_ctas", "nrc_plan_train_ctas",
    "nrc_server_create", "nrc_server_destroy", "nrc_server_open_session", "nrc_server_close_session",
    "nrc_server_frame_buffers", "nrc_server_session_cache", "nrc_server_submit", "nrc_server_wait",
    "nrc_server_get_stats", "nrc_screen", "nrc_checkpoint_bytes", "nrc_save_checkpoint", "nrc_load_checkpoint",
    "nrc_unpack_eval", "nrc_unpack_train", "nrc_infer_fp8", "nrc_fp8_refresh", "nrc_get_fp8",
    "nrc_frame_overlapped", "nrc_autotune_frame", "nrc_bvh_build", "nrc_bvh_destroy", "nrc_bvh_info",
    "nrc_path_trace", "nrc_optimize", "nrc_loss_gradient", "nrc_infer_packed", "nrc_infer_scatter_packed",
    "nrc_frame_packed", "nrc_frame_scatter_packed", "nrc_autotune_many", "nrc_scene_prepare",
    "nrc_scene_tables_destroy",
]


class NRCError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {STATUS.get(status, status)} ({status})")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("train_batch_size", ctypes.c_uint32), ("learning_rate", ctypes.c_float),
                ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("epsilon", ctypes.c_float),
                ("ema_alpha", ctypes.c_float), ("loss_scale", ctypes.c_float),
                ("use_ema_weights", ctypes.c_uint32), ("deterministic", ctypes.c_uint32),
                ("track_loss", ctypes.c_uint32), ("seed", ctypes.c_uint64), ("precision", ctypes.c_uint32),
                ("fp8_inference", ctypes.c_uint32)]


PRECISION_FP16, PRECISION_BF16 = 0, 1


class OptState(ctypes.Structure):
    _fields_ = [("t", ctypes.c_uint32), ("beta1_t", ctypes.c_float), ("beta2_t", ctypes.c_float),
                ("alpha_t", ctypes.c_float), ("alpha_t_1", ctypes.c_float)]


class ScatterTargets(ctypes.Structure):
    """nrc_scatter_targets: where the destination epilogue writes."""
    _fields_ = [("bias_factor_r", ctypes.c_void_p), ("factor_gb", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("train_records", ctypes.c_void_p * TRAIN_BATCH_COUNT),
                ("train_capacity", ctypes.c_uint32 * TRAIN_BATCH_COUNT)]


def scatter_targets(bias_factor_r=None, factor_gb=None, train_records: Sequence = ()) -> ScatterTargets:
    """Build the targets from CUDA tensors: bias_factor_r (H, W, 4) and
    factor_gb (H, W, 2) float32 images, up to four train record arrays: (cap, 20)
    nrc_train_record rows, or (cap, 10) nrc_packed_train_record rows for the
    packed-record calls (None entries are skipped)."""
    t = ScatterTargets()
    if bias_factor_r is not None:
        t.bias_factor_r = _ptr(bias_factor_r)
        t.factor_gb = _ptr(factor_gb)
        t.height, t.width = bias_factor_r.shape[0], bias_factor_r.shape[1]
    for b, r in enumerate(train_records):
        if r is not None:
            t.train_records[b] = _ptr(r)
            t.train_capacity[b] = r.shape[0]
    return t


class FramePlan(ctypes.Structure):
    """nrc_frame_plan: CTAs of the query and of the training in an overlapped frame."""
    _fields_ = [("query_ctas", ctypes.c_uint32), ("train_ctas", ctypes.c_uint32)]


class TraceParams(ctypes.Structure):
    """nrc_trace_params: camera, frame and methods of the path tracer."""
    _fields_ = [("origin", ctypes.c_float * 3), ("look", ctypes.c_float * 3), ("side", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("left_method", ctypes.c_uint32), ("right_method", ctypes.c_uint32),
                ("train_probability", ctypes.c_float)]


class TraceTargets(ctypes.Structure):
    _fields_ = [("eval_records", ctypes.c_void_p), ("eval_count", ctypes.c_void_p), ("eval_capacity", ctypes.c_uint32),
                ("train_records", ctypes.c_void_p * TRAIN_BATCH_COUNT),
                ("train_counts", ctypes.c_void_p * TRAIN_BATCH_COUNT), ("bias_factor_r", ctypes.c_void_p),
                ("factor_gb", ctypes.c_void_p)]


class QueryJob(ctypes.Structure):
    """nrc_query_job: one cache's queries in a batched launch."""
    _fields_ = [("ctx", ctypes.c_void_p), ("inputs", ctypes.c_void_p), ("d_count", ctypes.c_void_p),
                ("capacity", ctypes.c_uint32), ("out_rgb", ctypes.c_void_p), ("weight_set", ctypes.c_int)]


class TrainJob(ctypes.Structure):
    """nrc_train_job: one cache's chained training steps in a batched launch."""
    _fields_ = [("ctx", ctypes.c_void_p), ("records", ctypes.c_void_p * TRAIN_BATCH_COUNT),
                ("d_counts", ctypes.c_void_p * TRAIN_BATCH_COUNT), ("capacity", ctypes.c_uint32),
                ("nbatches", ctypes.c_int), ("write_use_last", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_batch_sessions", ctypes.c_uint32),
                ("max_inflight_batches", ctypes.c_uint32), ("device_loop", ctypes.c_uint32)]


class SessionDesc(ctypes.Structure):
    _fields_ = [("cache", Config), ("max_queries", ctypes.c_uint32), ("train_records", ctypes.c_uint32),
                ("frame_slots", ctypes.c_uint32), ("train_ctas", ctypes.c_uint32)]


class FrameBuffers(ctypes.Structure):
    _fields_ = [("queries", ctypes.c_void_p), ("query_count", ctypes.c_void_p), ("out_rgb", ctypes.c_void_p),
                ("train", ctypes.c_void_p * TRAIN_BATCH_COUNT), ("train_count", ctypes.c_void_p * TRAIN_BATCH_COUNT)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("bytes_in_use", ctypes.c_uint64), ("latency_p50_ms", ctypes.c_double),
                ("latency_p99_ms", ctypes.c_double), ("latency_max_ms", ctypes.c_double),
                ("mean_batch_sessions", ctypes.c_double)]


class SceneStruct(ctypes.Structure):
    """nrc_scene: device pointers of the scene buffers and their counts."""
    _fields_ = [("vertices", ctypes.c_void_p), ("vertex_indices", ctypes.c_void_p), ("texcoords", ctypes.c_void_p),
                ("texcoord_indices", ctypes.c_void_p), ("materials", ctypes.c_void_p),
                ("material_ids", ctypes.c_void_p), ("transforms", ctypes.c_void_p), ("textures", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("texcoord_count", ctypes.c_uint32),
                ("material_count", ctypes.c_uint32), ("primitive_count", ctypes.c_uint32),
                ("instance_count", ctypes.c_uint32), ("texture_count", ctypes.c_uint32),
                ("tables", ctypes.c_void_p)]


_lib: Optional[ctypes.CDLL] = None


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libnrc.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise RuntimeError(f"libnrc.so not built: {_build.LIB}")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    vp, u32, i32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64
    L.nrc_status_string.restype = ctypes.c_char_p
    L.nrc_status_string.argtypes = [i32]
    L.nrc_default_config.argtypes = [ctypes.POINTER(Config)]
    L.nrc_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    L.nrc_destroy.argtypes = [vp]
    L.nrc_reset.argtypes = [vp, u64]
    L.nrc_he_init_host.argtypes = [u64, vp]
    L.nrc_encode.argtypes = [vp, vp, vp, u32, vp, vp]
    L.nrc_sph_encode.argtypes = [vp, vp, u32, vp, vp]
    L.nrc_infer.argtypes = [vp, vp, vp, u32, vp, i32, vp]
    L.nrc_infer_encoded.argtypes = [vp, vp, vp, u32, vp, i32, vp]
    L.nrc_train.argtypes = [vp, vp, vp, u32, i32, vp]
    L.nrc_gradient.argtypes = [vp, vp, vp, u32, vp, vp]
    L.nrc_optimize.argtypes = [vp, vp, vp, i32, vp]
    L.nrc_loss_gradient.argtypes = [vp, vp, vp, u32, ctypes.c_float, u32, vp, vp]
    L.nrc_train_batches.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), u32, i32, i32, vp]
    L.nrc_frame.argtypes = [vp, vp, vp, u32, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), u32, vp]
    L.nrc_get_weights.argtypes = [vp, i32, vp]
    L.nrc_set_weights.argtypes = [vp, vp]
    L.nrc_get_optimizer.argtypes = [vp, ctypes.POINTER(OptState), vp]
    L.nrc_set_optimizer.argtypes = [vp, ctypes.POINTER(OptState), vp]
    L.nrc_get_loss.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]
    L.nrc_get_error.argtypes = [vp]
    L.nrc_train_noalloc.argtypes = [vp, vp, vp, vp, vp, vp, u32, ctypes.POINTER(Config), vp, vp]
    L.nrc_infer_scatter.argtypes = [vp, vp, vp, vp, u32, ctypes.POINTER(ScatterTargets), vp, i32, vp]
    L.nrc_frame_scatter.argtypes = [vp, vp, vp, vp, u32, ctypes.POINTER(ScatterTargets), ctypes.POINTER(vp), vp]
    L.nrc_get_device_buffers.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                         ctypes.POINTER(vp)]
    L.nrc_infer_many.argtypes = [ctypes.POINTER(QueryJob), u32, vp, vp]
    L.nrc_train_many.argtypes = [ctypes.POINTER(TrainJob), u32, vp, vp]
    L.nrc_plan_query_ctas.argtypes = [ctypes.POINTER(QueryJob), u32, vp]
    L.nrc_plan_train_ctas.argtypes = [ctypes.POINTER(TrainJob), u32, vp]
    L.nrc_autotune_many.argtypes = [ctypes.POINTER(QueryJob), u32, ctypes.POINTER(TrainJob), u32, vp, vp,
                                    ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.nrc_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]
    L.nrc_server_destroy.argtypes = [vp]
    L.nrc_server_open_session.argtypes = [vp, ctypes.POINTER(SessionDesc), ctypes.POINTER(u32)]
    L.nrc_server_close_session.argtypes = [vp, u32]
    L.nrc_server_frame_buffers.argtypes = [vp, u32, u32, ctypes.POINTER(FrameBuffers)]
    L.nrc_server_session_cache.argtypes = [vp, u32, ctypes.POINTER(vp)]
    L.nrc_server_submit.argtypes = [vp, u32, u32, vp, ctypes.POINTER(u64)]
    L.nrc_server_wait.argtypes = [vp, u64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    L.nrc_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats), i32]
    L.nrc_screen.argtypes = [vp, vp, u32, u32, i32, u32, vp, vp, vp]
    L.nrc_frame_overlapped.argtypes = [vp, vp, vp, u32, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), u32,
                                       ctypes.POINTER(FramePlan), vp, vp]
    L.nrc_autotune_frame.argtypes = [vp, vp, vp, u32, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), u32,
                                     ctypes.POINTER(FramePlan), ctypes.POINTER(ctypes.c_float)]
    L.nrc_infer_fp8.argtypes = [vp, vp, vp, u32, vp, vp]
    L.nrc_fp8_refresh.argtypes = [vp, vp]
    L.nrc_get_fp8.argtypes = [vp, vp, vp]
    L.nrc_bvh_build.argtypes = [ctypes.POINTER(SceneStruct), vp, ctypes.POINTER(vp)]
    L.nrc_bvh_destroy.argtypes = [vp]
    L.nrc_bvh_info.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.nrc_path_trace.argtypes = [ctypes.POINTER(SceneStruct), vp, ctypes.POINTER(TraceParams),
                                 ctypes.POINTER(TraceTargets), vp]
    L.nrc_unpack_eval.argtypes = [ctypes.POINTER(SceneStruct), vp, vp, u32, vp, vp, vp]
    L.nrc_scene_prepare.argtypes = [ctypes.POINTER(SceneStruct), vp, ctypes.POINTER(vp)]
    L.nrc_scene_tables_destroy.argtypes = [vp]
    L.nrc_infer_packed.argtypes = [vp, ctypes.POINTER(SceneStruct), vp, vp, u32, vp, i32, vp]
    L.nrc_infer_scatter_packed.argtypes = [vp, ctypes.POINTER(SceneStruct), vp, vp, u32,
                                           ctypes.POINTER(ScatterTargets), vp, i32, vp]
    L.nrc_frame_packed.argtypes = [vp, ctypes.POINTER(SceneStruct), vp, vp, u32, vp, ctypes.POINTER(vp),
                                   ctypes.POINTER(vp), u32, vp]
    L.nrc_frame_scatter_packed.argtypes = [vp, ctypes.POINTER(SceneStruct), vp, vp, u32,
                                           ctypes.POINTER(ScatterTargets), ctypes.POINTER(vp), vp]
    L.nrc_unpack_train.argtypes = [ctypes.POINTER(SceneStruct), vp, vp, u32, vp, vp]
    L.nrc_checkpoint_bytes.restype = ctypes.c_size_t
    L.nrc_checkpoint_bytes.argtypes = []
    L.nrc_save_checkpoint.argtypes = [vp, vp, ctypes.c_size_t]
    L.nrc_load_checkpoint.argtypes = [vp, vp, ctypes.c_size_t]
    _lib = L
    return L


def check(status: int, what: str) -> None:
    if status != 0:
        raise NRCError(status, what)


def default_config(**overrides) -> Config:
    c = Config()
    check(lib().nrc_default_config(ctypes.byref(c)), "nrc_default_config")
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


def he_init_host(seed: int) -> np.ndarray:
    w = np.empty(P, np.float32)
    check(lib().nrc_he_init_host(seed, w.ctypes.data_as(ctypes.c_void_p)), "nrc_he_init_host")
    return w


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    return t.data_ptr()


def _stream(stream) -> Optional[int]:
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


class Cache:
    """One neural radiance cache (an nrc_context): weights + Adam state on the GPU."""

    def __init__(self, **cfg):
        self.cfg = default_config(**cfg)
        h = ctypes.c_void_p()
        check(lib().nrc_create(ctypes.byref(self.cfg), ctypes.byref(h)), "nrc_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().nrc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------ compute --
    def encode(self, inputs, count, out, capacity=None, stream=None):
        cap = inputs.shape[0] if capacity is None else capacity
        check(lib().nrc_encode(self.h, _ptr(inputs), _ptr(count), cap, _ptr(out), _stream(stream)), "nrc_encode")

    def infer(self, inputs, count, out, capacity=None, weight_set=WEIGHTS_USE, stream=None):
        cap = inputs.shape[0] if capacity is None else capacity
        check(lib().nrc_infer(self.h, _ptr(inputs), _ptr(count), cap, _ptr(out), weight_set, _stream(stream)),
              "nrc_infer")

    def infer_encoded(self, enc, count, out, capacity=None, weight_set=WEIGHTS_USE, stream=None):
        cap = enc.shape[0] if capacity is None else capacity
        check(lib().nrc_infer_encoded(self.h, _ptr(enc), _ptr(count), cap, _ptr(out), weight_set,
                                      _stream(stream)), "nrc_infer_encoded")

    def infer_scatter(self, inputs, dst, count, targets: ScatterTargets, out=None, capacity=None,
                      weight_set=WEIGHTS_USE, stream=None):
        cap = inputs.shape[0] if capacity is None else capacity
        check(lib().nrc_infer_scatter(self.h, _ptr(inputs), _ptr(dst), _ptr(count), cap, ctypes.byref(targets),
                                      _ptr(out), weight_set, _stream(stream)), "nrc_infer_scatter")

    def frame_scatter(self, eval_inputs, eval_dst, eval_count, targets: ScatterTargets, train_counts: Sequence,
                      eval_capacity=None, stream=None):
        ecap = eval_inputs.shape[0] if eval_capacity is None else eval_capacity
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        check(lib().nrc_frame_scatter(self.h, _ptr(eval_inputs), _ptr(eval_dst), _ptr(eval_count), ecap,
                                      ctypes.byref(targets), cnts, _stream(stream)), "nrc_frame_scatter")

    # ------------------------------------------- the reference's record formats --
    def infer_packed(self, scene: "DeviceScene", records, count, out, capacity=None, weight_set=WEIGHTS_USE,
                     stream=None):
        """nrc_infer_packed: (n, 5) packed eval records of `scene` -> (n, 3) clamped rgb."""
        cap = records.shape[0] if capacity is None else capacity
        check(lib().nrc_infer_packed(self.h, ctypes.byref(scene.s), _ptr(records), _ptr(count), cap, _ptr(out),
                                     weight_set, _stream(stream)), "nrc_infer_packed")

    def infer_scatter_packed(self, scene: "DeviceScene", records, count, targets: ScatterTargets, out=None,
                             capacity=None, weight_set=WEIGHTS_USE, stream=None):
        """nrc_infer_scatter_packed: targets from scatter_targets() with (cap, 10) packed train records."""
        cap = records.shape[0] if capacity is None else capacity
        check(lib().nrc_infer_scatter_packed(self.h, ctypes.byref(scene.s), _ptr(records), _ptr(count), cap,
                                             ctypes.byref(targets), _ptr(out), weight_set, _stream(stream)),
              "nrc_infer_scatter_packed")

    def frame_packed(self, scene: "DeviceScene", eval_records, eval_count, out, train_records: Sequence,
                     train_counts: Sequence, eval_capacity=None, train_capacity=None, stream=None):
        """nrc_frame_packed: packed eval records (n, 5) and four packed train batches (cap, 10)."""
        ecap = eval_records.shape[0] if eval_capacity is None else eval_capacity
        tcap = train_records[0].shape[0] if train_capacity is None else train_capacity
        recs = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(r) for r in train_records])
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        check(lib().nrc_frame_packed(self.h, ctypes.byref(scene.s), _ptr(eval_records), _ptr(eval_count), ecap,
                                     _ptr(out), recs, cnts, tcap, _stream(stream)), "nrc_frame_packed")

    def frame_scatter_packed(self, scene: "DeviceScene", eval_records, eval_count, targets: ScatterTargets,
                             train_counts: Sequence, eval_capacity=None, stream=None):
        """nrc_frame_scatter_packed: the reference's frame on its record formats."""
        ecap = eval_records.shape[0] if eval_capacity is None else eval_capacity
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        check(lib().nrc_frame_scatter_packed(self.h, ctypes.byref(scene.s), _ptr(eval_records), _ptr(eval_count),
                                             ecap, ctypes.byref(targets), cnts, _stream(stream)),
              "nrc_frame_scatter_packed")

    def train(self, records, count, capacity=None, write_use=False, stream=None):
        cap = records.shape[0] if capacity is None else capacity
        check(lib().nrc_train(self.h, _ptr(records), _ptr(count), cap, int(write_use), _stream(stream)), "nrc_train")

    def gradient(self, records, count, grad, capacity=None, stream=None):
        cap = records.shape[0] if capacity is None else capacity
        check(lib().nrc_gradient(self.h, _ptr(records), _ptr(count), cap, _ptr(grad), _stream(stream)),
              "nrc_gradient")

    def optimize(self, grad_sum, count, write_use=True, stream=None):
        """nrc_optimize: the prepare + optimizer passes on a given gradient sum."""
        check(lib().nrc_optimize(self.h, _ptr(grad_sum), _ptr(count), int(write_use), _stream(stream)), "nrc_optimize")

    def train_batches(self, records: Sequence, counts: Sequence, capacity=None, write_use_last=True, stream=None):
        cap = records[0].shape[0] if capacity is None else capacity
        nb = len(records)
        recs = (ctypes.c_void_p * nb)(*[_ptr(r) for r in records])
        cnts = (ctypes.c_void_p * nb)(*[_ptr(c) for c in counts])
        check(lib().nrc_train_batches(self.h, recs, cnts, cap, nb, int(write_use_last), _stream(stream)),
              "nrc_train_batches")

    def frame(self, eval_inputs, eval_count, out, train_records: Sequence, train_counts: Sequence,
              eval_capacity=None, train_capacity=None, stream=None):
        ecap = eval_inputs.shape[0] if eval_capacity is None else eval_capacity
        tcap = train_records[0].shape[0] if train_capacity is None else train_capacity
        recs = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(r) for r in train_records])
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        check(lib().nrc_frame(self.h, _ptr(eval_inputs), _ptr(eval_count), ecap, _ptr(out), recs, cnts, tcap,
                              _stream(stream)), "nrc_frame")

    def frame_overlapped(self, eval_inputs, eval_count, out, train_records: Sequence, train_counts: Sequence,
                         plan=None, query_event=None, eval_capacity=None, train_capacity=None, stream=None):
        """nrc_frame_overlapped; plan = (query_ctas, train_ctas) or None (the tuned / default split);
        query_event: a torch.cuda.Event recorded when the query results are complete."""
        ecap = eval_inputs.shape[0] if eval_capacity is None else eval_capacity
        tcap = train_records[0].shape[0] if train_capacity is None else train_capacity
        recs = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(r) for r in train_records])
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        pl = ctypes.byref(FramePlan(*plan)) if plan is not None else None
        ev = None
        if query_event is not None:
            if query_event.cuda_event == 0:  # torch creates the CUDA event at its first record
                query_event.record(stream)
            ev = query_event.cuda_event
        check(lib().nrc_frame_overlapped(self.h, _ptr(eval_inputs), _ptr(eval_count), ecap, _ptr(out), recs, cnts,
                                         tcap, pl, ev, _stream(stream)), "nrc_frame_overlapped")

    def autotune_frame(self, eval_inputs, eval_count, out, train_records: Sequence, train_counts: Sequence):
        """nrc_autotune_frame: returns ((query_ctas, train_ctas), ms per frame)."""
        recs = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(r) for r in train_records])
        cnts = (ctypes.c_void_p * TRAIN_BATCH_COUNT)(*[_ptr(c) for c in train_counts])
        best = FramePlan()
        ms = ctypes.c_float()
        check(lib().nrc_autotune_frame(self.h, _ptr(eval_inputs), _ptr(eval_count), eval_inputs.shape[0], _ptr(out),
                                       recs, cnts, train_records[0].shape[0], ctypes.byref(best), ctypes.byref(ms)),
              "nrc_autotune_frame")
        return (best.query_ctas, best.train_ctas), ms.value

    # -------------------------------------------------------------- state --
    def get_weights(self, which=WEIGHTS_TRAIN) -> np.ndarray:
        w = np.empty(P, np.uint16)
        check(lib().nrc_get_weights(self.h, which, w.ctypes.data_as(ctypes.c_void_p)), "nrc_get_weights")
        return w

    def set_weights(self, w16: np.ndarray) -> None:
        w = np.ascontiguousarray(w16, np.uint16)
        assert w.size == P
        check(lib().nrc_set_weights(self.h, w.ctypes.data_as(ctypes.c_void_p)), "nrc_set_weights")

    def get_optimizer(self):
        st = OptState()
        ent = np.empty((P, 4), np.float32)
        check(lib().nrc_get_optimizer(self.h, ctypes.byref(st), ent.ctypes.data_as(ctypes.c_void_p)),
              "nrc_get_optimizer")
        return (st.t, st.beta1_t, st.beta2_t, st.alpha_t, st.alpha_t_1), ent

    def set_optimizer(self, state=None, entries: Optional[np.ndarray] = None) -> None:
        st = OptState(*state) if state is not None else None
        ent = np.ascontiguousarray(entries, np.float32) if entries is not None else None
        check(lib().nrc_set_optimizer(self.h, ctypes.byref(st) if st is not None else None,
                                      ent.ctypes.data_as(ctypes.c_void_p) if ent is not None else None),
              "nrc_set_optimizer")

    def reset(self, seed: int) -> None:
        check(lib().nrc_reset(self.h, seed), "nrc_reset")

    def get_loss(self):
        s, n = ctypes.c_double(), ctypes.c_uint64()
        check(lib().nrc_get_loss(self.h, ctypes.byref(s), ctypes.byref(n)), "nrc_get_loss")
        return s.value, n.value

    def error(self) -> int:
        return lib().nrc_get_error(self.h)

    def infer_fp8(self, inputs, count, out, capacity=None, stream=None):
        cap = inputs.shape[0] if capacity is None else capacity
        check(lib().nrc_infer_fp8(self.h, _ptr(inputs), _ptr(count), cap, _ptr(out), _stream(stream)),
              "nrc_infer_fp8")

    def fp8_refresh(self, stream=None):
        check(lib().nrc_fp8_refresh(self.h, _stream(stream)), "nrc_fp8_refresh")

    def get_fp8(self):
        """(w8 (P,) uint8 E4M3 bytes, scales dict)."""
        w8 = np.empty(P, np.uint8)
        sc = np.empty(25, np.float32)
        check(lib().nrc_get_fp8(self.h, w8.ctypes.data_as(ctypes.c_void_p), sc.ctypes.data_as(ctypes.c_void_p)),
              "nrc_get_fp8")
        return w8, {"scale_w": sc[0:6], "scale_x": sc[6:12], "c": sc[12:18], "inv_sx0": sc[18], "inv_w": sc[19:25]}

    def save_checkpoint(self) -> bytes:
        n = lib().nrc_checkpoint_bytes()
        buf = ctypes.create_string_buffer(n)
        check(lib().nrc_save_checkpoint(self.h, buf, n), "nrc_save_checkpoint")
        return buf.raw

    def load_checkpoint(self, blob: bytes) -> None:
        buf = ctypes.create_string_buffer(blob, len(blob))
        check(lib().nrc_load_checkpoint(self.h, buf, len(blob)), "nrc_load_checkpoint")

    def device_buffers(self):
        w, u, e, s = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().nrc_get_device_buffers(self.h, ctypes.byref(w), ctypes.byref(u), ctypes.byref(e), ctypes.byref(s)),
              "nrc_get_device_buffers")
        return w.value, u.value, e.value, s.value


# ------------------------------------------------------------ batched caches --
def query_job(cache: "Cache", inputs, count, out, capacity=None, weight_set=WEIGHTS_USE) -> QueryJob:
    """The job holds references to its tensors, so their device memory stays
    allocated (and distinct) for as long as the job object lives."""
    j = QueryJob(cache.h, _ptr(inputs), _ptr(count), inputs.shape[0] if capacity is None else capacity,
                 _ptr(out), weight_set)
    j._keep = (cache, inputs, count, out)
    return j


def train_job(cache: "Cache", records: Sequence, counts: Sequence, capacity=None, write_use_last=True) -> TrainJob:
    j = TrainJob()
    j.ctx = cache.h
    for b, (r, c) in enumerate(zip(records, counts)):
        j.records[b] = _ptr(r)
        j.d_counts[b] = _ptr(c)
    j.capacity = records[0].shape[0] if capacity is None else capacity
    j.nbatches = len(records)
    j.write_use_last = int(write_use_last)
    j._keep = (cache, list(records), list(counts))  # see query_job
    return j


def _ctas(ctas):
    if ctas is None:
        return None
    a = (ctypes.c_uint32 * len(ctas))(*ctas)
    return ctypes.cast(a, ctypes.c_void_p), a


def infer_many(jobs: Sequence[QueryJob], ctas=None, stream=None) -> None:
    """nrc_infer_many: every job's queries, one launch per 32 caches."""
    arr = (QueryJob * len(jobs))(*jobs)
    c = _ctas(ctas)
    check(lib().nrc_infer_many(arr, len(jobs), c[0] if c else None, _stream(stream)), "nrc_infer_many")


def train_many(jobs: Sequence[TrainJob], ctas=None, stream=None) -> None:
    """nrc_train_many: every job's chained training steps, one launch per 32 caches."""
    arr = (TrainJob * len(jobs))(*jobs)
    c = _ctas(ctas)
    check(lib().nrc_train_many(arr, len(jobs), c[0] if c else None, _stream(stream)), "nrc_train_many")


def autotune_many(qjobs: Sequence[QueryJob], tjobs: Sequence[TrainJob]):
    """nrc_autotune_many: (query CTA split, training CTA split, query ms, training ms)."""
    nq, nt = len(qjobs), len(tjobs)
    qa = (QueryJob * max(1, nq))(*qjobs)
    ta = (TrainJob * max(1, nt))(*tjobs)
    qc = np.zeros(max(1, nq), np.uint32)
    tc = np.zeros(max(1, nt), np.uint32)
    qms, tms = ctypes.c_float(0.0), ctypes.c_float(0.0)
    check(lib().nrc_autotune_many(qa, nq, ta, nt, qc.ctypes.data_as(ctypes.c_void_p),
                                  tc.ctypes.data_as(ctypes.c_void_p), ctypes.byref(qms), ctypes.byref(tms)),
          "nrc_autotune_many")
    return [int(x) for x in qc[:nq]], [int(x) for x in tc[:nt]], qms.value, tms.value


def plan_query_ctas(jobs: Sequence[QueryJob]) -> list:
    arr = (QueryJob * len(jobs))(*jobs)
    out = (ctypes.c_uint32 * len(jobs))()
    check(lib().nrc_plan_query_ctas(arr, len(jobs), ctypes.cast(out, ctypes.c_void_p)), "nrc_plan_query_ctas")
    return list(out)


def plan_train_ctas(jobs: Sequence[TrainJob]) -> list:
    arr = (TrainJob * len(jobs))(*jobs)
    out = (ctypes.c_uint32 * len(jobs))()
    check(lib().nrc_plan_train_ctas(arr, len(jobs), ctypes.cast(out, ctypes.c_void_p)), "nrc_plan_train_ctas")
    return list(out)


# ------------------------------------------------------------------ serving --
class SessionCache(Cache):
    """A view of a server session's cache (state reads only; the server owns it)."""

    def __init__(self, handle):
        self.h = handle

    def close(self) -> None:
        self.h = None


class _DeviceArray:
    """Exposes raw device memory through __cuda_array_interface__ (for torch.as_tensor)."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, shape, dtype):
    """A torch tensor viewing `ptr` (no copy); the memory must outlive the view."""
    import torch

    typestr = {torch.float32: "<f4", torch.int32: "<i4", torch.uint32: "<u4"}[dtype]
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")


class Server:
    """nrc_server: device-resident sessions whose frame requests are batched
    continuously, by a worker thread inside libnrc.so or (device_loop=True) by
    a loop that runs on the GPU."""

    def __init__(self, hbm_budget_bytes: int, max_batch_sessions: int = 32, max_inflight_batches: int = 2,
                 device_loop: bool = False):
        cfg = ServerConfig(hbm_budget_bytes, max_batch_sessions, max_inflight_batches, 1 if device_loop else 0)
        h = ctypes.c_void_p()
        check(lib().nrc_server_create(ctypes.byref(cfg), ctypes.byref(h)), "nrc_server_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            check(lib().nrc_server_destroy(self.h), "nrc_server_destroy")
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def open_session(self, max_queries: int, train_records: int, frame_slots: int = 2, train_ctas: int = 0,
                     **cfg) -> int:
        d = SessionDesc(default_config(**cfg), max_queries, train_records, frame_slots, train_ctas)
        sid = ctypes.c_uint32()
        check(lib().nrc_server_open_session(self.h, ctypes.byref(d), ctypes.byref(sid)), "nrc_server_open_session")
        return sid.value

    def close_session(self, sid: int) -> None:
        check(lib().nrc_server_close_session(self.h, sid), "nrc_server_close_session")

    def frame_buffers(self, sid: int, slot: int) -> FrameBuffers:
        f = FrameBuffers()
        check(lib().nrc_server_frame_buffers(self.h, sid, slot, ctypes.byref(f)), "nrc_server_frame_buffers")
        return f

    def frame_views(self, sid: int, slot: int, max_queries: int, train_records: int) -> dict:
        """Torch views of a frame slot: queries (Q, 14), query_count (1,), out (Q, 3),
        train [4 x (R, 20)], train_count [4 x (1,)]."""
        import torch

        f = self.frame_buffers(sid, slot)
        return {"queries": device_view(f.queries, (max_queries, IN_FLOATS), torch.float32),
                "query_count": device_view(f.query_count, (1,), torch.int32),
                "out": device_view(f.out_rgb, (max_queries, 3), torch.float32),
                "train": [device_view(f.train[b], (train_records, TRAIN_FLOATS), torch.float32)
                          for b in range(TRAIN_BATCH_COUNT)],
                "train_count": [device_view(f.train_count[b], (1,), torch.int32) for b in range(TRAIN_BATCH_COUNT)]}

    def cache(self, sid: int) -> SessionCache:
        c = ctypes.c_void_p()
        check(lib().nrc_server_session_cache(self.h, sid, ctypes.byref(c)), "nrc_server_session_cache")
        return SessionCache(c)

    def submit(self, sid: int, slot: int, ready_event=None) -> int:
        t = ctypes.c_uint64()
        ev = ready_event.cuda_event if ready_event is not None else None
        check(lib().nrc_server_submit(self.h, sid, slot, ev, ctypes.byref(t)), "nrc_server_submit")
        return t.value

    def wait(self, ticket: int, timeout_ms: float = -1.0) -> float:
        lat = ctypes.c_double()
        check(lib().nrc_server_wait(self.h, ticket, timeout_ms, ctypes.byref(lat)), "nrc_server_wait")
        return lat.value

    def stats(self, reset: bool = False) -> dict:
        st = ServerStats()
        check(lib().nrc_server_get_stats(self.h, ctypes.byref(st), int(reset)), "nrc_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}


def loss_gradient(pred, target, count, rows, loss_scale=1.0, precision=0, capacity=None, stream=None) -> None:
    """nrc_loss_gradient: the relative-L2 gradient row words (n x 2 uint32) of n (prediction, target) pairs."""
    cap = pred.shape[0] if capacity is None else capacity
    check(lib().nrc_loss_gradient(_ptr(pred), _ptr(target), _ptr(count), cap, float(loss_scale), int(precision),
                                  _ptr(rows), _stream(stream)), "nrc_loss_gradient")


def screen(color, accumulate=None, accumulate_count=0, out_rgba8=None, out_rgba=None, stream=None) -> None:
    """nrc_screen on (H, W, 4) float32 CUDA tensors; out_rgba8 is (H, W, 4) uint8."""
    h, w = color.shape[0], color.shape[1]
    check(lib().nrc_screen(_ptr(color), _ptr(accumulate), w, h, int(accumulate is not None), accumulate_count,
                           _ptr(out_rgba8), _ptr(out_rgba), _stream(stream)), "nrc_screen")


# ------------------------------------------------------------ scene unpack --
class DeviceScene:
    """A scene (the dict of numpy arrays that synthetic.scene makes) uploaded to
    the GPU, with its nrc_scene description."""

    def __init__(self, sc: dict):
        import torch

        def up(a):
            return torch.from_numpy(np.ascontiguousarray(a)).cuda()

        self.keep = {k: up(v) for k, v in sc.items() if k not in ("textures", "instance_ranges")}
        self.ranges = up(sc["instance_ranges"].astype(np.uint32).view(np.int32)) if "instance_ranges" in sc else None
        self.tex = [up(t) for t in sc["textures"]]
        table = np.zeros((max(1, len(self.tex)), 2), np.uint64)
        for i, t in enumerate(self.tex):
            table[i, 0] = t.data_ptr()
            table[i, 1] = np.uint64(t.shape[1]) | (np.uint64(t.shape[0]) << np.uint64(32))
        self.table = up(table.view(np.int64))
        k = self.keep
        self.s = SceneStruct(k["vertices"].data_ptr(), k["vertex_indices"].data_ptr(), k["texcoords"].data_ptr(),
                             k["texcoord_indices"].data_ptr(), k["materials"].data_ptr(), k["material_ids"].data_ptr(),
                             k["transforms"].data_ptr(), self.table.data_ptr(), k["vertices"].shape[0],
                             k["texcoords"].shape[0], k["materials"].shape[0], k["vertex_indices"].shape[0],
                             k["transforms"].shape[0], len(self.tex), None)
        self.tables = None

    def prepare(self, stream=None) -> "DeviceScene":
        """nrc_scene_prepare: build the gather tables and use them from now on."""
        self.release()
        h = ctypes.c_void_p()
        check(lib().nrc_scene_prepare(ctypes.byref(self.s), _stream(stream), ctypes.byref(h)), "nrc_scene_prepare")
        self.tables = h
        self.s.tables = h.value
        return self

    def unprepared(self) -> "DeviceScene":
        """A view of the same buffers without the tables (shares them; keep self alive)."""
        v = DeviceScene.__new__(DeviceScene)
        v.keep, v.ranges, v.tex, v.table, v.tables = self.keep, self.ranges, self.tex, self.table, None
        v.s = SceneStruct.from_buffer_copy(self.s)
        v.s.tables = None
        return v

    def release(self) -> None:
        """nrc_scene_tables_destroy of the tables made by prepare()."""
        if getattr(self, "tables", None) is not None:
            self.s.tables = None
            check(lib().nrc_scene_tables_destroy(self.tables), "nrc_scene_tables_destroy")
            self.tables = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def unpack_eval(scene: DeviceScene, records, count, out_inputs, out_dst=None, capacity=None, stream=None) -> None:
    """nrc_unpack_eval: records (n, 5) uint32/int32 CUDA tensor -> out_inputs (n, 14) float32, out_dst (n,)."""
    cap = records.shape[0] if capacity is None else capacity
    check(lib().nrc_unpack_eval(ctypes.byref(scene.s), _ptr(records), _ptr(count), cap, _ptr(out_inputs),
                                _ptr(out_dst), _stream(stream)), "nrc_unpack_eval")


def unpack_train(scene: DeviceScene, records, count, out_records, capacity=None, stream=None) -> None:
    """nrc_unpack_train: records (n, 10) 32-bit words -> out_records (n, 20) float32."""
    cap = records.shape[0] if capacity is None else capacity
    check(lib().nrc_unpack_train(ctypes.byref(scene.s), _ptr(records), _ptr(count), cap, _ptr(out_records),
                                 _stream(stream)), "nrc_unpack_train")


# ------------------------------------------------------------- path tracer --
class Bvh:
    """nrc_bvh over a DeviceScene's instance ranges (built on the GPU)."""

    def __init__(self, scene: "DeviceScene"):
        h = ctypes.c_void_p()
        check(lib().nrc_bvh_build(ctypes.byref(scene.s), _ptr(scene.ranges), ctypes.byref(h)), "nrc_bvh_build")
        self.h = h

    def info(self):
        t, n = ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().nrc_bvh_info(self.h, ctypes.byref(t), ctypes.byref(n)), "nrc_bvh_info")
        return t.value, n.value

    def close(self):
        if getattr(self, "h", None):
            lib().nrc_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TraceBuffers:
    """Device outputs of nrc_path_trace for a width x height frame."""

    def __init__(self, width: int, height: int, eval_capacity=None):
        import torch

        self.eval_capacity = width * height + 65536 if eval_capacity is None else eval_capacity
        self.eval = torch.zeros((self.eval_capacity, 5), dtype=torch.int32, device="cuda")
        self.eval_count = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.train = [torch.zeros((TRAIN_BATCH_SIZE, 10), dtype=torch.int32, device="cuda")
                      for _ in range(TRAIN_BATCH_COUNT)]
        self.train_counts = [torch.zeros(1, dtype=torch.int32, device="cuda") for _ in range(TRAIN_BATCH_COUNT)]
        self.bias_factor_r = torch.zeros((height, width, 4), dtype=torch.float32, device="cuda")
        self.factor_gb = torch.zeros((height, width, 2), dtype=torch.float32, device="cuda")

    def reset(self):
        self.eval_count.zero_()
        for c in self.train_counts:
            c.zero_()

    def targets(self) -> TraceTargets:
        t = TraceTargets()
        t.eval_records = _ptr(self.eval)
        t.eval_count = _ptr(self.eval_count)
        t.eval_capacity = self.eval_capacity
        for b in range(TRAIN_BATCH_COUNT):
            t.train_records[b] = _ptr(self.train[b])
            t.train_counts[b] = _ptr(self.train_counts[b])
        t.bias_factor_r = _ptr(self.bias_factor_r)
        t.factor_gb = _ptr(self.factor_gb)
        return t


def path_trace(scene: "DeviceScene", bvh: Bvh, params: TraceParams, buffers: TraceBuffers, stream=None) -> None:
    """nrc_path_trace (the caller zeroes the counters: TraceBuffers.reset)."""
    t = buffers.targets()
    check(lib().nrc_path_trace(ctypes.byref(scene.s), bvh.h, ctypes.byref(params), ctypes.byref(t), _stream(stream)),
          "nrc_path_trace")
