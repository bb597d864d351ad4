"""Seeded synthetic path-vertex records with the distributions of the benchmark
configurations (no dataset exists for this path: the reference's records come
from its path tracer, shader/src/path_tracer.comp:159-166, 302-371).

Inputs follow nrc_input / UnpackedNRCInput (shader/src/NRCRecord.glsl:40-45):
position U[0,1]^3; scattered direction and normal uniform on the sphere, then
sphere-encoded (NRCSphEncode), the direction quantised to unorm16 as the path
tracer stores it (path_tracer.comp:164); roughness U(0,1); diffuse and specular
albedo U(0,1)^3.

Training records follow nrc_train_record: bias = target radiance, factor = 1.
Targets: lognormal(0, 1.5) per channel, or a fixed smooth field of the inputs
times lognormal noise (for loss curves that can be compared across runs).
Per-frame redraws key a counter-based generator (Philox) by (seed, frame, stream).
"""
from __future__ import annotations

import numpy as np

IN_FLOATS = 14
TRAIN_FLOATS = 20


def rng_for(seed: int, frame: int = 0, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=[seed & 0xFFFFFFFFFFFFFFFF, (frame << 16) | stream]))


def sphere(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.standard_normal((n, 3))
    v /= np.maximum(np.linalg.norm(v, axis=1, keepdims=True), 1e-30)
    return v.astype(np.float32)


def sph_encode(d: np.ndarray) -> np.ndarray:
    """NRCSphEncode (NRCRecord.glsl:47-49) in float64, rounded to float32."""
    d = d.astype(np.float64)
    u = np.where((d[:, 0] == 0) & (d[:, 1] == 0), 0.5, 0.5 + np.arctan2(d[:, 1], d[:, 0]) / (2 * np.pi))
    v = np.arccos(np.clip(d[:, 2], -1, 1)) / np.pi
    return np.stack([u, v], 1).astype(np.float32)


def inputs(rng: np.random.Generator, n: int) -> np.ndarray:
    """(n, 14) float32 nrc_input records."""
    r = np.empty((n, IN_FLOATS), np.float32)
    r[:, 0:3] = rng.random((n, 3), dtype=np.float32)
    r[:, 3:5] = np.round(sph_encode(sphere(rng, n)) * 65535.0) / 65535.0
    r[:, 5:7] = sph_encode(sphere(rng, n))
    r[:, 7] = rng.random(n, dtype=np.float32)
    r[:, 8:14] = rng.random((n, 6), dtype=np.float32)
    return r


def smooth_field(x: np.ndarray) -> np.ndarray:
    """A fixed smooth positive radiance field of the inputs, (n, 3) float32."""
    p, d, nrm, rough = x[:, 0:3], x[:, 3:5], x[:, 5:7], x[:, 7]
    diff, spec = x[:, 8:11], x[:, 11:14]
    shade = 0.6 + 0.4 * np.sin(2 * np.pi * (p[:, 0] + 0.3 * p[:, 2])) * np.cos(np.pi * nrm[:, 1])
    gloss = np.exp(-4.0 * rough) * (0.5 + 0.5 * np.cos(2 * np.pi * (p[:, 1] + d[:, 0])))
    return (diff * shade[:, None] + spec * gloss[:, None] + 0.05).astype(np.float32)


def train_records(rng: np.random.Generator, n: int, target: str = "lognormal", sigma: float = 1.5) -> np.ndarray:
    """(n, 20) float32 nrc_train_record rows: bias[3], factor[3], input[14]."""
    x = inputs(rng, n)
    if target == "lognormal":
        t = rng.lognormal(0.0, sigma, (n, 3)).astype(np.float32)
    elif target == "field":
        t = smooth_field(x) * rng.lognormal(0.0, sigma, (n, 3)).astype(np.float32)
    else:
        raise ValueError(target)
    rec = np.empty((n, TRAIN_FLOATS), np.float32)
    rec[:, 0:3] = t
    rec[:, 3:6] = 1.0
    rec[:, 6:20] = x
    return rec


def dst_screen(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """EncodeNRCEvalDstScreen (NRCRecord.glsl:20): (x | y << 15) << 1."""
    return ((x.astype(np.uint32) | (y.astype(np.uint32) << 15)) << 1).astype(np.uint32)


def dst_train(b: np.ndarray, l: np.ndarray, r: np.ndarray) -> np.ndarray:
    """EncodeNRCEvalDstTrain (NRCRecord.glsl:21-23): (b | l << 2 | r << 16) << 1 | 1."""
    b, l, r = (np.asarray(v, np.uint32) for v in (b, l, r))
    return (((b | (l << 2) | (r << 16)) << 1) | 1).astype(np.uint32)


DST_INVALID = np.uint32(0xFFFFFFFF)


def frame_destinations(rng: np.random.Generator, width: int, height: int, train_counts, max_run: int = 8):
    """Destination words of one frame's queries, as the path tracer emits them:
    one per screen pixel, and for every train batch b its records 0..count-1
    split into consecutive runs [l, r] of 1..max_run records (one query per run,
    completing that run's targets). Returned in random order."""
    ys, xs = np.divmod(np.arange(width * height, dtype=np.uint32), np.uint32(width))
    words = [dst_screen(xs, ys)]
    for b, n in enumerate(train_counts):
        l = 0
        ls, rs = [], []
        while l < n:
            run = int(rng.integers(1, max_run + 1))
            r = min(n, l + run) - 1
            ls.append(l)
            rs.append(r)
            l = r + 1
        if ls:
            words.append(dst_train(np.full(len(ls), b), np.array(ls), np.array(rs)))
    d = np.concatenate(words)
    return d[rng.permutation(d.size)]


# ------------------------------------------------------------------ scenes --
def scene(rng: np.random.Generator, vertices: int = 300, primitives: int = 200, instances: int = 5,
          materials: int = 12, texture_sizes=((5, 3), (64, 32), (1, 1), (17, 9))) -> dict:
    """A seeded synthetic scene in the layout of the reference's scene buffers
    (shader/src/Scene.glsl:8-48): vertices, per-primitive vertex / texcoord
    index triples, texcoords (spanning several texture periods, negative ones
    included, to exercise REPEAT addressing), std430 materials (some textured,
    some constant, a few with texture ids past the table), per-primitive
    material ids, mat3x4 instance transforms and rgba8 sRGB textures."""
    sc = {}
    sc["vertices"] = rng.uniform(-1, 1, (vertices, 3)).astype(np.float32)
    # three distinct vertices per primitive (a degenerate triangle has no normal)
    sc["vertex_indices"] = rng.random((primitives, vertices)).argsort(axis=1)[:, :3].astype(np.uint32)
    n_tc = vertices // 2
    sc["texcoords"] = rng.uniform(-2, 3, (n_tc, 2)).astype(np.float32)
    sc["texcoord_indices"] = rng.integers(0, n_tc, (primitives, 3)).astype(np.uint32)
    mats = np.zeros((materials, 16), np.float32)
    ids = mats.view(np.uint32)
    mats[:, 0:3] = rng.uniform(0, 1, (materials, 3))
    mats[:, 4:7] = rng.uniform(0, 1, (materials, 3))
    mats[:, 8:11] = rng.uniform(0, 1, (materials, 3))
    mats[:, 12] = rng.uniform(0, 1, materials)  # metallic
    mats[:, 13] = rng.uniform(0, 1, materials)  # roughness
    mats[:, 14] = 1.5                          # ior
    nt = len(texture_sizes)
    choice = rng.integers(-1, nt + 1, (materials, 3))  # -1: constant; nt: past the table
    for col, word in ((0, 3), (1, 7), (2, 11)):
        ids[:, word] = np.where(choice[:, col] < 0, 0xFFFFFFFF, choice[:, col]).astype(np.uint32)
    sc["materials"] = mats
    sc["material_ids"] = rng.integers(0, materials, primitives).astype(np.uint32)
    t = np.zeros((instances, 3, 4), np.float32)
    for i in range(instances):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        m = q * rng.uniform(0.5, 2.0)
        t[i, :, :3] = m
        t[i, :, 3] = rng.uniform(-3, 3, 3)
    sc["transforms"] = t
    sc["textures"] = [rng.integers(0, 256, (h, w, 4), dtype=np.uint8) for (w, h) in texture_sizes]
    # each instance owns a contiguous range of primitives (the reference's instance
    # custom index + BLAS primitive index); the tracer renders these ranges
    cuts = np.linspace(0, primitives, instances + 1).astype(np.int64)
    sc["instance_ranges"] = np.stack([cuts[:-1], cuts[1:] - cuts[:-1]], 1).astype(np.uint32)
    return sc


def packed_inputs(rng: np.random.Generator, sc: dict, n: int, bad_fraction: float = 0.0) -> np.ndarray:
    """(n, 4) uint32 PackedNRCInput words (NRCRecord.glsl:6-9): primitive id,
    flip bit | instance id, barycentrics and sphere-encoded direction as unorm16
    pairs. A fraction of records carries out-of-range ids."""
    p = sc["vertex_indices"].shape[0]
    inst = sc["transforms"].shape[0]
    out = np.empty((n, 4), np.uint32)
    out[:, 0] = rng.integers(0, p, n)
    out[:, 1] = rng.integers(0, inst, n).astype(np.uint32) | (rng.integers(0, 2, n).astype(np.uint32) << 31)
    b = rng.uniform(0, 1, (n, 2))
    over = b.sum(1) > 1
    b[over] = 1 - b[over]
    bq = np.round(b * 65535).astype(np.uint32)
    out[:, 2] = bq[:, 0] | (bq[:, 1] << 16)
    d = np.round(sph_encode(sphere(rng, n)) * 65535).astype(np.uint32)
    out[:, 3] = d[:, 0] | (d[:, 1] << 16)
    if bad_fraction > 0:
        bad = rng.random(n) < bad_fraction
        half = rng.random(n) < 0.5
        out[bad & half, 0] = p + rng.integers(0, 10, int(np.sum(bad & half)))
        out[bad & ~half, 1] = (inst + rng.integers(0, 10, int(np.sum(bad & ~half)))).astype(np.uint32)
    return out


def eval_records(rng: np.random.Generator, sc: dict, n: int, bad_fraction: float = 0.0) -> np.ndarray:
    """(n, 5) uint32 NRCEvalRecord words: dst, then the packed input."""
    r = np.empty((n, 5), np.uint32)
    r[:, 0] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    r[:, 1:] = packed_inputs(rng, sc, n, bad_fraction)
    return r


def packed_train_records(rng: np.random.Generator, sc: dict, n: int) -> np.ndarray:
    """(n, 10) 32-bit words of NRCTrainRecord: bias rgb, factor rgb (float32), packed input."""
    r = np.empty((n, 10), np.uint32)
    f = r.view(np.float32)
    f[:, 0:3] = rng.lognormal(0, 1, (n, 3))
    f[:, 3:6] = rng.uniform(0, 1, (n, 3))
    r[:, 6:] = packed_inputs(rng, sc, n)
    return r


def terrain_scene(rng: np.random.Generator, n: int = 256, texture: int = 64) -> dict:
    """A seeded closed room for the path tracer and the renderer frame: a
    height-field floor (an n x n vertex grid over [-2, 2]^2 with smooth random
    heights, 2 (n-1)^2 triangles) inside four walls and a ceiling (the room is
    sized for the tracer's 4.0 secondary-ray range, so few paths escape),
    an emissive ceiling panel, two instances (the room and a raised, rotated,
    scaled copy of part of the floor), four materials of which two are
    textured."""
    g = np.linspace(-2.0, 2.0, n, dtype=np.float32)
    X, Z = np.meshgrid(g, g)
    H = np.zeros_like(X)
    for k in range(4):
        f = rng.uniform(0.6, 3.0) * (k + 1)
        H += rng.uniform(0.05, 0.2) / (k + 1) * np.sin(f * X + rng.uniform(0, 6)) * np.cos(f * Z + rng.uniform(0, 6))
    floor_v = np.stack([X, H - 0.6, Z], -1).reshape(-1, 3)
    i = np.arange(n - 1)
    a = (i[:, None] * n + i[None, :]).ravel()
    quads = np.stack([a, a + 1, a + n, a + n + 1], 1)
    floor_t = np.concatenate([quads[:, [0, 2, 1]], quads[:, [1, 2, 3]]], 0)
    # walls and ceiling: a box x, z in [-2.05, 2.05], y in [-0.8, 1.0]; two panels of the
    # ceiling are emitters
    lo, hi, y0, y1 = -2.05, 2.05, -0.8, 1.0
    box = np.array([[lo, y0, lo], [hi, y0, lo], [hi, y1, lo], [lo, y1, lo],
                    [lo, y0, hi], [hi, y0, hi], [hi, y1, hi], [lo, y1, hi],
                    [-0.6, y1 - 0.01, -0.6], [0.6, y1 - 0.01, -0.6], [0.6, y1 - 0.01, 0.6], [-0.6, y1 - 0.01, 0.6]],
                   np.float32)
    box_t = np.array([[0, 1, 2], [0, 2, 3], [4, 6, 5], [4, 7, 6], [0, 3, 7], [0, 7, 4], [1, 5, 6], [1, 6, 2],
                      [3, 2, 6], [3, 6, 7], [8, 10, 9], [8, 11, 10]]) + floor_v.shape[0]
    sc = {}
    sc["vertices"] = np.concatenate([floor_v, box], 0).astype(np.float32)
    tri = np.concatenate([floor_t, box_t], 0).astype(np.uint32)
    sc["vertex_indices"] = tri
    sc["texcoords"] = (sc["vertices"][:, [0, 2]] * 1.5).astype(np.float32)
    sc["texcoord_indices"] = tri.copy()
    mats = np.zeros((4, 16), np.float32)
    ids = mats.view(np.uint32)
    mats[:, 0:3] = rng.uniform(0.2, 0.9, (4, 3))
    mats[:, 4:7] = rng.uniform(0.0, 0.5, (4, 3))
    mats[:, 13] = [0.3, 0.7, 0.1, 0.5]  # roughness
    mats[:, 14] = 1.5
    mats[3, 8:11] = [6.0, 5.5, 5.0]     # the emitter
    ids[:, 3] = [0, 0xFFFFFFFF, 1, 0xFFFFFFFF]
    ids[:, 7] = [0xFFFFFFFF, 1, 0xFFFFFFFF, 0xFFFFFFFF]
    ids[:, 11] = 0xFFFFFFFF
    sc["materials"] = mats
    p = tri.shape[0]
    mid = rng.integers(0, 3, p).astype(np.uint32)
    mid[floor_t.shape[0]:] = 1          # walls and ceiling
    mid[-2:] = 3                        # the ceiling panel emits
    sc["material_ids"] = mid
    t = np.zeros((2, 3, 4), np.float32)
    t[0, :, :3] = np.eye(3)
    c, s_ = np.cos(0.6), np.sin(0.6)
    t[1, :, :3] = np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]]) * 0.3
    t[1, :, 3] = [0.6, 0.1, 0.4]
    sc["transforms"] = t
    sc["textures"] = [rng.integers(0, 256, (texture, texture, 4), dtype=np.uint8),
                      rng.integers(0, 256, (texture // 2, texture, 4), dtype=np.uint8)]
    sc["instance_ranges"] = np.array([[0, p], [0, floor_t.shape[0] // 8]], np.uint32)
    return sc


def train_records_device(gen, n: int, target: str = "field", sigma: float = 1.0, device: str = "cuda"):
    """The distributions of train_records, drawn on the device with a seeded
    torch.Generator (for runs of many frames, where host generation would
    dominate): an (n, 20) float32 tensor of nrc_train_record rows. The stream
    differs from the host generator's; the distributions are the same."""
    import torch

    def unif(*shape):
        return torch.rand(*shape, generator=gen, device=device, dtype=torch.float32)

    def sph(d):
        d = d.double()
        d = d / d.norm(dim=1, keepdim=True).clamp_min(1e-30)
        u = 0.5 + torch.atan2(d[:, 1], d[:, 0]) / (2 * np.pi)
        u = torch.where((d[:, 0] == 0) & (d[:, 1] == 0), torch.full_like(u, 0.5), u)
        v = torch.arccos(d[:, 2].clamp(-1, 1)) / np.pi
        return torch.stack([u, v], 1).float()

    rec = torch.empty((n, TRAIN_FLOATS), dtype=torch.float32, device=device)
    x = rec[:, 6:20]
    x[:, 0:3] = unif(n, 3)
    x[:, 3:5] = torch.round(sph(torch.randn(n, 3, generator=gen, device=device)) * 65535.0) / 65535.0
    x[:, 5:7] = sph(torch.randn(n, 3, generator=gen, device=device))
    x[:, 7] = unif(n)
    x[:, 8:14] = unif(n, 6)
    noise = torch.exp(sigma * torch.randn(n, 3, generator=gen, device=device))
    if target == "lognormal":
        rec[:, 0:3] = noise
    elif target == "field":
        p, d, nrm, rough = x[:, 0:3], x[:, 3:5], x[:, 5:7], x[:, 7]
        shade = 0.6 + 0.4 * torch.sin(2 * np.pi * (p[:, 0] + 0.3 * p[:, 2])) * torch.cos(np.pi * nrm[:, 1])
        gloss = torch.exp(-4.0 * rough) * (0.5 + 0.5 * torch.cos(2 * np.pi * (p[:, 1] + d[:, 0])))
        rec[:, 0:3] = (x[:, 8:11] * shade[:, None] + x[:, 11:14] * gloss[:, None] + 0.05) * noise
    else:
        raise ValueError(target)
    rec[:, 3:6] = 1.0
    return rec
