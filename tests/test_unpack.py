"""Scene unpack (UnpackNRCInput, shader/src/NRCRecord.glsl:97-125, over
shader/src/Scene.glsl:50-71 and the reference's bilinear / REPEAT / sRGB
texture sampler).

CPU: the oracle against an independent float64 restatement (geometry,
barycentric interpolation, texture lookups at texel centres and with wrap-around).
GPU: nrc_unpack_eval / nrc_unpack_train against the oracle on a seeded
synthetic scene: every field bit for bit except the sphere-encoded normal
(atan2 / acos, within 4e-7 as the stand-alone sphere encoding), out-of-range
records unpacked to zeros, destination words and train targets passed through;
then the unpacked records through the query with destinations, against the
same query on the oracle's unpacked records."""
import numpy as np
import pytest

from gpu_util import count, dev, host


def _f64_unpack(sc, w):
    """float64 restatement of the geometry part (position, dirs, normal, roughness)."""
    prim, iw = w[:, 0], w[:, 1]
    inst = iw & 0x7FFFFFFF
    flip = (iw >> 31) != 0
    V = sc["vertices"].astype(np.float64)
    T = sc["transforms"].astype(np.float64)
    vi = sc["vertex_indices"][prim]
    p = [np.einsum("nij,nj->ni", T[inst][:, :, :3], V[vi[:, k]]) + T[inst][:, :, 3] for k in range(3)]
    n = np.cross(p[1] - p[0], p[2] - p[0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n[flip] *= -1
    b1 = (w[:, 2] & 0xFFFF) / 65535.0
    b2 = (w[:, 2] >> 16) / 65535.0
    b0 = 1 - b1 - b2
    pos = p[0] * b0[:, None] + p[1] * b1[:, None] + p[2] * b2[:, None]
    sph = np.stack([0.5 + np.arctan2(n[:, 1], n[:, 0]) / (2 * np.pi), np.arccos(np.clip(n[:, 2], -1, 1)) / np.pi], 1)
    return pos, sph


def test_oracle_unpack_geometry_vs_float64(oracle):
    from vknrc_gb300 import synthetic as S

    sc = S.scene(S.rng_for(1))
    w = S.packed_inputs(S.rng_for(2), sc, 2000)
    u = oracle.unpack(sc, w)
    pos, sph = _f64_unpack(sc, w)
    assert np.allclose(u[:, 0:3], pos, atol=2e-5)
    assert np.allclose(u[:, 5:7], sph, atol=1e-5)
    assert np.array_equal(u[:, 3], (w[:, 3] & 0xFFFF).astype(np.float32) / np.float32(65535))
    rough = sc["materials"][sc["material_ids"][w[:, 0]], 13]
    assert np.array_equal(u[:, 7], rough)


def test_oracle_texture_sampling_texel_centres_and_wrap(oracle):
    """A one-triangle scene whose texcoords all sit at one point: at a texel
    centre the bilinear sample is that texel's sRGB-decoded value, one period
    away (REPEAT) it is the same, and between two texels it is their mean."""
    from vknrc_gb300 import synthetic as S

    sc = S.scene(S.rng_for(3), vertices=3, primitives=1, instances=1, materials=1, texture_sizes=((4, 2),))
    sc["vertex_indices"][:] = [0, 1, 2]
    ids = sc["materials"].view(np.uint32)
    ids[0, 3] = 0  # diffuse textured
    ids[0, 7] = 0xFFFFFFFF  # specular constant
    tex = sc["textures"][0].astype(np.float64) / 255.0
    lin = np.where(tex <= 0.04045, tex / 12.92, ((tex + 0.055) / 1.055) ** 2.4)
    w = S.packed_inputs(S.rng_for(4), sc, 1)
    for (tu, tv), want in [((2.5 / 4, 0.5 / 2), lin[0, 2]), ((2.5 / 4 + 3, 1.5 / 2 - 2), lin[1, 2]),
                           ((3.0 / 4, 0.5 / 2), 0.5 * (lin[0, 2] + lin[0, 3])),
                           ((0.0, 0.5 / 2), 0.5 * (lin[0, 3] + lin[0, 0]))]:
        sc["texcoords"] = np.tile(np.array([[tu, tv]], np.float32), (sc["texcoords"].shape[0], 1))
        u = oracle.unpack(sc, w)
        assert np.allclose(u[0, 8:11], want[:3], atol=2e-6), (tu, tv)
        assert np.array_equal(u[0, 11:14], sc["materials"][0, 4:7])


@pytest.mark.gpu
def test_gpu_unpack_eval_vs_oracle(cuda, oracle):
    import torch

    from vknrc_gb300 import nrc, synthetic as S

    sc = S.scene(S.rng_for(10))
    n = 20000
    ev = S.eval_records(S.rng_for(11), sc, n, bad_fraction=0.02)
    ref = oracle.unpack(sc, ev, 1)
    ds = nrc.DeviceScene(sc)
    out = torch.full((n + 7, 14), -1.0, dtype=torch.float32, device="cuda")
    dst = torch.zeros(n + 7, dtype=torch.int32, device="cuda")
    nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(n), out, dst)
    got = host(out)
    assert np.all(got[n:] == -1.0)  # nothing past the count
    exact = [0, 1, 2, 3, 4, 7, 8, 9, 10, 11, 12, 13]
    assert np.array_equal(got[:n, exact], ref[:, exact])
    assert np.max(np.abs(got[:n, 5:7] - ref[:, 5:7])) <= 4e-7
    assert np.array_equal(host(dst)[:n].view(np.uint32), ev[:, 0])
    bad = np.all(ref == 0, axis=1)
    assert bad.sum() > 0 and np.all(got[:n][bad] == 0)


@pytest.mark.gpu
def test_gpu_unpack_train_then_query_with_destinations(cuda, oracle):
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    sc = S.scene(S.rng_for(20))
    ds = nrc.DeviceScene(sc)
    r = 3000
    tr = S.packed_train_records(S.rng_for(21), sc, r)
    out = torch.zeros((r, 20), dtype=torch.float32, device="cuda")
    nrc.unpack_train(ds, dev(tr.view(np.int32)), count(r), out)
    got = host(out)
    ref = oracle.unpack(sc, tr, 6)
    assert np.array_equal(got[:, 0:6], tr[:, 0:6].view(np.float32))
    exact = [6 + k for k in (0, 1, 2, 3, 4, 7, 8, 9, 10, 11, 12, 13)]
    assert np.array_equal(got[:, exact], ref[:, [k - 6 for k in exact]])
    # unpacked eval records through the query with destinations (screen pixels only)
    n, W, H = 5000, 100, 50
    ev = S.eval_records(S.rng_for(22), sc, n)
    px = S.rng_for(23).permutation(W * H)[:n]
    ev[:, 0] = ((px % W) | ((px // W) << 15)).astype(np.uint32) << 1
    inputs = torch.zeros((n, 14), dtype=torch.float32, device="cuda")
    dst = torch.zeros(n, dtype=torch.int32, device="cuda")
    nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(n), inputs, dst)
    img0 = S.rng_for(24).uniform(0, 1, (H, W, 4)).astype(np.float32)
    gb = S.rng_for(25).uniform(0, 1, (H, W, 2)).astype(np.float32)
    with Cache(seed=26) as c:
        img = dev(img0)
        gb_d = dev(gb)  # held: the kernel reads it after the call returns
        c.infer_scatter(inputs, dst, count(n), nrc.scatter_targets(img, gb_d))
        got_img = host(img)
        pred_t = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        c.infer(inputs, count(n), pred_t)  # the kernel's own predictions, for the oracle's epilogue
        pred = host(pred_t)
        w16 = c.get_weights(0)
    ref_img = img0.copy()
    oracle.scatter(pred, ev[:, 0], ref_img, gb, [])
    assert np.array_equal(got_img, ref_img)
    ref_in = oracle.unpack(sc, ev, 1)  # the whole path from the oracle's unpacked records
    pred_o = np.maximum(oracle.forward_f32(w16, oracle.encode(ref_in)), 0)
    assert np.max(np.abs(pred_o - pred)) <= 1e-2 * max(1.0, float(np.abs(pred_o).max()))


def _corrupted_scene(seed):
    """A synthetic scene whose index buffers hold out-of-range entries (vertex,
    texcoord and material indices) and whose texture table has an empty
    texture, so every rejection of the unpack is met."""
    from vknrc_gb300 import synthetic as S

    rng = S.rng_for(seed)
    sc = S.scene(rng, texture_sizes=((5, 3), (64, 32), (0, 0), (17, 9)))
    p = sc["vertex_indices"].shape[0]
    sel = rng.choice(p, 15, replace=False)
    sc["vertex_indices"][sel[:5], 1] = sc["vertices"].shape[0] + 3
    sc["texcoord_indices"][sel[5:10], 2] = sc["texcoords"].shape[0]
    sc["material_ids"][sel[10:]] = sc["materials"].shape[0] + 1
    ids = sc["materials"].view(np.uint32)
    ids[0, 3], ids[1, 7] = 2, 2  # the empty texture, on one diffuse and one specular colour
    return sc


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 255, 256, 257, 20000])
def test_gpu_unpack_tables_equal_buffers_and_oracle(cuda, oracle, n):
    """nrc_scene_prepare's gather tables give the buffers' unpack bit for bit,
    records and index buffers with out-of-range entries included."""
    import torch

    from vknrc_gb300 import nrc, synthetic as S

    sc = _corrupted_scene(30)
    ev = S.eval_records(S.rng_for(31, n), sc, n, bad_fraction=0.05)
    tr = S.packed_train_records(S.rng_for(32, n), sc, n)
    plain = nrc.DeviceScene(sc)
    prepared = nrc.DeviceScene(sc).prepare()
    outs = []
    for ds in (plain, prepared):
        o = torch.full((n + 3, 14), -1.0, dtype=torch.float32, device="cuda")
        d = torch.zeros(n + 3, dtype=torch.int32, device="cuda")
        nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(n), o, d)
        t = torch.full((n + 3, 20), -1.0, dtype=torch.float32, device="cuda")
        nrc.unpack_train(ds, dev(tr.view(np.int32)), count(n), t)
        outs.append((host(o), host(d), host(t)))
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)
    got = outs[1][0]
    assert np.all(got[n:] == -1.0)
    ref = oracle.unpack(sc, ev, 1)
    exact = [0, 1, 2, 3, 4, 7, 8, 9, 10, 11, 12, 13]
    assert np.array_equal(got[:n, exact], ref[:, exact])
    assert np.max(np.abs(got[:n, 5:7] - ref[:, 5:7])) <= 4e-7
    ref_t = oracle.unpack(sc, tr, 6)
    assert np.array_equal(outs[1][2][:n, [6 + k for k in exact]], ref_t[:, exact])
    if n >= 20000:  # the rejections were met
        assert (np.all(ref == 0, axis=1)).sum() > 0.05 * n


@pytest.mark.gpu
def test_gpu_unpack_tables_of_another_scene_rejected(cuda):
    import torch

    from vknrc_gb300 import nrc, synthetic as S

    a = nrc.DeviceScene(S.scene(S.rng_for(33))).prepare()
    b = nrc.DeviceScene(S.scene(S.rng_for(34), primitives=150))
    b.s.tables = a.tables.value  # tables whose counts do not match this scene
    ev = S.eval_records(S.rng_for(35), S.scene(S.rng_for(34), primitives=150), 10)
    out = torch.zeros((10, 14), dtype=torch.float32, device="cuda")
    with pytest.raises(nrc.NRCError) as e:
        nrc.unpack_eval(b, dev(ev.view(np.int32)), count(10), out)
    assert e.value.status == 1  # NRC_ERROR_INVALID_ARGUMENT
    b.s.tables = None
