"""The query and the frame on the reference's record formats: packed eval
records (nrc_eval_record, 20 B) and packed train records
(nrc_packed_train_record, 40 B) over a scene, unpacked (UnpackNRCInput,
shader/src/NRCRecord.glsl:97-125, as nrc_inference.comp:33-36 does) into the
context's workspaces by the unpack kernel, then queried and trained.

Each packed call is checked bit for bit against the same work done in two
steps on the GPU (nrc_unpack_eval / nrc_unpack_train, then the unpacked-record
call), and against the
oracle: oracle_unpack + the oracle's forward within the query tolerance, and
the destination epilogue (oracle_scatter) bit for bit on the GPU's own
predictions."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def _scene(seed=40):
    from vknrc_gb300 import nrc, synthetic as S

    sc = S.scene(S.rng_for(seed))
    return sc, nrc.DeviceScene(sc)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 70001])
def test_infer_packed_equals_unpack_then_infer(cuda, oracle, n):
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    sc, ds = _scene()
    ev = S.eval_records(S.rng_for(41, n), sc, n, bad_fraction=0.02)
    rec = dev(ev.view(np.int32))
    with Cache(seed=42) as c:
        a = torch.full((n + 5, 3), float("nan"), dtype=torch.float32, device="cuda")
        c.infer_packed(ds, rec, count(n), a, capacity=n)
        inputs = torch.zeros((n, 14), dtype=torch.float32, device="cuda")
        nrc.unpack_eval(ds, rec, count(n), inputs)
        b = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        c.infer(inputs, count(n), b)
        got, want = host(a), host(b)
        w16 = c.get_weights(0)
        assert c.error() == 0
    np.testing.assert_array_equal(got[:n], want)
    assert np.isnan(got[n:]).all()  # nothing past the count
    ref = np.maximum(oracle.forward_f32(w16, oracle.encode(oracle.unpack(sc, ev, 1)), nthreads=8), 0)
    assert np.abs(got[:n] - ref).max() <= 1e-2 * max(1.0, float(np.abs(ref).max()))


def test_infer_scatter_packed_vs_unpacked_and_oracle(cuda, oracle):
    """Screen pixels and self-training targets in packed train records."""
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    sc, ds = _scene(43)
    W, H, ntrain = 96, 64, 600
    # every pixel once, and every train record in exactly one run (destinations
    # of one call do not repeat, as the path tracer emits them)
    dst = S.frame_destinations(S.rng_for(46), W, H, [ntrain] * 4, max_run=4)
    n = dst.size
    ev = S.eval_records(S.rng_for(44), sc, n)
    ev[:, 0] = dst
    img0 = S.rng_for(48).uniform(0, 1, (H, W, 4)).astype(np.float32)
    gb = S.rng_for(49).uniform(0, 1, (H, W, 2)).astype(np.float32)
    ptr = [S.packed_train_records(S.rng_for(50, b), sc, ntrain) for b in range(4)]
    gb_d = dev(gb)  # held: the kernels read it after the call returns
    with Cache(seed=51) as c:
        # packed: records, train batches in their 40-byte form
        img_a = dev(img0)
        tr_a = [dev(t.view(np.int32)) for t in ptr]
        out_a = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        c.infer_scatter_packed(ds, dev(ev.view(np.int32)), count(n), nrc.scatter_targets(img_a, gb_d, tr_a),
                               out=out_a)
        # unpacked: the same records and train batches unpacked first
        inputs = torch.zeros((n, 14), dtype=torch.float32, device="cuda")
        dst = torch.zeros(n, dtype=torch.int32, device="cuda")
        nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(n), inputs, dst)
        tr_b = []
        for t in ptr:
            u = torch.zeros((ntrain, 20), dtype=torch.float32, device="cuda")
            nrc.unpack_train(ds, dev(t.view(np.int32)), count(ntrain), u)
            tr_b.append(u)
        img_b = dev(img0)
        out_b = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        c.infer_scatter(inputs, dst, count(n), nrc.scatter_targets(img_b, gb_d, tr_b), out=out_b)
        got_img, pred = host(img_a), host(out_a)
        got_tr = [host(t).view(np.float32) for t in tr_a]
        np.testing.assert_array_equal(pred, host(out_b))
        np.testing.assert_array_equal(got_img, host(img_b))
        for a, b in zip(got_tr, tr_b):
            np.testing.assert_array_equal(a[:, 0:6], host(b)[:, 0:6])
        assert c.error() == 0
    # the oracle's epilogue on the kernel's own predictions
    ref_img = img0.copy()
    ref_tr = []
    for t in ptr:
        u = np.zeros((ntrain, 20), np.float32)  # the oracle's unpacked layout: bias, factor first
        u[:, 0:6] = t.view(np.float32)[:, 0:6]
        ref_tr.append(u)
    oracle.scatter(pred, ev[:, 0], ref_img, gb, ref_tr)
    np.testing.assert_array_equal(got_img, ref_img)
    for a, u in zip(got_tr, ref_tr):
        np.testing.assert_array_equal(a[:, 0:6], u[:, 0:6])
    assert any((a[:, 0:3] != t.view(np.float32)[:, 0:3]).any() for a, t in zip(got_tr, ptr))  # targets completed


def _packed_frame_inputs(sc, ds, q, r, seed):
    from vknrc_gb300 import synthetic as S

    ev = S.eval_records(S.rng_for(seed), sc, q)
    tr = [S.packed_train_records(S.rng_for(seed + 1, b), sc, r) for b in range(4)]
    return ev, tr


def test_frame_packed_equals_unpacked_frame(cuda):
    import torch

    from vknrc_gb300 import Cache, nrc

    sc, ds = _scene(52)
    q, r = 40000, 3000
    ev, tr = _packed_frame_inputs(sc, ds, q, r, 53)
    kw = dict(seed=54, learning_rate=1e-3, beta2=0.99)
    with Cache(**kw) as a, Cache(**kw) as b:
        out_a = torch.empty((q, 3), dtype=torch.float32, device="cuda")
        cnt_a = [count(r) for _ in range(4)]
        for _ in range(2):
            a.frame_packed(ds, dev(ev.view(np.int32)), count(q), out_a, [dev(t.view(np.int32)) for t in tr], cnt_a)
        inputs = torch.zeros((q, 14), dtype=torch.float32, device="cuda")
        nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(q), inputs)
        tr_u = []
        for t in tr:
            u = torch.zeros((r, 20), dtype=torch.float32, device="cuda")
            nrc.unpack_train(ds, dev(t.view(np.int32)), count(r), u)
            tr_u.append(u)
        out_b = torch.empty((q, 3), dtype=torch.float32, device="cuda")
        cnt_b = [count(r) for _ in range(4)]
        for _ in range(2):
            b.frame_overlapped(inputs, count(q), out_b, tr_u, cnt_b)
        np.testing.assert_array_equal(host(out_a), host(out_b))
        np.testing.assert_array_equal(a.get_weights(0), b.get_weights(0))
        np.testing.assert_array_equal(a.get_optimizer()[1], b.get_optimizer()[1])
        assert a.get_optimizer()[0][0] == 8
        assert a.error() == 0 and b.error() == 0


def test_frame_scatter_packed_equals_unpacked_frame(cuda):
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    sc, ds = _scene(55)
    W, H, r = 128, 96, 2048
    dst = S.frame_destinations(S.rng_for(58), W, H, [r] * 4, max_run=8)
    n = dst.size
    ev = S.eval_records(S.rng_for(56), sc, n)
    ev[:, 0] = dst
    tr = [S.packed_train_records(S.rng_for(59, b), sc, r) for b in range(4)]
    img0 = S.rng_for(60).uniform(0, 1, (H, W, 4)).astype(np.float32)
    gb = S.rng_for(61).uniform(0, 1, (H, W, 2)).astype(np.float32)
    kw = dict(seed=62, learning_rate=1e-3, beta2=0.99)
    gb_d = dev(gb)  # held: the kernels read it after the call returns
    cnt_a, cnt_b = [count(r) for _ in range(4)], [count(r) for _ in range(4)]
    with Cache(**kw) as a, Cache(**kw) as b:
        img_a = dev(img0)
        tr_a = [dev(t.view(np.int32)) for t in tr]
        ev_d, n_d = dev(ev.view(np.int32)), count(n)
        a.frame_scatter_packed(ds, ev_d, n_d, nrc.scatter_targets(img_a, gb_d, tr_a), cnt_a)
        inputs = torch.zeros((n, 14), dtype=torch.float32, device="cuda")
        dst = torch.zeros(n, dtype=torch.int32, device="cuda")
        nrc.unpack_eval(ds, dev(ev.view(np.int32)), count(n), inputs, dst)
        tr_b = []
        for t in tr:
            u = torch.zeros((r, 20), dtype=torch.float32, device="cuda")
            nrc.unpack_train(ds, dev(t.view(np.int32)), count(r), u)
            tr_b.append(u)
        img_b = dev(img0)
        b.frame_scatter(inputs, dst, n_d, nrc.scatter_targets(img_b, gb_d, tr_b), cnt_b)
        np.testing.assert_array_equal(host(img_a), host(img_b))
        for ta, tb in zip(tr_a, tr_b):
            np.testing.assert_array_equal(host(ta).view(np.float32)[:, 0:6], host(tb)[:, 0:6])
        np.testing.assert_array_equal(a.get_weights(0), b.get_weights(0))
        np.testing.assert_array_equal(a.get_optimizer()[1], b.get_optimizer()[1])
        assert a.error() == 0 and b.error() == 0


def test_frame_packed_scene_tables_equal_buffers(cuda):
    """The packed frame over a prepared scene (nrc_scene_prepare) equals the
    same frame over the scene buffers: outputs, weights and optimizer entries."""
    import torch

    from vknrc_gb300 import Cache, nrc

    sc, plain = _scene(63)
    prepared = nrc.DeviceScene(sc).prepare()
    q, r = 30000, 2500
    ev, tr = _packed_frame_inputs(sc, plain, q, r, 64)
    kw = dict(seed=65, learning_rate=1e-3, beta2=0.99)
    res = []
    for ds in (plain, prepared):
        with Cache(**kw) as c:
            out = torch.empty((q, 3), dtype=torch.float32, device="cuda")
            cnt = [count(r) for _ in range(4)]
            for _ in range(2):
                c.frame_packed(ds, dev(ev.view(np.int32)), count(q), out, [dev(t.view(np.int32)) for t in tr], cnt)
            res.append((host(out), c.get_weights(0), c.get_optimizer()[1]))
            assert c.error() == 0
    for a, b in zip(res[0], res[1]):
        np.testing.assert_array_equal(a, b)
