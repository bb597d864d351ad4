"""Query destination epilogue (nrc_inference.comp:50-73) fused into the query
kernel: screen pixels and self-training target completion, against the
oracle's scatter applied to the kernel's own predictions (bit-exact: the
epilogue is index work plus one fused multiply-add per channel), and the frame
with destinations against its two halves."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu

W, H = 96, 40
TRAIN_CAP = 512


def _frame(seed, train_counts=(500, 300, 512, 0), extra_invalid=37):
    from vknrc_gb300 import synthetic as S

    rng = S.rng_for(seed)
    dst = S.frame_destinations(rng, W, H, train_counts)
    # edge words: invalid, pixels outside the image, ranges running past the
    # capacity, an empty range (l > r), a batch without a buffer below
    edge = np.concatenate([
        np.full(extra_invalid, S.DST_INVALID, np.uint32),
        S.dst_screen(np.array([W, W + 5, 3]), np.array([0, H - 1, H])),
        # (on the batch with the fewest records, so it overlaps no other run)
        S.dst_train(np.array([int(np.argmin(train_counts))]), np.array([TRAIN_CAP - 2]),
                    np.array([TRAIN_CAP + 40])),
        S.dst_train(np.array([2]), np.array([9]), np.array([4])),
    ])
    dst = np.concatenate([dst, edge])
    dst = dst[rng.permutation(dst.size)]
    n = dst.size
    inputs = S.inputs(rng, n)
    img = rng.random((H, W, 4), dtype=np.float32)
    gb = rng.random((H, W, 2), dtype=np.float32)
    trains = [S.train_records(rng, TRAIN_CAP, target="lognormal", sigma=0.5) for _ in range(4)]
    for t in trains:
        t[:, 3:6] = rng.random((TRAIN_CAP, 3), dtype=np.float32)  # factors
    return inputs, dst, img, gb, trains


def test_infer_scatter_bit_exact(cuda, oracle):
    from vknrc_gb300 import Cache, nrc

    inputs, dst, img, gb, trains = _frame(21)
    n = dst.size
    with Cache(seed=5) as c:
        d_in = dev(inputs)
        pred = cuda.empty((n, 3), dtype=cuda.float32, device="cuda")
        c.infer(d_in, count(n), pred)
        d_img, d_gb = dev(img), dev(gb)
        d_tr = [dev(t) for t in trains]
        d_tr[3] = None  # batch 3 has no buffer: its words are skipped
        out = cuda.full((n, 3), -7.0, dtype=cuda.float32, device="cuda")
        targets = nrc.scatter_targets(d_img, d_gb, d_tr)
        c.infer_scatter(d_in, dev(dst.view(np.int32)), count(n), targets, out=out)
        assert c.error() == 0
        p = host(pred)
        got_img, got_tr = host(d_img), [host(t) if t is not None else None for t in d_tr]
        assert np.array_equal(host(out), p)
    want_img = img.copy()
    want_tr = [t.copy() for t in trains]
    want_tr[3] = None
    oracle.scatter(p, dst, want_img, gb, want_tr)
    assert np.array_equal(got_img, want_img)
    for b in range(3):
        assert np.array_equal(got_tr[b], want_tr[b]), b
    # something happened: every pixel was written (alpha 0), targets changed
    assert np.all(got_img[:, :, 3] == 0)
    assert not np.array_equal(got_tr[0][:, :3], trains[0][:, :3])


def test_infer_scatter_count_and_null_out(cuda, oracle):
    from vknrc_gb300 import Cache, nrc

    inputs, dst, img, gb, trains = _frame(22)
    n = dst.size
    m = n // 3  # only the first m queries count
    with Cache(seed=6) as c:
        d_in = dev(inputs)
        pred = cuda.empty((n, 3), dtype=cuda.float32, device="cuda")
        c.infer(d_in, count(n), pred)
        d_img, d_gb = dev(img), dev(gb)
        d_tr = [dev(t) for t in trains]
        c.infer_scatter(d_in, dev(dst.view(np.int32)), count(m), nrc.scatter_targets(d_img, d_gb, d_tr))
        got_img, got_tr = host(d_img), [host(t) for t in d_tr]
        p = host(pred)
    want_img, want_tr = img.copy(), [t.copy() for t in trains]
    oracle.scatter(p[:m], dst[:m], want_img, gb, want_tr)
    assert np.array_equal(got_img, want_img)
    for b in range(4):
        assert np.array_equal(got_tr[b], want_tr[b])


def test_scatter_argument_checks(cuda):
    from vknrc_gb300 import Cache, nrc

    with Cache(seed=7) as c:
        x = cuda.zeros((128, 14), dtype=cuda.float32, device="cuda")
        d = cuda.zeros(128, dtype=cuda.int32, device="cuda")
        img = cuda.zeros((4, 4, 4), dtype=cuda.float32, device="cuda")
        t = nrc.scatter_targets(img, None, [])
        with pytest.raises(nrc.NRCError) as e:
            c.infer_scatter(x, d, count(128), t)
        assert e.value.status == 1  # image without its factor_gb half
        big = nrc.ScatterTargets()
        big.width, big.height = 0x8001, 1
        with pytest.raises(nrc.NRCError):
            c.infer_scatter(x, d, count(128), big)


def test_frame_scatter_equals_its_halves(cuda):
    """nrc_frame_scatter = nrc_infer_scatter (screen + target completion) then
    four chained training steps on the completed records."""
    from vknrc_gb300 import Cache, nrc

    inputs, dst, img, gb, trains = _frame(23, train_counts=(512, 512, 400, 512))
    n = dst.size
    counts = [512, 512, 400, 512]
    res = []
    for split in (False, True):
        with Cache(seed=8) as c:
            d_img, d_gb = dev(img), dev(gb)
            d_tr = [dev(t) for t in trains]
            cnt = [count(k) for k in counts]
            targets = nrc.scatter_targets(d_img, d_gb, d_tr)
            if split:
                c.infer_scatter(dev(inputs), dev(dst.view(np.int32)), count(n), targets)
                c.train_batches(d_tr, cnt, write_use_last=True)
            else:
                c.frame_scatter(dev(inputs), dev(dst.view(np.int32)), count(n), targets, cnt)
            assert c.error() == 0
            res.append((host(d_img), [host(t) for t in d_tr], c.get_weights(0), c.get_weights(1),
                        c.get_optimizer()))
    a, b = res
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
    assert a[4][0] == b[4][0] and np.array_equal(a[4][1], b[4][1])
    assert a[4][0][0] == 4  # four optimizer steps ran
