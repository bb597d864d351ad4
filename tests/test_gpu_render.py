"""The whole renderer frame of the reference on the GPU
(src/rg/NRCRenderGraph.cpp: path tracer pass, cache query with the
destination epilogue, four chained training passes, screen pass), composed of
this library's calls: nrc_path_trace -> nrc_unpack_eval / nrc_unpack_train ->
nrc_frame_scatter -> nrc_screen, over several frames with the accumulation
image. Checks the hand-offs: the query consumes exactly the records the tracer
emitted (device counts), screen pixels that received a cache query differ from
the tracer's bias by factor * prediction, the train counts are clamped to the
batch size, the cache trains (its loss falls), and the screen output is
finite UNORM8."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def test_renderer_frames(cuda):
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    w, h = 160, 96
    sc = S.terrain_scene(S.rng_for(3), n=96)
    ds = nrc.DeviceScene(sc)
    bvh = nrc.Bvh(ds)
    buf = nrc.TraceBuffers(w, h)
    P = nrc.TraceParams()
    P.origin[:] = (0.0, 0.3, -1.9)
    P.look[:] = (0.0, -0.25, 1.0)
    P.side[:] = (0.8, 0.0, 0.0)
    P.up[:] = (0.0, 0.8 * h / w, 0.0)
    P.width, P.height, P.left_method, P.right_method, P.train_probability = w, h, 1, 1, 0.25
    cap = buf.eval_capacity
    inputs = torch.zeros((cap, 14), dtype=torch.float32, device="cuda")
    dst = torch.zeros(cap, dtype=torch.int32, device="cuda")
    train_u = [torch.zeros((16384, 20), dtype=torch.float32, device="cuda") for _ in range(4)]
    acc = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    out8 = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    losses = []
    with Cache(seed=4, track_loss=1, learning_rate=2e-3) as c:
        for f in range(6):
            P.seed = 1000 + f
            buf.reset()
            nrc.path_trace(ds, bvh, P, buf)
            trace_img = host(buf.bias_factor_r).copy()
            nrc.unpack_eval(ds, buf.eval, buf.eval_count, inputs, dst, capacity=cap)
            for b in range(4):
                nrc.unpack_train(ds, buf.train[b], buf.train_counts[b], train_u[b], capacity=16384)
            targets = nrc.scatter_targets(buf.bias_factor_r, buf.factor_gb, train_u)
            c.frame_scatter(inputs, dst, buf.eval_count, targets, buf.train_counts, eval_capacity=cap)
            nrc.screen(buf.bias_factor_r, acc, f, out8)
            n_eval = int(host(buf.eval_count)[0])
            counts = [int(host(x)[0]) for x in buf.train_counts]
            assert 0 < n_eval <= cap and all(0 < k <= 16384 for k in counts)  # clamped by the training
            img = host(buf.bias_factor_r)
            ev = host(buf.eval)[:n_eval].view(np.uint32)
            scr = ev[(ev[:, 0] & 1) == 0, 0] >> 1
            ys, xs = scr >> 15, scr & 0x7FFF
            gb = host(buf.factor_gb)
            # a queried pixel moved by factor * prediction (prediction >= 0, so not down)
            moved = img[ys, xs, :3] - trace_img[ys, xs, :3]
            fac = np.stack([trace_img[ys, xs, 3], gb[ys, xs, 0], gb[ys, xs, 1]], -1)
            assert np.all(moved >= -1e-6 * (1 + np.abs(trace_img[ys, xs, :3])))
            assert np.all((fac > 0) | (np.abs(moved) <= 1e-6))
            s, k = c.get_loss()
            losses.append(s / max(k, 1))
            assert c.error() == 0
    o8 = host(out8)
    assert np.all(o8[..., 3] == 255) and o8[..., :3].max() > 0
    assert np.all(np.isfinite(host(acc)))
    assert losses[-1] < losses[0], losses
    bvh.close()


def test_traced_records_unpack_equal_through_scene_tables(cuda):
    """The path tracer's own eval and train records unpack to the same inputs
    bit for bit over the scene's gather tables as over its buffers."""
    import torch

    from vknrc_gb300 import nrc, synthetic as S

    w, h = 128, 80
    sc = S.terrain_scene(S.rng_for(5), n=64)
    ds = nrc.DeviceScene(sc)
    dt = nrc.DeviceScene(sc).prepare()
    bvh = nrc.Bvh(ds)
    buf = nrc.TraceBuffers(w, h)
    P = nrc.TraceParams()
    P.origin[:] = (0.0, 0.3, -1.9)
    P.look[:] = (0.0, -0.25, 1.0)
    P.side[:] = (0.8, 0.0, 0.0)
    P.up[:] = (0.0, 0.8 * h / w, 0.0)
    P.width, P.height, P.left_method, P.right_method, P.train_probability = w, h, 1, 1, 0.25
    P.seed = 2024
    buf.reset()
    nrc.path_trace(ds, bvh, P, buf)
    cap = buf.eval_capacity
    outs = []
    for scene in (ds, dt):
        inputs = torch.full((cap, 14), -1.0, dtype=torch.float32, device="cuda")
        dst = torch.zeros(cap, dtype=torch.int32, device="cuda")
        nrc.unpack_eval(scene, buf.eval, buf.eval_count, inputs, dst, capacity=cap)
        tr = [torch.full((16384, 20), -1.0, dtype=torch.float32, device="cuda") for _ in range(4)]
        for b in range(4):
            nrc.unpack_train(scene, buf.train[b], buf.train_counts[b], tr[b], capacity=16384)
        outs.append((host(inputs), host(dst), [host(t) for t in tr]))
    n = int(host(buf.eval_count)[0])
    assert n > 0
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    for a, b in zip(outs[0][2], outs[1][2]):
        np.testing.assert_array_equal(a, b)
    assert np.all(outs[1][0][n:] == -1.0)  # nothing past the count
    bvh.close()
