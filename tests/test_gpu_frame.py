"""The frame schedule (src/rg/NRCRenderGraph.cpp:46-80): one query pass with
use_weights, then four chained training steps, the last writing use_weights.
Chained in one launch it must equal the same steps called one by one, and a
frame captured in a CUDA graph must replay to the same result."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def _batches(seed, n=16384):
    from vknrc_gb300 import synthetic as S

    return [dev(S.train_records(S.rng_for(seed, b), n, target="field", sigma=0.5)) for b in range(4)]


def test_chained_batches_equal_separate_steps(cuda):
    from vknrc_gb300 import Cache

    recs = _batches(60)
    with Cache(seed=61) as a, Cache(seed=61) as b:
        a.train_batches(recs, [count(16384) for _ in range(4)], write_use_last=True)
        for k in range(4):
            b.train(recs[k], count(16384), write_use=(k == 3))
        sa, ea = a.get_optimizer()
        sb, eb = b.get_optimizer()
        assert sa == sb and sa[0] == 4
        assert np.array_equal(ea, eb)
        assert np.array_equal(a.get_weights(0), b.get_weights(0))
        assert np.array_equal(a.get_weights(1), b.get_weights(1))
        assert a.error() == 0 and b.error() == 0


def test_frame_equals_query_then_chained_training(cuda):
    import torch

    from vknrc_gb300 import Cache, synthetic as S

    q = S.inputs(S.rng_for(62), 50000)
    recs = _batches(63, 4000)
    with Cache(seed=64) as a, Cache(seed=64) as b:
        oa = torch.empty((q.shape[0], 3), dtype=torch.float32, device="cuda")
        ob = torch.empty_like(oa)
        a.frame(dev(q), count(q.shape[0]), oa, recs, [count(4000) for _ in range(4)])
        b.infer(dev(q), count(q.shape[0]), ob)
        b.train_batches(recs, [count(4000) for _ in range(4)])
        assert np.array_equal(host(oa), host(ob))
        assert np.array_equal(a.get_optimizer()[1], b.get_optimizer()[1])


def test_frame_graph_capture_replays(cuda):
    import torch

    from vknrc_gb300 import Cache, synthetic as S

    q = dev(S.inputs(S.rng_for(65), 30000))
    recs = _batches(66, 8192)
    with Cache(seed=67) as a, Cache(seed=67) as b:
        cnt_q = count(30000)
        cnts_a = [count(8192) for _ in range(4)]
        out_a = torch.empty((30000, 3), dtype=torch.float32, device="cuda")
        # eager reference: two frames
        for _ in range(2):
            a.frame(q, cnt_q, out_a, recs, cnts_a)
        ref_out, ref_ent = host(out_a), a.get_optimizer()[1]
        # graph: capture one frame of context b, replay twice
        cnts_b = [count(8192) for _ in range(4)]
        out_b = torch.empty_like(out_a)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                b.frame(q, cnt_q, out_b, recs, cnts_b, stream=s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        # capture did not execute the frame
        assert b.get_optimizer()[0][0] == 0
        for _ in range(2):
            g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(host(out_b), ref_out)
        assert np.array_equal(b.get_optimizer()[1], ref_ent)
        assert b.error() == 0
