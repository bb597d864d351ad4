"""The overlapped frame (nrc_frame_overlapped): the query of a frame and its
four training steps at the same time (the training on its CTAs, the query's
tiles handed out by a counter to CTAs beside it and, as it finishes, on its
SMs), the training's new rendering weights staged and copied in once the
training has completed and every query CTA has loaded the previous ones, and
the autotuner that picks the split.

The query reads the same use_weights as in the sequential frame, so its
answers are the same bit for bit; the training with a group of train_ctas
CTAs equals nrc_train_many with that group size bit for bit (the same
fixed-order sums). The split chosen by the autotuner is valid, the tuning runs
on a scratch copy (the cache's step count does not move), and an overlapped
frame replays from a CUDA graph to the eager result."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def _frame_data(seed, q=60000, r=16384):
    from vknrc_gb300 import synthetic as S

    return (dev(S.inputs(S.rng_for(seed), q)),
            [dev(S.train_records(S.rng_for(seed, b + 1), r, target="field", sigma=0.5)) for b in range(4)])


@pytest.mark.parametrize("plan", [(112, 40), (140, 12), (152, 0)])
def test_overlapped_frame_equals_query_then_grouped_training(cuda, plan):
    import torch

    from vknrc_gb300 import Cache, nrc

    frames = [_frame_data(120 + k) for k in range(3)]
    with Cache(seed=121) as a, Cache(seed=121) as b:
        for k, (q, recs) in enumerate(frames):
            n = q.shape[0]
            oa = torch.full((n, 3), -1.0, dtype=torch.float32, device="cuda")
            ob = torch.full((n, 3), -1.0, dtype=torch.float32, device="cuda")
            ev = torch.cuda.Event()
            a.frame_overlapped(q, count(n), oa, recs, [count(16384) for _ in range(4)], plan=plan, query_event=ev)
            ev.synchronize()
            qa = oa.cpu().numpy()  # complete once the query event has fired (no device-wide sync)
            b.infer(q, count(n), ob)
            if plan[1] == 0:
                b.train_batches(recs, [count(16384) for _ in range(4)])
            else:
                nrc.train_many([nrc.train_job(b, recs, [count(16384) for _ in range(4)])], ctas=[plan[1]])
            assert np.array_equal(qa, host(ob)), k
            assert np.array_equal(a.get_weights(0), b.get_weights(0)), k
        assert np.array_equal(a.get_optimizer()[1], b.get_optimizer()[1])
        assert a.get_optimizer()[0][0] == 12 and a.error() == 0


def test_autotune_picks_a_valid_split_on_a_scratch_copy(cuda):
    import torch

    from vknrc_gb300 import Cache, NRCError

    q, recs = _frame_data(130)
    n = q.shape[0]
    out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    cnts = [count(16384) for _ in range(4)]
    with Cache(seed=131) as c:
        w0 = c.get_weights(0)
        (qc, tc), ms = c.autotune_frame(q, count(n), out, recs, cnts)
        assert ms > 0 and (tc == 0 or (qc >= 1 and qc + tc <= 152))
        assert c.get_optimizer()[0][0] == 0 and np.array_equal(c.get_weights(0), w0)  # untouched
        c.frame_overlapped(q, count(n), out, recs, cnts)  # with the tuned plan
        assert c.get_optimizer()[0][0] == 4 and c.error() == 0
        with pytest.raises(NRCError):
            c.frame_overlapped(q, count(n), out, recs, cnts, plan=(150, 10))  # more CTAs than SMs


def test_overlapped_frame_graph_replays(cuda):
    import torch

    from vknrc_gb300 import Cache

    q, recs = _frame_data(140, q=30000, r=8192)
    n = q.shape[0]
    with Cache(seed=141) as a, Cache(seed=141) as b:
        oa = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        ca = [count(8192) for _ in range(4)]
        for _ in range(3):
            a.frame_overlapped(q, count(n), oa, recs, ca, plan=(120, 32))
        ob = torch.empty_like(oa)
        cb = [count(8192) for _ in range(4)]
        cq = count(n)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                b.frame_overlapped(q, cq, ob, recs, cb, plan=(120, 32), stream=s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        assert b.get_optimizer()[0][0] == 0
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(host(oa), host(ob))
        assert np.array_equal(a.get_optimizer()[1], b.get_optimizer()[1])
        assert np.array_equal(a.get_weights(0), b.get_weights(0))
        assert b.error() == 0


@pytest.mark.parametrize("queries", ["none", "zero"])
def test_overlapped_frame_without_queries_publishes_the_weights(cuda, queries):
    """No query launched (capacity 0: the training's last CTA copies the staged
    rendering weights) or a query with no records (the query CTA that loads its
    weights last copies them after its wait for the training): use_weights
    match the grouped training's either way."""
    import torch

    from vknrc_gb300 import Cache, nrc
    from vknrc_gb300 import synthetic as S

    _, recs = _frame_data(150, q=1000)
    with Cache(seed=151) as a, Cache(seed=151) as b:
        for k in range(2):
            if queries == "none":
                q = torch.empty((0, 14), dtype=torch.float32, device="cuda")
                out = torch.empty((0, 3), dtype=torch.float32, device="cuda")
            else:
                q = dev(S.inputs(S.rng_for(152, k), 1000))
                out = torch.full((1000, 3), -1.0, dtype=torch.float32, device="cuda")
            a.frame_overlapped(q, count(0), out, recs, [count(16384) for _ in range(4)], plan=(120, 32))
            nrc.train_many([nrc.train_job(b, recs, [count(16384) for _ in range(4)])], ctas=[32])
            assert np.array_equal(a.get_weights(0), b.get_weights(0)), k
            assert np.array_equal(a.get_weights(1), b.get_weights(1)), k
            if queries == "zero":
                assert np.all(host(out) == -1.0)  # nothing answered
        assert a.error() == 0
