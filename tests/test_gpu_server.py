"""Serving loop (nrc_server_*): device-resident sessions, admission by a
device-memory budget, continuous batching of frame requests.

Each frame request runs the reference's frame schedule on one session
(src/rg/NRCRenderGraph.cpp:46-80): the query of its records with use_weights,
then four chained training steps, the last writing use_weights. A session's
results must be the same alone and in any mix of sessions: its query answers
are per-record computations and its training runs in a CTA group of a fixed
size, so the comparison is bit for bit, and it is also checked against the
same schedule driven through the batched-cache calls directly.

Every test runs on both forms of the loop: the host worker thread, and the
device-resident loop (a CUDA graph whose while node runs scheduler, batched
query, batched training and completion kernels on the GPU)."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu

GB = 1 << 30


def _frame(seed, frame, q, r):
    from vknrc_gb300 import synthetic as S

    queries = S.inputs(S.rng_for(seed, frame, 0), q)
    train = [S.train_records(S.rng_for(seed, frame, 1 + b), r, target="field", sigma=0.5) for b in range(4)]
    return queries, train


def _fill(views, queries, train):
    """Write one frame's records and counts into a slot (torch's current stream)."""
    import torch

    q = queries.shape[0]
    views["queries"][:q].copy_(torch.from_numpy(queries), non_blocking=False)
    views["query_count"].fill_(q)
    for b in range(4):
        views["train"][b][: train[b].shape[0]].copy_(torch.from_numpy(train[b]))
        views["train_count"][b].fill_(train[b].shape[0])
    ev = torch.cuda.Event()
    ev.record()
    return ev


def _run_session_frames(srv, sid, spec, frames, slots=2):
    """Submits `frames` frames of one session (slot k % slots), waiting only
    when a slot is reused. Returns per-frame outputs."""
    seed, q, r = spec
    pending, outs = {}, {}
    for k in range(frames):
        slot = k % slots
        if slot in pending:
            kk, t = pending.pop(slot)
            srv.wait(t, 60000)
            outs[kk] = host(srv.frame_views(sid, slot, q, r)["out"][:q]).copy()
        v = srv.frame_views(sid, slot, q, r)
        ev = _fill(v, *_frame(seed, k, q, r))
        pending[slot] = (k, srv.submit(sid, slot, ev))
    for slot, (kk, t) in pending.items():
        srv.wait(t, 60000)
        outs[kk] = host(srv.frame_views(sid, slot, q, r)["out"][:q]).copy()
    return [outs[k] for k in range(frames)]


SPECS = {"a": (11, 50000, 4096), "b": (12, 120000, 16384), "c": (13, 7000, 1000), "d": (14, 300000, 8192)}


@pytest.mark.parametrize("device_loop", [False, True])
def test_session_alone_equals_in_mix_and_direct_calls(cuda, device_loop):
    import threading

    from vknrc_gb300 import Cache, nrc

    frames = 3
    seed, q, r = SPECS["a"]
    with nrc.Server(8 * GB, device_loop=device_loop) as srv:
        sa = srv.open_session(q, r, seed=seed)
        alone = _run_session_frames(srv, sa, SPECS["a"], frames)
        c = srv.cache(sa)
        alone_w, alone_ent = c.get_weights(0), c.get_optimizer()[1]
    with nrc.Server(8 * GB, max_batch_sessions=4, device_loop=device_loop) as srv:
        ids = {k: srv.open_session(SPECS[k][1], SPECS[k][2], seed=SPECS[k][0]) for k in SPECS}
        results = {}
        threads = [threading.Thread(target=lambda k=k: results.__setitem__(
            k, _run_session_frames(srv, ids[k], SPECS[k], frames))) for k in SPECS]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        st = srv.stats()
        assert st["completed"] == st["submitted"] == frames * len(SPECS)
        c = srv.cache(ids["a"])
        for k in range(frames):
            assert np.array_equal(results["a"][k], alone[k]), k
        assert np.array_equal(c.get_weights(0), alone_w)
        assert np.array_equal(c.get_optimizer()[1], alone_ent)
        assert c.get_optimizer()[0][0] == 4 * frames
        assert c.error() == 0
    # the same schedule through the batched-cache calls, with the session's CTA group
    with Cache(seed=seed) as ref:
        g = max(1, min((r // 128 + 3) // 4, 152))
        for k in range(frames):
            queries, train = _frame(seed, k, q, r)
            out = dev(np.full((q, 3), -1, np.float32))
            nrc.infer_many([nrc.query_job(ref, dev(queries), count(q), out)])
            nrc.train_many([nrc.train_job(ref, [dev(t) for t in train], [count(r) for _ in range(4)])], ctas=[g])
            assert np.array_equal(host(out), alone[k]), k
        assert np.array_equal(ref.get_optimizer()[1], alone_ent)


@pytest.mark.parametrize("device_loop", [False, True])
def test_budget_admission_and_release(cuda, device_loop):
    from vknrc_gb300 import NRCError, nrc

    with nrc.Server(200 << 20, device_loop=device_loop) as srv:  # 200 MB
        ids = []
        with pytest.raises(NRCError) as e:
            for _ in range(64):
                ids.append(srv.open_session(100000, 4096, frame_slots=2))
        assert e.value.status == 5  # out of memory: the budget is full
        assert len(ids) >= 2
        used = srv.stats()["bytes_in_use"]
        assert used <= 200 << 20
        srv.close_session(ids.pop())
        assert srv.stats()["bytes_in_use"] < used
        ids.append(srv.open_session(100000, 4096, frame_slots=2))  # fits again
        with pytest.raises(NRCError):
            srv.submit(ids[0], 5)  # no such slot
        with pytest.raises(NRCError):
            srv.open_session(1000, 1000, frame_slots=0)


@pytest.mark.parametrize("device_loop", [False, True])
def test_requests_batch_and_complete_in_session_order(cuda, device_loop):
    """Many sessions submitting back to back: requests are batched (more than
    one session per launch on average), every request completes, and each
    session's step count equals its frames (its requests ran in order, one at
    a time)."""
    import torch

    from vknrc_gb300 import nrc

    n_sess, frames, q, r = 8, 4, 20000, 2048
    with nrc.Server(8 * GB, max_batch_sessions=8, max_inflight_batches=2, device_loop=device_loop) as srv:
        ids = [srv.open_session(q, r, frame_slots=frames, seed=900 + s) for s in range(n_sess)]
        for s in ids:
            for k in range(frames):
                _fill(srv.frame_views(s, k, q, r), *_frame(900 + s, k, q, r))
        torch.cuda.synchronize()
        tickets = [srv.submit(s, k) for k in range(frames) for s in ids]
        lat = [srv.wait(t, 60000) for t in tickets]
        assert all(x > 0 for x in lat)
        st = srv.stats()
        assert st["completed"] == n_sess * frames
        assert st["mean_batch_sessions"] > 1.0
        assert st["latency_p99_ms"] >= st["latency_p50_ms"] > 0
        for s in ids:
            c = srv.cache(s)
            assert c.get_optimizer()[0][0] == 4 * frames
            assert c.error() == 0


def test_device_loop_matches_host_worker_and_rejects_other_formats(cuda):
    """The same session frames through both loops give the same outputs and
    cache state bit for bit; the device loop takes fp16 caches only."""
    from vknrc_gb300 import NRCError, nrc

    frames = 3
    res = []
    for device_loop in (False, True):
        with nrc.Server(4 * GB, device_loop=device_loop) as srv:
            sid = srv.open_session(SPECS["c"][1], SPECS["c"][2], seed=SPECS["c"][0])
            outs = _run_session_frames(srv, sid, SPECS["c"], frames)
            c = srv.cache(sid)
            res.append((outs, c.get_weights(0), c.get_optimizer()[1]))
            if device_loop:
                with pytest.raises(NRCError) as e:
                    srv.open_session(1000, 1000, precision=1)
                assert e.value.status == 1
                st = srv.stats()
                assert st["batches"] >= frames and st["completed"] == frames
    for k in range(frames):
        assert np.array_equal(res[0][0][k], res[1][0][k]), k
    assert np.array_equal(res[0][1], res[1][1])
    assert np.array_equal(res[0][2], res[1][2])


@pytest.mark.parametrize("device_loop", [False, True])
def test_sessions_open_and_close_while_another_runs(cuda, device_loop):
    """Sessions opened and closed (their memory allocated and freed, which
    pauses the device loop) while another session's frames are in flight: the
    running session's results equal its results alone."""
    import threading

    from vknrc_gb300 import nrc

    frames = 4
    seed, q, r = SPECS["c"]
    with nrc.Server(4 * GB, device_loop=device_loop) as srv:
        sa = srv.open_session(q, r, seed=seed)
        alone = _run_session_frames(srv, sa, SPECS["c"], frames)
    with nrc.Server(4 * GB, device_loop=device_loop) as srv:
        sa = srv.open_session(q, r, seed=seed)
        out = {}
        t = threading.Thread(target=lambda: out.__setitem__("a", _run_session_frames(srv, sa, SPECS["c"], frames)))
        t.start()
        for k in range(3):
            sb = srv.open_session(20000, 2048, seed=70 + k)
            v = srv.frame_views(sb, 0, 20000, 2048)
            ev = _fill(v, *_frame(70 + k, 0, 20000, 2048))
            srv.wait(srv.submit(sb, 0, ev), 60000)
            srv.close_session(sb)
        t.join()
        for k in range(frames):
            assert np.array_equal(out["a"][k], alone[k]), k
        assert srv.cache(sa).error() == 0
