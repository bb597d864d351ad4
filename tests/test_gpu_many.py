"""Batched caches: many independent caches with uneven query and train counts in
one persistent launch per phase (nrc_infer_many, nrc_train_many).

Queries are per-record computations, so every cache's answers in a batched
launch equal its answers alone bit for bit, whatever CTA split is used.
Training sums the weight gradients per CTA group in a fixed order, so a cache
trained in a mix equals the same cache trained alone with the same CTA count;
against the single-cache path (152 CTAs, a different summation grouping) it
agrees within the training tolerance of the other tests."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu

QUERY_COUNTS = [1, 300, 4097, 65536, 256 * 256 + 17, 200_000, 0, 1280 * 720]
TRAIN_COUNTS = [4096, 65536, 129, 16384, 30000, 8192]


def _queries(seed, n):
    from vknrc_gb300 import synthetic as S

    return S.inputs(S.rng_for(seed), max(n, 1))


def test_infer_many_equals_each_cache_alone(cuda):
    import torch

    from vknrc_gb300 import Cache, nrc

    caches = [Cache(seed=100 + j) for j in range(len(QUERY_COUNTS))]
    try:
        qs = [dev(_queries(200 + j, n)) for j, n in enumerate(QUERY_COUNTS)]
        cnts = [count(n) for n in QUERY_COUNTS]
        solo = []
        for c, q, k in zip(caches, qs, cnts):
            o = torch.full((q.shape[0], 3), -1.0, dtype=torch.float32, device="cuda")
            c.infer(q, k, o)
            solo.append(host(o))
        for ctas in (None, [1] * len(caches), [3, 1, 7, 40, 2, 60, 1, 30]):
            outs = [torch.full((q.shape[0], 3), -1.0, dtype=torch.float32, device="cuda") for q in qs]
            jobs = [nrc.query_job(c, q, k, o) for c, q, k, o in zip(caches, qs, cnts, outs)]
            nrc.infer_many(jobs, ctas=ctas)
            for j, (o, ref, n) in enumerate(zip(outs, solo, QUERY_COUNTS)):
                got = host(o)
                assert np.array_equal(got[:n], ref[:n]), (ctas, j)
                assert np.all(got[n:] == -1.0)  # nothing written past the count
        plan = nrc.plan_query_ctas([nrc.query_job(c, q, k, o) for c, q, k, o in zip(caches, qs, cnts, outs)])
        assert sum(plan) <= 152 and min(plan) >= 1
        for c in caches:
            assert c.error() == 0
    finally:
        for c in caches:
            c.close()


def _train_set(seed, n):
    from vknrc_gb300 import synthetic as S

    return [dev(S.train_records(S.rng_for(seed, b), n, target="field", sigma=0.5)) for b in range(4)]


def test_train_many_in_mix_equals_alone(cuda):
    from vknrc_gb300 import Cache, nrc

    recs = [_train_set(300 + j, n) for j, n in enumerate(TRAIN_COUNTS)]
    mk = lambda j, n: Cache(seed=400 + j, train_batch_size=n, learning_rate=1e-3, beta2=0.99)
    mix = [mk(j, n) for j, n in enumerate(TRAIN_COUNTS)]
    alone = [mk(j, n) for j, n in enumerate(TRAIN_COUNTS)]
    try:
        jobs = lambda cs, idx: [nrc.train_job(cs[j], recs[j], [count(TRAIN_COUNTS[j]) for _ in range(4)])
                                for j in idx]
        plan = nrc.plan_train_ctas(jobs(mix, range(len(mix))))
        assert sum(plan) == 152 and min(plan) >= 1
        # records per CTA balanced: the largest cache gets the most CTAs
        assert plan[1] == max(plan)
        nrc.train_many(jobs(mix, range(len(mix))), ctas=plan)
        for j in range(len(alone)):
            nrc.train_many(jobs(alone, [j]), ctas=[plan[j]])
        for a, b in zip(mix, alone):
            sa, ea = a.get_optimizer()
            sb, eb = b.get_optimizer()
            assert sa == sb and sa[0] == 4
            assert np.array_equal(ea, eb)
            assert np.array_equal(a.get_weights(0), b.get_weights(0))
            assert a.error() == 0 and b.error() == 0
    finally:
        for c in mix + alone:
            c.close()


@pytest.mark.parametrize("ctas", [1, 5, 32, 152])
def test_train_many_group_size_gradient_vs_oracle(cuda, oracle, ctas):
    """One training step of a cache by a group of `ctas` CTAs: small groups run
    many tiles per CTA (one long TMEM accumulation) and keep the optimizer
    entries in memory rather than shared memory. After one Adam step the first
    moment is m = (1 - beta1) * g / n exactly enough to recover the summed
    gradient, which must match the oracle's (fp16 storage semantics) as the
    single-cache gradient test requires; the step state advances once."""
    from vknrc_gb300 import Cache, nrc, synthetic as S

    n = 16384
    tr = S.train_records(S.rng_for(500, 0), n, target="field", sigma=0.5)
    with Cache(seed=501, learning_rate=1e-3) as c:
        w = c.get_weights(1)
        nrc.train_many([nrc.train_job(c, [dev(tr)], [count(n)])], ctas=[ctas])
        st, ent = c.get_optimizer()
        assert st[0] == 1 and c.error() == 0
    ref, gabs, _ = oracle.train_grad(w, oracle.encode(tr[:, 6:]), tr[:, :3], mode=0, want_abs=True, nthreads=8)
    g = ent[:, 0].astype(np.float64) / np.float64(np.float32(0.1)) * n
    rel = np.abs(g - ref) / (gabs + 1e-30)
    assert np.median(rel) < 4e-5, np.median(rel)
    assert np.quantile(rel, 0.99) < 1e-3, np.quantile(rel, 0.99)
    assert rel.max() < 2e-2, rel.max()


def test_train_many_rejects_bad_jobs(cuda):
    from vknrc_gb300 import Cache, NRCError, nrc

    recs = _train_set(600, 256)
    with Cache(seed=601) as a:
        j = nrc.train_job(a, recs, [count(256) for _ in range(4)])
        with pytest.raises(NRCError):
            nrc.train_many([j, j])  # one context twice
        with pytest.raises(NRCError):
            nrc.train_many([j], ctas=[0])
        with pytest.raises(NRCError):
            nrc.train_many([j], ctas=[153])
        assert a.get_optimizer()[0][0] == 0


def test_batched_frame_graph_capture_replays(cuda):
    """The per-frame work of several caches (queries, then four chained training
    steps each) captured as one CUDA graph replays to the eager result."""
    import torch

    from vknrc_gb300 import Cache, nrc

    qn = [5000, 70000, 1000]
    tn = [4096, 16384, 8192]
    qs = [dev(_queries(700 + j, n)) for j, n in enumerate(qn)]
    recs = [_train_set(710 + j, n) for j, n in enumerate(tn)]

    def frame_jobs(cs, outs, qc, tc):
        return ([nrc.query_job(c, q, k, o) for c, q, k, o in zip(cs, qs, qc, outs)],
                [nrc.train_job(c, r, t) for c, r, t in zip(cs, recs, tc)])

    mk = lambda: [Cache(seed=720 + j, train_batch_size=n) for j, n in enumerate(tn)]
    eager, graphed = mk(), mk()
    try:
        outs_e = [torch.empty((n, 3), dtype=torch.float32, device="cuda") for n in qn]
        qc = [count(n) for n in qn]
        tc_e = [[count(n) for _ in range(4)] for n in tn]
        for _ in range(2):
            qj, tj = frame_jobs(eager, outs_e, qc, tc_e)
            nrc.infer_many(qj)
            nrc.train_many(tj)
        outs_g = [torch.empty_like(o) for o in outs_e]
        tc_g = [[count(n) for _ in range(4)] for n in tn]
        qj, tj = frame_jobs(graphed, outs_g, qc, tc_g)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                nrc.infer_many(qj, stream=s)
                nrc.train_many(tj, stream=s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        assert graphed[0].get_optimizer()[0][0] == 0  # capture ran nothing
        for _ in range(2):
            g.replay()
        torch.cuda.synchronize()
        for a, b, oa, ob in zip(eager, graphed, outs_e, outs_g):
            assert np.array_equal(host(oa), host(ob))
            assert np.array_equal(a.get_optimizer()[1], b.get_optimizer()[1])
            assert b.error() == 0
    finally:
        for c in eager + graphed:
            c.close()


def test_autotune_many_valid_split_and_caches_untouched(cuda):
    """nrc_autotune_many returns a split that fits on the SMs with at least one
    CTA per job, leaves the caches' training state as it was (the training
    candidates run on scratch copies), and the batched launches run with it."""
    import torch

    from vknrc_gb300 import Cache, nrc, synthetic as S

    qn = [256 * 256, 4097, 1280 * 720]
    tn = [4096, 16384, 30000]
    caches = [Cache(seed=700 + j, train_batch_size=tn[j]) for j in range(3)]
    try:
        qs = [dev(_queries(710 + j, n)) for j, n in enumerate(qn)]
        qc = [count(n) for n in qn]
        outs = [torch.empty((n, 3), dtype=torch.float32, device="cuda") for n in qn]
        recs = [[dev(S.train_records(S.rng_for(720 + j, b), n, sigma=0.5)) for b in range(4)] for j, n in enumerate(tn)]
        tc = [[count(n) for _ in range(4)] for n in tn]
        qjobs = [nrc.query_job(c, q, k, o) for c, q, k, o in zip(caches, qs, qc, outs)]
        tjobs = [nrc.train_job(c, r, t) for c, r, t in zip(caches, recs, tc)]
        before = [c.get_optimizer() for c in caches]
        w_before = [c.get_weights(1) for c in caches]
        gq, gt, qms, tms = nrc.autotune_many(qjobs, tjobs)
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        assert len(gq) == 3 and len(gt) == 3 and min(gq) >= 1 and min(gt) >= 1
        assert sum(gq) <= sms and sum(gt) <= sms
        assert qms > 0 and tms > 0
        for c, (st, ent), w in zip(caches, before, w_before):
            st2, ent2 = c.get_optimizer()
            assert st2 == st
            np.testing.assert_array_equal(ent2, ent)
            np.testing.assert_array_equal(c.get_weights(1), w)
        nrc.infer_many(qjobs, ctas=gq)
        nrc.train_many(tjobs, ctas=gt)
        torch.cuda.synchronize()
        assert all(c.get_optimizer()[0][0] == 4 for c in caches)
        assert all(c.error() == 0 for c in caches)
    finally:
        for c in caches:
            c.close()
