"""Record producer: the path tracer (shader/src/path_tracer.comp) over a BVH
built on the GPU, against the oracle's restatement with brute-force hits.

Every floating-point step is fixed on both sides (no contraction, explicit
fused multiply-adds, the same series for log / sin / cos / atan2 / exp), so
the per-pixel images are equal bit for bit and so are the records. Records are
appended through atomic counters in an order that differs between the two, so
they are compared as multisets: eval records by content, with a self-training
record's destination range replaced by the train records it points at; train
records batch by batch."""
import numpy as np
import pytest

from gpu_util import dev, host


def _scene(seed=7):
    from vknrc_gb300 import synthetic as S

    return S.scene(S.rng_for(seed), vertices=600, primitives=400, instances=6, materials=10)


def _params(oracle_mod, w, h, seed=5, left=1, right=2, p=0.35):
    P = oracle_mod.TraceParams()
    for k, v in {"origin": (0.0, 0.3, -7.5), "look": (0.0, 0.0, 1.0), "side": (0.55, 0.0, 0.0),
                 "up": (0.0, 0.55 * h / w, 0.0)}.items():
        getattr(P, k)[:] = v
    P.width, P.height, P.seed, P.left_method, P.right_method, P.train_probability = w, h, seed, left, right, p
    return P


def _canonical(eval_rec, train):
    """Eval records as a sorted list of tuples; a train destination (bit 0 set)
    becomes (batch, contents of its record range)."""
    out = []
    for r in eval_rec:
        dst = int(r[0])
        if dst & 1:
            e = dst >> 1
            b, l, rr = e & 3, (e >> 2) & 0x3FFF, e >> 16
            key = ("train", b, tuple(map(tuple, train[b][l:rr + 1].tolist())), tuple(r[1:].tolist()))
        else:
            key = ("screen", dst, tuple(r[1:].tolist()))
        out.append(key)
    return sorted(out)


def test_oracle_trace_is_deterministic_and_emits_records(oracle):
    sc = _scene()
    P = _params(oracle, 40, 24)
    a = oracle.path_trace(sc, P, 40 * 24 + 65536)
    b = oracle.path_trace(sc, P, 40 * 24 + 65536)
    assert np.array_equal(a["bias_factor_r"], b["bias_factor_r"])
    assert a["eval_count"] > 0 and sum(a["train_counts"]) > 0
    assert np.all(np.isfinite(a["bias_factor_r"])) and np.all(a["bias_factor_r"] >= 0)
    # every screen record points at a pixel of the frame
    scr = a["eval"][(a["eval"][:, 0] & 1) == 0, 0] >> 1
    assert np.all((scr & 0x7FFF) < 40) and np.all((scr >> 15) < 24)


@pytest.mark.gpu
@pytest.mark.parametrize("methods", [(1, 2), (1, 1), (0, 2)])
def test_gpu_trace_equals_oracle(cuda, oracle, methods):
    from vknrc_gb300 import nrc

    sc = _scene()
    w, h = 72, 40
    P = _params(oracle, w, h, left=methods[0], right=methods[1])
    ref = oracle.path_trace(sc, P, w * h + 65536)
    ds = nrc.DeviceScene(sc)
    bvh = nrc.Bvh(ds)
    assert bvh.info() == (400, 399)
    buf = nrc.TraceBuffers(w, h)
    buf.reset()
    GP = nrc.TraceParams.from_buffer_copy(bytes(P))
    nrc.path_trace(ds, bvh, GP, buf)
    assert np.array_equal(host(buf.bias_factor_r), ref["bias_factor_r"])
    assert np.array_equal(host(buf.factor_gb), ref["factor_gb"])
    n_eval = int(host(buf.eval_count)[0])
    counts = [int(host(c)[0]) for c in buf.train_counts]
    assert n_eval == ref["eval_count"] and counts == ref["train_counts"]
    ev = host(buf.eval)[:n_eval].view(np.uint32)
    tr = [host(buf.train[b])[: counts[b]].view(np.uint32) for b in range(4)]
    for b in range(4):
        assert sorted(map(tuple, tr[b].tolist())) == sorted(map(tuple, ref["train"][b].tolist())), b
    assert _canonical(ev, tr) == _canonical(ref["eval"], ref["train"])
    bvh.close()
