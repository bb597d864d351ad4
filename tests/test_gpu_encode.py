"""nrc_encode / nrc_sph_encode on the GPU against the oracle and the reference's
own encoding (golden vectors)."""
import numpy as np
import pytest

from gpu_util import count, dev, host

pytestmark = pytest.mark.gpu


def test_encode_bit_exact_vs_oracle(cuda, oracle, golden):
    from vknrc_gb300 import Cache, synthetic as S

    rec = np.concatenate([golden["encode"]["records"], S.inputs(S.rng_for(3), 10007)])
    with Cache() as c:
        out = cuda.full((rec.shape[0], 64), -1, dtype=cuda.int16, device="cuda")
        c.encode(dev(rec), count(rec.shape[0]), out)
        got = host(out).view(np.uint16)
    assert np.array_equal(got, oracle.encode(rec))


def test_encode_edge_positions_bit_exact(cuda, oracle):
    """Positions where the frequency features' roundings are delicate: exact
    dyadic points, values just off them, tiny and subnormal magnitudes, and
    magnitudes where p * 2^11 overflows (the kernel's fallback form)."""
    from vknrc_gb300 import Cache, synthetic as S

    vals = np.array([0.0, -0.0, 1.0, 0.5, 0.25, 1.0 / 2048, 3.0 / 4096, 1e-30, 1e-40, -1e-40, 0.999999,
                     np.nextafter(np.float32(0.5), np.float32(1)), np.nextafter(np.float32(0.5), np.float32(0)),
                     -0.75, 7.3, -1234.5, 2.0 ** 99, 1.5 * 2.0 ** 100, 1e30, 3e38, -3e38, np.inf, -np.inf],
                    dtype=np.float32)
    rec = S.inputs(S.rng_for(5), vals.size * 3)
    rec[:, 0] = np.tile(vals, 3)
    rec[:, 1] = np.roll(np.tile(vals, 3), 7)
    rec[:, 2] = np.roll(np.tile(vals, 3), 13)
    with Cache() as c:
        out = cuda.full((rec.shape[0], 64), -1, dtype=cuda.int16, device="cuda")
        c.encode(dev(rec), count(rec.shape[0]), out)
        got = host(out).view(np.uint16)
    want = oracle.encode(rec)
    nan_got = np.isnan(got.view(np.float16))
    nan_want = np.isnan(want.view(np.float16))
    assert np.array_equal(nan_got, nan_want)
    assert np.array_equal(got[~nan_got], want[~nan_want])


def test_encode_vs_reference_golden(cuda, golden):
    from vknrc_gb300 import Cache

    g = golden["encode"]
    with Cache() as c:
        out = cuda.zeros((g["records"].shape[0], 64), dtype=cuda.int16, device="cuda")
        c.encode(dev(g["records"]), count(g["records"].shape[0]), out)
        got = host(out).view(np.uint16)
    exact = np.r_[0:36, 56:64]
    assert np.array_equal(got[:, exact], g["encoded"][:, exact])
    d = np.abs(got[:, 36:56].view(np.float16).astype(np.float64) - g["encoded"][:, 36:56].view(np.float16))
    assert d.max() <= 2.0 ** -11


@pytest.mark.parametrize("n,cap", [(0, 64), (1, 64), (300, 200), (129, 129)])
def test_encode_count_and_capacity(cuda, oracle, n, cap):
    from vknrc_gb300 import Cache, synthetic as S

    rec = S.inputs(S.rng_for(4), max(cap, 1))
    with Cache() as c:
        out = cuda.full((max(cap, 1), 64), 0x7777, dtype=cuda.int16, device="cuda")
        c.encode(dev(rec), count(n), out, capacity=cap)
        got = host(out).view(np.uint16)
    m = min(n, cap)
    assert np.array_equal(got[:m], oracle.encode(rec[:m]))
    assert np.all(got[m:] == 0x7777)


def test_sph_encode_vs_reference_golden(cuda, golden):
    import ctypes

    from vknrc_gb300 import nrc

    g = golden["encode"]
    d = dev(g["dirs"])
    out = cuda.zeros((d.shape[0], 2), dtype=cuda.float32, device="cuda")
    nrc.check(nrc.lib().nrc_sph_encode(d.data_ptr(), count(d.shape[0]).data_ptr(), d.shape[0], out.data_ptr(),
                                       cuda.cuda.current_stream().cuda_stream), "sph")
    assert np.max(np.abs(host(out) - g["sph"])) <= 4e-7
