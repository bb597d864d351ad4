"""The seeded synthetic records the bench and tests use in place of the
reference's path-tracer output follow the benchmark configuration's
distributions: position U[0,1]^3, direction and normal uniform on the sphere
(sphere-encoded, the direction quantised to unorm16), roughness U(0,1),
diffuse/specular albedo U(0,1)^3, target radiance lognormal(0, 1.5) per
channel; the generators are counter-based and reproducible (CPU only)."""
import numpy as np

from vknrc_gb300 import synthetic as S

N = 200_000


def _uniform_ok(x, lo=0.0, hi=1.0):
    x = np.asarray(x, np.float64)
    assert x.min() >= lo and x.max() <= hi
    m, v = (lo + hi) / 2, (hi - lo) ** 2 / 12
    assert abs(x.mean() - m) < 0.005 * (hi - lo) and abs(x.var() - v) < 0.02 * v
    # the empirical CDF against the uniform one (Kolmogorov-Smirnov distance)
    xs = np.sort(x)
    cdf = (xs - lo) / (hi - lo)
    assert np.max(np.abs(cdf - np.arange(1, len(xs) + 1) / len(xs))) < 0.01


def test_inputs_follow_the_configuration():
    r = S.inputs(S.rng_for(7), N)
    assert r.shape == (N, 14) and r.dtype == np.float32
    for k in [0, 1, 2, 7, 8, 9, 10, 11, 12, 13]:  # position, roughness, albedos
        _uniform_ok(r[:, k])
    for cols in ([3, 4], [5, 6]):  # sphere-encoded direction and normal
        u, v = r[:, cols[0]].astype(np.float64), r[:, cols[1]].astype(np.float64)
        _uniform_ok(u)  # azimuth uniform
        _uniform_ok(np.cos(np.pi * v), -1.0, 1.0)  # z = cos(pi v) uniform for directions uniform on S^2
    q = r[:, 3:5].astype(np.float64) * 65535.0
    assert np.max(np.abs(q - np.round(q))) < 1e-2  # the direction is unorm16-quantised


def test_train_records_follow_the_configuration():
    t = S.train_records(S.rng_for(8), N, target="lognormal", sigma=1.5)
    assert t.shape == (N, 20)
    assert np.all(t[:, 3:6] == 1.0)  # factor = 1: the bias is the target
    lt = np.log(t[:, 0:3].astype(np.float64))
    assert np.all(np.abs(lt.mean(0)) < 0.02) and np.all(np.abs(lt.std(0) - 1.5) < 0.02)
    f = S.train_records(S.rng_for(8), 1000, target="field", sigma=1.0)
    assert np.all(f[:, 0:3] > 0)


def test_generators_are_counter_based_and_reproducible():
    a = S.inputs(S.rng_for(9, 3, 1), 1000)
    assert np.array_equal(a, S.inputs(S.rng_for(9, 3, 1), 1000))
    assert not np.array_equal(a, S.inputs(S.rng_for(9, 4, 1), 1000))  # another frame
    assert not np.array_equal(a, S.inputs(S.rng_for(9, 3, 2), 1000))  # another stream
