"""The learned-opening-test oracle checks itself on the CPU: the analytic
gradient against central finite differences, the BF16 rounding against
known values, the label against a direct multipole expansion check (a point
mass is its own monopole), and the feature map's invariances."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import lmac_oracle as lo  # noqa: E402


def rand_params(seed, scale=0.5):
    return np.random.default_rng(seed).standard_normal(lo.NPARAMS) * scale


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    P = rand_params(1)
    X = rng.standard_normal((64, lo.NIN))
    y = (rng.random(64) < 0.5).astype(np.float64)
    w = rng.random(64)
    g, _ = lo.grad(P, X, y, w, scale=0.5)
    h = 1e-6
    for q in rng.choice(lo.NPARAMS, 60, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[q] += h
        Pm[q] -= h
        fd = 0.5 * (lo.grad(Pp, X, y, w)[1] - lo.grad(Pm, X, y, w)[1]) / (2 * h)
        assert g[q] == pytest.approx(fd, rel=1e-5, abs=1e-8), q


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0, 1.0 + 2 ** -9], np.float32)
    got = lo.bf16(x)
    # BF16 spacing at 1 is 2^-7: 1 + 2^-9 rounds down, 1 + 2^-8 is a tie and
    # goes to the even neighbour 1.0.
    assert got[0] == 1.0 and got[5] == 1.0
    assert got[1] == 1.0
    assert got[2] == np.float32(1.0078125)
    assert abs(got[3] - x[3]) <= abs(x[3]) * 2 ** -8
    assert got[4] == 65536.0


def test_label_of_a_point_mass_is_zero():
    # A single particle is exactly its monopole (quadrupole zero): r = 0.
    t = np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0]])
    src = np.array([[2.0, 1.0, -1.0]])
    r = lo.label(t, np.ones(2), src, np.array([0.5]), src[0], 0.5, np.zeros(5), 1.0, 0.01)
    assert r < 1e-12


def test_label_shrinks_with_distance():
    rng = np.random.default_rng(0)
    src = rng.standard_normal((50, 3)) * 0.1
    m = rng.random(50)
    M = m.sum()
    com = (m[:, None] * src).sum(0) / M
    d = src - com
    Q = np.zeros(5)
    for k in range(50):
        dd = d[k] @ d[k]
        Q += m[k] * np.array([3 * d[k, 0] ** 2 - dd, 3 * d[k, 1] ** 2 - dd, 3 * d[k, 0] * d[k, 1],
                              3 * d[k, 0] * d[k, 2], 3 * d[k, 1] * d[k, 2]])
    rs = []
    for dist in (1.0, 2.0, 4.0):
        t = com[None, :] + np.array([[dist, 0.3 * dist, 0.0]])
        a = lo.exact_accel(t, src, m, 1.0, 0.0)
        rs.append(lo.label(t, np.linalg.norm(a, axis=1), src, m, com, M, Q, 1.0, 0.0))
    # quadrupole-corrected: the relative error falls like (s/d)^3
    assert rs[0] > rs[1] > rs[2]
    assert rs[1] / rs[2] > 4.0


def test_features_scale_free():
    rng = np.random.default_rng(5)
    n = 20
    gcom, ncom = rng.standard_normal((n, 3)), rng.standard_normal((n, 3)) * 4
    gR, M, maxR, size = rng.random(n) * 0.1, rng.random(n) + 0.1, rng.random(n) * 0.3, rng.random(n) * 0.5
    Q = rng.standard_normal((n, 5)) * 0.01
    amin = rng.random(n) + 0.5
    cnt = rng.integers(2, 1000, n)
    f1, _ = lo.features(gcom, gR, amin, ncom, M, maxR, size, Q, cnt, 1.0, 0.01)
    s = 3.0  # scale lengths by s, masses by s^3, accelerations then scale by s
    f2, _ = lo.features(gcom * s, gR * s, amin * s, ncom * s, M * s ** 3, maxR * s, size * s, Q * s ** 5, cnt,
                        1.0, 0.01 * s)
    np.testing.assert_allclose(f1, f2, rtol=1e-10, atol=1e-10)
