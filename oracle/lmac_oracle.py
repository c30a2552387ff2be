"""Oracle of the learned opening test (test infrastructure only).

numpy restatements, in FP64 unless stated, of what the GPU computes for the
learned multipole-acceptance test:

* ``features``     -- the 8 features of a (group, node) pair;
* ``label``        -- the worst relative error of a node's multipole
                      (softened monopole + unsoftened traceless quadrupole,
                      the P2C of projects/nbody_core/src/Solvers.cpp:147-179)
                      against the exact softened sum over the node's
                      particles (AccumPairPlummer, Solvers.cpp:19-38), over
                      the members of the group;
* ``forward`` / ``grad`` / ``adam`` -- the 8 -> 32 -> 32 -> 1 ReLU network,
                      binary cross-entropy on the logit, Adam;
* ``forward_bf16`` -- the tensor-core path: standardised inputs, weights and
                      first-layer activations rounded to BF16, sums in FP64.

The geometric test these replace is the reference's (include/ngrav/Mac.hpp:25-29,
src/Solvers.cpp:261-271); there is no reference counterpart of the network.
"""
from __future__ import annotations

import numpy as np

NIN, NH = 8, 32
W1, B1 = 0, NH * NIN
W2 = B1 + NH
B2 = W2 + NH * NH
W3 = B2 + NH
B3 = W3 + NH
NPARAMS = B3 + 1


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    return (P[W1:B1].reshape(NH, NIN), P[B1:W2], P[W2:B2].reshape(NH, NH), P[B2:W3], P[W3:B3], P[B3])


def _log2c(v):
    return np.clip(np.log2(np.maximum(v, 1e-30)), -30.0, 30.0)


def features(gcom, gR, amin, ncom, M, maxR, size, Q5, count, G, eps, log2b=0.0):
    """Features of pairs: group COM (n,3), group maxRadius, group min |a|; node
    COM (n,3), mass, maxRadius, size 2h, quadrupole (n,5: xx, yy, xy, xz, yz),
    particle count.  Returns (n, 8) and worst = |d| - maxR_G."""
    d = np.asarray(ncom, np.float64) - np.asarray(gcom, np.float64)
    d2 = np.sum(d * d, axis=1)
    dist = np.sqrt(d2)
    worst = dist - gR
    iw = 1.0 / np.maximum(worst, 1e-30)
    Q = np.asarray(Q5, np.float64)
    qxx, qyy, qxy, qxz, qyz = Q.T
    qzz = -qxx - qyy
    s2 = np.maximum(M * maxR * maxR, 1e-30)
    qn = np.sqrt(qxx ** 2 + qyy ** 2 + qzz ** 2 + 2.0 * (qxy ** 2 + qxz ** 2 + qyz ** 2))
    dx, dy, dz = d.T
    dqd = qxx * dx * dx + qyy * dy * dy + qzz * dz * dz + 2.0 * (qxy * dx * dy + qxz * dx * dz + qyz * dy * dz)
    f = np.empty((len(d2), NIN))
    f[:, 0] = _log2c(size * iw)
    f[:, 1] = _log2c(maxR * iw)
    f[:, 2] = _log2c(gR * iw)
    f[:, 3] = _log2c(G * M * iw * iw / np.maximum(amin, 1e-30)) - log2b
    f[:, 4] = qn / s2
    f[:, 5] = dqd / (s2 * np.maximum(d2, 1e-30))
    f[:, 6] = np.minimum(eps * iw, 16.0)
    f[:, 7] = np.log2(np.maximum(count, 1))
    return f, worst


def multipole_accel(targets, com, M, Q5, G, eps):
    """Acceleration of a node's multipole on target points (n,3)."""
    d = np.asarray(com, np.float64)[None, :] - targets
    r2 = np.sum(d * d, axis=1)
    a = (M / (r2 + eps * eps) ** 1.5)[:, None] * d
    qxx, qyy, qxy, qxz, qyz = Q5
    qzz = -qxx - qyy
    Q = np.array([[qxx, qxy, qxz], [qxy, qyy, qyz], [qxz, qyz, qzz]])
    qd = d @ Q
    qd2 = np.sum(d * qd, axis=1)
    ir = 1.0 / np.sqrt(r2)
    ir5 = ir ** 5
    ir7 = ir5 * ir * ir
    a += -ir5[:, None] * qd + (2.5 * qd2 * ir7)[:, None] * d
    return G * a


def exact_accel(targets, src, msrc, G, eps):
    d = src[None, :, :] - targets[:, None, :]
    r2 = np.sum(d * d, axis=2) + eps * eps
    w = msrc[None, :] / r2 ** 1.5
    return G * np.einsum("ts,tsk->tk", w, d)


def label(targets, amag, src, msrc, com, M, Q5, G, eps):
    """max over targets of |exact - multipole| / |a(target)|."""
    e = exact_accel(targets, src, msrc, G, eps) - multipole_accel(targets, com, M, Q5, G, eps)
    return float(np.max(np.sqrt(np.sum(e * e, axis=1)) / np.maximum(amag, 1e-30)))


def forward(P, X):
    w1, b1, w2, b2, w3, b3 = unpack(P)
    X = np.asarray(X, np.float64)
    a1 = X @ w1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ w2.T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w3 + b3
    return z, (X, a1, h1, a2, h2)


def bce(z, y):
    return np.maximum(z, 0.0) - y * z + np.log1p(np.exp(-np.abs(z)))


def grad(P, X, y, w=None, scale=1.0):
    """Gradient of scale * sum_k w_k BCE(z_k, y_k); returns (grad, loss sum)."""
    w1, b1, w2, b2, w3, b3 = unpack(P)
    y = np.asarray(y, np.float64)
    w = np.ones_like(y) if w is None else np.asarray(w, np.float64)
    z, (X, a1, h1, a2, h2) = forward(P, X)
    p = 1.0 / (1.0 + np.exp(-z))
    dz = w * scale * (p - y)
    g = np.zeros(NPARAMS)
    g[W3:B3] = h2.T @ dz
    g[B3] = dz.sum()
    d2 = np.outer(dz, w3) * (a2 > 0)
    g[W2:B2] = (d2.T @ h1).ravel()
    g[B2:W3] = d2.sum(axis=0)
    d1 = (d2 @ w2) * (a1 > 0)
    g[W1:B1] = (d1.T @ X).ravel()
    g[B1:W2] = d1.sum(axis=0)
    return g, float(np.sum(w * bce(z, y)))


def adam(P, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    P = P - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return P, m, v


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return (u & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def forward_bf16(P, norm, Xraw):
    """The tensor-core forward pass on raw features with norm = (mu[8], 1/sd[8])."""
    w1, b1, w2, b2, w3, b3 = unpack(P)
    mu = np.asarray(norm[:NIN], np.float32)
    isd = np.asarray(norm[NIN:], np.float32)
    xs = bf16((np.asarray(Xraw, np.float32) - mu) * isd).astype(np.float64)
    a1 = xs @ bf16(w1).astype(np.float64).T + np.float32(b1).astype(np.float64)
    h1 = bf16(np.maximum(a1, 0.0).astype(np.float32)).astype(np.float64)
    a2 = h1 @ bf16(w2).astype(np.float64).T + b2
    return np.maximum(a2, 0.0) @ w3 + b3
