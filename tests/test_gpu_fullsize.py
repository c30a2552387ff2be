"""The bench's full-size workload (the two-component galaxy, N = 4,194,304,
leaf capacity 32) through size-independent properties, where a per-element
comparison with the oracle would take the CPU minutes:

* the 63-bit keys equal the FP64 centre recurrence (numpy restatement of
  Tree.cpp:11-20,54-112), bit for bit;
* `order` is a permutation that sorts the keys; the leaves partition it;
* every internal node's count is the sum of its children's; leaves hold at
  most the leaf capacity; the root's mass and centre of mass are the FP64
  sums of the particles;
* the theta = 0.6 force error against the FP64-summed direct sum on 4,096
  targets stays at the Barnes-Hut truncation level;
* KDK steps conserve linear momentum to round-off of the force sums.
"""
import numpy as np
import pytest

from conftest import octant_keys

pytestmark = pytest.mark.gpu

NCRIT = 32


@pytest.fixture(scope="module")
def galaxy(ic):
    # FP32-rounded: the GPU state then holds exactly these values
    return tuple(np.asarray(a, np.float32).astype(np.float64) for a in ic.galaxy())


def test_fullsize_tree_invariants(pkg, galaxy):
    x, y, z, vx, vy, vz, m = galaxy
    n = len(x)
    with pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.002, theta=0.6), leaf_capacity=NCRIT) as sim:
        sim.set_particles(x, y, z, vx, vy, vz, m)
        sim.compute_accel()
        st = sim.stats()
        t = sim.debug_tree()
    assert st["status_bits"] == 0
    xs, ys, zs = x, y, z
    keys = octant_keys(xs, ys, zs)
    assert np.array_equal(t["keys"], keys)
    order = t["order"]
    assert np.array_equal(np.sort(order), np.arange(n))
    assert np.all(np.diff(keys[order].astype(np.uint64)) >= 0)

    c = pkg.canonical(t)
    level, prefix, count, leaf = c["level"], c["prefix"].astype(np.uint64), c["count"], c["is_leaf"] != 0
    assert count[0] == n and level[0] == 0
    assert np.all(count[leaf] <= NCRIT) or np.all(level[leaf & (count > NCRIT)] == 21)
    assert count[leaf].sum() == n
    # children of (l, p) are the nodes (l + 1, p * 8 + d): sum their counts per parent
    child = level > 0
    parent_key = (level[child] - 1).astype(np.uint64) << np.uint64(60) | (prefix[child] >> np.uint64(3))
    node_key = level.astype(np.uint64) << np.uint64(60) | prefix
    uniq, inv = np.unique(parent_key, return_inverse=True)
    sums = np.bincount(inv, weights=count[child].astype(np.float64))
    pos = np.searchsorted(node_key[np.argsort(node_key)], uniq)
    idx = np.argsort(node_key)[pos]
    assert np.array_equal(node_key[idx], uniq)
    assert np.array_equal(sums.astype(np.int64), count[idx].astype(np.int64))
    assert not np.any(leaf[idx])
    assert int((~leaf).sum()) == len(uniq)  # every internal node has children
    # each leaf's count is the number of keys under its prefix
    for L in np.unique(level[leaf]):
        sel = leaf & (level == L)
        pk = keys >> np.uint64(3 * (21 - int(L)))
        u, cnt = np.unique(pk, return_counts=True)
        at = np.searchsorted(u, prefix[sel])
        assert np.array_equal(u[at], prefix[sel])
        assert np.array_equal(cnt[at], count[sel])
    M = float(np.sum(m))
    assert c["mass"][0] == pytest.approx(M, rel=1e-12)
    mm = m
    com = np.array([np.sum(mm * xs), np.sum(mm * ys), np.sum(mm * zs)]) / M
    np.testing.assert_allclose(c["com"][0], com, rtol=0, atol=1e-9 * max(1.0, np.abs(com).max()))


def test_fullsize_force_error_and_momentum(pkg, galaxy):
    x, y, z, vx, vy, vz, m = galaxy
    with pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.002, theta=0.6, dt=2e-4), leaf_capacity=NCRIT) as sim:
        sim.set_particles(x, y, z, vx, vy, vz, m)
        sim.compute_accel()
        fe = sim.force_error(4096, seed=11, fp64_pairs=True)
        assert 1e-5 < fe["rms"] < 2e-3 and fe["max"] < 2e-2, fe
        p0 = np.asarray(sim.diagnostics()["P"])
        sim.step(5, 2e-4)
        p1 = np.asarray(sim.diagnostics()["P"])
        _, _, _, ux, uy, uz = sim.state()
    mm = np.asarray(m, np.float64)
    scale = np.sum(mm * np.sqrt(ux ** 2 + uy ** 2 + uz ** 2))
    assert np.linalg.norm(p1 - p0) < 1e-4 * scale
