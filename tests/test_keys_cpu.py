"""The 63-bit key definition reproduces the reference's tree (CPU check).

The CUDA key kernel evaluates the same FP64 recurrence as octant_keys(); this
test shows, on the CPU, that sorting by those keys and cutting at the golden
trees' leaves yields exactly the reference's leaf membership and `order`.
"""
import numpy as np
import pytest

from conftest import edge_cases, golden_tree, leaf_order_from_keys, load_golden, octant_keys

CASES = [("plummer16k.npz", "tree"), ("selftest_uniform1000.npz", "tree"), ("selftest_ball4000.npz", "tree")]


@pytest.mark.parametrize("fname,tag", CASES)
def test_keys_reproduce_reference_order(fname, tag):
    d = load_golden(fname)
    t = golden_tree(d, tag)
    keys = octant_keys(d["x"], d["y"], d["z"])
    order, counts = leaf_order_from_keys(keys, t)
    assert all(a == b for a, b in counts)
    assert np.array_equal(order, t["order"])
    # Every node's members share its octant-path prefix.
    for lvl, pfx, cnt in zip(t["level"], t["prefix"], t["count"]):
        if lvl == 0:
            assert cnt == len(keys)
            continue
        s = np.uint64(3 * (21 - lvl))
        assert int(np.sum((keys >> s) == np.uint64(pfx))) == cnt


@pytest.mark.parametrize("name", edge_cases()[0])
def test_keys_edge_cases(name):
    _, d = edge_cases()
    t = golden_tree(d, f"{name}_tree")
    keys = octant_keys(d[f"{name}_x"], d[f"{name}_y"], d[f"{name}_z"])
    if np.max(t["level"]) >= 21:
        pytest.skip("tree deeper than the 21 key levels")
    order, counts = leaf_order_from_keys(keys, t)
    assert all(a == b for a, b in counts)
    assert np.array_equal(order, t["order"])


def test_spread_interleave_matches_digits():
    """Bit layout: digit l of a key is the level-l octant (x:1, y:2, z:4)."""
    rng = np.random.default_rng(5)
    x, y, z = rng.random((3, 64))
    keys = octant_keys(x, y, z)
    k2 = octant_keys(x, y, z, levels=1)
    assert np.array_equal(keys >> np.uint64(60), k2)
