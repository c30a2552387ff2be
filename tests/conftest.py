import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

TREE_EXACT = ("level", "prefix", "count", "is_leaf", "center", "half")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def ic(pkg):
    import importlib
    return importlib.import_module(ge.PKG_NAME + ".ic")


@pytest.fixture(scope="session")
def oracle():
    orc = ge.load_oracle()
    orc.build_oracle()
    return orc.Oracle()


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def golden_tree(d, tag="tree"):
    keys = TREE_EXACT + ("com", "mass", "max_radius", "quad", "order")
    return {k: d[f"{tag}_{k}"] for k in keys}


def rel_err(ax, ay, az, rx, ry, rz):
    ref = np.sqrt(rx ** 2 + ry ** 2 + rz ** 2)
    return np.sqrt((ax - rx) ** 2 + (ay - ry) ** 2 + (az - rz) ** 2) / np.maximum(ref, 1e-300)


def edge_cases():
    d = load_golden("edge_cases.npz")
    return [str(s) for s in d["names"]], d


def octant_keys(x, y, z, levels=21):
    """63-bit octant-path keys by the reference's FP64 centre recurrence.

    Root cube as in Tree.cpp:54-88, octant bit p >= centre (Tree.cpp:11-20),
    child centre = centre +/- 0.5*half (Tree.cpp:90-112).  numpy FP64 adds
    round to nearest like the C++ code.  Digit l sits at bits 3*(20-l).
    """
    p = [np.asarray(a, dtype=np.float64) for a in (x, y, z)]
    n = len(p[0])
    if n == 0:
        return np.zeros(0, np.uint64)
    lo = [a.min() for a in p]
    hi = [a.max() for a in p]
    half = max(0.5 * (h - l) for l, h in zip(lo, hi))
    if not half > 1e-12:
        half = 1.0
    h = half * 1.001
    c = [np.full(n, 0.5 * (l + hh)) for l, hh in zip(lo, hi)]
    key = np.zeros(n, np.uint64)
    for _ in range(levels):
        b = [p[k] >= c[k] for k in range(3)]
        digit = b[0].astype(np.uint64) | (b[1].astype(np.uint64) << np.uint64(1)) | \
            (b[2].astype(np.uint64) << np.uint64(2))
        key = (key << np.uint64(3)) | digit
        h = 0.5 * h
        for k in range(3):
            c[k] = np.where(b[k], c[k] + h, c[k] - h)
    return key


def leaf_order_from_keys(keys, tree):
    """Reference `order` implied by keys and a canonical tree: leaves in key
    order, members by ascending original index."""
    sk = np.argsort(keys, kind="stable")
    ks = keys[sk]
    leaves = np.nonzero(tree["is_leaf"])[0]
    shift = (3 * (21 - tree["level"][leaves])).astype(np.uint64)
    lo_key = tree["prefix"][leaves].astype(np.uint64) << shift
    out, counts = [], []
    for j in np.argsort(lo_key, kind="stable"):
        li = leaves[j]
        s = np.uint64(3 * (21 - tree["level"][li]))
        pfx = np.uint64(tree["prefix"][li])
        a = np.searchsorted(ks, pfx << s, side="left")
        b = np.searchsorted(ks, (pfx + np.uint64(1)) << s, side="left") if tree["level"][li] > 0 else len(ks)
        counts.append((b - a, tree["count"][li]))
        out.append(np.sort(sk[a:b]))
    return (np.concatenate(out) if out else np.zeros(0, np.int64)), counts
