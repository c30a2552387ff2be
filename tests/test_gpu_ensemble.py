"""Ensembles of independent systems in one context (one launch per phase).

Each system of an ensemble is exactly the system alone: its tree is built
from its own root cube, its walk never leaves its own tree, so accelerations,
KDK trajectories, force errors and diagnostics equal those of a context that
holds that system only.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def systems(ic, sizes, seed0=10):
    out = []
    for k, n in enumerate(sizes):
        x, y, z, vx, vy, vz, m = ic.plummer(n, seed=seed0 + k)
        shift = np.array([10.0 * k, -3.0 * k, 0.5 * k])  # systems overlap nothing and share no frame
        out.append((x + shift[0], y + shift[1], z + shift[2], vx, vy, vz, m))
    return out


def new_sim(pkg, **kw):
    return pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.01, theta=0.6, dt=1e-3), leaf_capacity=16, **kw)


def concat(parts):
    return [np.concatenate([p[c] for p in parts]) for c in range(7)]


@pytest.mark.parametrize("sizes", [(1024, 3000, 777), (2048,) * 9])
def test_each_system_equals_the_system_alone(pkg, ic, sizes):
    parts = systems(ic, sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    ens = new_sim(pkg)
    ens.set_particles(*concat(parts))
    ens.set_ensemble(off)
    a_ens = ens.compute_accel()
    st = ens.stats()
    pairs = 0
    for k, p in enumerate(parts):
        with new_sim(pkg) as one:
            one.set_particles(*p)
            a_one = one.compute_accel()
            pairs += one.stats()["p2p_pairs"]
        for c in range(3):
            np.testing.assert_array_equal(a_ens[c][off[k]:off[k + 1]], a_one[c])
    assert st["p2p_pairs"] == pairs
    ens.close()


def test_each_system_matches_the_oracle_on_that_system(pkg, ic, oracle):
    """Pinned per system against the oracle, not only against the
    single-system GPU path: every system of an uneven ensemble has the
    oracle's accelerations (the reference's grouped walk at the same theta
    and leaf capacity, FP64) and its interaction counts."""
    sizes = (1024, 3000, 777, 2048)
    parts = systems(ic, sizes, seed0=60)
    off = np.concatenate([[0], np.cumsum(sizes)])
    with new_sim(pkg) as ens:
        ens.set_particles(*concat(parts))
        ens.set_ensemble(off)
        ax, ay, az = ens.compute_accel()
        st = ens.stats()
    pairs = terms = 0
    for k, (x, y, z, _, _, _, m) in enumerate(parts):
        rx, ry, rz, cnt = oracle.bh_accel(x, y, z, m, 1.0, 0.01, 0.6, 16, counters=True)
        sl = slice(off[k], off[k + 1])
        e = rel_err(ax[sl], ay[sl], az[sl], rx, ry, rz)
        assert np.median(e) <= 1e-5 and e.max() <= 1e-4, (k, np.median(e), e.max())
        pairs += cnt["p2p_pairs"]
        terms += cnt["p2c_terms"]
    assert st["p2p_pairs"] == pairs and st["p2c_terms"] == terms


def test_ensemble_kdk_and_checks(pkg, ic):
    sizes = (1500, 4096, 2048, 999, 3333)
    parts = systems(ic, sizes, seed0=40)
    off = np.concatenate([[0], np.cumsum(sizes)])
    ens = new_sim(pkg)
    ens.set_particles(*concat(parts))
    ens.set_ensemble(off)
    ens.prime()
    ens.step(4, 1e-3)
    rms, mx = ens.ensemble_force_error(256, seed=5)
    diags = ens.ensemble_diagnostics(exact_potential=True)
    state = ens.state()
    for k, p in enumerate(parts):
        with new_sim(pkg) as one:
            one.set_particles(*p)
            one.prime()
            one.step(4, 1e-3)
            s1 = one.state()
            d1 = one.diagnostics(exact_potential=True)
            fe = one.force_error(min(256, sizes[k]), seed=5)
        for c in range(6):
            np.testing.assert_allclose(state[c][off[k]:off[k + 1]], s1[c], rtol=0, atol=1e-12)
        assert diags[k]["energy"] == pytest.approx(d1["energy"], rel=1e-9)
        np.testing.assert_allclose(diags[k]["L"], d1["L"], rtol=1e-9, atol=1e-13)
        np.testing.assert_allclose(diags[k]["com"], d1["com"], atol=1e-12)
        assert 0.0 < rms[k] < 1e-2 and rms[k] <= mx[k]
        assert rms[k] == pytest.approx(fe["rms"], rel=0.5)  # different samples, same error level
    ens.close()


def test_ensemble_steps_are_graph_replays(pkg, ic):
    sizes = (2048, 1024, 4096)
    parts = systems(ic, sizes, seed0=70)
    ens = new_sim(pkg)
    ens.set_particles(*concat(parts))
    ens.set_ensemble(np.concatenate([[0], np.cumsum(sizes)]))
    ens.prime()
    ens.step(5, 1e-3)
    st = ens.stats()
    assert st["graph_captures"] == 2 and st["graph_replays"] == 3
    ens.close()


def test_ensemble_argument_checks(pkg, ic):
    sim = new_sim(pkg)
    sim.set_particles(*concat(systems(ic, (100, 200))))
    with pytest.raises(pkg.NgravError):
        sim.set_ensemble([0, 150, 250])  # does not end at n
    with pytest.raises(pkg.NgravError):
        sim.set_ensemble([0, 200, 100, 300])  # decreasing
    sim.set_ensemble([0, 100, 300])
    sim.compute_accel()
    sim.close()
