"""Pins the oracle (the C restatement) against the reference's own outputs.

The golden fixtures were produced by the reference's CPU path compiled from
its sources (tests/golden/make_golden.py).  These checks run on the CPU.
"""
import numpy as np
import pytest

from conftest import TREE_EXACT, edge_cases, golden_tree, load_golden, rel_err


def _check_tree(O, x, y, z, m, ncrit, gold):
    t = O.tree(x, y, z, m, ncrit)
    c = t.canonical()
    for k in TREE_EXACT:
        assert np.array_equal(c[k], gold[k]), k
    assert np.array_equal(t["order"], gold["order"])
    np.testing.assert_allclose(c["mass"], gold["mass"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(c["com"], gold["com"], rtol=0, atol=1e-13 * max(1.0, np.abs(gold["com"]).max()))
    np.testing.assert_allclose(c["max_radius"], gold["max_radius"], rtol=1e-12, atol=1e-14)
    qs = gold["mass"].max() * gold["half"].max() ** 2  # natural scale of a quadrupole
    np.testing.assert_allclose(c["quad"], gold["quad"], rtol=0, atol=1e-12 * qs)


def test_plummer16k_tree_and_accel(oracle):
    d = load_golden("plummer16k.npz")
    args = (d["x"], d["y"], d["z"], d["m"])
    _check_tree(oracle, *args, int(d["ncrit"]), golden_tree(d))
    ax, ay, az, cnt = oracle.bh_accel(*args, float(d["G"]), float(d["eps"]), float(d["theta"]), int(d["ncrit"]),
                                      counters=True)
    e = rel_err(ax, ay, az, d["ax"], d["ay"], d["az"])
    assert e.max() < 1e-12
    assert cnt["groups"] == int(np.sum(d["tree_is_leaf"]))


def test_plummer16k_direct(oracle):
    d = load_golden("plummer16k.npz")
    ax, ay, az = oracle.direct(d["x"], d["y"], d["z"], d["m"], float(d["G"]), float(d["eps"]))
    assert rel_err(ax, ay, az, d["dax"], d["day"], d["daz"]).max() < 1e-12


def test_plummer16k_leapfrog_and_diagnostics(oracle):
    d = load_golden("plummer16k.npz")
    st = (d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"])
    (x, y, z, vx, vy, vz), _ = oracle.leapfrog(st, d["m"], float(d["G"]), float(d["eps"]), float(d["theta"]),
                                               int(d["ncrit"]), float(d["dt"]), int(d["steps"]))
    for a, k in zip((x, y, z, vx, vy, vz), ("kdk_x", "kdk_y", "kdk_z", "kdk_vx", "kdk_vy", "kdk_vz")):
        np.testing.assert_allclose(a, d[k], rtol=0, atol=1e-12)
    diag = oracle.diagnostics(d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"], d["m"], float(d["G"]),
                              float(d["eps"]))
    np.testing.assert_allclose(diag, d["diag0"], rtol=1e-11, atol=1e-14)


def test_selftest_theta0_matches_direct(oracle):
    """The reference's own gate (SelfTest.cpp:43-74): BH at theta 0 equals Direct to 1e-12."""
    d = load_golden("selftest_uniform1000.npz")
    args = (d["x"], d["y"], d["z"], d["m"])
    _check_tree(oracle, *args, 8, golden_tree(d))
    ax, ay, az = oracle.bh_accel(*args, 1.0, 0.02, 0.0, 8)
    assert rel_err(ax, ay, az, d["dax"], d["day"], d["daz"]).max() <= 1e-12
    assert rel_err(ax, ay, az, d["ax"], d["ay"], d["az"]).max() <= 1e-13


def test_selftest_quadrupole_gain(oracle):
    """The reference's own gate (SelfTest.cpp:212-265): quadrupole cuts max error >= 3x."""
    d = load_golden("selftest_ball4000.npz")
    args = (d["x"], d["y"], d["z"], d["m"])
    _check_tree(oracle, *args, 8, golden_tree(d))
    errs = {}
    for tag, quad in (("mono", False), ("quad", True)):
        ax, ay, az = oracle.bh_accel(*args, 1.0, 0.01, 0.5, 8, quad=quad)
        assert rel_err(ax, ay, az, d[f"{tag}_ax"], d[f"{tag}_ay"], d[f"{tag}_az"]).max() < 1e-12
        errs[tag] = rel_err(ax, ay, az, d["dax"], d["day"], d["daz"]).max()
    assert errs["mono"] / errs["quad"] >= 3.0


@pytest.mark.parametrize("name", edge_cases()[0])
def test_edge_cases(oracle, name):
    _, d = edge_cases()
    x, y, z, m = (d[f"{name}_{k}"] for k in "xyzm")
    ncrit = int(d[f"{name}_ncrit"])
    _check_tree(oracle, x, y, z, m, ncrit, golden_tree(d, f"{name}_tree"))
    ax, ay, az = oracle.bh_accel(x, y, z, m, 1.0, 0.05, 0.5, ncrit)
    gx, gy, gz = d[f"{name}_ax"], d[f"{name}_ay"], d[f"{name}_az"]
    np.testing.assert_allclose(np.stack([ax, ay, az]), np.stack([gx, gy, gz]), rtol=1e-12,
                               atol=1e-12 * max(1e-300, np.abs(np.stack([gx, gy, gz])).max()))


def test_oracle_spline_softening_matches_reference(oracle):
    """Cubic-spline softening (Softening.hpp:30-56): the C restatement against
    the reference's own output on the same Plummer sphere."""
    d = load_golden("spline4k.npz")
    oracle.set_softening(1)
    try:
        G, h, th, nc = float(d["G"]), float(d["eps"]), float(d["theta"]), int(d["ncrit"])
        ax, ay, az = oracle.bh_accel(d["x"], d["y"], d["z"], d["m"], G, h, th, nc)
        for got, want in ((ax, d["ax"]), (ay, d["ay"]), (az, d["az"])):
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
        dx, dy, dz = oracle.direct(d["x"], d["y"], d["z"], d["m"], G, h)
        np.testing.assert_allclose(dx, d["dax"], rtol=0, atol=1e-12 * np.abs(d["dax"]).max())
        diag = oracle.diagnostics(d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"], d["m"], G, h)
        assert diag[0] == pytest.approx(d["diag0"][0], rel=1e-12)
    finally:
        oracle.set_softening(0)


def test_oracle_per_particle_walk_matches_reference(oracle):
    """WalkBH (Solvers.cpp:181-227): relative MAC with a given previous |a|, and
    the geometric walk on a target subset, against the reference's output."""
    d = load_golden("pp4k.npz")
    G, eps, th, nc = float(d["G"]), float(d["eps"]), float(d["theta"]), int(d["ncrit"])
    rx, ry, rz = oracle.bh_pp_accel(d["x"], d["y"], d["z"], d["m"], G, eps, th, nc, relative=True,
                                    alpha=float(d["alpha"]), aold=d["aold"])
    for got, want in ((rx, d["rel_ax"]), (ry, d["rel_ay"]), (rz, d["rel_az"])):
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
    t = d["targets"].astype(bool)
    gx, gy, gz = oracle.bh_pp_accel(d["x"], d["y"], d["z"], d["m"], G, eps, th, nc, targets=t)
    for got, want in ((gx, d["tgt_ax"]), (gy, d["tgt_ay"]), (gz, d["tgt_az"])):
        np.testing.assert_allclose(got[t], want[t], rtol=0, atol=1e-12 * np.abs(want).max())
    # the relative MAC meets its purpose: error well below the geometric walk's at this alpha
    e = rel_err(rx, ry, rz, d["dax"], d["day"], d["daz"])
    assert np.sqrt(np.mean(e ** 2)) < 5e-3


def test_oracle_block_step_matches_reference(oracle):
    """System::BlockStep (System.hpp:239-294): rungs, state and a(t + dt) after
    block steps (max rung 8, two steps; max rung 1, one step) against the
    reference's output."""
    d = load_golden("block4k.npz")
    G, eps, th, dt, eta = (float(d[k]) for k in ("G", "eps", "theta", "dt", "eta"))
    st0 = tuple(d[k] for k in ("x", "y", "z", "vx", "vy", "vz"))
    for tag in ("r8", "r1"):
        st, acc = st0, oracle.bh_accel(d["x"], d["y"], d["z"], d["m"], G, eps, th, 8)
        for _ in range(int(d[f"{tag}_steps"])):
            st, acc, rung, rmax = oracle.block_step(st, d["m"], G, eps, th, 8, dt, eta, int(d[f"{tag}_max_rung"]), acc)
        np.testing.assert_array_equal(rung, d[f"{tag}_rung"])
        assert rmax == d[f"{tag}_rung"].max() and rmax <= int(d[f"{tag}_max_rung"])
        for k, got in zip(("x", "y", "z", "vx", "vy", "vz"), st):
            want = d[f"{tag}_{k}"]
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
        for k, got in zip(("ax", "ay", "az"), acc):
            want = d[f"{tag}_{k}"]
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
    assert len(np.unique(d["r8_rung"])) >= 3  # several rungs in use
