"""The learned opening test on the GPU, against the oracle (oracle/lmac_oracle.py).

* tensor-core forward pass (BF16, tcgen05) vs the oracle's BF16 emulation,
  and the FP32 forward pass vs FP64;
* the training gradient vs the oracle's analytic gradient;
* features and exact-vs-multipole labels of recorded pairs vs FP64 numpy on
  the exported tree;
* the learned walk with the network silenced (gate above every logit) makes
  exactly the geometric walk's decisions: identical interaction counts;
* GPU training lowers the loss and classifies held-out pairs; the trained
  test runs inside the walk, within the error budget, and the FP64 check
  reverts the run to the geometric test when its threshold is breached.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import lmac_oracle as lo  # noqa: E402

pytestmark = pytest.mark.gpu


def plummer_system(pkg, ic, n, seed=3, ncrit=16, eps=0.01, theta=0.5, retest=True):
    x, y, z, vx, vy, vz, m = ic.plummer(n, seed=seed)
    sim = pkg.NBodySystem(pkg.StepParams(G=1.0, eps=eps, theta=theta), leaf_capacity=ncrit,
                          fp64_mac_retest=retest)
    sim.set_particles(x, y, z, vx, vy, vz, m)
    return sim, (x, y, z, vx, vy, vz, m)


def random_model(seed):
    rng = np.random.default_rng(seed)
    P = (rng.standard_normal(lo.NPARAMS) * 0.4).astype(np.float32)
    norm = np.concatenate([rng.standard_normal(8) * 0.5, 0.5 + rng.random(8)]).astype(np.float32)
    return P, norm


def test_tc_forward_matches_bf16_emulation(pkg, ic):
    sim, _ = plummer_system(pkg, ic, 1024)
    P, norm = random_model(7)
    sim.lmac_set_model(P, norm)
    rng = np.random.default_rng(11)
    n = 1000  # not a multiple of the 256-pair flush
    X = (rng.standard_normal((n, 8)) * 2.0).astype(np.float32)
    z_tc = sim.lmac_forward_tc(X)
    z_em = lo.forward_bf16(P, norm, X)
    np.testing.assert_allclose(z_tc, z_em, rtol=2e-2, atol=2e-2 * (1 + np.abs(z_em).mean()))
    # and the FP32 path on standardised inputs against FP64
    xs = (X - norm[:8]) * norm[8:]
    z32 = sim.lmac_forward(xs)
    z64, _ = lo.forward(P, xs.astype(np.float64))
    np.testing.assert_allclose(z32, z64, rtol=1e-4, atol=1e-4)
    # BF16 quantisation moves logits, but not far
    assert np.median(np.abs(z_tc - z64)) < 0.05 * (1 + np.median(np.abs(z64)))
    sim.close()


def test_grad_matches_oracle(pkg, ic):
    sim, _ = plummer_system(pkg, ic, 1024)
    rng = np.random.default_rng(5)
    P, _ = random_model(3)
    n = 1000
    X = rng.standard_normal((n, 8)).astype(np.float32)
    y = (rng.random(n) < 0.4).astype(np.float32)
    w = (rng.random(n) < 0.9).astype(np.float32)
    g, loss = sim.lmac_grad(X, y, w, params=P, scale=1.0 / n)
    g_ref, loss_ref = lo.grad(P.astype(np.float64), X.astype(np.float64), y, w, scale=1.0 / n)
    assert loss == pytest.approx(loss_ref, rel=1e-5)
    np.testing.assert_allclose(g, g_ref, rtol=1e-3, atol=1e-6 * np.abs(g_ref).max())
    sim.close()


def node_members(tree, v):
    L = int(tree["level"][v])
    if L == 0:
        return np.arange(len(tree["keys"]))
    return np.nonzero((tree["keys"] >> np.uint64(3 * (21 - L))) == tree["prefix"][v])[0]


def test_features_and_labels_match_oracle(pkg, ic):
    sim, (x, y, z, _, _, _, m) = plummer_system(pkg, ic, 8192, ncrit=8)
    sim.compute_accel()
    rec = sim.lmac_collect(theta_record=0.3, rho_lo=0.25, rho_hi=1.25, keep=1.0, seed=2, cap=1 << 20)
    assert len(rec["r"]) > 1000 and rec["nband"] == len(rec["r"])
    tree = sim.debug_tree()
    ax, ay, az = sim.accel()
    amag = np.sqrt(ax ** 2 + ay ** 2 + az ** 2)
    pos = np.stack([x, y, z], 1).astype(np.float64)
    mm = np.asarray(m, np.float64)
    rng = np.random.default_rng(0)
    pick = rng.choice(len(rec["r"]), 400, replace=False)
    g_idx, n_idx = rec["group"][pick], rec["node"][pick]
    members = [node_members(tree, int(v)) for v in g_idx]
    amin = np.array([amag[mb].min() for mb in members])
    f, worst = lo.features(tree["com"][g_idx], tree["max_radius"][g_idx], amin, tree["com"][n_idx],
                           tree["mass"][n_idx], tree["max_radius"][n_idx], 2 * tree["half"][n_idx],
                           tree["quad"][n_idx], tree["count"][n_idx], 1.0, 0.01)
    assert np.all(worst > 0)
    Xg = rec["X"][pick]
    np.testing.assert_allclose(Xg[:, [0, 1, 2, 3, 7]], f[:, [0, 1, 2, 3, 7]], atol=1e-4)
    np.testing.assert_allclose(Xg[:, 6], f[:, 6], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(Xg[:, 4:6], f[:, 4:6], rtol=1e-3, atol=1e-5)
    checked = 0
    for k in range(len(pick)):
        nm = node_members(tree, int(n_idx[k]))
        if len(nm) > 4096:
            continue
        gm = members[k]
        r_ref = lo.label(pos[gm], amag[gm], pos[nm], mm[nm], tree["com"][n_idx[k]], tree["mass"][n_idx[k]],
                         tree["quad"][n_idx[k]], 1.0, 0.01)
        scale = tree["mass"][n_idx[k]] / worst[k] ** 2 / amag[gm].min()  # |a_node| / |a| at the nearest member
        assert abs(rec["r"][pick[k]] - r_ref) <= 1e-2 * r_ref + 2e-6 * scale, (k, rec["r"][pick[k]], r_ref)
        checked += 1
    assert checked > 300
    sim.close()


def test_silenced_network_reproduces_geometric_walk(pkg, ic):
    n, theta = 65536, 0.5
    sim, arrs = plummer_system(pkg, ic, n, theta=theta, retest=False)
    a_geo = sim.compute_accel()
    s_geo = sim.stats()
    P, norm = random_model(9)
    sim.lmac_set_model(P, norm)
    # rho_lo below theta, rho_hi above: outside the band both tests agree;
    # inside it the gate silences the network, so the geometric test decides.
    sim.lmac_set_opts(gate=1e30, rho_lo=0.25, rho_hi=1.25, check_every=0, screen=0.0)
    sim.set_opts(mac=pkg.MAC_LEARNED)
    a_lm = sim.compute_accel()
    s_lm = sim.stats()
    assert s_lm["lmac_queries"] > 0 and s_lm["lmac_fallbacks"] == s_lm["lmac_queries"]
    assert s_lm["lmac_flushes"] > 0
    assert s_lm["p2p_pairs"] == s_geo["p2p_pairs"] and s_lm["p2c_terms"] == s_geo["p2c_terms"]
    ref = np.sqrt(sum(c ** 2 for c in a_geo))
    err = np.sqrt(sum((u - v) ** 2 for u, v in zip(a_lm, a_geo))) / ref
    assert np.max(err) < 1e-5  # same interactions, summed in another order
    sim.close()


def test_training_and_learned_walk(pkg, ic):
    n = 65536
    sim, _ = plummer_system(pkg, ic, n, ncrit=16, theta=0.5)
    rep = sim.lmac_train(snapshots=2, steps_between=0, pairs=1 << 17, epochs=3, batch=4096, seed=4)
    assert rep["pairs"] > 100000
    assert rep["loss_last"] < 0.7 * rep["loss_first"]
    assert rep["val_acc"] > 0.8
    sim.lmac_set_opts(budget=3e-5, check_every=0)
    sim.set_opts(mac=pkg.MAC_LEARNED)
    sim.compute_accel()
    st = sim.stats()
    assert st["lmac_active"] == 1 and st["lmac_queries"] > 0
    fe = sim.force_error(2048, seed=9, fp64_pairs=True)
    assert np.isfinite(fe["rms"]) and fe["rms"] < 5e-3
    # the FP64 check: an unreachable threshold reverts the run after one evaluation
    sim.lmac_set_opts(budget=3e-5, check_every=1, check_targets=512, revert_rms=1e-12)
    sim.compute_accel()
    st = sim.stats()
    assert st["lmac_reverted"] == 1 and st["lmac_checks"] == 1 and st["lmac_last_check_rms"] > 0
    sim.compute_accel()
    assert sim.stats()["lmac_queries"] == 0  # geometric test from now on
    sim.lmac_reset()
    sim.compute_accel()
    assert sim.stats()["lmac_queries"] > 0
    sim.close()


def test_error_bound_screen_is_safe(pkg, ic):
    """Pairs the quadrupole truncation bound accepts without the network meet
    the budget: with a budget so small that the network opens nearly
    everything, screening only removes queries, it does not add error."""
    n = 65536
    sim, _ = plummer_system(pkg, ic, n, ncrit=16, theta=0.5)
    sim.lmac_train(snapshots=2, steps_between=0, pairs=1 << 16, epochs=2, batch=4096, seed=2)
    sim.set_opts(mac=pkg.MAC_LEARNED)
    out = {}
    for screen in (0.0, 1.0):
        sim.lmac_set_opts(budget=1e-4, check_every=0, screen=screen)
        sim.compute_accel()
        st = sim.stats()
        out[screen] = (st, sim.force_error(2048, seed=3, fp64_pairs=True))
    assert out[0.0][0]["lmac_screened"] == 0
    assert out[1.0][0]["lmac_screened"] > 0
    assert out[1.0][0]["lmac_queries"] < out[0.0][0]["lmac_queries"]
    assert out[1.0][1]["rms"] <= 1.2 * out[0.0][1]["rms"] + 1e-6
    sim.close()
