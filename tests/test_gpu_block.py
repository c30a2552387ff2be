"""Block (power-of-two rung) timesteps on the GPU (System::BlockStep,
include/ngrav/System.hpp:239-294) against the reference's output
(tests/golden/block4k.npz) and the oracle.

Each coarse step assigns rungs from the current |a|, drifts everyone by the
finest substep, and refreshes the forces of the particles whose rung step
ends there with the geometric per-particle walk on a rebuilt tree; every
particle ends the step with a fresh acceleration."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

STATE = ("x", "y", "z", "vx", "vy", "vz")


def sim_for(pkg, d, precision):
    s = pkg.NBodySystem(pkg.StepParams(G=float(d["G"]), eps=float(d["eps"]), theta=float(d["theta"])),
                        leaf_capacity=8, precision=precision)
    s.set_particles(*(d[k] for k in STATE), d["m"])
    return s


@pytest.mark.parametrize("precision", ["split", "plain"])
@pytest.mark.parametrize("tag", ["r8", "r1"])
def test_block_step_matches_reference(pkg, tag, precision):
    d = load_golden("block4k.npz")
    prec = pkg.PRECISION_SPLIT if precision == "split" else pkg.PRECISION_PLAIN
    dt, eta, max_rung = float(d["dt"]), float(d["eta"]), int(d[f"{tag}_max_rung"])
    with sim_for(pkg, d, prec) as sim:
        sim.prime()
        for _ in range(int(d[f"{tag}_steps"])):
            rmax = sim.block_step(dt, eta=eta, max_rung=max_rung)
        rung = sim.rungs()
        st = sim.state()
        acc = sim.accel()
    want_rung = d[f"{tag}_rung"]
    assert rmax == want_rung.max()
    # rungs come from ceil(log2(dt / tau)): only a particle whose |a| sits
    # within FP32 rounding of a rung boundary may land one rung off
    assert np.mean(rung == want_rung) >= 0.999 and np.all(np.abs(rung - want_rung) <= 1)
    same = rung == want_rung
    e = rel_err(*acc, *(d[f"{tag}_{k}"] for k in ("ax", "ay", "az")))[same]
    assert np.median(e) <= 1e-5 and e.max() <= 1e-4, (np.median(e), e.max())
    # positions and velocities: FP32 forces over a coarse step of 0.01
    vscale = np.sqrt(sum(d[f"{tag}_{k}"] ** 2 for k in ("vx", "vy", "vz")))[same]
    dv = np.sqrt(sum((st[3 + c] - d[f"{tag}_{k}"]) ** 2 for c, k in enumerate(("vx", "vy", "vz"))))[same]
    assert np.median(dv / vscale) <= 1e-5 and np.max(dv / vscale) <= 1e-3
    dx = np.sqrt(sum((st[c] - d[f"{tag}_{k}"]) ** 2 for c, k in enumerate(("x", "y", "z"))))[same]
    if precision == "split":
        assert np.max(dx) <= 1e-6, np.max(dx)
    else:  # FP32 positions: each of up to 16 drifts rounds to half an ulp of |x|
        r = np.sqrt(sum(d[f"{tag}_{k}"] ** 2 for k in ("x", "y", "z")))[same]
        assert np.all(dx <= 2e-6 + 16 * 2.0 ** -24 * r), np.max(dx / (2e-6 + 16 * 2.0 ** -24 * r))


def test_block_step_matches_oracle_from_gpu_state(pkg, oracle):
    """One more block step from the GPU's own state and a(t), against the
    oracle restarted from that same state: isolates one step's error."""
    d = load_golden("block4k.npz")
    G, eps, th, dt, eta = (float(d[k]) for k in ("G", "eps", "theta", "dt", "eta"))
    with sim_for(pkg, d, pkg.PRECISION_SPLIT) as sim:
        sim.prime()
        sim.block_step(dt, eta=eta, max_rung=8)
        st0, a0 = sim.state(), sim.accel()
        sim.block_step(dt, eta=eta, max_rung=8)
        st1, a1, r1 = sim.state(), sim.accel(), sim.rungs()
    so, ao, ro, _ = oracle.block_step(st0, d["m"], G, eps, th, 8, dt, eta, 8, a0)
    assert np.mean(r1 == ro) >= 0.999
    same = r1 == ro
    e = rel_err(*a1, *ao)[same]
    assert np.median(e) <= 1e-5 and e.max() <= 1e-4, (np.median(e), e.max())
    dx = np.sqrt(sum((st1[c] - so[c]) ** 2 for c in range(3)))[same]
    assert np.max(dx) <= 1e-6


def test_block_step_energy_and_rung_zero_limit(pkg, ic):
    """Energy stays conserved over block steps; with max rung 0 a block step
    is one global KDK step (closing forces from the per-particle walk)."""
    x, y, z, vx, vy, vz, m = ic.plummer(8192, seed=21)
    sp = pkg.StepParams(G=1.0, eps=0.01, theta=0.5)
    with pkg.NBodySystem(sp, leaf_capacity=8) as sim:
        sim.set_particles(x, y, z, vx, vy, vz, m)
        sim.prime()
        e0 = sim.diagnostics(exact_potential=True)["energy"]
        for _ in range(5):
            rmax = sim.block_step(0.01, eta=0.025, max_rung=6)
        e1 = sim.diagnostics(exact_potential=True)["energy"]
        assert rmax >= 2
        assert abs(e1 - e0) < 2e-4 * abs(e0), (e0, e1)
    a = pkg.NBodySystem(sp, leaf_capacity=8)
    b = pkg.NBodySystem(sp, leaf_capacity=8)
    for s in (a, b):
        s.set_particles(x, y, z, vx, vy, vz, m)
        s.prime()
    assert a.block_step(1e-3, eta=0.025, max_rung=0) == 0
    assert np.all(a.rungs() == 0)
    b.step(1, 1e-3)
    sa, sb = a.state(), b.state()
    # the same KDK step; the closing forces differ only by the grouped vs
    # per-particle walk's opening decisions
    dv = np.sqrt(sum((sa[c] - sb[c]) ** 2 for c in (3, 4, 5)))
    v = np.sqrt(sum(sb[c] ** 2 for c in (3, 4, 5)))
    assert np.median(dv / v) < 1e-5
    for c in range(3):
        np.testing.assert_allclose(sa[c], sb[c], rtol=0, atol=1e-7)
    a.close()
    b.close()


def test_block_step_argument_checks(pkg, ic):
    x, y, z, vx, vy, vz, m = ic.plummer(256, seed=1)
    with pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.01, theta=0.5)) as sim:
        sim.set_particles(x, y, z, vx, vy, vz, m)
        with pytest.raises(pkg.NgravError):
            sim.block_step(0.0)
        with pytest.raises(pkg.NgravError):
            sim.block_step(0.01, eta=-1.0)
        with pytest.raises(pkg.NgravError):
            sim.block_step(0.01, max_rung=-1)
        assert np.all(sim.rungs() == 0)
        sim.block_step(0.01)  # primes itself
