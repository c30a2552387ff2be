"""Cubic-spline softening (Hernquist & Katz; Softening.hpp:30-56) on the GPU
against the reference's own output (tests/golden/spline4k.npz)."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def spline_sim(pkg, d, precision):
    prec = pkg.PRECISION_SPLIT if precision == "split" else pkg.PRECISION_PLAIN
    s = pkg.NBodySystem(pkg.StepParams(G=float(d["G"]), eps=float(d["eps"]), theta=float(d["theta"]),
                                       dt=float(d["dt"])), leaf_capacity=int(d["ncrit"]), precision=prec)
    s.set_softening(pkg.SOFTENING_SPLINE)
    s.set_particles(d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"], d["m"])
    return s


@pytest.mark.parametrize("precision", ["split", "plain"])
def test_spline_accelerations_match_reference(pkg, precision):
    d = load_golden("spline4k.npz")
    with spline_sim(pkg, d, precision) as sim:
        ax, ay, az = sim.compute_accel()
        fe = sim.force_error(1024, seed=3, fp64_pairs=True)
    e = rel_err(ax, ay, az, d["ax"], d["ay"], d["az"])
    assert np.median(e) <= 1e-5 and e.max() <= 1e-4, (np.median(e), e.max())
    # the sampler's direct sum is the spline one too: same error level as the reference BH's
    e_ref = rel_err(d["ax"], d["ay"], d["az"], d["dax"], d["day"], d["daz"])
    assert fe["rms"] == pytest.approx(np.sqrt(np.mean(e_ref ** 2)), rel=0.5)


def test_spline_kdk_and_energy(pkg):
    d = load_golden("spline4k.npz")
    with spline_sim(pkg, d, "split") as sim:
        g0 = sim.diagnostics(exact_potential=True)
        sim.prime()
        sim.step(int(d["steps"]), float(d["dt"]))
        x, y, z, vx, vy, vz = sim.state()
        g10 = sim.diagnostics(exact_potential=True)
    assert g0["energy"] == pytest.approx(d["diag0"][0], rel=1e-10)
    assert g10["energy"] == pytest.approx(d["diag10"][0], rel=1e-6)
    dpos = np.sqrt((x - d["kdk_x"]) ** 2 + (y - d["kdk_y"]) ** 2 + (z - d["kdk_z"]) ** 2)
    assert dpos.max() <= 2e-6, dpos.max()


def test_spline_needs_positive_eps(pkg):
    s = pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.0, theta=0.5))
    with pytest.raises(pkg.NgravError):
        s.set_softening(pkg.SOFTENING_SPLINE)
    s.close()
