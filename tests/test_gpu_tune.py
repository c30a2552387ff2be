"""The autotuner: candidates it times, the error constraint it keeps, and the
kernel shapes it switches between (which change speed, never the result)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def plummer(pkg, ic, n=65536, ncrit=16):
    sim = pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.01, theta=0.6), leaf_capacity=ncrit)
    sim.set_particles(*ic.plummer(n, seed=21))
    return sim


def test_autotune_keeps_the_error_bar_and_does_not_slow_down(pkg, ic):
    sim = plummer(pkg, ic)
    rep = sim.autotune(reps=2, check_targets=1024, rms_tolerance=1.1)
    assert rep["leaf_capacity"] in (8, 12, 16, 24, 32, 48)
    assert rep["p2p_tile"] in (64, 128, 256) and rep["walk_stack"] in (1024, 2048, 4096)
    assert rep["rms_after"] <= 1.1 * rep["rms_before"] * 1.02
    checked = [t for t in rep["tried"] if t[4] >= 0]
    assert len(rep["tried"]) >= 8 and len(checked) >= 6
    # the choice is the fastest admissible leaf capacity among those measured
    ok = [t for t in checked if t[4] <= 1.1 * rep["rms_before"]]
    assert rep["leaf_capacity"] == min(ok, key=lambda t: t[3])[0] or rep["ms_after"] <= min(t[3] for t in ok) * 1.1
    assert sim.opts.leaf_capacity == rep["leaf_capacity"]
    sim.close()


@pytest.mark.parametrize("tile,stack", [(64, 1024), (128, 4096), (256, 2048)])
def test_kernel_shapes_change_speed_not_results(pkg, ic, tile, stack):
    sim = plummer(pkg, ic, n=32768)
    a0 = sim.compute_accel()
    s0 = sim.stats()
    sim.set_tuning(p2p_tile=tile, walk_stack=stack)
    a1 = sim.compute_accel()
    s1 = sim.stats()
    assert s1["p2p_pairs"] == s0["p2p_pairs"] and s1["p2c_terms"] == s0["p2c_terms"]
    ref = np.sqrt(sum(c ** 2 for c in a0))
    err = np.sqrt(sum((u - v) ** 2 for u, v in zip(a1, a0))) / ref
    assert err.max() < 1e-5
    with pytest.raises(pkg.NgravError):
        sim.set_tuning(p2p_tile=100, walk_stack=2048)
    sim.close()
