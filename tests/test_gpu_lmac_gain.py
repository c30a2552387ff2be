"""What the trained network adds to the learned opening test, at equal error.

Three arms on one system (the two-component galaxy, 262,144 bodies, eps
0.002, leaf capacity 32), each calibrated by bisection to the same rms
relative force error, 1e-3 within 3 % (direct sum with FP64 sums on 4,096
targets):
  theta    the reference's geometric group test alone
           (include/ngrav/Mac.hpp:25-29, src/Solvers.cpp:261-271), theta
           bisected;
  screen   the learned walk with the network silenced (gate above every
           logit): band pairs the quadrupole error bound does not accept
           fall to the geometric test at the theta arm's theta; budget
           bisected;
  network  the learned walk with the network trained on this system (the
           method), the same fallback theta; budget bisected.
The network arm must do the least work of the three: the fewest algorithmic
flops (20 per P2P pair + 60 per P2C term, device counters) and the lowest
event-timed force evaluation (all phases, best of five).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TARGET, TOL = 1e-3, 0.03


def rms_now(sim):
    sim.compute_accel()
    return sim.force_error(4096, seed=2024, fp64_pairs=False)["rms"]


def bisect(sim, setter, lo, hi, log):
    """Knob value whose rms is within TOL of TARGET (rms grows with the knob)."""
    best = None
    for _ in range(24):
        mid = float(np.sqrt(lo * hi)) if log else 0.5 * (lo + hi)
        setter(mid)
        r = rms_now(sim)
        if best is None or abs(r / TARGET - 1) < abs(best[1] / TARGET - 1):
            best = (mid, r)
        if abs(r / TARGET - 1) <= TOL:
            return mid, r
        if r < TARGET:
            lo = mid
        else:
            hi = mid
    raise AssertionError(f"no setting within {TOL:.0%} of the target rms (closest {best})")


def cost(sim):
    """(algorithmic flops, best event-timed evaluation ms) of the current setting."""
    ms = []
    for _ in range(5):
        sim.compute_accel()
        st = sim.stats()
        ms.append(sum(st[k] for k in ("ms_bbox_keys", "ms_sort", "ms_build", "ms_moments", "ms_walk", "ms_force")))
    return 20.0 * st["p2p_pairs"] + 60.0 * st["p2c_terms"], min(ms), st


def test_trained_network_beats_screen_and_theta_at_equal_error(pkg, ic):
    arrs = ic.galaxy(n_halo=235930, n_disk=26214, seed=8)
    with pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.002, theta=0.6, dt=2e-4), leaf_capacity=32,
                         timing=True) as sim:
        sim.set_particles_f32(*arrs)
        rep = sim.lmac_train(snapshots=4, steps_between=1, dt=2e-4, pairs=1 << 20, epochs=4, batch=8192, seed=1)
        assert rep["val_acc"] > 0.8
        model = sim.lmac_get_model()
        sim.set_particles_f32(*arrs)  # training stepped the system
        sim.prime()

        # theta alone
        sim.set_opts(mac=pkg.MAC_GEOMETRIC)
        theta, r_theta = bisect(sim, lambda v: sim.set_opts(theta=v), 0.3, 1.0, log=False)
        f_theta, ms_theta, _ = cost(sim)

        # error-bound screen, the rest to the geometric test at that theta
        sim.lmac_set_model(*model)
        sim.set_opts(mac=pkg.MAC_LEARNED, theta=theta)
        silent = dict(gate=1e30, check_every=0)
        b_s, r_s = bisect(sim, lambda v: sim.lmac_set_opts(budget=v, **silent), 1e-6, 1e-1, log=True)
        f_s, ms_s, st_s = cost(sim)
        assert st_s["lmac_fallbacks"] == st_s["lmac_queries"]  # the network decided nothing

        # the method: screen + trained network
        b_n, r_n = bisect(sim, lambda v: sim.lmac_set_opts(budget=v, check_every=0), 1e-6, 1e-1, log=True)
        f_n, ms_n, st_n = cost(sim)
        assert st_n["lmac_queries"] > 0 and st_n["lmac_accepts"] > 0

    report = (f"theta {theta:.4f} rms {r_theta:.3e}: {f_theta:.3e} flop {ms_theta:.2f} ms | "
              f"screen {b_s:.3e} rms {r_s:.3e}: {f_s:.3e} flop {ms_s:.2f} ms | "
              f"network {b_n:.3e} rms {r_n:.3e}: {f_n:.3e} flop {ms_n:.2f} ms")
    print(report)
    assert f_n < f_s and f_n < f_theta, report
    assert ms_n < ms_s and ms_n < ms_theta, report
