"""Failure detection and recovery, driven from the host (no GPU fault).

The reference's GPU path fails silently where its pools run out
(src/gpu/GpuBarnesHut.cpp:259-260 node pool, :428 walk stack) and never
checks its inputs.  Here every kernel writes a sticky device status word that
the host reads after each evaluation:
- a NaN or Inf position or mass is reported as NGRAV_ERR_NONFINITE (set
  before a step, or planted between steps), the kernels downstream return at
  once, and the context stays usable;
- node-pool and interaction-list overflows, forced with tiny pools
  (ngrav_gpu_debug_shrink_pools), are detected, the pools grow and the
  evaluation re-runs, also inside a graph-captured KDK step; the states are
  bit-identical to a run that never overflowed;
- the learned walk's deferred-pair pool overflows the same way, and the
  re-run evaluation still counts toward the FP64 check cadence;
- the keys are sorted only as deep as the last tree went (plus a level);
  a tree that suddenly goes deeper stops its build (a node at the deepest
  sorted level would still split) and the evaluation re-runs on the full
  key, with the same tree and accelerations as a fresh context.
"""
import numpy as np
import pytest

from conftest import TREE_EXACT, load_golden

pytestmark = pytest.mark.gpu

NONFINITE = 5
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m")


def golden_sim(pkg, d, **kw):
    sim = pkg.NBodySystem(pkg.StepParams(G=float(d["G"]), eps=float(d["eps"]), theta=float(d["theta"])),
                          leaf_capacity=int(d["ncrit"]), **kw)
    sim.set_particles(*(d[k] for k in FIELDS))
    return sim


@pytest.mark.parametrize("field,index,value", [("x", 5, np.nan), ("z", 16000, np.inf), ("m", 7, np.nan)])
def test_nonfinite_input_is_reported_and_context_recovers(pkg, field, index, value):
    d = load_golden("plummer16k.npz")
    bad = {k: np.array(d[k], dtype=np.float64) for k in FIELDS}
    bad[field][index] = value
    with golden_sim(pkg, d) as sim:
        sim.set_particles(*(bad[k] for k in FIELDS))
        with pytest.raises(pkg.NgravError) as e:
            sim.compute_accel()
        assert e.value.code == NONFINITE
        # the same context takes a good set and evaluates it correctly
        sim.set_particles(*(d[k] for k in FIELDS))
        ax, ay, az = sim.compute_accel()
    ref = np.sqrt(d["ax"] ** 2 + d["ay"] ** 2 + d["az"] ** 2)
    rel = np.sqrt((ax - d["ax"]) ** 2 + (ay - d["ay"]) ** 2 + (az - d["az"]) ** 2) / ref
    assert np.median(rel) <= 1e-5 and rel.max() <= 1e-4


def test_nonfinite_planted_between_steps(pkg):
    d = load_golden("plummer16k.npz")
    with golden_sim(pkg, d) as sim:
        sim.prime()
        sim.step(2, float(d["dt"]))
        x, y, z, vx, vy, vz = sim.state()
        x[123] = np.nan
        sim.set_state(x, y, z, vx, vy, vz)
        with pytest.raises(pkg.NgravError) as e:
            sim.step(1, float(d["dt"]))
        assert e.value.code == NONFINITE


def _run(pkg, d, shrink, steps=10):
    with golden_sim(pkg, d) as sim:
        if shrink:
            sim.debug_shrink_pools(node_cap=64, far_chunks=1, near_chunks=1)
        sim.prime()  # an evaluation that overflows, grows and re-runs
        if shrink:
            # again, so the first graph-captured step overflows too
            sim.debug_shrink_pools(node_cap=64, far_chunks=1, near_chunks=1)
        sim.reset_cumulative()
        sim.step(steps, float(d["dt"]))
        st = sim.stats()
        return sim.state(), sim.accel(), st


def test_pool_overflow_grows_and_reruns_bit_identically(pkg):
    d = load_golden("plummer16k.npz")
    (s0, a0, st0) = _run(pkg, d, shrink=False)
    (s1, a1, st1) = _run(pkg, d, shrink=True)
    for u, v in zip(s0 + a0, s1 + a1):
        assert np.array_equal(u, v)
    assert st1["graph_captures"] >= 1
    # the overflowing step re-ran its evaluation: more kernels for the same steps
    assert st1["cum_launches"] > st0["cum_launches"]
    assert st1["status_bits"] & 0x7F == 0  # the last evaluation ended clean


def test_learned_pool_overflow_reruns_and_keeps_check_cadence(pkg, ic):
    n, dt, steps = 65536, 1e-3, 3
    arrs = ic.plummer(n, seed=3)
    out = []
    model = None
    for shrink in (False, True):
        with pkg.NBodySystem(pkg.StepParams(G=1.0, eps=0.01, theta=0.5), leaf_capacity=16) as sim:
            sim.set_particles(*arrs)
            if model is None:
                sim.lmac_train(snapshots=2, steps_between=0, pairs=1 << 15, epochs=2, batch=4096, seed=4)
                model = sim.lmac_get_model()
                sim.set_particles(*arrs)
            else:
                sim.lmac_set_model(*model)
            sim.lmac_set_opts(budget=1e-4, check_every=1, check_targets=256, revert_rms=1.0)
            sim.set_opts(mac=pkg.MAC_LEARNED)
            sim.prime()  # geometric (no accelerations yet), then learned steps
            if shrink:
                sim.debug_shrink_pools(pend_chunks=1)
            sim.reset_cumulative()
            sim.step(steps, dt)
            st = sim.stats()
            assert st["lmac_active"] == 1 and not st["lmac_reverted"]
            out.append((sim.state(), st))
    (s0, st0), (s1, st1) = out
    for u, v in zip(s0, s1):
        assert np.array_equal(u, v)
    # one FP64 check per learned evaluation, the re-run one included
    assert st1["lmac_checks"] == st0["lmac_checks"]
    assert st1["cum_launches"] > st0["cum_launches"]


def test_tree_deeper_than_the_sorted_key_levels_rebuilds_on_the_full_key(pkg):
    d = load_golden("plummer16k.npz")
    x, y, z = (np.array(d[k], dtype=np.float64) for k in ("x", "y", "z"))
    vx, vy, vz = (np.array(d[k], dtype=np.float64) for k in ("vx", "vy", "vz"))
    # 400 particles pulled into a cube of half-size 1e-3 around particle 0:
    # the tree there needs several more levels than the sphere's (and still
    # far fewer than 21, so every key stays distinct)
    rng = np.random.default_rng(7)
    idx = rng.choice(np.arange(1, len(x)), size=400, replace=False)
    x2, y2, z2 = x.copy(), y.copy(), z.copy()
    for a, b in ((x2, x), (y2, y), (z2, z)):
        a[idx] = b[0] + 1e-3 * rng.uniform(-1, 1, idx.size)
    with golden_sim(pkg, d) as sim:
        sim.compute_accel()
        shallow = sim.stats()["levels"]
        sim.compute_accel()  # sorted to the shallow tree's depth from here on
        launches0 = sim.stats()["cum_launches"]
        sim.compute_accel()
        launches1 = sim.stats()["cum_launches"] - launches0
        sim.set_state(x2, y2, z2, vx, vy, vz)
        sim.reset_cumulative()
        a1 = sim.compute_accel()
        st1 = sim.stats()
        t1 = sim.debug_tree()
    with golden_sim(pkg, d) as fresh:
        fresh.set_particles(x2, y2, z2, vx, vy, vz, d["m"])
        a0 = fresh.compute_accel()
        st0 = fresh.stats()
        t0 = fresh.debug_tree()
    assert st1["levels"] > shallow + 1  # deeper than the sorted levels: the build was redone
    assert st1["cum_launches"] > launches1  # one evaluation, two builds
    assert st1["status_bits"] & 0x1FF == 0 and st1["levels"] == st0["levels"]
    assert np.array_equal(t1["order"], t0["order"])
    c1, c0 = pkg.canonical(t1), pkg.canonical(t0)
    for k in TREE_EXACT:
        assert np.array_equal(c1[k], c0[k]), k
    assert st1["p2p_pairs"] == st0["p2p_pairs"] and st1["p2c_terms"] == st0["p2c_terms"]
    for u, v in zip(a1, a0):
        np.testing.assert_array_equal(u, v)
