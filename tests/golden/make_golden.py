"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own CPU Barnes-Hut path (projects/nbody_core, compiled
from its sources by oracle/build_ref.sh into oracle/_ref/libngrav_ref.so) on
seeded inputs and stores inputs + outputs as compressed .npz files.  Needs
that library (oracle/build_ref.sh builds it where the reference's sources
are present); the fixtures it writes are committed so that tests never need
the reference at run time.

All positions and masses are rounded to FP32 before the reference sees them,
so the GPU state (FP32 / double-float) holds exactly the same inputs.

    python tests/golden/make_golden.py              # every fixture
    python tests/golden/make_golden.py scenarios    # scenarios.npz only
    python tests/golden/make_golden.py spline       # spline4k.npz only
    python tests/golden/make_golden.py pp           # pp4k.npz only
    python tests/golden/make_golden.py writer       # writer_run.npz only
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

TREE_KEYS = ("level", "prefix", "count", "is_leaf", "center", "half", "com", "mass", "max_radius", "quad")


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def tree_fields(R, x, y, z, m, ncrit, tag):
    t = R.tree(x, y, z, m, ncrit).canonical()
    out = {f"{tag}_{k}": t[k] for k in TREE_KEYS}
    out[f"{tag}_order"] = t["order"]
    return out


# Deck scenarios (Scenarios.cpp:355-384) as the reference generates them,
# stored as the raw 7 x float32 records its ic_file / --dump-ic format holds
# (x, y, z, m, vx, vy, vz), plus the scenario's G, softening and dt.
SCENARIOS = (("plummer", 3000, 5), ("cluster", 2500, 2), ("cold_collapse", 5000, 1), ("plummer_sphere", 100, 9))


def make_scenarios(R):
    d = {}
    for kind, n, seed in SCENARIOS:
        (x, y, z, vx, vy, vz, m), par = R.scenario(kind, n, seed)
        d[f"{kind}_rec"] = np.stack([x, y, z, m, vx, vy, vz], 1).astype(np.float32)
        d[f"{kind}_params"] = np.array(par)
        d[f"{kind}_n"] = n
        d[f"{kind}_seed"] = seed
    # The --bench / --dump-ic Plummer sphere (main.cpp:243-280): seed 1.
    for n in (1000, 4097):
        x, y, z, vx, vy, vz, m = R.plummer(n, 1)
        d[f"bench{n}_rec"] = np.stack([x, y, z, m, vx, vy, vz], 1).astype(np.float32)
    d["names"] = np.array([k for k, _, _ in SCENARIOS])
    np.savez_compressed(os.path.join(HERE, "scenarios.npz"), **d)


def make_spline(R, ic):
    """Cubic-spline softening (Softening.hpp:30-56): Plummer 4,096 (seed 11),
    h = 0.02, leaf capacity 16, theta 0.5, 10 KDK steps of 1e-3."""
    n, ncrit, G, h, theta, dt, steps = 4096, 16, 1.0, 0.02, 0.5, 1e-3, 10
    x, y, z, vx, vy, vz, m = (f32(a) for a in ic.plummer(n, seed=11))
    R.set_softening(1)
    try:
        d = dict(x=x, y=y, z=z, vx=vx, vy=vy, vz=vz, m=m, G=G, eps=h, theta=theta, ncrit=ncrit, dt=dt, steps=steps)
        ax, ay, az = R.bh_accel(x, y, z, m, G, h, theta, ncrit)
        d.update(ax=ax, ay=ay, az=az)
        dx, dy, dz = R.direct(x, y, z, m, G, h)
        d.update(dax=dx, day=dy, daz=dz)
        (sx, sy, sz, svx, svy, svz), _ = R.leapfrog((x, y, z, vx, vy, vz), m, G, h, theta, ncrit, dt, steps)
        d.update(kdk_x=sx, kdk_y=sy, kdk_z=sz, kdk_vx=svx, kdk_vy=svy, kdk_vz=svz)
        d["diag0"] = R.diagnostics(x, y, z, vx, vy, vz, m, G, h)
        d["diag10"] = R.diagnostics(sx, sy, sz, svx, svy, svz, m, G, h)
    finally:
        R.set_softening(0)
    np.savez_compressed(os.path.join(HERE, "spline4k.npz"), **d)


def make_pp(R, ic):
    """The per-particle walk: relative MAC (alpha 1e-3, previous |a| = the
    direct-sum |a|) and the geometric walk on every third particle; Plummer
    4,096 (seed 13), eps 0.02, leaf capacity 8, theta 0.5."""
    n, ncrit, G, eps, theta, alpha = 4096, 8, 1.0, 0.02, 0.5, 1e-3
    x, y, z, vx, vy, vz, m = (f32(a) for a in ic.plummer(n, seed=13))
    dx, dy, dz = R.direct(x, y, z, m, G, eps)
    aold = np.sqrt(dx ** 2 + dy ** 2 + dz ** 2)
    rx, ry, rz = R.bh_pp_accel(x, y, z, m, G, eps, theta, ncrit, alpha=alpha, aold=aold)
    tg = (np.arange(n) % 3 == 0).astype(np.uint8)
    gx, gy, gz = R.bh_pp_accel(x, y, z, m, G, eps, theta, ncrit, targets=tg)
    np.savez_compressed(os.path.join(HERE, "pp4k.npz"), x=x, y=y, z=z, m=m, G=G, eps=eps, theta=theta, ncrit=ncrit,
                        alpha=alpha, aold=aold, rel_ax=rx, rel_ay=ry, rel_az=rz, targets=tg, tgt_ax=gx, tgt_ay=gy,
                        tgt_az=gz, dax=dx, day=dy, daz=dz)


def make_block(R, ic):
    """Block (power-of-two rung) timesteps, System::Step with
    StepParams::block: Plummer 4,096 (seed 17), eps 0.01, theta 0.5, coarse
    dt 0.01, eta 0.025; two steps with max rung 8 (rungs 0-3 in use) and one
    with max rung 1 (the clamp).  The reference's block path builds its
    trees with leaf capacity 8."""
    n, G, eps, theta, dt, eta = 4096, 1.0, 0.01, 0.5, 0.01, 0.025
    x, y, z, vx, vy, vz, m = (f32(a) for a in ic.plummer(n, seed=17))
    out = dict(x=x, y=y, z=z, vx=vx, vy=vy, vz=vz, m=m, G=G, eps=eps, theta=theta, dt=dt, eta=eta)
    for tag, max_rung, steps in (("r8", 8, 2), ("r1", 1, 1)):
        st, a, rung = R.block_step((x, y, z, vx, vy, vz), m, G, eps, theta, dt, eta, max_rung, nsteps=steps)
        out.update({f"{tag}_{k}": v for k, v in zip(("x", "y", "z", "vx", "vy", "vz"), st)})
        out.update({f"{tag}_{k}": v for k, v in zip(("ax", "ay", "az"), a)})
        out[f"{tag}_rung"] = rung
        out[f"{tag}_steps"] = steps
        out[f"{tag}_max_rung"] = max_rung
    np.savez_compressed(os.path.join(HERE, "block4k.npz"), **out)


def make_writer():
    """writer_run.npz: every file of the reference's own run-directory writer
    (fw::OutputWriter, driven through oracle/writer_driver.cpp's fixed
    three-frame run), keyed by its path in the run directory with '/' as
    '__', as raw bytes."""
    import subprocess
    import tempfile
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_writer")
    with tempfile.TemporaryDirectory() as tmp:
        run = os.path.join(tmp, "run")
        subprocess.run([exe, run], check=True)
        out = {}
        for dirpath, _, files in os.walk(run):
            for f in files:
                rel = os.path.relpath(os.path.join(dirpath, f), run)
                with open(os.path.join(dirpath, f), "rb") as fh:
                    out[rel.replace(os.sep, "__")] = np.frombuffer(fh.read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "writer_run.npz"), **out)


def main():
    orc = ge.load_oracle()
    if orc.build_reference() is None:
        raise SystemExit("reference sources not found; set NGRAV_REFERENCE")
    R = orc.Reference()
    pkg_ic = __import__(ge.PKG_NAME + ".ic", fromlist=["ic"]) if ge.load_package() else None
    if sys.argv[1:] == ["writer"]:
        make_writer()
        return
    if sys.argv[1:] == ["spline"]:
        make_spline(R, pkg_ic)
        return
    if sys.argv[1:] == ["pp"]:
        make_pp(R, pkg_ic)
        return
    if sys.argv[1:] == ["block"]:
        make_block(R, pkg_ic)
        return
    make_scenarios(R)
    if sys.argv[1:] == ["scenarios"]:
        return
    make_spline(R, pkg_ic)
    make_pp(R, pkg_ic)
    make_block(R, pkg_ic)
    make_writer()
    ic = __import__(ge.PKG_NAME + ".ic", fromlist=["ic"]) if ge.load_package() else None

    # 1) Plummer N=16,384, seed 0: leaf capacity 16, theta 0.5, eps 0.01, dt 1e-3, 10 KDK steps.
    n, ncrit, G, eps, theta, dt, steps = 16384, 16, 1.0, 0.01, 0.5, 1e-3, 10
    x, y, z, vx, vy, vz, m = (f32(a) for a in ic.plummer(n, seed=0))
    d = dict(x=x, y=y, z=z, vx=vx, vy=vy, vz=vz, m=m, G=G, eps=eps, theta=theta, ncrit=ncrit, dt=dt, steps=steps)
    d.update(tree_fields(R, x, y, z, m, ncrit, "tree"))
    ax, ay, az = R.bh_accel(x, y, z, m, G, eps, theta, ncrit)
    d.update(ax=ax, ay=ay, az=az)
    dx, dy, dz = R.direct(x, y, z, m, G, eps)
    d.update(dax=dx, day=dy, daz=dz)
    (sx, sy, sz, svx, svy, svz), _ = R.leapfrog((x, y, z, vx, vy, vz), m, G, eps, theta, ncrit, dt, steps)
    d.update(kdk_x=sx, kdk_y=sy, kdk_z=sz, kdk_vx=svx, kdk_vy=svy, kdk_vz=svz)
    d["diag0"] = R.diagnostics(x, y, z, vx, vy, vz, m, G, eps)
    d["diag10"] = R.diagnostics(sx, sy, sz, svx, svy, svz, m, G, eps)
    np.savez_compressed(os.path.join(HERE, "plummer16k.npz"), **d)

    # 2) BH-vs-Direct self-test cloud (SelfTest.cpp:43-74): theta 0, eps 0.02, default ncrit 8.
    x, y, z, m = (f32(a) for a in R.cloud("uniform", 1000, 12345))
    d = dict(x=x, y=y, z=z, m=m, G=1.0, eps=0.02, theta=0.0, ncrit=8)
    d.update(tree_fields(R, x, y, z, m, 8, "tree"))
    ax, ay, az = R.bh_accel(x, y, z, m, 1.0, 0.02, 0.0, 8)
    d.update(ax=ax, ay=ay, az=az)
    dx, dy, dz = R.direct(x, y, z, m, 1.0, 0.02)
    d.update(dax=dx, day=dy, daz=dz)
    np.savez_compressed(os.path.join(HERE, "selftest_uniform1000.npz"), **d)

    # 3) Quadrupole self-test cloud (SelfTest.cpp:212-265): eps 0.01, theta 0.5, ncrit 8.
    x, y, z, m = (f32(a) for a in R.cloud("ball", 4000, 2024))
    d = dict(x=x, y=y, z=z, m=m, G=1.0, eps=0.01, theta=0.5, ncrit=8)
    d.update(tree_fields(R, x, y, z, m, 8, "tree"))
    for tag, quad in (("mono", False), ("quad", True)):
        ax, ay, az = R.bh_accel(x, y, z, m, 1.0, 0.01, 0.5, 8, quad=quad)
        d.update({f"{tag}_ax": ax, f"{tag}_ay": ay, f"{tag}_az": az})
    dx, dy, dz = R.direct(x, y, z, m, 1.0, 0.01)
    d.update(dax=dx, day=dy, daz=dz)
    np.savez_compressed(os.path.join(HERE, "selftest_ball4000.npz"), **d)

    # 4) Edge cases: tiny and degenerate inputs, leaf capacities 1..16.
    rng = np.random.default_rng(99)
    cases = []
    for n, ncrit in ((1, 8), (2, 8), (8, 8), (9, 8), (17, 16), (300, 1), (257, 4), (1000, 32)):
        cases.append((f"n{n}_c{ncrit}", rng.standard_normal((n, 3)), ncrit))
    # A cluster of exact duplicates plus a cold clump: exercises deep splits.
    dup = np.concatenate([np.repeat(rng.standard_normal((1, 3)), 5, axis=0), rng.standard_normal((60, 3)) * 1e-4,
                          rng.standard_normal((200, 3))])
    cases.append(("dups_c4", dup, 4))
    # Points on a lattice: many exact ties with cell centres.
    g = np.arange(-4, 4, dtype=np.float64) * 0.25
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    cases.append(("lattice_c8", lat, 8))
    d = {}
    names = []
    for name, p, ncrit in cases:
        x, y, z = (f32(p[:, k]) for k in range(3))
        m = f32(np.full(len(x), 1.0 / len(x)))
        d.update({f"{name}_x": x, f"{name}_y": y, f"{name}_z": z, f"{name}_m": m, f"{name}_ncrit": ncrit})
        d.update(tree_fields(R, x, y, z, m, ncrit, f"{name}_tree"))
        ax, ay, az = R.bh_accel(x, y, z, m, 1.0, 0.05, 0.5, ncrit)
        d.update({f"{name}_ax": ax, f"{name}_ay": ay, f"{name}_az": az})
        names.append(name)
    d["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "edge_cases.npz"), **d)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
