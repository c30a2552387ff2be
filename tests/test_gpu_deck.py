"""The deck front end (nbody_gb300) on the GPU: a headless deck run, --bench
and --selftest, all through the C-ABI library.

- A deck run writes the reference's output layout (framework/src/
  OutputWriter.cpp:38-167: deck.toml copy, frames/<field>_NNNN.npy,
  diagnostics.csv with t,step + the DeckSim columns, manifest.json), and its
  trajectory follows the oracle's KDK leapfrog (src/Integrator.cpp:9-39) on
  the same ic_file input within FP32 force tolerances.
- --bench prints the reference's CSV line (main.cpp:389-391) with a mean
  relative force error that is the Barnes-Hut truncation error, not an FP32
  artefact.
- --selftest, --rung-selftest and --dt-selftest run the gates of
  SelfTest.cpp (Barnes-Hut, block timesteps, adaptive dt) on the GPU.
"""
import csv
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe(pkg):
    return pkg.executable()


def run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"{args} exited {r.returncode}: {r.stderr}"
    return r


def test_deck_run_layout_and_trajectory(exe, ic, oracle, tmp_path):
    n, G, eps, theta, ncrit, dt, frames, sub = 2048, 1.0, 0.05, 0.5, 16, 1e-3, 4, 5
    x, y, z, vx, vy, vz, m = ic.plummer(n, seed=3)
    rec = np.stack([x, y, z, m, vx, vy, vz], 1).astype(np.float32)
    icf = tmp_path / "ic.bin"
    rec.tofile(icf)
    deck_text = (f'title = "deck parity"\n[sim]\nG = {G}\n[softening]\neps = {eps}\n'
                 f'[time]\nframes = {frames}\nsubsteps_per_frame = {sub}\ndt = {dt}\n'
                 f'[solver]\nkind = "barnes_hut"\ntheta = {theta}\nleaf_capacity = {ncrit}\n'
                 f'[scenario]\ntype = "ic_file"\nic_file = "{icf}"\n')
    deck = tmp_path / "run.toml"
    deck.write_text(deck_text)
    out = tmp_path / "out"
    run(exe, "--deck", str(deck), "--out", str(out))

    assert (out / "deck.toml").read_text() == deck_text
    man = json.loads((out / "manifest.json").read_text())
    assert man["frames"] == frames and man["substeps_per_frame"] == sub and man["dt"] == dt
    assert man["fields"] == {"pos": {"dtype": "<f4", "shape": [n, 3]}, "vel": {"dtype": "<f4", "shape": [n, 3]}}
    cols = ["energy", "energy_drift_pct", "L_mag", "L_drift_pct", "p_mag", "com_x", "com_y", "com_z", "dt_last",
            "rung_max"]
    assert man["diagnostics"] == cols
    with open(out / "diagnostics.csv") as f:
        rows = list(csv.reader(f))
    assert rows[0] == ["t", "step"] + cols and len(rows) == frames + 1
    assert [int(r[1]) for r in rows[1:]] == [f * sub for f in range(frames)]

    pos0 = np.load(out / "frames" / "pos_0000.npy")
    assert pos0.dtype == np.float32 and pos0.shape == (n, 3)
    assert np.array_equal(pos0, rec[:, 0:3])

    st = tuple(rec[:, k].astype(np.float64) for k in (0, 1, 2, 4, 5, 6))
    mm = rec[:, 3].astype(np.float64)
    acc = None
    for f in range(1, frames):
        st, acc = oracle.leapfrog(st, mm, G, eps, theta, ncrit, dt, sub, acc)
        pos = np.load(out / "frames" / f"pos_{f:04d}.npy").astype(np.float64)
        vel = np.load(out / "frames" / f"vel_{f:04d}.npy").astype(np.float64)
        np.testing.assert_allclose(pos, np.stack(st[0:3], 1), rtol=0, atol=2e-6)
        np.testing.assert_allclose(vel, np.stack(st[3:6], 1), rtol=0, atol=2e-6)
        d = oracle.diagnostics(*st, mm, G, eps)
        row = [float(v) for v in rows[f + 1]]
        assert abs(row[2] - d[0]) <= 1e-6 * abs(d[0])          # energy (exact FP64 sum on both sides)
        np.testing.assert_allclose(row[7:10], d[1:4], atol=1e-7)  # centre of mass
        assert row[10] == dt and row[11] == 0.0


def test_bench_csv_line(exe):
    r = run(exe, "--bench", "barnes_hut", "--bench-n", "20000", "--bench-reps", "2")
    assert r.stderr.strip().splitlines()[-1] == "solver,n,theta,order,ms_per_eval,mean_rel_err"
    f = r.stdout.strip().split(",")
    assert f[0:4] == ["barnes_hut", "20000", "0.500", "5"]
    ms, err = float(f[4]), float(f[5])
    assert ms > 0.0
    # theta 0.5 with quadrupoles: truncation error of order 1e-4, far above FP32 round-off.
    assert 1e-6 < err < 2e-3
    r = run(exe, "--bench", "direct", "--bench-n", "20000", "--bench-reps", "1")
    assert float(r.stdout.strip().split(",")[5]) < 1e-5


def test_selftest_passes(exe):
    r = run(exe, "--selftest")
    assert "selftest: PASS" in r.stdout


def test_rung_selftest_passes(exe):
    """CoreRungSelfTest's gates (SelfTest.cpp:821-924) through the C-ABI: the
    block scheme conserves energy and needs >= 2x fewer particle evaluations
    than the global-adaptive scheme on a cloud with one tight binary."""
    r = run(exe, "--rung-selftest")
    assert "rung-selftest: PASS" in r.stdout, r.stdout


def test_dt_selftest_passes(exe):
    """CoreDtSelfTest's gates (SelfTest.cpp:438-482): adaptive dt on an e = 0.9
    orbit matches a fixed dt's accuracy with >= 2x fewer evaluations."""
    r = run(exe, "--dt-selftest")
    assert "dt-selftest: PASS" in r.stdout, r.stdout


def ic_deck(tmp_path, ic, n, seed, body, binary=False):
    x, y, z, vx, vy, vz, m = ic.plummer(n, seed=seed)
    if binary:  # one heavy tight pair (|a| ~ 30): shrinks the adaptive step / takes deep rungs
        x[0], y[0], z[0], x[1], y[1], z[1] = 0.02, 0.0, 0.0, -0.02, 0.0, 0.0
        vx[0], vy[0], vz[0], vx[1], vy[1], vz[1] = 0.0, 0.75, 0.0, 0.0, -0.75, 0.0
        m[0] = m[1] = 0.05
    rec = np.stack([x, y, z, m, vx, vy, vz], 1).astype(np.float32)
    icf = tmp_path / "ic.bin"
    rec.tofile(icf)
    deck = tmp_path / "run.toml"
    deck.write_text(f'title = "deck keys"\n{body}[scenario]\ntype = "ic_file"\nic_file = "{icf}"\n')
    st = tuple(rec[:, k].astype(np.float64) for k in (0, 1, 2, 4, 5, 6))
    return deck, st, rec[:, 3].astype(np.float64)


def frame(out, f):
    return (np.load(out / "frames" / f"pos_{f:04d}.npy").astype(np.float64),
            np.load(out / "frames" / f"vel_{f:04d}.npy").astype(np.float64))


def diag_rows(out):
    with open(out / "diagnostics.csv") as f:
        return [[float(v) for v in r] for r in list(csv.reader(f))[1:]]


def test_deck_block_scheme_follows_oracle(exe, ic, oracle, tmp_path):
    """time.scheme = "block": each substep is System::BlockStep; frames and
    the rung_max column follow the oracle's block step."""
    G, eps, theta, dt, eta, max_rung, frames, sub = 1.0, 0.01, 0.5, 4e-3, 0.03, 6, 3, 2
    body = (f'[sim]\nG = {G}\n[softening]\neps = {eps}\n[time]\nframes = {frames}\nsubsteps_per_frame = {sub}\n'
            f'dt = {dt}\nscheme = "block"\nblock_max_rung = {max_rung}\neta = {eta}\n'
            f'[solver]\nkind = "barnes_hut"\ntheta = {theta}\n')
    deck, st, mm = ic_deck(tmp_path, ic, 2048, 8, body, binary=True)
    out = tmp_path / "out"
    r = run(exe, "--deck", str(deck), "--out", str(out))
    assert "warning" not in r.stderr
    rows = diag_rows(out)
    acc = oracle.bh_accel(*st[0:3], mm, G, eps, theta, 8)
    for f in range(1, frames):
        for _ in range(sub):
            st, acc, rung, rmax = oracle.block_step(st, mm, G, eps, theta, 8, dt, eta, max_rung, acc)
        pos, vel = frame(out, f)
        np.testing.assert_allclose(pos, np.stack(st[0:3], 1), rtol=0, atol=5e-6)
        np.testing.assert_allclose(vel, np.stack(st[3:6], 1), rtol=0, atol=5e-4 * np.abs(st[3]).max())
        assert rows[f][11] == rmax and rmax >= 3
        assert rows[f][10] == dt


def test_deck_adaptive_dt_follows_oracle(exe, ic, oracle, tmp_path):
    """time.adaptive: every substep takes ChooseAdaptiveDt of the current
    accelerations (src/Integrator.cpp:41-59); dt_last reports it."""
    G, eps, theta, dt, eta, frames, sub = 1.0, 0.01, 0.5, 1e-2, 0.02, 3, 3
    body = (f'[sim]\nG = {G}\n[softening]\neps = {eps}\n[time]\nframes = {frames}\nsubsteps_per_frame = {sub}\n'
            f'dt = {dt}\nadaptive = true\neta = {eta}\n[solver]\nkind = "barnes_hut"\ntheta = {theta}\n')
    deck, st, mm = ic_deck(tmp_path, ic, 2048, 9, body, binary=True)
    out = tmp_path / "out"
    r = run(exe, "--deck", str(deck), "--out", str(out))
    assert "warning" not in r.stderr
    rows = diag_rows(out)
    acc = oracle.bh_accel(*st[0:3], mm, G, eps, theta, 8)
    for f in range(1, frames):
        for _ in range(sub):
            a = np.sqrt(acc[0] ** 2 + acc[1] ** 2 + acc[2] ** 2)
            h = float(np.clip(eta * np.sqrt(eps / a.max()), dt / 4096, dt))
            st, acc = oracle.leapfrog(st, mm, G, eps, theta, 8, h, 1, acc)
        assert h < dt
        assert rows[f][10] == pytest.approx(h, rel=1e-5)
        assert rows[f][0] == f * sub * dt  # the runner's t is step x nominal dt (HeadlessRunner.cpp:21-23)
        pos, vel = frame(out, f)
        np.testing.assert_allclose(pos, np.stack(st[0:3], 1), rtol=0, atol=5e-6)


def test_deck_spline_and_relative_mac(exe, ic, oracle, tmp_path):
    """softening.kind = "spline" follows the oracle's spline leapfrog; and
    solver.mac = "relative" runs the relative test (no fallback warning),
    conserving energy."""
    G, eps, theta, dt, frames, sub = 1.0, 0.05, 0.5, 1e-3, 3, 4
    body = (f'[sim]\nG = {G}\n[softening]\nkind = "spline"\neps = {eps}\n[time]\nframes = {frames}\n'
            f'substeps_per_frame = {sub}\ndt = {dt}\n[solver]\nkind = "barnes_hut"\ntheta = {theta}\n')
    deck, st, mm = ic_deck(tmp_path, ic, 2048, 10, body)
    out = tmp_path / "out"
    r = run(exe, "--deck", str(deck), "--out", str(out))
    assert "warning" not in r.stderr
    rows = diag_rows(out)
    oracle.set_softening(1)
    try:
        acc = None
        for f in range(1, frames):
            st, acc = oracle.leapfrog(st, mm, G, eps, theta, 8, dt, sub, acc)
            pos, vel = frame(out, f)
            np.testing.assert_allclose(pos, np.stack(st[0:3], 1), rtol=0, atol=2e-6)
            d = oracle.diagnostics(*st, mm, G, eps)
            assert abs(rows[f][2] - d[0]) <= 1e-6 * abs(d[0])
    finally:
        oracle.set_softening(0)

    body = (f'[sim]\nG = {G}\n[softening]\neps = {eps}\n[time]\nframes = 4\nsubsteps_per_frame = 5\n'
            f'dt = {dt}\n[solver]\nkind = "barnes_hut"\nmac = "relative"\nalpha = 0.004\n')
    deck, _, _ = ic_deck(tmp_path, ic, 2048, 11, body)
    out = tmp_path / "out_rel"
    r = run(exe, "--deck", str(deck), "--out", str(out))
    assert "warning" not in r.stderr
    rows = diag_rows(out)
    assert abs(rows[-1][3]) < 0.01  # energy_drift_pct
