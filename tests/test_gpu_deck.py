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
- --selftest runs the Barnes-Hut gates of SelfTest.cpp on the GPU.
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
