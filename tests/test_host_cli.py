"""The deck front end (nbody_gb300) on the CPU: deck parsing, scenario
generation and the raw ic_file format.  No GPU is touched: --print-deck and
--dump-ic never create a device context.

Pins:
- the TOML reader against Python's tomllib on the same files (the reference
  reads decks with toml++; framework/src/Deck.cpp:24-47);
- parse errors exit 1 and name the line (Deck.cpp:29-33 reports the source
  and position);
- every supported deck scenario and the --bench Plummer sphere, byte for byte
  against fixtures the reference's own generator wrote (tests/golden/
  scenarios.npz, from Scenarios.cpp:355-384 and ic/Plummer.hpp:26-112);
- the ic_file reader (Scenarios.cpp:292-329) round-trips the writer's format
  (main.cpp:253-280);
- the run-directory writer (deck.toml, frames/*.npy, diagnostics.csv,
  manifest.json) byte for byte against the reference's own OutputWriter on a
  fixed three-frame run (tests/golden/writer_run.npz, written by
  oracle/writer_driver.cpp linked to framework/src/OutputWriter.cpp).
"""
import json
import os
import re
import subprocess
import tomllib

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

DECKS = os.path.join(GOLDEN, "decks")


@pytest.fixture(scope="module")
def exe(pkg):
    return pkg.executable()


def run(exe, *args, check=True):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)
    if check and r.returncode != 0:
        raise AssertionError(f"{args} exited {r.returncode}: {r.stderr}")
    return r


@pytest.mark.parametrize("deck", ["plummer_gpu.toml", "syntax_mix.toml"])
def test_print_deck_matches_tomllib(exe, deck):
    path = os.path.join(DECKS, deck)
    got = json.loads(run(exe, "--print-deck", path).stdout)
    with open(path, "rb") as f:
        want = tomllib.load(f)
    assert got == want
    # Floats stay floats and integers stay integers.
    def kinds(v):
        if isinstance(v, dict):
            return {k: kinds(c) for k, c in v.items()}
        if isinstance(v, list):
            return [kinds(c) for c in v]
        return type(v).__name__
    assert kinds(got) == kinds(want)


@pytest.mark.parametrize("deck,line,what", [("bad_duplicate.toml", 5, "duplicate key 'dt'"),
                                            ("bad_value.toml", 3, "bad number")])
def test_parse_error_names_line(exe, deck, line, what):
    r = run(exe, "--print-deck", os.path.join(DECKS, deck), check=False)
    assert r.returncode == 1
    assert what in r.stderr and f"at line {line}" in r.stderr


def test_missing_deck_is_an_error(exe, tmp_path):
    r = run(exe, "--print-deck", str(tmp_path / "absent.toml"), check=False)
    assert r.returncode == 1 and "absent.toml" in r.stderr


def test_usage_without_mode(exe):
    r = run(exe, check=False)
    assert r.returncode == 2 and "usage" in r.stderr


def _dump(exe, tmp_path, *args):
    out = tmp_path / "ic.bin"
    r = run(exe, *args, "--dump-ic", str(out))
    return np.fromfile(out, dtype=np.float32).reshape(-1, 7), r.stderr


@pytest.mark.parametrize("n", [1000, 4097])
def test_bench_plummer_matches_reference(exe, tmp_path, n):
    g = load_golden("scenarios.npz")
    rec, err = _dump(exe, tmp_path, "--bench-n", str(n))
    assert rec.shape == (n, 7)
    assert np.array_equal(rec.view(np.uint32), g[f"bench{n}_rec"].view(np.uint32))
    assert re.search(rf"# dump-ic path=\S+ N={n} eps=0.02 G=1.0000 seed=1 ", err)


def test_deck_scenarios_match_reference(exe, tmp_path):
    g = load_golden("scenarios.npz")
    for kind in g["names"]:
        kind = str(kind)
        deck = tmp_path / f"{kind}.toml"
        deck.write_text(f'[scenario]\ntype = "{kind}"\nn = {int(g[kind + "_n"])}\nseed = {int(g[kind + "_seed"])}\n')
        rec, err = _dump(exe, tmp_path, "--deck", str(deck))
        assert np.array_equal(rec.view(np.uint32), g[kind + "_rec"].view(np.uint32)), kind
        m = re.search(r"G=(\S+) eps=(\S+) dt=(\S+)", err)
        assert [float(v) for v in m.groups()] == list(g[kind + "_params"]), kind


def test_unknown_scenario_falls_back_to_plummer(exe, tmp_path):
    g = load_golden("scenarios.npz")
    deck = tmp_path / "x.toml"
    deck.write_text('[scenario]\ntype = "no_such_model"\nn = 3000\nseed = 5\n')
    rec, err = _dump(exe, tmp_path, "--deck", str(deck))
    assert "not available" in err
    assert np.array_equal(rec.view(np.uint32), g["plummer_rec"].view(np.uint32))


def test_ic_file_round_trip(exe, tmp_path):
    rng = np.random.default_rng(11)
    rec = rng.standard_normal((777, 7)).astype(np.float32)
    rec[:, 3] = np.abs(rec[:, 3]) + 0.1
    src = tmp_path / "src.bin"
    rec.tofile(src)
    deck = tmp_path / "ic.toml"
    deck.write_text(f'[scenario]\ntype = "ic_file"\nic_file = "{src}"\n')
    got, err = _dump(exe, tmp_path, "--deck", str(deck))
    assert np.array_equal(got.view(np.uint32), rec.view(np.uint32))
    # Scenarios.cpp:323-327: G 1, softening 0.05, dt 1e-3 for a raw file.
    m = re.search(r"N=(\d+) G=(\S+) eps=(\S+) dt=(\S+)", err)
    assert int(m.group(1)) == 777 and [float(v) for v in m.groups()[1:]] == [1.0, 0.05, 1e-3]


def test_ic_file_errors(exe, tmp_path):
    empty = tmp_path / "empty.bin"
    empty.write_bytes(b"")
    for path, what in ((tmp_path / "absent.bin", "cannot open"), (empty, "no particles")):
        deck = tmp_path / "bad.toml"
        deck.write_text(f'[scenario]\ntype = "ic_file"\nic_file = "{path}"\n')
        r = run(exe, "--deck", str(deck), "--dump-ic", str(tmp_path / "o.bin"), check=False)
        assert r.returncode == 1 and what in r.stderr


def test_run_directory_bytes_match_reference_writer(tmp_path):
    """The same driver (oracle/writer_driver.cpp) compiled against this
    project's writer must write every file of the reference writer's run
    directory with identical bytes, and no other file."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    host = os.path.join(root, "opengl-physics_gb300", "host")
    drv = tmp_path / "writer_driver"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", host, os.path.join(root, "oracle", "writer_driver.cpp"),
                    os.path.join(host, "output_writer.cpp"), os.path.join(host, "deck.cpp"), "-o", str(drv)],
                   check=True, capture_output=True, timeout=300)
    run_dir = tmp_path / "run"
    subprocess.run([str(drv), str(run_dir)], check=True, capture_output=True, timeout=60)
    got = {}
    for dirpath, _, files in os.walk(run_dir):
        for f in files:
            rel = os.path.relpath(os.path.join(dirpath, f), run_dir).replace(os.sep, "__")
            with open(os.path.join(dirpath, f), "rb") as fh:
                got[rel] = fh.read()
    want = {k: bytes(v) for k, v in load_golden("writer_run.npz").items()}
    assert sorted(got) == sorted(want)
    for k in sorted(want):
        assert got[k] == want[k], f"{k} differs"
    # and NumPy reads what was written
    pos = np.load(run_dir / "frames" / "pos_0002.npy")
    assert pos.dtype == np.float32 and pos.shape == (5, 3)
    assert np.load(run_dir / "frames" / "ids_0001.npy").shape == (7,)
