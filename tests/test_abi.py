"""The C-ABI library builds, loads without a GPU, and exports every entry
point include/ngrav_gpu.h declares.  No compute calls are made here."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def header_functions():
    text = open(os.path.join(ROOT, "include", "ngrav_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ngrav_gpu_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    fns = header_functions()
    assert "ngrav_gpu_compute_accel" in fns and "ngrav_gpu_step" in fns
    assert len(fns) >= 16


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.load_library()._name)
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_python_mirror_lists_the_header(pkg):
    assert sorted(pkg.EXPORTS) == header_functions()


def test_default_opts_without_gpu(pkg):
    L = pkg.load_library()
    o = pkg.Opts()
    assert L.ngrav_gpu_default_opts(ctypes.byref(o)) == 0
    assert o.abi_version == pkg.ABI_VERSION and o.leaf_capacity == 8 and o.max_depth == 40
    assert o.theta == pytest.approx(0.5) and o.G == 1.0 and o.quadrupole == 1


def test_struct_layouts_match_header(pkg, tmp_path):
    """ctypes mirrors of the C structs match the C compiler's layout."""
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "ngrav_gpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(ngrav_gpu_opts),"
        " sizeof(ngrav_gpu_diag), sizeof(ngrav_gpu_ferr), sizeof(ngrav_gpu_stats), offsetof(ngrav_gpu_opts, G),"
        " offsetof(ngrav_gpu_stats, p2p_pairs), offsetof(ngrav_gpu_stats, lmac_last_check_rms),"
        " sizeof(ngrav_gpu_lmac_opts), sizeof(ngrav_gpu_lmac_train_opts), offsetof(ngrav_gpu_lmac_train_opts, seed),"
        " sizeof(ngrav_gpu_lmac_report)); printf(\"%zu %zu %zu\\n\", sizeof(ngrav_gpu_tune_opts),"
        " sizeof(ngrav_gpu_tune_report), offsetof(ngrav_gpu_tune_report, tried));return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(pkg.Opts), ctypes.sizeof(pkg.Diag), ctypes.sizeof(pkg.Ferr), ctypes.sizeof(pkg.Stats),
            pkg.Opts.G.offset, pkg.Stats.p2p_pairs.offset, pkg.Stats.lmac_last_check_rms.offset,
            ctypes.sizeof(pkg.LmacOpts), ctypes.sizeof(pkg.LmacTrainOpts), pkg.LmacTrainOpts.seed.offset,
            ctypes.sizeof(pkg.LmacReport), ctypes.sizeof(pkg.TuneOpts), ctypes.sizeof(pkg.TuneReport),
            pkg.TuneReport.tried.offset]
    assert got == want


def test_lmac_default_opts_without_gpu(pkg):
    L = pkg.load_library()
    o = pkg.LmacOpts()
    assert L.ngrav_gpu_lmac_default_opts(ctypes.byref(o)) == 0
    assert o.check_every == 10 and o.check_targets == 4096 and o.revert_rms == pytest.approx(1e-3)
    assert 0.0 < o.rho_lo < o.rho_hi and o.budget > 0.0
    t = pkg.LmacTrainOpts()
    assert L.ngrav_gpu_lmac_default_train_opts(ctypes.byref(t)) == 0
    assert t.snapshots == 16 and t.pairs == 1 << 22 and t.batch % 128 == 0
