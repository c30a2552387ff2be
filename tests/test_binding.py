"""The reference-side C++ binding of INTEGRATION.md.

INTEGRATION.md shows two pieces: an edit to the reference's
System<3>::ComputeAccel (include/ngrav/System.hpp:57-66) that consults a
Barnes-Hut evaluator registered with SetAuxSolver (System.hpp:40), and the
AccelFn<3> adapter include/ngrav_gpu_accelfn.hpp.  These tests hold both to
the document's text and make sure they build and run:
- the adapter block in INTEGRATION.md is the header, byte for byte;
- the header compiles and links against stand-ins of the reference
  declarations it uses (tests/binding/ngrav/Integrator.hpp) and
  libngrav_gpu.so;
- where the reference was compiled here (oracle/_ref/REF_ROOT names its
  sources), the diff applies to the reference's own System.hpp and the
  adapter compiles and links against the reference's real headers, its CPU
  path (oracle/_ref/libngrav_ref.so) and libngrav_gpu.so;
- on the GPU, the registered adapter -- called through the copy
  SetAuxSolver holds after the original is destroyed -- reproduces the
  reference's accelerations on the 16,384-body Plummer golden, twice.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "opengl-physics_gb300")
BINDING = os.path.join(ROOT, "tests", "binding")
REF_ROOT_FILE = os.path.join(ROOT, "oracle", "_ref", "REF_ROOT")


def _blocks(lang):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```" + lang + r"\n(.*?)```", text, flags=re.S)


def test_integration_md_quotes_the_adapter_header():
    header = open(os.path.join(INCLUDE, "ngrav_gpu_accelfn.hpp")).read()
    assert header in _blocks("cpp")


def _link_flags():
    return ["-L", PKG, "-lngrav_gpu", "-Wl,-rpath," + PKG]


@pytest.fixture(scope="module")
def binding_exe(pkg, tmp_path_factory):
    pkg.load_library()  # builds nothing; the library must exist
    exe = str(tmp_path_factory.mktemp("binding") / "binding_main")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", INCLUDE, "-I", BINDING,
                    os.path.join(BINDING, "binding_main.cpp"), "-o", exe] + _link_flags(),
                   check=True, capture_output=True, timeout=300)
    return exe


def test_adapter_compiles_and_links_against_standins(binding_exe):
    assert os.access(binding_exe, os.X_OK)


def _apply_diff(src, diff):
    """Apply one unified-diff hunk without line numbers: the context and '-'
    lines must appear verbatim in src."""
    old, new = [], []
    for line in diff.splitlines():
        tag, body = line[:1], line[1:]
        if tag in (" ", "-"):
            old.append(body)
        if tag in (" ", "+"):
            new.append(body)
    old_t, new_t = "\n".join(old) + "\n", "\n".join(new) + "\n"
    assert src.count(old_t) == 1, "the INTEGRATION.md diff does not apply to System.hpp"
    return src.replace(old_t, new_t)


def test_binding_builds_against_reference_headers(pkg, tmp_path):
    if not os.path.isfile(REF_ROOT_FILE):
        pytest.skip("the reference was not compiled on this machine")
    ref = open(REF_ROOT_FILE).read().strip()
    ref_inc = os.path.join(ref, "projects", "nbody_core", "include")
    if not os.path.isdir(ref_inc):
        pytest.skip("the reference's headers are not present")
    pkg.load_library()
    (diff,) = _blocks("diff")
    patched = tmp_path / "inc" / "ngrav"
    patched.mkdir(parents=True)
    src = open(os.path.join(ref_inc, "ngrav", "System.hpp")).read()
    (patched / "System.hpp").write_text(_apply_diff(src, diff))
    tu = tmp_path / "uses_binding.cpp"
    tu.write_text(
        '#include "ngrav/System.hpp"\n'
        '#include "ngrav_gpu_accelfn.hpp"\n'
        "int main() {\n"
        "    ngrav::System<3> sys;\n"
        "    ngrav::StepParams sp;\n"
        "    sys.SetAuxSolver(ngrav::Solver::BarnesHut, ngrav_gpu::GpuBarnesHut(sp, 16));\n"
        "    ngrav::SoA<3> s, out;\n"
        "    sys.ComputeAccel(ngrav::Solver::BarnesHut, s, sp, out);\n"
        "    return 0;\n"
        "}\n")
    ref_lib = os.path.join(ROOT, "oracle", "_ref")
    subprocess.run(["g++", "-std=gnu++20", "-O1", "-fopenmp", "-I", str(tmp_path / "inc"),
                    "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", ref_inc,
                    "-I", os.path.join(ref_inc, "ngrav"),  # the copy's sibling includes ("Integrator.hpp")
                    "-I", INCLUDE, str(tu),
                    "-o", str(tmp_path / "uses_binding"), "-L", ref_lib, "-lngrav_ref", "-Wl,-rpath," + ref_lib]
                   + _link_flags(), check=True, capture_output=True, timeout=600)


@pytest.mark.gpu
def test_registered_adapter_matches_reference_accelerations(binding_exe, tmp_path):
    d = load_golden("plummer16k.npz")
    n = len(d["x"])
    inp = np.concatenate([d["x"], d["y"], d["z"], d["m"],
                          [float(d["G"]), float(d["eps"]), float(d["theta"]), float(d["ncrit"])]]).astype(np.float64)
    inp.tofile(tmp_path / "in.f64")
    r = subprocess.run([binding_exe, str(n), str(tmp_path / "in.f64"), str(tmp_path / "out.f64")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(tmp_path / "out.f64").reshape(2, 3, n)
    ref = np.stack([d["ax"], d["ay"], d["az"]])
    for k in range(2):
        rel = np.linalg.norm(out[k] - ref, axis=0) / np.linalg.norm(ref, axis=0)
        assert np.median(rel) <= 1e-5 and rel.max() <= 1e-4, (k, np.median(rel), rel.max())
