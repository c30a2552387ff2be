"""ngrav_gpu_diagnostics_noalloc: diagnostics without any device allocation.

It exists for callers that cannot allocate device memory (a loop under a
framework's caching allocator that owns the device memory, or one that must
keep cudaMalloc/cudaFree out of its frame loop).  Through the C-ABI it must
give the same FP64 diagnostics as the context entry point
ngrav_gpu_diagnostics, on two calls in a row (the static scratch keeps the
previous call's contents, which must not leak into the next result).

This file is collected last on purpose, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_noalloc_matches_context_diagnostics_twice(pkg):
    torch = pytest.importorskip("torch")
    d = load_golden("plummer16k.npz")
    G, eps = float(d["G"]), float(d["eps"])
    with pkg.NBodySystem(pkg.StepParams(G=G, eps=eps), leaf_capacity=16) as sim:
        sim.set_particles(d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"], d["m"])
        ref = sim.diagnostics(exact_potential=True)
    dev = [torch.tensor(np.asarray(d[k], dtype=np.float32), device="cuda:0")
           for k in ("x", "y", "z", "vx", "vy", "vz", "m")]
    torch.cuda.synchronize()
    n = len(d["x"])
    for _ in range(2):
        got = pkg.diagnostics_noalloc(0, n, *[t.data_ptr() for t in dev], G, eps, with_potential=True)
        assert got["potential_exact"]
        assert got["kinetic"] == pytest.approx(ref["kinetic"], rel=1e-12)
        assert got["potential"] == pytest.approx(ref["potential"], rel=1e-10)
        assert got["energy"] == pytest.approx(ref["energy"], rel=1e-10)
        np.testing.assert_allclose(got["com"], ref["com"], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(got["L"], ref["L"], rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(got["P"], ref["P"], rtol=1e-12, atol=1e-14)


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    L = pkg.load_library()
    out = pkg.Diag()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ngrav_gpu_diagnostics_noalloc(0, pkg.NOALLOC_MAX_N + 1, *([dummy] * 7), 1.0, 0.01, 0, ctypes.byref(out))
    assert rc == 1  # NGRAV_ERR_INVALID_ARG
