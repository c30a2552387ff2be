"""ngrav_gpu_diagnostics_noalloc: diagnostics without any device allocation.

It exists for callers that cannot allocate device memory (a loop under a
framework's caching allocator that owns the device memory, or one that must
keep cudaMalloc/cudaFree out of its frame loop).  Through the C-ABI it must
give the same FP64 diagnostics as the reference's System diagnostics (the
golden diag0 of the 16,384-particle Plummer sphere, and the oracle on a size
that leaves a partial last block) and as the context entry point
ngrav_gpu_diagnostics, on two calls in a row (the static scratch keeps the
previous call's contents, which must not leak into the next result).

This file is collected last on purpose, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes
import math

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m")


def _device_arrays(torch, d, n):
    dev = [torch.tensor(np.asarray(d[k][:n], dtype=np.float32), device="cuda:0") for k in FIELDS]
    torch.cuda.synchronize()
    return dev


def test_noalloc_matches_golden_and_context_twice(pkg):
    torch = pytest.importorskip("torch")
    d = load_golden("plummer16k.npz")
    G, eps = float(d["G"]), float(d["eps"])
    ref = d["diag0"]  # the reference's E, COM, L, P of the initial state
    with pkg.NBodySystem(pkg.StepParams(G=G, eps=eps), leaf_capacity=16) as sim:
        sim.set_particles(*(d[k] for k in FIELDS))
        ctx = sim.diagnostics(exact_potential=True)
    n = len(d["x"])
    dev = _device_arrays(torch, d, n)
    for _ in range(2):
        got = pkg.diagnostics_noalloc(0, n, *[t.data_ptr() for t in dev], G, eps, with_potential=True)
        assert got["potential_exact"]
        assert got["energy"] == pytest.approx(ref[0], rel=1e-10)
        np.testing.assert_allclose(got["com"], ref[1:4], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(got["L"], ref[4:7], rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(got["P"], ref[7:10], rtol=1e-12, atol=1e-14)
        assert got["kinetic"] == pytest.approx(ctx["kinetic"], rel=1e-12)
        assert got["potential"] == pytest.approx(ctx["potential"], rel=1e-10)


def test_noalloc_partial_last_block_matches_oracle_twice(pkg, oracle):
    """n = 10,007: three 4,096-particle blocks, the last one partial, and a
    partial last 256-target potential tile."""
    torch = pytest.importorskip("torch")
    d = load_golden("plummer16k.npz")
    G, eps, n = float(d["G"]), float(d["eps"]), 10007
    ref = oracle.diagnostics(*(np.asarray(d[k][:n], dtype=np.float32) for k in FIELDS), G, eps)
    dev = _device_arrays(torch, d, n)
    for _ in range(2):
        got = pkg.diagnostics_noalloc(0, n, *[t.data_ptr() for t in dev], G, eps, with_potential=True)
        assert got["energy"] == pytest.approx(ref[0], rel=1e-10)
        np.testing.assert_allclose(got["com"], ref[1:4], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(got["L"], ref[4:7], rtol=1e-9, atol=1e-14)
        np.testing.assert_allclose(got["P"], ref[7:10], rtol=1e-12, atol=1e-14)


def test_noalloc_without_potential_reports_nan_energy(pkg):
    torch = pytest.importorskip("torch")
    d = load_golden("plummer16k.npz")
    G, eps, n = float(d["G"]), float(d["eps"]), 10007
    dev = _device_arrays(torch, d, n)
    with_pot = pkg.diagnostics_noalloc(0, n, *[t.data_ptr() for t in dev], G, eps, with_potential=True)
    got = pkg.diagnostics_noalloc(0, n, *[t.data_ptr() for t in dev], G, eps, with_potential=False)
    assert not got["potential_exact"]
    assert math.isnan(got["potential"]) and math.isnan(got["energy"])
    assert got["kinetic"] == with_pot["kinetic"]
    assert got["L"] == with_pot["L"] and got["P"] == with_pot["P"] and got["com"] == with_pot["com"]


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    L = pkg.load_library()
    out = pkg.Diag()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ngrav_gpu_diagnostics_noalloc(0, pkg.NOALLOC_MAX_N + 1, *([dummy] * 7), 1.0, 0.01, 0, ctypes.byref(out))
    assert rc == 1  # NGRAV_ERR_INVALID_ARG
