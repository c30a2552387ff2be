"""GB300 Barnes-Hut force evaluation and KDK step (Python host side).

A thin ctypes mirror of ``include/ngrav_gpu.h`` that reads like the
reference's ``ngrav::System<3>`` (projects/nbody_core/include/ngrav/System.hpp):

    sim = NBodySystem(StepParams(G=1.0, eps=0.01, theta=0.5), leaf_capacity=16)
    sim.set_particles(x, y, z, vx, vy, vz, m)     # System::SetParticles
    sim.prime()                                     # System::Prime
    sim.step(nsteps, dt)                            # System::Step (KDK)
    ax, ay, az = sim.compute_accel()                # ComputeAccelBarnesHut
    d = sim.diagnostics()                           # TotalEnergy / COM / L / P

All compute runs in ``libngrav_gpu.so`` (hand-written sm_103a kernels).  There
is no CPU fallback: constructing a system without the library or without a
GPU raises.  The directory name contains a hyphen, so import it through
``load()`` or ``importlib`` (module name ``opengl_physics_gb300``).
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libngrav_gpu.so")
HEADER = os.path.join(os.path.dirname(PKG_DIR), "include", "ngrav_gpu.h")

ABI_VERSION = 1
OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "no particles", 4: "capacity", 5: "non-finite input",
          6: "out of memory", 7: "timeout", 8: "depth limit"}
MAC_GEOMETRIC, MAC_LEARNED, MAC_RELATIVE = 0, 1, 2
SOFTENING_PLUMMER, SOFTENING_SPLINE = 0, 1
PRECISION_PLAIN, PRECISION_SPLIT = 0, 1

# Every extern "C" entry point declared in include/ngrav_gpu.h.
EXPORTS = (
    "ngrav_gpu_default_opts", "ngrav_gpu_create", "ngrav_gpu_destroy", "ngrav_gpu_last_error",
    "ngrav_gpu_set_opts", "ngrav_gpu_set_particles", "ngrav_gpu_set_particles_f32", "ngrav_gpu_compute_accel",
    "ngrav_gpu_set_state", "ngrav_gpu_set_state_f32", "ngrav_gpu_set_softening", "ngrav_gpu_set_mac_alpha",
    "ngrav_gpu_block_step", "ngrav_gpu_get_rungs", "ngrav_gpu_adaptive_dt",
    "ngrav_gpu_get_frame_f32",
    "ngrav_gpu_prime", "ngrav_gpu_step", "ngrav_gpu_get_state", "ngrav_gpu_get_accel", "ngrav_gpu_diagnostics",
    "ngrav_gpu_force_error", "ngrav_gpu_get_stats", "ngrav_gpu_debug_tree", "ngrav_gpu_debug_shrink_pools",
    "ngrav_gpu_reset_cumulative",
    "ngrav_gpu_probe_fp32_peak", "ngrav_gpu_diagnostics_noalloc",
    "ngrav_gpu_set_ensemble", "ngrav_gpu_ensemble_force_error", "ngrav_gpu_ensemble_diagnostics",
    "ngrav_gpu_default_tune_opts", "ngrav_gpu_autotune", "ngrav_gpu_set_tuning",
    "ngrav_gpu_lmac_default_opts", "ngrav_gpu_lmac_set_opts", "ngrav_gpu_lmac_default_train_opts",
    "ngrav_gpu_lmac_train", "ngrav_gpu_lmac_get_model", "ngrav_gpu_lmac_set_model", "ngrav_gpu_lmac_reset",
    "ngrav_gpu_lmac_collect", "ngrav_gpu_lmac_forward", "ngrav_gpu_lmac_forward_tc", "ngrav_gpu_lmac_grad",
)
LMAC_PARAMS = 1377
LMAC_FEATURES = 8
NOALLOC_MAX_N = 16777216


class Opts(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int), ("device", ctypes.c_int), ("leaf_capacity", ctypes.c_int),
                ("max_depth", ctypes.c_int), ("quadrupole", ctypes.c_int), ("mac", ctypes.c_int),
                ("precision", ctypes.c_int), ("fp64_mac_retest", ctypes.c_int), ("strict_depth", ctypes.c_int),
                ("timing", ctypes.c_int), ("G", ctypes.c_double), ("eps", ctypes.c_double),
                ("theta", ctypes.c_double)]


class Diag(ctypes.Structure):
    _fields_ = [("kinetic", ctypes.c_double), ("potential", ctypes.c_double), ("energy", ctypes.c_double),
                ("com", ctypes.c_double * 3), ("L", ctypes.c_double * 3), ("P", ctypes.c_double * 3),
                ("potential_exact", ctypes.c_int)]


class Ferr(ctypes.Structure):
    _fields_ = [("rms", ctypes.c_double), ("max", ctypes.c_double), ("median", ctypes.c_double),
                ("mean", ctypes.c_double),
                ("nsample", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_bbox_keys", ctypes.c_double), ("ms_sort", ctypes.c_double), ("ms_build", ctypes.c_double),
                ("ms_moments", ctypes.c_double), ("ms_walk", ctypes.c_double), ("ms_force", ctypes.c_double),
                ("ms_total", ctypes.c_double), ("p2p_pairs", ctypes.c_longlong), ("p2c_terms", ctypes.c_longlong),
                ("mac_tests", ctypes.c_longlong), ("mac_retests", ctypes.c_longlong), ("groups", ctypes.c_longlong),
                ("nodes", ctypes.c_int), ("leaves", ctypes.c_int), ("levels", ctypes.c_int),
                ("max_leaf_count", ctypes.c_int), ("depth_limited_leaves", ctypes.c_int),
                ("walk_stack_max", ctypes.c_int), ("status_bits", ctypes.c_uint), ("force_evals", ctypes.c_longlong),
                ("n", ctypes.c_longlong), ("cum_evals", ctypes.c_longlong), ("cum_p2p_pairs", ctypes.c_longlong),
                ("cum_p2c_terms", ctypes.c_longlong), ("cum_ms_walk", ctypes.c_double),
                ("cum_ms_force", ctypes.c_double), ("cum_ms_eval", ctypes.c_double),
                ("cum_ms_step", ctypes.c_double), ("cum_launches", ctypes.c_longlong),
                ("far_entries", ctypes.c_longlong), ("near_entries", ctypes.c_longlong), ("list_max", ctypes.c_int),
                ("lmac_queries", ctypes.c_longlong), ("lmac_accepts", ctypes.c_longlong),
                ("lmac_fallbacks", ctypes.c_longlong), ("lmac_flushes", ctypes.c_longlong),
                ("lmac_screened", ctypes.c_longlong),
                ("lmac_active", ctypes.c_int), ("lmac_reverted", ctypes.c_int), ("lmac_checks", ctypes.c_int),
                ("lmac_last_check_rms", ctypes.c_double), ("graph_captures", ctypes.c_longlong),
                ("graph_replays", ctypes.c_longlong), ("cum_particle_evals", ctypes.c_longlong),
                ("sort_passes", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneOpts(ctypes.Structure):
    _fields_ = [("reps", ctypes.c_int), ("check_targets", ctypes.c_int), ("rms_tolerance", ctypes.c_double),
                ("leaf_capacities", ctypes.c_int * 8)]


class TuneReport(ctypes.Structure):
    _fields_ = [("leaf_capacity", ctypes.c_int), ("p2p_tile", ctypes.c_int), ("walk_stack", ctypes.c_int),
                ("ms_before", ctypes.c_double), ("ms_after", ctypes.c_double), ("rms_before", ctypes.c_double),
                ("rms_after", ctypes.c_double), ("ntried", ctypes.c_int), ("tried", (ctypes.c_double * 5) * 32)]


class LmacOpts(ctypes.Structure):
    _fields_ = [("budget", ctypes.c_double), ("gate", ctypes.c_double), ("rho_lo", ctypes.c_double),
                ("rho_hi", ctypes.c_double), ("check_every", ctypes.c_int), ("check_targets", ctypes.c_int),
                ("revert_rms", ctypes.c_double), ("rounds", ctypes.c_int), ("screen", ctypes.c_double)]


class LmacTrainOpts(ctypes.Structure):
    _fields_ = [("snapshots", ctypes.c_int), ("steps_between", ctypes.c_int), ("dt", ctypes.c_double),
                ("pairs", ctypes.c_longlong), ("theta_record", ctypes.c_double), ("u_range", ctypes.c_double),
                ("epochs", ctypes.c_int), ("batch", ctypes.c_int), ("lr", ctypes.c_double), ("seed", ctypes.c_uint64)]


class LmacReport(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_longlong), ("band_pairs", ctypes.c_longlong), ("loss_first", ctypes.c_double),
                ("loss_last", ctypes.c_double), ("acc_last", ctypes.c_double), ("val_loss", ctypes.c_double),
                ("val_acc", ctypes.c_double), ("ms_data", ctypes.c_double), ("ms_train", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)
_U64 = ctypes.POINTER(ctypes.c_uint64)
_lib = None


def library_path() -> str:
    return LIB_PATH


EXE_PATH = os.path.join(PKG_DIR, "nbody_gb300")


def _run_build():
    from importlib import util as _u
    spec = _u.spec_from_file_location("_ngrav_build", os.path.join(PKG_DIR, "build.py"))
    mod = _u.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


def executable() -> str:
    """Path of the deck front end, nbody_gb300 (built with the library if absent)."""
    if not os.path.isfile(EXE_PATH):
        _run_build()
    return EXE_PATH


def load_library(path: str | None = None):
    """Load libngrav_gpu.so (building it if absent) and declare the C-ABI."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.isfile(path):
        _run_build()
    L = ctypes.CDLL(path)
    L.ngrav_gpu_default_opts.argtypes = [ctypes.POINTER(Opts)]
    L.ngrav_gpu_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Opts)]
    L.ngrav_gpu_destroy.argtypes = [ctypes.c_void_p]
    L.ngrav_gpu_destroy.restype = None
    L.ngrav_gpu_last_error.argtypes = [ctypes.c_void_p]
    L.ngrav_gpu_last_error.restype = ctypes.c_char_p
    L.ngrav_gpu_set_opts.argtypes = [ctypes.c_void_p, ctypes.POINTER(Opts)]
    L.ngrav_gpu_set_particles.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [_D] * 7
    L.ngrav_gpu_set_particles_f32.argtypes = [ctypes.c_void_p, ctypes.c_int64] + [_F] * 7
    L.ngrav_gpu_compute_accel.argtypes = [ctypes.c_void_p, _D, _D, _D]
    L.ngrav_gpu_set_state.argtypes = [ctypes.c_void_p] + [_D] * 6
    L.ngrav_gpu_set_softening.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.ngrav_gpu_set_mac_alpha.argtypes = [ctypes.c_void_p, ctypes.c_double]
    L.ngrav_gpu_adaptive_dt.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_double)]
    L.ngrav_gpu_get_frame_f32.argtypes = [ctypes.c_void_p, _F, _F]
    L.ngrav_gpu_get_rungs.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    L.ngrav_gpu_block_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]
    L.ngrav_gpu_set_state_f32.argtypes = [ctypes.c_void_p] + [_F] * 6
    L.ngrav_gpu_prime.argtypes = [ctypes.c_void_p]
    L.ngrav_gpu_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
    L.ngrav_gpu_get_state.argtypes = [ctypes.c_void_p] + [_D] * 6
    L.ngrav_gpu_get_accel.argtypes = [ctypes.c_void_p] + [_D] * 3
    L.ngrav_gpu_diagnostics.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Diag)]
    L.ngrav_gpu_force_error.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.POINTER(Ferr)]
    L.ngrav_gpu_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
    L.ngrav_gpu_debug_tree.argtypes = [ctypes.c_void_p, _I, _U64, _I, _I, _U64, _I, _I, _D, _D, _D, _D, _D, _D]
    L.ngrav_gpu_reset_cumulative.argtypes = [ctypes.c_void_p]
    L.ngrav_gpu_debug_shrink_pools.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4
    L.ngrav_gpu_probe_fp32_peak.argtypes = [ctypes.c_int, _D]
    L.ngrav_gpu_diagnostics_noalloc.argtypes = [ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 7 + \
        [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.POINTER(Diag)]
    L.ngrav_gpu_default_tune_opts.argtypes = [ctypes.POINTER(TuneOpts)]
    L.ngrav_gpu_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(TuneOpts), ctypes.POINTER(TuneReport)]
    L.ngrav_gpu_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.ngrav_gpu_set_ensemble.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.ngrav_gpu_ensemble_force_error.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, _D, _D]
    L.ngrav_gpu_ensemble_diagnostics.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Diag)]
    L.ngrav_gpu_lmac_default_opts.argtypes = [ctypes.POINTER(LmacOpts)]
    L.ngrav_gpu_lmac_set_opts.argtypes = [ctypes.c_void_p, ctypes.POINTER(LmacOpts)]
    L.ngrav_gpu_lmac_default_train_opts.argtypes = [ctypes.POINTER(LmacTrainOpts)]
    L.ngrav_gpu_lmac_train.argtypes = [ctypes.c_void_p, ctypes.POINTER(LmacTrainOpts), ctypes.POINTER(LmacReport)]
    L.ngrav_gpu_lmac_get_model.argtypes = [ctypes.c_void_p, _F, _F]
    L.ngrav_gpu_lmac_set_model.argtypes = [ctypes.c_void_p, _F, _F]
    L.ngrav_gpu_lmac_reset.argtypes = [ctypes.c_void_p]
    L.ngrav_gpu_lmac_collect.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_uint64, ctypes.c_int, _I,
                                         ctypes.POINTER(ctypes.c_longlong), _I, _I, _F, _F]
    L.ngrav_gpu_lmac_forward.argtypes = [ctypes.c_void_p, _F, ctypes.c_int, _F]
    L.ngrav_gpu_lmac_forward_tc.argtypes = [ctypes.c_void_p, _F, ctypes.c_int, _F]
    L.ngrav_gpu_lmac_grad.argtypes = [ctypes.c_void_p, _F, _F, _F, ctypes.c_int, _F, ctypes.c_double, _F,
                                      ctypes.POINTER(ctypes.c_double)]
    _lib = L
    return L


def diagnostics_noalloc(device, n, x, y, z, vx, vy, vz, m, G, eps, with_potential=False):
    """Conservation diagnostics of caller-owned device FP32 arrays (raw device
    pointers as ints), allocating no device memory (see the C header).  The
    exact potential costs n^2/2 FP64 pair terms, so it is opt-in; without it
    potential and energy are NaN."""
    L = load_library()
    d = Diag()
    rc = L.ngrav_gpu_diagnostics_noalloc(int(device), int(n), *[ctypes.c_void_p(int(p)) for p in
                                                                (x, y, z, vx, vy, vz, m)],
                                         float(G), float(eps), int(with_potential), ctypes.byref(d))
    if rc != OK:
        raise NgravError(rc, "ngrav_gpu_diagnostics_noalloc failed")
    return dict(kinetic=d.kinetic, potential=d.potential, energy=d.energy, com=list(d.com), L=list(d.L),
                P=list(d.P), potential_exact=int(d.potential_exact))


def probe_fp32_peak(device: int = 0) -> float:
    """Measured FP32 FMA throughput (TFLOP/s) of the device."""
    L = load_library()
    out = ctypes.c_double()
    rc = L.ngrav_gpu_probe_fp32_peak(device, ctypes.byref(out))
    if rc != OK:
        raise NgravError(rc, "FP32 peak probe failed")
    return out.value


class NgravError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ngrav_gpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


@dataclasses.dataclass
class StepParams:
    """Mirror of ngrav::StepParams (include/ngrav/Solvers.hpp:22-36) for the BH path."""
    G: float = 1.0
    eps: float = 0.05          # Plummer softening length
    theta: float = 0.5
    dt: float = 1e-3


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _c64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class NBodySystem:
    """One GPU context; mirrors System<3> for the Barnes-Hut solver."""

    def __init__(self, sp: StepParams | None = None, leaf_capacity: int = 8, precision: int = PRECISION_SPLIT,
                 quadrupole: bool = True, mac: int = MAC_GEOMETRIC, fp64_mac_retest: bool = True, device: int = 0,
                 max_depth: int = 40, timing: bool = False, strict_depth: bool = False):
        self.L = load_library()
        self.sp = sp or StepParams()
        o = Opts()
        self._check(self.L.ngrav_gpu_default_opts(ctypes.byref(o)), None)
        o.device = device
        o.leaf_capacity = leaf_capacity
        o.max_depth = max_depth
        o.quadrupole = int(quadrupole)
        o.mac = mac
        o.precision = precision
        o.fp64_mac_retest = int(fp64_mac_retest)
        o.strict_depth = int(strict_depth)
        o.timing = int(timing)
        o.G, o.eps, o.theta = self.sp.G, self.sp.eps, self.sp.theta
        self.opts = o
        h = ctypes.c_void_p()
        rc = self.L.ngrav_gpu_create(ctypes.byref(h), ctypes.byref(o))
        if rc != OK:
            raise NgravError(rc, "context creation failed (is a CUDA device visible?)")
        self.h = h
        self.n = 0

    def _check(self, rc, h):
        if rc != OK:
            msg = self.L.ngrav_gpu_last_error(h).decode() if h else ""
            raise NgravError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.L.ngrav_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_opts(self, **kw):
        for k, v in kw.items():
            setattr(self.opts, k, v)
        self._check(self.L.ngrav_gpu_set_opts(self.h, ctypes.byref(self.opts)), self.h)

    def set_particles(self, x, y, z, vx=None, vy=None, vz=None, m=None):
        arrs = [_c64(a) for a in (x, y, z, vx, vy, vz, m)]
        self.n = len(arrs[0])
        self.nsys = 1
        self._check(self.L.ngrav_gpu_set_particles(self.h, self.n, *[_p(a, _D) for a in arrs]), self.h)

    def set_particles_f32(self, x, y, z, vx, vy, vz, m):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, vx, vy, vz, m)]
        self.n = len(arrs[0])
        self.nsys = 1
        self._check(self.L.ngrav_gpu_set_particles_f32(self.h, self.n, *[_p(a, _F) for a in arrs]), self.h)

    def set_softening(self, kind):
        """SOFTENING_PLUMMER or SOFTENING_SPLINE (h = eps)."""
        self._check(self.L.ngrav_gpu_set_softening(self.h, int(kind)), self.h)

    def block_step(self, dt, eta=0.025, max_rung=8):
        """One coarse step with power-of-two rung timesteps; returns the largest rung used."""
        r = ctypes.c_int()
        self._check(self.L.ngrav_gpu_block_step(self.h, float(dt), float(eta), int(max_rung), ctypes.byref(r)),
                    self.h)
        return r.value

    def adaptive_dt(self, eta, dt_max):
        """ChooseAdaptiveDt on the current accelerations."""
        d = ctypes.c_double()
        self._check(self.L.ngrav_gpu_adaptive_dt(self.h, float(eta), float(dt_max), ctypes.byref(d)), self.h)
        return d.value

    def frame_f32(self):
        """(pos, vel) as N x 3 float32 in input order: the deck writer's frame fields."""
        pos = np.empty((self.n, 3), np.float32)
        vel = np.empty((self.n, 3), np.float32)
        self._check(self.L.ngrav_gpu_get_frame_f32(self.h, _p(pos, _F), _p(vel, _F)), self.h)
        return pos, vel

    def rungs(self):
        """Each particle's rung from the last block step (input order)."""
        out = np.zeros(self.n, np.int32)
        self._check(self.L.ngrav_gpu_get_rungs(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), self.h)
        return out

    def set_mac_alpha(self, alpha):
        """MacParams::alpha of the relative opening test."""
        self._check(self.L.ngrav_gpu_set_mac_alpha(self.h, float(alpha)), self.h)

    def set_state(self, x, y, z, vx=None, vy=None, vz=None):
        """New positions / velocities of the current particles (masses and the
        carried accelerations stay)."""
        arrs = [_c64(a) for a in (x, y, z, vx, vy, vz)]
        self._check(self.L.ngrav_gpu_set_state(self.h, *[_p(a, _D) for a in arrs]), self.h)

    def compute_accel(self):
        ax, ay, az = (np.empty(self.n) for _ in range(3))
        self._check(self.L.ngrav_gpu_compute_accel(self.h, _p(ax, _D), _p(ay, _D), _p(az, _D)), self.h)
        return ax, ay, az

    def prime(self):
        self._check(self.L.ngrav_gpu_prime(self.h), self.h)

    def step(self, nsteps=1, dt=None):
        self._check(self.L.ngrav_gpu_step(self.h, int(nsteps), float(self.sp.dt if dt is None else dt)), self.h)

    def state(self):
        out = [np.empty(self.n) for _ in range(6)]
        self._check(self.L.ngrav_gpu_get_state(self.h, *[_p(a, _D) for a in out]), self.h)
        return tuple(out)

    def accel(self):
        out = [np.empty(self.n) for _ in range(3)]
        self._check(self.L.ngrav_gpu_get_accel(self.h, *[_p(a, _D) for a in out]), self.h)
        return tuple(out)

    def diagnostics(self, exact_potential=False):
        d = Diag()
        self._check(self.L.ngrav_gpu_diagnostics(self.h, int(exact_potential), ctypes.byref(d)), self.h)
        return dict(kinetic=d.kinetic, potential=d.potential, energy=d.energy, com=list(d.com), L=list(d.L),
                    P=list(d.P), potential_exact=int(d.potential_exact))

    def force_error(self, nsample=4096, seed=12345, fp64_pairs=False):
        f = Ferr()
        self._check(self.L.ngrav_gpu_force_error(self.h, int(nsample), int(seed), int(fp64_pairs),
                                                 ctypes.byref(f)), self.h)
        return dict(rms=f.rms, max=f.max, median=f.median, mean=f.mean, nsample=f.nsample)

    def stats(self):
        s = Stats()
        self._check(self.L.ngrav_gpu_get_stats(self.h, ctypes.byref(s)), self.h)
        return s.as_dict()

    def reset_cumulative(self):
        self._check(self.L.ngrav_gpu_reset_cumulative(self.h), self.h)

    def debug_shrink_pools(self, node_cap=0, far_chunks=0, near_chunks=0, pend_chunks=0):
        """Testing: replace each pool given (> 0) by one of exactly that size,
        so the next evaluation must detect the overflow, grow and re-run."""
        self._check(self.L.ngrav_gpu_debug_shrink_pools(self.h, int(node_cap), int(far_chunks), int(near_chunks),
                                                        int(pend_chunks)), self.h)

    def debug_tree(self):
        nn = ctypes.c_int()
        self._check(self.L.ngrav_gpu_debug_tree(self.h, ctypes.byref(nn), *([None] * 12)), self.h)
        k, n = nn.value, self.n
        t = dict(keys=np.zeros(n, np.uint64), order=np.zeros(n, np.int32), level=np.zeros(k, np.int32),
                 prefix=np.zeros(k, np.uint64), count=np.zeros(k, np.int32), is_leaf=np.zeros(k, np.int32),
                 center=np.zeros((k, 3)), half=np.zeros(k), com=np.zeros((k, 3)), mass=np.zeros(k),
                 max_radius=np.zeros(k), quad=np.zeros((k, 5)))
        self._check(self.L.ngrav_gpu_debug_tree(
            self.h, ctypes.byref(nn), _p(t["keys"], _U64), _p(t["order"], _I), _p(t["level"], _I),
            _p(t["prefix"], _U64), _p(t["count"], _I), _p(t["is_leaf"], _I), _p(t["center"], _D),
            _p(t["half"], _D), _p(t["com"], _D), _p(t["mass"], _D), _p(t["max_radius"], _D),
            _p(t["quad"], _D)), self.h)
        return t


    # ---- autotuner ----
    def autotune(self, reps=2, check_targets=2048, rms_tolerance=1.1, leaf_capacities=None):
        """Pick leaf capacity, P2P tile and walk stack by timing this state; installs the choice."""
        o = TuneOpts()
        self._check(self.L.ngrav_gpu_default_tune_opts(ctypes.byref(o)), None)
        o.reps, o.check_targets, o.rms_tolerance = reps, check_targets, rms_tolerance
        if leaf_capacities is not None:
            for i in range(8):
                o.leaf_capacities[i] = leaf_capacities[i] if i < len(leaf_capacities) else 0
        r = TuneReport()
        self._check(self.L.ngrav_gpu_autotune(self.h, ctypes.byref(o), ctypes.byref(r)), self.h)
        self.opts.leaf_capacity = r.leaf_capacity
        tried = [list(r.tried[i]) for i in range(r.ntried)]
        return dict(leaf_capacity=r.leaf_capacity, p2p_tile=r.p2p_tile, walk_stack=r.walk_stack,
                    ms_before=r.ms_before, ms_after=r.ms_after, rms_before=r.rms_before, rms_after=r.rms_after,
                    tried=tried)

    def set_tuning(self, p2p_tile=0, walk_stack=2048):
        self._check(self.L.ngrav_gpu_set_tuning(self.h, int(p2p_tile), int(walk_stack)), self.h)

    # ---- ensembles ----
    def set_ensemble(self, offsets):
        """Treat the particles as independent systems: system s is
        [offsets[s], offsets[s+1]) of the arrays passed to set_particles."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        self.nsys = len(off) - 1
        self._check(self.L.ngrav_gpu_set_ensemble(self.h, self.nsys, off.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64))), self.h)

    def ensemble_force_error(self, targets_per_system=256, seed=1):
        k = getattr(self, "nsys", 1)
        rms, mx = np.zeros(k), np.zeros(k)
        self._check(self.L.ngrav_gpu_ensemble_force_error(self.h, int(targets_per_system), int(seed), _p(rms, _D),
                                                          _p(mx, _D)), self.h)
        return rms, mx

    def ensemble_diagnostics(self, exact_potential=False):
        k = getattr(self, "nsys", 1)
        arr = (Diag * k)()
        self._check(self.L.ngrav_gpu_ensemble_diagnostics(self.h, int(exact_potential), arr), self.h)
        return [dict(kinetic=d.kinetic, potential=d.potential, energy=d.energy, com=list(d.com), L=list(d.L),
                     P=list(d.P), potential_exact=int(d.potential_exact)) for d in arr]

    # ---- learned opening test ----
    def lmac_set_opts(self, **kw):
        """Run-time options of the learned test (budget, gate, rho_lo/rho_hi, check_every,
        check_targets, revert_rms); unspecified ones keep the library defaults."""
        o = LmacOpts()
        self._check(self.L.ngrav_gpu_lmac_default_opts(ctypes.byref(o)), None)
        for k, v in kw.items():
            setattr(o, k, v)
        self._check(self.L.ngrav_gpu_lmac_set_opts(self.h, ctypes.byref(o)), self.h)

    def lmac_train(self, **kw):
        """Generate labelled pairs on this system and train the network; returns the report."""
        o = LmacTrainOpts()
        self._check(self.L.ngrav_gpu_lmac_default_train_opts(ctypes.byref(o)), None)
        for k, v in kw.items():
            setattr(o, k, v)
        r = LmacReport()
        self._check(self.L.ngrav_gpu_lmac_train(self.h, ctypes.byref(o), ctypes.byref(r)), self.h)
        return r.as_dict()

    def lmac_get_model(self):
        p = np.zeros(LMAC_PARAMS, np.float32)
        nrm = np.zeros(2 * LMAC_FEATURES, np.float32)
        self._check(self.L.ngrav_gpu_lmac_get_model(self.h, _p(p, _F), _p(nrm, _F)), self.h)
        return p, nrm

    def lmac_set_model(self, params, norm):
        p = np.ascontiguousarray(params, dtype=np.float32)
        nrm = np.ascontiguousarray(norm, dtype=np.float32)
        self._check(self.L.ngrav_gpu_lmac_set_model(self.h, _p(p, _F), _p(nrm, _F)), self.h)

    def lmac_reset(self):
        self._check(self.L.ngrav_gpu_lmac_reset(self.h), self.h)

    def lmac_collect(self, theta_record=0.3, rho_lo=0.25, rho_hi=1.25, keep=1.0, seed=1, cap=65536):
        """Band pairs of the current tree with their features and labels."""
        npairs = ctypes.c_int()
        nband = ctypes.c_longlong()
        g = np.zeros(cap, np.int32)
        nd = np.zeros(cap, np.int32)
        X = np.zeros((cap, LMAC_FEATURES), np.float32)
        r = np.zeros(cap, np.float32)
        self._check(self.L.ngrav_gpu_lmac_collect(self.h, theta_record, rho_lo, rho_hi, keep, int(seed), int(cap),
                                                  ctypes.byref(npairs), ctypes.byref(nband), _p(g, _I), _p(nd, _I),
                                                  _p(X, _F), _p(r, _F)), self.h)
        k = npairs.value
        return dict(group=g[:k], node=nd[:k], X=X[:k], r=r[:k], nband=nband.value)

    def lmac_forward(self, x_std):
        x = np.ascontiguousarray(x_std, dtype=np.float32)
        z = np.zeros(len(x), np.float32)
        self._check(self.L.ngrav_gpu_lmac_forward(self.h, _p(x, _F), len(x), _p(z, _F)), self.h)
        return z

    def lmac_forward_tc(self, x_raw):
        x = np.ascontiguousarray(x_raw, dtype=np.float32)
        z = np.zeros(len(x), np.float32)
        self._check(self.L.ngrav_gpu_lmac_forward_tc(self.h, _p(x, _F), len(x), _p(z, _F)), self.h)
        return z

    def lmac_grad(self, x_std, y, w=None, params=None, scale=1.0):
        x = np.ascontiguousarray(x_std, dtype=np.float32)
        yy = np.ascontiguousarray(y, dtype=np.float32)
        ww = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        pp = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        g = np.zeros(LMAC_PARAMS, np.float32)
        loss = ctypes.c_double()
        self._check(self.L.ngrav_gpu_lmac_grad(self.h, _p(x, _F), _p(yy, _F), _p(ww, _F), len(x), _p(pp, _F),
                                               float(scale), _p(g, _F), ctypes.byref(loss)), self.h)
        return g, loss.value


def canonical(tree: dict) -> dict:
    """Node rows sorted by (level, prefix) -- a numbering-independent topology."""
    idx = np.lexsort((tree["prefix"], tree["level"]))
    return {k: (v[idx] if k not in ("keys", "order") else v) for k, v in tree.items()}
