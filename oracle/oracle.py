"""ctypes front end of the oracle and of the compiled reference.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline legs, never by the product package.

* :class:`Oracle` wraps ``oracle/libngrav_oracle.so`` -- the C restatement of
  the reference's CPU Barnes-Hut path (oracle/ngrav_oracle.c).  It builds on
  any host with gcc (``make -C oracle``).
* :class:`Reference` wraps ``oracle/_ref/libngrav_ref.so`` -- the reference's
  own sources compiled by ``oracle/build_ref.sh``.  It exists only where the
  reference sources are present (the build container); the golden fixtures in
  ``tests/golden/`` carry its results elsewhere.

Both expose the same methods, so a test can run either side on the same input.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libngrav_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libngrav_ref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_U64 = ctypes.POINTER(ctypes.c_ulonglong)


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def build_oracle() -> str:
    """Compile the C restatement with ``make -C oracle``; returns the .so path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


def build_reference(ref_root: str | None = None) -> str | None:
    """Compile the reference's own CPU path if its sources are present.

    ref_root, else $NGRAV_REFERENCE, else the location build_ref.sh knows; the
    recipe exits 3 when the sources are absent (e.g. on a machine that only
    runs the prebuilt files), and then this returns None."""
    root = ref_root or os.environ.get("NGRAV_REFERENCE")
    cmd = ["bash", os.path.join(HERE, "build_ref.sh")] + ([root] if root else [])
    r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode == 3:
        return None
    if r.returncode != 0:
        raise RuntimeError("build_ref.sh failed:\n" + r.stderr)
    return REF_SO


class _Tree(dict):
    """Node arrays of one tree (creation-order numbering) + its permutation."""

    def canonical(self):
        """Rows sorted by (level, prefix): numbering-independent topology."""
        idx = np.lexsort((self["prefix"], self["level"]))
        return {k: (self[k][idx] if k != "order" else self[k]) for k in self}


class _Common:
    _prefix = ""

    def _fn(self, name):
        return getattr(self.lib, self._prefix + name)

    def tree(self, x, y, z, m, ncrit=8, max_depth=40):
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        nn = ctypes.c_int()
        h = self._tree_create(n, x, y, z, m, ncrit, max_depth, ctypes.byref(nn))
        if not h:
            raise RuntimeError("tree build failed")
        k = nn.value
        t = _Tree(
            level=np.zeros(k, np.int32), prefix=np.zeros(k, np.uint64), count=np.zeros(k, np.int32),
            is_leaf=np.zeros(k, np.int32), center=np.zeros((k, 3)), half=np.zeros(k), com=np.zeros((k, 3)),
            mass=np.zeros(k), max_radius=np.zeros(k), quad=np.zeros((k, 5)), order=np.zeros(n, np.int32),
            parent=np.zeros(k, np.int32), first=np.zeros(k, np.int32))
        self._tree_export(h, n, t)
        self._tree_free(h)
        return t

    def direct(self, x, y, z, m, G, eps):
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
        self._direct(n, x, y, z, m, G, eps, ax, ay, az)
        return ax, ay, az

    def diagnostics(self, x, y, z, vx, vy, vz, m, G, eps):
        arrs = list(map(_f64, (x, y, z, vx, vy, vz, m)))
        out = np.zeros(10)
        self._fn("diagnostics")(len(arrs[0]), *[_dp(a) for a in arrs], ctypes.c_double(G), ctypes.c_double(eps),
                                _dp(out))
        return out


def _set_softening(self, kind):
    """0: Plummer, 1: cubic spline with h = eps, for every later call."""
    self.lib.or_set_softening(int(kind))


class Oracle(_Common):
    """The C restatement (oracle/ngrav_oracle.c)."""

    _prefix = "or_"
    set_softening = _set_softening

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.isfile(path):
            build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.or_tree_create.restype = ctypes.c_void_p
        L.or_tree_create.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I]
        L.or_tree_export.argtypes = [ctypes.c_void_p, _I, _U64, _I, _I, _D, _D, _D, _D, _D, _D, _I, _I, _I]
        L.or_tree_destroy.argtypes = [ctypes.c_void_p]
        L.or_bh_accel.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_void_p]
        L.or_direct.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, _D, _D, _D]
        L.or_direct_targets.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, _I, _D, _D, _D]
        L.or_leapfrog.argtypes = [ctypes.c_int] + [_D] * 10 + [ctypes.c_double] * 3 + [ctypes.c_int,
                                                                                       ctypes.c_double,
                                                                                       ctypes.c_int, ctypes.c_int]
        L.or_force_error.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                     _I, _D, _D, _D, _D]
        L.or_num_threads.restype = ctypes.c_int

    def num_threads(self) -> int:
        return int(self.lib.or_num_threads())

    def time_sampled(self, x, y, z, m, G, eps, theta, ncrit, group_stride, quad=True, with_acc=False):
        """(build_ms, walk_ms, fraction_walked, pairs) of a sampled grouped walk on a full tree;
        with_acc: also (ax, ay, az) of the walked targets (NaN for the others)."""
        x, y, z, m = map(_f64, (x, y, z, m))
        out = np.zeros(4)
        acc = np.empty(3 * len(x)) if with_acc else None
        fn = self.lib.or_bh_time_sampled
        fn.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                       ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
        if fn(len(x), _dp(x), _dp(y), _dp(z), _dp(m), G, eps, theta, ncrit, int(quad), int(group_stride), _dp(out),
              _dp(acc) if with_acc else None):
            raise RuntimeError("or_bh_time_sampled failed")
        res = (float(out[0]), float(out[1]), float(out[2]), float(out[3]))
        if with_acc:
            n = len(x)
            return res + ((acc[:n], acc[n:2 * n], acc[2 * n:]),)
        return res

    def _tree_create(self, n, x, y, z, m, ncrit, max_depth, nn):
        return self.lib.or_tree_create(n, _dp(x), _dp(y), _dp(z), _dp(m), ncrit, max_depth, 1, nn)

    def _tree_export(self, h, n, t):
        self.lib.or_tree_export(h, _ip(t["level"]), t["prefix"].ctypes.data_as(_U64), _ip(t["count"]),
                                _ip(t["is_leaf"]), _dp(t["center"]), _dp(t["half"]), _dp(t["com"]),
                                _dp(t["mass"]), _dp(t["max_radius"]), _dp(t["quad"]), _ip(t["order"]),
                                _ip(t["parent"]), _ip(t["first"]))

    def _tree_free(self, h):
        self.lib.or_tree_destroy(h)

    def _direct(self, n, x, y, z, m, G, eps, ax, ay, az):
        self.lib.or_direct(n, _dp(x), _dp(y), _dp(z), _dp(m), G, eps * eps, _dp(ax), _dp(ay), _dp(az))

    def bh_accel(self, x, y, z, m, G, eps, theta, ncrit=8, quad=True, counters=False):
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
        cnt = (ctypes.c_longlong * 4)()
        rc = self.lib.or_bh_accel(n, _dp(x), _dp(y), _dp(z), _dp(m), G, eps, theta, ncrit, int(quad), _dp(ax),
                                  _dp(ay), _dp(az), ctypes.cast(cnt, ctypes.c_void_p))
        if rc:
            raise RuntimeError("or_bh_accel failed")
        if counters:
            return ax, ay, az, dict(p2p_pairs=cnt[0], p2c_terms=cnt[1], mac_tests=cnt[2], groups=cnt[3])
        return ax, ay, az

    def direct_targets(self, x, y, z, m, G, eps, targets):
        x, y, z, m = map(_f64, (x, y, z, m))
        tg = np.ascontiguousarray(targets, dtype=np.int32)
        nt = len(tg)
        ax, ay, az = np.zeros(nt), np.zeros(nt), np.zeros(nt)
        self.lib.or_direct_targets(len(x), _dp(x), _dp(y), _dp(z), _dp(m), G, eps * eps, nt, _ip(tg), _dp(ax),
                                   _dp(ay), _dp(az))
        return ax, ay, az

    def bh_pp_accel(self, x, y, z, m, G, eps, theta, ncrit=8, quad=True, relative=False, alpha=0.001, aold=None,
                    targets=None, counters=False):
        """Per-particle walk (WalkBH): geometric or relative MAC; targets = bool mask."""
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
        ao = None if aold is None else _f64(aold)
        tg = None if targets is None else np.ascontiguousarray(targets, dtype=np.uint8)
        cnt = np.zeros(4, np.int64)
        fn = self.lib.or_bh_pp_accel
        fn.restype = ctypes.c_int
        rc = fn(n, _dp(x), _dp(y), _dp(z), _dp(m), ctypes.c_double(G), ctypes.c_double(eps), ctypes.c_double(theta),
                ncrit, int(quad), int(relative), ctypes.c_double(alpha), None if ao is None else _dp(ao),
                None if tg is None else tg.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), _dp(ax), _dp(ay), _dp(az),
                cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        if rc:
            raise RuntimeError("or_bh_pp_accel failed")
        return (ax, ay, az, cnt) if counters else (ax, ay, az)

    def leapfrog(self, state, m, G, eps, theta, ncrit, dt, nsteps, acc=None):
        """KDK steps; state = (x, y, z, vx, vy, vz); returns (state, acc)."""
        st = [np.array(a, dtype=np.float64) for a in state]
        m = _f64(m)
        n = len(m)
        primed = acc is not None
        a = [np.array(c, dtype=np.float64) for c in acc] if primed else [np.zeros(n) for _ in range(3)]
        rc = self.lib.or_leapfrog(n, *[_dp(v) for v in st], _dp(m), *[_dp(v) for v in a], G, eps, theta, ncrit, dt,
                                  nsteps, int(primed))
        if rc:
            raise RuntimeError("or_leapfrog failed")
        return tuple(st), tuple(a)

    def block_step(self, state, m, G, eps, theta, ncrit, dt, eta, max_rung, acc):
        """One block (rung) step from (state, acc); returns (state, acc, rungs, rung_max)."""
        st = [np.array(a, dtype=np.float64) for a in state]
        a = [np.array(c, dtype=np.float64) for c in acc]
        m = _f64(m)
        rung = np.zeros(len(m), np.int32)
        fn = self.lib.or_block_step
        fn.restype = ctypes.c_int
        rmax = fn(len(m), *[_dp(v) for v in st], _dp(m), *[_dp(v) for v in a], ctypes.c_double(G),
                  ctypes.c_double(eps), ctypes.c_double(theta), ncrit, ctypes.c_double(dt), ctypes.c_double(eta),
                  int(max_rung), _ip(rung))
        if rmax < 0:
            raise RuntimeError("or_block_step failed")
        return tuple(st), tuple(a), rung, rmax

    def force_error(self, x, y, z, m, G, eps, targets, ax, ay, az):
        """(rms, max, median) relative error of (ax, ay, az) vs the FP64 direct sum on targets."""
        x, y, z, m, ax, ay, az = map(_f64, (x, y, z, m, ax, ay, az))
        tg = np.ascontiguousarray(targets, dtype=np.int32)
        out = np.zeros(3)
        self.lib.or_force_error(len(x), _dp(x), _dp(y), _dp(z), _dp(m), G, eps * eps, len(tg), _ip(tg), _dp(ax),
                                _dp(ay), _dp(az), _dp(out))
        return float(out[0]), float(out[1]), float(out[2])


class Reference(_Common):
    """The reference's own sources, compiled by oracle/build_ref.sh."""

    _prefix = "ref_"

    def __init__(self, path: str = REF_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_tree_build.restype = ctypes.c_void_p
        L.ref_tree_build.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int, _I]
        L.ref_tree_export.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _U64, _I, _I, _D, _D, _D, _D, _D, _D,
                                      _I, _I, _I]
        L.ref_tree_free.argtypes = [ctypes.c_void_p]
        L.ref_bh_accel.restype = ctypes.c_double
        L.ref_bh_accel.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _D, _D]
        L.ref_direct_accel.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, _D, _D,
                                       _D]
        L.ref_leapfrog.restype = ctypes.c_double
        L.ref_leapfrog.argtypes = [ctypes.c_int] + [_D] * 10 + [ctypes.c_double] * 3 + [ctypes.c_int,
                                                                                        ctypes.c_double,
                                                                                        ctypes.c_int,
                                                                                        ctypes.c_int]
        L.ref_plummer.argtypes = [ctypes.c_int, ctypes.c_uint] + [_D] * 7

    def _tree_create(self, n, x, y, z, m, ncrit, max_depth, nn):
        return self.lib.ref_tree_build(n, _dp(x), _dp(y), _dp(z), _dp(m), ncrit, max_depth, nn)

    def _tree_export(self, h, n, t):
        self.lib.ref_tree_export(h, n, _ip(t["level"]), t["prefix"].ctypes.data_as(_U64), _ip(t["count"]),
                                 _ip(t["is_leaf"]), _dp(t["center"]), _dp(t["half"]), _dp(t["com"]),
                                 _dp(t["mass"]), _dp(t["max_radius"]), _dp(t["quad"]), _ip(t["order"]),
                                 _ip(t["parent"]), _ip(t["first"]))

    def _tree_free(self, h):
        self.lib.ref_tree_free(h)

    def _direct(self, n, x, y, z, m, G, eps, ax, ay, az):
        self.lib.ref_direct_accel(n, _dp(x), _dp(y), _dp(z), _dp(m), G, eps, _dp(ax), _dp(ay), _dp(az))

    def set_softening(self, kind):
        """0: Plummer, 1: cubic spline with h = eps, for every later call."""
        self.lib.ref_set_softening(int(kind))

    def bh_pp_accel(self, x, y, z, m, G, eps, theta, ncrit=8, alpha=0.001, aold=None, targets=None):
        """The reference's relative-MAC walk (aold given) or geometric target walk (targets given)."""
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
        ao = np.zeros(n) if aold is None else _f64(aold)
        tg = None if targets is None else np.ascontiguousarray(targets, dtype=np.uint8)
        fn = self.lib.ref_bh_pp_accel
        fn.restype = None
        fn(n, _dp(x), _dp(y), _dp(z), _dp(m), ctypes.c_double(G), ctypes.c_double(eps), ctypes.c_double(theta), ncrit,
           ctypes.c_double(alpha), _dp(ao), None if tg is None else tg.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
           _dp(ax), _dp(ay), _dp(az))
        return ax, ay, az

    def plummer(self, n, seed):
        """The reference's own Plummer generator (mt19937; clips r at 20)."""
        arrs = [np.zeros(n) for _ in range(7)]
        self.lib.ref_plummer(n, seed, *[_dp(a) for a in arrs])
        return arrs

    def scenario(self, kind, n, seed, ic_file=None):
        """The reference's deck scenario generator: (x, y, z, vx, vy, vz, m), (G, eps, dt)."""
        L = self.lib
        L.ref_scenario.restype = ctypes.c_int
        L.ref_scenario.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint, ctypes.c_char_p, ctypes.c_int] + \
            [_D] * 8
        par = np.zeros(3)
        icb = ic_file.encode() if ic_file else None
        count = L.ref_scenario(kind.encode(), n, seed, icb, 0, *([None] * 7), _dp(par))
        if count < 0:
            raise RuntimeError(f"reference scenario '{kind}' failed")
        arrs = [np.zeros(count) for _ in range(7)]
        L.ref_scenario(kind.encode(), n, seed, icb, count, *[_dp(a) for a in arrs], _dp(par))
        return arrs, (float(par[0]), float(par[1]), float(par[2]))

    def cloud(self, kind, n, seed):
        """Input clouds of the reference self-tests: 'uniform' (BH vs Direct) or 'ball' (quadrupole)."""
        arrs = [np.zeros(n) for _ in range(4)]
        fn = self.lib.ref_cloud_uniform if kind == "uniform" else self.lib.ref_cloud_ball
        fn.argtypes = [ctypes.c_int, ctypes.c_uint] + [_D] * 4
        fn(n, seed, *[_dp(a) for a in arrs])
        return arrs

    def bh_accel(self, x, y, z, m, G, eps, theta, ncrit=8, quad=True, timed=False):
        x, y, z, m = map(_f64, (x, y, z, m))
        n = len(x)
        ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
        ms = self.lib.ref_bh_accel(n, _dp(x), _dp(y), _dp(z), _dp(m), G, eps, theta, ncrit, int(quad), _dp(ax),
                                   _dp(ay), _dp(az))
        return (ax, ay, az, ms) if timed else (ax, ay, az)

    def block_step(self, state, m, G, eps, theta, dt, eta, max_rung, nsteps=1):
        """System::Step with StepParams::block, primed from the positions (ncrit 8);
        returns (state, acc, rungs of the last step)."""
        st = [np.array(a, dtype=np.float64) for a in state]
        m = _f64(m)
        n = len(m)
        a = [np.zeros(n) for _ in range(3)]
        rung = np.zeros(n, np.int32)
        fn = self.lib.ref_block_step
        fn.restype = None
        fn(n, *[_dp(v) for v in st], _dp(m), *[_dp(v) for v in a], ctypes.c_double(G), ctypes.c_double(eps),
           ctypes.c_double(theta), ctypes.c_double(dt), ctypes.c_double(eta), int(max_rung), int(nsteps), _ip(rung))
        return tuple(st), tuple(a), rung

    def leapfrog(self, state, m, G, eps, theta, ncrit, dt, nsteps, acc=None):
        st = [np.array(a, dtype=np.float64) for a in state]
        m = _f64(m)
        n = len(m)
        primed = acc is not None
        a = [np.array(c, dtype=np.float64) for c in acc] if primed else [np.zeros(n) for _ in range(3)]
        self.lib.ref_leapfrog(n, *[_dp(v) for v in st], _dp(m), *[_dp(v) for v in a], G, eps, theta, ncrit, dt,
                              nsteps, int(primed))
        return tuple(st), tuple(a)
