"""ctypes binding of the CPU oracle (liboracle.so) and of the reference cross-check
library (_ref/librefhost.so).  TEST INFRASTRUCTURE.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
use this module, as the checker.  The GPU library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "librefhost.so")

_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


class MercParams(C.Structure):
    """Mirror of ``merc_params`` in include/merc.h."""

    _fields_ = [
        ("dt", C.c_double),
        ("softening2", C.c_double),
        ("hill_factor", C.c_double),
        ("kepler_tol", C.c_double),
        ("eject_r", C.c_double),
        ("kepler_iters", C.c_int32),
        ("bs_rows", C.c_int32),
        ("compat_block", C.c_int32),
        ("drift", C.c_int32),
        ("kepler_max_iter", C.c_int32),
        ("warm_start", C.c_int32),
    ]


def default_params(**kw) -> MercParams:
    p = MercParams(dt=0.8219, softening2=1e-8, hill_factor=1.0, kepler_tol=1e-13, eject_r=0.0,
                   kepler_iters=8, bs_rows=3, compat_block=0, drift=0, kepler_max_iter=30, warm_start=2)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (and the reference cross-check when its sources exist)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "all", "ref"], stdout=out)


def ref_dir():
    """Directory of the reference checkout (environment MERC_REF_DIR, else the
    build recipe's default), or None where it is absent (as on a GPU host)."""
    try:
        out = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "refdir"], capture_output=True,
                             text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return out if out and os.path.isdir(out) else None


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.L = L
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_load_elements.argtypes = [C.POINTER(MercParams), C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                           _f64p, C.c_int]
        L.oracle_run.argtypes = [C.POINTER(MercParams), C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p, _u32p,
                                 C.c_int64, C.c_int, _i64p]
        L.oracle_run_collide.argtypes = [C.POINTER(MercParams), C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                         _f64p, _u32p, C.c_int64, C.c_int, _i64p, C.c_int64, _i64p, C.c_int64, _i64p]
        L.oracle_roundtrip.argtypes = [C.POINTER(MercParams), C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                       C.c_int]
        L.oracle_to_elements.argtypes = [C.POINTER(MercParams), C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                         C.c_int]
        L.oracle_mm_eval.argtypes = [C.c_int, C.c_int64, _f64p, _f64p, _f64p]
        L.oracle_energy.argtypes = [C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p, C.c_int]
        L.oracle_danby.argtypes = [C.c_int64, _f64p, _f64p, C.c_int, _f64p]
        L.oracle_cart_from_elem.argtypes = [C.c_int64, _f64p, C.c_int, _f64p, _f64p]
        L.oracle_elem_from_cart.argtypes = [C.c_int64, _f64p, _f64p, _f64p]
        L.oracle_universal.argtypes = [C.c_int64, _f64p, _f64p, C.c_double, C.c_double, C.c_int, _f64p, _f64p, _f64p,
                                       _i32p, C.c_int]
        L.oracle_stumpff.argtypes = [C.c_int64, _f64p, _f64p]

    def threads(self) -> int:
        return self.L.oracle_num_threads()

    def set_threads(self, n: int) -> None:
        self.L.oracle_set_threads(n)

    # ---- system level ----
    # precision: 0 binary64 + host C library, 1 long double, 2 binary64 +
    # the GPU library's merc_math functions (bitwise comparable with the GPU)
    def load_elements(self, params, offsets, n_massive, mass, elements, precision=0):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        n = int(off[-1])
        pos = np.zeros(3 * n)
        vel = np.zeros(3 * n)
        alag = np.zeros(n)
        st = self.L.oracle_load_elements(C.byref(params), len(nm), _ptr(off, _i64p), _ptr(nm, _i32p),
                                         _ptr(_f64(mass), _f64p), _ptr(_f64(elements), _f64p), _ptr(pos, _f64p),
                                         _ptr(vel, _f64p), _ptr(alag, _f64p), int(precision))
        if st:
            raise ValueError(f"oracle_load_elements status {st}")
        return pos, vel, alag

    def run(self, params, offsets, n_massive, mass, pos, vel, alag, flags=None, steps=1, precision=0):
        """Integrate in place-copies; returns (pos, vel, alag, flags, stats[4])."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        n = int(off[-1])
        pos = _f64(pos).copy()
        vel = _f64(vel).copy()
        alag = _f64(alag).copy()
        flags = np.zeros(n, np.uint32) if flags is None else np.ascontiguousarray(flags, np.uint32).copy()
        stats = np.zeros(4, np.int64)
        st = self.L.oracle_run(C.byref(params), len(nm), _ptr(off, _i64p), _ptr(nm, _i32p), _ptr(_f64(mass), _f64p),
                               _ptr(pos, _f64p), _ptr(vel, _f64p), _ptr(alag, _f64p), _ptr(flags, _u32p),
                               int(steps), int(precision), _ptr(stats, _i64p))
        if st:
            raise ValueError(f"oracle_run status {st}")
        return pos, vel, alag, flags, stats

    def run_collide(self, params, offsets, n_massive, mass, radius, pos, vel, alag, flags=None, steps=1,
                    precision=0, step0=0, max_events=65536):
        """run() with physical collisions: returns (pos, vel, alag, flags,
        stats[4], mass, events (k x 3: step, survivor, absorbed))."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        n = int(off[-1])
        pos = _f64(pos).copy()
        vel = _f64(vel).copy()
        alag = _f64(alag).copy()
        mass = _f64(mass).copy()
        rad = _f64(radius)
        flags = np.zeros(n, np.uint32) if flags is None else np.ascontiguousarray(flags, np.uint32).copy()
        stats = np.zeros(4, np.int64)
        ev = np.zeros(3 * max_events, np.int64)
        ne = C.c_int64(0)
        st = self.L.oracle_run_collide(C.byref(params), len(nm), _ptr(off, _i64p), _ptr(nm, _i32p),
                                       _ptr(mass, _f64p), _ptr(rad, _f64p), _ptr(pos, _f64p), _ptr(vel, _f64p),
                                       _ptr(alag, _f64p), _ptr(flags, _u32p), int(steps), int(precision),
                                       _ptr(stats, _i64p), int(step0), _ptr(ev, _i64p), int(max_events),
                                       C.byref(ne))
        if st:
            raise ValueError(f"oracle_run_collide status {st}")
        k = min(ne.value, max_events)
        return pos, vel, alag, flags, stats, mass, ev[:3 * k].reshape(-1, 3)

    def roundtrip(self, params, offsets, n_massive, mass, pos, vel, precision=0):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        n = int(off[-1])
        pos = _f64(pos).copy()
        vel = _f64(vel).copy()
        alag = np.zeros(n)
        st = self.L.oracle_roundtrip(C.byref(params), len(nm), _ptr(off, _i64p), _ptr(nm, _i32p),
                                     _ptr(_f64(mass), _f64p), _ptr(pos, _f64p), _ptr(vel, _f64p), _ptr(alag, _f64p),
                                     int(precision))
        if st:
            raise ValueError(f"oracle_roundtrip status {st}")
        return pos, vel, alag

    def to_elements(self, params, offsets, n_massive, mass, pos, vel, precision=0):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        n = int(off[-1])
        el = np.zeros(6 * n)
        st = self.L.oracle_to_elements(C.byref(params), len(nm), _ptr(off, _i64p), _ptr(nm, _i32p),
                                       _ptr(_f64(mass), _f64p), _ptr(_f64(pos), _f64p), _ptr(_f64(vel), _f64p),
                                       _ptr(el, _f64p), int(precision))
        if st:
            raise ValueError(f"oracle_to_elements status {st}")
        return el

    def energy(self, offsets, n_massive, mass, pos, vel):
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nm = np.ascontiguousarray(n_massive, dtype=np.int32)
        e = np.zeros(len(nm))
        st = self.L.oracle_energy(len(nm), _ptr(off, _i64p), _ptr(nm, _i32p), _ptr(_f64(mass), _f64p),
                                  _ptr(_f64(pos), _f64p), _ptr(_f64(vel), _f64p), _ptr(e, _f64p), 0)
        if st:
            raise ValueError(f"oracle_energy status {st}")
        return e

    # ---- unit level ----
    def danby(self, M, e, iters=8):
        M = _f64(M)
        e = _f64(e)
        out = np.zeros_like(M)
        self.L.oracle_danby(M.size, _ptr(M, _f64p), _ptr(e, _f64p), iters, _ptr(out, _f64p))
        return out

    def cart_from_elem(self, el, iters=8):
        el = _f64(el)
        n = el.size // 6
        pos = np.zeros(3 * n)
        vel = np.zeros(3 * n)
        self.L.oracle_cart_from_elem(n, _ptr(el, _f64p), iters, _ptr(pos, _f64p), _ptr(vel, _f64p))
        return pos, vel

    def elem_from_cart(self, pos, vel):
        pos = _f64(pos)
        vel = _f64(vel)
        n = pos.size // 3
        el = np.zeros(6 * n)
        self.L.oracle_elem_from_cart(n, _ptr(pos, _f64p), _ptr(vel, _f64p), _ptr(el, _f64p))
        return el

    def universal(self, pos, vel, dt, tol=1e-13, max_iter=30, s0=None, precision=0):
        pos = _f64(pos)
        vel = _f64(vel)
        n = pos.size // 3
        po = np.zeros(3 * n)
        vo = np.zeros(3 * n)
        its = np.zeros(n, np.int32)
        s0a = _f64(s0) if s0 is not None else None
        self.L.oracle_universal(n, _ptr(pos, _f64p), _ptr(vel, _f64p), dt, tol, max_iter, _ptr(s0a, _f64p),
                                _ptr(po, _f64p), _ptr(vo, _f64p), _ptr(its, _i32p), precision)
        return po, vo, its

    MM_FUNCS = {"sin": 0, "cos": 1, "atan2": 2, "acos": 3, "log": 4, "sinh": 5, "cosh": 6, "cbrt": 7, "exp": 8}

    def mm_eval(self, fn, x, y=None):
        """Host evaluation of a merc_math function (the GPU library's libm)."""
        x = _f64(x)
        yy = _f64(y) if y is not None else x
        out = np.zeros_like(x)
        self.L.oracle_mm_eval(self.MM_FUNCS[fn], x.size, _ptr(x, _f64p), _ptr(yy, _f64p), _ptr(out, _f64p))
        return out

    def stumpff(self, z):
        z = _f64(z)
        c = np.zeros(4 * z.size)
        self.L.oracle_stumpff(z.size, _ptr(z, _f64p), _ptr(c, _f64p))
        return c.reshape(4, -1)


class RefHost:
    """The reference's own src/sim.cuh compiled for the host (oracle/_ref)."""

    def __init__(self, path: str = REF_PATH):
        L = C.CDLL(path)
        self.L = L
        L.refhost_run.argtypes = [C.c_int, C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_double, C.c_long, _f64p,
                                  _f64p, _f64p, _f64p, _u8p]
        L.refhost_run.restype = C.c_int
        L.refhost_danby.argtypes = [C.c_long, _f64p, _f64p, _f64p]
        L.refhost_cart_from_elem.argtypes = [C.c_long, _f64p, _f64p, _f64p]
        L.refhost_elem_from_cart.argtypes = [C.c_long, _f64p, _f64p, _f64p]

    @staticmethod
    def available(path: str = REF_PATH) -> bool:
        return os.path.exists(path)

    def run(self, elements, mass, n_massive, block, dt, hill_factor, steps, want_elements=False):
        el = _f64(elements)
        m = _f64(mass)
        n = m.size
        pos = np.zeros(3 * n)
        vel = np.zeros(3 * n)
        alag = np.zeros(n)
        out_el = np.zeros(6 * n) if want_elements else None
        ce = np.zeros(n, np.uint8)
        st = self.L.refhost_run(n, int(n_massive), int(block), _ptr(el, _f64p), _ptr(m, _f64p), dt, hill_factor,
                                int(steps), _ptr(pos, _f64p), _ptr(vel, _f64p), _ptr(alag, _f64p),
                                _ptr(out_el, _f64p), _ptr(ce, _u8p))
        if st:
            raise ValueError("refhost_run rejected the shape (needs n % block == 0 and n_massive <= block)")
        return pos, vel, alag, out_el, ce

    def danby(self, M, e):
        M = _f64(M)
        e = _f64(e)
        out = np.zeros_like(M)
        self.L.refhost_danby(M.size, _ptr(M, _f64p), _ptr(e, _f64p), _ptr(out, _f64p))
        return out

    def cart_from_elem(self, el):
        el = _f64(el)
        n = el.size // 6
        pos = np.zeros(3 * n)
        vel = np.zeros(3 * n)
        self.L.refhost_cart_from_elem(n, _ptr(el, _f64p), _ptr(pos, _f64p), _ptr(vel, _f64p))
        return pos, vel

    def elem_from_cart(self, pos, vel):
        pos = _f64(pos)
        vel = _f64(vel)
        n = pos.size // 3
        el = np.zeros(6 * n)
        self.L.refhost_elem_from_cart(n, _ptr(pos, _f64p), _ptr(vel, _f64p), _ptr(el, _f64p))
        return el
