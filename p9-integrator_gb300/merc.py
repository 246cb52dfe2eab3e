"""Python binding of libmerc.so, the GB300 Mercurius integrator (C ABI in
include/merc.h).

This is a thin ctypes layer: every call goes to the CUDA library.  There is no
CPU path; if libmerc.so has not been built the import of :class:`Integrator`
fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmerc.so")

MERC_OK = 0
MERC_ERR_CONFIG = 1
MERC_ERR_CUDA = 2
MERC_ERR_TIMEOUT = 3
MERC_ERR_NONCONV = 4
MERC_ERR_STATE = 5

DRIFT_ELEMENTS = 0
DRIFT_UNIVERSAL = 1
WARM_PLAIN = 0
WARM_MLP = 1
WARM_SERIES = 2

FLAG_CE_LAST = 1
FLAG_CE_EVER = 2
FLAG_EJECTED = 4
FLAG_NONFINITE = 8
FLAG_MERGED = 16
FLAG_GREW = 32
MERGED_MASS = 1e-300
PARK_R = 1e6

_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_f64p = C.POINTER(C.c_double)


class MercParams(C.Structure):
    """``merc_params`` of include/merc.h."""

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


class MercStats(C.Structure):
    _fields_ = [
        ("steps_done", C.c_int64),
        ("ce_body_steps", C.c_int64),
        ("kepler_iterations", C.c_int64),
        ("kepler_solves", C.c_int64),
        ("kepler_nonconverged", C.c_int64),
        ("n_bodies", C.c_int64),
        ("n_systems", C.c_int64),
        ("last_step_ms", C.c_double),
        ("kepler_simt_iterations", C.c_int64),
    ]


class MercError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"merc error {code}: {msg}")
        self.code = code


_LIB = None


class Collision(C.Structure):
    """Mirror of ``merc_collision`` in include/merc.h."""

    _fields_ = [("step", C.c_int64), ("survivor", C.c_int64), ("absorbed", C.c_int64)]


def lib() -> C.CDLL:
    """Load libmerc.so (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.merc_default_params.argtypes = [C.POINTER(MercParams)]
    L.merc_default_params.restype = None
    L.merc_create.argtypes = [C.c_int, C.POINTER(MercParams), C.POINTER(vp)]
    L.merc_destroy.argtypes = [vp]
    L.merc_last_error.argtypes = [vp]
    L.merc_last_error.restype = C.c_char_p
    L.merc_set_params.argtypes = [vp, C.POINTER(MercParams)]
    L.merc_load_elements.argtypes = [vp, C.c_int32, _i64p, _i32p, _f64p, _f64p]
    L.merc_load_state.argtypes = [vp, C.c_int32, _i64p, _i32p, _f64p, _f64p, _f64p, _f64p]
    L.merc_step.argtypes = [vp, C.c_int64]
    L.merc_set_state.argtypes = [vp, _f64p, _f64p, _f64p]
    L.merc_diag_flush_l2.argtypes = [vp, C.c_int64]
    L.merc_roundtrip.argtypes = [vp]
    L.merc_get_state.argtypes = [vp, _f64p, _f64p, _u32p]
    L.merc_get_a_lag.argtypes = [vp, _f64p]
    L.merc_get_elements.argtypes = [vp, _f64p]
    L.merc_get_stats.argtypes = [vp, C.POINTER(MercStats)]
    L.merc_energy.argtypes = [vp, _f64p]
    L.merc_angular_momentum.argtypes = [vp, _f64p]
    L.merc_save_checkpoint.argtypes = [vp, C.c_char_p]
    L.merc_load_checkpoint.argtypes = [vp, C.c_char_p]
    L.merc_load_systems.argtypes = [vp, C.POINTER(SystemDesc), C.c_int32]
    L.merc_launch_count.argtypes = [vp]
    L.merc_launch_count.restype = C.c_int64
    L.merc_set_radii.argtypes = [vp, _f64p]
    L.merc_get_collisions.argtypes = [vp, C.POINTER(Collision), C.c_int64, C.POINTER(C.c_int64)]
    L.merc_get_masses.argtypes = [vp, _f64p]
    L.merc_step_static.argtypes = [C.c_int, C.POINTER(MercParams), C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    _f32p = C.POINTER(C.c_float)
    L.merc_mlp_log.argtypes = [vp, C.c_int64]
    L.merc_mlp_log_count.argtypes = [vp]
    L.merc_mlp_log_count.restype = C.c_int64
    L.merc_mlp_get_log.argtypes = [vp, _f32p, C.c_int64]
    L.merc_mlp_append_log.argtypes = [vp, _f32p, C.c_int64]
    L.merc_mlp_train.argtypes = [vp, C.c_int32, C.c_int32, C.c_float, C.c_uint64, _f32p]
    L.merc_mlp_set_weights.argtypes = [vp, _f32p]
    L.merc_mlp_get_weights.argtypes = [vp, _f32p]
    L.merc_diag_mlp_grad.argtypes = [C.c_int, C.c_int64, _f32p, _f32p, _f32p, _f32p]
    L.merc_diag_warm_start.argtypes = [C.c_int, C.c_int64, _f64p, _f64p, C.c_double, _f32p, C.c_double, C.c_int32,
                                       _f64p, _f64p, _i32p]
    L.merc_diag_math.argtypes = [C.c_int, C.c_int, C.c_int64, _f64p, _f64p, _f64p]
    L.merc_diag_fp64_peak.argtypes = [C.c_int, _f64p]
    L.merc_diag_time_kicks.argtypes = [vp, C.c_int]
    L.merc_diag_kick_ms.argtypes = [vp, _f64p, _i32p]
    L.merc_diag_far_recomputes.argtypes = [vp, C.POINTER(C.c_int64)]
    L.merc_diag_pdl.argtypes = [vp, C.c_int]
    L.merc_diag_encounter_wait.argtypes = [vp, C.POINTER(C.c_int32)]
    L.merc_diag_time_encounter.argtypes = [vp, C.c_int]
    L.merc_diag_encounter_ms.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    _LIB = L
    return L


class SystemDesc(C.Structure):
    """Mirror of ``merc_system_desc`` in include/merc.h."""

    _fields_ = [("n_bodies", C.c_int32), ("n_massive", C.c_int32), ("mass", _f64p), ("elements", _f64p),
                ("pos", _f64p), ("vel", _f64p)]


def default_params(**kw) -> MercParams:
    p = MercParams()
    lib().merc_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


@dataclass
class State:
    pos: np.ndarray  # 3 x n (component-major, flattened)
    vel: np.ndarray
    flags: np.ndarray


class Integrator:
    """One integrator context on one GPU (merc_create ... merc_destroy)."""

    def __init__(self, params: MercParams | None = None, device: int = 0):
        self.L = lib()
        self.h = C.c_void_p()
        self.params = params if params is not None else default_params()
        st = self.L.merc_create(device, C.byref(self.params), C.byref(self.h))
        if st:
            raise MercError(st, "merc_create failed (no CUDA device or invalid parameters)")
        self.n = 0
        self.nsys = 0

    def _check(self, st):
        if st:
            raise MercError(st, self.L.merc_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.merc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: MercParams):
        self._check(self.L.merc_set_params(self.h, C.byref(params)))
        self.params = params

    def load_elements(self, body_offset, n_massive, mass, elements):
        off = np.ascontiguousarray(body_offset, np.int64)
        nm = np.ascontiguousarray(n_massive, np.int32)
        self._check(self.L.merc_load_elements(self.h, len(nm), _p(off, _i64p), _p(nm, _i32p), _p(_f64(mass), _f64p),
                                              _p(_f64(elements), _f64p)))
        self.n, self.nsys = int(off[-1]), len(nm)

    def load_systems(self, sysm):
        """Load a systems.Systems batch from its elements (or from its cartesian
        state, for batches that carry one in extra["pos"] / extra["vel"])."""
        if "pos" in sysm.extra:
            self.load_state(sysm.body_offset, sysm.n_massive, sysm.mass, sysm.extra["pos"], sysm.extra["vel"])
        else:
            self.load_elements(sysm.body_offset, sysm.n_massive, sysm.mass, sysm.elements)

    def load_system_list(self, descs):
        """Load systems given one dict each: n_massive, mass and either
        elements (6 x n) or pos and vel (3 x n), through merc_load_systems."""
        keep = []
        arr = (SystemDesc * len(descs))()
        for k, d in enumerate(descs):
            m = _f64(d["mass"])
            keep.append(m)
            arr[k].n_bodies = m.size
            arr[k].n_massive = int(d["n_massive"])
            arr[k].mass = _p(m, _f64p)
            for key in ("elements", "pos", "vel"):
                if d.get(key) is not None:
                    a = _f64(np.ascontiguousarray(d[key]).reshape(-1))
                    keep.append(a)
                    setattr(arr[k], key, _p(a, _f64p))
        self._check(self.L.merc_load_systems(self.h, arr, len(descs)))
        self.n = sum(int(np.asarray(d["mass"]).size) for d in descs)
        self.nsys = len(descs)

    def save_checkpoint(self, path):
        self._check(self.L.merc_save_checkpoint(self.h, str(path).encode()))

    def load_checkpoint(self, path):
        """Restore a checkpoint (parameters, layout and state) into this context."""
        self._check(self.L.merc_load_checkpoint(self.h, str(path).encode()))
        st = self.stats()
        self.n, self.nsys = int(st.n_bodies), int(st.n_systems)

    def load_state(self, body_offset, n_massive, mass, pos, vel, a_lag=None):
        off = np.ascontiguousarray(body_offset, np.int64)
        nm = np.ascontiguousarray(n_massive, np.int32)
        al = _f64(a_lag) if a_lag is not None else None
        self._check(self.L.merc_load_state(self.h, len(nm), _p(off, _i64p), _p(nm, _i32p), _p(_f64(mass), _f64p),
                                           _p(_f64(pos), _f64p), _p(_f64(vel), _f64p), _p(al, _f64p)))
        self.n, self.nsys = int(off[-1]), len(nm)

    def set_state(self, pos=None, vel=None, a_lag=None):
        """Overwrite the loaded state from host arrays (None keeps a part)."""
        self._check(self.L.merc_set_state(self.h, _p(_f64(pos) if pos is not None else None, _f64p),
                                          _p(_f64(vel) if vel is not None else None, _f64p),
                                          _p(_f64(a_lag) if a_lag is not None else None, _f64p)))

    def flush_l2(self, nbytes: int = 512 << 20):
        self._check(self.L.merc_diag_flush_l2(self.h, int(nbytes)))

    def step(self, n_steps: int = 1):
        self._check(self.L.merc_step(self.h, int(n_steps)))

    def roundtrip(self):
        self._check(self.L.merc_roundtrip(self.h))

    def state(self, out: State | None = None) -> State:
        """The state (merc_get_state); `out` gives the host arrays to fill
        (e.g. pinned buffers), C-contiguous float64 / uint32 of the right sizes."""
        if out is not None:
            pos, vel, flags = out.pos, out.vel, out.flags
            if (pos.dtype != np.float64 or vel.dtype != np.float64 or flags.dtype != np.uint32
                    or pos.size != 3 * self.n or vel.size != 3 * self.n or flags.size != self.n
                    or not (pos.flags.c_contiguous and vel.flags.c_contiguous and flags.flags.c_contiguous)):
                raise ValueError("state(out=...): arrays of the wrong type, size or layout")
        else:
            pos = np.empty(3 * self.n)
            vel = np.empty(3 * self.n)
            flags = np.empty(self.n, np.uint32)
        self._check(self.L.merc_get_state(self.h, _p(pos, _f64p), _p(vel, _f64p), _p(flags, _u32p)))
        return State(pos, vel, flags)

    def set_radii(self, radius=None):
        """Physical collisions (merc_set_radii): radii in AU for every body, or
        None to switch detection off."""
        r = _f64(radius) if radius is not None else None
        if r is not None and r.size != self.n:
            raise ValueError("one radius per body")
        self._check(self.L.merc_set_radii(self.h, _p(r, _f64p)))

    def collisions(self) -> np.ndarray:
        """Resolved collisions: int64 array of rows (step, survivor, absorbed)."""
        cnt = C.c_int64(0)
        self._check(self.L.merc_get_collisions(self.h, None, 0, C.byref(cnt)))
        k = min(cnt.value, 65536)
        buf = (Collision * max(k, 1))()
        self._check(self.L.merc_get_collisions(self.h, buf, k, C.byref(cnt)))
        return np.array([(c.step, c.survivor, c.absorbed) for c in buf[:k]], dtype=np.int64).reshape(-1, 3)

    def masses(self) -> np.ndarray:
        m = np.empty(self.n)
        self._check(self.L.merc_get_masses(self.h, _p(m, _f64p)))
        return m

    def a_lag(self) -> np.ndarray:
        a = np.empty(self.n)
        self._check(self.L.merc_get_a_lag(self.h, _p(a, _f64p)))
        return a

    def elements(self) -> np.ndarray:
        el = np.empty(6 * self.n)
        self._check(self.L.merc_get_elements(self.h, _p(el, _f64p)))
        return el

    def stats(self) -> MercStats:
        s = MercStats()
        self._check(self.L.merc_get_stats(self.h, C.byref(s)))
        return s

    def energy(self) -> np.ndarray:
        e = np.empty(self.nsys)
        self._check(self.L.merc_energy(self.h, _p(e, _f64p)))
        return e

    def angular_momentum(self) -> np.ndarray:
        """Total angular momentum of each system: n_systems x 3."""
        L = np.empty(3 * self.nsys)
        self._check(self.L.merc_angular_momentum(self.h, _p(L, _f64p)))
        return L.reshape(self.nsys, 3)

    def launch_count(self) -> int:
        return int(self.L.merc_launch_count(self.h))

    # ---- learned warm start ----
    def mlp_log(self, capacity: int):
        self._check(self.L.merc_mlp_log(self.h, int(capacity)))

    def mlp_log_count(self) -> int:
        return int(self.L.merc_mlp_log_count(self.h))

    def mlp_get_log(self, max_samples: int | None = None) -> np.ndarray:
        n = self.mlp_log_count() if max_samples is None else int(max_samples)
        out = np.zeros(5 * n, np.float32)
        self._check(self.L.merc_mlp_get_log(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), n))
        return out.reshape(-1, 5)

    def mlp_append_log(self, samples):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1)
        self._check(self.L.merc_mlp_append_log(self.h, s.ctypes.data_as(C.POINTER(C.c_float)), s.size // 5))

    def mlp_train(self, epochs=20, batch=8192, lr=3e-3, seed=1):
        loss = np.zeros(epochs, np.float32)
        self._check(self.L.merc_mlp_train(self.h, int(epochs), int(batch), float(lr), int(seed),
                                          loss.ctypes.data_as(C.POINTER(C.c_float))))
        return loss

    def mlp_weights(self) -> np.ndarray:
        w = np.zeros(MLP_BLOB, np.float32)
        self._check(self.L.merc_mlp_get_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float))))
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == MLP_BLOB
        self._check(self.L.merc_mlp_set_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float))))

    def time_kicks(self, on: bool = True):
        self._check(self.L.merc_diag_time_kicks(self.h, 1 if on else 0))

    def kick_ms(self):
        ms = C.c_double()
        cnt = C.c_int32()
        self._check(self.L.merc_diag_kick_ms(self.h, C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    def programmatic_launches(self, on: bool = True):
        """Programmatic dependent launches inside the step graphs (default on)."""
        self._check(self.L.merc_diag_pdl(self.h, 1 if on else 0))

    def far_recomputes(self) -> int:
        """Merged kicks whose far field had to be summed a second time."""
        c = C.c_int64()
        self._check(self.L.merc_diag_far_recomputes(self.h, C.byref(c)))
        return c.value

    def time_encounter(self, on: bool = True):
        """Record CUDA events around the big systems' encounter sub-step."""
        self._check(self.L.merc_diag_time_encounter(self.h, 1 if on else 0))

    def encounter_ms(self):
        """Mean encounter sub-step duration (ms) of the last call and the
        number of launches averaged."""
        ms, cnt = C.c_double(), C.c_int32()
        self._check(self.L.merc_diag_encounter_ms(self.h, C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    def encounter_wait_check(self) -> bool:
        """Runs the encounter task kernel with a dependency that is never
        published and a short wait limit; True when the kernel reported that
        the wait gave up (merc_diag_encounter_wait)."""
        g = C.c_int32()
        self._check(self.L.merc_diag_encounter_wait(self.h, C.byref(g)))
        return bool(g.value)


MLP_BLOB = 1267


def mlp_grad(samples, blob, device: int = 0):
    """GPU loss and gradient of the warm-start network (diagnostic)."""
    L = lib()
    f32 = C.POINTER(C.c_float)
    s = np.ascontiguousarray(samples, np.float32).reshape(-1)
    b = np.ascontiguousarray(blob, np.float32)
    g = np.zeros(MLP_BLOB - 18, np.float32)
    loss = C.c_float()
    st = L.merc_diag_mlp_grad(device, s.size // 5, s.ctypes.data_as(f32), b.ctypes.data_as(f32), C.byref(loss),
                              g.ctypes.data_as(f32))
    if st:
        raise MercError(st, "merc_diag_mlp_grad failed")
    return loss.value, g


def warm_start_probe(pos, vel, dt, blob=None, tol=1e-13, max_iter=30, device: int = 0):
    """GPU warm-start guess, converged s and Newton iterations for drift inputs."""
    L = lib()
    pos = _f64(pos)
    vel = _f64(vel)
    n = pos.size // 3
    g = np.zeros(n)
    s = np.zeros(n)
    it = np.zeros(n, np.int32)
    b = np.ascontiguousarray(blob, np.float32) if blob is not None else None
    st = L.merc_diag_warm_start(device, n, _p(pos, _f64p), _p(vel, _f64p), dt,
                                b.ctypes.data_as(C.POINTER(C.c_float)) if b is not None else None, tol, max_iter,
                                _p(g, _f64p), _p(s, _f64p), _p(it, _i32p))
    if st:
        raise MercError(st, "merc_diag_warm_start failed")
    return g, s, it


MM_FUNCS = {"sin": 0, "cos": 1, "atan2": 2, "acos": 3, "log": 4, "sinh": 5, "cosh": 6, "cbrt": 7, "exp": 8,
            "div3": 9, "div": 10, "div15": 11, "div63": 12}


def device_math(fn: str, x, y=None, device: int = 0) -> np.ndarray:
    """Evaluate a merc_math function on the GPU (diagnostic)."""
    L = lib()
    x = _f64(x)
    yy = _f64(y) if y is not None else None
    out = np.empty_like(x)
    st = L.merc_diag_math(device, MM_FUNCS[fn], x.size, _p(x, _f64p), _p(yy, _f64p), _p(out, _f64p))
    if st:
        raise MercError(st, "merc_diag_math failed")
    return out


def fp64_peak_tflops(device: int = 0) -> float:
    L = lib()
    t = C.c_double()
    st = L.merc_diag_fp64_peak(device, C.byref(t))
    if st:
        raise MercError(st, "merc_diag_fp64_peak failed")
    return t.value
