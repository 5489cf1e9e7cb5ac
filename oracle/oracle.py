"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a CPU FP64 restatement of VOLCANOR's free-wake UVLM path
(oracle/vlm_oracle.cpp).  Only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of bench.py may import this module;
the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB_PATH = BUILD / "libvlm_oracle.so"

_CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False) -> Path:
    """Compile oracle/vlm_oracle.cpp into oracle/_build/libvlm_oracle.so."""
    src = HERE / "vlm_oracle.cpp"
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime:
        return LIB_PATH
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f"libvlm_oracle.{os.getpid()}.so"
    subprocess.check_call(["g++", *_CXXFLAGS, "-o", str(tmp), str(src)])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp, dp, cp, i32, i64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, ctypes.c_int, ctypes.c_long
        L.or_last_error.restype = cp
        L.or_sim_create.restype = vp
        L.or_sim_create.argtypes = [cp, cp, cp]
        L.or_sim_free.argtypes = [vp]
        L.or_set_threads.argtypes = [i32]
        L.or_sim_start.argtypes = [vp]
        L.or_set_sum_chunk.argtypes = [vp, i32]
        L.or_sim_step.argtypes = [vp, i32]
        L.or_rot_pitch.argtypes = [vp, i32, ctypes.c_double]
        L.or_gettheta.argtypes = [vp, ctypes.c_double, i32]
        L.or_gettheta.restype = ctypes.c_double
        L.or_set_blade_theta.argtypes = [vp, i32, ctypes.c_double]
        L.or_calc_aic.argtypes = [vp]
        L.or_test_freestream.argtypes = [vp, i32]
        L.or_dir_lift_drag.argtypes = [vp]
        L.or_calc_sec_alpha.argtypes = [vp]
        L.or_calc_force.argtypes = [vp]
        L.or_geti.argtypes = [vp, cp]
        L.or_geti.restype = i64
        L.or_get.argtypes = [vp, cp, i32, dp, i64]
        L.or_get.restype = i64
        L.or_sim_vind_points.argtypes = [vp, dp, i64, dp, i32]
        L.or_sim_skip_to.argtypes = [vp, i32]
        L.or_sim_step_open.argtypes = [vp]
        L.or_sim_step_close.argtypes = [vp]
        L.or_set.argtypes = [vp, cp, i32, dp, i64]
        L.or_vind_rings.argtypes = [dp, dp, dp, i64, dp, i64, dp, i32]
        L.or_vind_filaments.argtypes = [dp, dp, dp, i64, dp, i64, dp, i32]
        L.or_vf_vind.argtypes = [dp, dp, ctypes.c_double, dp, dp]
        L.or_inv2.argtypes = [dp, i32, dp]
        L.or_matvec.argtypes = [dp, dp, i32, dp]
        L.or_lsq2.argtypes = [ctypes.c_double, dp, dp, i32]
        L.or_lsq2.restype = ctypes.c_double
        L.or_sys_create.restype = vp
        L.or_sys_create.argtypes = [i32, cp, ctypes.POINTER(cp), cp]
        L.or_sys_free.argtypes = [vp]
        L.or_sys_set_sum_chunk.argtypes = [vp, i32]
        L.or_sys_start.argtypes = [vp]
        L.or_sys_step.argtypes = [vp, i32]
        L.or_sys_rotor.restype = vp
        L.or_sys_rotor.argtypes = [vp, i32]
        L.or_c81_lookup.restype = ctypes.c_double
        L.or_c81_lookup.argtypes = [cp, i32, ctypes.c_double, ctypes.c_double]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleError(RuntimeError):
    pass


def _check(rc: int):
    if rc != 0:
        raise OracleError(lib().or_last_error().decode())


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


class Sim:
    """One rotor case (config.nml + geom01.nml) inside the oracle."""

    def __init__(self, config_text: str, geom_text: str, base_dir: str | os.PathLike = ""):
        L = lib()
        self._h = L.or_sim_create(config_text.encode(), geom_text.encode(), str(base_dir).encode())
        if not self._h:
            raise OracleError(L.or_last_error().decode())

    @classmethod
    def from_case_dir(cls, case_dir: str | os.PathLike, geom: str = "geom01.nml") -> "Sim":
        d = Path(case_dir)
        return cls((d / "config.nml").read_text(), (d / geom).read_text(), d)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_sim_free(h)
            self._h = None

    def set_sum_chunk(self, c: int):
        """Chunked Biot-Savart summation order (0 = the reference's sequential order)."""
        lib().or_set_sum_chunk(self._h, int(c))

    # main program
    def start(self):
        _check(lib().or_sim_start(self._h))

    def step(self, n: int = 1):
        _check(lib().or_sim_step(self._h, int(n)))

    def step_open(self):
        """The next iteration up to its loads (the reference's mid-step state)."""
        _check(lib().or_sim_step_open(self._h))

    def step_close(self):
        """The rest of an opened iteration (the wake update)."""
        _check(lib().or_sim_step_close(self._h))

    def skip_to(self, k: int):
        """Advance to iteration k with the prescribed kinematics only (no
        flow); the flow state of iteration k is then set with :meth:`set`."""
        _check(lib().or_sim_skip_to(self._h, int(k)))

    def set(self, name: str, ib: int, values) -> None:
        """Set a named flow-state array (layouts of :meth:`get`)."""
        v = _f64(values).reshape(-1)
        _check(lib().or_set(self._h, name.encode(), int(ib), _ptr(v), v.size))

    # unit-test primitives
    def rot_pitch(self, ib: int, theta: float):
        _check(lib().or_rot_pitch(self._h, ib, float(theta)))

    def gettheta(self, psi: float, ib: int) -> float:
        return lib().or_gettheta(self._h, float(psi), ib)

    def set_blade_theta(self, ib: int, theta: float):
        lib().or_set_blade_theta(self._h, ib, float(theta))

    def calc_aic(self):
        _check(lib().or_calc_aic(self._h))

    def test_freestream(self, with_omega: bool):
        _check(lib().or_test_freestream(self._h, int(with_omega)))

    def dir_lift_drag(self):
        _check(lib().or_dir_lift_drag(self._h))

    def calc_sec_alpha(self):
        _check(lib().or_calc_sec_alpha(self._h))

    def calc_force(self):
        _check(lib().or_calc_force(self._h))

    # state access
    def geti(self, name: str) -> int:
        return int(lib().or_geti(self._h, name.encode()))

    def get(self, name: str, ib: int = 1) -> np.ndarray:
        L = lib()
        n = L.or_get(self._h, name.encode(), ib, None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(max(n, 1), dtype=np.float64)
        L.or_get(self._h, name.encode(), ib, _ptr(out), n)
        return out[:n]

    def ct_hist(self) -> np.ndarray:
        return self.get("ct_hist").reshape(-1, 10)

    def vind_points(self, P: np.ndarray, predicted: bool = False) -> np.ndarray:
        P = _f64(P).reshape(-1, 3)
        V = np.zeros_like(P)
        _check(lib().or_sim_vind_points(self._h, _ptr(P), P.shape[0], _ptr(V), int(predicted)))
        return V


class _RotorView(Sim):
    """One rotor of a System (the handle belongs to the system)."""

    def __init__(self, handle, owner):
        self._h = handle
        self._owner = owner

    def __del__(self):
        pass


class System:
    """Coupled rotors (nr > 1): config.nml and one geomXX.nml per rotor,
    stepped with every rotor's wing and wake in every induced-velocity sum."""

    def __init__(self, config_text: str, geom_texts, base_dir: str | os.PathLike = ""):
        L = lib()
        g = [t.encode() for t in geom_texts]
        arr = (ctypes.c_char_p * len(g))(*g)
        self._h = L.or_sys_create(len(g), config_text.encode(), arr, str(base_dir).encode())
        if not self._h:
            raise OracleError(L.or_last_error().decode())
        self.rotors = [_RotorView(L.or_sys_rotor(self._h, i), self) for i in range(len(g))]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_sys_free(h)
            self._h = None

    def set_sum_chunk(self, c: int):
        _check(lib().or_sys_set_sum_chunk(self._h, int(c)))

    def start(self):
        _check(lib().or_sys_start(self._h))

    def step(self, n: int = 1):
        _check(lib().or_sys_step(self._h, int(n)))


def c81_lookup(path, coeff: int, alpha_deg: float, mach: float) -> float:
    """CL (0), CD (1) or CM (2) of a C81 file at (alpha in degrees, Mach)."""
    return float(lib().or_c81_lookup(str(path).encode(), int(coeff), float(alpha_deg), float(mach)))


def vind_rings(corners, rvc, gam, P, chunk: int = 0) -> np.ndarray:
    """V[m] = sum_n vr_vind(ring n, P[m]) * gam[n] (reference order; chunked when chunk > 0)."""
    corners = _f64(corners).reshape(-1, 4, 3)
    rvc = _f64(rvc).reshape(-1, 4)
    gam = _f64(gam).reshape(-1)
    P = _f64(P).reshape(-1, 3)
    V = np.zeros_like(P)
    _check(lib().or_vind_rings(_ptr(corners), _ptr(rvc), _ptr(gam), corners.shape[0], _ptr(P), P.shape[0], _ptr(V), int(chunk)))
    return V


def vind_filaments(fc, rvc, gam, P, chunk: int = 0) -> np.ndarray:
    """V[m] = sum_n vf_vind(filament n, P[m]) * gam[n] (in order; chunked when chunk > 0)."""
    fc = _f64(fc).reshape(-1, 2, 3)
    rvc = _f64(rvc).reshape(-1)
    gam = _f64(gam).reshape(-1)
    P = _f64(P).reshape(-1, 3)
    V = np.zeros_like(P)
    _check(lib().or_vind_filaments(_ptr(fc), _ptr(rvc), _ptr(gam), fc.shape[0], _ptr(P), P.shape[0], _ptr(V), int(chunk)))
    return V


def vf_vind(fc1, fc2, rvc, P) -> np.ndarray:
    a, b, p = _f64(fc1), _f64(fc2), _f64(P)
    V = np.zeros(3)
    lib().or_vf_vind(_ptr(a), _ptr(b), float(rvc), _ptr(p), _ptr(V))
    return V


def inv2(A) -> np.ndarray:
    """Explicit inverse as in libMath.f90:48-83 (column-major storage)."""
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    flat = _f64(A.ravel(order="F"))
    out = np.zeros(n * n)
    _check(lib().or_inv2(_ptr(flat), n, _ptr(out)))
    return out.reshape(n, n, order="F")


def matvec(A, x) -> np.ndarray:
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    flat = _f64(A.ravel(order="F"))
    xv = _f64(x)
    y = np.zeros(n)
    lib().or_matvec(_ptr(flat), _ptr(xv), n, _ptr(y))
    return y
