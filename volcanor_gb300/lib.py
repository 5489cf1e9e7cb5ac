"""ctypes binding of libvlm_gb300.so (the C ABI in include/vlm.h).

The Python classes mirror the reference's object API for the hot path: a
:class:`Case` is one rotor/wing case read from ``config.nml`` +
``geom01.nml`` (the reference's ``rotor`` object after ``readGeom`` and
``init``), advanced with :meth:`Case.step` (one iteration of
src/main.f90:400-1452 per step).  There is no CPU fallback: if the CUDA
library is missing or no GPU is usable, every call raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Optional

import numpy as np

from . import build as _build

PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP32_NEAR64 = 2

VLM_OK = 0
_STATUS = {1: "invalid argument", 2: "CUDA error", 3: "I/O error", 4: "unsupported case feature",
           5: "singular AIC", 6: "non-finite result", 7: "call out of order"}


class VlmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("sum_chunk", ctypes.c_int), ("near_factor", ctypes.c_double),
                ("device", ctypes.c_int), ("use_graph", ctypes.c_int), ("solve_mode", ctypes.c_int),
                ("nbody_slots", ctypes.c_int), ("lattice", ctypes.c_int),
                ("incremental", ctypes.c_int)]


class SurrogateOptions(ctypes.Structure):
    _fields_ = [("enable", ctypes.c_int), ("young_far", ctypes.c_int), ("min_far", ctypes.c_int),
                ("collect_steps", ctypes.c_int),
                ("sample_stride", ctypes.c_int), ("train_iters", ctypes.c_int), ("batch", ctypes.c_int),
                ("lr", ctypes.c_float), ("audit_samples", ctypes.c_int), ("audit_tol", ctypes.c_double),
                ("hidden", ctypes.c_int), ("layers", ctypes.c_int), ("seed", ctypes.c_uint64)]


class SurrogateStats(ctypes.Structure):
    _fields_ = [("phase", ctypes.c_int), ("trainings", ctypes.c_int), ("audits", ctypes.c_int),
                ("reverts", ctypes.c_int), ("active_steps", ctypes.c_int), ("samples", ctypes.c_int64),
                ("last_audit_err", ctypes.c_double), ("max_audit_err", ctypes.c_double), ("last_loss", ctypes.c_float)]


# exported symbols and their signatures (include/vlm.h)
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64 = ctypes.c_int64
_vp = ctypes.c_void_p
SIGNATURES = {
    "vlm_version": (ctypes.c_char_p, []),
    "vlm_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "vlm_default_options": (None, [ctypes.POINTER(Options)]),
    "vlm_kernel_launch_count": (_i64, []),
    "vlm_device_info": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int)]),
    "vlm_measure_fp32_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "vlm_biot_savart_rings": (ctypes.c_int, [_dp, _dp, _dp, _i64, _dp, _i64, _dp, ctypes.c_int]),
    "vlm_biot_savart_rings_device": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_int, _vp]),
    "vlm_biot_savart_rings_scratch_bytes": (_i64, [_i64, _i64, ctypes.c_int]),
    "vlm_biot_savart_rings_sum_chunk": (_i64, [_i64, _i64, ctypes.c_int]),
    "vlm_biot_savart_rings_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_int, _vp]),
    "vlm_biot_savart_filaments": (ctypes.c_int, [_dp, _dp, _dp, _i64, _dp, _i64, _dp, ctypes.c_int]),
    "vlm_biot_savart_filaments_device": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _i64, _vp, ctypes.c_int, _vp]),
    "vlm_case_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(Options),
                                       ctypes.POINTER(_vp)]),
    "vlm_case_create_from_dir": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Options), ctypes.POINTER(_vp)]),
    "vlm_case_destroy": (ctypes.c_int, [_vp]),
    "vlm_case_start": (ctypes.c_int, [_vp]),
    "vlm_case_step": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "vlm_case_aic_factor": (ctypes.c_int, [_vp]),
    "vlm_case_solve_circulation": (ctypes.c_int, [_vp, _dp, _dp]),
    "vlm_case_loads": (ctypes.c_int, [_vp, _dp]),
    "vlm_case_wake_step": (ctypes.c_int, [_vp]),
    "vlm_case_get_wake": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp]),
    "vlm_case_get_int": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_i64)]),
    "vlm_case_get": (_i64, [_vp, ctypes.c_char_p, ctypes.c_int, _dp, _i64]),
    "vlm_case_vind_points": (ctypes.c_int, [_vp, _dp, _i64, _dp]),
    "vlm_case_params_json": (_i64, [_vp, ctypes.c_char_p, _i64]),
    "vlm_params_json": (_i64, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _i64]),
    "vlm_wing_kinematics": (_i64, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
                                   ctypes.c_int, _dp, _i64]),
    "vlm_case_last_step_ms": (ctypes.c_int, [_vp, _dp]),
    "vlm_case_profile_eval": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp]),
    "vlm_case_checkpoint_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "vlm_case_checkpoint_load": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "vlm_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "vlm_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_char_p),
                                        ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(Options), ctypes.POINTER(_vp)]),
    "vlm_batch_destroy": (ctypes.c_int, [_vp]),
    "vlm_case_set_tile": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "vlm_system_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                         ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(_vp)]),
    "vlm_system_create_from_dir": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.POINTER(_vp)]),
    "vlm_system_destroy": (ctypes.c_int, [_vp]),
    "vlm_system_rotor_count": (ctypes.c_int, [_vp]),
    "vlm_system_rotor": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "vlm_system_start": (ctypes.c_int, [_vp]),
    "vlm_system_step": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "vlm_system_last_step_ms": (ctypes.c_int, [_vp, _dp]),
    "vlm_batch_case": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "vlm_batch_start": (ctypes.c_int, [_vp]),
    "vlm_batch_step": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "vlm_batch_last_step_ms": (ctypes.c_int, [_vp, _dp]),
    "vlm_default_surrogate_options": (None, [ctypes.POINTER(SurrogateOptions)]),
    "vlm_case_set_surrogate": (ctypes.c_int, [_vp, ctypes.POINTER(SurrogateOptions)]),
    "vlm_case_surrogate_stats": (ctypes.c_int, [_vp, ctypes.POINTER(SurrogateStats)]),
    "vlm_mlp_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_vp)]),
    "vlm_mlp_destroy": (ctypes.c_int, [_vp]),
    "vlm_mlp_param_count": (_i64, [_vp]),
    "vlm_mlp_get_params": (ctypes.c_int, [_vp, _fp]),
    "vlm_mlp_set_params": (ctypes.c_int, [_vp, _fp]),
    "vlm_mlp_forward": (ctypes.c_int, [_vp, _fp, _i64, _fp]),
    "vlm_mlp_set_inference": (ctypes.c_int, [_vp, ctypes.c_int]),
    "vlm_mlp_get_inference": (ctypes.c_int, [_vp]),
    "vlm_mlp_gradient": (ctypes.c_int, [_vp, _fp, _fp, _i64, _fp, _fp]),
    "vlm_mlp_train": (ctypes.c_int, [_vp, _fp, _fp, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_float, _fp]),
}

_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libvlm_gb300.so (building it in-tree if it is missing or stale)."""
    global _lib
    if _lib is None:
        if build_if_missing:
            _build.build()
        if not _build.LIB.exists():
            raise RuntimeError(f"{_build.LIB} not built; run __graft_entry__.build()")
        L = ctypes.CDLL(str(_build.LIB))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().vlm_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _err(code: int):
    if code != VLM_OK:
        raise VlmError(code, last_error())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def options(precision: int = PREC_FP64, sum_chunk: Optional[int] = None, near_factor: Optional[float] = None,
            device: int = 0, use_graph: bool = True, solve_mode: Optional[int] = None) -> Options:
    o = Options()
    load().vlm_default_options(ctypes.byref(o))
    o.precision = precision
    if sum_chunk is not None:
        o.sum_chunk = sum_chunk
    if near_factor is not None:
        o.near_factor = near_factor
    o.device = device
    o.use_graph = int(use_graph)
    if solve_mode is not None:
        o.solve_mode = solve_mode
    return o


def launch_count() -> int:
    """Kernels this library has launched so far."""
    return int(load().vlm_kernel_launch_count())


def device_info(device: int = 0):
    sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _err(load().vlm_device_info(device, ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi)))
    return sm.value, ma.value, mi.value


def measure_fp32_peak(device: int = 0, reps: int = 20):
    """(TFLOP/s, ms per launch) of the library's FP32 FMA-chain kernel on all SMs."""
    tf, ms = ctypes.c_double(), ctypes.c_double()
    _err(load().vlm_measure_fp32_peak(device, reps, ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value, ms.value


def params_json(config_text: str, geom_text: str, base_dir: str | os.PathLike = "") -> str:
    """The rXXParams.json text of a case from its config.nml / geomXX.nml
    text (host-side parsing only; no GPU needed)."""
    L = load()
    args = (config_text.encode(), geom_text.encode(), str(base_dir).encode())
    n = L.vlm_params_json(*args, None, 0)
    if n < 0:
        raise VlmError(1, last_error())
    buf = ctypes.create_string_buffer(int(n) + 1)
    L.vlm_params_json(*args, buf, n + 1)
    return buf.value.decode()


def wing_kinematics(config_text: str, geom_text: str, iteration: int, name: str, blade: int = 1,
                    base_dir: str | os.PathLike = "") -> np.ndarray:
    """A wing array (PC, vr, CP, nCap, secCP) after the prescribed motion of
    iterations 1..iteration, from the case files alone (host side, no GPU)."""
    L = load()
    args = (config_text.encode(), geom_text.encode(), str(base_dir).encode(), int(iteration), name.encode(),
            int(blade))
    n = L.vlm_wing_kinematics(*args, None, 0)
    if n < 0:
        raise VlmError(1, last_error())
    out = np.zeros(max(n, 1))
    L.vlm_wing_kinematics(*args, _ptr(out), n)
    return out[:n]


def biot_savart_rings(corners, rvc, gam, P, precision: int = PREC_FP64) -> np.ndarray:
    """Ring-sum Biot-Savart through the host-buffer C entry point."""
    corners = _c64(corners).reshape(-1, 4, 3)
    rvc = _c64(rvc).reshape(-1, 4)
    gam = _c64(gam).reshape(-1)
    P = _c64(P).reshape(-1, 3)
    V = np.zeros_like(P)
    _err(load().vlm_biot_savart_rings(_ptr(corners), _ptr(rvc), _ptr(gam), corners.shape[0], _ptr(P), P.shape[0],
                                      _ptr(V), precision))
    return V


def biot_savart_filaments(fc, rvc, gam, P, precision: int = PREC_FP64) -> np.ndarray:
    """Single-filament Biot-Savart sum (vf_vind x gam) through the host-buffer
    C entry point; fc is N x 2 x 3 (start, end)."""
    fc = _c64(fc).reshape(-1, 2, 3)
    rvc = _c64(rvc).reshape(-1)
    gam = _c64(gam).reshape(-1)
    P = _c64(P).reshape(-1, 3)
    V = np.zeros_like(P)
    _err(load().vlm_biot_savart_filaments(_ptr(fc), _ptr(rvc), _ptr(gam), fc.shape[0], _ptr(P), P.shape[0],
                                          _ptr(V), precision))
    return V


def rings_sum_chunk(N: int, M: int, precision: int = PREC_FP64) -> int:
    """Summation block size of the ring kernel for (N, M): see include/vlm.h."""
    return int(load().vlm_biot_savart_rings_sum_chunk(N, M, precision))


def biot_savart_rings_device(corners_ptr: int, rvc_ptr: int, gam_ptr: int, N: int, P_ptr: int, M: int, V_ptr: int,
                             precision: int = PREC_FP64, stream: int = 0) -> None:
    """Device-buffer entry point: raw CUDA pointers (e.g. torch tensor data_ptr())."""
    _err(load().vlm_biot_savart_rings_device(corners_ptr, rvc_ptr, gam_ptr, N, P_ptr, M, V_ptr, precision,
                                             stream or None))


def biot_savart_rings_noalloc(corners_ptr: int, rvc_ptr: int, gam_ptr: int, N: int, P_ptr: int, M: int, V_ptr: int,
                              precision: int = PREC_FP64, stream: int = 0) -> None:
    """Allocation-free device-buffer ring kernel (fixed scratch; N <= 16384, M <= 65536).

    For callers that cannot allocate device memory at call time; see
    include/vlm.h for the limits and the shared-scratch rules.
    """
    _err(load().vlm_biot_savart_rings_noalloc(corners_ptr, rvc_ptr, gam_ptr, N, P_ptr, M, V_ptr, precision,
                                              stream or None))


class Case:
    """One rotor case on the GPU: the reference's rotor object + time loop."""

    def __init__(self, config_text: str, geom_text: str, base_dir: str | os.PathLike = "",
                 precision: int = PREC_FP64, sum_chunk: Optional[int] = None, near_factor: Optional[float] = None,
                 solve_mode: Optional[int] = None, use_graph: bool = True, nbody_slots: int = 0,
                 device: int = 0, lattice: Optional[bool] = None, incremental: Optional[bool] = None):
        L = load()
        self._h = _vp()
        self.opt = options(precision, sum_chunk, near_factor, device=device, use_graph=use_graph,
                           solve_mode=solve_mode)
        self.opt.nbody_slots = nbody_slots
        if lattice is not None:
            self.opt.lattice = 1 if lattice else 0
        if incremental is not None:
            self.opt.incremental = 1 if incremental else 0
        _err(L.vlm_case_create(config_text.encode(), geom_text.encode(), str(base_dir).encode(),
                               ctypes.byref(self.opt), ctypes.byref(self._h)))

    @classmethod
    def from_case_dir(cls, case_dir: str | os.PathLike, **kw) -> "Case":
        d = Path(case_dir)
        return cls((d / "config.nml").read_text(), (d / "geom01.nml").read_text(), d, **kw)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().vlm_case_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def start(self):
        _err(load().vlm_case_start(self._h))

    def step(self, n: int = 1, with_ct: bool = True) -> Optional[np.ndarray]:
        rows = np.zeros((n, 10)) if with_ct else None
        _err(load().vlm_case_step(self._h, int(n), _ptr(rows) if with_ct else None))
        return rows

    def set_tile(self, shape: int, chunks: int = 0):
        """FP32 N-body tile shape for the steps to come (-1: autotune)."""
        _err(load().vlm_case_set_tile(self._h, int(shape), int(chunks)))

    def autotune(self) -> np.ndarray:
        """Autotuner records: rows of rowNear, rowFar, candidates, then per
        evaluation (wake nodes, collocation points) shape, chunks, ms, model ms."""
        return self.get("autotune").reshape(-1, 11)

    def incremental_plans(self) -> np.ndarray:
        """Incremental predicted-wake evaluation, one row per measured wake
        signature: rowNear, rowFar, used (0/1), changed records, moved nodes,
        record capacity, node capacity, records, nodes."""
        return self.get("incremental").reshape(-1, 9)

    # the step as separate calls (include/vlm.h): solve -> [loads] -> wake
    def aic_factor(self):
        _err(load().vlm_case_aic_factor(self._h))

    def solve_circulation(self, kinematic_vel=None) -> np.ndarray:
        """Opens iteration iter+1: RHS + solve; returns gamVec (n).
        kinematic_vel (n x 3) replaces the library's kinematic velocity."""
        n = self.geti("n")
        gam = np.zeros(n)
        kv = None if kinematic_vel is None else _c64(kinematic_vel).reshape(-1)
        if kv is not None and kv.size != 3 * n:
            raise ValueError("kinematic_vel must have 3 x n values")
        _err(load().vlm_case_solve_circulation(self._h, _ptr(kv) if kv is not None else None, _ptr(gam)))
        return gam

    def loads(self) -> np.ndarray:
        row = np.zeros(10)
        _err(load().vlm_case_loads(self._h, _ptr(row)))
        return row

    def wake_step(self):
        _err(load().vlm_case_wake_step(self._h))

    def get_wake(self, blade: int = 1):
        """(waN (nNwake*ns, 4, 3), waN_gam, waF (nFwake, 2, 3), waF_gam) of a blade."""
        NW, NF, ns = self.geti("nNwake"), self.geti("nFwake"), self.geti("ns")
        wn, wg = np.zeros(12 * NW * ns), np.zeros(max(NW * ns, 1))
        fn, fg = np.zeros(max(6 * NF, 1)), np.zeros(max(NF, 1))
        _err(load().vlm_case_get_wake(self._h, blade, _ptr(wn), _ptr(wg), _ptr(fn), _ptr(fg)))
        return wn.reshape(-1, 4, 3), wg[:NW * ns], fn[:6 * NF].reshape(-1, 2, 3), fg[:NF]

    def geti(self, name: str) -> int:
        v = _i64()
        _err(load().vlm_case_get_int(self._h, name.encode(), ctypes.byref(v)))
        return int(v.value)

    def get(self, name: str, blade: int = 1) -> np.ndarray:
        L = load()
        n = L.vlm_case_get(self._h, name.encode(), blade, None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(max(n, 1))
        L.vlm_case_get(self._h, name.encode(), blade, _ptr(out), n)
        return out[:n]

    def checkpoint_save(self, path) -> None:
        _err(load().vlm_case_checkpoint_save(self._h, str(path).encode()))

    def checkpoint_load(self, path) -> None:
        _err(load().vlm_case_checkpoint_load(self._h, str(path).encode()))

    def set_surrogate(self, **kw) -> None:
        """Enable the learned far-wake surrogate (before start); keywords
        override the defaults of vlm_surrogate_options."""
        o = SurrogateOptions()
        load().vlm_default_surrogate_options(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        _err(load().vlm_case_set_surrogate(self._h, ctypes.byref(o)))

    def surrogate_stats(self) -> dict:
        st = SurrogateStats()
        _err(load().vlm_case_surrogate_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def ct_hist(self) -> np.ndarray:
        return self.get("ct_hist").reshape(-1, 10)

    def force_dist(self, blade: int = 1) -> np.ndarray:
        """(ns, 16) sectional loads of the current iteration in the columns of
        rXXbYYForceDistNNNNN.csv (blade 1..nbConvect)."""
        return self.get("forceDist", blade).reshape(-1, 16)

    def force_dim(self) -> np.ndarray:
        """The eleven rXXForceDim.csv values of the current iteration."""
        return self.get("forceDim")

    def params_json(self) -> str:
        """The rXXParams.json text of this case."""
        L = load()
        n = L.vlm_case_params_json(self._h, None, 0)
        if n < 0:
            raise VlmError(1, "vlm_case_params_json failed")
        buf = ctypes.create_string_buffer(int(n) + 1)
        L.vlm_case_params_json(self._h, buf, n + 1)
        return buf.value.decode()

    def vind_points(self, P) -> np.ndarray:
        P = _c64(P).reshape(-1, 3)
        V = np.zeros_like(P)
        _err(load().vlm_case_vind_points(self._h, _ptr(P), P.shape[0], _ptr(V)))
        return V

    def profile_eval(self, reps: int = 10):
        """(ms per launch, ring-target pairs, filament-target pairs) of the hot kernel."""
        ms, rp, fp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _err(load().vlm_case_profile_eval(self._h, reps, ctypes.byref(ms), ctypes.byref(rp), ctypes.byref(fp)))
        return ms.value, rp.value, fp.value

    def last_step_ms(self) -> float:
        ms = ctypes.c_double()
        _err(load().vlm_case_last_step_ms(self._h, ctypes.byref(ms)))
        return ms.value


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_fp)


class Mlp:
    """The surrogate's FP32 MLP (tanh hidden layers, linear output) on the GPU:
    forward, MSE gradient and Adam training by the library's own kernels."""

    def __init__(self, sizes, seed: int = 0):
        arr = (ctypes.c_int * len(sizes))(*sizes)
        self.sizes = list(sizes)
        self._h = _vp()
        _err(load().vlm_mlp_create(arr, len(sizes), seed, ctypes.byref(self._h)))

    @property
    def nparam(self) -> int:
        return int(load().vlm_mlp_param_count(self._h))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.nparam, dtype=np.float32)
        _err(load().vlm_mlp_get_params(self._h, _fptr(out)))
        return out

    def set_params(self, p) -> None:
        p = _f32(p)
        assert p.size == self.nparam
        _err(load().vlm_mlp_set_params(self._h, _fptr(p)))

    def forward(self, X) -> np.ndarray:
        X = _f32(X).reshape(-1, self.sizes[0])
        Y = np.zeros((X.shape[0], self.sizes[-1]), dtype=np.float32)
        _err(load().vlm_mlp_forward(self._h, _fptr(X), X.shape[0], _fptr(Y)))
        return Y

    INFER_FP32, INFER_TENSOR_CORES = 0, 1

    def set_inference(self, mode: int) -> None:
        """Forward-pass arithmetic: INFER_TENSOR_CORES (BF16 tcgen05 MMAs,
        the default when the network fits) or INFER_FP32 (CUDA cores)."""
        _err(load().vlm_mlp_set_inference(self._h, int(mode)))

    @property
    def inference(self) -> int:
        return int(load().vlm_mlp_get_inference(self._h))

    def gradient(self, X, T):
        X = _f32(X).reshape(-1, self.sizes[0])
        T = _f32(T).reshape(-1, self.sizes[-1])
        g = np.zeros(self.nparam, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _err(load().vlm_mlp_gradient(self._h, _fptr(X), _fptr(T), X.shape[0], _fptr(g), _fptr(loss)))
        return g, float(loss[0])

    def train(self, X, T, batch: int, iters: int, lr: float) -> float:
        X = _f32(X).reshape(-1, self.sizes[0])
        T = _f32(T).reshape(-1, self.sizes[-1])
        loss = np.zeros(1, dtype=np.float32)
        _err(load().vlm_mlp_train(self._h, _fptr(X), _fptr(T), X.shape[0], batch, iters, lr, _fptr(loss)))
        return float(loss[0])

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().vlm_mlp_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _BorrowedCase(Case):
    """A case owned by a batch (getters only)."""

    def __init__(self, handle, batch):
        self._h = handle
        self._batch = batch  # keeps the batch alive

    def close(self):
        self._h = _vp()


class System:
    """Coupled rotors (nr > 1): config.nml and one geomXX.nml per rotor,
    every induced-velocity sum over all rotors (include/vlm.h, vlm_system_*).
    ``rotors[i]`` are borrowed Case handles for the getters."""

    def __init__(self, config_text: str, geom_texts, base_dir: str | os.PathLike = "",
                 precision: int = PREC_FP64, sum_chunk: Optional[int] = None, near_factor: Optional[float] = None,
                 solve_mode: Optional[int] = None, device: int = 0, lattice: Optional[bool] = None):
        n = len(geom_texts)
        self._geo = (ctypes.c_char_p * n)(*[g.encode() for g in geom_texts])
        self.opt = options(precision, sum_chunk, near_factor, device=device, use_graph=False, solve_mode=solve_mode)
        if lattice is not None:
            self.opt.lattice = 1 if lattice else 0
        self.nr = n
        self._h = _vp()
        _err(load().vlm_system_create(config_text.encode(), n, self._geo, str(base_dir).encode(),
                                      ctypes.byref(self.opt), ctypes.byref(self._h)))
        self.rotors = []
        for i in range(n):
            h = _vp()
            _err(load().vlm_system_rotor(self._h, i, ctypes.byref(h)))
            self.rotors.append(_BorrowedCase(h, self))

    def start(self):
        _err(load().vlm_system_start(self._h))

    def step(self, n: int = 1, with_ct: bool = True) -> Optional[np.ndarray]:
        """n iterations; CT rows as [step][rotor][10]."""
        rows = np.zeros((n, self.nr, 10)) if with_ct else None
        _err(load().vlm_system_step(self._h, int(n), _ptr(rows) if with_ct else None))
        return rows

    def last_step_ms(self) -> float:
        ms = ctypes.c_double()
        _err(load().vlm_system_last_step_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            for r in self.rotors:
                r._h = _vp()
            load().vlm_system_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent cases advanced together (one graph launch per step in
    steady state); cases = [(config_text, geom_text, base_dir), ...]."""

    def __init__(self, cases, precision: int = PREC_FP64, sum_chunk: Optional[int] = None,
                 nbody_slots: int = 0, use_graph: bool = True, lattice: Optional[bool] = None,
                 incremental: Optional[bool] = None):
        n = len(cases)
        enc = lambda i: (ctypes.c_char_p * n)(*[str(c[i]).encode() for c in cases])
        self._cfg, self._geo, self._dir = enc(0), enc(1), enc(2)
        self.opt = options(precision, sum_chunk, use_graph=use_graph)
        self.opt.nbody_slots = nbody_slots
        if lattice is not None:
            self.opt.lattice = 1 if lattice else 0
        if incremental is not None:
            self.opt.incremental = 1 if incremental else 0
        self.n = n
        self._h = _vp()
        _err(load().vlm_batch_create(n, self._cfg, self._geo, self._dir, ctypes.byref(self.opt), ctypes.byref(self._h)))

    def case(self, i: int) -> Case:
        h = _vp()
        _err(load().vlm_batch_case(self._h, i, ctypes.byref(h)))
        return _BorrowedCase(h, self)

    def start(self):
        _err(load().vlm_batch_start(self._h))

    def step(self, n: int = 1, with_ct: bool = True) -> Optional[np.ndarray]:
        rows = np.zeros((self.n, n, 10)) if with_ct else None
        _err(load().vlm_batch_step(self._h, n, _ptr(rows) if with_ct else None))
        return rows

    def last_step_ms(self) -> float:
        ms = ctypes.c_double()
        _err(load().vlm_batch_last_step_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().vlm_batch_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_bounded_wait(limit: int = 4096) -> bool:
    """True when a device wait that nothing releases gave up and reported."""
    out = ctypes.c_int(-1)
    _err(load().vlm_selftest_bounded_wait(limit, ctypes.byref(out)))
    return out.value == 1
