"""ORACLE - test infrastructure only.  ctypes bindings of the CPU restatement (liboracle.so) and of
the loader that runs the reference's own kernels (librefrun.so + _ref/*.cubin).  Imported only by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REFRUN_LIB = os.path.join(HERE, "librefrun.so")
REF_UNIFORM_CUBIN = os.path.join(HERE, "_ref", "ref_uniform_mb8.cubin")
REF_AMR_CUBIN = os.path.join(HERE, "_ref", "ref_amr_mb8.cubin")
Q = 19

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)

_orc = None
_ref = None


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError("liboracle.so missing: run python oracle/build.py")
        L = C.CDLL(ORACLE_LIB)
        L.orc_init_tgv_f32.argtypes = [_F, C.c_int, C.c_int, C.c_double]
        L.orc_init_tgv_f64.argtypes = [_D, C.c_int, C.c_int, C.c_double]
        L.orc_step_f32.argtypes = [_F, _F, C.c_int, C.c_int, C.c_float]
        L.orc_step_f64.argtypes = [_D, _D, C.c_int, C.c_int, C.c_double]
        L.orc_macro_f32.argtypes = [_F, C.c_int, C.c_int, _F]
        L.orc_macro_f64.argtypes = [_D, C.c_int, C.c_int, _D]
        L.orc_diag_f32.argtypes = [_F, C.c_int, _D]
        L.orc_diag_f64.argtypes = [_D, C.c_int, _D]
        L.orc_run_f32.argtypes = [_F, _F, C.c_int, C.c_int, C.c_float, C.c_long]
        L.orc_run_f32.restype = C.c_int
        _orc = L
    return _orc


# ---- layouts --------------------------------------------------------------------------------------

def blocked_to_flat(fb: np.ndarray, n: int, mb: int) -> np.ndarray:
    """[block][q][cell] (block=(bz*gx+by)*gx+bx, cell=(k*mb+j)*mb+i) -> [q][z][y][x]."""
    gx = n // mb
    a = fb.reshape(gx, gx, gx, Q, mb, mb, mb)          # bz by bx q k j i
    a = a.transpose(3, 0, 4, 1, 5, 2, 6)                # q bz k by j bx i
    return np.ascontiguousarray(a.reshape(Q, n, n, n))


def flat_to_blocked(ff: np.ndarray, n: int, mb: int) -> np.ndarray:
    gx = n // mb
    a = ff.reshape(Q, gx, mb, gx, mb, gx, mb)           # q bz k by j bx i
    a = a.transpose(1, 3, 5, 0, 2, 4, 6)                # bz by bx q k j i
    return np.ascontiguousarray(a.reshape(-1))


# ---- uniform oracle (reference blocked layout) ----------------------------------------------------

def params(n: int, re: float, u0: float = 0.05, tstar: float = 12.0) -> dict:
    """nu, tau, omega (float), steps as src/tgv3d_uniform.cu:151-153 derives them."""
    nu = u0 * n / (2.0 * np.pi * re)
    tau = 3.0 * nu + 0.5
    kf = 2.0 * np.pi / n
    return {"nu": nu, "tau": tau, "omega": float(np.float32(1.0 / tau)), "omega_d": 1.0 / tau, "kf": kf,
            "steps": int(tstar / (u0 * kf) + 0.5)}


def init_tgv(n: int, mb: int = 8, u0: float = 0.05, dtype=np.float32) -> np.ndarray:
    f = np.empty(Q * n ** 3, dtype=dtype)
    if dtype == np.float32:
        orc().orc_init_tgv_f32(_fp(f), n, mb, u0)
    else:
        orc().orc_init_tgv_f64(_dp(f), n, mb, u0)
    return f


def step(f: np.ndarray, n: int, mb: int, omega: float, nsteps: int = 1) -> np.ndarray:
    a = np.array(f, copy=True)
    b = np.empty_like(a)
    for _ in range(nsteps):
        if a.dtype == np.float32:
            orc().orc_step_f32(_fp(a), _fp(b), n, mb, omega)
        else:
            orc().orc_step_f64(_dp(a), _dp(b), n, mb, omega)
        a, b = b, a
    return a


def macro(f: np.ndarray, n: int, mb: int) -> np.ndarray:
    out = np.empty(4 * n ** 3, dtype=f.dtype)
    if f.dtype == np.float32:
        orc().orc_macro_f32(_fp(f), n, mb, _fp(out))
    else:
        orc().orc_macro_f64(_dp(f), n, mb, _dp(out))
    return out


def diag_field(F: np.ndarray, n: int) -> tuple:
    out = np.empty(3, dtype=np.float64)
    if F.dtype == np.float32:
        orc().orc_diag_f32(_fp(F), n, _dp(out))
    else:
        orc().orc_diag_f64(_dp(F), n, _dp(out))
    return float(out[0]), float(out[1]), float(out[2])


def diag(f: np.ndarray, n: int, mb: int) -> tuple:
    return diag_field(macro(f, n, mb), n)


# ---- the reference's own kernels on the GPU ------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REFRUN_LIB) and os.path.exists(REF_UNIFORM_CUBIN)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        L = C.CDLL(REFRUN_LIB)
        L.refrun_last_error.restype = C.c_char_p
        L.refrun_load_uniform.argtypes = [C.c_char_p]
        L.ref_uniform_init.argtypes = [_F, C.c_int, C.c_double]
        L.ref_uniform_run.argtypes = [_F, C.c_int, C.c_float, C.c_long]
        L.ref_uniform_macro.argtypes = [_F, C.c_int, _F]
        L.ref_uniform_time.argtypes = [C.c_int, C.c_double, C.c_float, C.c_long, C.c_long, _F]
        rc = L.refrun_load_uniform(REF_UNIFORM_CUBIN.encode())
        if rc:
            raise RuntimeError("reference cubin load failed: %s" % L.refrun_last_error().decode())
        _ref = L
    return _ref


def _rck(rc: int) -> None:
    if rc:
        raise RuntimeError("reference kernel run failed (%d): %s" % (rc, ref().refrun_last_error().decode()))


def ref_init(n: int, u0: float = 0.05) -> np.ndarray:
    f = np.empty(Q * n ** 3, dtype=np.float32)
    _rck(ref().ref_uniform_init(_fp(f), n, u0))
    return f


def ref_run(f: np.ndarray, n: int, omega: float, nsteps: int) -> np.ndarray:
    a = np.array(f, dtype=np.float32, copy=True)
    _rck(ref().ref_uniform_run(_fp(a), n, omega, nsteps))
    return a


def ref_macro(f: np.ndarray, n: int) -> np.ndarray:
    F = np.empty(4 * n ** 3, dtype=np.float32)
    _rck(ref().ref_uniform_macro(_fp(np.ascontiguousarray(f, dtype=np.float32)), n, _fp(F)))
    return F


def ref_time(n: int, omega: float, warmup: int, nsteps: int, u0: float = 0.05) -> float:
    ms = C.c_float()
    _rck(ref().ref_uniform_time(n, u0, omega, warmup, nsteps, C.byref(ms)))
    return ms.value
