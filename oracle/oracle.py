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
        L.orc_qspeed_f32.argtypes = [_F, C.c_int, _F, _F, _F]
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


def qspeed(F: np.ndarray, n: int) -> tuple:
    """(Q, speed, velocity) of a float macro field [cell][rho,u,v,w] as the uniform program's VTK
    writer forms them (src/tgv3d_uniform.cu:112-121)."""
    F = np.ascontiguousarray(F, dtype=np.float32).reshape(-1)
    q, sp, v = (np.empty(n ** 3, dtype=np.float32), np.empty(n ** 3, dtype=np.float32),
                np.empty(3 * n ** 3, dtype=np.float32))
    orc().orc_qspeed_f32(_fp(F), n, _fp(q), _fp(sp), _fp(v))
    return q, sp, v


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


def ref_run_inplace(f: np.ndarray, n: int, omega: float, nsteps: int) -> None:
    """ref_run on f itself (no host copy: the N=512 state is 10.2 GB)."""
    assert f.dtype == np.float32 and f.flags.c_contiguous
    _rck(ref().ref_uniform_run(_fp(f), n, omega, nsteps))


def ref_macro(f: np.ndarray, n: int) -> np.ndarray:
    F = np.empty(4 * n ** 3, dtype=np.float32)
    _rck(ref().ref_uniform_macro(_fp(np.ascontiguousarray(f, dtype=np.float32)), n, _fp(F)))
    return F


def ref_time(n: int, omega: float, warmup: int, nsteps: int, u0: float = 0.05) -> float:
    ms = C.c_float()
    _rck(ref().ref_uniform_time(n, u0, omega, warmup, nsteps, C.byref(ms)))
    return ms.value


# ---- AMR: CPU restatement (liboracle) and the reference's kernels (librefrun) ----------------------

TABLES = {"ref0": 0, "fof0": 1, "rl0": 2, "l1pcb": 3, "l1oct": 4, "f1pos": 5, "l1grid": 6, "ref1": 7, "fof1": 8,
          "rl1": 9, "l2pl1": 10, "l2oct": 11, "skin0": 12, "skin1": 13, "deep": 14}
COUNTS = ["nref0", "nf1", "nref1", "nf2", "n_skin0", "n_skin1", "cap1", "cap2", "cnb0", "ng1", "hw_nf1", "hw_nf2",
          "ndeep", "cap_nref0", "cap_nref1", "steps"]
MODES = {"all": 0, "slab": 1, "sensor": 2}
BIG_BUDGET = float(1 << 40)


def _amr_sigs(L, prefix):
    vp = C.c_void_p
    getattr(L, prefix + "_destroy").argtypes = [vp]
    getattr(L, prefix + "_set_sensor_override").argtypes = [vp, _F, _F]
    getattr(L, prefix + "_regrid").argtypes = [vp]
    getattr(L, prefix + "_step").argtypes = [vp, C.c_long]
    getattr(L, prefix + "_diag").argtypes = [vp, _D]
    getattr(L, prefix + "_counts").argtypes = [vp, C.POINTER(C.c_long)]
    getattr(L, prefix + "_get_table").argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.c_long]
    getattr(L, prefix + "_get_sensor").argtypes = [vp, C.c_int, _F, C.c_long]
    getattr(L, prefix + "_get_pops").argtypes = [vp, C.c_int, _F, C.c_long]
    getattr(L, prefix + "_get_pops").restype = C.c_long
    getattr(L, prefix + "_set_pops").argtypes = [vp, C.c_int, _F, C.c_long]
    getattr(L, prefix + "_set_pops").restype = C.c_long


_amr_orc_ready = False


class AmrBackend:
    """Common driver of the CPU oracle ('oracle') and of the reference's kernels ('reference')."""

    def __init__(self, which: str, n: int, re: float, l1: str = "all", l2: str = "all", frac1: float = 0.35,
                 frac2: float = 0.35, u0: float = 0.05, tstar: float = 12.0, develop: int = 300,
                 budget: float = BIG_BUDGET, mb: int = 8, build: bool = True, grow: bool = False):
        global _amr_orc_ready
        self.which = which
        self.n, self.mb = n, mb
        if which == "oracle":
            L = orc()
            if not _amr_orc_ready:
                L.orc_amr_create.restype = C.c_void_p
                L.orc_amr_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                             C.c_double, C.c_double, C.c_int, C.c_double]
                L.orc_amr_initial_build.argtypes = [C.c_void_p]
                _amr_sigs(L, "orc_amr")
                _amr_orc_ready = True
            self.L, self.p = L, "orc_amr"
            self.h = L.orc_amr_create(n, mb, re, u0, tstar, MODES[l1], MODES[l2], frac1, frac2, develop, budget)
            if self.h and grow:
                L.orc_amr_set_growth.argtypes = [C.c_void_p, C.c_int]
                L.orc_amr_set_growth(C.c_void_p(self.h), 1)
        else:
            L = ref_amr()
            if mb != 8:
                raise ValueError("the reference cubin is built with MB=8")
            self.L, self.p = L, "ref_amr"
            self.h = L.ref_amr_create(n, re, u0, tstar, MODES[l1], MODES[l2], frac1, frac2, develop, budget)
        if not self.h:
            raise RuntimeError("AMR %s create failed" % which)
        if build:
            self.initial_build()

    def _f(self, name):
        return getattr(self.L, self.p + "_" + name)

    def initial_build(self):
        rc = self._f("initial_build")(C.c_void_p(self.h))
        if rc:
            raise RuntimeError("%s initial build failed (%d)" % (self.which, rc))

    def close(self):
        if self.h:
            self._f("destroy")(C.c_void_p(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_sensor_override(self, sen0, sen1pos):
        s0 = np.ascontiguousarray(sen0, dtype=np.float32)
        s1 = np.ascontiguousarray(sen1pos, dtype=np.float32)
        self._keep = (s0, s1)
        self._f("set_sensor_override")(C.c_void_p(self.h), _fp(s0), _fp(s1))

    def regrid(self):
        rc = self._f("regrid")(C.c_void_p(self.h))
        if rc:
            raise RuntimeError("%s regrid failed (%d)" % (self.which, rc))

    def step(self, k: int = 1):
        rc = self._f("step")(C.c_void_p(self.h), k)
        if rc:
            raise RuntimeError("%s step failed (%d)" % (self.which, rc))

    def diag(self):
        out = np.empty(3)
        self._f("diag")(C.c_void_p(self.h), _dp(out))
        return tuple(float(x) for x in out)

    def counts(self) -> dict:
        v = (C.c_long * 16)()
        self._f("counts")(C.c_void_p(self.h), v)
        return dict(zip(COUNTS, list(v)))

    def table(self, name: str) -> np.ndarray:
        c = self.counts()
        cap = max(c["ng1"], c["cnb0"], c["cap1"], c["cap2"], 1)
        a = np.empty(cap, dtype=np.int32)
        n = self._f("get_table")(C.c_void_p(self.h), TABLES[name], a.ctypes.data_as(C.POINTER(C.c_int)), cap)
        if n < 0:
            raise RuntimeError("table %s: %d" % (name, n))
        return a[:n].copy()

    def sensor(self, level: int) -> np.ndarray:
        c = self.counts()
        a = np.empty(max(c["cnb0"], c["cap1"], 1), dtype=np.float32)
        n = self._f("get_sensor")(C.c_void_p(self.h), level, _fp(a), a.size)
        return a[:n].copy()

    def pops(self, level: int) -> np.ndarray:
        c = self.counts()
        nb = {0: c["cnb0"], 1: c["nf1"], 2: c["nf2"]}[level]
        a = np.empty(max(nb * Q * self.mb ** 3, 1), dtype=np.float32)
        n = self._f("get_pops")(C.c_void_p(self.h), level, _fp(a), a.size)
        if n < 0:
            raise RuntimeError("pops: %d" % n)
        return a[:n].copy()

    def qspeed(self) -> tuple:
        """(Q, speed) on the (4 n)^3 composite: the reference's k_composite + k_qspeed."""
        nn = (4 * self.n) ** 3
        q, sp = np.empty(nn, dtype=np.float32), np.empty(nn, dtype=np.float32)
        rc = self.L.ref_amr_qspeed(C.c_void_p(self.h), _fp(q), _fp(sp))
        if rc:
            raise RuntimeError("reference qspeed failed (%d): %s" % (rc, self.L.refrun_last_error().decode()))
        return q, sp

    def set_pops(self, level: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        n = self._f("set_pops")(C.c_void_p(self.h), level, _fp(a), a.size)
        if n < 0:
            raise RuntimeError("set_pops: %d" % n)


_ref_amr_ready = False


def ref_amr_available() -> bool:
    return os.path.exists(REFRUN_LIB) and os.path.exists(REF_AMR_CUBIN)


def ref_amr() -> C.CDLL:
    global _ref_amr_ready
    L = ref()
    if not _ref_amr_ready:
        L.refrun_load_amr.argtypes = [C.c_char_p]
        rc = L.refrun_load_amr(REF_AMR_CUBIN.encode())
        if rc:
            raise RuntimeError("reference AMR cubin load failed: %s" % L.refrun_last_error().decode())
        L.ref_amr_create.restype = C.c_void_p
        L.ref_amr_create.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double,
                                     C.c_double, C.c_int, C.c_double]
        L.ref_amr_initial_build.argtypes = [C.c_void_p]
        L.ref_amr_time.argtypes = [C.c_void_p, C.c_long, C.c_long, _F]
        L.ref_amr_qspeed.argtypes = [C.c_void_p, _F, _F]
        _amr_sigs(L, "ref_amr")
        _ref_amr_ready = True
    return L


def random_sensor_fields(n: int, mb: int = 8, seed: int = 0, ties: bool = False):
    """Seeded sensor fields for bit-exact table comparisons: one value per coarse block and one per
    level-1 grid position.  ties=True draws from a few levels so thresholds fall on ties."""
    rng = np.random.default_rng(seed)
    cgx = n // mb
    cnb0, ng1 = cgx ** 3, (2 * cgx) ** 3
    if ties:
        return (rng.integers(0, 4, cnb0).astype(np.float32) * 0.25, rng.integers(0, 5, ng1).astype(np.float32) * 0.2)
    return rng.random(cnb0, dtype=np.float32), rng.random(ng1, dtype=np.float32)
