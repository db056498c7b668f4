"""ctypes binding of libjpsolver.so (the C ABI in include/jp.h).

This is the reference-facing boundary seen from Python: tests and bench.py drive the engine only
through these calls.  There is no fallback: if the shared library is missing, importing works but
creating a solver raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libjpsolver.so")

UNIFORM, AMR = 0, 1
STORAGE = {"fp32": 0, "fp16": 1, "bf16": 2, "fp64": 3}
REFINE = {"all": 0, "slab": 1, "sensor": 2}
LAYOUT = {"flat": 0, "blocked": 1}
Q = 19


class JPError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("jp status %d: %s" % (status, msg))
        self.status = status


class Config(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("n", C.c_int32),
        ("re", C.c_double), ("u0", C.c_double), ("tstar", C.c_double),
        ("storage", C.c_int32), ("mb", C.c_int32),
        ("l1_mode", C.c_int32), ("l2_mode", C.c_int32),
        ("frac1", C.c_double), ("frac2", C.c_double),
        ("adapt_every", C.c_int32), ("develop_steps", C.c_int32),
        ("max_gb", C.c_double),
        ("device", C.c_int32), ("threads_per_block", C.c_int32), ("vec", C.c_int32),
        ("flags", C.c_int32), ("buffer", C.c_int32), ("reserved", C.c_int32 * 6),
    ]


FLAG_SKIP_PREP, FLAG_SKIP_RESTRICT, FLAG_GRAPH, FLAG_DEFER_INIT, FLAG_INPLACE = 1, 2, 4, 8, 16


class Info(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("n", C.c_int32), ("mb", C.c_int32), ("storage", C.c_int32),
        ("cells", C.c_int64), ("steps", C.c_int64),
        ("nu", C.c_double), ("tau", C.c_double), ("omega", C.c_double),
        ("tau1", C.c_double), ("tau2", C.c_double), ("kf", C.c_double),
        ("bytes_state", C.c_int64), ("step_count", C.c_int64),
        ("reserved", C.c_int32 * 8),
    ]


class AmrCounts(C.Structure):
    _fields_ = [
        ("nref0", C.c_int32), ("nf1", C.c_int32), ("nref1", C.c_int32), ("nf2", C.c_int32),
        ("n_skin0", C.c_int32), ("n_skin1", C.c_int32), ("ndeep", C.c_int32),
        ("cnb0", C.c_int32), ("ng1", C.c_int32), ("cap_nref0", C.c_int32), ("cap1", C.c_int32),
        ("cap_nref1", C.c_int32), ("cap2", C.c_int32), ("pad", C.c_int32),
        ("hw_nf1", C.c_int64), ("hw_nf2", C.c_int64),
        ("reserved", C.c_int32 * 8),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_active", C.c_int32), ("pool_gb", C.c_double),
                ("tick_steps", C.c_int32), ("workers", C.c_int32), ("uniform_first", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class ServerStats(C.Structure):
    _fields_ = [("create_s", C.c_double), ("step_s", C.c_double), ("regrid_s", C.c_double),
                ("diag_s", C.c_double), ("destroy_s", C.c_double), ("tick_s", C.c_double),
                ("solves", C.c_int64), ("regrids", C.c_int64), ("diags", C.c_int64),
                ("coarse_steps", C.c_int64), ("uniform_gpu_s", C.c_double), ("amr_gpu_s", C.c_double),
                ("reserved", C.c_int64 * 6)]


class Request(C.Structure):
    _fields_ = [("id", C.c_int64), ("cfg", Config), ("diag_every", C.c_int32), ("reserved", C.c_int32 * 7)]


class Result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("valid", C.c_int32), ("steps", C.c_int64),
                ("samples", C.c_int32), ("pad", C.c_int32),
                ("peak_tstar", C.c_double), ("peak_enstrophy", C.c_double), ("energy_ratio", C.c_double),
                ("mass_drift", C.c_double), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_end", C.c_double), ("bytes", C.c_int64), ("reserved", C.c_int32 * 8)]


TABLES = {"ref0": 0, "fof0": 1, "rl0": 2, "l1pcb": 3, "l1oct": 4, "f1pos": 5, "l1grid": 6, "ref1": 7, "fof1": 8,
          "rl1": 9, "l2pl1": 10, "l2oct": 11, "skin0": 12, "skin1": 13, "deep": 14}

_lib: Optional[C.CDLL] = None

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "jp_config_default": (None, [C.POINTER(Config), C.c_int32]),
    "jp_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "jp_destroy": (None, [C.c_void_p]),
    "jp_last_error": (C.c_char_p, []),
    "jp_abi_version": (C.c_int32, []),
    "jp_build_info": (C.c_char_p, []),
    "jp_sizeof": (C.c_size_t, [C.c_int32]),
    "jp_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "jp_init_tgv": (C.c_int, [C.c_void_p]),
    "jp_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "jp_sync": (C.c_int, [C.c_void_p]),
    "jp_diag": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "jp_population_count": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "jp_get_populations": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64]),
    "jp_set_populations": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64]),
    "jp_stage_populations": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64]),
    "jp_get_macro": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "jp_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "jp_host_free": (None, [C.c_void_p]),
    "jp_step_timed": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float)]),
    "jp_save_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "jp_load_state": (C.c_int, [C.c_void_p, C.c_char_p]),
    "jp_launch_count": (C.c_int64, []),
    "jp_regrid": (C.c_int, [C.c_void_p]),
    "jp_autotune": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(C.c_double)]),
    "jp_ensemble_create": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p)]),
    "jp_ensemble_destroy": (None, [C.c_void_p]),
    "jp_ensemble_add": (C.c_int, [C.c_void_p, C.c_void_p]),
    "jp_ensemble_remove": (C.c_int, [C.c_void_p, C.c_void_p]),
    "jp_ensemble_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "jp_ensemble_set_persistent": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_int32]),
    "jp_ensemble_sync": (C.c_int, [C.c_void_p]),
    "jp_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "jp_server_destroy": (None, [C.c_void_p]),
    "jp_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request)]),
    "jp_server_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "jp_server_poll": (C.c_int32, [C.c_void_p, C.POINTER(Result), C.c_int32]),
    "jp_server_clock": (C.c_double, [C.c_void_p]),
    "jp_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "jp_get_output_fields": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                       C.c_int64]),
    "jp_memory_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "jp_diag_field_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "jp_amr_get_counts": (C.c_int, [C.c_void_p, C.POINTER(AmrCounts)]),
    "jp_get_table": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int64)]),
    "jp_get_sensor": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_int64)]),
    "jp_set_sensor_override": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
}


def lib() -> C.CDLL:
    """Load libjpsolver.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libjpsolver.so not found at %s: run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(st: int) -> None:
    if st != 0:
        raise JPError(st, lib().jp_last_error().decode())


def config(kind: str = "uniform", **kw) -> Config:
    c = Config()
    lib().jp_config_default(C.byref(c), UNIFORM if kind == "uniform" else AMR)
    for k, v in kw.items():
        if k == "storage" and isinstance(v, str):
            v = STORAGE[v]
        if k in ("l1_mode", "l2_mode") and isinstance(v, str):
            v = REFINE[v]
        if not hasattr(c, k):
            raise KeyError("unknown config field %r" % k)
        setattr(c, k, v)
    return c


def autotune(kind: str = "uniform", steps: int = 10, **kw) -> tuple:
    """(tuned config fields, lattice updates per second) from jp_autotune."""
    c = config(kind, **kw)
    best = C.c_double()
    _check(lib().jp_autotune(C.byref(c), steps, C.byref(best)))
    return {"vec": c.vec, "threads_per_block": c.threads_per_block, "mb": c.mb}, best.value


class Solver:
    """One solve on the GPU (uniform periodic cube or 3-level AMR)."""

    def __init__(self, kind: str = "uniform", **kw):
        self.cfg = config(kind, **kw)
        h = C.c_void_p()
        _check(lib().jp_create(C.byref(self.cfg), C.byref(h)))
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().jp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def info(self) -> dict:
        i = Info()
        _check(lib().jp_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in Info._fields_ if k != "reserved"}

    def init_tgv(self) -> None:
        _check(lib().jp_init_tgv(self.h))

    def step(self, n: int = 1) -> None:
        _check(lib().jp_step(self.h, n))

    def sync(self) -> None:
        _check(lib().jp_sync(self.h))

    def save_state(self, path: str) -> None:
        """Write the solve's state to a file (jp_save_state)."""
        _check(lib().jp_save_state(self.h, str(path).encode()))

    def load_state(self, path: str) -> None:
        """Continue from a state file written by a solver of the same configuration (jp_load_state)."""
        _check(lib().jp_load_state(self.h, str(path).encode()))

    def step_timed(self, n: int) -> float:
        ms = C.c_float()
        _check(lib().jp_step_timed(self.h, n, C.byref(ms)))
        return ms.value

    def diag(self) -> tuple:
        out = (C.c_double * 3)()
        _check(lib().jp_diag(self.h, out))
        return out[0], out[1], out[2]

    def population_count(self, level: int = 0) -> int:
        c = C.c_int64()
        _check(lib().jp_population_count(self.h, level, C.byref(c)))
        return c.value

    def get_populations(self, level: int = 0, layout: str = "flat", dtype=np.float32) -> np.ndarray:
        cnt = self.population_count(level)
        if cnt == 0:
            return np.empty(0, dtype=dtype)
        a = np.empty(cnt, dtype=dtype)
        dt = 0 if a.dtype == np.float32 else 1
        _check(lib().jp_get_populations(self.h, level, LAYOUT[layout], dt, a.ctypes.data_as(C.c_void_p), cnt))
        return a

    def set_populations(self, a: np.ndarray, level: int = 0, layout: str = "flat") -> None:
        a = np.ascontiguousarray(a)
        if a.dtype not in (np.float32, np.float64):
            raise TypeError("populations must be float32 or float64")
        dt = 0 if a.dtype == np.float32 else 1
        _check(lib().jp_set_populations(self.h, level, LAYOUT[layout], dt, a.ctypes.data_as(C.c_void_p), a.size))
        self.sync()

    def stage_populations(self, buf: "PinnedBuffer") -> None:
        """Upload populations (flat layout, the storage's own type) from pinned memory for the next
        step, overlapping the work already queued (jp_stage_populations); the next step takes them.
        `buf` must stay unchanged until that step has been synchronised."""
        dt = 0 if buf.dtype == np.float32 else 1
        _check(lib().jp_stage_populations(self.h, LAYOUT["flat"], dt, C.c_void_p(buf.ptr.value), buf.array.size))

    # ---- AMR ----
    def regrid(self) -> None:
        _check(lib().jp_regrid(self.h))

    def counts(self) -> dict:
        c = AmrCounts()
        _check(lib().jp_amr_get_counts(self.h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in AmrCounts._fields_ if k not in ("reserved", "pad")}

    def table(self, name: str) -> np.ndarray:
        n = C.c_int64()
        lib().jp_get_table(self.h, TABLES[name], None, 0, C.byref(n))
        a = np.empty(max(n.value, 1), dtype=np.int32)
        _check(lib().jp_get_table(self.h, TABLES[name], a.ctypes.data_as(C.POINTER(C.c_int32)), a.size, C.byref(n)))
        return a[:n.value]

    def sensor(self, level: int) -> np.ndarray:
        n = C.c_int64()
        lib().jp_get_sensor(self.h, level, None, 0, C.byref(n))
        a = np.empty(max(n.value, 1), dtype=np.float32)
        _check(lib().jp_get_sensor(self.h, level, a.ctypes.data_as(C.POINTER(C.c_float)), a.size, C.byref(n)))
        return a[:n.value]

    def set_sensor_override(self, sen0=None, sen1_by_pos=None) -> None:
        if sen0 is None or sen1_by_pos is None:
            _check(lib().jp_set_sensor_override(self.h, None, None))
            return
        s0 = np.ascontiguousarray(sen0, dtype=np.float32)
        s1 = np.ascontiguousarray(sen1_by_pos, dtype=np.float32)
        _check(lib().jp_set_sensor_override(self.h, s0.ctypes.data_as(C.POINTER(C.c_float)),
                                            s1.ctypes.data_as(C.POINTER(C.c_float))))

    def output_fields(self, velocity: bool = False):
        """(Q, speed[, velocity]) on the output grid (uniform: n^3; AMR: (4 n)^3), z-y-x order."""
        n = self.cfg.n * (4 if self.cfg.kind == AMR else 1)
        c = n ** 3
        q = np.empty(c, dtype=np.float32)
        sp = np.empty(c, dtype=np.float32)
        v = np.empty(3 * c, dtype=np.float32) if velocity else None
        fp = C.POINTER(C.c_float)
        _check(lib().jp_get_output_fields(self.h, q.ctypes.data_as(fp), sp.ctypes.data_as(fp),
                                          v.ctypes.data_as(fp) if v is not None else None, c))
        return (q, sp, v) if velocity else (q, sp)

    def memory_info(self) -> tuple:
        f, t = C.c_int64(), C.c_int64()
        _check(lib().jp_memory_info(self.h, C.byref(f), C.byref(t)))
        return f.value, t.value

    def macro(self) -> np.ndarray:
        n = self.cfg.n
        a = np.empty(4 * n ** 3, dtype=np.float32)
        _check(lib().jp_get_macro(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))
        return a.reshape(n, n, n, 4)


def launch_count() -> int:
    return int(lib().jp_launch_count())


class PinnedBuffer:
    """Page-locked host memory from jp_host_alloc, viewed as a numpy array."""

    def __init__(self, count: int, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        self.nbytes = int(count) * self.dtype.itemsize
        p = C.c_void_p()
        _check(lib().jp_host_alloc(C.byref(p), self.nbytes))
        self.ptr = p
        buf = (C.c_char * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(count))

    def free(self) -> None:
        if self.ptr:
            self.array = None
            lib().jp_host_free(self.ptr)
            self.ptr = None


class Ensemble:
    """Uniform solvers stepped together in batched launches."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().jp_ensemble_create(device, C.byref(h)))
        self.h = h
        self.members = []

    def add(self, s: Solver) -> None:
        _check(lib().jp_ensemble_add(self.h, s.h))
        self.members.append(s)

    def remove(self, s: Solver) -> None:
        _check(lib().jp_ensemble_remove(self.h, s.h))
        self.members.remove(s)

    def step(self, n: int = 1) -> None:
        _check(lib().jp_ensemble_step(self.h, n))

    def set_persistent(self, mode: int = 1, wait_limit_ns: int = 0, grid: int = 0) -> None:
        """mode 1: AMR members' coarse steps in one persistent launch per jp_ensemble_step."""
        _check(lib().jp_ensemble_set_persistent(self.h, mode, wait_limit_ns, grid))

    def sync(self) -> None:
        """Wait for the queued steps; raises JPError (JP_ERR_TIMEOUT = 6) if a barrier gave up."""
        _check(lib().jp_ensemble_sync(self.h))

    def close(self) -> None:
        if self.h:
            lib().jp_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching solve server (jp_server_*)."""

    def __init__(self, device: int = 0, max_active: int = 0, pool_gb: float = 0.0, tick_steps: int = 64,
                 workers: int = 0, uniform_first: int = 0):
        c = ServerConfig()
        c.device, c.max_active, c.pool_gb, c.tick_steps, c.workers = device, max_active, pool_gb, tick_steps, workers
        c.uniform_first = uniform_first
        h = C.c_void_p()
        _check(lib().jp_server_create(C.byref(c), C.byref(h)))
        self.h = h

    def submit(self, rid: int, kind: str = "uniform", diag_every: int = 0, **kw) -> int:
        r = Request()
        r.id = rid
        r.cfg = config(kind, **kw)
        r.diag_every = diag_every
        return lib().jp_server_submit(self.h, C.byref(r))

    def tick(self) -> tuple:
        a, q = C.c_int32(), C.c_int32()
        _check(lib().jp_server_tick(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def poll(self, max_results: int = 256) -> list:
        buf = (Result * max_results)()
        n = lib().jp_server_poll(self.h, buf, max_results)
        return [{k: getattr(buf[i], k) for k, _ in Result._fields_ if k not in ("reserved", "pad")} for i in range(n)]

    def clock(self) -> float:
        return lib().jp_server_clock(self.h)

    def stats(self) -> dict:
        """Host seconds per phase (summed over threads) and event counts (jp_server_get_stats)."""
        st = ServerStats()
        _check(lib().jp_server_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_ if k != "reserved"}

    def close(self) -> None:
        if self.h:
            lib().jp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
