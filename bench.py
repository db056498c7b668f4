"""Benchmark: uniform D3Q19 BGK Taylor-Green vortex at N=512, Re=1600 (GLUPS and fraction of the HBM
roofline), FP32 storage as the headline with shifted FP16 and BF16 storage beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--n 512]

One JSON line on stdout (rank 0).  A "step" is one lattice time step over the whole N^3 cube.
  value   device throughput, populations resident in HBM (CUDA events on the solver's stream)
  e2e     the same metric through the C ABI with the state in pinned HOST memory: each e2e step
          copies the state in, advances `lattice_steps_per_call` steps and reads back the diagnostics
--impl reference times the CPU restatement of the reference's step (OpenMP, all host cores); the
reference itself has no CPU path.  With --gpus N > 1 (torchrun) every rank runs an independent
replica (the solve does not shard); the slowest rank's time counts.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "jp-solver_gb300"))

Q = 19
BYTES_PER_UPDATE = {"fp32": 152, "fp16": 76, "bf16": 76, "fp64": 304}
RE = 1600.0
U0 = 0.05


def dist_setup(ngpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return rank, local, world, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def load_traffic(key: str):
    """DRAM bytes per lattice update of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(key)


def bench_storage(J, n: int, storage: str, steps: int, warmup: int, device: int, pg, sampler=None) -> dict:
    s = J.Solver("uniform", n=n, re=RE, u0=U0, storage=storage, device=device)
    try:
        s.step(warmup)
        s.sync()
        barrier(pg)
        l0 = J.launch_count()
        if sampler:
            sampler.start()
        ms = s.step_timed(steps)
        clocks = sampler.stop() if sampler else None
        launches = J.launch_count() - l0
        barrier(pg)
        ms = max_over_ranks(pg, ms)
        d = s.diag()
    finally:
        s.close()
    cells = n ** 3
    per_launch_s = ms / 1e3 / steps
    return {"ms_per_step": ms / steps, "glups": cells * steps / (ms / 1e3) / 1e9, "launches": launches,
            "per_launch_s": per_launch_s, "clocks": clocks, "diag": d,
            "achieved_gbs": BYTES_PER_UPDATE[storage] * cells / per_launch_s / 1e9}


def bench_e2e(J, n: int, calls: int, k: int, device: int, pg) -> dict:
    """State in pinned host memory; per call: H2D of the state, k lattice steps, diagnostics D2H."""
    import ctypes as C

    s = J.Solver("uniform", n=n, re=RE, u0=U0, storage="fp32", device=device)
    buf = None
    try:
        cnt = s.population_count()
        buf = J.PinnedBuffer(cnt)
        L = J.lib()
        out = (C.c_double * 3)()
        # the initial state comes from the host like every later call's
        st = L.jp_get_populations(s.h, 0, 0, 0, C.c_void_p(buf.ptr.value), cnt)
        assert st == 0, L.jp_last_error()

        def one():
            assert L.jp_set_populations(s.h, 0, 0, 0, C.c_void_p(buf.ptr.value), cnt) == 0
            assert L.jp_step(s.h, k) == 0
            assert L.jp_diag(s.h, out) == 0

        one()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(calls):
            one()
        dt = time.perf_counter() - t0
        barrier(pg)
        dt = max_over_ranks(pg, dt)
    finally:
        if buf is not None:
            buf.free()
        s.close()
    return {"seconds": dt, "glups": n ** 3 * k * calls / dt / 1e9, "h2d_bytes": cnt * 4, "d2h_bytes": 24}


def cpu_baseline(n: int, steps: int) -> dict:
    """The oracle (CPU restatement of the reference's step, OpenMP) on this host's cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import oracle as O

    p = O.params(n, RE, U0)
    f = O.init_tgv(n, 8, U0)
    g = np.empty_like(f)
    O.orc().orc_step_f32(O._fp(f), O._fp(g), n, 8, p["omega"])  # warm
    t0 = time.perf_counter()
    O.orc().orc_run_f32(O._fp(f), O._fp(g), n, 8, p["omega"], steps)
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n ** 3 * steps / dt / 1e9, "unit": "GLUPS", "cores": cores, "kind": "port",
            "sample": "oracle FP32 step, N=%d cube, %d steps (%.1f s)" % (n, steps, dt)}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--no-variants", action="store_true", help="skip the FP16/BF16 lines")
    ap.add_argument("--e2e-calls", type=int, default=4)
    ap.add_argument("--cpu-steps", type=int, default=3)
    a = ap.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    rank, local, world, pg = dist_setup(a.gpus)
    n = a.n
    config = {"workload": "uniform TGV D3Q19 BGK, N=%d, Re=%g, u0=%g, periodic" % (n, RE, U0),
              "n": n, "re": RE, "storage": "fp32", "cells": n ** 3,
              "l2": "inputs larger than L2 (%.1f GB of populations per step)" % (2 * Q * 4 * n ** 3 / 1e9),
              "parallelism": "replicas x%d" % world}

    if a.impl == "reference":
        if rank != 0:
            return 0
        steps = max(1, min(a.steps, 5))
        cb = cpu_baseline(n, steps)
        line = {"metric": "GLUPS", "value": cb["value"], "unit": "GLUPS", "impl": "reference", "n_gpus": a.gpus,
                "steps": steps, "warmup": a.warmup, "ms_per_step": 1e3 * n ** 3 / (cb["value"] * 1e9),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (analytic Taylor-Green initial state)", "config": config,
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import jpsolver as J

    peaks = load_peaks()
    sampler = ClockSampler(local)
    main_r = bench_storage(J, n, "fp32", a.steps, a.warmup, local, pg, sampler)
    variants = {}
    if not a.no_variants:
        for st in ("fp16", "bf16"):
            r = bench_storage(J, n, st, a.steps, a.warmup, local, pg)
            variants[st] = {"glups": r["glups"], "ms_per_step": r["ms_per_step"],
                            "bytes_per_update": BYTES_PER_UPDATE[st],
                            "achieved_gbs": r["achieved_gbs"], "frac": r["achieved_gbs"] / peaks["hbm_gbs"],
                            "speedup_vs_fp32": r["glups"] / main_r["glups"]}
    k = max(1, int(O_diag_every(n)))
    e2e = bench_e2e(J, n, a.e2e_calls, k, local, pg)
    traffic = load_traffic("stream_collide_fp32")
    value = main_r["glups"] * world
    line = {
        "metric": "GLUPS", "value": value, "unit": "GLUPS", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": main_r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic Taylor-Green initial state)", "config": config,
        "roofline": {"bound": "hbm", "kernel": "k_stream_collide<fp32>", "achieved": main_r["achieved_gbs"],
                     "peak": peaks["hbm_gbs"], "peak_source": peaks["source"], "unit": "GB/s",
                     "frac": main_r["achieved_gbs"] / peaks["hbm_gbs"],
                     "bytes_per_update": BYTES_PER_UPDATE["fp32"],
                     "traffic": (traffic * n ** 3) if traffic else None},
        "variants": variants,
        "e2e": {"value": e2e["glups"] * world, "unit": "GLUPS", "h2d_bytes_per_step": e2e["h2d_bytes"],
                "d2h_bytes_per_step": e2e["d2h_bytes"], "lattice_steps_per_call": k,
                "calls": a.e2e_calls},
        "gpu_launches": main_r["launches"],
        "clocks": main_r["clocks"],
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(n, a.cpu_steps)
    if rank == 0:
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()
    return 0


def O_diag_every(n: int) -> int:
    """The reference's diagnostic cadence max(1, steps/240) (src/tgv3d_uniform.cu:163) at t*=12."""
    import math

    steps = int(12.0 / (U0 * 2 * math.pi / n) + 0.5)
    return max(1, steps // 240)


if __name__ == "__main__":
    sys.exit(main())
