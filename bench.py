"""Benchmark: uniform D3Q19 BGK Taylor-Green vortex at N=512, Re=1600 (GLUPS and fraction of the HBM
roofline), FP32 storage as the headline with shifted FP16 and BF16 storage beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--n 512]

One JSON line on stdout (rank 0).  A "step" is one lattice time step over the whole N^3 cube.
  value   device throughput, populations resident in HBM (CUDA events on the solver's stream)
  e2e     the same metric through the C ABI with the state in pinned HOST memory: each e2e step
          copies the state in, advances `lattice_steps_per_call` steps and reads back the diagnostics
          (each copy staged on a copy stream while the previous call's steps run)
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


def bench_storage(J, n: int, storage: str, steps: int, warmup: int, device: int, pg, sampler=None, vec: int = 0,
                  tpb: int = 0, flags: int = 0) -> dict:
    s = J.Solver("uniform", n=n, re=RE, u0=U0, storage=storage, device=device, vec=vec, threads_per_block=tpb,
                 flags=flags)
    try:
        bytes_state = s.info["bytes_state"]
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
        diag_s = []
        for _ in range(3):  # one diagnostic (populations -> energy, enstrophy, mass; read-back), host clock
            t0 = time.perf_counter()
            s.diag()
            diag_s.append(time.perf_counter() - t0)
    finally:
        s.close()
    cells = n ** 3
    per_launch_s = ms / 1e3 / steps
    return {"ms_per_step": ms / steps, "glups": cells * steps / (ms / 1e3) / 1e9, "launches": launches,
            "per_launch_s": per_launch_s, "clocks": clocks, "diag": d, "diag_ms": 1e3 * min(diag_s),
            "bytes_state": bytes_state,
            "achieved_gbs": BYTES_PER_UPDATE[storage] * cells / per_launch_s / 1e9}


def bench_amr(J, device: int, steps: int = 20) -> dict:
    """The AMR static gold case (coarse N=64, both levels refined everywhere, finest 256^3, MB=8,
    Re=800, graph replay of the 1:2:4 coarse step): work-normalised GLUPS of the timed coarse steps,
    work = (cnb0 + 2 nf1 + 4 nf2) MB^3 per coarse step as the reference counts it, against the FP32
    (152 B) and FP16 (76 B) per-update roofline, in both storages."""
    peaks = load_peaks()
    out = {"workload": "AMR static gold: N0=64, --l1 all --l2 all, MB=8, Re=800, CUDA-graph step",
           "work_per_coarse_step": None}
    for st in ("fp32", "fp16"):
        s = J.Solver("amr", n=64, re=800.0, u0=U0, l1_mode="all", l2_mode="all", storage=st, device=device,
                     flags=J.FLAG_GRAPH)
        try:
            c = s.counts()
            work = (c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512
            s.step(4)
            s.sync()
            ms = s.step_timed(steps)
        finally:
            s.close()
        glups = work * steps / (ms / 1e3) / 1e9
        gbs = glups * BYTES_PER_UPDATE[st]
        out["work_per_coarse_step"] = work
        out[st] = {"glups_work": glups, "ms_per_coarse_step": ms / steps, "achieved_gbs": gbs,
                   "frac_of_fp32_roofline": glups * 152.0 / peaks["hbm_gbs"], "frac_of_own_roofline": gbs / peaks["hbm_gbs"]}
    out["dynamic"] = bench_amr_dynamic(J, device)
    return out


def bench_amr_dynamic(J, device: int, steps: int = 200) -> dict:
    """The dynamic AMR case (coarse N=96, sensor refinement on both levels, frac1 0.3, frac2 0.1,
    Re=1600, MB=8, a regrid every 20 coarse steps in the warm-up): graph replay of the coarse step,
    timed without regrids as the reference's bench mode does, work-normalised as above."""
    peaks = load_peaks()
    out = {"workload": "AMR dynamic: N0=96, --l1 sensor --l2 sensor, frac1 0.3, frac2 0.1, MB=8, Re=1600, "
                       "CUDA-graph step"}
    for st in ("fp32", "fp16"):
        s = J.Solver("amr", n=96, re=1600.0, u0=U0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.1,
                     adapt_every=20, storage=st, device=device, flags=J.FLAG_GRAPH)
        try:
            for w in range(20):
                if w % 20 == 0:
                    s.regrid()
                s.step(1)
            s.sync()
            c = s.counts()
            work = (c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512
            ms = s.step_timed(steps)
        finally:
            s.close()
        glups = work * steps / (ms / 1e3) / 1e9
        out[st] = {"glups_work": glups, "ms_per_coarse_step": ms / steps, "work_per_coarse_step": work,
                   "frac_of_fp32_roofline": glups * 152.0 / peaks["hbm_gbs"],
                   "frac_of_own_roofline": glups * BYTES_PER_UPDATE[st] / peaks["hbm_gbs"]}
    return out


def bench_e2e(J, n: int, calls: int, k: int, device: int, pg) -> dict:
    """State in pinned host memory; per call: H2D of the call's input state, k lattice steps,
    diagnostics D2H.  The input of call i+1 is staged (jp_stage_populations: a copy stream into a
    second state buffer) right after call i's steps are queued, so the upload overlaps those steps;
    every timed call's upload is inside the timed region (the first is issued after the clock
    starts) and the next jp_step waits for it on the device."""
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

        def stage():
            assert L.jp_stage_populations(s.h, 0, 0, C.c_void_p(buf.ptr.value), cnt) == 0, L.jp_last_error()

        def one(stage_next):
            assert L.jp_step(s.h, k) == 0          # takes the state staged for this call
            if stage_next:
                stage()                            # the next call's input, during these steps
            assert L.jp_diag(s.h, out) == 0

        stage()
        one(False)
        barrier(pg)
        t0 = time.perf_counter()
        stage()
        for i in range(calls):
            one(i + 1 < calls)
        dt = time.perf_counter() - t0
        barrier(pg)
        dt = max_over_ranks(pg, dt)
        # the machine's host-to-device rate for one call's state, outside the timed region: the one
        # upload that no steps hide (the first call's) costs bytes / this rate
        assert L.jp_sync(s.h) == 0
        t1 = time.perf_counter()
        assert L.jp_set_populations(s.h, 0, 0, 0, C.c_void_p(buf.ptr.value), cnt) == 0, L.jp_last_error()
        assert L.jp_sync(s.h) == 0
        h2d_s = time.perf_counter() - t1
    finally:
        if buf is not None:
            buf.free()
        s.close()
    return {"seconds": dt, "glups": n ** 3 * k * calls / dt / 1e9, "h2d_bytes": cnt * 4, "d2h_bytes": 24,
            "h2d_gbs": cnt * 4 / h2d_s / 1e9}


def c5_requests(J, n_req: int, rate: float, seed: int) -> list:
    """The served-ensemble workload: Poisson(rate) arrivals from a seed; each request a uniform solve
    with N in {32,48,64,96,128} or an AMR solve with coarse N in {16,24,32,48} (sensor refinement on
    both levels, frac1 0.3, frac2 0.1, regrid every 20 coarse steps, graph replay); Re log-uniform in
    [200, 3200]; t* uniform in [2, 10]; FP32 or FP16 storage 50/50."""
    import numpy as np

    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_req))
    out = []
    for i in range(n_req):
        amr = bool(rng.random() < 0.5)
        n = int(rng.choice([16, 24, 32, 48] if amr else [32, 48, 64, 96, 128]))
        re = float(np.exp(rng.uniform(np.log(200.0), np.log(3200.0))))
        ts = float(rng.uniform(2.0, 10.0))
        half = bool(rng.random() < 0.5)
        r = dict(rid=i, kind="amr" if amr else "uniform", n=n, re=re, tstar=ts, storage="fp16" if half else "fp32")
        if amr:
            r.update(l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.1, adapt_every=20, flags=J.FLAG_GRAPH)
        out.append((float(t[i]), r))
    return out


def serve_run(J, reqs: list, device: int, open_loop: bool, max_active: int = 0, tick: int = 64,
              workers: int = 0) -> dict:
    """Drive the server: open loop submits each request at its arrival time, closed loop submits all
    at once.  Returns throughput and latency percentiles (submit to result)."""
    import numpy as np

    sv = J.Server(device=device, pool_gb=120.0, max_active=max_active, tick_steps=tick, workers=workers)
    t0 = time.perf_counter()
    i, res = 0, {}
    if not open_loop:
        for _, r in reqs:
            sv.submit(**r)
        i = len(reqs)
    while len(res) < len(reqs):
        now = time.perf_counter() - t0
        while i < len(reqs) and reqs[i][0] <= now:
            sv.submit(**reqs[i][1])
            i += 1
        a, q = sv.tick()
        for r in sv.poll(1024):
            res[r["id"]] = r
        if a == 0 and q == 0 and i < len(reqs):
            time.sleep(min(0.002, max(0.0, reqs[i][0] - (time.perf_counter() - t0))))
    span = time.perf_counter() - t0
    stats = sv.stats()
    sv.close()
    lat = np.array([r["t_end"] - r["t_submit"] for r in res.values()])
    ok = sum(1 for r in res.values() if r["status"] == 0)
    return {"solves": len(res), "ok": ok, "seconds": span, "solves_per_s": len(res) / span,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "valid": sum(1 for r in res.values() if r["valid"]),
            "host_seconds": {k: round(v, 3) for k, v in stats.items() if k.endswith("_s")},
            "events": {k: v for k, v in stats.items() if not k.endswith("_s")}}


def program_args(J, r: dict, device: int) -> list:
    """The drop-in program and flags that run request r as a solve of its own."""
    prog = os.path.join(ROOT, "jp-solver_gb300", "bin", "amr" if r["kind"] == "amr" else "uniform")
    a = [prog, "--n", str(r["n"]), "--re", repr(r["re"]), "--tstar", repr(r["tstar"]), "--prec", r["storage"],
         "--device", str(device)]
    if r["kind"] == "amr":
        a += ["--l1", r["l1_mode"], "--l2", r["l2_mode"], "--frac1", repr(r["frac1"]), "--frac2", repr(r["frac2"]),
              "--adapt", str(r["adapt_every"]), "--graph", "1" if r.get("flags", 0) & J.FLAG_GRAPH else "0"]
    return a


def programs_one_at_a_time(J, reqs: list, device: int) -> dict:
    """The reference's way to run an ensemble: one program per solve, one after another (here the
    drop-in programs, each a process with its own CUDA context)."""
    import subprocess

    t0 = time.perf_counter()
    codes = [subprocess.run(program_args(J, r, device), stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode
             for _, r in reqs]
    span = time.perf_counter() - t0
    return {"solves": len(reqs), "seconds": span, "solves_per_s": len(reqs) / span,
            "exit_codes": {str(c): codes.count(c) for c in sorted(set(codes))}}


def bench_serve(J, args, device: int) -> dict:
    reqs = c5_requests(J, args.requests, args.rate, args.seed)
    open_r = serve_run(J, reqs, device, open_loop=True)
    m = min(args.compare, len(reqs))
    sample = reqs[:m]
    batched = serve_run(J, sample, device, open_loop=False)
    single = serve_run(J, sample, device, open_loop=False, max_active=1)
    closed = {"sample": m, "batched_solves_per_s": batched["solves_per_s"],
              "one_at_a_time_solves_per_s": single["solves_per_s"],
              "speedup": batched["solves_per_s"] / single["solves_per_s"]}
    if args.programs:
        pr = programs_one_at_a_time(J, sample, device)
        closed["programs_one_at_a_time"] = pr
        closed["speedup_vs_programs"] = batched["solves_per_s"] / pr["solves_per_s"]
    return {"open_loop": open_r, "closed_loop": closed}


def precision_run(J, n: int, storage: str, every: int, device: int, tstar: float = 12.0) -> dict:
    """One full TGV run (Re=1600) with diagnostics every `every` steps: the energy and enstrophy
    histories, the enstrophy peak time and the mass drift."""
    import numpy as np

    with J.Solver("uniform", n=n, re=RE, u0=U0, tstar=tstar, storage=storage, device=device) as s:
        info = s.info
        steps, kf = info["steps"], info["kf"]
        ts, E, Z, M = [], [], [], []
        t0 = time.perf_counter()
        for k in range(0, steps + 1, every):
            e, z, m = s.diag()
            ts.append(k * U0 * kf)
            E.append(e)
            Z.append(z)
            M.append(m)
            if k + every <= steps:
                s.step(every)
        wall = time.perf_counter() - t0
    E, Z, M = np.array(E), np.array(Z), np.array(M)
    i = int(np.argmax(Z))
    return {"storage": storage, "n": n, "steps": steps, "seconds": wall, "t": np.array(ts), "E": E / E[0], "Z": Z,
            "peak_tstar": float(ts[i]), "peak_enstrophy": float(Z[i]),
            "mass_drift": float(np.max(np.abs(M - M[0]) / M[0])), "energy_monotonic": bool(np.all(np.diff(E) <= 0))}


def bench_precision(J, args, device: int) -> dict:
    """Storage precision study: FP32, shifted FP16 and BF16 storage against an FP64 run at the same N
    (256 by default), Re=1600, t*=12; errors of the enstrophy peak time, the energy curve and the
    enstrophy curve relative to FP64."""
    import numpy as np

    n, every = args.n or 256, args.every
    ref = precision_run(J, n, "fp64", every, device)
    out = {"n": n, "every_steps": every, "dt_star_per_sample": float(ref["t"][1] - ref["t"][0]),
           "fp64": {k: ref[k] for k in ("peak_tstar", "peak_enstrophy", "mass_drift", "energy_monotonic", "seconds")}}
    for st in ("fp32", "fp16", "bf16"):
        r = precision_run(J, n, st, every, device)
        out[st] = {k: r[k] for k in ("peak_tstar", "peak_enstrophy", "mass_drift", "energy_monotonic", "seconds")}
        out[st]["peak_tstar_error"] = r["peak_tstar"] - ref["peak_tstar"]
        out[st]["energy_max_rel_error"] = float(np.max(np.abs(r["E"] - ref["E"]) / ref["E"]))
        out[st]["enstrophy_max_rel_error"] = float(np.max(np.abs(r["Z"] - ref["Z"]) / ref["Z"]))
    return out


def precision_summary(J, device: int, every: int) -> dict:
    """The storage precision figures of the headline line: the Re=1600, t*=12 run at N=256 in FP64,
    FP32, shifted FP16 and shifted BF16 storage, each with its enstrophy-peak time error against the
    FP64 run (bar for FP16: 0.05 t*), its largest energy-curve error and its mass drift."""
    class Args:
        pass

    args = Args()
    args.n, args.every = 256, every
    pr = bench_precision(J, args, device)
    out = {"n": 256, "re": RE, "tstar": 12.0, "every_steps": every, "dt_star_per_sample": pr["dt_star_per_sample"],
           "fp64": {"peak_tstar": pr["fp64"]["peak_tstar"], "mass_drift": pr["fp64"]["mass_drift"],
                    "seconds": pr["fp64"]["seconds"]}}
    for st in ("fp32", "fp16", "bf16"):
        out[st] = {k: pr[st][k] for k in ("peak_tstar", "peak_tstar_error", "energy_max_rel_error",
                                          "enstrophy_max_rel_error", "mass_drift", "energy_monotonic")}
    return out


ENSEMBLE_SHAPES = {  # AMR ensembles of the served-ensemble shapes: (coarse N, count), sensor/sensor, 0.3/0.1
    "served": [(16, 8), (24, 16), (32, 16), (48, 4)],
    "n16x8": [(16, 8)],
    "n24_32x32": [(24, 16), (32, 16)],
    "n48x4": [(48, 4)],
    "n96x1": [(96, 1)],
}


def bench_ensemble(J, shape: str, calls: int, k: int, device: int) -> dict:
    """Coarse steps of an AMR ensemble (seeded sensor grids, FP32, MB=8) with one launch per stage
    (per-stage) against one persistent launch per call of k coarse steps: device time per coarse step
    of all members (host clock around the timed calls, synchronised at both ends) and GLUPS(work)."""
    import numpy as np

    out = {"shape": shape, "members": [list(x) for x in ENSEMBLE_SHAPES[shape]], "calls": calls,
           "coarse_steps_per_call": k}
    for mode, name in ((0, "per_stage"), (1, "persistent")):
        solvers = []
        seed = 0
        for n0, cnt in ENSEMBLE_SHAPES[shape]:
            for _ in range(cnt):
                rng = np.random.default_rng(seed)
                seed += 1
                cgx = n0 // 8
                s0 = rng.random(cgx ** 3, dtype=np.float32)
                s1 = rng.random((2 * cgx) ** 3, dtype=np.float32)
                s = J.Solver("amr", n=n0, re=1600.0, u0=U0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.1,
                             develop_steps=2, max_gb=64.0, device=device, flags=J.FLAG_DEFER_INIT)
                s.set_sensor_override(s0, s1)
                s.init_tgv()
                solvers.append(s)
        ens = J.Ensemble(device)
        try:
            ens.set_persistent(mode)
            for s in solvers:
                ens.add(s)
            ens.step(2)
            ens.sync()
            l0 = J.launch_count()
            t0 = time.perf_counter()
            for _ in range(calls):
                ens.step(k)
            ens.sync()
            dt = time.perf_counter() - t0
            launches = J.launch_count() - l0
            work = sum((c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512 for c in (s.counts() for s in solvers))
        finally:
            ens.close()
            for s in solvers:
                s.close()
        steps = calls * k
        out[name] = {"us_per_coarse_step": dt / steps * 1e6, "glups_work": work * steps / dt / 1e9,
                     "launches_per_coarse_step": launches / steps, "work_per_coarse_step": work}
    out["speedup"] = out["per_stage"]["us_per_coarse_step"] / out["persistent"]["us_per_coarse_step"]
    return out


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
            "nproc": os.cpu_count(), "cpu_model": cpu_model(),
            "sample": "oracle FP32 step, N=%d cube, %d steps (%.1f s)" % (n, steps, dt)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu), read at run time."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = dict(ln.split(":", 1) for ln in out.splitlines() if ":" in ln)
        name = fields.get("Model name", "").strip()
        vendor = fields.get("Vendor ID", "").strip()
        if name:
            return (vendor + " " + name).strip()
    except (OSError, subprocess.SubprocessError, ValueError):
        pass
    import platform

    return platform.machine() + " " + (platform.processor() or "unknown")


def reference_gpu(n: int, steps: int) -> dict:
    """The reference's own CUDA kernels (compiled from its checkout into oracle/_ref/*.cubin) rerun on
    this GPU, timed with CUDA events: the uniform k_step at N=n (src/tgv3d_uniform.cu:41-61) and the
    AMR base_step launch sequence (src/tgv3d_amr.cu:821-837) on the static gold case (N0=64 all/all,
    Re=800) and on the dynamic case (N0=96 sensor/sensor, frac1 0.3, frac2 0.1, Re=1600, after the
    300 develop steps; no regrid timed), work-normalised as the reference's --bench counts it."""
    import ctypes as C

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if not O.ref_amr_available():
        return {"unavailable": "reference cubins not built (no reference checkout where build() ran)"}
    p = O.params(n, RE, U0)
    ms = O.ref_time(n, p["omega"], 3, steps, U0)
    out = {"uniform": {"n": n, "kernel": "k_step (reference, MB=8)", "glups": n ** 3 * steps / (ms / 1e3) / 1e9,
                       "ms_per_step": ms / steps, "steps": steps}}
    cases = {"amr_static_gold": (64, 800.0, "all", "all", 0.35, 0.35),
             "amr_dynamic": (96, 1600.0, "sensor", "sensor", 0.3, 0.1)}
    for key, (n0, re, l1, l2, f1, f2) in cases.items():
        b = O.AmrBackend("reference", n0, re, l1, l2, f1, f2, u0=U0, budget=float(1 << 40))
        try:
            c = b.counts()
            work = (c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512
            t = C.c_float()
            k = 10 if key == "amr_static_gold" else 100
            rc = O.ref_amr().ref_amr_time(C.c_void_p(b.h), 2, k, C.byref(t))
            if rc:
                raise RuntimeError(O.ref().refrun_last_error().decode())
        finally:
            b.close()
        out[key] = {"n0": n0, "glups_work": work * k / (t.value / 1e3) / 1e9, "ms_per_coarse_step": t.value / k,
                    "work_per_coarse_step": work, "coarse_steps": k}
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=None, help="cube edge (default 512; the precision study 256)")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP16/BF16 lines")
    ap.add_argument("--no-amr", action="store_true", help="skip the AMR static gold line")
    ap.add_argument("--e2e-calls", type=int, default=4)
    ap.add_argument("--cpu-steps", type=int, default=3, help="0 skips the CPU baseline")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16", "bf16", "fp64"],
                    help="storage of the timed run (the headline is fp32)")
    ap.add_argument("--vec", type=int, default=0)
    ap.add_argument("--tpb", type=int, default=0)
    ap.add_argument("--workload", default="uniform", choices=["uniform", "serve", "precision", "ensemble"])
    ap.add_argument("--shape", default="served", choices=list(ENSEMBLE_SHAPES),
                    help="ensemble: the AMR members (coarse N x count)")
    ap.add_argument("--every", type=int, default=10, help="precision study: steps between diagnostics")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the storage precision study (FP16/BF16 against FP64 at N=256) in the headline line")
    ap.add_argument("--reference-gpu", type=int, default=1,
                    help="--impl reference: also time the reference's own CUDA kernels on this GPU (0: skip)")
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--compare", type=int, default=200, help="requests in the batched vs one-at-a-time comparison")
    ap.add_argument("--programs", type=int, default=1,
                    help="serve: also time the comparison sample as one drop-in program per solve (0: skip)")
    a = ap.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    if a.workload == "serve":  # concurrent AMR solves: one hardware queue per stream (before any CUDA call)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    rank, local, world, pg = dist_setup(a.gpus)
    n = a.n or 512
    config = {"workload": "uniform TGV D3Q19 BGK, N=%d, Re=%g, u0=%g, periodic" % (n, RE, U0),
              "n": n, "re": RE, "storage": a.storage, "cells": n ** 3,
              "l2": "inputs larger than L2 (%.1f GB of populations per step)" % (2 * Q * 4 * n ** 3 / 1e9),
              "parallelism": "replicas x%d" % world}

    if a.impl == "reference":
        if rank != 0:
            return 0
        steps = max(1, min(a.steps, 5))
        cb = cpu_baseline(n, steps)
        rg = None
        if a.reference_gpu:
            try:
                rg = reference_gpu(n, 20)
            except Exception as exc:  # the CPU arm's line is still printed
                rg = {"unavailable": "reference kernels failed: %s" % exc}
        line = {"metric": "GLUPS", "value": cb["value"], "unit": "GLUPS", "impl": "reference", "n_gpus": a.gpus,
                "steps": steps, "warmup": a.warmup, "ms_per_step": 1e3 * n ** 3 / (cb["value"] * 1e9),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (analytic Taylor-Green initial state)", "config": config,
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "GLUPS", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        if rg is not None:
            line["reference_gpu"] = rg
        print(json.dumps(line))
        return 0

    import jpsolver as J

    if a.workload == "precision":
        pr = bench_precision(J, a, local)
        line = {"metric": "enstrophy-peak t* error vs FP64 storage", "value": pr["fp16"]["peak_tstar_error"],
                "unit": "t*", "n_gpus": world, "steps": pr["fp64"]["seconds"], "warmup": 0, "ms_per_step": None,
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (analytic Taylor-Green initial state)",
                "config": {"workload": "uniform TGV N=%d Re=%g t*=12, FP64/FP32/FP16/BF16 storage" % (pr["n"], RE)},
                "precision": pr}
        if rank == 0:
            print(json.dumps(line))
        return 0

    if a.workload == "ensemble":
        en = bench_ensemble(J, a.shape, max(1, a.steps // 8), 8, local)
        line = {"metric": "AMR ensemble GLUPS(work)", "value": en["persistent"]["glups_work"], "unit": "GLUPS(work)",
                "n_gpus": world, "steps": max(1, a.steps // 8) * 8, "warmup": 2,
                "ms_per_step": en["persistent"]["us_per_coarse_step"] / 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded sensor grids of Taylor-Green solves)",
                "config": {"workload": "AMR ensemble %s, sensor/sensor 0.3/0.1, FP32, MB=8" % a.shape},
                "ensemble": en}
        if rank == 0:
            print(json.dumps(line))
        return 0

    if a.workload == "serve":
        sv = bench_serve(J, a, local)
        o = sv["open_loop"]
        line = {"metric": "ensemble solves/s", "value": o["solves_per_s"], "unit": "solves/s", "n_gpus": world,
                "steps": o["solves"], "warmup": 0, "ms_per_step": 1e3 / o["solves_per_s"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded Poisson requests of Taylor-Green solves)",
                "config": {"workload": "served TGV ensemble: %d requests, Poisson %.0f/s, seed %d, 120 GB pool"
                                       % (a.requests, a.rate, a.seed)},
                "serving": sv, "p50_latency_s": o["p50_s"], "p99_latency_s": o["p99_s"]}
        if rank == 0:
            print(json.dumps(line))
        return 0

    peaks = load_peaks()
    sampler = ClockSampler(local)
    main_r = bench_storage(J, n, a.storage, a.steps, a.warmup, local, pg, sampler, a.vec, a.tpb)
    variants = {}
    if not a.no_variants:
        for st in ("fp16", "bf16"):
            r = bench_storage(J, n, st, a.steps, a.warmup, local, pg)
            variants[st] = {"glups": r["glups"], "ms_per_step": r["ms_per_step"],
                            "bytes_per_update": BYTES_PER_UPDATE[st],
                            "achieved_gbs": r["achieved_gbs"], "frac": r["achieved_gbs"] / peaks["hbm_gbs"],
                            "speedup_vs_fp32": r["glups"] / main_r["glups"]}
        # in-place (AA) streaming: one population array, the same bytes per update
        for st in ("fp32", "fp16"):
            r = bench_storage(J, n, st, a.steps, a.warmup, local, pg, flags=J.FLAG_INPLACE)
            variants[st + "_inplace"] = {"glups": r["glups"], "ms_per_step": r["ms_per_step"],
                                         "bytes_per_update": BYTES_PER_UPDATE[st], "bytes_state": r["bytes_state"],
                                         "achieved_gbs": r["achieved_gbs"], "frac": r["achieved_gbs"] / peaks["hbm_gbs"]}
    k = max(1, int(O_diag_every(n)))
    e2e = bench_e2e(J, n, a.e2e_calls, k, local, pg) if a.e2e_calls > 0 else None
    traffic = load_traffic("stream_collide_" + a.storage)
    value = main_r["glups"] * world
    line = {
        "metric": "GLUPS", "value": value, "unit": "GLUPS", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": main_r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic Taylor-Green initial state)", "config": config,
        "roofline": {"bound": "hbm", "kernel": "k_stream_collide<%s>" % a.storage, "achieved": main_r["achieved_gbs"],
                     "peak": peaks["hbm_gbs"], "peak_source": peaks["source"], "unit": "GB/s",
                     "frac": main_r["achieved_gbs"] / peaks["hbm_gbs"],
                     "bytes_per_update": BYTES_PER_UPDATE[a.storage],
                     "traffic": (traffic * n ** 3) if traffic else None},
        "variants": variants,
        "e2e": ({"value": e2e["glups"] * world, "unit": "GLUPS", "h2d_bytes_per_step": e2e["h2d_bytes"] // k,
                 "d2h_bytes_per_step": e2e["d2h_bytes"] / k, "h2d_bytes_per_call": e2e["h2d_bytes"],
                 "d2h_bytes_per_call": e2e["d2h_bytes"], "lattice_steps_per_call": k,
                 "calls": a.e2e_calls, "h2d_gbs": e2e["h2d_gbs"],
                 "overlap": "each call's H2D staged on a copy stream during the previous call's steps"}
                if e2e else None),
        "gpu_launches": main_r["launches"],
        "clocks": main_r["clocks"],
        "diagnostic": {"ms": main_r["diag_ms"], "step_equivalents": main_r["diag_ms"] / main_r["ms_per_step"],
                       "what": "one jp_diag (energy, enstrophy, mass straight from the populations: k_diag_pop + "
                               "k_diag_finish, read-back), host clock, best of 3",
                       "bytes": BYTES_PER_UPDATE[a.storage] // 2 * n ** 3,
                       "achieved_gbs": BYTES_PER_UPDATE[a.storage] // 2 * n ** 3 / (main_r["diag_ms"] * 1e-3) / 1e9},
    }
    if not a.no_amr and rank == 0:
        line["amr"] = bench_amr(J, local)
    if not a.no_precision and rank == 0:
        line["precision"] = precision_summary(J, local, a.every)
    if rank == 0 and world == 1 and a.cpu_steps > 0:
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
