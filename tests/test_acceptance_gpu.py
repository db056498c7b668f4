"""Physics acceptance of whole runs against the reference's own CUDA kernels (compiled from its
checkout into oracle/_ref/*.cubin and driven in its launch order by oracle/refrun.cpp) on the same GPU.

The reference states its gold tolerances in docs/validation.md:11-13 and README.md:114-115:
enstrophy-peak time within 0.3 t*, energy curve within 2 %, mass drift below 1e-4, energy strictly
decreasing.  Here the engine and the reference run the same configuration from the same analytic
state, each with its own kernels, and their curves are held to bars far tighter than those (stated
per test); the gold criteria are checked on both sides as well.

  C1  uniform N=64, Re=400, 2000 steps, diagnostics every 50 steps
  C3  AMR static gold: coarse N=64, --l1 all --l2 all, Re=800, t*=12, against uniform N=256
  C4  AMR dynamic: coarse N=96, --l1 sensor --l2 sensor, frac1 0.3, frac2 0.1, Re=1600, regrid
      every 20 coarse steps: tables bit-exact at each regrid when the reference is fed the engine's
      sensor, populations within 1e-5 relative per coarse step from a shared state, and the whole
      t*=20 run of both sides on the same grids against the dynamic gold criteria
  N=256 one FP32 step from the reference's state against the reference's k_step
  N=512 the same at the benchmark size (10.2 GB of state; skipped where the host or the GPU lacks the
        memory for two copies on each)
"""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_amr_available(), reason="reference cubins / librefrun.so not built")]
U0 = 0.05
BUDGET = 1024.0 * 2 ** 30
TABLES = ["ref0", "fof0", "rl0", "l1pcb", "l1oct", "f1pos", "l1grid", "ref1", "fof1", "rl1", "l2pl1", "l2oct",
          "skin0", "skin1", "deep"]
COUNTS = ["nref0", "nf1", "nref1", "nf2", "n_skin0", "n_skin1", "cap1", "cap2", "cap_nref0", "cap_nref1"]


def rel_err(a, b):
    if a.size == 0 and b.size == 0:
        return 0.0
    worst = 0.0
    for i in range(0, a.size, 1 << 26):       # chunks keep the FP64 temporaries small at N=256
        x = a[i:i + (1 << 26)].astype(np.float64)
        y = b[i:i + (1 << 26)].astype(np.float64)
        worst = max(worst, float(np.max(np.abs(x - y) / np.abs(y))))
    return worst


class Curve:
    """Diagnostic samples of one run: t*, E/E0, enstrophy, mass; with the program's summary figures
    (src/tgv3d_uniform.cu:179-199, src/tgv3d_amr.cu:883-903)."""

    def __init__(self, rows):
        a = np.array(rows, dtype=np.float64)
        self.t, E, self.Z, M = a[:, 0], a[:, 1], a[:, 2], a[:, 3]
        self.E = E / E[0]
        i = int(np.argmax(self.Z))
        self.peak_t, self.peak_z = float(self.t[i]), float(self.Z[i])
        self.mass_drift = float(np.max(np.abs(M - M[0]) / M[0]))
        self.monotonic = bool(np.all(E[1:] <= E[:-1] * 1.0000001))

    def valid(self):
        """The programs' VALID gate."""
        return np.isfinite(self.peak_z) and 4.0 < self.peak_t < 10.0 and self.monotonic and self.mass_drift < 5e-4

    def energy_gap(self, other):
        """Largest relative gap of E/E0 against another curve, at this curve's sample times."""
        e = np.interp(self.t, other.t, other.E)
        return float(np.max(np.abs(self.E - e) / e))

    def enstrophy_gap(self, other):
        z = np.interp(self.t, other.t, other.Z)
        return float(np.max(np.abs(self.Z - z) / np.max(other.Z)))


# ---- C1: uniform N=64, Re=400, 2000 steps ---------------------------------------------------------

def engine_uniform_curve(n, re, tstar, every, storage="fp32"):
    with J.Solver("uniform", n=n, re=re, u0=U0, tstar=tstar, storage=storage) as s:
        steps, kf = s.info["steps"], s.info["kf"]
        rows = []
        for k in range(0, steps + 1, every):
            rows.append((k * U0 * kf,) + s.diag())
            if k + every <= steps:
                s.step(every)
    return steps, Curve(rows)


def reference_uniform_curve(n, re, tstar, every):
    """The reference's k_init_tgv3d and k_step on the GPU; each sample is its k_macro field reduced
    as its host loop does (src/tgv3d_uniform.cu:168-189, restated by the oracle)."""
    p = O.params(n, re, U0, tstar)
    f = O.ref_init(n, U0)
    rows = []
    for k in range(0, p["steps"] + 1, every):
        rows.append((k * U0 * p["kf"],) + O.diag_field(O.ref_macro(f, n), n))
        if k + every <= p["steps"]:
            f = O.ref_run(f, n, p["omega"], every)
    return p["steps"], Curve(rows)


def test_c1_uniform_run_matches_reference_build():
    # The reference's FP32 collision lets mass drift (5.9e-5 over these 2000 steps, measured) while
    # the engine's, which relaxes the shifts f - w_q, holds it (2e-8); at fixed momentum E scales as
    # 1/rho^2, so the E/E0 curves part by about twice the reference's drift (1.0e-4 measured).  Bars:
    # E/E0 within 5e-4 relative and enstrophy within 1e-3 of its peak at every sample, the same peak
    # sample, mass drift below 1e-6 (engine) and the reference's own gate 5e-4 (gold: 2 %, 0.3 t*, 1e-4)
    n, re, tstar, every = 64, 400.0, 9.8175, 50
    se, e = engine_uniform_curve(n, re, tstar, every)
    sr, r = reference_uniform_curve(n, re, tstar, every)
    assert se == sr == 2000 and len(e.t) == len(r.t) == 41
    de, dz = e.energy_gap(r), e.enstrophy_gap(r)
    print("\nC1 N=64 Re=400 2000 steps: engine peak t*=%.4f drift %.2e, reference peak t*=%.4f drift %.2e; "
          "max E/E0 gap %.2e, enstrophy gap %.2e of peak" % (e.peak_t, e.mass_drift, r.peak_t, r.mass_drift, de, dz))
    assert de < 5e-4
    assert dz < 1e-3
    assert e.peak_t == r.peak_t
    assert e.mass_drift < 1e-6 and r.mass_drift < 5e-4
    assert e.valid() and e.monotonic and r.monotonic


# ---- C3: AMR static gold ----------------------------------------------------------------------------

def next_event(k, steps, every, adapt, dynamic):
    """The next coarse step at which the amr program samples, regrids or ends."""
    nxt = min(steps, k + every - k % every)
    if dynamic:
        nxt = min(nxt, k + adapt - k % adapt)
    return nxt


def amr_loop_rows(side, steps, kf, adapt, dynamic):
    """The amr program's loop (src/tgv3d_amr.cu:880-891): a regrid at every positive multiple of
    `adapt` coarse steps on a sensor grid, diagnostics every max(1, steps/160) coarse steps; the steps
    between two events go in one call.  Rows (t*, diagnostics...)."""
    every = max(1, steps // 160)
    rows, k = [], 0
    while True:
        if dynamic and k > 0 and k % adapt == 0:
            side.regrid()
        if k % every == 0:
            rows.append((k * U0 * kf,) + tuple(side.diag()))
        if k == steps:
            return rows
        nxt = next_event(k, steps, every, adapt, dynamic)
        side.step(nxt - k)
        k = nxt


def amr_loop(side, steps, kf, adapt, dynamic):
    return Curve(amr_loop_rows(side, steps, kf, adapt, dynamic))


def engine_amr_curve(n, re, tstar, l1="all", l2="all", frac1=0.35, frac2=0.35, adapt=100, storage="fp32", flags=0):
    """The engine through the C ABI."""
    with J.Solver("amr", n=n, re=re, u0=U0, tstar=tstar, l1_mode=l1, l2_mode=l2, frac1=frac1, frac2=frac2,
                  adapt_every=adapt, storage=storage, max_gb=1024.0, flags=flags) as s:
        steps = s.info["steps"]
        return steps, amr_loop(s, steps, s.info["kf"], adapt, "sensor" in (l1, l2))


def reference_amr_curve(n, re, tstar, l1="all", l2="all", frac1=0.35, frac2=0.35, adapt=100):
    """The reference's AMR kernels in its launch order (initial build, base_step, gpurce_regrid,
    k_composite + k_diag_reduce) over the same loop."""
    p = O.params(n, re, U0, tstar)
    b = O.AmrBackend("reference", n, re, l1, l2, frac1, frac2, u0=U0, tstar=tstar, budget=BUDGET)
    try:
        return p["steps"], amr_loop(b, p["steps"], p["kf"], adapt, "sensor" in (l1, l2))
    finally:
        b.close()


def test_c3_static_gold_against_uniform_4n_and_reference_build():
    # The gold criterion (docs/validation.md:13): refine-all AMR at N0=64 against uniform N=256 at
    # Re=800, t*=12: peak time within 0.3 t*, energy within 2 %, on the engine and on the reference;
    # mass drift below 1e-4 on the engine (the reference's own gate, 5e-4, on the reference: its
    # FP32 collision drifts 2.9e-4 over the run, measured).  Engine against the reference's AMR
    # kernels over the same run: E/E0 within 2e-3 relative (the reference's drift moves its E/E0 by
    # about twice that drift, 4.9e-4 measured), enstrophy within 3e-3 of its peak, the same peak
    # sample (one diagnostic interval = 0.074 t*).
    sa, a = engine_amr_curve(64, 800.0, 12.0)
    su, u = engine_uniform_curve(256, 800.0, 12.0, 40)
    sr, r = reference_amr_curve(64, 800.0, 12.0)
    assert sa == sr == 2445 and su == 9778
    print("\nC3 static gold: engine AMR peak t*=%.4f (uniform 256: %.4f, delta %.3f), energy gap %.4f, drift %.2e; "
          "reference AMR peak t*=%.4f (delta %.3f), energy gap %.4f, drift %.2e; engine vs reference: E/E0 %.2e, "
          "enstrophy %.2e" % (a.peak_t, u.peak_t, abs(a.peak_t - u.peak_t), a.energy_gap(u), a.mass_drift, r.peak_t,
                              abs(r.peak_t - u.peak_t), r.energy_gap(u), r.mass_drift, a.energy_gap(r),
                              a.enstrophy_gap(r)))
    for side in (a, r):
        assert abs(side.peak_t - u.peak_t) <= 0.3
        assert side.energy_gap(u) <= 0.02
        assert side.valid()
    assert a.mass_drift < 1e-4 and u.mass_drift < 1e-4 and u.valid()
    assert a.energy_gap(r) < 2e-3
    assert a.enstrophy_gap(r) < 3e-3
    assert a.peak_t == r.peak_t


# ---- C4: AMR dynamic ---------------------------------------------------------------------------------

def engine_sensors_by_position(e):
    """The sensor values the engine's last build used: level 0 per coarse block, level 1 per level-1
    grid position (the form the reference's override takes)."""
    c = e.counts()
    s1 = np.zeros(c["ng1"], dtype=np.float32)
    s1[e.table("f1pos")] = e.sensor(1)
    return e.sensor(0), s1


def same_grid(e, r, where):
    ce, cr = e.counts(), r.counts()
    for k in COUNTS:
        assert ce[k] == cr[k], "%s %s: engine %s reference %s" % (where, k, ce[k], cr[k])
    for t in TABLES:
        np.testing.assert_array_equal(e.table(t), r.table(t), err_msg="%s %s" % (where, t))


def share_state(e, r):
    for lv in range(3):
        e.set_populations(r.pops(lv), level=lv, layout="blocked")


def test_c4_dynamic_tables_and_steps_against_reference_build():
    # Tables, marks, skin lists and the 2:1 mask bit-exact at the initial build and at 6 regrids 20
    # coarse steps apart, with the reference fed the engine's own sensor (computed by the engine on
    # the shared state); populations within 1e-5 relative after the first coarse step from each
    # shared state and after each migration
    n, re, f1, f2, adapt = 96, 1600.0, 0.3, 0.1, 20
    with J.Solver("amr", n=n, re=re, u0=U0, l1_mode="sensor", l2_mode="sensor", frac1=f1, frac2=f2,
                  adapt_every=adapt, develop_steps=300, max_gb=1024.0) as e:
        r = O.AmrBackend("reference", n, re, "sensor", "sensor", f1, f2, u0=U0, develop=300, budget=BUDGET,
                         build=False)
        try:
            r.set_sensor_override(*engine_sensors_by_position(e))
            r.initial_build()
            same_grid(e, r, "initial build")
            worst_step, worst_migr, grids = 0.0, 0.0, []
            for g in range(6):
                share_state(e, r)
                e.step(1)
                r.step(1)
                for lv in range(3):
                    worst_step = max(worst_step, rel_err(e.get_populations(lv, layout="blocked"), r.pops(lv)))
                e.step(adapt - 1)
                r.step(adapt - 1)
                share_state(e, r)
                e.regrid()                           # the engine's own sensor on the shared state
                r.set_sensor_override(*engine_sensors_by_position(e))
                r.regrid()
                same_grid(e, r, "regrid %d" % g)
                for lv in range(3):
                    worst_migr = max(worst_migr, rel_err(e.get_populations(lv, layout="blocked"), r.pops(lv)))
                c = e.counts()
                grids.append((c["nf1"], c["nf2"]))
        finally:
            r.close()
    print("\nC4 N0=96 sensor/sensor: 6 regrids bit-exact, grids (nf1, nf2) %s; worst population error after a "
          "coarse step %.2e, after a migration %.2e" % (grids, worst_step, worst_migr))
    assert worst_step < 1e-5 and worst_migr < 1e-5
    assert all(g[1] > 0 for g in grids)


class FollowEngineGrid:
    """The reference's AMR kernels driven in the program's loop, each regrid fed the sensor the
    engine's regrid just used: both sides then keep identical grids for the whole run while each
    advances its own populations with its own kernels (the tables are compared at every regrid)."""

    def __init__(self, ref, engine):
        self.r, self.e, self.regrids = ref, engine, 0

    def regrid(self):
        self.r.set_sensor_override(*engine_sensors_by_position(self.e))
        self.r.regrid()
        same_grid(self.e, self.r, "regrid %d" % self.regrids)
        self.regrids += 1

    def step(self, k):
        self.r.step(k)

    def diag(self):
        return self.r.diag()


def test_c4_dynamic_whole_run_against_reference_build():
    # C4 over the whole t*=20 run (6112 coarse steps, a regrid every 20): the engine in the program's
    # loop (graph replay), and the reference's kernels on the grids the engine's sensor chose (fed at
    # each of the 305 regrids; tables, marks, skins and the 2:1 mask bit-exact every time).  The
    # dynamic gold (docs/validation.md:14): breakdown present (peak in (4, 10)), energy monotonic,
    # mass held (the programs' gate, 5e-4) on the engine; the interface interpolation and regrids are
    # not conservative, so mass drifts in this case on both sides (measured: engine 3.2e-4, the
    # reference 5.6e-4, past its own gate).  Engine against reference: the same peak sample, E/E0
    # within 3e-3 relative, enstrophy within 5e-3 of its peak, and no more mass drift than the reference.
    n, re, f1, f2, adapt = 96, 1600.0, 0.3, 0.1, 20
    with J.Solver("amr", n=n, re=re, u0=U0, tstar=20.0, l1_mode="sensor", l2_mode="sensor", frac1=f1, frac2=f2,
                  adapt_every=adapt, max_gb=1024.0, flags=J.FLAG_GRAPH) as e:
        steps, kf = e.info["steps"], e.info["kf"]
        r = O.AmrBackend("reference", n, re, "sensor", "sensor", f1, f2, u0=U0, tstar=20.0, budget=BUDGET,
                         build=False)
        try:
            r.set_sensor_override(*engine_sensors_by_position(e))
            r.initial_build()
            same_grid(e, r, "initial build")
            ref = FollowEngineGrid(r, e)

            class Lockstep:                    # one loop drives both: the engine's event first
                def regrid(self_):
                    e.regrid()
                    ref.regrid()

                def step(self_, k):
                    e.step(k)
                    ref.step(k)

                def diag(self_):
                    return e.diag() + ref.diag()

            rows = amr_loop_rows(Lockstep(), steps, kf, adapt, True)
        finally:
            r.close()
    ec = Curve([row[:4] for row in rows])
    rc = Curve([row[:1] + row[4:] for row in rows])
    assert steps == 6112 and ref.regrids == steps // adapt
    print("\nC4 whole run, %d regrids bit-exact: engine peak t*=%.4f drift %.2e monotonic %s; reference peak "
          "t*=%.4f drift %.2e monotonic %s; E/E0 gap %.2e, enstrophy gap %.2e of peak"
          % (ref.regrids, ec.peak_t, ec.mass_drift, ec.monotonic, rc.peak_t, rc.mass_drift, rc.monotonic,
             ec.energy_gap(rc), ec.enstrophy_gap(rc)))
    assert ec.valid()
    assert ec.mass_drift <= rc.mass_drift
    assert ec.peak_t == rc.peak_t
    assert ec.energy_gap(rc) < 3e-3
    assert ec.enstrophy_gap(rc) < 5e-3


# ---- N=256: one FP32 step from the reference's state -------------------------------------------------

def test_uniform_n256_step_from_reference_state():
    # the per-step bar at a production size: one engine step from the reference's state after 200
    # steps lands within 1e-5 relative of the reference's k_step on every population of 256^3 cells
    n = 256
    p = O.params(n, 1600.0)
    f = O.ref_run(O.ref_init(n), n, p["omega"], 200)
    g = O.ref_run(f, n, p["omega"], 1)
    with J.Solver("uniform", n=n, re=1600.0) as s:
        s.set_populations(f, layout="blocked")
        s.step(1)
        err = rel_err(s.get_populations(layout="blocked"), g)
    print("\nN=256 one step from the reference's state: max relative error %.2e" % err)
    assert err < 1e-5


def test_uniform_n512_step_from_reference_state():
    # the per-step bar at the benchmark size: one engine step from the reference's state after 20
    # steps, against the reference's k_step, on every population of 512^3 cells
    import torch
    n = 512
    need = 19 * n ** 3 * 4                      # one state, 10.2 GB
    avail = 0
    with open("/proc/meminfo") as fh:
        for line in fh:
            if line.startswith("MemAvailable:"):
                avail = int(line.split()[1]) * 1024
    if avail < 5 * need:
        pytest.skip("host memory: %.0f GB available, the test holds up to 4 states of 10.2 GB" % (avail / 1e9))
    if torch.cuda.mem_get_info()[0] < 5 * need:
        pytest.skip("device memory: two states on each side")
    p = O.params(n, 1600.0)
    f = O.ref_init(n)
    O.ref_run_inplace(f, n, p["omega"], 20)
    with J.Solver("uniform", n=n, re=1600.0) as s:
        s.set_populations(f, layout="blocked")
        s.step(1)
        e = s.get_populations(layout="blocked")
    O.ref_run_inplace(f, n, p["omega"], 1)
    err = rel_err(e, f)
    print("\nN=512 one step from the reference's state: max relative error %.2e" % err)
    assert err < 1e-5
