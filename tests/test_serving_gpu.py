"""Ensembles (batched launches over many cubes) and the continuous-batching server, on a GB300.

Bars: a cube stepped inside a batch gives the same bits as stepped alone (same kernel, same per-cell
arithmetic); a solve's result is identical alone and in a mix; admission never exceeds the pool
budget; an oversized request is refused, not run."""
import numpy as np
import pytest

import jpsolver as J

pytestmark = pytest.mark.gpu


def test_ensemble_step_matches_individual_steps_bit_exact():
    cfgs = [dict(n=16, re=400.0), dict(n=24, re=800.0, storage="fp16"), dict(n=32, re=1600.0),
            dict(n=40, re=200.0, storage="bf16"), dict(n=8, re=400.0)]
    alone = []
    for c in cfgs:
        with J.Solver("uniform", **c) as s:
            s.step(13)
            alone.append(s.get_populations(dtype=np.float64))
    solvers = [J.Solver("uniform", **c) for c in cfgs]
    ens = J.Ensemble()
    for s in solvers:
        ens.add(s)
    ens.step(5)
    solvers[0].step(3)            # a member's own steps interleave with the ensemble's
    ens.remove(solvers[0])
    ens.step(5)
    solvers[0].step(2)
    ens.add(solvers[0])
    ens.step(3)
    for s, ref, c in zip(solvers, alone, cfgs):
        got = s.get_populations(dtype=np.float64)
        assert s.info["step_count"] == 13
        np.testing.assert_array_equal(got, ref, err_msg=str(c))
    ens.close()
    for s in solvers:
        s.close()


def test_ensemble_with_more_members_than_one_launch():
    cfgs = [dict(n=8 + 8 * (i % 3), re=400.0 + 10 * i) for i in range(60)]   # > 48 cubes: two launches
    solvers = [J.Solver("uniform", **c) for c in cfgs]
    ens = J.Ensemble()
    for s in solvers:
        ens.add(s)
    ens.step(4)
    for s, c in zip(solvers, cfgs):
        with J.Solver("uniform", **c) as r:
            r.step(4)
            np.testing.assert_array_equal(s.get_populations(), r.get_populations())
    ens.close()
    for s in solvers:
        s.close()


def run_server(requests, **kw):
    sv = J.Server(**kw)
    for r in requests:
        assert sv.submit(**r) == 0
    results, peak_active = {}, 0
    while len(results) < len(requests):
        a, q = sv.tick()
        peak_active = max(peak_active, a)
        for res in sv.poll():
            results[res["id"]] = res
    sv.close()
    return results, peak_active


R0 = dict(rid=1, kind="uniform", n=32, re=400.0, tstar=2.0)
MIX = [dict(rid=10, kind="uniform", n=48, re=800.0, tstar=1.5, storage="fp16"),
       dict(rid=11, kind="uniform", n=16, re=300.0, tstar=3.0),
       dict(rid=12, kind="amr", n=16, re=800.0, tstar=1.0, l1_mode="sensor", l2_mode="sensor", frac1=0.3,
            frac2=0.2, develop_steps=20, adapt_every=20),
       dict(rid=13, kind="uniform", n=64, re=1600.0, tstar=0.5, storage="bf16"),
       dict(rid=14, kind="amr", n=16, re=400.0, tstar=1.0),
       dict(rid=15, kind="uniform", n=24, re=200.0, tstar=2.5)]


def test_server_result_same_alone_and_in_mix():
    # a uniform solve (batched launches) and an AMR solve (worker thread, own stream) each give the
    # same result alone and in a mix of six solves that run concurrently
    alone, _ = run_server([R0], tick_steps=16)
    alone_amr, _ = run_server([MIX[2]], tick_steps=16)
    mixed, peak = run_server([MIX[0], MIX[1], R0] + MIX[2:], tick_steps=16)
    for a, m in ((alone[1], mixed[1]), (alone_amr[12], mixed[12])):
        assert a["status"] == 0 and m["status"] == 0
        for k in ("steps", "samples", "peak_tstar", "peak_enstrophy", "energy_ratio", "mass_drift", "valid"):
            assert a[k] == m[k], (a["id"], k)
    assert peak >= 3                                   # solves really ran concurrently
    assert all(r["status"] == 0 for r in mixed.values())


def test_server_one_worker_gives_the_same_results():
    # one worker thread (creations and regrids one at a time) changes nothing but the timing: the AMR
    # solves still advance together in the batched launches, with the same results
    reqs = [dict(MIX[2], rid=40), dict(MIX[4], rid=41), dict(R0, rid=42)]
    one, _ = run_server(reqs, tick_steps=16, workers=1)
    many, _ = run_server(reqs, tick_steps=16)
    for rid in (40, 41, 42):
        assert one[rid]["status"] == 0
        for k in ("samples", "peak_tstar", "peak_enstrophy", "energy_ratio", "mass_drift", "valid"):
            assert one[rid][k] == many[rid][k], (rid, k)


def test_server_amr_result_matches_program_loop():
    req = MIX[2]
    res, _ = run_server([req], tick_steps=16)
    r = res[12]
    # the `amr` program's loop: regrid (s>0, s % adapt == 0), diagnostic (s % diagK == 0), step
    cfg = {k: v for k, v in req.items() if k not in ("rid", "kind")}
    with J.Solver("amr", **cfg) as s:
        steps = s.info["steps"]
        diagK = max(1, steps // 160)
        E0, peak, peak_ts, samples, Elast = None, -1.0, -1.0, 0, None
        kf = s.info["kf"]
        for step in range(steps + 1):
            if step > 0 and step % cfg["adapt_every"] == 0:
                s.regrid()
            if step % diagK == 0:
                E, ens, mass = s.diag()
                E0 = E if E0 is None else E0
                Elast = E
                samples += 1
                if ens > peak:
                    peak, peak_ts = ens, step * 0.05 * kf
            if step < steps:
                s.step(1)
    assert r["samples"] == samples
    assert r["peak_enstrophy"] == peak and r["peak_tstar"] == peak_ts
    assert r["energy_ratio"] == Elast / E0


@pytest.mark.parametrize("diag_every", [0, 3, 7])
def test_server_uniform_result_matches_program_loop(diag_every):
    # the `uniform` program's loop: a diagnostic at every step s % diagK == 0 (diagK = steps/240,
    # here 1: 305 steps), then steps to the next one; the served solve reports the same samples and
    # peak, bit for bit.  The server interleaves a solve's diagnostics with its batched steps inside
    # a tick (16 steps here), so intervals of 1, 3 and 7 steps put several samples in one tick, and
    # 305 steps leave a last interval that no sample follows
    req = dict(rid=21, kind="uniform", n=24, re=300.0, tstar=4.0, storage="fp16")
    if diag_every:
        req["diag_every"] = diag_every
    res, _ = run_server([req, dict(R0, rid=22), dict(MIX[0], rid=23)], tick_steps=16)
    r = res[21]
    cfg = {k: v for k, v in req.items() if k not in ("rid", "kind", "diag_every")}
    with J.Solver("uniform", **cfg) as s:
        steps, kf = s.info["steps"], s.info["kf"]
        diagK = diag_every or max(1, steps // 240)
        E0, peak, peak_ts, samples, Elast = None, -1.0, -1.0, 0, None
        for step in range(0, steps + 1, diagK):
            E, ens, mass = s.diag()
            E0 = E if E0 is None else E0
            Elast = E
            samples += 1
            if ens > peak:
                peak, peak_ts = ens, step * 0.05 * kf
            if step + diagK <= steps:
                s.step(diagK)
    assert r["steps"] == steps and r["samples"] == samples
    assert r["peak_enstrophy"] == peak and r["peak_tstar"] == peak_ts
    assert r["energy_ratio"] == Elast / E0


def test_server_admission_respects_budget():
    big = [dict(rid=100 + i, kind="uniform", n=96, re=800.0, tstar=0.3) for i in range(4)]
    one = 2 * 19 * 4 * 96 ** 3 + 16 * 96 ** 3 + (1 << 20)
    budget_gb = 2.5 * one / 2 ** 30                   # room for two at a time
    res, peak = run_server(big, pool_gb=budget_gb, tick_steps=32)
    assert peak == 2
    assert all(r["status"] == 0 for r in res.values())
    # later requests started only after earlier ones ended
    starts = sorted(r["t_start"] for r in res.values())
    ends = sorted(r["t_end"] for r in res.values())
    assert starts[2] >= ends[0]


def test_server_inplace_requests_fit_twice_as_many_with_the_same_results():
    base = [dict(rid=200 + i, kind="uniform", n=96, re=800.0, tstar=0.3) for i in range(4)]
    one = 2 * 19 * 4 * 96 ** 3 + 16 * 96 ** 3 + (1 << 20)
    budget_gb = 2.5 * one / 2 ** 30                   # two two-array cubes at a time, four in place
    two, peak2 = run_server(base, pool_gb=budget_gb, tick_steps=32)
    inp, peak1 = run_server([dict(r, flags=J.FLAG_INPLACE) for r in base], pool_gb=budget_gb, tick_steps=32)
    assert peak2 == 2 and peak1 == 4
    for rid in two:
        assert inp[rid]["status"] == 0
        for k in ("steps", "samples", "peak_tstar", "peak_enstrophy", "energy_ratio", "mass_drift", "valid"):
            assert inp[rid][k] == two[rid][k], (rid, k)


def test_server_refuses_request_larger_than_pool():
    sv = J.Server(pool_gb=0.001)
    assert sv.submit(rid=7, kind="uniform", n=64, re=400.0, tstar=0.2) == 4     # JP_ERR_NOMEM
    res = sv.poll()
    assert len(res) == 1 and res[0]["id"] == 7 and res[0]["status"] == 4
    sv.close()


def test_amr_ensemble_batched_coarse_steps_bit_exact():
    # AMR solves of different sizes and refinements stepped in one launch per stage give the same
    # bits as stepped alone, with regrids between ensemble steps and a uniform member alongside
    import oracle as O
    cfgs = [dict(n=16, re=800.0, l1_mode="all", l2_mode="all"),
            dict(n=24, re=1600.0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.3, develop_steps=5),
            dict(n=32, re=400.0, l1_mode="slab", l2_mode="sensor", frac2=0.4, develop_steps=5),
            dict(n=16, re=800.0, l1_mode="sensor", l2_mode="all", frac1=0.5, develop_steps=5, storage="fp16")]
    sens = [None, O.random_sensor_fields(24, seed=2), O.random_sensor_fields(32, seed=3),
            O.random_sensor_fields(16, seed=4)]

    def make(c, sv):
        s = J.Solver("amr", max_gb=64.0, **c)
        if sv is not None:
            s.set_sensor_override(*sv)
            s.init_tgv()
        return s

    alone = []
    for c, sv in zip(cfgs, sens):
        with make(c, sv) as s:
            s.step(3)
            s.regrid()
            s.step(2)
            alone.append([s.get_populations(lv, layout="blocked") for lv in range(3)] + [s.diag()])
    members = [make(c, sv) for c, sv in zip(cfgs, sens)]
    uni = J.Solver("uniform", n=16, re=400.0)
    ens = J.Ensemble()
    for m in members + [uni]:
        ens.add(m)
    ens.step(3)
    for m in members:
        m.regrid()
    ens.step(2)
    for m, ref, c in zip(members, alone, cfgs):
        assert m.info["step_count"] == 5
        for lv in range(3):
            np.testing.assert_array_equal(m.get_populations(lv, layout="blocked"), ref[lv], err_msg=str(c))
        assert m.diag() == ref[3]
    ens.close()
    for m in members + [uni]:
        m.close()
