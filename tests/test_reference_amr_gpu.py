"""The reference's own AMR kernels (src/tgv3d_amr.cu compiled from its checkout into a cubin), driven in
the reference's launch order, against the AMR oracle and the engine on the same inputs.  Pins the
oracle and checks the engine directly.  Skipped when the cubin was not built."""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_amr_available(), reason="reference AMR cubin / librefrun.so not built")]
TABLES = ["ref0", "fof0", "rl0", "l1pcb", "l1oct", "f1pos", "l1grid", "ref1", "fof1", "rl1", "l2pl1", "l2oct",
          "skin0", "skin1"]
BUDGET = 1024.0 * 2 ** 30


def rel_err(a, b):
    if a.size == 0 and b.size == 0:
        return 0.0
    return float(np.max(np.abs(a.astype(np.float64) - b) / np.abs(b)))


def pair(n, re, l1, l2, f1, f2, seed, develop=3):
    s0, s1 = O.random_sensor_fields(n, seed=seed)
    r = O.AmrBackend("reference", n, re, l1, l2, f1, f2, develop=develop, budget=BUDGET, build=False)
    o = O.AmrBackend("oracle", n, re, l1, l2, f1, f2, develop=develop, budget=BUDGET, build=False)
    for b in (r, o):
        b.set_sensor_override(s0, s1)
        b.initial_build()
    return r, o


def same_tables(a, b, where):
    ca, cb = a.counts(), b.counts()
    for k in ("nref0", "nf1", "nref1", "nf2", "n_skin0", "n_skin1", "cap1", "cap2"):
        assert ca[k] == cb[k], "%s %s: %s vs %s" % (where, k, ca[k], cb[k])
    for t in TABLES:
        np.testing.assert_array_equal(a.table(t), b.table(t), err_msg="%s %s" % (where, t))


CASES = [(16, "all", "all", 0.35, 0.35), (16, "slab", "sensor", 0.35, 0.5), (32, "sensor", "sensor", 0.3, 0.3),
         (24, "all", "sensor", 0.5, 0.2)]


@pytest.mark.parametrize("n,l1,l2,f1,f2", CASES)
def test_oracle_matches_reference_amr(n, l1, l2, f1, f2):
    r, o = pair(n, 1600.0, l1, l2, f1, f2, seed=n)
    same_tables(r, o, "initial build")
    for lv in range(3):
        assert rel_err(o.pops(lv), r.pops(lv)) < 2e-6, "seed level %d" % lv
    for lv in range(3):
        r.set_pops(lv, o.pops(lv))
    r.step(1)
    o.step(1)
    for lv in range(3):
        assert rel_err(o.pops(lv), r.pops(lv)) < 1e-5, "step level %d" % lv
    for lv in range(3):      # diagnostics of identical populations (the reference sums with atomics)
        r.set_pops(lv, o.pops(lv))
    dr, do = r.diag(), o.diag()
    for x, y in zip(dr, do):
        assert abs(x - y) <= 1e-11 * abs(x)
    t0, t1 = O.random_sensor_fields(n, seed=n + 1)
    for b in (r, o):
        b.set_sensor_override(t0, t1)
        b.regrid()
    same_tables(r, o, "regrid")
    for lv in range(3):
        assert rel_err(o.pops(lv), r.pops(lv)) < 1e-5, "migrated level %d" % lv
    r.close()
    o.close()


@pytest.mark.parametrize("n,l1,l2,f1,f2", CASES)
def test_engine_matches_reference_amr(n, l1, l2, f1, f2):
    s0, s1 = O.random_sensor_fields(n, seed=2 * n)
    r = O.AmrBackend("reference", n, 1600.0, l1, l2, f1, f2, develop=3, budget=BUDGET, build=False)
    r.set_sensor_override(s0, s1)
    r.initial_build()
    with J.Solver("amr", n=n, re=1600.0, l1_mode=l1, l2_mode=l2, frac1=f1, frac2=f2, develop_steps=3,
                  max_gb=1024.0, flags=J.FLAG_DEFER_INIT) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        ce, cr = e.counts(), r.counts()
        for k in ("nref0", "nf1", "nref1", "nf2", "n_skin0", "n_skin1", "cap1", "cap2"):
            assert ce[k] == cr[k], k
        for t in TABLES:
            np.testing.assert_array_equal(e.table(t), r.table(t), err_msg=t)
        for lv in range(3):
            e.set_populations(r.pops(lv), level=lv, layout="blocked")
        for _ in range(3):   # per coarse step from the reference's own state
            e.step(1)
            r.step(1)
            for lv in range(3):
                assert rel_err(e.get_populations(lv, layout="blocked"), r.pops(lv)) < 1e-5, "level %d" % lv
            for lv in range(3):
                e.set_populations(r.pops(lv), level=lv, layout="blocked")
    r.close()


def test_reference_sensor_matches_oracle_sensor():
    n = 32
    r = O.AmrBackend("reference", n, 1600.0, "sensor", "sensor", 0.3, 0.3, develop=30, budget=BUDGET)
    o = O.AmrBackend("oracle", n, 1600.0, "sensor", "sensor", 0.3, 0.3, develop=30, budget=BUDGET)
    assert rel_err(o.sensor(0), r.sensor(0)) < 1e-4
    r.close()
    o.close()
