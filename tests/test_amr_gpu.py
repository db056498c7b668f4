"""Parity of the engine's three-level AMR (through the C ABI) with the AMR oracle on a GB300.

Bars: block tables, marks, skin lists and the 2:1 (deep) mask are bit-exact when both sides are fed
the same sensor field (jp_set_sensor_override); populations agree within 1e-5 relative after one
coarse step from the same state; diagnostics within 1e-10 relative (deterministic sums in a
different order).
"""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu
TABLES = ["ref0", "fof0", "rl0", "l1pcb", "l1oct", "f1pos", "l1grid", "ref1", "fof1", "rl1", "l2pl1", "l2oct",
          "skin0", "skin1"]
COUNT_KEYS = ["nref0", "nf1", "nref1", "nf2", "n_skin0", "n_skin1", "cap1", "cap2", "cap_nref0", "cap_nref1"]


def engine(n, re, l1, l2, frac1=0.35, frac2=0.35, develop=300, mb=8, defer=False):
    # defer: no build at creation, so the first build is the one the test feeds a sensor to
    return J.Solver("amr", n=n, re=re, l1_mode=l1, l2_mode=l2, frac1=frac1, frac2=frac2, develop_steps=develop,
                    max_gb=1024.0, mb=mb, flags=J.FLAG_DEFER_INIT if defer else 0)


def oracle(n, re, l1, l2, frac1=0.35, frac2=0.35, develop=300, mb=8, build=True):
    return O.AmrBackend("oracle", n, re, l1, l2, frac1, frac2, develop=develop, budget=1024.0 * 2 ** 30, mb=mb,
                        build=build)


def assert_tables_equal(e, o, where="", caps=True):
    ce, co = e.counts(), o.counts()
    for k in COUNT_KEYS if caps else [k for k in COUNT_KEYS if not k.startswith("cap")]:
        assert ce[k] == co[k], "%s count %s: engine %s oracle %s" % (where, k, ce[k], co[k])
    for t in TABLES:
        np.testing.assert_array_equal(e.table(t), o.table(t), err_msg="%s table %s" % (where, t))
    if co["nf1"]:
        np.testing.assert_array_equal(e.table("deep"), o.table("deep"), err_msg=where + " deep mask")


def rel_err(a, b):
    if a.size == 0 and b.size == 0:
        return 0.0
    return float(np.max(np.abs(a.astype(np.float64) - b) / np.abs(b)))


CASES = [  # n, l1, l2, frac1, frac2, ties
    (16, "all", "all", 0.35, 0.35, False),
    (16, "slab", "sensor", 0.35, 0.35, False),
    (24, "sensor", "sensor", 0.3, 0.1, False),
    (32, "sensor", "sensor", 0.35, 0.35, True),
    (32, "slab", "slab", 0.35, 0.5, False),
    (32, "all", "sensor", 0.5, 0.3, True),
    (40, "sensor", "sensor", 0.25, 0.3, True),
]


def build_both(n, l1, l2, f1, f2, s0, s1, develop=5):
    """Initial build on both sides with the same sensor.  Ties can over-admit past a pool (the
    reference sizes it with a 1.4 margin and then writes out of bounds); the engine grows the pool,
    and so does the oracle here (grow=True), so tables still compare bit for bit."""
    e = engine(n, 800.0, l1, l2, f1, f2, develop=develop, defer=True)
    e.set_sensor_override(s0, s1)
    o = O.AmrBackend("oracle", n, 800.0, l1, l2, f1, f2, develop=develop, budget=1024.0 * 2 ** 30, build=False,
                     grow=True)
    o.set_sensor_override(s0, s1)
    o.initial_build()
    e.init_tgv()
    return e, o


@pytest.mark.parametrize("n,l1,l2,f1,f2,ties", CASES)
def test_tables_bit_exact_with_shared_sensor(n, l1, l2, f1, f2, ties):
    s0, s1 = O.random_sensor_fields(n, seed=n + len(l1) + len(l2), ties=ties)
    e, o = build_both(n, l1, l2, f1, f2, s0, s1)
    with e:
        assert_tables_equal(e, o, "initial build")
        np.testing.assert_array_equal(e.sensor(0), o.sensor(0))
        for r in range(2):
            t0, t1 = O.random_sensor_fields(n, seed=100 + r, ties=ties)
            e.set_sensor_override(t0, t1)
            o.set_sensor_override(t0, t1)
            e.step(1)
            o.step(1)
            o.regrid()
            e.regrid()
            assert_tables_equal(e, o, "regrid %d" % r)
        o.close()


@pytest.mark.parametrize("n,l1,l2,f1,f2", [(16, "all", "all", 0.35, 0.35), (16, "slab", "sensor", 0.35, 0.5),
                                            (32, "sensor", "sensor", 0.3, 0.3), (24, "all", "sensor", 0.5, 0.2)])
def test_populations_one_coarse_step(n, l1, l2, f1, f2):
    s0, s1 = O.random_sensor_fields(n, seed=7)
    with engine(n, 1600.0, l1, l2, f1, f2, develop=3, defer=True) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        o = oracle(n, 1600.0, l1, l2, f1, f2, develop=3, build=False)
        o.set_sensor_override(s0, s1)
        o.initial_build()
        assert_tables_equal(e, o)
        # seeded fine levels: prolongation of the same coarse state
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 2e-6, "seed level %d" % lv
        # same state on both sides, then one coarse step (1 + 2 + 4 level steps, fills, restrictions)
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        e.step(1)
        o.step(1)
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 1e-5, "level %d" % lv
        o.close()


@pytest.mark.parametrize("n,mb,f1", [(16, 4, 0.35), (64, 16, 0.5)])
def test_populations_one_coarse_step_other_block_edges(n, mb, f1):
    # the interface work (fill and prep lists, pulled populations only) at block edges 4 and 16: the
    # ghost-shell size, the interface cells and the step kernels all depend on MB
    s0, s1 = O.random_sensor_fields(n, mb=mb, seed=9)
    with engine(n, 1600.0, "sensor", "sensor", f1, 0.4, develop=3, mb=mb, defer=True) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        o = oracle(n, 1600.0, "sensor", "sensor", f1, 0.4, develop=3, mb=mb, build=False)
        o.set_sensor_override(s0, s1)
        o.initial_build()
        assert_tables_equal(e, o)
        counts = e.counts()
        assert counts["nf1"] > 0 and counts["nf2"] > 0
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        e.step(1)
        o.step(1)
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 1e-5, "level %d" % lv
        o.close()


def test_populations_across_regrid_migration():
    n = 32
    s0, s1 = O.random_sensor_fields(n, seed=3)
    t0, t1 = O.random_sensor_fields(n, seed=4)
    with engine(n, 1600.0, "sensor", "sensor", 0.4, 0.4, develop=2, defer=True) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        o = oracle(n, 1600.0, "sensor", "sensor", 0.4, 0.4, develop=2, build=False)
        o.set_sensor_override(s0, s1)
        o.initial_build()
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        e.step(2)
        o.step(2)
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        e.set_sensor_override(t0, t1)
        o.set_sensor_override(t0, t1)
        e.regrid()
        o.regrid()
        assert_tables_equal(e, o, "after regrid")
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 2e-6, "migrated level %d" % lv
        o.close()


@pytest.mark.parametrize("n,l1,l2", [(16, "all", "all"), (16, "slab", "sensor")])
def test_diag_matches_oracle(n, l1, l2):
    s0, s1 = O.random_sensor_fields(n, seed=11)
    with engine(n, 800.0, l1, l2, develop=2, defer=True) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        o = oracle(n, 800.0, l1, l2, develop=2, build=False)
        o.set_sensor_override(s0, s1)
        o.initial_build()
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        d = e.diag()
        do = o.diag()
        for x, y in zip(d, do):
            assert abs(x - y) <= 1e-10 * abs(y)
        o.close()


def test_computed_sensor_tables_match_oracle_on_smooth_flow():
    # without an override both sides compute the sensor themselves; on the initial TGV the ranking
    # of block sensors is far from ties, so the tables agree
    n = 32
    with engine(n, 1600.0, "sensor", "sensor", 0.3, 0.3, develop=40) as e:
        o = oracle(n, 1600.0, "sensor", "sensor", 0.3, 0.3, develop=40)
        s_e, s_o = e.sensor(0), o.sensor(0)
        assert rel_err(s_e, s_o) < 1e-4
        assert e.counts()["nf1"] == o.counts()["nf1"]


def test_static_gold_all_levels_track_uniform_4n():
    # refine-all AMR at N0 = uniform at 4 N0 (src/tgv3d_amr.cu:13, docs/validation.md:13): the
    # normalised energy E/E0 agrees within 2 % after the same physical time.  (E0 itself differs: the
    # fine levels start from a trilinear prolongation of the coarse TGV, whose amplitude is lower.)
    n0, re, steps = 16, 400.0, 40
    with engine(n0, re, "all", "all") as a:
        ea0 = a.diag()[0]
        a.step(steps)
        ea, za, ma = a.diag()
    with J.Solver("uniform", n=4 * n0, re=re) as u:
        eu0 = u.diag()[0]
        u.step(4 * steps)
        eu, zu, mu = u.diag()
    assert abs(ea / ea0 - eu / eu0) / (eu / eu0) < 0.02
    assert abs(ma - 1.0) < 1e-5


def test_pool_grows_when_ties_over_admit():
    # every coarse block ties at the threshold: 512 level-1 blocks against a pool of 72; the engine
    # grows the pool (the reference would write past it) and the tables equal the growing oracle's
    n = 32
    cnb0, ng1 = (n // 8) ** 3, (2 * n // 8) ** 3
    ones0, ones1 = np.ones(cnb0, dtype=np.float32), np.linspace(0, 1, ng1, dtype=np.float32)
    s0, s1 = O.random_sensor_fields(n, seed=21)
    with J.Solver("amr", n=n, re=800.0, l1_mode="sensor", l2_mode="sensor", frac1=0.1, frac2=0.2, develop_steps=2,
                  max_gb=1024.0, flags=J.FLAG_DEFER_INIT) as e:
        o = O.AmrBackend("oracle", n, 800.0, "sensor", "sensor", 0.1, 0.2, develop=2, budget=1024.0 * 2 ** 30,
                         grow=True, build=False)
        for b in (e, o):                 # the same initial grid on both sides
            b.set_sensor_override(s0, s1)
        e.init_tgv()
        o.initial_build()
        assert_tables_equal(e, o, "initial build")
        assert e.counts()["cap1"] == 72
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")
        for b in (e, o):
            b.set_sensor_override(ones0, ones1)
            b.regrid()
        assert e.counts()["nf1"] == 512 and e.counts()["cap1"] >= 512
        assert_tables_equal(e, o, "grown pool")
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 2e-6
        e.step(1)
        o.step(1)
        for lv in range(3):
            assert rel_err(e.get_populations(lv, layout="blocked"), o.pops(lv)) < 1e-5
        o.close()


def test_capacity_overflow_is_reported_not_written():
    # a regrid that would need more level-1 blocks than the pool holds, with no budget left to grow it,
    # is rejected before any table is written; the previous grid stays valid and the solver steps on
    n = 32
    with J.Solver("amr", n=n, re=800.0, l1_mode="sensor", l2_mode="sensor", frac1=0.1, frac2=0.1, develop_steps=2,
                  max_gb=0.04) as e:
        cap1 = e.counts()["cap1"]
        cnb0 = e.counts()["cnb0"]
        ones0 = np.ones(cnb0, dtype=np.float32)              # every block ties at the threshold
        ones1 = np.ones((2 * n // 8) ** 3, dtype=np.float32)
        e.set_sensor_override(ones0, ones1)
        before = {t: e.table(t) for t in TABLES}
        with pytest.raises(J.JPError) as exc:
            e.regrid()
        assert exc.value.status == 3
        assert 8 * cnb0 > cap1
        for t in TABLES:
            np.testing.assert_array_equal(e.table(t), before[t], err_msg=t)
        e.step(2)
        assert np.isfinite(e.diag()[0])


def test_autotune_amr_block_edge():
    # the AMR tuner times the block edges that divide N0 and returns one of them
    tuned, lups = J.autotune("amr", steps=2, n=32, re=800.0, l1_mode="all", l2_mode="all", max_gb=4.0)
    assert tuned["mb"] in (4, 8, 16) and lups > 0


@pytest.mark.parametrize("mb,tpbs", [(8, (128, 256, 512)), (16, (128, 256, 512)), (4, (64,))])
def test_step_threads_per_block_bit_exact(mb, tpbs):
    # the level steps split a block's cells over 64..512 threads; every split computes the same
    # per-cell arithmetic, so the populations agree bit for bit with the default split
    n = 32
    s0, s1 = O.random_sensor_fields(n, mb=mb, seed=5)
    out = {}
    for t in (0,) + tpbs:
        with J.Solver("amr", n=n, re=800.0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.3,
                      develop_steps=2, max_gb=1024.0, mb=mb, threads_per_block=t) as e:
            e.set_sensor_override(s0, s1)
            e.init_tgv()
            e.step(2)
            out[t] = [e.get_populations(lv, layout="blocked") for lv in range(3)]
    for t in tpbs:
        for lv in range(3):
            np.testing.assert_array_equal(out[t][lv], out[0][lv], err_msg="tpb %d level %d" % (t, lv))


def test_graph_replay_matches_direct_launches_across_regrids():
    # the captured step (launch shapes from the pool capacities, block counts read on the device)
    # stays valid across regrids that change every table and count: replay gives the same bits as
    # direct launches, including after seeding flips the fine levels' ping-pong parity
    n = 32
    runs = {}
    for flags in (0, J.FLAG_GRAPH):
        with J.Solver("amr", n=n, re=1600.0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.4,
                      develop_steps=2, max_gb=1024.0, flags=flags) as e:
            e.set_sensor_override(*O.random_sensor_fields(n, seed=31))
            e.init_tgv()
            seen = []
            for r in range(4):
                e.step(3)
                e.set_sensor_override(*O.random_sensor_fields(n, seed=40 + r))
                e.regrid()
                seen.append((e.counts()["nf1"], e.counts()["nf2"]))
            e.step(3)
            runs[flags] = ([e.get_populations(lv, layout="blocked") for lv in range(3)], seen, e.diag())
    assert len(set(runs[0][1])) > 1                    # the grids really changed
    assert runs[0][1] == runs[J.FLAG_GRAPH][1]
    for lv in range(3):
        np.testing.assert_array_equal(runs[J.FLAG_GRAPH][0][lv], runs[0][0][lv], err_msg="level %d" % lv)
    assert runs[0][2] == runs[J.FLAG_GRAPH][2]


@pytest.mark.parametrize("storage,atol", [("fp16", 2e-5), ("bf16", 1e-4)])
def test_shifted_storage_one_coarse_step_tracks_oracle(storage, atol):
    # AMR pools, prolongation sources and ghosts stored as shifted 16-bit values (f - w_q), FP32
    # arithmetic: from the same (rounded) state, one coarse step stays within the format's rounding
    # of the FP32 oracle.  The deviations |f - w_q| reach ~8e-3, whose rounding is ~4e-6 in FP16
    # (11-bit significand) and ~3e-5 in BF16 (8-bit); level 2 is stored four times in a coarse step
    # and the restrictions average rounded values, so the bars are 2e-5 and 1e-4 absolute (measured
    # 1.02e-5 and 3.9e-5).  Tables are identical for the same sensor.
    n = 24
    s0, s1 = O.random_sensor_fields(n, seed=17)
    with J.Solver("amr", n=n, re=1600.0, l1_mode="sensor", l2_mode="sensor", frac1=0.35, frac2=0.4,
                  develop_steps=3, max_gb=1024.0, storage=storage, flags=J.FLAG_DEFER_INIT) as e:
        e.set_sensor_override(s0, s1)
        e.init_tgv()
        o = oracle(n, 1600.0, "sensor", "sensor", 0.35, 0.4, develop=3, build=False)
        o.set_sensor_override(s0, s1)
        o.initial_build()
        assert_tables_equal(e, o, storage)
        for lv in range(3):
            e.set_populations(o.pops(lv), level=lv, layout="blocked")      # rounds to the format
            o.set_pops(lv, e.get_populations(lv, layout="blocked"))        # the same rounded state
        e.step(1)
        o.step(1)
        for lv in range(3):
            err = float(np.max(np.abs(e.get_populations(lv, layout="blocked").astype(np.float64) - o.pops(lv))))
            assert err < atol, "level %d: %.3g" % (lv, err)
        d, do = e.diag(), o.diag()
        assert abs(d[2] - do[2]) < 1e-6 and abs(d[0] - do[0]) < 1e-3 * do[0]
        o.close()


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_shifted_storage_static_gold_holds_mass(storage):
    # refine-all AMR in shifted storage over 60 coarse steps: the energy decays like the FP32 run's,
    # mass is held (shifted collision), and the graph replay gives the same bits as direct launches
    n0, re, steps = 16, 400.0, 60
    res = {}
    for st, flags in (("fp32", 0), (storage, 0), (storage, J.FLAG_GRAPH)):
        with J.Solver("amr", n=n0, re=re, l1_mode="all", l2_mode="all", storage=st, flags=flags) as a:
            e0, z0, m0 = a.diag()
            a.step(steps)
            e1, z1, m1 = a.diag()
            res[(st, flags)] = (e1 / e0, abs(m1 - m0) / m0, a.get_populations(2, layout="blocked"))
    r32, r16, r16g = res[("fp32", 0)], res[(storage, 0)], res[(storage, J.FLAG_GRAPH)]
    assert abs(r16[0] - r32[0]) < (2e-4 if storage == "fp16" else 3e-3)
    assert r16[1] < (1e-6 if storage == "fp16" else 1e-5)
    np.testing.assert_array_equal(r16[2], r16g[2])


def _dilate(mask, gx):
    """One 26-neighbour periodic dilation layer of a block mask on a gx^3 grid (x fastest)."""
    m = mask.reshape(gx, gx, gx).astype(bool)
    out = m.copy()
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out |= np.roll(m, (dz, dy, dx), axis=(0, 1, 2))
    return out.reshape(-1).astype(np.int32)


@pytest.mark.parametrize("layers", [1, 2])
def test_buffer_dilates_the_sensor_marks(layers):
    # --buffer N (parsed but unused by the reference): the refined coarse blocks are the sensor
    # marks dilated by N layers; level-2 marks grow only into deep level-1 blocks (2:1 balance)
    n = 48
    s0, s1 = O.random_sensor_fields(n, seed=8)
    res = {}
    for b in (0, layers):
        with J.Solver("amr", n=n, re=800.0, l1_mode="sensor", l2_mode="sensor", frac1=0.1, frac2=0.1,
                      develop_steps=2, max_gb=64.0, buffer=b) as e:
            e.set_sensor_override(s0, s1)
            e.init_tgv()
            res[b] = {t: e.table(t) for t in ("ref0", "ref1", "deep", "f1pos")}
            res[b]["counts"] = e.counts()
    ref0, cgx = res[0]["ref0"], n // 8
    want = ref0
    for _ in range(layers):
        want = _dilate(want, cgx)
    np.testing.assert_array_equal(res[layers]["ref0"], want)
    assert res[layers]["counts"]["nf1"] > res[0]["counts"]["nf1"]
    r1, deep = res[layers]["ref1"], res[layers]["deep"]
    assert np.all(r1[deep == 0] == 0)                  # level-2 marks only on deep blocks
    assert res[layers]["counts"]["nref1"] >= res[0]["counts"]["nref1"]


def buffer_level2_spec(sen1, deep, f1pos, l1grid, l1gx, frac2, cap, layers):
    """The level-2 marks of --buffer N, written out: the sensor threshold over the deep level-1
    blocks (tgt = min(cap, max(1, int(frac2 * ndeep))), thr = the (ndeep - tgt)-th smallest, marks =
    deep and sensor >= thr), then N dilation layers over the periodic level-1 grid, each marking a
    deep block when it or one of its 26 neighbour positions holds a marked level-1 block."""
    d = deep != 0
    vals = np.sort(sen1[d])
    nd = vals.size
    tgt = max(1, int(frac2 * nd))
    if cap is not None:
        tgt = min(cap, tgt)
    ref = (d & (sen1 >= vals[nd - tgt])).astype(np.int32)
    px, py, pz = f1pos % l1gx, (f1pos // l1gx) % l1gx, f1pos // (l1gx * l1gx)
    for _ in range(layers):
        out = ref.copy()
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    q = (((pz + dz) % l1gx) * l1gx + (py + dy) % l1gx) * l1gx + (px + dx) % l1gx
                    nb = l1grid[q]
                    out |= np.where(nb >= 0, ref[np.maximum(nb, 0)], 0)
        ref = np.where(d, out, 0).astype(np.int32)
    return ref


@pytest.mark.parametrize("layers", [1, 2])
def test_buffer_level2_marks_match_written_spec(layers):
    # --buffer N on level 2, pinned exactly: at the initial build (threshold without a cap) and at a
    # regrid (capped by cap_nref1), the engine's level-2 marks equal the written specification
    # computed from its own level-1 grid, sensor and deep mask; nf2 follows from them
    n, f2 = 48, 0.1
    with J.Solver("amr", n=n, re=800.0, l1_mode="sensor", l2_mode="sensor", frac1=0.2, frac2=f2, develop_steps=2,
                  max_gb=64.0, buffer=layers, flags=J.FLAG_DEFER_INIT) as e:
        e.set_sensor_override(*O.random_sensor_fields(n, seed=19))
        e.init_tgv()
        l1gx = 2 * n // 8
        for where in ("initial build", "regrid"):
            cap = None
            if where == "regrid":
                cap = e.counts()["cap_nref1"]          # the cap the regrid's threshold uses
                e.step(1)
                e.set_sensor_override(*O.random_sensor_fields(n, seed=23))
                e.regrid()
            c = e.counts()
            want = buffer_level2_spec(e.sensor(1), e.table("deep"), e.table("f1pos"), e.table("l1grid"), l1gx, f2,
                                      cap, layers)
            got = e.table("ref1")
            np.testing.assert_array_equal(got, want, err_msg=where)
            assert c["nf2"] == 8 * int(want.sum()) and c["nref1"] == int(want.sum())
            assert int(want.sum()) > int(np.sum(e.table("deep") != 0) * f2)   # the buffer added blocks


@pytest.mark.parametrize("mb,storage", [(8, "fp32"), (8, "fp16"), (16, "fp32"), (16, "bf16")])
def test_row_steps_bit_exact_with_cell_steps(mb, storage):
    # the fine steps on rows of four cells per thread (vector loads, shuffles at the row inside, the
    # x-neighbour block or ghost shell at the faces) compute each cell as the per-cell steps do:
    # same bits, on a grid with ghost shells on both fine levels and the fused restriction
    n = 32
    s0, s1 = O.random_sensor_fields(n, mb=mb, seed=12)
    out = {}
    for vec in (1, 4):
        with J.Solver("amr", n=n, re=1600.0, l1_mode="sensor", l2_mode="sensor", frac1=0.35, frac2=0.4,
                      develop_steps=2, max_gb=64.0, mb=mb, storage=storage, vec=vec) as e:
            e.set_sensor_override(s0, s1)
            e.init_tgv()
            e.step(3)
            out[vec] = [e.get_populations(lv, layout="blocked") for lv in range(3)]
    for lv in range(3):
        np.testing.assert_array_equal(out[4][lv], out[1][lv], err_msg="level %d" % lv)
