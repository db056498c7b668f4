"""Persistent AMR coarse steps: many solves and several coarse steps in one cooperative launch
(jp_ensemble_set_persistent), against the per-stage batched launches of the same ensemble.

Bars: populations of every level bit-exact with the per-stage path (the same device bodies on the
same inputs), across regrids and for every storage format; one launch per jp_ensemble_step; a grid
barrier that runs past its wait limit stops the launch and jp_ensemble_sync reports JP_ERR_TIMEOUT,
with the GPU still usable afterwards."""
import time

import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu

MEMBERS = [  # n, l1, l2, frac1, frac2, seed
    (32, "sensor", "sensor", 0.3, 0.3, 1),
    (24, "all", "all", 0.35, 0.35, 2),
    (32, "slab", "sensor", 0.35, 0.5, 3),
    (40, "sensor", "sensor", 0.25, 0.4, 4),
    (16, "sensor", "sensor", 0.5, 0.5, 5),
]


def make(spec, storage, vec=0):
    n, l1, l2, f1, f2, seed = spec
    s = J.Solver("amr", n=n, re=1600.0, l1_mode=l1, l2_mode=l2, frac1=f1, frac2=f2, develop_steps=2, max_gb=64.0,
                 storage=storage, vec=vec, flags=J.FLAG_DEFER_INIT)
    s.set_sensor_override(*O.random_sensor_fields(n, seed=seed))
    s.init_tgv()
    return s


def pops(s):
    return [s.get_populations(lv, layout="blocked") for lv in range(3)]


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
def test_persistent_steps_bit_exact_with_per_stage_launches(storage):
    runs = {}
    for mode in (0, 1):
        solvers = [make(sp, storage) for sp in MEMBERS]
        ens = J.Ensemble()
        ens.set_persistent(mode)
        for s in solvers:
            ens.add(s)
        l0 = J.launch_count()
        ens.step(3)
        ens.sync()
        launches = J.launch_count() - l0
        snap = [pops(s) for s in solvers]
        for i, s in enumerate(solvers):       # new grids, then more steps (odd count: coarse parity)
            s.set_sensor_override(*O.random_sensor_fields(MEMBERS[i][0], seed=50 + i))
            s.regrid()
        ens.step(2)
        ens.sync()
        runs[mode] = (snap, [pops(s) for s in solvers], [s.diag() for s in solvers], launches)
        ens.close()
        for s in solvers:
            s.close()
    assert runs[1][3] == 1                      # every coarse step of every member: one launch
    assert runs[0][3] >= 3 * 13
    for k in (0, 1):
        for i in range(len(MEMBERS)):
            for lv in range(3):
                np.testing.assert_array_equal(runs[1][k][i][lv], runs[0][k][i][lv],
                                              err_msg="%s member %d level %d" % ("after regrid" if k else "first", i, lv))
    assert runs[1][2] == runs[0][2]


def test_persistent_steps_bit_exact_with_solo_graph_steps():
    # one member alone, stepped with its own captured graph, against the persistent launch
    spec = MEMBERS[0]
    a = make(spec, "fp32")
    b = J.Solver("amr", n=spec[0], re=1600.0, l1_mode=spec[1], l2_mode=spec[2], frac1=spec[3], frac2=spec[4],
                 develop_steps=2, max_gb=64.0, flags=J.FLAG_DEFER_INIT | J.FLAG_GRAPH)
    b.set_sensor_override(*O.random_sensor_fields(spec[0], seed=spec[5]))
    b.init_tgv()
    ens = J.Ensemble()
    ens.set_persistent(1)
    ens.add(a)
    ens.step(5)
    ens.sync()
    b.step(5)
    for lv in range(3):
        np.testing.assert_array_equal(a.get_populations(lv, layout="blocked"), b.get_populations(lv, layout="blocked"))
    ens.close()
    a.close()
    b.close()


def test_persistent_barrier_wait_limit_reports_timeout():
    # a wait limit of 1 ns: the first CTA at the first grid barrier gives up, records the error and
    # returns, the others return at their next barrier; the host learns it at jp_ensemble_sync
    solvers = [make(sp, "fp32") for sp in MEMBERS[:2]]
    ens = J.Ensemble()
    ens.set_persistent(1, wait_limit_ns=1)
    for s in solvers:
        ens.add(s)
    ens.step(2)
    with pytest.raises(J.JPError) as exc:
        ens.sync()
    assert exc.value.status == 6 and b"grid barrier" in J.lib().jp_last_error()
    ens.sync()                                  # reported once, then cleared
    ens.close()
    for s in solvers:
        s.close()
    with J.Solver("uniform", n=16, re=400.0) as u:   # the context is still usable
        u.step(4)
        assert np.isfinite(u.diag()[0])


SHAPES = {  # name: member specs (n, l1, l2, frac1, frac2, seed); all with 300 develop steps skipped
    "32 solves N0 24/32 sensor": [(24 if i % 2 else 32, "sensor", "sensor", 0.3, 0.1, 100 + i) for i in range(32)],
    "8 solves N0 16 sensor": [(16, "sensor", "sensor", 0.3, 0.1, 200 + i) for i in range(8)],
    "4 solves N0 48 sensor": [(48, "sensor", "sensor", 0.3, 0.1, 300 + i) for i in range(4)],
    "1 solve N0 96 sensor": [(96, "sensor", "sensor", 0.3, 0.1, 400)],
    "1 solve N0 64 all/all": [(64, "all", "all", 0.35, 0.35, 500)],
}


@pytest.mark.parametrize("shape", list(SHAPES))
def test_persistent_steps_throughput(shape):
    # coarse steps of the whole ensemble per second: per-stage launches against one persistent launch
    # per call of 8 coarse steps (printed with -s; both must run)
    specs = SHAPES[shape]
    out = {}
    for mode in (0, 1):
        solvers = [make(sp, "fp32") for sp in specs]
        ens = J.Ensemble()
        ens.set_persistent(mode)
        for s in solvers:
            ens.add(s)
        ens.step(2)
        ens.sync()
        t0 = time.perf_counter()
        for _ in range(10):
            ens.step(8)
        ens.sync()
        out[mode] = (time.perf_counter() - t0) / 80
        work = sum((c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512 for c in (s.counts() for s in solvers))
        ens.close()
        for s in solvers:
            s.close()
    print("\n%s: per-stage launches %.1f us per coarse step, persistent %.1f us (%.2fx); %.1f vs %.1f GLUPS(work)"
          % (shape, out[0] * 1e6, out[1] * 1e6, out[0] / out[1], work / out[0] / 1e9, work / out[1] / 1e9))
    assert out[0] > 0 and out[1] > 0
