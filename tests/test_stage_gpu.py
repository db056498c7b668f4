"""jp_stage_populations: the next step's state uploaded on a copy stream while the solver works.

Bar: bit-identical to jp_set_populations followed by the same steps (the staged buffer becomes the
state; every step runs the same kernel on the same inputs).  Calls in between (diagnostics, reads)
see the current state; a pipelined sequence of calls (step, stage the next input, diagnostics)
gives the results of the same calls made one after another; ensemble members take their staged
state; misuse is refused with a status, not a fault."""
import numpy as np
import pytest

import jpsolver as J

pytestmark = pytest.mark.gpu
Q = 19


def perturbed(base, seed):
    rng = np.random.default_rng(seed)
    return (base * (1.0 + 1e-3 * rng.standard_normal(base.shape))).astype(base.dtype)


@pytest.mark.parametrize("n", [16, 48])
def test_staged_state_matches_set_populations(n):
    with J.Solver("uniform", n=n, re=800.0) as a, J.Solver("uniform", n=n, re=800.0) as b:
        f = perturbed(a.get_populations(), 1)
        buf = J.PinnedBuffer(f.size)
        try:
            buf.array[:] = f
            a.step(3)
            a.set_populations(f)
            a.step(5)
            b.step(3)
            b.stage_populations(buf)
            b.step(5)
            np.testing.assert_array_equal(b.get_populations(), a.get_populations())
            assert b.diag() == a.diag()
            assert b.info["step_count"] == a.info["step_count"] == 8
        finally:
            buf.free()


def test_calls_between_stage_and_step_see_the_current_state():
    n = 24
    with J.Solver("uniform", n=n, re=800.0) as s:
        s.step(2)
        before_f, before_d = s.get_populations(), s.diag()
        buf = J.PinnedBuffer(before_f.size)
        try:
            buf.array[:] = perturbed(before_f, 2)
            s.stage_populations(buf)
            assert s.diag() == before_d
            np.testing.assert_array_equal(s.get_populations(), before_f)
            s.step(1)                                         # takes the staged state first
            with J.Solver("uniform", n=n, re=800.0) as r:
                r.step(2)
                r.set_populations(buf.array.copy())
                r.step(1)
                np.testing.assert_array_equal(s.get_populations(), r.get_populations())
        finally:
            buf.free()


def test_explicit_state_discards_staged_populations():
    # init_tgv, set_populations and load_state set the state; an upload staged before them is dropped
    n = 16
    with J.Solver("uniform", n=n, re=800.0) as s, J.Solver("uniform", n=n, re=800.0) as r:
        f0 = s.get_populations()
        g = perturbed(f0, 4)
        buf = J.PinnedBuffer(f0.size)
        try:
            buf.array[:] = perturbed(f0, 5)
            s.stage_populations(buf)
            s.set_populations(g)
            s.step(2)
            r.set_populations(g)
            r.step(2)
            np.testing.assert_array_equal(s.get_populations(), r.get_populations())
            s.stage_populations(buf)
            s.init_tgv()
            s.step(1)
            r.init_tgv()
            r.step(1)
            np.testing.assert_array_equal(s.get_populations(), r.get_populations())
        finally:
            buf.free()


def test_pipelined_calls_match_sequential_calls():
    # per call: the state comes from the host, k steps, diagnostics; pipelined, call i+1's upload is
    # staged right after call i's steps are queued
    n, k, calls = 32, 7, 4
    with J.Solver("uniform", n=n, re=1600.0) as s0:
        base = s0.get_populations()
    inputs = [perturbed(base, 10 + i) for i in range(calls)]
    seq = []
    with J.Solver("uniform", n=n, re=1600.0) as s:
        for f in inputs:
            s.set_populations(f)
            s.step(k)
            seq.append((s.diag(), s.get_populations()))
    bufs = [J.PinnedBuffer(base.size) for _ in range(calls)]
    try:
        for b, f in zip(bufs, inputs):
            b.array[:] = f
        got = []
        with J.Solver("uniform", n=n, re=1600.0) as s:
            s.stage_populations(bufs[0])
            for i in range(calls):
                s.step(k)
                if i + 1 < calls:
                    s.stage_populations(bufs[i + 1])
                got.append((s.diag(), s.get_populations()))
        for (d0, f0), (d1, f1) in zip(seq, got):
            assert d0 == d1
            np.testing.assert_array_equal(f0, f1)
    finally:
        for b in bufs:
            b.free()


def test_ensemble_members_take_their_staged_state():
    cfgs = [dict(n=16, re=400.0), dict(n=24, re=800.0)]
    refs, bufs, solvers = [], [], []
    try:
        for i, c in enumerate(cfgs):
            with J.Solver("uniform", **c) as r:
                f = perturbed(r.get_populations(), 20 + i)
                r.set_populations(f)
                r.step(3)
                refs.append(r.get_populations())
            b = J.PinnedBuffer(f.size)
            b.array[:] = f
            bufs.append(b)
            s = J.Solver("uniform", **c)
            s.stage_populations(b)
            solvers.append(s)
        ens = J.Ensemble()
        for s in solvers:
            ens.add(s)
        ens.step(3)
        for s, ref in zip(solvers, refs):
            np.testing.assert_array_equal(s.get_populations(), ref)
        ens.close()
    finally:
        for s in solvers:
            s.close()
        for b in bufs:
            b.free()


def test_fp64_storage_stages_fp64():
    n = 16
    with J.Solver("uniform", n=n, re=800.0, storage="fp64") as a, \
            J.Solver("uniform", n=n, re=800.0, storage="fp64") as b:
        f = perturbed(a.get_populations(dtype=np.float64), 3)
        buf = J.PinnedBuffer(f.size, dtype=np.float64)
        try:
            buf.array[:] = f
            a.set_populations(f)
            a.step(2)
            b.stage_populations(buf)
            b.step(2)
            np.testing.assert_array_equal(b.get_populations(dtype=np.float64), a.get_populations(dtype=np.float64))
        finally:
            buf.free()


def test_staging_refused_where_unsupported():
    n = 16
    buf = J.PinnedBuffer(Q * n ** 3)
    try:
        with J.Solver("uniform", n=n, re=400.0) as s:
            buf.array[:] = s.get_populations()
            before = s.info["bytes_state"]
            s.stage_populations(buf)
            assert s.info["bytes_state"] == before + buf.nbytes     # the second state buffer
            with pytest.raises(J.JPError) as e:
                s.stage_populations(buf)                            # one staged state at a time
            assert e.value.status == 5
            s.step(1)
            s.stage_populations(buf)                                # free again once taken
            s.step(1)
        with J.Solver("uniform", n=n, re=400.0, storage="fp16") as s:
            with pytest.raises(J.JPError) as e:
                s.stage_populations(buf)                            # FP32 values for 16-bit storage
            assert e.value.status == 7
        with J.Solver("uniform", n=n, re=400.0, flags=J.FLAG_INPLACE) as s:
            with pytest.raises(J.JPError) as e:
                s.stage_populations(buf)
            assert e.value.status == 7
        with J.Solver("amr", n=n, l1_mode="all", l2_mode="all") as s:
            with pytest.raises(J.JPError) as e:
                s.stage_populations(buf)
            assert e.value.status == 7
    finally:
        buf.free()
