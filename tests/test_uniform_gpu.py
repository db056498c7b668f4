"""Parity of the engine's uniform path (through the C ABI) with the oracle, on a GB300.

Tolerances: FP32 populations within 1e-5 relative of the oracle after one step (the bar for FP32
parity); FP64 storage within 1e-12; shifted FP16/BF16 storage within the absolute errors stated per
test against the FP64 oracle.  Integer/index work has no tolerance.
"""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu
Q = 19


def rel_err(a, b):
    return float(np.max(np.abs(a.astype(np.float64) - b) / np.abs(b)))


@pytest.mark.parametrize("n", [8, 16, 24, 32, 48, 64])
def test_init_matches_oracle(n):
    with J.Solver("uniform", n=n, re=400.0) as s:
        a = s.get_populations(layout="blocked")
    b = O.init_tgv(n, 8, 0.05)
    assert rel_err(a, b) < 1e-6          # same float formula, contraction may move a few ulp


@pytest.mark.parametrize("n,steps", [(8, 1), (16, 1), (24, 1), (32, 1), (48, 1), (64, 1), (16, 100), (32, 50)])
def test_fp32_steps_match_oracle(n, steps):
    # 1e-5 relative per step; free-running trajectories add at most 5e-7 per step of last-bit drift
    tol = 1e-5 + 5e-7 * (steps - 1)
    p = O.params(n, 400.0)
    with J.Solver("uniform", n=n, re=400.0) as s:
        f0 = s.get_populations(layout="blocked")
        s.step(steps)
        a = s.get_populations(layout="blocked")
    b = O.step(f0, n, 8, p["omega"], steps)
    assert rel_err(a, b) < tol


@pytest.mark.parametrize("vec,tpb", [(1, 256), (2, 128), (4, 64), (4, 128), (4, 256), (4, 512)])
def test_fp32_thread_mappings_agree(vec, tpb):
    n = 32
    p = O.params(n, 1600.0)
    with J.Solver("uniform", n=n, re=1600.0, vec=vec, threads_per_block=tpb) as s:
        f0 = s.get_populations(layout="blocked")
        s.step(3)
        a = s.get_populations(layout="blocked")
    b = O.step(f0, n, 8, p["omega"], 3)
    assert rel_err(a, b) < 1e-5


@pytest.mark.parametrize("n", [16, 24, 32])
def test_fp64_storage_matches_fp64_oracle(n):
    p = O.params(n, 800.0)
    with J.Solver("uniform", n=n, re=800.0, storage="fp64") as s:
        f0 = s.get_populations(layout="blocked", dtype=np.float64)
        b0 = O.init_tgv(n, 8, 0.05, np.float64)
        assert rel_err(f0, b0) < 1e-14
        s.step(10)
        a = s.get_populations(layout="blocked", dtype=np.float64)
    b = O.step(b0, n, 8, p["omega_d"], 10)
    assert rel_err(a, b) < 1e-12


# one rounding of the largest deviation (|f - w| ~ 1e-2 at u0 = 0.05): 2^-11 (fp16), 2^-8 (bf16)
@pytest.mark.parametrize("storage,atol0,atol", [("fp16", 5e-6, 5e-5), ("bf16", 4e-5, 5e-4)])
def test_shifted_storage_tracks_fp64_oracle(storage, atol0, atol):
    n = 32
    p = O.params(n, 400.0)
    b0 = O.init_tgv(n, 8, 0.05, np.float64)
    with J.Solver("uniform", n=n, re=400.0, storage=storage) as s:
        a0 = s.get_populations(layout="blocked", dtype=np.float64)
        assert np.max(np.abs(a0 - b0)) < atol0          # one rounding of the deviation f - w
        s.step(20)
        a = s.get_populations(layout="blocked", dtype=np.float64)
    b = O.step(b0, n, 8, p["omega_d"], 20)
    print("%s: max |f - f_fp64| after init %.2e, after 20 steps %.2e" % (storage, np.max(np.abs(a0 - b0)),
                                                                      np.max(np.abs(a - b))))
    assert np.max(np.abs(a - b)) < atol


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("vec", [2, 4, 8])
def test_shifted_thread_mappings_agree(storage, vec):
    n = 16
    with J.Solver("uniform", n=n, re=400.0, storage=storage, vec=vec) as s:
        s.step(4)
        a = s.get_populations(layout="flat", dtype=np.float64)
    with J.Solver("uniform", n=n, re=400.0, storage=storage, vec=2, threads_per_block=64) as s:
        s.step(4)
        b = s.get_populations(layout="flat", dtype=np.float64)
    assert np.max(np.abs(a - b)) < 1e-6


@pytest.mark.parametrize("n", [16, 32])
def test_diag_matches_oracle(n):
    with J.Solver("uniform", n=n, re=400.0) as s:
        s.step(25)
        d = s.diag()
        f = s.get_populations(layout="blocked")
        F = s.macro().reshape(-1)
    Fo = O.macro(f, n, 8)
    np.testing.assert_array_equal(F, Fo)       # identical float arithmetic per cell
    e = O.diag_field(Fo, n)
    for x, y in zip(d, e):
        assert abs(x - y) <= 1e-12 * abs(y)      # only the summation order differs


def test_populations_round_trip_bit_exact():
    n = 16
    rng = np.random.default_rng(7)
    with J.Solver("uniform", n=n, re=400.0) as s:
        x = (rng.random(Q * n ** 3, dtype=np.float32) + 0.5).astype(np.float32)
        s.set_populations(x, layout="blocked")
        np.testing.assert_array_equal(s.get_populations(layout="blocked"), x)
        np.testing.assert_array_equal(s.get_populations(layout="flat"), O.blocked_to_flat(x, n, 8).reshape(-1))
        s.set_populations(x, layout="flat")
        np.testing.assert_array_equal(s.get_populations(layout="flat"), x)


def test_pinned_host_round_trip_and_step():
    n = 32
    with J.Solver("uniform", n=n, re=400.0) as s:
        f0 = s.get_populations()
        buf = J.PinnedBuffer(f0.size)
        buf.array[:] = f0
        s.set_populations(buf.array)
        s.step(2)
        a = s.get_populations()
        buf.free()
    with J.Solver("uniform", n=n, re=400.0) as s:
        s.step(2)
        b = s.get_populations()
    np.testing.assert_array_equal(a, b)


def test_large_state_round_trip_in_stream_order():
    # 1.27 GB of FP32 populations through pinned memory: the read-back follows the steps before it,
    # the write precedes the steps after it (asynchronous, in the solver's stream order)
    n = 256
    with J.Solver("uniform", n=n, re=1600.0) as a, J.Solver("uniform", n=n, re=1600.0) as b:
        a.step(3)
        buf = J.PinnedBuffer(Q * n ** 3)
        try:
            assert J.lib().jp_get_populations(a.h, 0, 0, 0, J.C.c_void_p(buf.ptr.value), buf.array.size) == 0
            ref = buf.array.copy()
            b.step(1)                          # b's own state, overwritten below in stream order
            assert J.lib().jp_set_populations(b.h, 0, 0, 0, J.C.c_void_p(buf.ptr.value), buf.array.size) == 0
            b.step(2)
            a.step(2)
            np.testing.assert_array_equal(b.get_populations(), a.get_populations())
            np.testing.assert_array_equal(ref, buf.array)
        finally:
            buf.free()


def test_step_counter_and_reinit():
    with J.Solver("uniform", n=16, re=400.0) as s:
        f0 = s.get_populations()
        s.step(7)
        assert s.info["step_count"] == 7
        s.init_tgv()
        assert s.info["step_count"] == 0
        np.testing.assert_array_equal(s.get_populations(), f0)


def test_nan_populations_are_visible_in_diag():
    # fault injected on the host: a NaN population must surface in the diagnostics (the reference's
    # gate checks isfinite, src/tgv3d_uniform.cu:199)
    n = 16
    with J.Solver("uniform", n=n, re=400.0) as s:
        f = s.get_populations()
        f[12345] = np.nan
        s.set_populations(f)
        s.step(1)
        d = s.diag()
    assert not np.isfinite(d[0]) or not np.isfinite(d[1])


def test_full_size_512_conserves_mass():
    # size-independent properties at the benchmark size: mass is conserved to FP32 round-off, the
    # energy decays, and the TGV's mean velocity stays zero
    with J.Solver("uniform", n=512, re=1600.0) as s:
        e0, z0, m0 = s.diag()
        assert abs(e0 - 0.05 ** 2 / 8) < 1e-8
        s.step(20)
        e1, z1, m1 = s.diag()
    assert abs(m1 - m0) / m0 < 2e-6                 # FP32 round-off of 20 steps on 1.3e8 cells
    assert e1 < e0
    assert z1 > 0


def test_autotune_picks_a_supported_mapping_that_matches_oracle():
    # the tuner times the candidate (vec, threads/block) pairs and hands back one of them; a solver
    # built with it steps like the oracle
    n = 64
    tuned, lups = J.autotune("uniform", steps=3, n=n, re=1600.0)
    assert tuned["vec"] in (1, 2, 4, 8) and tuned["threads_per_block"] in (64, 128, 256, 512)
    assert lups > 0
    p = O.params(n, 1600.0)
    with J.Solver("uniform", n=n, re=1600.0, vec=tuned["vec"], threads_per_block=tuned["threads_per_block"]) as s:
        f0 = s.get_populations(layout="blocked")
        s.step(2)
        a = s.get_populations(layout="blocked")
    assert rel_err(a, O.step(f0, n, 8, p["omega"], 2)) < 1.1e-5


def test_deferred_init_refuses_steps_until_initialised():
    # JP_FLAG_DEFER_INIT: the solver allocates only; stepping or diagnosing before jp_init_tgv is a
    # state error, after it the solver is the one jp_create would have made
    with J.Solver("uniform", n=16, re=400.0, flags=J.FLAG_DEFER_INIT) as s:
        with pytest.raises(J.JPError) as e:
            s.step(1)
        assert e.value.status == 5
        with pytest.raises(J.JPError):
            s.diag()
        s.init_tgv()
        s.step(3)
        a = s.get_populations()
    with J.Solver("uniform", n=16, re=400.0) as r:
        r.step(3)
        np.testing.assert_array_equal(a, r.get_populations())
