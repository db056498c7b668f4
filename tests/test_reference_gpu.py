"""The reference's own kernels (compiled from its checkout into oracle/_ref/*.cubin) run on the GB300
beside the oracle and the engine.  This pins the oracle to the reference and checks the engine
against the reference directly.  Skipped when the cubins were not built (no reference checkout)."""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_available(), reason="reference cubins / librefrun.so not built")]


def rel_err(a, b):
    b = b.astype(np.float64)
    return float(np.max(np.abs(a.astype(np.float64) - b) / np.abs(b)))


@pytest.mark.parametrize("n", [8, 16, 32])
def test_oracle_init_matches_reference_kernel(n):
    assert rel_err(O.init_tgv(n, 8, 0.05), O.ref_init(n)) < 1e-6


@pytest.mark.parametrize("n,steps", [(16, 1), (16, 20), (32, 5)])
def test_oracle_step_matches_reference_kernel(n, steps):
    p = O.params(n, 400.0)
    f0 = O.ref_init(n)
    a = O.step(f0, n, 8, p["omega"], steps)
    b = O.ref_run(f0, n, p["omega"], steps)
    assert rel_err(a, b) < 1e-5


def test_oracle_macro_matches_reference_kernel():
    n = 16
    p = O.params(n, 400.0)
    f = O.ref_run(O.ref_init(n), n, p["omega"], 10)
    np.testing.assert_array_equal(O.macro(f, n, 8), O.ref_macro(f, n))


@pytest.mark.parametrize("n,steps", [(16, 10), (24, 10), (32, 50)])
def test_engine_matches_reference_kernel_every_step(n, steps):
    # the per-step bar: from the reference's own state at step s, one engine step lands within 1e-5
    # relative of the reference's step s+1, at every s of the trajectory
    p = O.params(n, 1600.0)
    f = O.ref_init(n)
    with J.Solver("uniform", n=n, re=1600.0) as s:
        for _ in range(steps):
            g = O.ref_run(f, n, p["omega"], 1)
            s.set_populations(f, layout="blocked")
            s.step(1)
            assert rel_err(s.get_populations(layout="blocked"), g) < 1e-5
            f = g


@pytest.mark.parametrize("n,steps", [(16, 1), (24, 10), (32, 50)])
def test_engine_trajectory_tracks_reference_kernel(n, steps):
    # free-running trajectories: last-bit differences accumulate (tau ~ 0.5005 over-relaxes, so
    # round-off is not damped); budget 1e-5 + 5e-7 per step
    p = O.params(n, 1600.0)
    f0 = O.ref_init(n)
    with J.Solver("uniform", n=n, re=1600.0) as s:
        s.set_populations(f0, layout="blocked")
        s.step(steps)
        a = s.get_populations(layout="blocked")
    b = O.ref_run(f0, n, p["omega"], steps)
    assert rel_err(a, b) < 1e-5 + 5e-7 * steps


def test_engine_init_matches_reference_kernel():
    n = 32
    with J.Solver("uniform", n=n, re=1600.0) as s:
        a = s.get_populations(layout="blocked")
    assert rel_err(a, O.ref_init(n)) < 1e-6
