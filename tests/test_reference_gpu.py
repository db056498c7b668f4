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


@pytest.mark.parametrize("n,steps", [(16, 1), (24, 10), (32, 50)])
def test_engine_matches_reference_kernel(n, steps):
    p = O.params(n, 1600.0)
    f0 = O.ref_init(n)
    with J.Solver("uniform", n=n, re=1600.0) as s:
        s.set_populations(f0, layout="blocked")
        s.step(steps)
        a = s.get_populations(layout="blocked")
    b = O.ref_run(f0, n, p["omega"], steps)
    assert rel_err(a, b) < 1e-5


def test_engine_init_matches_reference_kernel():
    n = 32
    with J.Solver("uniform", n=n, re=1600.0) as s:
        a = s.get_populations(layout="blocked")
    assert rel_err(a, O.ref_init(n)) < 1e-6
