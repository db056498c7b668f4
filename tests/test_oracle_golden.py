"""Pins the CPU oracle to the reference: golden fixtures made by running the reference's OWN kernels
(src/tgv3d_uniform.cu, compiled from its checkout) on a GB300 (tests/golden/make_golden.py).

The oracle restates the reference's float arithmetic without FMA contraction, the reference build
contracts, so values agree to a few ulp (init, macro field) and within 1e-5 relative per step."""
import os

import numpy as np
import oracle as O
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    p = os.path.join(GOLD, name)
    if not os.path.exists(p):
        pytest.skip("fixture %s missing" % name)
    return np.load(p)


def rel_err(a, b):
    return float(np.max(np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.abs(b.astype(np.float64))))


@pytest.mark.parametrize("name", ["uniform_n8.npz", "uniform_n16.npz"])
def test_oracle_init_matches_reference(name):
    g = load(name)
    n = int(g["n"])
    a = O.init_tgv(n, int(g["mb"]), 0.05)
    assert rel_err(a, g["init"]) < 1e-6
    # most values are bit-identical; the rest differ by contraction in the last bits
    assert np.mean(a == g["init"]) > 0.5


def test_oracle_steps_match_reference():
    g = load("uniform_n8.npz")
    n, om = int(g["n"]), float(g["omega"])
    # one step from the reference's own state: the per-step bar
    assert rel_err(O.step(g["init"], n, 8, om, 1), g["step1"]) < 1e-5
    # ten steps: accumulated last-bit differences stay small
    assert rel_err(O.step(g["init"], n, 8, om, 10), g["step10"]) < 2e-5
    g16 = load("uniform_n16.npz")
    assert rel_err(O.step(g16["init"], 16, 8, float(g16["omega"]), 5), g16["step5"]) < 2e-5


def test_oracle_macro_matches_reference_bit_exact():
    g = load("uniform_n8.npz")
    # k_macro's sums have no products to contract: identical bits
    np.testing.assert_array_equal(O.macro(g["step10"], 8, 8), g["macro10"])


def test_oracle_gate_check_pins_mass_of_reference_state():
    g = load("uniform_n16.npz")
    E0, ens0, m0 = O.diag(g["init"], 16, 8)
    E5, ens5, m5 = O.diag(g["step5"], 16, 8)
    assert abs(m5 - m0) / m0 < 1e-6
    assert E5 < E0
