"""CPU checks of the uniform oracle (the restatement of src/tgv3d_uniform.cu): invariants that hold
for the reference's algorithm by construction.  The oracle's agreement with the reference's own
kernels is pinned separately against golden fixtures (test_oracle_golden.py)."""
import numpy as np
import oracle as O
import pytest

Q = 19
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])


def test_layout_round_trip():
    n, mb = 16, 8
    a = np.arange(Q * n ** 3, dtype=np.float32)
    f = O.blocked_to_flat(a, n, mb)
    assert f.shape == (Q, n, n, n)
    np.testing.assert_array_equal(O.flat_to_blocked(f, n, mb), a)
    # cell (x=9, y=2, z=13), q=5 lives in block (1,0,1), cell (1,2,5)
    b = (1 * 2 + 0) * 2 + 1
    c = (5 * mb + 2) * mb + 1
    assert f[5, 13, 2, 9] == a[(b * Q + 5) * mb ** 3 + c]


def test_params_match_reference_formulas():
    p = O.params(64, 400.0)
    assert p["steps"] == 2445  # round(12/(0.05*2pi/64))
    assert abs(p["tau"] - (3 * 0.05 * 64 / (2 * np.pi * 400) + 0.5)) < 1e-15
    assert O.params(512, 1600.0)["steps"] == 19557


def test_init_is_tgv_field():
    n, mb, u0 = 16, 8, 0.05
    f = O.init_tgv(n, mb, u0)
    F = O.macro(f, n, mb).reshape(n, n, n, 4)           # z y x
    x = (np.arange(n) + 0.5) * 2 * np.pi / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    np.testing.assert_allclose(F[..., 1], u0 * np.sin(X) * np.cos(Y) * np.cos(Z), atol=1e-7)
    np.testing.assert_allclose(F[..., 2], -u0 * np.cos(X) * np.sin(Y) * np.cos(Z), atol=1e-7)
    np.testing.assert_allclose(F[..., 3], 0.0, atol=1e-7)
    p = (u0 * u0 / 16) * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2)
    np.testing.assert_allclose(F[..., 0], 1 + 3 * p, atol=3e-7)
    E, ens, mass = O.diag_field(O.macro(f, n, mb), n)
    assert abs(E - u0 * u0 / 8) < 1e-8           # mean 1/2|u|^2 of the TGV field
    assert abs(mass - 1.0) < 1e-7


def test_step_conserves_mass_and_momentum():
    n, mb = 16, 8
    p = O.params(n, 100.0)
    f = O.init_tgv(n, mb, 0.05, np.float64)
    g = O.step(f, n, mb, p["omega_d"], 5)
    fa = O.blocked_to_flat(f, n, mb).reshape(Q, -1)
    ga = O.blocked_to_flat(g, n, mb).reshape(Q, -1)
    assert abs(ga.sum() - fa.sum()) < 1e-9 * fa.sum()
    for c in (CX, CY, CZ):
        assert abs((c[:, None] * ga).sum() - (c[:, None] * fa).sum()) < 1e-10


def test_translation_commutes_with_step_bit_exact():
    # the step is the same operation at every cell of the periodic cube, so shifting the state by whole
    # cells before or after a step gives identical bits
    n, mb = 16, 4
    p = O.params(n, 400.0)
    f = O.init_tgv(n, mb, 0.05)
    ff = O.blocked_to_flat(f, n, mb)
    sh = np.roll(ff, shift=(3, 5, 7), axis=(1, 2, 3))
    a = O.blocked_to_flat(O.step(O.flat_to_blocked(sh, n, mb), n, mb, p["omega"], 2), n, mb)
    b = np.roll(O.blocked_to_flat(O.step(f, n, mb, p["omega"], 2), n, mb), shift=(3, 5, 7), axis=(1, 2, 3))
    np.testing.assert_array_equal(a, b)


def test_block_edge_does_not_change_result():
    # MB only changes the storage order (src/tgv3d_uniform.cu:43-53), not the arithmetic
    n = 16
    p = O.params(n, 400.0)
    a = O.blocked_to_flat(O.step(O.init_tgv(n, 8), n, 8, p["omega"], 3), n, 8)
    b = O.blocked_to_flat(O.step(O.init_tgv(n, 4), n, 4, p["omega"], 3), n, 4)
    np.testing.assert_array_equal(a, b)


def numpy_step(ff, omega):
    """Independent numpy statement of one pull stream-collide step on the flat layout (float64)."""
    fin = np.stack([np.roll(ff[q], shift=(CZ[q], CY[q], CX[q]), axis=(0, 1, 2)) for q in range(Q)])
    rho = fin.sum(0)
    ux = (CX[:, None, None, None] * fin).sum(0) / rho
    uy = (CY[:, None, None, None] * fin).sum(0) / rho
    uz = (CZ[:, None, None, None] * fin).sum(0) / rho
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    cu = 3 * (CX[:, None, None, None] * ux + CY[:, None, None, None] * uy + CZ[:, None, None, None] * uz)
    feq = w[:, None, None, None] * rho * (1 + cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy + uz * uz))
    return fin - omega * (fin - feq)


def test_oracle_step_matches_independent_numpy_step():
    n, mb = 16, 8
    p = O.params(n, 800.0)
    f = O.init_tgv(n, mb, 0.05, np.float64)
    a = O.blocked_to_flat(O.step(f, n, mb, p["omega_d"], 1), n, mb)
    b = numpy_step(O.blocked_to_flat(f, n, mb), p["omega_d"])
    np.testing.assert_allclose(a, b, rtol=1e-13, atol=0)


def test_fp32_oracle_tracks_fp64():
    n, mb = 16, 8
    p = O.params(n, 400.0)
    a = O.step(O.init_tgv(n, mb, 0.05, np.float32), n, mb, p["omega"], 20)
    b = O.step(O.init_tgv(n, mb, 0.05, np.float64), n, mb, p["omega_d"], 20)
    assert np.max(np.abs(a - b) / np.abs(b)) < 1e-5


def test_diag_enstrophy_of_tgv_initial_field():
    # the central difference of sin(k i) over one cell is cos(k i) sin(k): the discrete enstrophy is the
    # continuous one with k replaced by sin(k)
    n, mb, u0 = 32, 8, 0.05
    f = O.init_tgv(n, mb, u0, np.float64)
    E, ens, mass = O.diag(f, n, mb)
    kf = 2 * np.pi / n
    s = np.sin(kf) / kf       # central-difference attenuation of one derivative
    # |curl u|^2 of TGV: omega = u0 k (-cos x sin y sin z, -sin x cos y sin z, 2 sin x sin y cos z);
    # mean 1/2|omega|^2 = 1/2 u0^2 k^2 (1/8 + 1/8 + 4/8) = 3/8 u0^2 k^2
    expect = 3.0 / 8.0 * u0 ** 2 * kf ** 2 * s ** 2
    assert abs(ens - expect) < 1e-3 * expect
