"""Diagnostics of the float storages straight from the populations (k_diag_pop), on a GB300.

The per-cell terms are those of the macro-field path (k_macro's rho and u, float differences of the
uniform program's host loop, src/tgv3d_uniform.cu:172-181), so the energy, enstrophy and mass must
match the oracle's reduction of the solver's own macro field to 1e-12 relative: only the sums differ
(double-float partials in another fixed order, ~1e-13 of the result).  Sizes cover tiles cut by the cube's edge (n not a multiple of the 32 x 16 tile),
a cube smaller than one tile, z chunks with a ragged last chunk, the in-place layouts after odd and
even step counts, the 16-bit storages, and n=256 (many tiles and chunks per CTA)."""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu


def check(s, n, tol=1e-12):
    d = s.diag()
    F = s.macro().reshape(-1)
    e = O.diag_field(F, n)
    for x, y in zip(d, e):
        assert abs(x - y) <= tol * abs(y), (n, d, e)
    return d


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("n", [8, 24, 40, 72])
def test_diag_from_populations_matches_oracle(storage, n):
    with J.Solver("uniform", n=n, re=800.0, storage=storage) as s:
        check(s, n)
        s.step(3)
        check(s, n)


@pytest.mark.parametrize("steps", [1, 2, 5])
@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_inplace_layouts_match_oracle(storage, steps):
    n = 40
    with J.Solver("uniform", n=n, re=800.0, storage=storage, flags=J.FLAG_INPLACE) as s:
        s.step(steps)
        check(s, n)


def test_random_state_and_repeatability():
    # a field far from the Taylor-Green vortex (every velocity component and density varies per cell)
    n = 48
    rng = np.random.default_rng(11)
    with J.Solver("uniform", n=n, re=800.0) as s:
        f = s.get_populations()
        f *= (1.0 + 0.05 * rng.standard_normal(f.size)).astype(np.float32)
        s.set_populations(f)
        a = check(s, n)
        assert s.diag() == a          # fixed summation order: the same bits every call


def pairwise(F, n):
    """The oracle's per-cell terms (float differences halved, then FP64) summed pairwise by numpy:
    at 16.7M cells the reference's sequential FP64 loop is itself off by ~1e-12."""
    F = F.reshape(n, n, n, 4)                       # [z][y][x][rho, ux, uy, uz]
    u, v, w = F[..., 1], F[..., 2], F[..., 3]

    def d(a, axis):                                 # (a[+1] - a[-1]) in float, then halved in FP64
        return (np.roll(a, -1, axis) - np.roll(a, 1, axis)).astype(np.float64) * 0.5

    ox = d(w, 1) - d(v, 0)
    oy = d(u, 0) - d(w, 2)
    oz = d(v, 2) - d(u, 1)
    u64, v64, w64 = (a.astype(np.float64) for a in (u, v, w))
    cells = float(n) ** 3
    return (np.sum(0.5 * (u64 * u64 + v64 * v64 + w64 * w64)) / cells,
            np.sum(0.5 * (ox * ox + oy * oy + oz * oz)) / cells,
            np.sum(F[..., 0].astype(np.float64)) / cells)


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_diag_at_256(storage):
    n = 256
    with J.Solver("uniform", n=n, re=1600.0, storage=storage) as s:
        s.step(4)
        d = s.diag()
        F = s.macro().reshape(-1)
    for x, y in zip(d, pairwise(F, n)):
        assert abs(x - y) <= 1e-12 * abs(y), (d, y)
    for x, y in zip(d, O.diag_field(F, n)):         # the reference's loop, its own rounding included
        assert abs(x - y) <= 1e-11 * abs(y), (d, y)
