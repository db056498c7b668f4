"""In-place (AA pattern) streaming of the uniform cube (JP_FLAG_INPLACE), on a GB300.

Bar: bit-identical to the two-array pull step, which the oracle tests pin.  Every collision of the
AA run sees the same inputs as the pull run and relaxes with the same code, so populations (read
back in the flat order of the two-array step) and diagnostics agree exactly after every step count,
odd (slots swapped in place) and even (populations already moved to where the next step reads
them).  Sizes cover rows held inside one warp (n=16, 32 at 4 cells per thread), rows across warps
(n=256: 64 threads per row), rows that straddle warps unevenly (n=48: 12 threads per row, ten rows
per 128-thread block), and FP64's two cells per thread."""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu
IN = J.FLAG_INPLACE


def pair(kw, steps):
    """(two-array, in-place) populations and diagnostics after `steps` steps."""
    out = []
    for flags in (0, IN):
        with J.Solver("uniform", flags=flags, **kw) as s:
            s.step(steps)
            out.append((s.get_populations(dtype=np.float64), s.diag(), s.info))
    return out


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16", "fp64"])
@pytest.mark.parametrize("n", [16, 48])
def test_inplace_matches_two_array_bit_exact(storage, n):
    kw = dict(n=n, re=800.0, storage=storage)
    for steps in (0, 1, 2, 5):
        (fa, da, ia), (fb, db, ib) = pair(kw, steps)
        np.testing.assert_array_equal(fb, fa, err_msg="%s n=%d after %d steps" % (storage, n, steps))
        assert db == da, (storage, n, steps)
        assert ib["bytes_state"] * 2 == ia["bytes_state"]


@pytest.mark.parametrize("n,tpb", [(32, 128), (64, 256), (256, 128)])
def test_inplace_row_mappings(n, tpb):
    # n=32: one row per warp; 64 at 256 threads: 16 threads per row, 16 rows per block; 256: each row
    # spans two warps, the vector-edge values crossing warps through shared memory
    kw = dict(n=n, re=1600.0, threads_per_block=tpb)
    (fa, da, _), (fb, db, _) = pair(kw, 3)
    np.testing.assert_array_equal(fb, fa)
    assert db == da


def test_inplace_matches_oracle():
    n = 32
    p = O.params(n, 400.0)
    with J.Solver("uniform", n=n, re=400.0, flags=IN) as s:
        f0 = s.get_populations(layout="blocked")
        s.step(3)
        a = s.get_populations(layout="blocked")
    b = O.step(f0, n, 8, p["omega"], 3)
    assert float(np.max(np.abs(a.astype(np.float64) - b) / np.abs(b))) < 1e-5


def test_inplace_set_populations_then_steps():
    # populations written at an odd step count land in the swapped layout, at an even one shifted
    n = 24
    rng = np.random.default_rng(7)
    with J.Solver("uniform", n=n, re=400.0) as a, J.Solver("uniform", n=n, re=400.0, flags=IN) as b:
        base = a.get_populations()
        for pre in (1, 2):
            f = (base * (1.0 + 1e-3 * rng.standard_normal(base.shape))).astype(np.float32)
            a.step(pre)
            b.step(pre)
            a.set_populations(f)
            b.set_populations(f)
            np.testing.assert_array_equal(b.get_populations(), f)
            a.step(3)
            b.step(3)
            np.testing.assert_array_equal(b.get_populations(), a.get_populations())


@pytest.mark.parametrize("save_flags,load_flags", [(IN, 0), (0, IN), (IN, IN)])
def test_state_files_move_between_layouts(tmp_path, save_flags, load_flags):
    path = str(tmp_path / "s.state")
    kw = dict(n=24, re=800.0)
    with J.Solver("uniform", **kw) as r:
        r.step(12)
        ref = r.get_populations()
    for k in (7, 8):          # odd and even step counts at the save
        with J.Solver("uniform", flags=save_flags, **kw) as a:
            a.step(k)
            a.save_state(path)
        with J.Solver("uniform", flags=load_flags, **kw) as b:
            b.load_state(path)
            b.step(12 - k)
            np.testing.assert_array_equal(b.get_populations(), ref)


def test_ensemble_of_inplace_members_at_mixed_parity():
    cfgs = [dict(n=16, re=400.0), dict(n=24, re=800.0, storage="fp16"), dict(n=32, re=1600.0),
            dict(n=48, re=200.0, storage="bf16")]
    refs = []
    for c in cfgs:
        with J.Solver("uniform", **c) as s:
            s.step(9)
            refs.append(s.get_populations(dtype=np.float64))
    solvers = [J.Solver("uniform", flags=IN, **c) for c in cfgs]
    solvers[0].step(1)
    solvers[2].step(1)          # members at odd and even step counts in the same ensemble step
    ens = J.Ensemble()
    for s in solvers:
        ens.add(s)
    ens.step(8)
    solvers[1].step(1)
    solvers[3].step(1)
    for s, ref, c in zip(solvers, refs, cfgs):
        assert s.info["step_count"] == 9
        np.testing.assert_array_equal(s.get_populations(dtype=np.float64), ref, err_msg=str(c))
    ens.close()
    for s in solvers:
        s.close()


def test_autotune_of_an_inplace_solve_keeps_its_vector_width():
    tuned, lups = J.autotune("uniform", steps=3, n=64, re=400.0, flags=IN)
    assert tuned["vec"] == 4 and tuned["threads_per_block"] in (64, 128, 256, 512) and lups > 0
    with J.Solver("uniform", n=64, re=400.0, flags=IN, threads_per_block=tuned["threads_per_block"]) as s:
        s.step(2)


def test_inplace_refused_where_unsupported():
    with pytest.raises(J.JPError):
        J.Solver("amr", n=16, flags=IN, l1_mode="all", l2_mode="all")
    with pytest.raises(J.JPError):
        J.Solver("uniform", n=16, vec=2, flags=IN)      # FP32 in place runs four cells per thread
