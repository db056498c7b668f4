"""State files (jp_save_state / jp_load_state): a solve written to disk and continued in a fresh
solver follows the uninterrupted run bit for bit, for the uniform cube in every storage and for the
three-level AMR across later regrids; files of another configuration or truncated files are
refused."""
import os

import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16", "fp64"])
def test_uniform_restart_bit_exact(tmp_path, storage):
    path = str(tmp_path / "u.state")
    kw = dict(n=24, re=800.0, storage=storage)
    with J.Solver("uniform", **kw) as a:
        a.step(7)
        a.save_state(path)
        a.step(5)
        ref = a.get_populations(dtype=np.float64)
        dref = a.diag()
    with J.Solver("uniform", **kw) as b:
        b.load_state(path)
        assert b.info["step_count"] == 7
        b.step(5)
        np.testing.assert_array_equal(b.get_populations(dtype=np.float64), ref)
        assert b.diag() == dref


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_amr_restart_bit_exact_across_regrids(tmp_path, storage):
    path = str(tmp_path / "a.state")
    n = 32
    kw = dict(n=n, re=1600.0, l1_mode="sensor", l2_mode="sensor", frac1=0.3, frac2=0.4, develop_steps=4,
              max_gb=64.0, storage=storage)
    sens = [O.random_sensor_fields(n, seed=50 + r) for r in range(3)]

    def cont(s, start):
        for r in range(start, 3):
            s.set_sensor_override(*sens[r])
            s.regrid()
            s.step(2)
        return [s.get_populations(lv, layout="blocked") for lv in range(3)], s.counts(), s.diag()

    with J.Solver("amr", **kw) as a:
        a.set_sensor_override(*sens[0])
        a.init_tgv()
        a.step(3)
        a.set_sensor_override(*sens[1])
        a.regrid()
        a.step(2)
        a.save_state(path)
        ref = cont(a, 2)
    with J.Solver("amr", **kw) as b:             # a fresh solve on its own initial grid
        b.load_state(path)
        got = cont(b, 2)
    for lv in range(3):
        np.testing.assert_array_equal(got[0][lv], ref[0][lv], err_msg="level %d" % lv)
    assert got[1] == ref[1]
    assert got[2] == ref[2]


def test_state_file_of_another_configuration_is_refused(tmp_path):
    path = str(tmp_path / "x.state")
    with J.Solver("uniform", n=16, re=400.0) as a:
        a.save_state(path)
    with J.Solver("uniform", n=16, re=800.0) as b:
        with pytest.raises(J.JPError) as e:
            b.load_state(path)
        assert e.value.status == 1
    with J.Solver("uniform", n=24, re=400.0) as b:
        with pytest.raises(J.JPError):
            b.load_state(path)
    with open(path, "r+b") as f:                   # truncated payload
        f.truncate(os.path.getsize(path) // 2)
    with J.Solver("uniform", n=16, re=400.0) as b:
        with pytest.raises(J.JPError):
            b.load_state(path)
