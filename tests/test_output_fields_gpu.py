"""Output fields (the VTK payload of --vtk/--frames): Q-criterion, speed and velocity.

Uniform: jp_get_output_fields against the oracle's restatement of the reference program's host writer
(src/tgv3d_uniform.cu:98-121: differences of float field values, widened, gradient and Q in double)
on the engine's own macro field, which is bit-exact with the reference's k_macro.
AMR: jp_get_output_fields on the (4 N0)^3 composite against the reference's own k_composite + k_qspeed
(src/tgv3d_amr.cu:523-536,553-564) run on the same populations and tables.

Bars: speed and velocity bit-exact (the same conversions of the same floats); Q within 1e-6 (uniform)
and 1e-5 (AMR) of max |Q| (FP64 sums that the GPU compiler may contract into fused multiply-adds; the
AMR composite's velocities divide by rho in a different order)."""
import numpy as np
import pytest

import jpsolver as J
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,steps", [(16, 0), (32, 40), (48, 25)])
def test_uniform_output_fields_match_reference_writer(n, steps):
    with J.Solver("uniform", n=n, re=400.0) as s:
        s.step(steps)
        F = s.macro()
        q, sp, v = s.output_fields(velocity=True)
    qo, spo, vo = O.qspeed(F, n)
    np.testing.assert_array_equal(sp, spo)
    np.testing.assert_array_equal(v, vo)
    scale = float(np.max(np.abs(qo)))
    assert scale > 0
    err = float(np.max(np.abs(q.astype(np.float64) - qo))) / scale
    assert err < 1e-6, err


@pytest.mark.skipif(not O.ref_amr_available(), reason="reference AMR cubin / librefrun.so not built")
@pytest.mark.parametrize("n,l1,l2,f1,f2", [(32, "slab", "sensor", 0.35, 0.5), (24, "sensor", "sensor", 0.4, 0.4)])
def test_amr_output_fields_match_reference_kqspeed(n, l1, l2, f1, f2):
    s0, s1 = O.random_sensor_fields(n, seed=5 * n)
    r = O.AmrBackend("reference", n, 800.0, l1, l2, f1, f2, develop=2, budget=1024.0 * 2 ** 30, build=False)
    try:
        r.set_sensor_override(s0, s1)
        r.initial_build()
        r.step(3)
        with J.Solver("amr", n=n, re=800.0, l1_mode=l1, l2_mode=l2, frac1=f1, frac2=f2, develop_steps=2,
                      max_gb=1024.0, flags=J.FLAG_DEFER_INIT) as e:
            e.set_sensor_override(s0, s1)
            e.init_tgv()
            c = e.counts()
            assert c["nf1"] > 0 and c["nf2"] > 0          # the composite draws on all three levels
            for t in ("ref1", "fof1", "l1grid"):
                np.testing.assert_array_equal(e.table(t), r.table(t))
            for lv in range(3):
                e.set_populations(r.pops(lv), level=lv, layout="blocked")
            q, sp = e.output_fields()
        qr, spr = r.qspeed()
    finally:
        r.close()
    scale = float(np.max(np.abs(qr)))
    assert scale > 0
    err_q = float(np.max(np.abs(q.astype(np.float64) - qr))) / scale
    err_s = float(np.max(np.abs(sp.astype(np.float64) - spr) / np.maximum(spr, 1e-30)))
    assert err_q < 1e-5, err_q
    assert err_s < 1e-6, err_s
