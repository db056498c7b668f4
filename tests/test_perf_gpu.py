"""Speed against the reference's own CUDA kernels rerun on the same GB300 (compiled from its checkout
into oracle/_ref/*.cubin).  Run with -s to see the figures:

    python -m pytest tests/test_perf_gpu.py -m gpu -s

The engine must beat the reference on its own hot path: the uniform k_step (src/tgv3d_uniform.cu:41)
and the AMR base_step launch sequence (src/tgv3d_amr.cu:821-837)."""
import time

import pytest

import jpsolver as J
import oracle as O

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_amr_available(), reason="reference cubins / librefrun.so not built")]


def engine_uniform_glups(n, steps, storage="fp32"):
    with J.Solver("uniform", n=n, re=1600.0, storage=storage) as s:
        s.step(3)
        s.sync()
        ms = s.step_timed(steps)
    return n ** 3 * steps / (ms / 1e3) / 1e9


@pytest.mark.parametrize("n", [128, 256])
def test_uniform_step_faster_than_reference_kernel(n):
    steps = 20
    p = O.params(n, 1600.0)
    ref_ms = O.ref_time(n, p["omega"], 3, steps)
    ref = n ** 3 * steps / (ref_ms / 1e3) / 1e9
    eng = engine_uniform_glups(n, steps)
    eng16 = engine_uniform_glups(n, steps, "fp16")
    print("\nuniform N=%d: reference k_step %.2f GLUPS (%.0f GB/s), engine fp32 %.2f GLUPS (%.0f GB/s, %.2fx), "
          "engine fp16 %.2f GLUPS (%.2fx)" % (n, ref, ref * 152, eng, eng * 152, eng / ref, eng16, eng16 / ref))
    assert eng > ref


@pytest.mark.parametrize("n,l1,l2", [(32, "all", "all"), (64, "all", "all")])
def test_amr_step_faster_than_reference_kernels(n, l1, l2):
    steps = 10
    r = O.AmrBackend("reference", n, 800.0, l1, l2, budget=1024.0 * 2 ** 30)
    c = r.counts()
    import ctypes
    ms = ctypes.c_float()
    rc = O.ref_amr().ref_amr_time(ctypes.c_void_p(r.h), 2, steps, ctypes.byref(ms))
    assert rc == 0
    work = (c["cnb0"] + 2 * c["nf1"] + 4 * c["nf2"]) * 512 * steps
    ref = work / (ms.value / 1e3) / 1e9
    r.close()
    with J.Solver("amr", n=n, re=800.0, l1_mode=l1, l2_mode=l2) as e:
        e.step(2)
        e.sync()
        ems = e.step_timed(steps)
        ce = e.counts()
    eng = (ce["cnb0"] + 2 * ce["nf1"] + 4 * ce["nf2"]) * 512 * steps / (ems / 1e3) / 1e9
    with J.Solver("amr", n=n, re=800.0, l1_mode=l1, l2_mode=l2, flags=J.FLAG_GRAPH) as g:
        g.step(2)
        g.sync()
        gms = g.step_timed(steps)
    geng = (ce["cnb0"] + 2 * ce["nf1"] + 4 * ce["nf2"]) * 512 * steps / (gms / 1e3) / 1e9
    print("\namr N0=%d %s/%s (L1=%d L2=%d blocks): reference %.2f GLUPS(work), engine %.2f (%.2fx), engine+graph %.2f "
          "(%.1f%% of the FP32 roofline at 152 B/update)" % (n, l1, l2, ce["nf1"], ce["nf2"], ref, eng, eng / ref, geng,
                                                             100 * geng * 152 / 6787.6))
    assert eng > ref
