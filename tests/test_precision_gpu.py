"""Storage precision pinned: the Taylor-Green run at Re=1600 to t*=12 in FP32, shifted FP16 and shifted
BF16 storage against the same run in FP64 storage, on a GB300.

The reference's gold bar for the enstrophy-peak time is 0.3 t* (docs/validation.md:12-13); the FP16
bar of this engine is 0.05 t* (one diagnostic sample of a fine run).  BF16 keeps 8 bits of mantissa,
so its figures are pinned, not held to the FP16 bar: at N=512 it lands 0.104 t* off the FP64 peak,
at N=256 0.06.  N=128 keeps the test to seconds; the samples are taken every 10 steps (0.0245 t*).
"""
import numpy as np
import pytest

import jpsolver as J

pytestmark = pytest.mark.gpu
N, RE, U0, TSTAR, EVERY = 128, 1600.0, 0.05, 12.0, 10


def run(storage):
    with J.Solver("uniform", n=N, re=RE, u0=U0, tstar=TSTAR, storage=storage) as s:
        steps, kf = s.info["steps"], s.info["kf"]
        rows = []
        for k in range(0, steps + 1, EVERY):
            rows.append((k * U0 * kf,) + tuple(s.diag()))
            if k + EVERY <= steps:
                s.step(EVERY)
    a = np.array(rows)
    i = int(np.argmax(a[:, 2]))
    return {"t": a[:, 0], "E": a[:, 1] / a[0, 1], "Z": a[:, 2], "peak": float(a[i, 0]),
            "drift": float(np.max(np.abs(a[:, 3] - a[0, 3]) / a[0, 3])),
            # the programs' energy test, with the acceptance tests' round-off allowance
            "monotonic": bool(np.all(a[1:, 1] <= a[:-1, 1] * 1.0000001))}


@pytest.fixture(scope="module")
def fp64():
    return run("fp64")


# storage: (peak-t* error bar, energy-curve error bar, mass-drift bar); measured on a GB300: FP32 0.0,
# 1.2e-4, 5.4e-8; FP16 0.0, 8.3e-4, 5.2e-7; BF16 0.0245 (one sample), 2.7e-2, 1.1e-5
BARS = {"fp32": (0.03, 5e-4, 5e-7), "fp16": (0.05, 2e-3, 2e-6), "bf16": (0.075, 0.05, 5e-5)}


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
def test_storage_precision_against_fp64(fp64, storage):
    r = run(storage)
    dpeak = abs(r["peak"] - fp64["peak"])
    dE = float(np.max(np.abs(r["E"] - fp64["E"]) / fp64["E"]))
    print("\n%s N=%d: peak t* %.4f (FP64 %.4f, error %.4f), energy curve max rel error %.2e, mass drift %.2e, "
          "energy decreasing %s" % (storage, N, r["peak"], fp64["peak"], dpeak, dE, r["drift"], r["monotonic"]))
    bar_peak, bar_E, bar_drift = BARS[storage]
    assert 4.0 < fp64["peak"] < 10.0
    assert dpeak <= bar_peak
    assert dE <= bar_E
    assert r["drift"] <= bar_drift
    # whether the energy decreases at every sample is reported only: at N=128, Re=1600 the sampled
    # energy of the FP64 run itself rises by more than round-off between some samples
