"""Generate the golden fixtures of tests/golden/ by running the reference's OWN kernels (compiled from
its checkout into oracle/_ref/*.cubin) on a GPU.  The fixtures pin the CPU oracle to the reference:
tests/test_oracle_golden.py checks the oracle against them on any machine, without a GPU.

    python tests/golden/make_golden.py --out tests/golden

Uniform fixtures (reference kernels k_init_tgv3d, k_step, k_macro of src/tgv3d_uniform.cu, MB=8):
  uniform_n8.npz   N=8,  Re=400:  init, after 1 and 10 steps, macro field after 10 steps
  uniform_n16.npz  N=16, Re=1600: init, after 5 steps
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle as O  # noqa: E402


def uniform(out: str) -> None:
    n, re = 8, 400.0
    p = O.params(n, re)
    f0 = O.ref_init(n)
    f1 = O.ref_run(f0, n, p["omega"], 1)
    f10 = O.ref_run(f0, n, p["omega"], 10)
    F10 = O.ref_macro(f10, n)
    np.savez_compressed(os.path.join(out, "uniform_n8.npz"), n=n, re=re, omega=np.float32(p["omega"]), mb=8,
                        init=f0, step1=f1, step10=f10, macro10=F10)
    n, re = 16, 1600.0
    p = O.params(n, re)
    f0 = O.ref_init(n)
    f5 = O.ref_run(f0, n, p["omega"], 5)
    np.savez_compressed(os.path.join(out, "uniform_n16.npz"), n=n, re=re, omega=np.float32(p["omega"]), mb=8,
                        init=f0, step5=f5)


TABLES = ["ref0", "fof0", "rl0", "l1pcb", "l1oct", "f1pos", "l1grid", "ref1", "fof1", "rl1", "l2pl1", "l2oct",
          "skin0", "skin1"]


def block_sums(f: np.ndarray, mb: int = 8) -> np.ndarray:
    """Per-block, per-population sums in float64: a compact fingerprint of a level's payload."""
    return f.reshape(-1, O.Q, mb ** 3).astype(np.float64).sum(axis=2)


def amr(out: str) -> None:
    """AMR fixtures (reference kernels of src/tgv3d_amr.cu, MB=8, seeded sensor field fed to the
    adaptation): tables after the initial build and after one regrid, per-block sums of each level after
    the build, after one coarse step and after the regrid, and the reference's diagnostics."""
    for n, l1, l2, f1, f2, seed in [(16, "slab", "sensor", 0.35, 0.5, 16), (24, "sensor", "sensor", 0.3, 0.2, 24)]:
        s0, s1 = O.random_sensor_fields(n, seed=seed)
        t0, t1 = O.random_sensor_fields(n, seed=seed + 1)
        r = O.AmrBackend("reference", n, 1600.0, l1, l2, f1, f2, develop=3, budget=1024.0 * 2 ** 30, build=False)
        r.set_sensor_override(s0, s1)
        r.initial_build()
        d = {"n": n, "re": 1600.0, "l1": l1, "l2": l2, "frac1": f1, "frac2": f2, "develop": 3, "seed": seed,
             "sen0": s0, "sen1": s1, "sen0_b": t0, "sen1_b": t1}
        for t in TABLES:
            d["init_" + t] = r.table(t)
        for lv in range(3):
            d["init_sums%d" % lv] = block_sums(r.pops(lv))
        r.step(1)
        for lv in range(3):
            d["step1_sums%d" % lv] = block_sums(r.pops(lv))
        d["step1_diag"] = np.array(r.diag())
        r.set_sensor_override(t0, t1)
        r.regrid()
        for t in TABLES:
            d["regrid_" + t] = r.table(t)
        for lv in range(3):
            d["regrid_sums%d" % lv] = block_sums(r.pops(lv))
        r.close()
        np.savez_compressed(os.path.join(out, "amr_n%d_%s_%s.npz" % (n, l1, l2)), **d)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", choices=["uniform", "amr"], default=None)
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    if not O.ref_available():
        sys.exit("reference cubins / librefrun.so missing: run python oracle/build.py on a host with the checkout")
    if a.only in (None, "uniform"):
        uniform(a.out)
    if a.only in (None, "amr"):
        amr(a.out)
    print("wrote fixtures to", a.out)
