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


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    if not O.ref_available():
        sys.exit("reference cubins / librefrun.so missing: run python oracle/build.py on a host with the checkout")
    uniform(a.out)
    print("wrote fixtures to", a.out)
