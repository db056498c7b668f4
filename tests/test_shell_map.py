"""The compact ghost-shell numbering of the AMR fine blocks (faces + edges, no corners) is a bijection
onto [0, 6 MB^2 + 12 MB), each shell cell maps to the neighbour slot of its offset, and it covers
every cell a D3Q19 pull can reach; the fine steps' pull
addressing (neighbour slot + masked cell) equals the global-coordinate pull.  Host-compiled check of
the device header (no GPU)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = r'''
#include "amr_common.cuh"
#include <cstdio>
#include <set>
template <int MB> int check() {
    const int SH = jp::amr::Geo<MB>::SH;
    std::set<int> seen;
    for (int t = 0; t < SH; ++t) {
        int i, j, k;
        jp::amr::shell_coord<MB>(t, i, j, k);
        if (jp::amr::shell_index<MB>(i, j, k) != t) return 1;
        seen.insert(t);
    }
    if ((int)seen.size() != SH) return 2;
    // the neighbour slot of every shell cell is the slot of its offset from the block
    for (int t = 0; t < SH; ++t) {
        int i, j, k;
        jp::amr::shell_coord<MB>(t, i, j, k);
        const int sx = i < 0 ? 0 : (i >= MB ? 2 : 1), sy = j < 0 ? 0 : (j >= MB ? 2 : 1), sz = k < 0 ? 0 : (k >= MB ? 2 : 1);
        if (jp::amr::shell_slot<MB>(i, j, k) != sz * 9 + sy * 3 + sx || sz * 9 + sy * 3 + sx == 13) return 2;
    }
    for (int k = 0; k < MB; ++k) for (int j = 0; j < MB; ++j) for (int i = 0; i < MB; ++i)
        for (int q = 1; q < 19; ++q) {
            int li = i - jp::cx(q), lj = j - jp::cy(q), lk = k - jp::cz(q);
            bool in = li >= 0 && li < MB && lj >= 0 && lj < MB && lk >= 0 && lk < MB;
            int s = jp::amr::shell_index<MB>(li, lj, lk);
            if (!in && (s < 0 || s >= SH)) return 3;
        }
    // pull_src against the global coordinates of a block at (1,1,1) in a 3^3 grid of blocks
    for (int k = 0; k < MB; ++k) for (int j = 0; j < MB; ++j) for (int i = 0; i < MB; ++i)
        for (int q = 0; q < 19; ++q) {
            const int gi = MB + i - jp::cx(q), gj = MB + j - jp::cy(q), gk = MB + k - jp::cz(q);
            const int e_ref = (gk / MB) * 9 + (gj / MB) * 3 + gi / MB;
            const int sc_ref = ((gk % MB) * MB + gj % MB) * MB + gi % MB;
            int e, sc;
            jp::amr::pull_src<MB>(q, i, j, k, e, sc);
            if (e != e_ref || sc != sc_ref) return 3;
        }
    return 0;
}
int main() { int r = check<4>() | (check<8>() << 2) | (check<16>() << 4); std::printf("%d\n", r); return r; }
'''


@pytest.mark.skipif(shutil.which("g++") is None or not os.path.exists("/usr/local/cuda/include/cuda_runtime.h"),
                    reason="needs g++ and the CUDA headers")
def test_shell_numbering_bijective_and_complete():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "shell.cpp")
        exe = os.path.join(d, "shell")
        open(src, "w").write(SRC)
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "jp-solver_gb300", "csrc"),
                            "-I", "/usr/local/cuda/include", src, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, "shell map check failed with code %s" % out.stdout
