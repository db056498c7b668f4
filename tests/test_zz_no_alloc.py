"""jp_diag_field_noalloc: the diagnostics entry point for callers that cannot allocate device memory
(a framework that owns all device memory through its own pool, a loop that must not allocate after
start-up).  Through the C ABI it must give the same energy, enstrophy and mass as the solver's own
jp_diag, on two calls in a row (the fixed scratch array keeps the previous call's contents), refuse
buffers that are not device memory and a field larger than its scratch can reduce, and keep working
after the device's context was replaced.

The caller's buffers come from PyTorch here: the entry point itself allocates nothing.  Collected
last (file name) so that a failure here does not hide the other tests."""
import ctypes

import numpy as np
import pytest

import jpsolver as J

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def call(field, n, float_diff, out):
    stream = torch.cuda.current_stream().cuda_stream
    return J.lib().jp_diag_field_noalloc(ctypes.c_void_p(field.data_ptr()), n, float_diff,
                                         ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))


@pytest.mark.parametrize("n,storage", [(32, "fp32"), (48, "fp16")])
def test_noalloc_diag_matches_jp_diag_on_two_calls(n, storage):
    with J.Solver("uniform", n=n, re=800.0, storage=storage) as s:
        s.step(25)
        expect = s.diag()                                  # the solver's own entry point
        field = torch.from_numpy(s.macro().reshape(-1).copy()).cuda()
    out = torch.full((3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(-1.0)
        assert call(field, n, 1, out) == 0, J.lib().jp_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for x, y in zip(got, expect):
            assert abs(x - y) <= 1e-12 * abs(y)            # same per-cell FP64 terms, other summation order


def test_noalloc_diag_rejects_field_beyond_scratch():
    field = torch.zeros(4 * 8, dtype=torch.float32, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    assert call(field, 646, 1, out) == 3                   # JP_ERR_CAPACITY, checked before any launch
    assert b"645" in J.lib().jp_last_error()
    torch.cuda.synchronize()


def test_noalloc_diag_rejects_host_buffers():
    # a host pointer would fault in the kernel: refused before any launch, nothing written
    host_field = np.zeros(4 * 16 ** 3, dtype=np.float32)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    st = J.lib().jp_diag_field_noalloc(ctypes.c_void_p(host_field.ctypes.data), 16, 1, ctypes.c_void_p(out.data_ptr()),
                                       None)
    assert st == 1 and b"not device memory" in J.lib().jp_last_error()
    field = torch.zeros(4 * 16 ** 3, dtype=torch.float32, device="cuda")
    host_out = np.zeros(3)
    st = J.lib().jp_diag_field_noalloc(ctypes.c_void_p(field.data_ptr()), 16, 1, ctypes.c_void_p(host_out.ctypes.data),
                                       None)
    assert st == 1 and b"not device memory" in J.lib().jp_last_error()
    torch.cuda.synchronize()


RESET_SCRIPT = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import jpsolver as J
L = J.lib()
rt = ctypes.CDLL("libcudart.so.13")
n = 16
rng = np.random.default_rng(3)
F = np.empty((n ** 3, 4), dtype=np.float32)
F[:, 0] = 1.0 + 0.01 * rng.standard_normal(n ** 3)
F[:, 1:] = 0.05 * rng.standard_normal((n ** 3, 3))
res = []
for rnd in range(2):
    f, o = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(f), ctypes.c_size_t(F.nbytes)) == 0
    assert rt.cudaMalloc(ctypes.byref(o), ctypes.c_size_t(24)) == 0
    assert rt.cudaMemcpy(f, F.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(F.nbytes), 1) == 0
    assert L.jp_diag_field_noalloc(f, n, 1, o, None) == 0, L.jp_last_error()
    out = np.zeros(3)
    assert rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), o, ctypes.c_size_t(24), 2) == 0
    res.append(out)
    rt.cudaFree(f)
    rt.cudaFree(o)
    if rnd == 0:
        assert rt.cudaDeviceReset() == 0   # the next call runs in a new primary context
assert np.array_equal(res[0], res[1]), res
print("reset ok", res[1])
"""


def test_noalloc_diag_after_context_reset(tmp_path):
    # in a process of its own (no torch): a call, cudaDeviceReset, a call in the new context; the
    # scratch address is looked up again and both calls give the same bits
    import os
    import subprocess
    import sys

    pkg = os.path.dirname(J.__file__)
    script = tmp_path / "reset.py"
    script.write_text(RESET_SCRIPT)
    r = subprocess.run([sys.executable, str(script), pkg], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reset ok" in r.stdout


def fp64_diag(F, n, float_diff):
    """The reference's per-cell arithmetic in FP64 (numpy): 1/2|u|^2, 1/2|curl u|^2 with central
    differences (periodic), rho; float_diff rounds each velocity difference to float first."""
    G = F.reshape(n, n, n, 4)                                   # [k][j][i][comp]

    def dif(comp, axis):                                        # (f(x+1) - f(x-1)) / 2 along axis
        a, b = np.roll(G[..., comp], -1, axis), np.roll(G[..., comp], 1, axis)
        if float_diff:
            return (a - b).astype(np.float64) * 0.5             # float32 subtraction, then widened
        return (a.astype(np.float64) - b.astype(np.float64)) * 0.5

    u, v, w = (G[..., c].astype(np.float64) for c in (1, 2, 3))
    ox = dif(3, 1) - dif(2, 0)                                  # dw/dy - dv/dz
    oy = dif(1, 0) - dif(3, 2)                                  # du/dz - dw/dx
    oz = dif(2, 2) - dif(1, 1)                                  # dv/dx - du/dy
    cells = float(n) ** 3
    return (float(np.sum(0.5 * (u * u + v * v + w * w))) / cells,
            float(np.sum(0.5 * (ox * ox + oy * oy + oz * oz))) / cells,
            float(np.sum(G[..., 0].astype(np.float64))) / cells)


def adversarial_field(kind, n, rng):
    F = np.empty((n ** 3, 4), dtype=np.float32)
    F[:, 0] = 1.0 + 0.01 * rng.standard_normal(n ** 3)
    if kind == "wide":          # signs mixed, magnitudes over six decades from cell to cell
        F[:, 1:] = rng.uniform(-1, 1, (n ** 3, 3)) * 10.0 ** rng.uniform(-6, 0, (n ** 3, 3))
    elif kind == "cancel":      # nearly equal neighbours: differences lose most leading bits
        F[:, 1:] = 0.7 + 1e-6 * rng.standard_normal((n ** 3, 3))
    else:                       # large and small blocks of cells side by side
        F[:, 1:] = np.where(rng.random((n ** 3, 1)) < 0.5, 1e3, 1e-3) * rng.standard_normal((n ** 3, 3))
    return F.reshape(-1)


@pytest.mark.parametrize("kind", ["wide", "cancel", "mixed"])
@pytest.mark.parametrize("float_diff", [1, 0])
def test_double_float_terms_match_fp64_on_adversarial_fields(kind, float_diff):
    # the per-cell terms are carried in double-float (error-free products and sums), the sums in
    # FP64: within 1e-13 relative of the FP64 computation on fields chosen to stress it
    n = 24
    F = adversarial_field(kind, n, np.random.default_rng(5))
    field = torch.from_numpy(F.copy()).cuda()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    assert call(field, n, float_diff, out) == 0, J.lib().jp_last_error().decode()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = fp64_diag(F, n, float_diff)
    for g, w in zip(got, want):
        assert abs(g - w) <= 1e-13 * abs(w), (kind, float_diff, g, w)
