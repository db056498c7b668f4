"""jp_diag_field_noalloc: the diagnostics entry point for callers that cannot allocate device memory
(a framework that owns all device memory, a loop that must not allocate after start-up, graph
capture).  Through the C ABI it must give the same energy, enstrophy and mass as the solver's own
jp_diag, on two calls in a row (the fixed scratch array keeps the previous call's contents), and
reject a field larger than its scratch can reduce.

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
