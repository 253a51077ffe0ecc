"""fftwf_gb300_dft_1d_noalloc, the entry point that allocates no device
memory: its output must match the plan-based entry point's on the same
inputs (float tolerance: rel L2 <= 1e-6), on calls made back to back while
the library's fixed scratch array still holds the previous call's contents.

Named to be collected last, so that a run stopping at the first failure has
already run every other test.  Passes alone in a fresh process (the first
call does the per-device set-up) and after the other tests."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 21
TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _input(torch, n, howmany, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n * howmany) + 1j * rng.standard_normal(n * howmany)).astype(np.complex64)
    return torch.from_numpy(x).cuda()


def _noalloc(lib, torch, x, y, n, howmany, sign):
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.fftwf_gb300_dft_1d_noalloc(n, howmany, x.data_ptr(), y.data_ptr(), sign, st)
    assert rc == 0, lib.fftw_gb300_last_error()


def _planned(torch, x, n, howmany, sign):
    import fftw3_gb300 as g
    y = torch.empty_like(x)
    p = g.plan_many_dft([n], howmany, x.data_ptr(), y.data_ptr(), sign, g.FFTW_ESTIMATE, "f")
    p.execute()
    torch.cuda.synchronize()
    return y.cpu().numpy()


def test_noalloc_matches_plan_on_consecutive_calls(lib, torch_cuda):
    torch = torch_cuda
    lib.fftwf_gb300_dft_1d_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_int, ctypes.c_void_p]
    lib.fftw_gb300_last_error.restype = ctypes.c_char_p
    # (n, howmany, sign): the first fills the whole fixed scratch; the second
    # repeats its shape on new data; the third changes n and direction
    calls = [(1 << 20, 2, -1), (1 << 20, 2, -1), (4096, 64, 1)]
    xs = [_input(torch, n, hm, 100 + i) for i, (n, hm, _) in enumerate(calls)]
    ys = [torch.empty_like(x) for x in xs]
    _noalloc(lib, torch, xs[0], ys[0], *calls[0])
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _noalloc(lib, torch, xs[1], ys[1], *calls[1])
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    _noalloc(lib, torch, xs[2], ys[2], *calls[2])
    torch.cuda.synchronize()
    # once set up, a call takes no device memory
    assert free1 == free0
    for (n, hm, sign), x, y in zip(calls, xs, ys):
        ref = _planned(torch, x, n, hm, sign)
        err = rel_l2(y.cpu().numpy(), ref)
        assert err <= TOL, f"n={n} howmany={hm} sign={sign}: rel L2 {err:.3e}"


def test_noalloc_in_place_and_limits(lib, torch_cuda):
    torch = torch_cuda
    n, hm = 65536, 32                   # exactly the maximum number of points
    x = _input(torch, n, hm, 7)
    ref = _planned(torch, x, n, hm, -1)
    _noalloc(lib, torch, x, x, n, hm, -1)
    torch.cuda.synchronize()
    assert rel_l2(x.cpu().numpy(), ref) <= TOL
    # beyond the fixed scratch, or an unsupported length: refused, nothing launched
    before = lib.fftw_gb300_launch_count()
    st = torch.cuda.current_stream().cuda_stream
    assert lib.fftwf_gb300_dft_1d_noalloc(n, hm + 1, x.data_ptr(), x.data_ptr(), -1, st) == -1
    assert b"exceeds the fixed scratch" in lib.fftw_gb300_last_error()
    assert lib.fftwf_gb300_dft_1d_noalloc(3 << 12, 1, x.data_ptr(), x.data_ptr(), -1, st) == -1
    assert b"power of two" in lib.fftw_gb300_last_error()
    assert lib.fftwf_gb300_dft_1d_noalloc(1 << 22, 0, x.data_ptr(), x.data_ptr(), -1, st) == -1
    assert lib.fftw_gb300_launch_count() == before
    assert MAX_POINTS == n * hm


@pytest.mark.parametrize("sign", [-1, 1])
def test_noalloc_every_length(lib, torch_cuda, sign):
    """Every length the entry point accepts, one transform each (n = 2^21
    uses the largest twiddle tables, right below the scratch region), and
    2^19 with several transforms; each call follows the previous one on the
    same stream, so every call meets the array as its predecessor left it."""
    torch = torch_cuda
    cases = [(1 << L, 1) for L in range(12, 22)] + [(1 << 19, 4)]
    xs = [_input(torch, n, hm, 300 + 7 * i + (sign > 0)) for i, (n, hm) in enumerate(cases)]
    ys = [torch.empty_like(x) for x in xs]
    for (n, hm), x, y in zip(cases, xs, ys):
        _noalloc(lib, torch, x, y, n, hm, sign)
    torch.cuda.synchronize()
    for (n, hm), x, y in zip(cases, xs, ys):
        ref = _planned(torch, x, n, hm, sign)
        err = rel_l2(y.cpu().numpy(), ref)
        assert err <= TOL, f"n={n} howmany={hm} sign={sign}: rel L2 {err:.3e}"

