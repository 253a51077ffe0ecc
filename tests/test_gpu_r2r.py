"""1D r2r transforms (plan_r2r_1d, plan_many_r2r, execute_r2r) on the GPU
against the oracle's defining sums (long double): float rel L2 <= 1e-6,
double <= 1e-14; round trips of each kind with its unnormalized inverse."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

KINDS = {0: "R2HC", 1: "HC2R", 2: "DHT", 4: "REDFT01", 5: "REDFT10", 8: "RODFT01", 9: "RODFT10"}
INVERSE = {0: 1, 1: 0, 2: 2, 4: 5, 5: 4, 8: 9, 9: 8}
TOL = {"f": 1e-6, "d": 1e-14}
RT = {"f": np.float32, "d": np.float64}


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def plan_many(lib, prec, n, hm, inp, out, kind, istride=1, idist=None, ostride=1, odist=None):
    pfx = "fftwf_" if prec == "f" else "fftw_"
    f = getattr(lib, pfx + "plan_many_r2r")
    f.restype = ctypes.c_void_p
    nn = (ctypes.c_int * 1)(n)
    kk = (ctypes.c_int * 1)(kind)
    p = f(1, nn, hm, inp, None, istride, idist if idist is not None else n, out, None, ostride,
          odist if odist is not None else n, kk, 64)
    assert p, lib.fftw_gb300_last_error()
    return p


def run(lib, prec, p, inp, out):
    pfx = "fftwf_" if prec == "f" else "fftw_"
    getattr(lib, pfx + "execute_r2r").argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    getattr(lib, pfx + "execute_r2r")(p, inp, out)
    getattr(lib, pfx + "destroy_plan").argtypes = [ctypes.c_void_p]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("kind", sorted(KINDS), ids=[KINDS[k] for k in sorted(KINDS)])
@pytest.mark.parametrize("n", [1, 2, 5, 8, 17, 100, 1024])
def test_r2r_device(lib, torch_cuda, restatement, prec, kind, n):
    torch = torch_cuda
    hm = 2
    rng = np.random.default_rng(n + 31 * kind)
    x = rng.standard_normal(n * hm).astype(RT[prec])
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros_like(dx)
    p = plan_many(lib, prec, n, hm, dx.data_ptr(), dy.data_ptr(), kind)
    run(lib, prec, p, dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    ref = restatement.r2r(x.astype(np.float64 if prec == "f" else np.longdouble), n, kind, "d" if prec == "f" else "l")
    assert rel_l2(dy.cpu().numpy().astype(np.float64), ref.astype(np.float64)) <= TOL[prec]


@pytest.mark.parametrize("kind", sorted(KINDS), ids=[KINDS[k] for k in sorted(KINDS)])
def test_r2r_round_trip_and_layouts(lib, torch_cuda, restatement, kind):
    """Strided input (stride 2, distance 2n+1), host output; then the inverse
    kind on device arrays gives back N x the input (N = n, or 2n for the
    DCT/DST pairs)."""
    torch = torch_cuda
    n, hm = 96, 4
    rng = np.random.default_rng(40 + kind)
    src = rng.standard_normal((2 * n + 1) * hm).astype(np.float32)
    x = np.stack([src[t * (2 * n + 1): t * (2 * n + 1) + 2 * n: 2] for t in range(hm)])
    dsrc = torch.from_numpy(src).cuda()
    y = np.zeros(n * hm, dtype=np.float32)
    p = plan_many(lib, "f", n, hm, dsrc.data_ptr(), y.ctypes.data, kind, istride=2, idist=2 * n + 1)
    run(lib, "f", p, dsrc.data_ptr(), y.ctypes.data)
    ref = restatement.r2r(x.astype(np.float64).ravel(), n, kind, "d")
    assert rel_l2(y.astype(np.float64), ref) <= 1e-6
    dy = torch.from_numpy(y).cuda()
    dz = torch.zeros_like(dy)
    q = plan_many(lib, "f", n, hm, dy.data_ptr(), dz.data_ptr(), INVERSE[kind])
    run(lib, "f", q, dy.data_ptr(), dz.data_ptr())
    scale = 2 * n if kind in (4, 5, 8, 9) else n
    assert rel_l2(dz.cpu().numpy().astype(np.float64) / scale, x.ravel().astype(np.float64)) <= 2e-6


def test_r2r_1d_in_place_and_execute(lib, torch_cuda, restatement):
    """plan_r2r_1d in place on a device array, run through fftwf_execute."""
    torch = torch_cuda
    n = 1000
    rng = np.random.default_rng(41)
    x = rng.standard_normal(n).astype(np.float32)
    dx = torch.from_numpy(x.copy()).cuda()
    f = lib.fftwf_plan_r2r_1d
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint]
    p = f(n, dx.data_ptr(), dx.data_ptr(), 5, 64)
    assert p
    lib.fftwf_execute.argtypes = [ctypes.c_void_p]
    lib.fftwf_execute(p)
    torch.cuda.synchronize()
    ref = restatement.r2r(x.astype(np.float64), n, 5, "d")
    assert rel_l2(dx.cpu().numpy().astype(np.float64), ref) <= 1e-6
