"""r2r transforms (plan_r2r_1d/2d/3d, plan_many_r2r, plan_guru_r2r,
execute_r2r) on the GPU against the oracle's defining sums (double for float
results, long double for double results): float rel L2 <= 1e-6, double <=
1e-14; round trips of each kind with its unnormalized inverse; multi-d r2r as
the separable product of the 1D kinds."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

KINDS = {0: "R2HC", 1: "HC2R", 2: "DHT", 3: "REDFT00", 4: "REDFT01", 5: "REDFT10", 6: "REDFT11", 7: "RODFT00",
         8: "RODFT01", 9: "RODFT10", 10: "RODFT11"}
INVERSE = {0: 1, 1: 0, 2: 2, 3: 3, 4: 5, 5: 4, 6: 6, 7: 7, 8: 9, 9: 8, 10: 10}


def logical(kind, n):
    """The logical DFT size N: the inverse kind undoes a kind up to N."""
    return {3: 2 * (n - 1), 7: 2 * (n + 1)}.get(kind, 2 * n if kind >= 4 else n)


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
    if kind == 3 and n == 1:
        pytest.skip("a size-1 REDFT00 is not defined")
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
    kind on device arrays gives back N x the input (N the logical DFT size:
    n for R2HC/HC2R/DHT, 2(n-1) for REDFT00, 2(n+1) for RODFT00, else 2n)."""
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
    scale = logical(kind, n)
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


def plan_r2r_nd(lib, prec, shape, kinds, inp, out):
    pfx = "fftwf_" if prec == "f" else "fftw_"
    f = getattr(lib, pfx + "plan_r2r")
    f.restype = ctypes.c_void_p
    r = len(shape)
    p = f(r, (ctypes.c_int * r)(*shape), inp, out, (ctypes.c_int * r)(*kinds), 64)
    assert p, lib.fftw_gb300_last_error()
    return p


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("shape,kinds", [([12, 17], [5, 10]), ([9, 16], [3, 0]), ([6, 9, 10], [3, 2, 7]),
                                         ([8, 5, 4], [6, 1, 9])])
def test_r2r_multid_device(lib, torch_cuda, restatement, prec, shape, kinds):
    """plan_r2r of rank 2 and 3 with a different kind per dim, device arrays."""
    torch = torch_cuda
    tot = int(np.prod(shape))
    rng = np.random.default_rng(tot + sum(kinds))
    x = rng.standard_normal(tot).astype(RT[prec])
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros_like(dx)
    p = plan_r2r_nd(lib, prec, shape, kinds, dx.data_ptr(), dy.data_ptr())
    run(lib, prec, p, dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    op = "d" if prec == "f" else "l"
    ref = restatement.r2r_nd(x.astype(np.float64 if prec == "f" else np.longdouble), shape, kinds, op)
    assert rel_l2(dy.cpu().numpy().astype(np.float64), ref.astype(np.float64)) <= TOL[prec]


def test_r2r_multid_many_host_strided(lib, restatement):
    """plan_many_r2r rank 2 with howmany 3 on pageable host arrays: input
    elements 2 reals apart (inembed pads the rows), output dense; then the
    inverse kinds in place give back N0 N1 x the input."""
    n0, n1, hm = 10, 14, 3
    kinds, inv = [7, 4], [7, 5]
    ie = [n0, 16]
    idist = 2 * n0 * 16 + 5
    rng = np.random.default_rng(50)
    src = rng.standard_normal(idist * hm).astype(np.float32)
    keep = src.copy()
    x = np.stack([src[t * idist: t * idist + 2 * n0 * 16: 2].reshape(n0, 16)[:, :n1] for t in range(hm)])
    y = np.full(n0 * n1 * hm, 3.0, dtype=np.float32)
    f = lib.fftwf_plan_many_r2r
    f.restype = ctypes.c_void_p
    nn = (ctypes.c_int * 2)(n0, n1)
    p = f(2, nn, hm, src.ctypes.data, (ctypes.c_int * 2)(*ie), 2, idist, y.ctypes.data, None, 1, n0 * n1,
          (ctypes.c_int * 2)(*kinds), 64)
    assert p, lib.fftw_gb300_last_error()
    run(lib, "f", p, src.ctypes.data, y.ctypes.data)
    assert np.array_equal(src, keep)
    ref = restatement.r2r_nd(x.astype(np.float64).ravel(), [n0, n1], kinds, "d")
    assert rel_l2(y.astype(np.float64), ref) <= 1e-6
    q = f(2, nn, hm, y.ctypes.data, None, 1, n0 * n1, y.ctypes.data, None, 1, n0 * n1, (ctypes.c_int * 2)(*inv), 64)
    assert q, lib.fftw_gb300_last_error()
    run(lib, "f", q, y.ctypes.data, y.ctypes.data)
    scale = logical(7, n0) * logical(4, n1)
    assert rel_l2(y.astype(np.float64) / scale, x.ravel().astype(np.float64)) <= 2e-6


def test_r2r_guru_rank2_in_place_device(lib, torch_cuda, restatement):
    """plan_guru_r2r rank 2 (REDFT11 x R2HC) with one howmany dim, in place on a device array."""
    torch = torch_cuda
    n0, n1, hm = 16, 24, 2
    rng = np.random.default_rng(51)
    x = rng.standard_normal(n0 * n1 * hm)
    dx = torch.from_numpy(x.copy()).cuda()

    class IoDim(ctypes.Structure):
        _fields_ = [("n", ctypes.c_int), ("is_", ctypes.c_int), ("os", ctypes.c_int)]
    dims = (IoDim * 2)(IoDim(n0, n1, n1), IoDim(n1, 1, 1))
    hdims = (IoDim * 1)(IoDim(hm, n0 * n1, n0 * n1))
    f = lib.fftw_plan_guru_r2r
    f.restype = ctypes.c_void_p
    p = f(2, dims, 1, hdims, dx.data_ptr(), dx.data_ptr(), (ctypes.c_int * 2)(6, 0), 64)
    assert p, lib.fftw_gb300_last_error()
    run(lib, "d", p, dx.data_ptr(), dx.data_ptr())
    torch.cuda.synchronize()
    ref = restatement.r2r_nd(x.astype(np.longdouble), [n0, n1], [6, 0], "l")
    assert rel_l2(dx.cpu().numpy(), ref.astype(np.float64)) <= 1e-14


def test_r2r_rank0_copy(lib, torch_cuda):
    """plan_guru_r2r of rank 0: a copy of the howmany elements (2D howmany
    dims with strides 3 and 2 reals in, dense out), as in the reference."""
    torch = torch_cuda
    rng = np.random.default_rng(52)
    src = rng.standard_normal(3 * 40 * 7).astype(np.float32)
    ds = torch.from_numpy(src).cuda()
    dd = torch.zeros(40 * 7, dtype=torch.float32, device="cuda")

    class IoDim(ctypes.Structure):
        _fields_ = [("n", ctypes.c_int), ("is_", ctypes.c_int), ("os", ctypes.c_int)]
    hdims = (IoDim * 2)(IoDim(40, 21, 7), IoDim(7, 3, 1))
    f = lib.fftwf_plan_guru_r2r
    f.restype = ctypes.c_void_p
    p = f(0, None, 2, hdims, ds.data_ptr(), dd.data_ptr(), None, 64)
    assert p, lib.fftw_gb300_last_error()
    run(lib, "f", p, ds.data_ptr(), dd.data_ptr())
    torch.cuda.synchronize()
    want = src.reshape(40, 21)[:, 0:21:3].ravel()
    assert np.array_equal(dd.cpu().numpy(), want)


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n,hm", [(128, 37), (256, 9), (2048, 5), (4096, 3), (16384, 2), (4096, 4096)])
@pytest.mark.parametrize("inplace", [False, True])
def test_redft10_fused_pass(lib, torch_cuda, restatement, prec, n, hm, inplace):
    """DCT-II of unit-stride rows of a power-of-two length runs as one pass
    (the permuted load, the r2c and the cosine post-twiddle in one kernel):
    against the oracle's defining sum on rows spread over the batch."""
    torch = torch_cuda
    rng = np.random.default_rng(n + hm + inplace)
    x = rng.standard_normal(n * hm).astype(RT[prec])
    dx = torch.from_numpy(x).cuda()
    dy = dx if inplace else torch.zeros_like(dx)
    p = plan_many(lib, prec, n, hm, dx.data_ptr(), dy.data_ptr(), 5)
    pfx = "fftwf_" if prec == "f" else "fftw_"
    sp = getattr(lib, pfx + "sprint_plan")
    sp.restype = ctypes.c_char_p
    sp.argtypes = [ctypes.c_void_p]
    # (a double transform of 8192 complex points takes more shared memory
    # than the bulk-copy kernel has: it keeps the three-kernel form)
    fused = not (prec == "d" and n > 8192)
    assert (b"fused-dct2" in sp(p)) == fused
    before = lib.fftw_gb300_launch_count()
    run(lib, prec, p, dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    if fused:
        assert lib.fftw_gb300_launch_count() - before == 1
    rows = sorted(set(np.linspace(0, hm - 1, min(hm, 8)).astype(int).tolist()))
    y = dy.cpu().numpy().reshape(hm, n)
    xs = x.reshape(hm, n)
    for t in rows:
        xt = xs[t].astype(np.float64 if prec == "f" else np.longdouble)
        if n <= 2048:
            ref = restatement.r2r(xt, n, 5, "d" if prec == "f" else "l")
        else:
            ref = restatement.r2r_fast(xt, n, 5, "d" if prec == "f" else "l", 1)
        assert rel_l2(y[t].astype(np.float64), ref.astype(np.float64)) <= TOL[prec], f"row {t}"
