"""Parity of the CUDA path against the oracle, through the C ABI.

Every transform here is planned and executed with the fftw3.h entry points of
libfftw3_gb300 on device (or host) arrays, and compared with the oracle: the
reference's own outputs (golden vectors) or the C restatement of the
reference algorithms run in long double (double results) / double (float
results).  Bounds: relative L2 error <= 1e-6 for float, <= 1e-14 for double,
as the accuracy target of this path states.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden_cases, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f": 1e-6, "d": 1e-14}
CT = {"f": np.complex64, "d": np.complex128}
RT = {"f": np.float32, "d": np.float64}


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    return t.cpu().numpy()


def oracle_c2c(restatement, x, shape, sign, prec):
    return restatement.c2c(x.astype(np.clongdouble if prec == "d" else np.complex128), shape, sign,
                           "l" if prec == "d" else "d", nthreads=4)


def run_c2c(torch, x, shape, sign, prec, howmany):
    import fftw3_gb300 as g
    xi = _dev(torch, x.astype(CT[prec]))
    yo = torch.empty_like(xi)
    p = g.plan_many_dft(list(shape), howmany, xi.data_ptr(), yo.data_ptr(), sign, g.FFTW_ESTIMATE, prec)
    p.execute()
    torch.cuda.synchronize()
    return _host(yo), p


GC = golden_cases()


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("case", GC, ids=[f"{c['kind']}-{'x'.join(map(str, c['shape']))}-s{c['sign']}" for c in GC])
def test_golden(lib, torch_cuda, case, prec):
    """Our library against the reference FFTW's own outputs (golden vectors)."""
    import fftw3_gb300 as g
    torch = torch_cuda
    kind, shape, hm, x = case["kind"], case["shape"], case["howmany"], case["x"]
    if kind == "c2c":
        y, _ = run_c2c(torch, x, shape, case["sign"], prec, hm)
    elif kind == "r2c":
        xi = _dev(torch, x.astype(RT[prec]))
        nc = int(np.prod(shape[:-1])) * (shape[-1] // 2 + 1)
        yo = torch.empty(hm * nc, dtype=torch.complex64 if prec == "f" else torch.complex128, device="cuda")
        p = g.plan_many_dft_r2c(list(shape), hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, prec)
        p.execute()
        y = _host(yo)
    else:
        xi = _dev(torch, x.astype(CT[prec]))
        yo = torch.empty(hm * int(np.prod(shape)), dtype=torch.float32 if prec == "f" else torch.float64, device="cuda")
        p = g.plan_many_dft_c2r(list(shape), hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, prec)
        p.execute()
        y = _host(yo)
    err = rel_l2(y, case["yl"])
    assert err <= TOL[prec], f"rel L2 {err:.3e} > {TOL[prec]}"


POW2 = [1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n", POW2)
def test_c2c_pow2(lib, torch_cuda, restatement, n, prec):
    rng = np.random.default_rng(n)
    hm = max(1, min(64, 65536 // n))
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, _ = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert rel_l2(y, oracle_c2c(restatement, x, [n], sign, prec)) <= TOL[prec]


MIXED = [3, 5, 6, 7, 9, 10, 11, 12, 13, 14, 15, 20, 60, 100, 143, 210, 360, 1000, 1001, 2310, 3000, 6561, 10000]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n", MIXED)
def test_c2c_mixed_radix(lib, torch_cuda, restatement, n, prec):
    rng = np.random.default_rng(n + 1)
    hm = max(1, min(32, 65536 // n))
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, _ = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert rel_l2(y, oracle_c2c(restatement, x, [n], sign, prec)) <= TOL[prec]


PRIMES = [17, 19, 31, 101, 173, 257, 1021, 2039, 4093]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n", PRIMES)
def test_c2c_bluestein(lib, torch_cuda, restatement, n, prec):
    if prec == "d" and n > 2048:
        pytest.skip("double Bluestein convolution above 4096 points is a two-pass plan")
    rng = np.random.default_rng(n + 2)
    hm = 4
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, _ = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert rel_l2(y, oracle_c2c(restatement, x, [n], sign, prec)) <= TOL[prec]


LARGE = [(1 << 15, "f"), (1 << 16, "f"), (1 << 18, "f"), (1 << 20, "f"), (3 << 14, "f"), (60000, "f"),
         (1 << 14, "d"), (1 << 16, "d"), (3 * 5 * 7 * 256, "d")]


@pytest.mark.parametrize("n,prec", LARGE)
def test_c2c_fourstep(lib, torch_cuda, restatement, n, prec):
    rng = np.random.default_rng(n + 3)
    hm = 2
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, p = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert rel_l2(y, oracle_c2c(restatement, x, [n], sign, prec)) <= TOL[prec]


MULTI = [[16, 16], [8, 12], [32, 64], [4, 6, 10], [8, 8, 8], [64, 64, 64], [128, 256], [5, 7, 9], [2, 3, 4, 5]]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("shape", MULTI, ids=["x".join(map(str, s)) for s in MULTI])
def test_c2c_multid(lib, torch_cuda, restatement, shape, prec):
    rng = np.random.default_rng(len(shape) * 100 + shape[0])
    tot = int(np.prod(shape))
    hm = 2
    x = rng.standard_normal(tot * hm) + 1j * rng.standard_normal(tot * hm)
    for sign in (-1, 1):
        y, _ = run_c2c(torch_cuda, x, shape, sign, prec, hm)
        assert rel_l2(y, oracle_c2c(restatement, x, shape, sign, prec)) <= TOL[prec]


COLS4 = [([4096, 16], "f"), ([16384, 8], "f"), ([8192, 64], "f"), ([4096, 1024], "f"),
         ([8192, 128], "d"), ([4096, 64], "d")]


@pytest.mark.parametrize("shape,prec", COLS4, ids=[f"{'x'.join(map(str, s))}-{p}" for s, p in COLS4])
def test_c2c_column_fourstep(lib, torch_cuda, restatement, shape, prec):
    """A long strided axis whose single column pass would move tiles narrower
    than 32 bytes runs as two column passes (four-step, twiddle indexed by a
    vector dimension of the first pass)."""
    import fftw3_gb300 as g
    g.set_dry_run(True)
    try:
        d = g.plan_many_dft(shape, 2, 1 << 20, 1 << 30, prec=prec).describe()
    finally:
        g.set_dry_run(False)
    assert "ld=cols st=cols" in d and "+twiddle" in d
    rng = np.random.default_rng(shape[0] + shape[1])
    tot = int(np.prod(shape))
    x = rng.standard_normal(tot * 2) + 1j * rng.standard_normal(tot * 2)
    for sign in (-1, 1):
        y, _ = run_c2c(torch_cuda, x, shape, sign, prec, 2)
        assert rel_l2(y, oracle_c2c(restatement, x, shape, sign, prec)) <= TOL[prec]


def test_c2c_inplace_3d(lib, torch_cuda, restatement):
    """plan_dft_3d in place, forward then backward (the 3D in-place workload's layout)."""
    import fftw3_gb300 as g
    torch = torch_cuda
    shape = [32, 48, 64]
    rng = np.random.default_rng(5)
    x = (rng.uniform(-1, 1, int(np.prod(shape))) + 1j * rng.uniform(-1, 1, int(np.prod(shape)))).astype(np.complex64)
    a = _dev(torch, x)
    lib_ = g.load()
    pf = g.Plan(lib_.fftwf_plan_dft_3d(*shape, a.data_ptr(), a.data_ptr(), -1, g.FFTW_ESTIMATE), "f")
    pb = g.Plan(lib_.fftwf_plan_dft_3d(*shape, a.data_ptr(), a.data_ptr(), 1, g.FFTW_ESTIMATE), "f")
    pf.execute()
    yf = _host(a)
    assert rel_l2(yf, restatement.c2c(x.astype(np.complex128), shape, -1, "d")) <= 1e-6
    pb.execute()
    back = _host(a) / np.prod(shape)
    assert rel_l2(back, x) <= 1e-6


def test_c2c_inplace_3d_256_forward(lib, torch_cuda, restatement):
    """plan_dft_3d 256^3 in place: the forward transform of the whole array
    against the oracle (the round trip alone cannot see errors that cancel
    between the two directions), then backward / N back to the input."""
    import fftw3_gb300 as g
    torch = torch_cuda
    shape = [256, 256, 256]
    tot = int(np.prod(shape))
    rng = np.random.default_rng(256)
    x = (rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)).astype(np.complex64)
    a = _dev(torch, x)
    lib_ = g.load()
    pf = g.Plan(lib_.fftwf_plan_dft_3d(*shape, a.data_ptr(), a.data_ptr(), -1, g.FFTW_ESTIMATE), "f")
    pb = g.Plan(lib_.fftwf_plan_dft_3d(*shape, a.data_ptr(), a.data_ptr(), 1, g.FFTW_ESTIMATE), "f")
    assert len(pf.passes()) == 3
    pf.execute()
    yf = _host(a).astype(np.complex128)
    ref = restatement.c2c(x.astype(np.complex128), shape, -1, "d", nthreads=8)
    err = float(np.linalg.norm(yf - ref.ravel()) / np.linalg.norm(ref))
    assert err <= 1e-6, f"forward rel L2 {err:.3e}"
    del yf, ref
    pb.execute()
    back = _host(a) / tot
    assert rel_l2(back, x) <= 1e-6


def test_strided_embedded(lib, torch_cuda, restatement):
    """plan_many_dft with istride/idist/inembed/onembed (the advanced layout)."""
    import fftw3_gb300 as g
    torch = torch_cuda
    rng = np.random.default_rng(9)
    n, hm = 64, 12
    # input: howmany interleaved (istride = hm, idist = 1); output: padded rows
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
    xi = _dev(torch, x)
    odist = n + 5
    yo = torch.zeros(hm * odist, dtype=torch.complex64, device="cuda")
    p = g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_ESTIMATE, "f",
                        inembed=[n], istride=hm, idist=1, onembed=[odist], ostride=1, odist=odist)
    p.execute()
    y = _host(yo).reshape(hm, odist)
    ref = restatement.c2c(x.reshape(n, hm).T.copy().astype(np.complex128), [n], -1, "d").reshape(hm, n)
    assert rel_l2(y[:, :n], ref) <= 1e-6
    assert np.all(y[:, n:] == 0), "gaps in the output must stay untouched"
    # 2D with embedded input rows
    n0, n1, emb = 12, 20, 24
    x2 = (rng.standard_normal(n0 * emb) + 1j * rng.standard_normal(n0 * emb)).astype(np.complex64)
    xi = _dev(torch, x2)
    yo = torch.zeros(n0 * n1, dtype=torch.complex64, device="cuda")
    p = g.plan_many_dft([n0, n1], 1, xi.data_ptr(), yo.data_ptr(), 1, g.FFTW_ESTIMATE, "f",
                        inembed=[n0, emb], istride=1, idist=0, onembed=[n0, n1], ostride=1, odist=0)
    p.execute()
    ref = restatement.c2c(x2.reshape(n0, emb)[:, :n1].copy().astype(np.complex128), [n0, n1], 1, "d")
    assert rel_l2(_host(yo), ref) <= 1e-6


R2C_SIZES = [2, 4, 6, 15, 16, 30, 64, 100, 1024, 1000, 4096, 16384, 32768,
             17, 97, 1021, 34, 2042]   # odd and even lengths with a prime factor > 13


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n", R2C_SIZES)
def test_r2c_c2r_1d(lib, torch_cuda, restatement, n, prec):
    import fftw3_gb300 as g
    torch = torch_cuda
    if prec == "d" and n > 16384:
        pytest.skip("double r2c above 16384 points is a two-pass plan")
    rng = np.random.default_rng(n + 4)
    hm = max(1, min(16, 65536 // n))
    nc = n // 2 + 1
    x = rng.standard_normal(n * hm)
    xi = _dev(torch, x.astype(RT[prec]))
    yo = torch.empty(hm * nc, dtype=torch.complex64 if prec == "f" else torch.complex128, device="cuda")
    p = g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, prec)
    p.execute()
    op = "l" if prec == "d" else "d"
    ref = restatement.r2c(x.astype(np.longdouble if prec == "d" else np.float64), [n], op)
    assert rel_l2(_host(yo), ref) <= TOL[prec]
    z = rng.standard_normal(nc * hm) + 1j * rng.standard_normal(nc * hm)
    zi = _dev(torch, z.astype(CT[prec]))
    ro = torch.empty(hm * n, dtype=torch.float32 if prec == "f" else torch.float64, device="cuda")
    q = g.plan_many_dft_c2r([n], hm, zi.data_ptr(), ro.data_ptr(), g.FFTW_ESTIMATE, prec)
    q.execute()
    ref = restatement.c2r(z.astype(np.clongdouble if prec == "d" else np.complex128), [n], op)
    assert rel_l2(_host(ro), ref) <= TOL[prec]


@pytest.mark.parametrize("shape", [[8, 6], [64, 64], [5, 7, 9], [16, 32, 30], [256, 512], [2048, 2048], [4096, 100]],
                         ids=str)
def test_r2c_c2r_multid(lib, torch_cuda, restatement, shape):
    import fftw3_gb300 as g
    torch = torch_cuda
    rng = np.random.default_rng(sum(shape))
    tot = int(np.prod(shape))
    nc = tot // shape[-1] * (shape[-1] // 2 + 1)
    x = rng.standard_normal(tot)
    xi = _dev(torch, x.astype(np.float32))
    yo = torch.empty(nc, dtype=torch.complex64, device="cuda")
    p = g.plan_many_dft_r2c(shape, 1, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, "f")
    p.execute()
    assert rel_l2(_host(yo), restatement.r2c(x, shape, "d")) <= 1e-6
    z = rng.standard_normal(nc) + 1j * rng.standard_normal(nc)
    zi = _dev(torch, z.astype(np.complex64))
    ro = torch.empty(tot, dtype=torch.float32, device="cuda")
    q = g.plan_many_dft_c2r(shape, 1, zi.data_ptr(), ro.data_ptr(), g.FFTW_ESTIMATE, "f")
    q.execute()
    assert rel_l2(_host(ro), restatement.c2r(z, shape, "d")) <= 1e-6


def test_r2c_inplace_padded(lib, torch_cuda, restatement):
    """In-place r2c with rows padded to 2*(n/2+1) reals (api/rdft2-pad.c:33)."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 30, 5
    pad = 2 * (n // 2 + 1)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((hm, n))
    buf = np.zeros((hm, pad), dtype=np.float32)
    buf[:, :n] = x
    a = _dev(torch, buf.ravel())
    p = g.plan_many_dft_r2c([n], hm, a.data_ptr(), a.data_ptr(), g.FFTW_ESTIMATE, "f", idist=pad, odist=pad // 2)
    p.execute()
    y = _host(a).view(np.complex64)
    assert rel_l2(y, restatement.r2c(x.ravel(), [n], "d")) <= 1e-6


def test_host_arrays_staged(lib, torch_cuda, restatement):
    """Host (numpy / fftwf_malloc) arrays go through device staging."""
    import ctypes
    import fftw3_gb300 as g
    rng = np.random.default_rng(12)
    n, hm = 1024, 8
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
    y = np.zeros_like(x)
    p = g.plan_many_dft([n], hm, x.ctypes.data, y.ctypes.data, -1, g.FFTW_ESTIMATE, "f")
    p.execute()
    assert rel_l2(y, restatement.c2c(x.astype(np.complex128), [n], -1, "d")) <= 1e-6
    # fftwf_malloc memory (page-locked), in place
    lib_ = g.load()
    ptr = lib_.fftwf_malloc(x.nbytes)
    buf = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), shape=(2 * n * hm,))
    buf[:] = x.view(np.float32)
    q = g.plan_many_dft([n], hm, ptr, ptr, 1, g.FFTW_ESTIMATE, "f")
    q.execute()
    got = buf.view(np.complex64).copy()
    assert rel_l2(got, restatement.c2c(x.astype(np.complex128), [n], 1, "d")) <= 1e-6
    q.destroy()
    lib_.fftwf_free(ptr)


def test_new_array_execute_and_roundtrip(lib, torch_cuda):
    """execute_dft on new arrays; backward(forward(x)) / N == x."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 4096, 64
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
    a, b = _dev(torch, x), torch.empty(n * hm, dtype=torch.complex64, device="cuda")
    c = torch.empty_like(b)
    pf = g.plan_many_dft([n], hm, a.data_ptr(), b.data_ptr(), -1, g.FFTW_ESTIMATE, "f")
    pb = g.plan_many_dft([n], hm, a.data_ptr(), b.data_ptr(), 1, g.FFTW_ESTIMATE, "f")
    pf.execute_dft(a.data_ptr(), b.data_ptr())
    pb.execute_dft(b.data_ptr(), c.data_ptr())
    assert rel_l2(_host(c) / n, x) <= 1e-6
    before = g.launch_count()
    pf.execute()
    assert g.launch_count() == before + 1


RADER_PRIMES = [17, 31, 61, 97, 101, 257, 401, 673, 1201, 3001]


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n", RADER_PRIMES)
def test_c2c_rader(lib, torch_cuda, restatement, n, prec, monkeypatch):
    """Primes through Rader's algorithm (dft/rader.c): generator permutation
    and a cyclic convolution of length n-1, against the oracle's Rader."""
    if prec == "d" and 2 * n * 16 > 227 * 1024:
        pytest.skip("double Rader buffers exceed one CTA's shared memory")
    monkeypatch.setenv("FFTW_GB300_PRIME", "rader")
    rng = np.random.default_rng(n + 5)
    hm = 3
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, p = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert "rader" in p.describe()
        ref = np.concatenate([restatement.dft_method(x[i * n:(i + 1) * n].astype(np.clongdouble), sign, 3, "l")
                              for i in range(hm)])
        assert rel_l2(y, ref) <= TOL[prec]


LARGE_BLUESTEIN = [(10007, "f"), (20011, "f"), (2 * 10007, "f"), (5003, "d"), (8191, "d")]


@pytest.mark.parametrize("n,prec", LARGE_BLUESTEIN)
def test_c2c_bluestein_multipass(lib, torch_cuda, restatement, n, prec):
    """Lengths whose convolution exceeds one CTA: chirp multiply, FFT(nb) in
    two passes, spectrum multiply, inverse FFT(nb), chirp multiply."""
    rng = np.random.default_rng(n + 6)
    hm = 2
    x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    for sign in (-1, 1):
        y, p = run_c2c(torch_cuda, x, [n], sign, prec, hm)
        assert "pointwise" in p.describe()
        assert rel_l2(y, oracle_c2c(restatement, x, [n], sign, prec)) <= TOL[prec]


LARGE_REAL = [(1 << 16, "f"), (40000, "f"), (1 << 20, "f"), (1 << 15, "d"), (60000, "d"),
              (4099, "f"), (12297, "f"), (2049, "d"), (4099, "d"), (8198, "d")]


@pytest.mark.parametrize("n,prec", LARGE_REAL)
def test_r2c_c2r_multipass(lib, torch_cuda, restatement, n, prec):
    """Real lengths beyond one CTA: even lengths as a half-length c2c over the
    real array as pairs plus an element-wise hc2c pass; lengths with a prime
    factor > 13 beyond one CTA (4099, 3 x 4099, and in double 2049, 4099,
    2 x 4099) as Bluestein's convolution read from the real array (r2c) or
    the Hermitian-extended half spectrum (c2r)."""
    import fftw3_gb300 as g
    torch = torch_cuda
    rng = np.random.default_rng(n + 7)
    hm = 2
    nc = n // 2 + 1
    x = rng.standard_normal(n * hm)
    xi = _dev(torch, x.astype(RT[prec]))
    yo = torch.empty(hm * nc, dtype=torch.complex64 if prec == "f" else torch.complex128, device="cuda")
    p = g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, prec)
    p.execute()
    op = "l" if prec == "d" else "d"
    ref = restatement.r2c(x.astype(np.longdouble if prec == "d" else np.float64), [n], op, nthreads=4)
    assert rel_l2(_host(yo), ref) <= TOL[prec]
    z = rng.standard_normal(nc * hm) + 1j * rng.standard_normal(nc * hm)
    zi = _dev(torch, z.astype(CT[prec]))
    ro = torch.empty(hm * n, dtype=torch.float32 if prec == "f" else torch.float64, device="cuda")
    q = g.plan_many_dft_c2r([n], hm, zi.data_ptr(), ro.data_ptr(), g.FFTW_ESTIMATE, prec)
    q.execute()
    ref = restatement.c2r(z.astype(np.clongdouble if prec == "d" else np.complex128), [n], op, nthreads=4)
    assert rel_l2(_host(ro), ref) <= TOL[prec]


@pytest.mark.parametrize("prec", ["f", "d"])
def test_r2c_c2r_strided_beyond_one_cta(lib, torch_cuda, restatement, prec):
    """An even length beyond one CTA with a real stride of 2 (r2c input, c2r
    output): not a complex array of pairs, so it runs as the convolution."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 40000, 2
    nc = n // 2 + 1
    rng = np.random.default_rng(77)
    src = rng.standard_normal(2 * n * hm)
    xi = _dev(torch, src.astype(RT[prec]))
    yo = torch.empty(hm * nc, dtype=torch.complex64 if prec == "f" else torch.complex128, device="cuda")
    p = g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE, prec, istride=2, idist=2 * n)
    assert "pointwise" in p.describe()
    p.execute()
    op = "l" if prec == "d" else "d"
    x = src.reshape(hm, 2 * n)[:, ::2].ravel()
    ref = restatement.r2c(x.astype(np.longdouble if prec == "d" else np.float64), [n], op, nthreads=4)
    assert rel_l2(_host(yo), ref) <= TOL[prec]
    z = rng.standard_normal(nc * hm) + 1j * rng.standard_normal(nc * hm)
    zi = _dev(torch, z.astype(CT[prec]))
    ro = torch.zeros(hm * 2 * n, dtype=torch.float32 if prec == "f" else torch.float64, device="cuda")
    q = g.plan_many_dft_c2r([n], hm, zi.data_ptr(), ro.data_ptr(), g.FFTW_ESTIMATE, prec, ostride=2, odist=2 * n)
    q.execute()
    ref = restatement.c2r(z.astype(np.clongdouble if prec == "d" else np.complex128), [n], op, nthreads=4)
    out = _host(ro).reshape(hm, 2 * n)
    assert rel_l2(out[:, ::2].ravel(), ref) <= TOL[prec]
    assert np.all(out[:, 1::2] == 0)


def test_c2r_multid_preserve_input_is_null(lib):
    """Like the reference, a multi-dimensional c2r cannot preserve its input."""
    import fftw3_gb300 as g
    lib_ = g.load()
    n = (ctypes.c_int * 2)(16, 16)
    p = lib_.fftwf_plan_many_dft_c2r(2, n, 1, 1 << 20, None, 1, 16 * 9, 1 << 21, None, 1, 256,
                                     g.FFTW_ESTIMATE | g.FFTW_PRESERVE_INPUT)
    assert not p
    q = lib_.fftwf_plan_many_dft_c2r(1, n, 1, 1 << 20, None, 1, 9, 1 << 21, None, 1, 16,
                                     g.FFTW_ESTIMATE | g.FFTW_PRESERVE_INPUT)
    assert q
    lib_.fftwf_destroy_plan(q)
