"""Split-array transforms: fftw[f]_plan_guru_split_dft / execute_split_dft
(always the forward DFT of ri + i*ii into ro + i*io) and the r2c / c2r forms
plan_guru_split_dft_r2c / _c2r with execute_split_dft_r2c / _c2r, strides
counted in reals.  Checked against the oracle (float: rel L2 <= 1e-6 vs FP64;
double: <= 1e-14 vs long double) for separate arrays (copy / transform /
copy), arrays that interleave (an ordinary complex, r2c or c2r plan) or
interleave swapped, host and device arrays, strided layouts, in place, and
new-array execute."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f": 1e-6, "d": 1e-14}
RT = {"f": np.float32, "d": np.float64}


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def oracle(restatement, x, shape, prec):
    return restatement.c2c(x.astype(np.clongdouble if prec == "d" else np.complex128), shape, -1,
                           "l" if prec == "d" else "d", nthreads=4)


@pytest.mark.parametrize("prec", ["f", "d"])
def test_split_separate_host_arrays(lib, restatement, prec):
    import fftw3_gb300 as g
    shape, hm = [12, 20], 3
    tot = 240
    rng = np.random.default_rng(31)
    ri = rng.standard_normal(tot * hm).astype(RT[prec])
    ii = rng.standard_normal(tot * hm).astype(RT[prec])
    ro = np.zeros_like(ri)
    io = np.zeros_like(ii)
    p = g.plan_guru_split_dft([(12, 20, 20), (20, 1, 1)], [(hm, tot, tot)], ri.ctypes.data, ii.ctypes.data,
                              ro.ctypes.data, io.ctypes.data, g.FFTW_ESTIMATE, prec)
    assert "split" in p.describe()
    p.execute()
    ref = oracle(restatement, ri.astype(np.float64) + 1j * ii.astype(np.float64), shape, prec)
    assert rel_l2(ro + 1j * io.astype(np.float64), ref) <= TOL[prec]


def test_split_strided_device_arrays_and_new_arrays(lib, torch_cuda, restatement):
    """Input elements 3 reals apart, transforms 3001 apart; output dense."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm, s, dist = 1000, 4, 3, 3001
    rng = np.random.default_rng(32)
    a = rng.standard_normal(dist * hm).astype(np.float32)
    b = rng.standard_normal(dist * hm).astype(np.float32)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    ro = torch.zeros(n * hm, dtype=torch.float32, device="cuda")
    io = torch.zeros_like(ro)
    p = g.plan_guru_split_dft([(n, s, 1)], [(hm, dist, n)], da.data_ptr(), db.data_ptr(), ro.data_ptr(),
                              io.data_ptr(), g.FFTW_ESTIMATE, "f")
    p.execute()
    idx = (np.arange(hm)[:, None] * dist + np.arange(n)[None, :] * s).ravel()
    x = a[idx].astype(np.float64) + 1j * b[idx].astype(np.float64)
    ref = oracle(restatement, x, [n], "f")
    assert rel_l2(ro.cpu().numpy() + 1j * io.cpu().numpy().astype(np.float64), ref) <= 1e-6
    # the same plan on new arrays of the same layout
    a2 = rng.standard_normal(dist * hm).astype(np.float32)
    b2 = rng.standard_normal(dist * hm).astype(np.float32)
    da2, db2 = torch.from_numpy(a2).cuda(), torch.from_numpy(b2).cuda()
    ro2, io2 = torch.zeros_like(ro), torch.zeros_like(io)
    p.execute_split_dft(da2.data_ptr(), db2.data_ptr(), ro2.data_ptr(), io2.data_ptr())
    ref2 = oracle(restatement, a2[idx].astype(np.float64) + 1j * b2[idx].astype(np.float64), [n], "f")
    assert rel_l2(ro2.cpu().numpy() + 1j * io2.cpu().numpy().astype(np.float64), ref2) <= 1e-6


def test_split_in_place(lib, restatement):
    import fftw3_gb300 as g
    n = 4096
    rng = np.random.default_rng(33)
    re = rng.standard_normal(n).astype(np.float32)
    im = rng.standard_normal(n).astype(np.float32)
    x = re.astype(np.float64) + 1j * im.astype(np.float64)
    p = g.plan_guru_split_dft([(n, 1, 1)], [], re.ctypes.data, im.ctypes.data, re.ctypes.data, im.ctypes.data,
                              g.FFTW_ESTIMATE, "f")
    p.execute()
    assert rel_l2(re + 1j * im.astype(np.float64), oracle(restatement, x, [n], "f")) <= 1e-6


@pytest.mark.parametrize("swapped", [False, True])
def test_split_interleaved_views(lib, torch_cuda, restatement, swapped):
    """ii = ri + 1 (or ri = ii + 1) with even strides: an ordinary complex plan."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 2048, 8
    rng = np.random.default_rng(34 + swapped)
    z = rng.standard_normal(2 * n * hm).astype(np.float32)
    dz = torch.from_numpy(z).cuda()
    dy = torch.zeros_like(dz)
    b, o = dz.data_ptr(), dy.data_ptr()
    ri, ii, ro, io = (b + 4, b, o + 4, o) if swapped else (b, b + 4, o, o + 4)
    p = g.plan_guru_split_dft([(n, 2, 2)], [(hm, 2 * n, 2 * n)], ri, ii, ro, io, g.FFTW_ESTIMATE, "f")
    assert "split" not in p.describe()
    p.execute()
    zz = z.reshape(hm, n, 2).astype(np.float64)
    zo = dy.cpu().numpy().reshape(hm, n, 2).astype(np.float64)
    if swapped:
        x, y = zz[..., 1] + 1j * zz[..., 0], zo[..., 1] + 1j * zo[..., 0]
    else:
        x, y = zz[..., 0] + 1j * zz[..., 1], zo[..., 0] + 1j * zo[..., 1]
    assert rel_l2(y.ravel(), oracle(restatement, x.ravel(), [n], "f")) <= 1e-6


def test_split_overlapping_spans_odd_stride(lib, restatement):
    """ii = ri + 1 with an odd stride (3 reals): not an interleaved complex
    array, and the real and imaginary spans overlap inside one buffer."""
    import fftw3_gb300 as g
    n = 1500
    rng = np.random.default_rng(35)
    buf = rng.standard_normal(3 * n + 1).astype(np.float32)
    keep = buf.copy()
    out = np.full(3 * n + 1, 7.0, dtype=np.float32)
    b, o = buf.ctypes.data, out.ctypes.data
    p = g.plan_guru_split_dft([(n, 3, 3)], [], b, b + 4, o, o + 4, g.FFTW_ESTIMATE, "f")
    assert "split" in p.describe()
    p.execute()
    x = keep[0:3 * n:3].astype(np.float64) + 1j * keep[1:3 * n:3].astype(np.float64)
    y = out[0:3 * n:3].astype(np.float64) + 1j * out[1:3 * n:3].astype(np.float64)
    assert rel_l2(y, oracle(restatement, x, [n], "f")) <= 1e-6
    assert np.all(out[2:3 * n:3] == 7.0) and out[-1] == 7.0      # gaps untouched
    assert np.array_equal(buf, keep)                              # input untouched


@pytest.mark.parametrize("prec", ["f", "d"])
def test_split_r2c_separate_host_arrays(lib, restatement, prec):
    """plan_guru_split_dft_r2c, rank 2 with one howmany dim: real input on
    pageable host memory, ro and io separate host arrays (last dim n/2+1)."""
    import fftw3_gb300 as g
    n0, n1, hm = 12, 20, 3
    nc = n1 // 2 + 1
    rng = np.random.default_rng(36)
    x = rng.standard_normal(n0 * n1 * hm).astype(RT[prec])
    ro = np.zeros(n0 * nc * hm, dtype=RT[prec])
    io = np.zeros_like(ro)
    p = g.plan_guru_split_dft_r2c([(n0, n1, nc), (n1, 1, 1)], [(hm, n0 * n1, n0 * nc)], x.ctypes.data,
                                  ro.ctypes.data, io.ctypes.data, g.FFTW_ESTIMATE, prec)
    assert "split-dft-r2c" in p.describe()
    p.execute()
    op = "l" if prec == "d" else "d"
    ref = restatement.r2c(x.astype(np.longdouble if prec == "d" else np.float64), [n0, n1], op)
    assert rel_l2(ro.astype(np.float64) + 1j * io.astype(np.float64), ref.astype(np.complex128)) <= TOL[prec]


@pytest.mark.parametrize("prec", ["f", "d"])
def test_split_c2r_strided_device_and_new_arrays(lib, torch_cuda, restatement, prec):
    """plan_guru_split_dft_c2r: ri / ii elements 3 reals apart on the device,
    dense real output; then execute_split_dft_c2r on new arrays."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 1000, 4
    nc = n // 2 + 1
    dist = 3 * nc + 1
    rng = np.random.default_rng(37)
    idx = (np.arange(hm)[:, None] * dist + np.arange(nc)[None, :] * 3).ravel()
    p = None
    for trial in range(2):
        a = rng.standard_normal(dist * hm).astype(RT[prec])
        b = rng.standard_normal(dist * hm).astype(RT[prec])
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        out = torch.zeros(n * hm, dtype=da.dtype, device="cuda")
        if p is None:
            p = g.plan_guru_split_dft_c2r([(n, 3, 1)], [(hm, dist, n)], da.data_ptr(), db.data_ptr(),
                                          out.data_ptr(), g.FFTW_ESTIMATE, prec)
            assert "split-dft-c2r" in p.describe()
            p.execute()
        else:
            p.execute_split_dft_c2r(da.data_ptr(), db.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        z = a[idx].astype(np.float64) + 1j * b[idx].astype(np.float64)
        op = "l" if prec == "d" else "d"
        ref = restatement.c2r(z.astype(np.clongdouble if prec == "d" else np.complex128), [n], op)
        assert rel_l2(out.cpu().numpy().astype(np.float64), ref.astype(np.float64)) <= TOL[prec]
        assert np.array_equal(da.cpu().numpy(), a)                 # input preserved


def test_split_r2c_c2r_interleaved_views(lib, torch_cuda, restatement):
    """io = ro + 1 (r2c) and ii = ri + 1 (c2r) with even strides: ordinary
    r2c / c2r plans, run through execute_split_dft_r2c / _c2r."""
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 2048, 8
    nc = n // 2 + 1
    rng = np.random.default_rng(38)
    x = rng.standard_normal(n * hm).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros(2 * nc * hm, dtype=torch.float32, device="cuda")
    o = dy.data_ptr()
    p = g.plan_guru_split_dft_r2c([(n, 1, 2)], [(hm, n, 2 * nc)], dx.data_ptr(), o, o + 4, g.FFTW_ESTIMATE, "f")
    assert "split" not in p.describe()
    p.execute_split_dft_r2c(dx.data_ptr(), o, o + 4)
    torch.cuda.synchronize()
    y = dy.cpu().numpy().reshape(hm * nc, 2).astype(np.float64)
    ref = restatement.r2c(x.astype(np.float64), [n], "d")
    assert rel_l2(y[:, 0] + 1j * y[:, 1], ref) <= 1e-6
    dz = torch.zeros(n * hm, dtype=torch.float32, device="cuda")
    q = g.plan_guru_split_dft_c2r([(n, 2, 1)], [(hm, 2 * nc, n)], o, o + 4, dz.data_ptr(), g.FFTW_ESTIMATE, "f")
    assert "split" not in q.describe()
    q.execute()
    torch.cuda.synchronize()
    zc = y[:, 0] + 1j * y[:, 1]
    ref = restatement.c2r(zc, [n], "d")
    assert rel_l2(dz.cpu().numpy().astype(np.float64), ref) <= 1e-6
