"""Host arrays large enough for pipelined staging: the batch is cut into
chunks that are copied in, transformed and copied out on three streams.
This is the path of multi-pass plans on host arrays, and of any plan on
pageable memory (single-pass plans on page-locked arrays read and write
host memory directly).  Checked against the oracle on transforms at chunk
boundaries (first, last, either side of each cut, the shorter last chunk)
and, for the whole batch, against the same plan run on device arrays."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CHUNK_BYTES = 96 << 20     # input bytes per chunk (the executor's constant)


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _pinned(lib, pfx, nbytes, dtype):
    ptr = getattr(lib, pfx + "malloc")(nbytes)
    assert ptr
    arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_ubyte)), shape=(nbytes,)).view(dtype)
    return ptr, arr


def _sample_rows(hm, per_chunk):
    rows = {0, 1, hm - 1, hm - 2}
    for c in range(1, (hm + per_chunk - 1) // per_chunk):
        rows |= {c * per_chunk - 1, c * per_chunk}
    return sorted(r for r in rows if 0 <= r < hm)


@pytest.mark.parametrize("prec,n,hm,inplace", [("f", 65536, 520, False), ("d", 32768, 1100, True),
                                               ("f", 1 << 18, 100, True)])
def test_c2c_pinned_chunks(lib, torch_cuda, restatement, prec, n, hm, inplace):
    import fftw3_gb300 as g
    torch = torch_cuda
    ct = np.complex64 if prec == "f" else np.complex128
    pfx = "fftwf_" if prec == "f" else "fftw_"
    cs = np.dtype(ct).itemsize
    assert n * hm * cs >= 2 * CHUNK_BYTES
    rng = np.random.default_rng(n + hm)
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(ct)
    pin, ain = _pinned(lib, pfx, x.nbytes, ct)
    pout, aout = (pin, ain) if inplace else _pinned(lib, pfx, x.nbytes, ct)
    ain[:] = x
    p = g.plan_many_dft([n], hm, pin, pout, -1, g.FFTW_ESTIMATE, prec)
    assert len(p.passes()) > 1
    p.execute()
    y = aout.copy()
    # whole batch against the same plan on device arrays
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    q = g.plan_many_dft([n], hm, xd.data_ptr(), yd.data_ptr(), -1, g.FFTW_ESTIMATE, prec)
    q.execute()
    assert rel_l2(y, yd.cpu().numpy()) <= (1e-6 if prec == "f" else 1e-14)
    # rows at the chunk boundaries against the oracle
    rows = _sample_rows(hm, max(1, CHUNK_BYTES // (n * cs)))
    xs = x.reshape(hm, n)[rows]
    ref = restatement.c2c(xs.astype(np.complex128 if prec == "f" else np.clongdouble).ravel(), [n], -1,
                          "d" if prec == "f" else "l", nthreads=4)
    tol = 1e-6 if prec == "f" else 1e-14
    assert rel_l2(y.reshape(hm, n)[rows].ravel(), ref) <= tol
    p.destroy()
    getattr(lib, pfx + "free")(pin)
    if not inplace:
        getattr(lib, pfx + "free")(pout)


def test_r2c_inplace_padded_pinned_chunks(lib, torch_cuda, restatement):
    """In-place r2c with FFTW's padded rows (2*(n/2+1) reals per row), a
    length planned as several passes."""
    import fftw3_gb300 as g
    n, hm = 65536, 1000
    pad = 2 * (n // 2 + 1)
    nbytes = hm * pad * 4
    assert nbytes >= 2 * CHUNK_BYTES
    rng = np.random.default_rng(5)
    x = rng.standard_normal((hm, n)).astype(np.float32)
    ptr, buf = _pinned(lib, "fftwf_", nbytes, np.float32)
    buf.reshape(hm, pad)[:, :n] = x
    nn = (ctypes.c_int * 1)(n)
    p = g.Plan(lib.fftwf_plan_many_dft_r2c(1, nn, hm, ptr, None, 1, pad, ptr, None, 1, pad // 2,
                                           g.FFTW_ESTIMATE), "f")
    assert len(p.passes()) > 1
    p.execute()
    y = buf.view(np.complex64).reshape(hm, pad // 2)
    rows = _sample_rows(hm, max(1, CHUNK_BYTES // (pad * 4)))
    ref = restatement.r2c(x[rows].astype(np.float64).ravel(), [n], "d", nthreads=4)
    assert rel_l2(y[rows].ravel(), ref) <= 1e-6
    p.destroy()
    lib.fftwf_free(ptr)


def test_pageable_numpy_chunks(lib, torch_cuda, restatement):
    """Pageable numpy arrays take the same pipelined path."""
    import fftw3_gb300 as g
    n, hm = 2048, 16000
    rng = np.random.default_rng(9)
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
    y = np.zeros_like(x)
    p = g.plan_many_dft([n], hm, x.ctypes.data, y.ctypes.data, 1, g.FFTW_ESTIMATE, "f")
    p.execute()
    rows = _sample_rows(hm, max(1, CHUNK_BYTES // (n * 8)))
    ref = restatement.c2c(x.reshape(hm, n)[rows].astype(np.complex128).ravel(), [n], 1, "d", nthreads=4)
    assert rel_l2(y.reshape(hm, n)[rows].ravel(), ref) <= 1e-6
    # untouched by the transform: the input
    assert np.isfinite(x).all()


def test_whole_extent_staging_repeats(lib, restatement):
    """A multi-pass plan on page-locked host arrays that cannot be cut into
    chunks (one transform) stages the whole extent, on every execute."""
    import fftw3_gb300 as g
    shape = [256, 512]
    tot = 256 * 512
    ptr_in, ain = _pinned(lib, "fftwf_", tot * 8, np.complex64)
    ptr_out, aout = _pinned(lib, "fftwf_", tot * 8, np.complex64)
    p = g.plan_many_dft(shape, 1, ptr_in, ptr_out, -1, g.FFTW_ESTIMATE, "f")
    assert len(p.passes()) > 1
    before = lib.fftw_gb300_failures()
    rng = np.random.default_rng(36)
    for _ in range(3):
        x = (rng.standard_normal(tot) + 1j * rng.standard_normal(tot)).astype(np.complex64)
        ain[:] = x
        p.execute()
        ref = restatement.c2c(x.astype(np.complex128), shape, -1, "d", nthreads=4)
        assert rel_l2(aout.copy(), ref) <= 1e-6
    assert lib.fftw_gb300_failures() == before
    p.destroy()
    lib.fftwf_free(ptr_in)
    lib.fftwf_free(ptr_out)
