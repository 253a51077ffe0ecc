"""Executing one plan from several host threads at once.

The reference allows it: "it is safe to execute the same plan in parallel
by multiple threads" through the new-array execute functions
(doc/threads.texi:243-247; a plan is read-only once made,
doc/reference.texi:227).  Here each execute takes the plan's lock while it
enqueues its work, so calls on one plan reach the GPU one whole call after
another and never share the plan's scratch or staging buffers while in
flight.  Four threads x 50 calls on one single-pass plan (4096 x 256) and on
one four-step plan (2^20 x 4, which owns a scratch array), each thread with
its own arrays and alternating between two inputs, every output checked
against the oracle (float tolerance: rel L2 <= 1e-6)."""
import ctypes
import threading

import numpy as np
import pytest

from conftest import rel_l2_f as rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-6
THREADS = 4
CALLS = 50


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _pinned(lib, nbytes):
    ptr = lib.fftwf_malloc(nbytes)
    assert ptr
    arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_ubyte)), shape=(nbytes,)).view(np.complex64)
    return ptr, arr


def _run_threads(work):
    errors = []

    def wrap(t):
        try:
            work(t)
        except BaseException as e:      # reported by the main thread
            errors.append(f"thread {t}: {e!r}")

    ts = [threading.Thread(target=wrap, args=(t,)) for t in range(THREADS)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, "\n".join(errors)


@pytest.mark.parametrize("n,hm", [(4096, 256), (1 << 20, 4)])
def test_same_plan_device_arrays_from_threads(lib, torch_cuda, restatement, n, hm):
    import fftw3_gb300 as g
    torch = torch_cuda
    rng = np.random.default_rng(n + hm)
    xs = [(rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
          for _ in range(2 * THREADS)]
    refs = [restatement.c2c(x.astype(np.complex128), [n], -1, "d", nthreads=8) for x in xs]
    xd = [torch.from_numpy(x).cuda() for x in xs]
    yd = [torch.empty_like(xd[0]) for _ in range(THREADS)]
    p = g.plan_many_dft([n], hm, xd[0].data_ptr(), yd[0].data_ptr(), -1, g.FFTW_ESTIMATE, "f")
    failures0 = lib.fftw_gb300_failures()
    if n > 16384:
        assert len(p.passes()) == 2 and lib.fftwf_gb300_scratch_bytes(p.ptr) > 0

    def work(t):
        for c in range(CALLS):
            k = 2 * t + (c & 1)
            # a synchronous execute: returns once the transform is done
            p.execute_dft(xd[k].data_ptr(), yd[t].data_ptr())
            y = yd[t].cpu().numpy()
            e = rel_l2(y, refs[k])
            assert e <= TOL, f"call {c}: rel L2 {e:.3e}"

    _run_threads(work)
    assert lib.fftw_gb300_failures() == failures0


@pytest.mark.parametrize("n,hm", [(4096, 256), (1 << 20, 4)])
def test_same_plan_host_arrays_from_threads(lib, torch_cuda, restatement, n, hm):
    """Host arrays: page-locked ones go straight through the kernel for a
    single-pass plan; a multi-pass plan stages them through the plan's
    device buffers, which concurrent calls must not share."""
    import fftw3_gb300 as g
    rng = np.random.default_rng(7 * n + hm)
    xs = [(rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
          for _ in range(2 * THREADS)]
    refs = [restatement.c2c(x.astype(np.complex128), [n], -1, "d", nthreads=8) for x in xs]
    nbytes = xs[0].nbytes
    ins = [_pinned(lib, nbytes) for _ in range(2 * THREADS)]
    outs = [_pinned(lib, nbytes) for _ in range(THREADS)]
    for (ptr, arr), x in zip(ins, xs):
        arr[:] = x
    p = g.plan_many_dft([n], hm, ins[0][0], outs[0][0], -1, g.FFTW_ESTIMATE, "f")
    failures0 = lib.fftw_gb300_failures()

    def work(t):
        for c in range(CALLS):
            k = 2 * t + (c & 1)
            p.execute_dft(ins[k][0], outs[t][0])
            e = rel_l2(outs[t][1], refs[k])
            assert e <= TOL, f"call {c}: rel L2 {e:.3e}"

    try:
        _run_threads(work)
        assert lib.fftw_gb300_failures() == failures0
    finally:
        p.destroy()
        for ptr, _ in ins + outs:
            lib.fftwf_free(ptr)
