"""Plan sets: many c2c plans of uneven lengths run as one work-queue kernel
launch (captured in a CUDA graph), checked transform by transform against
the oracle and against executing the same plans one by one."""
import ctypes
import os
import sys

import numpy as np
import pytest

from conftest import rel_l2, rel_l2_f

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _make_set(torch, lengths, prec="f", sign=-1, seed=0):
    import fftw3_gb300 as g
    ct = torch.complex64 if prec == "f" else torch.complex128
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    xin = torch.randn(int(offs[-1]), dtype=ct, device="cuda", generator=gen)
    yout = torch.zeros_like(xin)
    es = xin.element_size()
    plans = []
    for i, n in enumerate(lengths):
        p = g.plan_many_dft([int(n)], 1, xin.data_ptr() + int(offs[i]) * es, yout.data_ptr() + int(offs[i]) * es,
                            sign, g.FFTW_ESTIMATE, prec)
        plans.append(p)
    return xin, yout, offs, plans


def _check(restatement, xin, yout, offs, lengths, prec, sign, sample=None):
    x = xin.cpu().numpy()
    y = yout.cpu().numpy()
    tol = 1e-6 if prec == "f" else 1e-14
    idx = range(len(lengths)) if sample is None else sample
    worst = 0.0
    for i in idx:
        a, b = int(offs[i]), int(offs[i + 1])
        xo = x[a:b].astype(np.clongdouble if prec == "d" else np.complex128)
        ref = restatement.c2c(xo, [b - a], sign, "l" if prec == "d" else "d")
        e = (rel_l2_f if prec == "f" else rel_l2)(y[a:b], ref)
        worst = max(worst, e)
        assert e <= tol, f"transform {i} (n={b - a}): rel L2 {e:.3e}"
    return worst


def _set_of(plans, prec, flags=None):
    import fftw3_gb300 as g
    lib = g.load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    arr = (ctypes.c_void_p * len(plans))(*[p.ptr for p in plans])
    f = getattr(lib, pfx + "gb300_plan_set")
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint]
    s = f(len(plans), arr, g.FFTW_ESTIMATE if flags is None else flags)
    assert s, g.last_error()
    getattr(lib, pfx + "gb300_execute_set").argtypes = [ctypes.c_void_p]
    getattr(lib, pfx + "gb300_destroy_set").argtypes = [ctypes.c_void_p]
    return lib, pfx, s


@pytest.mark.parametrize("prec", ["f", "d"])
def test_planset_mixed_lengths(lib, torch_cuda_set, restatement, prec):
    torch = torch_cuda_set
    import bench
    rng = np.random.default_rng(42)
    if prec == "f":
        lengths = bench.uneven_lengths(rng, 240)
        lengths += [64, 128, 4096, 8192, 16384, 65536, 60000, 17, 4093, 2039, 97, 1]
    else:
        lengths = bench.uneven_lengths(rng, 160, max_pow2=14, max_smooth=20000, max_prime=2047)
        lengths += [64, 4096, 8192, 16384, 17, 2039, 1]
    xin, yout, offs, plans = _make_set(torch, lengths, prec)
    lib_, pfx, s = _set_of(plans, prec)
    import fftw3_gb300 as g
    before = g.launch_count()
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0, g.last_error()
    torch.cuda.synchronize()
    _check(restatement, xin, yout, offs, lengths, prec, -1)
    # executing again gives the same result (counters and queue head reset by the graph)
    y1 = yout.clone()
    yout.zero_()
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0
    torch.cuda.synchronize()
    assert torch.equal(y1, yout)
    assert lib_.fftw_gb300_device_status() == 0
    # the same plans one by one give the same transforms (within tolerance)
    y2 = torch.zeros_like(yout)
    es = yout.element_size()
    for i, p in enumerate(plans):
        p.execute_dft(xin.data_ptr() + int(offs[i]) * es, y2.data_ptr() + int(offs[i]) * es)
    torch.cuda.synchronize()
    assert rel_l2(y2.cpu().numpy(), y1.cpu().numpy()) < (2e-6 if prec == "f" else 1e-13)
    getattr(lib_, pfx + "gb300_destroy_set")(s)


def test_planset_register_body(lib, torch_cuda_set, restatement, monkeypatch):
    """Power-of-two float items (64..4096 points: singles and the passes of
    long lengths) with the register-stage body instead of the runtime-radix
    one: every transform against the oracle, and the same set with the
    runtime-radix body agrees."""
    torch = torch_cuda_set
    import bench
    lengths = bench.uneven_lengths(np.random.default_rng(9), 200)
    lengths += [64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536, 60000, 97]
    xin, yout, offs, plans = _make_set(torch, lengths, "f", seed=9)
    monkeypatch.setenv("FFTW_GB300_QUEUE_BODY", "reg")
    lib_, pfx, s = _set_of(plans, "f")
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0
    torch.cuda.synchronize()
    assert lib_.fftw_gb300_device_status() == 0
    _check(restatement, xin, yout, offs, lengths, "f", -1)
    y_reg = yout.clone()
    getattr(lib_, pfx + "gb300_destroy_set")(s)
    monkeypatch.setenv("FFTW_GB300_QUEUE_BODY", "gen")
    lib_, pfx, s = _set_of(plans, "f")
    yout.zero_()
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0
    torch.cuda.synchronize()
    assert rel_l2(yout.cpu().numpy(), y_reg.cpu().numpy()) < 2e-6
    getattr(lib_, pfx + "gb300_destroy_set")(s)


def test_planset_tuned(lib, torch_cuda_set, restatement):
    """A set planned with FFTW_MEASURE: every length is tuned (item body,
    radix order, Rader or Bluestein, long split) on scratch arrays and
    recorded in wisdom as "set p4 n<n>"; the tuned set is correct; the same
    set plans under FFTW_WISDOM_ONLY from the exported wisdom, and a length
    wisdom does not cover is refused."""
    import fftw3_gb300 as g
    torch = torch_cuda_set
    lib_ = g.load()
    lib_.fftwf_forget_wisdom()
    lengths = [64, 64, 256, 1024, 4096, 60, 210, 1000, 3000, 97, 193, 4093, 8192, 16384, 65536, 60000, 6000] * 3
    xin, yout, offs, plans = _make_set(torch, lengths, "f", seed=13)
    lib_.fftwf_set_timelimit(120.0)
    xin_copy = xin.clone()
    _, pfx, s = _set_of(plans, "f", flags=g.FFTW_MEASURE)
    lib_.fftwf_set_timelimit(-1.0)
    # tuning ran on scratch arrays: the caller's input is untouched
    assert torch.equal(xin, xin_copy)
    w = ctypes.string_at(lib_.fftwf_export_wisdom_to_string()).decode()
    for n in set(lengths):
        assert f'"set p4 n{n}"' in w, n
    assert lib_.fftwf_gb300_execute_set(s) == 0
    torch.cuda.synchronize()
    assert lib_.fftw_gb300_device_status() == 0
    _check(restatement, xin, yout, offs, lengths, "f", -1)
    lib_.fftwf_gb300_destroy_set(s)
    # wisdom round trip: forget, import, plan with FFTW_WISDOM_ONLY
    lib_.fftwf_forget_wisdom()
    assert lib_.fftwf_import_wisdom_from_string(w.encode()) == 1
    _, pfx, s = _set_of(plans, "f", flags=g.FFTW_ESTIMATE | g.FFTW_WISDOM_ONLY)
    yout.zero_()
    assert lib_.fftwf_gb300_execute_set(s) == 0
    torch.cuda.synchronize()
    _check(restatement, xin, yout, offs, lengths, "f", -1)
    lib_.fftwf_gb300_destroy_set(s)
    extra = g.plan_many_dft([5000], 1, xin.data_ptr(), yout.data_ptr(), -1, g.FFTW_ESTIMATE, "f")
    arr = (ctypes.c_void_p * (len(plans) + 1))(*([p.ptr for p in plans] + [extra.ptr]))
    assert not lib_.fftwf_gb300_plan_set(len(plans) + 1, arr, g.FFTW_ESTIMATE | g.FFTW_WISDOM_ONLY)
    lib_.fftwf_forget_wisdom()


def test_planset_backward_and_rader(lib, torch_cuda_set, restatement, monkeypatch):
    monkeypatch.setenv("FFTW_GB300_PRIME", "rader")
    torch = torch_cuda_set
    lengths = [17, 31, 61, 97, 401, 673, 1201, 3001, 64, 60, 210, 5000, 32768]
    xin, yout, offs, plans = _make_set(torch, lengths, "f", sign=1, seed=3)
    lib_, pfx, s = _set_of(plans, "f")
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0
    torch.cuda.synchronize()
    _check(restatement, xin, yout, offs, lengths, "f", 1)
    getattr(lib_, pfx + "gb300_destroy_set")(s)


@pytest.fixture(scope="module")
def torch_cuda_set():
    import torch
    assert torch.cuda.is_available()
    return torch


def test_planset_first_use_in_fresh_process(lib):
    """A plan set built and executed before any other launch of the library in
    the process (its device status word is allocated outside the capture)."""
    import subprocess
    code = (
        "import sys, ctypes, numpy as np, torch; sys.path.insert(0, %r)\n"
        "import fftw3_gb300 as g\n"
        "x = torch.randn(3000, dtype=torch.complex64, device='cuda'); y = torch.zeros_like(x)\n"
        "ps = [g.plan_many_dft([n], 1, x.data_ptr() + o * 8, y.data_ptr() + o * 8, -1, g.FFTW_ESTIMATE, 'f')"
        " for n, o in ((1000, 0), (2000, 1000))]\n"
        "lib = g.load(); f = lib.fftwf_gb300_plan_set; f.restype = ctypes.c_void_p\n"
        "f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint]\n"
        "arr = (ctypes.c_void_p * 2)(*[p.ptr for p in ps]); s = f(2, arr, 0)\n"
        "lib.fftwf_gb300_execute_set.argtypes = [ctypes.c_void_p]\n"
        "rc = lib.fftwf_gb300_execute_set(s); torch.cuda.synchronize()\n"
        "ref = np.concatenate([np.fft.fft(x[:1000].cpu().numpy().astype(np.complex128)),"
        " np.fft.fft(x[1000:].cpu().numpy().astype(np.complex128))])\n"
        "err = np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref)\n"
        "print(rc, err); sys.exit(0 if rc == 0 and err < 1e-6 else 1)\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_planset_bounded_wait_runs_out(lib, torch_cuda_set, restatement):
    """A row tile whose column tiles never all arrive: its wait gives up after
    the set's limit (5 ms here), the tile is skipped, the launch finishes and
    the device status reads 2 (GB_STATUS_QUEUE_TIMEOUT); nothing traps or
    hangs, and the next execute of the unchanged set is correct."""
    torch = torch_cuda_set
    lengths = [65536, 32768, 4096, 1000, 97]
    xin, yout, offs, plans = _make_set(torch, lengths, "f", seed=11)
    lib_, pfx, s = _set_of(plans, "f")
    ex = getattr(lib_, pfx + "gb300_execute_set")
    wait = getattr(lib_, pfx + "gb300_set_wait_limit")
    wait.argtypes = [ctypes.c_void_p, ctypes.c_double]
    stall = getattr(lib_, pfx + "gb300_set_test_stall")
    stall.argtypes = [ctypes.c_void_p, ctypes.c_int]
    assert lib_.fftw_gb300_device_status() == 0
    assert wait(s, 0.005) == 0
    assert stall(s, 1) == 0
    assert ex(s) == 0
    torch.cuda.synchronize()
    assert lib_.fftw_gb300_device_status() == 2
    # the status word was cleared by the read
    assert lib_.fftw_gb300_device_status() == 0
    assert stall(s, 0) == 0
    assert wait(s, 2.0) == 0
    yout.zero_()
    assert ex(s) == 0
    torch.cuda.synchronize()
    assert lib_.fftw_gb300_device_status() == 0
    _check(restatement, xin, yout, offs, lengths, "f", -1)
    # a limit outside (0, 60] s is refused
    assert wait(s, 0.0) == -1 and wait(s, 100.0) == -1
    getattr(lib_, pfx + "gb300_destroy_set")(s)


def test_planset_uneven10k(lib, torch_cuda_set, restatement):
    """The 10,000-transform uneven set (60% powers of two 2^6..2^16, 30%
    7-smooth lengths in [60, 60000], 10% primes in [17, 4093], seed 7) as one
    graph launch: every prime transform and a seeded sample of 200 others
    against the oracle."""
    torch = torch_cuda_set
    import bench
    lengths = bench.uneven_lengths(np.random.default_rng(7), 10000)
    xin, yout, offs, plans = _make_set(torch, lengths, "f", seed=5)
    lib_, pfx, s = _set_of(plans, "f")
    assert getattr(lib_, pfx + "gb300_execute_set")(s) == 0
    torch.cuda.synchronize()
    assert lib_.fftw_gb300_device_status() == 0
    primes = set(bench.primes_in(17, 4093))
    prime_idx = [i for i, n in enumerate(lengths) if n in primes]
    others = [i for i in range(len(lengths)) if lengths[i] not in primes]
    sample = sorted(prime_idx + list(np.random.default_rng(1).choice(others, 200, replace=False)))
    assert len(prime_idx) > 800
    _check(restatement, xin, yout, offs, lengths, "f", -1, sample=sample)
    getattr(lib_, pfx + "gb300_destroy_set")(s)
    for p in plans:
        p.destroy()
