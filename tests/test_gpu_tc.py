"""The tensor-core (tcgen05, split FP16) form: the GEMM building block against
numpy, then whole transforms against the FP64 oracle at the float bound,
including inputs whose magnitudes span 1e-3..1e3."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FFTW_GB300_TENSOR_CORE = 1 << 28


@pytest.fixture(scope="module")
def torch_tc():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("ks", [1, 6])
def test_tc_gemm_selftest(lib, torch_tc, ks):
    """D = A . B^T through the shared-memory descriptors, tcgen05.mma and
    tcgen05.ld used by the FFT stages; exact for small-integer operands."""
    import fftw3_gb300 as g
    torch = torch_tc
    rng = np.random.default_rng(ks)
    K = 16 * ks
    A = rng.integers(-4, 5, size=(128, K)).astype(np.float16)
    B = rng.integers(-4, 5, size=(32, K)).astype(np.float16)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dD = torch.zeros(128 * 32, dtype=torch.float32, device="cuda")
    lib_ = g.load()
    lib_.fftw_gb300_tc_selftest.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    assert lib_.fftw_gb300_tc_selftest(dA.data_ptr(), dB.data_ptr(), dD.data_ptr(), ks) == 0
    D = dD.cpu().numpy().reshape(128, 32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    assert np.array_equal(D, ref.astype(np.float32))
    assert lib_.fftw_gb300_device_status() == 0


@pytest.fixture(params=["2", "3"])
def tc_ctas(request, monkeypatch):
    """The two builds of the tensor-core kernel: two CTAs per SM with bulk
    copies into a second buffer, three CTAs per SM with plain loads (read
    when planning)."""
    monkeypatch.setenv("FFTW_GB300_TC_CTAS", request.param)
    return request.param


def _tc_plan_ok(p, ctas):
    d = p.describe()
    assert "tc-split-fp16" in d
    assert ("ctas=3" in d) == (ctas == "3")


@pytest.mark.parametrize("n", [256, 512, 1024, 2048, 4096, 65536])
@pytest.mark.parametrize("dist", ["normal", "loguniform"])
@pytest.mark.parametrize("sign", [-1, 1])
def test_tc_fft_parity(lib, torch_tc, restatement, tc_ctas, n, dist, sign):
    """1D batches; 512, 1024 and 2048 begin with an FP32 stage of radix 2,
    4 or 8; 65536 runs as two tensor-core passes of 256 (four-step)."""
    import fftw3_gb300 as g
    torch = torch_tc
    hm = {256: 1024, 512: 512, 1024: 256, 2048: 129, 4096: 64, 65536: 4}[n]
    rng = np.random.default_rng(n + (sign > 0))
    if dist == "normal":
        x = rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)
    else:
        mag = lambda: 10.0 ** rng.uniform(-3, 3, n * hm) * rng.choice([-1.0, 1.0], n * hm)
        x = mag() + 1j * mag()
    x = x.astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    yo = torch.empty_like(xi)
    p = g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), sign, g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    _tc_plan_ok(p, tc_ctas)
    p.execute()
    y = yo.cpu().numpy()
    ref = restatement.c2c(x.astype(np.complex128), [n], sign, "d", nthreads=4)
    err = rel_l2(y, ref)
    assert err <= 1e-6, f"rel L2 {err:.3e}"
    assert g.load().fftw_gb300_device_status() == 0


def test_tc_2d_512(lib, torch_tc, restatement, tc_ctas):
    """2D 512 x 512 (the 3D workload's axis length): rows and columns in the
    tensor-core form, each beginning with a radix-2 FP32 stage."""
    import fftw3_gb300 as g
    torch = torch_tc
    shape = [512, 512]
    rng = np.random.default_rng(512)
    tot = 512 * 512 * 2
    x = (rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    yo = torch.empty_like(xi)
    p = g.plan_many_dft(shape, 2, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    assert p.describe().count("tc-split-fp16") == 2
    p.execute()
    ref = restatement.c2c(x.astype(np.complex128), shape, -1, "d", nthreads=4)
    assert rel_l2(yo.cpu().numpy(), ref) <= 1e-6
    assert g.load().fftw_gb300_device_status() == 0


def test_tc_multid_columns(lib, torch_tc, restatement, tc_ctas):
    """2D 256 x 256: the column axis runs through the tensor-core kernel with
    column tiles (strided loads and stores)."""
    import fftw3_gb300 as g
    torch = torch_tc
    shape = [256, 256]
    rng = np.random.default_rng(77)
    x = (rng.standard_normal(2 * 65536) + 1j * rng.standard_normal(2 * 65536)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    yo = torch.empty_like(xi)
    p = g.plan_many_dft(shape, 2, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    assert p.describe().count("tc-split-fp16") == 2
    p.execute()
    ref = restatement.c2c(x.astype(np.complex128), shape, -1, "d", nthreads=4)
    assert rel_l2(yo.cpu().numpy(), ref) <= 1e-6


@pytest.mark.parametrize("n", [256, 4096, 65536])
def test_tc_fft_loguniform_large_batch(lib, torch_tc, restatement, tc_ctas, n):
    """The precision-form workload's log-uniform variant (re and im with
    magnitudes 10^U[-3,3) and random signs, generated on the device) at 2^26
    points per length: transforms spread over the whole batch against the
    FP64 oracle, each within the float bound."""
    import fftw3_gb300 as g
    from conftest import rel_l2_f
    torch = torch_tc
    hm = (1 << 26) // n
    gen = torch.Generator(device="cuda").manual_seed(n + 3)

    def mag():
        m = torch.pow(10.0, torch.rand(n * hm, device="cuda", generator=gen, dtype=torch.float64) * 6 - 3)
        s = torch.randint(0, 2, (n * hm,), device="cuda", generator=gen).to(torch.float64) * 2 - 1
        return (m * s).to(torch.float32)

    x = torch.complex(mag(), mag())
    y = torch.empty_like(x)
    p = g.plan_many_dft([n], hm, x.data_ptr(), y.data_ptr(), -1, g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    _tc_plan_ok(p, tc_ctas)
    p.execute()
    torch.cuda.synchronize()
    sel = np.linspace(0, hm - 1, 16).astype(int)
    xs = x.view(hm, n).cpu().numpy()[sel]
    ys = y.view(hm, n).cpu().numpy()[sel]
    worst = 0.0
    for a, b in zip(xs, ys):
        err = rel_l2_f(b, restatement.c2c(a.astype(np.complex128), [n], -1, "d"))
        worst = max(worst, err)
    assert worst <= 1e-6, f"worst rel L2 {worst:.3e}"
    assert g.load().fftw_gb300_device_status() == 0


def test_tc_3d_stage_budget(lib, torch_tc, restatement):
    """3D 256^3 in place: the tensor-core form takes passes until the plan
    holds four GEMM stages (two axes here), the third axis stays FP32, and
    the forward transform of the whole array stays within the float bound."""
    import fftw3_gb300 as g
    from conftest import rel_l2_f
    torch = torch_tc
    shape = [256, 256, 256]
    tot = 256 ** 3
    rng = np.random.default_rng(3)
    x = (rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)).astype(np.complex64)
    a = torch.from_numpy(x).cuda()
    p = g.Plan(g.load().fftwf_plan_dft_3d(*shape, a.data_ptr(), a.data_ptr(), -1,
                                          g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE), "f")
    assert p.describe().count("tc-split-fp16") == 2 and len(p.passes()) == 3
    p.execute()
    ref = restatement.c2c(x.astype(np.complex128), shape, -1, "d", nthreads=8)
    assert rel_l2_f(a.cpu().numpy(), ref) <= 1e-6
    assert g.load().fftw_gb300_device_status() == 0


@pytest.mark.parametrize("n,hm", [(8192, 32), (512, 64)])
def test_tc_real_forms(lib, torch_tc, restatement, n, hm):
    """r2c and c2r in the tensor-core form: the half-length c2c as tcgen05
    GEMM stages beside the hc2c post- / pre-pass; r2c of N(0,1) reals and c2r
    of that spectrum against the FP64 oracle (float bound)."""
    import fftw3_gb300 as g
    torch = torch_tc
    rng = np.random.default_rng(n + hm)
    nc = n // 2 + 1
    x = rng.standard_normal(n * hm).astype(np.float32)
    xi = torch.from_numpy(x).cuda()
    yo = torch.empty(hm * nc, dtype=torch.complex64, device="cuda")
    p = g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    assert "tc-split-fp16" in p.describe()
    p.execute()
    torch.cuda.synchronize()
    y = yo.cpu().numpy()
    assert rel_l2(y, restatement.r2c(x.astype(np.float64), [n], "d")) <= 1e-6
    zi = yo.clone()
    ro = torch.empty(hm * n, dtype=torch.float32, device="cuda")
    q = g.plan_many_dft_c2r([n], hm, zi.data_ptr(), ro.data_ptr(), g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE, "f")
    assert "tc-split-fp16" in q.describe()
    q.execute()
    torch.cuda.synchronize()
    assert rel_l2(ro.cpu().numpy(), restatement.c2r(y.astype(np.complex128), [n], "d")) <= 1e-6
    assert g.load().fftw_gb300_device_status() == 0


def test_tc_real_2d(lib, torch_tc, restatement):
    """2D r2c 2048^2 in the tensor-core form (rows: the 1024-point half-length
    c2c as GEMMs and the hc2c pass; columns FP32) against the oracle."""
    import fftw3_gb300 as g
    torch = torch_tc
    rng = np.random.default_rng(2048)
    x = rng.standard_normal(2048 * 2048).astype(np.float32)
    xi = torch.from_numpy(x).cuda()
    yo = torch.empty(2048 * 1025, dtype=torch.complex64, device="cuda")
    p = g.plan_many_dft_r2c([2048, 2048], 1, xi.data_ptr(), yo.data_ptr(), g.FFTW_ESTIMATE | FFTW_GB300_TENSOR_CORE,
                            "f")
    assert "tc-split-fp16" in p.describe()
    p.execute()
    torch.cuda.synchronize()
    assert rel_l2(yo.cpu().numpy(), restatement.r2c(x.astype(np.float64), [2048, 2048], "d")) <= 1e-6
    assert g.load().fftw_gb300_device_status() == 0
