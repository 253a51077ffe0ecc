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


@pytest.mark.parametrize("n", [256, 4096, 65536])
@pytest.mark.parametrize("dist", ["normal", "loguniform"])
@pytest.mark.parametrize("sign", [-1, 1])
def test_tc_fft_parity(lib, torch_tc, restatement, n, dist, sign):
    """1D batches; 65536 runs as two tensor-core passes of 256 (four-step)."""
    import fftw3_gb300 as g
    torch = torch_tc
    hm = {256: 1024, 4096: 64, 65536: 4}[n]
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
    assert "tc-split-fp16" in p.describe()
    p.execute()
    y = yo.cpu().numpy()
    ref = restatement.c2c(x.astype(np.complex128), [n], sign, "d", nthreads=4)
    err = rel_l2(y, ref)
    assert err <= 1e-6, f"rel L2 {err:.3e}"
    assert g.load().fftw_gb300_device_status() == 0


def test_tc_multid_columns(lib, torch_tc, restatement):
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
