"""The persistent, bulk-copy fed kernels over long batches: a CTA walks many
tiles, with one or two compute groups sharing its shared-memory buffers, the
next tile's copy in flight while the groups transform theirs.  Short batches
(one or two tiles per CTA) never exercise the hand-over of a buffer from one
group to the other, so these cases give every CTA dozens of tiles, and check
(a) that one and two groups give the same result on every transform of the
batch, and (b) transforms spread over the whole batch against the oracle
(float tolerance: rel L2 <= 1e-6)."""
import os

import numpy as np
import pytest

from conftest import rel_l2_f

pytestmark = pytest.mark.gpu

TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def _run(torch, make, groups):
    """Plan with FFTW_GB300_TMA_GROUPS=groups (read when planning), execute."""
    old = os.environ.get("FFTW_GB300_TMA_GROUPS")
    os.environ["FFTW_GB300_TMA_GROUPS"] = str(groups)
    try:
        p, run = make()
    finally:
        if old is None:
            del os.environ["FFTW_GB300_TMA_GROUPS"]
        else:
            os.environ["FFTW_GB300_TMA_GROUPS"] = old
    out = run(p)
    torch.cuda.synchronize()
    return out.clone()


def _spread(count, k=24):
    return sorted(set(np.linspace(0, count - 1, k).astype(int).tolist()))


@pytest.mark.parametrize("n,hm", [(4096, 16384), (256, 1 << 19), (1024, 32768)])
def test_c2c_rows_one_and_two_groups(lib, torch_cuda, restatement, n, hm):
    import fftw3_gb300 as g
    torch = torch_cuda
    gen = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(n * hm, dtype=torch.complex64, device="cuda", generator=gen)
    y = torch.empty_like(x)

    def make():
        p = g.plan_many_dft([n], hm, x.data_ptr(), y.data_ptr(), -1, g.FFTW_ESTIMATE, "f")
        assert "reg-tma" in p.describe()
        return p, lambda p: (p.execute(), y)[1]

    y1 = _run(torch, make, 1)
    y2 = _run(torch, make, 2)
    assert rel_l2_f(y2.cpu().numpy(), y1.cpu().numpy()) <= 1e-7
    xs = x.view(hm, n).cpu().numpy()
    ys = y2.view(hm, n).cpu().numpy()
    for t in _spread(hm):
        ref = restatement.c2c(xs[t].astype(np.complex128), [n], -1, "d")
        assert rel_l2_f(ys[t], ref) <= TOL, f"transform {t}"


def test_r2c_one_and_two_groups(lib, torch_cuda, restatement):
    import fftw3_gb300 as g
    torch = torch_cuda
    n, hm = 16384, 4096
    gen = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(n * hm, dtype=torch.float32, device="cuda", generator=gen)
    y = torch.empty(hm * (n // 2 + 1), dtype=torch.complex64, device="cuda")

    def make():
        p = g.plan_many_dft_r2c([n], hm, x.data_ptr(), y.data_ptr(), g.FFTW_ESTIMATE, "f")
        assert "reg-tma" in p.describe()
        return p, lambda p: (p.execute(), y)[1]

    y1 = _run(torch, make, 1)
    y2 = _run(torch, make, 2)
    assert rel_l2_f(y2.cpu().numpy(), y1.cpu().numpy()) <= 1e-7
    xs = x.view(hm, n).cpu().numpy()
    ys = y2.view(hm, n // 2 + 1).cpu().numpy()
    for t in _spread(hm, 12):
        ref = restatement.r2c(xs[t].astype(np.float64), [n], "d")
        assert rel_l2_f(ys[t], ref) <= TOL, f"transform {t}"


@pytest.mark.parametrize("shape,hm", [([1024, 1024], 32), ([65536], 512), ([128, 256, 256], 4)])
def test_column_tiles_one_and_two_groups(lib, torch_cuda, restatement, shape, hm):
    """Column passes (tensor-map tiles): the strided axes of multi-d plans
    and the four-step passes of a long 1D length."""
    import fftw3_gb300 as g
    torch = torch_cuda
    tot = int(np.prod(shape))
    gen = torch.Generator(device="cuda").manual_seed(tot + hm)
    x = torch.randn(tot * hm, dtype=torch.complex64, device="cuda", generator=gen)
    y = torch.empty_like(x)

    def make():
        p = g.plan_many_dft(shape, hm, x.data_ptr(), y.data_ptr(), -1, g.FFTW_ESTIMATE, "f")
        assert "cols-tma" in p.describe()
        return p, lambda p: (p.execute(), y)[1]

    y1 = _run(torch, make, 1)
    y2 = _run(torch, make, 2)
    assert rel_l2_f(y2.cpu().numpy(), y1.cpu().numpy()) <= 1e-7
    xs = x.view(hm, tot).cpu().numpy()
    ys = y2.view(hm, tot).cpu().numpy()
    for t in _spread(hm, 4):
        ref = restatement.c2c(xs[t].astype(np.complex128), shape, -1, "d", nthreads=8)
        assert rel_l2_f(ys[t], ref) <= TOL, f"transform {t}"
