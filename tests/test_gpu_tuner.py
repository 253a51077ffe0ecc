"""FFTW_MEASURE: the tuner times candidate configurations on scratch arrays
(the caller's arrays are untouched), keeps the fastest as wisdom, and the
wisdom round-trips through export/import; FFTW_WISDOM_ONLY then plans."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [4096, 60, 1021, 1 << 16])
def test_measure_records_wisdom_and_keeps_inputs(lib, restatement, n):
    import torch
    import fftw3_gb300 as g
    lib_ = g.load()
    lib_.fftwf_forget_wisdom()
    hm = 8
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n * hm) + 1j * rng.standard_normal(n * hm)).astype(np.complex64)
    xi = torch.from_numpy(x).cuda()
    yo = torch.full_like(xi, 7 + 7j)
    p = g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_MEASURE, "f")
    # planning with FFTW_MEASURE did not touch the caller's arrays
    assert np.array_equal(xi.cpu().numpy(), x)
    assert torch.all(yo == 7 + 7j)
    w = ctypes.string_at(lib_.fftwf_export_wisdom_to_string())
    assert f'"c2c p4 n{n}"'.encode() in w
    assert lib_.fftwf_cost(p.ptr) > 0
    p.execute()
    assert rel_l2(yo.cpu().numpy(), restatement.c2c(x.astype(np.complex128), [n], -1, "d")) <= 1e-6
    # the exported wisdom imports again and serves FFTW_WISDOM_ONLY
    lib_.fftwf_forget_wisdom()
    assert lib_.fftwf_import_wisdom_from_string(w) == 1
    q = g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_WISDOM_ONLY, "f")
    q.execute()
    assert rel_l2(yo.cpu().numpy(), restatement.c2c(x.astype(np.complex128), [n], -1, "d")) <= 1e-6
    lib_.fftwf_forget_wisdom()
