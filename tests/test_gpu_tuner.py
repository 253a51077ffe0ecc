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


def test_wisdom_only_keys_the_whole_problem(lib):
    """FFTW_WISDOM_ONLY plans only a problem whose exact shape was planned
    with tuning (api/apiplan.c:102-107, wisdom keyed by the whole problem,
    kernel/planner.c:651-703): wisdom of a c2c of length n serves neither an
    r2c of n, a c2c of n with another batch size, nor the other direction."""
    import torch
    import fftw3_gb300 as g
    lib_ = g.load()
    lib_.fftwf_forget_wisdom()
    n, hm = 4096, 8
    xi = torch.zeros(n * hm, dtype=torch.complex64, device="cuda")
    yo = torch.zeros_like(xi)
    g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, g.FFTW_MEASURE, "f").destroy()
    w = ctypes.string_at(lib_.fftwf_export_wisdom_to_string())
    assert f'"c2c p4 n{n}"'.encode() in w and b'"prob p4 k0 r1 ' in w
    only = g.FFTW_WISDOM_ONLY
    # the tuned problem itself plans
    g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, only, "f").destroy()
    for make in (lambda: g.plan_many_dft([n], 2 * hm, xi.data_ptr(), yo.data_ptr(), -1, only, "f"),
                 lambda: g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), 1, only, "f"),
                 lambda: g.plan_many_dft([n], hm, xi.data_ptr(), xi.data_ptr(), -1, only, "f"),
                 lambda: g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), only, "f"),
                 lambda: g.plan_many_dft([64, 64], hm, xi.data_ptr(), yo.data_ptr(), -1, only, "f")):
        with pytest.raises(RuntimeError, match="WISDOM_ONLY"):
            make()
    # after a round trip through the exported text the same holds
    lib_.fftwf_forget_wisdom()
    assert lib_.fftwf_import_wisdom_from_string(w) == 1
    g.plan_many_dft([n], hm, xi.data_ptr(), yo.data_ptr(), -1, only, "f").destroy()
    with pytest.raises(RuntimeError, match="WISDOM_ONLY"):
        g.plan_many_dft_r2c([n], hm, xi.data_ptr(), yo.data_ptr(), only, "f")
    lib_.fftwf_forget_wisdom()
