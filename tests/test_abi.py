"""The C-ABI boundary, checked without a GPU: the library loads, exports every
symbol the public headers declare, keeps the reference's flag values and
argument checks, and fails loudly (NULL plan + message) when no GPU exists.
No transform is computed here."""
import ctypes
import os
import re

import pytest

import fftw3_gb300 as g
from conftest import has_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exports_every_declared_symbol(lib):
    names = g.declared_symbols()
    assert len(names) > 150
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_flag_values_match_reference_header():
    """api/fftw3.h:489-519 values, bit for bit."""
    txt = open(os.path.join(ROOT, "include", "fftw3.h")).read()
    want = {
        "FFTW_MEASURE": 0, "FFTW_DESTROY_INPUT": 1, "FFTW_UNALIGNED": 2, "FFTW_CONSERVE_MEMORY": 4,
        "FFTW_EXHAUSTIVE": 8, "FFTW_PRESERVE_INPUT": 16, "FFTW_PATIENT": 32, "FFTW_ESTIMATE": 64,
        "FFTW_WISDOM_ONLY": 1 << 21, "FFTW_ESTIMATE_PATIENT": 1 << 7, "FFTW_BELIEVE_PCOST": 1 << 8,
        "FFTW_NO_DFT_R2HC": 1 << 9, "FFTW_NO_NONTHREADED": 1 << 10, "FFTW_NO_BUFFERING": 1 << 11,
        "FFTW_NO_INDIRECT_OP": 1 << 12, "FFTW_ALLOW_LARGE_GENERIC": 1 << 13, "FFTW_NO_RANK_SPLITS": 1 << 14,
        "FFTW_NO_VRANK_SPLITS": 1 << 15, "FFTW_NO_VRECURSE": 1 << 16, "FFTW_NO_SIMD": 1 << 17,
        "FFTW_NO_SLOW": 1 << 18, "FFTW_NO_FIXED_RADIX_LARGE_N": 1 << 19, "FFTW_ALLOW_PRUNING": 1 << 20,
    }
    for name, v in want.items():
        m = re.search(r"#define %s \((\d+)U(?: << (\d+))?\)" % name, txt)
        assert m, name
        got = int(m.group(1)) << int(m.group(2) or 0)
        assert got == v, name
    assert "#define FFTW_FORWARD (-1)" in txt and "#define FFTW_BACKWARD (+1)" in txt


def test_version_strings(lib):
    for pfx in ("fftw_", "fftwf_"):
        s = ctypes.c_char_p.in_dll(lib, pfx + "version")
        assert ctypes.string_at(ctypes.addressof(s)).startswith(b"fftw-3.3")


def test_invalid_arguments_return_null(lib):
    """api/mktensor-rowmajor.c:58-61: rank < 0, n <= 0, howmany < 0 -> NULL."""
    g.set_dry_run(True)
    try:
        n = (ctypes.c_int * 1)(64)
        bad = (ctypes.c_int * 1)(0)
        for pfx in ("fftw_", "fftwf_"):
            f = getattr(lib, pfx + "plan_many_dft")
            assert not f(-1, n, 1, 16, None, 1, 64, 32, None, 1, 64, -1, g.FFTW_ESTIMATE)
            assert not f(1, bad, 1, 16, None, 1, 64, 32, None, 1, 64, -1, g.FFTW_ESTIMATE)
            assert not f(1, n, -1, 16, None, 1, 64, 32, None, 1, 64, -1, g.FFTW_ESTIMATE)
            assert not f(1, n, 1, 16, None, 1, 64, 32, None, 1, 64, 0, g.FFTW_ESTIMATE)   # sign must be +-1
            assert f(1, n, 1, 16, None, 1, 64, 32, None, 1, 64, -1, g.FFTW_ESTIMATE)
            # r2r: every fftw_r2r_kind (api/fftw3.h:96-100), any rank; a kind
            # out of range and a size-1 REDFT00 (not defined) return NULL
            f = getattr(lib, pfx + "plan_many_r2r")
            f.restype = ctypes.c_void_p
            for kind in range(11):
                kinds = (ctypes.c_int * 2)(kind, kind)
                assert f(1, n, 1, 16, None, 1, 64, 32, None, 1, 64, kinds, 64), kind
            assert not f(1, n, 1, 16, None, 1, 64, 32, None, 1, 64, (ctypes.c_int * 1)(11), 64)
            one = (ctypes.c_int * 1)(1)
            assert not f(1, one, 1, 16, None, 1, 1, 32, None, 1, 1, (ctypes.c_int * 1)(3), 64)
            assert "REDFT00" in g.last_error()
            assert f(1, one, 1, 16, None, 1, 1, 32, None, 1, 1, (ctypes.c_int * 1)(7), 64)
            assert f(0, n, 5, 16, None, 1, 2, 32, None, 1, 3, (ctypes.c_int * 1)(0), 64)   # rank 0: a copy
            n3 = (ctypes.c_int * 3)(6, 5, 8)
            p = f(3, n3, 2, 16, None, 1, 240, 32, None, 1, 240, (ctypes.c_int * 3)(3, 10, 1), 64)
            assert p
            assert getattr(lib, pfx + "sprint_plan")(p).decode().count("(dim ") == 3
    finally:
        g.set_dry_run(False)


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(lib):
    """Without a GPU the planner refuses (no CPU fallback) and says why."""
    n = (ctypes.c_int * 1)(64)
    p = lib.fftwf_plan_many_dft(1, n, 1, 16, None, 1, 64, 32, None, 1, 64, -1, g.FFTW_ESTIMATE)
    assert not p
    assert "GPU" in g.last_error()


def test_malloc_alignment_and_free(lib):
    for pfx in ("fftw_", "fftwf_"):
        p = getattr(lib, pfx + "malloc")(1000)
        assert p and p % 64 == 0
        ctypes.memset(p, 1, 1000)
        assert getattr(lib, pfx + "alignment_of")(p) == 0
        assert getattr(lib, pfx + "alignment_of")(p + 4) == 4
        getattr(lib, pfx + "free")(p)


def test_threads_api(lib):
    """threads/api.c:39-95: accepted; the GPU replaces the thread pool."""
    assert lib.fftw_init_threads() == 1
    lib.fftwf_plan_with_nthreads(8)
    assert lib.fftwf_planner_nthreads() == 8
    lib.fftwf_plan_with_nthreads(1)
    lib.fftw_cleanup_threads()


def test_header_declares_exactly_the_reference_api():
    """include/fftw3.h declares the same function and data names as the
    reference's FFTW_DEFINE_API list (api/fftw3.h:127-466), no more, no less."""
    from oracle.oracle import ref_source
    path = ref_source(os.path.join("api", "fftw3.h"))
    if path is None:
        pytest.skip("the reference sources are not on this machine")
    ref = open(path).read()
    body = ref[ref.index("#define FFTW_DEFINE_API"):ref.index("FFTW_DEFINE_API(FFTW_MANGLE_DOUBLE")]
    want = set(re.findall(r"X\((\w+)\)\s*[\(\[]", body))
    ours = open(os.path.join(ROOT, "include", "fftw3.h")).read()
    have = set(re.findall(r"PFX##(\w+)\s*[\(\[]", ours))
    assert len(want) > 70 and want == have, (sorted(want - have), sorted(have - want))
