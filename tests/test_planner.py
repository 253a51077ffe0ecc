"""Host planner logic, checked without a GPU (dry-run plans): how problems
become passes (per-axis multi-d, four-step split for long transforms,
Bluestein for large primes, tile/move choices for strided axes), and the
wisdom text format."""
import ctypes

import numpy as np

import pytest

import fftw3_gb300 as g


@pytest.fixture(autouse=True)
def dry(lib):
    g.set_dry_run(True)
    yield
    g.set_dry_run(False)


def passes(p):
    return p.passes()


def test_batched_1d_is_one_pass():
    p = g.plan_many_dft([4096], 65536, 1 << 20, 1 << 30, prec="f")
    (ps,) = passes(p)
    assert ps["nfft"] == 4096 and ps["variant"] in (0, 2) and ps["blocks"] * ps["tb"] >= 65536


def test_double_precision_pass():
    p = g.plan_many_dft([1024], 4096, 1 << 20, 1 << 30, prec="d")
    (ps,) = passes(p)
    assert ps["nfft"] == 1024 and ps["variant"] in (0, 2)


def test_long_transform_is_two_passes_with_scratch(lib):
    p = g.plan_many_dft([1 << 20], 64, 1 << 20, 1 << 30, prec="f")
    ps = passes(p)
    assert len(ps) == 2
    assert ps[0]["nfft"] * ps[1]["nfft"] == 1 << 20
    assert lib.fftwf_gb300_scratch_bytes(p.ptr) == (1 << 20) * 64 * 8


def test_smooth_nonpow2_uses_generic_stages():
    p = g.plan_many_dft([60], 100, 1 << 20, 1 << 30, prec="f")
    (ps,) = passes(p)
    assert ps["variant"] == 1 and ps["nfft"] == 60


def test_prime_uses_bluestein_power_of_two():
    p = g.plan_many_dft([1021], 10, 1 << 20, 1 << 30, prec="f")
    (ps,) = passes(p)
    assert ps["kind"] == 3 and ps["nfft"] == 2048


def test_3d_is_one_pass_per_axis():
    p = g.plan_many_dft([512, 512, 512], 1, 1 << 20, 1 << 20, prec="f")
    ps = passes(p)
    assert [x["nfft"] for x in ps] == [512, 512, 512]
    d = p.describe()
    assert d.count("ld=cols") == 2   # the two strided axes move tiles of columns


def test_r2c_2d_is_r2c_then_c2c():
    p = g.plan_many_dft_r2c([8192, 8192], 1, 1 << 20, 1 << 30, prec="f")
    ps = passes(p)
    assert ps[0]["kind"] == 1 and ps[0]["nfft"] == 4096
    # the 8192-point column axis: one column pass would move tiles one
    # column (8 bytes) wide, so it runs as a four-step pair of column passes
    # with wide tiles whose lengths multiply to 8192
    assert all(x["kind"] == 0 for x in ps[1:])
    assert int(np.prod([x["nfft"] for x in ps[1:]])) == 8192
    assert p.describe().count("ld=cols") == len(ps) - 1


def test_c2r_multid_does_c2c_first():
    p = g.plan_many_dft_c2r([64, 64], 1, 1 << 20, 1 << 30, prec="f")
    ps = passes(p)
    assert ps[0]["kind"] == 0 and ps[1]["kind"] == 2


def test_vector_dims_merge():
    """Contiguous howmany dims collapse into one (kernel/tensor7.c)."""
    lib = g.load()
    IOD = g.IODim * 1
    H = g.IODim * 2
    dims = IOD(g.IODim(256, 1, 1))
    hm = H(g.IODim(10, 256 * 20, 256 * 20), g.IODim(20, 256, 256))
    p = g.Plan(lib.fftwf_plan_guru_dft(1, dims, 2, hm, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE), "f")
    (ps,) = passes(p)
    assert ps["blocks"] * ps["tb"] >= 200


def test_rank0_copy_and_inplace_noop():
    lib = g.load()
    n = (ctypes.c_int * 1)(1)
    p = lib.fftwf_plan_many_dft(0, n, 5, 1 << 20, None, 1, 1, 1 << 21, None, 1, 1, -1, g.FFTW_ESTIMATE)
    assert p
    lib.fftwf_destroy_plan(p)


def test_wisdom_roundtrip_and_rejection(lib):
    lib.fftwf_forget_wisdom()
    w = b'(fftw-3.3.10-gb300 fftwf_wisdom #x67623330304c4942\n  (gb300-pass "c2c p4 n1024" #x0 #x2 #x0 #x0 #x0)\n)\n'
    assert lib.fftwf_import_wisdom_from_string(w) == 1
    out = ctypes.string_at(lib.fftwf_export_wisdom_to_string())
    assert b'"c2c p4 n1024" #x0 #x2' in out
    # the reference's own wisdom format is rejected, and existing wisdom kept
    ref_style = b"(fftw-3.3.10 fftwf_wisdom #x4be12fff #x7b2df9b2 #xa5975329 #x385b0041\n)\n"
    assert lib.fftwf_import_wisdom_from_string(ref_style) == 0
    assert lib.fftwf_import_wisdom_from_string(b"(fftw-3.3.10-gb300 fftwf_wisdom #x1\n)") == 0
    assert lib.fftwf_import_wisdom_from_string(w[:-10]) == 0     # truncated
    assert lib.fftw_import_wisdom_from_string(w) == 0            # other precision
    out2 = ctypes.string_at(lib.fftwf_export_wisdom_to_string())
    assert out2 == out
    # tb from wisdom is used by the planner
    p = g.plan_many_dft([1024], 64, 1 << 20, 1 << 30, prec="f")
    assert passes(p)[0]["tb"] == 2
    lib.fftwf_forget_wisdom()
    assert b"gb300-pass" not in ctypes.string_at(lib.fftwf_export_wisdom_to_string())


def test_wisdom_only_without_wisdom_is_null(lib):
    lib.fftwf_forget_wisdom()
    n = (ctypes.c_int * 1)(4096)
    p = lib.fftwf_plan_many_dft(1, n, 1, 1 << 20, None, 1, 4096, 1 << 21, None, 1, 4096, -1, g.FFTW_WISDOM_ONLY)
    assert not p


def test_print_plan_names_passes():
    p = g.plan_many_dft([4096], 16, 1 << 20, 1 << 30, prec="f")
    s = p.describe()
    assert s.startswith("(gb300-dft-f32") and "nfft=4096" in s


def test_prime_rader_when_asked(monkeypatch):
    monkeypatch.setenv("FFTW_GB300_PRIME", "rader")
    p = g.plan_many_dft([401], 10, 1 << 20, 1 << 30, prec="f")
    (ps,) = passes(p)
    assert ps["kind"] == 5 and ps["nfft"] == 400
    # p-1 with a prime factor > 13 falls back to Bluestein
    p = g.plan_many_dft([1021], 10, 1 << 20, 1 << 30, prec="f")
    assert passes(p)[0]["kind"] == 3


def test_split_array_plans(lib):
    """plan_guru_split_dft: interleaved arrays (ii = ri + 1) become an ordinary
    complex plan; separate arrays a pack / c2c / unpack plan."""
    base = 1 << 20
    p = g.plan_guru_split_dft([(64, 2, 2)], [(10, 128, 128)], base, base + 4, base + 8192, base + 8196, prec="f")
    assert p.describe().startswith("(gb300-dft-f32")
    q = g.plan_guru_split_dft([(64, 1, 1)], [(10, 64, 64)], base, base + 4096, base + 8192, base + 12288, prec="f")
    assert q.describe().startswith("(gb300-split-dft-f32") and len(q.passes()) == 1
    r = g.plan_guru_split_dft([(12, 20, 1), (20, 1, 12)], [(3, 240, 240)], base, base + 8192, base + 16384,
                              base + 24576, prec="d")
    assert r.describe().startswith("(gb300-split-dft-f64")


def test_split_real_plans(lib):
    """plan_guru_split_dft_r2c/c2r: interleaved complex sides (io = ro + 1,
    ii = ri + 1, even strides) become ordinary r2c / c2r plans; separate
    arrays a copy / r2c or c2r / copy plan."""
    base = 1 << 20
    p = g.plan_guru_split_dft_r2c([(64, 1, 2)], [(10, 64, 66)], base, base + 8192, base + 8196, prec="f")
    assert p.describe().startswith("(gb300-rdft2-r2c-f32")
    q = g.plan_guru_split_dft_r2c([(64, 1, 1)], [(10, 64, 33)], base, base + 8192, base + 16384, prec="f")
    assert q.describe().startswith("(gb300-split-dft-r2c-f32")
    r = g.plan_guru_split_dft_c2r([(12, 9, 20), (16, 1, 1)], [], base, base + 8192, base + 16384, prec="d")
    assert r.describe().startswith("(gb300-split-dft-c2r-f64")
    t = g.plan_guru_split_dft_c2r([(64, 2, 1)], [(3, 66, 64)], base, base + 8, base + 16384, prec="d")
    assert t.describe().startswith("(gb300-rdft2-c2r-f64")
    with pytest.raises(RuntimeError):
        g.plan_guru_split_dft_r2c([], [(3, 1, 1)], base, base + 8192, base + 16384, prec="f")


@pytest.mark.parametrize("n,prec", [(4099, "f"), (12297, "f"), (1000003, "f"), (2049, "d"), (8198, "d")])
def test_long_real_prime_lengths_run_as_convolution(n, prec):
    """Real lengths with a prime factor > 13 beyond one CTA: Bluestein's
    convolution straight from the real array (r2c) or from the
    Hermitian-extended half spectrum (c2r), FFTs of a power of two >= 2n-1
    in between."""
    nb = 1 << (2 * n - 2).bit_length()
    for make, pin, pout in ((g.plan_many_dft_r2c, "chirp-in-real", "chirp-out-half"),
                            (g.plan_many_dft_c2r, "chirp-in-herm", "chirp-out-real")):
        p = make([n], 2, 1 << 20, 1 << 30, prec=prec)
        lines = p.describe().splitlines()
        assert f"pointwise:{pin} n={n} nfft={nb} " in lines[1]
        assert f"pointwise:{pout} n={n} " in lines[-1]
        assert sum("pointwise:spec-mul" in x for x in lines) == 1


def test_strided_long_real_runs_as_convolution():
    p = g.plan_many_dft_r2c([40000], 2, 1 << 20, 1 << 30, prec="f", istride=2, idist=80000)
    lines = p.describe().splitlines()
    assert "pointwise:chirp-in-real" in lines[1] and "pointwise:chirp-out-half" in lines[-1]


def test_r2r_stages_per_dim():
    """A rank-3 r2r plan is one stage per dim, last dim first: a c2r core for
    HC2R (8), a complex DFT of 2n for odd-length RODFT11 (5), an r2c of
    2(n-1) for REDFT00 (6)."""
    lib = g.load()
    f = lib.fftwf_plan_many_r2r
    f.restype = ctypes.c_void_p
    p = f(3, (ctypes.c_int * 3)(6, 5, 8), 2, 1 << 20, None, 1, 240, 1 << 30, None, 1, 240,
          (ctypes.c_int * 3)(3, 10, 1), 64)
    assert p
    d = lib.fftwf_sprint_plan(p).decode()
    i2, i1, i0 = d.index("(dim 2 kind 1"), d.index("(dim 1 kind 10"), d.index("(dim 0 kind 3")
    assert i2 < i1 < i0
    assert "rdft2-c2r" in d[i2:i1] and "n=10" in d[i1:i0] and "r2c n=10" in d[i0:]


def test_long_description_is_truncated_not_overflowed():
    """A plan with many passes (3D r2c whose axes all run as multi-pass
    convolutions) describes itself within the fixed description buffer."""
    p = g.plan_many_dft_r2c([4099, 2049, 17], 1, 1 << 20, 1 << 36, prec="d", istride=2,
                            idist=2 * 4099 * 2049 * 17)
    d = p.describe()
    assert d.startswith("(gb300-rdft2-r2c-f64") and len(d) <= 1023
    assert len(p.passes()) > 6


def test_c2r_multid_preserve_input_in_place(lib):
    """The reference plans an in-place multi-dimensional c2r under
    FFTW_PRESERVE_INPUT (the input is overwritten by definition,
    rdft/rank-geq2-rdft2.c:118-124); out of place it returns NULL."""
    f = lib.fftwf_plan_dft_c2r_2d
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint]
    assert f(64, 64, 1 << 20, 1 << 20, g.FFTW_ESTIMATE | g.FFTW_PRESERVE_INPUT)
    assert not f(64, 64, 1 << 20, 1 << 30, g.FFTW_ESTIMATE | g.FFTW_PRESERVE_INPUT)


def test_wisdom_groups_and_radix_order(lib):
    """Wisdom records the tuner's threads per CTA of a bulk-copy pass (one
    or two compute groups) and the radix order of a runtime-radix pass; the
    planner follows both, and entries written with five numbers (no groups,
    no order) still import."""
    import fftw3_gb300 as g
    g.set_dry_run(True)
    try:
        lib.fftwf_forget_wisdom()
        w = (b'(fftw-3.3.10-gb300 fftwf_wisdom #x67623330304c4942\n'
             b'  (gb300-pass "c2c p4 n4096" #xffffffff #x0 #x0 #x0 #x0 #x2 #x0)\n'
             b'  (gb300-pass "c2c p4 n6000" #xffffffff #x0 #x0 #x0 #x0 #x0 #x1)\n'
             b'  (gb300-pass "c2c p4 n3000" #xffffffff #x0 #x0 #x0 #x0 #x0 #x2)\n)\n')
        assert lib.fftwf_import_wisdom_from_string(w) == 1
        p = g.plan_many_dft([4096], 64, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        assert "reg-tma groups=2" in p.describe()
        p = g.plan_many_dft([6000], 8, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        assert "rad=8.2.5.5.5.3" in p.describe(), p.describe()
        p = g.plan_many_dft([3000], 8, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        assert "rad=5.5.5.3.8" in p.describe(), p.describe()
        exported = ctypes.string_at(lib.fftwf_export_wisdom_to_string())
        assert b'"c2c p4 n4096" #xffffffff #x0 #x0 #x0 #x0 #x2 #x0)' in exported
        # out-of-range choices are refused and leave the wisdom as it was
        bad = w.replace(b"#x2 #x0)", b"#x7 #x0)")
        assert lib.fftwf_import_wisdom_from_string(bad) == 0
        lib.fftwf_forget_wisdom()
        p = g.plan_many_dft([6000], 8, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        assert "rad=16.3.5.5.5" in p.describe() or "rad=16" in p.describe(), p.describe()
    finally:
        lib.fftwf_forget_wisdom()
        g.set_dry_run(False)


def test_tensor_core_builds(monkeypatch):
    """FFTW_GB300_TENSOR_CORE plans: unit-stride rows take the two-CTA build
    (a bulk copy-in buffer, 87 KB of shared memory), the strided passes of a
    four-step length the three-CTA build (54 KB, no second buffer);
    FFTW_GB300_TC_CTAS overrides; the four-GEMM-stage budget leaves a third
    axis of 256^3 in FP32."""
    TC = 1 << 28
    monkeypatch.delenv("FFTW_GB300_TC_CTAS", raising=False)
    rows = g.plan_many_dft([4096], 1024, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE | TC, "f")
    (ps,) = passes(rows)
    assert ps["variant"] == 3 and ps["threads"] == 256
    assert "tc-split-fp16" in rows.describe() and "ctas=3" not in rows.describe()
    four = g.plan_many_dft([65536], 16, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE | TC, "f")
    ps4 = passes(four)
    assert len(ps4) == 2 and all(p["variant"] == 3 for p in ps4)
    assert four.describe().count("ctas=3") == 2
    assert all(p["smem"] < rows.passes()[0]["smem"] for p in ps4)
    monkeypatch.setenv("FFTW_GB300_TC_CTAS", "3")
    rows3 = g.plan_many_dft([4096], 1024, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE | TC, "f")
    assert "ctas=3" in rows3.describe()
    monkeypatch.setenv("FFTW_GB300_TC_CTAS", "2")
    four2 = g.plan_many_dft([65536], 16, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE | TC, "f")
    assert "ctas=3" not in four2.describe()
    monkeypatch.delenv("FFTW_GB300_TC_CTAS")
    cube = g.plan_many_dft([256, 256, 256], 1, 1 << 20, 1 << 20, -1, g.FFTW_ESTIMATE | TC, "f")
    assert [p["variant"] for p in passes(cube)].count(3) == 2


def test_benchmark_workload_passes():
    """The passes the measured workloads run (kind, FFT length, variant):
    one bulk-copy fed pass for the unit-stride batches (c2c 4096, c2c 1024
    double, r2c 16384 on its 8192-point core), tensor-map column passes for
    both four-step passes of 65536 and 2^20 and for the strided axes of 512^3
    and of the 8192^2 r2c (whose 8192-point column axis is itself a
    four-step)."""
    TMA, COLS = 2, 4
    def shape(p):
        return [(x["kind"], x["nfft"], x["variant"]) for x in p.passes()]
    assert shape(g.plan_many_dft([4096], 65536, 1 << 20, 1 << 32, -1, g.FFTW_ESTIMATE, "f")) == [(0, 4096, TMA)]
    assert shape(g.plan_many_dft([1024], 4096, 1 << 20, 1 << 32, -1, g.FFTW_ESTIMATE, "d")) == [(0, 1024, TMA)]
    assert shape(g.plan_many_dft_r2c([16384], 16384, 1 << 20, 1 << 34, g.FFTW_ESTIMATE, "f")) == [(1, 8192, TMA)]
    assert shape(g.plan_many_dft([65536], 4096, 1 << 20, 1 << 32, -1, g.FFTW_ESTIMATE, "f")) == \
        [(0, 256, COLS), (0, 256, COLS)]
    assert shape(g.plan_many_dft([1 << 20], 64, 1 << 20, 1 << 32, -1, g.FFTW_ESTIMATE, "f")) == \
        [(0, 1024, COLS), (0, 1024, COLS)]
    assert shape(g.plan_many_dft([512, 512, 512], 1, 1 << 20, 1 << 20, -1, g.FFTW_ESTIMATE, "f")) == \
        [(0, 512, TMA), (0, 512, COLS), (0, 512, COLS)]
    r2d = shape(g.plan_many_dft_r2c([8192, 8192], 1, 1 << 20, 1 << 32, g.FFTW_ESTIMATE, "f"))
    assert r2d[0] == (1, 4096, TMA) and [v for _, _, v in r2d[1:]] == [COLS, COLS]
    assert r2d[1][1] * r2d[2][1] == 8192


@pytest.mark.parametrize("after", [0, 1, 3])
def test_failed_device_allocation_gives_null_plan(lib, after):
    """A device table allocation that fails (injected on the host, as a
    refused cudaMalloc would) makes the planner return NULL with the reason in
    fftw_gb300_last_error, for single-pass, four-step and r2c plans; the
    injection fires once and the next plan is whole."""
    lib.fftw_gb300_fail_alloc_after.argtypes = [ctypes.c_int]
    for make in (lambda: g.plan_many_dft([4096], 64, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f"),
                 lambda: g.plan_many_dft([1 << 20], 4, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f"),
                 lambda: g.plan_many_dft_r2c([16384], 8, 1 << 20, 1 << 30, g.FFTW_ESTIMATE, "f")):
        lib.fftw_gb300_fail_alloc_after(after)
        try:
            p = make()
        except Exception:
            p = None
        failed = p is None or not getattr(p, "ptr", None)
        lib.fftw_gb300_fail_alloc_after(-1)
        if failed:
            assert "injected" in g.last_error()
        q = make()
        assert q is not None and q.ptr and len(q.passes()) >= 1
    # the single-pass plan needs more than one table, so the first allocation fails it
    lib.fftw_gb300_fail_alloc_after(0)
    with pytest.raises(Exception):
        p = g.plan_many_dft([4096], 64, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        if p is None or not p.ptr:
            raise RuntimeError(g.last_error())
    lib.fftw_gb300_fail_alloc_after(-1)


def test_infeasible_wisdom_still_plans(lib):
    """Wisdom entries whose configuration cannot apply (an unknown variant, a
    tile too large for one CTA, a split that does not divide the length,
    Rader for a prime whose n-1 has a factor above 13) leave the planner to
    its own choices: every plan builds and stays within the launch limits,
    as the reference forgets infeasible wisdom and re-plans
    (api/apiplan.c:51-84)."""
    lib.fftwf_forget_wisdom()
    head = ctypes.string_at(lib.fftwf_export_wisdom_to_string()).decode().rstrip().rstrip(")")
    ent = lambda key, *f: '  (gb300-pass "%s" %s)\n' % (key, " ".join("#x%x" % (v & 0xffffffff) for v in f))
    cases = [("c2c p4 n4096", 7, 1000, 2, 2, 0, 0, 0), ("c2c p4 n4096", 1, 1000, 0, 0, 0, 0, 0),
             ("c2c p4 n65536", -1, 0, 0, 0, 3, 0, 0), ("c2c p4 n1021", 5, 0, 0, 0, 0, 0, 0)]
    for c in cases:
        lib.fftwf_forget_wisdom()
        assert lib.fftwf_import_wisdom_from_string((head + ent(*c) + ")\n").encode()) == 1
        n = int(c[0].split("n")[-1])
        p = g.plan_many_dft([n], 64, 1 << 20, 1 << 30, -1, g.FFTW_ESTIMATE, "f")
        ps = p.passes()
        assert ps and all(x["threads"] <= 1024 and x["smem"] <= 232448 and x["tb"] >= 1 for x in ps), (c, ps)
        tot = 1
        for x in ps:
            if x["kind"] == 0:
                tot *= x["nfft"]
        assert tot == n or ps[0]["kind"] == 3, (c, ps)
    lib.fftwf_forget_wisdom()


def test_real_tensor_core_form(monkeypatch):
    """FFTW_GB300_TENSOR_CORE r2c / c2r of an even length whose half length is
    a power of two of 256..4096: the half-length c2c runs in the tensor-core
    form beside the hc2c post- (r2c) or pre-pass (c2r); the 2D 8192^2 r2c
    takes it for its rows, the columns stay FP32; without the flag the
    single fused r2c pass is kept, and r2c 16384 (an 8192-point core) stays
    FP32."""
    TC, HC2C = 1 << 28, 6
    monkeypatch.delenv("FFTW_GB300_TC_CTAS", raising=False)
    def shape(p):
        return [(x["kind"], x["nfft"], x["variant"]) for x in p.passes()]
    assert shape(g.plan_many_dft_r2c([8192], 64, 1 << 20, 1 << 30, g.FFTW_ESTIMATE | TC, "f")) == \
        [(0, 4096, 3), (HC2C, 4096, 1)]
    assert shape(g.plan_many_dft_c2r([8192], 64, 1 << 20, 1 << 30, g.FFTW_ESTIMATE | TC, "f")) == \
        [(HC2C, 4096, 1), (0, 4096, 3)]
    assert shape(g.plan_many_dft_r2c([8192], 64, 1 << 20, 1 << 30, g.FFTW_ESTIMATE, "f")) == [(1, 4096, 2)]
    assert shape(g.plan_many_dft_r2c([16384], 64, 1 << 20, 1 << 30, g.FFTW_ESTIMATE | TC, "f")) == [(1, 8192, 2)]
    r2d = shape(g.plan_many_dft_r2c([8192, 8192], 1, 1 << 20, 1 << 32, g.FFTW_ESTIMATE | TC, "f"))
    assert r2d[:2] == [(0, 4096, 3), (HC2C, 4096, 1)] and all(v != 3 for _, _, v in r2d[2:])
