"""Planner robustness, checked without a GPU (dry-run plans): seeded random
problems of every planner family — c2c up to rank 4 with prime, smooth and
long lengths, strided and in place; r2c / c2r with long prime last dims and
real strides; r2r of any kind and rank; split-array c2c / r2c / c2r — must
all plan (non-NULL) and describe themselves within the description buffer,
with every pass inside the launch limits."""
import ctypes
import random

import pytest

import fftw3_gb300 as g


@pytest.fixture(autouse=True)
def dry(lib):
    g.set_dry_run(True)
    yield
    g.set_dry_run(False)


def check(p):
    assert len(p.describe()) <= 1023
    for ps in p.passes():
        assert 1 <= ps["threads"] <= 1024 and ps["tb"] >= 1 and 0 <= ps["smem"] <= 232448


@pytest.mark.parametrize("prec", ["f", "d"])
def test_c2c_sweep(prec):
    rng = random.Random(3)
    lens = [1, 2, 3, 13, 17, 64, 97, 173, 1000, 1021, 4093, 4096, 4099, 8192, 12289, 65537, 100003, 1 << 20]
    planned = 0
    for _ in range(300):
        rank = rng.choice([1, 1, 2, 3, 4])
        n = [rng.choice(lens) for _ in range(rank)]
        tot = 1
        for x in n:
            tot *= x
        if tot > 1 << 28:
            continue
        ist, inplace = rng.choice([1, 2, 3]), rng.random() < 0.2
        ost = ist if inplace else rng.choice([1, 2])
        out = 1 << 20 if inplace else 1 << 40
        check(g.plan_many_dft(n, rng.choice([1, 5]), 1 << 20, out, rng.choice([-1, 1]), g.FFTW_ESTIMATE, prec,
                              istride=ist, idist=tot * ist, ostride=ost, odist=tot * ost))
        planned += 1
    assert planned >= 150


@pytest.mark.parametrize("prec", ["f", "d"])
def test_real_sweep(prec):
    rng = random.Random(4)
    lens = [2, 3, 15, 16, 17, 97, 1021, 2049, 4096, 4099, 8198, 12297, 65537, 131074]
    planned = 0
    for _ in range(120):
        rank = rng.choice([1, 1, 2, 3])
        n = [min(rng.choice(lens), 3000) for _ in range(rank - 1)] + [rng.choice(lens)]
        nr = 1
        for x in n:
            nr *= x
        if nr > 1 << 28:
            continue
        nc = nr // n[-1] * (n[-1] // 2 + 1)
        st = rng.choice([1, 2])
        check(g.plan_many_dft_r2c(n, 2, 1 << 20, 1 << 40, g.FFTW_ESTIMATE, prec, istride=st, idist=nr * st,
                                  odist=nc))
        check(g.plan_many_dft_c2r(n, 2, 1 << 40, 1 << 20, g.FFTW_ESTIMATE, prec, idist=nc, ostride=st,
                                  odist=nr * st))
        planned += 1
    assert planned >= 60


@pytest.mark.parametrize("prec", ["f", "d"])
def test_r2r_sweep(lib, prec):
    rng = random.Random(5)
    f = getattr(lib, ("fftwf_" if prec == "f" else "fftw_") + "plan_many_r2r")
    f.restype = ctypes.c_void_p
    for _ in range(300):
        rank = rng.choice([1, 1, 2, 3])
        n = [rng.choice([1, 2, 3, 5, 8, 17, 100, 127, 256, 1021, 4096, 4097, 100003]) for _ in range(rank)]
        if rank > 1:
            n = [min(x, 300) for x in n]
        kinds = [rng.randrange(11) for _ in range(rank)]
        if any(k == 3 and x == 1 for k, x in zip(kinds, n)):
            continue
        tot = 1
        for x in n:
            tot *= x
        p = f(rank, (ctypes.c_int * rank)(*n), 2, 1 << 20, None, 1, tot, 1 << 40, None, 1, tot,
              (ctypes.c_int * rank)(*kinds), 64)
        assert p, (n, kinds, g.last_error())
        assert len(getattr(lib, ("fftwf_" if prec == "f" else "fftw_") + "sprint_plan")(p)) <= 1023


def test_split_sweep():
    rng = random.Random(6)
    base = 1 << 20
    for _ in range(200):
        prec, kind = rng.choice("fd"), rng.choice(["c2c", "r2c", "c2r"])
        rank = rng.choice([1, 1, 2, 3])
        n = [rng.choice([1, 2, 3, 16, 17, 100, 1021, 4096, 4099]) for _ in range(rank)]
        si, so = rng.choice([1, 2, 3]), rng.choice([1, 2, 3])
        dims = []
        for d in reversed(range(rank)):
            dims.insert(0, (n[d], si, so))
            si *= n[d]
            so *= (n[d] // 2 + 1) if (d == rank - 1 and kind != "c2c") else n[d]
        hd = [(3, si, so)]
        if kind == "c2c":
            p = g.plan_guru_split_dft(dims, hd, base, base + (1 << 34), base + (2 << 34), base + (3 << 34), prec=prec)
        elif kind == "r2c":
            p = g.plan_guru_split_dft_r2c(dims, hd, base, base + (2 << 34), base + (3 << 34), prec=prec)
        else:
            p = g.plan_guru_split_dft_c2r(dims, hd, base, base + (1 << 34), base + (2 << 34), prec=prec)
        check(p)


@pytest.mark.parametrize("groups", [None, "2"])
def test_two_group_passes_are_whole_warps(lib, monkeypatch, groups):
    """A persistent pass with two compute groups per CTA synchronises each
    group with its own named barrier, which counts whole warps: every such
    pass the planner emits has a thread count per group that is a multiple
    of 32 (small column tiles keep one group and the CTA-wide barrier), by
    default and when two groups are asked for everywhere."""
    import re
    import fftw3_gb300 as g
    if groups:
        monkeypatch.setenv("FFTW_GB300_TMA_GROUPS", groups)
    g.set_dry_run(True)
    try:
        shapes = [[16, 16], [32, 16], [16, 64], [8, 8, 8], [64, 64], [128, 32], [512, 512, 512], [256, 256],
                  [2048, 8], [16, 2048], [65536], [1 << 20], [4096], [256], [64], [2, 1024], [1024, 4], [8192]]
        seen = 0
        for shape in shapes:
            for hm in (1, 3, 64):
                for prec in ("f", "d"):
                    p = g.plan_many_dft(shape, hm, 1 << 20, 1 << 24, -1, g.FFTW_ESTIMATE, prec)
                    for line in p.describe().splitlines():
                        m = re.search(r"(reg-tma|cols-tma)( groups=2)? tb=(\d+) thr=(\d+)", line)
                        if m and m.group(2):
                            seen += 1
                            assert int(m.group(4)) % 32 == 0, (shape, hm, prec, line)
        assert seen > 0
    finally:
        g.set_dry_run(False)
