"""The oracle (C restatement of the reference algorithms) against the golden
vectors produced by the reference FFTW itself (tests/golden/gen_golden.py),
and against the reference live when oracle/_ref is built here."""
import numpy as np
import pytest

from conftest import golden_cases, rel_l2

CASES = golden_cases()


@pytest.mark.parametrize("case", CASES, ids=[f"{c['kind']}-{'x'.join(map(str, c['shape']))}-h{c['howmany']}-s{c['sign']}" for c in CASES])
def test_restatement_matches_reference_golden(restatement, case):
    kind, shape, x = case["kind"], case["shape"], case["x"]
    for prec, tol_d, tol_l in (("d", 1e-14, 1e-14), ("l", 1e-14, 1e-17)):
        if kind == "c2c":
            y = restatement.c2c(x.astype(np.clongdouble if prec == "l" else np.complex128), shape, case["sign"], prec)
        elif kind == "r2c":
            y = restatement.r2c(x, shape, prec)
        else:
            y = restatement.c2r(x, shape, prec)
        assert rel_l2(y, case["yd"]) <= tol_d, (prec, "vs reference double")
        assert rel_l2(y, case["yl"]) <= tol_l, (prec, "vs reference long double")


def test_restatement_solvers_agree(restatement):
    """Cooley-Tukey, generic O(n^2), Rader and Bluestein give the same DFT
    (dft/ct.c, dft/generic.c, dft/rader.c, dft/bluestein.c)."""
    rng = np.random.default_rng(7)
    for n in (17, 31, 101, 257, 1021):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        ref = restatement.dft_method(x, -1, 2, "l")
        for m in (1, 3, 4):
            assert rel_l2(restatement.dft_method(x, -1, m, "l"), ref) < 1e-17


def test_restatement_twiddle_octants(restatement):
    """Octant-reduced twiddles (kernel/trig.c:57-80) equal exp(-2 pi i m/n)
    to within one double rounding (checked against long-double sin/cos)."""
    pi_l = np.longdouble("3.14159265358979323846264338327950288")
    for n in (7, 8, 12, 1000, 4096):
        for m in range(0, n, max(1, n // 37)):
            w = restatement.twiddle(m, n, -1, "d")
            th = 2 * pi_l * np.longdouble(m) / np.longdouble(n)
            assert abs(w.real - float(np.cos(th))) <= 2.3e-16
            assert abs(w.imag + float(np.sin(th))) <= 2.3e-16


def _ref_ok():
    from oracle.oracle import ref_available
    return ref_available()


@pytest.mark.skipif(not _ref_ok(), reason="oracle/_ref not built (reference sources absent)")
def test_restatement_matches_reference_live(restatement):
    from oracle.oracle import Reference
    refd = Reference("d")
    rng = np.random.default_rng(11)
    for shape in ([12], [96], [243], [625], [1001], [4100], [6, 35], [3, 4, 5]):
        x = rng.standard_normal(2 * int(np.prod(shape))) + 1j * rng.standard_normal(2 * int(np.prod(shape)))
        for sign in (-1, 1):
            assert rel_l2(restatement.c2c(x, shape, sign, "d"), refd.c2c(x, shape, sign)) < 1e-14
