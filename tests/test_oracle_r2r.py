"""The oracle's r2r restatement against the defining sums of the reference
manual, evaluated independently here with numpy in float64, and against the
reference's own r2r planner (oracle/_ref, built from the reference sources
where they are present) for the lengths its codelet-free build can plan
(CPU only)."""
import numpy as np
import pytest

from oracle.oracle import Reference, ref_available

KINDS = {0: "R2HC", 1: "HC2R", 2: "DHT", 3: "REDFT00", 4: "REDFT01", 5: "REDFT10", 6: "REDFT11", 7: "RODFT00",
         8: "RODFT01", 9: "RODFT10", 10: "RODFT11"}


def definition(kind, x):
    n = len(x)
    j = np.arange(n)
    k = j[:, None]
    if kind == 0:
        X = np.fft.fft(x)
        return np.concatenate([X.real[: n // 2 + 1], X.imag[1:(n + 1) // 2][::-1]])
    if kind == 1:
        X = np.zeros(n, dtype=complex)
        X[: n // 2 + 1] = x[: n // 2 + 1]
        for m in range(1, (n + 1) // 2):
            X[m] += 1j * x[n - m]
            X[n - m] = np.conj(X[m])
        return np.real(np.fft.ifft(X) * n)
    if kind == 2:
        return (np.cos(2 * np.pi * j * k / n) + np.sin(2 * np.pi * j * k / n)) @ x
    if kind == 3:
        return x[0] + ((-1.0) ** j) * x[-1] + 2 * np.cos(np.pi * j[1:-1] * k / (n - 1)) @ x[1:-1]
    if kind == 6:
        return 2 * np.cos(np.pi * (2 * j + 1) * (2 * k + 1) / (4 * n)) @ x
    if kind == 7:
        return 2 * np.sin(np.pi * (j + 1) * (k + 1) / (n + 1)) @ x
    if kind == 10:
        return 2 * np.sin(np.pi * (2 * j + 1) * (2 * k + 1) / (4 * n)) @ x
    if kind == 4:
        return x[0] + 2 * np.cos(np.pi * j[1:] * (2 * k + 1) / (2 * n)) @ x[1:]
    if kind == 5:
        return 2 * np.cos(np.pi * (2 * j + 1) * k / (2 * n)) @ x
    if kind == 8:
        return ((-1.0) ** j) * x[-1] + 2 * np.sin(np.pi * (j[:-1] + 1) * (2 * k + 1) / (2 * n)) @ x[:-1]
    return 2 * np.sin(np.pi * (2 * j + 1) * (k + 1) / (2 * n)) @ x


@pytest.mark.parametrize("kind", sorted(KINDS), ids=[KINDS[k] for k in sorted(KINDS)])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 16, 33, 100])
def test_r2r_oracle_matches_definition(restatement, kind, n):
    if kind == 3 and n == 1:
        pytest.skip("a size-1 REDFT00 is not defined")
    rng = np.random.default_rng(n * 16 + kind)
    x = rng.standard_normal((3, n))
    y = restatement.r2r(x.ravel(), n, kind, "l").astype(np.float64).reshape(3, n)
    ref = np.stack([definition(kind, r) for r in x])
    assert np.abs(y - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_r2r_oracle_rejects_size1_redft00(restatement):
    with pytest.raises(AssertionError):
        restatement.r2r(np.ones(1), 1, 3, "d")


def test_r2r_nd_oracle_is_separable(restatement):
    """r2r_nd applies the 1D kind of each dim along that dim: a 2D DCT-II x
    DST-I equals the matrix product of the two 1D transform matrices."""
    rng = np.random.default_rng(7)
    n0, n1 = 5, 6
    x = rng.standard_normal((2, n0, n1))
    y = restatement.r2r_nd(x.ravel(), [n0, n1], [5, 7], "d").reshape(2, n0, n1)
    m0 = np.stack([definition(5, e) for e in np.eye(n0)], axis=1)
    m1 = np.stack([definition(7, e) for e in np.eye(n1)], axis=1)
    ref = np.einsum("ia,bj,tab->tij", m0, m1.T, x)
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.skipif(not ref_available(), reason="the reference build (oracle/_ref) is not on this machine")
@pytest.mark.parametrize("kind", [k for k in sorted(KINDS) if k not in (3, 7)], ids=lambda k: KINDS[k])
@pytest.mark.parametrize("n", [1, 3, 5, 7, 9, 15, 21, 105])
def test_r2r_oracle_matches_reference(restatement, kind, n):
    """Pins the restatement to the reference itself: odd lengths of the nine
    kinds its codelet-free build plans (REDFT00 / RODFT00 have even logical
    sizes, which that build cannot plan)."""
    rng = np.random.default_rng(1000 + 16 * n + kind)
    x = rng.standard_normal(4 * n)
    ref = Reference("d").r2r(x, n, kind)
    assert ref is not None, "the reference planner returned NULL"
    y = restatement.r2r(x, n, kind, "l").astype(np.float64)
    assert np.abs(y - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


@pytest.mark.skipif(not ref_available(), reason="the reference build (oracle/_ref) is not on this machine")
@pytest.mark.parametrize("kind", [3, 7], ids=lambda k: KINDS[k])
@pytest.mark.parametrize("n", [2, 3, 8, 17, 100])
def test_r2r_oracle_dct1_dst1_match_reference_dft(restatement, kind, n):
    """REDFT00 / RODFT00 pinned through the reference's complex DFT of the
    even / odd extension (logical sizes 2(n-1) / 2(n+1)): DCT-I is the real
    part of bins 0..n-1, DST-I minus the imaginary part of bins 1..n."""
    rng = np.random.default_rng(2000 + 16 * n + kind)
    x = rng.standard_normal((3, n))
    if kind == 3:
        ext = np.concatenate([x, x[:, -2:0:-1]], axis=1)
    else:
        z = np.zeros((3, 1))
        ext = np.concatenate([z, x, z, -x[:, ::-1]], axis=1)
    N = ext.shape[1]
    full = Reference("d").c2c(ext.astype(np.complex128).ravel(), [N]).reshape(3, N)
    ref = full[:, :n].real if kind == 3 else -full[:, 1:n + 1].imag
    y = restatement.r2r(x.ravel(), n, kind, "l").astype(np.float64).reshape(3, n)
    assert np.abs(y - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


def _golden_r2r():
    import json
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_r2r.npz"))
    out = []
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["key"]
        yl = z[k + "_yl_hi"].astype(np.longdouble) + z[k + "_yl_lo"].astype(np.longdouble)
        out.append(dict(m, x=z[k + "_x"], yd=z[k + "_yd"], yl=yl))
    return out


GOLDEN_R2R = _golden_r2r()


@pytest.mark.parametrize("case", GOLDEN_R2R, ids=[f"{KINDS[c['kind']]}-n{c['n']}" for c in GOLDEN_R2R])
def test_r2r_oracle_matches_reference_golden(restatement, case):
    """The restatement against the reference's own r2r outputs committed in
    tests/golden/golden_r2r.npz (gen_golden_r2r.py): double vs the reference's
    double, long double vs its long double."""
    x, n, kind = case["x"], case["n"], case["kind"]
    yd = restatement.r2r(x, n, kind, "d")
    yl = restatement.r2r(x.astype(np.longdouble), n, kind, "l")
    scale = max(1.0, float(np.abs(case["yd"]).max()))
    assert np.abs(yd - case["yd"]).max() <= 1e-14 * scale
    assert float(np.abs(yl - case["yl"]).max()) <= 1e-17 * scale


@pytest.mark.parametrize("kind", sorted(KINDS), ids=[KINDS[k] for k in sorted(KINDS)])
def test_r2r_fast_oracle_matches_defining_sums(restatement, kind):
    """The O(n log n) restatement (real DFT of the symmetric extension)
    against the defining sums, and against the reference's golden outputs."""
    for n in (1, 2, 3, 4, 7, 16, 33, 100, 257):
        if kind == 3 and n == 1:
            continue
        x = np.random.default_rng(3000 + 16 * n + kind).standard_normal(3 * n)
        ref = restatement.r2r(x.astype(np.longdouble), n, kind, "l").astype(np.float64)
        y = restatement.r2r_fast(x, n, kind, "d")
        assert np.abs(y - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), n
    for case in GOLDEN_R2R:
        if case["kind"] == kind:
            y = restatement.r2r_fast(case["x"], case["n"], kind, "d")
            assert np.abs(y - case["yd"]).max() <= 1e-14 * max(1.0, float(np.abs(case["yd"]).max()))
