"""Python access to the oracle.  TEST INFRASTRUCTURE ONLY.

Two CPU implementations of the reference algorithms are reachable here:

* ``Restatement`` -- ``oracle/_build/liboracle_fft.so``, the C restatement in
  ``fft_oracle_impl.h`` (float / double / long double, threaded).  Builds
  anywhere gcc is present, including the GPU host.
* ``Reference`` -- ``oracle/_ref/libfftw3_ref{,f,l}.so``, the reference FFTW
  compiled from its own sources without generated codelets (only where the
  reference checkout exists).  Used to pin the restatement and to generate
  the golden fixtures under ``tests/golden/``.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")

_PREC = {
    "f": (np.float32, np.complex64),
    "d": (np.float64, np.complex128),
    "l": (np.longdouble, np.clongdouble),
}

FFTW_FORWARD = -1
FFTW_BACKWARD = 1
FFTW_ESTIMATE = 1 << 6
FFTW_ALLOW_LARGE_GENERIC = 1 << 13


def ref_root() -> str | None:
    """The reference FFTW checkout: the directory FFTW_REF_SRC names, else a
    checkout named ``reference`` beside this repository; None where neither
    exists (the reference is then only present through the committed
    fixtures under tests/golden/)."""
    env = os.environ.get("FFTW_REF_SRC")
    cands = [env] if env else [os.path.join(os.path.dirname(HERE), os.pardir, "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "api", "fftw3.h")):
            return os.path.realpath(c)
    return None


def build(ref: bool = False) -> None:
    """Compile the restatement (and, if asked and possible, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "restate"], check=True)
    src = ref_root()
    if ref and src:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + src], check=True)


def ref_source(rel: str) -> str | None:
    """Path of a file of the reference checkout, or None where the
    reference sources are absent."""
    src = ref_root()
    path = os.path.join(src, rel) if src else None
    return path if path and os.path.isfile(path) else None


def harness() -> str | None:
    """Build the reference's own benchmark harness (tests/bench.c +
    libbench2) against this library's fftw3.h and libfftw3_gb300.so, where
    the reference sources exist; returns the executable's path, else None.
    The executable answers `--can-do <problem>` from this library's planner
    in dry-run mode (oracle/ref/harness_shim.c)."""
    if ref_source(os.path.join("tests", "bench.c")) is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "harness", "REF=" + ref_root()], check=True)
    return os.path.join(REFDIR, "bench_gb300")


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REFDIR, f"libfftw3_ref{p}.so")) for p in ("", "f", "l"))


def _as(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Restatement:
    """The C restatement of the reference algorithms."""

    _lib = None

    def __init__(self):
        if Restatement._lib is None:
            path = os.path.join(BUILD, "liboracle_fft.so")
            if not os.path.exists(path):
                build()
            lib = ctypes.CDLL(path)
            I = ctypes.c_longlong
            for p in "fdl":
                getattr(lib, f"orc_{p}_c2c").argtypes = [ctypes.c_int, ctypes.c_void_p, I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
                getattr(lib, f"orc_{p}_r2c").argtypes = [ctypes.c_int, ctypes.c_void_p, I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
                getattr(lib, f"orc_{p}_c2r").argtypes = [ctypes.c_int, ctypes.c_void_p, I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
                getattr(lib, f"orc_{p}_dft_method").argtypes = [I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
                getattr(lib, f"orc_{p}_twiddle").argtypes = [I, I, ctypes.c_int, ctypes.c_void_p]
                getattr(lib, f"orc_{p}_r2r").argtypes = [ctypes.c_int, I, I, ctypes.c_void_p, ctypes.c_void_p]
                getattr(lib, f"orc_{p}_r2r_fast").argtypes = [ctypes.c_int, I, I, ctypes.c_void_p, ctypes.c_void_p,
                                                              ctypes.c_int]
            Restatement._lib = lib
        self.lib = Restatement._lib

    def c2c(self, x, shape, sign=FFTW_FORWARD, prec="d", nthreads=1):
        """Batched row-major c2c; x has shape (howmany, *shape) or flat."""
        rt, ct = _PREC[prec]
        x = _as(x, ct)
        tot = int(np.prod(shape))
        howmany = x.size // tot
        y = np.empty(x.size, dtype=ct)
        n = (ctypes.c_int * len(shape))(*shape)
        rc = getattr(self.lib, f"orc_{prec}_c2c")(len(shape), n, howmany, x.ctypes.data, y.ctypes.data, sign, nthreads)
        assert rc == 0
        return y.reshape(x.shape)

    def r2c(self, x, shape, prec="d", nthreads=1):
        rt, ct = _PREC[prec]
        x = _as(x, rt)
        tot = int(np.prod(shape))
        howmany = x.size // tot
        nc = tot // shape[-1] * (shape[-1] // 2 + 1)
        y = np.empty(howmany * nc, dtype=ct)
        n = (ctypes.c_int * len(shape))(*shape)
        rc = getattr(self.lib, f"orc_{prec}_r2c")(len(shape), n, howmany, x.ctypes.data, y.ctypes.data, nthreads)
        assert rc == 0
        return y

    def c2r(self, x, shape, prec="d", nthreads=1):
        rt, ct = _PREC[prec]
        x = _as(x, ct)
        tot = int(np.prod(shape))
        nc = tot // shape[-1] * (shape[-1] // 2 + 1)
        howmany = x.size // nc
        y = np.empty(howmany * tot, dtype=rt)
        n = (ctypes.c_int * len(shape))(*shape)
        rc = getattr(self.lib, f"orc_{prec}_c2r")(len(shape), n, howmany, x.ctypes.data, y.ctypes.data, nthreads)
        assert rc == 0
        return y

    def r2r(self, x, n, kind, prec="d"):
        """Batched 1D r2r of length n by its defining sum (kinds: fftw_r2r_kind values)."""
        rt, _ = _PREC[prec]
        x = _as(x, rt)
        y = np.empty(x.size, dtype=rt)
        rc = getattr(self.lib, f"orc_{prec}_r2r")(int(kind), int(n), x.size // int(n), x.ctypes.data, y.ctypes.data)
        assert rc == 0, f"r2r kind {kind} is not restated"
        return y

    def r2r_fast(self, x, n, kind, prec="d", nthreads=1):
        """Batched 1D r2r of length n in O(n log n): the real DFT of the
        kind's symmetric extension (same results as r2r, for large n)."""
        rt, _ = _PREC[prec]
        x = _as(x, rt)
        y = np.empty(x.size, dtype=rt)
        rc = getattr(self.lib, f"orc_{prec}_r2r_fast")(int(kind), int(n), x.size // int(n), x.ctypes.data,
                                                       y.ctypes.data, int(nthreads))
        assert rc == 0, f"r2r kind {kind} of size {n} is not defined"
        return y

    def r2r_nd(self, x, shape, kinds, prec="d"):
        """Multi-dimensional r2r of a row-major array of the given shape
        (batched over any leading elements): the 1D r2r of kinds[d] along each
        dim d, the separable product the reference defines."""
        rt, _ = _PREC[prec]
        r = len(shape)
        a = _as(x, rt).reshape((-1,) + tuple(shape))
        for d in range(r):
            ax = 1 + d
            b = np.ascontiguousarray(np.moveaxis(a, ax, -1))
            y = self.r2r(b.ravel(), shape[d], kinds[d], prec).reshape(b.shape)
            a = np.moveaxis(y, -1, ax)
        return np.ascontiguousarray(a).ravel()

    def dft_method(self, x, sign=FFTW_FORWARD, method=1, prec="d"):
        """One 1D DFT with a named solver: 1 CT, 2 generic, 3 Rader, 4 Bluestein."""
        rt, ct = _PREC[prec]
        x = _as(x, ct)
        y = np.empty_like(x)
        rc = getattr(self.lib, f"orc_{prec}_dft_method")(x.size, x.ctypes.data, y.ctypes.data, sign, method)
        assert rc == 0
        return y

    def twiddle(self, m, n, sign=FFTW_FORWARD, prec="d"):
        rt, ct = _PREC[prec]
        out = np.empty(2, dtype=rt)
        getattr(self.lib, f"orc_{prec}_twiddle")(m, n, sign, out.ctypes.data)
        return complex(out[0], out[1])


class Reference:
    """The reference FFTW (codelet-free build) through its public API."""

    _libs: dict = {}

    def __init__(self, prec="d"):
        self.prec = prec
        pfx = {"d": "fftw_", "f": "fftwf_", "l": "fftwl_"}[prec]
        self.pfx = pfx
        if prec not in Reference._libs:
            path = os.path.join(REFDIR, f"libfftw3_ref{'' if prec == 'd' else prec}.so")
            lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL)
            vp, ci, cu = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint
            ip = ctypes.POINTER(ctypes.c_int)
            f = getattr(lib, pfx + "plan_many_dft")
            f.restype = vp
            f.argtypes = [ci, ip, ci, vp, vp, ci, ci, vp, vp, ci, ci, ci, cu]
            for nm in ("plan_many_dft_r2c", "plan_many_dft_c2r"):
                f = getattr(lib, pfx + nm)
                f.restype = vp
                f.argtypes = [ci, ip, ci, vp, vp, ci, ci, vp, vp, ci, ci, cu]
            f = getattr(lib, pfx + "plan_many_r2r")
            f.restype = vp
            f.argtypes = [ci, ip, ci, vp, vp, ci, ci, vp, vp, ci, ci, ip, cu]
            getattr(lib, pfx + "execute").argtypes = [vp]
            getattr(lib, pfx + "destroy_plan").argtypes = [vp]
            getattr(lib, pfx + "plan_with_nthreads").argtypes = [ci]
            getattr(lib, pfx + "init_threads").restype = ci
            getattr(lib, pfx + "init_threads")()
            Reference._libs[prec] = lib
        self.lib = Reference._libs[prec]

    def _fn(self, name):
        return getattr(self.lib, self.pfx + name)

    def c2c(self, x, shape, sign=FFTW_FORWARD, flags=FFTW_ESTIMATE | FFTW_ALLOW_LARGE_GENERIC, nthreads=1):
        rt, ct = _PREC[self.prec]
        x = np.array(x, dtype=ct).ravel()   # planner may scribble; work on a copy
        tot = int(np.prod(shape))
        howmany = x.size // tot
        y = np.zeros(x.size, dtype=ct)
        n = (ctypes.c_int * len(shape))(*shape)
        self._fn("plan_with_nthreads")(nthreads)
        p = self._fn("plan_many_dft")(len(shape), n, howmany, x.ctypes.data, None, 1, tot,
                                      y.ctypes.data, None, 1, tot, sign, flags)
        if not p:
            raise RuntimeError(f"reference could not plan c2c {shape}")
        self._fn("execute")(p)
        self._fn("destroy_plan")(p)
        return y

    def r2r(self, x, n, kind, flags=FFTW_ESTIMATE | FFTW_ALLOW_LARGE_GENERIC):
        """Batched 1D r2r of length n through the reference's own r2r planner.
        The codelet-free build plans odd lengths of every kind but REDFT00 and
        RODFT00 (whose logical sizes 2(n-1), 2(n+1) are even); None when the
        planner returns NULL."""
        rt, _ = _PREC[self.prec]
        x = np.array(x, dtype=rt).ravel()
        howmany = x.size // int(n)
        y = np.zeros(x.size, dtype=rt)
        nn = (ctypes.c_int * 1)(int(n))
        kk = (ctypes.c_int * 1)(int(kind))
        p = self._fn("plan_many_r2r")(1, nn, howmany, x.ctypes.data, None, 1, int(n), y.ctypes.data, None, 1,
                                      int(n), kk, flags)
        if not p:
            return None
        self._fn("execute")(p)
        self._fn("destroy_plan")(p)
        return y

    def r2c(self, x, shape, **kw):
        """Reference r2c: the codelet-free build cannot plan even-length r2c,
        so the r2c result is its c2c of the real data, bins 0..n/2 of the
        last axis kept (the reference's own arithmetic via its complex path)."""
        rt, ct = _PREC[self.prec]
        x = np.asarray(x, dtype=rt).reshape(-1, *shape)
        full = self.c2c(x.astype(ct), shape, FFTW_FORWARD, **kw).reshape(x.shape)
        return np.ascontiguousarray(full[..., : shape[-1] // 2 + 1]).ravel()

    def c2r(self, x, shape, **kw):
        """Reference c2r semantics via its complex path: c2c backward over
        the leading axes, then the last axis as a Hermitian-extended
        backward c2c whose real part is kept (rdft/rank-geq2-rdft2.c:56-69)."""
        rt, ct = _PREC[self.prec]
        nl = shape[-1]
        nc = nl // 2 + 1
        x = np.array(x, dtype=ct).reshape(-1, *shape[:-1], nc)
        if len(shape) > 1:
            lead = list(shape[:-1])
            # c2c backward over leading axes: move last axis into the batch
            xt = np.moveaxis(x, -1, 1).copy()  # (B, nc, *lead)
            yt = self.c2c(xt, lead, FFTW_BACKWARD, **kw).reshape(xt.shape)
            x = np.moveaxis(yt, 1, -1)
        full = np.zeros(x.shape[:-1] + (nl,), dtype=ct)
        full[..., :nc] = x
        full[..., 0] = full[..., 0].real
        for k in range(1, nc):
            if nl - k >= nc:
                full[..., nl - k] = np.conj(x[..., k])
        if nl % 2 == 0:
            full[..., nl // 2] = full[..., nl // 2].real
        y = self.c2c(full.reshape(-1, nl), [nl], FFTW_BACKWARD, **kw)
        return np.ascontiguousarray(y.real.astype(rt)).ravel()


def rel_l2(y, ref):
    y = np.asarray(y).astype(np.clongdouble if np.iscomplexobj(y) or np.iscomplexobj(ref) else np.longdouble).ravel()
    ref = np.asarray(ref).astype(y.dtype).ravel()
    den = np.sqrt(np.sum(np.abs(ref) ** 2))
    num = np.sqrt(np.sum(np.abs(y - ref) ** 2))
    return float(num / den) if den > 0 else float(num)
