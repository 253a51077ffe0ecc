"""Python binding of libfftw3_gb300 (ctypes over the C ABI in include/fftw3.h).

The product is the C shared library ``libfftw3_gb300.so``: a GB300-native
implementation of FFTW's plan/execute path.  This module only loads it and
declares the C signatures, so tests and the benchmark can call the same entry
points a C program would (``fftwf_plan_many_dft``, ``fftwf_execute_dft``, ...).
It never computes a transform itself: if the library is missing, loading
fails loudly.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIBPATH = os.path.join(PKG, "libfftw3_gb300.so")
HEADERS = [os.path.join(ROOT, "include", "fftw3.h"), os.path.join(ROOT, "include", "fftw3_gb300.h")]

FFTW_FORWARD = -1
FFTW_BACKWARD = 1
FFTW_MEASURE = 0
FFTW_DESTROY_INPUT = 1 << 0
FFTW_UNALIGNED = 1 << 1
FFTW_EXHAUSTIVE = 1 << 3
FFTW_PRESERVE_INPUT = 1 << 4
FFTW_PATIENT = 1 << 5
FFTW_ESTIMATE = 1 << 6
FFTW_WISDOM_ONLY = 1 << 21

_lib = None

vp = ctypes.c_void_p
ci = ctypes.c_int
cu = ctypes.c_uint
ip = ctypes.POINTER(ctypes.c_int)


class IODim(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("is_", ctypes.c_int), ("os", ctypes.c_int)]


class IODim64(ctypes.Structure):
    _fields_ = [("n", ctypes.c_ssize_t), ("is_", ctypes.c_ssize_t), ("os", ctypes.c_ssize_t)]


def _sigs(lib, pfx):
    def f(name, res, args):
        fn = getattr(lib, pfx + name)
        fn.restype = res
        fn.argtypes = args

    f("plan_many_dft", vp, [ci, ip, ci, vp, ip, ci, ci, vp, ip, ci, ci, ci, cu])
    f("plan_dft", vp, [ci, ip, vp, vp, ci, cu])
    f("plan_dft_1d", vp, [ci, vp, vp, ci, cu])
    f("plan_dft_2d", vp, [ci, ci, vp, vp, ci, cu])
    f("plan_dft_3d", vp, [ci, ci, ci, vp, vp, ci, cu])
    f("plan_guru_dft", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, ci, cu])
    f("plan_guru64_dft", vp, [ci, ctypes.POINTER(IODim64), ci, ctypes.POINTER(IODim64), vp, vp, ci, cu])
    f("plan_many_dft_r2c", vp, [ci, ip, ci, vp, ip, ci, ci, vp, ip, ci, ci, cu])
    f("plan_many_dft_c2r", vp, [ci, ip, ci, vp, ip, ci, ci, vp, ip, ci, ci, cu])
    f("plan_dft_r2c", vp, [ci, ip, vp, vp, cu])
    f("plan_dft_c2r", vp, [ci, ip, vp, vp, cu])
    f("plan_dft_r2c_1d", vp, [ci, vp, vp, cu])
    f("plan_dft_r2c_2d", vp, [ci, ci, vp, vp, cu])
    f("plan_dft_r2c_3d", vp, [ci, ci, ci, vp, vp, cu])
    f("plan_dft_c2r_1d", vp, [ci, vp, vp, cu])
    f("plan_dft_c2r_2d", vp, [ci, ci, vp, vp, cu])
    f("plan_dft_c2r_3d", vp, [ci, ci, ci, vp, vp, cu])
    f("plan_guru_dft_r2c", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, cu])
    f("plan_guru_dft_c2r", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, cu])
    f("plan_many_r2r", vp, [ci, ip, ci, vp, ip, ci, ci, vp, ip, ci, ci, vp, cu])
    f("execute_r2r", None, [vp, vp, vp])
    f("plan_guru_split_dft", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, vp, vp, cu])
    f("plan_guru64_split_dft", vp, [ci, ctypes.POINTER(IODim64), ci, ctypes.POINTER(IODim64), vp, vp, vp, vp, cu])
    f("execute_split_dft", None, [vp, vp, vp, vp, vp])
    f("plan_guru_split_dft_r2c", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, vp, cu])
    f("plan_guru_split_dft_c2r", vp, [ci, ctypes.POINTER(IODim), ci, ctypes.POINTER(IODim), vp, vp, vp, cu])
    f("execute_split_dft_r2c", None, [vp, vp, vp, vp])
    f("execute_split_dft_c2r", None, [vp, vp, vp, vp])
    f("execute", None, [vp])
    f("execute_dft", None, [vp, vp, vp])
    f("execute_dft_r2c", None, [vp, vp, vp])
    f("execute_dft_c2r", None, [vp, vp, vp])
    f("destroy_plan", None, [vp])
    f("copy_plan", vp, [vp])
    f("sprint_plan", ctypes.c_char_p, [vp])
    f("export_wisdom_to_string", ctypes.c_void_p, [])
    f("import_wisdom_from_string", ci, [ctypes.c_char_p])
    f("export_wisdom_to_filename", ci, [ctypes.c_char_p])
    f("import_wisdom_from_filename", ci, [ctypes.c_char_p])
    f("forget_wisdom", None, [])
    f("cleanup", None, [])
    f("malloc", vp, [ctypes.c_size_t])
    f("free", None, [vp])
    f("flops", None, [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                      ctypes.POINTER(ctypes.c_double)])
    f("alignment_of", ci, [vp])
    f("init_threads", ci, [])
    f("plan_with_nthreads", None, [ci])
    f("planner_nthreads", ci, [])
    f("set_timelimit", None, [ctypes.c_double])
    f("cost", ctypes.c_double, [vp])
    f("estimate_cost", ctypes.c_double, [vp])
    f("gb300_set_stream", ci, [vp, vp])
    f("gb300_set_async", ci, [vp, ci])
    f("gb300_npasses", ci, [vp])
    f("gb300_pass_info", ci, [vp, ci, ip, ip, ip, ip, ip, ip, ctypes.POINTER(ctypes.c_longlong)])
    f("gb300_scratch_bytes", ctypes.c_size_t, [vp])


def load(path: str | None = None):
    """Load the library (once).  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIBPATH
    if not os.path.exists(path):
        raise RuntimeError(f"libfftw3_gb300.so not built ({path}); run python -m fftw3_gb300.build")
    lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL)
    for pfx in ("fftw_", "fftwf_"):
        _sigs(lib, pfx)
    lib.fftw_gb300_last_error.restype = ctypes.c_char_p
    lib.fftw_gb300_last_error.argtypes = []
    lib.fftw_gb300_failures.restype = ci
    lib.fftw_gb300_set_dry_run.argtypes = [ci]
    lib.fftw_gb300_launch_count.restype = ctypes.c_longlong
    lib.fftw_gb300_fp64_fma_gflops.restype = ctypes.c_double
    lib.fftw_gb300_fp64_fma_gflops.argtypes = []
    lib.fftwf_gb300_dft_1d_noalloc.restype = ci
    lib.fftwf_gb300_dft_1d_noalloc.argtypes = [ci, ci, vp, vp, ci, vp]
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    """Every function/data symbol the public headers declare, per prefix."""
    names = []
    txt = open(HEADERS[0]).read()
    body = txt[txt.index("#define GB_FFTW_DECLARE"):txt.index("GB_FFTW_DECLARE(fftw_, double")]
    per = sorted(set(re.findall(r"PFX##(\w+)\s*[\(\[]", body)))
    for pfx in ("fftw_", "fftwf_"):
        names += [pfx + n for n in per]
    ext = open(HEADERS[1]).read()
    names += re.findall(r"extern [^;(]*?\b(fftwf?_gb300_\w+)\s*\(", ext)
    body = ext[ext.index("#define GB_FFTW_EXT_DECLARE"):ext.index("GB_FFTW_EXT_DECLARE(fftw_)")]
    per = sorted(set(re.findall(r"PFX##(\w+)\s*\(", body)))
    for pfx in ("fftw_", "fftwf_"):
        names += [pfx + n for n in per]
    return names


def last_error() -> str:
    return (load().fftw_gb300_last_error() or b"").decode()


class Plan:
    """A plan handle (owns one fftw[f]_plan)."""

    def __init__(self, ptr, prec: str):
        if not ptr:
            raise RuntimeError("planner returned NULL: " + last_error())
        self.ptr = ptr
        self.prec = prec
        self.pfx = "fftwf_" if prec == "f" else "fftw_"
        self.lib = load()

    def _f(self, name):
        return getattr(self.lib, self.pfx + name)

    def execute(self):
        self._f("execute")(self.ptr)

    def execute_dft(self, i, o):
        self._f("execute_dft")(self.ptr, i, o)

    def execute_dft_r2c(self, i, o):
        self._f("execute_dft_r2c")(self.ptr, i, o)

    def execute_dft_c2r(self, i, o):
        self._f("execute_dft_c2r")(self.ptr, i, o)

    def execute_r2r(self, i, o):
        self._f("execute_r2r")(self.ptr, i, o)

    def execute_split_dft(self, ri, ii, ro, io):
        self._f("execute_split_dft")(self.ptr, ri, ii, ro, io)

    def execute_split_dft_r2c(self, inp, ro, io):
        self._f("execute_split_dft_r2c")(self.ptr, inp, ro, io)

    def execute_split_dft_c2r(self, ri, ii, out):
        self._f("execute_split_dft_c2r")(self.ptr, ri, ii, out)

    def set_stream(self, stream_ptr: int):
        return self._f("gb300_set_stream")(self.ptr, stream_ptr)

    def set_async(self, on: bool):
        return self._f("gb300_set_async")(self.ptr, int(on))

    def describe(self) -> str:
        s = self._f("sprint_plan")(self.ptr)
        return s.decode() if s else ""

    def passes(self):
        out = []
        for i in range(self._f("gb300_npasses")(self.ptr)):
            v = [ctypes.c_int() for _ in range(6)]
            b = ctypes.c_longlong()
            self._f("gb300_pass_info")(self.ptr, i, *[ctypes.byref(x) for x in v], ctypes.byref(b))
            out.append(dict(kind=v[0].value, nfft=v[1].value, variant=v[2].value, tb=v[3].value,
                            threads=v[4].value, smem=v[5].value, blocks=b.value))
        return out

    def destroy(self):
        if self.ptr:
            self._f("destroy_plan")(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def _iarr(v):
    if v is None:
        return None
    return (ctypes.c_int * len(v))(*v)


def plan_many_dft(n, howmany, inp, out, sign=FFTW_FORWARD, flags=FFTW_ESTIMATE, prec="f",
                  inembed=None, istride=1, idist=None, onembed=None, ostride=1, odist=None) -> Plan:
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    tot = 1
    for d in n:
        tot *= d
    idist = tot if idist is None else idist
    odist = tot if odist is None else odist
    p = getattr(lib, pfx + "plan_many_dft")(len(n), _iarr(n), howmany, inp, _iarr(inembed), istride, idist,
                                          out, _iarr(onembed), ostride, odist, sign, flags)
    return Plan(p, prec)


def plan_many_dft_r2c(n, howmany, inp, out, flags=FFTW_ESTIMATE, prec="f", inembed=None, istride=1,
                      idist=None, onembed=None, ostride=1, odist=None) -> Plan:
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    tot = 1
    for d in n[:-1]:
        tot *= d
    idist = tot * n[-1] if idist is None else idist
    odist = tot * (n[-1] // 2 + 1) if odist is None else odist
    p = getattr(lib, pfx + "plan_many_dft_r2c")(len(n), _iarr(n), howmany, inp, _iarr(inembed), istride, idist,
                                              out, _iarr(onembed), ostride, odist, flags)
    return Plan(p, prec)


def plan_many_dft_c2r(n, howmany, inp, out, flags=FFTW_ESTIMATE, prec="f", inembed=None, istride=1,
                      idist=None, onembed=None, ostride=1, odist=None) -> Plan:
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    tot = 1
    for d in n[:-1]:
        tot *= d
    idist = tot * (n[-1] // 2 + 1) if idist is None else idist
    odist = tot * n[-1] if odist is None else odist
    p = getattr(lib, pfx + "plan_many_dft_c2r")(len(n), _iarr(n), howmany, inp, _iarr(inembed), istride, idist,
                                              out, _iarr(onembed), ostride, odist, flags)
    return Plan(p, prec)


def plan_guru_dft(dims, howmany_dims, inp, out, sign=FFTW_FORWARD, flags=FFTW_ESTIMATE, prec="f") -> Plan:
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    d = (IODim * max(1, len(dims)))(*[IODim(*x) for x in dims])
    h = (IODim * max(1, len(howmany_dims)))(*[IODim(*x) for x in howmany_dims])
    p = getattr(lib, pfx + "plan_guru_dft")(len(dims), d, len(howmany_dims), h, inp, out, sign, flags)
    return Plan(p, prec)


def plan_guru_split_dft(dims, howmany_dims, ri, ii, ro, io, flags=FFTW_ESTIMATE, prec="f") -> Plan:
    """Forward DFT of ri + i*ii into ro + i*io; (n, is, os) strides in reals."""
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    d = (IODim * max(1, len(dims)))(*[IODim(*x) for x in dims])
    h = (IODim * max(1, len(howmany_dims)))(*[IODim(*x) for x in howmany_dims])
    p = getattr(lib, pfx + "plan_guru_split_dft")(len(dims), d, len(howmany_dims), h, ri, ii, ro, io, flags)
    return Plan(p, prec)


def plan_many_r2r(n, howmany, inp, out, kinds, flags=FFTW_ESTIMATE, prec="f", inembed=None, istride=1,
                  idist=None, onembed=None, ostride=1, odist=None) -> Plan:
    """r2r of rank len(n), one fftw_r2r_kind value per dim; strides in reals."""
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    tot = 1
    for d in n:
        tot *= d
    k = (ctypes.c_int * len(kinds))(*kinds)
    p = getattr(lib, pfx + "plan_many_r2r")(len(n), _iarr(n), howmany, inp, _iarr(inembed), istride,
                                            tot if idist is None else idist, out, _iarr(onembed), ostride,
                                            tot if odist is None else odist, k, flags)
    return Plan(p, prec)


def plan_guru_split_dft_r2c(dims, howmany_dims, inp, ro, io, flags=FFTW_ESTIMATE, prec="f") -> Plan:
    """r2c of the real array inp into ro + i*io (last dim n/2+1); (n, is, os) strides in reals."""
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    d = (IODim * max(1, len(dims)))(*[IODim(*x) for x in dims])
    h = (IODim * max(1, len(howmany_dims)))(*[IODim(*x) for x in howmany_dims])
    p = getattr(lib, pfx + "plan_guru_split_dft_r2c")(len(dims), d, len(howmany_dims), h, inp, ro, io, flags)
    return Plan(p, prec)


def plan_guru_split_dft_c2r(dims, howmany_dims, ri, ii, out, flags=FFTW_ESTIMATE, prec="f") -> Plan:
    """c2r of ri + i*ii (last dim n/2+1) into the real array out; (n, is, os) strides in reals."""
    lib = load()
    pfx = "fftwf_" if prec == "f" else "fftw_"
    d = (IODim * max(1, len(dims)))(*[IODim(*x) for x in dims])
    h = (IODim * max(1, len(howmany_dims)))(*[IODim(*x) for x in howmany_dims])
    p = getattr(lib, pfx + "plan_guru_split_dft_c2r")(len(dims), d, len(howmany_dims), h, ri, ii, out, flags)
    return Plan(p, prec)


def set_dry_run(on: bool):
    load().fftw_gb300_set_dry_run(int(on))


def launch_count() -> int:
    return int(load().fftw_gb300_launch_count())
