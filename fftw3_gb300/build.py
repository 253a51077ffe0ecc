"""Build libfftw3_gb300.so in-tree.

    python -m fftw3_gb300.build            # or fftw3_gb300.build.build()

CUDA sources are compiled for sm_103a only (-gencode arch=compute_103a,
code=sm_103a) with nvcc, the host C sources with gcc, in parallel, into
fftw3_gb300/_build/; the shared library lands at
fftw3_gb300/libfftw3_gb300.so with the CUDA runtime linked statically.
Objects are reused when newer than every source and header.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libfftw3_gb300.so")
# the wisdom tool (fftw-wisdom counterpart), one binary per precision
TOOLS = {os.path.join(PKG, "fftw-wisdom-gb300"): [], os.path.join(PKG, "fftwf-wisdom-gb300"): ["-DGB_TOOL_SINGLE"]}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newest_dep() -> float:
    deps = (glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(CSRC, "cli", "*")) +
            glob.glob(os.path.join(INC, "*.h")) + [__file__])
    return max(os.path.getmtime(d) for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, jobs: int | None = None) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    newest = _newest_dep()
    if all(os.path.exists(f) and os.path.getmtime(f) >= newest for f in [LIB, *TOOLS]):
        return LIB
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cc = sorted(glob.glob(os.path.join(CSRC, "*.c")))
    objs, cmds = [], []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
            continue
        cmds.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-I", CSRC, "-I", INC, "-c", src, "-o", obj])
    for src in cc:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
            continue
        cmds.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
                     "-pthread", "-I", CSRC, "-I", INC, "-I", os.path.join(cuda, "include"),
                     "-c", src, "-o", obj])
    jobs = jobs or min(len(cmds), os.cpu_count() or 4) or 1
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared", *ARCH, "-cudart=static", "-o", tmp, *objs, "-Xlinker", "-Bsymbolic-functions",
          "-lpthread", "-lm"])
    os.replace(tmp, LIB)
    tool_src = os.path.join(CSRC, "cli", "wisdom_tool.c")
    for exe, defs in TOOLS.items():
        _run(["gcc", "-std=gnu11", "-O2", "-Wall", *defs, "-I", INC, tool_src, "-o", exe, "-L", PKG,
              "-lfftw3_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
