import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    """The product library, built in-tree if needed."""
    from fftw3_gb300 import build, load
    build.build()
    return load()


@pytest.fixture(scope="session")
def restatement():
    from oracle.oracle import Restatement, build
    build()
    return Restatement()


GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def golden_cases():
    import json
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    out = []
    for m in meta:
        k = m["key"]
        yl = z[k + "_yl_hi"].astype(np.clongdouble if np.iscomplexobj(z[k + "_yl_hi"]) else np.longdouble)
        yl = yl + z[k + "_yl_lo"].astype(yl.dtype)
        out.append(dict(m, x=z[k + "_x"], yd=z[k + "_yd"], yl=yl))
    return out


def rel_l2_f(y, ref):
    """rel_l2 in double precision: for float results, whose errors (~1e-7)
    double arithmetic resolves exactly enough, on arrays too large for the
    long-double sum (software quad precision on some hosts)."""
    y = np.asarray(y).ravel().astype(np.complex128)
    ref = np.asarray(ref).ravel().astype(np.complex128)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(y - ref) / den) if den > 0 else float(np.linalg.norm(y))


def rel_l2(y, ref):
    y = np.asarray(y).ravel()
    ref = np.asarray(ref).ravel()
    dt = np.clongdouble if (np.iscomplexobj(y) or np.iscomplexobj(ref)) else np.longdouble
    y = y.astype(dt)
    ref = ref.astype(dt)
    den = np.sqrt(np.sum(np.abs(ref) ** 2))
    num = np.sqrt(np.sum(np.abs(y - ref) ** 2))
    return float(num / den) if den > 0 else float(num)
