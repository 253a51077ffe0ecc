"""The wisdom tool (counterpart of the reference's fftw-wisdom): command
line, size syntax, and — on a GPU — wisdom that the library imports."""
import os
import subprocess

import pytest

from conftest import has_gpu

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fftw3_gb300")


def tool(prec, *args, **kw):
    exe = os.path.join(PKG, ("fftwf" if prec == "f" else "fftw") + "-wisdom-gb300")
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=kw.get("timeout", 60))


@pytest.mark.parametrize("prec", ["f", "d"])
def test_help_and_version(lib, prec):
    r = tool(prec, "-h")
    assert r.returncode == 0 and "<type><inplace><direction><geometry>" in r.stdout
    r = tool(prec, "--version")
    assert r.returncode == 0 and "gb300" in r.stdout


def test_rejects_bad_sizes_and_options(lib):
    # r2r (type k) sizes take no direction and a kind after each dim
    for bad in ("kof1024", "koe12x16", "kx10e10", "ko10e12", "cof", "cxf64"):
        r = tool("f", "-e", "-n", bad)
        assert r.returncode == 1 and f"cannot parse size {bad}" in r.stderr, bad
    r = tool("f", "--bogus")
    assert r.returncode == 1 and "unknown option" in r.stderr


@pytest.mark.skipif(has_gpu(), reason="checks the message given without a GPU")
def test_without_gpu_reports_each_size(lib):
    for size in ("cof64", "ko10e10x16o11", "ki64", "ki32hx8e00"):
        r = tool("f", "-e", "-n", size)
        assert r.returncode == 1 and f"cannot plan {size}" in r.stderr, size


@pytest.mark.gpu
def test_tuned_wisdom_round_trip(lib, tmp_path):
    out = tmp_path / "w.txt"
    r = tool("f", "-m", "-n", "-o", str(out), "cof4096", "cib1024", "rof2048", "cof64x64", "ko96e10x100o11",
             timeout=600)
    assert r.returncode == 0, r.stderr
    text = out.read_text()
    assert text.startswith("(fftw-3.3.10-gb300 fftwf_wisdom") and '"c2c p4 n4096"' in text
    lib.fftwf_forget_wisdom()
    assert lib.fftwf_import_wisdom_from_filename(str(out).encode()) == 1
