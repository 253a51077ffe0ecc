"""The reference's own benchmark / self-test harness (tests/bench.c,
tests/fftw-bench.c and libbench2, compiled where the reference sources are)
built unchanged against include/fftw3.h and linked with libfftw3_gb300.so:
it compiles, links, and every problem of its own problem syntax that the
reference can plan — c2c, r2c/c2r, r2r of every kind, split arrays
(`//`), vector loops (`*`), strides (`:`), in place and out, forward and
backward, destroy-input — plans through this library (dry run, no GPU).
Skipped where the reference sources are absent."""
import subprocess

import pytest

from oracle.oracle import harness

PLANNED = [
    "cof1", "cof2", "cof17", "cof4099", "cof100003", "cif1000x1000", "cob2x3x5x7", "cof16x16x16x16",
    "cof64*3", "cof64:2:3*4", "cif64*8:64:64", "cof4096*65536", "co1*1", "tcof8x8", "dcob16x16",
    "rof2", "rof17", "rof1024", "rof4097", "rob4097", "rib4097", "rof16*3", "rib9x10", "rob3x5x7",
    "rib64x64", "rob64x64", "rif64x64", "rib8x6x10", "rof1x1",
    "ki1e01", "ko5o00", "ki100e11x3o10", "ko64fx64b", "ko10e10x16o11", "ko16hx16hx16h", "ki32h", "ko7o00",
    "//cif64", "//cof100", "//rof64", "//rob64",
]
NOT_PLANNED = ["ko1e00"]     # a size-1 REDFT00 is not defined (the reference returns NULL too)


@pytest.fixture(scope="module")
def bench_exe(lib):
    exe = harness()
    if exe is None:
        pytest.skip("the reference sources are not on this machine")
    return exe


def can_do(exe, problem):
    r = subprocess.run([exe, "--can-do", problem], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip().splitlines()[-1]


@pytest.mark.parametrize("problem", PLANNED)
def test_harness_plans(bench_exe, problem):
    assert can_do(bench_exe, problem) == "#t"


@pytest.mark.parametrize("problem", NOT_PLANNED)
def test_harness_rejects_what_the_reference_rejects(bench_exe, problem):
    assert can_do(bench_exe, problem) == "#f"
