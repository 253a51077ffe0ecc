"""The drop-in boundary from C and C++: a program written against the
reference's API compiles with include/fftw3.h under strict warnings (as C99
and as C++), links against libfftw3_gb300.so, and plans every planner
family through it (dry-run plans: no GPU is needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fftw3_gb300")

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <fftw3.h>
#include <fftw3_gb300.h>

static int check(const char *what, void *p)
{
    if (!p) { printf("NULL %s: %s\n", what, fftw_gb300_last_error()); return 1; }
    return 0;
}

int main(void)
{
    int bad = 0, n[3] = {8, 12, 16};
    fftwf_complex *c = (fftwf_complex *)(size_t)(1 << 20), *d = (fftwf_complex *)(size_t)(1 << 30);
    float *r = (float *)(size_t)(1 << 20), *s = (float *)(size_t)(1 << 30);
    double *rd = (double *)(size_t)(1 << 20), *sd = (double *)(size_t)(1 << 30);
    fftwf_r2r_kind k3[3] = {FFTW_REDFT10, FFTW_RODFT11, FFTW_DHT};
    fftw_r2r_kind k1 = FFTW_REDFT00;
    fftwf_iodim dims[1] = {{64, 1, 1}}, hdims[1] = {{4, 64, 64}};
    fftwf_plan p;
    char *txt;
    fftw_gb300_set_dry_run(1);
    p = fftwf_plan_many_dft(1, n, 10, c, NULL, 1, 8, d, NULL, 1, 8, FFTW_FORWARD, FFTW_ESTIMATE);
    bad += check("plan_many_dft", p);
    txt = fftwf_sprint_plan(p);
    if (!txt || strncmp(txt, "(gb300-dft-f32", 14)) { printf("sprint_plan: %s\n", txt ? txt : "NULL"); ++bad; }
    free(txt);
    fftwf_destroy_plan(p);
    p = fftwf_plan_dft_3d(8, 12, 16, c, c, FFTW_BACKWARD, FFTW_ESTIMATE);
    bad += check("plan_dft_3d", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_dft_r2c_2d(8, 16, r, d, FFTW_ESTIMATE);
    bad += check("plan_dft_r2c_2d", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_many_dft_c2r(1, n + 2, 3, c, NULL, 1, 9, s, NULL, 1, 16, FFTW_ESTIMATE);
    bad += check("plan_many_dft_c2r", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_guru_dft(1, dims, 1, hdims, c, d, FFTW_FORWARD, FFTW_ESTIMATE);
    bad += check("plan_guru_dft", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_guru_split_dft(1, dims, 1, hdims, r, r + 4096, s, s + 4096, FFTW_ESTIMATE);
    bad += check("plan_guru_split_dft", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_guru_split_dft_r2c(1, dims, 1, hdims, r, s, s + 4096, FFTW_ESTIMATE);
    bad += check("plan_guru_split_dft_r2c", p);
    fftwf_destroy_plan(p);
    p = fftwf_plan_r2r(3, n, r, s, k3, FFTW_ESTIMATE);
    bad += check("plan_r2r", p);
    fftwf_destroy_plan(p);
    {
        fftw_plan q = fftw_plan_r2r_1d(33, rd, sd, k1, FFTW_ESTIMATE);
        bad += check("fftw_plan_r2r_1d", q);
        fftw_destroy_plan(q);
        q = fftw_plan_r2r_1d(1, rd, sd, k1, FFTW_ESTIMATE);      /* size-1 REDFT00: not defined */
        if (q) { printf("size-1 REDFT00 planned\n"); ++bad; fftw_destroy_plan(q); }
    }
    {
        char *w = fftwf_export_wisdom_to_string();
        if (!w || fftwf_import_wisdom_from_string(w) != 1) { printf("wisdom round trip\n"); ++bad; }
        free(w);
    }
    printf("%s %d\n", bad ? "FAILED" : "OK", bad);
    return bad != 0;
}
"""


@pytest.mark.parametrize("compiler,flags", [("gcc", ["-std=c99", "-x", "c"]), ("g++", ["-std=c++17", "-x", "c++"])])
def test_reference_style_program_builds_and_plans(lib, tmp_path, compiler, flags):
    if not shutil.which(compiler):
        pytest.skip(f"{compiler} not found")
    src = tmp_path / "app.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "app"
    cmd = [compiler, *flags, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           str(src), "-x", "none", "-L", PKG, "-lfftw3_gb300", "-Wl,-rpath," + PKG, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK 0"), r.stdout + r.stderr
