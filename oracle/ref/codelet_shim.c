/* The reference checkout carries no generated codelets (they are produced by
 * its OCaml generator, which is not available here).  dft/conf.c and
 * rdft/conf.c register the codelet tables by name; this file supplies those
 * four tables empty, so the reference planner falls back to its hand-written
 * generic solvers (ct + dft-generic/dftw-generic, rader, bluestein).  Test-only. */
#include "kernel/ifftw.h"
const solvtab X(solvtab_dft_standard) = { SOLVTAB_END };
const solvtab X(solvtab_rdft_r2cf) = { SOLVTAB_END };
const solvtab X(solvtab_rdft_r2cb) = { SOLVTAB_END };
const solvtab X(solvtab_rdft_r2r) = { SOLVTAB_END };
