/*
 * fftw-wisdom-gb300 / fftwf-wisdom-gb300: create wisdom for a list of
 * transform sizes ahead of time, the counterpart of the reference's
 * fftw-wisdom tool (tools/fftw-wisdom.c:100-131 usage, 134-148 canonical
 * sizes, 280-330 main loop).  Each size is planned with the tuner
 * (PATIENT unless told otherwise), which times the candidate kernels on
 * scratch device arrays and records the winners; the accumulated wisdom is
 * written to stdout or to -o FILE in this library's wisdom format, ready for
 * fftw_import_wisdom_from_filename or the system wisdom file.
 *
 * Size syntax (as the reference's): <type><inplace><direction><geometry>,
 * type c (complex), r (r2c forward / c2r backward) or k (r2r, no
 * direction), inplace i or o, direction f or b, geometry n1[xn2[x...]];
 * for k each dim is followed by its kind, f/b/h/e00/e01/e10/e11/o00/o01/
 * o10/o11 for R2HC/HC2R/DHT/REDFT00/.../RODFT11 (R2HC when omitted).
 *
 * Built twice by fftw3_gb300/build.py: with GB_TOOL_SINGLE for the fftwf_
 * API, without for fftw_.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "fftw3.h"
#include "fftw3_gb300.h"

#ifdef GB_TOOL_SINGLE
#define FX(name) fftwf_##name
#define TOOL_NAME "fftwf-wisdom-gb300"
typedef float real_t;
typedef fftwf_plan plan_t;
typedef fftwf_complex cpx_t;
#else
#define FX(name) fftw_##name
#define TOOL_NAME "fftw-wisdom-gb300"
typedef double real_t;
typedef fftw_plan plan_t;
typedef fftw_complex cpx_t;
#endif

/* powers of two to 2^20, powers of ten to 10^6, square 2D and cubic 3D */
static const char *const canonical[] = {
     "1", "2", "4", "8", "16", "32", "64", "128", "256", "512", "1024", "2048", "4096", "8192", "16384",
     "32768", "65536", "131072", "262144", "524288", "1048576", "10", "100", "1000", "10000", "100000",
     "1000000", "2x2", "4x4", "8x8", "10x10", "16x16", "32x32", "64x64", "100x100", "128x128", "256x256",
     "512x512", "1000x1000", "1024x1024", "2x2x2", "4x4x4", "8x8x8", "10x10x10", "16x16x16", "32x32x32",
     "64x64x64", "100x100x100"};

static void usage(FILE *f)
{
     fprintf(f,
             "Usage: " TOOL_NAME " [options] [sizes]\n"
             "  Create wisdom (tuned kernel choices) for the given sizes and write it to\n"
             "  stdout, or to a file with -o.\n\n"
             "Options:\n"
             "  -h, --help                 this help\n"
             "  -V, --version              library version\n"
             "  -v, --verbose              print each size as it is planned\n"
             "  -c, --canonical            add the canonical set of sizes\n"
             "  -t H, --time-limit=H       stop planning after H hours (default: no limit)\n"
             "  -o FILE, --output-file=FILE  write wisdom to FILE\n"
             "  -i, --impatient, -m, --measure  plan in MEASURE mode (PATIENT is the default)\n"
             "  -e, --estimate             plan in ESTIMATE mode (no tuning)\n"
             "  -x, --exhaustive           plan in EXHAUSTIVE mode\n"
             "  -n, --no-system-wisdom     do not read the system wisdom file\n"
             "  -w FILE, --wisdom-file=FILE  read wisdom from FILE first (- for stdin)\n"
             "  -T N, --threads=N          accepted; the GPU replaces the thread pool\n\n"
             "Size syntax: <type><inplace><direction><geometry>\n"
             "  <type> = c, r or k (complex, real r2c/c2r, or r2r); <inplace> = i or o;\n"
             "  <direction> = f or b (omitted for k); <geometry> = n1[xn2[x...]],\n"
             "  e.g. cof4096, rib512x512; for k each dim is followed by its kind,\n"
             "  f/b/h/e00/e01/e10/e11/o00/o01/o10/o11 (R2HC/HC2R/DHT/REDFT00/.../RODFT11),\n"
             "  e.g. koe10x16o11\n"
             "  Sizes may also be read from stdin by giving - as a size.\n");
}

typedef struct {
     char type, place, dir;
     int rank;
     int n[8];
     int kind[8];           /* r2r kinds (fftw_r2r_kind values) */
} problem;

/* an r2r kind after a dim of a k size: f, b, h, e<ab>, o<ab> */
static int parse_kind(const char **q, int *kind)
{
     const char c = **q;
     char *end;
     long ab;
     *kind = FFTW_R2HC;
     if (c == 'f' || c == 'b' || c == 'h') {
          *kind = c == 'f' ? FFTW_R2HC : c == 'b' ? FFTW_HC2R : FFTW_DHT;
          ++*q;
          return 0;
     }
     if (c != 'e' && c != 'o') return 0;
     ab = strtol(*q + 1, &end, 10);
     if (end == *q + 1) return -1;
     *q = end;
     if (ab == 0) *kind = c == 'e' ? FFTW_REDFT00 : FFTW_RODFT00;
     else if (ab == 1) *kind = c == 'e' ? FFTW_REDFT01 : FFTW_RODFT01;
     else if (ab == 10) *kind = c == 'e' ? FFTW_REDFT10 : FFTW_RODFT10;
     else if (ab == 11) *kind = c == 'e' ? FFTW_REDFT11 : FFTW_RODFT11;
     else return -1;
     return 0;
}

static int parse(const char *s, problem *p)
{
     const char *q = s;
     char *end;
     memset(p, 0, sizeof *p);
     if (strlen(s) < 4) return -1;
     p->type = *q++;
     p->place = *q++;
     p->dir = p->type == 'k' ? 'f' : *q++;
     if ((p->type != 'c' && p->type != 'r' && p->type != 'k') || (p->place != 'i' && p->place != 'o') ||
         (p->dir != 'f' && p->dir != 'b'))
          return -1;
     for (;;) {
          long v = strtol(q, &end, 10);
          if (end == q || v <= 0 || v > (1L << 30) || p->rank >= 8) return -1;
          p->n[p->rank] = (int)v;
          if (p->type == 'k') {
               const char *e = end;
               if (parse_kind(&e, &p->kind[p->rank])) return -1;
               end = (char *)e;
          }
          p->rank++;
          if (*end == 'x') { q = end + 1; continue; }
          if (*end) return -1;
          break;
     }
     return 0;
}

/* Plan (and so tune) one problem on host arrays of its size; the tuner
 * works on its own device scratch arrays, so these are never written. */
static int plan_one(const problem *p, unsigned flags, int verbose, const char *spec)
{
     size_t tot = 1, last;
     int i;
     plan_t pl;
     void *in, *out;
     for (i = 0; i < p->rank; ++i) tot *= (size_t)p->n[i];
     last = (size_t)p->n[p->rank - 1];
     if (verbose) fprintf(stderr, "Planning transform: %s\n", spec);
     if (p->type == 'k') {
          FX(r2r_kind) k[8];
          for (i = 0; i < p->rank; ++i) k[i] = (FX(r2r_kind))p->kind[i];
          in = FX(malloc)(tot * sizeof(real_t));
          out = p->place == 'i' ? in : FX(malloc)(tot * sizeof(real_t));
          if (!in || !out) return -1;
          pl = FX(plan_r2r)(p->rank, p->n, (real_t *)in, (real_t *)out, k, flags);
     } else if (p->type == 'c') {
          in = FX(malloc)(tot * sizeof(cpx_t));
          out = p->place == 'i' ? in : FX(malloc)(tot * sizeof(cpx_t));
          if (!in || !out) return -1;
          pl = FX(plan_dft)(p->rank, p->n, (cpx_t *)in, (cpx_t *)out, p->dir == 'f' ? FFTW_FORWARD : FFTW_BACKWARD,
                            flags);
     } else {
          size_t nc = tot / last * (last / 2 + 1);
          in = FX(malloc)(2 * nc * sizeof(real_t));
          out = p->place == 'i' ? in : FX(malloc)(nc * sizeof(cpx_t));
          if (!in || !out) return -1;
          if (p->dir == 'f') pl = FX(plan_dft_r2c)(p->rank, p->n, (real_t *)in, (cpx_t *)out, flags);
          else pl = FX(plan_dft_c2r)(p->rank, p->n, (cpx_t *)out, (real_t *)in, flags);
     }
     if (!pl) fprintf(stderr, TOOL_NAME ": cannot plan %s: %s\n", spec, fftw_gb300_last_error());
     else FX(destroy_plan)(pl);
     FX(free)(in);
     if (out != in) FX(free)(out);
     return pl ? 0 : -1;
}

static int add(char ***list, int *n, int *cap, const char *s)
{
     if (*n == *cap) {
          int c = *cap ? 2 * *cap : 64;
          char **l = (char **)realloc(*list, (size_t)c * sizeof *l);
          if (!l) return -1;
          *list = l;
          *cap = c;
     }
     (*list)[(*n)++] = strdup(s);
     return 0;
}

int main(int argc, char **argv)
{
     unsigned flags = FFTW_PATIENT;
     int verbose = 0, canon = 0, system_wisdom = 1, i, j, nprob = 0, cap = 0, failed = 0;
     double hours = 0;
     const char *outname = 0;
     char **probs = 0;
     FILE *out;
     time_t t0 = time(0);

     for (i = 1; i < argc; ++i) {
          const char *a = argv[i];
          const char *val = 0;
#define OPT(s, l) (!strcmp(a, s) || !strcmp(a, l))
#define ARG(s, l)                                                                  \
     ((!strcmp(a, s) && i + 1 < argc && (val = argv[++i])) ||                     \
      (!strncmp(a, l "=", strlen(l) + 1) && (val = a + strlen(l) + 1)))
          if (OPT("-h", "--help")) { usage(stdout); return 0; }
          else if (OPT("-V", "--version")) { printf("%s\n", FX(version)); return 0; }
          else if (OPT("-v", "--verbose")) verbose = 1;
          else if (OPT("-c", "--canonical")) canon = 1;
          else if (OPT("-i", "--impatient") || OPT("-m", "--measure")) flags = FFTW_MEASURE;
          else if (OPT("-e", "--estimate")) flags = FFTW_ESTIMATE;
          else if (OPT("-x", "--exhaustive")) flags = FFTW_EXHAUSTIVE;
          else if (OPT("-n", "--no-system-wisdom")) system_wisdom = 0;
          else if (ARG("-t", "--time-limit")) hours = atof(val);
          else if (ARG("-o", "--output-file")) outname = val;
          else if (ARG("-T", "--threads")) FX(plan_with_nthreads)(atoi(val));
          else if (ARG("-w", "--wisdom-file")) {
               int ok = !strcmp(val, "-") ? FX(import_wisdom_from_file)(stdin) : FX(import_wisdom_from_filename)(val);
               if (!ok) { fprintf(stderr, TOOL_NAME ": cannot read wisdom from %s\n", val); return 1; }
          } else if (!strcmp(a, "-")) {
               char s[1025];
               while (fscanf(stdin, "%1024s", s) == 1)
                    if (add(&probs, &nprob, &cap, s)) return 1;
          } else if (a[0] == '-') {
               fprintf(stderr, TOOL_NAME ": unknown option %s\n", a);
               usage(stderr);
               return 1;
          } else if (add(&probs, &nprob, &cap, a)) return 1;
#undef OPT
#undef ARG
     }
     if (system_wisdom && !FX(import_system_wisdom)() && verbose)
          fprintf(stderr, TOOL_NAME ": system-wisdom import failed\n");
     if (canon) {
          static const char *const types[] = {"cof", "cob", "cif", "cib", "rof", "rob", "rif", "rib"};
          char ps[64];
          for (i = 0; i < (int)(sizeof canonical / sizeof canonical[0]); ++i)
               for (j = 0; j < 8; ++j) {
                    if (strchr(canonical[i], 'x') && !strchr(types[j], 'o')) continue;
                    snprintf(ps, sizeof ps, "%s%s", types[j], canonical[i]);
                    if (add(&probs, &nprob, &cap, ps)) return 1;
               }
     }
     for (i = 0; i < nprob; ++i) {
          problem p;
          if (hours > 0 && difftime(time(0), t0) > hours * 3600.0) {
               if (verbose) fprintf(stderr, TOOL_NAME ": time limit reached, %d sizes left\n", nprob - i);
               break;
          }
          if (parse(probs[i], &p)) {
               fprintf(stderr, TOOL_NAME ": cannot parse size %s\n", probs[i]);
               failed = 1;
               continue;
          }
          if (plan_one(&p, flags, verbose, probs[i])) failed = 1;
     }
     out = outname ? fopen(outname, "w") : stdout;
     if (!out) { fprintf(stderr, TOOL_NAME ": cannot open %s\n", outname); return 1; }
     FX(export_wisdom_to_file)(out);
     if (outname) fclose(out);
     for (i = 0; i < nprob; ++i) free(probs[i]);
     free(probs);
     return failed;
}
