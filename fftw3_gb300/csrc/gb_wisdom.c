/*
 * Wisdom: the tuner's choices, exported and imported with the reference's
 * wisdom calls (api/export-wisdom*.c, api/import-wisdom*.c,
 * api/forget-wisdom.c).  The text keeps the reference's s-expression shape
 * (kernel/planner.c:790-826):
 *
 *   (fftw-3.3.10-gb300 fftwf_wisdom #x<signature>
 *     (gb300-pass "c2c p4 n4096" #x<variant> #x<tb> #x<load> #x<store> #x<n1> #x<groups> #x<order>)
 *   )
 *
 * (an entry with only the first five numbers, as earlier versions wrote
 * them, reads with groups and order 0: the planner's choices)
 *
 * The preamble and signature differ from the reference's, so a file written
 * by one library is rejected by the other (the reference rejects a
 * mismatched registry signature the same way, kernel/planner.c:847-852).
 * Import returns 0 and leaves the current wisdom untouched on any error
 * (kernel/planner.c:901-905).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gb_host.h"

#define GB_WISDOM_SIG 0x67623330304c4942ULL   /* registry signature of this library */

typedef struct node { gb_wisdom_entry e; int prec; struct node *next; } node;
static node *wis = 0;

static int prec_of_key(const char *key)
{
     const char *p = strstr(key, " p");
     return p ? atoi(p + 2) : 0;
}

const gb_wisdom_entry *gb_wisdom_lookup(const char *key)
{
     node *n;
     for (n = wis; n; n = n->next)
          if (!strcmp(n->e.key, key)) return &n->e;
     return 0;
}

void gb_wisdom_store(const gb_wisdom_entry *e)
{
     node *n;
     for (n = wis; n; n = n->next)
          if (!strcmp(n->e.key, e->key)) { n->e = *e; return; }
     n = (node *)malloc(sizeof *n);
     n->e = *e;
     n->prec = prec_of_key(e->key);
     n->next = wis;
     wis = n;
}

void gb_wisdom_forget(void)
{
     while (wis) {
          node *n = wis;
          wis = n->next;
          free(n);
     }
}

static void emits(void (*emit)(char, void *), void *d, const char *s)
{
     while (*s) emit(*s++, d);
}

int gb_wisdom_export(int prec, void (*emit)(char c, void *), void *data)
{
     char buf[512];
     node *n;
     snprintf(buf, sizeof buf, "(fftw-3.3.10-gb300 %s_wisdom #x%llx\n", prec == 4 ? "fftwf" : "fftw",
              (unsigned long long)GB_WISDOM_SIG);
     emits(emit, data, buf);
     for (n = wis; n; n = n->next) {
          if (n->prec != prec) continue;
          snprintf(buf, sizeof buf, "  (gb300-pass \"%s\" #x%x #x%x #x%x #x%x #x%x #x%x #x%x)\n", n->e.key,
                   n->e.variant, n->e.tb, n->e.load_mode, n->e.store_mode, n->e.n1, n->e.groups, n->e.order);
          emits(emit, data, buf);
     }
     emits(emit, data, ")\n");
     return 0;
}

/* ---- a small reader over the caller's getc ---- */
typedef struct { int (*g)(void *); void *d; int c; } rd;
static void adv(rd *r) { r->c = r->g(r->d); }
static void skipws(rd *r) { while (r->c == ' ' || r->c == '\n' || r->c == '\t' || r->c == '\r') adv(r); }
static int expect(rd *r, const char *s)
{
     skipws(r);
     while (*s) { if (r->c != *s) return 0; adv(r); ++s; }
     return 1;
}
static int read_hex(rd *r, unsigned long long *v)
{
     int any = 0;
     skipws(r);
     if (r->c != '#') return 0;
     adv(r);
     if (r->c != 'x') return 0;
     adv(r);
     *v = 0;
     for (;;) {
          int c = r->c, d;
          if (c >= '0' && c <= '9') d = c - '0';
          else if (c >= 'a' && c <= 'f') d = c - 'a' + 10;
          else if (c >= 'A' && c <= 'F') d = c - 'A' + 10;
          else break;
          *v = *v * 16 + (unsigned)d;
          any = 1;
          adv(r);
     }
     return any;
}
static int read_str(rd *r, char *out, int cap)
{
     int k = 0;
     skipws(r);
     if (r->c != '"') return 0;
     adv(r);
     while (r->c != '"' && r->c != EOF) {
          if (k + 1 >= cap) return 0;
          out[k++] = (char)r->c;
          adv(r);
     }
     if (r->c != '"') return 0;
     adv(r);
     out[k] = 0;
     return 1;
}

int gb_wisdom_import(int prec, int (*getc_fn)(void *), void *data)
{
     rd r;
     unsigned long long sig, v[7];
     gb_wisdom_entry got[1024];
     int ngot = 0, i;
     r.g = getc_fn; r.d = data;
     adv(&r);
     if (!expect(&r, "(fftw-3.3.10-gb300")) return 0;
     if (!expect(&r, prec == 4 ? "fftwf_wisdom" : "fftw_wisdom")) return 0;
     if (!read_hex(&r, &sig) || sig != GB_WISDOM_SIG) return 0;
     for (;;) {
          skipws(&r);
          if (r.c == ')') break;
          if (!expect(&r, "(gb300-pass")) return 0;
          if (ngot >= 1024) return 0;
          memset(&got[ngot], 0, sizeof got[ngot]);
          if (!read_str(&r, got[ngot].key, sizeof got[ngot].key)) return 0;
          for (i = 0; i < 5; ++i)
               if (!read_hex(&r, &v[i])) return 0;
          v[5] = v[6] = 0;
          skipws(&r);
          if (r.c == '#' && (!read_hex(&r, &v[5]) || !read_hex(&r, &v[6]))) return 0;
          if (!expect(&r, ")")) return 0;
          if (prec_of_key(got[ngot].key) != prec) return 0;
          got[ngot].variant = (int)v[0]; got[ngot].tb = (int)v[1];
          got[ngot].load_mode = (int)v[2]; got[ngot].store_mode = (int)v[3]; got[ngot].n1 = (int)v[4];
          got[ngot].groups = (int)v[5]; got[ngot].order = (int)v[6];
          if (got[ngot].tb < 0 || got[ngot].tb > 1024 || got[ngot].n1 < 0 || v[5] > 2 || v[6] >= GB_RADIX_ORDERS)
               return 0;
          ++ngot;
     }
     for (i = 0; i < ngot; ++i) gb_wisdom_store(&got[i]);
     return 1;
}
