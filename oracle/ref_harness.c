/* Runtime and harness of the translated reference step (test infrastructure).
 *
 * oracle/f90sub2c.py turns the reference's own Fortran step routines into C
 * (oracle/_ref/ref_step.c, a build product).  This file supplies what the
 * Fortran runtime and the reference's C helper did for them:
 *   - array descriptors (allocate/deallocate, dummy-argument views);
 *   - Fortran unformatted sequential records (4-byte length markers, the
 *     gfortran layout; optional byte swap for the big-endian SGI files the
 *     reference's test/2d case ships), read and written in a run directory;
 *   - formatted writes: the numeric items of each line, at full precision,
 *     appended to the unit's file (the history file of resstat/resstat3D);
 *   - the reference's error()/stop paths, trapped with setjmp so that a
 *     failing routine returns a status to the caller instead of exiting;
 *   - igetver/addver (src/getver.c:28-62): versioned file names base.ext.N,
 *     resolved by scanning the run directory instead of running verlist;
 *   - second() (src/second.f90), a constant so runs are reproducible.
 * Python (oracle/refstep.py) drives it through ctypes: every translated
 * procedure takes pointer arguments only, so ref_call() can call any of
 * them with an argument vector.
 */
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <unistd.h>
#ifndef REF_HDR
#define REF_HDR "_ref/ref_step.h"
#endif
#include REF_HDR

/* ---------------- descriptors ---------------- */

void fd_view(fdesc* d, void* p, unsigned long es, int rank, const long* lb, const long* ub) {
  (void)es;
  d->p = p;
  d->rank = rank;
  d->owned = 0;
  long st = 1;
  for (int k = 0; k < rank; ++k) {
    d->lb[k] = lb[k];
    d->n[k] = ub[k] == FD_ASSUMED ? (1L << 40) : (ub[k] - lb[k] + 1);
    if (d->n[k] < 0) d->n[k] = 0;
    d->st[k] = st;
    st *= d->n[k];
  }
}

void fd_alloc(fdesc* d, unsigned long es, int rank, const long* lb, const long* ub) {
  long n = 1;
  for (int k = 0; k < rank; ++k) {
    long e = ub[k] - lb[k] + 1;
    n *= e > 0 ? e : 0;
  }
  void* p = calloc((size_t)(n > 0 ? n : 1), es);
  fd_view(d, p, es, rank, lb, ub);
  d->owned = 1;
}

void fd_free(fdesc* d) {
  if (d->owned) free(d->p);
  d->p = 0;
  d->owned = 0;
}

/* ---------------- strings ---------------- */

static char str_ring[16][512];
static int str_pos;

static char* str_slot(void) {
  str_pos = (str_pos + 1) & 15;
  return str_ring[str_pos];
}

const char* fstr_cat(const char* a, const char* b) {
  char* s = str_slot();
  snprintf(s, 512, "%s%s", a, b);
  return s;
}

const char* fstr_char(int c) {
  char* s = str_slot();
  s[0] = (char)c;
  s[1] = 0;
  return s;
}

const char* fstr_trim(const char* a) {
  char* s = str_slot();
  snprintf(s, 512, "%s", a);
  size_t n = strlen(s);
  while (n > 0 && s[n - 1] == ' ') s[--n] = 0;
  return s;
}

const char* fstr_adjustl(const char* a) {
  while (*a == ' ') ++a;
  return fstr_trim(a);
}

const char* fstr_sub(const char* a, long lo, long hi) {
  char* s = str_slot();
  long n = (long)strlen(a);
  if (hi < 0 || hi > n) hi = n;
  long k = 0;
  for (long i = lo; i <= hi && k < 511; ++i) s[k++] = a[i - 1];
  s[k] = 0;
  return s;
}

int fstr_cmp(const char* a, const char* b) { return strcmp(fstr_trim(a), fstr_trim(b)); }

int fstr_index(const char* a, const char* b) {
  if (!*b) return (int)strlen(a) + 1; /* char(0): the end of the C string */
  const char* p = strstr(a, b);
  return p ? (int)(p - a) + 1 : 0;
}

void fstr_assign(char* dst, int len, const char* src) {
  int n = (int)strlen(src);
  char tmp[1024];
  snprintf(tmp, sizeof tmp, "%s", src);
  for (int i = 0; i < len; ++i) dst[i] = i < n ? tmp[i] : ' ';
  dst[len] = 0;
}

/* ---------------- error trapping ---------------- */

static jmp_buf* ref_jmp;
static char ref_msg[512];
int ref_status;

const char* ref_last_message(void) { return ref_msg; }

static void trap(int status, const char* msg) {
  ref_status = status;
  snprintf(ref_msg, sizeof ref_msg, "%s", msg);
  if (ref_jmp) longjmp(*ref_jmp, status);
  fprintf(stderr, "reference stopped outside ref_call: %s\n", msg);
  abort();
}

void f_error(char* code, char* msg) { trap(1, fstr_cat(fstr_trim(code), fstr_cat(": ", fstr_trim(msg)))); }
void f_stop_(void) { trap(2, "stop"); }
void f_ioerror_(void) { trap(3, "I/O error"); }
void f_unsupported_(const char* what) { trap(4, what); }

typedef void (*fn0)(void);
typedef void (*fnv)(void*, ...);

/* Call a translated procedure with n pointer arguments; 0, or the trap status. */
int ref_call(void* fn, int n, void** a) {
  jmp_buf jb;
  jmp_buf* saved = ref_jmp;
  ref_jmp = &jb;
  ref_status = 0;
  ref_msg[0] = 0;
  if (setjmp(jb) == 0) {
    fnv f = (fnv)fn;
    switch (n) {
      case 0: ((fn0)fn)(); break;
      case 1: f(a[0]); break;
      case 2: f(a[0], a[1]); break;
      case 3: f(a[0], a[1], a[2]); break;
      case 4: f(a[0], a[1], a[2], a[3]); break;
      case 5: f(a[0], a[1], a[2], a[3], a[4]); break;
      case 6: f(a[0], a[1], a[2], a[3], a[4], a[5]); break;
      case 7: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6]); break;
      case 8: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]); break;
      case 9: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]); break;
      case 10: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9]); break;
      case 11: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10]); break;
      case 12: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11]); break;
      case 13: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12]); break;
      case 14: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13]); break;
      case 15: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14]); break;
      case 16: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15]); break;
      case 17: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15], a[16]); break;
      case 18: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15], a[16], a[17]); break;
      case 19: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15], a[16], a[17], a[18]); break;
      case 20: f(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15], a[16], a[17], a[18], a[19]); break;
      default: ref_status = 5; snprintf(ref_msg, sizeof ref_msg, "too many arguments"); break;
    }
  }
  ref_jmp = saved;
  return ref_status;
}

/* ---------------- files ---------------- */

static char run_dir[1024] = ".";
static int swap_bytes;

void ref_set_dir(const char* d) { snprintf(run_dir, sizeof run_dir, "%s", d); }
void ref_set_swap(int s) { swap_bytes = s; }

typedef struct {
  FILE* f;
  int formatted;
  unsigned char* buf; /* current record */
  size_t len, pos, cap;
  int bad;
  int trunc; /* opened on an existing file: the first write ends the file there */
} unit_t;
static unit_t units[128];

static void path_of(char* out, size_t n, const char* file) {
  const char* t = fstr_trim(file);
  while (*t == ' ') ++t;
  if (t[0] == '/') snprintf(out, n, "%s", t);
  else snprintf(out, n, "%s/%s", run_dir, t);
}

int fio_open(int unit, const char* file, const char* form, const char* status) {
  if (unit < 0 || unit >= 128) return 1;
  if (units[unit].f) fclose(units[unit].f);
  char path[2048];
  path_of(path, sizeof path, file);
  const char* fm = fstr_trim(form);
  int formatted = !(fm[0] == 'u' || fm[0] == 'U');
  const char* stt = fstr_trim(status);
  FILE* f;
  int trunc = 0;
  if (stt[0] == 'o' || stt[0] == 'O') {
    f = fopen(path, formatted ? "r" : "rb");
  } else if (stt[0] == 'n' || stt[0] == 'N' || stt[0] == 'r' || stt[0] == 'R' || stt[0] == 's' || stt[0] == 'S') {
    f = fopen(path, formatted ? "w+" : "w+b");
  } else {
    /* unknown: an existing file is opened at its start for reading, and a
     * sequential write there ends the file after the record written */
    f = fopen(path, formatted ? "r+" : "r+b");
    if (f) trunc = 1;
    else f = fopen(path, formatted ? "w+" : "w+b");
  }
  if (!f) return 1;
  units[unit].f = f;
  units[unit].formatted = formatted;
  units[unit].trunc = trunc;
  return 0;
}

void fio_close(int unit) {
  if (unit >= 0 && unit < 128 && units[unit].f) {
    fclose(units[unit].f);
    units[unit].f = 0;
  }
}

static uint32_t rd_marker(FILE* f, int* ok) {
  unsigned char b[4];
  if (fread(b, 1, 4, f) != 4) {
    *ok = 0;
    return 0;
  }
  if (swap_bytes) return (uint32_t)b[3] | (uint32_t)b[2] << 8 | (uint32_t)b[1] << 16 | (uint32_t)b[0] << 24;
  return (uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24;
}

static void wr_marker(FILE* f, uint32_t v) {
  unsigned char b[4];
  for (int i = 0; i < 4; ++i) b[swap_bytes ? 3 - i : i] = (unsigned char)(v >> (8 * i));
  fwrite(b, 1, 4, f);
}

static unit_t* cur;

void fio_rbegin(int unit) {
  cur = (unit >= 0 && unit < 128) ? &units[unit] : 0;
  if (!cur || !cur->f) {
    if (cur) cur->bad = 1;
    return;
  }
  int ok = 1;
  uint32_t n = rd_marker(cur->f, &ok);
  cur->bad = !ok;
  if (!ok) return;
  if (cur->cap < n) {
    cur->buf = realloc(cur->buf, n);
    cur->cap = n;
  }
  if (fread(cur->buf, 1, n, cur->f) != n) cur->bad = 1;
  uint32_t n2 = rd_marker(cur->f, &ok);
  if (!ok || n2 != n) cur->bad = 1;
  cur->len = n;
  cur->pos = 0;
}

/* es: bytes of one swap unit (4 for integer, 8 for real and each complex part) */
void fio_ritem(void* p, unsigned long bytes) {
  if (!cur || cur->bad) return;
  if (cur->pos + bytes > cur->len) {
    cur->bad = 1;
    return;
  }
  memcpy(p, cur->buf + cur->pos, bytes);
  cur->pos += bytes;
}

void fio_ritem_es(void* p, unsigned long es, unsigned long count) {
  unsigned long bytes = es * count;
  if (!cur || cur->bad) return;
  if (cur->pos + bytes > cur->len) {
    cur->bad = 1;
    return;
  }
  unsigned char* d = p;
  memcpy(d, cur->buf + cur->pos, bytes);
  if (swap_bytes)
    for (unsigned long i = 0; i < count; ++i)
      for (unsigned long k = 0; k < es / 2; ++k) {
        unsigned char t = d[i * es + k];
        d[i * es + k] = d[i * es + es - 1 - k];
        d[i * es + es - 1 - k] = t;
      }
  cur->pos += bytes;
}

int fio_rend(void) { return !cur || cur->bad; }

static unsigned char* wbuf;
static size_t wlen, wcap;
static int wunit;

void fio_wbegin(int unit) {
  wunit = unit;
  wlen = 0;
}

void fio_witem_es(const void* p, unsigned long es, unsigned long count) {
  unsigned long bytes = es * count;
  if (wlen + bytes > wcap) {
    wcap = (wlen + bytes) * 2;
    wbuf = realloc(wbuf, wcap);
  }
  unsigned char* d = wbuf + wlen;
  memcpy(d, p, bytes);
  if (swap_bytes)
    for (unsigned long i = 0; i < count; ++i)
      for (unsigned long k = 0; k < es / 2; ++k) {
        unsigned char t = d[i * es + k];
        d[i * es + k] = d[i * es + es - 1 - k];
        d[i * es + es - 1 - k] = t;
      }
  wlen += bytes;
}

void fio_witem(const void* p, unsigned long bytes) { fio_witem_es(p, bytes, 1); }

int fio_wend(void) {
  if (wunit < 0 || wunit >= 128 || !units[wunit].f) return 1;
  FILE* f = units[wunit].f;
  if (units[wunit].trunc) {
    fflush(f);
    if (ftruncate(fileno(f), ftell(f)) != 0) return 1;
    units[wunit].trunc = 0;
  }
  wr_marker(f, (uint32_t)wlen);
  fwrite(wbuf, 1, wlen, f);
  wr_marker(f, (uint32_t)wlen);
  fflush(f);
  return 0;
}

/* formatted writes: numeric items only, one line per statement */
static int funit;
static char fline[4096];
static size_t fpos;

void fio_fbegin(int unit) {
  funit = unit;
  fpos = 0;
  fline[0] = 0;
}

void fio_fnum(double v) {
  if (fpos < sizeof fline - 40) fpos += (size_t)snprintf(fline + fpos, sizeof fline - fpos, "%.17g ", v);
}

void fio_fend(void) {
  if (funit >= 0 && funit < 128 && units[funit].f && units[funit].formatted) {
    fprintf(units[funit].f, "%s\n", fline);
    fflush(units[funit].f);
  }
}

/* list-directed reads: values separated by blanks or commas, continuing to
 * further records when a statement needs more values; the rest of the last
 * record is skipped (so the deck's trailing "! comment" text is never read).
 * Unit 5 (or *) reads the deck text given with ref_set_stdin. */
static char* stdin_text;
static size_t stdin_pos;
static char lline[4096];
static size_t lpos;
static int lunit, lbad;

void ref_set_stdin(const char* text) {
  free(stdin_text);
  stdin_text = strdup(text ? text : "");
  stdin_pos = 0;
}

static int next_record(void) {
  lline[0] = 0;
  lpos = 0;
  if (lunit == 5 || lunit < 0) {
    if (!stdin_text || !stdin_text[stdin_pos]) return 0;
    size_t k = 0;
    while (stdin_text[stdin_pos] && stdin_text[stdin_pos] != '\n' && k < sizeof lline - 1)
      lline[k++] = stdin_text[stdin_pos++];
    if (stdin_text[stdin_pos] == '\n') ++stdin_pos;
    lline[k] = 0;
    return 1;
  }
  if (lunit >= 128 || !units[lunit].f) return 0;
  return fgets(lline, sizeof lline, units[lunit].f) != 0;
}

void fio_lbegin(int unit) {
  lunit = unit;
  lbad = !next_record();
}

static int next_token(char* tok, size_t n) {
  for (;;) {
    if (lbad) return 0;
    while (lline[lpos] == ' ' || lline[lpos] == '\t' || lline[lpos] == '\r' || lline[lpos] == '\n') ++lpos;
    if (lline[lpos] == ',') {
      ++lpos;
      continue;
    }
    if (!lline[lpos]) {
      if (!next_record()) {
        lbad = 1;
        return 0;
      }
      continue;
    }
    size_t k = 0;
    if (lline[lpos] == '\'' || lline[lpos] == '"') {
      char q = lline[lpos++];
      while (lline[lpos] && lline[lpos] != q && k < n - 1) tok[k++] = lline[lpos++];
      if (lline[lpos] == q) ++lpos;
    } else {
      while (lline[lpos] && !strchr(" \t,\r\n", lline[lpos]) && k < n - 1) tok[k++] = lline[lpos++];
    }
    tok[k] = 0;
    return 1;
  }
}

void fio_lint(int* p) {
  char t[128];
  if (next_token(t, sizeof t)) *p = (int)strtol(t, 0, 10);
}

void fio_lreal(double* p) {
  char t[128];
  if (!next_token(t, sizeof t)) return;
  for (char* c = t; *c; ++c)
    if (*c == 'd' || *c == 'D') *c = 'e';
  *p = strtod(t, 0);
}

void fio_lreal4(float* p) {
  double d = 0;
  fio_lreal(&d);
  *p = (float)d;
}

void fio_lcx(cx* p) {
  char t[256];
  if (!next_token(t, sizeof t)) return;
  double a = 0, b = 0;
  sscanf(t, "(%lf", &a);
  if (next_token(t, sizeof t)) sscanf(t, "%lf", &b);
  p->re = a;
  p->im = b;
}

void fio_llog(int* p) {
  char t[128];
  if (!next_token(t, sizeof t)) return;
  const char* c = t[0] == '.' ? t + 1 : t;
  *p = (*c == 't' || *c == 'T');
}

void fio_lchar(char* p, int len) {
  char t[512];
  if (next_token(t, sizeof t)) fstr_assign(p, len, t);
}

int fio_lend(void) { return lbad; }

/* formatted read of one character item under (aW): the record's first W
 * characters (the whole record for W < 0), blank-padded to len */
int fio_aread(int unit, char* p, int len, int width) {
  lunit = unit;
  if (!next_record()) return 1;
  char t[4096];
  size_t k = 0;
  while (lline[k] && lline[k] != '\r' && lline[k] != '\n' && (width < 0 || (int)k < width) && k < sizeof t - 1) {
    t[k] = lline[k];
    ++k;
  }
  t[k] = 0;
  fstr_assign(p, len, t);
  return 0;
}

int fio_exists(const char* file) {
  char path[2048];
  path_of(path, sizeof path, file);
  FILE* f = fopen(path, "rb");
  if (f) fclose(f);
  return f != 0;
}

/* ---------------- the reference's C and utility routines ---------------- */

int f_iargc(void) { return 0; }
void f_getarg(int* i, char* arg) { (void)i; fstr_assign(arg, 1, " "); }

/* diagnostics the benchmark decks never turn on */
#ifndef REF_HAVE_wdata
void f_wdata() { trap(4, "wdata is not translated"); }
#endif
void f_fstat3d() { trap(4, "fstat3d is not translated"); }
void f_fstat2d() { trap(4, "fstat2d is not translated"); }
void f_cfilter() { trap(4, "cfilter stops the reference on entry"); }
void f_traces() { trap(4, "traces is not translated"); }
void f_sstat() { trap(4, "sstat is not translated"); }
void f_expdrv() { trap(4, "the explicit drivers are not translated"); }
void f_expdrv3d() { trap(4, "the explicit drivers are not translated"); }
void f_warning() {}

/* src/getver.c igetver: the highest version N of base.ext.N present, 0 if none */
int f_igetver(char* base, char* ext) {
  char pat[1024];
  snprintf(pat, sizeof pat, "%s.%s.", fstr_trim(base), fstr_trim(ext));
  int best = 0;
  for (int v = 1; v < 10000; ++v) {
    char path[2048];
    snprintf(path, sizeof path, "%s/%s%d", run_dir, pat, v);
    FILE* f = fopen(path, "rb");
    if (f) {
      fclose(f);
      best = v;
    } else if (v > best + 64) {
      break;
    }
  }
  return best;
}

/* src/getver.c addver: fname = base.ext.iver */
void f_addver(char* base, char* ext, int* iver, char* fname, int* lfile) {
  char s[1024];
  snprintf(s, sizeof s, "%s.%s.%d", fstr_trim(base), fstr_trim(ext), *iver);
  fstr_assign(fname, *lfile, s);
}

/* src/second.f90: CPU time; a constant keeps the history reproducible */
double f_second(void) { return 0.0; }
float f_second4(void) { return 0.0f; }

/* ---------------- access for the Python driver ---------------- */

void* ref_scalar(const char* name, int* type) {
  for (const ref_sym* s = ref_scalars; s->name; ++s)
    if (!strcmp(s->name, name)) {
      *type = s->type;
      return s->addr;
    }
  return 0;
}

fdesc* ref_array(const char* name, int* type) {
  for (const ref_sym* s = ref_arrays; s->name; ++s)
    if (!strcmp(s->name, name)) {
      *type = s->type;
      return (fdesc*)s->addr;
    }
  return 0;
}

const ref_proc* ref_proc_find(const char* name) {
  for (const ref_proc* p = ref_procs; p->name; ++p)
    if (!strcmp(p->name, name)) return p;
  return 0;
}

void ref_reset_oob(void) { ref_oob_count = 0; ref_dim_count = 0; }
long ref_get_oob(void) { return ref_oob_count; }
long ref_get_dim(void) { return ref_dim_count; }
