/*
 * catalog.c -- ASCII catalogue reading as FCFC does it
 * (src/io/read_ascii.c:540-800, formatter src/io/ascii_fmtr.c:114-300):
 * the first ASCII_SKIP lines are dropped, then empty lines and lines that
 * start (after blanks) with the ASCII_COMMENT character; every other line is
 * read with the scanf conversions of ASCII_FORMATTER, one conversion at a
 * time; `$n` is the n-th conversion not suppressed with `*`.  POSITION and
 * WEIGHT are numeric expressions of the columns, SELECTION a boolean one.
 * A `%f` column is read into a float, as FCFC reads it; only int, long,
 * float, double and string columns are usable in expressions (the others,
 * e.g. `%Lf` or `%hd`, are read past), as in read_ascii.c:113-121.
 *
 * Like FCFC (which parses the lines of a file chunk with OpenMP), the file
 * is read in chunks whose lines are parsed by several threads; the rows keep
 * the file's order.  Formatters made only of numeric conversions separated
 * by blanks take a fast path (strtod / strtof / strtol, the conversions
 * scanf itself uses); a line the fast path cannot take as a whole -- a
 * number not followed by a blank or the end of the line, an int out of
 * range -- is read again with sscanf, so both paths give the same values.
 */
#define _POSIX_C_SOURCE 200809L
#include "catalog.h"

#include <ctype.h>
#include <errno.h>
#include <limits.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "expr.h"

/* C_NULL: a conversion FCFC's expressions cannot use (other integer
 * widths, unsigned, long double, %n): read past, unusable in expressions */
enum { C_SKIP, C_INT, C_LONG, C_FLT, C_DBL, C_STR, C_NULL };

typedef struct {
  char fmt[96];      /* literal text since the previous conversion + the
                        conversion (suppressed for strings) + "%n" */
  int type;
  /* fast path: numeric conversion without width after blank-only text */
  int fast;
  char spec;         /* conversion character */
  int num;           /* numeric: 0 none, 'i' integer, 'f' float, 'd' double */
} conv_t;

static int parse_fmtr(const char *f, conv_t **out, int *nconv, char *err,
    size_t errlen) {
  int cap = 16, n = 0;
  conv_t *cv = malloc(sizeof *cv * cap);
  if (!cv) return -1;
  const char *start = f;
  while (*f) {
    if (*f != '%') {
      f++;
      continue;
    }
    if (f[1] == '%') {
      f += 2;
      continue;
    }
    const char *p = f + 1;
    int skip = 0;
    if (*p == '*') {
      skip = 1;
      p++;
    }
    int width = 0;
    while (isdigit((unsigned char) *p)) {
      width = 1;
      p++;
    }
    char l1 = 0, l2 = 0;
    if (*p == 'h' || *p == 'l' || *p == 'j' || *p == 'z' || *p == 't' ||
        *p == 'L') {
      l1 = *p++;
      if ((l1 == 'h' || l1 == 'l') && *p == l1) l2 = *p++;
    }
    char c = *p++;
    int type, num = 0;
    if (c && strchr("di", c)) {
      type = (!l1) ? C_INT : ((l1 == 'l' && !l2) ? C_LONG : C_NULL);
      num = (!l1 || (l1 == 'l' && !l2)) ? 'i' : 0;
    } else if (c && strchr("ouxXn", c)) {
      type = C_NULL;
    } else if (c && strchr("aAeEfFgG", c)) {
      type = (!l1) ? C_FLT : ((l1 == 'l' && !l2) ? C_DBL : C_NULL);
      num = (!l1) ? 'f' : ((l1 == 'l' && !l2) ? 'd' : 0);
    } else if (c == 's' || c == 'c') {
      type = C_STR;
    } else if (c == '[') {
      type = C_STR;
      if (*p == '^') p++;
      if (*p == ']') p++;
      while (*p && *p != ']') p++;
      if (*p == ']') p++;
    } else {
      snprintf(err, errlen, "invalid ASCII_FORMATTER `%s'", start);
      free(cv);
      return -1;
    }
    if (n == cap) {
      cap *= 2;
      conv_t *t = realloc(cv, sizeof *cv * cap);
      if (!t) {
        free(cv);
        return -1;
      }
      cv = t;
    }
    /* the literal text before this conversion belongs to it */
    size_t pre = (size_t) (f - start);
    size_t body = (size_t) (p - f);
    if (pre + body + 4 >= sizeof cv[n].fmt) {
      snprintf(err, errlen, "ASCII_FORMATTER too long");
      free(cv);
      return -1;
    }
    int blank = 1;
    for (const char *q = start; q < f; q++)
      if (!isspace((unsigned char) *q)) blank = 0;
    char *o = cv[n].fmt;
    memcpy(o, start, pre);
    o += pre;
    if (skip || type == C_STR || type == C_NULL) {
      /* read past it: suppressed conversion */
      *o++ = '%';
      *o++ = '*';
      const char *q = f + 1 + (skip ? 1 : 0);
      memcpy(o, q, (size_t) (p - q));
      o += p - q;
    } else {
      memcpy(o, f, body);
      o += body;
    }
    memcpy(o, "%n", 3);
    cv[n].type = skip ? C_SKIP : type;
    cv[n].spec = c;
    cv[n].num = num;
    cv[n].fast = (num != 0) && !width && blank && c != 'n';
    n++;
    start = p;
    f = p;
  }
  *out = cv;
  *nconv = n;
  return 0;
}

/* The lines of one thread: [beg, end), each ending in '\n' (or at end). */
typedef struct {
  char *beg, *end;
  const conv_t *cv;
  int nconv, nread, fast;
  expr_node *const *ex;      /* POSITION x, y, z, WEIGHT, SELECTION */
  char comment;
  expr_val *cols;
  double *o[4];
  size_t n, cap;
  size_t nlines;             /* lines looked at (failing one included) */
  int fail;                  /* 0, or what failed on the last line */
  int fail_expr;
} part_t;

enum { F_READ = 1, F_SEL, F_EXPR, F_MEM };

/* All conversions of a line by the fast path: 0, or -1 where the line has
 * to be read with sscanf. */
static int fast_line(const part_t *P, const char *q) {
  int j = 0;
  for (int i = 0; i < P->nconv; i++) {
    const conv_t *c = P->cv + i;
    char *e;
    expr_val *v = (c->type == C_SKIP) ? NULL : P->cols + j;
    errno = 0;
    if (c->num == 'd') {
      const double x = strtod(q, &e);
      if (v) {
        v->is_str = 0;
        v->num = x;
      }
    } else if (c->num == 'f') {
      const float x = strtof(q, &e);
      if (v) {
        v->is_str = 0;
        v->num = (double) x;
      }
    } else {
      const long x = strtol(q, &e, c->spec == 'i' ? 0 : 10);
      if (errno == ERANGE) return -1;
      if (c->type == C_INT && (x < INT_MIN || x > INT_MAX)) return -1;
      if (v) {
        v->is_str = 0;
        v->num = (double) x;
      }
    }
    if (e == q || (*e && !isspace((unsigned char) *e))) return -1;
    q = e;
    if (c->type != C_SKIP) j++;
  }
  return 0;
}

/* All conversions of a line with sscanf: 0, or -1 if one fails. */
static int scanf_line(const part_t *P, const char *q) {
  int j = 0;
  for (int i = 0; i < P->nconv; i++) {
    const conv_t *cv = P->cv + i;
    int used = 0, got = 0;
    expr_val *c = (cv->type == C_SKIP) ? NULL : P->cols + j;
    switch (cv->type) {
      case C_SKIP:
        got = sscanf(q, cv->fmt, &used);
        got = (got == 0 && used > 0);
        break;
      case C_INT: {
        int v = 0;
        got = (sscanf(q, cv->fmt, &v, &used) == 1 && used > 0);
        c->is_str = 0;
        c->num = (double) v;
        break;
      }
      case C_LONG: {
        long v = 0;
        got = (sscanf(q, cv->fmt, &v, &used) == 1 && used > 0);
        c->is_str = 0;
        c->num = (double) v;
        break;
      }
      case C_NULL:
        got = sscanf(q, cv->fmt, &used);
        got = (got == 0 && used > 0);
        c->is_str = -1;
        break;
      case C_FLT: {
        float v = 0;
        got = (sscanf(q, cv->fmt, &v, &used) == 1 && used > 0);
        c->is_str = 0;
        c->num = (double) v;
        break;
      }
      case C_DBL: {
        double v = 0;
        got = (sscanf(q, cv->fmt, &v, &used) == 1 && used > 0);
        c->is_str = 0;
        c->num = v;
        break;
      }
      default: {   /* string: its position and length */
        const char *s = q;
        while (isspace((unsigned char) *s)) s++;
        got = sscanf(q, cv->fmt, &used);
        got = (got == 0 && used > 0);
        c->is_str = 1;
        c->str = s;
        c->len = (size_t) (q + used - s);
        break;
      }
    }
    if (!got) return -1;
    q += used;
    if (cv->type != C_SKIP) j++;
  }
  return 0;
}

static void *part_run(void *arg) {
  part_t *P = arg;
  char *p = P->beg;
  while (p < P->end) {
    char *nl = memchr(p, '\n', (size_t) (P->end - p));
    char *le = nl ? nl : P->end;
    *le = '\0';                      /* conversions stop at the line's end */
    char *line = p;
    p = le + 1;
    P->nlines++;
    while (isspace((unsigned char) *line)) line++;
    if (!*line || (P->comment && *line == P->comment)) continue;
    if (!(P->fast && fast_line(P, line) == 0) && scanf_line(P, line)) {
      P->fail = F_READ;
      return NULL;
    }
    if (P->ex[4]) {
      int keep = 0;
      if (expr_eval_bool(P->ex[4], P->cols, &keep)) {
        P->fail = F_SEL;
        return NULL;
      }
      if (!keep) continue;
    }
    if (P->n == P->cap) {
      size_t cap = P->cap ? 2 * P->cap : 16384;
      for (int k = 0; k < 4; k++) {
        if (!P->ex[k]) continue;
        double *t = realloc(P->o[k], sizeof(double) * cap);
        if (!t) {
          P->fail = F_MEM;
          return NULL;
        }
        P->o[k] = t;
      }
      P->cap = cap;
    }
    for (int k = 0; k < 4; k++) {
      if (!P->ex[k]) continue;
      if (expr_eval_num(P->ex[k], P->cols, P->o[k] + P->n)) {
        P->fail = F_EXPR;
        P->fail_expr = k;
        return NULL;
      }
    }
    P->n++;
  }
  return NULL;
}

static int reader_threads(void) {
  const char *e = getenv("OMP_NUM_THREADS");
  long t = e ? strtol(e, NULL, 10) : sysconf(_SC_NPROCESSORS_ONLN);
  if (t < 1) t = 1;
  if (t > 64) t = 64;
  return (int) t;
}

/* Bytes read per chunk: 64 MiB, or FCFCG_ASCII_CHUNK (at least 4 KiB). */
static size_t chunk_bytes(void) {
  const char *e = getenv("FCFCG_ASCII_CHUNK");
  long v = e ? strtol(e, NULL, 10) : 0;
  return v >= 4096 ? (size_t) v : ((size_t) 64 << 20);
}

int cat_read_ascii(const char *fname, const char *fmtr, const char *const pos[3],
    const char *wexpr, const char *sel, long skip, char comment,
    double **xyz, double **w, size_t *num, char *err, size_t errlen) {
  conv_t *cv = NULL;
  int nconv = 0, rc = -1;
  expr_node *ex[5] = {NULL, NULL, NULL, NULL, NULL};
  FILE *fp = NULL;
  char *buf = NULL;
  size_t n = 0, cap = 0;
  double *o[4] = {NULL, NULL, NULL, NULL};
  const int nth = reader_threads();
  part_t *parts = calloc((size_t) nth, sizeof *parts);
  *num = 0;
  if (!parts) return -1;
  if (parse_fmtr(fmtr, &cv, &nconv, err, errlen)) goto done;
  int nread = 0, fast = 1;
  for (int i = 0; i < nconv; i++) {
    nread += (cv[i].type != C_SKIP);
    fast &= cv[i].fast;
  }
  const char *txt[5] = {pos[0], pos[1], pos[2], wexpr, sel};
  int maxc = 0;
  for (int k = 0; k < 5; k++) {
    if (!txt[k] || !*txt[k]) continue;
    if (!(ex[k] = expr_compile(txt[k], err, errlen))) goto done;
    if (expr_max_col(ex[k]) > maxc) maxc = expr_max_col(ex[k]);
  }
  if (maxc > nread) {
    snprintf(err, errlen, "not enough columns in ASCII_FORMATTER for the "
             "column expressions");
    goto done;
  }
  for (int t = 0; t < nth; t++) {
    parts[t].cv = cv;
    parts[t].nconv = nconv;
    parts[t].nread = nread;
    parts[t].fast = fast;
    parts[t].ex = ex;
    parts[t].comment = comment;
    parts[t].cols = calloc((size_t) (nread > 0 ? nread : 1), sizeof(expr_val));
    if (!parts[t].cols) goto done;
  }
  if (!(fp = fopen(fname, "r"))) {
    snprintf(err, errlen, "cannot read `%s'", fname);
    goto done;
  }
  size_t bcap = chunk_bytes(), have = 0;
  long lineno = 0;   /* lines before the current chunk */
  if (!(buf = malloc(bcap + 1))) goto done;
  for (;;) {
    size_t got = fread(buf + have, 1, bcap - have, fp);
    have += got;
    const int eof = (got == 0);
    if (have == 0) break;
    /* complete lines: up to the last newline (all of it at the end) */
    size_t stop = have;
    if (!eof) {
      while (stop > 0 && buf[stop - 1] != '\n') stop--;
      if (stop == 0) {   /* a line longer than the buffer */
        char *t = realloc(buf, 2 * bcap + 1);
        if (!t) goto done;
        buf = t;
        bcap *= 2;
        continue;
      }
    }
    char *beg = buf, *end = buf + stop;
    if (eof) *end = '\0';   /* a last line without a newline ends here
                              (buf has a byte to spare); otherwise buf[stop]
                              starts the line carried over */
    while (skip > 0 && beg < end) {    /* ASCII_SKIP */
      char *nl = memchr(beg, '\n', (size_t) (end - beg));
      beg = nl ? nl + 1 : end;
      skip--;
      lineno++;
    }
    /* split at line starts, one range per thread */
    int np = 0;
    const size_t len = (size_t) (end - beg);
    const int want = (len < (1u << 16)) ? 1 : nth;
    char *cur = beg;
    for (int t = 0; t < want && cur < end; t++) {
      char *e = (t == want - 1) ? end : beg + len * (size_t) (t + 1) / want;
      if (e < cur) e = cur;
      if (e < end) {
        char *nl = memchr(e, '\n', (size_t) (end - e));
        e = nl ? nl + 1 : end;
      }
      part_t *P = parts + np++;
      P->beg = cur;
      P->end = e;
      P->n = 0;
      P->nlines = 0;
      P->fail = 0;
      cur = e;
    }
    pthread_t tid[64];
    int started[64] = {0};
    for (int t = 1; t < np; t++)
      started[t] = !pthread_create(tid + t, NULL, part_run, parts + t);
    part_run(parts);
    for (int t = 1; t < np; t++) {
      if (started[t]) pthread_join(tid[t], NULL);
      else part_run(parts + t);
    }
    /* the first failure in file order */
    long before = lineno;
    for (int t = 0; t < np; t++) {
      part_t *P = parts + t;
      if (P->fail) {
        const long ln = before + (long) P->nlines;
        if (P->fail == F_READ)
          snprintf(err, errlen, "failed to read line %ld of `%s' with format "
                   "`%s'", ln, fname, fmtr);
        else if (P->fail == F_SEL)
          snprintf(err, errlen, "cannot evaluate SELECTION `%s' (line %ld)",
                   sel, ln);
        else if (P->fail == F_EXPR)
          snprintf(err, errlen, "cannot evaluate `%s' (line %ld)",
                   txt[P->fail_expr], ln);
        else
          snprintf(err, errlen, "out of memory");
        goto done;
      }
      before += (long) P->nlines;
    }
    lineno = before;
    /* append the rows in file order */
    size_t add = 0;
    for (int t = 0; t < np; t++) add += parts[t].n;
    if (n + add > cap) {
      size_t nc = cap ? cap : 65536;
      while (nc < n + add) nc *= 2;
      for (int k = 0; k < 4; k++) {
        if (!ex[k]) continue;
        double *t = realloc(o[k], sizeof(double) * nc);
        if (!t) {
          snprintf(err, errlen, "out of memory");
          goto done;
        }
        o[k] = t;
      }
      cap = nc;
    }
    for (int t = 0; t < np; t++) {
      for (int k = 0; k < 4; k++)
        if (ex[k] && parts[t].n)
          memcpy(o[k] + n, parts[t].o[k], sizeof(double) * parts[t].n);
      n += parts[t].n;
    }
    /* carry the incomplete last line over */
    memmove(buf, buf + stop, have - stop);
    have -= stop;
    if (eof) break;
  }
  if (ferror(fp)) {
    snprintf(err, errlen, "cannot read `%s'", fname);
    goto done;
  }
  for (int k = 0; k < 3; k++) xyz[k] = o[k];
  *w = o[3];
  o[0] = o[1] = o[2] = o[3] = NULL;
  *num = n;
  rc = 0;
done:
  for (int k = 0; k < 4; k++) free(o[k]);
  for (int k = 0; k < 5; k++) expr_free(ex[k]);
  for (int t = 0; t < nth; t++) {
    for (int k = 0; k < 4; k++) free(parts[t].o[k]);
    free(parts[t].cols);
  }
  free(parts);
  free(cv);
  free(buf);
  if (fp) fclose(fp);
  return rc;
}

int cat_read_table(const char *fname, double **a, double **b, size_t *num,
    char *err, size_t errlen) {
  FILE *fp = fopen(fname, "r");
  if (!fp) {
    snprintf(err, errlen, "cannot read `%s'", fname);
    return -1;
  }
  char *line = NULL;
  size_t lcap = 0, n = 0, cap = 0;
  double *x = NULL, *y = NULL;
  int rc = 0;
  while (getline(&line, &lcap, fp) >= 0) {
    char *p = line;
    while (isspace((unsigned char) *p)) p++;
    if (!*p || *p == '#') continue;
    double u, v;
    if (sscanf(p, "%lf %lf", &u, &v) != 2) {
      snprintf(err, errlen, "failed to read a line of `%s'", fname);
      rc = -1;
      break;
    }
    if (n == cap) {
      cap = cap ? 2 * cap : 64;
      double *t1 = realloc(x, sizeof(double) * cap);
      if (t1) x = t1;
      double *t2 = realloc(y, sizeof(double) * cap);
      if (t2) y = t2;
      if (!t1 || !t2) {
        rc = -1;
        break;
      }
    }
    x[n] = u;
    y[n] = v;
    n++;
  }
  free(line);
  fclose(fp);
  if (rc) {
    free(x);
    free(y);
    return rc;
  }
  *a = x;
  *b = y;
  *num = n;
  return 0;
}
