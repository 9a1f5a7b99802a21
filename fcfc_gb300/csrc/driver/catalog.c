/*
 * catalog.c -- ASCII catalogue reading as FCFC does it
 * (src/io/read_ascii.c:540-800, formatter src/io/ascii_fmtr.c:114-300):
 * the first ASCII_SKIP lines are dropped, then empty lines and lines that
 * start (after blanks) with the ASCII_COMMENT character; every other line is
 * read with the scanf conversions of ASCII_FORMATTER, one conversion at a
 * time; `$n` is the n-th conversion not suppressed with `*`.  POSITION and
 * WEIGHT are numeric expressions of the columns, SELECTION a boolean one.
 * A `%f` column is read into a float, as FCFC reads it.
 */
#define _POSIX_C_SOURCE 200809L
#include "catalog.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "expr.h"

/* C_NULL: a conversion FCFC's expressions cannot use (other integer
 * widths, unsigned, %n): read past, unusable in expressions */
enum { C_SKIP, C_INT, C_LONG, C_FLT, C_DBL, C_STR, C_NULL };

typedef struct {
  char fmt[96];      /* literal text since the previous conversion + the
                        conversion (suppressed for strings) + "%n" */
  int type;
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
    while (isdigit((unsigned char) *p)) p++;
    char l1 = 0, l2 = 0;
    if (*p == 'h' || *p == 'l' || *p == 'j' || *p == 'z' || *p == 't' ||
        *p == 'L') {
      l1 = *p++;
      if ((l1 == 'h' || l1 == 'l') && *p == l1) l2 = *p++;
    }
    char c = *p++;
    int type;
    if (c && strchr("di", c))
      type = (!l1) ? C_INT : ((l1 == 'l' && !l2) ? C_LONG : C_NULL);
    else if (c && strchr("ouxXn", c))
      type = C_NULL;
    else if (c && strchr("aAeEfFgG", c))
      type = (!l1) ? C_FLT : ((l1 == 'l' || l1 == 'L') && !l2 ? C_DBL : C_NULL);
    else if (c == 's' || c == 'c')
      type = C_STR;
    else if (c == '[') {
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
    n++;
    start = p;
    f = p;
  }
  *out = cv;
  *nconv = n;
  return 0;
}

int cat_read_ascii(const char *fname, const char *fmtr, const char *const pos[3],
    const char *wexpr, const char *sel, long skip, char comment,
    double **xyz, double **w, size_t *num, char *err, size_t errlen) {
  conv_t *cv = NULL;
  int nconv = 0, rc = -1;
  expr_node *ex[5] = {NULL, NULL, NULL, NULL, NULL};
  expr_val *cols = NULL;
  FILE *fp = NULL;
  char *line = NULL;
  size_t lcap = 0, n = 0, cap = 0;
  double *o[4] = {NULL, NULL, NULL, NULL};
  *num = 0;
  if (parse_fmtr(fmtr, &cv, &nconv, err, errlen)) return -1;
  int nread = 0;
  for (int i = 0; i < nconv; i++) nread += (cv[i].type != C_SKIP);
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
  cols = calloc((size_t) (nread > 0 ? nread : 1), sizeof *cols);
  if (!cols || !(fp = fopen(fname, "r"))) {
    snprintf(err, errlen, "cannot read `%s'", fname);
    goto done;
  }
  long lineno = 0;
  ssize_t len;
  while ((len = getline(&line, &lcap, fp)) >= 0) {
    if (lineno++ < skip) continue;
    char *p = line;
    while (isspace((unsigned char) *p)) p++;
    if (!*p || (comment && *p == comment)) continue;
    /* the conversions, one at a time */
    const char *q = p;
    int j = 0;
    for (int i = 0; i < nconv; i++) {
      int used = 0, got = 0;
      expr_val *c = (cv[i].type == C_SKIP) ? NULL : cols + j;
      switch (cv[i].type) {
        case C_SKIP:
          got = sscanf(q, cv[i].fmt, &used);
          got = (got == 0 && used > 0);
          break;
        case C_INT: {
          int v = 0;
          got = (sscanf(q, cv[i].fmt, &v, &used) == 1 && used > 0);
          c->is_str = 0;
          c->num = (double) v;
          break;
        }
        case C_LONG: {
          long v = 0;
          got = (sscanf(q, cv[i].fmt, &v, &used) == 1 && used > 0);
          c->is_str = 0;
          c->num = (double) v;
          break;
        }
        case C_NULL:
          got = sscanf(q, cv[i].fmt, &used);
          got = (got == 0 && used > 0);
          c->is_str = -1;
          break;
        case C_FLT: {
          float v = 0;
          got = (sscanf(q, cv[i].fmt, &v, &used) == 1 && used > 0);
          c->is_str = 0;
          c->num = (double) v;
          break;
        }
        case C_DBL: {
          double v = 0;
          got = (sscanf(q, cv[i].fmt, &v, &used) == 1 && used > 0);
          c->is_str = 0;
          c->num = v;
          break;
        }
        default: {   /* string: its position and length */
          const char *s = q;
          while (isspace((unsigned char) *s)) s++;
          got = sscanf(q, cv[i].fmt, &used);
          got = (got == 0 && used > 0);
          c->is_str = 1;
          c->str = s;
          c->len = (size_t) (q + used - s);
          break;
        }
      }
      if (!got) {
        snprintf(err, errlen, "failed to read line %ld of `%s' with format "
                 "`%s'", lineno, fname, fmtr);
        goto done;
      }
      q += used;
      if (cv[i].type != C_SKIP) j++;
    }
    if (ex[4]) {
      int keep = 0;
      if (expr_eval_bool(ex[4], cols, &keep)) {
        snprintf(err, errlen, "cannot evaluate SELECTION `%s'", sel);
        goto done;
      }
      if (!keep) continue;
    }
    if (n == cap) {
      cap = cap ? 2 * cap : 65536;
      for (int k = 0; k < 4; k++) {
        if (k == 3 && !ex[3]) continue;
        double *t = realloc(o[k], sizeof(double) * cap);
        if (!t) {
          snprintf(err, errlen, "out of memory");
          goto done;
        }
        o[k] = t;
      }
    }
    for (int k = 0; k < 4; k++) {
      if (!ex[k]) continue;
      if (expr_eval_num(ex[k], cols, o[k] + n)) {
        snprintf(err, errlen, "cannot evaluate `%s'", txt[k]);
        goto done;
      }
    }
    n++;
  }
  for (int k = 0; k < 3; k++) xyz[k] = o[k];
  *w = o[3];
  o[0] = o[1] = o[2] = o[3] = NULL;
  *num = n;
  rc = 0;
done:
  for (int k = 0; k < 4; k++) free(o[k]);
  for (int k = 0; k < 5; k++) expr_free(ex[k]);
  free(cols);
  free(cv);
  free(line);
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
