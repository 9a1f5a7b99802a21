/*
 * expr.c -- parser and evaluator of catalogue column expressions
 * (precedence climbing; see expr.h for the syntax).
 */
#include "expr.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { N_NUM, N_STR, N_COL, N_FN, N_UN, N_BIN };
enum { F_ABS, F_SQRT, F_LN, F_LOG, F_ISFINITE };
enum {
  O_POW, O_MUL, O_DIV, O_REM, O_ADD, O_SUB, O_SHL, O_SHR, O_LT, O_LE, O_GT,
  O_GE, O_EQ, O_NE, O_BAND, O_BXOR, O_BOR, O_LAND, O_LOR,
  O_NEG, O_POS, O_LNOT, O_BNOT
};

struct expr_node {
  int kind, op;
  double num;
  char *str;
  size_t len;
  int col;
  expr_node *a, *b;
};

static const struct {
  const char *tok;
  int op, prec;
} BIN[] = {
  {"**", O_POW, 11}, {"<<", O_SHL, 8}, {">>", O_SHR, 8}, {"<=", O_LE, 7},
  {">=", O_GE, 7}, {"==", O_EQ, 6}, {"!=", O_NE, 6}, {"&&", O_LAND, 2},
  {"||", O_LOR, 1}, {"*", O_MUL, 10}, {"/", O_DIV, 10}, {"%", O_REM, 10},
  {"+", O_ADD, 9}, {"-", O_SUB, 9}, {"<", O_LT, 7}, {">", O_GT, 7},
  {"&", O_BAND, 5}, {"^", O_BXOR, 4}, {"|", O_BOR, 3},
};

typedef struct {
  const char *s, *p;
  char *err;
  size_t errlen;
  int fail;
} parser;

static expr_node *node_new(int kind) {
  expr_node *n = calloc(1, sizeof *n);
  if (n) n->kind = kind;
  return n;
}

void expr_free(expr_node *e) {
  if (!e) return;
  expr_free(e->a);
  expr_free(e->b);
  free(e->str);
  free(e);
}

static void perr(parser *P, const char *what) {
  if (!P->fail && P->err && P->errlen)
    snprintf(P->err, P->errlen, "%s at offset %d of `%s'", what,
             (int) (P->p - P->s), P->s);
  P->fail = 1;
}

static void skipws(parser *P) {
  while (isspace((unsigned char) *P->p)) P->p++;
}

static expr_node *binary(parser *P, int minp);

static expr_node *atom(parser *P) {
  skipws(P);
  const char *c = P->p;
  if (*c == '(') {
    P->p++;
    expr_node *n = binary(P, 1);
    skipws(P);
    if (*P->p != ')') {
      perr(P, "missing `)'");
      expr_free(n);
      return NULL;
    }
    P->p++;
    return n;
  }
  if (*c == '$') {
    int brace = (c[1] == '{');
    const char *d = c + 1 + brace;
    if (!isdigit((unsigned char) *d)) {
      perr(P, "bad column");
      return NULL;
    }
    long k = strtol(d, (char **) &d, 10);
    if (brace) {
      if (*d != '}') {
        perr(P, "missing `}'");
        return NULL;
      }
      d++;
    }
    if (k < 1 || k > 100000) {
      perr(P, "bad column index");
      return NULL;
    }
    expr_node *n = node_new(N_COL);
    if (!n) return NULL;
    n->col = (int) k;
    P->p = d;
    return n;
  }
  if (*c == '"' || *c == '\'') {
    const char *e = strchr(c + 1, *c);
    if (!e) {
      perr(P, "unterminated string");
      return NULL;
    }
    expr_node *n = node_new(N_STR);
    if (!n) return NULL;
    n->len = (size_t) (e - c - 1);
    n->str = malloc(n->len + 1);
    if (!n->str) {
      free(n);
      return NULL;
    }
    memcpy(n->str, c + 1, n->len);
    n->str[n->len] = '\0';
    P->p = e + 1;
    return n;
  }
  if (isdigit((unsigned char) *c) || (*c == '.' && isdigit((unsigned char) c[1]))) {
    char *end;
    double v = strtod(c, &end);
    expr_node *n = node_new(N_NUM);
    if (!n) return NULL;
    n->num = v;
    P->p = end;
    return n;
  }
  static const struct {
    const char *name;
    int fn;
  } FN[] = {{"isfinite", F_ISFINITE}, {"sqrt", F_SQRT}, {"abs", F_ABS},
            {"log", F_LOG}, {"ln", F_LN}};
  for (size_t i = 0; i < sizeof FN / sizeof FN[0]; i++) {
    size_t l = strlen(FN[i].name);
    if (!strncmp(c, FN[i].name, l) && !isalnum((unsigned char) c[l])) {
      P->p = c + l;
      skipws(P);
      if (*P->p != '(') {
        perr(P, "missing `(' after a function");
        return NULL;
      }
      P->p++;
      expr_node *arg = binary(P, 1);
      skipws(P);
      if (!arg || *P->p != ')') {
        perr(P, "missing `)'");
        expr_free(arg);
        return NULL;
      }
      P->p++;
      expr_node *n = node_new(N_FN);
      if (!n) {
        expr_free(arg);
        return NULL;
      }
      n->op = FN[i].fn;
      n->a = arg;
      return n;
    }
  }
  perr(P, "unexpected token");
  return NULL;
}

static expr_node *unary(parser *P) {
  skipws(P);
  int op = -1;
  switch (*P->p) {
    case '-': op = O_NEG; break;
    case '+': op = O_POS; break;
    case '!':
      if (P->p[1] != '=') op = O_LNOT;
      break;
    case '~': op = O_BNOT; break;
  }
  if (op < 0) return atom(P);
  P->p++;
  expr_node *a = unary(P);
  if (!a) return NULL;
  expr_node *n = node_new(N_UN);
  if (!n) {
    expr_free(a);
    return NULL;
  }
  n->op = op;
  n->a = a;
  return n;
}

static expr_node *binary(parser *P, int minp) {
  expr_node *left = unary(P);
  while (left) {
    skipws(P);
    int hit = -1;
    for (size_t i = 0; i < sizeof BIN / sizeof BIN[0]; i++)
      if (!strncmp(P->p, BIN[i].tok, strlen(BIN[i].tok))) {
        hit = (int) i;
        break;
      }
    if (hit < 0 || BIN[hit].prec < minp) return left;
    P->p += strlen(BIN[hit].tok);
    expr_node *right = binary(P, BIN[hit].prec + 1);   /* left-associative */
    if (!right) {
      expr_free(left);
      return NULL;
    }
    expr_node *n = node_new(N_BIN);
    if (!n) {
      expr_free(left);
      expr_free(right);
      return NULL;
    }
    n->op = BIN[hit].op;
    n->a = left;
    n->b = right;
    left = n;
  }
  return left;
}

expr_node *expr_compile(const char *text, char *err, size_t errlen) {
  parser P = {text, text, err, errlen, 0};
  expr_node *e = binary(&P, 1);
  skipws(&P);
  if (e && *P.p) {
    perr(&P, "trailing characters");
    expr_free(e);
    return NULL;
  }
  if (!e) perr(&P, "invalid expression");
  return e;
}

int expr_max_col(const expr_node *e) {
  if (!e) return 0;
  int m = (e->kind == N_COL) ? e->col : 0;
  int a = expr_max_col(e->a), b = expr_max_col(e->b);
  if (a > m) m = a;
  if (b > m) m = b;
  return m;
}

/* value of a node: numbers, or strings for == and != */
typedef struct {
  int is_str;
  double v;
  const char *s;
  size_t len;
} val;

static int as_int(double v, long long *out) {
  if (!(v == floor(v)) || fabs(v) > 9.2e18) return -1;
  *out = (long long) v;
  return 0;
}

static int eval(const expr_node *e, const expr_val *cols, val *out) {
  val a, b;
  long long ia, ib;
  switch (e->kind) {
    case N_NUM:
      out->is_str = 0;
      out->v = e->num;
      return 0;
    case N_STR:
      out->is_str = 1;
      out->s = e->str;
      out->len = e->len;
      return 0;
    case N_COL: {
      const expr_val *c = cols + (e->col - 1);
      if (c->is_str < 0) return -1;   /* a column expressions cannot use */
      out->is_str = c->is_str;
      out->v = c->num;
      out->s = c->str;
      out->len = c->len;
      return 0;
    }
    case N_FN:
      if (eval(e->a, cols, &a) || a.is_str) return -1;
      out->is_str = 0;
      switch (e->op) {
        case F_ABS: out->v = fabs(a.v); break;
        case F_SQRT: out->v = sqrt(a.v); break;
        case F_LN: out->v = log(a.v); break;
        case F_LOG: out->v = log10(a.v); break;
        default: out->v = isfinite(a.v) ? 1 : 0; break;
      }
      return 0;
    case N_UN:
      if (eval(e->a, cols, &a) || a.is_str) return -1;
      out->is_str = 0;
      switch (e->op) {
        case O_NEG: out->v = -a.v; break;
        case O_POS: out->v = a.v; break;
        case O_LNOT: out->v = (a.v == 0); break;
        default:
          if (as_int(a.v, &ia)) return -1;
          out->v = (double) ~ia;
          break;
      }
      return 0;
    default:
      break;
  }
  if (eval(e->a, cols, &a) || eval(e->b, cols, &b)) return -1;
  out->is_str = 0;
  if (e->op == O_EQ || e->op == O_NE) {
    int eq;
    if (a.is_str != b.is_str) return -1;
    if (a.is_str)
      eq = (a.len == b.len && !memcmp(a.s, b.s, a.len));
    else
      eq = (a.v == b.v);
    out->v = (e->op == O_EQ) ? eq : !eq;
    return 0;
  }
  if (a.is_str || b.is_str) return -1;
  switch (e->op) {
    case O_POW: out->v = pow(a.v, b.v); break;
    case O_MUL: out->v = a.v * b.v; break;
    case O_DIV: out->v = a.v / b.v; break;
    case O_REM: out->v = fmod(a.v, b.v); break;
    case O_ADD: out->v = a.v + b.v; break;
    case O_SUB: out->v = a.v - b.v; break;
    case O_LT: out->v = a.v < b.v; break;
    case O_LE: out->v = a.v <= b.v; break;
    case O_GT: out->v = a.v > b.v; break;
    case O_GE: out->v = a.v >= b.v; break;
    case O_LAND: out->v = (a.v != 0) && (b.v != 0); break;
    case O_LOR: out->v = (a.v != 0) || (b.v != 0); break;
    default:
      if (as_int(a.v, &ia) || as_int(b.v, &ib)) return -1;
      switch (e->op) {
        case O_SHL: out->v = (double) (ia << ib); break;
        case O_SHR: out->v = (double) (ia >> ib); break;
        case O_BAND: out->v = (double) (ia & ib); break;
        case O_BXOR: out->v = (double) (ia ^ ib); break;
        default: out->v = (double) (ia | ib); break;
      }
  }
  return 0;
}

int expr_eval_num(const expr_node *e, const expr_val *cols, double *out) {
  val v;
  if (eval(e, cols, &v) || v.is_str) return -1;
  *out = v.v;
  return 0;
}

int expr_eval_bool(const expr_node *e, const expr_val *cols, int *out) {
  val v;
  if (eval(e, cols, &v) || v.is_str) return -1;
  *out = (v.v != 0);
  return 0;
}
