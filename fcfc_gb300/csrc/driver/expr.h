/*
 * expr.h -- column expressions of FCFC's catalogue keys (POSITION, WEIGHT,
 * SELECTION) in the syntax of its expression library (src/lib/libast.h):
 * numbers, "strings", $n / ${n} columns, parentheses, abs sqrt ln log
 * isfinite, unary - + ! ~, ** * / % + - << >> < <= > >= == != & ^ | && ||.
 * Unary operators bind above `**`; every binary operator is
 * left-associative, as in libast's precedence table (libast.c:134-201).
 * Numbers are evaluated in double precision; strings only compare.
 */
#ifndef FCFCG_EXPR_H
#define FCFCG_EXPR_H

#include <stddef.h>

typedef struct expr_node expr_node;

/* One column value of a catalogue line. */
typedef struct {
  int is_str;           /* 1 string, 0 number, -1 unusable column */
  double num;
  const char *str;      /* not terminated: str[0 .. len) */
  size_t len;
} expr_val;

/* Compile an expression; NULL on a syntax error (message in err). */
expr_node *expr_compile(const char *text, char *err, size_t errlen);
void expr_free(expr_node *e);
/* Largest column index the expression uses (0: none). */
int expr_max_col(const expr_node *e);
/* Evaluate with cols[k - 1] the value of $k; 0 on success. */
int expr_eval_num(const expr_node *e, const expr_val *cols, double *out);
int expr_eval_bool(const expr_node *e, const expr_val *cols, int *out);

#endif
