/*
 * conf.c -- configuration of the command line drivers: the KEY = value
 * parser, FCFC's command line options with libcfg's rules and priorities,
 * and FCFC's checks of the output files (OVERWRITE).
 */
#define _POSIX_C_SOURCE 200809L
#include <ctype.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "conf.h"

void die(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "Error: ");
  vfprintf(stderr, fmt, ap);
  fprintf(stderr, "\n");
  va_end(ap);
  exit(1);
}

static char *trim(char *s) {
  while (isspace((unsigned char) *s)) s++;
  char *e = s + strlen(s);
  while (e > s && isspace((unsigned char) e[-1])) *--e = '\0';
  return s;
}

static char *unquote(char *s) {
  s = trim(s);
  size_t l = strlen(s);
  if (l >= 2 && (s[0] == '"' || s[0] == '\'') && s[l - 1] == s[0]) {
    s[l - 1] = '\0';
    s++;
  }
  return s;
}

static char *strip_comment(char *s) {
  char q = 0;
  for (char *p = s; *p; p++) {
    if (q) {
      if (*p == q) q = 0;
    } else if (*p == '"' || *p == '\'') {
      q = *p;
    } else if (*p == '#') {
      *p = '\0';
      break;
    }
  }
  return s;
}

void conf_add(conf_t *C, const char *key, char *val, int prio) {
  for (int i = 0; i < C->n; i++)
    if (C->e[i].prio == prio && !strcmp(C->e[i].key, key)) {
      fprintf(stderr, "Warning: omitting duplicate entry of parameter `%s'\n",
              key);
      return;
    }
  if (C->n == C->cap) {
    C->cap = C->cap ? 2 * C->cap : 32;
    C->e = realloc(C->e, sizeof *C->e * C->cap);
    if (!C->e) die("out of memory");
  }
  entry_t *E = C->e + C->n++;
  E->key = strdup(key);
  E->n = 0;
  E->v = NULL;
  E->prio = prio;
  val = trim(val);
  if (*val == '[') {
    char *end = strrchr(val, ']');
    if (end) *end = '\0';
    char *p = val + 1;
    for (;;) {
      /* split at commas outside quotes */
      char q = 0, *s = p;
      while (*p && (q || *p != ',')) {
        if (q && *p == q) q = 0;
        else if (!q && (*p == '"' || *p == '\'')) q = *p;
        p++;
      }
      int last = (*p == '\0');
      *p = '\0';
      E->v = realloc(E->v, sizeof(char *) * (E->n + 1));
      E->v[E->n++] = strdup(unquote(s));
      if (last) break;
      p++;
    }
    if (E->n == 1 && !*E->v[0]) E->n = 0;
  } else {
    E->v = malloc(sizeof(char *));
    E->v[0] = strdup(unquote(val));
    E->n = 1;
  }
}

void conf_read(conf_t *C, const char *fname) {
  FILE *fp = fopen(fname, "r");
  if (!fp) die("cannot open the configuration file `%s'", fname);
  char *line = NULL, *acc = NULL;
  size_t cap = 0, alen = 0;
  while (getline(&line, &cap, fp) >= 0) {
    char *l = strip_comment(line);
    size_t len = strlen(l);
    while (len && isspace((unsigned char) l[len - 1])) l[--len] = '\0';
    int cont = (len && l[len - 1] == '\\');
    if (cont) l[--len] = ' ';
    acc = realloc(acc, alen + len + 2);
    memcpy(acc + alen, l, len);
    alen += len;
    acc[alen] = '\0';
    if (cont) continue;
    char *eq = strchr(acc, '=');
    if (eq) {
      *eq = '\0';
      char *k = trim(acc);
      if (*k) conf_add(C, k, eq + 1, PRIO_FILE);
    }
    alen = 0;
  }
  free(line);
  free(acc);
  fclose(fp);
}

const entry_t *conf_get(const conf_t *C, const char *key) {
  const entry_t *best = NULL;
  for (int i = 0; i < C->n; i++)
    if (!strcmp(C->e[i].key, key) && (!best || C->e[i].prio > best->prio))
      best = C->e + i;
  return best;
}

/* the i-th value, a single value broadcast, or NULL */
const char *conf_str(const conf_t *C, const char *key, int i) {
  const entry_t *E = conf_get(C, key);
  if (!E || E->n == 0) return NULL;
  if (E->n == 1) return E->v[0];
  return (i < E->n) ? E->v[i] : NULL;
}

int conf_len(const conf_t *C, const char *key) {
  const entry_t *E = conf_get(C, key);
  return E ? E->n : 0;
}

double conf_dbl(const conf_t *C, const char *key, double def) {
  const char *s = conf_str(C, key, 0);
  if (!s || !*s) return def;
  char *end;
  double v = strtod(s, &end);
  if (*trim(end)) die("invalid value of %s: `%s'", key, s);
  return v;
}

long conf_long(const conf_t *C, const char *key, int i, long def) {
  const char *s = conf_str(C, key, i);
  if (!s || !*s) return def;
  return strtol(s, NULL, 10);
}

int is_true(const char *s) {
  return s && (s[0] == 'T' || s[0] == 't' || s[0] == '1' || s[0] == 'Y' ||
               s[0] == 'y');
}

/* FCFC's check_output (src/fcfc/2pt_box/load_conf.c:582-650) for one output
 * file: 0 to write it, 1 to read it back (an existing pair-count file with
 * 0 < OVERWRITE < force); FCFC's refusals end the run.  force: 2 for
 * PAIR_COUNT_FILE, 1 for the correlation function outputs.  A negative
 * OVERWRITE asks on the terminal, up to |OVERWRITE| times. */
int check_output(const char *fname, const char *key, int ovw,
    int force) {
  if (!fname || !*fname) die("the output file %s is not set", key);
  if (access(fname, F_OK) == 0) {
    if (ovw < 0) {
      fprintf(stderr, "Warning: the output file %s exists: `%s'\n", key,
              fname);
      int decided = 0;
      for (int i = 0; i < -ovw && !decided; i++) {
        fprintf(stderr, "Are you going to overwrite it? (y/n): ");
        const int ch = getchar();
        if (ch == EOF) continue;
        for (int c = ch; c != '\n' && c != EOF;) c = getchar();
        if (ch == 'n' || ch == 'N') {
          ovw = force - 1;
          decided = 1;
        } else if (ch == 'y' || ch == 'Y') {
          ovw = force;
          decided = 1;
        }
      }
      if (!decided) die("too many failed inputs");
    }
    if (ovw <= 0) die("abort to avoid overwriting %s: `%s'", key, fname);
    if (ovw < force) {
      if (access(fname, R_OK)) die("cannot access %s: `%s'", key, fname);
      return 1;
    }
    fprintf(stderr, "Warning: %s will be overwritten: `%s'\n", key, fname);
    if (access(fname, W_OK)) die("cannot write to file: `%s'", fname);
  } else {
    const char *sl = strrchr(fname, '/');
    if (sl && sl > fname) {
      char *dir = strndup(fname, (size_t) (sl - fname));
      if (!dir) die("out of memory");
      if (access(dir, X_OK)) die("cannot access the directory `%s'", dir);
      free(dir);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Command line: FCFC's options (src/fcfc/2pt_box/load_conf.c:477-515,     */
/* survey src/fcfc/2pt/load_conf.c:512-553), each setting one configuration */
/* key, parsed by libcfg's rules (src/lib/libcfg.c:1009-1139): `-x VALUE',  */
/* `-x=VALUE', `--long VALUE', `--long=VALUE'; a Boolean option without a   */
/* value means T; `--' ends the options; unknown options are reported and   */
/* skipped.                                                                 */

typedef struct {
  char sopt;            /* short option, 0 for none */
  const char *lopt;     /* long option */
  const char *key;      /* configuration key */
  int is_bool;
  const char *help;
} option_t;

static const option_t OPTIONS[] = {
  {'c', "conf", "CONFIG_FILE", 0, "configuration file"},
  {'i', "input", "CATALOG", 0, "input catalogues"},
  {'l', "label", "CATALOG_LABEL", 0, "catalogue labels"},
  {'T', "type", "CATALOG_TYPE", 0, "catalogue formats (0: ASCII)"},
  {0, "skip", "ASCII_SKIP", 0, "lines skipped at the start of each file"},
  {0, "comment", "ASCII_COMMENT", 0, "comment characters"},
  {'f', "formatter", "ASCII_FORMATTER", 0, "column formatters"},
  {'x', "position", "POSITION", 0, "columns or expressions of x, y, z"},
  {'w', "weight", "WEIGHT", 0, "columns or expressions of the weights"},
  {'s', "select", "SELECTION", 0, "selection expressions"},
#ifdef FCFCG_SURVEY
  {0, "convert", "COORD_CONVERT", 1, "RA, Dec, z to comoving coordinates"},
  {'d', "omega-m", "OMEGA_M", 0, "matter density parameter"},
  {0, "omega-l", "OMEGA_LAMBDA", 0, "dark energy density parameter"},
  {0, "eos-w", "DE_EOS_W", 0, "dark energy equation of state"},
  {0, "cmvdst-err", "CMVDST_ERR", 0, "error of the distance integration"},
  {0, "cmvdst-file", "Z_CMVDST_FILE", 0, "table of redshift and distance"},
#else
  {'b', "box", "BOX_SIZE", 0, "side lengths of the periodic box"},
#endif
  {'S', "data-struct", "DATA_STRUCT", 0, "data structure (0 or 1: cell grid)"},
  {'B', "bin", "BINNING_SCHEME", 0, "0: s, 1: (s, mu), 2: (s_perp, pi)"},
  {'p', "pair", "PAIR_COUNT", 0, "pairs to count or read, by label"},
  {'P', "pair-output", "PAIR_COUNT_FILE", 0, "pair-count files"},
  {'e', "cf", "CF_ESTIMATOR", 0, "correlation function estimators"},
  {'E', "cf-output", "CF_OUTPUT_FILE", 0, "correlation function files"},
  {'m', "multipole", "MULTIPOLE", 0, "Legendre multipole orders"},
  {'M', "mp-output", "MULTIPOLE_FILE", 0, "multipole files"},
  {'u', "wp", "PROJECTED_CF", 1, "projected correlation function"},
  {'U', "wp-output", "PROJECTED_FILE", 0, "projected correlation files"},
  {0, "s-file", "SEP_BIN_FILE", 0, "separation (or s_perp) bin edges file"},
  {0, "s-min", "SEP_BIN_MIN", 0, "lower limit of linear separation bins"},
  {0, "s-max", "SEP_BIN_MAX", 0, "upper limit of linear separation bins"},
  {0, "s-step", "SEP_BIN_SIZE", 0, "width of linear separation bins"},
  {0, "mu-num", "MU_BIN_NUM", 0, "number of mu bins"},
  {0, "pi-file", "PI_BIN_FILE", 0, "pi bin edges file"},
  {0, "pi-min", "PI_BIN_MIN", 0, "lower limit of linear pi bins"},
  {0, "pi-max", "PI_BIN_MAX", 0, "upper limit of linear pi bins"},
  {0, "pi-step", "PI_BIN_SIZE", 0, "width of linear pi bins"},
  {'F', "out-format", "OUTPUT_FORMAT", 0, "pair-count file format"},
  {'O', "overwrite", "OVERWRITE", 0, "overwrite policy for existing files"},
  {'v', "verbose", "VERBOSE", 1, "detailed standard output"},
};
#define NOPT ((int) (sizeof OPTIONS / sizeof OPTIONS[0]))


static void usage(void) {
  printf("Usage: %s [OPTION]\n"
         "FCFC's run flow with the pair counts on the GPU.  Every option sets "
         "the\nconfiguration key beside it, over the configuration file's "
         "value.\n"
         "  -h, --help       this message\n"
         "  -V, --version    version information\n"
         "  -t, --template   print a configuration template\n", PROG);
  for (int i = 0; i < NOPT; i++) {
    const option_t *o = OPTIONS + i;
    char s[8] = "    ";
    if (o->sopt) snprintf(s, sizeof s, "-%c, ", o->sopt);
    printf("  %s--%-13s %-16s %s%s\n", s, o->lopt, o->key, o->help,
           o->is_bool ? " (T/F)" : "");
  }
  printf("Engine options:\n"
         "      --fp64           count in FP64 only (no FP32 pass)\n"
         "      --with-mu-one    count mu = 1 in the last mu bin\n"
         "      --no-graph       run the counts one by one, not as one CUDA "
         "graph\n"
         "Default configuration file: `%s'.\n", DEFAULT_CONF);
  exit(0);
}

static void version(void) {
  printf("%s (fcfc-gb300): pair counts on one GPU, FP32 with an FP64 "
         "recheck;\nFCFC's configuration keys, estimators and file formats, "
         "FP64 counts.\n", PROG);
  exit(0);
}

static void conf_template(void) {
  printf("# Configuration for %s: KEY = value or KEY = [v1, v2, ...].\n"
         "# Arrays give one value per catalogue or per pair; '#' starts a "
         "comment.\n", PROG);
  for (int i = 0; i < NOPT; i++) {
    if (!strcmp(OPTIONS[i].key, "CONFIG_FILE")) continue;
    printf("\n# %s%s\n%s = \n", OPTIONS[i].help,
           OPTIONS[i].is_bool ? " (T or F)" : "", OPTIONS[i].key);
  }
  exit(0);
}

/* libcfg's test for an option: `-x', `-x=...', `--', or `--name...' */
static int is_opt(const char *a) {
  if (a[0] != '-' || !a[1]) return 0;
  if (isalpha((unsigned char) a[1])) return !a[2] || a[2] == '=';
  if (a[1] == '-') return !a[2] || (a[2] != '=' && isgraph((unsigned char) a[2]));
  return 0;
}

/* Command line options into C (PRIO_CMD); the engine's own flags are
 * returned through the pointers. */
void conf_parse_args(conf_t *C, int argc, char **argv, int *fp64,
    int *mu_one, int *graph) {
  for (int i = 1; i < argc; i++) {
    char *arg = argv[i];
    if (!strcmp(arg, "--fp64")) {
      *fp64 = 1;
      continue;
    }
    if (!strcmp(arg, "--with-mu-one")) {
      *mu_one = 1;
      continue;
    }
    if (!strcmp(arg, "--no-graph")) {
      *graph = 0;
      continue;
    }
    if (!is_opt(arg)) {
      fprintf(stderr, "Warning: unrecognised command line option `%s'\n", arg);
      continue;
    }
    if (!strcmp(arg, "--")) break;
    char *val = NULL, *eq = strchr(arg, '=');
    char name[64];
    size_t nl = eq ? (size_t) (eq - arg) : strlen(arg);
    if (nl >= sizeof name) {
      fprintf(stderr, "Warning: unrecognised command line option `%s'\n", arg);
      continue;
    }
    memcpy(name, arg, nl);
    name[nl] = '\0';
    if (eq) val = eq + 1;
    else if (i + 1 < argc && !is_opt(argv[i + 1])) val = argv[++i];
    const int lng = (name[1] == '-');
    if ((!lng && name[1] == 'h') || (lng && !strcmp(name + 2, "help"))) usage();
    if ((!lng && name[1] == 'V') || (lng && !strcmp(name + 2, "version")))
      version();
    if ((!lng && name[1] == 't') || (lng && !strcmp(name + 2, "template")))
      conf_template();
    const option_t *o = NULL;
    for (int k = 0; k < NOPT && !o; k++)
      if (lng ? !strcmp(name + 2, OPTIONS[k].lopt)
              : (OPTIONS[k].sopt && name[1] == OPTIONS[k].sopt))
        o = OPTIONS + k;
    if (!o) {
      fprintf(stderr, "Warning: unrecognised command line option `%s'\n", name);
      continue;
    }
    if (!val || !*val) {
      if (!o->is_bool) die("argument not found for option `%s'", name);
      val = "T";
    }
    char *copy = strdup(val);
    conf_add(C, o->key, copy, PRIO_CMD);
    free(copy);
  }
}

