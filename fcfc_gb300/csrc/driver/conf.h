/*
 * conf.h -- configuration of the command line drivers: FCFC's keys from a
 * file and from FCFC's command line options, with libcfg's priorities, and
 * FCFC's checks of the output files.
 */
#ifndef FCFCG_DRIVER_CONF_H
#define FCFCG_DRIVER_CONF_H

#ifdef FCFCG_SURVEY
#define PROG "FCFC_2PT_GPU"
#define DEFAULT_CONF "fcfc_2pt.conf"   /* src/fcfc/2pt/define.h:112 */
#else
#define PROG "FCFC_2PT_BOX_GPU"
#define DEFAULT_CONF "fcfc_2pt_box.conf"   /* src/fcfc/2pt_box/define.h:110 */
#endif

/* Configuration: KEY = value | [v1, v2, ...]; '#' comments outside quotes;  */
/* a trailing '\' joins lines; values may be quoted with ' or ".            */

typedef struct {
  char *key;
  int n;          /* number of values (1 for a scalar) */
  char **v;
  int prio;       /* PRIO_FILE or PRIO_CMD */
} entry_t;

/* As FCFC's configuration reader (libcfg, with FCFC's priorities in
 * src/util/define_comm.h:143-144): a command line value beats the file's,
 * and within one source the first value of a key is kept. */
#define PRIO_FILE 1
#define PRIO_CMD 5

typedef struct {
  entry_t *e;
  int n, cap;
} conf_t;

/* "Error: ..." on stderr, exit status 1 */
void die(const char *fmt, ...) __attribute__((noreturn, format(printf, 1, 2)));

/* Add KEY = val (val is modified); a second value of a key at the same
 * priority is reported and dropped. */
void conf_add(conf_t *C, const char *key, char *val, int prio);
/* KEY = value lines of a file (PRIO_FILE); dies if it cannot be read */
void conf_read(conf_t *C, const char *fname);
/* the entry of a key with the highest priority (the first among equals) */
const entry_t *conf_get(const conf_t *C, const char *key);
/* the i-th value, a single value broadcast, or NULL */
const char *conf_str(const conf_t *C, const char *key, int i);
int conf_len(const conf_t *C, const char *key);
double conf_dbl(const conf_t *C, const char *key, double def);
long conf_long(const conf_t *C, const char *key, int i, long def);
int is_true(const char *s);

/* FCFC's command line options into C (PRIO_CMD); -h, -V and -t print and
 * exit.  The engine's own flags (--fp64, --with-mu-one, --no-graph) are
 * returned through the pointers. */
void conf_parse_args(conf_t *C, int argc, char **argv, int *fp64,
    int *mu_one, int *graph);

/* FCFC's check_output: 0 to write the file, 1 to read it back; dies on
 * FCFC's refusals.  force: 2 for PAIR_COUNT_FILE, 1 for the correlation
 * function outputs. */
int check_output(const char *fname, const char *key, int ovw, int force);

#endif
