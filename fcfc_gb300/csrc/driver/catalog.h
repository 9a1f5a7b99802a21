/*
 * catalog.h -- ASCII catalogue and two-column table reading for the command
 * line drivers (see catalog.c).
 */
#ifndef FCFCG_CATALOG_H
#define FCFCG_CATALOG_H

#include <stddef.h>

/* Read a catalogue: xyz[0..2] and *w (NULL without wexpr) are malloc'ed
 * arrays of *num rows.  comment 0: none.  Returns 0, or -1 with a message. */
int cat_read_ascii(const char *fname, const char *fmtr,
    const char *const pos[3], const char *wexpr, const char *sel, long skip,
    char comment, double **xyz, double **w, size_t *num, char *err,
    size_t errlen);

/* Two numbers per line ('#' lines and blank lines skipped). */
int cat_read_table(const char *fname, double **a, double **b, size_t *num,
    char *err, size_t errlen);

#endif
