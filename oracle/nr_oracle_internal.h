/* Helpers shared by nr_oracle.c and nr_oracle_mesh.c (test infrastructure,
 * see nr_oracle.h). */
#ifndef NR_ORACLE_INTERNAL_H
#define NR_ORACLE_INTERNAL_H

#include <stdio.h>

/* Line reader with std::getline / istream::eof semantics. */
typedef struct {
    FILE *f;
    int eof;
    char *buf;
    size_t cap;
} or_lines;

const char *or_getline(or_lines *r);

#endif
