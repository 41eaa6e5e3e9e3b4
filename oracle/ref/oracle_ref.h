/* Test infrastructure: shared declarations of the reference-ngspice oracle
 * driver (glue.c, driver.c).  Not part of the product. */
#ifndef ORACLE_REF_H
#define ORACLE_REF_H

typedef struct oracle_trace {
    int nvars;          /* number of unknowns reported by CKTdump */
    char **names;       /* unknown names, in equation order 1..n */
    int npoints;        /* accepted time points recorded */
    int cap;
    double *times;      /* [npoints] */
    double *values;     /* [npoints][nvars] */
} oracle_trace_t;

extern oracle_trace_t oracle_trace;
void oracle_init(void);

/* von47.c: appends every BSIM4v7 instance's von to (*buf)[nv..], growing
 * the buffer (capacity *cap) as needed; returns the new count.  The
 * argument is a CKTcircuit *. */
int oracle_v47_von(void *ckt, double **buf, int *cap, int nv);

#endif
