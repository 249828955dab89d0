/* Minimal stand-in for SuiteSparse's cs.h (see cholmod.h beside it). */
#ifndef MDZ_ORACLE_STUB_CS_H
#define MDZ_ORACLE_STUB_CS_H
typedef struct mdz_stub_cs { int nzmax, m, n; int *p, *i; double *x; int nz; } cs_di;
typedef cs_di cs;
#endif
