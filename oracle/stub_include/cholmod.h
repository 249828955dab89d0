/* Minimal stand-in for SuiteSparse's cholmod.h so that MDOODZ7.0's headers
 * parse when only the local-rheology sources are compiled (oracle/_ref).
 * None of these types is used on the rheology path. */
#ifndef MDZ_ORACLE_STUB_CHOLMOD_H
#define MDZ_ORACLE_STUB_CHOLMOD_H
typedef struct { int unused; } cholmod_common;
typedef struct mdz_stub_cholmod_factor cholmod_factor;
typedef struct mdz_stub_cholmod_dense cholmod_dense;
typedef struct mdz_stub_cholmod_sparse cholmod_sparse;
#endif
