/* Empty stand-in for SuiteSparse umfpack.h: the oracle build compiles
 * StokesRoutines.c for RheologicalOperators only, which uses no UMFPACK symbol. */
