/* Empty stand-in for SuiteSparse amd.h (see umfpack.h). */
