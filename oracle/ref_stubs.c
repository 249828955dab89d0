/* Empty definitions for the MDOODZ7.0 symbols that the compiled rheology
 * sources reference but never reach on the local-rheology path with
 * melting=0 and no HDF5 output, and for the Stokes solvers that the other
 * routines of StokesRoutines.c call (oracle/_ref only; RheologicalOperators
 * reaches none of them).  Deliberately compiled without the MDOODZ headers so
 * their prototypes do not apply. */
void AddFieldToGroup(void) {}
void AddGroupToHDF5(void) {}
void CreateOutputHDF5(void) {}
void isoutPart(void) {}
void PartialMelting(void) {}
void ScaleBackD(void) {}
void BuildStokesOperatorDecoupled(void) {}
void DirectStokesDecoupled(void) {}
void DirectStokesDecoupledComp(void) {}
void KSPStokesDecoupled(void) {}
void KillerSolver(void) {}
