/* Empty definitions for the MDOODZ7.0 symbols that the compiled rheology
 * sources reference but never reach on the local-rheology path with
 * melting=0 and no HDF5 output (oracle/_ref only).  Deliberately compiled
 * without the MDOODZ headers so their prototypes do not apply. */
void AddFieldToGroup(void) {}
void AddGroupToHDF5(void) {}
void ApplyBC(void) {}
void CreateOutputHDF5(void) {}
void P2Mastah(void) {}
void PartialMelting(void) {}
void ScaleBackD(void) {}
