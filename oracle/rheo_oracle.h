/*
 * rheo_oracle.h -- CPU restatement of MDOODZ7.0's local rheology update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the GPU library is
 * compared against; only tests/, the smoke check and the CPU-baseline leg of
 * bench.py may load it.  The product library never links or calls it.
 *
 * It restates, in plain C and in the reference's floating-point evaluation
 * order, MDLIB/RheologyDensity.c:116-1426 and MDLIB/AnisotropyRoutines.c:
 * 257-727, 885-1217, MDLIB/StokesRoutines.c:75-410 with MDLIB/FD_Jacobian.c:48-323,
 * StrainRateComponents (MDLIB/RheologyDensity.c:2001-2097), Softening /
 * CohesionFrictionDilationGrid and ShearModCompExpGrid (:1432-1755),
 * UpdateParticleStress (MDLIB/RheologyParticles.c:1725-2004), plus
 * InterpCentroidsToVerticesDouble (MDLIB/GridRoutines.c:108-210).  Built with
 * -ffp-contract=off it is bit-identical to the reference compiled from its own sources on x86-64
 * (pinned by tests/test_oracle_vs_reference.py and the committed golden
 * fixtures).  Unlike the reference it never calls exit(): errors come back as
 * MDZ_* status codes, and it also reports local iteration counts.
 *
 * The interface uses the same plain-pointer structs as include/mdz_rheo.h so
 * one set of test buffers feeds both.
 */
#ifndef MDZ_RHEO_ORACLE_H
#define MDZ_RHEO_ORACLE_H
#include "../include/mdz_rheo.h"

#ifdef __cplusplus
extern "C" {
#endif

/* NonNewtonianViscosityGrid (RheologyDensity.c:1131).  iters_n/iters_s
 * (may be NULL) receive per-(phase,node) VE iteration counts, laid out
 * [p*Nc + c0] / [p*Nv + c1].  Returns the first status met. */
int orc_sweep(const mdz_model *model, const mdz_materials *mat, const mdz_grid_fields *f,
              int final_update, int32_t *iters_n, int32_t *iters_s, mdz_sweep_stats *stats);

/* NonNewtonianViscosityGridAniso (AnisotropyRoutines.c:885). */
int orc_sweep_aniso(const mdz_model *model, const mdz_materials *mat, const mdz_grid_fields *f,
                    int final_update, int32_t *iters_n, int32_t *iters_s, mdz_sweep_stats *stats);

/* ViscosityConcise / ViscosityConciseAniso on n independent points. */
int orc_points(const mdz_model *model, const mdz_materials *mat, const mdz_point_inputs *in,
               mdz_point_outputs *out, int64_t n, int aniso);

/* RheologicalOperators (StokesRoutines.c:75-410), finite-difference derivatives of
 * DerivativesOnTheFly_n/_s (FD_Jacobian.c:48-323) when jacobian = 1. */
int orc_operators(const mdz_model *model, const mdz_materials *mat, const mdz_grid_fields *f,
                  mdz_operator_fields *ops, int jacobian, int compressible, int aniso);

/* StrainRateComponents (RheologyDensity.c:2001-2097). */
int orc_strain_rates(const mdz_model *model, double dx, double dz, int out_of_plane, double compressible,
                     mdz_strain_rate_fields *sr);

/* CohesionFrictionDilationGrid (RheologyDensity.c:1539-1628) after its P2Mastah step:
 * Softening (:1432-1532) of every node from f->strain_pl_n/_s. */
int orc_softening(const mdz_model *model, const mdz_prep_materials *mat, mdz_prep_fields *f, int smooth_softening,
                  int hardening_modulus, int marker_noise);

/* ShearModCompExpGrid (RheologyDensity.c:1634-1755); MDZ_ESHEAR_INF where the
 * reference exits with code 32. */
int orc_shear_modulus(const mdz_model *model, const mdz_prep_materials *mat, mdz_prep_fields *f);

/* UpdateParticleStress (RheologyParticles.c:1725-2004), subgrid_diffusion 0 or 1. */
int orc_marker_stress(const mdz_model *model, const mdz_marker_opts *opts, mdz_marker_grid *grid, mdz_markers *mk);
/* P2Mastah of a marker array (ParticleRoutines.c:2170-2665), serial order */
int orc_p2mastah(const mdz_model *m, const mdz_marker_grid *g, const mdz_markers *mk, const double *val, int avg,
                 int stencil, double *node_n, double *node_s);

/* InterpCentroidsToVerticesDouble (GridRoutines.c:108) alone. */
void orc_interp_c2v(const mdz_model *model, const double *centroid, const signed char *BCp_type,
                    const signed char *BCg_type, double *vertex);

/* Number of OpenMP threads the oracle uses (for timing reports). */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
