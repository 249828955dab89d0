/*
 * shim_backend.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU stand-in for the context, sweep, operator, strain-rate, preparation and marker
 * entry points of libmdz_rheo_gb300.so (include/mdz_rheo.h) that forwards every call to
 * the C restatement (rheo_oracle.c).  Linked with the MDOODZ-side drop-in
 * (mdoodz7.0_gb300/host/mdz_rheo_mdoodz.c) and with the reference's own sources
 * into oracle/_ref/libmdz_shimtest.so, it lets a CPU test run the drop-in's
 * NonNewtonianViscosityGrid(Aniso), RheologicalOperators and StrainRateComponents
 * on a real `grid` and compare them with the reference's, which checks how the
 * drop-in unpacks grid / mat_prop / params / scale.  The GPU library itself is never part of this build.
 */
#include <stdlib.h>

#include "../include/mdz_rheo.h"
#include "rheo_oracle.h"

struct mdz_rheo_ctx {
  int device;
};

int mdz_rheo_create(int device, mdz_rheo_ctx **out) {
  if (!out) return MDZ_EINVAL;
  *out = (mdz_rheo_ctx *)calloc(1, sizeof(mdz_rheo_ctx));
  if (!*out) return MDZ_ENOMEM;
  (*out)->device = device;
  return MDZ_OK;
}

int mdz_rheo_destroy(mdz_rheo_ctx *ctx) {
  free(ctx);
  return MDZ_OK;
}

const char *mdz_rheo_status_string(int status) { return status == MDZ_OK ? "ok" : "error"; }

int mdz_rheo_sweep(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat, const mdz_grid_fields *f,
                   int final_update, int mem, int flags, mdz_sweep_stats *stats) {
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_sweep(model, mat, f, final_update, NULL, NULL, stats);
}

int mdz_rheo_sweep_aniso(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                         const mdz_grid_fields *f, int final_update, int mem, int flags, mdz_sweep_stats *stats) {
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_sweep_aniso(model, mat, f, final_update, NULL, NULL, stats);
}

int mdz_rheo_operators(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat, const mdz_grid_fields *f,
                       mdz_operator_fields *ops, int jacobian, int compressible, int aniso, int mem, int flags,
                       mdz_sweep_stats *stats) {
  (void)stats;
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_operators(model, mat, f, ops, jacobian, compressible, aniso);
}

int mdz_rheo_strain_rates(mdz_rheo_ctx *ctx, const mdz_model *model, double dx, double dz, int out_of_plane,
                          double compressible, mdz_strain_rate_fields *sr, int mem, int flags,
                          mdz_sweep_stats *stats) {
  (void)stats;
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_strain_rates(model, dx, dz, out_of_plane, compressible, sr);
}

int mdz_rheo_softening(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_prep_materials *mat, mdz_prep_fields *f,
                       int smooth_softening, int hardening_modulus, int marker_noise, int mem, int flags,
                       mdz_sweep_stats *stats) {
  (void)stats;
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_softening(model, mat, f, smooth_softening, hardening_modulus, marker_noise);
}

int mdz_rheo_shear_modulus(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_prep_materials *mat,
                           mdz_prep_fields *f, int mem, int flags, mdz_sweep_stats *stats) {
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_shear_modulus(model, mat, f);
}

int mdz_rheo_p2mastah(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_marker_grid *grid,
                      const mdz_markers *markers, const double *values, int avg, int interp_stencil,
                      double *node_n, double *node_s, int mem, int flags, mdz_sweep_stats *stats) {
  (void)stats;
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_p2mastah(model, grid, markers, values, avg, interp_stencil, node_n, node_s);
}

int mdz_rheo_marker_stress(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_marker_opts *opts,
                           mdz_marker_grid *grid, mdz_markers *markers, int mem, int flags, mdz_sweep_stats *stats) {
  (void)stats;
  if (!ctx || mem != MDZ_MEM_HOST || flags != 0) return MDZ_EINVAL;
  return orc_marker_stress(model, opts, grid, markers);
}
