/*
 * ref_harness.c -- drives the reference's own NonNewtonianViscosityGrid(Aniso),
 * ViscosityConcise(Aniso), RheologicalOperators, StrainRateComponents,
 * CohesionFrictionDilationGrid (with its marker interpolation), ShearModCompExpGrid and
 * UpdateParticleStress,
 * compiled from the MDOODZ7.0 sources, from the plain-pointer structs of
 * include/mdz_rheo.h.
 *
 * TEST INFRASTRUCTURE ONLY: it is built by oracle/Makefile (target `ref`)
 * into oracle/_ref/ when the reference tree is present, and is used to pin the
 * C restatement (rheo_oracle.c) and to generate the golden fixtures.
 *
 * It fills a zeroed `grid` (MDLIB/mdoodz-private.h:75-147) with the caller's
 * arrays, the identity index maps kp/lp/kn/ln that GridIndices builds
 * (MDLIB/GridRoutines.c:543-585), a `mat_prop` and a `params` with the fields
 * the path reads, and calls the reference.  The reference exits the process on
 * a local-solve failure, so callers only hand it inputs that converge.
 */
#include <stdlib.h>
#include <string.h>

#include "mdoodz-private.h"
#include "../include/mdz_rheo.h"
#include <omp.h>

static void fill_materials(mat_prop *mp, const mdz_materials *m) {
  memset(mp, 0, sizeof(*mp));
  mp->Nb_phases = m->Nb_phases;
  mp->R         = m->R;
  for (int p = 0; p < MDZ_MAX_PHASES; p++) {
#define CP(name) mp->name[p] = m->name[p]
    CP(cstv); CP(pwlv); CP(linv); CP(gbsv); CP(expv); CP(gs); CP(kin); CP(plast); CP(density_model);
    CP(phase_mix); CP(phase_two); CP(reac_soft); CP(reac_phase); CP(melt);
    CP(eta0); CP(rho); CP(drho); CP(alp); CP(bet); CP(T0); CP(P0); CP(Slim); CP(eta_vp); CP(n_vp);
    CP(T_st); CP(gs_ref);
    CP(Qpwl); CP(Vpwl); CP(npwl); CP(mpwl); CP(rpwl); CP(Apwl); CP(fpwl); CP(apwl); CP(Fpwl); CP(pref_pwl);
    CP(Qlin); CP(Vlin); CP(nlin); CP(mlin); CP(rlin); CP(Alin); CP(flin); CP(alin); CP(Flin);
    CP(Qgbs); CP(Vgbs); CP(ngbs); CP(mgbs); CP(rgbs); CP(Agbs); CP(fgbs); CP(agbs); CP(Fgbs);
    CP(Qexp); CP(Sexp); CP(Eexp); CP(Gexp); CP(nexp);
    CP(Kpzm); CP(Qpzm); CP(Gpzm); CP(Lpzm); CP(cpzm); CP(ppzm);
#undef CP
  }
}

static void fill_params(params *pm, scale *sc, const mdz_model *m) {
  memset(pm, 0, sizeof(*pm));
  memset(sc, 0, sizeof(*sc));
  pm->Nx = m->Nx; pm->Nz = m->Nz; pm->Nb_phases = m->Nb_phases;
  pm->step = m->step; pm->elastic = m->elastic; pm->eta_average = m->eta_average;
  pm->periodic_x = m->periodic_x; pm->density_variations = m->density_variations;
  pm->tensile_line_search = m->tensile_line_search; pm->melting = m->melting;
  pm->chemical_production = m->chemical_production; pm->diffuse_X = m->diffuse_X;
  pm->diffuse_avg = m->diffuse_avg; pm->dt = m->dt; pm->min_eta = m->min_eta;
  pm->max_eta = m->max_eta; pm->eta_tol = m->eta_tol;
  sc->eta = m->scale_eta; sc->L = m->scale_L; sc->T = m->scale_T; sc->S = m->scale_S; sc->E = m->scale_E;
}

static void quiet_log(void) {
  static int done = 0;
  if (done) return;
  MdoodzLogConfig cfg = {MDOODZ_LOG_CONSOLE, MDOODZ_LOG_ERROR, 0, MDOODZ_TS_RELATIVE, 0, NULL};
  mdoodz_log_init(&cfg);
  done = 1;
}

#define W(x) ((double *)(x))

/* A zeroed `grid` over the caller's arrays, with the identity index maps. */
static grid *make_grid(const mdz_model *m, const mdz_grid_fields *f) {
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1, Nc = Ncx * Ncz, Nv = Nx * Nz;
  grid *g = calloc(1, sizeof(grid));
  g->Nx = Nx; g->Nz = Nz;
  g->kp = malloc(sizeof(int) * Nc); g->lp = malloc(sizeof(int) * Nc);
  g->kn = malloc(sizeof(int) * Nv); g->ln = malloc(sizeof(int) * Nv);
  for (int i = 0; i < Nc; i++) { g->kp[i] = i % Ncx; g->lp[i] = i / Ncx; }
  for (int i = 0; i < Nv; i++) { g->kn[i] = i % Nx; g->ln[i] = i / Nx; }
  /* centroid inputs */
  g->mu_n = W(f->mu_n); g->T = W(f->T); g->p_in = W(f->p_in); g->d0_n = W(f->d0_n);
  g->phi0_n = W(f->phi0_n); g->X0_n = W(f->X0_n); g->exxd = W(f->exxd); g->ezzd = W(f->ezzd);
  g->exz_n = W(f->exz_n); g->sxxd0 = W(f->sxxd0); g->szzd0 = W(f->szzd0); g->sxz0_n = W(f->sxz0_n);
  g->strain_n = W(f->strain_n); g->dil_n = W(f->dil_n); g->fric_n = W(f->fric_n); g->C_n = W(f->C_n);
  g->p0_n = W(f->p0_n); g->T0_n = W(f->T0_n); g->bet_n = W(f->bet_n); g->div_u = W(f->div_u);
  g->phase_perc_n = (double **)f->phase_perc_n;
  g->BCp.type = (signed char *)f->BCp_type;
  /* vertex inputs */
  g->mu_s = W(f->mu_s); g->X0_s = W(f->X0_s); g->exxd_s = W(f->exxd_s); g->ezzd_s = W(f->ezzd_s);
  g->exz = W(f->exz); g->sxxd0_s = W(f->sxxd0_s); g->szzd0_s = W(f->szzd0_s); g->sxz0 = W(f->sxz0);
  g->strain_s = W(f->strain_s); g->dil_s = W(f->dil_s); g->fric_s = W(f->fric_s); g->C_s = W(f->C_s);
  g->p0_s = W(f->p0_s); g->bet_s = W(f->bet_s); g->div_u_s = W(f->div_u_s);
  g->phase_perc_s = (double **)f->phase_perc_s;
  g->BCg.type = (signed char *)f->BCg_type;
  /* anisotropy */
  g->d1_n = W(f->d1_n); g->d2_n = W(f->d2_n); g->angle_n = W(f->angle_n);
  g->aniso_factor_n = W(f->aniso_factor_n); g->d1_s = W(f->d1_s); g->d2_s = W(f->d2_s);
  g->angle_s = W(f->angle_s); g->aniso_factor_s = W(f->aniso_factor_s);
  /* interpolated + outputs */
  g->T_s = f->T_s; g->P_s = f->P_s; g->d0_s = f->d0_s; g->phi0_s = f->phi0_s;
  g->eta_n = f->eta_n; g->eta_phys_n = f->eta_phys_n; g->VE_n = f->VE_n; g->sxxd = f->sxxd;
  g->szzd = f->szzd; g->sxz_n = f->sxz_n; g->eII_el = f->eII_el; g->eII_pl = f->eII_pl;
  g->eII_pwl = f->eII_pwl; g->eII_exp = f->eII_exp; g->eII_lin = f->eII_lin; g->eII_gbs = f->eII_gbs;
  g->eII_cst = f->eII_cst; g->d_n = f->d_n; g->p_corr = f->p_corr; g->div_u_el = f->div_u_el;
  g->div_u_pl = f->div_u_pl; g->div_u_r = f->div_u_r; g->Wtot = f->Wtot; g->Wel = f->Wel;
  g->Wdiss = f->Wdiss; g->X_n = f->X_n; g->OverS_n = f->OverS_n; g->rho_n = f->rho_n;
  g->phase_eta_n = (double **)f->phase_eta_n;
  g->sxxd_s = f->sxxd_s; g->szzd_s = f->szzd_s; g->sxz = f->sxz; g->eta_phys_s = f->eta_phys_s;
  g->eta_s = f->eta_s; g->X_s = f->X_s; g->VE_s = f->VE_s;
  g->phase_eta_s = (double **)f->phase_eta_s;
  return g;
}

static void free_grid(grid *g) {
  free(g->kp); free(g->lp); free(g->kn); free(g->ln);
  free(g);
}

int ref_sweep(const mdz_model *m, const mdz_materials *mat, const mdz_grid_fields *f,
              int final_update, int aniso) {
  quiet_log();
  mat_prop *mp = malloc(sizeof(mat_prop));
  params pm;
  scale sc;
  Nparams np;
  memset(&np, 0, sizeof(np));
  fill_materials(mp, mat);
  fill_params(&pm, &sc, m);
  grid *g = make_grid(m, f);
  if (aniso) NonNewtonianViscosityGridAniso(g, mp, &pm, np, &sc, final_update);
  else       NonNewtonianViscosityGrid(g, mp, &pm, np, &sc, final_update);
  free_grid(g);
  free(mp);
  return 0;
}

/* RheologicalOperators (StokesRoutines.c:75) on the same kind of grid, writing `ops`.
 * The anisotropic Newton branch reads FS_AR_n / FS_AR_s without using them in the
 * coefficients; they are set to 1. */
int ref_operators(const mdz_model *m, const mdz_materials *mat, const mdz_grid_fields *f,
                  mdz_operator_fields *ops, int jacobian, int compressible, int aniso) {
  quiet_log();
  const int Nc = (m->Nx - 1) * (m->Nz - 1), Nv = m->Nx * m->Nz;
  mat_prop *mp = malloc(sizeof(mat_prop));
  params pm;
  scale sc;
  fill_materials(mp, mat);
  fill_params(&pm, &sc, m);
  pm.compressible = compressible;
  pm.anisotropy = aniso;
  grid *g = make_grid(m, f);
  g->D11_n = ops->D11_n; g->D12_n = ops->D12_n; g->D13_n = ops->D13_n; g->D14_n = ops->D14_n;
  g->D21_n = ops->D21_n; g->D22_n = ops->D22_n; g->D23_n = ops->D23_n; g->D24_n = ops->D24_n;
  g->D31_s = ops->D31_s; g->D32_s = ops->D32_s; g->D33_s = ops->D33_s; g->D34_s = ops->D34_s;
  g->drhodp_n = ops->drhodp_n;
  g->FS_AR_n = malloc(sizeof(double) * Nc);
  g->FS_AR_s = malloc(sizeof(double) * Nv);
  for (int i = 0; i < Nc; i++) g->FS_AR_n[i] = 1.0;
  for (int i = 0; i < Nv; i++) g->FS_AR_s[i] = 1.0;
  RheologicalOperators(g, &pm, mp, &sc, jacobian, aniso);
  free(g->FS_AR_n); free(g->FS_AR_s);
  free_grid(g);
  free(mp);
  return 0;
}

/* StrainRateComponents (RheologyDensity.c:2001) on a grid holding only the arrays it
 * touches. */
int ref_strain_rates(const mdz_model *m, double dx, double dz, int out_of_plane, double compressible,
                     mdz_strain_rate_fields *sr) {
  quiet_log();
  params pm;
  scale sc;
  fill_params(&pm, &sc, m);
  pm.out_of_plane = out_of_plane;
  pm.compressible = compressible;
  mdz_grid_fields none;
  memset(&none, 0, sizeof(none));
  grid *g = make_grid(m, &none);
  g->dx = dx; g->dz = dz;
  g->u_in = W(sr->u_in); g->v_in = W(sr->v_in);
  g->BCp.type = (signed char *)sr->BCp_type; g->BCg.type = (signed char *)sr->BCg_type;
  g->div_u = sr->div_u; g->exxd = sr->exxd; g->ezzd = sr->ezzd; g->exz_n = sr->exz_n; g->wxz_n = sr->wxz_n;
  g->exz = sr->exz; g->wxz = sr->wxz; g->exxd_s = sr->exxd_s; g->ezzd_s = sr->ezzd_s; g->div_u_s = sr->div_u_s;
  StrainRateComponents(g, sc, &pm);
  free_grid(g);
  return 0;
}

/* The mat_prop fields of Softening and ShearModCompExpGrid. */
static mat_prop *prep_materials(const mdz_prep_materials *m) {
  mat_prop *mp = calloc(1, sizeof(mat_prop));
  mp->Nb_phases = m->Nb_phases;
  for (int p = 0; p < MDZ_MAX_PHASES; p++) {
#define CP(name) mp->name[p] = m->name[p]
    CP(G); CP(bet); CP(alp); CP(C); CP(phi); CP(psi); CP(H_c); CP(C_end); CP(phi_end); CP(psi_end);
    CP(pls_start); CP(pls_end); CP(phi_soft); CP(psi_soft); CP(coh_soft);
#undef CP
  }
  return mp;
}

/* A grid with mesh spacing, node coordinates from (xmin, zmin) and the preparation
 * fields of `f`. */
static grid *prep_grid(const mdz_model *m, mdz_prep_fields *f, double xmin, double zmin, double dx, double dz) {
  mdz_grid_fields none;
  memset(&none, 0, sizeof(none));
  grid *g = make_grid(m, &none);
  const int Nx = m->Nx, Nz = m->Nz;
  g->dx = dx; g->dz = dz;
  g->xg_coord = malloc(sizeof(double) * Nx); g->zg_coord = malloc(sizeof(double) * Nz);
  g->xc_coord = malloc(sizeof(double) * (Nx - 1)); g->zc_coord = malloc(sizeof(double) * (Nz - 1));
  for (int k = 0; k < Nx; k++) g->xg_coord[k] = xmin + k * dx;
  for (int l = 0; l < Nz; l++) g->zg_coord[l] = zmin + l * dz;
  for (int k = 0; k < Nx - 1; k++) g->xc_coord[k] = xmin + 0.5 * dx + k * dx;
  for (int l = 0; l < Nz - 1; l++) g->zc_coord[l] = zmin + 0.5 * dz + l * dz;
  g->BCp.type = (signed char *)f->BCp_type; g->BCg.type = (signed char *)f->BCg_type;
  g->BCt.type = (signed char *)f->BCp_type;
  g->phase_perc_n = (double **)f->phase_perc_n; g->phase_perc_s = (double **)f->phase_perc_s;
  g->noise_n = W(f->noise_n); g->noise_s = W(f->noise_s);
  g->fric_n = f->fric_n; g->dil_n = f->dil_n; g->C_n = f->C_n;
  g->fric_s = f->fric_s; g->dil_s = f->dil_s; g->C_s = f->C_s;
  g->mu_n = f->mu_n; g->bet_n = f->bet_n; g->alp = f->alp; g->mu_s = f->mu_s; g->bet_s = f->bet_s;
  return g;
}

static void free_prep_grid(grid *g) {
  free(g->xg_coord); free(g->zg_coord); free(g->xc_coord); free(g->zc_coord);
  free_grid(g);
}

/* CohesionFrictionDilationGrid (RheologyDensity.c:1539) itself, markers included: its
 * P2Mastah interpolates the markers' plastic strain to centroids and vertices, then
 * Softening runs per node.  The same two P2Mastah calls (:1558, :1595) are repeated
 * here into strain_n / strain_s, the plastic strain the GPU path and the restatement
 * take as input. */
int ref_softening_markers(const mdz_model *m, const mdz_prep_materials *pmat, mdz_prep_fields *f, int64_t n_part,
                          const double *px, const double *pz, const int *pphase, const double *pstrain, double xmin,
                          double zmin, double dx, double dz, int interp_stencil, int smooth_softening,
                          int hardening_modulus, int marker_noise, double *strain_n, double *strain_s) {
  quiet_log();
  mat_prop *mp = prep_materials(pmat);
  params pm;
  scale sc;
  fill_params(&pm, &sc, m);
  pm.interp_stencil = interp_stencil;
  pm.smooth_softening = smooth_softening;
  pm.hardening_modulus = hardening_modulus;
  pm.marker_noise = marker_noise;
  grid *g = prep_grid(m, f, xmin, zmin, dx, dz);
  markers P;
  memset(&P, 0, sizeof(P));
  P.Nb_part = (int)n_part;
  P.x = (double *)px; P.z = (double *)pz; P.phase = (int *)pphase; P.strain_pl = (double *)pstrain;
  /* one OpenMP thread: P2Mastah's per-thread partial sums then run in marker order */
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);
  CohesionFrictionDilationGrid(g, &P, *mp, pm, sc);
  const int Nc = (m->Nx - 1) * (m->Nz - 1), Nv = m->Nx * m->Nz;
  memset(strain_n, 0, sizeof(double) * Nc);
  memset(strain_s, 0, sizeof(double) * Nv);
  P2Mastah(&pm, P, P.strain_pl, g, strain_n, (char *)g->BCp.type, 1, 0, 0, 1, pm.interp_stencil, NULL);
  P2Mastah(&pm, P, P.strain_pl, g, strain_s, (char *)g->BCg.type, 1, 0, 0, 0, pm.interp_stencil, NULL);
  omp_set_num_threads(threads);
  free_prep_grid(g);
  free(mp);
  return 0;
}

/* ShearModCompExpGrid (RheologyDensity.c:1634).  The reference exits on an infinite
 * centroid modulus, so callers only hand it inputs without one. */
int ref_shear_modulus(const mdz_model *m, const mdz_prep_materials *pmat, mdz_prep_fields *f) {
  quiet_log();
  mat_prop *mp = prep_materials(pmat);
  params pm;
  scale sc;
  fill_params(&pm, &sc, m);
  grid *g = prep_grid(m, f, 0.0, 0.0, 1.0, 1.0);
  ShearModCompExpGrid(g, mp, &pm, sc);
  free_prep_grid(g);
  free(mp);
  return 0;
}

/* UpdateParticleStress (RheologyParticles.c:1725) on a grid and marker set holding the
 * arrays it touches; the marker arrays are updated in place, wxz likewise. */
int ref_marker_stress(const mdz_model *m, const mdz_marker_opts *o, mdz_marker_grid *mg, mdz_markers *mk) {
  quiet_log();
  mat_prop *mp = calloc(1, sizeof(mat_prop));
  params pm;
  scale sc;
  fill_params(&pm, &sc, m);
  pm.dx = mg->dx; pm.dz = mg->dz;
  pm.elastic = o->elastic; pm.subgrid_diffusion = o->subgrid_diffusion; pm.stress_rotation = o->stress_rotation;
  pm.anisotropy = o->anisotropy; pm.advection = o->advection; pm.interp_stencil = o->interp_stencil;
  mdz_grid_fields none;
  memset(&none, 0, sizeof(none));
  grid *g = make_grid(m, &none);
  g->dx = mg->dx; g->dz = mg->dz;
  g->xg_coord = W(mg->xg_coord); g->zg_coord = W(mg->zg_coord);
  g->xvz_coord = W(mg->xvz_coord); g->zvx_coord = W(mg->zvx_coord);
  g->BCp.type = (signed char *)mg->BCp_type; g->BCg.type = (signed char *)mg->BCg_type;
  g->sxxd = W(mg->sxxd); g->szzd = W(mg->szzd); g->sxxd0 = W(mg->sxxd0); g->szzd0 = W(mg->szzd0);
  g->sxz = W(mg->sxz); g->sxz0 = W(mg->sxz0);
  g->u_in = W(mg->u_in); g->v_in = W(mg->v_in);
  g->wxz = mg->wxz;
  g->xc_coord = W(mg->xc_coord); g->zc_coord = W(mg->zc_coord);
  g->eta_phys_s = W(mg->eta_phys_s);
  if (o->G)
    for (int p = 0; p < m->Nb_phases && p < 20; p++) mp->G[p] = o->G[p];
  markers P;
  memset(&P, 0, sizeof(P));
  P.Nb_part = (int)mk->n;
  P.x = (double *)mk->x; P.z = (double *)mk->z; P.phase = (int *)mk->phase;
  P.sxxd = mk->sxxd; P.szzd = mk->szzd; P.sxz = mk->sxz; P.nx = mk->nx; P.nz = mk->nz;
  /* one thread: P2Mastah's sums (subgrid diffusion 2) then run in marker order, the
   * order the restatement sums in; with more threads the reference's own result moves
   * in the last bits with the thread count */
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);
  UpdateParticleStress(g, &P, &pm, mp, &sc);
  omp_set_num_threads(threads);
  free_grid(g);
  free(mp);
  return 0;
}

/* The reference's P2Mastah (flag 1, prop 0) of a marker array onto the centroids and/or
 * vertices, on one OpenMP thread (its per-thread partial sums then run in marker order). */
int ref_p2mastah(const mdz_model *m, const mdz_marker_grid *mg, const mdz_markers *mk, const double *val, int avg,
                 int stencil, double *node_n, double *node_s) {
  quiet_log();
  params pm;
  scale sc;
  fill_params(&pm, &sc, m);
  pm.dx = mg->dx; pm.dz = mg->dz; pm.interp_stencil = stencil;
  mdz_grid_fields none;
  memset(&none, 0, sizeof(none));
  grid *g = make_grid(m, &none);
  g->dx = mg->dx; g->dz = mg->dz;
  g->xg_coord = W(mg->xg_coord); g->zg_coord = W(mg->zg_coord);
  g->xc_coord = W(mg->xc_coord); g->zc_coord = W(mg->zc_coord);
  markers P;
  memset(&P, 0, sizeof(P));
  P.Nb_part = (int)mk->n;
  P.x = (double *)mk->x; P.z = (double *)mk->z; P.phase = (int *)mk->phase;
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);
  if (node_n) P2Mastah(&pm, P, (double *)val, g, node_n, (char *)mg->BCp_type, 1, avg, 0, 1, stencil, NULL);
  if (node_s) P2Mastah(&pm, P, (double *)val, g, node_s, (char *)mg->BCg_type, 1, avg, 0, 0, stencil, NULL);
  omp_set_num_threads(threads);
  free_grid(g);
  return 0;
}

int ref_points(const mdz_model *m, const mdz_materials *mat, const mdz_point_inputs *in,
               mdz_point_outputs *out, int64_t n, int aniso) {
  quiet_log();
  mat_prop *mp = malloc(sizeof(mat_prop));
  params pm;
  scale sc;
  fill_materials(mp, mat);
  fill_params(&pm, &sc, m);
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) {
    double r[24];
    double eta;
    if (aniso) {
      /* eta_vep takes the etaVE slot; VEcoeff stays 0 */
      r[5] = 0.0;
      eta = ViscosityConciseAniso(in->phase[i], in->lxlz[i], in->lx2[i], in->angle[i], in->ani_fac[i],
                                  in->G[i], in->T[i], in->P[i], in->d[i], in->phi[i], in->X0[i],
                                  in->Exx[i], in->Ezz[i], in->Exz[i], in->Txx0[i], in->Tzz0[i],
                                  in->Txz0[i], mp, &pm, &sc, &r[1], &r[2], &r[3], &r[4], &r[6],
                                  &r[7], &r[8], &r[9], &r[10], &r[11], &r[12], &r[13],
                                  in->strain_acc[i], in->dil[i], in->fric[i], in->C[i], in->P0[i],
                                  in->T0[i], &r[14], &r[15], &r[16], &r[17], in->beta[i], in->div[i],
                                  &r[18], &r[19], &r[20], &r[21], &r[22], &r[23], in->post_process,
                                  in->centroid, in->final_update, (int)i);
    } else {
      eta = ViscosityConcise(in->phase[i], in->G[i], in->T[i], in->P[i], in->d[i], in->phi[i],
                             in->X0[i], in->Exx[i], in->Ezz[i], in->Exz[i], in->Txx0[i], in->Tzz0[i],
                             in->Txz0[i], mp, &pm, &sc, &r[1], &r[2], &r[3], &r[4], &r[5], &r[6],
                             &r[7], &r[8], &r[9], &r[10], &r[11], &r[12], &r[13], in->strain_acc[i],
                             in->dil[i], in->fric[i], in->C[i], in->P0[i], in->T0[i], &r[14], &r[15],
                             &r[16], &r[17], in->beta[i], in->div[i], &r[18], &r[19], &r[20], &r[21],
                             &r[22], &r[23], in->post_process, in->centroid, in->final_update, (int)i);
    }
    r[0] = eta;
    double *dst[24] = {out->eta, out->Txx, out->Tzz, out->Txz, out->etaVE, out->VEcoeff, out->Eii_el,
                       out->Eii_pl, out->Eii_pwl, out->Eii_exp, out->Eii_lin, out->Eii_gbs,
                       out->Eii_cst, out->d1, out->X1, out->OverS, out->Pcorr, out->rho,
                       out->div_el, out->div_pl, out->div_r, out->Wtot, out->Wel, out->Wdiss};
    for (int j = 0; j < 24; j++) if (dst[j]) dst[j][i] = r[j];
  }
  free(mp);
  return 0;
}
