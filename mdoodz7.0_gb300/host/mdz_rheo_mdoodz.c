/*
 * mdz_rheo_mdoodz.c -- the MDOODZ7.0-side drop-in: NonNewtonianViscosityGrid,
 * NonNewtonianViscosityGridAniso, RheologicalOperators, StrainRateComponents,
 * CohesionFrictionDilationGrid, ShearModCompExpGrid and UpdateParticleStress with the
 * reference's own signatures (MDLIB/mdoodz-private.h:423, :437, :607, :426, :417, :416
 * and :415), evaluated on the GPU by libmdz_rheo_gb300.so through the C ABI of
 * include/mdz_rheo.h.
 *
 * It is compiled inside the MDOODZ build, against MDLIB/mdoodz-private.h, in place of
 * the definitions at MDLIB/RheologyDensity.c:1131, :1539, :1634, :2001,
 * MDLIB/AnisotropyRoutines.c:885, MDLIB/StokesRoutines.c:75 and
 * MDLIB/RheologyParticles.c:1725 (those are compiled out under MDZ_RHEO_GB300).
 * Each call unpacks `grid`, `mat_prop`, `params` and `scale` into the library's
 * plain-pointer structs and runs one sweep on host memory: the library uploads the
 * inputs, runs the kernel and writes every output back into the caller's arrays in
 * place, as the reference does (including the vertex fields T_s, P_s, d0_s, phi0_s).
 *
 * Errors: where the reference logs and calls exit() from inside the local solve,
 * the library returns a status; this file logs the reference's message for it and
 * exits with the reference's code (RheologyDensity.c:175-177, :312-315, :839-841,
 * :1045-1050, :1274-1301; AnisotropyRoutines.c:543, :580-583).
 *
 * One library context per process, created on first use on the device named by the
 * environment variable MDZ_RHEO_DEVICE (default 0).  Like the reference, the calls
 * are blocking and are made from one host thread.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mdoodz-private.h"
#include "mdz_rheo.h"

static mdz_rheo_ctx *s_ctx = NULL;

static mdz_rheo_ctx *mdz_context(void) {
  if (s_ctx == NULL) {
    const char *dev = getenv("MDZ_RHEO_DEVICE");
    const int rc = mdz_rheo_create(dev ? atoi(dev) : 0, &s_ctx);
    if (rc != MDZ_OK) {
      fprintf(stderr, "GB300 rheology: cannot open the device context (%s)\n", mdz_rheo_status_string(rc));
      exit(1);
    }
  }
  return s_ctx;
}

static void mdz_model_from(mdz_model *md, const grid *mesh, const params *model, const scale *scaling) {
  memset(md, 0, sizeof(*md));
  md->Nx = mesh->Nx;
  md->Nz = mesh->Nz;
  md->Nb_phases = model->Nb_phases;
  md->step = model->step;
  md->elastic = model->elastic;
  md->eta_average = model->eta_average;
  md->periodic_x = model->periodic_x;
  md->density_variations = model->density_variations;
  md->tensile_line_search = model->tensile_line_search;
  md->melting = model->melting;
  md->chemical_production = model->chemical_production;
  md->diffuse_X = model->diffuse_X;
  md->diffuse_avg = model->diffuse_avg;
  md->dt = model->dt;
  md->min_eta = model->min_eta;
  md->max_eta = model->max_eta;
  md->eta_tol = model->eta_tol;
  md->scale_eta = scaling->eta;
  md->scale_L = scaling->L;
  md->scale_T = scaling->T;
  md->scale_S = scaling->S;
  md->scale_E = scaling->E;
}

static void mdz_materials_from(mdz_materials *m, const mat_prop *mp) {
  memset(m, 0, sizeof(*m));
  m->Nb_phases = mp->Nb_phases;
  m->R = mp->R;
  for (int p = 0; p < MDZ_MAX_PHASES; p++) {
#define MDZ_COPY(name) m->name[p] = mp->name[p]
    MDZ_COPY(cstv); MDZ_COPY(pwlv); MDZ_COPY(linv); MDZ_COPY(gbsv); MDZ_COPY(expv); MDZ_COPY(gs);
    MDZ_COPY(kin); MDZ_COPY(plast); MDZ_COPY(density_model); MDZ_COPY(phase_mix); MDZ_COPY(phase_two);
    MDZ_COPY(reac_soft); MDZ_COPY(reac_phase); MDZ_COPY(melt);
    MDZ_COPY(eta0); MDZ_COPY(rho); MDZ_COPY(drho); MDZ_COPY(alp); MDZ_COPY(bet); MDZ_COPY(T0);
    MDZ_COPY(P0); MDZ_COPY(Slim); MDZ_COPY(eta_vp); MDZ_COPY(n_vp); MDZ_COPY(T_st); MDZ_COPY(gs_ref);
    MDZ_COPY(Qpwl); MDZ_COPY(Vpwl); MDZ_COPY(npwl); MDZ_COPY(mpwl); MDZ_COPY(rpwl); MDZ_COPY(Apwl);
    MDZ_COPY(fpwl); MDZ_COPY(apwl); MDZ_COPY(Fpwl); MDZ_COPY(pref_pwl);
    MDZ_COPY(Qlin); MDZ_COPY(Vlin); MDZ_COPY(nlin); MDZ_COPY(mlin); MDZ_COPY(rlin); MDZ_COPY(Alin);
    MDZ_COPY(flin); MDZ_COPY(alin); MDZ_COPY(Flin);
    MDZ_COPY(Qgbs); MDZ_COPY(Vgbs); MDZ_COPY(ngbs); MDZ_COPY(mgbs); MDZ_COPY(rgbs); MDZ_COPY(Agbs);
    MDZ_COPY(fgbs); MDZ_COPY(agbs); MDZ_COPY(Fgbs);
    MDZ_COPY(Qexp); MDZ_COPY(Sexp); MDZ_COPY(Eexp); MDZ_COPY(Gexp); MDZ_COPY(nexp);
    MDZ_COPY(Kpzm); MDZ_COPY(Qpzm); MDZ_COPY(Gpzm); MDZ_COPY(Lpzm); MDZ_COPY(cpzm); MDZ_COPY(ppzm);
#undef MDZ_COPY
  }
}

static void mdz_fields_from(mdz_grid_fields *f, grid *g, int aniso) {
  memset(f, 0, sizeof(*f));
  /* centroid inputs */
  f->mu_n = g->mu_n; f->T = g->T; f->p_in = g->p_in; f->d0_n = g->d0_n; f->phi0_n = g->phi0_n;
  f->X0_n = g->X0_n; f->exxd = g->exxd; f->ezzd = g->ezzd; f->exz_n = g->exz_n; f->sxxd0 = g->sxxd0;
  f->szzd0 = g->szzd0; f->sxz0_n = g->sxz0_n; f->strain_n = g->strain_n; f->dil_n = g->dil_n;
  f->fric_n = g->fric_n; f->C_n = g->C_n; f->p0_n = g->p0_n; f->T0_n = g->T0_n; f->bet_n = g->bet_n;
  f->div_u = g->div_u;
  f->phase_perc_n = (const double *const *)g->phase_perc_n;
  f->BCp_type = g->BCp.type;
  /* vertex inputs */
  f->mu_s = g->mu_s; f->X0_s = g->X0_s; f->exxd_s = g->exxd_s; f->ezzd_s = g->ezzd_s; f->exz = g->exz;
  f->sxxd0_s = g->sxxd0_s; f->szzd0_s = g->szzd0_s; f->sxz0 = g->sxz0; f->strain_s = g->strain_s;
  f->dil_s = g->dil_s; f->fric_s = g->fric_s; f->C_s = g->C_s; f->p0_s = g->p0_s; f->bet_s = g->bet_s;
  f->div_u_s = g->div_u_s;
  f->phase_perc_s = (const double *const *)g->phase_perc_s;
  f->BCg_type = g->BCg.type;
  if (aniso) {
    f->d1_n = g->d1_n; f->d2_n = g->d2_n; f->angle_n = g->angle_n; f->aniso_factor_n = g->aniso_factor_n;
    f->d1_s = g->d1_s; f->d2_s = g->d2_s; f->angle_s = g->angle_s; f->aniso_factor_s = g->aniso_factor_s;
  }
  /* written: interpolated vertex fields and outputs */
  f->T_s = g->T_s; f->P_s = g->P_s; f->d0_s = g->d0_s; f->phi0_s = g->phi0_s;
  f->eta_n = g->eta_n; f->eta_phys_n = g->eta_phys_n; f->VE_n = g->VE_n; f->sxxd = g->sxxd;
  f->szzd = g->szzd; f->sxz_n = g->sxz_n; f->eII_el = g->eII_el; f->eII_pl = g->eII_pl;
  f->eII_pwl = g->eII_pwl; f->eII_exp = g->eII_exp; f->eII_lin = g->eII_lin; f->eII_gbs = g->eII_gbs;
  f->eII_cst = g->eII_cst; f->d_n = g->d_n; f->p_corr = g->p_corr; f->div_u_el = g->div_u_el;
  f->div_u_pl = g->div_u_pl; f->div_u_r = g->div_u_r; f->Wtot = g->Wtot; f->Wel = g->Wel;
  f->Wdiss = g->Wdiss; f->X_n = g->X_n; f->OverS_n = g->OverS_n; f->rho_n = g->rho_n;
  f->phase_eta_n = (double *const *)g->phase_eta_n;
  f->sxxd_s = g->sxxd_s; f->szzd_s = g->szzd_s; f->sxz = g->sxz; f->eta_phys_s = g->eta_phys_s;
  f->eta_s = g->eta_s; f->X_s = g->X_s; f->VE_s = aniso ? g->VE_s : NULL;
  f->phase_eta_s = (double *const *)g->phase_eta_s;
}

/* The reference's message and exit code for a failed sweep. */
static void mdz_fail(int rc, const mdz_sweep_stats *st) {
  int code = 1;
  const char *msg = mdz_rheo_status_string(rc);
  switch (rc) {
    case MDZ_EVE_ITER: msg = "Visco-Elastic iterations failed!"; code = 0; break;   /* :175-177 */
    case MDZ_EGSE_ITER: code = 346; break;                                         /* :312-315, :366-368 */
    case MDZ_EEMPTY_CELL: msg = "Cell went empty!!! Exiting..."; code = 345; break; /* :1274-1277 */
    case MDZ_ELINESEARCH: code = 0; break;                                         /* :868-872 */
    case MDZ_EANISO_ITER: code = 0; break;                                         /* Aniso :580-583 */
    default: code = 1; break;
  }
  fprintf(stderr, "%s (node %lld)\n", msg, (long long)st->error_node);
  exit(code);
}

static void mdz_sweep_grid(grid *mesh, mat_prop *materials, params *model, scale *scaling, int final_update,
                           int aniso) {
  mdz_model md;
  mdz_materials mt;
  mdz_grid_fields f;
  mdz_sweep_stats st;
  mdz_model_from(&md, mesh, model, scaling);
  mdz_materials_from(&mt, materials);
  mdz_fields_from(&f, mesh, aniso);
  memset(&st, 0, sizeof(st));
  const int rc = aniso ? mdz_rheo_sweep_aniso(mdz_context(), &md, &mt, &f, final_update, MDZ_MEM_HOST, 0, &st)
                       : mdz_rheo_sweep(mdz_context(), &md, &mt, &f, final_update, MDZ_MEM_HOST, 0, &st);
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

void NonNewtonianViscosityGrid(grid *mesh, mat_prop *materials, params *model, Nparams Nmodel, scale *scaling,
                               int final_update) {
  (void)Nmodel; /* passed by value and unused, as in the reference */
  mdz_sweep_grid(mesh, materials, model, scaling, final_update, 0);
  ApplySetGridDensityOverride(mesh, model); /* RheologyDensity.c:1425 */
}

/* RheologicalOperators (StokesRoutines.c:75): the D tensors, with the Newton operator's
 * finite-difference derivatives (FD_Jacobian.c) solved on the GPU. */
void RheologicalOperators(grid *mesh, params *model, mat_prop *materials, scale *scaling, int Jacobian,
                          int anisotropy) {
  mdz_model md;
  mdz_materials mt;
  mdz_grid_fields f;
  mdz_operator_fields ops;
  mdz_sweep_stats st;
  mdz_model_from(&md, mesh, model, scaling);
  mdz_materials_from(&mt, materials);
  mdz_fields_from(&f, mesh, anisotropy);
  ops.D11_n = mesh->D11_n; ops.D12_n = mesh->D12_n; ops.D13_n = mesh->D13_n; ops.D14_n = mesh->D14_n;
  ops.D21_n = mesh->D21_n; ops.D22_n = mesh->D22_n; ops.D23_n = mesh->D23_n; ops.D24_n = mesh->D24_n;
  ops.drhodp_n = mesh->drhodp_n;
  ops.D31_s = mesh->D31_s; ops.D32_s = mesh->D32_s; ops.D33_s = mesh->D33_s; ops.D34_s = mesh->D34_s;
  memset(&st, 0, sizeof(st));
  const int rc = mdz_rheo_operators(mdz_context(), &md, &mt, &f, &ops, Jacobian, (int)model->compressible,
                                    anisotropy, MDZ_MEM_HOST, 0, &st);
  if (rc == MDZ_ENONFINITE) { /* :375-376, by the value at the first such vertex */
    const int64_t v = st.error_node - (int64_t)(mesh->Nx - 1) * (mesh->Nz - 1);
    const int inf = v >= 0 && v < (int64_t)mesh->Nx * mesh->Nz && isinf(mesh->D34_s[v]);
    fprintf(stderr, inf ? "EXIT: D34 is INF!\n" : "EXIT: D34 is NAN!\n");
    exit(1);
  }
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

/* StrainRateComponents (RheologyDensity.c:2001): strain rates, spin and their vertex /
 * centroid interpolations from u_in, v_in, in one GPU launch.  `scaling` is unused, as
 * in the reference. */
void StrainRateComponents(grid *mesh, scale scaling, params *model) {
  (void)scaling;
  mdz_model md;
  mdz_strain_rate_fields sr;
  mdz_sweep_stats st;
  memset(&md, 0, sizeof(md));
  md.Nx = mesh->Nx; md.Nz = mesh->Nz; md.periodic_x = model->periodic_x;
  sr.u_in = mesh->u_in; sr.v_in = mesh->v_in;
  sr.BCp_type = mesh->BCp.type; sr.BCg_type = mesh->BCg.type;
  sr.div_u = mesh->div_u; sr.exxd = mesh->exxd; sr.ezzd = mesh->ezzd; sr.exz_n = mesh->exz_n;
  sr.wxz_n = mesh->wxz_n; sr.exz = mesh->exz; sr.wxz = mesh->wxz; sr.exxd_s = mesh->exxd_s;
  sr.ezzd_s = mesh->ezzd_s; sr.div_u_s = mesh->div_u_s;
  memset(&st, 0, sizeof(st));
  const int rc = mdz_rheo_strain_rates(mdz_context(), &md, mesh->dx, mesh->dz, model->out_of_plane,
                                       model->compressible, &sr, MDZ_MEM_HOST, 0, &st);
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

/* The mat_prop fields of the preparation steps. */
static void mdz_prep_materials_from(mdz_prep_materials *m, const mat_prop *mp, int nphases) {
  memset(m, 0, sizeof(*m));
  m->Nb_phases = nphases;
  for (int p = 0; p < MDZ_MAX_PHASES; p++) {
    m->G[p] = mp->G[p]; m->bet[p] = mp->bet[p]; m->alp[p] = mp->alp[p];
    m->C[p] = mp->C[p]; m->phi[p] = mp->phi[p]; m->psi[p] = mp->psi[p]; m->H_c[p] = mp->H_c[p];
    m->C_end[p] = mp->C_end[p]; m->phi_end[p] = mp->phi_end[p]; m->psi_end[p] = mp->psi_end[p];
    m->pls_start[p] = mp->pls_start[p]; m->pls_end[p] = mp->pls_end[p];
    m->phi_soft[p] = mp->phi_soft[p]; m->psi_soft[p] = mp->psi_soft[p]; m->coh_soft[p] = mp->coh_soft[p];
  }
}

static void mdz_prep_fields_from(mdz_prep_fields *f, grid *g) {
  memset(f, 0, sizeof(*f));
  f->phase_perc_n = (const double *const *)g->phase_perc_n;
  f->phase_perc_s = (const double *const *)g->phase_perc_s;
  f->BCp_type = g->BCp.type; f->BCg_type = g->BCg.type;
  f->noise_n = g->noise_n; f->noise_s = g->noise_s;
  f->fric_n = g->fric_n; f->dil_n = g->dil_n; f->C_n = g->C_n;
  f->fric_s = g->fric_s; f->dil_s = g->dil_s; f->C_s = g->C_s;
  f->mu_n = g->mu_n; f->bet_n = g->bet_n; f->alp = g->alp; f->mu_s = g->mu_s; f->bet_s = g->bet_s;
}

/* CohesionFrictionDilationGrid (RheologyDensity.c:1539): the markers' plastic strain is
 * interpolated to the centroids and vertices by the reference's own P2Mastah, exactly as
 * there (:1557-1558, :1594-1595); Softening of every node then runs on the GPU. */
void CohesionFrictionDilationGrid(grid *mesh, markers *particles, mat_prop materials, params model, scale scaling) {
  (void)scaling;
  mdz_model md;
  mdz_prep_materials pm;
  mdz_prep_fields f;
  mdz_sweep_stats st;
  double *strain_n = DoodzCalloc((model.Nx - 1) * (model.Nz - 1), sizeof(double));
  double *strain_s = DoodzCalloc(model.Nx * model.Nz, sizeof(double));
  memset(&md, 0, sizeof(md));
  md.Nx = mesh->Nx; md.Nz = mesh->Nz; md.Nb_phases = model.Nb_phases; md.periodic_x = model.periodic_x;
  /* the plastic strain on the centroids and vertices: the two P2Mastah calls of
   * RheologyDensity.c:1552-1553 (arithmetic, interpolated), on the GPU */
  mdz_marker_grid mg;
  mdz_markers mk;
  memset(&mg, 0, sizeof(mg));
  memset(&mk, 0, sizeof(mk));
  mg.dx = mesh->dx; mg.dz = mesh->dz;
  mg.xg_coord = mesh->xg_coord; mg.zg_coord = mesh->zg_coord;
  mg.xc_coord = mesh->xc_coord; mg.zc_coord = mesh->zc_coord;
  mg.BCp_type = mesh->BCp.type; mg.BCg_type = mesh->BCg.type;
  mk.n = particles->Nb_part;
  mk.x = particles->x; mk.z = particles->z; mk.phase = particles->phase;
  memset(&st, 0, sizeof(st));
  int rc = mdz_rheo_p2mastah(mdz_context(), &md, &mg, &mk, particles->strain_pl, 0, model.interp_stencil, strain_n,
                             strain_s, MDZ_MEM_HOST, 0, &st);
  if (rc != MDZ_OK) mdz_fail(rc, &st);
  mdz_prep_materials_from(&pm, &materials, model.Nb_phases);
  mdz_prep_fields_from(&f, mesh);
  f.strain_pl_n = strain_n; f.strain_pl_s = strain_s;
  memset(&st, 0, sizeof(st));
  rc = mdz_rheo_softening(mdz_context(), &md, &pm, &f, model.smooth_softening, model.hardening_modulus,
                          model.marker_noise, MDZ_MEM_HOST, 0, &st);
  DoodzFree(strain_n);
  DoodzFree(strain_s);
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

/* ShearModCompExpGrid (RheologyDensity.c:1634): harmonic phase averages of G and bet,
 * arithmetic alp, on the GPU.  An infinite centroid modulus gets the reference's message
 * and exit code 32 (:1688-1690). */
void ShearModCompExpGrid(grid *mesh, mat_prop *materials, params *model, scale scaling) {
  mdz_model md;
  mdz_prep_materials pm;
  mdz_prep_fields f;
  mdz_sweep_stats st;
  memset(&md, 0, sizeof(md));
  md.Nx = mesh->Nx; md.Nz = mesh->Nz; md.Nb_phases = model->Nb_phases; md.periodic_x = model->periodic_x;
  mdz_prep_materials_from(&pm, materials, model->Nb_phases);
  mdz_prep_fields_from(&f, mesh);
  memset(&st, 0, sizeof(st));
  const int rc = mdz_rheo_shear_modulus(mdz_context(), &md, &pm, &f, MDZ_MEM_HOST, 0, &st);
  if (rc == MDZ_ESHEAR_INF) {
    const int Ncx = mesh->Nx - 1, c0 = (int)st.error_node, k = c0 % Ncx, l = c0 / Ncx;
    fprintf(stderr, "%f x = %2.6e z = %2.6e - BCp %d BCt %d\n", mesh->mu_n[c0], mesh->xc_coord[k] * scaling.L,
            mesh->zc_coord[l] * scaling.L, mesh->BCp.type[c0], mesh->BCt.type[c0]);
    exit(32);
  }
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

/* UpdateParticleStress (RheologyParticles.c:1725): the markers' stress update from the
 * grid's stress change (with subgrid stress diffusion when subgrid_diffusion is 2), the
 * stress rotation and the director rotation, on the GPU. */
void UpdateParticleStress(grid *mesh, markers *particles, params *model, mat_prop *materials, scale *scaling) {
  (void)scaling;
  mdz_model md;
  mdz_marker_opts o;
  mdz_marker_grid g;
  mdz_markers mk;
  mdz_sweep_stats st;
  memset(&md, 0, sizeof(md));
  md.Nx = mesh->Nx; md.Nz = mesh->Nz; md.periodic_x = model->periodic_x; md.dt = model->dt;
  md.Nb_phases = model->Nb_phases;
  o.G = materials->G;
  o.elastic = model->elastic; o.subgrid_diffusion = model->subgrid_diffusion;
  o.stress_rotation = model->stress_rotation; o.anisotropy = model->anisotropy;
  o.advection = model->advection; o.interp_stencil = model->interp_stencil;
  g.dx = mesh->dx; g.dz = mesh->dz;
  g.xg_coord = mesh->xg_coord; g.zg_coord = mesh->zg_coord;
  g.xvz_coord = mesh->xvz_coord; g.zvx_coord = mesh->zvx_coord;
  g.BCp_type = mesh->BCp.type; g.BCg_type = mesh->BCg.type;
  g.sxxd = mesh->sxxd; g.szzd = mesh->szzd; g.sxxd0 = mesh->sxxd0; g.szzd0 = mesh->szzd0;
  g.sxz = mesh->sxz; g.sxz0 = mesh->sxz0;
  g.u_in = mesh->u_in; g.v_in = mesh->v_in;
  g.wxz = mesh->wxz;
  g.xc_coord = mesh->xc_coord; g.zc_coord = mesh->zc_coord;
  g.eta_phys_s = mesh->eta_phys_s;
  mk.n = particles->Nb_part;
  mk.x = particles->x; mk.z = particles->z; mk.phase = particles->phase;
  mk.sxxd = particles->sxxd; mk.szzd = particles->szzd; mk.sxz = particles->sxz;
  mk.nx = particles->nx; mk.nz = particles->nz;
  memset(&st, 0, sizeof(st));
  const int rc = mdz_rheo_marker_stress(mdz_context(), &md, &o, &g, &mk, MDZ_MEM_HOST, 0, &st);
  if (rc == MDZ_EMARKER_OUT) {
    fprintf(stderr, "marker beyond the grid in x (UpdateParticleStress)\n"); /* ParticleRoutines.c:1261-1265 */
    exit(89);
  }
  if (rc != MDZ_OK) mdz_fail(rc, &st);
}

void NonNewtonianViscosityGridAniso(grid *mesh, mat_prop *materials, params *model, Nparams Nmodel,
                                    scale *scaling, int final_update) {
  (void)Nmodel;
  mdz_sweep_grid(mesh, materials, model, scaling, final_update, 1);
  ApplySetGridDensityOverride(mesh, model); /* AnisotropyRoutines.c:1216 */
}
