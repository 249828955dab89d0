/*
 * rheo_oracle.c -- CPU restatement of MDOODZ7.0's local rheology update.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  See
 * rheo_oracle.h.  Every block cites the reference lines it restates; the
 * floating-point expressions keep the reference's evaluation order so that,
 * compiled with -ffp-contract=off, results are bit-identical to the reference
 * built from its own sources on x86-64.  Dead computations of the reference
 * (values that never reach an output) are left out and noted.
 */
#include "rheo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ZEROC 273.15 /* MDLIB/include/mdoodz.h:4 */
#define ORC_MIN(a, b) ((a) <= (b) ? (a) : (b)) /* MINV, MDLIB/mdoodz-private.h:11 */
#define ORC_MAX(a, b) ((a) >= (b) ? (a) : (b)) /* MAXV, MDLIB/mdoodz-private.h:12 */

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* one point: scalar inputs and outputs                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  int    phase;
  double G, T, P, d, phi, X0, Exx, Ezz, Exz, Txx0, Tzz0, Txz0, dil, fric, C, P0, T0, beta;
  double lxlz, lx2, angle, ani_fac; /* aniso only */
  int    post_process, centroid, final_update;
} orc_pt;

typedef struct {
  double eta, Txx, Tzz, Txz, etaVE, VEcoeff, Eii_el, Eii_pl, Eii_pwl, Eii_exp, Eii_lin, Eii_gbs,
         Eii_cst, d1, X1, OverS, Pcorr, rho, div_el, div_pl, div_r, Wtot, Wel, Wdiss;
  int    iters, is_pl, status;
  int    mech;  /* MDZ_MECH_* bits: the switches of :471-483 (aniso :322-326) and is_pl */
} orc_res;

static void set_status(int *st, int code) {
  if (*st == MDZ_OK) *st = code;
}

/* ------------------------------------------------------------------------ */
/* local visco-elastic solves: LocalIterationParams (RheologyDensity.h:17-48) */
/* ------------------------------------------------------------------------ */
typedef struct {
  int    elastic, peierls, dislocation, diffusion, constant, gbs;
  double Eii, eta_el, eta_cst, C_pwl, n_pwl, C_gbs, n_gbs, C_lin, n_lin, m_lin, C_exp, ST, n_exp;
  double d, eta_up, eta_lo, Ag, gam, lam, cg, pg;
} orc_ve;

typedef struct {
  double eta, Tii, d1, e_cst, e_pwl, e_gbs, e_exp, e_lin;
  int    iters, status;
} orc_ve_out;

/* LocalIterationViscoElastic, RheologyDensity.c:152-197 */
static void orc_ve_newton(const orc_ve *q, orc_ve_out *o) {
  const int    nitmax = 20;
  const double tol    = 1.0e-11;
  double eta = o->eta, Tii = o->Tii;
  double e_cst = 0., e_pwl = 0., e_gbs = 0., e_exp = 0., e_lin = 0.;
  int    it, iters = nitmax;
  for (it = 0; it < nitmax; it++) {
    Tii = 2.0 * eta * q->Eii;
    if (q->constant) e_cst = Tii / 2.0 / q->eta_cst;
    if (q->dislocation) e_pwl = q->C_pwl * pow(Tii, q->n_pwl);
    if (q->gbs) e_gbs = q->C_gbs * pow(Tii, q->n_gbs);
    if (q->peierls) e_exp = q->C_exp * pow(Tii, q->ST + q->n_exp);
    if (q->diffusion) e_lin = q->C_lin * pow(Tii, q->n_lin) * pow(q->d, -q->m_lin);
    const double e_vis = e_pwl + e_exp + e_lin + e_gbs + e_cst;
    const double r     = q->Eii - q->elastic * Tii / (2.0 * q->eta_el) - e_vis;
    const double res   = fabs(r / q->Eii);
    if (res < tol / 100) {
      iters = it + 1;
      break;
    } else if (it == nitmax - 1 && res > tol) { /* reference: exit(0) */
      set_status(&o->status, MDZ_EVE_ITER);
      break;
    }
    double dfdeta = 0.0;
    if (q->elastic) dfdeta += -q->Eii / q->eta_el;
    if (q->peierls) dfdeta += -(e_exp) * (q->ST + q->n_exp) / eta;
    if (q->diffusion) dfdeta += -(e_lin) * q->n_lin / eta;
    if (q->dislocation) dfdeta += -(e_pwl) * q->n_pwl / eta;
    if (q->constant) dfdeta += -q->Eii / q->eta_cst;
    eta -= r / dfdeta;
  }
  o->eta = eta; o->Tii = Tii; o->iters = iters;
  o->e_cst = e_cst; o->e_exp = e_exp; o->e_gbs = e_gbs; o->e_pwl = e_pwl; o->e_lin = e_lin;
}

/* LocalIterationViscoElasticGrainSize, RheologyDensity.c:203-379.  The two
 * bracket-end evaluations at :221-243 only feed the unused r_eta_lo/r_eta_up
 * and are overwritten inside the loop, so they are not restated. */
static void orc_ve_gse(const orc_ve *q, orc_ve_out *o) {
  const int    nitmax = 50, bisection_steps = 20;
  const double tol    = 1.0e-11;
  double d_ve = o->d1, eta = o->eta, Tii = o->Tii;
  const double p = q->pg, Eii = q->Eii, n_pwl = q->n_pwl, Ag = q->Ag;
  const double Bg    = q->lam / (q->cg * q->gam);
  const double C_pwl = q->C_pwl;
  double eta_up = q->eta_up, eta_lo = q->eta_lo;
  double e_cst = 0., e_pwl = 0., e_gbs = 0., e_exp = 0., e_lin = 0.;
  int    it, iters = nitmax;
  for (it = 0; it < nitmax; it++) {
    if (it < bisection_steps) eta = sqrt(eta_up * eta_lo);
    Tii = 2.0 * eta * q->Eii;
    if (q->constant) e_cst = Tii / 2.0 / q->eta_cst;
    if (q->dislocation) e_pwl = q->C_pwl * pow(Tii, q->n_pwl);
    d_ve = pow(2 * Bg * q->Eii * e_pwl * eta * p / q->Ag, (-1.0 / (p + 1)));
    if (q->gbs) e_gbs = q->C_gbs * pow(Tii, q->n_gbs);
    if (q->peierls) e_exp = q->C_exp * pow(Tii, q->ST + q->n_exp);
    if (q->diffusion) e_lin = q->C_lin * pow(Tii, q->n_lin) * pow(d_ve, -q->m_lin);
    const double e_vis = e_pwl + e_exp + e_lin + e_gbs + e_cst;
    const double r     = q->Eii - q->elastic * Tii / (2.0 * q->eta_el) - e_vis;
    const double res   = fabs(r / q->Eii);
    if (res < tol / 100) { iters = it + 1; break; }
    if (it == bisection_steps - 1 && res < tol) { iters = it + 1; break; }
    if (it < bisection_steps) {
      if (r > 0.0) eta_up = eta;
      else         eta_lo = eta;
    } else {
      const double dddeta = -1.0 / 2.0 * Ag * d_ve * pow(2 * Eii * eta, -n_pwl) *
                            (2 * Bg * C_pwl * Eii * n_pwl * p * pow(2 * Eii * eta, n_pwl) / Ag +
                             2 * Bg * C_pwl * Eii * p * pow(2 * Eii * eta, n_pwl) / Ag) /
                            (Bg * C_pwl * Eii * eta * p * (p + 1));
      double dfdeta = 0.0;
      if (q->elastic) dfdeta += -q->Eii / q->eta_el;
      if (q->constant) dfdeta += -q->Eii / q->eta_cst;
      if (q->peierls) dfdeta += -(e_exp) * (q->ST + q->n_exp) / eta;
      if (q->diffusion) dfdeta += -(e_lin) * q->n_lin / eta;
      if (q->dislocation) dfdeta += -(e_pwl) * q->n_pwl / eta;
      dfdeta += q->m_lin * e_lin * dddeta / d_ve;
      eta -= r / dfdeta;
    }
    if (it == nitmax - 1 && res > tol) { /* reference: exit(346) */
      set_status(&o->status, MDZ_EGSE_ITER);
      break;
    }
  }
  if (isnan(eta) || isinf(eta)) set_status(&o->status, MDZ_EGSE_ITER);
  o->eta = eta; o->d1 = d_ve; o->Tii = Tii; o->iters = iters;
  o->e_cst = e_cst; o->e_exp = e_exp; o->e_gbs = e_gbs; o->e_pwl = e_pwl; o->e_lin = e_lin;
}

/* solve_local_3x3, RheologyDensity.c:1082-1125 */
static int orc_solve3(double J11, double J12, double J13, double J21, double J22, double J23,
                      double J31, double J32, double J33, double R1, double R2, double R3,
                      double *dT, double *dP, double *dl) {
  const double det = J11 * (J22 * J33 - J23 * J32) - J12 * (J21 * J33 - J23 * J31) +
                     J13 * (J21 * J32 - J22 * J31);
  if (fabs(det) < 1e-30) return 0;
  const double inv = 1.0 / det;
  *dT = -inv * ((J22 * J33 - J23 * J32) * R1 + (J13 * J32 - J12 * J33) * R2 +
                (J12 * J23 - J13 * J22) * R3);
  *dP = -inv * ((J23 * J31 - J21 * J33) * R1 + (J11 * J33 - J13 * J31) * R2 +
                (J13 * J21 - J11 * J23) * R3);
  *dl = -inv * ((J21 * J32 - J22 * J31) * R1 + (J12 * J31 - J11 * J32) * R2 +
                (J11 * J22 - J12 * J21) * R3);
  return 1;
}

/* EvaluateDensity, RheologyDensity.c:1761-1831 (models 0, 1, 3, 5; 2 and 4
 * need phase-diagram tables and are rejected before the sweep when their
 * value is used). */
static double orc_density(const mdz_model *m, const mdz_materials *mt, int p, double T, double P,
                          double X, double phi) {
  double rho = 0.0;
  const int dm = mt->density_model[p];
  if (dm == 0) rho = mt->rho[p];
  if (dm == 1) {
    rho = (1.0 - mt->alp[p] * (T - mt->T0[p])) * (1.0 + mt->bet[p] * (P - mt->P0[p]));
    rho = ((1.0 - X) * mt->rho[p] + X * (mt->rho[p] + mt->drho[p])) * rho;
  }
  if (dm == 3 && m->density_variations == 0) rho = mt->rho[p] * exp(mt->bet[p] * P - mt->alp[p] * T);
  if (dm == 3 && m->density_variations == 1) {
    const double rho_ref = (1.0 - X) * mt->rho[p] + X * mt->rho[mt->reac_phase[p]];
    rho = rho_ref * exp(mt->bet[p] * P - mt->alp[p] * T);
  }
  if (dm == 5) {
    const double rs = mt->rho[p] * exp(mt->bet[p] * P - mt->alp[p] * T);
    const double rl = (mt->rho[p] + mt->drho[p]) * exp(mt->bet[p] * P - mt->alp[p] * T);
    rho = (1 - phi) * rs + phi * rl;
  }
  return rho;
}

/* ------------------------------------------------------------------------ */
/* ViscosityConcise, RheologyDensity.c:385-1080                              */
/* ------------------------------------------------------------------------ */
static void orc_viscosity_concise(const mdz_model *m, const mdz_materials *mt, const orc_pt *in,
                                  orc_res *o) {
  const int phase = in->phase;
  const int nitmax = 20;
  double G = in->G, T = in->T, P = in->P, d = in->d, dil = in->dil, C = in->C;
  const double phi = in->phi, X0 = in->X0, Exx = in->Exx, Ezz = in->Ezz, Exz = in->Exz;
  const double Txx0 = in->Txx0, Tzz0 = in->Tzz0, Txz0 = in->Txz0, fric = in->fric;
  const double R = mt->R, min_eta = m->min_eta, max_eta = m->max_eta;
  const double TmaxPeierls = (1200.0 + ZEROC) / m->scale_T; /* :390 */
  const double dt = (m->step == 0) ? 1e100 : m->dt;      /* :392-394 */
  const double tol = m->eta_tol;
  int    plastic = 0, constant = 0, dislocation = 0, peierls = 0, diffusion = 0, gbs = 0;
  int    elastic = m->elastic, gs = 0, is_pl = 0;
  double K = 1.0 / in->beta;
  const double Tiimin = 1e5 / m->scale_S;                  /* :427 */
  const double n_pwl = mt->npwl[phase], n_lin = mt->nlin[phase], m_lin = mt->mlin[phase];
  const double n_gbs = mt->ngbs[phase], n_exp = mt->nexp[phase];
  const double eta_vp0 = mt->eta_vp[phase], n_vp = mt->n_vp[phase];
  double eta_vp = mt->eta_vp[phase];
  int    constant_mix = mt->phase_mix[phase];
  if (m->diffuse_X == 0) constant_mix = 0;                 /* :440 */

  memset(o, 0, sizeof(*o));                                /* :451-455 */
  /* invariants, :461-464 */
  const double Eyy = -(Exx + Ezz);
  double Eii = sqrt(1.0 / 2.0 * (Exx * Exx + Ezz * Ezz + Eyy * Eyy) + Exz * Exz);
  if (Eii * m->scale_E < 1e-30) Eii = 1e-30 / m->scale_E;
  o->Pcorr = P;                                            /* :467 */
  /* mechanism switches, :471-483 */
  if (mt->cstv[phase] != 0) constant = 1;
  if (mt->pwlv[phase] != 0) dislocation = 1;
  if (mt->expv[phase] != 0 && T < TmaxPeierls) peierls = 1;
  if (mt->linv[phase] != 0) diffusion = 1;
  if (mt->gbsv[phase] != 0) gbs = 1;
  if (mt->gs[phase] != 0) gs = 1;
  if (mt->plast[phase] == 1) plastic = 1;
  if (mt->plast[phase] == 2) plastic = 2;
  if (m->step == 0) { elastic = 0; plastic = 0; }
  o->mech = constant * MDZ_MECH_CONSTANT | dislocation * MDZ_MECH_DISLOCATION | peierls * MDZ_MECH_PEIERLS |
            diffusion * MDZ_MECH_DIFFUSION | gbs * MDZ_MECH_GBS | gs * MDZ_MECH_GRAIN_SIZE |
            (plastic != 0) * MDZ_MECH_PLASTIC | (elastic != 0) * MDZ_MECH_ELASTIC;
  o->d1 = mt->gs_ref[phase];                               /* :486 */
  if (elastic == 0) { G = 1e1; dil = 0.0; K = 1e10; }      /* :493 */
  if (T < ZEROC / m->scale_T) T = ZEROC / m->scale_T;      /* :496 */

  /* Arrhenius pre-factors, :501-523 */
  double B_pwl = 0.0, C_pwl = 0.0, B_lin = 0.0, C_lin = 0.0, B_gbs = 0.0, B_exp = 0.0, C_exp = 0.0;
  double ST = 0.0;
  if (dislocation == 1) {
    B_pwl = mt->pref_pwl[phase] * mt->Fpwl[phase] * pow(mt->Apwl[phase], -1.0 / n_pwl) *
            exp((mt->Qpwl[phase] + P * mt->Vpwl[phase]) / R / n_pwl / T) *
            pow(d, mt->mpwl[phase] / n_pwl) * pow(mt->fpwl[phase], -mt->rpwl[phase] / n_pwl) *
            exp(-mt->apwl[phase] * phi / n_pwl);
    C_pwl = pow(2.0 * B_pwl, -n_pwl);
  }
  if (diffusion == 1) {
    if (m_lin > 0.0 && d < 1e-13 / m->scale_L) set_status(&o->status, MDZ_EGRAIN_ZERO);
    B_lin = mt->Flin[phase] * pow(mt->Alin[phase], -1.0 / n_lin) *
            exp((mt->Qlin[phase] + P * mt->Vlin[phase]) / R / n_lin / T) *
            pow(mt->flin[phase], -mt->rlin[phase] / n_lin) * exp(-mt->alin[phase] * phi / n_lin);
    C_lin = pow(2.0 * B_lin, -n_lin);
  }
  if (gbs == 1) {
    B_gbs = mt->Fgbs[phase] * pow(mt->Agbs[phase], -1.0 / n_gbs) *
            exp((mt->Qgbs[phase] + P * mt->Vgbs[phase]) / R / n_gbs / T) *
            pow(d, mt->mgbs[phase] / n_gbs) * pow(mt->fgbs[phase], -mt->rgbs[phase] / n_gbs) *
            exp(-mt->agbs[phase] * phi / n_gbs);
  }
  if (peierls == 1) {
    const double Ea = mt->Qexp[phase], gamma = mt->Gexp[phase];
    ST = Ea / R / T * 2.0 * gamma * (1 - gamma);
    const double Arr = exp(-Ea / R / T * pow(1.0 - gamma, 2.0));
    const double F_exp = pow(pow(2.0, 1.0 - ST - n_exp) / pow(sqrt(3.0), ST + n_exp + 1.0),
                             1.0 / (ST + n_exp));
    B_exp = F_exp * (pow(gamma * mt->Sexp[phase], ST / (ST + n_exp)) /
                     pow(mt->Eexp[phase] * Arr, 1.0 / (ST + n_exp)));
    C_exp = pow(2.0 * B_exp, -(ST + n_exp));
  }
  const double cos_fric = cos(fric), sin_fric = sin(fric), sin_dil = sin(dil);
  double Tyield = 0.0;
  if (plastic == 1) {                                      /* :530-539 */
    Tyield = C * cos_fric + P * sin_fric;
    if (mt->Slim[phase] < Tyield) { C = mt->Slim[phase]; Tyield = mt->Slim[phase]; }
  }
  o->X1 = X0;                                              /* :545, :554 */

  /* isolated viscosities, :559-592 */
  const double eta_el = G * dt;
  double eta_cst = 0.0, eta_pwl = 0.0, eta_lin = 0.0, eta_gbs = 0.0, eta_exp = 0.0, Ag = 0.0;
  if (constant == 1) eta_cst = mt->eta0[phase];
  if (constant_mix == 1) {
    const double e1 = mt->eta0[phase], e2 = mt->eta0[mt->phase_two[phase]];
    if (m->diffuse_avg == 0) eta_cst = X0 * e1 + (1 - X0) * e2;
    if (m->diffuse_avg == 1) eta_cst = pow(X0 / e1 + (1 - X0) / e2, -1.0);
    if (m->diffuse_avg == 2) eta_cst = exp(X0 * log(e1) + (1 - X0) * log(e2));
  }
  if (dislocation == 1) eta_pwl = B_pwl * pow(Eii, 1.0 / n_pwl - 1.0);
  double Tii = 0.0;
  if (gs == 1) {                                           /* :567-576 */
    Ag = mt->Kpzm[phase] * exp(-mt->Qpzm[phase] / R / T);
    const double gam = mt->Gpzm[phase], lam = mt->Lpzm[phase], cg = mt->cpzm[phase], pg = mt->ppzm[phase];
    Tii = 2. * eta_el * Eii;
    o->Eii_pwl = Tii / 2.0 / eta_pwl;
    d = exp(log(Ag * gam / (lam * (1.0 / cg) * Tii * (o->Eii_pwl) * pg)) / (1.0 + pg));
  }
  if (diffusion == 1) eta_lin = B_lin * pow(Eii, 1.0 / n_lin - 1.0) * pow(d, m_lin / n_lin);
  if (gbs == 1) eta_gbs = B_gbs * pow(Eii, 1.0 / n_gbs - 1.0);
  if (peierls == 1) eta_exp = B_exp * pow(Eii, 1.0 / (ST + n_exp) - 1.0);
  o->Eii_pl = 0.0;
  double eta_up = 1.0e100 / m->scale_eta, eta_lo = -1.0e100 / m->scale_eta;
  if (constant == 1)    { eta_up = ORC_MIN(eta_up, eta_cst); eta_lo = ORC_MAX(eta_lo, eta_cst); }
  if (dislocation == 1) { eta_up = ORC_MIN(eta_up, eta_pwl); eta_lo = ORC_MAX(eta_lo, eta_pwl); }
  if (elastic == 1)     { eta_up = ORC_MIN(eta_up, eta_el);  eta_lo = ORC_MAX(eta_lo, eta_el);  }
  if (peierls == 1)     { eta_up = ORC_MIN(eta_up, eta_exp); eta_lo = ORC_MAX(eta_lo, eta_exp); }
  if (diffusion == 1)   { eta_up = ORC_MIN(eta_up, eta_lin); eta_lo = ORC_MAX(eta_lo, eta_lin); }
  if (gbs == 1)         { eta_up = ORC_MIN(eta_up, eta_gbs); eta_lo = ORC_MAX(eta_lo, eta_gbs); }

  /* initial guess and local solve, :597-647 (the d_it of :610 is unused) */
  double eta_ve = eta_up;
  Tii = 2.0 * eta_ve * Eii;
  if (gs == 1) o->d1 = d;
  orc_ve q = {0};
  q.elastic = elastic; q.peierls = peierls; q.dislocation = dislocation; q.diffusion = diffusion;
  q.constant = constant; q.gbs = gbs; q.Eii = Eii; q.eta_el = eta_el; q.eta_cst = eta_cst;
  q.C_pwl = C_pwl; q.n_pwl = n_pwl; q.C_gbs = 0.0; /* C_gbs is never set, :616-642 */
  q.n_gbs = n_gbs; q.C_lin = C_lin; q.n_lin = n_lin; q.m_lin = m_lin; q.C_exp = C_exp; q.ST = ST;
  q.n_exp = n_exp; q.d = d; q.eta_up = eta_up; q.eta_lo = eta_lo; q.Ag = Ag;
  q.gam = mt->Gpzm[phase]; q.lam = mt->Lpzm[phase]; q.cg = mt->cpzm[phase]; q.pg = mt->ppzm[phase];
  orc_ve_out vo = {0};
  vo.eta = eta_ve; vo.Tii = Tii; vo.d1 = o->d1; vo.status = MDZ_OK;
  if (gs) orc_ve_gse(&q, &vo);
  else    orc_ve_newton(&q, &vo);
  set_status(&o->status, vo.status);
  eta_ve = vo.eta; Tii = vo.Tii; o->iters = vo.iters;
  if (gs) o->d1 = vo.d1;
  o->Eii_cst = vo.e_cst; o->Eii_exp = vo.e_exp; o->Eii_gbs = vo.e_gbs; o->Eii_pwl = vo.e_pwl;
  o->Eii_lin = vo.e_lin;

  /* plastic corrections */
  double gdot = 0.0, divp = 0.0, Pc = P, eta_vep = 0.0, lam_dot = 0.0, A_tau = 1.0, A_P = 0.0;
  if (plastic == 1) {                                      /* :655-707 */
    double F_trial = Tii - Tyield;
    if (F_trial > 1e-17) {
      double Tiic = 0.0, res_pl;
      is_pl   = 1;
      eta_vp  = eta_vp0 * pow(Eii, 1.0 / n_vp - 1);
      gdot    = F_trial / (eta_ve + eta_vp + K * dt * sin_fric * sin_dil);
      A_P     = -sin_dil;
      const double F_trial0 = F_trial;
      for (int it = 0; it < nitmax; it++) {
        A_P     = -sin_dil;
        divp    = -gdot * A_P;
        Pc      = P + K * dt * divp;
        eta_vp  = eta_vp0 * pow(fabs(gdot), 1.0 / n_vp - 1.0);
        Tyield  = Tyield + gdot * eta_vp;
        Tiic    = Tii - eta_ve * gdot;
        F_trial = Tiic - Tyield;
        res_pl  = fabs(F_trial);
        if (res_pl < tol || res_pl / F_trial0 < tol) break;
        const double dFdgdot = -eta_ve - eta_vp / n_vp - K * dt * sin_fric * sin_dil;
        gdot -= F_trial / dFdgdot;
      }
      if (Tiic < 0.0) {                                    /* :697-704 */
        F_trial = Tii - Tiimin;
        gdot    = F_trial / (eta_ve);
        Tiic    = Tiimin;
        Pc      = P;
      }
      o->Pcorr = Pc;
      eta_vep  = Tiic / (2.0 * Eii);
      Tii      = Tiic;
    }
  }
  if (plastic == 2) {                                      /* :710-930 */
    const double k = sin_fric, kq = sin_dil, c = C * cos_fric;
    const double a = sqrt(1.0 + k * k), b = sqrt(1.0 + kq * kq);
    const double T_st = mt->T_st[phase];
    const double py = (T_st + c / a) / (1.0 - k / a);
    const double Ry = py - T_st;
    const double pd = py - Ry * k / a;
    const double tau_d = k * pd + c;
    const double pq = pd + kq * tau_d;
    double R_haty = sqrt(Tii * Tii + (P - py) * (P - py));
    double R_hatq;
    int on_yield = (Tii * (py - pd)) >= (tau_d * (py - P)), on_flow;
    double F_trial = on_yield ? Tii - k * P - c : a * (R_haty - Ry);
    divp = 0.0;
    if (F_trial > 1e-17) {
      const double atol = 1e-10, rtol = 1e-8;
      double Tiic = Tii, R0n = 2.0 * atol, Rn;
      double A_tau_2 = 0, A_P_2 = 0, A_tau_P = 0, A_P_tau = 0, dFdT, dFdP;
      is_pl = 1; Pc = P; lam_dot = 0.0;
      for (int it = 0; it < nitmax; it++) {
        if (Tiic < 0.0) Tiic = 0.0;
        on_yield = (Tiic * (py - pd)) >= (tau_d * (py - Pc));
        on_flow  = (Tiic * (pq - pd)) >= (tau_d * (pq - Pc));
        eta_vp   = eta_vp0;
        R_haty   = sqrt(Tiic * Tiic + (Pc - py) * (Pc - py));
        R_hatq   = sqrt(Tiic * Tiic + (Pc - pq) * (Pc - pq));
        if (on_yield) { F_trial = Tiic - k * Pc - c; dFdT = 1.0; dFdP = -k; }
        else { F_trial = a * (R_haty - Ry); dFdT = a * Tiic / R_haty; dFdP = a * (Pc - py) / R_haty; }
        if (on_flow) { A_tau = 0.5; A_P = kq; A_tau_2 = 0.0; A_P_2 = 0.0; A_tau_P = 0.0; A_P_tau = 0.0; }
        else {
          A_tau   = b * Tiic / (2.0 * R_hatq);
          A_P     = -b * (Pc - pq) / R_hatq;
          A_tau_2 = b * (R_hatq * R_hatq - Tiic * Tiic) / (2.0 * R_hatq * R_hatq * R_hatq);
          A_P_2   = -b * (R_hatq * R_hatq - (Pc - pq) * (Pc - pq)) / (R_hatq * R_hatq * R_hatq);
          A_tau_P = -b * Tiic * (Pc - pq) / (2.0 * R_hatq * R_hatq * R_hatq);
          A_P_tau = b * Tiic * (Pc - pq) / (R_hatq * R_hatq * R_hatq);
        }
        double R1 = (Tii - Tiic) / (2.0 * eta_ve) - lam_dot * A_tau;
        double R2 = (Pc - P) / (K * dt) - lam_dot * A_P;
        double R3 = F_trial - lam_dot * eta_vp;
        Rn = sqrt(R1 * R1 + R2 * R2 + R3 * R3);
        if (Rn < atol || Rn / R0n < rtol) break;
        R0n = Rn;
        const double J11 = -1.0 / 2.0 / eta_ve - lam_dot * A_tau_2, J12 = -lam_dot * A_tau_P, J13 = -A_tau;
        const double J21 = -lam_dot * A_P_tau, J22 = 1.0 / K / dt - lam_dot * A_P_2, J23 = -A_P;
        const double J31 = dFdT, J32 = dFdP, J33 = -eta_vp;
        double dT, dP, dl;
        if (!orc_solve3(J11, J12, J13, J21, J22, J23, J31, J32, J33, R1, R2, R3, &dT, &dP, &dl)) {
          set_status(&o->status, MDZ_ESINGULAR);           /* reference: exit(1) */
          break;
        }
        double alpha = 1.0;
        if (m->tensile_line_search == 1) {                 /* :845-887 */
          const double c_ls = 1e-4, R0ls = 0.5 * (R1 * R1 + R2 * R2 + R3 * R3);
          int failed = 0;
          for (int ls = 0; ls < 100; ls++) {
            const double Tl = Tiic + dT * alpha, Pl = Pc + dP * alpha;
            on_yield = (Tl * (py - pd) >= tau_d * (py - Pl));
            on_flow  = (Tl * (pq - pd) >= tau_d * (pq - Pl));
            eta_vp   = eta_vp0;
            R_haty   = sqrt(Tl * Tl + (Pl - py) * (Pl - py));
            R_hatq   = sqrt(Tl * Tl + (Pl - pq) * (Pl - pq));
            const double Fl = on_yield ? Tl - k * Pl - c : a * (R_haty - Ry);
            if (on_flow) { A_tau = 0.5; A_P = kq; }
            else { A_tau = b * Tl / (2.0 * R_hatq); A_P = -b * (Pl - pq) / R_hatq; }
            R1 = (Tii - Tl) / (2.0 * eta_ve) - lam_dot * A_tau;
            R2 = (Pl - P) / (K * dt) - lam_dot * A_P;
            R3 = Fl - lam_dot * eta_vp;
            const double Rls = 0.5 * (R1 * R1 + R2 * R2 + R3 * R3);
            if (Rls < R0ls - 2.0 * c_ls * alpha * Rls && ls > 0) break;
            alpha *= 0.5;
            if (alpha < 1e-2) { failed = 1; break; }
          }
          if (failed) { set_status(&o->status, MDZ_ELINESEARCH); break; } /* reference: exit(0) */
        }
        Tiic += alpha * dT;
        Pc += alpha * dP;
        lam_dot += alpha * dl;
      }
      o->Pcorr = Pc;
      eta_vep  = Tiic / (2.0 * Eii);
      Tii      = Tiic;
      divp     = lam_dot * A_P;
    }
  }

  /* density, :934-960 (kinetics only alters rho when density_variations==0,
   * where the grid never reads it) */
  if (in->centroid > 0) {
    const double Pd = (in->final_update == 1) ? Pc : P;
    o->rho = orc_density(m, mt, phase, T, Pd, X0, phi);
  }

  double eta_pl = 0.0;
  if (is_pl == 0) { o->etaVE = eta_ve; o->div_pl = 0.0; }
  else if (plastic == 1) { o->etaVE = eta_vep; o->div_pl = divp; eta_pl = Tii / gdot; }
  else if (plastic == 2) { o->etaVE = eta_vep; o->div_pl = divp; eta_pl = Tii / (2.0 * lam_dot * A_tau); }
  o->is_pl = is_pl;
  if (is_pl) o->mech |= MDZ_MECH_YIELD;
  o->Txx = 2.0 * (o->etaVE) * Exx;                         /* :981-983 */
  o->Tzz = 2.0 * (o->etaVE) * Ezz;
  o->Txz = 2.0 * (o->etaVE) * Exz;

  double eta = 0.0;
  if (in->post_process == 1) {                             /* :986-1053 */
    if (dislocation == 1) eta_pwl = B_pwl * pow(o->Eii_pwl, 1.0 / n_pwl - 1.0);
    if (diffusion == 1) eta_lin = B_lin * pow(o->Eii_lin, 1.0 / n_lin - 1.0) * pow(o->d1, m_lin / n_lin);
    if (peierls == 1) eta_exp = B_exp * pow(o->Eii_exp, 1.0 / (ST + n_exp) - 1.0);
    if (elastic) {
      const double Tyy = -(o->Txx + o->Tzz), Tyy0 = -(Txx0 + Tzz0);
      const double Exx_el = (o->Txx - Txx0) / 2 / eta_el, Ezz_el = (o->Tzz - Tzz0) / 2 / eta_el;
      const double Eyy_el = (Tyy - Tyy0) / 2 / eta_el, Exz_el = (o->Txz - Txz0) / 2 / eta_el;
      o->Eii_el = sqrt(0.5 * (Exx_el * Exx_el + Ezz_el * Ezz_el + Eyy_el * Eyy_el) + Exz_el * Exz_el);
    }
    if (is_pl && plastic == 1) o->Eii_pl = gdot / 2.0;
    else if (is_pl && plastic == 2) o->Eii_pl = lam_dot * A_tau;
    else o->Eii_pl = 0.0;
    o->div_pl = divp;
    o->div_el = -(Pc - in->P0) / (K * dt);
    o->div_r  = 0.0;
    double inv = 0.0;
    if (peierls == 1) inv += (1.0 / eta_exp);
    if (dislocation == 1) inv += (1.0 / eta_pwl);
    if (diffusion == 1) inv += (1.0 / eta_lin);
    if (constant == 1) inv += (1.0 / eta_cst);
    if (is_pl == 1) inv += (1.0 / eta_pl);
    eta = 1.0 / (inv);
    if (plastic == 1) o->OverS = eta_vp * gdot;
    if (plastic == 2) o->OverS = eta_vp * lam_dot * A_tau;
    if (in->centroid == 1) {
      o->Wtot  = Tii * Tii / eta_ve;
      o->Wel   = Tii * Tii / eta_el;
      o->Wdiss = Tii * Tii / eta;
      if (o->Wdiss < 0.0) set_status(&o->status, MDZ_EWDISS); /* reference: exit(1) */
    }
  }
  /* limiters, :1058-1073 */
  if (o->etaVE > max_eta) o->etaVE = max_eta;
  if (o->etaVE < min_eta) o->etaVE = min_eta;
  if (eta > max_eta) eta = max_eta;
  if (eta < min_eta) eta = min_eta;
  o->eta = eta;
}

/* ------------------------------------------------------------------------ */
/* ViscosityConciseAniso, AnisotropyRoutines.c:282-727                        */
/* ------------------------------------------------------------------------ */
static void orc_viscosity_concise_aniso(const mdz_model *m, const mdz_materials *mt,
                                        const orc_pt *in, orc_res *o) {
  const int    phase = in->phase;
  const double tol = 1e-11, R = mt->R, dt = m->dt, min_eta = m->min_eta, max_eta = m->max_eta;
  const int    nitmax = 50;
  const double TmaxPeierls = (1200.0 + ZEROC) / m->scale_T;
  double G = in->G, T = in->T, P = in->P, dil = in->dil, Coh = in->C;
  const double fric = in->fric, phi = in->phi, lxlz = in->lxlz, lx2 = in->lx2, ani_fac = in->ani_fac;
  int    plastic = 0, constant = 0, dislocation = 0, peierls = 0, diffusion = 0;
  int    elastic = m->elastic, is_pl = 0;
  double eta_el = 1e20, eta_cst = 0.0;
  const double n_pwl = mt->npwl[phase], n_lin = mt->nlin[phase], m_lin = mt->mlin[phase];
  const double n_exp = mt->nexp[phase];

  memset(o, 0, sizeof(*o));                                /* :310-318 */
  o->Pcorr = P;
  o->d1    = in->d;
  if (mt->cstv[phase] != 0) constant = 1;                  /* :322-326 */
  if (mt->pwlv[phase] != 0) dislocation = 1;
  if (mt->expv[phase] != 0 && T < TmaxPeierls) peierls = 1;
  if (mt->linv[phase] != 0) diffusion = 1;
  if (mt->plast[phase] != 0) plastic = 1;
  if (m->step == 0) elastic = 0;
  o->mech = constant * MDZ_MECH_CONSTANT | dislocation * MDZ_MECH_DISLOCATION | peierls * MDZ_MECH_PEIERLS |
            diffusion * MDZ_MECH_DIFFUSION | (mt->gs[phase] != 0) * MDZ_MECH_GRAIN_SIZE |
            plastic * MDZ_MECH_PLASTIC | (elastic != 0) * MDZ_MECH_ELASTIC;
  if (elastic == 0) { G = 1e1; dil = 0.0; }
  if (T < ZEROC / m->scale_T) T = ZEROC / m->scale_T;

  double B_pwl = 0.0, C_pwl = 0.0, B_lin = 0.0, C_lin = 0.0, B_exp = 0.0, C_exp = 0.0, ST = 0.0;
  if (dislocation == 1) {                                  /* :334-337 */
    B_pwl = mt->pref_pwl[phase] * mt->Fpwl[phase] * pow(mt->Apwl[phase], -1.0 / n_pwl) *
            exp((mt->Qpwl[phase] + P * mt->Vpwl[phase]) / R / n_pwl / T) *
            pow(in->d, mt->mpwl[phase] / n_pwl) * pow(mt->fpwl[phase], -mt->rpwl[phase] / n_pwl) *
            exp(-mt->apwl[phase] * phi / n_pwl);
    C_pwl = pow(2.0 * B_pwl, -n_pwl);
  }
  if (diffusion == 1) {                                    /* :342-349 */
    if (m_lin > 0.0 && o->d1 < 1e-13 / m->scale_L) set_status(&o->status, MDZ_EGRAIN_ZERO);
    B_lin = mt->Flin[phase] * pow(mt->Alin[phase], -1.0 / n_lin) *
            exp((mt->Qlin[phase] + P * mt->Vlin[phase]) / R / n_lin / T) *
            pow(mt->flin[phase], -mt->rlin[phase] / n_lin) * exp(-mt->alin[phase] * phi / n_lin);
    C_lin = pow(2.0 * B_lin, -n_lin);
  }
  if (peierls == 1) {                                      /* :355-362 */
    const double Ea = mt->Qexp[phase], gamma = mt->Gexp[phase];
    ST = Ea / R / T * 2.0 * gamma * (1 - gamma);
    const double Arr = exp(-Ea / R / T * pow(1.0 - gamma, 2.0));
    const double F_exp = pow(pow(2.0, 1.0 - ST - n_exp) / pow(sqrt(3.0), ST + n_exp + 1.0),
                             1.0 / (ST + n_exp));
    B_exp = F_exp * (pow(gamma * mt->Sexp[phase], ST / (ST + n_exp)) /
                     pow(mt->Eexp[phase] * Arr, 1.0 / (ST + n_exp)));
    C_exp = pow(2.0 * B_exp, -(ST + n_exp));
  }
  double Tyield = 0.0;
  const double K = 1.0 / in->beta;
  if (plastic == 1) {                                      /* :370-377 */
    Tyield = Coh * cos(fric) + P * sin(fric);
    if (mt->Slim[phase] < Tyield) { Coh = mt->Slim[phase]; Tyield = mt->Slim[phase]; }
  }
  /* rotate the strain rate, :379-383 */
  const double nz2 = 1.0 - lx2;
  const double Er_xx = lx2 * in->Exx + nz2 * in->Ezz + 2. * lxlz * in->Exz;
  const double Er_zz = nz2 * in->Exx + lx2 * in->Ezz - 2. * lxlz * in->Exz;
  const double Er_xz = -lxlz * in->Exx + lxlz * in->Ezz + (lx2 - nz2) * in->Exz;
  const double Er_yy = -Er_xx - Er_zz;
  /* I2, :263-265 */
  const double Eii = sqrt(0.5 * (pow(Er_xx, 2) + pow(Er_zz, 2) + pow(Er_yy, 2)) + pow(Er_xz, 2));
  double eta_pwl = 0.0, eta_lin = 0.0, eta_exp = 0.0;
  if (constant) eta_cst = mt->eta0[phase];                 /* :390-397 */
  if (dislocation) eta_pwl = B_pwl * pow(Eii, (1 - n_pwl) / n_pwl);
  if (elastic) eta_el = G * dt;
  if (diffusion == 1) eta_lin = B_lin * pow(Eii, 1.0 / n_lin - 1.0) * pow(o->d1, m_lin / n_lin);
  if (peierls == 1) eta_exp = B_exp * pow(Eii, 1.0 / (ST + n_exp) - 1.0);
  double eta_up = 1.0e100 / m->scale_eta, eta_lo = -1.0e100 / m->scale_eta; /* :409-415 */
  if (constant)    { eta_up = ORC_MIN(eta_up, eta_cst); eta_lo = ORC_MAX(eta_lo, eta_cst); }
  if (dislocation) { eta_up = ORC_MIN(eta_up, eta_pwl); eta_lo = ORC_MAX(eta_lo, eta_pwl); }
  if (elastic)     { eta_up = ORC_MIN(eta_up, eta_el);  eta_lo = ORC_MAX(eta_lo, eta_el);  }
  if (peierls)     { eta_up = ORC_MIN(eta_up, eta_exp); eta_lo = ORC_MAX(eta_lo, eta_exp); }
  if (diffusion)   { eta_up = ORC_MIN(eta_up, eta_lin); eta_lo = ORC_MAX(eta_lo, eta_lin); }
  double eta_ve = eta_up, Tii = 0.0;

  if (mt->gs[phase] != 0) {                                /* :429-473 */
    orc_ve q = {0};
    q.Ag = mt->Kpzm[phase] * exp(-mt->Qpzm[phase] / (R * T));
    q.gam = mt->Gpzm[phase]; q.lam = mt->Lpzm[phase]; q.cg = mt->cpzm[phase]; q.pg = mt->ppzm[phase];
    q.Eii = Eii; q.C_pwl = C_pwl; q.n_pwl = n_pwl; q.C_lin = C_lin; q.n_lin = n_lin; q.m_lin = m_lin;
    q.ST = ST; q.n_exp = n_exp; q.elastic = elastic; q.eta_el = eta_el; q.peierls = peierls;
    q.C_exp = C_exp; q.dislocation = dislocation; q.diffusion = diffusion; q.constant = constant;
    q.eta_cst = eta_cst; q.gbs = 0; q.C_gbs = 0.0; q.n_gbs = 1.0; q.d = o->d1;
    q.eta_up = eta_up; q.eta_lo = eta_lo;
    orc_ve_out vo = {0};
    vo.eta = eta_ve; vo.Tii = Tii; vo.d1 = o->d1; vo.status = MDZ_OK;
    orc_ve_gse(&q, &vo);
    set_status(&o->status, vo.status);
    eta_ve = vo.eta; Tii = vo.Tii; o->d1 = vo.d1; o->iters = vo.iters;
    o->Eii_cst = vo.e_cst; o->Eii_lin = vo.e_lin; o->Eii_gbs = vo.e_gbs; o->Eii_pwl = vo.e_pwl;
    o->Eii_exp = vo.e_exp;
  } else {                                                 /* :474-585 */
    double r = 0.0, eta_bi_lo = min_eta * 1.0e-3, eta_bi_hi = 10.0 * ORC_MAX(eta_lo, max_eta);
    const double d = o->d1;
    for (int bit = 0; bit < 10; bit++) {
      eta_ve = sqrt(eta_bi_lo * eta_bi_hi);
      Tii = 2.0 * eta_ve * Eii;
      if (constant) o->Eii_cst = Tii / 2.0 / eta_cst;
      if (dislocation) o->Eii_pwl = C_pwl * pow(Tii, n_pwl);
      if (peierls) o->Eii_exp = C_exp * pow(Tii, ST + n_exp);
      if (diffusion) o->Eii_lin = C_lin * pow(Tii, n_lin) * pow(d, -m_lin);
      const double Eii_vis = o->Eii_pwl + o->Eii_cst + o->Eii_exp + o->Eii_lin;
      const double r_bi = Eii - elastic * Tii / 2 / eta_el - Eii_vis;
      if (r_bi > 0.0) eta_bi_lo = eta_ve;
      else eta_bi_hi = eta_ve;
      if (fabs(r_bi / Eii) < tol / 100) break;
    }
    eta_ve = sqrt(eta_bi_lo * eta_bi_hi);
    o->iters = nitmax;
    for (int it = 0; it < nitmax; it++) {
      Tii = 2.0 * eta_ve * Eii;
      if (constant) o->Eii_cst = Tii / 2.0 / eta_cst;
      if (dislocation) o->Eii_pwl = C_pwl * pow(Tii, n_pwl);
      if (peierls) o->Eii_exp = C_exp * pow(Tii, ST + n_exp);
      if (diffusion) o->Eii_lin = C_lin * pow(Tii, n_lin) * pow(d, -m_lin);
      const double Eii_vis = o->Eii_pwl + o->Eii_cst + o->Eii_exp + o->Eii_lin;
      r = Eii - elastic * Tii / 2 / eta_el - Eii_vis;
      if (isnan(r)) { set_status(&o->status, MDZ_EANISO_NAN); o->iters = it + 1; break; }
      double drdeta = 0.0;
      if (elastic) drdeta += -elastic * Eii / eta_el;
      if (dislocation) drdeta += -o->Eii_pwl * n_pwl / eta_ve;
      if (constant) drdeta += -constant * Eii / eta_cst;
      if (peierls) drdeta += -(o->Eii_exp) * (ST + n_exp) / eta_ve;
      if (diffusion) drdeta += -(o->Eii_lin) * n_lin / eta_ve;
      eta_ve -= r / drdeta;
      if (eta_ve <= 0.0) eta_ve = min_eta;
      if (fabs(r / Eii) < tol / 100) { o->iters = it + 1; break; }
      if (it == nitmax - 1 && fabs(r / Eii) < 10.0 * tol) break;
      if (it == nitmax - 1 && (fabs(r / Eii) > tol)) { set_status(&o->status, MDZ_EANISO_ITER); break; }
    }
  }
  if (eta_ve < min_eta) eta_ve = min_eta;                  /* :589-603 */
  if (eta_ve > max_eta) eta_ve = max_eta;
  double Tr_xx = 2.0 * eta_ve * Er_xx, Tr_zz = 2.0 * eta_ve * Er_zz;
  double Tr_xz = 2.0 * eta_ve * Er_xz / ani_fac;
  double eta_vep = eta_ve;
  const double eta_vp = mt->eta_vp[phase], eta_vp0 = mt->eta_vp[phase];
  const double Ft = Tii - Tyield;
  double gdot = 0.0, Pc = P;
  if (Ft > 1e-17 && plastic == 1) {                        /* :625-648 */
    is_pl = 1;
    gdot = Ft / (eta_ve + eta_vp0 + K * dt * sin(dil) * sin(fric));
    const double Tiic = Tii - gdot * eta_ve;
    Pc = P + K * dt * sin(dil) * gdot;
    eta_vep = Tiic / 2.0 / Eii;
    Tr_xx = 2.0 * (eta_vep) * Er_xx;
    Tr_zz = 2.0 * (eta_vep) * Er_zz;
    Tr_xz = 2.0 * (eta_vep) * Er_xz / ani_fac;
    o->div_pl = gdot * sin(dil);
    o->Eii_pl = gdot / 2.0;
    Tii = Tiic;
  }
  o->Txx = lx2 * Tr_xx + nz2 * Tr_zz - 2. * lxlz * Tr_xz; /* :650-652 */
  o->Tzz = nz2 * Tr_xx + lx2 * Tr_zz + 2. * lxlz * Tr_xz;
  o->Txz = lxlz * Tr_xx - lxlz * Tr_zz + (lx2 - nz2) * Tr_xz;
  o->Pcorr = Pc;
  if (eta_vep < min_eta) eta_vep = min_eta;                /* :664-677 */
  if (eta_vep > max_eta) eta_vep = max_eta;
  o->etaVE = eta_vep;
  o->is_pl = is_pl;
  if (is_pl) o->mech |= MDZ_MECH_YIELD;
  double eta = eta_vep;
  const double eta_pl = Tii / gdot, divp = gdot * sin(dil);
  if (in->post_process == 1) {                             /* :681-714 */
    if (dislocation == 1) eta_pwl = B_pwl * pow(o->Eii_pwl, 1.0 / n_pwl - 1.0);
    if (diffusion == 1) eta_lin = B_lin * pow(o->Eii_lin, 1.0 / n_lin - 1.0) * pow(o->d1, m_lin / n_lin);
    if (peierls == 1) eta_exp = B_exp * pow(o->Eii_exp, 1.0 / (ST + n_exp) - 1.0);
    if (elastic) o->Eii_el = Tii * Tii / (4 * eta_el * eta_el);
    if (is_pl) o->Eii_pl = gdot / 2.0;
    o->div_pl = divp;
    o->div_el = -(Pc - in->P0) / (K * dt);
    double inv = 0.0;
    if (diffusion == 1) inv += (1.0 / eta_lin);
    if (peierls == 1) inv += (1.0 / eta_exp);
    if (dislocation == 1) inv += (1.0 / eta_pwl);
    if (constant == 1) inv += (1.0 / eta_cst);
    if (is_pl == 1) inv += (1.0 / eta_pl);
    eta = 1.0 / (inv);
    o->OverS = eta_vp * gdot;
    if (in->centroid == 1) {
      o->Wtot  = Tii * Tii / eta_ve;
      o->Wel   = Tii * Tii / eta_el;
      o->Wdiss = Tii * Tii / eta;
    }
  }
  if (eta > max_eta) eta = max_eta;                        /* :720-721 */
  if (eta < min_eta) eta = min_eta;
  o->eta = eta;
}

/* EffectiveStrainRate, RheologyDensity.c:116-146 */
static void orc_effective_strain_rate(double *Exx, double *Ezz, double *Exz, double exx, double ezz,
                                      double exz, double Txx, double Tzz, double Txz, double d1,
                                      double d2, double ani, double eta_e, int elastic) {
  if (!elastic) { *Exx = exx; *Ezz = ezz; *Exz = exz; return; }
  const double Da11 = 2.0 - 2.0 * ani * d1, Da12 = 2.0 * ani * d1, Da13 = -2.0 * ani * d2;
  const double Da22 = 2.0 - 2.0 * ani * d1, Da23 = 2.0 * ani * d2;
  const double Da33 = 1.0 + 2.0 * ani * (d1 - 0.5);
  const double a11 = Da33 * Da22 - pow(Da23, 2), a12 = Da13 * Da23 - Da33 * Da12;
  const double a13 = Da12 * Da23 - Da13 * Da22, a22 = Da33 * Da11 - pow(Da13, 2);
  const double a23 = Da12 * Da13 - Da11 * Da23, a33 = Da11 * Da22 - pow(Da12, 2);
  const double det = (Da11 * a11) + (Da12 * a12) + (Da13 * a13);
  const double i11 = a11 / det, i12 = a12 / det, i13 = a13 / det, i22 = a22 / det, i23 = a23 / det,
               i33 = a33 / det;
  *Exx = exx + (i11 * Txx + i12 * Tzz + i13 * Txz) / eta_e;
  *Ezz = ezz + (i12 * Txx + i22 * Tzz + i23 * Txz) / eta_e;
  *Exz = exz + (i13 * Txx + i23 * Tzz + i33 * Txz) / eta_e / 2.0;
}

/* ------------------------------------------------------------------------ */
/* InterpCentroidsToVerticesDouble, GridRoutines.c:108-210.  The reference   */
/* builds a ghost-ringed copy of the centroid field; vertex (k,l) reads ring  */
/* cells (k..k+1, l..l+1), each of which maps to one centroid.                */
/* ------------------------------------------------------------------------ */
static int orc_ring_to_centroid(int i, int j, int Ncx, int Ncz, int per) {
  int cj = j - 1, ci;
  if (cj < 0) cj = 0;
  if (cj > Ncz - 1) cj = Ncz - 1;
  if (per == 1) ci = (i == 0) ? Ncx - 1 : (i == Ncx + 1) ? 0 : i - 1;
  else { ci = i - 1; if (ci < 0) ci = 0; if (ci > Ncx - 1) ci = Ncx - 1; }
  return ci + cj * Ncx;
}

static double orc_interp_vertex(const double *cen, const signed char *BCp, const signed char *BCg,
                                int k, int l, int Nx, int Nz, int per) {
  const int Ncx = Nx - 1, Ncz = Nz - 1, c1 = k + l * Nx;
  if (BCg[c1] == 30) return 0.0;
  const int sw = orc_ring_to_centroid(k, l, Ncx, Ncz, per), se = orc_ring_to_centroid(k + 1, l, Ncx, Ncz, per);
  const int nw = orc_ring_to_centroid(k, l + 1, Ncx, Ncz, per), ne = orc_ring_to_centroid(k + 1, l + 1, Ncx, Ncz, per);
  const int inSW = !(BCp[sw] == 30 || BCp[sw] == 31), inSE = !(BCp[se] == 30 || BCp[se] == 31);
  const int inNW = !(BCp[nw] == 30 || BCp[nw] == 31), inNE = !(BCp[ne] == 30 || BCp[ne] == 31);
  return 0.25 * (inSW * cen[sw] + inSE * cen[se] + inNW * cen[nw] + inNE * cen[ne]);
}

void orc_interp_c2v(const mdz_model *m, const double *cen, const signed char *BCp,
                    const signed char *BCg, double *vert) {
  const int Nx = m->Nx, Nz = m->Nz;
#pragma omp parallel for
  for (int c1 = 0; c1 < Nx * Nz; c1++)
    vert[c1] = orc_interp_vertex(cen, BCp, BCg, c1 % Nx, c1 / Nx, Nx, Nz, m->periodic_x);
}

/* ------------------------------------------------------------------------ */
/* sweeps                                                                     */
/* ------------------------------------------------------------------------ */
static int orc_check_supported(const mdz_model *m, const mdz_materials *mt) {
  if (m->Nx < 2 || m->Nz < 2 || m->Nb_phases < 1 || m->Nb_phases > MDZ_MAX_PHASES) return MDZ_EINVAL;
  if (m->melting || m->chemical_production) return MDZ_EUNSUPPORTED;
  for (int p = 0; p < m->Nb_phases; p++) {
    const int dm = mt->density_model[p];
    if (m->density_variations == 1 && (dm == 2 || dm == 4)) return MDZ_EUNSUPPORTED;
  }
  return MDZ_OK;
}

typedef struct {
  uint64_t calls, iters, plastic;
  uint32_t maxit;
  int      status;
  int64_t  node;
} orc_acc;

static void acc_error(orc_acc *a, int status, int64_t node) {
  if (status == MDZ_OK) return;
#pragma omp critical(orc_err)
  {
    if (a->status == MDZ_OK || node < a->node) { a->status = status; a->node = node; }
  }
}

static void fill_stats(mdz_sweep_stats *s, const orc_acc *a) {
  if (!s) return;
  s->phase_calls = a->calls; s->newton_iters = a->iters; s->max_newton_iters = a->maxit;
  s->plastic_calls = a->plastic; s->status = a->status; s->error_node = a->status ? a->node : -1;
  s->elapsed_ms = 0.0;
}

/* NonNewtonianViscosityGrid(Aniso): RheologyDensity.c:1131-1426,
 * AnisotropyRoutines.c:885-1217.  kp/lp/kn/ln are the identity maps built by
 * GridIndices (GridRoutines.c:543-585), so the loop index is the node. */
static int orc_sweep_impl(const mdz_model *m, const mdz_materials *mt, const mdz_grid_fields *f,
                          int final_update, int32_t *iters_n, int32_t *iters_s,
                          mdz_sweep_stats *stats, int aniso) {
  int st = orc_check_supported(m, mt);
  if (st != MDZ_OK) return st;
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1, Nc = Ncx * Ncz, Nv = Nx * Nz;
  const int np = m->Nb_phases, avg = m->eta_average;
  const double el = (m->elastic == 1) ? 1.0 : 0.0;
  orc_acc acc = {0, 0, 0, 0, MDZ_OK, -1};
  uint64_t calls = 0, iters = 0, plastic = 0;
  uint32_t maxit = 0;

  /* :1150-1153 / :903-906 */
  orc_interp_c2v(m, f->T, f->BCp_type, f->BCg_type, f->T_s);
  orc_interp_c2v(m, f->p_in, f->BCp_type, f->BCg_type, f->P_s);
  orc_interp_c2v(m, f->d0_n, f->BCp_type, f->BCg_type, f->d0_s);
  orc_interp_c2v(m, f->phi0_n, f->BCp_type, f->BCg_type, f->phi0_s);

#pragma omp parallel for reduction(+ : calls, iters, plastic) reduction(max : maxit)
  for (int c0 = 0; c0 < Nc; c0++) {
    double *outs[23] = {f->eta_n, f->eta_phys_n, f->VE_n, f->sxxd, f->szzd, f->sxz_n, f->eII_el,
                        f->eII_pl, f->eII_pwl, f->eII_exp, f->eII_lin, f->eII_gbs, f->eII_cst,
                        f->d_n, f->p_corr, f->div_u_el, f->div_u_pl, f->div_u_r, f->Wtot, f->Wel,
                        f->Wdiss, f->X_n, f->OverS_n};
    for (int i = 0; i < 23; i++) outs[i][c0] = 0.0;
    if (m->density_variations == 1) f->rho_n[c0] = 0.0;
    if (iters_n) for (int p = 0; p < np; p++) iters_n[(int64_t)p * Nc + c0] = 0;
    if (f->BCp_type[c0] == 30 || f->BCp_type[c0] == 31) continue;
    const double eta_e = (m->elastic == 1) ? m->dt * f->mu_n[c0] : 1.0;
    double Exx, Ezz, Exz, d1 = 0, d2 = 0;
    orc_pt pt;
    memset(&pt, 0, sizeof(pt));
    if (!aniso) {
      Exx = f->exxd[c0] + el * f->sxxd0[c0] / eta_e / 2.0;
      Ezz = f->ezzd[c0] + el * f->szzd0[c0] / eta_e / 2.0;
      Exz = f->exz_n[c0] + el * f->sxz0_n[c0] / eta_e / 2.0;
    } else {
      d1 = f->d1_n[c0]; d2 = f->d2_n[c0];
      const double angle = f->angle_n[c0], lay = angle - M_PI / 2.0;
      pt.lxlz = cos(lay) * sin(lay); pt.lx2 = cos(lay) * cos(lay); pt.angle = angle;
      pt.ani_fac = f->aniso_factor_n[c0];
      const double aniS_e = 1.0 - 1.0 / f->aniso_factor_n[c0];
      orc_effective_strain_rate(&Exx, &Ezz, &Exz, f->exxd[c0], f->ezzd[c0], f->exz_n[c0], f->sxxd0[c0],
                                f->szzd0[c0], f->sxz0_n[c0], d1, d2, aniS_e, eta_e, m->elastic);
    }
    pt.G = f->mu_n[c0]; pt.T = f->T[c0]; pt.P = f->p_in[c0]; pt.d = f->d0_n[c0];
    pt.phi = f->phi0_n[c0]; pt.X0 = f->X0_n[c0]; pt.Exx = Exx; pt.Ezz = Ezz; pt.Exz = Exz;
    pt.Txx0 = f->sxxd0[c0]; pt.Tzz0 = f->szzd0[c0]; pt.Txz0 = f->sxz0_n[c0]; pt.dil = f->dil_n[c0];
    pt.fric = f->fric_n[c0]; pt.C = f->C_n[c0]; pt.P0 = f->p0_n[c0]; pt.T0 = f->T0_n[c0];
    pt.beta = f->bet_n[c0]; pt.post_process = 1; pt.centroid = 1; pt.final_update = final_update;
    for (int p = 0; p < np; p++) {
      const double perc = f->phase_perc_n[p][c0];
      if (!(fabs(perc) > 1e-13)) continue;                 /* :1210-1212 */
      orc_res r;
      pt.phase = p;
      if (aniso) orc_viscosity_concise_aniso(m, mt, &pt, &r);
      else       orc_viscosity_concise(m, mt, &pt, &r);
      acc_error(&acc, r.status, c0);
      calls++; iters += (uint64_t)r.iters; plastic += (uint64_t)r.is_pl;
      if ((uint32_t)r.iters > maxit) maxit = (uint32_t)r.iters;
      if (iters_n) iters_n[(int64_t)p * Nc + c0] = MDZ_ITEM_WORD(r.iters, r.mech);
      f->phase_eta_n[p][c0] = r.etaVE;
      switch (avg) {
        case 0: f->eta_n[c0] += perc * r.etaVE; f->eta_phys_n[c0] += perc * r.eta; break;
        case 1: f->eta_n[c0] += perc * 1.0 / r.etaVE; f->eta_phys_n[c0] += perc * 1.0 / r.eta; break;
        case 2: f->eta_n[c0] += perc * log(r.etaVE); f->eta_phys_n[c0] += perc * log(r.eta); break;
      }
      if (aniso) f->VE_n[c0] += perc * r.etaVE / eta_e;
      else       f->VE_n[c0] += perc * r.VEcoeff;
      f->eII_el[c0] += perc * r.Eii_el;
      f->eII_pl[c0] += perc * r.Eii_pl;
      f->eII_pwl[c0] += perc * r.Eii_pwl;
      f->eII_exp[c0] += perc * r.Eii_exp;
      f->eII_lin[c0] += perc * r.Eii_lin;
      f->eII_gbs[c0] += perc * r.Eii_gbs;
      f->eII_cst[c0] += perc * r.Eii_cst;
      f->d_n[c0] += perc * 1.0 / r.d1;
      f->Wtot[c0] += perc * r.Wtot;
      f->Wdiss[c0] += perc * r.Wdiss;
      f->Wel[c0] += perc * r.Wel;
      f->p_corr[c0] += perc * r.Pcorr;
      f->div_u_el[c0] += perc * r.div_el;
      f->div_u_pl[c0] += perc * r.div_pl;
      f->div_u_r[c0] += perc * r.div_r;
      f->X_n[c0] += perc * r.X1;
      f->OverS_n[c0] += perc * r.OverS;
      if (m->density_variations == 1) f->rho_n[c0] += perc * (aniso ? 0.0 : r.rho);
    }
    f->d_n[c0] = 1.0 / f->d_n[c0];
    if (!aniso && (isinf(f->d_n[c0]) || isnan(f->d_n[c0]))) acc_error(&acc, MDZ_EEMPTY_CELL, c0);
    if (avg == 1) {
      f->eta_n[c0] = 1.0 / f->eta_n[c0];
      f->eta_phys_n[c0] = 1.0 / f->eta_phys_n[c0];
      if (isinf(f->eta_phys_n[c0]) || isnan(f->eta_phys_n[c0])) acc_error(&acc, MDZ_ENONFINITE, c0);
    }
    if (avg == 2) {
      f->eta_n[c0] = exp(f->eta_n[c0]);
      f->eta_phys_n[c0] = exp(f->eta_phys_n[c0]);
    }
    if (!aniso) {                                          /* :1311-1313 */
      f->sxxd[c0] = 2.0 * f->eta_n[c0] * Exx;
      f->szzd[c0] = 2.0 * f->eta_n[c0] * Ezz;
      f->sxz_n[c0] = 2.0 * f->eta_n[c0] * Exz;
    } else {                                               /* AnisotropyRoutines.c:1079-1086 */
      const double a = 1.0 - 1.0 / f->aniso_factor_n[c0];
      const double Dxx = Exx * (1.0 - a * d1) + Ezz * a * d1 - 2.0 * Exz * a * d2;
      const double Dzz = Ezz * (1.0 - a * d1) + Exx * a * d1 + 2.0 * Exz * a * d2;
      const double Dxz = -Exx * a * d2 + Ezz * a * d2 + 2 * Exz * (a * (d1 - 0.5) + 0.5);
      f->sxxd[c0] = 2.0 * f->eta_n[c0] * Dxx;
      f->szzd[c0] = 2.0 * f->eta_n[c0] * Dzz;
      f->sxz_n[c0] = 2.0 * f->eta_n[c0] * Dxz;
    }
  }

#pragma omp parallel for reduction(+ : calls, iters, plastic) reduction(max : maxit)
  for (int c1 = 0; c1 < Nv; c1++) {
    f->sxxd_s[c1] = 0.0; f->szzd_s[c1] = 0.0; f->sxz[c1] = 0.0;
    f->eta_phys_s[c1] = 0.0; f->eta_s[c1] = 0.0; f->X_s[c1] = 0.0;
    if (aniso && f->VE_s) f->VE_s[c1] = 0.0;
    if (iters_s) for (int p = 0; p < np; p++) iters_s[(int64_t)p * Nv + c1] = 0;
    if (f->BCg_type[c1] == 30) continue;
    const double eta_e = (m->elastic == 1) ? m->dt * f->mu_s[c1] : 1.0;
    double Exx, Ezz, Exz, d1 = 0, d2 = 0;
    orc_pt pt;
    memset(&pt, 0, sizeof(pt));
    if (!aniso) {
      Exx = f->exxd_s[c1] + el * f->sxxd0_s[c1] / eta_e / 2.0;
      Ezz = f->ezzd_s[c1] + el * f->szzd0_s[c1] / eta_e / 2.0;
      Exz = f->exz[c1] + el * f->sxz0[c1] / eta_e / 2.0;
    } else {
      d1 = f->d1_s[c1]; d2 = f->d2_s[c1];
      const double angle = f->angle_s[c1], lay = angle - M_PI / 2.0;
      pt.lxlz = cos(lay) * sin(lay); pt.lx2 = cos(lay) * cos(lay); pt.angle = angle;
      pt.ani_fac = f->aniso_factor_s[c1];
      const double aniS_e = 1.0 - 1.0 / f->aniso_factor_s[c1];
      orc_effective_strain_rate(&Exx, &Ezz, &Exz, f->exxd_s[c1], f->ezzd_s[c1], f->exz[c1],
                                f->sxxd0_s[c1], f->szzd0_s[c1], f->sxz0[c1], d1, d2, aniS_e, eta_e,
                                m->elastic);
    }
    pt.G = f->mu_s[c1]; pt.T = f->T_s[c1]; pt.P = f->P_s[c1]; pt.d = f->d0_s[c1];
    pt.phi = f->phi0_s[c1]; pt.X0 = f->X0_s[c1]; pt.Exx = Exx; pt.Ezz = Ezz; pt.Exz = Exz;
    pt.Txx0 = f->sxxd0_s[c1]; pt.Tzz0 = f->szzd0_s[c1]; pt.Txz0 = f->sxz0[c1]; pt.dil = f->dil_s[c1];
    pt.fric = f->fric_s[c1]; pt.C = f->C_s[c1]; pt.P0 = f->p0_s[c1]; pt.T0 = 0.0;
    pt.beta = f->bet_s[c1]; pt.post_process = 1; pt.centroid = 0; pt.final_update = final_update;
    for (int p = 0; p < np; p++) {
      const double perc = f->phase_perc_s[p][c1];
      if (!(fabs(perc) > 1e-13)) continue;
      orc_res r;
      pt.phase = p;
      if (aniso) orc_viscosity_concise_aniso(m, mt, &pt, &r);
      else       orc_viscosity_concise(m, mt, &pt, &r);
      acc_error(&acc, r.status, (int64_t)Nc + c1);
      calls++; iters += (uint64_t)r.iters; plastic += (uint64_t)r.is_pl;
      if ((uint32_t)r.iters > maxit) maxit = (uint32_t)r.iters;
      if (iters_s) iters_s[(int64_t)p * Nv + c1] = MDZ_ITEM_WORD(r.iters, r.mech);
      f->phase_eta_s[p][c1] = r.etaVE;
      switch (avg) {
        case 0: f->eta_s[c1] += perc * r.etaVE; f->eta_phys_s[c1] += perc * r.eta; break;
        case 1: f->eta_s[c1] += perc * 1.0 / r.etaVE; f->eta_phys_s[c1] += perc * 1.0 / r.eta; break;
        case 2: f->eta_s[c1] += perc * log(r.etaVE); f->eta_phys_s[c1] += perc * log(r.eta); break;
      }
      if (aniso && f->VE_s) f->VE_s[c1] += perc * r.etaVE / eta_e;
      f->X_s[c1] += perc * r.X1;
    }
    if (avg == 1) {
      f->eta_s[c1] = 1.0 / f->eta_s[c1];
      f->eta_phys_s[c1] = 1.0 / f->eta_phys_s[c1];
      if (isinf(f->eta_phys_s[c1]) || isnan(f->eta_phys_s[c1])) acc_error(&acc, MDZ_ENONFINITE, (int64_t)Nc + c1);
    }
    if (avg == 2) {
      f->eta_s[c1] = exp(f->eta_s[c1]);
      f->eta_phys_s[c1] = exp(f->eta_phys_s[c1]);
    }
    if (!aniso) {
      f->sxxd_s[c1] = 2.0 * f->eta_s[c1] * Exx;
      f->szzd_s[c1] = 2.0 * f->eta_s[c1] * Ezz;
      f->sxz[c1] = 2.0 * f->eta_s[c1] * Exz;
    } else {
      const double a = 1.0 - 1.0 / f->aniso_factor_s[c1];
      const double Dxx = Exx * (1.0 - a * d1) + Ezz * a * d1 - 2.0 * Exz * a * d2;
      const double Dzz = Ezz * (1.0 - a * d1) + Exx * a * d1 + 2.0 * Exz * a * d2;
      const double Dxz = -Exx * a * d2 + Ezz * a * d2 + 2 * Exz * (a * (d1 - 0.5) + 0.5);
      f->sxxd_s[c1] = 2.0 * f->eta_s[c1] * Dxx;
      f->szzd_s[c1] = 2.0 * f->eta_s[c1] * Dzz;
      f->sxz[c1] = 2.0 * f->eta_s[c1] * Dxz;
    }
  }
  acc.calls = calls; acc.iters = iters; acc.plastic = plastic; acc.maxit = maxit;
  fill_stats(stats, &acc);
  return acc.status;
}

int orc_sweep(const mdz_model *m, const mdz_materials *mt, const mdz_grid_fields *f, int fu,
              int32_t *in_, int32_t *is_, mdz_sweep_stats *s) {
  return orc_sweep_impl(m, mt, f, fu, in_, is_, s, 0);
}

int orc_sweep_aniso(const mdz_model *m, const mdz_materials *mt, const mdz_grid_fields *f, int fu,
                    int32_t *in_, int32_t *is_, mdz_sweep_stats *s) {
  return orc_sweep_impl(m, mt, f, fu, in_, is_, s, 1);
}

int orc_points(const mdz_model *m, const mdz_materials *mt, const mdz_point_inputs *in,
               mdz_point_outputs *out, int64_t n, int aniso) {
  int status = MDZ_OK;
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) {
    orc_pt pt;
    memset(&pt, 0, sizeof(pt));
    pt.phase = in->phase[i]; pt.G = in->G[i]; pt.T = in->T[i]; pt.P = in->P[i]; pt.d = in->d[i];
    pt.phi = in->phi[i]; pt.X0 = in->X0[i]; pt.Exx = in->Exx[i]; pt.Ezz = in->Ezz[i];
    pt.Exz = in->Exz[i]; pt.Txx0 = in->Txx0[i]; pt.Tzz0 = in->Tzz0[i]; pt.Txz0 = in->Txz0[i];
    pt.dil = in->dil[i]; pt.fric = in->fric[i]; pt.C = in->C[i]; pt.P0 = in->P0[i];
    pt.T0 = in->T0[i]; pt.beta = in->beta[i];
    if (aniso) { pt.lxlz = in->lxlz[i]; pt.lx2 = in->lx2[i]; pt.angle = in->angle[i]; pt.ani_fac = in->ani_fac[i]; }
    pt.post_process = in->post_process; pt.centroid = in->centroid; pt.final_update = in->final_update;
    orc_res r;
    if (aniso) orc_viscosity_concise_aniso(m, mt, &pt, &r);
    else       orc_viscosity_concise(m, mt, &pt, &r);
    double *dst[24] = {out->eta, out->Txx, out->Tzz, out->Txz, out->etaVE, out->VEcoeff, out->Eii_el,
                       out->Eii_pl, out->Eii_pwl, out->Eii_exp, out->Eii_lin, out->Eii_gbs,
                       out->Eii_cst, out->d1, out->X1, out->OverS, out->Pcorr, out->rho,
                       out->div_el, out->div_pl, out->div_r, out->Wtot, out->Wel, out->Wdiss};
    const double src[24] = {r.eta, r.Txx, r.Tzz, r.Txz, r.etaVE, r.VEcoeff, r.Eii_el, r.Eii_pl,
                            r.Eii_pwl, r.Eii_exp, r.Eii_lin, r.Eii_gbs, r.Eii_cst, r.d1, r.X1,
                            r.OverS, r.Pcorr, r.rho, r.div_el, r.div_pl, r.div_r, r.Wtot, r.Wel,
                            r.Wdiss};
    for (int j = 0; j < 24; j++) if (dst[j]) dst[j][i] = src[j];
    if (out->iters) out->iters[i] = r.iters;
    if (out->status) out->status[i] = r.status;
    if (r.status != MDZ_OK) {
#pragma omp critical(orc_pts)
      if (status == MDZ_OK) status = r.status;
    }
  }
  return status;
}

/* ------------------------------------------------------------------------ */
/* RheologicalOperators (StokesRoutines.c:75-410) with the finite-difference */
/* derivatives of DerivativesOnTheFly_n / _s and PhaseRheologyLoop_v1        */
/* (FD_Jacobian.c:48-323).                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {  /* the per-node fields PhaseRheologyLoop_v1 reads */
  const double *const *vol, *const *eta_phase;
  const double *G, *T, *P0, *d, *phi, *X0, *txx0, *tzz0, *txz0, *beta, *dil, *fric, *C;
  double T0;
} orc_fd_node;

typedef struct { double *detadE, *ddivpdE, *danidE, *drhodP; } orc_fd_acc;

/* PhaseRheologyLoop_v1, FD_Jacobian.c:48-100 */
static void orc_phase_loop(const mdz_model *m, const mdz_materials *mt, int aniso, int is_centroid, double sign,
                           double denom, double Exx, double Ezz, double Exz, double P, double ani_fac,
                           double angle, double lx2, double lxlz, int64_t c, const orc_fd_node *nd,
                           orc_fd_acc a) {
  const double ani_vep = 1.0;
  for (int p = 0; p < m->Nb_phases; p++) {
    if (!(fabs(nd->vol[p][c]) > 1e-13)) continue;
    orc_pt pt;
    memset(&pt, 0, sizeof(pt));
    pt.phase = p; pt.G = nd->G[c]; pt.T = nd->T[c]; pt.P = P; pt.d = nd->d[c]; pt.phi = nd->phi[c];
    pt.X0 = nd->X0[c]; pt.Exx = Exx; pt.Ezz = Ezz; pt.Exz = Exz; pt.Txx0 = nd->txx0[c];
    pt.Tzz0 = nd->tzz0[c]; pt.Txz0 = nd->txz0[c]; pt.dil = nd->dil[c]; pt.fric = nd->fric[c];
    pt.C = nd->C[c]; pt.P0 = nd->P0[c]; pt.T0 = nd->T0; pt.beta = nd->beta[c];
    pt.lxlz = lxlz; pt.lx2 = lx2; pt.angle = angle; pt.ani_fac = ani_fac;
    pt.post_process = 0; pt.centroid = is_centroid; pt.final_update = 0;
    orc_res r;
    if (aniso) orc_viscosity_concise_aniso(m, mt, &pt, &r);
    else       orc_viscosity_concise(m, mt, &pt, &r);
    const double eta_vep = r.etaVE;
    if (m->eta_average == 0) *a.detadE += sign * nd->vol[p][c] * eta_vep / (denom);
    if (m->eta_average == 1) *a.detadE += sign * nd->vol[p][c] * eta_vep / (denom) / pow(nd->eta_phase[p][c], 2.0);
    if (m->eta_average == 2) *a.detadE += sign * nd->vol[p][c] * eta_vep / (denom) / nd->eta_phase[p][c];
    *a.danidE += sign * nd->vol[p][c] * ani_vep / (denom);
    if (is_centroid > 0) *a.ddivpdE += sign * nd->vol[p][c] * r.div_pl / (denom);
    if (is_centroid == 2) *a.drhodP += sign * nd->vol[p][c] * r.rho / (denom);
  }
}

/* DerivativesOnTheFly_n (is_centroid = 1, tol 1e-5) and _s (0, 1e-7): central
 * differences in Exx, Ezz, Exz (denominator 4 pert: Gxz = 2 Exz) and P. d[0..3] are
 * d/dExx, d/dEzz, d/dGxz, d/dP of eta; v[], n[] of div_pl and the anisotropy factor. */
static void orc_fd_derivatives(const mdz_model *m, const mdz_materials *mt, int aniso, int centroid,
                               double Exx_ref, double Ezz_ref, double Exz_ref, double P_ref, double ani_fac,
                               double angle, double lx2, double lxlz, int64_t c, const orc_fd_node *nd,
                               double eta_node, double d[4], double v[4], double an[4], double *drhodp) {
  const double tol = centroid ? 1e-5 : 1e-7;
  const double pert_xx = tol * fabs(Exx_ref) + tol / 1e10;
  const double pert_zz = tol * fabs(Ezz_ref) + tol / 1e10;
  const double pert_xz = tol * fabs(Exz_ref) + tol / 1e10;
  const double pert_p = tol * fabs(P_ref) + tol / 1e10;
  double scratch = 0.0;
  for (int s = 0; s < 2; s++) {
    const double sign = s == 0 ? 1.0 : -1.0;
    orc_fd_acc a = {&d[0], centroid ? &v[0] : &scratch, &an[0], NULL};
    orc_phase_loop(m, mt, aniso, centroid ? 1 : 0, sign, 2.0 * pert_xx, Exx_ref + sign * pert_xx, Ezz_ref, Exz_ref,
                   P_ref, ani_fac, angle, lx2, lxlz, c, nd, a);
  }
  for (int s = 0; s < 2; s++) {
    const double sign = s == 0 ? 1.0 : -1.0;
    orc_fd_acc a = {&d[1], centroid ? &v[1] : &scratch, &an[1], NULL};
    orc_phase_loop(m, mt, aniso, centroid ? 1 : 0, sign, 2.0 * pert_zz, Exx_ref, Ezz_ref + sign * pert_zz, Exz_ref,
                   P_ref, ani_fac, angle, lx2, lxlz, c, nd, a);
  }
  for (int s = 0; s < 2; s++) {
    const double sign = s == 0 ? 1.0 : -1.0;
    orc_fd_acc a = {&d[2], centroid ? &v[2] : &scratch, &an[2], NULL};
    orc_phase_loop(m, mt, aniso, centroid ? 1 : 0, sign, 4.0 * pert_xz, Exx_ref, Ezz_ref, Exz_ref + sign * pert_xz,
                   P_ref, ani_fac, angle, lx2, lxlz, c, nd, a);
  }
  for (int s = 0; s < 2; s++) {
    const double sign = s == 0 ? 1.0 : -1.0;
    orc_fd_acc a = {&d[3], centroid ? &v[3] : &scratch, &an[3], centroid ? drhodp : &scratch};
    orc_phase_loop(m, mt, aniso, centroid ? 2 : 0, sign, 2.0 * pert_p, Exx_ref, Ezz_ref, Exz_ref,
                   P_ref + sign * pert_p, ani_fac, angle, lx2, lxlz, c, nd, a);
  }
  if (m->eta_average == 1) for (int k = 0; k < 4; k++) d[k] *= pow(eta_node, 2);
  if (m->eta_average == 2) for (int k = 0; k < 4; k++) d[k] *= eta_node;
}

int orc_operators(const mdz_model *m, const mdz_materials *mt, const mdz_grid_fields *f,
                  mdz_operator_fields *ops, int jacobian, int compressible, int aniso) {
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1;
  const int64_t Nc = (int64_t)Ncx * Ncz, Nv = (int64_t)Nx * Nz;
  const double dt = m->dt;
  int status = MDZ_OK;
  const orc_fd_node nn = {f->phase_perc_n, (const double *const *)f->phase_eta_n, f->mu_n, f->T, f->p0_n, f->d0_n,
                          f->phi0_n, f->X0_n, f->sxxd0, f->szzd0, f->sxz0_n, f->bet_n, f->dil_n, f->fric_n,
                          f->C_n, 0.0};
  const orc_fd_node ns = {f->phase_perc_s, (const double *const *)f->phase_eta_s, f->mu_s, f->T_s, f->p0_s,
                          f->d0_s, f->phi0_s, f->X0_s, f->sxxd0_s, f->szzd0_s, f->sxz0, f->bet_s, f->dil_s,
                          f->fric_s, f->C_s, 0.0};
  /* centroids: StokesRoutines.c:94-120 (Picard), :251-320 (Newton) */
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t k = 0; k < Nc; k++) {
    double *D[8] = {ops->D11_n, ops->D12_n, ops->D13_n, ops->D14_n, ops->D21_n, ops->D22_n, ops->D23_n, ops->D24_n};
    if (f->BCp_type[k] == 30 || f->BCp_type[k] == 31) {
      for (int j = 0; j < 8; j++) D[j][k] = 0.0;
      continue;
    }
    const double eta_vep = f->eta_n[k];
    double ani_vep = 1.0, aniS_vep = 0.0, d1 = 0.0, d2 = 0.0, angle = 0.0, lxlz = 0.0, lx2 = 0.0;
    if (aniso) {
      ani_vep = f->aniso_factor_n[k];
      aniS_vep = 1.0 - 1.0 / ani_vep;
      d1 = f->d1_n[k];
      d2 = f->d2_n[k];
    }
    if (!jacobian) {
      D[0][k] = 2.0 * f->eta_n[k] - 2.0 * aniS_vep * d1 * eta_vep;
      D[1][k] = 2.0 * aniS_vep * d1 * eta_vep;
      D[2][k] = -2.0 * aniS_vep * d2 * eta_vep;
      D[3][k] = 0.0;
      D[4][k] = 2.0 * aniS_vep * d1 * eta_vep;
      D[5][k] = 2.0 * f->eta_n[k] - 2.0 * aniS_vep * d1 * eta_vep;
      D[6][k] = 2.0 * aniS_vep * d2 * eta_vep;
      D[7][k] = 0.0;
      continue;
    }
    const double eta_e = (m->elastic == 1) ? dt * f->mu_n[k] : 1.0;
    const double K = (compressible == 1) ? 1.0 / f->bet_n[k] : 0.0;
    if (aniso) {
      angle = f->angle_n[k];
      const double lay_ang = angle - M_PI / 2.0;
      lxlz = cos(lay_ang) * sin(lay_ang);
      lx2 = cos(lay_ang) * cos(lay_ang);
    }
    double Exx, Ezz, Exz;
    orc_effective_strain_rate(&Exx, &Ezz, &Exz, f->exxd[k], f->ezzd[k], f->exz_n[k], f->sxxd0[k], f->szzd0[k],
                              f->sxz0_n[k], d1, d2, aniS_vep, eta_e, m->elastic);
    const double e_a2 = eta_vep / (ani_vep * ani_vep);
    const double Gxz = 2.0 * Exz;
    const double Dxx = Exx * (1.0 - aniS_vep * d1) + Ezz * aniS_vep * d1 - Gxz * aniS_vep * d2;
    const double Dzz = Ezz * (1.0 - aniS_vep * d1) + Exx * aniS_vep * d1 + Gxz * aniS_vep * d2;
    const double Axx = -Exx * d1 * e_a2 + Ezz * d1 * e_a2 - Gxz * d2 * e_a2;
    const double Azz = Exx * d1 * e_a2 - Ezz * d1 * e_a2 + Gxz * d2 * e_a2;
    double de[4] = {0, 0, 0, 0}, dv[4] = {0, 0, 0, 0}, da[4] = {0, 0, 0, 0}, drhodp = 0.0;
    orc_fd_node nk = nn;
    nk.T0 = f->T0_n[k];
    orc_fd_derivatives(m, mt, aniso, 1, Exx, Ezz, Exz, f->p_in[k], ani_vep, angle, lx2, lxlz, k, &nk, f->eta_n[k],
                       de, dv, da, &drhodp);
    if (ops->drhodp_n) ops->drhodp_n[k] = drhodp;
    D[0][k] = 2.0 * (1.0 - aniS_vep * d1) * eta_vep + 2.0 * de[0] * Dxx - K * dt * dv[0] + 2.0 * da[0] * Axx;
    D[1][k] = 2.0 * aniS_vep * d1 * eta_vep + 2.0 * de[1] * Dxx - K * dt * dv[1] + 2.0 * da[1] * Axx;
    D[2][k] = -2.0 * aniS_vep * d2 * eta_vep + 2.0 * de[2] * Dxx - K * dt * dv[2] + 2.0 * da[2] * Axx;
    D[3][k] = 2.0 * de[3] * Dxx - K * dt * dv[3] + 2.0 * da[3] * Axx;
    D[4][k] = 2.0 * aniS_vep * d1 * eta_vep + 2.0 * de[0] * Dzz - K * dt * dv[0] + 2.0 * da[0] * Azz;
    D[5][k] = 2.0 * (1.0 - aniS_vep * d1) * eta_vep + 2.0 * de[1] * Dzz - K * dt * dv[1] + 2.0 * da[1] * Azz;
    D[6][k] = 2.0 * aniS_vep * d2 * eta_vep + 2.0 * de[2] * Dzz - K * dt * dv[2] + 2.0 * da[2] * Azz;
    D[7][k] = 2.0 * de[3] * Dzz - K * dt * dv[3] + 2.0 * da[3] * Azz;
  }
  /* vertices: StokesRoutines.c:170-200 (Picard), :325-380 (Newton) */
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t k = 0; k < Nv; k++) {
    double *D[4] = {ops->D31_s, ops->D32_s, ops->D33_s, ops->D34_s};
    if (f->BCg_type[k] == 30) {
      for (int j = 0; j < 4; j++) D[j][k] = 0.0;
      continue;
    }
    const double eta_vep = f->eta_s[k];
    double ani_vep = 1.0, aniS_vep = 0.0, d1 = 0.0, d2 = 0.0, angle = 0.0, lxlz = 0.0, lx2 = 0.0;
    if (aniso) {
      ani_vep = f->aniso_factor_s[k];
      aniS_vep = 1.0 - 1.0 / ani_vep;
      d1 = f->d1_s[k];
      d2 = f->d2_s[k];
    }
    if (!jacobian) {
      D[0][k] = -2.0 * aniS_vep * d2 * eta_vep;
      D[1][k] = 2.0 * aniS_vep * d2 * eta_vep;
      D[2][k] = eta_vep + 2.0 * aniS_vep * (d1 - 0.5) * eta_vep;
      D[3][k] = 0.0;
      continue;
    }
    const double eta_e = (m->elastic == 1) ? dt * f->mu_s[k] : 1.0;
    if (aniso) {
      angle = f->angle_s[k];
      const double lay_ang = angle - M_PI / 2.0;
      lxlz = cos(lay_ang) * sin(lay_ang);
      lx2 = cos(lay_ang) * cos(lay_ang);
    }
    double Exx, Ezz, Exz;
    orc_effective_strain_rate(&Exx, &Ezz, &Exz, f->exxd_s[k], f->ezzd_s[k], f->exz[k], f->sxxd0_s[k],
                              f->szzd0_s[k], f->sxz0[k], d1, d2, aniS_vep, eta_e, m->elastic);
    const double e_a2 = eta_vep / (ani_vep * ani_vep);
    const double Gxz = 2. * Exz;
    const double Dxz = -Exx * aniS_vep * d2 + Ezz * aniS_vep * d2 + Gxz * (aniS_vep * (d1 - 0.5) + 0.5);
    const double Axz = -Exx * d2 * e_a2 + Ezz * d2 * e_a2 + Gxz * e_a2 * (d1 - 0.5);
    double de[4] = {0, 0, 0, 0}, dv[4] = {0, 0, 0, 0}, da[4] = {0, 0, 0, 0};
    orc_fd_derivatives(m, mt, aniso, 0, Exx, Ezz, Exz, f->P_s[k], ani_vep, angle, lx2, lxlz, k, &ns, f->eta_s[k],
                       de, dv, da, NULL);
    D[0][k] = -2.0 * aniS_vep * d2 * eta_vep + 2.0 * de[0] * Dxz + 2.0 * da[0] * Axz;
    D[1][k] = 2.0 * aniS_vep * d2 * eta_vep + 2.0 * de[1] * Dxz + 2.0 * da[1] * Axz;
    D[2][k] = (2.0 * aniS_vep * (d1 - 0.5) + 1.0) * eta_vep + 2.0 * de[2] * Dxz + 2.0 * da[2] * Axz;
    D[3][k] = 2.0 * de[3] * Dxz + 2.0 * da[3] * Axz;
    if (isnan(D[3][k]) || isinf(D[3][k])) {  /* :384-385 */
#pragma omp critical(orc_ops)
      if (status == MDZ_OK) status = MDZ_ENONFINITE;
    }
  }
  return status;
}

/* ------------------------------------------------------------------------ */
/* StrainRateComponents, RheologyDensity.c:2001-2097: the reference's four    */
/* passes in its order -- centroid divergence and deviatoric normal rates,    */
/* vertex shear rate and spin (wxz is left alone at air vertices), their      */
/* 4-vertex centroid averages, and the vertex interpolation of exxd, ezzd and */
/* div_u (InterpCentroidsToVerticesDouble, restated above).                   */
/* ------------------------------------------------------------------------ */
int orc_strain_rates(const mdz_model *m, double dx, double dz, int out_of_plane, double compressible,
                     mdz_strain_rate_fields *sr) {
  if (m->Nx < 2 || m->Nz < 2) return MDZ_EINVAL;
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1;
  const double oop = (out_of_plane == 1) ? 1.0 : 0.0;
  const double *u = sr->u_in, *v = sr->v_in;
  const signed char *BCp = sr->BCp_type, *BCg = sr->BCg_type;
#pragma omp parallel for
  for (int c0 = 0; c0 < Ncx * Ncz; c0++) {
    const int k = c0 % Ncx, l = c0 / Ncx, c1 = k + l * Nx, c2 = k + l * (Nx + 1);
    sr->div_u[c0] = 0.0;
    sr->exxd[c0] = 0.0;
    sr->ezzd[c0] = 0.0;
    if (BCp[c0] != 30 && BCp[c0] != 31) {
      const double dvxdx = (u[c1 + 1 + Nx] - u[c1 + Nx]) / dx;
      const double dvzdz = (v[c2 + Nx + 1 + 1] - v[c2 + 1]) / dz;
      const double dvydy = oop * 0.5 * (dvxdx + dvzdz);
      sr->div_u[c0] = dvxdx + dvzdz + dvydy;
      sr->exxd[c0] = dvxdx - compressible * 1.0 / 3.0 * sr->div_u[c0];
      sr->ezzd[c0] = dvzdz - compressible * 1.0 / 3.0 * sr->div_u[c0];
    }
  }
#pragma omp parallel for
  for (int c1 = 0; c1 < Nx * Nz; c1++) {
    const int k = c1 % Nx, l = c1 / Nx, c2 = k + l * (Nx + 1);
    sr->exz[c1] = 0.0;
    if (BCg[c1] != 30) {
      const double dvxdz = (u[c1 + Nx] - u[c1]) / dz;
      const double dvzdx = (v[c2 + 1] - v[c2]) / dx;
      sr->exz[c1] = 0.5 * (dvxdz + dvzdx);
      sr->wxz[c1] = 0.5 * (dvzdx - dvxdz);
    }
  }
#pragma omp parallel for
  for (int c0 = 0; c0 < Ncx * Ncz; c0++) {
    const int k = c0 % Ncx, l = c0 / Ncx, c1 = k + l * Nx;
    const int corner[4] = {c1, c1 + 1, c1 + Nx, c1 + Nx + 1};
    sr->exz_n[c0] = 0.0;
    sr->wxz_n[c0] = 0.0;
    if (BCp[c0] != 30 && BCp[c0] != 31) {
      for (int q = 0; q < 4; q++)
        if (BCg[corner[q]] != 30) sr->exz_n[c0] += 0.25 * sr->exz[corner[q]];
      for (int q = 0; q < 4; q++)
        if (BCg[corner[q]] != 30) sr->wxz_n[c0] += 0.25 * sr->wxz[corner[q]];
    }
  }
  orc_interp_c2v(m, sr->exxd, BCp, BCg, sr->exxd_s);
  orc_interp_c2v(m, sr->ezzd, BCp, BCg, sr->ezzd_s);
  orc_interp_c2v(m, sr->div_u, BCp, BCg, sr->div_u_s);
  return MDZ_OK;
}

/* ------------------------------------------------------------------------ */
/* Softening (RheologyDensity.c:1432-1532) as CohesionFrictionDilationGrid    */
/* (:1539-1628) applies it, after P2Mastah: arithmetic phase average          */
/* (average = 0, :1541), marker noise on the cohesion, zeros at air nodes.    */
/* ------------------------------------------------------------------------ */
static void orc_soften(const mdz_prep_materials *m, int p, int style, double s, double *fric, double *dil,
                       double *C) {
  *fric = m->phi[p];
  *dil = m->psi[p];
  *C = m->C[p];
  const double dstrain = m->pls_end[p] - m->pls_start[p];
  if (style == 1) {
    const double mu_strain = 0.5 * (m->pls_end[p] + m->pls_start[p]);
    if (m->phi_soft[p] == 1) {
      const double dfric = m->phi[p] - m->phi_end[p];
      double f = m->phi[p] - dfric / 2.0 * erfc(-(s - mu_strain) / dstrain) - m->phi_end[p];
      const double f0 = m->phi[p] - dfric / 2.0 * erfc(-(0.0 - mu_strain) / dstrain) - m->phi_end[p];
      *fric = f * dfric / f0 + m->phi_end[p];
    }
    if (m->psi_soft[p] == 1) {
      const double ddil = m->psi[p] - m->psi_end[p];
      double d = m->psi[p] - ddil / 2.0 * erfc(-(s - mu_strain) / dstrain) - m->psi_end[p];
      const double d0 = m->psi[p] - ddil / 2.0 * erfc(-(0.0 - mu_strain) / dstrain) - m->psi_end[p];
      *dil = d * ddil / d0 + m->psi_end[p];
    }
    if (m->coh_soft[p] == 1) {
      const double dcoh = m->C[p] - m->C_end[p];
      double c = m->C[p] - dcoh / 2.0 * erfc(-(s - mu_strain) / dstrain) - m->C_end[p];
      const double c0 = m->C[p] - dcoh / 2.0 * erfc(-(0.0 - mu_strain) / dstrain) - m->C_end[p];
      *C = c * dcoh / c0 + m->C_end[p];
    }
  } else if (style == 2) {
    *C = fmax(m->C[p] + m->H_c[p] * s, m->C_end[p]);
  } else {
    if (s < m->pls_start[p]) {
      if (m->phi_soft[p] == 1) *fric = m->phi[p];
      if (m->psi_soft[p] == 1) *dil = m->psi[p];
      if (m->coh_soft[p] == 1) *C = m->C[p];
    }
    if (s >= m->pls_end[p]) {
      if (m->phi_soft[p] == 1) *fric = m->phi_end[p];
      if (m->psi_soft[p] == 1) *dil = m->psi_end[p];
      if (m->coh_soft[p] == 1) *C = m->C_end[p];
    }
    if (s >= m->pls_start[p] && s < m->pls_end[p]) {
      if (m->phi_soft[p] == 1) *fric = m->phi[p] + (m->phi_end[p] - m->phi[p]) / dstrain * s;
      if (m->psi_soft[p] == 1) *dil = m->psi[p] + (m->psi_end[p] - m->psi[p]) / dstrain * s;
      if (m->coh_soft[p] == 1) *C = m->C[p] + (m->C_end[p] - m->C[p]) / dstrain * s;
    }
  }
}

static void orc_soften_node(const mdz_prep_materials *m, int np, int style, int noise, const double *const *perc,
                            int64_t i, int solid, double s, const double *nz, double *fric, double *dil, double *C) {
  fric[i] = 0.0;
  dil[i] = 0.0;
  C[i] = 0.0;
  if (!solid) return;
  for (int p = 0; p < np; p++) {
    double f, d, c;
    orc_soften(m, p, style, s, &f, &d, &c);
    fric[i] += perc[p][i] * f;
    dil[i] += perc[p][i] * d;
    C[i] += perc[p][i] * c;
  }
  if (noise == 1) C[i] += nz[i] * C[i];
}

int orc_softening(const mdz_model *md, const mdz_prep_materials *m, mdz_prep_fields *f, int smooth_softening,
                  int hardening_modulus, int marker_noise) {
  if (md->Nx < 2 || md->Nz < 2 || md->Nb_phases < 1 || md->Nb_phases > MDZ_MAX_PHASES) return MDZ_EINVAL;
  const int64_t Nc = (int64_t)(md->Nx - 1) * (md->Nz - 1), Nv = (int64_t)md->Nx * md->Nz;
  int style = 0;
  if (smooth_softening == 1) style = 1;
  if (hardening_modulus == 1) style = 2;
#pragma omp parallel for
  for (int64_t c0 = 0; c0 < Nc; c0++)
    orc_soften_node(m, md->Nb_phases, style, marker_noise, f->phase_perc_n, c0,
                    f->BCp_type[c0] != 30 && f->BCp_type[c0] != 31, f->strain_pl_n[c0], f->noise_n, f->fric_n,
                    f->dil_n, f->C_n);
#pragma omp parallel for
  for (int64_t c1 = 0; c1 < Nv; c1++)
    orc_soften_node(m, md->Nb_phases, style, marker_noise, f->phase_perc_s, c1, f->BCg_type[c1] != 30,
                    f->strain_pl_s[c1], f->noise_s, f->fric_s, f->dil_s, f->C_s);
  return MDZ_OK;
}

/* ShearModCompExpGrid, RheologyDensity.c:1634-1755 (average = 1, :1637). */
int orc_shear_modulus(const mdz_model *md, const mdz_prep_materials *m, mdz_prep_fields *f) {
  if (md->Nx < 2 || md->Nz < 2 || md->Nb_phases < 1 || md->Nb_phases > MDZ_MAX_PHASES) return MDZ_EINVAL;
  const int Nx = md->Nx, Nz = md->Nz, Ncx = Nx - 1, Ncz = Nz - 1, np = md->Nb_phases;
  int64_t bad = -1;
  for (int64_t c0 = 0; c0 < (int64_t)Ncx * Ncz; c0++) {
    f->mu_n[c0] = 0.0;
    f->bet_n[c0] = 0.0;
    f->alp[c0] = 0.0;
    if (f->BCp_type[c0] != 30 && f->BCp_type[c0] != 31) {
      for (int p = 0; p < np; p++) {
        f->mu_n[c0] += f->phase_perc_n[p][c0] * 1.0 / m->G[p];
        f->bet_n[c0] += f->phase_perc_n[p][c0] * 1.0 / m->bet[p];
        f->alp[c0] += f->phase_perc_n[p][c0] * m->alp[p];
      }
      f->mu_n[c0] = 1.0 / f->mu_n[c0];
      f->bet_n[c0] = 1.0 / f->bet_n[c0];
    }
    if (isinf(f->mu_n[c0]) && bad < 0) bad = c0;
  }
  for (int64_t c1 = 0; c1 < (int64_t)Nx * Nz; c1++) {
    f->mu_s[c1] = 0.0;
    f->bet_s[c1] = 0.0;
    if (f->BCg_type[c1] != 30) {
      for (int p = 0; p < np; p++) {
        f->mu_s[c1] += f->phase_perc_s[p][c1] * 1.0 / m->G[p];
        f->bet_s[c1] += f->phase_perc_s[p][c1] * 1.0 / m->bet[p];
      }
      f->mu_s[c1] = 1.0 / f->mu_s[c1];
      f->bet_s[c1] = 1.0 / f->bet_s[c1];
    }
  }
  if (md->periodic_x == 1) {
    for (int l = 0; l < Nz; l++) {
      const int64_t c1 = (int64_t)l * Nx + Nx - 1, c = (int64_t)l * Nx;
      double av = 0.5 * (f->mu_s[c1] + f->mu_s[c]);
      f->mu_s[c1] = av; f->mu_s[c] = av;
      av = 0.5 * (f->bet_s[c1] + f->bet_s[c]);
      f->bet_s[c1] = av; f->bet_s[c] = av;
    }
  }
  return bad >= 0 ? MDZ_ESHEAR_INF : MDZ_OK;
}

/* ------------------------------------------------------------------------ */
/* UpdateParticleStress, RheologyParticles.c:1725-2004, for subgrid_diffusion */
/* 0 or 1, with the grid <-> marker interpolations it calls.                  */
/* ------------------------------------------------------------------------ */

/* The four centroid corners of a marker in the ghost-extended centroid frame
 * (Interp_Grid2P_centroids2, ParticleRoutines.c:1349-1514; Centers2Particle, :270-430):
 * Nx, Nz count centroids, X/Z hold Nx+1 / Nz+1 coordinates (one ghost at each end).
 * Returns 0, or -1 where the marker lies outside every case the reference handles. */
static int orc_cell_corners(double x, double z, const double *X, const double *Z, int Nx, int Nz, double dx,
                            double dz, int per, int *jp, int *ip, int c[4]) {
  const int j = (int)ceil((x - X[0]) / dx) - 1, i = (int)ceil((z - Z[0]) / dz) - 1;
  int SW, SE, NW, NE;
  *jp = j; *ip = i;
  if (j > 0 && j < Nx && i > 0 && i < Nz) {
    SW = (j - 1) + (i - 1) * Nx; SE = SW + 1; NW = SW + Nx; NE = NW + 1;
  } else if (j == 0 && i > 0 && i < Nz) {
    if (per == 1) { SW = (Nx - 1) + (i - 1) * Nx; SE = (i - 1) * Nx; NW = (Nx - 1) + i * Nx; NE = i * Nx; }
    else { SW = SE = (i - 1) * Nx; NW = NE = i * Nx; }
  } else if (j == Nx && i > 0 && i < Nz) {
    if (per == 1) { SW = (Nx - 1) + (i - 1) * Nx; SE = (i - 1) * Nx; NW = (Nx - 1) + i * Nx; NE = i * Nx; }
    else { SW = SE = (Nx - 1) + (i - 1) * Nx; NW = NE = (Nx - 1) + i * Nx; }
  } else if (i == 0 && j > 0 && j < Nx) {
    SW = NW = j - 1; SE = NE = j;
  } else if (i == Nz && j > 0 && j < Nx) {
    SW = NW = (j - 1) + (Nz - 1) * Nx; SE = NE = SW + 1;
  } else if (i == 0 && j == 0) {
    if (per == 1) { SW = NW = Nx - 1; SE = NE = 0; }
    else SW = SE = NW = NE = 0;
  } else if (i == 0 && j == Nx) {
    if (per == 1) { SW = NW = Nx - 1; SE = NE = 0; }
    else SW = SE = NW = NE = Nx - 1;
  } else if (i == Nz && j == 0) {
    if (per == 1) { SW = NW = (Nx - 1) + (Nz - 1) * Nx; SE = NE = (Nz - 1) * Nx; }
    else SW = SE = NW = NE = (Nz - 1) * Nx;
  } else if (i == Nz && j == Nx) {
    if (per == 1) { SW = NW = (Nx - 1) + (Nz - 1) * Nx; SE = NE = (Nz - 1) * Nx; }
    else SW = SE = NW = NE = (Nx - 1) + (Nz - 1) * Nx;
  } else {
    return -1;
  }
  c[0] = SW; c[1] = SE; c[2] = NW; c[3] = NE;
  return 0;
}

static int orc_air(signed char t) { return t == 30 || t == 31; }

/* the bilinear weights of the four corners, in the reference's order (SW, SE, NW, NE) */
static void orc_weights(double dxm, double dzm, double dx, double dz, double w[4]) {
  w[0] = (1.0 - dxm / dx) * (1.0 - dzm / dz);
  w[1] = (dxm / dx) * (1.0 - dzm / dz);
  w[2] = (1.0 - dxm / dx) * (dzm / dz);
  w[3] = (dxm / dx) * (dzm / dz);
}

/* Interp_Grid2P_centroids2 (ParticleRoutines.c:1332-1573) for one active marker: an air
 * corner lends its weight to the corner across (SW<->NW, SE<->NE); divided by the weight
 * sum when that exceeds 1e-13.  `field(c)` is the centroid value. */
static double orc_c2p_sub(const double *F, const signed char *tag, const int c[4], const double w[4]) {
  const int alt[4] = {c[2], c[3], c[0], c[1]};
  double v = 0.0, sw = 0.0;
  for (int q = 0; q < 4; q++) {
    v += w[q] * F[orc_air(tag[c[q]]) ? alt[q] : c[q]];
    sw += w[q];
  }
  if (sw > 1e-13) v /= sw;
  return v;
}

/* Centers2Particle / Vertices2Particle (ParticleRoutines.c:262-455, :464-536): air corners
 * are left out. */
static double orc_c2p_skip(const double *F, const signed char *tag, const int c[4], const double w[4]) {
  double v = 0.0, sw = 0.0;
  for (int q = 0; q < 4; q++)
    if (!orc_air(tag[c[q]])) { v += w[q] * F[c[q]]; sw += w[q]; }
  if (sw > 1e-13) v /= sw;
  return v;
}

/* Interp_Grid2P (ParticleRoutines.c:1223-1321) for one active marker: the vertex cell of
 * (x - X[0]) / dx clamped to the grid (beyond it in x the reference exits with 89), the
 * weights of |x - X[j]|, an air corner (30, 31) replaced by the corner across, no
 * normalisation. */
static double orc_v2p(const double *F, const signed char *tag, double x, double z, const double *X, const double *Z,
                      int Nx, int Nz, double dx, double dz, int *status) {
  int j = (int)ceil((x - X[0]) / dx) - 1;
  if (j < 0) j = 0;
  if (j > Nx - 2) { j = Nx - 2; *status = MDZ_EMARKER_OUT; }
  int i = (int)ceil((z - Z[0]) / dz) - 1;
  if (i < 0) i = 0;
  if (i > Nz - 2) i = Nz - 2;
  const int cv[4] = {j + i * Nx, j + i * Nx + 1, j + (i + 1) * Nx, j + (i + 1) * Nx + 1};
  const int alt[4] = {cv[2], cv[3], cv[0], cv[1]};
  double w[4];
  orc_weights(fabs(x - X[j]), fabs(z - Z[i]), dx, dz, w);
  double v = 0.0;
  for (int q = 0; q < 4; q++) v += w[q] * F[orc_air(tag[cv[q]]) ? alt[q] : cv[q]];
  return v;
}

/* P2Mastah's sums (ParticleRoutines.c:2288-2575) over the active markers in order, on a
 * grid of Nxn x Nzn nodes at X, Z: WM += w and, when BM is given, BM += val * w at the
 * marker's nearest node and, with the 9-node stencil, the eight around it (N, S, E, W,
 * SW, NW, NE, SE, as in the reference), wrapped in x when periodic.  One thread of the
 * reference sums in this order. */
static void orc_p2m(const mdz_markers *mk, const double *val, const double *X, const double *Z, int Nxn, int Nzn,
                    double dx, double dz, int stencil, int per, double *WM, double *BM) {
  const double dx_itp = (stencil == 9) ? 3.0 * dx / 2.0 : dx / 2.0;
  const double dz_itp = (stencil == 9) ? 3.0 * dz / 2.0 : dz / 2.0;
  for (int64_t p = 0; p < mk->n; p++) {
    if (mk->phase[p] == -1) continue;
    const double x = mk->x[p], z = mk->z[p], mv = val ? val[p] : 0.0;
    int ip = (int)ceil((x - X[0]) / dx + 0.5) - 1, jp = (int)ceil((z - Z[0]) / dz + 0.5) - 1;
    if (ip < 0) ip = 0;
    if (ip > Nxn - 1) ip = Nxn - 1;
    if (jp < 0) jp = 0;
    if (jp > Nzn - 1) jp = Nzn - 1;
    const double Xp = X[ip], Zp = Z[jp];
#define ORC_W(cond, kk, xx, zz)                                                        \
    if (cond) {                                                                        \
      const int64_t kp_ = (kk);                                                        \
      const double w_ = (1.0 - fabs(xx - x) / dx_itp) * (1.0 - fabs(zz - z) / dz_itp); \
      WM[kp_] += w_;                                                                   \
      if (BM) BM[kp_] += mv * w_;                                                      \
    }
    ORC_W(1, ip + (int64_t)jp * Nxn, Xp, Zp);
    if (stencil == 9) {
      const int peE = (ip == Nxn - 1 && per == 1), peW = (ip == 0 && per == 1);
      const double xE = Xp + dx, xW = Xp - dx, zN = Zp + dz, zS = Zp - dz;
      const int kE = ip + 1 - peE * Nxn, kW = ip - 1 + peW * Nxn;
      ORC_W(jp < Nzn - 1, ip + (int64_t)(jp + 1) * Nxn, Xp, zN);
      ORC_W(jp > 0, ip + (int64_t)(jp - 1) * Nxn, Xp, zS);
      ORC_W(ip < Nxn - 1 || peE, kE + (int64_t)jp * Nxn, xE, Zp);
      ORC_W(ip > 0 || peW, kW + (int64_t)jp * Nxn, xW, Zp);
      ORC_W(jp > 0 && (ip > 0 || peW), kW + (int64_t)(jp - 1) * Nxn, xW, zS);
      ORC_W(jp < Nzn - 1 && (ip > 0 || peW), kW + (int64_t)(jp + 1) * Nxn, xW, zN);
      ORC_W(jp < Nzn - 1 && (ip < Nxn - 1 || peE), kE + (int64_t)(jp + 1) * Nxn, xE, zN);
      ORC_W(jp > 0 && (ip < Nxn - 1 || peE), kE + (int64_t)(jp - 1) * Nxn, xE, zS);
    }
#undef ORC_W
  }
}

/* P2Mastah's node values (flag 1; :2603-2641): BM / WM where |WM| reaches 1e-30 away
 * from air (its reciprocal for avg 1, its exponential for avg 2), else F keeps its value;
 * with periodic x the two ends of each row of a vertex field take their mean. */
static void orc_p2m_nodes_avg(double *F, const double *WM, const double *BM, const signed char *tag, int Nxn,
                              int Nzn, int vertex, int per, int avg) {
  for (int64_t i = 0; i < (int64_t)Nxn * Nzn; i++)
    if (!(fabs(WM[i]) < 1e-30 || orc_air(tag[i]))) {
      F[i] = BM[i] / WM[i];
      if (avg == 1) F[i] = 1.0 / F[i];
      if (avg == 2) F[i] = exp(F[i]);
    }
  if (vertex && per == 1)
    for (int l = 0; l < Nzn; l++) {
      const int64_t c1 = (int64_t)l * Nxn + Nxn - 1, c = (int64_t)l * Nxn;
      const double av = 0.5 * (F[c1] + F[c]);
      F[c1] = av; F[c] = av;
    }
}

static void orc_p2m_nodes(double *F, const double *WM, const double *BM, const signed char *tag, int Nxn, int Nzn,
                          int vertex, int per) {
  orc_p2m_nodes_avg(F, WM, BM, tag, Nxn, Nzn, vertex, per, 0);
}

/* P2Mastah of a marker array (flag 1, prop 0) onto the centroids and/or vertices, avg 0,
 * 1 or 2 (ParticleRoutines.c:2170-2665): the values go in as v, 1/v or log v
 * (:2346-2352) and the node means come back as m, 1/m or exp m. */
int orc_p2mastah(const mdz_model *m, const mdz_marker_grid *g, const mdz_markers *mk, const double *val, int avg,
                 int stencil, double *node_n, double *node_s) {
  if (m->Nx < 2 || m->Nz < 2 || avg < 0 || avg > 2 || (stencil != 1 && stencil != 9)) return MDZ_EINVAL;
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1, per = m->periodic_x;
  const int64_t Nc = (int64_t)Ncx * Ncz, Nv = (int64_t)Nx * Nz, n = mk->n;
  for (int64_t p = 0; p < n; p++)
    if (mk->phase[p] != -1 && (mk->phase[p] < 0 || mk->phase[p] >= m->Nb_phases)) return MDZ_EINVAL;
  double *v = malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  for (int64_t p = 0; p < n; p++) v[p] = avg == 1 ? 1.0 / val[p] : (avg == 2 ? log(val[p]) : val[p]);
  if (node_n) {
    double *s = calloc(2 * (size_t)Nc, sizeof(double));
    orc_p2m(mk, v, g->xc_coord, g->zc_coord, Ncx, Ncz, g->dx, g->dz, stencil, per, s, s + Nc);
    orc_p2m_nodes_avg(node_n, s, s + Nc, g->BCp_type, Ncx, Ncz, 0, per, avg);
    free(s);
  }
  if (node_s) {
    double *s = calloc(2 * (size_t)Nv, sizeof(double));
    orc_p2m(mk, v, g->xg_coord, g->zg_coord, Nx, Nz, g->dx, g->dz, stencil, per, s, s + Nv);
    orc_p2m_nodes_avg(node_s, s, s + Nv, g->BCg_type, Nx, Nz, 1, per, avg);
    free(s);
  }
  free(v);
  return MDZ_OK;
}

/* UpdateParticleStress with subgrid_diffusion 2 (RheologyParticles.c:1811-1903): the old
 * grid stresses and the vertex viscosity go to the markers; each active marker relaxes
 * towards the old stress over its Maxwell time (the subgrid increment); P2Mastah takes
 * the subgrid increments to the grid; what remains of the grid's increment comes back
 * to the markers, and both are added to the marker stress. */
static int orc_subgrid_stress(const mdz_model *m, const mdz_marker_opts *o, mdz_marker_grid *g, mdz_markers *mk,
                              int status) {
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1, per = m->periodic_x;
  const int64_t Nc = (int64_t)Ncx * Ncz, Nv = (int64_t)Nx * Nz, n = mk->n;
  const double dx = g->dx, dz = g->dz, dt = m->dt, d = 1.0;
  double *ms = calloc(3 * (size_t)(n > 0 ? n : 1), sizeof(double)); /* dtxxms, dtzzms, dtxzms */
  double *gs = calloc(4 * (size_t)Nc + 2 * (size_t)Nv, sizeof(double)); /* 4 centroid, 2 vertex fields */
  double *wmc = calloc(3 * (size_t)Nc, sizeof(double)), *wmv = calloc(2 * (size_t)Nv, sizeof(double));
  double *dtxxms = ms, *dtzzms = ms + n, *dtxzms = ms + 2 * n;
  double *dtxxgs = gs, *dtzzgs = gs + Nc, *dtxzgs = gs + 2 * Nc, *dtxxgr = gs + 2 * Nc + Nv,
         *dtzzgr = dtxxgr + Nc, *dtxzgr = dtzzgr + Nc;
  for (int64_t p = 0; p < n; p++) {
    if (mk->phase[p] == -1) continue;
    const int ph = mk->phase[p];
    if (ph < 0 || ph >= m->Nb_phases) { status = MDZ_EINVAL; continue; }
    const double x = mk->x[p], z = mk->z[p];
    int jp, ip, c[4];
    double w[4], txxm0 = 0.0, tzzm0 = 0.0;
    if (orc_cell_corners(x, z, g->xvz_coord, g->zvx_coord, Ncx, Ncz, dx, dz, per, &jp, &ip, c) != 0) {
      status = MDZ_EMARKER_OUT;
    } else {
      orc_weights(x - g->xvz_coord[jp], z - g->zvx_coord[ip], dx, dz, w);
      txxm0 = orc_c2p_sub(g->sxxd0, g->BCp_type, c, w);
      tzzm0 = orc_c2p_sub(g->szzd0, g->BCp_type, c, w);
      if (isinf(txxm0) || isinf(tzzm0)) status = MDZ_ENONFINITE; /* ParticleRoutines.c:1565-1569 */
    }
    const double txzm0 = orc_v2p(g->sxz0, g->BCg_type, x, z, g->xg_coord, g->zg_coord, Nx, Nz, dx, dz, &status);
    const double etam = orc_v2p(g->eta_phys_s, g->BCg_type, x, z, g->xg_coord, g->zg_coord, Nx, Nz, dx, dz, &status);
    const double dtaum = etam / o->G[ph];
    const double f = 1.0 - exp(-d * dt / dtaum);
    dtxxms[p] = -(mk->sxxd[p] - txxm0) * f;
    dtzzms[p] = -(mk->szzd[p] - tzzm0) * f;
    dtxzms[p] = -(mk->sxz[p] - txzm0) * f;
    if (isinf(dtxxms[p]) || isnan(dtxxms[p])) status = MDZ_ENONFINITE; /* :1846-1855, exit 1 */
  }
  /* subgrid increments markers -> grid, three P2Mastah calls (:1859-1861) */
  orc_p2m(mk, dtxxms, g->xc_coord, g->zc_coord, Ncx, Ncz, dx, dz, o->interp_stencil, per, wmc, wmc + Nc);
  orc_p2m_nodes(dtxxgs, wmc, wmc + Nc, g->BCp_type, Ncx, Ncz, 0, per);
  memset(wmc, 0, 2 * (size_t)Nc * sizeof(double));
  orc_p2m(mk, dtzzms, g->xc_coord, g->zc_coord, Ncx, Ncz, dx, dz, o->interp_stencil, per, wmc, wmc + Nc);
  orc_p2m_nodes(dtzzgs, wmc, wmc + Nc, g->BCp_type, Ncx, Ncz, 0, per);
  orc_p2m(mk, dtxzms, g->xg_coord, g->zg_coord, Nx, Nz, dx, dz, o->interp_stencil, per, wmv, wmv + Nv);
  orc_p2m_nodes(dtxzgs, wmv, wmv + Nv, g->BCg_type, Nx, Nz, 1, per);
  /* remaining increments on the grid (:1864-1872) */
  for (int64_t c0 = 0; c0 < Nc; c0++)
    if (!orc_air(g->BCp_type[c0])) {
      dtxxgr[c0] = (g->sxxd[c0] - g->sxxd0[c0]) - dtxxgs[c0];
      dtzzgr[c0] = (g->szzd[c0] - g->szzd0[c0]) - dtzzgs[c0];
    }
  for (int64_t c1 = 0; c1 < Nv; c1++)
    if (g->BCg_type[c1] != 30) dtxzgr[c1] = (g->sxz[c1] - g->sxz0[c1]) - dtxzgs[c1];
  /* remaining increments grid -> markers and the final update (:1875-1885) */
  for (int64_t p = 0; p < n; p++) {
    if (mk->phase[p] == -1) continue;
    const double x = mk->x[p], z = mk->z[p];
    int jp, ip, c[4];
    double w[4], dtxxmr = 0.0, dtzzmr = 0.0;
    if (orc_cell_corners(x, z, g->xvz_coord, g->zvx_coord, Ncx, Ncz, dx, dz, per, &jp, &ip, c) == 0) {
      orc_weights(x - g->xvz_coord[jp], z - g->zvx_coord[ip], dx, dz, w);
      dtxxmr = orc_c2p_sub(dtxxgr, g->BCp_type, c, w);
      dtzzmr = orc_c2p_sub(dtzzgr, g->BCp_type, c, w);
      if (isinf(dtxxmr) || isinf(dtzzmr)) status = MDZ_ENONFINITE;
    }
    const double dtxzmr = orc_v2p(dtxzgr, g->BCg_type, x, z, g->xg_coord, g->zg_coord, Nx, Nz, dx, dz, &status);
    mk->sxxd[p] = mk->sxxd[p] + dtxxms[p] + dtxxmr;
    mk->szzd[p] = mk->szzd[p] + dtzzms[p] + dtzzmr;
    mk->sxz[p] = mk->sxz[p] + dtxzms[p] + dtxzmr;
  }
  free(ms); free(gs); free(wmc); free(wmv);
  return status;
}

int orc_marker_stress(const mdz_model *m, const mdz_marker_opts *o, mdz_marker_grid *g, mdz_markers *mk) {
  if (m->Nx < 2 || m->Nz < 2) return MDZ_EINVAL;
  if (o->elastic == 1 && o->subgrid_diffusion == 2 &&
      (!o->G || !g->xc_coord || !g->zc_coord || !g->eta_phys_s || m->Nb_phases < 1))
    return MDZ_EINVAL;
  const int Nx = m->Nx, Nz = m->Nz, Ncx = Nx - 1, Ncz = Nz - 1, per = m->periodic_x;
  const int64_t Nc = (int64_t)Ncx * Ncz, Nv = (int64_t)Nx * Nz, n = mk->n;
  const double dx = g->dx, dz = g->dz, dt = m->dt;
  const double *u = g->u_in, *v = g->v_in;
  int status = MDZ_OK;
  /* velocity gradients: centroids and vertices below the surface, else 0 (:1751-1782) */
  const int director = (o->anisotropy == 1 && o->advection == 1);
  double *dudx_n = NULL, *dvdz_n = NULL, *dudz_s = NULL, *dvdx_s = NULL;
  if (director) {
    dudx_n = calloc(Nc, sizeof(double)); dvdz_n = calloc(Nc, sizeof(double));
    dudz_s = calloc(Nv, sizeof(double)); dvdx_s = calloc(Nv, sizeof(double));
    for (int64_t c1 = 0; c1 < Nv; c1++) {
      const int64_t k = c1 % Nx, l = c1 / Nx, c3 = k + l * (Nx + 1);
      if (g->BCg_type[c1] != 30) {
        dudz_s[c1] = (u[c1 + Nx] - u[c1]) / dz;
        dvdx_s[c1] = (v[c3 + 1] - v[c3]) / dx;
      }
    }
    for (int64_t c0 = 0; c0 < Nc; c0++) {
      const int64_t k = c0 % Ncx, l = c0 / Ncx, c1 = k + l * Nx, c2 = k + l * (Nx + 1);
      if (!orc_air(g->BCp_type[c0])) {
        dudx_n[c0] = (u[c1 + 1 + Nx] - u[c1 + Nx]) / dx;
        dvdz_n[c0] = (v[c2 + 1 + (Nx + 1)] - v[c2 + 1]) / dz;
      }
    }
  }
  for (int64_t p = 0; p < n; p++) {
    if (mk->phase[p] == -1) continue;
    const double x = mk->x[p], z = mk->z[p];
    if (director) { /* :1784-1802 */
      int jp, ip, c[4];
      double w[4];
      double mdudx = 0.0, mdvdz = 0.0, mdudz = 0.0, mdvdx = 0.0;
      if (orc_cell_corners(x, z, g->xvz_coord, g->zvx_coord, Ncx, Ncz, dx, dz, per, &jp, &ip, c) != 0) {
        status = MDZ_EMARKER_OUT;
        continue;
      }
      orc_weights(x - g->xvz_coord[jp], z - g->zvx_coord[ip], dx, dz, w);
      mdudx = orc_c2p_skip(dudx_n, g->BCp_type, c, w);
      mdvdz = orc_c2p_skip(dvdz_n, g->BCp_type, c, w);
      /* Vertices2Particle: cell from |x - X0|, clamped to the grid */
      int j = (int)ceil(fabs(x - g->xg_coord[0]) / dx) - 1, i = (int)ceil(fabs(z - g->zg_coord[0]) / dz) - 1;
      if (j < 0) j = 0;
      if (j > Nx - 2) j = Nx - 2;
      if (i < 0) i = 0;
      if (i > Nz - 2) i = Nz - 2;
      const int cv[4] = {j + i * Nx, j + i * Nx + 1, j + (i + 1) * Nx, j + (i + 1) * Nx + 1};
      orc_weights(x - g->xg_coord[j], z - g->zg_coord[i], dx, dz, w);
      mdudz = orc_c2p_skip(dudz_s, g->BCg_type, cv, w);
      mdvdx = orc_c2p_skip(dvdx_s, g->BCg_type, cv, w);
      const double nx = mk->nx[p], nz = mk->nz[p];
      mk->nx[p] += dt * (-(mdudx - mdvdz) * nx * nz - mdvdx * nz * nz + mdudz * nx * nx) * nz;
      mk->nz[p] += dt * ((mdudx - mdvdz) * nx * nz + mdvdx * nz * nz - mdudz * nx * nx) * nx;
      const double norm = sqrt(pow(mk->nx[p], 2) + pow(mk->nz[p], 2));
      mk->nx[p] /= norm;
      mk->nz[p] /= norm;
    }
  }
  free(dudx_n); free(dvdz_n); free(dudz_s); free(dvdx_s);
  if (o->elastic != 1) return status;

  if (o->subgrid_diffusion == 2) status = orc_subgrid_stress(m, o, g, mk, status);
  /* stress increments grid -> markers (:1919-1966), then ArrayPlusArray on every marker */
  for (int64_t p = 0; p < n && o->subgrid_diffusion != 2; p++) {
    double dsx = 0.0, dsz = 0.0, dsxz = 0.0;
    if (mk->phase[p] != -1) {
      const double x = mk->x[p], z = mk->z[p];
      int jp, ip, c[4];
      double w[4];
      if (orc_cell_corners(x, z, g->xvz_coord, g->zvx_coord, Ncx, Ncz, dx, dz, per, &jp, &ip, c) != 0) {
        status = MDZ_EMARKER_OUT;
      } else {
        double fx[4], fz[4];
        const int alt[4] = {c[2], c[3], c[0], c[1]};
        orc_weights(x - g->xvz_coord[jp], z - g->zvx_coord[ip], dx, dz, w);
        double sw = 0.0;
        for (int q = 0; q < 4; q++) {
          const int cc = orc_air(g->BCp_type[c[q]]) ? alt[q] : c[q];
          /* dsxxd / dszzd: the change at cells below the surface, else 0 (calloc) */
          fx[q] = orc_air(g->BCp_type[cc]) ? 0.0 : g->sxxd[cc] - g->sxxd0[cc];
          fz[q] = orc_air(g->BCp_type[cc]) ? 0.0 : g->szzd[cc] - g->szzd0[cc];
          dsx += w[q] * fx[q];
          dsz += w[q] * fz[q];
          sw += w[q];
        }
        if (sw > 1e-13) { dsx /= sw; dsz /= sw; }
        if (isinf(dsx) || isinf(dsz)) status = MDZ_ENONFINITE; /* ParticleRoutines.c:1565-1569, exit 1 */
      }
      /* Interp_Grid2P (ParticleRoutines.c:1223-1321): vertex cell clamped to the grid */
      int j = (int)ceil((x - g->xg_coord[0]) / dx) - 1;
      if (j < 0) j = 0;
      if (j > Nx - 2) { j = Nx - 2; status = MDZ_EMARKER_OUT; }
      int i = (int)ceil((z - g->zg_coord[0]) / dz) - 1;
      if (i < 0) i = 0;
      if (i > Nz - 2) i = Nz - 2;
      const int cv[4] = {j + i * Nx, j + i * Nx + 1, j + (i + 1) * Nx, j + (i + 1) * Nx + 1};
      const int alt[4] = {cv[2], cv[3], cv[0], cv[1]};
      orc_weights(fabs(x - g->xg_coord[j]), fabs(z - g->zg_coord[i]), dx, dz, w);
      for (int q = 0; q < 4; q++) {
        const int cc = orc_air(g->BCg_type[cv[q]]) ? alt[q] : cv[q];
        const double d = (g->BCg_type[cc] != 30) ? g->sxz[cc] - g->sxz0[cc] : 0.0;
        dsxz += w[q] * d;
      }
    }
    mk->sxxd[p] = mk->sxxd[p] + dsx;
    mk->szzd[p] = mk->szzd[p] + dsz;
    mk->sxz[p] = mk->sxz[p] + dsxz;
  }

  /* :1967-1992: P2Mastah of a zeroed marker array onto wxz (vertices), so wxz becomes
   * 0 / (sum of marker weights) wherever that sum reaches 1e-30 below the surface; the
   * marker spin stays zero and the rotation below turns by zero */
  double *WM = calloc(Nv, sizeof(double));
  orc_p2m(mk, NULL, g->xg_coord, g->zg_coord, Nx, Nz, dx, dz, o->interp_stencil, per, WM, NULL);
  for (int64_t c1 = 0; c1 < Nv; c1++)
    if (!(fabs(WM[c1]) < 1e-30 || orc_air(g->BCg_type[c1]))) g->wxz[c1] = 0.0 / WM[c1];
  if (per == 1)
    for (int l = 0; l < Nz; l++) {
      const int64_t c1 = (int64_t)l * Nx + Nx - 1, c = (int64_t)l * Nx;
      const double av = 0.5 * (g->wxz[c1] + g->wxz[c]);
      g->wxz[c1] = av; g->wxz[c] = av;
    }
  free(WM);
  for (int64_t p = 0; p < n; p++) {
    if (mk->phase[p] == -1) continue;
    const double txx = mk->sxxd[p], tzz = mk->szzd[p], txz = mk->sxz[p], wxzm = 0.0;
    if (o->stress_rotation == 1) { /* Jaumann rate */
      mk->sxxd[p] -= dt * 2.0 * txz * wxzm;
      mk->szzd[p] -= -dt * 2.0 * txz * wxzm;
      mk->sxz[p] -= dt * (tzz - txx) * wxzm;
    }
    if (o->stress_rotation == 2) { /* analytical rotation */
      const double angle = dt * wxzm;
      mk->sxxd[p] = (txx * cos(angle) + txz * sin(angle)) * cos(angle) + (txz * cos(angle) + tzz * sin(angle)) * sin(angle);
      mk->szzd[p] = -(-txx * sin(angle) + txz * cos(angle)) * sin(angle) + (-txz * sin(angle) + tzz * cos(angle)) * cos(angle);
      mk->sxz[p] = -(txx * cos(angle) + txz * sin(angle)) * sin(angle) + (txz * cos(angle) + tzz * sin(angle)) * cos(angle);
    }
  }
  return status;
}
