// rheo_device.cuh -- device-side local rheology update (FP64) for sm_103a.
//
// One call of `point_iso` is one ViscosityConcise (MDLIB/RheologyDensity.c:385-1080);
// `point_aniso` is ViscosityConciseAniso (MDLIB/AnisotropyRoutines.c:282-727).
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and this path is bound by the FP64 pipe,
// so the formulation minimises FP64 instructions while keeping every quantity
// well conditioned:
//  * per-phase constants (log pre-factors, 1/(R n), 1/n, ...) are folded on the host;
//  * each creep law k is carried as the logarithm of the reciprocal of its isolated
//    viscosity at the node's strain rate, ln(1/eta_k), a sum of well-conditioned logs
//    (no exp); its strain rate at trial viscosity eta is then
//        Eii_k(eta) = Eii (eta / eta_k)^n_k,
//    the reference's C_k Tii^n_k with Tii = 2 eta Eii rewritten.  The Peierls law is
//    used in the equivalent physical form A (sqrt(3) Tii / (gamma sigma_P))^(ST+n);
//  * the local Newton iterates on s = eta / eta_up (eta_up: the reference's start
//    point); a step takes one log, of s, and one exp per non-linear law, with the laws
//    offset from the softest one p by n_k ln(eta_p / eta_k) <= 0 and from eta_up by
//    ln(eta_up / eta_p), so no large logarithms cancel;
//  * once a Newton step is small (|n step| < 1e-5) the next residual carries the law
//    terms by the binomial series instead of a new log and exps (exact to 2e-16);
//  * post-processing uses eta_k = Tii / (2 Eii_k), the reference's
//    B_k pow(Eii_k, 1/n_k - 1) rewritten with the same identity.
// These are identities of the reference's formulas: results differ only by rounding
// (a few 1e-14 relative, checked by the parity tests).  The Newton iteration itself
// (start point, update, stopping test, cap) is the reference's, so from the reference's
// start (MDZ_SWEEP_REF_START) iteration counts agree except where rounding moves a
// residual across the stopping threshold.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mdz_rheo.h"
#include "dd_math.cuh"
#include "fp64_bits.cuh"
#include "fp64_div.cuh"
#include "fp64_math.cuh"

namespace mdz {

constexpr double kZeroC = 273.15;                 // MDLIB/include/mdoodz.h:4
constexpr double kLn2 = 0.69314718055994530942;
constexpr double kInf = __builtin_huge_val();
constexpr double kLnSqrt3 = 0.54930614433405484570;  // log(sqrt(3))
constexpr double kSqrt3 = 1.73205080756887729353;

// mechanism / option bits of PhaseConst::flags
enum : int {
  F_CST = 1 << 0,   // cstv != 0
  F_PWL = 1 << 1,   // pwlv != 0
  F_EXPV = 1 << 2,  // expv != 0 (Peierls, still gated by T < TmaxPeierls)
  F_LIN = 1 << 3,   // linv != 0
  F_GBS = 1 << 4,   // gbsv != 0
  F_GS = 1 << 5,    // gs != 0 (paleowattmeter grain size)
  F_PL1 = 1 << 6,   // plast == 1
  F_PL2 = 1 << 7,   // plast == 2
  F_PLANY = 1 << 8, // plast != 0 (anisotropic path)
  F_CMIX = 1 << 9,  // phase_mix with diffuse_X
  F_LIN1 = 1 << 10, // nlin == 1: Newtonian diffusion creep (linear in eta)
  F_PWL_M = 1 << 11,// mpwl != 0
  F_PWL_A = 1 << 12,// apwl != 0
  F_LIN_A = 1 << 13,// alin != 0
  F_VP1 = 1 << 14,  // n_vp == 1 (pow(x, 1/n_vp - 1) == 1)
  F_PWL1 = 1 << 15, // npwl == 1
};

// Per-phase constants folded on the host (mdz_rheo_capi.cu: fold_phase).
struct PhaseConst {
  int flags, density_model, phase_two, reac_phase;
  // dislocation: ln B = lnK + (Q + P V) invRn / T + mn ln d - an phi
  double pwl_n, pwl_invn, pwl_lnK, pwl_Q, pwl_V, pwl_invRn, pwl_mn, pwl_an;
  // diffusion: ln B = lnK + (Q + P V) invRn / T - an phi; eta also carries d^(m/n)
  double lin_n, lin_invn, lin_lnK, lin_Q, lin_V, lin_invRn, lin_m, lin_mn, lin_an;
  // grain-boundary sliding (bracket only: C_gbs is never set by the reference)
  double gbs_n, gbs_invn, gbs_lnK, gbs_Q, gbs_V, gbs_invRn, gbs_m, gbs_mn, gbs_an;
  // Peierls: ST = EaR g2 / T; Eii_exp = exp(lnA0 - EaR om2 / T) (s3gS Tii)^(ST+n)
  double exp_EaR, exp_g2, exp_om2, exp_n, exp_lnA0, exp_s3gS, exp_ln_s3gS;
  // constant viscosity
  double eta0, eta0_two;
  // plasticity
  double Slim, eta_vp, n_vp, T_st;
  // grain size / wattmeter
  double gs_ref, inv_gs_ref, ln_gs_ref, Kpzm, Qpzm, Gpzm, Lpzm, cpzm, ppzm;
  // density
  double rho, drho, alp, bet, T0, P0, rho_reac;
};

struct ModelConst {
  int np, elastic, step, eta_average, periodic_x, density_variations, tensile_line_search;
  int diffuse_avg, Nx, Nz, Ncx, Ncz;
  long long Nc, Nv;
  double dt, dt_model, min_eta, max_eta, eta_tol, R;
  double scale_eta, scale_L, scale_T, scale_S, scale_E;
  double TmaxPeierls, Tmin, Tiimin, Eii_floor, eta_up0, ln_eta_up0, eta_lo0, d_min;
};

// Per-node values shared by all phases of one node.
struct NodeIn {
  double Exx, Ezz, Exz, Txx0, Tzz0, Txz0;
  double G, T, P, d, phi, X0, dil, fric, C, P0, T0, beta;
  double lxlz, lx2, ani_fac;  // anisotropic nodes
  // post_process: 0 none, 1 every output (ViscosityConcise's post_process = 1), 2 only what
  // the sweep keeps of a vertex (etaVE, the dissipative viscosity, X): the per-phase stress
  // components, strain-rate partition, divergences and overstress are left unset
  int centroid, final_update, post_process, want_rho;
};

struct NodeCtx {
  double Eii, lnEii, T, Traw, invT, lnd, K, G, dil, eta_el, inv_eta_el, sin_fric, cos_fric, sin_dil;
  double inv2Eii, inv_Kdt, inv_d;
  double ln_eta_el;         // ln(eta_el), set where elasticity is on
  int elastic, plastic_on;  // plastic_on = (step != 0)
};

struct PointOut {
  double eta, Txx, Tzz, Txz, etaVE, Eii_el, Eii_pl, Eii_pwl, Eii_exp, Eii_lin, Eii_gbs, Eii_cst, d1, inv_d1,
      X1, OverS, Pcorr, rho, div_el, div_pl, Wtot, Wel, Wdiss;
  int iters, is_pl, status;
  int f32_steps;  // FP32 Newton steps taken by the start of the local solve
  int mech;       // MDZ_MECH_* bits of the local solve (its switches, and MDZ_MECH_YIELD)
};

__device__ __forceinline__ void set_status(int &st, int code) {
  if (st == MDZ_OK) st = code;
}

// ---------------------------------------------------------------------------------------
// node set-up: invariants and switches shared by the phases (RheologyDensity.c:461-496)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void node_strain_update(NodeCtx &c);

__device__ __forceinline__ void node_common(const ModelConst &M, const NodeIn &in, bool need_lnd, NodeCtx &c) {
  node_strain_update(c);
  c.Traw = in.T;
  c.T = fp64_lt(in.T, M.Tmin) ? M.Tmin : in.T;
  c.invT = quotient(1.0, c.T);
  c.lnd = need_lnd ? fast_log(in.d) : 0.0;
  c.inv_d = 0.0;
  sincos(in.fric, &c.sin_fric, &c.cos_fric);
  c.sin_dil = fp64_is_zero(c.dil) ? 0.0 : sin(c.dil);
}

// The strain-rate invariant and what depends on it (RheologyDensity.c:455-459); the
// rest of the node set-up does not depend on the strain rate.
__device__ __forceinline__ void node_strain_iso(const ModelConst &M, const NodeIn &in, NodeCtx &c) {
  const double Eyy = -(in.Exx + in.Ezz);
  double Eii = sqrt(0.5 * (in.Exx * in.Exx + in.Ezz * in.Ezz + Eyy * Eyy) + in.Exz * in.Exz);
  if (fp64_lt(Eii * M.scale_E, 1e-30)) Eii = M.Eii_floor;
  c.Eii = Eii;
}

__device__ __forceinline__ void node_strain_update(NodeCtx &c) {
  c.lnEii = fast_log(c.Eii);
  c.inv2Eii = quotient(0.5, c.Eii);
}

__device__ __forceinline__ void node_setup_iso(const ModelConst &M, const NodeIn &in, bool need_lnd,
                                               NodeCtx &c) {
  node_strain_iso(M, in, c);
  c.elastic = (M.step == 0) ? 0 : M.elastic;
  c.plastic_on = (M.step != 0);
  c.K = quotient(1.0, in.beta);
  c.G = in.G;
  c.dil = in.dil;
  if (c.elastic == 0) { c.G = 1e1; c.dil = 0.0; c.K = 1e10; }
  c.eta_el = c.G * M.dt;
  c.inv_eta_el = quotient(1.0, c.eta_el);
  c.ln_eta_el = c.elastic ? fast_log(c.eta_el) : 0.0;
  c.inv_Kdt = quotient(1.0, c.K * M.dt);
  node_common(M, in, need_lnd, c);
}

// EvaluateDensity, RheologyDensity.c:1761-1831 (models 0, 1, 3, 5)
__device__ __forceinline__ double density(const ModelConst &M, const PhaseConst &ph, double T, double P,
                                          double X, double phi) {
  double rho = 0.0;
  const int dm = ph.density_model;
  if (dm == 0) rho = ph.rho;
  if (dm == 1) {
    rho = (1.0 - ph.alp * (T - ph.T0)) * (1.0 + ph.bet * (P - ph.P0));
    rho = ((1.0 - X) * ph.rho + X * (ph.rho + ph.drho)) * rho;
  }
  if (dm == 3 && M.density_variations == 0) rho = ph.rho * exp(ph.bet * P - ph.alp * T);
  if (dm == 3 && M.density_variations == 1)
    rho = ((1.0 - X) * ph.rho + X * ph.rho_reac) * exp(ph.bet * P - ph.alp * T);
  if (dm == 5) {
    const double e = exp(ph.bet * P - ph.alp * T);
    rho = (1 - phi) * (ph.rho * e) + phi * ((ph.rho + ph.drho) * e);
  }
  return rho;
}

// ---------------------------------------------------------------------------------------
// Creep laws of one (node, phase).  ln B and the isolated-viscosity reciprocals 1/eta_k
// (RheologyDensity.c:501-523, 559-592), the forms documented at the top of the file.
// ---------------------------------------------------------------------------------------
enum { K_PWL = 0, K_EXP = 1, K_LIN = 2, K_COUNT = 3 };

struct Laws {
  int mech;               // F_CST | F_PWL | F_EXPV (active) | F_LIN | F_GBS
  double ln_inv[K_COUNT]; // ln(1/eta_k) at the node's Eii (-inf where inactive)
  double n[K_COUNT];      // exponents n_pwl, ST + n_exp, n_lin
  double lnB_pwl, lnB_lin, lnA_exp, ST, ln_inv_gbs;
};

// 1/eta_k itself, where a caller needs it in linear form
__device__ __forceinline__ double law_inv(const Laws &L, int k) { return fast_exp(L.ln_inv[k]); }

__device__ __forceinline__ void creep_laws(const ModelConst &M, const PhaseConst &ph, const NodeCtx &c, double P,
                                           double phi, double lnd, int peierls, Laws &L) {
  const int fl = ph.flags;
  L.mech = (fl & (F_CST | F_PWL | F_LIN | F_GBS)) | (peierls ? F_EXPV : 0);
  L.ln_inv[0] = L.ln_inv[1] = L.ln_inv[2] = -kInf;
  L.n[0] = ph.pwl_n; L.n[1] = 0.0; L.n[2] = ph.lin_n;
  L.lnB_pwl = L.lnB_lin = L.lnA_exp = L.ST = 0.0;
  L.ln_inv_gbs = -kInf;
  const double lnEii = c.lnEii;
  if (fl & F_PWL) {
    // B = pref F A^(-1/n) exp((Q+PV)/(RnT)) d^(m/n) f^(-r/n) exp(-a phi/n);
    // 1/eta_pwl = Eii^(1-1/n) / B:  ln(1/eta_pwl) = lnEii - lnEii/n - lnB
    double lnB = ph.pwl_lnK + (ph.pwl_Q + P * ph.pwl_V) * ph.pwl_invRn * c.invT;
    if (fl & F_PWL_M) lnB += ph.pwl_mn * lnd;
    if (fl & F_PWL_A) lnB -= ph.pwl_an * phi;
    L.lnB_pwl = lnB;
    L.ln_inv[K_PWL] = lnEii - fma(lnEii, ph.pwl_invn, lnB);
  }
  if (fl & F_LIN) {
    // 1/eta_lin = Eii^(1-1/n) / (B d^(m/n))
    double lnB = ph.lin_lnK + (ph.lin_Q + P * ph.lin_V) * ph.lin_invRn * c.invT;
    if (fl & F_LIN_A) lnB -= ph.lin_an * phi;
    L.lnB_lin = lnB;
    const double lnBd = !fp64_is_zero(ph.lin_m) ? fma(ph.lin_mn, lnd, lnB) : lnB;
    L.ln_inv[K_LIN] = lnEii - fma(lnEii, ph.lin_invn, lnBd);
  }
  if (peierls) {
    // Eii_exp(Tii) = A (sqrt3 Tii / (gamma S))^nE, A = (sqrt3/2) E Arr (gamma S)^n;
    // isolated: Tii* = (gamma S / sqrt3) (Eii/A)^(1/nE), 1/eta_exp = 2 Eii / Tii*
    L.ST = ph.exp_EaR * c.invT * ph.exp_g2;
    const double nE = L.ST + ph.exp_n;
    L.n[K_EXP] = nE;
    L.lnA_exp = ph.exp_lnA0 - ph.exp_EaR * ph.exp_om2 * c.invT;
    L.ln_inv[K_EXP] = (kLn2 + ph.exp_ln_s3gS + lnEii) - quotient(lnEii - L.lnA_exp, nE);
  }
  if (fl & F_GBS) {
    double lnB = ph.gbs_lnK + (ph.gbs_Q + P * ph.gbs_V) * ph.gbs_invRn * c.invT - ph.gbs_an * phi;
    if (!fp64_is_zero(ph.gbs_m)) lnB += ph.gbs_mn * lnd;
    L.ln_inv_gbs = lnEii - fma(lnEii, ph.gbs_invn, lnB);
  }
}

// ---------------------------------------------------------------------------------------
// Local VE residual  r(eta) = Eii - el Tii/(2 eta_el) - sum_k Eii_k(eta),  Tii = 2 eta Eii
// (LocalIterationViscoElastic, RheologyDensity.c:152-197), written in the normalised
// unknown s = eta / eta_up (eta_up: the reference's start point).  Linear terms
// (elasticity, constant viscosity, Newtonian laws) are s Aup with Aup = eta_up A;
// non-linear ones Eii exp(n_k (ln s + lp) + nc_k), where lp = ln(eta_up / eta_p) for
// the softest non-linear law p and nc_k = n_k ln(eta_p / eta_k) <= 0.  Every quantity
// in the exponent is O(1) for the terms that carry strain rate, so nothing large cancels.
// ---------------------------------------------------------------------------------------
struct VeCoef {
  double Eii, thr_conv, thr_fail;  // Eii * tol/100, Eii * tol
  double inv_Eii;                  // 1 / Eii
  double eta_up;                   // eta = s eta_up
  double Aup;                      // eta_up x the sum of the linear coefficients (el, cst, Newtonian laws)
  double a_cst, a_lin1, a_pwl1;    // e_cst = eta a_cst, e_lin = eta a_lin1 (n_lin==1), e_pwl = eta a_pwl1 (n_pwl==1)
  double lp;                       // ln(eta_up / eta_p)
  double n[K_COUNT], nc[K_COUNT];  // exponent and n_k * ln(eta_p / eta_k) per non-linear law
  double hn[K_COUNT];              // (n_k - 1) / 2
  double nmax;                     // largest exponent of the non-linear laws (0 without)
  int nl;                          // bit k: law k is non-linear and active
};

struct VeState {
  double eta, Tii, e_cst, e_pwl, e_exp, e_lin;
  double e[K_COUNT];  // strain rates of the non-linear laws at the last evaluated point
  int iters, status;
};

__device__ __forceinline__ void ve_coef(const Laws &L, const NodeCtx &c, double eta_cst, double eta_up,
                                        double ln_eta_up, VeCoef &q) {
  const double Eii = c.Eii;
  const double tol = 1.0e-11;  // hard-coded in LocalIterationViscoElastic (:154)
  q.Eii = Eii;
  q.inv_Eii = 2.0 * c.inv2Eii;
  q.thr_conv = Eii * (tol / 100);
  q.thr_fail = Eii * tol;
  q.eta_up = eta_up;
  q.a_cst = (L.mech & F_CST) ? Eii / eta_cst : 0.0;
  double A = (c.elastic ? Eii * c.inv_eta_el : 0.0) + q.a_cst;
  q.a_lin1 = q.a_pwl1 = 0.0;
  q.nl = 0;
  double ln_inv_p = -kInf;
  int p = -1;
#pragma unroll
  for (int k = 0; k < K_COUNT; k++) {
    const int bit = (k == K_PWL) ? F_PWL : ((k == K_EXP) ? F_EXPV : F_LIN);
    q.n[k] = L.n[k];
    q.nc[k] = 0.0;
    if (!(L.mech & bit)) continue;
    if (k != K_EXP && fp64_eq_nonzero(L.n[k], 1.0)) {  // Newtonian law: Eii eta / eta_k
      const double a = Eii * law_inv(L, k);
      if (k == K_LIN) q.a_lin1 = a;
      else q.a_pwl1 = a;
      A += a;
    } else {
      q.nl |= 1 << k;
      if (fp64_gt(L.ln_inv[k], ln_inv_p)) { ln_inv_p = L.ln_inv[k]; p = k; }
    }
  }
  if (!fp64_gt(ln_inv_p, -kInf)) q.nl = 0;
  q.lp = ln_eta_up + ln_inv_p;
  q.nmax = 0.0;
#pragma unroll
  for (int k = 0; k < K_COUNT; k++) {
    q.hn[k] = 0.5 * (q.n[k] - 1.0);
    if (q.nl >> k & 1) q.nmax = fp64_fmax(q.nmax, q.n[k]);
    if ((q.nl >> k & 1) && k != p) q.nc[k] = q.n[k] * (L.ln_inv[k] - ln_inv_p);
  }
  q.Aup = A * eta_up;
}

// Residual r at sv; the strain rates of the non-linear laws stay in s.e.  With step >= 0
// the non-linear terms are carried from the previous point sv / (1 + step) by the
// binomial series
//     (1 + step)^n = 1 + n step (1 + (n - 1) step / 2) + O((n step)^3),
// used only where |n step| < 1e-5, so the dropped term is below 2e-16 relative: the same
// residual as a fresh evaluation to rounding, without its log and exps.
__device__ __forceinline__ void ve_eval(const VeCoef &q, double sv, VeState &s, double &r, double step = -1.0) {
  double *e = s.e;
  if (fp64_ge(step, -0.5)) {
#pragma unroll
    for (int k = 0; k < K_COUNT; k++)
      if (q.nl >> k & 1) {
        const double t = step * q.n[k];
        e[k] = fma(e[k] * t, fma(step, q.hn[k], 1.0), e[k]);
      }
  } else {
    e[0] = e[1] = e[2] = 0.0;
    if (q.nl) {
      const double lx = fast_log(sv) + q.lp;
#pragma unroll
      for (int k = 0; k < K_COUNT; k++)
        if (q.nl >> k & 1) e[k] = q.Eii * fast_exp(fma(q.n[k], lx, q.nc[k]));
    }
  }
  const double eta = sv * q.eta_up;
  s.e_cst = eta * q.a_cst;
  s.e_pwl = (q.nl >> K_PWL & 1) ? e[K_PWL] : eta * q.a_pwl1;
  s.e_lin = (q.nl >> K_LIN & 1) ? e[K_LIN] : eta * q.a_lin1;
  s.e_exp = e[K_EXP];
  s.Tii = 2.0 * eta * q.Eii;
  r = q.Eii - sv * q.Aup - (e[K_PWL] + e[K_EXP] + e[K_LIN]);
}

// S = sum_k n_k Eii_k at the last evaluated point (the non-linear part of -s r'(s))
__device__ __forceinline__ double ve_S(const VeCoef &q, const VeState &s) {
  double S = 0.0;
#pragma unroll
  for (int k = 0; k < K_COUNT; k++)
    if (q.nl >> k & 1) S = fma(q.n[k], s.e[k], S);
  return S;
}

// Newton on s from sv: s <- s (1 + step), step = r / (Aup s + S), i.e. s - r / r'(s)
// with r' = -Aup - S/s (LocalIterationViscoElastic); returns eta = s eta_up in st.eta.
// A moved start (one the start stages chose) that has not converged within the cap is
// abandoned: the iteration runs again from the upper bound eta_up (s_up), with the
// reference's cap, and the evaluations of both runs count.
__device__ __forceinline__ void ve_newton(const VeCoef &q, double sv, VeState &s, float s_up = 1.0f,
                                          bool moved = false) {
  const int nitmax = 20;
  s.iters = 0;
  double step = -1.0;  // no previous point yet
  for (int it = 0; it < nitmax; it++) {
    double r;
    ve_eval(q, sv, s, r, step);
    s.iters++;
    if (fp64_abs_lt(r, q.thr_conv)) break;
    if (it == nitmax - 1 && moved) {  // back to the upper bound
      moved = false;
      sv = f64_of_f32(s_up);
      step = -1.0;
      it = -1;
      continue;
    }
    if (it == nitmax - 1 && fabs(r) > q.thr_fail) { set_status(s.status, MDZ_EVE_ITER); break; }
    const double d = newton_quotient(r, fma(q.Aup, sv, ve_S(q, s)));
    sv = fma(sv, d, sv);
    step = fp64_lt(fabs(d) * q.nmax, 1e-5) ? d : -1.0;
  }
  s.eta = sv * q.eta_up;
}

// Start point of the FP64 Newton, in two stages on the same normalised residual
//     r(s)/Eii = 1 - a s - sum_k exp(n_k ln s + c_k),   a = Aup/Eii,  c_k = n_k lp + nc_k.
// The FP64 iteration that follows is unchanged and runs to the same residual tolerance, so
// these stages only move its start; every quantity in them is O(1).
//
// Stage 1, `fp32` FP32 Newton steps (ve_polish_f32): within FP32 rounding of the root,
// about 3e-7 relative.  The coefficients go to FP32 by truncating their bit patterns on
// the integer pipe (a starting guess needs no rounding), since GB300 runs the
// FP32<->FP64 conversions on its FP64 pipe: values beyond the FP32 range become
// +-FLT_MAX (NaN too) and the step guard returns 1 should they upset the iteration;
// values below it become 0.  r is decreasing and concave, so Newton from above the root
// (r < 0; the reference's start eta_up, s = 1, is such a point) descends monotonically,
// and from below it (a learned guess may be) the first step lands above it.  A step that
// leaves (0, 2] abandons the guess for s = 1.
//
// Stage 2 (ve_halley_dd): one Halley step whose residual and derivative are evaluated in
// double-float (dd_math.cuh): s <- s (1 + d / (1 + d Q / (2 D))) with D = a s + sum_k n_k
// e_k (= -s r'(s)), d = r / D, Q = sum_k n_k (n_k - 1) e_k (= -s^2 r''(s)).  From the FP32
// root the step's own error is third order (about 1e-20), so the start lands within the
// double-float evaluation's error (a few 1e-14 of the exponents) of the root, and the
// FP64 residual there is already below the reference's stopping threshold 1e-13 Eii:
// the FP64 iteration stops at its first evaluation, whose outputs it returns.  Where it
// does not (an unresolved polish, a huge exponent), the FP64 Newton simply continues.
struct StartCoef {
  double a;              // Aup / Eii
  double c[K_COUNT];     // n_k lp + nc_k for the non-linear laws
};

__device__ __forceinline__ void start_coef(const VeCoef &q, StartCoef &sc) {
  sc.a = q.Aup * q.inv_Eii;
#pragma unroll
  for (int k = 0; k < K_COUNT; k++) sc.c[k] = (q.nl >> k & 1) ? fma(q.n[k], q.lp, q.nc[k]) : 0.0;
}

// s_hi: the upper bound the iteration falls back to
__device__ __forceinline__ float ve_polish_f32(const VeCoef &q, const StartCoef &sc, float s0, int iters,
                                               int &taken, float s_hi) {
  taken = 0;
  if (iters <= 0) return s0;
  const float a = f32_trunc(sc.a);
  float c[K_COUNT] = {0.f, 0.f, 0.f}, n[K_COUNT] = {0.f, 0.f, 0.f};
  if (q.nl) {
#pragma unroll
    for (int k = 0; k < K_COUNT; k++)
      if (q.nl >> k & 1) { n[k] = f32_trunc(q.n[k]); c[k] = f32_trunc(sc.c[k]); }
  }
  float s = s0;
  for (int it = 0; it < iters; it++) {
    float e = 0.f, S = 0.f;
    if (q.nl) {
      const float ls = __logf(s);
#pragma unroll
      for (int k = 0; k < K_COUNT; k++)
        if (q.nl >> k & 1) {
          const float ek = __expf(fmaf(n[k], ls, c[k]));
          e += ek;
          S = fmaf(n[k], ek, S);
        }
    }
    const float r = 1.0f - a * s - e;
    if (fabsf(r) < 1e-6f) break;
    const float sn = s + r * s / fmaf(a, s, S);
    taken = it + 1;
    if (!(sn > 0.0f && sn <= 2.0f)) return s_hi;  // the upper bound eta_up: right of the root
    s = sn;
  }
  return s;
}

// Stage 2 from the FP32 point s (see above).  Where s is not a positive normal number in
// (0, 2], or the correction is not small (the polish did not settle), the FP64 Newton
// starts at s itself if s lies above the root and at the upper bound s = 1 otherwise.
__device__ __forceinline__ double ve_halley_dd(const VeCoef &q, const StartCoef &sc, float s, float s_hi) {
  if (!(s >= 1.17549435e-38f && s <= 2.0f)) return f64_of_f32(s_hi);
  const f2 a = dd_of_f64(sc.a);
  const f2 as = dd_mul_f(a, s);
  f2 E = {0.0f, 0.0f}, D = as;
  float Q = 0.0f;
  if (q.nl) {
    const f2 ls = dd_log_f(s);
#pragma unroll
    for (int k = 0; k < K_COUNT; k++)
      if (q.nl >> k & 1) {
        const f2 nk = dd_of_f64(q.n[k]);
        const f2 e = dd_exp(dd_add(dd_mul(nk, ls), dd_of_f64(sc.c[k])));
        const f2 ne = dd_mul(nk, e);
        E = dd_add(E, e);
        D = dd_add(D, ne);
        Q = __fmaf_rn(ne.hi, __fsub_rn(nk.hi, 1.0f), Q);
      }
  }
  const f2 r = dd_add(dd_add_f(dd_neg(as), 1.0f), dd_neg(E));  // 1 - a s - sum_k e_k
  // d = r / D in double-float: a first quotient and the quotient of its remainder
  const float q1 = __fdividef(r.hi, D.hi);
  // an unsettled point: the FP64 Newton takes it from there if it lies above the root
  // (r <= 0, monotone descent), from the upper bound s = 1 otherwise
  if (!(fabsf(q1) < 1e-3f)) return f64_of_f32((r.hi > 0.0f) ? s_hi : s);
  const f2 rem = dd_add(r, dd_neg(dd_mul_f(D, q1)));
  const float q2 = __fdividef(rem.hi, D.hi);
  const float h = __fdividef(__fmul_rn(__fmul_rn(q1, q1), Q), 2.0f * D.hi);  // Halley's term d^2 Q / (2 D)
  // s (1 + d - d^2 Q / (2 D))
  f2 sn = two_prod(s, q1);
  sn.lo = __fmaf_rn(s, __fsub_rn(q2, h), sn.lo);
  sn = dd_add_f(sn, s);
  return f64_of_dd(sn);
}

// The start of the FP64 Newton: `fp32` FP32 Newton steps from s0, then, with `dd`, the
// double-float Halley step.
__device__ __forceinline__ double ve_start(const VeCoef &q, float s0, int fp32, bool dd, int &taken,
                                           float s_hi = 1.0f) {
  taken = 0;
  if (fp32 <= 0 && !dd) return f64_of_f32(s0);
  StartCoef sc;
  start_coef(q, sc);
  const float s = ve_polish_f32(q, sc, s0, fp32, taken, s_hi);
  return dd ? ve_halley_dd(q, sc, s, s_hi) : f64_of_f32(s);
}

// The start descriptor carried by the kernels' `polish` argument: FP32 Newton steps in the
// low byte, the double-float Halley step in bit 8 (MDZ_START_DD); 0 is the reference's
// start.
__device__ __forceinline__ int start_fp32(int polish) { return polish & 0xff; }
__device__ __forceinline__ bool start_dd(int polish) { return (polish & MDZ_START_DD) != 0; }

struct GseIn {
  double Eii, eta_el, eta_cst, C_pwl, n_pwl, C_lin, n_lin, m_lin, C_exp, ST, n_exp, eta_up, eta_lo, Ag,
      gam, lam, cg, pg;
  int elastic, constant, dislocation, peierls, diffusion;
};

__device__ inline void ve_gse(const GseIn &q, double &eta_io, double &Tii_o, double &d_io, double &e_cst,
                              double &e_pwl, double &e_exp, double &e_lin, int &iters, int &status) {
  const int nitmax = 50, bisection_steps = 20;
  const double tol = 1.0e-11;
  double d_ve = d_io, eta = eta_io, Tii = Tii_o;
  const double p = q.pg, Eii = q.Eii, n_pwl = q.n_pwl, Ag = q.Ag;
  const double Bg = q.lam / (q.cg * q.gam);
  const double C_pwl = q.C_pwl;
  double eta_up = q.eta_up, eta_lo = q.eta_lo;
  e_cst = e_pwl = e_exp = e_lin = 0.0;
  iters = nitmax;
  for (int it = 0; it < nitmax; it++) {
    if (it < bisection_steps) eta = sqrt(eta_up * eta_lo);
    Tii = 2.0 * eta * Eii;
    if (q.constant) e_cst = Tii / 2.0 / q.eta_cst;
    if (q.dislocation) e_pwl = C_pwl * pow(Tii, n_pwl);
    d_ve = pow(2 * Bg * Eii * e_pwl * eta * p / Ag, (-1.0 / (p + 1)));
    if (q.peierls) e_exp = q.C_exp * pow(Tii, q.ST + q.n_exp);
    if (q.diffusion) e_lin = q.C_lin * pow(Tii, q.n_lin) * pow(d_ve, -q.m_lin);
    const double e_vis = e_pwl + e_exp + e_lin + e_cst;
    const double r = Eii - q.elastic * Tii / (2.0 * q.eta_el) - e_vis;
    const double res = fabs(r / Eii);
    if (res < tol / 100) { iters = it + 1; break; }
    if (it == bisection_steps - 1 && res < tol) { iters = it + 1; break; }
    if (it < bisection_steps) {
      if (r > 0.0) eta_up = eta;
      else eta_lo = eta;
    } else {
      const double pw = pow(2 * Eii * eta, n_pwl);
      const double dddeta = -1.0 / 2.0 * Ag * d_ve * pow(2 * Eii * eta, -n_pwl) *
                            (2 * Bg * C_pwl * Eii * n_pwl * p * pw / Ag + 2 * Bg * C_pwl * Eii * p * pw / Ag) /
                            (Bg * C_pwl * Eii * eta * p * (p + 1));
      double dfdeta = 0.0;
      if (q.elastic) dfdeta += -Eii / q.eta_el;
      if (q.constant) dfdeta += -Eii / q.eta_cst;
      if (q.peierls) dfdeta += -(e_exp) * (q.ST + q.n_exp) / eta;
      if (q.diffusion) dfdeta += -(e_lin) * q.n_lin / eta;
      if (q.dislocation) dfdeta += -(e_pwl) * n_pwl / eta;
      dfdeta += q.m_lin * e_lin * dddeta / d_ve;
      eta -= r / dfdeta;
    }
    if (it == nitmax - 1 && res > tol) { set_status(status, MDZ_EGSE_ITER); break; }
  }
  if (isnan(eta) || isinf(eta)) set_status(status, MDZ_EGSE_ITER);
  eta_io = eta; Tii_o = Tii; d_io = d_ve;
}

// solve_local_3x3, RheologyDensity.c:1082-1125
__device__ __forceinline__ bool solve3(double J11, double J12, double J13, double J21, double J22, double J23,
                                       double J31, double J32, double J33, double R1, double R2, double R3,
                                       double &dT, double &dP, double &dl) {
  const double det = J11 * (J22 * J33 - J23 * J32) - J12 * (J21 * J33 - J23 * J31) + J13 * (J21 * J32 - J22 * J31);
  if (fabs(det) < 1e-30) return false;
  const double inv = 1.0 / det;
  dT = -inv * ((J22 * J33 - J23 * J32) * R1 + (J13 * J32 - J12 * J33) * R2 + (J12 * J23 - J13 * J22) * R3);
  dP = -inv * ((J23 * J31 - J21 * J33) * R1 + (J11 * J33 - J13 * J31) * R2 + (J13 * J21 - J11 * J23) * R3);
  dl = -inv * ((J21 * J32 - J22 * J31) * R1 + (J12 * J31 - J11 * J32) * R2 + (J11 * J22 - J12 * J21) * R3);
  return true;
}

// Combined mode-I/mode-II return of Popov et al. 2025 (RheologyDensity.c:710-930).
// Returns is_pl and updates Tii, Pc, lam_dot, A_tau, A_P, eta_vp.
__device__ inline int plastic_popov(const ModelConst &M, const PhaseConst &ph, double Tii_in, double P, double C,
                                    double cos_fric, double sin_fric, double sin_dil, double eta_ve, double K,
                                    double &Tii, double &Pc, double &lam_dot, double &A_tau, double &A_P,
                                    double &eta_vp, int &status) {
  const int nitmax = 20;
  const double k = sin_fric, kq = sin_dil, c = C * cos_fric, dt = M.dt;
  const double a = sqrt(1.0 + k * k), b = sqrt(1.0 + kq * kq);
  const double py = (ph.T_st + c / a) / (1.0 - k / a);
  const double Ry = py - ph.T_st;
  const double pd = py - Ry * k / a;
  const double tau_d = k * pd + c;
  const double pq = pd + kq * tau_d;
  double R_haty = sqrt(Tii_in * Tii_in + (P - py) * (P - py)), R_hatq;
  int on_yield = (Tii_in * (py - pd)) >= (tau_d * (py - P)), on_flow;
  double F = on_yield ? Tii_in - k * P - c : a * (R_haty - Ry);
  Tii = Tii_in;
  if (!(F > 1e-17)) return 0;
  const double atol = 1e-10, rtol = 1e-8;
  const double eta_vp0 = ph.eta_vp;
  double Tiic = Tii_in, R0n = 2.0 * atol;
  double A_tau_2 = 0, A_P_2 = 0, A_tau_P = 0, A_P_tau = 0, dFdT, dFdP;
  Pc = P; lam_dot = 0.0;
  for (int it = 0; it < nitmax; it++) {
    if (Tiic < 0.0) Tiic = 0.0;
    on_yield = (Tiic * (py - pd)) >= (tau_d * (py - Pc));
    on_flow = (Tiic * (pq - pd)) >= (tau_d * (pq - Pc));
    eta_vp = eta_vp0;
    R_haty = sqrt(Tiic * Tiic + (Pc - py) * (Pc - py));
    R_hatq = sqrt(Tiic * Tiic + (Pc - pq) * (Pc - pq));
    if (on_yield) { F = Tiic - k * Pc - c; dFdT = 1.0; dFdP = -k; }
    else { F = a * (R_haty - Ry); dFdT = a * Tiic / R_haty; dFdP = a * (Pc - py) / R_haty; }
    if (on_flow) { A_tau = 0.5; A_P = kq; A_tau_2 = 0.0; A_P_2 = 0.0; A_tau_P = 0.0; A_P_tau = 0.0; }
    else {
      const double R3h = R_hatq * R_hatq * R_hatq;
      A_tau = b * Tiic / (2.0 * R_hatq);
      A_P = -b * (Pc - pq) / R_hatq;
      A_tau_2 = b * (R_hatq * R_hatq - Tiic * Tiic) / (2.0 * R3h);
      A_P_2 = -b * (R_hatq * R_hatq - (Pc - pq) * (Pc - pq)) / R3h;
      A_tau_P = -b * Tiic * (Pc - pq) / (2.0 * R3h);
      A_P_tau = b * Tiic * (Pc - pq) / R3h;
    }
    double R1 = (Tii_in - Tiic) / (2.0 * eta_ve) - lam_dot * A_tau;
    double R2 = (Pc - P) / (K * dt) - lam_dot * A_P;
    double R3 = F - lam_dot * eta_vp;
    const double Rn = sqrt(R1 * R1 + R2 * R2 + R3 * R3);
    if (Rn < atol || Rn / R0n < rtol) break;
    R0n = Rn;
    double dT, dP, dl;
    if (!solve3(-1.0 / 2.0 / eta_ve - lam_dot * A_tau_2, -lam_dot * A_tau_P, -A_tau, -lam_dot * A_P_tau,
                1.0 / K / dt - lam_dot * A_P_2, -A_P, dFdT, dFdP, -eta_vp, R1, R2, R3, dT, dP, dl)) {
      set_status(status, MDZ_ESINGULAR);
      break;
    }
    double alpha = 1.0;
    if (M.tensile_line_search == 1) {  // :845-887
      const double c_ls = 1e-4, R0ls = 0.5 * (R1 * R1 + R2 * R2 + R3 * R3);
      bool failed = false;
      for (int ls = 0; ls < 100; ls++) {
        const double Tl = Tiic + dT * alpha, Pl = Pc + dP * alpha;
        on_yield = (Tl * (py - pd) >= tau_d * (py - Pl));
        on_flow = (Tl * (pq - pd) >= tau_d * (pq - Pl));
        eta_vp = eta_vp0;
        R_haty = sqrt(Tl * Tl + (Pl - py) * (Pl - py));
        R_hatq = sqrt(Tl * Tl + (Pl - pq) * (Pl - pq));
        const double Fl = on_yield ? Tl - k * Pl - c : a * (R_haty - Ry);
        if (on_flow) { A_tau = 0.5; A_P = kq; }
        else { A_tau = b * Tl / (2.0 * R_hatq); A_P = -b * (Pl - pq) / R_hatq; }
        R1 = (Tii_in - Tl) / (2.0 * eta_ve) - lam_dot * A_tau;
        R2 = (Pl - P) / (K * dt) - lam_dot * A_P;
        R3 = Fl - lam_dot * eta_vp;
        const double Rls = 0.5 * (R1 * R1 + R2 * R2 + R3 * R3);
        if (Rls < R0ls - 2.0 * c_ls * alpha * Rls && ls > 0) break;
        alpha *= 0.5;
        if (alpha < 1e-2) { failed = true; break; }
      }
      if (failed) { set_status(status, MDZ_ELINESEARCH); break; }
    }
    Tiic += alpha * dT;
    Pc += alpha * dP;
    lam_dot += alpha * dl;
  }
  Tii = Tiic;
  return 1;
}


// ---------------------------------------------------------------------------------------
// ViscosityConcise (RheologyDensity.c:385-1080) for phase `ph` at a node prepared by
// node_setup_iso.  `warm_eta` > 0 replaces the initial guess eta_up (learned warm start).
// ---------------------------------------------------------------------------------------
// State carried from the set-up of one (node, phase) to its local solve.
struct IsoState {
  Laws L;
  double eta_up, ln_eta_up, eta_cst, Tyield, C, Ag, lnd;
  // normalisation of the local Newton's unknown s = eta / eta_n: eta_n = eta_up where the
  // start is the reference's (exact), else the power of two nearest eta_up; s_up = the
  // start point eta_up in that unknown (1 when exact)
  double eta_n, ln_eta_n;
  float s_up;
};

// Start point of the local solve (RheologyDensity.c:582-592, AnisotropyRoutines.c:409-415):
// the smallest of the initial bound, eta_cst, the isolated creep viscosities and eta_el,
// with its logarithm for the normalised residual.
__device__ __forceinline__ void start_viscosity(const ModelConst &M, double ln_inv_max, bool constant,
                                                double eta_cst, bool elastic, const NodeCtx &c, double &eta_up,
                                                double &ln_eta_up) {
  eta_up = M.eta_up0;
  ln_eta_up = M.ln_eta_up0;
  bool from_cst = false;
  if (constant && fp64_lt(eta_cst, eta_up)) { eta_up = eta_cst; from_cst = true; }
  if (fp64_gt(ln_inv_max, -kInf)) {
    const double e = fast_exp(-ln_inv_max);
    if (fp64_lt(e, eta_up)) { eta_up = e; ln_eta_up = -ln_inv_max; from_cst = false; }
  }
  if (elastic && fp64_lt(c.eta_el, eta_up)) { eta_up = c.eta_el; ln_eta_up = c.ln_eta_el; from_cst = false; }
  if (from_cst) ln_eta_up = fast_log(eta_cst);
}

// The start point and the normalisation of the local solve.  Exact (the reference's start,
// and the grain-size and bisection solves, which need its bracket): eta_up as the
// reference forms it, and eta_n = eta_up.  Otherwise eta_up is only the upper bound where
// the start stages begin (s_up), and nothing needs its FP64 value: its logarithm is the
// smallest of the candidates' logarithms (compared on the integer pipe; no exp), and the
// unknown is normalised by eta_n = 2^k, k the nearest integer to log2(eta_up), built from
// bits, with ln(eta_n) = k ln2; s_up = exp(ln eta_up - k ln2) in [0.7, 1.42] in FP32.
__device__ __forceinline__ void start_point(const ModelConst &M, double ln_inv_max, bool constant, double eta_cst,
                                            bool elastic, const NodeCtx &c, bool exact, IsoState &S) {
  if (!exact) {
    double ln = M.ln_eta_up0;
    if (constant) {
      const double lc = fast_log(eta_cst);
      if (fp64_lt(lc, ln)) ln = lc;
    }
    if (fp64_gt(ln_inv_max, -kInf) && fp64_lt(-ln_inv_max, ln)) ln = -ln_inv_max;
    if (elastic && fp64_lt(c.ln_eta_el, ln)) ln = c.ln_eta_el;
    const float lf = f32_trunc(ln);
    if (fabsf(lf) < 690.0f) {  // finite, and 2^k a normal double
      const int k = __float2int_rn(lf * 1.44269504f);
      S.ln_eta_up = ln;
      S.eta_up = 0.0;  // not formed
      S.eta_n = __hiloint2double((k + 1023) << 20, 0);
      const double kd = __hiloint2double(0x43300000, k ^ (int)0x80000000) - 4503601774854144.0;  // (double)k
      S.ln_eta_n = fma(kd, MDZ_LN2_HI, kd * MDZ_LN2_LO);
      S.s_up = __expf(fmaf((float)-k, 0.693147182f, lf));
      return;
    }
  }
  start_viscosity(M, ln_inv_max, constant, eta_cst, elastic, c, S.eta_up, S.ln_eta_up);
  S.eta_n = S.eta_up;
  S.ln_eta_n = S.ln_eta_up;
  S.s_up = 1.0f;
}

// Lower end of the reference's bracket: the largest of the lower bound, eta_cst, eta_el and
// the isolated creep viscosities (needed by the grain-size solve and the bisection only).
__device__ __forceinline__ double lower_viscosity(const ModelConst &M, const Laws &L, bool constant, double eta_cst,
                                                  bool elastic, double eta_el, bool gbs) {
  double eta_lo = M.eta_lo0;
  if (constant) eta_lo = fmax(eta_lo, eta_cst);
  if (L.mech & F_PWL) eta_lo = fmax(eta_lo, fast_exp(-L.ln_inv[K_PWL]));
  if (elastic) eta_lo = fmax(eta_lo, eta_el);
  if (L.mech & F_EXPV) eta_lo = fmax(eta_lo, fast_exp(-L.ln_inv[K_EXP]));
  if (L.mech & F_LIN) eta_lo = fmax(eta_lo, fast_exp(-L.ln_inv[K_LIN]));
  if (gbs) eta_lo = fmax(eta_lo, fast_exp(-L.ln_inv_gbs));
  return eta_lo;
}

// exact: the local solve starts where the reference's does (start descriptor 0)
__device__ inline void iso_setup(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                 IsoState &S, PointOut &o, bool exact = true) {
  const int fl = ph.flags;
  const int constant = (fl & F_CST) != 0, diffusion = (fl & F_LIN) != 0, gs = (fl & F_GS) != 0;
  const int peierls = ((fl & F_EXPV) != 0) && fp64_lt(c.Traw, M.TmaxPeierls);
  const int plastic = c.plastic_on ? ((fl & F_PL1) ? 1 : ((fl & F_PL2) ? 2 : 0)) : 0;
  const int elastic = c.elastic;
  const double T = c.T, P = in.P, Eii = c.Eii, eta_el = c.eta_el;
  o.status = MDZ_OK;
  o.f32_steps = 0;
  o.mech = (constant ? MDZ_MECH_CONSTANT : 0) | ((fl & F_PWL) ? MDZ_MECH_DISLOCATION : 0) |
           (peierls ? MDZ_MECH_PEIERLS : 0) | (diffusion ? MDZ_MECH_DIFFUSION : 0) |
           ((fl & F_GBS) ? MDZ_MECH_GBS : 0) | (gs ? MDZ_MECH_GRAIN_SIZE : 0) |
           (plastic ? MDZ_MECH_PLASTIC : 0) | (elastic ? MDZ_MECH_ELASTIC : 0);
  o.Pcorr = P;
  o.X1 = in.X0;
  o.Eii_gbs = 0.0;  // C_gbs is never set by the reference (:616-642)
  o.OverS = 0.0;
  o.Wtot = o.Wel = o.Wdiss = 0.0;
  o.Eii_el = 0.0;
  o.rho = 0.0;
  o.d1 = ph.gs_ref;
  o.inv_d1 = ph.inv_gs_ref;
  if (diffusion && fp64_gt(ph.lin_m, 0.0) && fp64_lt(in.d, M.d_min)) set_status(o.status, MDZ_EGRAIN_ZERO);

  Laws &L = S.L;
  creep_laws(M, ph, c, P, in.phi, c.lnd, peierls, L);
  double Tyield = 0.0, C = in.C;
  if (plastic == 1) {  // :530-539 (products and sum rounded apart: the same bits in every kernel)
    Tyield = __dadd_rn(__dmul_rn(C, c.cos_fric), __dmul_rn(P, c.sin_fric));
    if (fp64_lt(ph.Slim, Tyield)) { C = ph.Slim; Tyield = ph.Slim; }
  }
  double eta_cst = 0.0, Ag = 0.0, lnd = c.lnd;
  if (constant) eta_cst = ph.eta0;
  if (fl & F_CMIX) {  // :563-565
    const double X0 = in.X0, e1 = ph.eta0, e2 = ph.eta0_two;
    if (M.diffuse_avg == 0) eta_cst = X0 * e1 + (1 - X0) * e2;
    if (M.diffuse_avg == 1) eta_cst = pow(X0 / e1 + (1 - X0) / e2, -1.0);
    if (M.diffuse_avg == 2) eta_cst = exp(X0 * log(e1) + (1 - X0) * log(e2));
  }
  if (gs) {  // wattmeter grain size before eta_lin (:567-576)
    Ag = ph.Kpzm * exp(-ph.Qpzm / M.R / T);
    const double Tii0 = 2. * eta_el * Eii;
    const double epwl0 = Tii0 / 2.0 * law_inv(L, K_PWL);
    const double d = exp(log(Ag * ph.Gpzm / (ph.Lpzm * (1.0 / ph.cpzm) * Tii0 * epwl0 * ph.ppzm)) / (1.0 + ph.ppzm));
    o.d1 = d;
    lnd = log(d);
    if (diffusion) {
      const double lnBd = !fp64_is_zero(ph.lin_m) ? fma(ph.lin_mn, lnd, L.lnB_lin) : L.lnB_lin;
      L.ln_inv[K_LIN] = c.lnEii - fma(c.lnEii, ph.lin_invn, lnBd);
    }
  }
  // bracket (:582-592): the smallest isolated viscosity is 1 / the largest reciprocal
  const double ln_inv_max =
      fp64_fmax(fp64_fmax(L.ln_inv[K_PWL], L.ln_inv[K_EXP]), fp64_fmax(L.ln_inv[K_LIN], L.ln_inv_gbs));
  start_point(M, ln_inv_max, constant, eta_cst, elastic == 1, c, exact || gs, S);
  S.eta_cst = eta_cst; S.Tyield = Tyield; S.C = C; S.Ag = Ag; S.lnd = lnd;
}

// The state of one (node, phase) between its visco-elastic solve and its post-processing.
struct IsoMid {
  double eta_ve, Tii, Tii_ve, Tyield, e_cst, e_pwl, e_exp, e_lin;
  double gdot, divp, Pc, eta_vep, lam_dot, A_tau, A_P, eta_vp;
  int is_pl;
};

// Inputs and results of the Drucker-Prager return of one (node, phase) (plastic == 1,
// RheologyDensity.c:655-707).  It depends only on these and on the phase's constants, so a
// CTA can run the returns of all its yielding items together, one per thread
// (k_sweep_compact), with the bits of the inline return.
struct DpItem {
  double Tii, Tyield, eta_ve, P, K, sin_fric, sin_dil, Eii, inv2Eii;  // in; Tii, Tyield out
  double gdot, divp, Pc, eta_vp, eta_vep;                              // out
};

__device__ __forceinline__ bool iso_yields_dp(const ModelConst &M, const PhaseConst &ph, const NodeCtx &c,
                                              const IsoMid &m) {
  const int plastic = c.plastic_on ? ((ph.flags & F_PL1) ? 1 : ((ph.flags & F_PL2) ? 2 : 0)) : 0;
  return plastic == 1 && fp64_gt(m.Tii - m.Tyield, 1e-17);
}

__device__ __forceinline__ void dp_load(DpItem &d, const IsoMid &m, const NodeIn &in, const NodeCtx &c) {
  d.Tii = m.Tii; d.Tyield = m.Tyield; d.eta_ve = m.eta_ve; d.P = in.P; d.K = c.K;
  d.sin_fric = c.sin_fric; d.sin_dil = c.sin_dil; d.Eii = c.Eii; d.inv2Eii = c.inv2Eii;
}

__device__ __forceinline__ void dp_store(IsoMid &m, const DpItem &d) {
  m.is_pl = 1;
  m.Tii = d.Tii; m.Tyield = d.Tyield; m.gdot = d.gdot; m.divp = d.divp; m.Pc = d.Pc; m.eta_vp = d.eta_vp;
  m.eta_vep = d.eta_vep;
}

// The Drucker-Prager return (:655-707) of an item that yields (Tii - Tyield > 1e-17).
__device__ inline void dp_return(const ModelConst &M, const PhaseConst &ph, DpItem &d) {
  const int fl = ph.flags;
  const double Tii = d.Tii, eta_ve = d.eta_ve, P = d.P, dt = M.dt;
  double Tyield = d.Tyield;
  double F = Tii - Tyield;
  const double tol = M.eta_tol, eta_vp0 = ph.eta_vp, n_vp = ph.n_vp;
  const bool vp1 = (fl & F_VP1) != 0;
  // The products and sums of this return are rounded one by one (explicit intrinsics, which
  // the compiler never fuses), as the reference's unfused arithmetic does: left to the
  // compiler, whether a product fused into the following sum depended on the kernel the
  // function was inlined into, and the iteration magnified that last bit.
  const double Kdt = __dmul_rn(d.K, dt);
  const double ksd = __dmul_rn(__dmul_rn(Kdt, d.sin_fric), d.sin_dil);
  double Tiic = 0.0, divp = 0.0, Pc = P;
  double eta_vp = vp1 ? eta_vp0 : eta_vp0 * pow(d.Eii, 1.0 / n_vp - 1);
  double gdot = quotient(F, eta_ve + eta_vp + ksd);
  const double F0 = F, tolF0 = tol * F0;
  // with n_vp == 1, eta_vp / n_vp is eta_vp exactly and the derivative is a constant
  const double dF1 = __dsub_rn(__dsub_rn(-eta_ve, eta_vp0), ksd);
  // The return is a fixed map of the state (gdot, Tyield) entering each iteration.  When
  // the state that the update produces equals one already entered -- the previous
  // iteration's (the Newton step rounds away) or the one before (two states alternate
  // in the last bit) -- every later iteration repeats one already done, and the values
  // the loop ends with at its cap of 20 are known now: stop there instead of running
  // the repeats.  The results are those of the full loop, bit for bit.
  unsigned long long g1 = ~0ull, y1 = ~0ull;  // state entering the previous iteration
  int last = 19;
  for (int it = 0; it <= last; it++) {
    const unsigned long long g0 = fp64_bits(gdot), y0 = fp64_bits(Tyield);
    divp = __dmul_rn(gdot, d.sin_dil);
    Pc = __dadd_rn(P, __dmul_rn(Kdt, divp));
    eta_vp = vp1 ? eta_vp0 : eta_vp0 * pow(fabs(gdot), 1.0 / n_vp - 1.0);
    Tyield = __dadd_rn(Tyield, __dmul_rn(gdot, eta_vp));
    Tiic = __dsub_rn(Tii, __dmul_rn(eta_ve, gdot));
    F = Tiic - Tyield;
    if (fp64_abs_lt(F, tol) || fp64_abs_lt(F, tolF0)) break;
    gdot -= F / (vp1 ? dF1 : (-eta_ve - eta_vp / n_vp - ksd));
    if (it == last) break;
    const unsigned long long gn = fp64_bits(gdot), yn = fp64_bits(Tyield);
    if (gn == g0 && yn == y0) break;  // period 1: iteration 19 would be this one
    if (gn == g1 && yn == y1) {       // period 2: iteration 19 repeats this one or the next
      if (((19 - it) & 1) == 0) break;
      last = it + 1;
    }
    g1 = g0; y1 = y0;
  }
  if (fp64_lt(Tiic, 0.0)) { gdot = (Tii - M.Tiimin) / (eta_ve); Tiic = M.Tiimin; Pc = P; }  // :697-704
  d.gdot = gdot; d.divp = divp; d.Pc = Pc; d.eta_vp = eta_vp; d.Tyield = Tyield;
  d.eta_vep = Tiic * d.inv2Eii;
  d.Tii = Tiic;
}

// Local solve (from s_start * eta_up, moved by the start stages that the descriptor
// `polish` names (ve_start); s_start = 1 and polish = 0 is the reference's start) of one
// (node, phase), up to its plastic corrections.  eta_conv (may be null) receives the
// converged visco-elastic viscosity, before plasticity.
__device__ inline void iso_ve(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                              IsoState &S, float s_start, int polish, PointOut &o, IsoMid &m,
                              double *eta_conv = nullptr) {
  const int fl = ph.flags;
  const int constant = (fl & F_CST) != 0, dislocation = (fl & F_PWL) != 0, diffusion = (fl & F_LIN) != 0;
  const int gbs = (fl & F_GBS) != 0, gs = (fl & F_GS) != 0;
  const int peierls = ((fl & F_EXPV) != 0) && fp64_lt(c.Traw, M.TmaxPeierls);
  const int elastic = c.elastic;
  const double P = in.P, Eii = c.Eii, eta_el = c.eta_el;
  Laws &L = S.L;
  const double eta_up = S.eta_up, eta_cst = S.eta_cst, Ag = S.Ag;
  const double Tyield = S.Tyield;
  double eta_ve, Tii, e_cst, e_pwl, e_exp, e_lin;
  if (!gs) {  // LocalIterationViscoElastic (:646)
    VeCoef q;
    ve_coef(L, c, eta_cst, S.eta_n, S.ln_eta_n, q);
    VeState s;
    s.status = MDZ_OK;
    ve_newton(q, ve_start(q, s_start * S.s_up, start_fp32(polish), start_dd(polish), o.f32_steps, S.s_up), s,
              S.s_up, polish != 0);
    set_status(o.status, s.status);
    eta_ve = s.eta; Tii = s.Tii; e_cst = s.e_cst; e_pwl = s.e_pwl; e_exp = s.e_exp; e_lin = s.e_lin;
    o.iters = s.iters;
  } else {  // LocalIterationViscoElasticGrainSize (:644)
    const double eta_lo = lower_viscosity(M, L, constant, eta_cst, elastic == 1, eta_el, gbs);
    GseIn g;
    g.Eii = Eii; g.eta_el = eta_el; g.eta_cst = eta_cst;
    g.C_pwl = exp(-ph.pwl_n * (kLn2 + L.lnB_pwl)); g.n_pwl = ph.pwl_n;
    g.C_lin = exp(-ph.lin_n * (kLn2 + L.lnB_lin)); g.n_lin = ph.lin_n; g.m_lin = ph.lin_m;
    g.C_exp = exp(fma(L.n[K_EXP], log(ph.exp_s3gS), L.lnA_exp)); g.ST = L.ST; g.n_exp = ph.exp_n;
    g.eta_up = eta_up; g.eta_lo = eta_lo; g.Ag = Ag; g.gam = ph.Gpzm; g.lam = ph.Lpzm;
    g.cg = ph.cpzm; g.pg = ph.ppzm; g.elastic = elastic; g.constant = constant; g.dislocation = dislocation;
    g.peierls = peierls; g.diffusion = diffusion;
    eta_ve = eta_up;
    Tii = 2.0 * eta_ve * Eii;
    double dd = o.d1;
    int st = MDZ_OK;
    ve_gse(g, eta_ve, Tii, dd, e_cst, e_pwl, e_exp, e_lin, o.iters, st);
    set_status(o.status, st);
    o.d1 = dd;
    o.inv_d1 = 1.0 / dd;
  }
  if (eta_conv) *eta_conv = eta_ve;
  m.eta_ve = eta_ve; m.Tii = Tii; m.Tii_ve = Tii; m.Tyield = Tyield;
  m.e_cst = e_cst; m.e_pwl = e_pwl; m.e_exp = e_exp; m.e_lin = e_lin;
  m.gdot = 0.0; m.divp = 0.0; m.Pc = P; m.eta_vep = 0.0; m.lam_dot = 0.0; m.A_tau = 1.0; m.A_P = 0.0;
  m.eta_vp = ph.eta_vp;
  m.is_pl = 0;
}

// Plastic corrections but the Drucker-Prager return (which dp_return does), and the
// post-processing of one (node, phase) after its visco-elastic solve (:655-1073).
__device__ inline void iso_post(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                IsoState &S, PointOut &o, IsoMid &m) {
  const int fl = ph.flags;
  const int constant = (fl & F_CST) != 0, dislocation = (fl & F_PWL) != 0, diffusion = (fl & F_LIN) != 0;
  const int gs = (fl & F_GS) != 0;
  const int peierls = ((fl & F_EXPV) != 0) && fp64_lt(c.Traw, M.TmaxPeierls);
  const int plastic = c.plastic_on ? ((fl & F_PL1) ? 1 : ((fl & F_PL2) ? 2 : 0)) : 0;
  const int elastic = c.elastic;
  const double T = c.T, P = in.P, Eii = c.Eii, K = c.K;
  const double eta_cst = S.eta_cst, C = S.C, lnd = S.lnd;
  (void)T;
  const double eta_ve = m.eta_ve, Tii_ve = m.Tii_ve;
  const double e_cst = m.e_cst, e_pwl = m.e_pwl, e_exp = m.e_exp, e_lin = m.e_lin;
  double Tii = m.Tii;
  int is_pl = m.is_pl;
  double gdot = m.gdot, divp = m.divp, Pc = m.Pc, eta_vep = m.eta_vep, lam_dot = m.lam_dot, A_tau = m.A_tau;
  double eta_vp = m.eta_vp;
  if (is_pl && plastic == 1) o.Pcorr = Pc;
  double A_P = 0.0;
  if (plastic == 2) {
    int st = MDZ_OK;
    double Tn = Tii;
    is_pl = plastic_popov(M, ph, Tii, P, C, c.cos_fric, c.sin_fric, c.sin_dil, eta_ve, K, Tn, Pc, lam_dot, A_tau,
                          A_P, eta_vp, st);
    set_status(o.status, st);
    if (is_pl) {
      o.Pcorr = Pc;
      eta_vep = Tn * c.inv2Eii;
      Tii = Tn;
      divp = lam_dot * A_P;
    }
  }

  // density on centroids (:934-960); only density_variations==1 lets it reach the grid
  if (in.centroid > 0 && in.want_rho) o.rho = density(M, ph, T, (in.final_update == 1) ? Pc : P, in.X0, in.phi);

  double inv_eta_pl = 0.0;
  if (is_pl == 0) o.etaVE = eta_ve;
  else if (plastic == 1) { o.etaVE = eta_vep; inv_eta_pl = quotient(gdot, Tii); }
  else { o.etaVE = eta_vep; inv_eta_pl = 2.0 * lam_dot * A_tau / Tii; }
  o.is_pl = is_pl;
  if (is_pl) o.mech |= MDZ_MECH_YIELD;
  o.Eii_cst = e_cst; o.Eii_pwl = e_pwl; o.Eii_exp = e_exp; o.Eii_lin = e_lin;
  // the dissipative viscosity: 1 / eta = sum_k 2 Eii_k / Tii (+ 1/eta_cst, 1/eta_pl)
  const auto dissipative = [&](double &inv_half_T) {
    inv_half_T = quotient(2.0, Tii_ve);  // 1/eta_k = 2 Eii_k / Tii
    double inv = 0.0;
    if (peierls) inv = __fma_rn(e_exp, inv_half_T, inv);
    if (dislocation) inv = __fma_rn(e_pwl, inv_half_T, inv);
    if (diffusion) {
      // eta_lin = B pow(Eii_lin, 1/n-1) pow(d1, m/n) = Tii/(2 Eii_lin) (d1/d)^(m/n), d1 = gs_ref
      double inv_lin = e_lin * inv_half_T;
      if (!fp64_is_zero(ph.lin_m) && !gs) inv_lin *= fast_exp(ph.lin_mn * (lnd - ph.ln_gs_ref));
      inv += inv_lin;
    }
    if (constant) inv += (1.0 / eta_cst);
    if (is_pl == 1) inv += inv_eta_pl;
    return inv;
  };

  double eta = 0.0;
  if (in.post_process == 2) {  // a vertex of the sweep: only etaVE, eta and X are kept
    double inv_half_T;
    eta = quotient(1.0, dissipative(inv_half_T));
  } else {
    o.Txx = 2.0 * o.etaVE * in.Exx;
    o.Tzz = 2.0 * o.etaVE * in.Ezz;
    o.Txz = 2.0 * o.etaVE * in.Exz;
    if (in.post_process == 1) {  // :986-1053
      double inv_half_T;
      const double inv = dissipative(inv_half_T);
      eta = quotient(1.0, inv);
      if (elastic) {
        const double h = 0.5 * c.inv_eta_el;
        const double Tyy = -(o.Txx + o.Tzz), Tyy0 = -(in.Txx0 + in.Tzz0);
        const double ex = (o.Txx - in.Txx0) * h, ez = (o.Tzz - in.Tzz0) * h;
        const double ey = (Tyy - Tyy0) * h, exz = (o.Txz - in.Txz0) * h;
        o.Eii_el = sqrt(__fma_rn(0.5, __fma_rn(ey, ey, __fma_rn(ez, ez, __dmul_rn(ex, ex))), __dmul_rn(exz, exz)));
      }
      o.Eii_pl = (is_pl && plastic == 1) ? gdot / 2.0 : ((is_pl && plastic == 2) ? lam_dot * A_tau : 0.0);
      o.div_pl = divp;
      o.div_el = -(Pc - in.P0) * c.inv_Kdt;
      if (plastic == 1) o.OverS = eta_vp * gdot;
      if (plastic == 2) o.OverS = eta_vp * lam_dot * A_tau;
      if (in.centroid == 1) {
        const double T2 = Tii * Tii;
        o.Wtot = T2 * (Eii * inv_half_T);  // T2 / eta_ve, with Tii_ve = 2 eta_ve Eii
        o.Wel = T2 * c.inv_eta_el;
        o.Wdiss = T2 * inv;
        if (fp64_lt(o.Wdiss, 0.0)) set_status(o.status, MDZ_EWDISS);
      }
    } else {
      o.Eii_pl = 0.0;
      o.div_pl = (is_pl ? divp : 0.0);
      o.div_el = 0.0;
    }
  }
  // limiters (:1058-1073)
  if (fp64_gt(o.etaVE, M.max_eta)) o.etaVE = M.max_eta;
  if (fp64_lt(o.etaVE, M.min_eta)) o.etaVE = M.min_eta;
  if (fp64_gt(eta, M.max_eta)) eta = M.max_eta;
  if (fp64_lt(eta, M.min_eta)) eta = M.min_eta;
  o.eta = eta;
}

// Local solve, plastic corrections and post-processing of one (node, phase): iso_ve, the
// Drucker-Prager return where the item yields, iso_post.
__device__ inline void iso_finish(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                  IsoState &S, float s_start, int polish, PointOut &o,
                                  double *eta_conv = nullptr) {
  IsoMid m;
  iso_ve(M, ph, in, c, S, s_start, polish, o, m, eta_conv);
  if (iso_yields_dp(M, ph, c, m)) {
    DpItem d;
    dp_load(d, m, in, c);
    dp_return(M, ph, d);
    dp_store(m, d);
  }
  iso_post(M, ph, in, c, S, o, m);
}

__device__ inline void point_iso(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                 int polish, PointOut &o) {
  IsoState S;
  iso_setup(M, ph, in, c, S, o, polish == 0);
  iso_finish(M, ph, in, c, S, 1.0f, polish, o);
}

// CTA-level compaction of the Drucker-Prager returns.  The return of an item that yields
// takes a few iterations with a division each, and about one item in eleven yields: inline,
// nearly every warp carries one or two yielding lanes through the return while the other
// lanes wait.  A kernel whose CTA (at most 128 threads) walks its items' phases in step
// calls dp_compact with every thread once per phase, after iso_ve: the yielding items are
// gathered by ballot into a queue in shared memory (one shared atomic per warp, slots by
// popcount), the first threads of the CTA run one return each, packed into as few warps as
// the queue needs, and every owner takes its result back for iso_post.  The same
// functions as iso_finish, so the same bits.
struct CompactQueue {
  DpItem item[128];
  int count[2];  // per phase parity: the counter of the phase in flight and of the next
};

__device__ __forceinline__ void compact_init(CompactQueue &Q) {
  if (threadIdx.x < 2) Q.count[threadIdx.x] = 0;
  __syncthreads();
}

// par: the phase parity, flipped here.  count[par ^ 1] is cleared between the two
// barriers, where no thread touches it; count[par] is read only between them.
__device__ __forceinline__ void dp_compact(const ModelConst &M, const PhaseConst &ph, CompactQueue &Q, int &par,
                                           bool yields, IsoMid &m, const NodeIn &in, const NodeCtx &c) {
  const int t = threadIdx.x, lane = t & 31;
  const unsigned ball = __ballot_sync(0xffffffffu, yields);
  int slot = 0;
  if (lane == 0 && ball) slot = atomicAdd(&Q.count[par], __popc(ball));
  slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(ball & ((1u << lane) - 1u));
  if (yields) dp_load(Q.item[slot], m, in, c);
  __syncthreads();
  const int q = Q.count[par];
  if (t == 0) Q.count[par ^ 1] = 0;
  if (t < q) {
    DpItem d = Q.item[t];
    dp_return(M, ph, d);
    Q.item[t] = d;
  }
  __syncthreads();
  if (yields) dp_store(m, Q.item[slot]);
  par ^= 1;
}

// ---------------------------------------------------------------------------------------
// ViscosityConciseAniso (AnisotropyRoutines.c:282-727).  The node context carries the
// rotated-frame invariant; Er_* are the rotated strain-rate components.
// ---------------------------------------------------------------------------------------
struct AnisoNode {
  double Er_xx, Er_zz, Er_xz, lxlz, lx2;
};

// Rotated strain rate and its invariant (AnisotropyRoutines.c:379-390).
__device__ __forceinline__ void node_strain_aniso(const NodeIn &in, NodeCtx &c, AnisoNode &a) {
  const double lx2 = in.lx2, lxlz = in.lxlz, nz2 = 1.0 - lx2;  // :379-383
  a.lx2 = lx2; a.lxlz = lxlz;
  a.Er_xx = lx2 * in.Exx + nz2 * in.Ezz + 2. * lxlz * in.Exz;
  a.Er_zz = nz2 * in.Exx + lx2 * in.Ezz - 2. * lxlz * in.Exz;
  a.Er_xz = -lxlz * in.Exx + lxlz * in.Ezz + (lx2 - nz2) * in.Exz;
  const double Er_yy = -a.Er_xx - a.Er_zz;
  c.Eii = sqrt(0.5 * (a.Er_xx * a.Er_xx + a.Er_zz * a.Er_zz + Er_yy * Er_yy) + a.Er_xz * a.Er_xz);
}

__device__ __forceinline__ void node_setup_aniso(const ModelConst &M, const NodeIn &in, bool need_lnd, NodeCtx &c,
                                                 AnisoNode &a) {
  node_strain_aniso(in, c, a);
  c.elastic = (M.step == 0) ? 0 : M.elastic;
  c.plastic_on = 1;
  c.K = quotient(1.0, in.beta);
  c.G = in.G;
  c.dil = in.dil;
  if (c.elastic == 0) { c.G = 1e1; c.dil = 0.0; }
  c.eta_el = c.elastic ? c.G * M.dt_model : 1e20;
  c.inv_eta_el = quotient(1.0, c.eta_el);
  c.ln_eta_el = c.elastic ? fast_log(c.eta_el) : 0.0;
  c.inv_Kdt = quotient(1.0, c.K * M.dt_model);
  node_common(M, in, need_lnd, c);
  c.inv_d = 1.0 / in.d;
}

__device__ inline void aniso_setup(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                   const AnisoNode &an, IsoState &S, PointOut &o, bool exact = true) {
  const int fl = ph.flags;
  const int constant = (fl & F_CST) != 0, dislocation = (fl & F_PWL) != 0, diffusion = (fl & F_LIN) != 0;
  const int peierls = ((fl & F_EXPV) != 0) && fp64_lt(c.Traw, M.TmaxPeierls);
  const int plastic = (fl & F_PLANY) != 0;
  const int elastic = c.elastic;
  const double T = c.T, P = in.P, eta_el = c.eta_el, K = c.K, dt = M.dt_model;
  const double min_eta = M.min_eta, max_eta = M.max_eta;
  o.status = MDZ_OK;
  o.f32_steps = 0;
  o.mech = (constant ? MDZ_MECH_CONSTANT : 0) | (dislocation ? MDZ_MECH_DISLOCATION : 0) |
           (peierls ? MDZ_MECH_PEIERLS : 0) | (diffusion ? MDZ_MECH_DIFFUSION : 0) |
           ((fl & F_GS) ? MDZ_MECH_GRAIN_SIZE : 0) | (plastic ? MDZ_MECH_PLASTIC : 0) |
           (elastic ? MDZ_MECH_ELASTIC : 0);
  o.Pcorr = P;
  o.X1 = 0.0; o.rho = 0.0; o.Eii_gbs = 0.0; o.Eii_el = 0.0; o.Eii_pl = 0.0; o.div_pl = 0.0; o.div_el = 0.0;
  o.OverS = 0.0; o.Wtot = o.Wel = o.Wdiss = 0.0;
  o.d1 = in.d;
  o.inv_d1 = c.inv_d;
  if (diffusion && fp64_gt(ph.lin_m, 0.0) && fp64_lt(in.d, M.d_min)) set_status(o.status, MDZ_EGRAIN_ZERO);

  Laws &L = S.L;
  creep_laws(M, ph, c, P, in.phi, c.lnd, peierls, L);
  L.mech &= ~F_GBS;  // the anisotropic path has no grain-boundary sliding
  L.ln_inv_gbs = -kInf;
  double Tyield = 0.0, Coh = in.C;
  if (plastic) {  // :370-377 (products and sum rounded apart: the same bits in every kernel)
    Tyield = __dadd_rn(__dmul_rn(Coh, c.cos_fric), __dmul_rn(P, c.sin_fric));
    if (ph.Slim < Tyield) { Coh = ph.Slim; Tyield = ph.Slim; }
  }
  const double eta_cst = constant ? ph.eta0 : 0.0;
  // bracket (:409-415); its lower end is formed only where it is used
  const double ln_inv_max = fp64_fmax(fp64_fmax(L.ln_inv[K_PWL], L.ln_inv[K_EXP]), L.ln_inv[K_LIN]);
  start_point(M, ln_inv_max, constant, eta_cst, elastic != 0, c, exact || (fl & F_GS), S);
  S.eta_cst = eta_cst; S.Tyield = Tyield; S.C = Coh; S.Ag = 0.0;
  S.lnd = c.lnd;
  (void)an; (void)T; (void)K; (void)dt; (void)min_eta; (void)max_eta; (void)dislocation; (void)eta_el;
}

// Local solve, plasticity, post-processing.  The Newton starts from the reference's
// bisection when s_start <= 0 and polish == 0; otherwise from s_start * eta_up (eta_up
// when s_start <= 0) moved by the start stages that the descriptor `polish` names.
__device__ inline void aniso_finish(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                   const AnisoNode &an, IsoState &S, float s_start, int polish, PointOut &o,
                                   double *eta_conv = nullptr) {
  const int fl = ph.flags;
  const int constant = (fl & F_CST) != 0, dislocation = (fl & F_PWL) != 0, diffusion = (fl & F_LIN) != 0;
  const int peierls = ((fl & F_EXPV) != 0) && fp64_lt(c.Traw, M.TmaxPeierls);
  const int plastic = (fl & F_PLANY) != 0;
  const int elastic = c.elastic;
  const double T = c.T, P = in.P, Eii = c.Eii, eta_el = c.eta_el, K = c.K, dt = M.dt_model;
  const double min_eta = M.min_eta, max_eta = M.max_eta;
  Laws &L = S.L;
  const double eta_up = S.eta_up, eta_cst = S.eta_cst, Tyield = S.Tyield;
  double eta_ve = eta_up, Tii = 0.0, e_cst = 0.0, e_pwl = 0.0, e_exp = 0.0, e_lin = 0.0;
  if (fl & F_GS) {  // :429-473
    GseIn g;
    g.Eii = Eii; g.eta_el = eta_el; g.eta_cst = eta_cst;
    g.C_pwl = exp(-ph.pwl_n * (kLn2 + L.lnB_pwl)); g.n_pwl = ph.pwl_n;
    g.C_lin = exp(-ph.lin_n * (kLn2 + L.lnB_lin)); g.n_lin = ph.lin_n; g.m_lin = ph.lin_m;
    g.C_exp = exp(fma(L.n[K_EXP], log(ph.exp_s3gS), L.lnA_exp)); g.ST = L.ST; g.n_exp = ph.exp_n;
    g.eta_up = eta_up; g.eta_lo = lower_viscosity(M, L, constant, eta_cst, elastic != 0, eta_el, false);
    g.Ag = ph.Kpzm * exp(-ph.Qpzm / (M.R * T));
    g.gam = ph.Gpzm; g.lam = ph.Lpzm; g.cg = ph.cpzm; g.pg = ph.ppzm; g.elastic = elastic; g.constant = constant;
    g.dislocation = dislocation; g.peierls = peierls; g.diffusion = diffusion;
    double dd = in.d;
    int st = MDZ_OK;
    ve_gse(g, eta_ve, Tii, dd, e_cst, e_pwl, e_exp, e_lin, o.iters, st);
    set_status(o.status, st);
    o.d1 = dd;
    o.inv_d1 = 1.0 / dd;
  } else {  // :474-585: 10 log-space bisection steps on [min_eta 1e-3, 10 max(eta_lo, max_eta)], then Newton
    const double tol = 1e-11;
    VeCoef q;
    ve_coef(L, c, eta_cst, S.eta_n, S.ln_eta_n, q);
    VeState s;
    s.status = MDZ_OK;
    double r, sv;  // sv = eta_ve / eta_n (eta_n = eta_up from the bisection: that start is exact)
    if (s_start > 0.0f || polish > 0) {
      sv = ve_start(q, ((s_start > 0.0f) ? s_start : 1.0f) * S.s_up, start_fp32(polish), start_dd(polish),
                    o.f32_steps, S.s_up);
    } else {
      const double inv_up = 1.0 / eta_up;
      const double eta_lo = lower_viscosity(M, L, constant, eta_cst, elastic != 0, eta_el, false);
      double lo = min_eta * 1.0e-3, hi = 10.0 * fmax(eta_lo, max_eta);
      for (int bit = 0; bit < 10; bit++) {
        eta_ve = sqrt(lo * hi);
        ve_eval(q, eta_ve * inv_up, s, r);
        if (r > 0.0) lo = eta_ve;
        else hi = eta_ve;
        if (fabs(r) < q.thr_conv) break;
      }
      sv = sqrt(lo * hi) * inv_up;
    }
    // a moved start (not the bisection's) that has not converged within the cap is
    // abandoned for the upper bound eta_up, above the root, with a fresh cap
    bool moved = s_start > 0.0f || polish > 0;
    o.iters = 0;
    double step = -1.0;  // binomial update of the previous point's terms (see ve_eval)
    for (int it = 0; it < 50; it++) {
      ve_eval(q, sv, s, r, step);
      o.iters++;
      if (fp64_is_nan(r)) { set_status(o.status, MDZ_EANISO_NAN); break; }
      const double d = newton_quotient(r, fma(q.Aup, sv, ve_S(q, s)));
      sv = fma(sv, d, sv);
      step = fp64_lt(fabs(d) * q.nmax, 1e-5) ? d : -1.0;
      if (fp64_le(sv, 0.0)) { sv = min_eta / q.eta_up; step = -1.0; }
      const double ar = fabs(r);
      if (fp64_abs_lt(r, q.thr_conv)) break;
      if (it == 49 && moved && !(ar < 10.0 * tol * Eii)) {
        moved = false;
        sv = f64_of_f32(S.s_up);
        step = -1.0;
        it = -1;
        continue;
      }
      if (it == 49 && ar < 10.0 * tol * Eii) break;
      if (it == 49 && ar > q.thr_fail) { set_status(o.status, MDZ_EANISO_ITER); break; }
    }
    eta_ve = sv * q.eta_up;
    Tii = s.Tii; e_cst = s.e_cst; e_pwl = s.e_pwl; e_exp = s.e_exp; e_lin = s.e_lin;
  }
  if (fp64_lt(eta_ve, min_eta)) eta_ve = min_eta;  // :589-603
  if (fp64_gt(eta_ve, max_eta)) eta_ve = max_eta;
  const double Tii_ve = Tii;
  if (eta_conv) *eta_conv = eta_ve;
  double Tr_xx = 2.0 * eta_ve * an.Er_xx, Tr_zz = 2.0 * eta_ve * an.Er_zz, Tr_xz = 2.0 * eta_ve * an.Er_xz / in.ani_fac;
  double eta_vep = eta_ve, gdot = 0.0, Pc = P;
  const double Ft = Tii - Tyield;
  int is_pl = 0;
  if (fp64_gt(Ft, 1e-17) && plastic) {  // :625-648
    is_pl = 1;
    // rounded one by one, as in the isotropic return
    const double Kdt_sd = __dmul_rn(__dmul_rn(K, dt), c.sin_dil);
    gdot = quotient(Ft, __dadd_rn(__dadd_rn(eta_ve, ph.eta_vp), __dmul_rn(Kdt_sd, c.sin_fric)));
    const double Tiic = __dsub_rn(Tii, __dmul_rn(gdot, eta_ve));
    Pc = __dadd_rn(P, __dmul_rn(Kdt_sd, gdot));
    eta_vep = Tiic * c.inv2Eii;
    Tr_xx = 2.0 * eta_vep * an.Er_xx;
    Tr_zz = 2.0 * eta_vep * an.Er_zz;
    Tr_xz = 2.0 * eta_vep * an.Er_xz / in.ani_fac;
    o.div_pl = gdot * c.sin_dil;
    o.Eii_pl = gdot / 2.0;
    Tii = Tiic;
  }
  if (in.post_process != 2) {
    const double lx2 = an.lx2, lxlz = an.lxlz, nz2 = 1.0 - lx2;  // :650-652
    o.Txx = lx2 * Tr_xx + nz2 * Tr_zz - 2. * lxlz * Tr_xz;
    o.Tzz = nz2 * Tr_xx + lx2 * Tr_zz + 2. * lxlz * Tr_xz;
    o.Txz = lxlz * Tr_xx - lxlz * Tr_zz + (lx2 - nz2) * Tr_xz;
  }
  o.Pcorr = Pc;
  if (fp64_lt(eta_vep, min_eta)) eta_vep = min_eta;
  if (fp64_gt(eta_vep, max_eta)) eta_vep = max_eta;
  o.etaVE = eta_vep;
  o.is_pl = is_pl;
  if (is_pl) o.mech |= MDZ_MECH_YIELD;
  o.Eii_cst = e_cst; o.Eii_pwl = e_pwl; o.Eii_exp = e_exp; o.Eii_lin = e_lin;
  double eta = eta_vep;
  double inv = 0.0;
  if (in.post_process != 0) {  // :681-714 (eta_lin uses *d, the same d as the Newton: no correction)
    const double inv_half_T = quotient(2.0, Tii_ve);
    if (diffusion) inv += e_lin * inv_half_T;
    if (peierls) inv += e_exp * inv_half_T;
    if (dislocation) inv += e_pwl * inv_half_T;
    if (constant) inv += 1.0 / eta_cst;
    if (is_pl) inv += quotient(gdot, Tii);
    eta = quotient(1.0, inv);
  }
  if (in.post_process == 1) {
    if (elastic) o.Eii_el = Tii * Tii * (0.25 * c.inv_eta_el * c.inv_eta_el);
    if (is_pl) o.Eii_pl = gdot / 2.0;
    o.div_pl = gdot * c.sin_dil;
    o.div_el = -(Pc - in.P0) * c.inv_Kdt;
    o.OverS = ph.eta_vp * gdot;
    if (in.centroid == 1) {
      const double T2 = Tii * Tii;
      o.Wtot = T2 / eta_ve;
      o.Wel = T2 * c.inv_eta_el;
      o.Wdiss = T2 * inv;
    }
  }
  if (fp64_gt(eta, max_eta)) eta = max_eta;  // :720-721
  if (fp64_lt(eta, min_eta)) eta = min_eta;
  o.eta = eta;
}

__device__ inline void point_aniso(const ModelConst &M, const PhaseConst &ph, const NodeIn &in, const NodeCtx &c,
                                   const AnisoNode &an, int polish, PointOut &o) {
  IsoState S;
  aniso_setup(M, ph, in, c, an, S, o, polish == 0);
  aniso_finish(M, ph, in, c, an, S, 0.0f, polish, o);
}

// EffectiveStrainRate, RheologyDensity.c:116-146
__device__ __forceinline__ void effective_strain_rate(double &Exx, double &Ezz, double &Exz, double exx, double ezz,
                                                      double exz, double Txx, double Tzz, double Txz, double d1,
                                                      double d2, double ani, double eta_e, int elastic) {
  if (!elastic) { Exx = exx; Ezz = ezz; Exz = exz; return; }
  const double Da11 = 2.0 - 2.0 * ani * d1, Da12 = 2.0 * ani * d1, Da13 = -2.0 * ani * d2;
  const double Da22 = 2.0 - 2.0 * ani * d1, Da23 = 2.0 * ani * d2, Da33 = 1.0 + 2.0 * ani * (d1 - 0.5);
  const double a11 = Da33 * Da22 - Da23 * Da23, a12 = Da13 * Da23 - Da33 * Da12, a13 = Da12 * Da23 - Da13 * Da22;
  const double a22 = Da33 * Da11 - Da13 * Da13, a23 = Da12 * Da13 - Da11 * Da23, a33 = Da11 * Da22 - Da12 * Da12;
  const double idet = 1.0 / ((Da11 * a11) + (Da12 * a12) + (Da13 * a13));
  const double ie = 1.0 / eta_e;
  Exx = exx + (a11 * Txx + a12 * Tzz + a13 * Txz) * idet * ie;
  Ezz = ezz + (a12 * Txx + a22 * Tzz + a23 * Txz) * idet * ie;
  Exz = exz + (a13 * Txx + a23 * Tzz + a33 * Txz) * idet * ie * 0.5;
}

// InterpCentroidsToVerticesDouble (GridRoutines.c:108-210): vertex (k,l) averages ring
// cells (k..k+1, l..l+1) of the ghost-ringed centroid field; each ring cell is one
// centroid (zero-flux edges, optional x-periodicity).  Air cells (30/31) count as 0.
__device__ __forceinline__ int ring_to_centroid(int i, int j, int Ncx, int Ncz, int per) {
  int cj = j - 1;
  cj = cj < 0 ? 0 : (cj > Ncz - 1 ? Ncz - 1 : cj);
  int ci;
  if (per == 1) ci = (i == 0) ? Ncx - 1 : ((i == Ncx + 1) ? 0 : i - 1);
  else { ci = i - 1; ci = ci < 0 ? 0 : (ci > Ncx - 1 ? Ncx - 1 : ci); }
  return ci + cj * Ncx;
}

}  // namespace mdz
