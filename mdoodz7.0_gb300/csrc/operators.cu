// operators.cu -- RheologicalOperators (MDLIB/StokesRoutines.c:75-410) on the GPU.
//
// k_operators<ANISO, JAC> writes the viscosity tensors D of the momentum equations,
// one thread per node over [centroids | vertices], from a grid that a sweep has just
// updated.  The Picard operator (JAC = false) is a few products per node.  The Newton
// operator (JAC = true) also needs d(eta)/dE, d(eta)/dP, d(div_pl)/dE and d(rho)/dP,
// which the reference forms by central differences over 8 perturbed local solves per
// node and active phase (DerivativesOnTheFly_n / _s, PhaseRheologyLoop_v1,
// MDLIB/FD_Jacobian.c:48-323).  Each thread runs its node's 8 x Nb_phases perturbed
// solves with the same device code as the sweep (post-processing off), so the whole
// Jacobian is one launch.
#include <cuda_runtime.h>

#include "operators.cuh"

namespace mdz {

namespace {

// Per-node inputs of the perturbed solves (PhaseRheologyLoop_v1's arguments).
struct OpNode {
  NodeIn in;       // base inputs: effective strain rates, P, fields of the node
  double eta;      // eta_n / eta_s of the node (the averaged viscosity)
  long long idx;   // c0 or c1
  bool centroid;
};

// PhaseRheologyLoop_v1 for one perturbed input: every active phase's local solve,
// accumulated into the derivative slots.  ctx / an: the node set-up of this input.
// COMPACT (isotropic): every thread of the CTA runs the phase loop together (has false: a
// thread without a node, which still takes part in the barriers) and the yielding items'
// Drucker-Prager returns run packed into the first warps (dp_compact); the same functions
// as point_iso, so the same bits.
template <bool ANISO, bool COMPACT>
__device__ __forceinline__ void phase_loop(const OpArgs &A, const OpNode &nd, bool has, const NodeIn &in,
                                           const NodeCtx &ctx, const AnisoNode &an, int is_centroid, double sign,
                                           double denom, double &detadE, double &ddivpdE, double &danidE,
                                           double *drhodP, CompactQueue *Q, int *par) {
  for (int p = 0; p < A.M.np; p++) {
    const double vol = has ? (nd.centroid ? A.perc_n[p][nd.idx] : A.perc_s[p][nd.idx]) : 0.0;
    const bool active = fp64_abs_gt(vol, 1e-13);
    if (!COMPACT && !active) continue;
    PointOut o;
    if (COMPACT) {
      IsoState st;
      IsoMid m;
      bool yields = false;
      if (active) {
        iso_setup(A.M, A.ph[p], in, ctx, st, o, A.polish == 0);
        iso_ve(A.M, A.ph[p], in, ctx, st, 1.0f, A.polish, o, m);
        yields = iso_yields_dp(A.M, A.ph[p], ctx, m);
      }
      dp_compact(A.M, A.ph[p], *Q, *par, yields, m, in, ctx);
      if (!active) continue;
      iso_post(A.M, A.ph[p], in, ctx, st, o, m);
    } else if (ANISO) {
      point_aniso(A.M, A.ph[p], in, ctx, an, A.polish, o);
    } else {
      point_iso(A.M, A.ph[p], in, ctx, A.polish, o);
    }
    const double eta_vep = o.etaVE;
    const int avg = A.M.eta_average;
    if (avg == 0) detadE += sign * vol * eta_vep / denom;
    else {
      const double ep = nd.centroid ? A.peta_n[p][nd.idx] : A.peta_s[p][nd.idx];
      if (avg == 1) detadE += sign * vol * eta_vep / denom / (ep * ep);
      else detadE += sign * vol * eta_vep / denom / ep;
    }
    danidE += sign * vol / denom;
    if (is_centroid > 0) ddivpdE += sign * vol * o.div_pl / denom;
    if (is_centroid == 2) *drhodP += sign * vol * o.rho / denom;
  }
}

// DerivativesOnTheFly_n (centroids, tol 1e-5) / _s (vertices, 1e-7).  d[]: d(eta)/d(Exx,
// Ezz, Gxz, P); v[]: d(div_pl)/d(...) (centroids); a[]: d(anisotropy factor)/d(...).
template <bool ANISO, bool COMPACT>
__device__ __forceinline__ void fd_derivatives(const OpArgs &A, const OpNode &nd, bool has, double d[4], double v[4],
                                               double a[4], double &drhodp, CompactQueue *Q = nullptr,
                                               int *par = nullptr) {
  const double tol = nd.centroid ? 1e-5 : 1e-7;
  const NodeIn &b = nd.in;
  const double pert[4] = {tol * fabs(b.Exx) + tol / 1e10, tol * fabs(b.Ezz) + tol / 1e10,
                          tol * fabs(b.Exz) + tol / 1e10, tol * fabs(b.P) + tol / 1e10};
  double vscratch = 0.0;
  // the node set-up once; a strain-rate perturbation then only changes the invariant
  NodeCtx base;
  AnisoNode base_an;
  if (has) {
    if (ANISO) node_setup_aniso(A.M, b, A.need_lnd != 0, base, base_an);
    else node_setup_iso(A.M, b, A.need_lnd != 0, base);
  }
#pragma unroll 1
  for (int dir = 0; dir < 4; dir++) {
#pragma unroll 1
    for (int s = 0; s < 2; s++) {
      const double sign = s == 0 ? 1.0 : -1.0;
      NodeIn in = b;
      if (dir == 0) in.Exx = b.Exx + sign * pert[0];
      if (dir == 1) in.Ezz = b.Ezz + sign * pert[1];
      if (dir == 2) in.Exz = b.Exz + sign * pert[2];
      if (dir == 3) in.P = b.P + sign * pert[3];
      const int is_centroid = nd.centroid ? (dir == 3 ? 2 : 1) : 0;
      in.centroid = is_centroid;
      in.want_rho = (is_centroid == 2);
      const double denom = (dir == 2 ? 4.0 : 2.0) * pert[dir];
      NodeCtx ctx = base;
      AnisoNode an = base_an;
      if (has && dir < 3) {
        if (ANISO) node_strain_aniso(in, ctx, an);
        else node_strain_iso(A.M, in, ctx);
        node_strain_update(ctx);
      }
      phase_loop<ANISO, COMPACT>(A, nd, has, in, ctx, an, is_centroid, sign, denom, d[dir],
                                 nd.centroid ? v[dir] : vscratch, a[dir], &drhodp, Q, par);
    }
  }
  if (A.M.eta_average == 1)
    for (int k = 0; k < 4; k++) d[k] *= nd.eta * nd.eta;
  if (A.M.eta_average == 2)
    for (int k = 0; k < 4; k++) d[k] *= nd.eta;
}

// The Newton operator's node: the base inputs of the perturbed solves and the averaged
// anisotropy terms (StokesRoutines.c:257-281 centroids, :328-351 vertices).
struct NewtonNode {
  OpNode nd;
  double ani_vep, aniS, d1, d2;
};

// Air nodes get zero operators (StokesRoutines.c:167-172, :240-243, :315-320, :370-373);
// returns false there.
template <bool ANISO>
__device__ __forceinline__ bool op_node_load(const OpArgs &A, long long i, NewtonNode &w) {
  const ModelConst &M = A.M;
  OpNode &nd = w.nd;
  nd.centroid = i < M.Nc;
  nd.idx = nd.centroid ? i : i - M.Nc;
  const long long c = nd.idx;
  const bool air = nd.centroid ? (A.bcp[c] == 30 || A.bcp[c] == 31) : (A.bcg[c] == 30);
  if (air) {
    if (nd.centroid) for (int j = 0; j < 8; j++) A.D[OP_D11 + j][c] = 0.0;
    else for (int j = 0; j < 4; j++) A.D[OP_D31 + j][c] = 0.0;
    return false;
  }
  nd.eta = nd.centroid ? A.eta_n[c] : A.eta_s[c];
  w.ani_vep = 1.0;
  w.aniS = w.d1 = w.d2 = 0.0;
  if (ANISO) {
    w.ani_vep = nd.centroid ? A.ci[CI_anif][c] : A.vi[VI_anif][c];
    w.aniS = 1.0 - 1.0 / w.ani_vep;
    w.d1 = nd.centroid ? A.ci[CI_d1][c] : A.vi[VI_d1][c];
    w.d2 = nd.centroid ? A.ci[CI_d2][c] : A.vi[VI_d2][c];
  }
  return true;
}

// Picard operator: StokesRoutines.c:94-166, :179-239
__device__ __forceinline__ void picard_store(const OpArgs &A, const NewtonNode &w) {
  const long long c = w.nd.idx;
  const double eta_vep = w.nd.eta, aniS = w.aniS, d1 = w.d1, d2 = w.d2;
  if (w.nd.centroid) {
    A.D[OP_D11][c] = 2.0 * eta_vep - 2.0 * aniS * d1 * eta_vep;
    A.D[OP_D12][c] = 2.0 * aniS * d1 * eta_vep;
    A.D[OP_D13][c] = -2.0 * aniS * d2 * eta_vep;
    A.D[OP_D14][c] = 0.0;
    A.D[OP_D21][c] = 2.0 * aniS * d1 * eta_vep;
    A.D[OP_D22][c] = 2.0 * eta_vep - 2.0 * aniS * d1 * eta_vep;
    A.D[OP_D23][c] = 2.0 * aniS * d2 * eta_vep;
    A.D[OP_D24][c] = 0.0;
  } else {
    A.D[OP_D31][c] = -2.0 * aniS * d2 * eta_vep;
    A.D[OP_D32][c] = 2.0 * aniS * d2 * eta_vep;
    A.D[OP_D33][c] = eta_vep + 2.0 * aniS * (d1 - 0.5) * eta_vep;
    A.D[OP_D34][c] = 0.0;
  }
}

// The base inputs of the Newton operator's perturbed solves: the node's fields and its
// effective strain rates (StokesRoutines.c:257-284, :328-354).
template <bool ANISO>
__device__ __forceinline__ void newton_inputs(const OpArgs &A, NewtonNode &w) {
  const ModelConst &M = A.M;
  OpNode &nd = w.nd;
  const long long c = nd.idx;
  NodeIn &in = nd.in;
  const double mu = nd.centroid ? A.ci[CI_mu][c] : A.vi[VI_mu][c];
  const double eta_e = (M.elastic == 1) ? M.dt_model * mu : 1.0;
  if (nd.centroid) {
    in.Txx0 = A.ci[CI_sxxd0][c]; in.Tzz0 = A.ci[CI_szzd0][c]; in.Txz0 = A.ci[CI_sxz0][c];
    in.T = A.ci[CI_T][c]; in.P = A.ci[CI_p_in][c]; in.d = A.ci[CI_d0][c]; in.phi = A.ci[CI_phi0][c];
    in.X0 = A.ci[CI_X0][c]; in.dil = A.ci[CI_dil][c]; in.fric = A.ci[CI_fric][c]; in.C = A.ci[CI_C][c];
    in.P0 = A.ci[CI_p0][c]; in.T0 = A.ci[CI_T0][c]; in.beta = A.ci[CI_bet][c];
  } else {
    in.Txx0 = A.vi[VI_sxxd0][c]; in.Tzz0 = A.vi[VI_szzd0][c]; in.Txz0 = A.vi[VI_sxz0][c];
    in.T = A.T_s[c]; in.P = A.P_s[c]; in.d = A.d0_s[c]; in.phi = A.phi0_s[c];
    in.X0 = A.vi[VI_X0][c]; in.dil = A.vi[VI_dil][c]; in.fric = A.vi[VI_fric][c]; in.C = A.vi[VI_C][c];
    in.P0 = A.vi[VI_p0][c]; in.T0 = 0.0; in.beta = A.vi[VI_bet][c];
  }
  in.G = mu;
  in.final_update = 0;
  in.post_process = 0;
  in.lxlz = in.lx2 = 0.0;
  in.ani_fac = w.ani_vep;
  if (ANISO) {
    const double angle = nd.centroid ? A.ci[CI_angle][c] : A.vi[VI_angle][c];
    double sn, cs;
    sincos(angle - M_PI / 2.0, &sn, &cs);
    in.lxlz = cs * sn;
    in.lx2 = cs * cs;
  }
  const double exx = nd.centroid ? A.ci[CI_exxd][c] : A.vi[VI_exxd][c];
  const double ezz = nd.centroid ? A.ci[CI_ezzd][c] : A.vi[VI_ezzd][c];
  const double exz = nd.centroid ? A.ci[CI_exz][c] : A.vi[VI_exz][c];
  effective_strain_rate(in.Exx, in.Ezz, in.Exz, exx, ezz, exz, in.Txx0, in.Tzz0, in.Txz0, w.d1, w.d2, w.aniS,
                        eta_e, M.elastic);
}

// The Newton operator's coefficients from the derivatives (StokesRoutines.c:285-312,
// :355-368); counts the node's perturbed solves.
__device__ __forceinline__ void newton_store(const OpArgs &A, const NewtonNode &w, const double dE[4],
                                             const double dV[4], const double dA[4], double drhodp,
                                             unsigned long long &calls, int &status) {
  const ModelConst &M = A.M;
  const OpNode &nd = w.nd;
  const NodeIn &in = nd.in;
  const long long c = nd.idx;
  const double eta_vep = nd.eta, ani_vep = w.ani_vep, aniS = w.aniS, d1 = w.d1, d2 = w.d2;
  const double e_a2 = eta_vep / (ani_vep * ani_vep);
  const double Gxz = 2.0 * in.Exz;
  for (int p = 0; p < M.np; p++) {
    const double vol = nd.centroid ? A.perc_n[p][c] : A.perc_s[p][c];
    if (fp64_abs_gt(vol, 1e-13)) calls += 8;
  }
  if (nd.centroid) {
    const double K = A.compressible ? 1.0 / in.beta : 0.0, Kdt = K * M.dt_model;
    const double Dxx = in.Exx * (1.0 - aniS * d1) + in.Ezz * aniS * d1 - Gxz * aniS * d2;
    const double Dzz = in.Ezz * (1.0 - aniS * d1) + in.Exx * aniS * d1 + Gxz * aniS * d2;
    const double Axx = -in.Exx * d1 * e_a2 + in.Ezz * d1 * e_a2 - Gxz * d2 * e_a2;
    const double Azz = in.Exx * d1 * e_a2 - in.Ezz * d1 * e_a2 + Gxz * d2 * e_a2;
    if (A.D[OP_DRHODP]) A.D[OP_DRHODP][c] = drhodp;
    A.D[OP_D11][c] = 2.0 * (1.0 - aniS * d1) * eta_vep + 2.0 * dE[0] * Dxx - Kdt * dV[0] + 2.0 * dA[0] * Axx;
    A.D[OP_D12][c] = 2.0 * aniS * d1 * eta_vep + 2.0 * dE[1] * Dxx - Kdt * dV[1] + 2.0 * dA[1] * Axx;
    A.D[OP_D13][c] = -2.0 * aniS * d2 * eta_vep + 2.0 * dE[2] * Dxx - Kdt * dV[2] + 2.0 * dA[2] * Axx;
    A.D[OP_D14][c] = 2.0 * dE[3] * Dxx - Kdt * dV[3] + 2.0 * dA[3] * Axx;
    A.D[OP_D21][c] = 2.0 * aniS * d1 * eta_vep + 2.0 * dE[0] * Dzz - Kdt * dV[0] + 2.0 * dA[0] * Azz;
    A.D[OP_D22][c] = 2.0 * (1.0 - aniS * d1) * eta_vep + 2.0 * dE[1] * Dzz - Kdt * dV[1] + 2.0 * dA[1] * Azz;
    A.D[OP_D23][c] = 2.0 * aniS * d2 * eta_vep + 2.0 * dE[2] * Dzz - Kdt * dV[2] + 2.0 * dA[2] * Azz;
    A.D[OP_D24][c] = 2.0 * dE[3] * Dzz - Kdt * dV[3] + 2.0 * dA[3] * Azz;
  } else {
    const double Dxz = -in.Exx * aniS * d2 + in.Ezz * aniS * d2 + Gxz * (aniS * (d1 - 0.5) + 0.5);
    const double Axz = -in.Exx * d2 * e_a2 + in.Ezz * d2 * e_a2 + Gxz * e_a2 * (d1 - 0.5);
    A.D[OP_D31][c] = -2.0 * aniS * d2 * eta_vep + 2.0 * dE[0] * Dxz + 2.0 * dA[0] * Axz;
    A.D[OP_D32][c] = 2.0 * aniS * d2 * eta_vep + 2.0 * dE[1] * Dxz + 2.0 * dA[1] * Axz;
    A.D[OP_D33][c] = (2.0 * aniS * (d1 - 0.5) + 1.0) * eta_vep + 2.0 * dE[2] * Dxz + 2.0 * dA[2] * Axz;
    const double d34 = 2.0 * dE[3] * Dxz + 2.0 * dA[3] * Axz;
    A.D[OP_D34][c] = d34;
    if (isnan(d34) || isinf(d34)) status = MDZ_ENONFINITE;  // :375-376
  }
}

__device__ __forceinline__ void op_report(const OpArgs &A, long long i, int &status) {
  if (status != MDZ_OK) {
    const unsigned long long key = ((unsigned long long)i << 8) | (unsigned long long)(-status & 0xff);
    atomicMin(&A.stats->err_key, key);
    status = MDZ_OK;
  }
}

__device__ __forceinline__ void op_flush_calls(const OpArgs &A, unsigned long long calls) {
  for (int o = 16; o > 0; o >>= 1) calls += __shfl_down_sync(0xffffffffu, calls, o);
  if ((threadIdx.x & 31) == 0 && calls) atomicAdd(&A.stats->calls, calls);
}

// One thread per node.  Registers capped for 4 CTAs of 128 per SM (3 for the anisotropic
// form): the extra resident warps hide more of the FP64 pipe's latency than the spills
// cost.  At 2049 x 2049 cells the Newton operator took 131.4 ms uncapped (232 registers,
// 2 CTAs per SM), 123.7 ms at 3 and 120.4 ms at 4 CTAs per SM; the anisotropic one 73.5,
// 65.3 and 66.6 ms.
template <bool ANISO, bool JAC>
__global__ void __launch_bounds__(128, ANISO ? 3 : 4) k_operators(const __grid_constant__ OpArgs A) {
  const long long total = A.M.Nc + A.M.Nv;
  unsigned long long calls = 0;
  int status = MDZ_OK;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    NewtonNode w;
    if (!op_node_load<ANISO>(A, i, w)) continue;
    if (!JAC) {
      picard_store(A, w);
      continue;
    }
    newton_inputs<ANISO>(A, w);
    double dE[4] = {0.0, 0.0, 0.0, 0.0}, dV[4] = {0.0, 0.0, 0.0, 0.0}, dA[4] = {0.0, 0.0, 0.0, 0.0};
    double drhodp = 0.0;
    fd_derivatives<ANISO, false>(A, w.nd, true, dE, dV, dA, drhodp);
    newton_store(A, w, dE, dV, dA, drhodp, calls, status);
    op_report(A, i, status);
  }
  op_flush_calls(A, calls);
}

// The isotropic Newton operator with its Drucker-Prager returns compacted per CTA: the
// node loop, the 8 perturbations and the phase loop are uniform over the CTA, and the
// returns of each phase's yielding items run packed into the first warps (dp_compact).
// The same bits as k_operators<false, true>.  5 CTAs per SM: 103.4 ms per 2049 x 2049
// launch against 104.9 ms at 4.
__global__ void __launch_bounds__(128, 5) k_operators_compact(const __grid_constant__ OpArgs A) {
  __shared__ CompactQueue Q;
  compact_init(Q);
  int par = 0;
  const long long total = A.M.Nc + A.M.Nv;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long calls = 0;
  int status = MDZ_OK;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < total; base += stride) {  // uniform
    const long long i = base + threadIdx.x;
    NewtonNode w;
    w.nd.centroid = true;
    w.nd.idx = 0;
    const bool has = i < total && op_node_load<false>(A, i, w);
    if (has) newton_inputs<false>(A, w);
    double dE[4] = {0.0, 0.0, 0.0, 0.0}, dV[4] = {0.0, 0.0, 0.0, 0.0}, dA[4] = {0.0, 0.0, 0.0, 0.0};
    double drhodp = 0.0;
    fd_derivatives<false, true>(A, w.nd, has, dE, dV, dA, drhodp, &Q, &par);
    if (has) {
      newton_store(A, w, dE, dV, dA, drhodp, calls, status);
      op_report(A, i, status);
    }
  }
  op_flush_calls(A, calls);
}

}  // namespace

cudaError_t launch_operators(const OpArgs &a, bool aniso, bool jacobian, bool compact, cudaStream_t s) {
  const long long total = a.M.Nc + a.M.Nv;
  const long long grid = (total + 127) / 128;
  if (grid < 1) return cudaSuccess;
  const unsigned g = (unsigned)(grid > 0x7fffffffLL ? 0x7fffffffLL : grid);
  if (!aniso && jacobian && compact) {
    k_operators_compact<<<g, 128, 0, s>>>(a);
  } else if (aniso) {
    if (jacobian) k_operators<true, true><<<g, 128, 0, s>>>(a);
    else k_operators<true, false><<<g, 128, 0, s>>>(a);
  } else {
    if (jacobian) k_operators<false, true><<<g, 128, 0, s>>>(a);
    else k_operators<false, false><<<g, 128, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace mdz
