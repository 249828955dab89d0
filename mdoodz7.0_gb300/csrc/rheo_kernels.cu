// rheo_kernels.cu -- sweep and point kernels of the local rheology update (sm_103a).
//
// k_sweep<ANISO> is NonNewtonianViscosityGrid (MDLIB/RheologyDensity.c:1131-1426) /
// NonNewtonianViscosityGridAniso (MDLIB/AnisotropyRoutines.c:885-1217) with the four
// InterpCentroidsToVerticesDouble calls (:1150-1153) fused into the vertex pass: one
// thread per node over the index space [centroids | vertices], per-phase tables in the
// kernel's constant parameter bank (uniform across a warp, so every lookup is a
// broadcast), SoA loads and stores coalesced along the node index.
#include <cuda_runtime.h>

#include "rheo_kernels.cuh"

namespace mdz {

__device__ __forceinline__ void record_error(DevStats *st, long long node, int status) {
  if (status == MDZ_OK) return;
  const unsigned long long key = ((unsigned long long)node << 8) | (unsigned long long)(-status & 0xff);
  atomicMin(&st->err_key, key);
}

struct Acc {
  unsigned long long calls, iters, plastic;
  unsigned int maxit;
};

// ---------------------------------------------------------------------------------
// one centroid (RheologyDensity.c:1156-1316 / AnisotropyRoutines.c:910-1087)
// ---------------------------------------------------------------------------------
template <bool ANISO>
__device__ __forceinline__ void do_centroid(const SweepArgs &A, long long c0, Acc &acc) {
  const ModelConst &M = A.M;
  const int np = M.np, avg = M.eta_average;
  double out[CO_COUNT];
#pragma unroll
  for (int i = 0; i < CO_COUNT; i++) out[i] = 0.0;
  const signed char bc = A.bcp[c0];
  if (bc != 30 && bc != 31) {
    NodeIn in;
    const double mu = A.ci[CI_mu][c0];
    const double eta_e = (M.elastic == 1) ? M.dt_model * mu : 1.0;
    const double inv_eta_e = ANISO ? 1.0 / eta_e : 0.0;
    const double el = (M.elastic == 1) ? 1.0 : 0.0;
    const double exxd = A.ci[CI_exxd][c0], ezzd = A.ci[CI_ezzd][c0], exz = A.ci[CI_exz][c0];
    in.Txx0 = A.ci[CI_sxxd0][c0]; in.Tzz0 = A.ci[CI_szzd0][c0]; in.Txz0 = A.ci[CI_sxz0][c0];
    double d1 = 0.0, d2 = 0.0, anif = 1.0;
    if (!ANISO) {
      const double h = el * 0.5 / eta_e;  // el / eta_e / 2
      in.Exx = exxd + in.Txx0 * h;
      in.Ezz = ezzd + in.Tzz0 * h;
      in.Exz = exz + in.Txz0 * h;
    } else {
      d1 = A.ci[CI_d1][c0]; d2 = A.ci[CI_d2][c0]; anif = A.ci[CI_anif][c0];
      double sn, cs;
      sincos(A.ci[CI_angle][c0] - M_PI / 2.0, &sn, &cs);
      in.lxlz = cs * sn; in.lx2 = cs * cs; in.ani_fac = anif;
      effective_strain_rate(in.Exx, in.Ezz, in.Exz, exxd, ezzd, exz, in.Txx0, in.Tzz0, in.Txz0, d1, d2,
                            1.0 - 1.0 / anif, eta_e, M.elastic);
    }
    in.G = mu; in.T = A.ci[CI_T][c0]; in.P = A.ci[CI_p_in][c0]; in.d = A.ci[CI_d0][c0];
    in.phi = A.ci[CI_phi0][c0]; in.X0 = A.ci[CI_X0][c0]; in.dil = A.ci[CI_dil][c0];
    in.fric = A.ci[CI_fric][c0]; in.C = A.ci[CI_C][c0]; in.P0 = A.ci[CI_p0][c0]; in.T0 = A.ci[CI_T0][c0];
    in.beta = A.ci[CI_bet][c0];
    in.centroid = 1; in.final_update = A.final_update; in.post_process = 1;
    in.want_rho = (M.density_variations == 1);
    NodeCtx ctx;
    AnisoNode an;
    if (ANISO) node_setup_aniso(M, in, A.need_lnd, ctx, an);
    else node_setup_iso(M, in, A.need_lnd, ctx);
    int status = MDZ_OK;
    for (int p = 0; p < np; p++) {
      const double perc = A.perc_n[p][c0];
      if (!(fabs(perc) > 1e-13)) {  // :1210-1212
        if (A.iters_n) A.iters_n[(long long)p * M.Nc + c0] = 0;
        continue;
      }
      PointOut o;
      if (ANISO) point_aniso(M, A.ph[p], in, ctx, an, 0.0, o);
      else point_iso(M, A.ph[p], in, ctx, 0.0, o);
      set_status(status, o.status);
      acc.calls++; acc.iters += o.iters; acc.plastic += o.is_pl;
      acc.maxit = max(acc.maxit, (unsigned)o.iters);
      if (A.iters_n) A.iters_n[(long long)p * M.Nc + c0] = o.iters;
      A.peta_n[p][c0] = o.etaVE;
      if (avg == 0) { out[CO_eta] += perc * o.etaVE; out[CO_eta_phys] += perc * o.eta; }
      else if (avg == 1) { out[CO_eta] += perc / o.etaVE; out[CO_eta_phys] += perc / o.eta; }
      else { out[CO_eta] += perc * log(o.etaVE); out[CO_eta_phys] += perc * log(o.eta); }
      if (ANISO) out[CO_VE] += perc * o.etaVE * inv_eta_e;
      out[CO_eII_el] += perc * o.Eii_el;
      out[CO_eII_pl] += perc * o.Eii_pl;
      out[CO_eII_pwl] += perc * o.Eii_pwl;
      out[CO_eII_exp] += perc * o.Eii_exp;
      out[CO_eII_lin] += perc * o.Eii_lin;
      out[CO_eII_gbs] += perc * o.Eii_gbs;
      out[CO_eII_cst] += perc * o.Eii_cst;
      out[CO_d] += perc * o.inv_d1;
      out[CO_Wtot] += perc * o.Wtot;
      out[CO_Wdiss] += perc * o.Wdiss;
      out[CO_Wel] += perc * o.Wel;
      out[CO_p_corr] += perc * o.Pcorr;
      out[CO_div_el] += perc * o.div_el;
      out[CO_div_pl] += perc * o.div_pl;
      out[CO_X] += perc * o.X1;
      out[CO_OverS] += perc * o.OverS;
      out[CO_rho] += perc * o.rho;
    }
    out[CO_d] = 1.0 / out[CO_d];
    if (!ANISO && (isinf(out[CO_d]) || isnan(out[CO_d]))) set_status(status, MDZ_EEMPTY_CELL);
    if (avg == 1) {
      out[CO_eta] = 1.0 / out[CO_eta];
      out[CO_eta_phys] = 1.0 / out[CO_eta_phys];
      if (isinf(out[CO_eta_phys]) || isnan(out[CO_eta_phys])) set_status(status, MDZ_ENONFINITE);
    } else if (avg == 2) {
      out[CO_eta] = exp(out[CO_eta]);
      out[CO_eta_phys] = exp(out[CO_eta_phys]);
    }
    const double eta2 = 2.0 * out[CO_eta];
    if (!ANISO) {
      out[CO_sxxd] = eta2 * in.Exx; out[CO_szzd] = eta2 * in.Ezz; out[CO_sxz] = eta2 * in.Exz;
    } else {  // AnisotropyRoutines.c:1079-1086
      const double a = 1.0 - 1.0 / anif;
      out[CO_sxxd] = eta2 * (in.Exx * (1.0 - a * d1) + in.Ezz * a * d1 - 2.0 * in.Exz * a * d2);
      out[CO_szzd] = eta2 * (in.Ezz * (1.0 - a * d1) + in.Exx * a * d1 + 2.0 * in.Exz * a * d2);
      out[CO_sxz] = eta2 * (-in.Exx * a * d2 + in.Ezz * a * d2 + 2 * in.Exz * (a * (d1 - 0.5) + 0.5));
    }
    record_error(A.stats, c0, status);
  } else if (A.iters_n) {
    for (int p = 0; p < np; p++) A.iters_n[(long long)p * M.Nc + c0] = 0;
  }
#pragma unroll
  for (int i = 0; i < CO_COUNT; i++)
    if (A.co[i]) A.co[i][c0] = out[i];
}

// ---------------------------------------------------------------------------------
// one vertex, with the fused centroid-to-vertex interpolation (GridRoutines.c:108-210)
// ---------------------------------------------------------------------------------
template <bool ANISO>
__device__ __forceinline__ void do_vertex(const SweepArgs &A, long long c1, Acc &acc) {
  const ModelConst &M = A.M;
  const int np = M.np, avg = M.eta_average, Nx = M.Nx;
  const int k = (int)(c1 % Nx), l = (int)(c1 / Nx);
  const signed char bcg = A.bcg[c1];
  double Ts = 0.0, Ps = 0.0, ds = 0.0, phis = 0.0;
  if (bcg != 30) {
    const int idx[4] = {ring_to_centroid(k, l, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k + 1, l, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k, l + 1, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k + 1, l + 1, M.Ncx, M.Ncz, M.periodic_x)};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const signed char f = A.bcp[idx[j]];
      const double w = (f == 30 || f == 31) ? 0.0 : 1.0;
      Ts += w * A.ci[CI_T][idx[j]];
      Ps += w * A.ci[CI_p_in][idx[j]];
      ds += w * A.ci[CI_d0][idx[j]];
      phis += w * A.ci[CI_phi0][idx[j]];
    }
    Ts *= 0.25; Ps *= 0.25; ds *= 0.25; phis *= 0.25;
  }
  A.vo[VO_T][c1] = Ts; A.vo[VO_P][c1] = Ps; A.vo[VO_d0][c1] = ds; A.vo[VO_phi0][c1] = phis;

  double eta = 0.0, eta_phys = 0.0, X = 0.0, VE = 0.0, sxx = 0.0, szz = 0.0, sxz = 0.0;
  if (bcg != 30) {
    NodeIn in;
    const double mu = A.vi[VI_mu][c1];
    const double eta_e = (M.elastic == 1) ? M.dt_model * mu : 1.0;
    const double inv_eta_e = ANISO ? 1.0 / eta_e : 0.0;
    const double el = (M.elastic == 1) ? 1.0 : 0.0;
    const double exxd = A.vi[VI_exxd][c1], ezzd = A.vi[VI_ezzd][c1], exz = A.vi[VI_exz][c1];
    in.Txx0 = A.vi[VI_sxxd0][c1]; in.Tzz0 = A.vi[VI_szzd0][c1]; in.Txz0 = A.vi[VI_sxz0][c1];
    double d1 = 0.0, d2 = 0.0, anif = 1.0;
    if (!ANISO) {
      const double h = el * 0.5 / eta_e;  // el / eta_e / 2
      in.Exx = exxd + in.Txx0 * h;
      in.Ezz = ezzd + in.Tzz0 * h;
      in.Exz = exz + in.Txz0 * h;
    } else {
      d1 = A.vi[VI_d1][c1]; d2 = A.vi[VI_d2][c1]; anif = A.vi[VI_anif][c1];
      double sn, cs;
      sincos(A.vi[VI_angle][c1] - M_PI / 2.0, &sn, &cs);
      in.lxlz = cs * sn; in.lx2 = cs * cs; in.ani_fac = anif;
      effective_strain_rate(in.Exx, in.Ezz, in.Exz, exxd, ezzd, exz, in.Txx0, in.Tzz0, in.Txz0, d1, d2,
                            1.0 - 1.0 / anif, eta_e, M.elastic);
    }
    in.G = mu; in.T = Ts; in.P = Ps; in.d = ds; in.phi = phis; in.X0 = A.vi[VI_X0][c1];
    in.dil = A.vi[VI_dil][c1]; in.fric = A.vi[VI_fric][c1]; in.C = A.vi[VI_C][c1]; in.P0 = A.vi[VI_p0][c1];
    in.T0 = 0.0; in.beta = A.vi[VI_bet][c1];
    in.centroid = 0; in.final_update = A.final_update; in.post_process = 1; in.want_rho = 0;
    NodeCtx ctx;
    AnisoNode an;
    if (ANISO) node_setup_aniso(M, in, A.need_lnd, ctx, an);
    else node_setup_iso(M, in, A.need_lnd, ctx);
    int status = MDZ_OK;
    for (int p = 0; p < np; p++) {
      const double perc = A.perc_s[p][c1];
      if (!(fabs(perc) > 1e-13)) {
        if (A.iters_s) A.iters_s[(long long)p * M.Nv + c1] = 0;
        continue;
      }
      PointOut o;
      if (ANISO) point_aniso(M, A.ph[p], in, ctx, an, 0.0, o);
      else point_iso(M, A.ph[p], in, ctx, 0.0, o);
      set_status(status, o.status);
      acc.calls++; acc.iters += o.iters; acc.plastic += o.is_pl;
      acc.maxit = max(acc.maxit, (unsigned)o.iters);
      if (A.iters_s) A.iters_s[(long long)p * M.Nv + c1] = o.iters;
      A.peta_s[p][c1] = o.etaVE;
      if (avg == 0) { eta += perc * o.etaVE; eta_phys += perc * o.eta; }
      else if (avg == 1) { eta += perc / o.etaVE; eta_phys += perc / o.eta; }
      else { eta += perc * log(o.etaVE); eta_phys += perc * log(o.eta); }
      if (ANISO) VE += perc * o.etaVE * inv_eta_e;
      X += perc * o.X1;
    }
    if (avg == 1) {
      eta = 1.0 / eta; eta_phys = 1.0 / eta_phys;
      if (isinf(eta_phys) || isnan(eta_phys)) set_status(status, MDZ_ENONFINITE);
    } else if (avg == 2) {
      eta = exp(eta); eta_phys = exp(eta_phys);
    }
    const double eta2 = 2.0 * eta;
    if (!ANISO) {
      sxx = eta2 * in.Exx; szz = eta2 * in.Ezz; sxz = eta2 * in.Exz;
    } else {
      const double a = 1.0 - 1.0 / anif;
      sxx = eta2 * (in.Exx * (1.0 - a * d1) + in.Ezz * a * d1 - 2.0 * in.Exz * a * d2);
      szz = eta2 * (in.Ezz * (1.0 - a * d1) + in.Exx * a * d1 + 2.0 * in.Exz * a * d2);
      sxz = eta2 * (-in.Exx * a * d2 + in.Ezz * a * d2 + 2 * in.Exz * (a * (d1 - 0.5) + 0.5));
    }
    record_error(A.stats, M.Nc + c1, status);
  } else if (A.iters_s) {
    for (int p = 0; p < np; p++) A.iters_s[(long long)p * M.Nv + c1] = 0;
  }
  A.vo[VO_sxxd][c1] = sxx; A.vo[VO_szzd][c1] = szz; A.vo[VO_sxz][c1] = sxz;
  A.vo[VO_eta_phys][c1] = eta_phys; A.vo[VO_eta][c1] = eta; A.vo[VO_X][c1] = X;
  if (A.vo[VO_VE]) A.vo[VO_VE][c1] = VE;
}

__device__ __forceinline__ void flush_acc(DevStats *st, Acc &acc) {
  // warp-aggregate, then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    acc.calls += __shfl_down_sync(0xffffffffu, acc.calls, o);
    acc.iters += __shfl_down_sync(0xffffffffu, acc.iters, o);
    acc.plastic += __shfl_down_sync(0xffffffffu, acc.plastic, o);
    acc.maxit = max(acc.maxit, __shfl_down_sync(0xffffffffu, acc.maxit, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&st->calls, acc.calls);
    atomicAdd(&st->iters, acc.iters);
    atomicAdd(&st->plastic, acc.plastic);
    atomicMax(&st->maxit, acc.maxit);
  }
}

template <bool ANISO>
__global__ void __launch_bounds__(128) k_sweep(const __grid_constant__ SweepArgs A) {
  Acc acc = {0, 0, 0, 0};
  const long long total = A.M.Nc + A.M.Nv;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    if (i < A.M.Nc) do_centroid<ANISO>(A, i, acc);
    else do_vertex<ANISO>(A, i - A.M.Nc, acc);
  }
  flush_acc(A.stats, acc);
}

// ---------------------------------------------------------------------------------
// independent points: ViscosityConcise / ViscosityConciseAniso
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_points(const __grid_constant__ PointArgs A) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Acc acc = {0, 0, 0, 0};
  if (i < A.n) {
    const mdz_point_inputs &I = A.in;
    NodeIn in;
    in.Exx = I.Exx[i]; in.Ezz = I.Ezz[i]; in.Exz = I.Exz[i];
    in.Txx0 = I.Txx0[i]; in.Tzz0 = I.Tzz0[i]; in.Txz0 = I.Txz0[i];
    in.G = I.G[i]; in.T = I.T[i]; in.P = I.P[i]; in.d = I.d[i]; in.phi = I.phi[i]; in.X0 = I.X0[i];
    in.dil = I.dil[i]; in.fric = I.fric[i]; in.C = I.C[i]; in.P0 = I.P0[i]; in.T0 = I.T0[i]; in.beta = I.beta[i];
    in.centroid = I.centroid; in.final_update = I.final_update; in.post_process = I.post_process;
    in.want_rho = 1;
    const int p = I.phase[i];
    PointOut o;
    NodeCtx ctx;
    if (A.aniso) {
      in.lxlz = I.lxlz[i]; in.lx2 = I.lx2[i]; in.ani_fac = I.ani_fac[i];
      AnisoNode an;
      node_setup_aniso(A.M, in, true, ctx, an);
      point_aniso(A.M, A.ph[p], in, ctx, an, 0.0, o);
    } else {
      node_setup_iso(A.M, in, true, ctx);
      point_iso(A.M, A.ph[p], in, ctx, 0.0, o);
    }
    const mdz_point_outputs &O = A.out;
    double *dst[24] = {O.eta, O.Txx, O.Tzz, O.Txz, O.etaVE, O.VEcoeff, O.Eii_el, O.Eii_pl, O.Eii_pwl, O.Eii_exp,
                       O.Eii_lin, O.Eii_gbs, O.Eii_cst, O.d1, O.X1, O.OverS, O.Pcorr, O.rho, O.div_el, O.div_pl,
                       O.div_r, O.Wtot, O.Wel, O.Wdiss};
    const double src[24] = {o.eta, o.Txx, o.Tzz, o.Txz, o.etaVE, 0.0, o.Eii_el, o.Eii_pl, o.Eii_pwl, o.Eii_exp,
                            o.Eii_lin, o.Eii_gbs, o.Eii_cst, o.d1, o.X1, o.OverS, o.Pcorr, o.rho, o.div_el,
                            o.div_pl, 0.0, o.Wtot, o.Wel, o.Wdiss};
#pragma unroll
    for (int j = 0; j < 24; j++)
      if (dst[j]) dst[j][i] = src[j];
    if (O.iters) O.iters[i] = o.iters;
    if (O.status) O.status[i] = o.status;
    record_error(A.stats, i, o.status);
    acc.calls = 1; acc.iters = o.iters; acc.plastic = o.is_pl; acc.maxit = o.iters;
  }
  flush_acc(A.stats, acc);
}

cudaError_t launch_sweep(const SweepArgs &a, bool aniso, cudaStream_t s, int block, int grid_cap) {
  const long long total = a.M.Nc + a.M.Nv;
  long long grid = (total + block - 1) / block;
  if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
  if (grid < 1) grid = 1;
  if (aniso) k_sweep<true><<<(unsigned)grid, block, 0, s>>>(a);
  else k_sweep<false><<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_points(const PointArgs &a, cudaStream_t s) {
  const int block = 128;
  const long long grid = (a.n + block - 1) / block;
  if (grid > 0) k_points<<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

void sweep_kernel_info(int aniso, int *regs, int *smem, int *max_blocks_per_sm, int block) {
  cudaFuncAttributes fa;
  const void *fn = aniso ? (const void *)k_sweep<true> : (const void *)k_sweep<false>;
  cudaFuncGetAttributes(&fa, fn);
  *regs = fa.numRegs;
  *smem = (int)fa.sharedSizeBytes;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(max_blocks_per_sm, fn, block, 0);
}

}  // namespace mdz
