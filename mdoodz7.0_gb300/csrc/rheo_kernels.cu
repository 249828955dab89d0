// rheo_kernels.cu -- sweep and point kernels of the local rheology update (sm_103a).
//
// k_sweep<ANISO, NODES> is NonNewtonianViscosityGrid (MDLIB/RheologyDensity.c:1131-1426) /
// NonNewtonianViscosityGridAniso (MDLIB/AnisotropyRoutines.c:885-1217) with the four
// InterpCentroidsToVerticesDouble calls (:1150-1153) fused into the vertex pass: one
// thread per node over the index space [centroids | vertices], launched once over the
// centroids (NODES 1) and once over the vertices (NODES 2) so that each kernel carries only
// its own kind's work (vertices skip the per-phase outputs only centroids keep), per-phase
// tables in the kernel's constant parameter bank (uniform across a warp, so every lookup
// is a broadcast), SoA loads and stores coalesced along the node index.  k_sweep_queue is
// the same sweep as a persistent grid on a work counter; k_sweep_warm puts the learned
// warm start (evaluated per warp on the tensor cores) before each local solve;
// k_sweep_batch sweeps many grids in one launch per kind of node.
//
// k_sweep_tiles<ANISO, MODE, NODES> walks the same index space in tiles of 128 nodes, one tile
// per CTA at a time, with the phase loop uniform over the CTA so that a block-wide stage
// can sit between each phase's set-up and its local solve: the learned warm start
// (MODE_WARM: the tcgen05 network's guess, then the start stages) or the training-data dump
// (MODE_COLLECT, from the reference's own start).
#include <cuda_runtime.h>

#include "mlp.cuh"
#include "mlp_warp.cuh"
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
  unsigned long long f32;  // FP32 Newton steps of the starts
};

// Multiplicative perturbation of the strain-rate inputs of every grid of a batch:
// x <- x (1 + amp u), u uniform in [-1, 1) from a counter hash (SplitMix64, Steele et
// al. 2014) of (seed, sweep, grid, node, component).  Rounded steps without
// contraction, so a host restatement reproduces the values exactly.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// u = m 2^-52 - 1 for the top 53 bits m of the hash, in [-1, 1).  Every such value is a
// double, so u is formed exactly without an integer-to-double conversion (an FP64-pipe
// instruction on this GPU): the low 52 bits of m as the fraction of a number in [1, 2),
// minus 1 where m >= 2^52 and minus 2 below (both subtractions exact).
__device__ __forceinline__ double perturb_factor(unsigned long long key, long long node, int comp, double amp) {
  const unsigned long long m = splitmix64(key ^ (unsigned long long)(node * 3 + comp)) >> 11;
  const double f = __longlong_as_double((long long)(0x3ff0000000000000ull | (m & 0xfffffffffffffull)));
  const double u = __dsub_rn(f, (m >> 52) ? 1.0 : 2.0);  // [-1, 1)
  return __dadd_rn(1.0, __dmul_rn(amp, u));
}

// The perturbation of one grid in one sweep, fused into the sweep's load of the strain
// rates: key = the hash of (seed, sweep, grid), amp > 0.
struct PerturbKey {
  unsigned long long key;
  double amp;
};

__device__ __forceinline__ unsigned long long perturb_key(unsigned long long seed, int sweep, int grid) {
  return splitmix64(splitmix64(seed ^ (unsigned long long)sweep) ^ (unsigned long long)grid);
}

// The node's three strain-rate inputs x[0..2] (exxd, ezzd, exz of a centroid or of a
// vertex, node index i over [centroids | vertices]) multiplied by their factors and stored
// back, so the next captured sweep starts from the perturbed rates.
__device__ __forceinline__ void perturb_inputs(const PerturbKey &pk, long long i, double *const *x) {
#pragma unroll
  for (int k = 0; k < 3; k++) *x[k] = __dmul_rn(*x[k], perturb_factor(pk.key, i, k, pk.amp));
}

// ---------------------------------------------------------------------------------
// one node: load and prepare (RheologyDensity.c:1165-1204, :1324-1340;
// AnisotropyRoutines.c:917-977, :1097-1131)
// ---------------------------------------------------------------------------------
struct Node {
  long long idx;  // centroid c0, or vertex c1
  bool centroid, solid;
  double eta_e, inv_eta_e, d1, d2, anif;
  double interp[4];  // vertex T_s, P_s, d0_s, phi0_s
  NodeIn in;
  NodeCtx ctx;
  AnisoNode an;
};

// NODES: 0 either kind (index i decides), 1 centroids only, 2 vertices only; a kernel
// specialised to one kind of node drops the other kind's code and registers
// pk (may be null): the strain rates are perturbed first, at every node, air included.
template <bool ANISO, int NODES = 0>
__device__ __forceinline__ void node_prepare(const SweepArgs &A, long long i, Node &n,
                                             const PerturbKey *pk = nullptr) {
  const ModelConst &M = A.M;
  n.centroid = NODES == 1 ? true : (NODES == 2 ? false : i < M.Nc);
  const double el = (M.elastic == 1) ? 1.0 : 0.0;
  double mu, exxd, ezzd, exz;
  if (pk) {
    double *x[3];
    if (n.centroid) {
      x[0] = const_cast<double *>(A.ci[CI_exxd]) + i;
      x[1] = const_cast<double *>(A.ci[CI_ezzd]) + i;
      x[2] = const_cast<double *>(A.ci[CI_exz]) + i;
    } else {
      x[0] = const_cast<double *>(A.vi[VI_exxd]) + (i - M.Nc);
      x[1] = const_cast<double *>(A.vi[VI_ezzd]) + (i - M.Nc);
      x[2] = const_cast<double *>(A.vi[VI_exz]) + (i - M.Nc);
    }
    perturb_inputs(*pk, i, x);
  }
  if (n.centroid) {
    const long long c0 = i;
    n.idx = c0;
    const signed char bc = A.bcp[c0];
    n.solid = (bc != 30 && bc != 31);
    if (!n.solid) return;
    mu = A.ci[CI_mu][c0];
    exxd = A.ci[CI_exxd][c0]; ezzd = A.ci[CI_ezzd][c0]; exz = A.ci[CI_exz][c0];
    n.in.Txx0 = A.ci[CI_sxxd0][c0]; n.in.Tzz0 = A.ci[CI_szzd0][c0]; n.in.Txz0 = A.ci[CI_sxz0][c0];
    n.in.T = A.ci[CI_T][c0]; n.in.P = A.ci[CI_p_in][c0]; n.in.d = A.ci[CI_d0][c0];
    n.in.phi = A.ci[CI_phi0][c0]; n.in.X0 = A.ci[CI_X0][c0]; n.in.dil = A.ci[CI_dil][c0];
    n.in.fric = A.ci[CI_fric][c0]; n.in.C = A.ci[CI_C][c0]; n.in.P0 = A.ci[CI_p0][c0]; n.in.T0 = A.ci[CI_T0][c0];
    n.in.beta = A.ci[CI_bet][c0];
    if (ANISO) { n.d1 = A.ci[CI_d1][c0]; n.d2 = A.ci[CI_d2][c0]; n.anif = A.ci[CI_anif][c0]; }
  } else {
    const long long c1 = i - M.Nc;
    n.idx = c1;
    const int Nx = M.Nx, k = (int)(c1 % Nx), l = (int)(c1 / Nx);
    const signed char bcg = A.bcg[c1];
    n.solid = (bcg != 30);
    n.interp[0] = n.interp[1] = n.interp[2] = n.interp[3] = 0.0;
    if (!n.solid) return;
    const int idx[4] = {ring_to_centroid(k, l, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k + 1, l, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k, l + 1, M.Ncx, M.Ncz, M.periodic_x),
                        ring_to_centroid(k + 1, l + 1, M.Ncx, M.Ncz, M.periodic_x)};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const signed char f = A.bcp[idx[j]];
      const double w = (f == 30 || f == 31) ? 0.0 : 1.0;
      n.interp[0] += w * A.ci[CI_T][idx[j]];
      n.interp[1] += w * A.ci[CI_p_in][idx[j]];
      n.interp[2] += w * A.ci[CI_d0][idx[j]];
      n.interp[3] += w * A.ci[CI_phi0][idx[j]];
    }
#pragma unroll
    for (int j = 0; j < 4; j++) n.interp[j] *= 0.25;
    mu = A.vi[VI_mu][c1];
    exxd = A.vi[VI_exxd][c1]; ezzd = A.vi[VI_ezzd][c1]; exz = A.vi[VI_exz][c1];
    n.in.Txx0 = A.vi[VI_sxxd0][c1]; n.in.Tzz0 = A.vi[VI_szzd0][c1]; n.in.Txz0 = A.vi[VI_sxz0][c1];
    n.in.T = n.interp[0]; n.in.P = n.interp[1]; n.in.d = n.interp[2]; n.in.phi = n.interp[3];
    n.in.X0 = A.vi[VI_X0][c1]; n.in.dil = A.vi[VI_dil][c1]; n.in.fric = A.vi[VI_fric][c1];
    n.in.C = A.vi[VI_C][c1]; n.in.P0 = A.vi[VI_p0][c1]; n.in.T0 = 0.0; n.in.beta = A.vi[VI_bet][c1];
    if (ANISO) { n.d1 = A.vi[VI_d1][c1]; n.d2 = A.vi[VI_d2][c1]; n.anif = A.vi[VI_anif][c1]; }
  }
  n.in.G = mu;
  n.eta_e = (M.elastic == 1) ? M.dt_model * mu : 1.0;
  n.inv_eta_e = ANISO ? 1.0 / n.eta_e : 0.0;
  if (!ANISO) {
    const double h = el * 0.5 / n.eta_e;  // el / eta_e / 2
    n.in.Exx = exxd + n.in.Txx0 * h;
    n.in.Ezz = ezzd + n.in.Tzz0 * h;
    n.in.Exz = exz + n.in.Txz0 * h;
  } else {
    const double angle = n.centroid ? A.ci[CI_angle][n.idx] : A.vi[VI_angle][n.idx];
    double sn, cs;
    sincos(angle - M_PI / 2.0, &sn, &cs);
    n.in.lxlz = cs * sn; n.in.lx2 = cs * cs; n.in.ani_fac = n.anif;
    effective_strain_rate(n.in.Exx, n.in.Ezz, n.in.Exz, exxd, ezzd, exz, n.in.Txx0, n.in.Tzz0, n.in.Txz0, n.d1,
                          n.d2, 1.0 - 1.0 / n.anif, n.eta_e, M.elastic);
  }
  n.in.centroid = n.centroid ? 1 : 0;
  n.in.final_update = A.final_update;
  n.in.post_process = n.centroid ? 1 : 2;  // a vertex keeps only etaVE, eta_phys and X
  n.in.want_rho = n.centroid && (M.density_variations == 1);
  if (ANISO) node_setup_aniso(M, n.in, A.need_lnd, n.ctx, n.an);
  else node_setup_iso(M, n.in, A.need_lnd, n.ctx);
}

__device__ __forceinline__ double node_perc(const SweepArgs &A, const Node &n, int p) {
  return n.centroid ? A.perc_n[p][n.idx] : A.perc_s[p][n.idx];
}

__device__ __forceinline__ void node_iters(const SweepArgs &A, const Node &n, int p, int it) {
  if (n.centroid) { if (A.iters_n) A.iters_n[(long long)p * A.M.Nc + n.idx] = it; }
  else if (A.iters_s) A.iters_s[(long long)p * A.M.Nv + n.idx] = it;
}

// accumulate one phase's result (RheologyDensity.c:1217-1270, :1359-1378)
template <bool ANISO>
__device__ __forceinline__ void node_accumulate(const SweepArgs &A, const Node &n, int p, double perc,
                                                const PointOut &o, double *out, Acc &acc, int &status) {
  set_status(status, o.status);
  acc.calls++; acc.iters += o.iters; acc.plastic += o.is_pl; acc.f32 += o.f32_steps;
  acc.maxit = max(acc.maxit, (unsigned)o.iters);
  node_iters(A, n, p, MDZ_ITEM_WORD(o.iters, o.mech));
  if (n.centroid) A.peta_n[p][n.idx] = o.etaVE;
  else A.peta_s[p][n.idx] = o.etaVE;
  const int avg = A.M.eta_average;
  if (avg == 0) { out[CO_eta] += perc * o.etaVE; out[CO_eta_phys] += perc * o.eta; }
  else if (avg == 1) { out[CO_eta] += perc / o.etaVE; out[CO_eta_phys] += perc / o.eta; }
  else { out[CO_eta] += perc * log(o.etaVE); out[CO_eta_phys] += perc * log(o.eta); }
  if (ANISO) out[CO_VE] += perc * o.etaVE * n.inv_eta_e;
  out[CO_X] += perc * o.X1;
  if (!n.centroid) return;
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
  out[CO_OverS] += perc * o.OverS;
  out[CO_rho] += perc * o.rho;
}

// finalize the averages and the stress, then store (:1274-1313, :1380-1405)
template <bool ANISO>
__device__ __forceinline__ void node_store(const SweepArgs &A, const Node &n, double *out, int status) {
  const ModelConst &M = A.M;
  const int avg = M.eta_average;
  if (n.solid) {
    if (n.centroid) {
      out[CO_d] = 1.0 / out[CO_d];
      if (!ANISO && !fp64_finite(out[CO_d])) set_status(status, MDZ_EEMPTY_CELL);
    }
    if (avg == 1) {
      out[CO_eta] = 1.0 / out[CO_eta];
      out[CO_eta_phys] = 1.0 / out[CO_eta_phys];
      if (!fp64_finite(out[CO_eta_phys])) set_status(status, MDZ_ENONFINITE);
    } else if (avg == 2) {
      out[CO_eta] = exp(out[CO_eta]);
      out[CO_eta_phys] = exp(out[CO_eta_phys]);
    }
    const double eta2 = 2.0 * out[CO_eta];
    const NodeIn &in = n.in;
    if (!ANISO) {
      out[CO_sxxd] = eta2 * in.Exx; out[CO_szzd] = eta2 * in.Ezz; out[CO_sxz] = eta2 * in.Exz;
    } else {  // AnisotropyRoutines.c:1079-1086
      const double a = 1.0 - 1.0 / n.anif, d1 = n.d1, d2 = n.d2;
      out[CO_sxxd] = eta2 * (in.Exx * (1.0 - a * d1) + in.Ezz * a * d1 - 2.0 * in.Exz * a * d2);
      out[CO_szzd] = eta2 * (in.Ezz * (1.0 - a * d1) + in.Exx * a * d1 + 2.0 * in.Exz * a * d2);
      out[CO_sxz] = eta2 * (-in.Exx * a * d2 + in.Ezz * a * d2 + 2 * in.Exz * (a * (d1 - 0.5) + 0.5));
    }
    record_error(A.stats, A.node_base + (n.centroid ? n.idx : M.Nc + n.idx), status);
  } else {
    for (int p = 0; p < M.np; p++) node_iters(A, n, p, 0);
  }
  if (n.centroid) {
#pragma unroll
    for (int i = 0; i < CO_COUNT; i++)
      if (A.co[i]) A.co[i][n.idx] = out[i];
  } else {
    const long long c1 = n.idx;
    A.vo[VO_T][c1] = n.interp[0]; A.vo[VO_P][c1] = n.interp[1];
    A.vo[VO_d0][c1] = n.interp[2]; A.vo[VO_phi0][c1] = n.interp[3];
    A.vo[VO_sxxd][c1] = out[CO_sxxd]; A.vo[VO_szzd][c1] = out[CO_szzd]; A.vo[VO_sxz][c1] = out[CO_sxz];
    A.vo[VO_eta_phys][c1] = out[CO_eta_phys]; A.vo[VO_eta][c1] = out[CO_eta]; A.vo[VO_X][c1] = out[CO_X];
    if (A.vo[VO_VE]) A.vo[VO_VE][c1] = out[CO_VE];
  }
}

__device__ __forceinline__ void flush_acc(DevStats *st, Acc &acc) {
  // warp-aggregate, then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    acc.calls += __shfl_down_sync(0xffffffffu, acc.calls, o);
    acc.iters += __shfl_down_sync(0xffffffffu, acc.iters, o);
    acc.plastic += __shfl_down_sync(0xffffffffu, acc.plastic, o);
    acc.maxit = max(acc.maxit, __shfl_down_sync(0xffffffffu, acc.maxit, o));
    acc.f32 += __shfl_down_sync(0xffffffffu, acc.f32, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&st->calls, acc.calls);
    atomicAdd(&st->iters, acc.iters);
    atomicAdd(&st->plastic, acc.plastic);
    atomicMax(&st->maxit, acc.maxit);
    if (acc.f32) atomicAdd(&st->f32_steps, acc.f32);
  }
}

// ---------------------------------------------------------------------------------
// plain sweep: one thread per node
// ---------------------------------------------------------------------------------
// One node of one grid: prepare, every active phase's local solve, averaging, store.
template <bool ANISO, int NODES = 0>
__device__ __forceinline__ void sweep_node(const SweepArgs &A, long long i, Acc &acc,
                                           const PerturbKey *pk = nullptr) {
  Node n;
  node_prepare<ANISO, NODES>(A, i, n, pk);
  double out[CO_COUNT];
#pragma unroll
  for (int j = 0; j < CO_COUNT; j++) out[j] = 0.0;
  int status = MDZ_OK;
  if (n.solid) {
    for (int p = 0; p < A.M.np; p++) {
      const double perc = node_perc(A, n, p);
      if (!fp64_abs_gt(perc, 1e-13)) {  // :1210-1212
        node_iters(A, n, p, 0);
        continue;
      }
      PointOut o;
      if (ANISO) point_aniso(A.M, A.ph[p], n.in, n.ctx, n.an, A.polish, o);
      else point_iso(A.M, A.ph[p], n.in, n.ctx, A.polish, o);
      node_accumulate<ANISO>(A, n, p, perc, o, out, acc, status);
    }
  }
  node_store<ANISO>(A, n, out, status);
}

// One sweep is two launches: the centroids (NODES 1), then the vertices (NODES 2), each
// over its whole range or over the band of rows a banded sweep gives it.
// Four CTAs of 128 per SM (128 registers, with spills: about 0.7 kB per vertex thread and
// 0.9 kB per centroid thread, which stay in L1 and L2).  Sixteen warps per SM hide more of
// the FP64 pipe's latency than the spills cost: at 2049 x 2049 cells the default-start
// sweep takes 19.1 ms against 19.5 ms at three CTAs per SM (168 registers) and 20.6 ms at
// two (255 registers, no spills); five CTAs gain another 0.4 % there but lose 1.6 % on the
// many-grid batch.
// MINB: CTAs of 128 per SM the register allocation is capped for (4: 128 registers; 2: 255
// registers, which wins where local solves take many Newton evaluations); the autotuner
// times both.
template <bool ANISO, int NODES, int MINB = 4>
__global__ void __launch_bounds__(128, MINB) k_sweep(const __grid_constant__ SweepArgs A) {
  Acc acc = {0, 0, 0, 0, 0};
  const long long total = NODES == 1 ? (A.ranged ? A.c_n : A.M.Nc) : (A.ranged ? A.v_n : A.M.Nv);
  const long long lo = NODES == 1 ? (A.ranged ? A.c_lo : 0) : A.M.Nc + (A.ranged ? A.v_lo : 0);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += stride)
    sweep_node<ANISO, NODES>(A, lo + j, acc);
  flush_acc(A.stats, acc);
}

// Persistent form: a grid of resident CTAs whose warps pull chunks of 32 consecutive
// nodes from a work counter until none is left.  A warp takes its next chunk as soon as
// its slowest lane is done, instead of a CTA waiting for all four of its warps and the
// block scheduler refilling the SM; one lane fetches for the warp (one atomic per chunk),
// the chunk start is broadcast by shuffle, and the lanes past the end are retired by a
// ballot.  The node body is the plain sweep's, so the results are the same bits.
template <bool ANISO, int NODES>
__global__ void __launch_bounds__(128, 4) k_sweep_queue(const __grid_constant__ SweepArgs A) {
  Acc acc = {0, 0, 0, 0, 0};
  const long long total = NODES == 1 ? A.M.Nc : A.M.Nv;
  const long long lo = NODES == 1 ? 0 : A.M.Nc;
  unsigned long long *counter = &A.stats->queue[NODES - 1];
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    const long long j = (long long)base + lane;
    const unsigned live = __ballot_sync(0xffffffffu, j < total);
    if (live == 0u) break;
    if ((live >> lane) & 1u) sweep_node<ANISO, NODES>(A, lo + j, acc);
  }
  flush_acc(A.stats, acc);
}

// Compacting form of the isotropic sweep: the CTA's 128 threads walk their nodes' phases
// in step (the node and phase loops are uniform over the CTA), and the Drucker-Prager
// returns of each phase's yielding items run packed into the first warps (dp_compact).
// Same functions, so the same bits as k_sweep.

// The warm-start declarations (used below with WARM)
__device__ __forceinline__ void warm_inputs(const MlpDevice &W, const float *f, int nfeat, float *x);

// One isotropic node per thread; every thread of the CTA calls it together (valid false: a
// thread without a node, which still takes part in the CTA's barriers and, WARM, in its
// warp's network).  WARM: the learned start, evaluated per warp, before each local solve.
template <int NODES, bool WARM>
__device__ __forceinline__ void compact_node(const SweepArgs &A, bool valid, long long i, Acc &acc,
                                             CompactQueue &Q, int &par, MlpWarpShared *S = nullptr,
                                             const MlpDevice *W = nullptr, const PerturbKey *pk = nullptr) {
  Node n;
  n.solid = false;
  n.centroid = NODES == 1;
  if (valid) node_prepare<false, NODES>(A, i, n, pk);
  double out[CO_COUNT];
#pragma unroll
  for (int k = 0; k < CO_COUNT; k++) out[k] = 0.0;
  int status = MDZ_OK;
  const int polish = WARM ? W->polish_iters : A.polish;
  for (int p = 0; p < A.M.np; p++) {  // uniform over the CTA
    const double perc = (valid && n.solid) ? node_perc(A, n, p) : 0.0;
    const bool active = fp64_abs_gt(perc, 1e-13);  // :1210-1212
    if (valid && n.solid && !active) node_iters(A, n, p, 0);
    IsoState st;
    PointOut o;
    IsoMid m;
    float s_start = 1.0f;
    if (WARM) {
      float f[kMlpIn], x[kMlpIn];
#pragma unroll
      for (int k = 0; k < kMlpIn; k++) f[k] = 0.0f;
      if (active) {
        iso_setup(A.M, A.ph[p], n.in, n.ctx, st, o, polish == 0);
        warm_features(A.M, n.in, n.ctx, st, false, f);
      }
      warm_inputs(*W, f, kFeatIso, x);
      __syncwarp();
      const float y = mlp_warp_predict(*S, x);
      s_start = warm_start_point(y, W->z_scale, W->z_shift);
    } else if (active) {
      iso_setup(A.M, A.ph[p], n.in, n.ctx, st, o, polish == 0);
    }
    bool yields = false;
    if (active) {
      iso_ve(A.M, A.ph[p], n.in, n.ctx, st, s_start, polish, o, m);
      yields = iso_yields_dp(A.M, A.ph[p], n.ctx, m);
    }
    dp_compact(A.M, A.ph[p], Q, par, yields, m, n.in, n.ctx);
    if (active) {
      iso_post(A.M, A.ph[p], n.in, n.ctx, st, o, m);
      node_accumulate<false>(A, n, p, perc, o, out, acc, status);
    }
  }
  if (valid) node_store<false>(A, n, out, status);
}

// 4 CTAs of 128 per SM (128 registers).  At 5 (96 registers) the sweep gained 0.3 % (17.15
// against 17.20 ms at 2049 x 2049 cells) while its spills' DRAM write-backs nearly doubled
// (751 against 415 B per node at 1025 x 1025).
template <int NODES>
__global__ void __launch_bounds__(128, 4) k_sweep_compact(const __grid_constant__ SweepArgs A) {
  __shared__ CompactQueue Q;
  compact_init(Q);
  Acc acc = {0, 0, 0, 0, 0};
  const long long total = NODES == 1 ? (A.ranged ? A.c_n : A.M.Nc) : (A.ranged ? A.v_n : A.M.Nv);
  const long long lo = NODES == 1 ? (A.ranged ? A.c_lo : 0) : A.M.Nc + (A.ranged ? A.v_lo : 0);
  const long long stride = (long long)gridDim.x * blockDim.x;
  int par = 0;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < total; base += stride) {  // uniform
    const long long j = base + threadIdx.x;
    compact_node<NODES, false>(A, j < total, lo + j, acc, Q, par);
  }
  flush_acc(A.stats, acc);
}

// ---------------------------------------------------------------------------------
// learned warm start, per warp: the plain sweep with the network between each phase's
// set-up and its local solve, evaluated by the warp's 32 lanes on the tensor cores
// (mlp_warp.cuh)
// ---------------------------------------------------------------------------------
// The network's normalised inputs for one (node, phase) (zeros where the lane has none).
__device__ __forceinline__ void warm_inputs(const MlpDevice &W, const float *f, int nfeat, float *x) {
#pragma unroll
  for (int j = 0; j < kMlpIn; j++) x[j] = (j < nfeat) ? (f[j] - W.x_shift[j]) * W.x_scale[j] : 0.0f;
}

// One node per lane, the warp's 32 nodes consecutive, so every lane of a warp runs the
// same number of node iterations and reaches the network at the same phase; lanes past
// the end or at inactive (node, phase) items feed zeros and discard the output.
// One node of the learned-warm-start sweep; every lane of the warp calls it together
// (valid false: a lane without a node, which still takes part in the network).
template <bool ANISO, int NODES>
__device__ __forceinline__ void warm_node(const SweepArgs &A, MlpWarpShared &S, const MlpDevice &W, bool valid,
                                          long long i, Acc &acc, const PerturbKey *pk = nullptr) {
  const int nfeat = ANISO ? kFeatAniso : kFeatIso;
  Node n;
  n.solid = false;
  n.centroid = NODES == 1;
  if (valid) node_prepare<ANISO, NODES>(A, i, n, pk);
  double out[CO_COUNT];
#pragma unroll
  for (int k = 0; k < CO_COUNT; k++) out[k] = 0.0;
  int status = MDZ_OK;
  for (int p = 0; p < A.M.np; p++) {  // uniform over the warp
    const double perc = (valid && n.solid) ? node_perc(A, n, p) : 0.0;
    const bool active = fp64_abs_gt(perc, 1e-13);
    if (valid && n.solid && !active) node_iters(A, n, p, 0);
    IsoState st;
    PointOut o;
    float f[kMlpIn], x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; k++) f[k] = 0.0f;
    if (active) {
      if (ANISO) aniso_setup(A.M, A.ph[p], n.in, n.ctx, n.an, st, o, W.polish_iters == 0);
      else iso_setup(A.M, A.ph[p], n.in, n.ctx, st, o, W.polish_iters == 0);
      warm_features(A.M, n.in, n.ctx, st, ANISO, f);
    }
    warm_inputs(W, f, nfeat, x);
    __syncwarp();
    const float y = mlp_warp_predict(S, x);
    if (!active) continue;
    const float s_start = warm_start_point(y, W.z_scale, W.z_shift);
    if (ANISO) aniso_finish(A.M, A.ph[p], n.in, n.ctx, n.an, st, s_start, W.polish_iters, o);
    else iso_finish(A.M, A.ph[p], n.in, n.ctx, st, s_start, W.polish_iters, o);
    node_accumulate<ANISO>(A, n, p, perc, o, out, acc, status);
  }
  if (valid) node_store<ANISO>(A, n, out, status);
}

// One node per lane, the warp's 32 nodes consecutive, so every lane of a warp runs the
// same number of node iterations and reaches the network at the same phase; lanes past
// the end or at inactive (node, phase) items feed zeros and discard the output.
template <bool ANISO, int NODES>
__global__ void __launch_bounds__(128, 4) k_sweep_warm(const __grid_constant__ SweepArgs A,
                                                    const __grid_constant__ MlpDevice W) {
  extern __shared__ __align__(16) unsigned char smem_warm[];
  MlpWarpShared &S = *reinterpret_cast<MlpWarpShared *>(smem_warm);
  mlp_warp_load(S, W);
  Acc acc = {0, 0, 0, 0, 0};
  const long long total = NODES == 1 ? A.M.Nc : A.M.Nv;
  const long long lo = NODES == 1 ? 0 : A.M.Nc;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if constexpr (ANISO) {
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
      const long long j = base + lane;
      warm_node<ANISO, NODES>(A, S, W, j < total, lo + j, acc);
    }
  } else {  // the isotropic sweep compacts its plastic returns per CTA (k_sweep_compact)
    __shared__ CompactQueue Q;
    compact_init(Q);
    int par = 0;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < total; base += stride) {  // uniform
      const long long j = base + threadIdx.x;
      compact_node<NODES, true>(A, j < total, lo + j, acc, Q, par, &S, &W);
    }
  }
  flush_acc(A.stats, acc);
}

// ---------------------------------------------------------------------------------
// many grids in one launch: the node range of every grid is cut into tiles of
// kBatchTile nodes, so a CTA's tile lies in one grid; the grid's arguments are read
// from global memory (uniform over the CTA, served by L1)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int batch_grid_of(const long long *tile_start, int n, long long tile) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&tile_start[mid]) <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One kernel per kind of node, as for a single grid (and with the same node body, so a
// grid swept here gives the single-grid results to the bit): the centroid tiles of every
// grid (NODES 1), then the vertex tiles (NODES 2).  A tile of kBatchTile nodes is one CTA
// and lies in one grid, so the phase loop is uniform over the CTA and the learned warm
// start (WARM) is evaluated per warp as in k_sweep_warm.  PERTURB: the strain rates are
// multiplied by the sweep's perturbation factors as they are loaded, in place (the
// captured multi-sweep graph), instead of by a separate pass over them.
template <bool ANISO, int NODES, bool WARM, bool PERTURB>
__global__ void __launch_bounds__(kBatchTile, 4) k_sweep_batch(const __grid_constant__ BatchArgs B,
                                                             const __grid_constant__ BatchSweepArgs X) {
  extern __shared__ __align__(16) unsigned char smem_batch[];
  MlpWarpShared &S = *reinterpret_cast<MlpWarpShared *>(smem_batch);
  if (WARM) mlp_warp_load(S, X.mlp);
  Acc acc = {0, 0, 0, 0, 0};
  const long long *ts = NODES == 1 ? B.tile_start_n : B.tile_start_s;
  const long long tiles = NODES == 1 ? B.tiles_n : B.tiles_s;
  [[maybe_unused]] int par = 0;
  if constexpr (!ANISO) {
    __shared__ CompactQueue Q;
    compact_init(Q);
    for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {  // uniform over the CTA
      const int g = batch_grid_of(ts, B.n, t);
      const SweepArgs &A = B.grids[g];
      const long long j = (t - __ldg(&ts[g])) * kBatchTile + threadIdx.x;
      const bool valid = j < (NODES == 1 ? A.M.Nc : A.M.Nv);
      const long long i = NODES == 1 ? j : A.M.Nc + j;
      PerturbKey pk;
      if (PERTURB) { pk.key = perturb_key(X.seed, X.sweep, g); pk.amp = X.amp; }
      compact_node<NODES, WARM>(A, valid, i, acc, Q, par, &S, &X.mlp, PERTURB ? &pk : nullptr);
    }
  } else {
    for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {  // uniform over the CTA
      const int g = batch_grid_of(ts, B.n, t);
      const SweepArgs &A = B.grids[g];
      const long long j = (t - __ldg(&ts[g])) * kBatchTile + threadIdx.x;
      const bool valid = j < (NODES == 1 ? A.M.Nc : A.M.Nv);
      const long long i = NODES == 1 ? j : A.M.Nc + j;
      PerturbKey pk;
      if (PERTURB) { pk.key = perturb_key(X.seed, X.sweep, g); pk.amp = X.amp; }
      if (WARM) warm_node<ANISO, NODES>(A, S, X.mlp, valid, i, acc, PERTURB ? &pk : nullptr);
      else if (valid) sweep_node<ANISO, NODES>(A, i, acc, PERTURB ? &pk : nullptr);
    }
  }
  flush_acc(B.stats, acc);
}

// ---------------------------------------------------------------------------------
// tiled sweep with a block-wide stage per phase (learned warm start / data collection)
// ---------------------------------------------------------------------------------
// NODES 1 sweeps the centroids, NODES 2 the vertices (one launch each, with the node
// bodies of the plain sweep's two kernels).
template <bool ANISO, int MODE, int NODES>
__global__ void __launch_bounds__(128, 2) k_sweep_tiles(const __grid_constant__ SweepArgs A,
                                                     const __grid_constant__ WarmArgs W) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  MlpShared &S = *reinterpret_cast<MlpShared *>(smem_raw);
  uint32_t phase = 0;
  if (MODE == MODE_WARM) mlp_begin(S, W.mlp);
  Acc acc = {0, 0, 0, 0, 0};
  const long long total = A.M.Nc + A.M.Nv;
  const long long count = NODES == 1 ? A.M.Nc : A.M.Nv, base = NODES == 1 ? 0 : A.M.Nc;
  const long long ntiles = (count + kMlpTile - 1) / kMlpTile;
  const int nfeat = ANISO ? kFeatAniso : kFeatIso;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {  // uniform over the CTA
    const long long j = tile * kMlpTile + threadIdx.x;
    const bool valid = j < count;
    const long long i = base + j;
    Node n;
    n.solid = false;
    n.centroid = NODES == 1;
    if (valid) node_prepare<ANISO, NODES>(A, i, n);
    double out[CO_COUNT];
#pragma unroll
    for (int j = 0; j < CO_COUNT; j++) out[j] = 0.0;
    int status = MDZ_OK;
    for (int p = 0; p < A.M.np; p++) {  // uniform over the CTA
      const double perc = (valid && n.solid) ? node_perc(A, n, p) : 0.0;
      const bool active = fp64_abs_gt(perc, 1e-13);
      if (valid && n.solid && !active) node_iters(A, n, p, 0);
      IsoState st;
      PointOut o;
      float f[kMlpIn];
#pragma unroll
      for (int j = 0; j < kMlpIn; j++) f[j] = 0.0f;
      float s_start = ANISO ? 0.0f : 1.0f;  // the reference's own start
      if (active) {
        const bool exact = (MODE == MODE_COLLECT) || W.mlp.polish_iters == 0;  // the pairs' targets need eta_up
        if (ANISO) aniso_setup(A.M, A.ph[p], n.in, n.ctx, n.an, st, o, exact);
        else iso_setup(A.M, A.ph[p], n.in, n.ctx, st, o, exact);
        warm_features(A.M, n.in, n.ctx, st, ANISO, f);
      }
      if (MODE == MODE_WARM) {
        float x[kMlpIn];
#pragma unroll
        for (int j = 0; j < kMlpIn; j++) x[j] = (j < nfeat) ? (f[j] - W.mlp.x_shift[j]) * W.mlp.x_scale[j] : 0.0f;
        float y[2];
        mlp_forward(S, x, y, phase, W.mlp.poll_limit);
        if (active && !S.fault) {
          s_start = warm_start_point(y[0], W.mlp.z_scale, W.mlp.z_shift);
        }
      }
      if (!active) continue;
      double eta_conv = 0.0;
      const int polish = (MODE == MODE_WARM) ? W.mlp.polish_iters : 0;
      if (ANISO) aniso_finish(A.M, A.ph[p], n.in, n.ctx, n.an, st, s_start, polish, o, &eta_conv);
      else iso_finish(A.M, A.ph[p], n.in, n.ctx, st, s_start, polish, o, &eta_conv);
      node_accumulate<ANISO>(A, n, p, perc, o, out, acc, status);
      if (MODE == MODE_COLLECT) {
        const long long item = (long long)p * total + i;
        float *xo = W.X_out + item * kMlpIn;
#pragma unroll
        for (int j = 0; j < kMlpIn; j++) xo[j] = f[j];
        W.Y_out[item * 2 + 0] = (eta_conv > 0.0) ? (float)log(st.eta_up / eta_conv) : __int_as_float(0x7fc00000);
        W.Y_out[item * 2 + 1] = (float)o.is_pl;
      }
    }
    if (valid) node_store<ANISO>(A, n, out, status);
    if (MODE == MODE_COLLECT && valid) {  // items of inactive phases carry a NaN target
      for (int p = 0; p < A.M.np; p++) {
        const double perc = n.solid ? node_perc(A, n, p) : 0.0;
        if (!fp64_abs_gt(perc, 1e-13)) W.Y_out[((long long)p * total + i) * 2] = __int_as_float(0x7fc00000);
      }
    }
  }
  if (MODE == MODE_WARM) {
    mlp_end(S);
    if (threadIdx.x == 0 && S.fault) atomicExch(&A.stats->mma_fault, 1u);
  }
  flush_acc(A.stats, acc);
}

// ---------------------------------------------------------------------------------
// independent points: ViscosityConcise / ViscosityConciseAniso
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_points(const __grid_constant__ PointArgs A) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Acc acc = {0, 0, 0, 0, 0};
  const bool bad_phase = (i < A.n) && (A.in.phase[i] < 0 || A.in.phase[i] >= A.M.np);
  if (bad_phase) {  // phase ids in device memory are only checked here
    if (A.out.status) A.out.status[i] = MDZ_EINVAL;
    record_error(A.stats, i, MDZ_EINVAL);
  }
  if (i < A.n && !bad_phase) {
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
      point_aniso(A.M, A.ph[p], in, ctx, an, A.polish, o);
    } else {
      node_setup_iso(A.M, in, true, ctx);
      point_iso(A.M, A.ph[p], in, ctx, A.polish, o);
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
    acc.calls = 1; acc.iters = o.iters; acc.plastic = o.is_pl; acc.maxit = o.iters; acc.f32 = o.f32_steps;
  }
  flush_acc(A.stats, acc);
}

template <bool ANISO, int NODES>
static void launch_kind(const SweepArgs &a, const LaunchShape &sh, long long count, cudaStream_t s) {
  if (sh.form == SHAPE_QUEUE) {
    k_sweep_queue<ANISO, NODES><<<(unsigned)sh.grid_cap, 128, 0, s>>>(a);
    return;
  }
  if (!ANISO && sh.form == SHAPE_COMPACT) {  // the isotropic sweep only
    long long grid = (count + 127) / 128;
    if (sh.grid_cap > 0 && grid > sh.grid_cap) grid = sh.grid_cap;
    k_sweep_compact<NODES><<<(unsigned)grid, 128, 0, s>>>(a);
    return;
  }
  long long grid = (count + sh.block - 1) / sh.block;
  if (sh.grid_cap > 0 && grid > sh.grid_cap) grid = sh.grid_cap;
  if (sh.form == SHAPE_REGS255) k_sweep<ANISO, NODES, 2><<<(unsigned)grid, sh.block, 0, s>>>(a);
  else k_sweep<ANISO, NODES, 4><<<(unsigned)grid, sh.block, 0, s>>>(a);
}

cudaError_t launch_sweep(const SweepArgs &a, bool aniso, cudaStream_t s, const LaunchShape &shape) {
  const long long counts[2] = {a.ranged ? a.c_n : a.M.Nc, a.ranged ? a.v_n : a.M.Nv};
  // the work counter of the persistent form covers a whole sweep, not a band of rows
  LaunchShape sh = shape;
  if (sh.form == SHAPE_QUEUE && (a.ranged || sh.grid_cap <= 0)) sh.form = SHAPE_THREAD;
  if (sh.form == SHAPE_QUEUE) sh.block = 128;
  for (int kind = 0; kind < 2; kind++) {
    if (counts[kind] <= 0) continue;
    if (kind == 0 && aniso) launch_kind<true, 1>(a, sh, counts[kind], s);
    else if (kind == 0) launch_kind<false, 1>(a, sh, counts[kind], s);
    else if (aniso) launch_kind<true, 2>(a, sh, counts[kind], s);
    else launch_kind<false, 2>(a, sh, counts[kind], s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <bool ANISO, int NODES>
static cudaError_t launch_warm_t(const SweepArgs &a, const MlpDevice &w, cudaStream_t s, long long count) {
  auto fn = k_sweep_warm<ANISO, NODES>;
  const size_t smem = sizeof(MlpWarpShared);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  fn<<<(unsigned)((count + 127) / 128), 128, smem, s>>>(a, w);
  return cudaGetLastError();
}

cudaError_t launch_sweep_warm(const SweepArgs &a, const MlpDevice &w, bool aniso, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (a.M.Nc > 0) e = aniso ? launch_warm_t<true, 1>(a, w, s, a.M.Nc) : launch_warm_t<false, 1>(a, w, s, a.M.Nc);
  if (e != cudaSuccess || a.M.Nv <= 0) return e;
  return aniso ? launch_warm_t<true, 2>(a, w, s, a.M.Nv) : launch_warm_t<false, 2>(a, w, s, a.M.Nv);
}

// The warm-start form keeps its MLP tiles in dynamic shared memory; asking for the
// largest shared-memory carve-out lets two of its CTAs share an SM (the register file
// allows two), which the occupancy query then reports.
template <bool ANISO, int MODE, int NODES>
static void tiles_attributes() {
  if (MODE != MODE_WARM) return;
  auto fn = k_sweep_tiles<ANISO, MODE, NODES>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpShared));
  cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
}

template <bool ANISO, int MODE>
static cudaError_t launch_tiles_t(const SweepArgs &a, const WarmArgs &w, cudaStream_t s, int grid) {
  const size_t smem = (MODE == MODE_WARM) ? sizeof(MlpShared) : 0;
  const long long tiles[2] = {(a.M.Nc + kMlpTile - 1) / kMlpTile, (a.M.Nv + kMlpTile - 1) / kMlpTile};
  tiles_attributes<ANISO, MODE, 1>();
  tiles_attributes<ANISO, MODE, 2>();
  if (tiles[0] > 0)
    k_sweep_tiles<ANISO, MODE, 1><<<(unsigned)(tiles[0] < grid ? tiles[0] : grid), kMlpTile, smem, s>>>(a, w);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || tiles[1] <= 0) return e;
  k_sweep_tiles<ANISO, MODE, 2><<<(unsigned)(tiles[1] < grid ? tiles[1] : grid), kMlpTile, smem, s>>>(a, w);
  return cudaGetLastError();
}

cudaError_t launch_sweep_tiles(const SweepArgs &a, const WarmArgs &w, bool aniso, int mode, cudaStream_t s,
                               int grid) {
  if (grid < 1) grid = 1;
  switch (mode * 2 + (aniso ? 1 : 0)) {
    case MODE_COLLECT * 2: return launch_tiles_t<false, MODE_COLLECT>(a, w, s, grid);
    case MODE_COLLECT * 2 + 1: return launch_tiles_t<true, MODE_COLLECT>(a, w, s, grid);
    case MODE_WARM * 2: return launch_tiles_t<false, MODE_WARM>(a, w, s, grid);
    case MODE_WARM * 2 + 1: return launch_tiles_t<true, MODE_WARM>(a, w, s, grid);
    default: return cudaErrorInvalidValue;
  }
}

int tiles_blocks_per_sm(bool aniso, int mode) {
  int n = 0;
  const void *fn = nullptr;
  switch (mode * 2 + (aniso ? 1 : 0)) {
    case MODE_COLLECT * 2: fn = (const void *)k_sweep_tiles<false, MODE_COLLECT, 1>; break;
    case MODE_COLLECT * 2 + 1: fn = (const void *)k_sweep_tiles<true, MODE_COLLECT, 1>; break;
    case MODE_WARM * 2: fn = (const void *)k_sweep_tiles<false, MODE_WARM, 1>; break;
    default: fn = (const void *)k_sweep_tiles<true, MODE_WARM, 1>; break;
  }
  const size_t smem = (mode == MODE_WARM) ? sizeof(MlpShared) : 0;
  if (mode == MODE_WARM) {
    if (aniso) tiles_attributes<true, MODE_WARM, 1>();
    else tiles_attributes<false, MODE_WARM, 1>();
  }
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kMlpTile, smem);
  // The query has been seen to report one CTA where registers (255 per thread, 2 CTAs
  // of 128) and the shared-memory carve-out allow two; bound it below by the register
  // file and shared memory directly.  A larger grid only changes residency, not results.
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess && fa.numRegs > 0) {
    const int regs = (fa.numRegs + 7) & ~7;
    int by_regs = 65536 / (kMlpTile * regs);
    int by_smem = (int)((227 * 1024) / (smem + fa.sharedSizeBytes + 1024));
    const int own = by_regs < by_smem ? by_regs : by_smem;
    if (own > n) n = own;
  }
  cudaGetLastError();
  return n > 0 ? n : 1;
}

template <bool ANISO, int NODES, bool WARM, bool PERTURB>
static cudaError_t launch_batch_t(const BatchArgs &b, const BatchSweepArgs &x, cudaStream_t s, long long grid) {
  auto fn = k_sweep_batch<ANISO, NODES, WARM, PERTURB>;
  const size_t smem = WARM ? sizeof(MlpWarpShared) : 0;
  if (WARM) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  fn<<<(unsigned)grid, kBatchTile, smem, s>>>(b, x);
  return cudaGetLastError();
}

template <bool ANISO, int NODES>
static cudaError_t launch_batch_kind(const BatchArgs &b, const BatchSweepArgs &x, cudaStream_t s, long long grid) {
  const bool pert = x.amp != 0.0;
  if (x.warm) return pert ? launch_batch_t<ANISO, NODES, true, true>(b, x, s, grid)
                          : launch_batch_t<ANISO, NODES, true, false>(b, x, s, grid);
  return pert ? launch_batch_t<ANISO, NODES, false, true>(b, x, s, grid)
              : launch_batch_t<ANISO, NODES, false, false>(b, x, s, grid);
}

cudaError_t launch_sweep_batch(const BatchArgs &b, const BatchSweepArgs &x, bool aniso, cudaStream_t s, int grid) {
  // one CTA per tile, up to `grid`, per kind
  const long long gn = b.tiles_n < grid ? b.tiles_n : grid, gs = b.tiles_s < grid ? b.tiles_s : grid;
  cudaError_t e = cudaSuccess;
  if (gn > 0) e = aniso ? launch_batch_kind<true, 1>(b, x, s, gn) : launch_batch_kind<false, 1>(b, x, s, gn);
  if (e != cudaSuccess) return e;
  if (gs > 0) e = aniso ? launch_batch_kind<true, 2>(b, x, s, gs) : launch_batch_kind<false, 2>(b, x, s, gs);
  return e;
}

cudaError_t launch_points(const PointArgs &a, cudaStream_t s) {
  const int block = 128;
  const long long grid = (a.n + block - 1) / block;
  if (grid > 0) k_points<<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

void sweep_kernel_info(int aniso, int *regs, int *smem, int *max_blocks_per_sm, int block, int form) {
  cudaFuncAttributes fa;
  // the centroid kernel: the larger of the two, it sets the launch shape
  const void *fn = aniso ? (const void *)k_sweep<true, 1, 4> : (const void *)k_sweep<false, 1, 4>;
  if (form == SHAPE_REGS255) fn = aniso ? (const void *)k_sweep<true, 1, 2> : (const void *)k_sweep<false, 1, 2>;
  if (form == SHAPE_QUEUE) fn = aniso ? (const void *)k_sweep_queue<true, 1> : (const void *)k_sweep_queue<false, 1>;
  if (form == SHAPE_COMPACT && !aniso) fn = (const void *)k_sweep_compact<1>;
  cudaFuncGetAttributes(&fa, fn);
  *regs = fa.numRegs;
  *smem = (int)fa.sharedSizeBytes;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(max_blocks_per_sm, fn, block, 0);
}

}  // namespace mdz
