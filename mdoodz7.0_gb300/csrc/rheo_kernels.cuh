// rheo_kernels.cuh -- launch-side declarations shared by the kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.cuh"
#include "mlp_warp.cuh"
#include "rheo_device.cuh"

namespace mdz {

// Centroid input fields (grid member names, MDLIB/mdoodz-private.h:75-147)
enum CenIn { CI_mu, CI_T, CI_p_in, CI_d0, CI_phi0, CI_X0, CI_exxd, CI_ezzd, CI_exz, CI_sxxd0, CI_szzd0, CI_sxz0,
             CI_fric, CI_C, CI_dil, CI_p0, CI_T0, CI_bet, CI_d1, CI_d2, CI_angle, CI_anif, CI_COUNT };
enum VerIn { VI_mu, VI_X0, VI_exxd, VI_ezzd, VI_exz, VI_sxxd0, VI_szzd0, VI_sxz0, VI_fric, VI_C, VI_dil, VI_p0,
             VI_bet, VI_d1, VI_d2, VI_angle, VI_anif, VI_COUNT };
enum CenOut { CO_eta, CO_eta_phys, CO_VE, CO_sxxd, CO_szzd, CO_sxz, CO_eII_el, CO_eII_pl, CO_eII_pwl, CO_eII_exp,
              CO_eII_lin, CO_eII_gbs, CO_eII_cst, CO_d, CO_p_corr, CO_div_el, CO_div_pl, CO_div_r, CO_Wtot,
              CO_Wel, CO_Wdiss, CO_X, CO_OverS, CO_rho, CO_COUNT };
enum VerOut { VO_sxxd, VO_szzd, VO_sxz, VO_eta_phys, VO_eta, VO_X, VO_VE, VO_T, VO_P, VO_d0, VO_phi0, VO_COUNT };

// Device statistics block (one per context)
struct DevStats {
  unsigned long long err_key;  // (node << 8) | -status of the lowest failing node; ~0 if none
  unsigned long long calls, iters, plastic;
  unsigned int maxit;
  unsigned int mma_fault;      // a tensor-core completion wait gave up (warm start)
  unsigned long long f32_steps;  // FP32 Newton steps taken by the starts of the local solves
  unsigned long long queue[2];   // work counters of the persistent sweep (centroids, vertices)
};

// Launch shape of the plain sweep: threads per block, grid cap (0: one thread per node;
// else a grid-stride loop over that many CTAs) and the kernel form.
enum { SHAPE_THREAD = 0, SHAPE_REGS255 = 1, SHAPE_QUEUE = 2, SHAPE_COMPACT = 3 };
struct LaunchShape {
  int block, grid_cap, form;
};

// modes of the tiled sweep
enum { MODE_COLLECT = 0, MODE_WARM = 1 };

struct WarmArgs {
  MlpDevice mlp;
  float *X_out;  // MODE_COLLECT: features [item][kMlpIn], item = p * (Nc + Nv) + node
  float *Y_out;  // MODE_COLLECT: targets [item][2] = (ln(eta_up / eta_ve), is_pl); NaN for inactive items
};

struct SweepArgs {
  ModelConst M;
  PhaseConst ph[MDZ_MAX_PHASES];
  const double *ci[CI_COUNT];
  const double *vi[VI_COUNT];
  double *co[CO_COUNT];
  double *vo[VO_COUNT];
  const double *perc_n[MDZ_MAX_PHASES];
  const double *perc_s[MDZ_MAX_PHASES];
  double *peta_n[MDZ_MAX_PHASES];
  double *peta_s[MDZ_MAX_PHASES];
  const signed char *bcp;
  const signed char *bcg;
  int32_t *iters_n, *iters_s;  // optional [p*N + node]
  DevStats *stats;
  int final_update, need_lnd;
  int polish;  // start descriptor of every local solve: FP32 Newton steps | MDZ_START_DD (0: the reference's start)
  long long node_base;  // added to node indices in error reports (batched grids)
  // k_sweep over a band of rows only: centroids [c_lo, c_lo + c_n) and vertices
  // [v_lo, v_lo + v_n); 0 sweeps every node
  int ranged;
  long long c_lo, c_n, v_lo, v_n;
};

// Many grids in one launch.  Grid g owns tiles [tile_start[g], tile_start[g + 1]) of
// kBatchTile nodes (centroids first, then vertices, as in one sweep).
constexpr int kBatchTile = 128;
struct BatchArgs {
  const SweepArgs *grids;       // device array [n]
  const long long *tile_start;  // device array [n + 1]: tiles over each grid's nodes
  // the same cut over the centroids and over the vertices separately, for the sweep's
  // two kernels (device arrays [n + 1])
  const long long *tile_start_n, *tile_start_s;
  int n;
  long long tiles, tiles_n, tiles_s;
  DevStats *stats;
};

struct PointArgs {
  ModelConst M;
  PhaseConst ph[MDZ_MAX_PHASES];
  mdz_point_inputs in;
  mdz_point_outputs out;
  long long n;
  int aniso;
  int polish;  // as in SweepArgs
  DevStats *stats;
};

cudaError_t launch_sweep(const SweepArgs &a, bool aniso, cudaStream_t s, const LaunchShape &shape);
// kernels launch_sweep issues for these arguments: one per kind of node (centroids,
// vertices) with nodes in range; launch_sweep_tiles issues the same over the whole grid
inline unsigned sweep_kernel_count(const SweepArgs &a) {
  const long long nc = a.ranged ? a.c_n : a.M.Nc, nv = a.ranged ? a.v_n : a.M.Nv;
  return (nc > 0 ? 1u : 0u) + (nv > 0 ? 1u : 0u);
}
// kernels launch_sweep_batch issues: one per kind of node with tiles
inline unsigned batch_kernel_count(const BatchArgs &b) { return (b.tiles_n > 0 ? 1u : 0u) + (b.tiles_s > 0 ? 1u : 0u); }
cudaError_t launch_points(const PointArgs &a, cudaStream_t s);
// Per-launch options of a batched sweep: the learned warm start (warm, mlp), and the
// strain-rate perturbation fused into the load (amp != 0: factors 1 + amp u, u uniform in
// [-1, 1) from the counter hash of (seed, sweep, grid, node, component)).
struct BatchSweepArgs {
  MlpDevice mlp;
  int warm;
  double amp;
  unsigned long long seed;
  int sweep;
};
cudaError_t launch_sweep_batch(const BatchArgs &b, const BatchSweepArgs &x, bool aniso, cudaStream_t s, int grid);
cudaError_t launch_sweep_tiles(const SweepArgs &a, const WarmArgs &w, bool aniso, int mode, cudaStream_t s,
                               int grid);
// the learned warm start evaluated per warp (mlp_warp.cuh): one launch per kind of node
cudaError_t launch_sweep_warm(const SweepArgs &a, const MlpDevice &w, bool aniso, cudaStream_t s);
int tiles_blocks_per_sm(bool aniso, int mode);
void sweep_kernel_info(int aniso, int *regs, int *smem, int *max_blocks_per_sm, int block, int form);

}  // namespace mdz
