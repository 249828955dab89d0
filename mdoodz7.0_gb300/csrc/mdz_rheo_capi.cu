// mdz_rheo_capi.cu -- the C ABI of include/mdz_rheo.h.
//
// A context owns one CUDA stream, a device statistics block and, for host-memory
// sweeps, device mirrors of the grid fields (grown on demand, kept until destroy).
// Per-phase material constants are folded here, once per call, into the PhaseConst
// table the kernels read from their constant parameter bank.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "mlp_train.cuh"
#include "operators.cuh"
#include "rheo_kernels.cuh"
#include "markers.cuh"
#include "prep.cuh"
#include "strain_rates.cuh"

#include <algorithm>
#include <random>

using namespace mdz;

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

struct mdz_rheo_ctx {
  int device = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DevStats *d_stats = nullptr, *h_stats = nullptr;
  std::vector<DevBuf> bufs;
  int32_t *d_iters_n = nullptr, *d_iters_s = nullptr;
  size_t cap_iters_n = 0, cap_iters_s = 0;
  long long last_Nc = 0, last_Nv = 0;
  int last_np = 0, have_iters = 0, pending = 0;
  unsigned long long h2d = 0, d2h = 0;
  unsigned launches = 0;
  // untuned shape, [iso, aniso]: the isotropic sweep compacts its plastic returns per CTA
  LaunchShape shape[2] = {{128, 0, SHAPE_COMPACT}, {128, 0, SHAPE_THREAD}};
  // shapes the autotuner chose, keyed by (anisotropic, phases, reference start, nodes); a
  // sweep takes the entry of its key with the nearest node count, else shape[aniso]
  struct Tuned {
    int aniso, np, ref;
    long long nodes;
    LaunchShape shape;
  };
  std::vector<Tuned> tuned;
  // host-memory sweeps in row bands: copies in, kernels and copies out overlap
  cudaStream_t copy_in = nullptr, copy_out = nullptr, compute2 = nullptr;
  cudaEvent_t band_ev[2 * 16 + 3] = {};
  int bands = 0;  // 0: automatic (rows / 128, at most 16); else this many
  int sms = 0;
  // learned warm start
  void *warm_buf = nullptr;  // tiles W1, W2, W3 + biases b1, b2, b3[16]
  MlpDevice warm{};
  int warm_ready = 0, polish_iters = MDZ_DEFAULT_START;
  unsigned mma_fault = 0;
  unsigned mma_poll_limit = 1u << 24;  // tcgen05 completion polls before a wait gives up
};

struct mdz_rheo_batch {
  mdz_rheo_ctx *ctx = nullptr;
  int n = 0;
  bool aniso = false, warm = false;  // warm: the learned warm start in every sweep of the batch
  SweepArgs *d_grids = nullptr;
  long long *d_tile_start = nullptr;
  long long tiles = 0, nodes = 0;
  BatchArgs args{};
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_sweeps = 0, graph_launches = 0;
};

namespace {

constexpr int kBatchMaxGrids = 4096;

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      fprintf(stderr, "mdz_rheo: %s failed: %s\n", #x, cudaGetErrorString(e_)); \
      return MDZ_ECUDA;                                                       \
    }                                                                         \
  } while (0)

int ensure(DevBuf &b, size_t bytes) {
  if (b.cap >= bytes) return MDZ_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  if (cudaMalloc(&b.p, bytes) != cudaSuccess) return MDZ_ENOMEM;
  b.cap = bytes;
  return MDZ_OK;
}

// PhaseConst from one column of mat_prop (flow-law conventions of
// MDLIB/RheologyDensity.c:501-539 folded into logs; see rheo_device.cuh).
void fold_phase(const mdz_materials *m, const mdz_model *md, int p, PhaseConst &c) {
  memset(&c, 0, sizeof(c));
  int fl = 0;
  if (m->cstv[p] != 0) fl |= F_CST;
  if (m->pwlv[p] != 0) fl |= F_PWL;
  if (m->expv[p] != 0) fl |= F_EXPV;
  if (m->linv[p] != 0) fl |= F_LIN;
  if (m->gbsv[p] != 0) fl |= F_GBS;
  if (m->gs[p] != 0) fl |= F_GS;
  if (m->plast[p] == 1) fl |= F_PL1;
  if (m->plast[p] == 2) fl |= F_PL2;
  if (m->plast[p] != 0) fl |= F_PLANY;
  if (m->phase_mix[p] == 1 && md->diffuse_X != 0) fl |= F_CMIX;
  if (m->nlin[p] == 1.0) fl |= F_LIN1;
  if (m->npwl[p] == 1.0) fl |= F_PWL1;
  if (m->mpwl[p] != 0.0) fl |= F_PWL_M;
  if (m->apwl[p] != 0.0) fl |= F_PWL_A;
  if (m->alin[p] != 0.0) fl |= F_LIN_A;
  if (1.0 / m->n_vp[p] - 1.0 == 0.0) fl |= F_VP1;
  c.flags = fl;
  c.density_model = m->density_model[p];
  c.phase_two = m->phase_two[p];
  c.reac_phase = m->reac_phase[p];
  const double R = m->R;
  // dislocation: B = pref F A^(-1/n) exp((Q+PV)/(R n T)) d^(m/n) f^(-r/n) exp(-a phi/n)
  {
    const double n = m->npwl[p];
    c.pwl_n = n; c.pwl_invn = 1.0 / n;
    c.pwl_lnK = log(m->pref_pwl[p]) + log(m->Fpwl[p]) - log(m->Apwl[p]) / n;
    if (m->rpwl[p] != 0.0) c.pwl_lnK += -(m->rpwl[p] / n) * log(m->fpwl[p]);
    c.pwl_Q = m->Qpwl[p]; c.pwl_V = m->Vpwl[p]; c.pwl_invRn = 1.0 / (R * n);
    c.pwl_mn = m->mpwl[p] / n; c.pwl_an = m->apwl[p] / n;
  }
  // diffusion: B = F A^(-1/n) exp((Q+PV)/(R n T)) f^(-r/n) exp(-a phi/n)
  {
    const double n = m->nlin[p];
    c.lin_n = n; c.lin_invn = 1.0 / n;
    c.lin_lnK = log(m->Flin[p]) - log(m->Alin[p]) / n;
    if (m->rlin[p] != 0.0) c.lin_lnK += -(m->rlin[p] / n) * log(m->flin[p]);
    c.lin_Q = m->Qlin[p]; c.lin_V = m->Vlin[p]; c.lin_invRn = 1.0 / (R * n);
    c.lin_m = m->mlin[p]; c.lin_mn = m->mlin[p] / n; c.lin_an = m->alin[p] / n;
  }
  // grain-boundary sliding (bracket only)
  {
    const double n = m->ngbs[p];
    c.gbs_n = n; c.gbs_invn = 1.0 / n;
    c.gbs_lnK = log(m->Fgbs[p]) - log(m->Agbs[p]) / n;
    if (m->rgbs[p] != 0.0) c.gbs_lnK += -(m->rgbs[p] / n) * log(m->fgbs[p]);
    c.gbs_Q = m->Qgbs[p]; c.gbs_V = m->Vgbs[p]; c.gbs_invRn = 1.0 / (R * n);
    c.gbs_m = m->mgbs[p]; c.gbs_mn = m->mgbs[p] / n; c.gbs_an = m->agbs[p] / n;
  }
  // Peierls (RheologyDensity.c:518-523): with nE = ST + n,
  //   C Tii^nE = (sqrt3/2) E Arr (gamma S)^n (sqrt3 Tii / (gamma S))^nE
  {
    const double g = m->Gexp[p], gS = g * m->Sexp[p];
    c.exp_EaR = m->Qexp[p] / R; c.exp_g2 = 2.0 * g * (1 - g); c.exp_om2 = (1.0 - g) * (1.0 - g);
    c.exp_n = m->nexp[p];
    c.exp_lnA0 = kLnSqrt3 - kLn2 + log(m->Eexp[p]) + (m->nexp[p] != 0.0 ? m->nexp[p] * log(gS) : 0.0);
    c.exp_s3gS = kSqrt3 / gS;
    c.exp_ln_s3gS = log(c.exp_s3gS);
  }
  c.eta0 = m->eta0[p];
  const int p2 = m->phase_two[p];
  c.eta0_two = (p2 >= 0 && p2 < MDZ_MAX_PHASES) ? m->eta0[p2] : m->eta0[p];
  c.Slim = m->Slim[p]; c.eta_vp = m->eta_vp[p]; c.n_vp = m->n_vp[p]; c.T_st = m->T_st[p];
  c.gs_ref = m->gs_ref[p]; c.inv_gs_ref = 1.0 / m->gs_ref[p]; c.ln_gs_ref = log(m->gs_ref[p]);
  c.Kpzm = m->Kpzm[p]; c.Qpzm = m->Qpzm[p]; c.Gpzm = m->Gpzm[p]; c.Lpzm = m->Lpzm[p];
  c.cpzm = m->cpzm[p]; c.ppzm = m->ppzm[p];
  c.rho = m->rho[p]; c.drho = m->drho[p]; c.alp = m->alp[p]; c.bet = m->bet[p]; c.T0 = m->T0[p]; c.P0 = m->P0[p];
  const int rp = m->reac_phase[p];
  c.rho_reac = (rp >= 0 && rp < MDZ_MAX_PHASES) ? m->rho[rp] : m->rho[p];
}

int fold_model(const mdz_model *md, const mdz_materials *m, ModelConst &M) {
  memset(&M, 0, sizeof(M));
  if (md->Nb_phases < 1 || md->Nb_phases > MDZ_MAX_PHASES) return MDZ_EINVAL;
  if (md->melting || md->chemical_production) return MDZ_EUNSUPPORTED;
  M.np = md->Nb_phases;
  M.elastic = md->elastic; M.step = md->step; M.eta_average = md->eta_average;
  M.periodic_x = md->periodic_x; M.density_variations = md->density_variations;
  M.tensile_line_search = md->tensile_line_search; M.diffuse_avg = md->diffuse_avg;
  M.Nx = md->Nx; M.Nz = md->Nz; M.Ncx = md->Nx - 1; M.Ncz = md->Nz - 1;
  M.Nc = (long long)M.Ncx * M.Ncz; M.Nv = (long long)M.Nx * M.Nz;
  M.dt_model = md->dt;
  M.dt = (md->step == 0) ? 1e100 : md->dt;  // RheologyDensity.c:392-394
  M.min_eta = md->min_eta; M.max_eta = md->max_eta; M.eta_tol = md->eta_tol; M.R = m->R;
  M.scale_eta = md->scale_eta; M.scale_L = md->scale_L; M.scale_T = md->scale_T; M.scale_S = md->scale_S;
  M.scale_E = md->scale_E;
  M.TmaxPeierls = (1200.0 + kZeroC) / md->scale_T;
  M.Tmin = kZeroC / md->scale_T;
  M.Tiimin = 1e5 / md->scale_S;
  M.Eii_floor = 1e-30 / md->scale_E;
  M.eta_up0 = 1.0e100 / md->scale_eta;
  M.ln_eta_up0 = log(M.eta_up0);
  M.eta_lo0 = -1.0e100 / md->scale_eta;
  M.d_min = 1e-13 / md->scale_L;
  for (int p = 0; p < M.np; p++) {
    const int dm = m->density_model[p];
    if (md->density_variations == 1 && (dm == 2 || dm == 4)) return MDZ_EUNSUPPORTED;
  }
  return MDZ_OK;
}

bool need_lnd(const mdz_materials *m, int np) {
  for (int p = 0; p < np; p++) {
    if (m->pwlv[p] && m->mpwl[p] != 0.0) return true;
    if (m->linv[p] && m->mlin[p] != 0.0) return true;
    if (m->gbsv[p] && m->mgbs[p] != 0.0) return true;
  }
  return false;
}

int stats_from_device(mdz_rheo_ctx *ctx, mdz_sweep_stats *st, float ms) {
  const DevStats &h = *ctx->h_stats;
  int status = MDZ_OK;
  long long node = -1;
  if (h.err_key != ~0ull) {
    status = -(int)(h.err_key & 0xff);
    node = (long long)(h.err_key >> 8);
  }
  if (st) {
    st->phase_calls = h.calls; st->newton_iters = h.iters; st->max_newton_iters = h.maxit;
    st->plastic_calls = h.plastic; st->status = status; st->error_node = node; st->elapsed_ms = ms;
    st->h2d_bytes = ctx->h2d; st->d2h_bytes = ctx->d2h; st->kernel_launches = ctx->launches;
    st->mma_fault = h.mma_fault;
    st->fp32_steps = h.f32_steps;
  }
  return status;
}

int reset_stats(mdz_rheo_ctx *ctx) {
  DevStats init;
  memset(&init, 0, sizeof(init));
  init.err_key = ~0ull;
  *ctx->h_stats = init;
  CK(cudaMemcpyAsync(ctx->d_stats, ctx->h_stats, sizeof(DevStats), cudaMemcpyHostToDevice, ctx->stream));
  return MDZ_OK;
}

int finish(mdz_rheo_ctx *ctx, mdz_sweep_stats *st) {
  CK(cudaMemcpyAsync(ctx->h_stats, ctx->d_stats, sizeof(DevStats), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  return stats_from_device(ctx, st, ms);
}

// slot numbering of the host-mode mirrors
enum { S_CI = 0, S_VI = S_CI + CI_COUNT, S_CO = S_VI + VI_COUNT, S_VO = S_CO + CO_COUNT,
       S_PN = S_VO + VO_COUNT, S_PS = S_PN + MDZ_MAX_PHASES, S_EN = S_PS + MDZ_MAX_PHASES,
       S_ES = S_EN + MDZ_MAX_PHASES, S_BCP = S_ES + MDZ_MAX_PHASES, S_BCG, S_OP, S_SR = S_OP + OP_COUNT,
       S_SRU = S_SR + SR_COUNT, S_SRV, S_PREP, S_MK = S_PREP + 16, S_P2M = S_MK + 33, S_COUNT = S_P2M + 12 };

bool host_mapped(const void *p, size_t bytes);

// Device copies of host arrays, one slot per array.  With `direct`, a page-locked host
// array that the device addresses at the same pointer (host_mapped) is used in place: the
// kernels read and write it over the host link, and its bytes count as crossing it.
struct Mirror {
  mdz_rheo_ctx *ctx;
  bool direct = false;
  int err = MDZ_OK;
  template <class T>
  bool mapped(const T *h, size_t n) const { return direct && host_mapped(h, n * sizeof(T)); }
  // upload (if host) a read-only array of n elements into slot s
  template <class T>
  T *in(const T *h, int slot, size_t n, bool host) {
    if (!h || err) return const_cast<T *>(h);
    if (!host) return const_cast<T *>(h);
    if (mapped(h, n)) {
      ctx->h2d += n * sizeof(T);
      return const_cast<T *>(h);
    }
    if ((err = ensure(ctx->bufs[slot], n * sizeof(T))) != MDZ_OK) return nullptr;
    if (cudaMemcpyAsync(ctx->bufs[slot].p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      err = MDZ_ECUDA;
    ctx->h2d += n * sizeof(T);
    return (T *)ctx->bufs[slot].p;
  }
  template <class T>
  T *out(T *h, int slot, size_t n, bool host) {
    if (!h || err) return h;
    if (!host || mapped(h, n)) return h;
    if ((err = ensure(ctx->bufs[slot], n * sizeof(T))) != MDZ_OK) return nullptr;
    return (T *)ctx->bufs[slot].p;
  }
  // an array that was `in` or `out`: copy it back unless the kernels wrote it in place
  template <class T>
  void back(T *h, int slot, size_t n, bool host) {
    if (!h || err || !host) return;
    if (mapped(h, n)) {
      ctx->d2h += n * sizeof(T);
      return;
    }
    if (cudaMemcpyAsync(h, ctx->bufs[slot].p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
      err = MDZ_ECUDA;
    ctx->d2h += n * sizeof(T);
  }
};

// The field pointers of one sweep in kernel order, checked for presence.
struct FieldLists {
  const double *cin[CI_COUNT];
  const double *vin[VI_COUNT];
  double *cout[CO_COUNT];
  double *vout[VO_COUNT];
  int nci, nvi;
};

int field_lists(const mdz_model *md, const mdz_grid_fields *f, bool aniso, FieldLists &L) {
  const double *cin[CI_COUNT] = {f->mu_n, f->T, f->p_in, f->d0_n, f->phi0_n, f->X0_n, f->exxd, f->ezzd, f->exz_n,
                                 f->sxxd0, f->szzd0, f->sxz0_n, f->fric_n, f->C_n, f->dil_n, f->p0_n, f->T0_n,
                                 f->bet_n, f->d1_n, f->d2_n, f->angle_n, f->aniso_factor_n};
  const double *vin[VI_COUNT] = {f->mu_s, f->X0_s, f->exxd_s, f->ezzd_s, f->exz, f->sxxd0_s, f->szzd0_s, f->sxz0,
                                 f->fric_s, f->C_s, f->dil_s, f->p0_s, f->bet_s, f->d1_s, f->d2_s, f->angle_s,
                                 f->aniso_factor_s};
  L.nci = aniso ? CI_COUNT : CI_d1;
  L.nvi = aniso ? VI_COUNT : VI_d1;
  for (int i = 0; i < CI_COUNT; i++) L.cin[i] = (i < L.nci) ? cin[i] : nullptr;
  for (int i = 0; i < VI_COUNT; i++) L.vin[i] = (i < L.nvi) ? vin[i] : nullptr;
  for (int i = 0; i < L.nci; i++) if (!L.cin[i]) return MDZ_EINVAL;
  for (int i = 0; i < L.nvi; i++) if (!L.vin[i]) return MDZ_EINVAL;
  if (!f->phase_perc_n || !f->phase_perc_s || !f->phase_eta_n || !f->phase_eta_s || !f->BCp_type || !f->BCg_type)
    return MDZ_EINVAL;
  double *cout[CO_COUNT] = {f->eta_n, f->eta_phys_n, f->VE_n, f->sxxd, f->szzd, f->sxz_n, f->eII_el, f->eII_pl,
                            f->eII_pwl, f->eII_exp, f->eII_lin, f->eII_gbs, f->eII_cst, f->d_n, f->p_corr,
                            f->div_u_el, f->div_u_pl, f->div_u_r, f->Wtot, f->Wel, f->Wdiss, f->X_n, f->OverS_n,
                            md->density_variations == 1 ? f->rho_n : nullptr};
  for (int i = 0; i < CO_rho; i++) if (!cout[i]) return MDZ_EINVAL;
  if (md->density_variations == 1 && !f->rho_n) return MDZ_EINVAL;
  double *vout[VO_COUNT] = {f->sxxd_s, f->szzd_s, f->sxz, f->eta_phys_s, f->eta_s, f->X_s,
                            aniso ? f->VE_s : nullptr, f->T_s, f->P_s, f->d0_s, f->phi0_s};
  for (int i = 0; i < VO_COUNT; i++) if (i != VO_VE && !vout[i]) return MDZ_EINVAL;
  if (aniso && !f->VE_s) return MDZ_EINVAL;
  for (int i = 0; i < CO_COUNT; i++) L.cout[i] = cout[i];
  for (int i = 0; i < VO_COUNT; i++) L.vout[i] = vout[i];
  return MDZ_OK;
}

constexpr int kMaxBands = 16;

int host_bands(const mdz_rheo_ctx *ctx, int Nz) {
  int b = ctx->bands > 0 ? ctx->bands : Nz / 128;
  if (b > kMaxBands) b = kMaxBands;
  if (b > Nz) b = Nz;
  return b < 1 ? 1 : b;
}

// Row boundaries of B bands over Nz vertex rows: band sizes in the ratio
// min(2^b, 2^(B-1-b), 8), so the first band's upload (before any kernel) and the last
// band's download (after every kernel) are short, and each band's upload stays shorter
// than the kernel before it while the bands grow; at least one row per band.
void band_rows(int Nz, int B, int *a) {
  double cum[kMaxBands + 1];
  cum[0] = 0.0;
  for (int b = 0; b < B; b++) {
    const int up = b < 3 ? b : 3, down = (B - 1 - b) < 3 ? (B - 1 - b) : 3;
    cum[b + 1] = cum[b] + (double)(1 << (up < down ? up : down));
  }
  a[0] = 0;
  for (int b = 1; b < B; b++) {
    long long r = llround(cum[b] / cum[B] * Nz);
    if (r < a[b - 1] + 1) r = a[b - 1] + 1;
    if (r > Nz - (B - b)) r = Nz - (B - b);
    a[b] = (int)r;
  }
  a[B] = Nz;
}

// A sweep of host arrays in B bands of vertex rows [a_b, a_{b+1}) with the centroid rows
// of the same indices.  Band b's inputs go up on copy_in; its kernel waits for them, on
// the context stream for even b and on a second stream for odd b (a band's kernel fills
// the SMs its predecessor's tail leaves idle); its outputs come back on copy_out once the
// kernel is done.  The copies of one band thus overlap the kernels of the others.  A
// vertex row l reads the centroid rows l - 1 and l, which bands up to b have uploaded by
// then (copy_in runs in order), and every node writes only its own outputs.
LaunchShape pick_shape(const mdz_rheo_ctx *ctx, bool aniso, int np, bool ref, long long nodes) {
  const mdz_rheo_ctx::Tuned *best = nullptr;
  double best_d = 1e300;
  for (const auto &t : ctx->tuned) {
    if (t.aniso != (int)aniso || t.np != np || t.ref != (int)ref) continue;
    const double d = fabs(log((double)t.nodes / (double)(nodes > 0 ? nodes : 1)));
    if (d < best_d) { best_d = d; best = &t; }
  }
  return best ? best->shape : ctx->shape[aniso ? 1 : 0];
}

int banded_sweep(mdz_rheo_ctx *ctx, SweepArgs &A, bool aniso, const FieldLists &L, const mdz_grid_fields *f,
                 int B) {
  const int Nx = A.M.Nx, Nz = A.M.Nz, Ncx = A.M.Ncx, Ncz = A.M.Ncz, np = A.M.np;
  const size_t Nc = (size_t)A.M.Nc, Nv = (size_t)A.M.Nv;
  if (!ctx->copy_in) {
    CK(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->compute2, cudaStreamNonBlocking));
    for (cudaEvent_t &e : ctx->band_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  int rows[kMaxBands + 1];
  band_rows(Nz, B, rows);
  // device arrays, full size, in the same slots as the one-shot path
  auto slot = [&](int s, size_t bytes) -> void * {
    return ensure(ctx->bufs[s], bytes) == MDZ_OK ? ctx->bufs[s].p : nullptr;
  };
  bool ok = true;
  for (int i = 0; i < L.nci; i++) ok = ok && (A.ci[i] = (const double *)slot(S_CI + i, Nc * 8));
  for (int i = 0; i < L.nvi; i++) ok = ok && (A.vi[i] = (const double *)slot(S_VI + i, Nv * 8));
  for (int p = 0; p < np; p++) {
    ok = ok && (A.perc_n[p] = (const double *)slot(S_PN + p, Nc * 8)) && (A.perc_s[p] = (const double *)slot(S_PS + p, Nv * 8));
    ok = ok && (A.peta_n[p] = (double *)slot(S_EN + p, Nc * 8)) && (A.peta_s[p] = (double *)slot(S_ES + p, Nv * 8));
  }
  ok = ok && (A.bcp = (const signed char *)slot(S_BCP, Nc)) && (A.bcg = (const signed char *)slot(S_BCG, Nv));
  for (int i = 0; i < CO_COUNT; i++) A.co[i] = L.cout[i] ? (double *)slot(S_CO + i, Nc * 8) : nullptr;
  for (int i = 0; i < VO_COUNT; i++) A.vo[i] = L.vout[i] ? (double *)slot(S_VO + i, Nv * 8) : nullptr;
  for (int i = 0; i < CO_COUNT; i++) ok = ok && (!L.cout[i] || A.co[i]);
  for (int i = 0; i < VO_COUNT; i++) ok = ok && (!L.vout[i] || A.vo[i]);
  if (!ok) return MDZ_ENOMEM;
  // [0] start, [1 + b] band b uploaded, [1 + B + b] band b swept, [1 + 2B] downloads
  // done, [2 + 2B] kernels of the second stream done
  cudaEvent_t *ev = ctx->band_ev;
  auto up = [&](const void *dst, const void *src, size_t off, size_t n, size_t es) -> cudaError_t {
    if (!src || !n) return cudaSuccess;
    ctx->h2d += n * es;
    return cudaMemcpyAsync((char *)dst + off * es, (const char *)src + off * es, n * es, cudaMemcpyHostToDevice,
                           ctx->copy_in);
  };
  auto down = [&](void *dst, const void *src, size_t off, size_t n, size_t es) -> cudaError_t {
    if (!dst || !n) return cudaSuccess;
    ctx->d2h += n * es;
    return cudaMemcpyAsync((char *)dst + off * es, (const char *)src + off * es, n * es, cudaMemcpyDeviceToHost,
                           ctx->copy_out);
  };
  CK(cudaEventRecord(ev[0], ctx->stream));  // earlier work on these buffers comes first
  CK(cudaStreamWaitEvent(ctx->copy_in, ev[0], 0));
  CK(cudaStreamWaitEvent(ctx->copy_out, ev[0], 0));
  for (int b = 0; b < B; b++) {
    const int vr0 = rows[b], vr1 = rows[b + 1];
    const int cr0 = vr0 < Ncz ? vr0 : Ncz, cr1 = vr1 < Ncz ? vr1 : Ncz;
    const size_t coff = (size_t)cr0 * Ncx, cn = (size_t)(cr1 - cr0) * Ncx;
    const size_t voff = (size_t)vr0 * Nx, vn = (size_t)(vr1 - vr0) * Nx;
    for (int i = 0; i < L.nci; i++) CK(up(A.ci[i], L.cin[i], coff, cn, 8));
    for (int i = 0; i < L.nvi; i++) CK(up(A.vi[i], L.vin[i], voff, vn, 8));
    for (int p = 0; p < np; p++) {
      CK(up(A.perc_n[p], f->phase_perc_n[p], coff, cn, 8));
      CK(up(A.perc_s[p], f->phase_perc_s[p], voff, vn, 8));
      CK(up(A.peta_n[p], f->phase_eta_n[p], coff, cn, 8));
      CK(up(A.peta_s[p], f->phase_eta_s[p], voff, vn, 8));
    }
    CK(up(A.bcp, f->BCp_type, coff, cn, 1));
    CK(up(A.bcg, f->BCg_type, voff, vn, 1));
    CK(cudaEventRecord(ev[1 + b], ctx->copy_in));
    cudaStream_t ks = (b & 1) ? ctx->compute2 : ctx->stream;
    CK(cudaStreamWaitEvent(ks, ev[1 + b], 0));
    if (b == 0) CK(cudaEventRecord(ctx->ev0, ks));
    A.ranged = 1;
    A.c_lo = (long long)coff; A.c_n = (long long)cn; A.v_lo = (long long)voff; A.v_n = (long long)vn;
    CK(launch_sweep(A, aniso, ks, pick_shape(ctx, aniso, A.M.np, A.polish == 0, A.M.Nc + A.M.Nv)));
    ctx->launches += sweep_kernel_count(A);
    CK(cudaEventRecord(ev[1 + B + b], ks));
    CK(cudaStreamWaitEvent(ctx->copy_out, ev[1 + B + b], 0));
    for (int i = 0; i < CO_COUNT; i++) CK(down(L.cout[i], A.co[i], coff, cn, 8));
    for (int i = 0; i < VO_COUNT; i++) CK(down(L.vout[i], A.vo[i], voff, vn, 8));
    for (int p = 0; p < np; p++) {
      CK(down(f->phase_eta_n[p], A.peta_n[p], coff, cn, 8));
      CK(down(f->phase_eta_s[p], A.peta_s[p], voff, vn, 8));
    }
  }
  A.ranged = 0;
  CK(cudaEventRecord(ev[2 + 2 * B], ctx->compute2));
  CK(cudaStreamWaitEvent(ctx->stream, ev[2 + 2 * B], 0));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventRecord(ev[1 + 2 * B], ctx->copy_out));
  CK(cudaStreamWaitEvent(ctx->stream, ev[1 + 2 * B], 0));
  return MDZ_OK;
}

// Whether the current device reads and writes pageable host memory (malloc, new, mmap)
// through the host's page tables, as the GPU of a Grace-Blackwell system does over its
// coherent NVLink-C2C link (cudaDevAttrPageableMemoryAccessUsesHostPageTables); cached per
// device.
bool pageable_in_place() {
  static std::atomic<int> cached[64];  // 0: not asked yet, 1: no, 2: yes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return false;
  }
  int v = cached[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    int a = 0, b = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) a = 0;
    if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) b = 0;
    cudaGetLastError();
    v = (a == 1 && b == 1) ? 2 : 1;
    cached[dev].store(v, std::memory_order_relaxed);
  }
  return v == 2;
}

// Host arrays the kernels can address directly, checked at the array's first and last
// byte: page-locked memory mapped into the device's address space at the same address
// (cudaHostAlloc, cudaMallocHost, or cudaHostRegister of the whole array), and, where the
// device reads pageable memory through the host page tables, ordinary pageable memory.  On
// a Grace-Blackwell system the host link is coherent and fast enough that the sweep reads
// its inputs and writes its outputs there during the kernels at nearly the speed of device
// memory (the kernels are bound by the FP64 pipe), with no staging copies.
bool host_mapped(const void *p, size_t bytes) {
  if (!p || !bytes) return true;
  const void *ends[2] = {p, (const char *)p + (bytes - 1)};
  for (const void *q : ends) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer == q) continue;
    if (a.type == cudaMemoryTypeUnregistered && pageable_in_place()) continue;
    return false;
  }
  return true;
}

// Every array of a host-memory sweep addressable by the kernels (host_mapped); the bytes
// the kernels then read from and write to host memory go into the context's counters.
bool sweep_arrays_mapped(mdz_rheo_ctx *ctx, const FieldLists &L, const mdz_grid_fields *f, int np, size_t Nc,
                         size_t Nv) {
  size_t in = 0, out = 0;
  for (int i = 0; i < L.nci; i++) { if (!host_mapped(L.cin[i], Nc * 8)) return false; in += L.cin[i] ? Nc * 8 : 0; }
  for (int i = 0; i < L.nvi; i++) { if (!host_mapped(L.vin[i], Nv * 8)) return false; in += L.vin[i] ? Nv * 8 : 0; }
  for (int i = 0; i < CO_COUNT; i++) { if (!host_mapped(L.cout[i], Nc * 8)) return false; out += L.cout[i] ? Nc * 8 : 0; }
  for (int i = 0; i < VO_COUNT; i++) { if (!host_mapped(L.vout[i], Nv * 8)) return false; out += L.vout[i] ? Nv * 8 : 0; }
  for (int p = 0; p < np; p++) {
    if (!host_mapped(f->phase_perc_n[p], Nc * 8) || !host_mapped(f->phase_perc_s[p], Nv * 8) ||
        !host_mapped(f->phase_eta_n[p], Nc * 8) || !host_mapped(f->phase_eta_s[p], Nv * 8))
      return false;
    in += 2 * (Nc + Nv) * 8;  // fractions, and the previous phase viscosities that inactive phases keep
    out += (Nc + Nv) * 8;
  }
  if (!host_mapped(f->BCp_type, Nc) || !host_mapped(f->BCg_type, Nv)) return false;
  in += Nc + Nv;
  ctx->h2d += in;
  ctx->d2h += out;
  return true;
}

int sweep_impl(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_materials *mat, const mdz_grid_fields *f,
               int final_update, int mem, int flags, mdz_sweep_stats *st, bool aniso, float *X = nullptr,
               float *Y = nullptr) {
  if (!ctx || !md || !mat || !f) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_ASYNC) && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_WARMSTART) && !ctx->warm_ready) return MDZ_ENOTREADY;
  if ((flags & MDZ_SWEEP_WARMSTART) && ctx->warm.n_feat != (aniso ? kFeatAniso : kFeatIso)) return MDZ_EINVAL;
  const bool collect = (X != nullptr);
  int mode = -1;  // plain
  if (collect) mode = MODE_COLLECT;
  else if (flags & MDZ_SWEEP_WARMSTART) mode = MODE_WARM;
  if (md->Nx < 2 || md->Nz < 2) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  static thread_local SweepArgs A;  // large: keep off the stack
  memset(&A, 0, sizeof(A));
  int rc = fold_model(md, mat, A.M);
  if (rc != MDZ_OK) return rc;
  for (int p = 0; p < A.M.np; p++) fold_phase(mat, md, p, A.ph[p]);
  A.final_update = final_update;
  A.need_lnd = need_lnd(mat, A.M.np);
  A.polish = (flags & MDZ_SWEEP_REF_START) ? 0 : ctx->polish_iters;
  const size_t Nc = (size_t)A.M.Nc, Nv = (size_t)A.M.Nv;
  const int np = A.M.np;
  const bool host_mem = (mem == MDZ_MEM_HOST);
  FieldLists L;
  if ((rc = field_lists(md, f, aniso, L)) != MDZ_OK) return rc;
  const double *const *cin = L.cin, *const *vin = L.vin;
  double *const *cout = L.cout, *const *vout = L.vout;
  const int nci = L.nci, nvi = L.nvi;

  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  // host arrays the kernels can address in place need no staging copies
  const bool direct = host_mem && !(flags & MDZ_SWEEP_STAGED) && sweep_arrays_mapped(ctx, L, f, np, Nc, Nv);
  const bool host = host_mem && !direct;  // staged through device mirrors
  const int bands = (host && mode < 0 && !(flags & MDZ_SWEEP_ITERS)) ? host_bands(ctx, md->Nz) : 1;
  if (bands > 1) {
    A.stats = ctx->d_stats;
    if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
    if ((rc = banded_sweep(ctx, A, aniso, L, f, bands)) != MDZ_OK) return rc;
    return finish(ctx, st);
  }
  Mirror mi{ctx};
  for (int i = 0; i < nci; i++) A.ci[i] = mi.in(cin[i], S_CI + i, Nc, host);
  for (int i = 0; i < nvi; i++) A.vi[i] = mi.in(vin[i], S_VI + i, Nv, host);
  for (int p = 0; p < np; p++) {
    A.perc_n[p] = mi.in(f->phase_perc_n[p], S_PN + p, Nc, host);
    A.perc_s[p] = mi.in(f->phase_perc_s[p], S_PS + p, Nv, host);
    // phase_eta of inactive phases keeps its previous value, as in the reference
    A.peta_n[p] = (double *)mi.in((const double *)f->phase_eta_n[p], S_EN + p, Nc, host);
    A.peta_s[p] = (double *)mi.in((const double *)f->phase_eta_s[p], S_ES + p, Nv, host);
  }
  A.bcp = mi.in(f->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(f->BCg_type, S_BCG, Nv, host);
  for (int i = 0; i < CO_COUNT; i++) A.co[i] = mi.out(cout[i], S_CO + i, Nc, host);
  for (int i = 0; i < VO_COUNT; i++) A.vo[i] = mi.out(vout[i], S_VO + i, Nv, host);
  if (mi.err) return mi.err;
  if (flags & MDZ_SWEEP_ITERS) {
    const size_t bn = Nc * np * sizeof(int32_t), bs = Nv * np * sizeof(int32_t);
    if (ctx->cap_iters_n < bn) {
      cudaFree(ctx->d_iters_n);
      ctx->d_iters_n = nullptr; ctx->cap_iters_n = 0;
      CK(cudaMalloc(&ctx->d_iters_n, bn));
      ctx->cap_iters_n = bn;
    }
    if (ctx->cap_iters_s < bs) {
      cudaFree(ctx->d_iters_s);
      ctx->d_iters_s = nullptr; ctx->cap_iters_s = 0;
      CK(cudaMalloc(&ctx->d_iters_s, bs));
      ctx->cap_iters_s = bs;
    }
    A.iters_n = ctx->d_iters_n; A.iters_s = ctx->d_iters_s;
    ctx->have_iters = 1;
    ctx->last_Nc = A.M.Nc; ctx->last_Nv = A.M.Nv; ctx->last_np = np;
  }
  A.stats = ctx->d_stats;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  // collected features / targets (device scratch when the caller's buffers are on the host)
  const size_t items = (size_t)np * (Nc + Nv);
  float *dX = X, *dY = Y;
  struct Scratch {  // freed on every return path
    DevBuf b;
    ~Scratch() { if (b.p) cudaFree(b.p); }
  } tmpX, tmpY;
  if (collect && host_mem) {
    if (ensure(tmpX.b, items * kMlpIn * sizeof(float)) != MDZ_OK || ensure(tmpY.b, items * 2 * sizeof(float)) != MDZ_OK)
      return MDZ_ENOMEM;
    dX = (float *)tmpX.b.p;
    dY = (float *)tmpY.b.p;
  }
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (mode < 0) {
    CK(launch_sweep(A, aniso, ctx->stream,
                    pick_shape(ctx, aniso, A.M.np, A.polish == 0, A.M.Nc + A.M.Nv)));
  } else if (mode == MODE_WARM && !(flags & MDZ_SWEEP_WARM_TILES)) {
    MlpDevice w = ctx->warm;
    w.polish_iters = ctx->polish_iters;
    CK(launch_sweep_warm(A, w, aniso, ctx->stream));
  } else {
    WarmArgs W;
    memset(&W, 0, sizeof(W));
    W.mlp = ctx->warm;
    W.mlp.polish_iters = ctx->polish_iters;
    W.mlp.poll_limit = ctx->mma_poll_limit;
    W.X_out = dX;
    W.Y_out = dY;
    const int grid = ctx->sms * tiles_blocks_per_sm(aniso, mode);
    CK(launch_sweep_tiles(A, W, aniso, mode, ctx->stream, grid));
  }
  ctx->launches += sweep_kernel_count(A);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if (collect && host_mem) {
    CK(cudaMemcpyAsync(X, dX, items * kMlpIn * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(Y, dY, items * 2 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  for (int i = 0; i < CO_COUNT; i++) mi.back(cout[i], S_CO + i, Nc, host);
  for (int i = 0; i < VO_COUNT; i++) mi.back(vout[i], S_VO + i, Nv, host);
  for (int p = 0; p < np; p++) {
    mi.back(f->phase_eta_n[p], S_EN + p, Nc, host);
    mi.back(f->phase_eta_s[p], S_ES + p, Nv, host);
  }
  if (mi.err) return mi.err;
  if (flags & MDZ_SWEEP_ASYNC) {
    ctx->pending = 1;
    return MDZ_OK;
  }
  return finish(ctx, st);
}


// ---------------------------------------------------------------------------------
// input preparation: Softening over the grid, ShearModCompExpGrid (helpers)
// ---------------------------------------------------------------------------------

// the per-phase constants of Softening, by the reference's own expressions
// (RheologyDensity.c:1448-1470, :1493-1497)
void fold_soft(const mdz_prep_materials *m, int p, SoftPhase &P) {
  P.phi = m->phi[p]; P.psi = m->psi[p]; P.C = m->C[p];
  P.phi_end = m->phi_end[p]; P.psi_end = m->psi_end[p]; P.C_end = m->C_end[p];
  P.pls_start = m->pls_start[p]; P.pls_end = m->pls_end[p]; P.Hc = m->H_c[p];
  P.key_start = order_key_host(m->pls_start[p]); P.key_end = order_key_host(m->pls_end[p]);
  P.start_nan = is_nan_host(m->pls_start[p]); P.end_nan = is_nan_host(m->pls_end[p]);
  P.phi_soft = m->phi_soft[p]; P.psi_soft = m->psi_soft[p]; P.coh_soft = m->coh_soft[p];
  const double dstrain = m->pls_end[p] - m->pls_start[p];
  P.q_phi = (m->phi_end[p] - m->phi[p]) / dstrain;
  P.q_psi = (m->psi_end[p] - m->psi[p]) / dstrain;
  P.q_C = (m->C_end[p] - m->C[p]) / dstrain;
  P.mu_strain = 0.5 * (m->pls_end[p] + m->pls_start[p]);
  P.dstrain = make_divisor(dstrain);
  const double e0 = erfc(-(0.0 - P.mu_strain) / dstrain);
  const double x[3] = {m->phi[p], m->psi[p], m->C[p]}, xe[3] = {m->phi_end[p], m->psi_end[p], m->C_end[p]};
  for (int k = 0; k < 3; k++) {
    const double d = x[k] - xe[k];
    const double half = d / 2.0;
    const double t = half * e0;
    const double x0 = (x[k] - t) - xe[k];
    P.d[k] = d; P.half_d[k] = half; P.x_end_[k] = xe[k];
    P.x0[k] = make_divisor(x0);
  }
}

bool prep_common(const mdz_model *md, const mdz_prep_materials *mat, const mdz_prep_fields *f, int mem, int flags) {
  if (!md || !mat || !f) return false;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return false;
  if (flags & ~(MDZ_SWEEP_ASYNC | MDZ_SWEEP_STAGED)) return false;
  if ((flags & MDZ_SWEEP_ASYNC) && mem != MDZ_MEM_DEVICE) return false;
  if (md->Nx < 2 || md->Nz < 2 || md->Nb_phases < 1 || md->Nb_phases > MDZ_MAX_PHASES) return false;
  if (!f->phase_perc_n || !f->phase_perc_s || !f->BCp_type || !f->BCg_type) return false;
  for (int p = 0; p < md->Nb_phases; p++) if (!f->phase_perc_n[p] || !f->phase_perc_s[p]) return false;
  return true;
}

int prep_finish(mdz_rheo_ctx *ctx, int flags, mdz_sweep_stats *st) {
  if (flags & MDZ_SWEEP_ASYNC) {
    ctx->pending = 1;
    return MDZ_OK;
  }
  return finish(ctx, st);
}

// ---------------------------------------------------------------------------------
// static scratch of mdz_rheo_points_static: one array per device, its address looked
// up once per device; the lock serialises the calls that share it
// ---------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_points_scratch[MDZ_STATIC_SCRATCH_BYTES];
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
void *g_static_addr[kStaticMaxDevices] = {};

// ---------------------------------------------------------------------------------
// learned warm start: host-side packing of the BF16 K-major tiles (umma.cuh layout)
// ---------------------------------------------------------------------------------
uint16_t f2bf(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

size_t kmajor_off(int r, int k, int K) {
  return (size_t)((r >> 3) * (16 * K) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// tile[rows_alloc x K] with tile(r, k) = W[r * ldw + k] (or W[k * ldw + r] if transposed)
void pack_tile(uint8_t *tile, int rows_alloc, int K, const float *W, int rows_used, int k_used, int ldw, bool tr) {
  memset(tile, 0, (size_t)rows_alloc * K * 2);
  for (int r = 0; r < rows_used; r++)
    for (int k = 0; k < k_used; k++) {
      const uint16_t b = f2bf(tr ? W[(size_t)k * ldw + r] : W[(size_t)r * ldw + k]);
      memcpy(tile + kmajor_off(r, k, K), &b, 2);
    }
}

constexpr size_t kT1 = kMlpHid * kMlpIn * 2, kT2 = kMlpHid * kMlpHid * 2, kT3 = kMlpOut * kMlpHid * 2;

// The B operands of the per-warp MMA (mma.sync m16n8k16, mlp_warp.cuh) in fragment order:
// entry (j * KC + c) * 32 + lane, lane = 4 g + t, holds the BF16 pairs
// (W[n][k], W[n][k + 1]) and (W[n][k + 8], W[n][k + 9]) with n = 8 j + g, k = 16 c + 2 t,
// W row-major [out][in] with `ldw` columns (zero beyond rows_used x k_used).
void pack_frags(uint32_t *dst, const float *W, int NT, int KC, int rows_used, int k_used, int ldw) {
  for (int j = 0; j < NT; j++)
    for (int c = 0; c < KC; c++)
      for (int lane = 0; lane < 32; lane++) {
        const int n = 8 * j + (lane >> 2), k = 16 * c + 2 * (lane & 3);
        auto el = [&](int kk) -> uint32_t {
          return (n < rows_used && kk < k_used) ? (uint32_t)f2bf(W[(size_t)n * ldw + kk]) : 0u;
        };
        uint32_t *o = dst + 2 * ((j * KC + c) * 32 + lane);
        o[0] = el(k) | (el(k + 1) << 16);
        o[1] = el(k + 8) | (el(k + 9) << 16);
      }
}

constexpr size_t kFB1 = (size_t)kF1 * 8, kFB2 = (size_t)kF2 * 8, kFB3 = (size_t)kF3 * 8;

int upload_warm(mdz_rheo_ctx *c, const mdz_mlp_weights *w) {
  const size_t fbytes = kFB1 + kFB2 + kFB3;
  const size_t bytes = kT1 + kT2 + kT3 + (64 + 64 + 16) * sizeof(float) + fbytes;
  if (!c->warm_buf) CK(cudaMalloc(&c->warm_buf, bytes));
  std::vector<uint8_t> h(bytes, 0);
  pack_tile(h.data(), kMlpHid, kMlpIn, w->W1, kMlpHid, w->n_feat, MDZ_MLP_IN, false);
  pack_tile(h.data() + kT1, kMlpHid, kMlpHid, w->W2, kMlpHid, kMlpHid, MDZ_MLP_HID, false);
  pack_tile(h.data() + kT1 + kT2, kMlpOut, kMlpHid, w->W3, 2, kMlpHid, MDZ_MLP_HID, false);
  float *b = (float *)(h.data() + kT1 + kT2 + kT3);
  memcpy(b, w->b1, 64 * sizeof(float));
  memcpy(b + 64, w->b2, 64 * sizeof(float));
  b[128] = w->b3[0];
  b[129] = w->b3[1];
  uint8_t *fr = h.data() + kT1 + kT2 + kT3 + (64 + 64 + 16) * sizeof(float);
  pack_frags((uint32_t *)fr, w->W1, 8, 1, kMlpHid, w->n_feat, MDZ_MLP_IN);
  pack_frags((uint32_t *)(fr + kFB1), w->W2, 8, 4, kMlpHid, kMlpHid, MDZ_MLP_HID);
  pack_frags((uint32_t *)(fr + kFB1 + kFB2), w->W3, 1, 4, 2, kMlpHid, MDZ_MLP_HID);
  CK(cudaMemcpy(c->warm_buf, h.data(), bytes, cudaMemcpyHostToDevice));
  uint8_t *d = (uint8_t *)c->warm_buf;
  c->warm.W1 = (const uint4 *)d;
  c->warm.W2 = (const uint4 *)(d + kT1);
  c->warm.W3 = (const uint4 *)(d + kT1 + kT2);
  const float *db = (const float *)(d + kT1 + kT2 + kT3);
  c->warm.b1 = db; c->warm.b2 = db + 64; c->warm.b3 = db + 128;
  const uint8_t *df = d + kT1 + kT2 + kT3 + (64 + 64 + 16) * sizeof(float);
  c->warm.F1 = (const uint2 *)df;
  c->warm.F2 = (const uint2 *)(df + kFB1);
  c->warm.F3 = (const uint2 *)(df + kFB1 + kFB2);
  for (int j = 0; j < kMlpIn; j++) { c->warm.x_shift[j] = w->x_shift[j]; c->warm.x_scale[j] = w->x_scale[j]; }
  c->warm.z_shift = w->z_shift;
  c->warm.z_scale = w->z_scale;
  c->warm.n_feat = w->n_feat;
  return MDZ_OK;
}

// Device state of one training run, in one allocation.
struct TrainBuffers {
  void *mem = nullptr;
  MlpTrainState S{};
  ~TrainBuffers() { if (mem) cudaFree(mem); }
};

constexpr int kP1 = kMlpHid * kMlpIn, kP2 = kMlpHid * kMlpHid, kP3 = 2 * kMlpHid;

int alloc_train(TrainBuffers &B) {
  const int P = kP1 + kP2 + kP3 + 64 + 64 + 16;
  const size_t fbytes = (size_t)P * 4 * sizeof(float);
  const size_t tbytes = kT1 + kT2 + kT3 + kT2 + kMlpHid * kMlpOut * 2;
  CK(cudaMalloc(&B.mem, fbytes + tbytes + 64));
  CK(cudaMemset(B.mem, 0, fbytes + tbytes + 64));
  float *f = (float *)B.mem;
  float **slots[4][6] = {{&B.S.W1, &B.S.W2, &B.S.W3, &B.S.b1, &B.S.b2, &B.S.b3},
                         {&B.S.mW1, &B.S.mW2, &B.S.mW3, &B.S.mb1, &B.S.mb2, &B.S.mb3},
                         {&B.S.vW1, &B.S.vW2, &B.S.vW3, &B.S.vb1, &B.S.vb2, &B.S.vb3},
                         {&B.S.gW1, &B.S.gW2, &B.S.gW3, &B.S.gb1, &B.S.gb2, &B.S.gb3}};
  const int sizes[6] = {kP1, kP2, kP3, 64, 64, 16};
  for (int g = 0; g < 4; g++)
    for (int i = 0; i < 6; i++) { *slots[g][i] = f; f += sizes[i]; }
  uint8_t *t = (uint8_t *)f;
  B.S.tW1 = (uint4 *)t; t += kT1;
  B.S.tW2 = (uint4 *)t; t += kT2;
  B.S.tW3 = (uint4 *)t; t += kT3;
  B.S.tW2t = (uint4 *)t; t += kT2;
  B.S.tW3t = (uint4 *)t; t += kMlpHid * kMlpOut * 2;
  B.S.loss = (float *)t;
  B.S.fault = (int *)(t + 16);
  return MDZ_OK;
}

int put_weights(TrainBuffers &B, const mdz_mlp_weights *w) {
  CK(cudaMemcpy(B.S.W1, w->W1, kP1 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.S.W2, w->W2, kP2 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.S.W3, w->W3, kP3 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.S.b1, w->b1, 64 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.S.b2, w->b2, 64 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.S.b3, w->b3, 2 * sizeof(float), cudaMemcpyHostToDevice));
  for (int j = 0; j < kMlpIn; j++) { B.S.x_shift[j] = w->x_shift[j]; B.S.x_scale[j] = w->x_scale[j]; }
  B.S.z_shift = w->z_shift;
  B.S.z_scale = w->z_scale;
  return MDZ_OK;
}

int get_weights(const TrainBuffers &B, mdz_mlp_weights *w) {
  CK(cudaMemcpy(w->W1, B.S.W1, kP1 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(w->W2, B.S.W2, kP2 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(w->W3, B.S.W3, kP3 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(w->b1, B.S.b1, 64 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(w->b2, B.S.b2, 64 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(w->b3, B.S.b3, 2 * sizeof(float), cudaMemcpyDeviceToHost));
  return MDZ_OK;
}

// Seeded initialisation (He-uniform for the hidden layers, small output layer) and
// feature / target normalisation from the data (finite targets only).
void init_weights(mdz_mlp_weights *w, const float *X, const float *Y, int64_t n, int n_feat, uint64_t seed) {
  std::mt19937_64 rng(seed);
  memset(w, 0, sizeof(*w));
  w->n_feat = n_feat;
  auto uni = [&](float a) { return (float)((double)rng() / 18446744073709551616.0 * 2.0 - 1.0) * a; };
  for (int h = 0; h < kMlpHid; h++)
    for (int f = 0; f < n_feat; f++) w->W1[h * kMlpIn + f] = uni(sqrtf(6.0f / n_feat));
  for (int i = 0; i < kP2; i++) w->W2[i] = uni(sqrtf(6.0f / kMlpHid));
  for (int i = 0; i < kP3; i++) w->W3[i] = uni(0.1f * sqrtf(6.0f / kMlpHid));
  std::vector<double> s(kMlpIn, 0.0), s2(kMlpIn, 0.0);
  double zs = 0.0, zs2 = 0.0;
  int64_t cnt = 0;
  for (int64_t i = 0; i < n; i++) {
    const float z = Y[i * 2];
    if (!std::isfinite(z)) continue;
    cnt++;
    zs += z; zs2 += (double)z * z;
    for (int f = 0; f < n_feat; f++) { const double x = X[i * kMlpIn + f]; s[f] += x; s2[f] += x * x; }
  }
  const double c = cnt > 0 ? (double)cnt : 1.0;
  for (int f = 0; f < kMlpIn; f++) {
    const double m = s[f] / c, v = s2[f] / c - m * m;
    w->x_shift[f] = (float)m;
    w->x_scale[f] = (f < n_feat && v > 1e-20) ? (float)(1.0 / sqrt(v)) : 0.0f;
  }
  const double zm = zs / c, zv = zs2 / c - zm * zm;
  w->z_shift = (float)zm;
  w->z_scale = (float)(zv > 1e-20 ? sqrt(zv) : 1.0);
}

}  // namespace

extern "C" {

int mdz_rheo_version(void) { return MDZ_RHEO_ABI_VERSION; }

void mdz_rheo_abi_sizes(size_t out[8]) {
  out[0] = sizeof(mdz_materials); out[1] = sizeof(mdz_model); out[2] = sizeof(mdz_grid_fields);
  out[3] = sizeof(mdz_sweep_stats); out[4] = sizeof(mdz_point_inputs); out[5] = sizeof(mdz_point_outputs);
  out[6] = 0; out[7] = 0;
}

const char *mdz_rheo_status_string(int s) {
  switch (s) {
    case MDZ_OK: return "ok";
    case MDZ_EINVAL: return "invalid argument";
    case MDZ_ECUDA: return "CUDA error";
    case MDZ_EUNSUPPORTED: return "unsupported option (melting, chemical production, tabulated density)";
    case MDZ_ENOMEM: return "out of device memory";
    case MDZ_ENOTREADY: return "not ready (warm start without weights?)";
    case MDZ_EVE_ITER: return "Visco-Elastic iterations failed!";
    case MDZ_EGSE_ITER: return "GSE local iter failed to converge";
    case MDZ_ESINGULAR: return "Singular Jacobian in Newton local solve";
    case MDZ_EEMPTY_CELL: return "Cell went empty";
    case MDZ_ENONFINITE: return "Inf/NaN viscosity";
    case MDZ_EWDISS: return "negative dissipation";
    case MDZ_EGRAIN_ZERO: return "grain size dependent viscosity with zero grain size";
    case MDZ_ELINESEARCH: return "tensile plasticity line search failed (alpha < 0.01)";
    case MDZ_EANISO_NAN: return "anisotropic VE residual is NaN";
    case MDZ_EANISO_ITER: return "anisotropic Visco-Elastic iterations failed";
    case MDZ_ESCRATCH: return "request larger than the static scratch (MDZ_STATIC_SCRATCH_BYTES)";
    case MDZ_ESHEAR_INF: return "infinite shear modulus at a cell centre";
    case MDZ_EMARKER_OUT: return "marker beyond the grid";
    default: return "unknown status";
  }
}

int mdz_rheo_create(int device, mdz_rheo_ctx **out) {
  if (!out) return MDZ_EINVAL;
  *out = nullptr;
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return MDZ_EINVAL;
  CK(cudaSetDevice(device));
  mdz_rheo_ctx *c = new mdz_rheo_ctx();
  c->device = device;
  c->bufs.resize(S_COUNT);
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaMalloc(&c->d_stats, sizeof(DevStats)) != cudaSuccess ||
      cudaMallocHost(&c->h_stats, sizeof(DevStats)) != cudaSuccess) {
    mdz_rheo_destroy(c);
    return MDZ_ECUDA;
  }
  c->stream = c->own;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return MDZ_OK;
}

int mdz_rheo_destroy(mdz_rheo_ctx *c) {
  if (!c) return MDZ_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto &b : c->bufs) if (b.p) cudaFree(b.p);
  if (c->d_iters_n) cudaFree(c->d_iters_n);
  if (c->d_iters_s) cudaFree(c->d_iters_s);
  if (c->d_stats) cudaFree(c->d_stats);
  if (c->warm_buf) cudaFree(c->warm_buf);
  if (c->h_stats) cudaFreeHost(c->h_stats);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t e : c->band_ev) if (e) cudaEventDestroy(e);
  if (c->copy_in) { cudaStreamSynchronize(c->copy_in); cudaStreamDestroy(c->copy_in); }
  if (c->copy_out) { cudaStreamSynchronize(c->copy_out); cudaStreamDestroy(c->copy_out); }
  if (c->compute2) { cudaStreamSynchronize(c->compute2); cudaStreamDestroy(c->compute2); }
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return MDZ_OK;
}

int mdz_rheo_set_host_bands(mdz_rheo_ctx *c, int bands) {
  if (!c || bands < 0 || bands > kMaxBands) return MDZ_EINVAL;
  c->bands = bands;
  return MDZ_OK;
}

int mdz_rheo_host_access(mdz_rheo_ctx *c, int *pageable) {
  if (!c || !pageable) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  *pageable = pageable_in_place() ? 1 : 0;
  return MDZ_OK;
}

int mdz_rheo_set_stream(mdz_rheo_ctx *c, void *stream) {
  if (!c) return MDZ_EINVAL;
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return MDZ_OK;
}

int mdz_rheo_sync(mdz_rheo_ctx *c, mdz_sweep_stats *st) {
  if (!c) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  c->pending = 0;
  return finish(c, st);
}

int mdz_rheo_sweep(mdz_rheo_ctx *c, const mdz_model *md, const mdz_materials *m, const mdz_grid_fields *f,
                   int final_update, int mem, int flags, mdz_sweep_stats *st) {
  return sweep_impl(c, md, m, f, final_update, mem, flags, st, false);
}

int mdz_rheo_sweep_aniso(mdz_rheo_ctx *c, const mdz_model *md, const mdz_materials *m, const mdz_grid_fields *f,
                         int final_update, int mem, int flags, mdz_sweep_stats *st) {
  return sweep_impl(c, md, m, f, final_update, mem, flags, st, true);
}

int mdz_rheo_points(mdz_rheo_ctx *c, const mdz_model *md, const mdz_materials *m, const mdz_point_inputs *in,
                    mdz_point_outputs *out, int64_t n, int aniso, int mem) {
  if (!c || !md || !m || !in || !out || n < 0) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  static thread_local PointArgs A;
  memset(&A, 0, sizeof(A));
  int rc = fold_model(md, m, A.M);
  if (rc != MDZ_OK) return rc;
  for (int p = 0; p < A.M.np; p++) fold_phase(m, md, p, A.ph[p]);
  A.n = n;
  A.aniso = aniso;
  A.polish = c->polish_iters;
  A.stats = c->d_stats;
  if (n == 0) return MDZ_OK;
  const bool host = (mem == MDZ_MEM_HOST);
  c->h2d = c->d2h = 0;
  std::vector<void *> tmp;
  // host arrays the device can address (host_mapped) are used in place; others are copied
  auto up = [&](const void *h, size_t bytes) -> void * {
    if (!h) return nullptr;
    if (!host) return const_cast<void *>(h);
    c->h2d += bytes;
    if (host_mapped(h, bytes)) return const_cast<void *>(h);
    void *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
    tmp.push_back(d);
    cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream);
    return d;
  };
  const size_t nb = (size_t)n * sizeof(double);
  A.in = *in;
  A.in.phase = (const int32_t *)up(in->phase, (size_t)n * sizeof(int32_t));
  // the inputs k_points reads (strain_acc, div and angle it never reads: not staged)
  A.in.strain_acc = A.in.div = A.in.angle = nullptr;
  const double **pin[] = {&A.in.G, &A.in.T, &A.in.P, &A.in.d, &A.in.phi, &A.in.X0, &A.in.Exx, &A.in.Ezz,
                          &A.in.Exz, &A.in.Txx0, &A.in.Tzz0, &A.in.Txz0, &A.in.dil,
                          &A.in.fric, &A.in.C, &A.in.P0, &A.in.T0, &A.in.beta,
                          &A.in.lxlz, &A.in.lx2, &A.in.ani_fac};
  if (!aniso) A.in.lxlz = A.in.lx2 = A.in.ani_fac = nullptr;
  for (auto pp : pin) *pp = (const double *)up(*pp, nb);
  // every input the kernel reads must be present
  const void *req[] = {A.in.phase, A.in.G, A.in.T, A.in.P, A.in.d, A.in.phi, A.in.X0, A.in.Exx, A.in.Ezz,
                       A.in.Exz, A.in.Txx0, A.in.Tzz0, A.in.Txz0, A.in.dil, A.in.fric, A.in.C, A.in.P0,
                       A.in.T0, A.in.beta};
  bool ok = true;
  for (auto r : req) ok = ok && r;
  if (aniso) ok = ok && A.in.lxlz && A.in.lx2 && A.in.ani_fac;
  A.out = *out;
  double **pout[] = {&A.out.eta, &A.out.Txx, &A.out.Tzz, &A.out.Txz, &A.out.etaVE, &A.out.VEcoeff,
                     &A.out.Eii_el, &A.out.Eii_pl, &A.out.Eii_pwl, &A.out.Eii_exp, &A.out.Eii_lin,
                     &A.out.Eii_gbs, &A.out.Eii_cst, &A.out.d1, &A.out.X1, &A.out.OverS, &A.out.Pcorr,
                     &A.out.rho, &A.out.div_el, &A.out.div_pl, &A.out.div_r, &A.out.Wtot, &A.out.Wel,
                     &A.out.Wdiss};
  std::vector<std::pair<void *, void *>> backs;  // (host, device)
  auto dn = [&](void *h, size_t bytes) -> void * {
    if (!h) return nullptr;
    if (!host) return h;
    c->d2h += bytes;
    if (host_mapped(h, bytes)) return h;
    void *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
    tmp.push_back(d);
    backs.push_back({h, d});
    return d;
  };
  for (auto pp : pout) *pp = (double *)dn(*pp, nb);
  A.out.iters = (int32_t *)dn(out->iters, (size_t)n * sizeof(int32_t));
  A.out.status = (int32_t *)dn(out->status, (size_t)n * sizeof(int32_t));
  if (ok) {
    for (int p = 0; p < n && host; p++) {
      if (in->phase[p] < 0 || in->phase[p] >= A.M.np) { ok = false; break; }
    }
  }
  if (!ok) {
    for (auto d : tmp) cudaFree(d);
    return MDZ_EINVAL;
  }
  if ((rc = reset_stats(c)) != MDZ_OK) return rc;
  c->launches = 1;
  CK(cudaEventRecord(c->ev0, c->stream));
  CK(launch_points(A, c->stream));
  CK(cudaEventRecord(c->ev1, c->stream));
  for (auto &b : backs) {
    size_t bytes = (b.first == (void *)out->iters || b.first == (void *)out->status) ? (size_t)n * sizeof(int32_t) : nb;
    cudaMemcpyAsync(b.first, b.second, bytes, cudaMemcpyDeviceToHost, c->stream);
  }
  rc = finish(c, nullptr);
  for (auto d : tmp) cudaFree(d);
  return rc;
}

int mdz_rheo_points_static(const mdz_model *md, const mdz_materials *m, const mdz_point_inputs *in,
                           mdz_point_outputs *out, int64_t n, int aniso, int mem, void *stream,
                           mdz_sweep_stats *st) {
  if (!md || !m || !in || !out || n < 0) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  const bool host = (mem == MDZ_MEM_HOST);
  // host memory stages n int32 at least: a count above the array's capacity is rejected
  // before any input is read or any byte count is formed (no size_t wrap-around for huge n)
  if (host && (uint64_t)n > (uint64_t)(MDZ_STATIC_SCRATCH_BYTES / sizeof(int32_t))) return MDZ_ESCRATCH;
  // every input the kernel reads must be present
  const void *req[] = {in->phase, in->G, in->T, in->P, in->d, in->phi, in->X0, in->Exx, in->Ezz, in->Exz,
                       in->Txx0, in->Tzz0, in->Txz0, in->dil, in->fric, in->C, in->P0, in->T0, in->beta};
  for (auto r : req) if (!r) return MDZ_EINVAL;
  if (aniso && (!in->lxlz || !in->lx2 || !in->ani_fac)) return MDZ_EINVAL;
  static thread_local PointArgs A;
  memset(&A, 0, sizeof(A));
  int rc = fold_model(md, m, A.M);
  if (rc != MDZ_OK) return rc;
  for (int p = 0; p < A.M.np; p++) fold_phase(m, md, p, A.ph[p]);
  if (host)
    for (int64_t i = 0; i < n; i++)
      if (in->phase[i] < 0 || in->phase[i] >= A.M.np) return MDZ_EINVAL;
  A.n = n;
  A.aniso = aniso;
  A.polish = MDZ_DEFAULT_START;
  A.in = *in;
  A.out = *out;
  // layout of the array: statistics, then (host memory) one 256-aligned slot per array
  const size_t nb = (size_t)n * sizeof(double), ni = (size_t)n * sizeof(int32_t);
  // the inputs k_points reads (strain_acc, div and angle it never reads: not staged)
  A.in.strain_acc = A.in.div = A.in.angle = nullptr;
  const double **pin[] = {&A.in.G, &A.in.T, &A.in.P, &A.in.d, &A.in.phi, &A.in.X0, &A.in.Exx, &A.in.Ezz,
                          &A.in.Exz, &A.in.Txx0, &A.in.Tzz0, &A.in.Txz0, &A.in.dil,
                          &A.in.fric, &A.in.C, &A.in.P0, &A.in.T0, &A.in.beta,
                          &A.in.lxlz, &A.in.lx2, &A.in.ani_fac};
  if (!aniso) A.in.lxlz = A.in.lx2 = A.in.ani_fac = nullptr;
  double **pout[] = {&A.out.eta, &A.out.Txx, &A.out.Tzz, &A.out.Txz, &A.out.etaVE, &A.out.VEcoeff,
                     &A.out.Eii_el, &A.out.Eii_pl, &A.out.Eii_pwl, &A.out.Eii_exp, &A.out.Eii_lin,
                     &A.out.Eii_gbs, &A.out.Eii_cst, &A.out.d1, &A.out.X1, &A.out.OverS, &A.out.Pcorr,
                     &A.out.rho, &A.out.div_el, &A.out.div_pl, &A.out.div_r, &A.out.Wtot, &A.out.Wel,
                     &A.out.Wdiss};
  constexpr size_t kStats = 256;
  static_assert(sizeof(DevStats) <= kStats, "statistics block");
  size_t need = kStats;
  auto round256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  if (host) {
    need += in->phase ? round256(ni) : 0;
    for (auto pp : pin) need += *pp ? round256(nb) : 0;
    for (auto pp : pout) need += *pp ? round256(nb) : 0;
    need += (out->iters ? round256(ni) : 0) + (out->status ? round256(ni) : 0);
  }
  if (need > (size_t)MDZ_STATIC_SCRATCH_BYTES) return MDZ_ESCRATCH;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kStaticMaxDevices) return MDZ_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {  // set-up, once per device, with that device current
    void *a = nullptr;
    CK(cudaGetSymbolAddress(&a, g_points_scratch));
    if (!a || ((uintptr_t)a & 255)) return MDZ_ECUDA;
    g_static_addr[dev] = a;
  }
  char *base = (char *)g_static_addr[dev];
  DevStats *dstats = (DevStats *)base;
  A.stats = dstats;
  // From the first enqueue on, every return waits for `stream` while the lock is still
  // held (this guard is destroyed before the lock): no copy or kernel of this call can
  // still touch the array when the next call takes it.
  struct Drain {
    cudaStream_t s;
    bool on = false;
    ~Drain() { if (on) cudaStreamSynchronize(s); }
  } drain{s};
  drain.on = true;
  CK(cudaMemsetAsync(dstats, 0, sizeof(DevStats), s));
  CK(cudaMemsetAsync(&dstats->err_key, 0xff, sizeof(dstats->err_key), s));
  if (n > 0) {
    std::vector<std::pair<void *, const void *>> backs;  // (host destination, device slot)
    size_t off = kStats;
    auto stage_in = [&](const void *h, size_t bytes) -> const void * {
      if (!h || !host) return h;
      void *d = base + off;
      off += round256(bytes);
      if (cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = MDZ_ECUDA;
      return d;
    };
    auto stage_out = [&](void *h, size_t bytes) -> void * {
      if (!h || !host) return h;
      void *d = base + off;
      off += round256(bytes);
      backs.push_back({h, d});
      return d;
    };
    A.in.phase = (const int32_t *)stage_in(in->phase, ni);
    for (auto pp : pin) *pp = (const double *)stage_in(*pp, nb);
    for (auto pp : pout) *pp = (double *)stage_out(*pp, nb);
    A.out.iters = (int32_t *)stage_out(out->iters, ni);
    A.out.status = (int32_t *)stage_out(out->status, ni);
    if (rc != MDZ_OK) return rc;
    CK(launch_points(A, s));
    for (auto &b : backs) {
      const size_t bytes = (b.first == (void *)out->iters || b.first == (void *)out->status) ? ni : nb;
      CK(cudaMemcpyAsync(b.first, b.second, bytes, cudaMemcpyDeviceToHost, s));
    }
  }
  DevStats h;
  CK(cudaMemcpyAsync(&h, dstats, sizeof(h), cudaMemcpyDeviceToHost, s));
  drain.on = false;
  CK(cudaStreamSynchronize(s));
  int status = MDZ_OK;
  long long node = -1;
  if (h.err_key != ~0ull) {
    status = -(int)(h.err_key & 0xff);
    node = (long long)(h.err_key >> 8);
  }
  if (st) {
    memset(st, 0, sizeof(*st));
    st->phase_calls = h.calls; st->newton_iters = h.iters; st->max_newton_iters = h.maxit;
    st->plastic_calls = h.plastic; st->status = status; st->error_node = node;
    st->kernel_launches = n > 0 ? 1 : 0;
    st->fp32_steps = h.f32_steps;
  }
  return status;
}

int mdz_rheo_batch_create(mdz_rheo_ctx *c, int n, const mdz_model *models, const mdz_materials *mats,
                          const mdz_grid_fields *fields, int aniso, int final_update, int flags,
                          mdz_rheo_batch **out) {
  if (!c || !models || !mats || !fields || !out || n < 1 || n > kBatchMaxGrids) return MDZ_EINVAL;
  if (flags & ~(MDZ_SWEEP_REF_START | MDZ_SWEEP_WARMSTART)) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_REF_START) && (flags & MDZ_SWEEP_WARMSTART)) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_WARMSTART) && !c->warm_ready) return MDZ_ENOTREADY;
  if ((flags & MDZ_SWEEP_WARMSTART) && c->warm.n_feat != (aniso ? kFeatAniso : kFeatIso)) return MDZ_EINVAL;
  *out = nullptr;
  CK(cudaSetDevice(c->device));
  std::vector<SweepArgs> h((size_t)n);
  std::vector<long long> tile_start((size_t)n + 1, 0), tile_n((size_t)n + 1, 0), tile_s((size_t)n + 1, 0);
  long long nodes = 0;
  for (int g = 0; g < n; g++) {
    SweepArgs &A = h[g];
    memset(&A, 0, sizeof(A));
    const mdz_model *md = models + g;
    const mdz_materials *mt = mats + g;
    const mdz_grid_fields *f = fields + g;
    if (md->Nx < 2 || md->Nz < 2) return MDZ_EINVAL;
    int rc = fold_model(md, mt, A.M);
    if (rc != MDZ_OK) return rc;
    for (int p = 0; p < A.M.np; p++) fold_phase(mt, md, p, A.ph[p]);
    FieldLists L;
    if ((rc = field_lists(md, f, aniso != 0, L)) != MDZ_OK) return rc;
    for (int i = 0; i < L.nci; i++) A.ci[i] = L.cin[i];
    for (int i = 0; i < L.nvi; i++) A.vi[i] = L.vin[i];
    for (int i = 0; i < CO_COUNT; i++) A.co[i] = L.cout[i];
    for (int i = 0; i < VO_COUNT; i++) A.vo[i] = L.vout[i];
    for (int p = 0; p < A.M.np; p++) {
      A.perc_n[p] = f->phase_perc_n[p];
      A.perc_s[p] = f->phase_perc_s[p];
      A.peta_n[p] = f->phase_eta_n[p];
      A.peta_s[p] = f->phase_eta_s[p];
      if (!A.perc_n[p] || !A.perc_s[p] || !A.peta_n[p] || !A.peta_s[p]) return MDZ_EINVAL;
    }
    A.bcp = f->BCp_type;
    A.bcg = f->BCg_type;
    A.stats = c->d_stats;
    A.final_update = final_update;
    A.need_lnd = need_lnd(mt, A.M.np);
    A.polish = (flags & MDZ_SWEEP_REF_START) ? 0 : c->polish_iters;
    A.node_base = nodes;
    const long long ng = A.M.Nc + A.M.Nv;
    nodes += ng;
    tile_start[g + 1] = tile_start[g] + (ng + kBatchTile - 1) / kBatchTile;
    tile_n[g + 1] = tile_n[g] + (A.M.Nc + kBatchTile - 1) / kBatchTile;
    tile_s[g + 1] = tile_s[g] + (A.M.Nv + kBatchTile - 1) / kBatchTile;
  }
  mdz_rheo_batch *b = new mdz_rheo_batch();
  b->ctx = c;
  b->n = n;
  b->aniso = aniso != 0;
  b->warm = (flags & MDZ_SWEEP_WARMSTART) != 0;
  b->nodes = nodes;
  b->tiles = tile_start[n];
  if (cudaMalloc(&b->d_grids, sizeof(SweepArgs) * n) != cudaSuccess ||
      cudaMalloc(&b->d_tile_start, sizeof(long long) * 3 * (n + 1)) != cudaSuccess ||
      cudaMemcpy(b->d_grids, h.data(), sizeof(SweepArgs) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_tile_start, tile_start.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->d_tile_start + (n + 1), tile_n.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->d_tile_start + 2 * (n + 1), tile_s.data(), sizeof(long long) * (n + 1),
                 cudaMemcpyHostToDevice) != cudaSuccess) {
    mdz_rheo_batch_destroy(b);
    return MDZ_ECUDA;
  }
  b->args.grids = b->d_grids;
  b->args.tile_start = b->d_tile_start;
  b->args.tile_start_n = b->d_tile_start + (n + 1);
  b->args.tile_start_s = b->d_tile_start + 2 * (n + 1);
  b->args.n = n;
  b->args.tiles = b->tiles;
  b->args.tiles_n = tile_n[n];
  b->args.tiles_s = tile_s[n];
  b->args.stats = c->d_stats;
  b->grid = (int)std::min<long long>(b->tiles, 0x7fffffffLL);
  *out = b;
  return MDZ_OK;
}

int mdz_rheo_batch_destroy(mdz_rheo_batch *b) {
  if (!b) return MDZ_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_grids) cudaFree(b->d_grids);
  if (b->d_tile_start) cudaFree(b->d_tile_start);
  delete b;
  return MDZ_OK;
}

// The per-launch options of a batch sweep: the context's network and start descriptor as
// they are now (a warm batch), and the perturbation of sweep `sweep` (amp 0: none).
BatchSweepArgs batch_launch_args(const mdz_rheo_batch *b, double amp, uint64_t seed, int sweep) {
  BatchSweepArgs x;
  memset(&x, 0, sizeof(x));
  x.warm = b->warm ? 1 : 0;
  if (b->warm) {
    x.mlp = b->ctx->warm;
    x.mlp.polish_iters = b->ctx->polish_iters;
  }
  x.amp = amp;
  x.seed = (unsigned long long)seed;
  x.sweep = sweep;
  return x;
}

int mdz_rheo_batch_sweep(mdz_rheo_batch *b, mdz_sweep_stats *st) {
  if (!b) return MDZ_EINVAL;
  mdz_rheo_ctx *c = b->ctx;
  CK(cudaSetDevice(c->device));
  int rc = reset_stats(c);
  if (rc != MDZ_OK) return rc;
  c->h2d = c->d2h = 0;
  c->launches = batch_kernel_count(b->args);
  CK(cudaEventRecord(c->ev0, c->stream));
  if (b->warm && !c->warm_ready) return MDZ_ENOTREADY;
  CK(launch_sweep_batch(b->args, batch_launch_args(b, 0.0, 0, 0), b->aniso, c->stream, b->grid));
  CK(cudaEventRecord(c->ev1, c->stream));
  return finish(c, st);
}

int mdz_rheo_batch_capture(mdz_rheo_batch *b, int nsweeps, double amp, uint64_t seed) {
  if (!b || nsweeps < 1 || nsweeps > 100000 || !(amp >= 0.0 && amp < 1.0)) return MDZ_EINVAL;
  mdz_rheo_ctx *c = b->ctx;
  if (b->warm && !c->warm_ready) return MDZ_ENOTREADY;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaMemsetAsync(c->d_stats, 0, sizeof(DevStats), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(&c->d_stats->err_key, 0xff, sizeof(c->d_stats->err_key), c->stream);
  // each sweep perturbs the strain rates as it loads them (fused: no separate pass)
  for (int s = 0; s < nsweeps && e == cudaSuccess; s++)
    e = launch_sweep_batch(b->args, batch_launch_args(b, amp, seed, s), b->aniso, c->stream, b->grid);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return MDZ_ECUDA;
  }
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    b->graph = nullptr;
    b->exec = nullptr;
    return MDZ_ECUDA;
  }
  b->graph_sweeps = nsweeps;
  b->graph_launches = nsweeps * (int)batch_kernel_count(b->args);
  return MDZ_OK;
}

int mdz_rheo_batch_set_grid(mdz_rheo_batch *b, int ctas) {
  if (!b || ctas < 0) return MDZ_EINVAL;
  CK(cudaSetDevice(b->ctx->device));
  CK(cudaStreamSynchronize(b->ctx->stream));
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  b->graph_sweeps = b->graph_launches = 0;
  b->grid = (int)std::min<long long>(ctas > 0 ? (long long)ctas : b->tiles, 0x7fffffffLL);
  return MDZ_OK;
}

int mdz_rheo_batch_launch(mdz_rheo_batch *b, mdz_sweep_stats *st) {
  if (!b) return MDZ_EINVAL;
  if (!b->exec) return MDZ_ENOTREADY;
  mdz_rheo_ctx *c = b->ctx;
  CK(cudaSetDevice(c->device));
  c->h2d = c->d2h = 0;
  c->launches = (unsigned)b->graph_launches;
  CK(cudaEventRecord(c->ev0, c->stream));
  CK(cudaGraphLaunch(b->exec, c->stream));
  CK(cudaEventRecord(c->ev1, c->stream));
  return finish(c, st);
}

int mdz_rheo_autotune(mdz_rheo_ctx *c, const mdz_model *md, const mdz_materials *m, const mdz_grid_fields *f,
                      int aniso, int flags, int reps, double *ms_out, int *best_out) {
  if (!c || !md || !m || !f || reps < 1 || reps > 1000) return MDZ_EINVAL;
  if (flags & (MDZ_SWEEP_ASYNC | MDZ_SWEEP_WARMSTART | MDZ_SWEEP_ITERS)) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  const int a = aniso ? 1 : 0;
  // the candidates, in the order of MDZ_AUTOTUNE_CANDIDATES
  std::vector<LaunchShape> cand;
  const int waves[5] = {0, 1, 2, 4, 8};  // 0: one thread per node
  for (int block : {128, 64})
    for (int w : waves) {
      int occ = 0, regs = 0, smem = 0;
      sweep_kernel_info(a, &regs, &smem, &occ, block, SHAPE_THREAD);
      cand.push_back({block, w ? c->sms * (occ > 0 ? occ : 1) * w : 0, SHAPE_THREAD});
    }
  cand.push_back({128, 0, SHAPE_REGS255});
  {
    int occ = 0, regs = 0, smem = 0;
    sweep_kernel_info(a, &regs, &smem, &occ, 128, SHAPE_QUEUE);
    cand.push_back({128, c->sms * (occ > 0 ? occ : 1), SHAPE_QUEUE});
  }
  // the compacting form; the anisotropic sweep, which has no iterated plastic return, runs
  // it as one thread per node
  cand.push_back({128, 0, aniso ? SHAPE_THREAD : SHAPE_COMPACT});
  static_assert(MDZ_AUTOTUNE_CANDIDATES == 13, "candidate list");
  const LaunchShape keep = c->shape[a];
  const auto keep_tuned = c->tuned;
  c->tuned.clear();  // every candidate below runs as the context's shape
  double best_ms = 1e300;
  int best = 0;
  for (int ci = 0; ci < (int)cand.size(); ci++) {
    c->shape[a] = cand[ci];
    double sum = 0.0;
    mdz_sweep_stats st;
    for (int r = 0; r <= reps; r++) {  // the first is a warm-up
      const int rc = sweep_impl(c, md, m, f, 0, MDZ_MEM_DEVICE, flags, &st, aniso != 0);
      if (rc != MDZ_OK) {
        c->shape[a] = keep;
        c->tuned = keep_tuned;
        return rc;
      }
      if (r > 0) sum += st.elapsed_ms;
    }
    const double ms = sum / reps;
    if (ms_out) ms_out[ci] = ms;
    if (ms < best_ms) { best_ms = ms; best = ci; }
  }
  c->shape[a] = cand[best];
  c->tuned = keep_tuned;
  // cache the choice for sweeps of this kind: phases, start, size
  const bool ref = (flags & MDZ_SWEEP_REF_START) != 0;
  const long long nodes = (long long)(md->Nx - 1) * (md->Nz - 1) + (long long)md->Nx * md->Nz;
  for (auto it = c->tuned.begin(); it != c->tuned.end();)
    if (it->aniso == a && it->np == m->Nb_phases && it->ref == (int)ref && it->nodes == nodes) it = c->tuned.erase(it);
    else ++it;
  c->tuned.push_back({a, m->Nb_phases, (int)ref, nodes, cand[best]});
  if (best_out) *best_out = best;
  return MDZ_OK;
}

int mdz_rheo_set_launch_shape(mdz_rheo_ctx *c, int aniso, int block, int grid_cap, int form) {
  if (!c || (block != 64 && block != 128) || grid_cap < 0) return MDZ_EINVAL;
  if (form != SHAPE_THREAD && form != SHAPE_REGS255 && form != SHAPE_QUEUE && form != SHAPE_COMPACT)
    return MDZ_EINVAL;
  if (form == SHAPE_COMPACT && (aniso || block != 128)) return MDZ_EINVAL;
  if (form == SHAPE_QUEUE && grid_cap == 0) {  // one wave of resident CTAs
    int occ = 0, regs = 0, smem = 0;
    CK(cudaSetDevice(c->device));
    sweep_kernel_info(aniso ? 1 : 0, &regs, &smem, &occ, 128, SHAPE_QUEUE);
    grid_cap = c->sms * (occ > 0 ? occ : 1);
  }
  c->shape[aniso ? 1 : 0] = {form == SHAPE_QUEUE ? 128 : block, grid_cap, form};
  c->tuned.clear();
  return MDZ_OK;
}

int mdz_rheo_get_launch_form(mdz_rheo_ctx *c, int aniso, int *form) {
  if (!c || !form) return MDZ_EINVAL;
  *form = c->shape[aniso ? 1 : 0].form;
  return MDZ_OK;
}

int mdz_rheo_get_launch_shape(mdz_rheo_ctx *c, int aniso, int *block, int *grid_cap) {
  if (!c || !block || !grid_cap) return MDZ_EINVAL;
  *block = c->shape[aniso ? 1 : 0].block;
  *grid_cap = c->shape[aniso ? 1 : 0].grid_cap;
  return MDZ_OK;
}

int mdz_rheo_operators(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_materials *mat, const mdz_grid_fields *f,
                       mdz_operator_fields *ops, int jacobian, int compressible, int aniso, int mem, int flags,
                       mdz_sweep_stats *st) {
  if (!ctx || !md || !mat || !f || !ops) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (flags & ~(MDZ_SWEEP_REF_START | MDZ_OPS_PER_NODE | MDZ_SWEEP_STAGED)) return MDZ_EINVAL;
  if (md->Nx < 2 || md->Nz < 2) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  static thread_local OpArgs A;
  memset(&A, 0, sizeof(A));
  int rc = fold_model(md, mat, A.M);
  if (rc != MDZ_OK) return rc;
  for (int p = 0; p < A.M.np; p++) fold_phase(mat, md, p, A.ph[p]);
  A.compressible = compressible != 0;
  A.need_lnd = need_lnd(mat, A.M.np);
  A.polish = (flags & MDZ_SWEEP_REF_START) ? 0 : ctx->polish_iters;
  const size_t Nc = (size_t)A.M.Nc, Nv = (size_t)A.M.Nv;
  const bool host = (mem == MDZ_MEM_HOST);
  const bool anis = aniso != 0, jac = jacobian != 0;
  // inputs: the sweep's inputs (the ones the local solve reads) and its outputs
  FieldLists L;
  {
    // the output lists are not written here; only their presence checks are shared
    mdz_grid_fields g = *f;
    if ((rc = field_lists(md, &g, anis, L)) != MDZ_OK) return rc;
  }
  if (!f->eta_n || !f->eta_s || !f->T_s || !f->P_s || !f->d0_s || !f->phi0_s) return MDZ_EINVAL;
  double *dout[OP_COUNT] = {ops->D11_n, ops->D12_n, ops->D13_n, ops->D14_n, ops->D21_n, ops->D22_n, ops->D23_n,
                            ops->D24_n, jac ? ops->drhodp_n : nullptr, ops->D31_s, ops->D32_s, ops->D33_s,
                            ops->D34_s};
  for (int i = 0; i < OP_COUNT; i++) if (i != OP_DRHODP && !dout[i]) return MDZ_EINVAL;
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  for (int i = 0; i < L.nci; i++) A.ci[i] = mi.in(L.cin[i], S_CI + i, Nc, host);
  for (int i = 0; i < L.nvi; i++) A.vi[i] = mi.in(L.vin[i], S_VI + i, Nv, host);
  for (int p = 0; p < A.M.np; p++) {
    A.perc_n[p] = mi.in(f->phase_perc_n[p], S_PN + p, Nc, host);
    A.perc_s[p] = mi.in(f->phase_perc_s[p], S_PS + p, Nv, host);
    A.peta_n[p] = mi.in((const double *)f->phase_eta_n[p], S_EN + p, Nc, host);
    A.peta_s[p] = mi.in((const double *)f->phase_eta_s[p], S_ES + p, Nv, host);
  }
  A.bcp = mi.in(f->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(f->BCg_type, S_BCG, Nv, host);
  A.eta_n = mi.in((const double *)f->eta_n, S_CO + CO_eta, Nc, host);
  A.eta_s = mi.in((const double *)f->eta_s, S_VO + VO_eta, Nv, host);
  A.T_s = mi.in((const double *)f->T_s, S_VO + VO_T, Nv, host);
  A.P_s = mi.in((const double *)f->P_s, S_VO + VO_P, Nv, host);
  A.d0_s = mi.in((const double *)f->d0_s, S_VO + VO_d0, Nv, host);
  A.phi0_s = mi.in((const double *)f->phi0_s, S_VO + VO_phi0, Nv, host);
  for (int i = 0; i < OP_COUNT; i++) {
    const size_t n = i < OP_D31 ? Nc : Nv;
    // drhodp_n is not written at air cells, as in the reference: keep the caller's values there
    A.D[i] = (i == OP_DRHODP) ? (double *)mi.in((const double *)dout[i], S_OP + i, n, host)
                              : mi.out(dout[i], S_OP + i, n, host);
  }
  if (mi.err) return mi.err;
  A.stats = ctx->d_stats;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launch_operators(A, anis, jac, !(flags & MDZ_OPS_PER_NODE), ctx->stream));
  ctx->launches = 1;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  for (int i = 0; i < OP_COUNT; i++) mi.back(dout[i], S_OP + i, i < OP_D31 ? Nc : Nv, host);
  if (mi.err) return mi.err;
  return finish(ctx, st);
}

int mdz_rheo_strain_rates(mdz_rheo_ctx *ctx, const mdz_model *md, double dx, double dz, int out_of_plane,
                          double compressible, mdz_strain_rate_fields *sr, int mem, int flags, mdz_sweep_stats *st) {
  if (!ctx || !md || !sr) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (flags & ~(MDZ_SWEEP_ASYNC | MDZ_SWEEP_STAGED)) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_ASYNC) && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (md->Nx < 2 || md->Nz < 2) return MDZ_EINVAL;
  double *out[SR_COUNT] = {sr->div_u, sr->exxd, sr->ezzd, sr->exz_n, sr->wxz_n,
                           sr->exz, sr->wxz, sr->exxd_s, sr->ezzd_s, sr->div_u_s};
  if (!sr->u_in || !sr->v_in || !sr->BCp_type || !sr->BCg_type) return MDZ_EINVAL;
  for (int i = 0; i < SR_COUNT; i++) if (!out[i]) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  StrainArgs A;
  memset(&A, 0, sizeof(A));
  A.Nx = md->Nx; A.Nz = md->Nz; A.Ncx = md->Nx - 1; A.Ncz = md->Nz - 1;
  A.periodic_x = md->periodic_x;
  A.dx = make_divisor(dx); A.dz = make_divisor(dz);
  A.oop_half = (out_of_plane == 1) ? 0.5 : 0.0;  // RheologyDensity.c:2006, :2033
  A.comp3 = compressible * 1.0 / 3.0;             // RheologyDensity.c:2039-2040
  const size_t Nx = (size_t)md->Nx, Nz = (size_t)md->Nz;
  const size_t Nc = (Nx - 1) * (Nz - 1), Nv = Nx * Nz;
  const bool host = (mem == MDZ_MEM_HOST);
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  A.u = mi.in(sr->u_in, S_SRU, Nx * (Nz + 1), host);
  A.v = mi.in(sr->v_in, S_SRV, (Nx + 1) * Nz, host);
  A.bcp = mi.in(sr->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(sr->BCg_type, S_BCG, Nv, host);
  for (int i = 0; i < SR_COUNT; i++) {
    const size_t n = i < SR_EXZ ? Nc : Nv;
    // wxz is not written at air vertices, as in the reference: keep the caller's values there
    A.out[i] = (i == SR_WXZ) ? (double *)mi.in((const double *)out[i], S_SR + i, n, host)
                             : mi.out(out[i], S_SR + i, n, host);
  }
  if (mi.err) return mi.err;
  int rc;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launch_strain_rates(A, ctx->stream));
  ctx->launches = 1;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  for (int i = 0; i < SR_COUNT; i++) mi.back(out[i], S_SR + i, i < SR_EXZ ? Nc : Nv, host);
  if (mi.err) return mi.err;
  if (flags & MDZ_SWEEP_ASYNC) {
    ctx->pending = 1;
    return MDZ_OK;
  }
  return finish(ctx, st);
}

int mdz_rheo_marker_stress(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_marker_opts *o, mdz_marker_grid *g,
                           mdz_markers *mk, int mem, int flags, mdz_sweep_stats *st) {
  if (!ctx || !md || !o || !g || !mk) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (flags & ~(MDZ_SWEEP_ASYNC | MDZ_SWEEP_STAGED)) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_ASYNC) && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (md->Nx < 2 || md->Nz < 2 || mk->n < 0 || mk->n > 0x7fffffffLL) return MDZ_EINVAL;
  if (o->interp_stencil != 1 && o->interp_stencil != 9) return MDZ_EINVAL;
  const bool el = (o->elastic == 1), dir = (o->anisotropy == 1 && o->advection == 1);
  const bool sub = el && o->subgrid_diffusion == 2;
  if (sub && (!o->G || !g->xc_coord || !g->zc_coord || !g->eta_phys_s || md->Nb_phases < 1 ||
              md->Nb_phases > MDZ_MAX_PHASES))
    return MDZ_EINVAL;
  if (!g->xg_coord || !g->zg_coord || !g->xvz_coord || !g->zvx_coord || !g->BCp_type || !g->BCg_type ||
      !mk->x || !mk->z || !mk->phase)
    return MDZ_EINVAL;
  if (el && (!g->sxxd || !g->szzd || !g->sxxd0 || !g->szzd0 || !g->sxz || !g->sxz0 || !g->wxz || !mk->sxxd ||
             !mk->szzd || !mk->sxz))
    return MDZ_EINVAL;
  if (dir && (!g->u_in || !g->v_in || !mk->nx || !mk->nz)) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  MarkerArgs A;
  memset(&A, 0, sizeof(A));
  const size_t Nx = (size_t)md->Nx, Nz = (size_t)md->Nz, Nc = (Nx - 1) * (Nz - 1), Nv = Nx * Nz;
  const size_t n = (size_t)mk->n;
  A.n = mk->n; A.Nx = md->Nx; A.Nz = md->Nz; A.periodic_x = md->periodic_x;
  A.elastic = o->elastic; A.rotation = o->stress_rotation; A.director = dir; A.stencil = o->interp_stencil;
  A.subgrid = sub ? 1 : 0;
  if (sub) {
    A.np = md->Nb_phases;
    for (int p = 0; p < A.np; p++) A.G[p] = make_divisor(o->G[p]);
  }
  A.dt = md->dt;
  A.dx = make_divisor(g->dx); A.dz = make_divisor(g->dz);
  // P2Mastah's weight lengths, by its own expressions (ParticleRoutines.c:2218-2221)
  A.dx_itp = make_divisor(o->interp_stencil == 9 ? 3.0 * g->dx / 2.0 : g->dx / 2.0);
  A.dz_itp = make_divisor(o->interp_stencil == 9 ? 3.0 * g->dz / 2.0 : g->dz / 2.0);
  const bool host = (mem == MDZ_MEM_HOST);
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  A.xg = mi.in(g->xg_coord, S_MK + 8, Nx, host);
  A.zg = mi.in(g->zg_coord, S_MK + 9, Nz, host);
  A.xvz = mi.in(g->xvz_coord, S_MK + 10, Nx + 1, host);
  A.zvx = mi.in(g->zvx_coord, S_MK + 11, Nz + 1, host);
  A.bcp = mi.in(g->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(g->BCg_type, S_BCG, Nv, host);
  A.x = mi.in(mk->x, S_MK + 0, n, host);
  A.z = mi.in(mk->z, S_MK + 1, n, host);
  A.phase = mi.in((const int *)mk->phase, S_MK + 2, n, host);
  if (el) {
    A.sxxd = mi.in(g->sxxd, S_MK + 12, Nc, host);
    A.szzd = mi.in(g->szzd, S_MK + 13, Nc, host);
    A.sxxd0 = mi.in(g->sxxd0, S_MK + 14, Nc, host);
    A.szzd0 = mi.in(g->szzd0, S_MK + 15, Nc, host);
    A.sxz = mi.in(g->sxz, S_MK + 16, Nv, host);
    A.sxz0 = mi.in(g->sxz0, S_MK + 17, Nv, host);
    A.wxz = (double *)mi.in((const double *)g->wxz, S_MK + 20, Nv, host);  // kept where not rewritten
    A.m_sxxd = (double *)mi.in((const double *)mk->sxxd, S_MK + 3, n, host);
    A.m_szzd = (double *)mi.in((const double *)mk->szzd, S_MK + 4, n, host);
    A.m_sxz = (double *)mi.in((const double *)mk->sxz, S_MK + 5, n, host);
  }
  if (sub) {
    A.xc = mi.in(g->xc_coord, S_MK + 27, Nx - 1, host);
    A.zc = mi.in(g->zc_coord, S_MK + 28, Nz - 1, host);
    A.eta_s = mi.in(g->eta_phys_s, S_MK + 29, Nv, host);
  }
  if (dir) {
    A.u = mi.in(g->u_in, S_MK + 18, Nx * (Nz + 1), host);
    A.v = mi.in(g->v_in, S_MK + 19, (Nx + 1) * Nz, host);
    A.m_nx = (double *)mi.in((const double *)mk->nx, S_MK + 6, n, host);
    A.m_nz = (double *)mi.in((const double *)mk->nz, S_MK + 7, n, host);
  }
  if (mi.err) return mi.err;
  // scratch: per-node increments and gradients, P2Mastah flags and exact sums
  const size_t scratch[6] = {el ? Nv * sizeof(double) : 0, el ? Nc * sizeof(double2) : 0, el ? Nv * sizeof(double) : 0,
                             dir ? Nc * sizeof(double2) : 0, dir ? Nv * sizeof(double2) : 0,
                             el ? Nv + sizeof(int) : 0};
  void *sp[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int b = 0; b < 6; b++) {
    if (!scratch[b]) continue;
    if (ensure(ctx->bufs[S_MK + 21 + b], scratch[b]) != MDZ_OK) return MDZ_ENOMEM;
    sp[b] = ctx->bufs[S_MK + 21 + b].p;
  }
  A.WM = (double *)sp[0];
  A.inc_n = (double2 *)sp[1];
  A.inc_s = (double *)sp[2];
  A.grad_n = (double2 *)sp[3];
  A.grad_s = (double2 *)sp[4];
  A.exotic = (int *)sp[5];
  A.hit = sp[5] ? (unsigned char *)sp[5] + sizeof(int) : nullptr;
  if (sub) {
    if (ensure(ctx->bufs[S_MK + 30], (n > 0 ? 3 * n : 1) * sizeof(double)) != MDZ_OK ||
        ensure(ctx->bufs[S_MK + 31], 3 * Nc * sizeof(double)) != MDZ_OK ||
        ensure(ctx->bufs[S_MK + 32], 2 * Nv * sizeof(double)) != MDZ_OK)
      return MDZ_ENOMEM;
    A.m_sub = (double *)ctx->bufs[S_MK + 30].p;
    A.sum_n = (double *)ctx->bufs[S_MK + 31].p;
    A.sum_s = (double *)ctx->bufs[S_MK + 32].p;
  }
  // A marker at most L (1 - 2^-40) from a vertex, L the weight length, has 1 - d/L >=
  // 2^-41 on that axis once rounded, so a P2Mastah weight >= 2^-82 > 1e-30
  const auto near = [](double L) { return (L >= 0x1p-900 && L <= 0x1p900) ? L - L * 0x1p-40 : -1.0; };
  A.near_x = near(A.dx_itp.b);
  A.near_z = near(A.dz_itp.b);
  A.stats = ctx->d_stats;
  int rc;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (el || dir) {
    CK(launch_marker_grid(A, ctx->stream));
    ctx->launches += 1;
  }
  if (sub) {
    CK(launch_marker_subgrid(A, ctx->stream));
    CK(launch_marker_remainder(A, ctx->stream));
    ctx->launches += 2;
  }
  if (el || dir) {
    CK(launch_marker_update(A, ctx->stream));
    ctx->launches += 1;
  }
  if (el) {
    if (!sub) {
      CK(launch_marker_weights(A, ctx->stream));
      ctx->launches += 1;
    }
    CK(launch_marker_wxz(A, ctx->stream));
    ctx->launches += 1;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if (el) {
    mi.back(mk->sxxd, S_MK + 3, n, host);
    mi.back(mk->szzd, S_MK + 4, n, host);
    mi.back(mk->sxz, S_MK + 5, n, host);
    mi.back(g->wxz, S_MK + 20, Nv, host);
  }
  if (dir) {
    mi.back(mk->nx, S_MK + 6, n, host);
    mi.back(mk->nz, S_MK + 7, n, host);
  }
  if (mi.err) return mi.err;
  return prep_finish(ctx, flags, st);
}

int mdz_rheo_p2mastah(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_marker_grid *g, const mdz_markers *mk,
                      const double *values, int avg, int interp_stencil, double *node_n, double *node_s, int mem,
                      int flags, mdz_sweep_stats *st) {
  if (!ctx || !md || !g || !mk || !values || (!node_n && !node_s)) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (flags & ~(MDZ_SWEEP_ASYNC | MDZ_SWEEP_STAGED)) return MDZ_EINVAL;
  if ((flags & MDZ_SWEEP_ASYNC) && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (md->Nx < 2 || md->Nz < 2 || md->Nb_phases < 1 || mk->n < 0 || mk->n > 0x7fffffffLL) return MDZ_EINVAL;
  if (avg < 0 || avg > 2 || (interp_stencil != 1 && interp_stencil != 9)) return MDZ_EINVAL;
  if (!mk->x || !mk->z || !mk->phase) return MDZ_EINVAL;
  if (node_n && (!g->xc_coord || !g->zc_coord || !g->BCp_type)) return MDZ_EINVAL;
  if (node_s && (!g->xg_coord || !g->zg_coord || !g->BCg_type)) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  MarkerArgs A;
  memset(&A, 0, sizeof(A));
  const size_t Nx = (size_t)md->Nx, Nz = (size_t)md->Nz, Nc = (Nx - 1) * (Nz - 1), Nv = Nx * Nz;
  const size_t n = (size_t)mk->n;
  A.n = mk->n; A.Nx = md->Nx; A.Nz = md->Nz; A.periodic_x = md->periodic_x; A.np = md->Nb_phases;
  A.stencil = interp_stencil; A.avg = avg;
  A.dx = make_divisor(g->dx); A.dz = make_divisor(g->dz);
  // P2Mastah's weight lengths, by its own expressions (ParticleRoutines.c:2218-2221)
  A.dx_itp = make_divisor(interp_stencil == 9 ? 3.0 * g->dx / 2.0 : g->dx / 2.0);
  A.dz_itp = make_divisor(interp_stencil == 9 ? 3.0 * g->dz / 2.0 : g->dz / 2.0);
  const bool host = (mem == MDZ_MEM_HOST);
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  A.x = mi.in(mk->x, S_P2M + 0, n, host);
  A.z = mi.in(mk->z, S_P2M + 1, n, host);
  A.phase = mi.in((const int *)mk->phase, S_P2M + 2, n, host);
  A.val = mi.in(values, S_P2M + 3, n, host);
  if (node_n) {
    A.xc = mi.in(g->xc_coord, S_P2M + 4, Nx - 1, host);
    A.zc = mi.in(g->zc_coord, S_P2M + 5, Nz - 1, host);
    A.bcp = mi.in(g->BCp_type, S_BCP, Nc, host);
    A.out_n = (double *)mi.in((const double *)node_n, S_P2M + 6, Nc, host);  // nodes P2Mastah skips keep theirs
  }
  if (node_s) {
    A.xg = mi.in(g->xg_coord, S_P2M + 7, Nx, host);
    A.zg = mi.in(g->zg_coord, S_P2M + 8, Nz, host);
    A.bcg = mi.in(g->BCg_type, S_BCG, Nv, host);
    A.out_s = (double *)mi.in((const double *)node_s, S_P2M + 9, Nv, host);
  }
  if (mi.err) return mi.err;
  if ((node_n && ensure(ctx->bufs[S_P2M + 10], 2 * Nc * sizeof(double)) != MDZ_OK) ||
      (node_s && ensure(ctx->bufs[S_P2M + 11], 2 * Nv * sizeof(double)) != MDZ_OK))
    return MDZ_ENOMEM;
  A.sum_n = node_n ? (double *)ctx->bufs[S_P2M + 10].p : nullptr;
  A.sum_s = node_s ? (double *)ctx->bufs[S_P2M + 11].p : nullptr;
  A.stats = ctx->d_stats;
  int rc;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  if (node_n) CK(cudaMemsetAsync(A.sum_n, 0, 2 * Nc * sizeof(double), ctx->stream));
  if (node_s) CK(cudaMemsetAsync(A.sum_s, 0, 2 * Nv * sizeof(double), ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launch_p2m_scatter(A, ctx->stream));
  CK(launch_p2m_nodes(A, ctx->stream));
  ctx->launches = 2;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if (node_n) mi.back(node_n, S_P2M + 6, Nc, host);
  if (node_s) mi.back(node_s, S_P2M + 9, Nv, host);
  if (mi.err) return mi.err;
  return prep_finish(ctx, flags, st);
}

// input preparation: Softening over the grid, ShearModCompExpGrid
int mdz_rheo_softening(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_prep_materials *mat, mdz_prep_fields *f,
                       int smooth_softening, int hardening_modulus, int marker_noise, int mem, int flags,
                       mdz_sweep_stats *st) {
  if (!ctx || !prep_common(md, mat, f, mem, flags)) return MDZ_EINVAL;
  if (!f->strain_pl_n || !f->strain_pl_s || !f->fric_n || !f->dil_n || !f->C_n || !f->fric_s || !f->dil_s ||
      !f->C_s)
    return MDZ_EINVAL;
  if (marker_noise == 1 && (!f->noise_n || !f->noise_s)) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  static thread_local SoftArgs A;
  memset(&A, 0, sizeof(A));
  const size_t Nc = (size_t)(md->Nx - 1) * (md->Nz - 1), Nv = (size_t)md->Nx * md->Nz;
  A.Nc = (long long)Nc; A.Nv = (long long)Nv;
  A.np = md->Nb_phases;
  // CohesionFrictionDilationGrid (RheologyDensity.c:1545-1546): the later switch wins
  A.style = 0;
  if (smooth_softening == 1) A.style = 1;
  if (hardening_modulus == 1) A.style = 2;
  A.noise = marker_noise == 1;
  for (int p = 0; p < A.np; p++) fold_soft(mat, p, A.ph[p]);
  const bool host = (mem == MDZ_MEM_HOST);
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  for (int p = 0; p < A.np; p++) {
    A.perc_n[p] = mi.in(f->phase_perc_n[p], S_PN + p, Nc, host);
    A.perc_s[p] = mi.in(f->phase_perc_s[p], S_PS + p, Nv, host);
  }
  A.bcp = mi.in(f->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(f->BCg_type, S_BCG, Nv, host);
  A.strain_n = mi.in(f->strain_pl_n, S_PREP + 0, Nc, host);
  A.strain_s = mi.in(f->strain_pl_s, S_PREP + 1, Nv, host);
  if (A.noise) {
    A.noise_n = mi.in(f->noise_n, S_PREP + 2, Nc, host);
    A.noise_s = mi.in(f->noise_s, S_PREP + 3, Nv, host);
  }
  double *outs[6] = {f->fric_n, f->dil_n, f->C_n, f->fric_s, f->dil_s, f->C_s};
  double *dev[6];
  for (int k = 0; k < 6; k++) dev[k] = mi.out(outs[k], S_PREP + 4 + k, k < 3 ? Nc : Nv, host);
  if (mi.err) return mi.err;
  A.fric_n = dev[0]; A.dil_n = dev[1]; A.C_n = dev[2]; A.fric_s = dev[3]; A.dil_s = dev[4]; A.C_s = dev[5];
  int rc;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launch_softening(A, ctx->stream));
  ctx->launches = 1;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  for (int k = 0; k < 6; k++) mi.back(outs[k], S_PREP + 4 + k, k < 3 ? Nc : Nv, host);
  if (mi.err) return mi.err;
  return prep_finish(ctx, flags, st);
}

int mdz_rheo_shear_modulus(mdz_rheo_ctx *ctx, const mdz_model *md, const mdz_prep_materials *mat,
                           mdz_prep_fields *f, int mem, int flags, mdz_sweep_stats *st) {
  if (!ctx || !prep_common(md, mat, f, mem, flags)) return MDZ_EINVAL;
  if (!f->mu_n || !f->bet_n || !f->alp || !f->mu_s || !f->bet_s) return MDZ_EINVAL;
  CK(cudaSetDevice(ctx->device));
  static thread_local ModArgs A;
  memset(&A, 0, sizeof(A));
  const size_t Nc = (size_t)(md->Nx - 1) * (md->Nz - 1), Nv = (size_t)md->Nx * md->Nz;
  A.Nc = (long long)Nc; A.Nv = (long long)Nv;
  A.Nx = md->Nx;
  A.np = md->Nb_phases;
  A.periodic_x = md->periodic_x;
  A.skip_zero = 1;
  for (int p = 0; p < A.np; p++) {
    A.G[p] = make_divisor(mat->G[p]);
    A.bet[p] = make_divisor(mat->bet[p]);
    A.alp[p] = mat->alp[p];
    if (!(std::isfinite(mat->G[p]) && mat->G[p] != 0.0 && std::isfinite(mat->bet[p]) && mat->bet[p] != 0.0 &&
          std::isfinite(mat->alp[p])))
      A.skip_zero = 0;
  }
  const bool host = (mem == MDZ_MEM_HOST);
  ctx->h2d = ctx->d2h = 0;
  ctx->launches = 0;
  Mirror mi{ctx, !(flags & MDZ_SWEEP_STAGED)};
  for (int p = 0; p < A.np; p++) {
    A.perc_n[p] = mi.in(f->phase_perc_n[p], S_PN + p, Nc, host);
    A.perc_s[p] = mi.in(f->phase_perc_s[p], S_PS + p, Nv, host);
  }
  A.bcp = mi.in(f->BCp_type, S_BCP, Nc, host);
  A.bcg = mi.in(f->BCg_type, S_BCG, Nv, host);
  double *outs[5] = {f->mu_n, f->bet_n, f->alp, f->mu_s, f->bet_s};
  double *dev[5];
  for (int k = 0; k < 5; k++) dev[k] = mi.out(outs[k], S_PREP + 10 + k, k < 3 ? Nc : Nv, host);
  if (mi.err) return mi.err;
  A.mu_n = dev[0]; A.bet_n = dev[1]; A.alp_n = dev[2]; A.mu_s = dev[3]; A.bet_s = dev[4];
  A.stats = ctx->d_stats;
  int rc;
  if ((rc = reset_stats(ctx)) != MDZ_OK) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launch_moduli(A, ctx->stream));
  ctx->launches = 1;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  for (int k = 0; k < 5; k++) mi.back(outs[k], S_PREP + 10 + k, k < 3 ? Nc : Nv, host);
  if (mi.err) return mi.err;
  return prep_finish(ctx, flags, st);
}

int mdz_rheo_get_iterations(mdz_rheo_ctx *c, int32_t *out_n, int32_t *out_s) {
  if (!c || !c->have_iters) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (out_n) CK(cudaMemcpy(out_n, c->d_iters_n, (size_t)c->last_Nc * c->last_np * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (out_s) CK(cudaMemcpy(out_s, c->d_iters_s, (size_t)c->last_Nv * c->last_np * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return MDZ_OK;
}


int mdz_rheo_set_warmstart(mdz_rheo_ctx *c, const mdz_mlp_weights *w, int polish_iters) {
  if (!c || polish_iters < 0 || (polish_iters & ~(0xff | MDZ_START_DD)) || (polish_iters & 0xff) > 64)
    return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  c->polish_iters = polish_iters;
  if (!w) { c->warm_ready = 0; return MDZ_OK; }
  if (w->n_feat < 1 || w->n_feat > kMlpIn || !(w->z_scale != 0.0f)) return MDZ_EINVAL;
  const int rc = upload_warm(c, w);
  c->warm_ready = (rc == MDZ_OK);
  return rc;
}

int mdz_rheo_set_mma_poll_limit(mdz_rheo_ctx *c, int32_t limit) {
  if (!c) return MDZ_EINVAL;
  c->mma_poll_limit = limit < 0 ? (1u << 24) : (unsigned)limit;
  return MDZ_OK;
}

int mdz_rheo_collect(mdz_rheo_ctx *c, const mdz_model *md, const mdz_materials *m, const mdz_grid_fields *f,
                     int final_update, int aniso, int mem, float *X, float *Y, mdz_sweep_stats *st) {
  if (!X || !Y) return MDZ_EINVAL;
  return sweep_impl(c, md, m, f, final_update, mem, 0, st, aniso != 0, X, Y);
}

int mdz_rheo_train_mlp(mdz_rheo_ctx *c, const float *X, const float *Y, int64_t n, int n_feat,
                       const mdz_mlp_train_cfg *cfg, mdz_mlp_weights *w, float *loss, int mem) {
  if (!c || !X || !Y || !cfg || !w || n < 128 || n_feat < 1 || n_feat > kMlpIn) return MDZ_EINVAL;
  if (cfg->batch < 128 || cfg->batch % 128 || cfg->epochs < 1) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  // samples with a finite target, on the host for the statistics and the order
  std::vector<float> hX, hY;
  const float *pX = X, *pY = Y;
  if (mem == MDZ_MEM_DEVICE) {
    hX.resize((size_t)n * kMlpIn);
    hY.resize((size_t)n * 2);
    CK(cudaMemcpy(hX.data(), X, hX.size() * sizeof(float), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hY.data(), Y, hY.size() * sizeof(float), cudaMemcpyDeviceToHost));
    pX = hX.data();
    pY = hY.data();
  }
  std::vector<int> keep;
  keep.reserve((size_t)n);
  for (int64_t i = 0; i < n; i++)
    if (std::isfinite(pY[i * 2]) && std::isfinite(pY[i * 2 + 1])) keep.push_back((int)i);
  if (keep.size() < 128) return MDZ_EINVAL;
  if (!(w->z_scale != 0.0f)) init_weights(w, pX, pY, n, n_feat, cfg->seed);
  w->n_feat = n_feat;
  TrainBuffers B;
  int rc = alloc_train(B);
  if (rc != MDZ_OK) return rc;
  if ((rc = put_weights(B, w)) != MDZ_OK) return rc;
  void *dXY = nullptr;
  int *dperm = nullptr;
  float *dpart = nullptr;
  const size_t xb = (size_t)n * kMlpIn * sizeof(float), yb = (size_t)n * 2 * sizeof(float);
  const size_t pb = (size_t)(cfg->batch / kMlpTile) * kGradCount * sizeof(float);  // one block per CTA of a step
  CK(cudaMalloc(&dXY, xb + yb));
  if (cudaMalloc(&dperm, keep.size() * sizeof(int)) != cudaSuccess) { cudaFree(dXY); return MDZ_ENOMEM; }
  if (cudaMalloc(&dpart, pb) != cudaSuccess || cudaMemset(dpart, 0, pb) != cudaSuccess) {
    cudaFree(dXY);
    cudaFree(dperm);
    cudaFree(dpart);
    return MDZ_ENOMEM;
  }
  CK(cudaMemcpy(dXY, pX, xb, cudaMemcpyHostToDevice));
  CK(cudaMemcpy((char *)dXY + xb, pY, yb, cudaMemcpyHostToDevice));
  MlpTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.W = B.S;
  a.part = dpart;
  a.X = (const float *)dXY;
  a.Y = (const float *)((char *)dXY + xb);
  a.perm = dperm;
  a.n_feat = n_feat;
  a.w_pl = cfg->w_pl;
  const size_t smem = mlp_step_smem();
  cudaFuncSetAttribute(k_mlp_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_mlp_pack<<<(kP2 + 255) / 256, 256, 0, c->stream>>>(a);
  std::mt19937_64 rng(cfg->seed ^ 0x9e3779b97f4a7c15ull);
  const long long nk = (long long)keep.size();
  const long long steps_per_epoch = (nk + cfg->batch - 1) / cfg->batch;
  const long long total_steps = steps_per_epoch * cfg->epochs;
  long long step = 0;
  std::vector<int> order(keep);
  rc = MDZ_OK;
  for (int e = 0; e < cfg->epochs && rc == MDZ_OK; e++) {
    std::shuffle(order.begin(), order.end(), rng);
    if (cudaMemcpyAsync(dperm, order.data(), nk * sizeof(int), cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaMemsetAsync(B.S.loss, 0, 2 * sizeof(float), c->stream) != cudaSuccess) { rc = MDZ_ECUDA; break; }
    for (long long off = 0; off < nk; off += cfg->batch, step++) {
      const long long nb = std::min<long long>(cfg->batch, nk - off);
      a.offset = off;
      a.n = off + nb;
      a.inv_batch = 1.0f / (float)nb;
      const int ctas = (int)((nb + kMlpTile - 1) / kMlpTile);
      k_mlp_step<<<(unsigned)ctas, kMlpTile, smem, c->stream>>>(a);
      k_mlp_reduce<<<(kGradCount + 255) / 256, 256, 0, c->stream>>>(a, ctas);
      MlpAdam o;
      const double frac = (double)step / (double)std::max<long long>(1, total_steps - 1);
      o.lr = (float)(cfg->lr_final + 0.5 * (cfg->lr - cfg->lr_final) * (1.0 + cos(3.14159265358979323846 * frac)));
      o.beta1 = cfg->beta1; o.beta2 = cfg->beta2; o.eps = cfg->eps;
      o.bc1 = (float)(1.0 / (1.0 - pow((double)cfg->beta1, (double)(step + 1))));
      o.bc2 = (float)(1.0 / (1.0 - pow((double)cfg->beta2, (double)(step + 1))));
      k_mlp_adam<<<(kP2 + 255) / 256, 256, 0, c->stream>>>(a, o);
    }
    if (cudaGetLastError() != cudaSuccess) { rc = MDZ_ECUDA; break; }
    float hl[2];
    if (cudaMemcpyAsync(hl, B.S.loss, sizeof(hl), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = MDZ_ECUDA; break; }
    if (loss) loss[e] = hl[0] / (float)nk;
  }
  int fault = 0;
  cudaMemcpy(&fault, B.S.fault, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(dXY);
  cudaFree(dperm);
  cudaFree(dpart);
  if (rc != MDZ_OK) return rc;
  if (fault) return MDZ_ECUDA;
  return get_weights(B, w);
}

int mdz_rheo_mlp_predict(mdz_rheo_ctx *c, const mdz_mlp_weights *w, const float *X, float *Yp, int64_t n, int mem) {
  if (!c || !w || !X || !Yp || n < 0) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  CK(cudaSetDevice(c->device));
  TrainBuffers B;
  int rc = alloc_train(B);
  if (rc != MDZ_OK) return rc;
  if ((rc = put_weights(B, w)) != MDZ_OK) return rc;
  const float *dX = X;
  float *dY = Yp;
  void *tmp = nullptr;
  const size_t xb = (size_t)n * kMlpIn * sizeof(float), yb = (size_t)n * 2 * sizeof(float);
  if (mem == MDZ_MEM_HOST) {
    CK(cudaMalloc(&tmp, xb + yb));
    CK(cudaMemcpy(tmp, X, xb, cudaMemcpyHostToDevice));
    dX = (const float *)tmp;
    dY = (float *)((char *)tmp + xb);
  }
  MlpTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.W = B.S;
  a.X = dX;
  a.n = n;
  a.n_feat = w->n_feat;
  k_mlp_pack<<<(kP2 + 255) / 256, 256, 0, c->stream>>>(a);
  const size_t smem = mlp_predict_smem();
  cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long tiles = (n + kMlpTile - 1) / kMlpTile;
  const int grid = (int)std::min<long long>(tiles, (long long)c->sms * 2);
  k_mlp_predict<<<grid, kMlpTile, smem, c->stream>>>(a, dY);
  rc = (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(c->stream) == cudaSuccess) ? MDZ_OK : MDZ_ECUDA;
  if (rc == MDZ_OK && mem == MDZ_MEM_HOST) rc = (cudaMemcpy(Yp, dY, yb, cudaMemcpyDeviceToHost) == cudaSuccess) ? MDZ_OK : MDZ_ECUDA;
  int fault = 0;
  cudaMemcpy(&fault, B.S.fault, sizeof(int), cudaMemcpyDeviceToHost);
  if (tmp) cudaFree(tmp);
  return (rc == MDZ_OK && fault) ? MDZ_ECUDA : rc;
}


int mdz_rheo_mlp_gradient(mdz_rheo_ctx *c, const mdz_mlp_weights *w, const float *X, const float *Y, int64_t n,
                          float w_pl, mdz_mlp_weights *grad, float *loss, int mem) {
  if (!c || !w || !X || !Y || !grad || n < 1) return MDZ_EINVAL;
  if (mem != MDZ_MEM_HOST && mem != MDZ_MEM_DEVICE) return MDZ_EINVAL;
  CK(cudaSetDevice(c->device));
  TrainBuffers B;
  int rc = alloc_train(B);
  if (rc != MDZ_OK) return rc;
  if ((rc = put_weights(B, w)) != MDZ_OK) return rc;
  const float *dX = X, *dY = Y;
  void *tmp = nullptr;
  const size_t xb = (size_t)n * kMlpIn * sizeof(float), yb = (size_t)n * 2 * sizeof(float);
  if (mem == MDZ_MEM_HOST) {
    CK(cudaMalloc(&tmp, xb + yb));
    CK(cudaMemcpy(tmp, X, xb, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((char *)tmp + xb, Y, yb, cudaMemcpyHostToDevice));
    dX = (const float *)tmp;
    dY = (const float *)((char *)tmp + xb);
  }
  const long long ctas = (n + kMlpTile - 1) / kMlpTile;
  const size_t pb = (size_t)ctas * kGradCount * sizeof(float);
  float *dpart = nullptr;
  if (ctas > 0x7fffffffLL || cudaMalloc(&dpart, pb) != cudaSuccess || cudaMemset(dpart, 0, pb) != cudaSuccess) {
    cudaFree(dpart);
    if (tmp) cudaFree(tmp);
    return MDZ_ENOMEM;
  }
  MlpTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.W = B.S;
  a.part = dpart;
  a.X = dX;
  a.Y = dY;
  a.n = n;
  a.n_feat = w->n_feat;
  a.inv_batch = 1.0f / (float)n;
  a.w_pl = w_pl;
  k_mlp_pack<<<(kP2 + 255) / 256, 256, 0, c->stream>>>(a);
  const size_t smem = mlp_step_smem();
  cudaFuncSetAttribute(k_mlp_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_mlp_step<<<(unsigned)ctas, kMlpTile, smem, c->stream>>>(a);
  k_mlp_reduce<<<(kGradCount + 255) / 256, 256, 0, c->stream>>>(a, (int)ctas);
  rc = (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(c->stream) == cudaSuccess) ? MDZ_OK : MDZ_ECUDA;
  cudaFree(dpart);
  if (tmp) cudaFree(tmp);
  if (rc != MDZ_OK) return rc;
  int fault = 0;
  CK(cudaMemcpy(&fault, B.S.fault, sizeof(int), cudaMemcpyDeviceToHost));
  if (fault) return MDZ_ECUDA;
  CK(cudaMemcpy(grad->W1, B.S.gW1, kP1 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad->W2, B.S.gW2, kP2 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad->W3, B.S.gW3, kP3 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad->b1, B.S.gb1, 64 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad->b2, B.S.gb2, 64 * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad->b3, B.S.gb3, 2 * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) CK(cudaMemcpy(loss, B.S.loss, 2 * sizeof(float), cudaMemcpyDeviceToHost));
  return MDZ_OK;
}

}  // extern "C"
