// mlp.cuh -- the learned warm start of the local visco-elastic solve.
//
// A 10(12) -> 64 -> 64 -> 2 perceptron with BF16 weights and activations and FP32
// accumulation predicts, for one (node, phase), z = ln(eta_up / eta_ve): how far below
// the reference's start point eta_up (the smallest isolated viscosity) the converged
// visco-elastic viscosity lies, and a plastic indicator.  It runs on the 5th-generation
// tensor cores (tcgen05): one CTA of 128 threads evaluates 128 items at once, thread t
// owning row t; weights and activations are K-major BF16 tiles in shared memory and the
// FP32 accumulators live in tensor memory (umma.cuh).
//
// The guess is refined by a few Newton steps in FP32 on the normalised residual
//     r(s) = 1 - a s - sum_k exp(n_k ln s + c_k),   s = eta / eta_up,
// where every quantity is O(1) (a = eta_up A / Eii, c_k = n_k ln(eta_up / eta_p) + nc_k).
// The FP64 Newton then starts from s eta_up and iterates exactly as the plain solver to
// the same residual tolerance, so the learned part only decides where it starts.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "rheo_device.cuh"
#include "umma.cuh"

namespace mdz {

constexpr int kMlpIn = 16;   // feature width (10 used, 12 for the anisotropic path), padded for the MMA K
constexpr int kMlpHid = 64;
constexpr int kMlpOut = 16;  // output width (2 used), padded for the MMA N
constexpr int kMlpTile = 128;
constexpr int kFeatIso = 10, kFeatAniso = 12;

// Start of the local solve from the network's output: s = eta_ve / eta_up = exp(-z).
// eta_up is an upper bound of the root that is exact where one mechanism dominates, and
// the FP32 steps from it stop at once there; a predicted z below the network's typical
// error (about 1e-3 on held-out data) carries no information, so such items keep eta_up.
constexpr float kWarmMinZ = 2e-3f;
__device__ __forceinline__ float warm_start_point(float y, float z_scale, float z_shift) {
  const float z = fmaxf(y * z_scale + z_shift, 0.0f);
  return (z > kWarmMinZ) ? __expf(-z) : 1.0f;
}

// Device-side weights: BF16 copies already in the K-major tile byte order of umma.cuh
// (B operands: rows = output units, K = input units), FP32 biases, feature and output
// normalisation.
struct MlpDevice {
  const uint4 *W1, *W2, *W3;  // 64x16, 64x64, 16x64 tiles
  const uint2 *F1, *F2, *F3;  // the same weights as the per-warp MMA's B fragments (mlp_warp.cuh)
  const float *b1, *b2, *b3;
  float x_shift[kMlpIn], x_scale[kMlpIn];
  float z_shift, z_scale;
  int n_feat;
  int polish_iters;            // start descriptor after the guess: FP32 Newton steps | MDZ_START_DD
  unsigned poll_limit;         // tcgen05 completion polls before a wait gives up
};

struct MlpShared {
  alignas(128) unsigned char W1[kMlpHid * kMlpIn * 2];
  alignas(128) unsigned char W2[kMlpHid * kMlpHid * 2];
  alignas(128) unsigned char W3[kMlpOut * kMlpHid * 2];
  alignas(128) unsigned char X[kMlpTile * kMlpIn * 2];
  alignas(128) unsigned char H[kMlpTile * kMlpHid * 2];
  float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  int fault;              // an MMA completion wait gave up: stop issuing, keep the plain start
  uint32_t fault_parity;  // the mbarrier phase that wait gave up on (drained before TMEM is freed)
};

constexpr uint32_t kMlpTmemCols = 128;  // D1 cols 0..63, D2 64..127, D3 reuses 0..15

__device__ __forceinline__ void copy16(void *dst, const void *src, int bytes, int t, int nt) {
  uint4 *d = (uint4 *)dst;
  const uint4 *s = (const uint4 *)src;
  for (int i = t; i < bytes / 16; i += nt) d[i] = __ldg(&s[i]);
}

// Block-wide set-up: weights to shared memory, TMEM allocation (warp 0), mbarrier.
__device__ __forceinline__ void mlp_begin(MlpShared &S, const MlpDevice &W) {
  const int t = threadIdx.x;
  copy16(S.W1, W.W1, sizeof(S.W1), t, blockDim.x);
  copy16(S.W2, W.W2, sizeof(S.W2), t, blockDim.x);
  copy16(S.W3, W.W3, sizeof(S.W3), t, blockDim.x);
  if (t < kMlpHid) { S.b1[t] = W.b1[t]; S.b2[t] = W.b2[t]; }
  if (t < kMlpOut) S.b3[t] = W.b3[t];
  if (t == 0) { umma::mbar_init(&S.mbar, 1); S.fault = 0; S.fault_parity = 0; }
  if ((t >> 5) == 0) umma::tmem_alloc(&S.tmem, kMlpTmemCols);
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// Block-wide tear-down.  After a wait that gave up, the MMA group it waited for may still
// be in flight: thread 0 waits (again bounded) for that phase before TMEM is freed.  At
// most one group is outstanding then, as no MMA is issued after a fault.
__device__ __forceinline__ void mlp_end(MlpShared &S) {
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (threadIdx.x == 0 && S.fault) umma::mbar_wait(&S.mbar, S.fault_parity);
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) umma::tmem_free(S.tmem, kMlpTmemCols);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Store 16 consecutive values v[0..15] of row r, columns k0..k0+15, into a K-major tile.
__device__ __forceinline__ void store_row16(unsigned char *tile, int r, int k0, int K, const float *v) {
  uint4 a, b;
  a.x = pack_bf16x2(v[0], v[1]); a.y = pack_bf16x2(v[2], v[3]); a.z = pack_bf16x2(v[4], v[5]); a.w = pack_bf16x2(v[6], v[7]);
  b.x = pack_bf16x2(v[8], v[9]); b.y = pack_bf16x2(v[10], v[11]); b.z = pack_bf16x2(v[12], v[13]); b.w = pack_bf16x2(v[14], v[15]);
  *reinterpret_cast<uint4 *>(tile + umma::kmajor_offset(r, k0, K)) = a;
  *reinterpret_cast<uint4 *>(tile + umma::kmajor_offset(r, k0 + 8, K)) = b;
}

__device__ __forceinline__ void mlp_sync_for_mma() {
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// Issue D[cols] = A(tile, K) * B^T over K in steps of 16, then wait for completion.
__device__ __forceinline__ void mlp_layer(MlpShared &S, uint32_t tcol, const unsigned char *Atile,
                                          const unsigned char *Btile, int K, int N, uint32_t &phase,
                                          uint32_t limit) {
  if (threadIdx.x == 0 && !S.fault) {
    const uint32_t idesc = umma::idesc_bf16_f32(kMlpTile, N);
    const uint32_t a0 = umma::smem_u32(Atile), b0 = umma::smem_u32(Btile);
    for (int kk = 0; kk < K / 16; kk++)
      umma::mma_bf16(S.tmem + tcol, umma::smem_desc(a0 + kk * 256, 128, 16 * K),
                     umma::smem_desc(b0 + kk * 256, 128, 16 * K), idesc, kk > 0);
    umma::commit(&S.mbar);
  }
  if (!S.fault) {
    if (!umma::mbar_wait(&S.mbar, phase, limit)) {  // benign race: every writer stores the same values
      S.fault_parity = phase;
      S.fault = 1;
    }
  }
  phase ^= 1;
  umma::fence_after_sync();
}

// Hidden-layer epilogue: TMEM columns tcol..tcol+63 of this thread's row, + bias, ReLU,
// back to the H tile as BF16.
__device__ __forceinline__ void mlp_hidden_epilogue(MlpShared &S, uint32_t tcol, const float *bias) {
  const int t = threadIdx.x, w = t >> 5;
#pragma unroll
  for (int c = 0; c < kMlpHid; c += 16) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, tcol + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + bias[c + i], 0.0f);
    store_row16(S.H, t, c, kMlpHid, v);
  }
}

// Forward pass of the whole CTA tile; every thread of the block must call it.
// x: this thread's (already normalised) features, kMlpIn wide.  Returns out[0..1].
// `limit`: completion polls per layer before giving up.
__device__ __forceinline__ void mlp_forward(MlpShared &S, const float *x, float *out, uint32_t &phase,
                                            uint32_t limit) {
  const int t = threadIdx.x, w = t >> 5;
  store_row16(S.X, t, 0, kMlpIn, x);
  mlp_sync_for_mma();
  // TMEM is read only by warps none of whose lanes has seen a wait give up (the decision is
  // warp-uniform, as tcgen05.ld is a warp-wide instruction): after a give-up the MMA group
  // may still be writing those columns
  mlp_layer(S, 0, S.X, S.W1, kMlpIn, kMlpHid, phase, limit);
  if (__all_sync(0xffffffffu, S.fault == 0)) mlp_hidden_epilogue(S, 0, S.b1);
  mlp_sync_for_mma();
  mlp_layer(S, 64, S.H, S.W2, kMlpHid, kMlpHid, phase, limit);
  if (__all_sync(0xffffffffu, S.fault == 0)) mlp_hidden_epilogue(S, 64, S.b2);
  mlp_sync_for_mma();
  mlp_layer(S, 0, S.H, S.W3, kMlpHid, kMlpOut, phase, limit);
  out[0] = out[1] = 0.0f;
  if (__all_sync(0xffffffffu, S.fault == 0)) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, 0), v);
    out[0] = v[0] + S.b3[0];
    out[1] = v[1] + S.b3[1];
  }
  umma::fence_before_sync();
  if (S.fault) { out[0] = 0.0f; out[1] = 0.0f; }
}

// Features of one (node, phase), in physical units so one network serves any scaling
// and any material table: strain-rate invariant, temperature, pressure, grain size,
// the isolated viscosities relative to the start point, and the stress memory.  Every
// double enters by truncation to FP32 on the integer pipe (f32_trunc) and the arithmetic
// is FP32, so the features cost the FP64 pipe nothing; their logarithms come from the
// FP64 ones the solve already carries (ln Eii, ln eta_up, ln(1/eta_k), ln eta_el).
__device__ __forceinline__ void warm_features(const ModelConst &M, const NodeIn &in, const NodeCtx &c,
                                              const IsoState &S, bool aniso, float *f) {
  const float lo = -40.0f;
  const float ln_up = f32_trunc(S.ln_eta_up);
  f[0] = f32_trunc(c.lnEii) + __logf(f32_trunc(M.scale_E));
  f[1] = 1000.0f * f32_trunc(c.invT) / f32_trunc(M.scale_T);
  f[2] = f32_trunc(in.P) * f32_trunc(M.scale_S) * 1e-9f;
  f[3] = fp64_gt(in.d, 0.0) ? __logf(f32_trunc(in.d) * f32_trunc(M.scale_L)) : -20.0f;
  f[4] = c.elastic ? f32_trunc(c.ln_eta_el) - ln_up : 0.0f;
  // ln(eta_up / eta_k); inactive laws carry ln(1/eta_k) = -inf, which truncates to -FLT_MAX
#pragma unroll
  for (int k = 0; k < K_COUNT; k++) f[5 + k] = fmaxf(ln_up + f32_trunc(S.L.ln_inv[k]), lo);
  f[8] = (S.L.mech & F_CST) ? fmaxf(ln_up - __logf(f32_trunc(S.eta_cst)), lo) : lo;
  // stress memory: the share of the effective strain rate carried by the old stress
  const float t0 = f32_trunc(in.Txx0), t1 = f32_trunc(in.Tzz0), t2 = f32_trunc(in.Txz0);
  const float T0 = sqrtf(0.5f * (t0 * t0 + t1 * t1 + (t0 + t1) * (t0 + t1)) + t2 * t2);
  f[9] = c.elastic ? T0 * f32_trunc(c.inv_eta_el) * 0.5f / f32_trunc(c.Eii) : 0.0f;
  if (aniso) {
    f[10] = 2.0f * f32_trunc(in.lx2) - 1.0f;   // cos(2 theta)
    f[11] = __logf(f32_trunc(in.ani_fac));     // ln(delta)
  }
}

}  // namespace mdz
