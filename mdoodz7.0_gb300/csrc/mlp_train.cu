// mlp_train.cu -- training and batch inference of the warm-start perceptron on tcgen05.
//
// k_mlp_step: one CTA = one tile of 128 samples.  Forward (X W1^T -> ReLU -> W2 -> ReLU
// -> W3) and the activation backward (dY W3, dZ2 W2) are M=128 tcgen05 GEMMs with the
// sample as the row; the weight gradients reduce over the 128 samples as M=64 GEMMs
// (rows = the layer's output or input units, K = samples) whose operands are the same
// activations stored transposed.  Bias gradients and the loss are warp reductions.
// Gradients are added to FP32 accumulators with one atomic per element and CTA.
// k_mlp_adam: Adam on the FP32 master weights, then re-packs the BF16 K-major tiles
// (W1, W2, W3 and the transposes W2^T, W3^T used by the backward pass).
// k_mlp_predict: forward only, for evaluation on held-out data.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp_train.cuh"
#include "umma.cuh"

namespace mdz {

namespace {

constexpr int T = kMlpTile;  // samples per CTA tile

struct TrainShared {
  // B operands (weights) of the forward and of the activation backward
  alignas(128) unsigned char W1[kMlpHid * kMlpIn * 2];    // [64 hid][16 in]
  alignas(128) unsigned char W2[kMlpHid * kMlpHid * 2];   // [64 out][64 in]
  alignas(128) unsigned char W3[kMlpOut * kMlpHid * 2];   // [16 out][64 in]
  alignas(128) unsigned char W2t[kMlpHid * kMlpHid * 2];  // [64 in][64 out]
  alignas(128) unsigned char W3t[kMlpHid * kMlpOut * 2];  // [64 in][16 out]
  // A operands (sample-major)
  alignas(128) unsigned char X[T * kMlpIn * 2];
  alignas(128) unsigned char A1[T * kMlpHid * 2];
  alignas(128) unsigned char A2[T * kMlpHid * 2];
  alignas(128) unsigned char dY[T * kMlpOut * 2];
  alignas(128) unsigned char dZ2[T * kMlpHid * 2];
  // transposed tiles (K = sample) for the weight gradients
  alignas(128) unsigned char Xt[kMlpIn * T * 2];
  alignas(128) unsigned char A1t[kMlpHid * T * 2];
  alignas(128) unsigned char A2t[kMlpHid * T * 2];
  alignas(128) unsigned char dYt[kMlpOut * T * 2];
  alignas(128) unsigned char dZ2t[kMlpHid * T * 2];
  alignas(128) unsigned char dZ1t[kMlpHid * T * 2];
  float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
  float red[4][kMlpHid];  // per-warp partial bias gradients
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  int fault;
  uint32_t fault_parity;  // the mbarrier phase a wait gave up on (drained before TMEM is freed)
};

constexpr uint32_t kTrainCols = 256;
// TMEM column map
constexpr int C_D1 = 0, C_D2 = 64, C_D3 = 0, C_DH2 = 0, C_DH1 = 64, C_GW3 = 128, C_GW1 = 160, C_GW2 = 192;

__device__ __forceinline__ void sync_mma() {
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// Issue D[tcol] = A * B^T, A = M x K tile, B = N x K tile (both K-major), from thread 0.
__device__ __forceinline__ void issue(TrainShared &S, int M, int N, int K, uint32_t tcol, const unsigned char *At,
                                      const unsigned char *Bt) {
  if (threadIdx.x == 0 && !S.fault) {
    const uint32_t idesc = umma::idesc_bf16_f32(M, N);
    const uint32_t a0 = umma::smem_u32(At), b0 = umma::smem_u32(Bt);
    for (int kk = 0; kk < K / 16; kk++)
      umma::mma_bf16(S.tmem + tcol, umma::smem_desc(a0 + kk * 256, 128, 16 * K),
                     umma::smem_desc(b0 + kk * 256, 128, 16 * K), idesc, kk > 0);
  }
}

// One commit for every MMA issued since the last, then the CTA waits for them.
__device__ __forceinline__ void complete(TrainShared &S, uint32_t &phase) {
  if (threadIdx.x == 0 && !S.fault) umma::commit(&S.mbar);
  if (!S.fault && !umma::mbar_wait(&S.mbar, phase)) {  // every writer stores the same values
    S.fault_parity = phase;
    S.fault = 1;
  }
  phase ^= 1;
  umma::fence_after_sync();
}

__device__ __forceinline__ void gemm(TrainShared &S, int M, int N, int K, uint32_t tcol, const unsigned char *At,
                                     const unsigned char *Bt, uint32_t &phase) {
  issue(S, M, N, K, tcol, At, Bt);
  complete(S, phase);
}

__device__ __forceinline__ void put_bf16(unsigned char *tile, int r, int k, int K, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(tile + umma::kmajor_offset(r, k, K)) = __float2bfloat16_rn(v);
}

// Row `row` of an M=64 accumulator is held by thread 32*(row/16) + row%16.
__device__ __forceinline__ int m64_row_of_thread(int t) { return ((t & 31) < 16) ? (t >> 5) * 16 + (t & 31) : -1; }

__device__ __forceinline__ void load_weights(TrainShared &S, const MlpTrainState &W) {
  const int t = threadIdx.x;
  copy16(S.W1, W.tW1, sizeof(S.W1), t, blockDim.x);
  copy16(S.W2, W.tW2, sizeof(S.W2), t, blockDim.x);
  copy16(S.W3, W.tW3, sizeof(S.W3), t, blockDim.x);
  copy16(S.W2t, W.tW2t, sizeof(S.W2t), t, blockDim.x);
  copy16(S.W3t, W.tW3t, sizeof(S.W3t), t, blockDim.x);
  if (t < kMlpHid) { S.b1[t] = W.b1[t]; S.b2[t] = W.b2[t]; }
  if (t < kMlpOut) S.b3[t] = (t < 2) ? W.b3[t] : 0.0f;
}

// Sum v over the 128 threads of the CTA for each of n columns; thread c < n gets column c.
__device__ __forceinline__ float block_colsum(TrainShared &S, const float *v, int n, int c_out) {
  const int t = threadIdx.x, w = t >> 5, l = t & 31;
  for (int c = 0; c < n; c++) {
    float x = v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (l == 0) S.red[w][c] = x;
  }
  __syncthreads();
  float r = 0.0f;
  if (c_out < n) r = S.red[0][c_out] + S.red[1][c_out] + S.red[2][c_out] + S.red[3][c_out];
  __syncthreads();
  return r;
}

}  // namespace

// Forward + backward of one tile per CTA; the CTA's gradient sums go to its block of
// a.part (k_mlp_reduce adds the blocks up).
__global__ void __launch_bounds__(128) k_mlp_step(const __grid_constant__ MlpTrainArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TrainShared &S = *reinterpret_cast<TrainShared *>(smem_raw);
  const int t = threadIdx.x, w = t >> 5;
  const MlpTrainState &W = a.W;
  float *gp = a.part + (size_t)blockIdx.x * kGradCount;
  load_weights(S, W);
  if (t == 0) { umma::mbar_init(&S.mbar, 1); S.fault = 0; S.fault_parity = 0; }
  if (w == 0) umma::tmem_alloc(&S.tmem, kTrainCols);
  sync_mma();
  uint32_t phase = 0;
  const long long base = a.offset + (long long)blockIdx.x * T;
  const long long s_idx = base + t;
  const bool valid = s_idx < a.n;
  const long long src = valid ? (a.perm ? (long long)a.perm[s_idx] : s_idx) : 0;
  // ---- inputs: normalised features (zero rows for padding samples)
  float x[kMlpIn];
#pragma unroll
  for (int j = 0; j < kMlpIn; j++)
    x[j] = (valid && j < a.n_feat) ? (a.X[src * kMlpIn + j] - W.x_shift[j]) * W.x_scale[j] : 0.0f;
  const float y0 = valid ? (a.Y[src * 2 + 0] - W.z_shift) / W.z_scale : 0.0f;
  const float y1 = valid ? a.Y[src * 2 + 1] : 0.0f;
  store_row16(S.X, t, 0, kMlpIn, x);
#pragma unroll
  for (int j = 0; j < kMlpIn; j++) put_bf16(S.Xt, j, t, T, x[j]);
  sync_mma();
  // ---- forward
  gemm(S, T, kMlpHid, kMlpIn, C_D1, S.X, S.W1, phase);
  for (int c = 0; c < kMlpHid; c += 16) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_D1 + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + S.b1[c + i], 0.0f);
    store_row16(S.A1, t, c, kMlpHid, v);
#pragma unroll
    for (int i = 0; i < 16; i++) put_bf16(S.A1t, c + i, t, T, v[i]);
  }
  sync_mma();
  gemm(S, T, kMlpHid, kMlpHid, C_D2, S.A1, S.W2, phase);
  for (int c = 0; c < kMlpHid; c += 16) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_D2 + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + S.b2[c + i], 0.0f);
    store_row16(S.A2, t, c, kMlpHid, v);
#pragma unroll
    for (int i = 0; i < 16; i++) put_bf16(S.A2t, c + i, t, T, v[i]);
  }
  sync_mma();
  gemm(S, T, kMlpOut, kMlpHid, C_D3, S.A2, S.W3, phase);
  float dy[kMlpOut];
  {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_D3), v);
    const float o0 = v[0] + S.b3[0], o1 = v[1] + S.b3[1];
    const float e0 = valid ? o0 - y0 : 0.0f, e1 = valid ? o1 - y1 : 0.0f;
#pragma unroll
    for (int i = 0; i < kMlpOut; i++) dy[i] = 0.0f;
    dy[0] = 2.0f * e0 * a.inv_batch;
    dy[1] = 2.0f * a.w_pl * e1 * a.inv_batch;
    float l2[2] = {e0 * e0, a.w_pl * e1 * e1};
    const float loss = block_colsum(S, l2, 2, t);
    if (t < 2) atomicAdd(&W.loss[t], loss);
  }
  store_row16(S.dY, t, 0, kMlpOut, dy);
#pragma unroll
  for (int j = 0; j < kMlpOut; j++) put_bf16(S.dYt, j, t, T, dy[j]);
  {
    const float gb = block_colsum(S, dy, 2, t);
    if (t < 2) gp[kGradB3 + t] = gb;
  }
  sync_mma();
  // ---- backward through layer 3: dH2 = dY W3, dZ2 = dH2 * (A2 > 0); with it, in the same
  // commit group, layer 3's weight gradient (its operands are ready: A2 and dY)
  issue(S, T, kMlpHid, kMlpOut, C_DH2, S.dY, S.W3t);
  issue(S, 64, kMlpOut, T, C_GW3, S.A2t, S.dYt);   // gW3^T[h][o]
  complete(S, phase);
  float gsum[kMlpHid];
  for (int c = 0; c < kMlpHid; c += 16) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_DH2 + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const float a2 = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(
          S.A2 + umma::kmajor_offset(t, c + i, kMlpHid)));
      v[i] = (a2 > 0.0f) ? v[i] : 0.0f;
      gsum[c + i] = v[i];
    }
    store_row16(S.dZ2, t, c, kMlpHid, v);
#pragma unroll
    for (int i = 0; i < 16; i++) put_bf16(S.dZ2t, c + i, t, T, v[i]);
  }
  {
    const float gb = block_colsum(S, gsum, kMlpHid, t);
    if (t < kMlpHid) gp[kGradB2 + t] = gb;
  }
  sync_mma();
  // ---- backward through layer 2: dH1 = dZ2 W2, dZ1 = dH1 * (A1 > 0); with it layer 2's
  // weight gradient (dZ2 and A1 are ready)
  issue(S, T, kMlpHid, kMlpHid, C_DH1, S.dZ2, S.W2t);
  issue(S, 64, kMlpHid, T, C_GW2, S.dZ2t, S.A1t);  // gW2[o][i]
  complete(S, phase);
  for (int c = 0; c < kMlpHid; c += 16) {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_DH1 + c), v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const float a1 = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(
          S.A1 + umma::kmajor_offset(t, c + i, kMlpHid)));
      v[i] = (a1 > 0.0f) ? v[i] : 0.0f;
      gsum[c + i] = v[i];
      put_bf16(S.dZ1t, c + i, t, T, v[i]);
    }
  }
  {
    const float gb = block_colsum(S, gsum, kMlpHid, t);
    if (t < kMlpHid) gp[kGradB1 + t] = gb;
  }
  sync_mma();
  // ---- weight gradients, reduction over the 128 samples (M = 64 tiles, K = samples);
  // layers 3 and 2 were issued with the backward GEMMs above, in the TMEM columns that
  // no later GEMM writes
  gemm(S, 64, kMlpIn, T, C_GW1, S.dZ1t, S.Xt, phase);    // gW1[h][f]
  const int row = m64_row_of_thread(t);
  {
    float v[16];
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_GW3), v);
    if (row >= 0) { gp[kGradW3 + 0 * kMlpHid + row] = v[0]; gp[kGradW3 + 1 * kMlpHid + row] = v[1]; }
    for (int c = 0; c < kMlpHid; c += 16) {
      umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_GW2 + c), v);
      if (row >= 0)
        for (int i = 0; i < 16; i++) gp[kGradW2 + row * kMlpHid + c + i] = v[i];
    }
    umma::tmem_ld16(umma::tmem_addr(S.tmem, w, C_GW1), v);
    if (row >= 0)
      for (int i = 0; i < a.n_feat; i++) gp[kGradW1 + row * kMlpIn + i] = v[i];
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  // after a wait that gave up, the group it waited for may still be in flight (no MMA is
  // issued after a fault, so at most one): wait for it, bounded, before freeing TMEM
  if (t == 0 && S.fault) umma::mbar_wait(&S.mbar, S.fault_parity);
  __syncthreads();
  if (w == 0) umma::tmem_free(S.tmem, kTrainCols);
  if (t == 0 && S.fault) atomicExch(W.fault, 1);
}

namespace {

__device__ __forceinline__ float adam_update(float &p, float &m, float &v, float g, const MlpAdam &o) {
  m = o.beta1 * m + (1.0f - o.beta1) * g;
  v = o.beta2 * v + (1.0f - o.beta2) * g * g;
  const float mh = m * o.bc1, vh = v * o.bc2;
  p -= o.lr * mh / (sqrtf(vh) + o.eps);
  return p;
}

__device__ __forceinline__ void put_tile(uint4 *tile, int r, int k, int K, float v) {
  put_bf16(reinterpret_cast<unsigned char *>(tile), r, k, K, v);
}

}  // namespace

// The step's gradient: the CTAs' blocks of a.part added in CTA order (deterministic).
__global__ void k_mlp_reduce(const __grid_constant__ MlpTrainArgs a, int ctas) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kGradCount) return;
  float s = 0.0f;
  for (int c = 0; c < ctas; c++) s += a.part[(size_t)c * kGradCount + i];
  const MlpTrainState &W = a.W;
  if (i < kGradW2) W.gW1[i - kGradW1] = s;
  else if (i < kGradW3) W.gW2[i - kGradW2] = s;
  else if (i < kGradB1) W.gW3[i - kGradW3] = s;
  else if (i < kGradB2) W.gb1[i - kGradB1] = s;
  else if (i < kGradB3) W.gb2[i - kGradB2] = s;
  else W.gb3[i - kGradB3] = s;
}

// One Adam step over every parameter, then the BF16 tiles; zeroes the gradients.
__global__ void k_mlp_adam(const __grid_constant__ MlpTrainArgs a, const __grid_constant__ MlpAdam o) {
  const MlpTrainState &W = a.W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // W1: [64][16] (features >= n_feat stay 0)
  if (i < kMlpHid * kMlpIn) {
    const int h = i / kMlpIn, f = i % kMlpIn;
    float p = W.W1[i];
    if (f < a.n_feat) p = adam_update(W.W1[i], W.mW1[i], W.vW1[i], W.gW1[i], o);
    W.gW1[i] = 0.0f;
    put_tile(W.tW1, h, f, kMlpIn, p);
  }
  // W2: [64][64]
  if (i < kMlpHid * kMlpHid) {
    const int r = i / kMlpHid, c = i % kMlpHid;
    const float p = adam_update(W.W2[i], W.mW2[i], W.vW2[i], W.gW2[i], o);
    W.gW2[i] = 0.0f;
    put_tile(W.tW2, r, c, kMlpHid, p);
    put_tile(W.tW2t, c, r, kMlpHid, p);
  }
  // W3: [2][64] (rows 2..15 of the tiles stay 0)
  if (i < 2 * kMlpHid) {
    const int r = i / kMlpHid, c = i % kMlpHid;
    const float p = adam_update(W.W3[i], W.mW3[i], W.vW3[i], W.gW3[i], o);
    W.gW3[i] = 0.0f;
    put_tile(W.tW3, r, c, kMlpHid, p);
    put_tile(W.tW3t, c, r, kMlpOut, p);
  }
  if (i < kMlpHid) {
    adam_update(W.b1[i], W.mb1[i], W.vb1[i], W.gb1[i], o);
    adam_update(W.b2[i], W.mb2[i], W.vb2[i], W.gb2[i], o);
    W.gb1[i] = 0.0f;
    W.gb2[i] = 0.0f;
  }
  if (i < 2) {
    adam_update(W.b3[i], W.mb3[i], W.vb3[i], W.gb3[i], o);
    W.gb3[i] = 0.0f;
  }
}

// Pack the FP32 master weights into the BF16 tiles (no update).
__global__ void k_mlp_pack(const __grid_constant__ MlpTrainArgs a) {
  const MlpTrainState &W = a.W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kMlpHid * kMlpIn) put_tile(W.tW1, i / kMlpIn, i % kMlpIn, kMlpIn, W.W1[i]);
  if (i < kMlpHid * kMlpHid) {
    put_tile(W.tW2, i / kMlpHid, i % kMlpHid, kMlpHid, W.W2[i]);
    put_tile(W.tW2t, i % kMlpHid, i / kMlpHid, kMlpHid, W.W2[i]);
  }
  if (i < kMlpOut * kMlpHid) {
    const int r = i / kMlpHid, c = i % kMlpHid;
    const float p = (r < 2) ? W.W3[r * kMlpHid + c] : 0.0f;
    put_tile(W.tW3, r, c, kMlpHid, p);
    put_tile(W.tW3t, c, r, kMlpOut, p);
  }
}

// Forward only: Y[s] = (z, plastic indicator) for n samples of raw features X.
__global__ void __launch_bounds__(128) k_mlp_predict(const __grid_constant__ MlpTrainArgs a, float *Yp) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  MlpShared &S = *reinterpret_cast<MlpShared *>(smem_raw);
  MlpDevice d;
  d.W1 = a.W.tW1; d.W2 = a.W.tW2; d.W3 = a.W.tW3; d.b1 = a.W.b1; d.b2 = a.W.b2; d.b3 = a.W.b3;
  mlp_begin(S, d);
  uint32_t phase = 0;
  const long long ntiles = (a.n + T - 1) / T;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long s = tile * T + threadIdx.x;
    float x[kMlpIn];
#pragma unroll
    for (int j = 0; j < kMlpIn; j++)
      x[j] = (s < a.n && j < a.n_feat) ? (a.X[s * kMlpIn + j] - a.W.x_shift[j]) * a.W.x_scale[j] : 0.0f;
    float y[2];
    mlp_forward(S, x, y, phase, 1u << 24);
    if (s < a.n) {
      Yp[s * 2 + 0] = y[0] * a.W.z_scale + a.W.z_shift;
      Yp[s * 2 + 1] = y[1];
    }
  }
  mlp_end(S);
  if (threadIdx.x == 0 && S.fault) atomicExch(a.W.fault, 1);
}

size_t mlp_step_smem() { return sizeof(TrainShared); }
size_t mlp_predict_smem() { return sizeof(MlpShared); }

}  // namespace mdz
