// mlp_warp.cuh -- the learned warm start evaluated by each warp on its own 32 nodes.
//
// Inside the sweep every thread owns one node and runs that node's phases one after the
// other.  The CTA-wide tcgen05 form of the network (mlp.cuh) must gather all 128 threads
// of a CTA at every layer of every phase (CTA barriers and mbarrier waits inside the
// phase loop); this form needs only the 32 lanes of one warp, which reach the network at
// the same phase because the phase loop is uniform.  It runs on the warp-level BF16
// tensor-core instruction (mma.sync m16n8k16, FP32 accumulation): a warp's 32 items are
// two 16-row tiles, the 10(12) -> 64 -> 64 -> 2 network is 2 x (8 + 32 + 4) MMAs, and
// each layer's accumulator fragments are already the next layer's A operand (the
// m16n8 accumulator of two adjacent column tiles is the m16k16 operand layout), so the
// activations never leave registers.  Weights sit in shared memory in fragment order,
// loaded once per CTA; the features pass through a 1.1 KB per-warp buffer to reach the
// operand layout; no barrier beyond __syncwarp is taken after the kernel's start.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.cuh"

namespace mdz {

constexpr int kWarpMlpWarps = 4;  // warps per CTA of the warm sweep (128 threads)
// B-operand fragments: [(n_tile * k_chunks + k_chunk) * 32 + lane] = two bf16x2 words
constexpr int kF1 = 8 * 1 * 32, kF2 = 8 * 4 * 32, kF3 = 1 * 4 * 32;

struct MlpWarpShared {
  uint2 F1[kF1], F2[kF2], F3[kF3];
  float b1[kMlpHid], b2[kMlpHid], b3[8];
  uint32_t X[kWarpMlpWarps][32 * 9];  // per warp: 32 rows of 16 bf16 features, row stride 9 words
  float Z[kWarpMlpWarps][32];
};

// Block-wide load of the weights (every thread of the block calls it once, at the start).
__device__ __forceinline__ void mlp_warp_load(MlpWarpShared &S, const MlpDevice &W) {
  const int t = threadIdx.x, nt = blockDim.x;
  for (int i = t; i < kF1; i += nt) S.F1[i] = __ldg(&W.F1[i]);
  for (int i = t; i < kF2; i += nt) S.F2[i] = __ldg(&W.F2[i]);
  for (int i = t; i < kF3; i += nt) S.F3[i] = __ldg(&W.F3[i]);
  for (int i = t; i < kMlpHid; i += nt) { S.b1[i] = __ldg(&W.b1[i]); S.b2[i] = __ldg(&W.b2[i]); }
  if (t < 8) S.b3[t] = (t < 2) ? __ldg(&W.b3[t]) : 0.0f;
  __syncthreads();
}

__device__ __forceinline__ void mma_bf16_16816(float *d, const uint32_t *a, uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// bias + ReLU of one accumulator fragment (columns col, col + 1; rows g and g + 8)
__device__ __forceinline__ void bias_relu(float *d, const float *bias, int col) {
  const float b0 = bias[col], b1 = bias[col + 1];
  d[0] = fmaxf(d[0] + b0, 0.0f); d[1] = fmaxf(d[1] + b1, 0.0f);
  d[2] = fmaxf(d[2] + b0, 0.0f); d[3] = fmaxf(d[3] + b1, 0.0f);
}

// Network output 0 for this lane's item, from its normalised features x[0..15].  All 32
// lanes of the warp must call it together (inactive lanes with any x).
__device__ __forceinline__ float mlp_warp_predict(MlpWarpShared &S, const float *x) {
  const int lane = threadIdx.x & 31, w = (threadIdx.x >> 5) & (kWarpMlpWarps - 1);
  const int g = lane >> 2, t = lane & 3;
  uint32_t *X = S.X[w];
  // rows 9 words apart: the 32 lanes' stores of one word fall in 32 different banks
#pragma unroll
  for (int i = 0; i < 8; i++) X[lane * 9 + i] = pack_bf16x2(x[2 * i], x[2 * i + 1]);
  __syncwarp();
#pragma unroll 1
  for (int mt = 0; mt < 2; mt++) {
    const int r0 = mt * 16 + g, r1 = r0 + 8;
    // A operand of layer 1: rows r0 / r1, feature pairs 2t (k 0..7) and 2t + 8 (k 8..15)
    const uint32_t a[4] = {X[r0 * 9 + t], X[r1 * 9 + t], X[r0 * 9 + 4 + t], X[r1 * 9 + 4 + t]};
    uint32_t h[4][4];  // layer-1 activations as the 4 k-chunks of layer 2's A operand
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float d0[4] = {0.f, 0.f, 0.f, 0.f}, d1[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16_16816(d0, a, S.F1[(2 * c) * 32 + lane]);
      mma_bf16_16816(d1, a, S.F1[(2 * c + 1) * 32 + lane]);
      bias_relu(d0, S.b1, 16 * c + 2 * t);
      bias_relu(d1, S.b1, 16 * c + 8 + 2 * t);
      h[c][0] = pack_bf16x2(d0[0], d0[1]); h[c][1] = pack_bf16x2(d0[2], d0[3]);
      h[c][2] = pack_bf16x2(d1[0], d1[1]); h[c][3] = pack_bf16x2(d1[2], d1[3]);
    }
    // layer 2, two column tiles (16 hidden units) at a time, each pair folded at once into
    // layer 3 as one k-chunk of its A operand
    float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float d0[4] = {0.f, 0.f, 0.f, 0.f}, d1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        mma_bf16_16816(d0, h[k], S.F2[((2 * c) * 4 + k) * 32 + lane]);
        mma_bf16_16816(d1, h[k], S.F2[((2 * c + 1) * 4 + k) * 32 + lane]);
      }
      bias_relu(d0, S.b2, 16 * c + 2 * t);
      bias_relu(d1, S.b2, 16 * c + 8 + 2 * t);
      const uint32_t a3[4] = {pack_bf16x2(d0[0], d0[1]), pack_bf16x2(d0[2], d0[3]), pack_bf16x2(d1[0], d1[1]),
                              pack_bf16x2(d1[2], d1[3])};
      mma_bf16_16816(o, a3, S.F3[c * 32 + lane]);
    }
    // output column 0 of rows r0 and r1 sits in the lanes with t == 0
    if (t == 0) { S.Z[w][r0] = o[0] + S.b3[0]; S.Z[w][r1] = o[2] + S.b3[0]; }
  }
  __syncwarp();
  const float z = S.Z[w][lane];
  __syncwarp();  // the buffers are free for the warp's next call
  return z;
}

}  // namespace mdz
