// strain_rates.cu -- StrainRateComponents (MDLIB/RheologyDensity.c:2001-2097) in one launch.
//
// The reference makes four passes over the grid: centroid divergence and deviatoric
// normal rates, vertex shear rate and spin, the 4-vertex centroid averages of exz/wxz,
// then InterpCentroidsToVerticesDouble (MDLIB/GridRoutines.c:108-210) three times
// through a ghost-ringed copy of each centroid field.  Here one block owns a tile of
// kSrTx x kSrTz vertices and the centroids of the same indices.  It first evaluates the
// per-node values its tile needs, with a one-node halo, into shared memory -- centroid
// values at the ghost-ring cells (ring cell (i, j) maps to one centroid, as in the
// reference's ringed copy) and vertex values -- then forms the averages and the
// interpolation from shared memory and writes every output once.  Each velocity is
// read from HBM about once and every output written once; the halo adds
// (kSrTx + kSrTz + 1) / (kSrTx * kSrTz) evaluations per node.  The kernel is bound by
// the FP64 pipe (GB300 runs FP64 at 1/64 of the FP32 rate), so the forms below keep
// the FP64 instruction count low wherever that leaves every result bit unchanged.
//
// Every operation rounds as the reference's does (divisions by the mesh spacing are
// correctly rounded, fp64_div.cuh; the products and sums that a compiler could contract
// into an FMA are written with explicit round-to-nearest intrinsics), so the results
// are bitwise those of the reference.
#include "strain_rates.cuh"

#include "fp64_bits.cuh"

namespace mdz {

namespace {

// ghost-ring column / row -> centroid column / row (GridRoutines.c:131-180): the
// border copies its inner neighbour, or the opposite side when periodic in x
__device__ __forceinline__ int ring_col(int i, int Ncx, int per) {
  if (per == 1) return (i == 0) ? Ncx - 1 : ((i == Ncx + 1) ? 0 : i - 1);
  const int c = i - 1;
  return c < 0 ? 0 : (c > Ncx - 1 ? Ncx - 1 : c);
}
__device__ __forceinline__ int ring_row(int j, int Ncz) {
  const int c = j - 1;
  return c < 0 ? 0 : (c > Ncz - 1 ? Ncz - 1 : c);
}

constexpr int kW = kSrTx + 1, kH = kSrTz + 1;  // tile plus the one-node halo

struct SrShared {
  double div[kH][kW], exx[kH][kW], ezz[kH][kW];  // centroid values at ring cells (k0+i, l0+j); +0.0 at air
  double exz[kH][kW], wxz[kH][kW];                // vertex values at vertices (k0+i, l0+j); +0.0 at air
  unsigned char cin[kH][kW];                      // ring cell's centroid is not air (BCp not 30/31)
  unsigned char vin[kH][kW];                      // bit 0: vertex not air (BCg != 30); bit 1: exz, wxz tame
};

// x == 0 or 2^-1000 <= |x| <= 2^1000: the range in which a quarter of a sum of such
// values rounds exactly like the sum of their quarters (no subnormal, no overflow)
__device__ __forceinline__ bool tame(double x) {
  return (fp64_exponent(x) - 23u) <= 2000u || fp64_is_zero(x);
}

// +0.0 in place of -0.0 (the reference's averages start from +0.0 and never end at -0.0)
__device__ __forceinline__ double no_negative_zero(double x) { return fp64_is_negative_zero(x) ? 0.0 : x; }

__global__ void __launch_bounds__(kSrTx * kSrTz) k_strain_rates(const StrainArgs A) {
  __shared__ SrShared S;
  const int Nx = A.Nx, Nz = A.Nz, Ncx = A.Ncx, Ncz = A.Ncz;
  const int k0 = blockIdx.x * kSrTx, l0 = blockIdx.y * kSrTz;
  const Divisor dx = A.dx, dz = A.dz;

  // ---- per-node values of the tile and its halo
  for (int t = threadIdx.x; t < kW * kH; t += blockDim.x) {
    const int i = t % kW, j = t / kW;
    const int ri = k0 + i, rj = l0 + j;
    if (ri <= Ncx + 1 && rj <= Ncz + 1) {
      // centroid behind ring cell (ri, rj): RheologyDensity.c:2016-2041
      const int ck = ring_col(ri, Ncx, A.periodic_x), cl = ring_row(rj, Ncz);
      const long long c0 = ck + (long long)cl * Ncx;
      const signed char bc = A.bcp[c0];
      const bool in = !(bc == 30 || bc == 31);
      double dv = 0.0, ex = 0.0, ez = 0.0;
      if (in) {
        const long long c1 = ck + (long long)cl * Nx, c2 = ck + (long long)cl * (Nx + 1);
        const double dvxdx = div_by(A.u[c1 + 1 + Nx] - A.u[c1 + Nx], dx);
        const double dvzdz = div_by(A.v[c2 + Nx + 2] - A.v[c2 + 1], dz);
        const double s = __dadd_rn(dvxdx, dvzdz);
        dv = __dadd_rn(s, __dmul_rn(A.oop_half, s));
        ex = __dsub_rn(dvxdx, __dmul_rn(A.comp3, dv));
        ez = __dsub_rn(dvzdz, __dmul_rn(A.comp3, dv));
      }
      S.div[j][i] = dv; S.exx[j][i] = ex; S.ezz[j][i] = ez;
      S.cin[j][i] = in;
    }
    if (ri < Nx && rj < Nz) {
      // vertex (ri, rj): RheologyDensity.c:2045-2063
      const long long c1 = ri + (long long)rj * Nx, c2 = ri + (long long)rj * (Nx + 1);
      const bool in = A.bcg[c1] != 30;
      double e = 0.0, w = 0.0;
      if (in) {
        const double dvxdz = div_by(A.u[c1 + Nx] - A.u[c1], dz);
        const double dvzdx = div_by(A.v[c2 + 1] - A.v[c2], dx);
        e = 0.5 * (dvxdz + dvzdx);
        w = 0.5 * (dvzdx - dvxdz);
      }
      S.exz[j][i] = e; S.wxz[j][i] = w;
      S.vin[j][i] = (unsigned char)(in | ((tame(e) && tame(w)) << 1));
    }
  }
  __syncthreads();

  const int tx = threadIdx.x % kSrTx, tz = threadIdx.x / kSrTx;
  const int k = k0 + tx, l = l0 + tz;
  if (k < Nx && l < Nz) {
    // vertex outputs: exz, wxz, and exxd_s / ezzd_s / div_u_s from the four ring cells
    // (k..k+1, l..l+1), GridRoutines.c:185-206.  The reference weights each ring value
    // by 0 (air) or 1; air ring cells hold +0.0 here, so the weighted and the plain sums
    // agree bit for bit and the weights are left out.
    const long long c1 = k + (long long)l * Nx;
    double xs = 0.0, zs = 0.0, ds = 0.0;
    if (S.vin[tz][tx] & 1) {
#define MDZ_RING4(F)                                                                                  \
  __dmul_rn(0.25, __dadd_rn(__dadd_rn(__dadd_rn(S.F[tz][tx], S.F[tz][tx + 1]), S.F[tz + 1][tx]), \
                            S.F[tz + 1][tx + 1]))
      xs = MDZ_RING4(exx);
      zs = MDZ_RING4(ezz);
      ds = MDZ_RING4(div);
#undef MDZ_RING4
      A.out[SR_WXZ][c1] = S.wxz[tz][tx];
    }
    A.out[SR_EXZ][c1] = S.exz[tz][tx];
    A.out[SR_EXXD_S][c1] = xs;
    A.out[SR_EZZD_S][c1] = zs;
    A.out[SR_DIV_S][c1] = ds;
  }
  if (k < Ncx && l < Ncz) {
    // centroid outputs: own values (ring cell (k+1, l+1)) and the averages of the four
    // vertices (k..k+1, l..l+1) that are not air, RheologyDensity.c:2067-2089
    const long long c0 = k + (long long)l * Ncx;
    double en = 0.0, wn = 0.0;
    if (S.cin[tz + 1][tx + 1]) {
      const unsigned char f0 = S.vin[tz][tx], f1 = S.vin[tz][tx + 1];
      const unsigned char f2 = S.vin[tz + 1][tx], f3 = S.vin[tz + 1][tx + 1];
      if (((f0 | f1 | f2 | f3) & 1) == 0) {
        // no vertex counts: both stay +0.0
      } else if ((f0 == 1) | (f1 == 1) | (f2 == 1) | (f3 == 1)) {
        // a counted value outside the tame range: the reference's sequence of
        // quarter-value additions, from +0.0, in SW, SE, NW, NE order
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int a = tx + (q & 1), b = tz + (q >> 1);
          if (S.vin[b][a] & 1) {
            en = __dadd_rn(en, __dmul_rn(0.25, S.exz[b][a]));
            wn = __dadd_rn(wn, __dmul_rn(0.25, S.wxz[b][a]));
          }
        }
      } else {
        // every counted value is tame and air vertices hold +0.0: a quarter of the plain
        // sum equals the reference's sum of quarters bit for bit, up to the sign of a
        // zero result
#define MDZ_QUAD4(F)                                                                                   \
  no_negative_zero(__dmul_rn(0.25, __dadd_rn(__dadd_rn(__dadd_rn(S.F[tz][tx], S.F[tz][tx + 1]),         \
                                                       S.F[tz + 1][tx]),                               \
                                             S.F[tz + 1][tx + 1])))
        en = MDZ_QUAD4(exz);
        wn = MDZ_QUAD4(wxz);
#undef MDZ_QUAD4
      }
    }
    A.out[SR_DIV][c0] = S.div[tz + 1][tx + 1];
    A.out[SR_EXXD][c0] = S.exx[tz + 1][tx + 1];
    A.out[SR_EZZD][c0] = S.ezz[tz + 1][tx + 1];
    A.out[SR_EXZ_N][c0] = en;
    A.out[SR_WXZ_N][c0] = wn;
  }
}

}  // namespace

cudaError_t launch_strain_rates(const StrainArgs &a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.Nx + kSrTx - 1) / kSrTx), (unsigned)((a.Nz + kSrTz - 1) / kSrTz));
  if (grid.y > 65535u) return cudaErrorInvalidValue;
  k_strain_rates<<<grid, kSrTx * kSrTz, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mdz
