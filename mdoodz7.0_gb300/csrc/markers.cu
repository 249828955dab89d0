// markers.cu -- UpdateParticleStress (MDLIB/RheologyParticles.c:1725-2004) on the GPU,
// for subgrid_diffusion 0 and 1.
//
// k_marker_update: one thread per marker.  It gathers what it needs from the grid
// directly -- the stress increments sxxd - sxxd0, szzd - szzd0 at the four centroid
// corners (Interp_Grid2P_centroids2, ParticleRoutines.c:1332-1573) and sxz - sxz0 at
// the four vertex corners (Interp_Grid2P, :1223-1321), the velocity gradients for the
// director (Centers2Particle, Vertices2Particle, :262-536) -- instead of building the
// reference's full-grid temporaries, then updates the marker and scatters its
// P2Mastah weights (:2170-2600) into WM.
// k_marker_wxz: one thread per vertex.  The reference's P2Mastah call at
// RheologyParticles.c:1971 interpolates a zeroed marker array onto wxz, so every vertex
// below the surface whose weight sum reaches 1e-30 gets 0 / WM; with periodic x, the
// first and last vertex of each row take their mean.  The marker spin stays zero, so
// the stress rotation that follows turns by zero; its arithmetic is kept as written.
//
// Every division by the mesh spacing or by the weight length is correctly rounded
// (fp64_div.cuh) and every product and sum is written with round-to-nearest intrinsics,
// so positions, weights and results are the reference's to the last bit.  The director
// normalisation squares by multiplication where the reference calls pow.
#include "markers.cuh"

#include "fp64_bits.cuh"

namespace mdz {

namespace {

__device__ __forceinline__ bool air(signed char t) { return t == 30 || t == 31; }

__device__ __forceinline__ void report(const MarkerArgs &A, long long k, int code) {
  atomicMin(&A.stats->err_key, ((unsigned long long)k << 8) | (unsigned long long)(-code));
}

// ceil(q) - 1 as the reference converts it to int, saturated far outside the grid (and
// for NaN) so that no conversion overflows; such markers fall outside every case
__device__ __forceinline__ int cell_of(double q) {
  const double c = ceil(q) - 1.0;
  if (!fp64_abs_lt(c, 1e9)) return fp64_lt(c, 0.0) ? -1000000000 : 1000000000;
  return (int)c;
}

// bilinear weights in the reference's order SW, SE, NW, NE: a = dxm/dx, b = dzm/dz
__device__ __forceinline__ void weights(double a, double b, double w[4]) {
  const double ia = __dsub_rn(1.0, a), ib = __dsub_rn(1.0, b);
  w[0] = __dmul_rn(ia, ib);
  w[1] = __dmul_rn(a, ib);
  w[2] = __dmul_rn(ia, b);
  w[3] = __dmul_rn(a, b);
}

// Corners of a marker in the ghost-extended centroid frame (Interp_Grid2P_centroids2,
// Centers2Particle): Ncx, Ncz centroids; returns false outside every handled case.
__device__ __forceinline__ bool cell_corners(const MarkerArgs &A, double x, double z, int &jp, int &ip, int c[4]) {
  const int Nx = A.Nx - 1, Nz = A.Nz - 1, per = A.periodic_x;
  const int j = cell_of(div_by(__dsub_rn(x, A.xvz[0]), A.dx)), i = cell_of(div_by(__dsub_rn(z, A.zvx[0]), A.dz));
  jp = j; ip = i;
  int SW, SE, NW, NE;
  if (j > 0 && j < Nx && i > 0 && i < Nz) {
    SW = (j - 1) + (i - 1) * Nx; SE = SW + 1; NW = SW + Nx; NE = NW + 1;
  } else if ((j == 0 || j == Nx) && i > 0 && i < Nz) {
    if (per == 1) { SW = (Nx - 1) + (i - 1) * Nx; SE = (i - 1) * Nx; NW = (Nx - 1) + i * Nx; NE = i * Nx; }
    else if (j == 0) { SW = SE = (i - 1) * Nx; NW = NE = i * Nx; }
    else { SW = SE = (Nx - 1) + (i - 1) * Nx; NW = NE = (Nx - 1) + i * Nx; }
  } else if (i == 0 && j > 0 && j < Nx) {
    SW = NW = j - 1; SE = NE = j;
  } else if (i == Nz && j > 0 && j < Nx) {
    SW = NW = (j - 1) + (Nz - 1) * Nx; SE = NE = SW + 1;
  } else if ((i == 0 || i == Nz) && (j == 0 || j == Nx)) {
    const int row = (i == 0) ? 0 : (Nz - 1) * Nx;
    if (per == 1) { SW = NW = (Nx - 1) + row; SE = NE = row; }
    else SW = SE = NW = NE = ((j == 0) ? 0 : Nx - 1) + row;
  } else {
    return false;
  }
  c[0] = SW; c[1] = SE; c[2] = NW; c[3] = NE;
  return true;
}

// Centers2Particle / Vertices2Particle: air corners left out, divided by the weight sum
// where it exceeds 1e-13
template <class F>
__device__ __forceinline__ double gather_skip(const signed char *tag, const int c[4], const double w[4], F field) {
  double v = 0.0, sw = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (!air(tag[c[q]])) {
      v = __dadd_rn(v, __dmul_rn(w[q], field(c[q])));
      sw = __dadd_rn(sw, w[q]);
    }
  if (fp64_gt(sw, 1e-13)) v = v / sw;
  return v;
}

// velocity gradients of StrainRateComponents' layout, zero at air nodes
// (RheologyParticles.c:1751-1782)
__device__ __forceinline__ double dudx_n(const MarkerArgs &A, int c0) {
  const int Ncx = A.Nx - 1, k = c0 % Ncx, l = c0 / Ncx;
  const long long c1 = k + (long long)l * A.Nx;
  return air(A.bcp[c0]) ? 0.0 : div_by(__dsub_rn(A.u[c1 + 1 + A.Nx], A.u[c1 + A.Nx]), A.dx);
}
__device__ __forceinline__ double dvdz_n(const MarkerArgs &A, int c0) {
  const int Ncx = A.Nx - 1, k = c0 % Ncx, l = c0 / Ncx;
  const long long c2 = k + (long long)l * (A.Nx + 1);
  return air(A.bcp[c0]) ? 0.0 : div_by(__dsub_rn(A.v[c2 + 1 + (A.Nx + 1)], A.v[c2 + 1]), A.dz);
}
__device__ __forceinline__ double dudz_s(const MarkerArgs &A, int c1) {
  return (A.bcg[c1] == 30) ? 0.0 : div_by(__dsub_rn(A.u[c1 + A.Nx], A.u[c1]), A.dz);
}
__device__ __forceinline__ double dvdx_s(const MarkerArgs &A, int c1) {
  const int k = c1 % A.Nx, l = c1 / A.Nx;
  const long long c3 = k + (long long)l * (A.Nx + 1);
  return (A.bcg[c1] == 30) ? 0.0 : div_by(__dsub_rn(A.v[c3 + 1], A.v[c3]), A.dx);
}

__device__ __forceinline__ void director(const MarkerArgs &A, long long k, double x, double z) {
  int jp, ip, c[4];
  double w[4];
  if (!cell_corners(A, x, z, jp, ip, c)) { report(A, k, MDZ_EMARKER_OUT); return; }
  weights(div_by(__dsub_rn(x, A.xvz[jp]), A.dx), div_by(__dsub_rn(z, A.zvx[ip]), A.dz), w);
  const double mdudx = gather_skip(A.bcp, c, w, [&](int i) { return dudx_n(A, i); });
  const double mdvdz = gather_skip(A.bcp, c, w, [&](int i) { return dvdz_n(A, i); });
  int j = cell_of(div_by(fabs(__dsub_rn(x, A.xg[0])), A.dx)), i = cell_of(div_by(fabs(__dsub_rn(z, A.zg[0])), A.dz));
  j = j < 0 ? 0 : (j > A.Nx - 2 ? A.Nx - 2 : j);
  i = i < 0 ? 0 : (i > A.Nz - 2 ? A.Nz - 2 : i);
  const int cv[4] = {j + i * A.Nx, j + i * A.Nx + 1, j + (i + 1) * A.Nx, j + (i + 1) * A.Nx + 1};
  weights(div_by(__dsub_rn(x, A.xg[j]), A.dx), div_by(__dsub_rn(z, A.zg[i]), A.dz), w);
  const double mdudz = gather_skip(A.bcg, cv, w, [&](int q) { return dudz_s(A, q); });
  const double mdvdx = gather_skip(A.bcg, cv, w, [&](int q) { return dvdx_s(A, q); });
  // :1795-1800 with the operations in the reference's order
  const double nx = A.m_nx[k], nz = A.m_nz[k], d = __dsub_rn(mdudx, mdvdz);
  const double E = __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(-d, nx), nz), __dmul_rn(__dmul_rn(mdvdx, nz), nz)),
                             __dmul_rn(__dmul_rn(mdudz, nx), nx));
  const double Fz = __dsub_rn(__dadd_rn(__dmul_rn(__dmul_rn(d, nx), nz), __dmul_rn(__dmul_rn(mdvdx, nz), nz)),
                              __dmul_rn(__dmul_rn(mdudz, nx), nx));
  const double nx1 = __dadd_rn(nx, __dmul_rn(__dmul_rn(A.dt, E), nz));
  const double nz1 = __dadd_rn(nz, __dmul_rn(__dmul_rn(A.dt, Fz), nx));
  const double norm = sqrt(__dadd_rn(__dmul_rn(nx1, nx1), __dmul_rn(nz1, nz1)));
  A.m_nx[k] = nx1 / norm;
  A.m_nz[k] = nz1 / norm;
}

__global__ void __launch_bounds__(256) k_marker_update(const MarkerArgs A) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.n) return;
  const bool active = A.phase[k] != -1;
  const double x = A.x[k], z = A.z[k];
  if (active && A.director) director(A, k, x, z);
  if (A.elastic != 1) return;
  double dsx = 0.0, dsz = 0.0, dsxz = 0.0;
  if (active) {
    int jp, ip, c[4];
    double w[4];
    if (!cell_corners(A, x, z, jp, ip, c)) {
      report(A, k, MDZ_EMARKER_OUT);
    } else {
      weights(div_by(__dsub_rn(x, A.xvz[jp]), A.dx), div_by(__dsub_rn(z, A.zvx[ip]), A.dz), w);
      const int alt[4] = {c[2], c[3], c[0], c[1]};
      double sw = 0.0;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        // an air corner lends its weight to the corner across; dsxxd, dszzd are 0 at air
        const int cc = air(A.bcp[c[q]]) ? alt[q] : c[q];
        const bool solid = !air(A.bcp[cc]);
        const double fx = solid ? __dsub_rn(A.sxxd[cc], A.sxxd0[cc]) : 0.0;
        const double fz = solid ? __dsub_rn(A.szzd[cc], A.szzd0[cc]) : 0.0;
        dsx = __dadd_rn(dsx, __dmul_rn(w[q], fx));
        dsz = __dadd_rn(dsz, __dmul_rn(w[q], fz));
        sw = __dadd_rn(sw, w[q]);
      }
      if (fp64_gt(sw, 1e-13)) { dsx = dsx / sw; dsz = dsz / sw; }
      if (fp64_is_inf(dsx) || fp64_is_inf(dsz)) report(A, k, MDZ_ENONFINITE);  // ParticleRoutines.c:1565-1569
    }
    // Interp_Grid2P: vertex cell clamped to the grid; beyond it in x the reference exits (89)
    int j = cell_of(div_by(__dsub_rn(x, A.xg[0]), A.dx));
    if (j < 0) j = 0;
    if (j > A.Nx - 2) { j = A.Nx - 2; report(A, k, MDZ_EMARKER_OUT); }
    int i = cell_of(div_by(__dsub_rn(z, A.zg[0]), A.dz));
    i = i < 0 ? 0 : (i > A.Nz - 2 ? A.Nz - 2 : i);
    const int cv[4] = {j + i * A.Nx, j + i * A.Nx + 1, j + (i + 1) * A.Nx, j + (i + 1) * A.Nx + 1};
    const int alt[4] = {cv[2], cv[3], cv[0], cv[1]};
    weights(div_by(fabs(__dsub_rn(x, A.xg[j])), A.dx), div_by(fabs(__dsub_rn(z, A.zg[i])), A.dz), w);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int cc = air(A.bcg[cv[q]]) ? alt[q] : cv[q];
      const double d = (A.bcg[cc] != 30) ? __dsub_rn(A.sxz[cc], A.sxz0[cc]) : 0.0;
      dsxz = __dadd_rn(dsxz, __dmul_rn(w[q], d));
    }
  }
  // ArrayPlusArray on every marker (:1954-1956)
  double txx = __dadd_rn(A.m_sxxd[k], dsx), tzz = __dadd_rn(A.m_szzd[k], dsz), txz = __dadd_rn(A.m_sxz[k], dsxz);
  if (active) {
    // rotation by the zeroed marker spin (:1972-1989), arithmetic as written
    const double wm = 0.0;
    if (A.rotation == 1) {
      const double a = __dsub_rn(txx, __dmul_rn(__dmul_rn(__dmul_rn(A.dt, 2.0), txz), wm));
      const double b = __dsub_rn(tzz, __dmul_rn(__dmul_rn(__dmul_rn(-A.dt, 2.0), txz), wm));
      const double c = __dsub_rn(txz, __dmul_rn(__dmul_rn(A.dt, __dsub_rn(tzz, txx)), wm));
      txx = a; tzz = b; txz = c;
    } else if (A.rotation == 2) {
      const double ang = __dmul_rn(A.dt, wm);
      const double cs = cos(ang), sn = sin(ang);
      const double a = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(txx, cs), __dmul_rn(txz, sn)), cs),
                                 __dmul_rn(__dadd_rn(__dmul_rn(txz, cs), __dmul_rn(tzz, sn)), sn));
      const double b = __dadd_rn(__dmul_rn(-__dadd_rn(__dmul_rn(-txx, sn), __dmul_rn(txz, cs)), sn),
                                 __dmul_rn(__dadd_rn(__dmul_rn(-txz, sn), __dmul_rn(tzz, cs)), cs));
      const double c = __dadd_rn(__dmul_rn(-__dadd_rn(__dmul_rn(txx, cs), __dmul_rn(txz, sn)), sn),
                                 __dmul_rn(__dadd_rn(__dmul_rn(txz, cs), __dmul_rn(tzz, sn)), cs));
      txx = a; tzz = b; txz = c;
    }
    // P2Mastah weights of this marker at its nearest vertex and, with the 9-node
    // stencil, the eight around it (ParticleRoutines.c:2288-2575)
    int ipx = cell_of(__dadd_rn(div_by(__dsub_rn(x, A.xg[0]), A.dx), 0.5));
    int jpz = cell_of(__dadd_rn(div_by(__dsub_rn(z, A.zg[0]), A.dz), 0.5));
    ipx = ipx < 0 ? 0 : (ipx > A.Nx - 1 ? A.Nx - 1 : ipx);
    jpz = jpz < 0 ? 0 : (jpz > A.Nz - 1 ? A.Nz - 1 : jpz);
    const double X = A.xg[ipx], Z = A.zg[jpz];
    auto w_at = [&](double xn, double zn) {
      return __dmul_rn(__dsub_rn(1.0, div_by(fabs(__dsub_rn(xn, x)), A.dx_itp)),
                       __dsub_rn(1.0, div_by(fabs(__dsub_rn(zn, z)), A.dz_itp)));
    };
    atomicAdd(&A.WM[ipx + (long long)jpz * A.Nx], w_at(X, Z));
    if (A.stencil == 9) {
      const int Nx = A.Nx, Nz = A.Nz, per = A.periodic_x;
      const bool peE = (ipx == Nx - 1 && per == 1), peW = (ipx == 0 && per == 1);
      const double xE = __dadd_rn(X, A.dx.b), xW = __dsub_rn(X, A.dx.b);
      const double zN = __dadd_rn(Z, A.dz.b), zS = __dsub_rn(Z, A.dz.b);
      const int kE = peE ? 0 : ipx + 1, kW = peW ? Nx - 1 : ipx - 1;
      const bool N = jpz < Nz - 1, S = jpz > 0, E = ipx < Nx - 1 || peE, Wst = ipx > 0 || peW;
      if (N) atomicAdd(&A.WM[ipx + (long long)(jpz + 1) * Nx], w_at(X, zN));
      if (S) atomicAdd(&A.WM[ipx + (long long)(jpz - 1) * Nx], w_at(X, zS));
      if (E) atomicAdd(&A.WM[kE + (long long)jpz * Nx], w_at(xE, Z));
      if (Wst) atomicAdd(&A.WM[kW + (long long)jpz * Nx], w_at(xW, Z));
      if (S && Wst) atomicAdd(&A.WM[kW + (long long)(jpz - 1) * Nx], w_at(xW, zS));
      if (N && Wst) atomicAdd(&A.WM[kW + (long long)(jpz + 1) * Nx], w_at(xW, zN));
      if (N && E) atomicAdd(&A.WM[kE + (long long)(jpz + 1) * Nx], w_at(xE, zN));
      if (S && E) atomicAdd(&A.WM[kE + (long long)(jpz - 1) * Nx], w_at(xE, zS));
    }
  }
  A.m_sxxd[k] = txx;
  A.m_szzd[k] = tzz;
  A.m_sxz[k] = txz;
}

// the value P2Mastah leaves at vertex c1 (:2603-2631)
__device__ __forceinline__ double wxz_after(const MarkerArgs &A, long long c1) {
  const double W = A.WM[c1];
  if (fp64_abs_lt(W, 1e-30) || air(A.bcg[c1])) return A.wxz[c1];
  return 0.0 / W;
}

__global__ void __launch_bounds__(256) k_marker_wxz(const MarkerArgs A) {
  const long long c1 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c1 >= (long long)A.Nx * A.Nz) return;
  const int k = (int)(c1 % A.Nx);
  if (A.periodic_x == 1) {
    if (k == A.Nx - 1) return;  // written by the row's first vertex
    if (k == 0) {
      // :2633-2641: both ends of the row take the mean of the two
      const double av = 0.5 * (wxz_after(A, c1 + A.Nx - 1) + wxz_after(A, c1));
      A.wxz[c1] = av;
      A.wxz[c1 + A.Nx - 1] = av;
      return;
    }
  }
  A.wxz[c1] = wxz_after(A, c1);
}

unsigned blocks_for(long long n) {
  const long long g = (n + 255) / 256;
  return (unsigned)(g > 0x7fffffffLL ? 0x7fffffffLL : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_marker_update(const MarkerArgs &a, cudaStream_t s) {
  if (a.n > 0) k_marker_update<<<blocks_for(a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_wxz(const MarkerArgs &a, cudaStream_t s) {
  k_marker_wxz<<<blocks_for((long long)a.Nx * a.Nz), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mdz
