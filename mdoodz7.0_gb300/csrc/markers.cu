// markers.cu -- UpdateParticleStress (MDLIB/RheologyParticles.c:1725-2004) on the GPU,
// for subgrid_diffusion 0 and 1.
//
// k_marker_grid: one thread per centroid and per vertex.  It forms the per-node fields
// the reference builds before interpolating to the markers -- the stress increments
// sxxd - sxxd0, szzd - szzd0, sxz - sxz0 and, for the director, the velocity gradients
// of RheologyParticles.c:1751-1782 -- once per node instead of once per marker and
// corner, and clears the scratch of the P2Mastah step.
// k_marker_update: one thread per marker.  Its centroid cell and weights
// (Interp_Grid2P_centroids2, ParticleRoutines.c:1332-1573, and Centers2Particle,
// :262-455) and its vertex cell and weights (Interp_Grid2P, :1223-1321, and
// Vertices2Particle, :464-536) are formed once and shared by the director and the
// stress update wherever the reference's expressions give the same bits; the column
// quotient (x - xg[0]) / dx also gives P2Mastah's nearest vertex (:2301-2311).
// P2Mastah at RheologyParticles.c:1971 interpolates a zeroed marker array onto wxz:
// every vertex below the surface whose weight sum WM reaches 1e-30 gets 0 / WM, the
// others keep wxz.  Every weight is non-negative for a marker on the grid, and a
// rounded sum of non-negative numbers is at least its largest term, so a vertex is
// decided by whether some weight reaches 1e-30: a byte flag, set with a plain store,
// replaces the reference's summation.  A weight is surely >= 1e-30 when the marker
// lies inside its support by more than 2^-40 of the weight length on both axes,
// tested without a division; a weight below 1e-30 that is not zero, or one that is not
// finite, sets *exotic, and k_marker_weights then forms the exact sums with atomics as
// P2Mastah does.
// k_marker_wxz: one thread per vertex; with periodic x the first and last vertex of
// each row take their mean.  The marker spin stays zero, so the stress rotation turns
// by zero; its arithmetic is kept as written, with cos(+-0) = 1 and sin(+-0) = +-0
// taken as the exact values they are.
//
// subgrid_diffusion 2 (RheologyParticles.c:1811-1903) adds two launches between the grid
// kernel and the update.  k_marker_subgrid, per marker: the old grid stresses and the
// vertex viscosity at the marker, its subgrid increment -(s - s0)(1 - exp(-dt/t_M)) with
// t_M = eta/G, and P2Mastah's sums of those increments on the centroid and vertex grids
// (atomics; the reference's own order depends on its thread count).  k_marker_remainder,
// per node: the grid's increment less the subgrid increment P2Mastah gives the node.
// k_marker_update then interpolates the remainders exactly as the plain increments and
// adds both to the marker; k_marker_wxz takes its vertex weight sums from the same P2Mastah.
//
// Every division by the mesh spacing or by the weight length is correctly rounded
// (fp64_div.cuh), every product and sum is written with round-to-nearest intrinsics,
// cell indices come from fp64_ceil_int (the reference's ceil, on the integer pipe), and
// a division by a weight sum that is exactly 1 is skipped (it returns its numerator),
// so positions, weights and results are the reference's to the last bit.  The director
// normalisation squares by multiplication where the reference calls pow.
#include "markers.cuh"

#include "fp64_bits.cuh"
#include "fp64_math.cuh"

namespace mdz {

namespace {

__device__ __forceinline__ bool air(signed char t) { return t == 30 || t == 31; }

__device__ __forceinline__ void report(const MarkerArgs &A, long long k, int code) {
  atomicMin(&A.stats->err_key, ((unsigned long long)k << 8) | (unsigned long long)(-code));
}

// ceil(q) - 1 as the reference converts it to int; beyond 2^30 in magnitude (and for
// NaN) saturated, which falls outside every case and every clamp the same way
__device__ __forceinline__ int cell_of(double q) { return fp64_ceil_int(q) - 1; }

__device__ __forceinline__ bool sign_clear(double v) { return (fp64_hi(v) >> 31) == 0u; }

// (a / sw, b / sw) as the reference writes them.  For sw == 1 a division returns its
// numerator; the bilinear weights of a cell without air sum to exactly 1 for most
// markers, and the divisions stay out of line so that a warp whose markers all have
// sw == 1 branches past them.
__device__ __noinline__ double2 div_pair(double a, double b, double sw) { return make_double2(a / sw, b / sw); }

__device__ __forceinline__ void div_sum(double &a, double &b, double sw) {
  if (fp64_bits(sw) != 0x3ff0000000000000ull) {
    const double2 q = div_pair(a, b, sw);
    a = q.x;
    b = q.y;
  }
}

// ceil(RN(t/b)) - 1 and ceil(RN(RN(t/b) + 1/2)) - 1: the cell of a marker at distance t
// from the first node of a frame, and (for the vertex frame) P2Mastah's nearest node
struct CellPair {
  int c, h;
};

__device__ __noinline__ CellPair cell_pair_exact(double t, Divisor d) {
  const double q = div_by(t, d);
  return {cell_of(q), cell_of(__dadd_rn(q, 0.5))};
}

// q0 = RN(t y) lies within 1.5 ulp of t/b (y = RN(1/b)), and RN(t/b) within half an
// ulp of it.  When q0 >= 1 lies more than 16 of its ulps from every integer and every
// half-integer, RN(t/b) and RN(RN(t/b) + 1/2) (whose rounding moves by at most one ulp
// of q0 more) have the ceilings of q0 and q0 + 1/2, which the integer pipe reads from
// the bits of q0; otherwise the correctly rounded quotient decides.
__device__ __forceinline__ CellPair cell_pair(double t, const Divisor &d) {
  const double q0 = __dmul_rn(t, d.y);
  unsigned lo, hi;
  fp64_words(q0, lo, hi);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  if (d.fast && (hi >> 31) == 0u && e >= 0 && e < 29) {
    const unsigned long long m = ((unsigned long long)(hi & 0xfffffu) << 32 | lo) | (1ull << 52);
    const int sh = 52 - e;  // fraction bits of q0
    const unsigned long long one = 1ull << sh, half = one >> 1, f = m & (one - 1ull);
    const unsigned long long dh = f > half ? f - half : half - f;
    if (f > 16ull && one - f > 16ull && dh > 16ull) {
      const int ip = (int)(m >> sh);
      return {ip, ip + (f > half ? 1 : 0)};
    }
  }
  return cell_pair_exact(t, d);
}

// bilinear weights in the reference's order SW, SE, NW, NE: a = dxm/dx, b = dzm/dz
__device__ __forceinline__ void weights(double a, double b, double w[4]) {
  const double ia = __dsub_rn(1.0, a), ib = __dsub_rn(1.0, b);
  w[0] = __dmul_rn(ia, ib);
  w[1] = __dmul_rn(a, ib);
  w[2] = __dmul_rn(ia, b);
  w[3] = __dmul_rn(a, b);
}

__device__ __forceinline__ int clamp_to(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

// Corners of a marker in the ghost-extended centroid frame (Interp_Grid2P_centroids2,
// Centers2Particle): Ncx, Ncz centroids; returns false outside every handled case.
__device__ __forceinline__ bool cell_corners(const MarkerArgs &A, double x, double z, int &jp, int &ip, int c[4]) {
  const int Nx = A.Nx - 1, Nz = A.Nz - 1, per = A.periodic_x;
  const int j = cell_pair(__dsub_rn(x, A.xvz[0]), A.dx).c, i = cell_pair(__dsub_rn(z, A.zvx[0]), A.dz).c;
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

// Centers2Particle / Vertices2Particle for a pair of fields: air corners left out, each
// sum divided by the weight sum where that exceeds 1e-13
__device__ __forceinline__ double2 gather_skip(const signed char *tag, const double2 *f, const int c[4],
                                               const double w[4]) {
  double a = 0.0, b = 0.0, sw = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (!air(tag[c[q]])) {
      const double2 v = f[c[q]];
      a = __dadd_rn(a, __dmul_rn(w[q], v.x));
      b = __dadd_rn(b, __dmul_rn(w[q], v.y));
      sw = __dadd_rn(sw, w[q]);
    }
  if (fp64_gt(sw, 1e-13)) div_sum(a, b, sw);
  return make_double2(a, b);
}

// :1784-1802 with the operations in the reference's order
__device__ __forceinline__ void director(const MarkerArgs &A, long long k, const int c[4], const double wc[4],
                                         const int cv[4], const double wv[4]) {
  const double2 gn = gather_skip(A.bcp, A.grad_n, c, wc);   // du/dx, dv/dz
  const double2 gs = gather_skip(A.bcg, A.grad_s, cv, wv);  // du/dz, dv/dx
  const double mdudx = gn.x, mdvdz = gn.y, mdudz = gs.x, mdvdx = gs.y;
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

// P2Mastah's weight (1 - ax/dx_itp) (1 - az/dz_itp) for the distances ax = |X - x|,
// az = |Z - z| of a marker to a vertex (ParticleRoutines.c:2320-2575)
__device__ __forceinline__ double p2m_weight(const MarkerArgs &A, double ax, double az) {
  return __dmul_rn(__dsub_rn(1.0, div_by(ax, A.dx_itp)), __dsub_rn(1.0, div_by(az, A.dz_itp)));
}

__device__ __forceinline__ void p2m_mark(const MarkerArgs &A, long long v, double ax, double az) {
  if (fp64_le(ax, A.near_x) && fp64_le(az, A.near_z)) {
    A.hit[v] = 1;
    return;
  }
  const double w = p2m_weight(A, ax, az);
  if (fp64_ge(w, 1e-30) && fp64_finite(w)) A.hit[v] = 1;
  else if (!fp64_is_zero(w)) *A.exotic = 1;
}

// The vertices P2Mastah gives a marker a weight at: its nearest vertex (ipx, jpz) and,
// with the 9-node stencil, the eight around it, wrapped in x when periodic
// (:2301-2575); hx, hz are ceil((x - xg[0]) / dx + 1/2) - 1 and its z twin, unclamped
template <class F>
__device__ __forceinline__ void p2m_vertices(const MarkerArgs &A, double x, double z, int hx, int hz, F visit) {
  const int ipx = clamp_to(hx, A.Nx - 1), jpz = clamp_to(hz, A.Nz - 1);
  const double X = A.xg[ipx], Z = A.zg[jpz];
  const double axc = fabs(__dsub_rn(X, x)), azc = fabs(__dsub_rn(Z, z));
  visit(ipx + (long long)jpz * A.Nx, axc, azc);
  if (A.stencil != 9) return;
  const int Nx = A.Nx, Nz = A.Nz, per = A.periodic_x;
  const bool peE = (ipx == Nx - 1 && per == 1), peW = (ipx == 0 && per == 1);
  const double axE = fabs(__dsub_rn(__dadd_rn(X, A.dx.b), x)), axW = fabs(__dsub_rn(__dsub_rn(X, A.dx.b), x));
  const double azN = fabs(__dsub_rn(__dadd_rn(Z, A.dz.b), z)), azS = fabs(__dsub_rn(__dsub_rn(Z, A.dz.b), z));
  const int kE = peE ? 0 : ipx + 1, kW = peW ? Nx - 1 : ipx - 1;
  const bool N = jpz < Nz - 1, S = jpz > 0, E = ipx < Nx - 1 || peE, Wst = ipx > 0 || peW;
  if (N) visit(ipx + (long long)(jpz + 1) * Nx, axc, azN);
  if (S) visit(ipx + (long long)(jpz - 1) * Nx, axc, azS);
  if (E) visit(kE + (long long)jpz * Nx, axE, azc);
  if (Wst) visit(kW + (long long)jpz * Nx, axW, azc);
  if (S && Wst) visit(kW + (long long)(jpz - 1) * Nx, axW, azS);
  if (N && Wst) visit(kW + (long long)(jpz + 1) * Nx, axW, azN);
  if (N && E) visit(kE + (long long)(jpz + 1) * Nx, axE, azN);
  if (S && E) visit(kE + (long long)(jpz - 1) * Nx, axE, azS);
}

// The rotation of :1972-1989 by the marker spin, which UpdateParticleStress leaves at
// zero, with the arithmetic as written.  For stresses that are nonzero and below 2^500
// in magnitude and a finite dt below 2^500, every product with the zero spin is a
// signed zero and every sum returns its nonzero term (Jaumann, rotation 1); with
// cos(0) = 1 and sin(+-0) = +-0 the same holds for finite nonzero stresses (rotation 2):
// the rotation is then the identity, and the caller skips this function.
__device__ __noinline__ void rotate(int rotation, double dt, double &txx, double &tzz, double &txz) {
  const double wm = 0.0;
  if (rotation == 1) {
    const double a = __dsub_rn(txx, __dmul_rn(__dmul_rn(__dmul_rn(dt, 2.0), txz), wm));
    const double b = __dsub_rn(tzz, __dmul_rn(__dmul_rn(__dmul_rn(-dt, 2.0), txz), wm));
    const double r = __dsub_rn(txz, __dmul_rn(__dmul_rn(dt, __dsub_rn(tzz, txx)), wm));
    txx = a; tzz = b; txz = r;
  } else {
    const double ang = __dmul_rn(dt, wm);
    double cs, sn;
    if (fp64_is_zero(ang)) { cs = 1.0; sn = ang; }
    else { cs = cos(ang); sn = sin(ang); }
    const double a = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(txx, cs), __dmul_rn(txz, sn)), cs),
                               __dmul_rn(__dadd_rn(__dmul_rn(txz, cs), __dmul_rn(tzz, sn)), sn));
    const double b = __dadd_rn(__dmul_rn(-__dadd_rn(__dmul_rn(-txx, sn), __dmul_rn(txz, cs)), sn),
                               __dmul_rn(__dadd_rn(__dmul_rn(-txz, sn), __dmul_rn(tzz, cs)), cs));
    const double r = __dadd_rn(__dmul_rn(-__dadd_rn(__dmul_rn(txx, cs), __dmul_rn(txz, sn)), sn),
                               __dmul_rn(__dadd_rn(__dmul_rn(txz, cs), __dmul_rn(tzz, sn)), cs));
    txx = a; tzz = b; txz = r;
  }
}

// P2Mastah's exact weights of a marker on a grid of Nxn x Nzn nodes at X, Z (:2301-2575),
// visit(node, w) in the reference's order.  hx, hz are ceil((x - X[0]) / dx + 1/2) - 1 and
// its z twin, unclamped.  The nine weights share three quotients per axis.
template <class F>
__device__ __forceinline__ void p2m_exact(const MarkerArgs &A, const double *X, const double *Z, int Nxn, int Nzn,
                                          double x, double z, int hx, int hz, F visit) {
  const int ip = clamp_to(hx, Nxn - 1), jp = clamp_to(hz, Nzn - 1);
  const double Xp = X[ip], Zp = Z[jp];
  const double fc = __dsub_rn(1.0, div_by(fabs(__dsub_rn(Xp, x)), A.dx_itp));
  const double gc = __dsub_rn(1.0, div_by(fabs(__dsub_rn(Zp, z)), A.dz_itp));
  visit(ip + (long long)jp * Nxn, __dmul_rn(fc, gc));
  if (A.stencil != 9) return;
  const int per = A.periodic_x;
  const bool peE = (ip == Nxn - 1 && per == 1), peW = (ip == 0 && per == 1);
  const double fE = __dsub_rn(1.0, div_by(fabs(__dsub_rn(__dadd_rn(Xp, A.dx.b), x)), A.dx_itp));
  const double fW = __dsub_rn(1.0, div_by(fabs(__dsub_rn(__dsub_rn(Xp, A.dx.b), x)), A.dx_itp));
  const double gN = __dsub_rn(1.0, div_by(fabs(__dsub_rn(__dadd_rn(Zp, A.dz.b), z)), A.dz_itp));
  const double gS = __dsub_rn(1.0, div_by(fabs(__dsub_rn(__dsub_rn(Zp, A.dz.b), z)), A.dz_itp));
  const int kE = peE ? 0 : ip + 1, kW = peW ? Nxn - 1 : ip - 1;
  const bool N = jp < Nzn - 1, S = jp > 0, E = ip < Nxn - 1 || peE, Wst = ip > 0 || peW;
  if (N) visit(ip + (long long)(jp + 1) * Nxn, __dmul_rn(fc, gN));
  if (S) visit(ip + (long long)(jp - 1) * Nxn, __dmul_rn(fc, gS));
  if (E) visit(kE + (long long)jp * Nxn, __dmul_rn(fE, gc));
  if (Wst) visit(kW + (long long)jp * Nxn, __dmul_rn(fW, gc));
  if (S && Wst) visit(kW + (long long)(jp - 1) * Nxn, __dmul_rn(fW, gS));
  if (N && Wst) visit(kW + (long long)(jp + 1) * Nxn, __dmul_rn(fW, gN));
  if (N && E) visit(kE + (long long)(jp + 1) * Nxn, __dmul_rn(fE, gN));
  if (S && E) visit(kE + (long long)(jp - 1) * Nxn, __dmul_rn(fE, gS));
}

// Interp_Grid2P_centroids2 of two raw centroid fields: an air corner takes the value of
// the corner across, the sum is divided by the weight sum where that exceeds 1e-13
__device__ __forceinline__ double2 gather_sub(const MarkerArgs &A, const double *fa, const double *fb, const int c[4],
                                              const double w[4]) {
  const int alt[4] = {c[2], c[3], c[0], c[1]};
  double a = 0.0, b = 0.0, sw = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int cc = air(A.bcp[c[q]]) ? alt[q] : c[q];
    a = __dadd_rn(a, __dmul_rn(w[q], fa[cc]));
    b = __dadd_rn(b, __dmul_rn(w[q], fb[cc]));
    sw = __dadd_rn(sw, w[q]);
  }
  if (fp64_gt(sw, 1e-13)) div_sum(a, b, sw);
  return make_double2(a, b);
}

// Interp_Grid2P of a raw vertex field: an air corner takes the value of the corner across
__device__ __forceinline__ double gather_vertex(const MarkerArgs &A, const double *f, const int cv[4],
                                                const double w[4]) {
  const int alt[4] = {cv[2], cv[3], cv[0], cv[1]};
  double v = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++) v = __dadd_rn(v, __dmul_rn(w[q], f[air(A.bcg[cv[q]]) ? alt[q] : cv[q]]));
  return v;
}

__global__ void __launch_bounds__(256) k_marker_grid(const MarkerArgs A) {
  const long long Nc = (long long)(A.Nx - 1) * (A.Nz - 1), Nv = (long long)A.Nx * A.Nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0 && A.elastic == 1 && !A.subgrid) *A.exotic = 0;
  if (t < Nc) {
    const long long c0 = t;
    const bool a = air(A.bcp[c0]);
    if (A.elastic == 1 && A.subgrid) {
      A.sum_n[c0] = 0.0; A.sum_n[Nc + c0] = 0.0; A.sum_n[2 * Nc + c0] = 0.0;
    } else if (A.elastic == 1) {
      A.inc_n[c0] = a ? make_double2(0.0, 0.0)
                      : make_double2(__dsub_rn(A.sxxd[c0], A.sxxd0[c0]), __dsub_rn(A.szzd[c0], A.szzd0[c0]));
    }
    if (A.director) {
      // RheologyParticles.c:1751-1766 in the layout of the velocity arrays
      const int Ncx = A.Nx - 1, k = (int)(c0 % Ncx), l = (int)(c0 / Ncx);
      const long long c1 = k + (long long)l * A.Nx, c2 = k + (long long)l * (A.Nx + 1);
      A.grad_n[c0] = a ? make_double2(0.0, 0.0)
                       : make_double2(div_by(__dsub_rn(A.u[c1 + 1 + A.Nx], A.u[c1 + A.Nx]), A.dx),
                                      div_by(__dsub_rn(A.v[c2 + 1 + (A.Nx + 1)], A.v[c2 + 1]), A.dz));
    }
  } else if (t < Nc + Nv) {
    const long long c1 = t - Nc;
    const bool wall = A.bcg[c1] == 30;
    if (A.elastic == 1 && A.subgrid) {
      A.sum_s[c1] = 0.0; A.sum_s[Nv + c1] = 0.0;
    } else if (A.elastic == 1) {
      A.inc_s[c1] = wall ? 0.0 : __dsub_rn(A.sxz[c1], A.sxz0[c1]);
      A.hit[c1] = 0;
      A.WM[c1] = 0.0;
    }
    if (A.director) {
      // :1768-1782
      const int k = (int)(c1 % A.Nx), l = (int)(c1 / A.Nx);
      const long long c3 = k + (long long)l * (A.Nx + 1);
      A.grad_s[c1] = wall ? make_double2(0.0, 0.0)
                          : make_double2(div_by(__dsub_rn(A.u[c1 + A.Nx], A.u[c1]), A.dz),
                                         div_by(__dsub_rn(A.v[c3 + 1], A.v[c3]), A.dx));
    }
  }
}

// subgrid diffusion 2, markers (:1822-1861)
__global__ void __launch_bounds__(256) k_marker_subgrid(const MarkerArgs A) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.n) return;
  const int ph = A.phase[k];
  if (ph == -1) return;
  if (ph < 0 || ph >= A.np) { report(A, k, MDZ_EINVAL); return; }
  const double x = A.x[k], z = A.z[k];
  int jp, ip, c[4];
  double txx0 = 0.0, tzz0 = 0.0;
  if (cell_corners(A, x, z, jp, ip, c)) {
    double wc[4];
    weights(div_by(__dsub_rn(x, A.xvz[jp]), A.dx), div_by(__dsub_rn(z, A.zvx[ip]), A.dz), wc);
    const double2 t0 = gather_sub(A, A.sxxd0, A.szzd0, c, wc);
    txx0 = t0.x; tzz0 = t0.y;
    if (fp64_is_inf(txx0) || fp64_is_inf(tzz0)) report(A, k, MDZ_ENONFINITE);  // ParticleRoutines.c:1565-1569
  } else {
    report(A, k, MDZ_EMARKER_OUT);
  }
  const double tx = __dsub_rn(x, A.xg[0]), tz = __dsub_rn(z, A.zg[0]);
  const CellPair px = cell_pair(tx, A.dx), pz = cell_pair(tz, A.dz);
  if (px.c > A.Nx - 2) report(A, k, MDZ_EMARKER_OUT);
  const int j = clamp_to(px.c, A.Nx - 2), i = clamp_to(pz.c, A.Nz - 2);
  double wv[4];
  weights(div_by(fabs(__dsub_rn(x, A.xg[j])), A.dx), div_by(fabs(__dsub_rn(z, A.zg[i])), A.dz), wv);
  const int cv[4] = {j + i * A.Nx, j + i * A.Nx + 1, j + (i + 1) * A.Nx, j + (i + 1) * A.Nx + 1};
  const double txz0 = gather_vertex(A, A.sxz0, cv, wv), etam = gather_vertex(A, A.eta_s, cv, wv);
  // -(s - s0) (1 - exp(-d dt / t_M)), d = 1, t_M = eta / G (:1844-1846); the table-driven
  // exp of fp64_math.cuh (about 1 ulp from the C library's)
  const double tM = div_by(etam, A.G[ph]);
  const double f = __dsub_rn(1.0, fast_exp(-A.dt / tM));
  const double dxx = __dmul_rn(-__dsub_rn(A.m_sxxd[k], txx0), f);
  const double dzz = __dmul_rn(-__dsub_rn(A.m_szzd[k], tzz0), f);
  const double dxz = __dmul_rn(-__dsub_rn(A.m_sxz[k], txz0), f);
  if (!fp64_finite(dxx)) report(A, k, MDZ_ENONFINITE);  // :1847-1855, exit 1
  A.m_sub[k] = dxx;
  A.m_sub[A.n + k] = dzz;
  A.m_sub[2 * A.n + k] = dxz;
  // P2Mastah's sums (:1859-1861): centroids at xc, zc, vertices at xg, zg
  const int Ncx = A.Nx - 1, Ncz = A.Nz - 1;
  const long long Nc = (long long)Ncx * Ncz, Nv = (long long)A.Nx * A.Nz;
  const CellPair qx = cell_pair(__dsub_rn(x, A.xc[0]), A.dx), qz = cell_pair(__dsub_rn(z, A.zc[0]), A.dz);
  p2m_exact(A, A.xc, A.zc, Ncx, Ncz, x, z, qx.h, qz.h, [&](long long v, double w) {
    atomicAdd(&A.sum_n[v], w);
    atomicAdd(&A.sum_n[Nc + v], __dmul_rn(dxx, w));
    atomicAdd(&A.sum_n[2 * Nc + v], __dmul_rn(dzz, w));
  });
  p2m_exact(A, A.xg, A.zg, A.Nx, A.Nz, x, z, px.h, pz.h, [&](long long v, double w) {
    atomicAdd(&A.sum_s[v], w);
    atomicAdd(&A.sum_s[Nv + v], __dmul_rn(dxz, w));
  });
}

// P2Mastah's node value BMWM / WM where |WM| reaches 1e-30 away from air, else 0 (the
// reference's zeroed target), for one sum pair (:2603-2631)
__device__ __forceinline__ double p2m_value(double W, double BM, bool air_node) {
  return (air_node || fp64_abs_lt(W, 1e-30)) ? 0.0 : BM / W;
}

// subgrid diffusion 2, grid (:1864-1872): what remains of each node's increment
__global__ void __launch_bounds__(256) k_marker_remainder(const MarkerArgs A) {
  const long long Nc = (long long)(A.Nx - 1) * (A.Nz - 1), Nv = (long long)A.Nx * A.Nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Nc) {
    const long long c0 = t;
    if (air(A.bcp[c0])) {
      A.inc_n[c0] = make_double2(0.0, 0.0);
      return;
    }
    const double W = A.sum_n[c0];
    const double gxx = p2m_value(W, A.sum_n[Nc + c0], false), gzz = p2m_value(W, A.sum_n[2 * Nc + c0], false);
    A.inc_n[c0] = make_double2(__dsub_rn(__dsub_rn(A.sxxd[c0], A.sxxd0[c0]), gxx),
                               __dsub_rn(__dsub_rn(A.szzd[c0], A.szzd0[c0]), gzz));
  } else if (t < Nc + Nv) {
    const long long c1 = t - Nc;
    const int k = (int)(c1 % A.Nx);
    double g = p2m_value(A.sum_s[c1], A.sum_s[Nv + c1], air(A.bcg[c1]));
    if (A.periodic_x == 1 && (k == 0 || k == A.Nx - 1)) {
      // :2633-2641: both ends of the row take the mean of the two
      const long long last = c1 - k + A.Nx - 1, first = c1 - k;
      g = 0.5 * (p2m_value(A.sum_s[last], A.sum_s[Nv + last], air(A.bcg[last])) +
                 p2m_value(A.sum_s[first], A.sum_s[Nv + first], air(A.bcg[first])));
    }
    A.inc_s[c1] = (A.bcg[c1] == 30) ? 0.0 : __dsub_rn(__dsub_rn(A.sxz[c1], A.sxz0[c1]), g);
  }
}

__global__ void __launch_bounds__(256) k_marker_update(const MarkerArgs A) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.n) return;
  if (A.phase[k] == -1) {
    // ArrayPlusArray adds the (zero) increment of an inactive marker too (:1954-1956);
    // the subgrid update leaves it alone (:1878-1884)
    if (A.elastic == 1 && !A.subgrid) {
      A.m_sxxd[k] = __dadd_rn(A.m_sxxd[k], 0.0);
      A.m_szzd[k] = __dadd_rn(A.m_szzd[k], 0.0);
      A.m_sxz[k] = __dadd_rn(A.m_sxz[k], 0.0);
    }
    return;
  }
  const double x = A.x[k], z = A.z[k];
  // centroid frame
  int jp, ip, c[4];
  double wc[4];
  const bool inside = cell_corners(A, x, z, jp, ip, c);
  if (inside) weights(div_by(__dsub_rn(x, A.xvz[jp]), A.dx), div_by(__dsub_rn(z, A.zvx[ip]), A.dz), wc);
  else report(A, k, MDZ_EMARKER_OUT);
  // vertex frame of Interp_Grid2P: cell clamped to the grid; beyond it in x the reference exits (89)
  const double tx = __dsub_rn(x, A.xg[0]), tz = __dsub_rn(z, A.zg[0]);
  const CellPair px = cell_pair(tx, A.dx), pz = cell_pair(tz, A.dz);
  const bool beyond = px.c > A.Nx - 2;
  const int j = clamp_to(px.c, A.Nx - 2), i = clamp_to(pz.c, A.Nz - 2);
  const double ex = __dsub_rn(x, A.xg[j]), ez = __dsub_rn(z, A.zg[i]);
  double wv[4];
  weights(div_by(fabs(ex), A.dx), div_by(fabs(ez), A.dz), wv);
  const int cv[4] = {j + i * A.Nx, j + i * A.Nx + 1, j + (i + 1) * A.Nx, j + (i + 1) * A.Nx + 1};

  if (A.director && inside) {
    // Vertices2Particle takes the cell of |x - xg[0]| and the weights of x - xg[j]: the
    // bits above whenever those differences carry no sign
    int jd = j, id = i;
    double wd[4] = {wv[0], wv[1], wv[2], wv[3]};
    if (!(sign_clear(tx) && sign_clear(tz) && sign_clear(ex) && sign_clear(ez))) {
      jd = clamp_to(cell_of(div_by(fabs(tx), A.dx)), A.Nx - 2);
      id = clamp_to(cell_of(div_by(fabs(tz), A.dz)), A.Nz - 2);
      weights(div_by(__dsub_rn(x, A.xg[jd]), A.dx), div_by(__dsub_rn(z, A.zg[id]), A.dz), wd);
    }
    const int cd[4] = {jd + id * A.Nx, jd + id * A.Nx + 1, jd + (id + 1) * A.Nx, jd + (id + 1) * A.Nx + 1};
    director(A, k, c, wc, cd, wd);
  }
  if (A.elastic != 1) return;

  double dsx = 0.0, dsz = 0.0, dsxz = 0.0;
  if (inside) {
    const int alt[4] = {c[2], c[3], c[0], c[1]};
    double sw = 0.0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      // an air corner lends its weight to the corner across; the increments are 0 at air
      const int cc = air(A.bcp[c[q]]) ? alt[q] : c[q];
      const double2 f = A.inc_n[cc];
      dsx = __dadd_rn(dsx, __dmul_rn(wc[q], f.x));
      dsz = __dadd_rn(dsz, __dmul_rn(wc[q], f.y));
      sw = __dadd_rn(sw, wc[q]);
    }
    if (fp64_gt(sw, 1e-13)) div_sum(dsx, dsz, sw);
    if (fp64_is_inf(dsx) || fp64_is_inf(dsz)) report(A, k, MDZ_ENONFINITE);  // ParticleRoutines.c:1565-1569
  }
  if (beyond) report(A, k, MDZ_EMARKER_OUT);
  {
    const int alt[4] = {cv[2], cv[3], cv[0], cv[1]};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int cc = air(A.bcg[cv[q]]) ? alt[q] : cv[q];
      dsxz = __dadd_rn(dsxz, __dmul_rn(wv[q], A.inc_s[cc]));
    }
  }
  // ArrayPlusArray (:1954-1956), or the subgrid update s + ds_sub + ds_rest (:1878-1884)
  double txx = A.m_sxxd[k], tzz = A.m_szzd[k], txz = A.m_sxz[k];
  if (A.subgrid) {
    txx = __dadd_rn(txx, A.m_sub[k]);
    tzz = __dadd_rn(tzz, A.m_sub[A.n + k]);
    txz = __dadd_rn(txz, A.m_sub[2 * A.n + k]);
  }
  txx = __dadd_rn(txx, dsx); tzz = __dadd_rn(tzz, dsz); txz = __dadd_rn(txz, dsxz);
  // rotation by the zeroed marker spin (:1972-1989)
  if (A.rotation == 1 || A.rotation == 2) {
    const unsigned exx = fp64_exponent(txx), ezz = fp64_exponent(tzz), exz = fp64_exponent(txz);
    const bool plain = exx - 1u < 1522u && ezz - 1u < 1522u && exz - 1u < 1522u;
    const bool identity = plain && (A.rotation == 1 ? fp64_exponent(A.dt) < 1523u : fp64_is_zero(__dmul_rn(A.dt, 0.0)));
    if (!identity) rotate(A.rotation, A.dt, txx, tzz, txz);
  }
  A.m_sxxd[k] = txx;
  A.m_szzd[k] = tzz;
  A.m_sxz[k] = txz;
  if (!A.subgrid)
    p2m_vertices(A, x, z, px.h, pz.h, [&](long long v, double ax, double az) { p2m_mark(A, v, ax, az); });
}

// The exact P2Mastah weight sums, only after a weight below 1e-30 that is not zero (or
// one that is not finite) was seen; otherwise every CTA reads the flag and returns
__global__ void __launch_bounds__(256) k_marker_weights(const MarkerArgs A) {
  if (*A.exotic == 0) return;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < A.n;
       k += (long long)gridDim.x * blockDim.x) {
    if (A.phase[k] == -1) continue;
    const double x = A.x[k], z = A.z[k];
    const int hx = cell_pair(__dsub_rn(x, A.xg[0]), A.dx).h, hz = cell_pair(__dsub_rn(z, A.zg[0]), A.dz).h;
    p2m_vertices(A, x, z, hx, hz,
                 [&](long long v, double ax, double az) { atomicAdd(&A.WM[v], p2m_weight(A, ax, az)); });
  }
}

// the value P2Mastah leaves at vertex c1 (:2603-2631)
__device__ __forceinline__ double wxz_after(const MarkerArgs &A, long long c1, bool exact) {
  if (air(A.bcg[c1])) return A.wxz[c1];
  if (exact) {
    const double W = A.subgrid ? A.sum_s[c1] : A.WM[c1];
    return fp64_abs_lt(W, 1e-30) ? A.wxz[c1] : 0.0 / W;
  }
  return A.hit[c1] ? 0.0 : A.wxz[c1];
}

__global__ void __launch_bounds__(256) k_marker_wxz(const MarkerArgs A) {
  const long long c1 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c1 >= (long long)A.Nx * A.Nz) return;
  const bool exact = A.subgrid || *A.exotic != 0;
  const int k = (int)(c1 % A.Nx);
  if (A.periodic_x == 1) {
    if (k == A.Nx - 1) return;  // written by the row's first vertex
    if (k == 0) {
      // :2633-2641: both ends of the row take the mean of the two
      const double av = 0.5 * (wxz_after(A, c1 + A.Nx - 1, exact) + wxz_after(A, c1, exact));
      A.wxz[c1] = av;
      A.wxz[c1 + A.Nx - 1] = av;
      return;
    }
  }
  A.wxz[c1] = wxz_after(A, c1, exact);
}

// P2Mastah of a marker array (ParticleRoutines.c:2288-2575): the sums of w and w v on
// the centroids (sum_n) and vertices (sum_s), v the marker's value, 1/v or log v
__global__ void __launch_bounds__(256) k_p2m_scatter(const MarkerArgs A) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.n) return;
  const int ph = A.phase[k];
  if (ph == -1) return;
  if (ph < 0 || ph >= A.np) { report(A, k, MDZ_EINVAL); return; }
  const double x = A.x[k], z = A.z[k];
  double v = A.val[k];
  if (A.avg == 1) v = 1.0 / v;
  else if (A.avg == 2) v = log(v);
  if (A.out_n) {
    const int Ncx = A.Nx - 1, Ncz = A.Nz - 1;
    const long long Nc = (long long)Ncx * Ncz;
    const int hx = cell_pair(__dsub_rn(x, A.xc[0]), A.dx).h, hz = cell_pair(__dsub_rn(z, A.zc[0]), A.dz).h;
    p2m_exact(A, A.xc, A.zc, Ncx, Ncz, x, z, hx, hz, [&](long long node, double w) {
      atomicAdd(&A.sum_n[node], w);
      atomicAdd(&A.sum_n[Nc + node], __dmul_rn(v, w));
    });
  }
  if (A.out_s) {
    const long long Nv = (long long)A.Nx * A.Nz;
    const int hx = cell_pair(__dsub_rn(x, A.xg[0]), A.dx).h, hz = cell_pair(__dsub_rn(z, A.zg[0]), A.dz).h;
    p2m_exact(A, A.xg, A.zg, A.Nx, A.Nz, x, z, hx, hz, [&](long long node, double w) {
      atomicAdd(&A.sum_s[node], w);
      atomicAdd(&A.sum_s[Nv + node], __dmul_rn(v, w));
    });
  }
}

// the node value P2Mastah writes (:2603-2631), or the one the node keeps
__device__ __forceinline__ double p2m_node(const MarkerArgs &A, double W, double BM, bool air_node, double old) {
  if (air_node || fp64_abs_lt(W, 1e-30)) return old;
  const double m = BM / W;
  return A.avg == 1 ? 1.0 / m : (A.avg == 2 ? exp(m) : m);
}

__global__ void __launch_bounds__(256) k_p2m_nodes(const MarkerArgs A) {
  const long long Nc = (long long)(A.Nx - 1) * (A.Nz - 1), Nv = (long long)A.Nx * A.Nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Nc) {
    if (A.out_n) A.out_n[t] = p2m_node(A, A.sum_n[t], A.sum_n[Nc + t], air(A.bcp[t]), A.out_n[t]);
  } else if (t < Nc + Nv && A.out_s) {
    const long long c1 = t - Nc;
    const int k = (int)(c1 % A.Nx);
    if (A.periodic_x == 1 && (k == 0 || k == A.Nx - 1)) {
      if (k == A.Nx - 1) return;  // written with the row's first vertex
      // :2633-2641: both ends of the row take the mean of the two
      const long long last = c1 + A.Nx - 1;
      const double fl = p2m_node(A, A.sum_s[last], A.sum_s[Nv + last], air(A.bcg[last]), A.out_s[last]);
      const double ff = p2m_node(A, A.sum_s[c1], A.sum_s[Nv + c1], air(A.bcg[c1]), A.out_s[c1]);
      const double av = 0.5 * (fl + ff);
      A.out_s[c1] = av;
      A.out_s[last] = av;
      return;
    }
    A.out_s[c1] = p2m_node(A, A.sum_s[c1], A.sum_s[Nv + c1], air(A.bcg[c1]), A.out_s[c1]);
  }
}

unsigned blocks_for(long long n) {
  const long long g = (n + 255) / 256;
  return (unsigned)(g > 0x7fffffffLL ? 0x7fffffffLL : (g < 1 ? 1 : g));
}

}  // namespace

cudaError_t launch_marker_grid(const MarkerArgs &a, cudaStream_t s) {
  k_marker_grid<<<blocks_for((long long)(a.Nx - 1) * (a.Nz - 1) + (long long)a.Nx * a.Nz), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_subgrid(const MarkerArgs &a, cudaStream_t s) {
  if (a.n > 0) k_marker_subgrid<<<blocks_for(a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_remainder(const MarkerArgs &a, cudaStream_t s) {
  k_marker_remainder<<<blocks_for((long long)(a.Nx - 1) * (a.Nz - 1) + (long long)a.Nx * a.Nz), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_update(const MarkerArgs &a, cudaStream_t s) {
  if (a.n > 0) k_marker_update<<<blocks_for(a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_weights(const MarkerArgs &a, cudaStream_t s) {
  // four CTAs per SM at most: in the common case each reads one flag and returns
  const unsigned g = blocks_for(a.n), cap = 152u * 4u;
  if (a.n > 0) k_marker_weights<<<g < cap ? g : cap, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_p2m_scatter(const MarkerArgs &a, cudaStream_t s) {
  if (a.n > 0) k_p2m_scatter<<<blocks_for(a.n), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_p2m_nodes(const MarkerArgs &a, cudaStream_t s) {
  k_p2m_nodes<<<blocks_for((long long)(a.Nx - 1) * (a.Nz - 1) + (long long)a.Nx * a.Nz), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_marker_wxz(const MarkerArgs &a, cudaStream_t s) {
  k_marker_wxz<<<blocks_for((long long)a.Nx * a.Nz), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mdz
