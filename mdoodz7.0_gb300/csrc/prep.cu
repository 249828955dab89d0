// prep.cu -- the sweep's per-node input preparation on the GPU.
//
// k_softening: CohesionFrictionDilationGrid (MDLIB/RheologyDensity.c:1539-1628) after
// its particle interpolation.  Per node: Softening (:1432-1532) of friction, dilation
// and cohesion of every phase against the node's plastic strain, the arithmetic phase
// average the caller fixes (average = 0, :1541), and the marker noise on the cohesion
// (:1573, :1610).  Air nodes get zeros.
// k_moduli: ShearModCompExpGrid (:1634-1755).  Per node: harmonic phase averages of G
// and bet (average = 1, :1637), arithmetic average of alp at centroids, and, when
// periodic in x, the mean of the first and last vertex of each row.
//
// One thread per node, centroids first, then vertices; every access is coalesced.
// Both kernels are short per node and bound by the FP64 pipe (divisions by the phase
// constants use the host reciprocal form of fp64_div.cuh; tests on the bits of a double
// run on the integer pipe, fp64_bits.cuh).  Every product and sum is
// written with explicit round-to-nearest intrinsics, so no FMA contraction changes a
// bit against the reference; the per-phase constants are folded on the host with the
// reference's own expressions.
#include "prep.cuh"

namespace mdz {

namespace {

// one field of the erfc form: ((x - (dX/2) t) - x_end) dX / x0 + x_end (:1451-1454)
__device__ __forceinline__ double erfc_soften(const SoftPhase &P, int k, double x, double t) {
  const double v = __dsub_rn(__dsub_rn(x, __dmul_rn(P.half_d[k], t)), P.x_end_[k]);
  return __dadd_rn(div_by(__dmul_rn(v, P.d[k]), P.x0[k]), P.x_end_[k]);
}

// Softening of one phase at plastic strain s (RheologyDensity.c:1440-1502); ks is
// fp64_order_key(s) and s_nan whether s is NaN, for the comparisons of style 0
__device__ __forceinline__ void soften(const SoftPhase &P, int style, double s, unsigned long long ks, bool s_nan,
                                       double &f, double &d, double &c) {
  f = P.phi; d = P.psi; c = P.C;
  if (style == 1) {
    // erfc form (:1446-1470); the three fields share the erfc argument
    if (P.phi_soft == 1 || P.psi_soft == 1 || P.coh_soft == 1) {
      const double t = erfc(div_by(-__dsub_rn(s, P.mu_strain), P.dstrain));
      if (P.phi_soft == 1) f = erfc_soften(P, 0, P.phi, t);
      if (P.psi_soft == 1) d = erfc_soften(P, 1, P.psi, t);
      if (P.coh_soft == 1) c = erfc_soften(P, 2, P.C, t);
    }
  } else if (style == 2) {
    c = fmax(__dadd_rn(P.C, __dmul_rn(P.Hc, s)), P.C_end);  // :1472-1475
  } else {
    // piecewise linear (:1478-1499): three tests applied in turn, as in the reference;
    // the comparisons run on integer keys (IEEE semantics: false when either side is NaN)
    const bool below_start = !s_nan && !P.start_nan && ks < P.key_start;
    const bool from_end = !s_nan && !P.end_nan && ks >= P.key_end;
    const bool from_start = !s_nan && !P.start_nan && ks >= P.key_start;
    const bool below_end = !s_nan && !P.end_nan && ks < P.key_end;
    if (below_start) {
      if (P.phi_soft == 1) f = P.phi;
      if (P.psi_soft == 1) d = P.psi;
      if (P.coh_soft == 1) c = P.C;
    }
    if (from_end) {
      if (P.phi_soft == 1) f = P.phi_end;
      if (P.psi_soft == 1) d = P.psi_end;
      if (P.coh_soft == 1) c = P.C_end;
    }
    if (from_start && below_end) {
      if (P.phi_soft == 1) f = __dadd_rn(P.phi, __dmul_rn(P.q_phi, s));
      if (P.psi_soft == 1) d = __dadd_rn(P.psi, __dmul_rn(P.q_psi, s));
      if (P.coh_soft == 1) c = __dadd_rn(P.C, __dmul_rn(P.q_C, s));
    }
  }
}

__global__ void __launch_bounds__(256) k_softening(const SoftArgs A) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.Nc + A.Nv) return;
  const bool cen = i < A.Nc;
  const long long n = cen ? i : i - A.Nc;
  const bool solid = cen ? (A.bcp[n] != 30 && A.bcp[n] != 31) : (A.bcg[n] != 30);
  double fric = 0.0, dil = 0.0, C = 0.0;
  if (solid) {
    const double s = cen ? A.strain_n[n] : A.strain_s[n];
    const unsigned long long ks = fp64_order_key(s);
    const bool s_nan = fp64_is_nan(s);
    for (int p = 0; p < A.np; p++) {
      const double w = cen ? A.perc_n[p][n] : A.perc_s[p][n];
      double f, d, c;
      soften(A.ph[p], A.style, s, ks, s_nan, f, d, c);
      // a zero fraction of finite values adds a zero, which leaves the sums unchanged
      if (fp64_is_zero(w) && fp64_finite(f) && fp64_finite(d) && fp64_finite(c)) continue;
      fric = __dadd_rn(fric, __dmul_rn(w, f));
      dil = __dadd_rn(dil, __dmul_rn(w, d));
      C = __dadd_rn(C, __dmul_rn(w, c));
    }
    if (A.noise == 1) {
      const double r = cen ? A.noise_n[n] : A.noise_s[n];
      C = __dadd_rn(C, __dmul_rn(r, C));
    }
  }
  double *fo = cen ? A.fric_n : A.fric_s, *dout = cen ? A.dil_n : A.dil_s, *co = cen ? A.C_n : A.C_s;
  fo[n] = fric;
  dout[n] = dil;
  co[n] = C;
}

// harmonic averages of G and bet over the phases of one node (RheologyDensity.c:1656-1684,
// :1707-1741); alp accumulates the arithmetic average when given
__device__ __forceinline__ void harmonic(const ModArgs &A, const double *const *perc, long long n, double &mu,
                                         double &bet, double *alp) {
  mu = 0.0; bet = 0.0;
  double a = 0.0;
  for (int p = 0; p < A.np; p++) {
    const double w = perc[p][n];
    if (A.skip_zero && fp64_is_zero(w)) continue;
    mu = __dadd_rn(mu, div_by(w, A.G[p]));
    bet = __dadd_rn(bet, div_by(w, A.bet[p]));
    if (alp) a = __dadd_rn(a, __dmul_rn(w, A.alp[p]));
  }
  mu = 1.0 / mu;
  bet = 1.0 / bet;
  if (alp) *alp = a;
}

__device__ __forceinline__ void vertex_moduli(const ModArgs &A, long long c1, double &mu, double &bet) {
  mu = 0.0; bet = 0.0;
  if (A.bcg[c1] != 30) harmonic(A, A.perc_s, c1, mu, bet, nullptr);
}

__global__ void __launch_bounds__(256) k_moduli(const ModArgs A) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.Nc + A.Nv) return;
  if (i < A.Nc) {
    const long long c0 = i;
    double mu = 0.0, bet = 0.0, alp = 0.0;
    const signed char bc = A.bcp[c0];
    if (bc != 30 && bc != 31) harmonic(A, A.perc_n, c0, mu, bet, &alp);
    if (fp64_is_inf(mu)) {  // :1688-1690
      const unsigned long long key = ((unsigned long long)c0 << 8) | (unsigned long long)(-MDZ_ESHEAR_INF);
      atomicMin(&A.stats->err_key, key);
    }
    A.mu_n[c0] = mu;
    A.bet_n[c0] = bet;
    A.alp_n[c0] = alp;
    return;
  }
  const long long c1 = i - A.Nc;
  const int k = (int)(c1 % A.Nx);
  double mu, bet;
  if (A.periodic_x == 1 && k == A.Nx - 1) return;  // written by the row's first vertex
  vertex_moduli(A, c1, mu, bet);
  if (A.periodic_x == 1 && k == 0) {
    // :1744-1752: both ends of the row take the mean of the two
    double mu_e, bet_e;
    vertex_moduli(A, c1 + A.Nx - 1, mu_e, bet_e);
    mu = 0.5 * (mu_e + mu);
    bet = 0.5 * (bet_e + bet);
    A.mu_s[c1 + A.Nx - 1] = mu;
    A.bet_s[c1 + A.Nx - 1] = bet;
  }
  A.mu_s[c1] = mu;
  A.bet_s[c1] = bet;
}

unsigned grid_for(long long n) {
  const long long g = (n + 255) / 256;
  return (unsigned)(g > 0x7fffffffLL ? 0x7fffffffLL : g);
}

}  // namespace

cudaError_t launch_softening(const SoftArgs &a, cudaStream_t s) {
  if (a.Nc + a.Nv > 0) k_softening<<<grid_for(a.Nc + a.Nv), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_moduli(const ModArgs &a, cudaStream_t s) {
  if (a.Nc + a.Nv > 0) k_moduli<<<grid_for(a.Nc + a.Nv), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mdz
