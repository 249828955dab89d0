// prep.cuh -- arguments of the sweep's input-preparation kernels (prep.cu):
// Softening over the grid (CohesionFrictionDilationGrid) and ShearModCompExpGrid.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/mdz_rheo.h"
#include "fp64_bits.cuh"
#include "fp64_div.cuh"
#include "rheo_kernels.cuh"

namespace mdz {

// host side of fp64_order_key (fp64_bits.cuh): the same key, for the folded thresholds
inline unsigned long long order_key_host(double x) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
inline bool is_nan_host(double x) {
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
  return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

// per-phase constants of Softening (RheologyDensity.c:1432-1532), folded on the host
// with the reference's own expressions so every folded value is bitwise the same
struct SoftPhase {
  double phi, psi, C, phi_end, psi_end, C_end, pls_start, pls_end, Hc;
  unsigned long long key_start, key_end;  // fp64_order_key of pls_start / pls_end
  int start_nan, end_nan;                 // a NaN bound makes its comparisons false
  double q_phi, q_psi, q_C;              // style 0: (x_end - x) / (pls_end - pls_start)
  double mu_strain;                      // style 1: 0.5 * (pls_end + pls_start)
  Divisor dstrain;                       //          pls_end - pls_start
  double half_d[3], d[3], x_end_[3];     //          dX / 2.0, dX = x - x_end, x_end  (fric, dil, C)
  Divisor x0[3];                         //          the erfc form at zero strain
  int phi_soft, psi_soft, coh_soft;
};

struct SoftArgs {
  long long Nc, Nv;
  int np, style, noise;
  SoftPhase ph[MDZ_MAX_PHASES];
  const double *perc_n[MDZ_MAX_PHASES], *perc_s[MDZ_MAX_PHASES];
  const signed char *bcp, *bcg;
  const double *strain_n, *strain_s, *noise_n, *noise_s;
  double *fric_n, *dil_n, *C_n, *fric_s, *dil_s, *C_s;
};

struct ModArgs {
  long long Nc, Nv;
  int Nx, np, periodic_x;
  int skip_zero;  // every G and bet is finite and nonzero: a zero fraction adds nothing
  Divisor G[MDZ_MAX_PHASES], bet[MDZ_MAX_PHASES];
  double alp[MDZ_MAX_PHASES];
  const double *perc_n[MDZ_MAX_PHASES], *perc_s[MDZ_MAX_PHASES];
  const signed char *bcp, *bcg;
  double *mu_n, *bet_n, *alp_n, *mu_s, *bet_s;
  DevStats *stats;
};

cudaError_t launch_softening(const SoftArgs &a, cudaStream_t s);
cudaError_t launch_moduli(const ModArgs &a, cudaStream_t s);

}  // namespace mdz
