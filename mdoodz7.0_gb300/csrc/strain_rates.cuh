// strain_rates.cuh -- arguments of the StrainRateComponents kernel (strain_rates.cu).
#pragma once
#include <cuda_runtime.h>

#include "fp64_div.cuh"

namespace mdz {

// output slots, in the order of mdz_strain_rate_fields
enum SrOut { SR_DIV, SR_EXXD, SR_EZZD, SR_EXZ_N, SR_WXZ_N, SR_EXZ, SR_WXZ, SR_EXXD_S, SR_EZZD_S, SR_DIV_S,
             SR_COUNT };

struct StrainArgs {
  int Nx, Nz, Ncx, Ncz, periodic_x;
  Divisor dx, dz;  // mesh spacings
  double oop_half;  // 0.5 when params.out_of_plane == 1, else 0 (the factor of d(vy)/dy)
  double comp3;     // params.compressible * 1.0 / 3.0
  const double *u, *v;
  const signed char *bcp, *bcg;
  double *out[SR_COUNT];
};

// centroids and vertices per tile of one block: kSrTx x kSrTz of each
constexpr int kSrTx = 32, kSrTz = 16;

cudaError_t launch_strain_rates(const StrainArgs &a, cudaStream_t s);

}  // namespace mdz
