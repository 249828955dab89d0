// markers.cuh -- arguments of the marker stress update (markers.cu): UpdateParticleStress.
#pragma once
#include <cuda_runtime.h>

#include "fp64_div.cuh"
#include "rheo_kernels.cuh"

namespace mdz {

struct MarkerArgs {
  long long n;                      // markers
  int Nx, Nz, periodic_x;           // vertices
  int elastic, rotation, director;  // switches (director: anisotropy and advection on)
  int stencil;                      // P2Mastah's interpolation stencil, 1 or 9
  double dt;
  Divisor dx, dz;                   // mesh spacing
  Divisor dx_itp, dz_itp;           // P2Mastah's weight lengths: dx/2 (stencil 1) or 3 dx/2 (stencil 9)
  const double *xg, *zg, *xvz, *zvx;
  const signed char *bcp, *bcg;
  const double *sxxd, *szzd, *sxxd0, *szzd0, *sxz, *sxz0, *u, *v;
  double *wxz;
  const double *x, *z;
  const int *phase;
  double *m_sxxd, *m_szzd, *m_sxz, *m_nx, *m_nz;
  double *WM;  // per-vertex sum of marker weights (scratch, zeroed before the launch)
  DevStats *stats;
};

// markers: director, stress increments, rotation, and the weight scatter into WM
cudaError_t launch_marker_update(const MarkerArgs &a, cudaStream_t s);
// vertices: wxz where the weight sum reaches 1e-30, and the periodic column average
cudaError_t launch_marker_wxz(const MarkerArgs &a, cudaStream_t s);

}  // namespace mdz
