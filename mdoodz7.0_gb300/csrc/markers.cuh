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
  double near_x, near_z;            // distances up to which a P2Mastah weight is surely >= 1e-30 (-1: none)
  const double *xg, *zg, *xvz, *zvx;
  const signed char *bcp, *bcg;
  const double *sxxd, *szzd, *sxxd0, *szzd0, *sxz, *sxz0, *u, *v;
  double *wxz;
  const double *x, *z;
  const int *phase;
  double *m_sxxd, *m_szzd, *m_sxz, *m_nx, *m_nz;
  // scratch written by k_marker_grid
  double2 *inc_n;    // centroids: sxxd - sxxd0, szzd - szzd0 (0 at air)
  double *inc_s;     // vertices: sxz - sxz0 (0 where BCg is 30)
  double2 *grad_n;   // centroids: du/dx, dv/dz (0 at air)
  double2 *grad_s;   // vertices: du/dz, dv/dx (0 where BCg is 30)
  unsigned char *hit;  // vertex received a P2Mastah weight >= 1e-30
  double *WM;          // exact per-vertex weight sums, filled only when *exotic is set
  int *exotic;         // a weight below 1e-30 that is not zero, or not finite, was seen
  DevStats *stats;
};

// grid: stress increments and velocity gradients per node, scratch cleared
cudaError_t launch_marker_grid(const MarkerArgs &a, cudaStream_t s);
// markers: director, stress increments, rotation, and the P2Mastah hit flags
cudaError_t launch_marker_update(const MarkerArgs &a, cudaStream_t s);
// markers again, only when *exotic is set: the exact P2Mastah weight sums
cudaError_t launch_marker_weights(const MarkerArgs &a, cudaStream_t s);
// vertices: wxz where the weight sum reaches 1e-30, and the periodic column average
cudaError_t launch_marker_wxz(const MarkerArgs &a, cudaStream_t s);

}  // namespace mdz
