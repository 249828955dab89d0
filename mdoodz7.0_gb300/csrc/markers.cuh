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
  int subgrid;                      // subgrid_diffusion 2: relaxation of marker stresses (elastic only)
  int np;                           // phases (subgrid diffusion 2)
  Divisor G[MDZ_MAX_PHASES];        // shear modulus per phase (subgrid diffusion 2)
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
  // subgrid diffusion 2
  const double *xc, *zc, *eta_s;  // centroid coordinates (Ncx, Ncz), vertex viscosity
  double *m_sub;                  // per marker: the subgrid increments of sxxd, szzd, sxz [3][n]
  double *sum_n;                  // centroids: P2Mastah's WM, BMWM of dsxx, BMWM of dszz [3][Nc]
  double *sum_s;                  // vertices: WM, BMWM of dsxz [2][Nv]
  // P2Mastah of a marker array (mdz_rheo_p2mastah)
  const double *val;              // per marker
  int avg;                        // 0 arithmetic, 1 harmonic, 2 geometric
  double *out_n, *out_s;          // node fields (either may be null)
  DevStats *stats;
};

// grid: stress increments and velocity gradients per node, scratch cleared
cudaError_t launch_marker_grid(const MarkerArgs &a, cudaStream_t s);
// markers (subgrid diffusion 2): the subgrid increments and their P2Mastah sums
cudaError_t launch_marker_subgrid(const MarkerArgs &a, cudaStream_t s);
// grid (subgrid diffusion 2): the grid's increments less the subgrid ones
cudaError_t launch_marker_remainder(const MarkerArgs &a, cudaStream_t s);
// markers: director, stress increments, rotation, and the P2Mastah hit flags
cudaError_t launch_marker_update(const MarkerArgs &a, cudaStream_t s);
// markers again, only when *exotic is set: the exact P2Mastah weight sums
cudaError_t launch_marker_weights(const MarkerArgs &a, cudaStream_t s);
// vertices: wxz where the weight sum reaches 1e-30, and the periodic column average
cudaError_t launch_marker_wxz(const MarkerArgs &a, cudaStream_t s);
// P2Mastah of a marker array: the weight sums (markers), then the node values (nodes)
cudaError_t launch_p2m_scatter(const MarkerArgs &a, cudaStream_t s);
cudaError_t launch_p2m_nodes(const MarkerArgs &a, cudaStream_t s);

}  // namespace mdz
