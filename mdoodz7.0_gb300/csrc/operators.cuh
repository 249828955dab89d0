// operators.cuh -- arguments of the RheologicalOperators kernel (operators.cu).
#pragma once
#include <cuda_runtime.h>

#include "rheo_kernels.cuh"

namespace mdz {

// output slots, in the order of mdz_operator_fields
enum OpOut { OP_D11, OP_D12, OP_D13, OP_D14, OP_D21, OP_D22, OP_D23, OP_D24, OP_DRHODP, OP_D31, OP_D32, OP_D33,
             OP_D34, OP_COUNT };

struct OpArgs {
  ModelConst M;
  PhaseConst ph[MDZ_MAX_PHASES];
  const double *ci[CI_COUNT];
  const double *vi[VI_COUNT];
  const double *T_s, *P_s, *d0_s, *phi0_s;  // vertex fields the sweep interpolated
  const double *eta_n, *eta_s;              // the sweep's averaged viscosities
  const double *perc_n[MDZ_MAX_PHASES], *perc_s[MDZ_MAX_PHASES];
  const double *peta_n[MDZ_MAX_PHASES], *peta_s[MDZ_MAX_PHASES];
  const signed char *bcp, *bcg;
  double *D[OP_COUNT];
  DevStats *stats;
  int compressible, need_lnd, polish;
};

// compact: the isotropic Newton operator with its plastic returns compacted per CTA (the
// same bits as one thread per node); ignored elsewhere.
cudaError_t launch_operators(const OpArgs &a, bool aniso, bool jacobian, bool compact, cudaStream_t s);

}  // namespace mdz
