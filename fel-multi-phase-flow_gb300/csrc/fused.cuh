// fused.cuh -- kernels of the fused time step (fmf_ctx_step).  These compute the
// same quantities as the drop-in kernels of ops.cuh but fuse reference
// subroutines, skip work whose result the step never reads, and let nvcc
// contract multiply-adds; they are checked against the oracle at 1e-10.
#pragma once
#include "fmf_common.cuh"

namespace fmf {
namespace fused {

void weno5_both(cudaStream_t s, const Grid& g, double dxi, double dyi, double dzi, const double* u,
                const double* v, const double* w, const double* uo, const double* vo, const double* wo,
                double* const* adv, double* const* advo);

}  // namespace fused
}  // namespace fmf
