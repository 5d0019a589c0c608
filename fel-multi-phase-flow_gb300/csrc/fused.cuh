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

// solphi_mthinc1 for the faces solphi_mthinc2 reads (every face of rows 1..n in
// the two directions normal to it, faces 0..n along it); list/count: device scratch
// of >= (ni+2)(nj+2)(nk+2) ints and one int.
void mthinc_fluxes(cudaStream_t s, const Grid& g, double dxinv, double dyinv, double dzinv, double dt, double bet,
                   const double* phi, const double* gx, const double* gy, const double* gz, const double* u,
                   const double* v, const double* w, double* fx, double* fy, double* fz, int* list, int* count);

}  // namespace fused
}  // namespace fmf
