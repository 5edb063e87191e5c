// adjoint.cuh -- reverse-mode (adjoint) pieces of the RK3 step.
//
// Every forward kernel of the step has a transpose here:
//   k_deriv_t      D^T of the compact first derivative (transposed tridiagonal
//                  solve, then the transposed right-hand-side band)
//   adjoint cell bodies of the primitive variables, the fluxes, Smagorinsky,
//   the RK update with its wall conditions, impeller forcing and conversions,
//   and the WENO5 level-set stage (linearised weights).
// The step-level driver is adjoint.cu.
#pragma once

#include "common.cuh"
#include "deriv.cuh"
#include "deriv_tma.cuh"
#include "impeller.cuh"
#include "pointwise.cuh"
#include "weno.cuh"

namespace emix {

// out = D^T in (acc = 0) or out += D^T in (acc = 1) along `axis`, for nf <= 6
// fields; w is scratch of the size of in.  With maps (y or z, a closed
// table) the rows come by TMA through them, the same values bit for bit.
int launch_deriv_t(const DerivTTable &T, int axis, int acc, int nf, const double *const *in,
                   double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st,
                   const PencilMaps *maps = nullptr);

} // namespace emix
