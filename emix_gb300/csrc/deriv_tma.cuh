// deriv_tma.cuh -- y/z pencil sweeps with their rows staged by TMA
// (deriv_tma.cu).
//
// The y/z derivative (out += D f, the flux divergence's y and z passes, or
// out = D f, the velocity gradients' y and z passes as one launch) and its
// transpose (the adjoint's D^T passes) of the load kernels with the same
// arithmetic, but every row the sweeps read comes
// through shared memory: a block of 32, 64 or 128 pencils (lanes along x)
// has one thread issue 3-D tiled copies of 4 rows x the block's pencils
// (4 KB at 128) into a ring of three buffers, completion on an mbarrier per
// buffer; the forward sweep reads f from the ring, the backward sweep w (and
// the accumulation target).  Every wait is bounded: a block whose copy does
// not arrive counts itself (emix_pencil_tma_timeouts), waits (bounded) for
// the copies it still has in flight and leaves its pencils unwritten.
#pragma once

#include "deriv.cuh"

#include <cuda.h>

namespace emix {

constexpr int kPtR = 4;     // rows per copy
constexpr int kPtS = 3;     // buffers in the ring

// tensor maps of one launch: per field its input f, forward-sweep buffer w
// and accumulation target out, as 3-D (nx, ny, nz) tensors with boxes of
// `width` pencils x kPtR rows along the launch's axis; width (32, 64 or
// 128, the block's threads) is the one that idles the fewest lanes of a row
struct PencilMaps {
    CUtensorMap in[kMaxFields], w[kMaxFields], out[kMaxFields];
    int axis[kMaxFields];   // 1 (y) or 2 (z) per field
    int width;
};

// Encodes the maps of nf fields, field f along axis[f]; false where the copy
// unit's rules do not hold (nx odd, a field not 16-byte aligned) or the
// driver lacks the encoder.
bool pencil_tma_maps(PencilMaps *M, const int *axis, int nf, const double *const *in, double *const *w,
                     double *const *out, int nx, int ny, int nz);

// D in along each field's axis, rows staged by TMA through the maps M:
// out += D in (EPI_ACCUM) or out = D in (EPI_STORE, w = out); fields [0, nfa)
// with table Ta, the rest with Tb (fields as in launch_deriv), the tables
// all closed or all cyclic.
int launch_deriv_yz_tma(const DerivTable &Ta, const DerivTable &Tb, const PencilMaps &M, int epi, int nfa, int nf,
                        const double *const *in, double *const *w, double *const *out, int nx, int ny, int nz,
                        cudaStream_t st);

// D^T in along each field's axis (a closed table T), rows staged by TMA
// through the maps M: out = D^T in (acc = 0) or out += D^T in (acc = 1), with
// w the forward sweep's buffer; the same values bit for bit as the load
// kernel of launch_deriv_t.
int launch_deriv_t_yz_tma(const DerivTTable &T, const PencilMaps &M, int acc, int nf, const double *const *in,
                          double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st);

} // namespace emix
