// common.cuh -- shared definitions for the eMix3d GB300 kernels.
//
// Layout everywhere: Fortran column-major, i fastest, linear index
// i + nx*(j + ny*k) (the reference's ArrayDev3D, src/Engine/cuArray.cu:123);
// multi-component fields stack components with stride nx*ny*nz.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "../../include/emix_gb300.h"

#define EMIX_DEV __device__ __forceinline__

namespace emix {

// Host-side CUDA error check that turns a failing call into a status code.
#define EMIX_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) {                                              \
            ::emix::set_last_error(_e, #expr, __FILE__, __LINE__);            \
            return EMIX_ERR_CUDA;                                             \
        }                                                                     \
    } while (0)

void set_last_error(cudaError_t e, const char *what, const char *file, int line);
void set_last_message(const char *msg);

inline size_t ncell(int nx, int ny, int nz) { return (size_t)nx * (size_t)ny * (size_t)nz; }

// Per-axis factor table of one compact first-derivative operator, built on
// the host by build_deriv_table() and read by the pencil kernels.
//
// For row i the kernels evaluate
//   r'_i = A_i (f_{i+1} - f_{i-1}) + B_i (f_{i+2} - f_{i-2})      (interior)
//   r'_i = sum_k C_{i,k} f_{idx(i,k)}                               (closure rows)
//   w_i  = r'_i - m_i w_{i-1}                                       (forward)
//   x_i  = w_i - g_i x_{i+1}                                        (backward)
// where the 1/h scale and the Thomas pivot 1/bet_i are already folded into
// A_i, B_i, C_{i,k}.  Periodic operators add the Sherman-Morrison terms.
struct DerivRow {
    double A, B, m, g;
};

constexpr int kMaxClosure = 4;   // closure rows at each end
constexpr int kTableMaxN = 4096; // longest supported pencil

struct DerivTable {
    int n;          // pencil length
    int scheme;     // EMIX_SCHEME_*
    int periodic;   // 1 for the cyclic operator
    int nlo, nhi;   // closure rows at the low / high end (explicit 4-point stencils)
    // periodic extras (Sherman-Morrison): y0 = sum_{k<ku} U0_k w_k,
    // fact = (y0 + sm1*y_{n-1})*sm2, x_i = y_i - fact*zz_i for i < zlo or i >= zhi
    int ku;
    int zlo, zhi;
    double sm1, sm2;
    const DerivRow *rows;  // n rows
    const double *clo;     // nlo x 4: row i < nlo, coefficients of f_0..f_3
    const double *chi;     // nhi x 4: row n-1-k, coefficients of f_{n-1}..f_{n-4}
    const double *u0;      // ku weights (periodic)
    const double *zz;      // n values (periodic)
};

// Build the table for (scheme, n, h); rows/u0/zz returned in host vectors.
// Host arrays: rows[n], clo[kMaxClosure*4], chi[kMaxClosure*4], u0[n], zz[n].
int build_deriv_table_host(int scheme, int n, double h, DerivTable &t, DerivRow *rows,
                           double *clo, double *chi, double *u0, double *zz);

// Device-resident table for (scheme, n, h) on the current device, built on
// first use and kept for the life of the process.  Not to be called while a
// stream is being captured.
int get_deriv_table(int scheme, int n, double h, DerivTable *out);

// per-device grow-only scratch of the library (deriv_ops.cu); calls that use
// it and overlap on one device race
int device_scratch(size_t bytes, double **out);

// Transposed operator D^T (the adjoint): y_i = r_i ib_i - m_i y_{i-1},
// z_i = y_i - g_i z_{i+1} solves A^T z = r; then out_j = sum_k bt[7j+k] z_{j+k-3}.
// For the cyclic scheme D^T = -D and `neg` is the forward table of -D.
struct DerivTRow {
    double ib, m, g;
};
struct DerivTTable {
    int n, periodic;
    const DerivTRow *rows;
    const double *bt;
    // rows jlo..jhi of B^T are the interior's antisymmetric stencil
    // tb z_{j-2} + ta z_{j-1} - ta z_{j+1} - tb z_{j+2} (jlo > jhi: none)
    int jlo, jhi;
    double ta, tb;
    DerivTable neg;
};
int get_deriv_t_table(int scheme, int n, double h, DerivTTable *out);

} // namespace emix
