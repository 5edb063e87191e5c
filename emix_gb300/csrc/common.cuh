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

// Streaming multiprocessors of the current device (queried once per device
// ordinal and cached; 1 if the query fails).
int device_sms();

// Blocks of `bs` threads for a grid-stride loop over n items: one block per
// bs items, at most `per_sm` blocks per SM of the current device.
inline int grid_cap(long n, int per_sm, int bs = 256) {
    long b = (n + bs - 1) / bs;
    const long cap = (long)device_sms() * per_sm;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

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
// Reciprocal seeded from the single-precision reciprocal of d's mantissa
// (d's exponent applied by integer arithmetic), then one third-order step of
// the iteration for 1/d: with e = 1 - d x, x <- x (1 + e + e^2), the first
// terms of x / (1 - e) (J.-M. Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed., section 4.7, on Newton-Raphson-like iterations).  The
// seed's relative error is below 2^-22, so the step's error e^3 is below
// 2^-66: a correctly rounded result up to the last operation's rounding.
// Three FMAs.  For normal d of either sign well inside the double range.
EMIX_DEV double rcp_newton(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int ebits = (int)(b >> 52) & 0x7ff;                       // biased exponent
    const unsigned int mant = (unsigned int)((b >> 29) & 0x7fffff); // top 23 mantissa bits
    const float m = __uint_as_float(0x3f800000u | mant);            // in [1, 2)
    const unsigned int rf = __float_as_uint(__frcp_rn(m));          // in (0.5, 1]
    // rebuild 1/m as a double and scale by 2^-(ebits-1023)
    const int fexp = (int)(rf >> 23) & 0xff;
    const unsigned long long rm = ((unsigned long long)(fexp - 127 + 1023 - (ebits - 1023)) << 52) |
                                  ((unsigned long long)(rf & 0x7fffff) << 29);
    // d's sign on the seed: the step below then converges for negative d too
    const double x = __longlong_as_double((long long)(rm | (b & 0x8000000000000000ull)));
    const double e = fma(-d, x, 1.0);
    return fma(x, fma(e, e, e), x);
}

// 1/d by rcp_newton where its exponent arithmetic is safe (|d| within
// 2^-1021 .. 2^1020), by division otherwise (zero, subnormal, huge, inf, NaN).
EMIX_DEV double rcp_fast(double d) {
    const int ebits = (int)((unsigned long long)__double_as_longlong(d) >> 52) & 0x7ff;
    return (ebits >= 2 && ebits <= 2043) ? rcp_newton(d) : 1.0 / d;
}

// sqrt(x) from the single-precision reciprocal square root of x's mantissa
// (exponent halved by integer arithmetic), then one third-order step: with
// s = x y and e = 1 - s y, sqrt(x) = s (1 - e)^(-1/2) ~ s (1 + e/2 + 3e^2/8),
// the first terms of the binomial series (the same family of iterations as
// rcp_newton, Muller et al., section 4.7).  The seed's relative error is below
// 2^-21, the step's below 2^-60: within an ulp of the correctly rounded root.
// Five FP64 operations; zero, negative, subnormal, huge, inf and NaN
// arguments go to sqrt().
EMIX_DEV double sqrt_fast(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ebits = (int)(b >> 52) & 0x7ff;
    if (ebits < 2 || ebits > 2045 || (b >> 63)) return sqrt(x);
    const int e = ebits - 1023;   // x = m 2^e, m in [1, 2)
    const int odd = e & 1;
    // f = m 2^odd in [1, 4), top 23 mantissa bits
    const float f = __uint_as_float(((127u + (unsigned)odd) << 23) | (unsigned int)((b >> 29) & 0x7fffff));
    const unsigned int rb = __float_as_uint(rsqrtf(f));
    // y = rsqrt(f) 2^-((e - odd) / 2)
    const int half = (e - odd) / 2;
    const int fexp = (int)(rb >> 23) & 0xff;
    const double y = __longlong_as_double(
        (long long)(((unsigned long long)(fexp - 127 + 1023 - half) << 52) | ((unsigned long long)(rb & 0x7fffff) << 29)));
    const double s = x * y;
    const double ee = fma(-s, y, 1.0);
    return fma(s, ee * fma(0.375, ee, 0.5), s);
}

// 1/sqrt(x): the seed of sqrt_fast, then one third-order step
// y (1 + e/2 + 3e^2/8) with e = 1 - x y^2 (the same binomial series).  Five
// FP64 operations; zero, negative, subnormal, huge, inf and NaN arguments go
// to 1 / sqrt().
EMIX_DEV double rsqrt_fast(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ebits = (int)(b >> 52) & 0x7ff;
    if (ebits < 2 || ebits > 2045 || (b >> 63)) return 1.0 / sqrt(x);
    const int e = ebits - 1023;
    const int odd = e & 1;
    const float f = __uint_as_float(((127u + (unsigned)odd) << 23) | (unsigned int)((b >> 29) & 0x7fffff));
    const unsigned int rb = __float_as_uint(rsqrtf(f));
    const int half = (e - odd) / 2;
    const int fexp = (int)(rb >> 23) & 0xff;
    const double y = __longlong_as_double(
        (long long)(((unsigned long long)(fexp - 127 + 1023 - half) << 52) | ((unsigned long long)(rb & 0x7fffff) << 29)));
    const double ee = fma(-x * y, y, 1.0);
    return fma(y, ee * fma(0.375, ee, 0.5), y);
}

struct DerivRow {
    double A, B, m, g;
};

// The same factorisation on the scaled unknowns u_i = w_i / k_i, z_i = x_i / k_i,
// k_i = A_i on stencil rows and 1 on closure rows: a stencil row's forward step
// is u_i = (d1 + c d2) - mu u_{i-1}, the backward z_i = u_i - gu z_{i+1}, and
// x_i = k z_i.  Used where the result is accumulated (out += k z in one FMA).
struct DerivRowU {
    double c, mu, gu, k;
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
    const DerivRowU *urows;  // n rows of the scaled form
    const double *u0s;     // ku weights of the scaled form: u0_k k_k (periodic)
    double sm1s;           // sm1 k_{n-1} (periodic)
};

// Parallel cyclic reduction (PCR) followed by Thomas, for one compact
// operator: `steps` PCR steps split the system into 2^steps interleaved
// subsystems (rows i = r (mod 2^steps)), each then solved by Thomas.  The
// matrix side of every step and the subsystems' factors are precomputed; a
// pencil costs per row the right-hand-side stencil, two FMAs per PCR step and
// the three operations of the factored Thomas sweeps.  The cyclic scheme
// solves the Sherman-Morrison-modified non-cyclic system A' and corrects by
// zz = A'^{-1} u at the end.
constexpr int kPcrMaxSteps = 5;
constexpr int kPcrMaxN = 160;      // pencils of up to 160 rows (5 per lane at 5 steps)
struct PcrTable {
    int n, steps, periodic;
    int nlo, nhi;               // closure rows at each end (non-cyclic schemes)
    const double *ra, *rb;      // n: interior right-hand side (1/h folded in)
    const double *cl;           // 4n: closure right-hand side (f_0..f_3 low, f_{n-1}..f_{n-4} high)
    const double *al, *ga;      // steps x n: d_i += al d_{i-h} + ga d_{i+h}, h = 2^k
    const double *ib, *mt, *gt; // n: Thomas of the subsystems: w = d ib - mt w_prev, x = w - gt x_next
    const double *zz;           // n (cyclic): A'^{-1} u
    double sm1, sm2;            // cyclic: fact = (y_0 + sm1 y_{n-1}) sm2, x = y - fact zz
};
int get_pcr_table(int scheme, int n, double h, int steps, PcrTable *out);

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
