// weno.cuh -- WENO5 level-set advection (one TVD-RK3 stage per launch).
//
// Semantics follow the reference's never-called driver cuAdvectLsJB
// (src/LevelSet/lsTransportEc.cu:201-418): Dev1thO_Downwind -> the
// left/right-biased Jiang-Peng reconstructions PhiDevPlusParameterJB /
// PhiDevMinusParameterJB (src/LevelSet/lsTools.cu:587-770) -> the upwind
// selection of advect_RS_WENO (:361-417) -> RunGK_First/Second/ThirdS
// (src/LevelSet/extrapol.cu:155-212), all on the ghost-padded grid, with the
// reference's index rules at the padded-grid edges.
//
// One fused kernel per stage instead of five launches and ten field passes:
// each block stages the backward differences of its tile (plus the stencil
// halo) in shared memory once per direction, and each cell evaluates only
// the upwind reconstruction its velocity selects (the other one is
// multiplied by zero in the reference).
#pragma once

#include "common.cuh"

namespace emix {

struct WenoArgs {
    const double *phi;   // padded field read with the stencil
    // precomputed per-cell scale factors (reflect mode only; may be null):
    // C_d = jbn_d/h_d and E_d = 12*1e-6/C_d^2, 3 components each, unpadded
    const double *wc;
    const double *we;
    // region of the padded grid to compute: [r0, r0 + rn) per axis
    int r0[3], rn[3];
    const double *phi0;  // padded field read at the cell (stages 2 and 3)
    double *out;         // padded output, or unpadded interior when out_interior
    const double *vel;   // 3 components
    const double *jbn;   // components 0, 4, 8 read
    int reflect;         // 1: vel/jbn are unpadded and read at mirrored indices
    int out_interior;
    int nxg, nyg, nzg;   // padded dimensions
    int g;               // ghost layers (used when reflect or out_interior)
    double sx, sy, sz;   // 1/h per axis
    double dt;
    int stage;           // 1, 2, 3
    int ref_bugs;
};

constexpr int kWX = 32, kWY = 4, kWZ = 2;

__global__ void __launch_bounds__(kWX *kWY *kWZ) k_weno_stage(WenoArgs a);

// Padding with mirrored ghost cells: cuSwapToGhost followed by
// cuGhostCellsMirror3dZ/Y/X (src/LevelSet/lsTools.cu:482-585,772-796).
__global__ void k_ghost_pad(double *__restrict__ ghost, const double *__restrict__ val, int g,
                            double dir, int nx, int ny, int nz);
__global__ void k_ghost_unpad(double *__restrict__ val, const double *__restrict__ ghost, int g,
                              int nx, int ny, int nz);

int launch_weno_stage(const WenoArgs &a, cudaStream_t st);

// C_d = jbn_d / h_d and E_d = 12e-6 / C_d^2 for the precomputed-scale path
__global__ void k_weno_scales(const double *__restrict__ jbn, double *__restrict__ wc,
                              double *__restrict__ we, double sx, double sy, double sz, long n);

// Reciprocal by Newton-Raphson iteration (x <- x + x(1 - d x)), seeded from the
// single-precision reciprocal of d's mantissa with d's exponent applied by
// integer arithmetic; two iterations take the ~24-bit seed to double
// precision (J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd
// ed., section 4.7).  For positive normal d well inside the double range.
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
    double x = __longlong_as_double((long long)rm);
    double e = fma(-d, x, 1.0);
    x = fma(x, e, x);
    e = fma(-d, x, 1.0);
    x = fma(x, e, x);
    return x;
}

} // namespace emix
