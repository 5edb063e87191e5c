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
// One fused kernel per stage instead of five launches and ten field passes
// (weno_march_body, weno_march.cuh): each cell evaluates only the upwind
// reconstruction its velocity selects (the other one is multiplied by zero in
// the reference).  This header holds the pieces the stage kernel, the batched
// form and the adjoint share: the arguments, the reconstruction, the edge
// rules of the stencil and the mirrored padding.
#pragma once

#include "common.cuh"

#include <cuda.h>   // CUtensorMap (the driver entry point is fetched at run time)

namespace emix {

struct WenoArgs {
    const double *phi;   // padded field read with the stencil
    // precomputed per-cell scale factors (reflect mode only; may be null):
    // pairs (C_d, E_d) with C_d = jbn_d/h_d and E_d = kWenoEps4/C_d^2, for
    // d = 0, 1, 2 in turn, each over the unpadded grid (16-byte aligned)
    const double *wce;
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

// Padding with mirrored ghost cells: cuSwapToGhost followed by
// cuGhostCellsMirror3dZ/Y/X (src/LevelSet/lsTools.cu:482-585,772-796).
struct PadArgs {
    double *ghost;
    const double *val;
    int g;
    double dir;
    int nx, ny, nz;
    long ng;
    long qbeg, qend;   // k_ghost_pad: padded cells [qbeg, qend) only (qend = 0: all)
};
__global__ void k_ghost_pad(PadArgs a);
__global__ void k_ghost_unpad(double *__restrict__ val, const double *__restrict__ ghost, int g,
                              int nx, int ny, int nz);

// one stage on one grid (region rn[d] <= 0: the whole padded axis); with a
// tensor map of a.phi (weno_tma_map) the plane tiles come by TMA copies
int launch_weno_stage(const WenoArgs &a, cudaStream_t st, const CUtensorMap *tmap = nullptr);
// the z-marching stage kernel (weno_march.cu); a's region normalised
int launch_weno_march(const WenoArgs &a, cudaStream_t st, const CUtensorMap *tmap = nullptr);
// the tiled-copy description of a.phi's plane tiles; false (and no map) when
// the copy unit's rules do not hold: a.phi 16-byte aligned, an even padded x
// extent (row pitch a multiple of 16 bytes), extents at least the tile's
bool weno_tma_map(CUtensorMap *m, const WenoArgs &a);

// the pairs (C_d, E_d) = (jbn_d / h_d, kWenoEps4 / C_d^2) of the precomputed-scale path
__global__ void k_weno_scales(const double *__restrict__ jbn, double *__restrict__ wce, double sx,
                              double sy, double sz, long n);

// (C_d, E_d) of unpadded cell iv (nv cells)
EMIX_DEV double2 weno_scale(const double *wce, int d, long nv, long iv) {
    return reinterpret_cast<const double2 *>(wce)[d * nv + iv];
}

// Jiang-Peng WENO5 reconstruction from five differences (Phi_x_WENO,
// src/LevelSet/lsTools.cu:9-50).  Same weights 0.1/0.6/0.3 and
// epsilon = 1e-6 on (beta + eps)^2, rearranged to cut FP64 operations:
//   with d_k, e_k the second and first differences of candidate stencil k,
//   4 beta_k = (13/3) d_k^2 + e_k^2, so alpha_k ~ c_k / (4 beta_k + 4 eps)^2;
//   the three candidate values are v3 + r_k / 12 with r_1 = d_1 + 3 e_1,
//   r_2 = d_2 - 3 e_2, r_3 = d_3 - 3 e_3, so the result is
//   v3 + sum(w_k r_k) / (12 sum w_k), with w_1 = t_2 t_3, w_2 = 6 t_1 t_3,
//   w_3 = 3 t_1 t_2 (the weights times t_1 t_2 t_3 / 0.1); one reciprocal.
// eps4 is 4*epsilon for differences already scaled by the metric, or
// 4*epsilon/C^2 for unscaled differences (WENO(C v; eps) = C WENO(v; eps/C^2)).
constexpr double kWenoEps4 = 4.0e-6;

EMIX_DEV double weno5(double v1, double v2, double v3, double v4, double v5, double eps4) {
    constexpr double c13 = 13.0 / 3.0;
    const double d1 = fma(-2.0, v2, v1 + v3);
    const double e1 = fma(-4.0, v2, fma(3.0, v3, v1));
    const double d2 = fma(-2.0, v3, v2 + v4);
    const double e2 = v2 - v4;
    const double d3 = fma(-2.0, v4, v3 + v5);
    const double e3 = fma(-4.0, v4, fma(3.0, v3, v5));
    double t1 = fma(c13 * d1, d1, fma(e1, e1, eps4)); t1 *= t1;
    double t2 = fma(c13 * d2, d2, fma(e2, e2, eps4)); t2 *= t2;
    double t3 = fma(c13 * d3, d3, fma(e3, e3, eps4)); t3 *= t3;
    const double w1 = t2 * t3;
    const double w2 = (6.0 * t1) * t3;
    const double w3 = (3.0 * t1) * t2;
    const double r1 = fma(3.0, e1, d1);
    const double r2 = fma(-3.0, e2, d2);
    const double r3 = fma(-3.0, e3, d3);
    const double num = fma(w1, r1, fma(w2, r2, w3 * r3));
    const double den = 12.0 * (w1 + w2 + w3);
    return fma(num, rcp_newton(den), v3);
}

// Positions (0..n-1) of the five differences for the left-biased (u >= 0)
// and right-biased (u < 0) reconstruction at index i, with the edge rules
// of PhiDevPlusParameterJB / PhiDevMinusParameterJB (lsTools.cu:623-636,
// 716-734).
EMIX_DEV void stencil_left(int i, int n, int p[5]) {
    p[0] = i - 2; p[1] = i - 1; p[2] = i; p[3] = i + 1; p[4] = i + 2;
    if (i == 0) { p[1] = i; p[0] = i + 1; }
    if (i == 1) { p[0] = p[1]; }
    if (i == n - 1) { p[3] = i; p[4] = p[1]; }
    if (i == n - 2) { p[4] = p[3]; }
}

EMIX_DEV void stencil_right(int i, int n, int p[5]) {
    // v1..v5 = D(i+3), D(i+2), D(i+1), D(i), D(i-1)
    int im1 = i - 1, im2 = i - 2, ip1 = i + 1, ip2 = i + 2, ip3 = i + 3;
    if (i == 0) { im1 = i; }
    if (i == n - 1) { ip1 = i; ip2 = im1; ip3 = im2; }
    if (i == n - 2) { ip2 = ip1; ip3 = i; }
    if (i == n - 3) { ip3 = ip2; }
    p[0] = ip3; p[1] = ip2; p[2] = ip1; p[3] = i; p[4] = im1;
}

// mirrored interior index of padded coordinate G (ghost width g, interior n)
EMIX_DEV int mirror(int G, int g, int n) {
    int I = G - g;
    if (I < 0) I = -I - 1;
    else if (I >= n) I = 2 * n - 1 - I;
    return I;
}

// Padded cell q <- the interior cell it mirrors (times dir per reflection).
EMIX_DEV void pad_cell(const PadArgs &a, long q) {
    const int g = a.g, nx = a.nx, ny = a.ny, nz = a.nz;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g;
    const int X = (int)(q % nxg);
    const int Y = (int)((q / nxg) % nyg);
    const int Z = (int)(q / ((long)nxg * nyg));
    const int cnt = (X < g || X >= nx + g) + (Y < g || Y >= ny + g) + (Z < g || Z >= nz + g);
    double v = a.val[mirror(X, g, nx) + (long)nx * (mirror(Y, g, ny) + (long)ny * mirror(Z, g, nz))];
    for (int c = 0; c < cnt; ++c) v *= a.dir;
    a.ghost[q] = v;
}

} // namespace emix
