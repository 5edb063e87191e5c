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

constexpr int kWX = 32, kWY = 4, kWZ = 2;

__global__ void __launch_bounds__(kWX *kWY *kWZ) k_weno_stage(WenoArgs a);

// Padding with mirrored ghost cells: cuSwapToGhost followed by
// cuGhostCellsMirror3dZ/Y/X (src/LevelSet/lsTools.cu:482-585,772-796).
struct PadArgs {
    double *ghost;
    const double *val;
    int g;
    double dir;
    int nx, ny, nz;
    long ng;
};
__global__ void k_ghost_pad(PadArgs a);
__global__ void k_ghost_unpad(double *__restrict__ val, const double *__restrict__ ghost, int g,
                              int nx, int ny, int nz);

int launch_weno_stage(const WenoArgs &a, cudaStream_t st);
// the z-marching form of the stage (weno_march.cu); a's region normalised
int launch_weno_march(const WenoArgs &a, cudaStream_t st);

// the pairs (C_d, E_d) = (jbn_d / h_d, kWenoEps4 / C_d^2) of the precomputed-scale path
__global__ void k_weno_scales(const double *__restrict__ jbn, double *__restrict__ wce, double sx,
                              double sy, double sz, long n);

// (C_d, E_d) of unpadded cell iv (nv cells)
EMIX_DEV double2 weno_scale(const double *wce, int d, long nv, long iv) {
    return reinterpret_cast<const double2 *>(wce)[d * nv + iv];
}

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

// One TVD stage on one (virtual) block of kWX x kWY x kWZ cells.
EMIX_DEV void weno_stage_body(const WenoArgs &a, uint3 bid, uint3 tid3) {
    // backward differences phi(p) - phi(p-1) (D(0) = phi(1) - phi(0)),
    // unscaled, for the tile plus the [-2, +3] stencil halo of each axis
    __shared__ double Dx[kWZ][kWY][kWX + 5];
    __shared__ double Dy[kWZ][kWY + 5][kWX];
    __shared__ double Dz[kWZ + 5][kWY][kWX];

    const int nxg = a.nxg, nyg = a.nyg, nzg = a.nzg;
    const int x0 = a.r0[0] + bid.x * kWX, y0 = a.r0[1] + bid.y * kWY,
              z0 = a.r0[2] + bid.z * kWZ;
    const int xe = a.r0[0] + a.rn[0], ye = a.r0[1] + a.rn[1], ze = a.r0[2] + a.rn[2];
    const long sxy = (long)nxg * nyg;
    const double *__restrict__ phi = a.phi;
    const int tid = tid3.x + kWX * (tid3.y + kWY * tid3.z);
    constexpr int NT = kWX * kWY * kWZ;

    for (int t = tid; t < kWZ * kWY * (kWX + 5); t += NT) {
        const int xi = t % (kWX + 5), yz = t / (kWX + 5);
        const int yi = yz % kWY, zi = yz / kWY;
        const int X = x0 - 2 + xi, Y = y0 + yi, Z = z0 + zi;
        double v = 0.0;
        if (X >= 0 && X < nxg && Y < nyg && Z < nzg) {
            const long id = X + (long)nxg * Y + sxy * Z;
            v = X == 0 ? phi[id + 1] - phi[id] : phi[id] - phi[id - 1];
        }
        Dx[zi][yi][xi] = v;
    }
    for (int t = tid; t < kWZ * (kWY + 5) * kWX; t += NT) {
        const int xi = t % kWX, yz = t / kWX;
        const int yi = yz % (kWY + 5), zi = yz / (kWY + 5);
        const int X = x0 + xi, Y = y0 - 2 + yi, Z = z0 + zi;
        double v = 0.0;
        if (X < nxg && Y >= 0 && Y < nyg && Z < nzg) {
            const long id = X + (long)nxg * Y + sxy * Z;
            v = Y == 0 ? phi[id + nxg] - phi[id] : phi[id] - phi[id - nxg];
        }
        Dy[zi][yi][xi] = v;
    }
    for (int t = tid; t < (kWZ + 5) * kWY * kWX; t += NT) {
        const int xi = t % kWX, yz = t / kWX;
        const int yi = yz % kWY, zi = yz / kWY;
        const int X = x0 + xi, Y = y0 + yi, Z = z0 - 2 + zi;
        double v = 0.0;
        if (X < nxg && Y < nyg && Z >= 0 && Z < nzg) {
            const long id = X + (long)nxg * Y + sxy * Z;
            v = Z == 0 ? phi[id + sxy] - phi[id] : phi[id] - phi[id - sxy];
        }
        Dz[zi][yi][xi] = v;
    }
    __syncthreads();

    const int tx = tid3.x, ty = tid3.y, tz = tid3.z;
    const int X = x0 + tx, Y = y0 + ty, Z = z0 + tz;
    if (X >= xe || Y >= ye || Z >= ze) return;
    const long id = X + (long)nxg * Y + sxy * Z;

    // velocity and metric at the cell
    long iv;
    long nv;
    if (a.reflect) {
        const int nx = nxg - 2 * a.g, ny = nyg - 2 * a.g, nz = nzg - 2 * a.g;
        iv = mirror(X, a.g, nx) + (long)nx * (mirror(Y, a.g, ny) + (long)ny * mirror(Z, a.g, nz));
        nv = (long)nx * ny * nz;
    } else {
        iv = id;
        nv = sxy * nzg;
    }
    const double ux = a.vel[iv], uy = a.vel[nv + iv], uz = a.vel[2 * nv + iv];
    // scale of the differences: either multiply the five differences by
    // C = jbn/h (as the reference does) or use the precomputed per-cell
    // factors and rescale epsilon instead (one multiply per direction)
    const bool pre = a.wce != nullptr;
    double cx, cy, cz, ex, ey, ez, mx, my, mz;
    if (pre) {
        cx = 1.0; cy = 1.0; cz = 1.0;
        const double2 sx2 = weno_scale(a.wce, 0, nv, iv), sy2 = weno_scale(a.wce, 1, nv, iv),
                      sz2 = weno_scale(a.wce, 2, nv, iv);
        mx = sx2.x; my = sy2.x; mz = sz2.x;
        ex = sx2.y; ey = sy2.y; ez = sz2.y;
    } else {
        cx = a.jbn[iv] * a.sx; cy = a.jbn[4 * nv + iv] * a.sy; cz = a.jbn[8 * nv + iv] * a.sz;
        mx = 1.0; my = 1.0; mz = 1.0;
        ex = kWenoEps4; ey = kWenoEps4; ez = kWenoEps4;
    }

    int p[5];
    double rs;
    // x
    {
        if (__double_as_longlong(ux) >= 0) stencil_left(X, nxg, p); else stencil_right(X, nxg, p);
        const double *d = &Dx[tz][ty][0];
        const int o = x0 - 2;
        double phx;
        if (pre)
            phx = mx * weno5(d[p[0] - o], d[p[1] - o], d[p[2] - o], d[p[3] - o], d[p[4] - o], ex);
        else
            phx = weno5(d[p[0] - o] * cx, d[p[1] - o] * cx, d[p[2] - o] * cx, d[p[3] - o] * cx,
                        d[p[4] - o] * cx, ex);
        rs = ux * phx;
    }
    // y
    {
        if (__double_as_longlong(uy) >= 0) stencil_left(Y, nyg, p); else stencil_right(Y, nyg, p);
        const int o = y0 - 2;
        const double v1 = Dy[tz][p[0] - o][tx], v2 = Dy[tz][p[1] - o][tx], v3 = Dy[tz][p[2] - o][tx],
                     v4 = Dy[tz][p[3] - o][tx], v5 = Dy[tz][p[4] - o][tx];
        double phy;
        if (pre)
            phy = my * weno5(v1, v2, v3, v4, v5, ey);
        else
            phy = weno5(v1 * cy, v2 * cy, v3 * cy, v4 * cy, v5 * cy, ey);
        rs = rs + uy * phy;
    }
    // z
    {
        const bool left = __double_as_longlong(uz) >= 0;
        if (left) stencil_left(Z, nzg, p); else stencil_right(Z, nzg, p);
        const int o = z0 - 2;
        double v5 = Dz[p[4] - o][ty][tx];
        if (left && a.ref_bugs && Z == nzg - 1) {
            // lsTools.cu:636: id_kp2 = id_jm1 -- the z-difference one row
            // down in y (same cell when Y == 0) at the top layer
            const int Yb = Y == 0 ? Y : Y - 1;
            const long ib = X + (long)nxg * Yb + sxy * Z;
            v5 = phi[ib] - phi[ib - sxy];
        }
        const double v1 = Dz[p[0] - o][ty][tx], v2 = Dz[p[1] - o][ty][tx], v3 = Dz[p[2] - o][ty][tx],
                     v4 = Dz[p[3] - o][ty][tx];
        double phz;
        if (pre)
            phz = mz * weno5(v1, v2, v3, v4, v5, ez);
        else
            phz = weno5(v1 * cz, v2 * cz, v3 * cz, v4 * cz, v5 * cz, ez);
        rs = rs + uz * phz;
    }

    // TVD-RK3 stage (extrapol.cu:155-212)
    const double pin = phi[id];
    double v;
    if (a.stage == 1) {
        v = fma(-a.dt, rs, pin);
    } else {
        const double t = fma(-a.dt, rs, pin);
        const double p0 = a.phi0[id];
        v = a.stage == 2 ? fma(0.25, t, 0.75 * p0) : fma(2.0, t, p0) * (1.0 / 3.0);
    }
    if (a.out_interior) {
        const int g = a.g;
        const int nx = nxg - 2 * g, ny = nyg - 2 * g, nz = nzg - 2 * g;
        const int I = X - g, J = Y - g, K = Z - g;
        if (I >= 0 && I < nx && J >= 0 && J < ny && K >= 0 && K < nz)
            a.out[I + (long)nx * (J + (long)ny * K)] = v;
    } else {
        a.out[id] = v;
    }
}

} // namespace emix
