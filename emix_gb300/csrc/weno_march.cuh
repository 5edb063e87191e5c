// weno_march.cuh -- the level-set TVD stage as a z-marching kernel body
// (k_weno_march in weno_march.cu; the batched form walks it over many grids).
//
// The TVD stage of weno.cuh (the reference's cuAdvectLsJB pieces), arranged
// to do few FP64 operations per cell:
//   * each block owns a 16 x 16 column of (x, y) cells and walks a range of z;
//     the z differences live in a per-thread register window (one new
//     difference per plane, no z halo), and the next plane's phi tile is
//     loaded into registers while the current plane is computed;
//   * besides the backward differences D(p) = phi(p) - phi(p-1), the second
//     differences A(p) = D(p) - D(p-1) are formed once per tile position, so
//     that a WENO5 evaluation needs 6 operations for its d_k, e_k instead of 11
//     (weno5a below);
//   * a warp with a cell within 2-3 cells of the padded grid's x or y faces
//     (where the reference's edge rules move the stencil) reads the five
//     differences of every lane at the rule's positions from the same tile;
//     planes near the z faces read them from global memory (weno_z_general).
#pragma once

#include "tma.cuh"
#include "weno.cuh"

namespace emix {

constexpr int kMX = 16, kMY = 16, kNT = kMX * kMY;
constexpr int kPX = kMX + 6, kPY = kMY + 6;   // phi tile: [x0-3, x0+kMX+3) x [y0-3, y0+kMY+3)
constexpr int kPN = kPX * kPY;
constexpr int kPR = (kPN + kNT - 1) / kNT;     // tile values each thread loads

// WENO5 of weno5() (weno.cuh) with the five differences given as v3 and the
// four consecutive second differences a_k = v_{k+1} - v_k:
//   d1 = a2 - a1, d2 = a3 - a2, d3 = a4 - a3,
//   e1 = d1 + 2 a2, e2 = -(a2 + a3), e3 = d3 - 2 a3.
// With c12 = -12 the a_k given are the negated second differences: d, e and
// r change sign, the smoothness terms do not, so the sign goes to the
// denominator (the right-biased stencil reads its second differences in
// reverse order with this sign, and needs no negations).
// The same with the third differences d1 = a2 - a1, d2 = a3 - a2, d3 = a4 - a3
// given (from the stage's third-difference tiles): a1 and a4 are not needed.
EMIX_DEV double weno5d(double v3, double a2, double a3, double d1, double d2, double d3, double eps4,
                       double c12) {
    constexpr double c13 = 13.0 / 3.0;
    const double e1 = fma(2.0, a2, d1);
    const double e2 = -(a2 + a3);
    const double e3 = fma(-2.0, a3, d3);
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
    const double den = c12 * (w1 + w2 + w3);
    return fma(num, rcp_newton(den), v3);
}

EMIX_DEV double weno5a(double v3, double a1, double a2, double a3, double a4, double eps4, double c12) {
    return weno5d(v3, a2, a3, a2 - a1, a3 - a2, a4 - a3, eps4, c12);
}

// sqrt(13/3), correctly rounded
constexpr double kSqrt13_3 = 2.0816659994661326;

// The same from the four second differences and the third differences scaled
// by sqrt(13/3), s_k = sqrt(13/3) d_k (from the stage's scaled tiles), so that
// the smoothness term c13 d_k^2 + e_k^2 is one FMA: with e1 = 3 a2 - a1,
// e2 = -(a2 + a3), e3 = a4 - 3 a3 and the candidates halved, r_k / 2 =
// 2 e1 - a2, a3 - e2, a3 - e3, the halving carried by c6 = c12 / 2.  The
// sign of s_k does not matter (it enters squared), so the right-biased side
// reads the tile's values as they are.
EMIX_DEV double weno5s(double v3, double a1, double a2, double a3, double a4, double s1, double s2,
                       double s3, double eps4, double c6) {
    const double e1 = fma(3.0, a2, -a1);
    const double e2 = -(a2 + a3);
    const double e3 = fma(-3.0, a3, a4);
    double t1 = fma(s1, s1, fma(e1, e1, eps4)); t1 *= t1;
    double t2 = fma(s2, s2, fma(e2, e2, eps4)); t2 *= t2;
    double t3 = fma(s3, s3, fma(e3, e3, eps4)); t3 *= t3;
    const double w1 = t2 * t3;
    const double w2 = (6.0 * t1) * t3;
    const double w3 = (3.0 * t1) * t2;
    const double r1 = fma(2.0, e1, -a2);
    const double r2 = a3 - e2;
    const double r3 = a3 - e3;
    const double num = fma(w1, r1, fma(w2, r2, w3 * r3));
    const double den = c6 * (w1 + w2 + w3);
    return fma(num, rcp_newton(den), v3);
}

// z direction of a plane near the z faces: the five differences at the edge
// rule's positions, read from global memory
EMIX_DEV void weno_z_general(const double *phi, long id, int Z, int nzg, bool left, bool ztop_bug, long nxg,
                             long sxy, double v[5]) {
    int p[5];
    if (left) stencil_left(Z, nzg, p); else stencil_right(Z, nzg, p);
    const long base = id - (long)Z * sxy;
    for (int k = 0; k < 5; ++k) {
        const int q = p[k];
        v[k] = q == 0 ? phi[base + sxy] - phi[base] : phi[base + q * sxy] - phi[base + (q - 1) * sxy];
    }
    if (ztop_bug) {
        // lsTools.cu:636: id_kp2 = id_jm1 -- the z difference one row down in y
        // (the same cell on the first row) at the top layer
        const long ib = ((id % sxy) / nxg == 0) ? id : id - nxg;
        v[4] = phi[ib] - phi[ib - sxy];
    }
}

struct Plane {
    double v[kPR];
};

EMIX_DEV void load_plane(const double *__restrict__ phi, int x0, int y0, int Z, int nxg, int nyg, int nzg,
                         long sxy, int tid, Plane &pl) {
#pragma unroll
    for (int r = 0; r < kPR; ++r) {
        const int t = tid + r * kNT;
        double v = 0.0;
        if (t < kPN && Z >= 0 && Z < nzg) {
            const int gx = x0 - 3 + t % kPX, gy = y0 - 3 + t / kPX;
            if (gx >= 0 && gx < nxg && gy >= 0 && gy < nyg) v = phi[gx + (long)nxg * gy + sxy * Z];
        }
        pl.v[r] = v;
    }
}

// TMA staging of the phi plane tiles (k_weno_march_tma): a 3-D tiled copy of
// a kTY x kTW box per plane into one of two shared buffers, completion on an
// mbarrier; the box starts at an even x (16-byte rule of the copy unit), so the
// tile sits kdx = 0 or 1 columns into the buffer.
constexpr int kTW = kPX + 2;                        // 24 doubles: 192 bytes per row
constexpr int kTY = kPY;                            // 22 rows
constexpr unsigned kTileBytes = kTW * kTY * 8;      // 4224

// one thread: expect the tile's bytes on bar, then copy the box at (x, y, z)
EMIX_DEV void tma_plane(const void *tmap, unsigned dst, unsigned bar, int x, int y, int z) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(kTileBytes)
                 : "memory");
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(dst), "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(z), "r"(bar)
                 : "memory");
}

// count of stage blocks that gave up waiting for a plane copy (read by
// emix_weno_tma_timeouts; the TMA kernel and that reader are in weno_march.cu)
static __device__ int g_weno_tma_timeouts = 0;
// test hook (emix_weno_tma_test_drop): nonzero makes the TMA stage issue no
// copies, so that its bounded waits run out and the timeout path is exercised
static __device__ int g_weno_tma_drop = 0;

// One (virtual) block: column tile (bx, by) of the region, z chunk bz of gz.
// TMA: the plane tiles come by tiled bulk copies described by *tmap (a
// __grid_constant__ kernel parameter); otherwise by register-staged loads.
template <bool TMA>
EMIX_DEV void weno_march_body_t(const WenoArgs &a, int bx, int by, int bz, int gz, const void *tmap) {
    __shared__ __align__(128) double Pbuf[2 * kTY * kTW];   // register path: [kPY][kPX]; TMA: [2][kTY][kTW]
    __shared__ double Dx[kMY][kMX + 5];      // positions x0-2 .. x0+kMX+2
    __shared__ double Ax[kMY][kMX + 4];      // positions x0-1 .. x0+kMX+2
    __shared__ double Dy[kMY + 5][kMX];      // rows y0-2 .. y0+kMY+2
    __shared__ double Ay[kMY + 4][kMX];      // rows y0-1 .. y0+kMY+2
    // scaled third differences S(p) = sqrt(13/3) (A(p) - A(p-1))
    __shared__ double Tx[kMY][kMX + 3];      // positions x0 .. x0+kMX+2
    __shared__ double Ty[kMY + 3][kMX];      // rows y0 .. y0+kMY+2

    const int nxg = a.nxg, nyg = a.nyg, nzg = a.nzg;
    const long sxy = (long)nxg * nyg;
    const double *__restrict__ phi = a.phi;
    const int tid = threadIdx.x, tx = tid % kMX, ty = tid / kMX;
    const int x0 = a.r0[0] + bx * kMX, y0 = a.r0[1] + by * kMY;
    const int xe = a.r0[0] + a.rn[0], ye = a.r0[1] + a.rn[1];
    const int zr0 = a.r0[2], zrn = a.rn[2];
    const int chunk = (zrn + gz - 1) / gz;
    const int zs = zr0 + bz * chunk, ze = min(zs + chunk, zr0 + zrn);
    const int X = x0 + tx, Y = y0 + ty;
    const bool active = X < xe && Y < ye;
    const long col = (long)X + (long)nxg * Y;
    // warps (two rows of 16 cells) with a cell whose x or y stencil follows
    // an edge rule of the padded grid
    const bool wedge_x = __any_sync(0xffffffffu, active && (X < 2 || X > nxg - 4));
    const bool wedge_y = __any_sync(0xffffffffu, active && (Y < 2 || Y > nyg - 4));

    const int g = a.g;
    const int nx = nxg - 2 * g, ny = nyg - 2 * g, nz = nzg - 2 * g;
    const long nv = a.reflect ? (long)nx * ny * nz : sxy * nzg;
    const bool pre = a.wce != nullptr;

    // z window of this column: phi(z), 0 outside the grid
    auto ld = [&](int z) { return (active && z >= 0 && z < nzg) ? phi[col + sxy * z] : 0.0; };
    // Dz[t] = D(Z - 2 + t), t = 0..5; Az[t] = A(Z - 1 + t), t = 0..4;
    // Tz[t] = S(Z + t) = sqrt(13/3) (A(Z + t) - A(Z + t - 1)), t = 0..3; fz = phi(Z + 3)
    double Dz[6], Az[5], Tz[4], fz;
    {
        double f[7];
#pragma unroll
        for (int t = 0; t < 7; ++t) f[t] = ld(zs - 3 + t);
#pragma unroll
        for (int t = 0; t < 6; ++t) Dz[t] = (zs - 2 + t == 0) ? ld(1) - ld(0) : f[t + 1] - f[t];
#pragma unroll
        for (int t = 0; t < 5; ++t) Az[t] = Dz[t + 1] - Dz[t];
#pragma unroll
        for (int t = 0; t < 4; ++t) Tz[t] = kSqrt13_3 * (Az[t + 1] - Az[t]);
        fz = f[6];
    }

    // plane tiles: register path one [kPY][kPX] tile, loaded into registers
    // during the previous plane; TMA path two [kTY][kTW] buffers, plane Z in
    // buffer (Z - zs) & 1, the copy of plane Z + 2 issued once plane Z is read
    const int xs = (x0 - 3) & ~1, kdx = (x0 - 3) - xs;   // box origin (even x), tile offset
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ int s_ok;
    Plane pl;
    if constexpr (TMA) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&mbar[0])), "r"(1) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&mbar[1])), "r"(1) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0 && !g_weno_tma_drop) {
            if (zs < ze) tma_plane(tmap, smem_u32(Pbuf), smem_u32(&mbar[0]), xs, y0 - 3, zs);
            if (zs + 1 < ze) tma_plane(tmap, smem_u32(Pbuf + kTY * kTW), smem_u32(&mbar[1]), xs, y0 - 3, zs + 1);
        }
    } else {
        if (zs < ze) load_plane(phi, x0, y0, zs, nxg, nyg, nzg, sxy, tid, pl);
    }
    for (int Z = zs; Z < ze; ++Z) {
        const int kk = Z - zs, b = kk & 1;
        const double *Pz;
        int pld, pcx;
        if constexpr (TMA) {
            if (tid == 0) s_ok = mbar_wait(smem_u32(&mbar[b]), (unsigned)((kk >> 1) & 1));
            __syncthreads();
            if (!s_ok) {
                // the copy did not arrive: count it, let the copies in flight
                // land (bounded), and leave this block's planes unwritten
                if (tid == 0) {
                    atomicAdd(&g_weno_tma_timeouts, 1);
                    mbar_wait(smem_u32(&mbar[b]), (unsigned)((kk >> 1) & 1));
                    if (Z + 1 < ze) mbar_wait(smem_u32(&mbar[b ^ 1]), (unsigned)(((kk + 1) >> 1) & 1));
                }
                return;
            }
            Pz = Pbuf + b * kTY * kTW;
            pld = kTW;
            pcx = kdx;
        } else {
            // ---- this plane's tile (loaded during the previous plane) ----
#pragma unroll
            for (int r = 0; r < kPR; ++r) {
                const int t = tid + r * kNT;
                if (t < kPN) Pbuf[t] = pl.v[r];
            }
            __syncthreads();
            // the next plane's tile, in flight during this plane
            if (Z + 1 < ze) load_plane(phi, x0, y0, Z + 1, nxg, nyg, nzg, sxy, tid, pl);
            Pz = Pbuf;
            pld = kPX;
            pcx = 0;
        }
        auto P = [&](int py, int px) { return Pz[py * pld + px + pcx]; };
        const double fnext = ld(Z + 4);
        for (int t = tid; t < kMY * (kMX + 5); t += kNT) {
            const int i = t % (kMX + 5), j = t / (kMX + 5);
            const int gx = x0 - 2 + i;   // P column i + 1
            Dx[j][i] = gx == 0 ? P(j + 3, i + 2) - P(j + 3, i + 1) : P(j + 3, i + 1) - P(j + 3, i);
        }
        for (int t = tid; t < (kMY + 5) * kMX; t += kNT) {
            const int i = t % kMX, j = t / kMX;
            const int gy = y0 - 2 + j;   // P row j + 1
            Dy[j][i] = gy == 0 ? P(j + 2, i + 3) - P(j + 1, i + 3) : P(j + 1, i + 3) - P(j, i + 3);
        }
        const double pin = active ? P(ty + 3, tx + 3) : 0.0;
        __syncthreads();
        if constexpr (TMA) {
            // buffer b is read: the copy of plane Z + 2 may overwrite it
            if (tid == 0 && Z + 2 < ze && !g_weno_tma_drop) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                tma_plane(tmap, smem_u32(Pbuf + b * kTY * kTW), smem_u32(&mbar[b]), xs, y0 - 3, Z + 2);
            }
        }
        for (int t = tid; t < kMY * (kMX + 4); t += kNT) {
            const int i = t % (kMX + 4), j = t / (kMX + 4);
            Ax[j][i] = Dx[j][i + 1] - Dx[j][i];
        }
        for (int t = tid; t < (kMY + 4) * kMX; t += kNT) {
            const int i = t % kMX, j = t / kMX;
            Ay[j][i] = Dy[j + 1][i] - Dy[j][i];
        }
        __syncthreads();
        // scaled third differences, once per position instead of three
        // differences and three products per evaluation
        for (int t = tid; t < kMY * (kMX + 3); t += kNT) {
            const int i = t % (kMX + 3), j = t / (kMX + 3);
            Tx[j][i] = kSqrt13_3 * (Ax[j][i + 1] - Ax[j][i]);
        }
        for (int t = tid; t < (kMY + 3) * kMX; t += kNT) {
            const int i = t % kMX, j = t / kMX;
            Ty[j][i] = kSqrt13_3 * (Ay[j + 1][i] - Ay[j][i]);
        }
        __syncthreads();

        if (active) {
            const long id = col + sxy * Z;
            long iv = id;
            if (a.reflect)
                iv = mirror(X, g, nx) + (long)nx * (mirror(Y, g, ny) + (long)ny * mirror(Z, g, nz));
            double rs = 0.0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double u = a.vel[d * nv + iv];
                double mx, ex;
                if (pre) {
                    const double2 ce = weno_scale(a.wce, d, nv, iv);
                    mx = ce.x;
                    ex = ce.y;
                } else {
                    const double jd = a.jbn[4 * d * nv + iv] * (d == 0 ? a.sx : (d == 1 ? a.sy : a.sz));
                    // W(C v; eps) = C W(v; eps / C^2)
                    mx = jd;
                    ex = kWenoEps4 / (jd * jd);
                }
                const bool left = __double_as_longlong(u) >= 0;
                // the five differences as v3, the second differences a1..a4
                // and the scaled third differences s1..s3; the upwind side is
                // chosen by selects (no divergent WENO5)
                double v3, a1, a2, a3, a4, c12 = left ? 12.0 : -12.0;
                bool tiled = true;
                double s1, s2, s3;
                if ((d == 0 && !wedge_x) || (d == 1 && !wedge_y)) {
                    // left: v3 = D(c), a = A(c-1..c+2), s = S(c..c+2); right:
                    // v3 = D(c+1), a = -A(c+3..c), given as A(c+3..c) with the
                    // sign in c12, s = S(c+3..c+1) -- tile index of D(c) is
                    // t + 2, of A(c) t + 1, of S(c) t
                    const int o = left ? 0 : 4, st = left ? 1 : -1, ov = left ? 2 : 3, os = left ? 0 : 3;
                    if (d == 0) {
                        const double *ar = &Ax[ty][tx];
                        const double *sr = &Tx[ty][tx];
                        v3 = Dx[ty][tx + ov];
                        a1 = ar[o]; a2 = ar[o + st]; a3 = ar[o + 2 * st]; a4 = ar[o + 3 * st];
                        s1 = sr[os]; s2 = sr[os + st]; s3 = sr[os + 2 * st];
                    } else {
                        v3 = Dy[ty + ov][tx];
                        a1 = Ay[ty + o][tx]; a2 = Ay[ty + o + st][tx]; a3 = Ay[ty + o + 2 * st][tx];
                        a4 = Ay[ty + o + 3 * st][tx];
                        s1 = Ty[ty + os][tx]; s2 = Ty[ty + os + st][tx]; s3 = Ty[ty + os + 2 * st][tx];
                    }
                } else if (d == 2 && Z >= 2 && Z <= nzg - 4) {
                    v3 = left ? Dz[2] : Dz[3];
                    a1 = left ? Az[0] : Az[4];
                    a2 = left ? Az[1] : Az[3];
                    a3 = Az[2];
                    a4 = left ? Az[3] : Az[1];
                    s1 = left ? Tz[0] : Tz[3];
                    s2 = left ? Tz[1] : Tz[2];
                    s3 = left ? Tz[2] : Tz[1];
                } else {
                    tiled = false;
                    // edge rules: the differences at the rule's positions
                    double v[5];
                    if (d == 2) {
                        const bool bug = left && a.ref_bugs && Z == nzg - 1;
                        weno_z_general(phi, id, Z, nzg, left, bug, nxg, sxy, v);
                    } else {
                        int p[5];
                        const int c = d == 0 ? X : Y, L = d == 0 ? nxg : nyg;
                        if (left) stencil_left(c, L, p); else stencil_right(c, L, p);
                        if (d == 0) {
                            for (int k = 0; k < 5; ++k) v[k] = Dx[ty][p[k] - (x0 - 2)];
                        } else {
                            for (int k = 0; k < 5; ++k) v[k] = Dy[p[k] - (y0 - 2)][tx];
                        }
                    }
                    v3 = v[2];
                    a1 = v[1] - v[0]; a2 = v[2] - v[1]; a3 = v[3] - v[2]; a4 = v[4] - v[3];
                    c12 = 12.0;
                }
                const double W = tiled ? weno5s(v3, a1, a2, a3, a4, s1, s2, s3, ex, left ? 6.0 : -6.0)
                                       : weno5a(v3, a1, a2, a3, a4, ex, c12);
                rs = fma(u, mx * W, rs);
            }
            // TVD-RK3 stage (extrapol.cu:155-212)
            double v;
            if (a.stage == 1) {
                v = fma(-a.dt, rs, pin);
            } else {
                const double t = fma(-a.dt, rs, pin);
                const double p0 = a.phi0[id];
                v = a.stage == 2 ? fma(0.25, t, 0.75 * p0) : fma(2.0, t, p0) * (1.0 / 3.0);
            }
            if (a.out_interior) {
                const int I = X - g, J = Y - g, K = Z - g;
                if (I >= 0 && I < nx && J >= 0 && J < ny && K >= 0 && K < nz)
                    a.out[I + (long)nx * (J + (long)ny * K)] = v;
            } else {
                a.out[id] = v;
            }
        }
        // ---- advance the z window ----
#pragma unroll
        for (int t = 0; t < 5; ++t) Dz[t] = Dz[t + 1];
        Dz[5] = fnext - fz;   // D(Z + 4); Z + 4 > 0
        fz = fnext;
#pragma unroll
        for (int t = 0; t < 4; ++t) Az[t] = Az[t + 1];
        Az[4] = Dz[5] - Dz[4];
#pragma unroll
        for (int t = 0; t < 3; ++t) Tz[t] = Tz[t + 1];
        Tz[3] = kSqrt13_3 * (Az[4] - Az[3]);
        __syncthreads();
    }
    if constexpr (TMA) {
        if (tid == 0) {
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(smem_u32(&mbar[0])) : "memory");
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(smem_u32(&mbar[1])) : "memory");
        }
    }
}

// the register-staged form (the batched ensemble walks it over many grids)
EMIX_DEV void weno_march_body(const WenoArgs &a, int bx, int by, int bz, int gz) {
    weno_march_body_t<false>(a, bx, by, bz, gz, nullptr);
}


} // namespace emix
