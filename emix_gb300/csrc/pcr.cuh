// pcr.cuh -- y/z compact derivatives by parallel cyclic reduction + Thomas.
//
// The Thomas kernels (deriv.cuh) give one pencil to one thread: six FP64
// operations per row, and a pencil's rows strictly one after another.  Here a
// pencil's rows are split over 2^S lanes of a warp: lane r holds rows
// i = r (mod 2^S) in registers, S PCR steps (each row taking its partners
// i -/+ 2^k from the lanes r -/+ 2^k by warp shuffles) decouple the 2^S
// subsystems, and each lane solves its own subsystem by the factored Thomas
// sweeps.  The reference solves each pencil serially
// (src/Schemes/derivCompact.cu:146-215); the matrix side of every PCR step and
// the subsystems' factors come from the host (get_pcr_table).  A warp covers
// 32 / 2^S consecutive x pencils: lanes r + 2^S p, p the pencil.
#pragma once

#include "deriv.cuh"

namespace emix {

// right-hand side of row i (the stencil with 1/h folded in), f at element 0
// of the pencil with element stride s
EMIX_DEV double pcr_rhs(const PcrTable &P, const double *__restrict__ f, long s, int i) {
    const int n = P.n;
    if (P.periodic) {
        int im1 = i - 1, im2 = i - 2, ip1 = i + 1, ip2 = i + 2;
        if (im1 < 0) im1 += n;
        if (im2 < 0) im2 += n;
        if (ip1 >= n) ip1 -= n;
        if (ip2 >= n) ip2 -= n;
        return P.ra[i] * (f[ip1 * s] - f[im1 * s]) + P.rb[i] * (f[ip2 * s] - f[im2 * s]);
    }
    const double *c = P.cl + 4 * i;
    if (i < P.nlo) return c[0] * f[0] + c[1] * f[s] + c[2] * f[2 * s] + c[3] * f[3 * s];
    if (i >= n - P.nhi) {
        const double *e = f + (long)(n - 1) * s;
        return c[0] * e[0] + c[1] * e[-s] + c[2] * e[-2 * s] + c[3] * e[-3 * s];
    }
    return P.ra[i] * (f[(i + 1) * s] - f[(i - 1) * s]) + P.rb[i] * (f[(i + 2) * s] - f[(i - 2) * s]);
}

// One warp's pencils: x0 .. x0 + 32/2^S - 1 at `o` (the other coordinate) of
// field f.  S PCR steps, M >= ceil(n / 2^S) rows per lane.  Every lane of the
// warp runs the whole body (the shuffles need them all); lanes past the grid
// neither load nor store.
template <int S, int M, int EPI>
EMIX_DEV void pcr_yz_warp(const PcrTable &P, const PencilFields &F, int nx, int nother, long s, long os,
                          int x0, int o, int fi) {
    constexpr int H = 1 << S;
    const int lane = threadIdx.x & 31, r = lane & (H - 1), base = lane & ~(H - 1);
    const int x = x0 + (lane >> S);
    const bool live = x < nx && o < nother;
    const int n = P.n;
    const int m = (n + H - 1) >> S;   // slots in use (<= M; the same in every lane)
    const long off = (long)(live ? x : 0) + (long)(live ? o : 0) * os;
    const double *__restrict__ in = pick(F.in, fi) + off;
    double *out = pick(F.out, fi) + off;

    double d[M];
#pragma unroll
    for (int t = 0; t < M; ++t) {
        const int i = r + H * t;
        d[t] = (t < m && live && i < n) ? pcr_rhs(P, in, s, i) : 0.0;
    }
    // PCR: d_i += al_i d_{i-h} + ga_i d_{i+h}, h = 2^k.  Row i - h lives in
    // lane r - h (slot t) or, for r < h, lane r - h + H (slot t - 1); row
    // i + h in lane r + h (slot t) or lane r + h - H (slot t + 1).  Slots are
    // updated in order, so slot t - 1's value before its update travels in
    // `prev`.
#pragma unroll
    for (int k = 0; k < S; ++k) {
        const int h = 1 << k;
        const int lo = base + ((r - h) & (H - 1)), hi = base + ((r + h) & (H - 1));
        const double *__restrict__ al = P.al + (long)k * n;
        const double *__restrict__ ga = P.ga + (long)k * n;
        double prev = 0.0;
#pragma unroll
        for (int t = 0; t < M; ++t) {
            if (t >= m) break;
            const int i = r + H * t;
            const double nxt = t + 1 < M ? d[t + 1] : 0.0;
            const double a0 = __shfl_sync(0xffffffffu, d[t], lo);
            const double a1 = __shfl_sync(0xffffffffu, prev, lo);
            const double b0 = __shfl_sync(0xffffffffu, d[t], hi);
            const double b1 = __shfl_sync(0xffffffffu, nxt, hi);
            const double dm = r >= h ? a0 : a1;
            const double dp = r + h < H ? b0 : b1;
            prev = d[t];
            if (i < n) d[t] = fma(ga[i], dp, fma(al[i], dm, d[t]));
        }
    }
    // Thomas on this lane's subsystem (rows r, r + H, ...)
    double w = 0.0;
#pragma unroll
    for (int t = 0; t < M; ++t) {
        if (t >= m) break;
        const int i = r + H * t;
        if (i < n) {
            w = fma(-P.mt[i], w, d[t] * P.ib[i]);
            d[t] = w;
        }
    }
    double xv = 0.0;
#pragma unroll
    for (int t = M - 1; t >= 0; --t) {
        const int i = r + H * t;
        if (t < m && i < n) {
            xv = d[t] - P.gt[i] * xv;
            d[t] = xv;
        }
    }
    if (P.periodic) {
        // x = y - fact zz with fact from y_0 (lane base, slot 0) and y_{n-1}
        const int re = (n - 1) & (H - 1), te = (n - 1) >> S;
        double ye = 0.0;
#pragma unroll
        for (int t = 0; t < M; ++t)
            if (t == te) ye = d[t];
        const double y0 = __shfl_sync(0xffffffffu, d[0], base);
        const double yn = __shfl_sync(0xffffffffu, ye, base + re);
        const double fact = (y0 + P.sm1 * yn) * P.sm2;
#pragma unroll
        for (int t = 0; t < M; ++t) {
            if (t >= m) break;
            const int i = r + H * t;
            if (i < n) d[t] -= fact * P.zz[i];
        }
    }
    if (!live) return;
#pragma unroll
    for (int t = 0; t < M; ++t) {
        if (t >= m) break;
        const int i = r + H * t;
        if (i < n) {
            double v = d[t];
            if (EPI == EPI_ACCUM) v += out[i * s];
            out[i * s] = v;
        }
    }
}

// Rows a lane holds at S steps, pencils of up to kPcrMaxN rows.
template <int S>
constexpr int pcr_rows() { return (kPcrMaxN + (1 << S) - 1) >> S; }

// Pencils one 128-thread block covers along x at S steps.
template <int S>
constexpr int pcr_block_x() { return 4 * (32 >> S); }

// y/z launch at S steps (S = 2..5): grid (ceil(nx / pcr_block_x<S>()),
// nother, nf), 128 threads.  axis 1: s = nx, os = nx*ny; axis 2: s = nx*ny,
// os = nx.
int launch_deriv_pcr(const PcrTable &P, int axis, int epi, int nf, const double *const *in,
                     double *const *out, int nx, int ny, int nz, cudaStream_t st);

} // namespace emix
