// deriv.cuh -- compact first-derivative pencil kernels (FP64).
//
// One thread owns one pencil and runs the factored Thomas sweeps serially;
// the right-hand-side stencil is fused into the forward sweep.  On GB300 the
// FP64 pipe (about 0.5 T lane-ops/s) is the binding resource, so the kernels
// are written to minimise FP64 instructions: per interior cell 2 DADD + 1 DMUL
// + 1 DFMA for the stencil, 1 DFMA forward, 1 DFMA backward, and no divides
// (the pivots live in the factor table).
//
//   y/z pencils: lanes map to consecutive x, so every load and store of a
//                warp is one 256-byte coalesced access; the pencil walk keeps
//                a five-value sliding window in registers.
//   x pencils:   a warp owns 32 pencils and stages 32-row chunks through a
//                [32][33] shared-memory tile: the stencil rows are computed
//                lane-per-row (coalesced loads), the sweeps lane-per-pencil.
//
// The forward sweep's intermediate w is written to a buffer (the output
// itself when the epilogue is a plain store) and read back by the backward
// sweep.  Field index = blockIdx.z, so nf fields give nf times more warps.
#pragma once

#include "common.cuh"

namespace emix {

enum { EPI_STORE = 0, EPI_ACCUM = 1 };

constexpr int kMaxFields = 6;

struct PencilFields {
    const double *in[kMaxFields];
    double *w[kMaxFields];
    double *out[kMaxFields];
};

template <typename P>
EMIX_DEV P pick(const P (&a)[kMaxFields], int f) {
    // uniform selection without dynamic indexing of the parameter array
    P r = a[0];
    if (f == 1) r = a[1];
    if (f == 2) r = a[2];
    if (f == 3) r = a[3];
    if (f == 4) r = a[4];
    if (f == 5) r = a[5];
    return r;
}

// Right-hand side r'_i of one pencil (already scaled by 1/h and the pivot).
// fp points at element 0 of the pencil, s is the element stride.
EMIX_DEV double rhs_row(const DerivTable &T, const double *__restrict__ fp, long s, int i) {
    const int n = T.n;
    const DerivRow row = T.rows[i];
    if (T.periodic) {
        int im1 = i - 1, im2 = i - 2, ip1 = i + 1, ip2 = i + 2;
        if (im1 < 0) im1 += n;
        if (im2 < 0) im2 += n;
        if (ip1 >= n) ip1 -= n;
        if (ip2 >= n) ip2 -= n;
        return row.A * (fp[ip1 * s] - fp[im1 * s]) + row.B * (fp[ip2 * s] - fp[im2 * s]);
    }
    if (i < T.nlo) {
        const double *c = T.clo + 4 * i;
        return c[0] * fp[0] + c[1] * fp[s] + c[2] * fp[2 * s] + c[3] * fp[3 * s];
    }
    if (i >= n - T.nhi) {
        const double *c = T.chi + 4 * (n - 1 - i);
        const double *e = fp + (long)(n - 1) * s;
        return c[0] * e[0] + c[1] * e[-s] + c[2] * e[-2 * s] + c[3] * e[-3 * s];
    }
    return row.A * (fp[(i + 1) * s] - fp[(i - 1) * s]) + row.B * (fp[(i + 2) * s] - fp[(i - 2) * s]);
}

// ---------------------------------------------------------------------------
// y / z pencils: thread per pencil.
//   axis 1 (y): pencils (x, z), element stride nx,    other stride nx*ny
//   axis 2 (z): pencils (x, y), element stride nx*ny, other stride nx
// grid: (ceil(nx/blockDim.x), nother, nf)
// ---------------------------------------------------------------------------
// K fields of one pencil in lockstep: K independent dependency chains per
// thread, interleaved so that the FP64 pipe always has work (ILP).
template <int EPI, int K>
EMIX_DEV void pencil_yz(const DerivTable &T, const PencilFields &F, int f0, long base, long s) {
    const double *in[K];
    double *w[K], *out[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        in[k] = pick(F.in, f0 + k) + base;
        w[k] = pick(F.w, f0 + k) + base;
        out[k] = pick(F.out, f0 + k) + base;
    }
    const int n = T.n;
    const DerivRow *__restrict__ rows = T.rows;

    // forward sweep
    double wp[K], y0[K];
#pragma unroll
    for (int k = 0; k < K; ++k) { wp[k] = 0.0; y0[k] = 0.0; }
    int i = 0;
    if (!T.periodic) {
        for (; i < T.nlo; ++i) {
            const double m = rows[i].m;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const double v = rhs_row(T, in[k], s, i) - m * wp[k];
                w[k][i * s] = v;
                wp[k] = v;
            }
        }
        const int iend = n - T.nhi;
        if (i < iend) {
            double fm2[K], fm1[K], f0c[K], fp1[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                fm2[k] = in[k][(i - 2) * s]; fm1[k] = in[k][(i - 1) * s];
                f0c[k] = in[k][i * s]; fp1[k] = in[k][(i + 1) * s];
            }
            for (; i < iend; ++i) {
                const DerivRow r = rows[i];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const double fp2 = in[k][(i + 2) * s];
                    const double v = r.A * (fp1[k] - fm1[k]) + r.B * (fp2 - fm2[k]) - r.m * wp[k];
                    w[k][i * s] = v;
                    wp[k] = v;
                    fm2[k] = fm1[k]; fm1[k] = f0c[k]; f0c[k] = fp1[k]; fp1[k] = fp2;
                }
            }
        }
        for (; i < n; ++i) {
            const double m = rows[i].m;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const double v = rhs_row(T, in[k], s, i) - m * wp[k];
                w[k][i * s] = v;
                wp[k] = v;
            }
        }
    } else {
        double fm2[K], fm1[K], f0c[K], fp1[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            fm2[k] = in[k][(n - 2) * s]; fm1[k] = in[k][(n - 1) * s];
            f0c[k] = in[k][0]; fp1[k] = in[k][s];
        }
        for (; i < n; ++i) {
            int j = i + 2;
            if (j >= n) j -= n;
            const DerivRow r = rows[i];
            const bool acc = i < T.ku;
            const double u0 = acc ? T.u0[i] : 0.0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const double fp2 = in[k][j * s];
                const double v = r.A * (fp1[k] - fm1[k]) + r.B * (fp2 - fm2[k]) - r.m * wp[k];
                w[k][i * s] = v;
                if (acc) y0[k] += u0 * v;
                wp[k] = v;
                fm2[k] = fm1[k]; fm1[k] = f0c[k]; f0c[k] = fp1[k]; fp1[k] = fp2;
            }
        }
    }

    // backward sweep
    double fact[K], yn[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        fact[k] = T.periodic ? (y0[k] + T.sm1 * wp[k]) * T.sm2 : 0.0;
        yn[k] = 0.0;
    }
    for (i = n - 1; i >= 0; --i) {
        const double g = rows[i].g;
        const bool corr = T.periodic && (i < T.zlo || i >= T.zhi);
        const double z = corr ? T.zz[i] : 0.0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const double y = w[k][i * s] - g * yn[k];
            yn[k] = y;
            double xv = y;
            if (corr) xv = y - fact[k] * z;
            if (EPI == EPI_ACCUM) xv += out[k][i * s];
            out[k][i * s] = xv;
        }
    }
}

// grid: (ceil(nx/blockDim.x), nother, ceil(nf/K)); block z-index g owns fields
// K*g .. K*g+K-1 (the last group may hold fewer)
template <int EPI, int K>
__global__ void __launch_bounds__(128)
k_deriv_yz(DerivTable T, PencilFields F, int nx, int nother, long s, long os, int nf) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int o = blockIdx.y;
    if (x >= nx || o >= nother) return;
    const long base = x + (long)o * os;
    const int f0 = blockIdx.z * K;
    if (K == 2 && f0 + 1 < nf)
        pencil_yz<EPI, K>(T, F, f0, base, s);
    else
        pencil_yz<EPI, 1>(T, F, f0, base, s);
}

// ---------------------------------------------------------------------------
// x pencils: a warp owns 32 consecutive pencils (flattened (j,k)); chunks of
// 32 rows go through a per-warp [32][33] shared tile.
// grid: (ceil(npencil / (32*warps_per_block)), 1, nf); block 32*warps
// ---------------------------------------------------------------------------
constexpr int kXTile = 32 * 33;

template <int EPI>
__global__ void __launch_bounds__(128)
k_deriv_x(DerivTable T, PencilFields F, long npencil) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *tile = smem + warp * kXTile;
    const long p0 = ((long)blockIdx.x * (blockDim.x >> 5) + warp) * 32;
    if (p0 >= npencil) return;  // whole warp
    const int npw = (int)min((long)32, npencil - p0);
    const int f = blockIdx.z;
    const int n = T.n;
    const double *__restrict__ in = pick(F.in, f) + p0 * n;
    double *w = pick(F.w, f) + p0 * n;
    double *out = pick(F.out, f) + p0 * n;
    const DerivRow *__restrict__ rows = T.rows;

    double wp = 0.0, y0 = 0.0;
    for (int c0 = 0; c0 < n; c0 += 32) {
        const int cl = min(32, n - c0);
        if (lane < cl) {
            const int i = c0 + lane;
            for (int q = 0; q < npw; ++q) tile[q * 33 + lane] = rhs_row(T, in + (long)q * n, 1, i);
        }
        __syncwarp();
        if (lane < npw) {
            double *t = tile + lane * 33;
            for (int r = 0; r < cl; ++r) {
                const int i = c0 + r;
                const double v = t[r] - rows[i].m * wp;
                t[r] = v;
                if (T.periodic && i < T.ku) y0 += T.u0[i] * v;
                wp = v;
            }
        }
        __syncwarp();
        if (lane < cl)
            for (int q = 0; q < npw; ++q) w[(long)q * n + c0 + lane] = tile[q * 33 + lane];
        __syncwarp();
    }

    double fact = 0.0;
    if (T.periodic) fact = (y0 + T.sm1 * wp) * T.sm2;
    double yn = 0.0;
    for (int c0 = ((n - 1) / 32) * 32; c0 >= 0; c0 -= 32) {
        const int cl = min(32, n - c0);
        if (lane < cl)
            for (int q = 0; q < npw; ++q) tile[q * 33 + lane] = w[(long)q * n + c0 + lane];
        __syncwarp();
        if (lane < npw) {
            double *t = tile + lane * 33;
            for (int r = cl - 1; r >= 0; --r) {
                const int i = c0 + r;
                const double y = t[r] - rows[i].g * yn;
                yn = y;
                double xv = y;
                if (T.periodic && (i < T.zlo || i >= T.zhi)) xv = y - fact * T.zz[i];
                t[r] = xv;
            }
        }
        __syncwarp();
        if (lane < cl) {
            for (int q = 0; q < npw; ++q) {
                double v = tile[q * 33 + lane];
                double *o = out + (long)q * n + c0 + lane;
                if (EPI == EPI_ACCUM) v += *o;
                *o = v;
            }
        }
        __syncwarp();
    }
}

// Launch helper: derivative of nf fields along axis; w may equal out when
// epi == EPI_STORE.  in must not alias w/out.
int launch_deriv(const DerivTable &T, int axis, int epi, int nf, const double *const *in,
                 double *const *w, double *const *out, int nx, int ny, int nz,
                 cudaStream_t st);

} // namespace emix
