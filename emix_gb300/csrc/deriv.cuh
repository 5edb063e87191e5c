// deriv.cuh -- compact first-derivative pencil kernels (FP64).
//
// One thread owns one pencil and runs the factored Thomas sweeps serially;
// the right-hand-side stencil is fused into the forward sweep.  On GB300 the
// FP64 pipe (about 0.5 T lane-ops/s) is the binding resource, so the kernels
// are written to minimise FP64 instructions: per interior cell 2 DADD + 1 DMUL
// + 1 DFMA for the stencil, 1 DFMA forward, 1 DFMA backward, and no divides
// (the pivots live in the factor table).  The accumulating y/z form (out +=
// D f) runs the sweeps on unknowns scaled by the stencil's leading
// coefficient and restores the scale in the accumulating FMA: 6 operations
// per cell instead of 7.
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
// out += D f along one y/z pencil, on the scaled unknowns of DerivRowU: a
// stencil row costs 2 DADD + 2 DFMA forward and 2 DFMA backward (the second
// one restores the scale and accumulates), one FP64 operation fewer than a
// store followed by an add.
EMIX_DEV void deriv_yz_accum(const DerivTable &T, const double *__restrict__ in, double *w,
                             double *out, long s) {
    const int n = T.n;
    const DerivRowU *__restrict__ ur = T.urows;
    double up = 0.0, y0 = 0.0;
    int i = 0;
    if (!T.periodic) {
        // closure rows: k = 1, so u = w
        for (; i < T.nlo; ++i) {
            const double v = rhs_row(T, in, s, i) - ur[i].mu * up;
            w[i * s] = v;
            up = v;
        }
        const int iend = n - T.nhi;
        if (i < iend) {
            double fm2 = in[(i - 2) * s], fm1 = in[(i - 1) * s], f0 = in[i * s], fp1 = in[(i + 1) * s];
            double q0 = in[(i + 2) * s];
            double q1 = i + 3 < n ? in[(i + 3) * s] : 0.0;
            double q2 = i + 4 < n ? in[(i + 4) * s] : 0.0;
            double q3 = i + 5 < n ? in[(i + 5) * s] : 0.0;
            for (; i < iend; ++i) {
                const double fp2 = q0;
                q0 = q1; q1 = q2; q2 = q3;
                if (i + 6 < n) q3 = in[(i + 6) * s];
                const DerivRowU r = ur[i];
                const double t = fma(r.c, fp2 - fm2, fp1 - fm1);
                const double v = t - r.mu * up;
                w[i * s] = v;
                up = v;
                fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
            }
        }
        for (; i < n; ++i) {
            const double v = rhs_row(T, in, s, i) - ur[i].mu * up;
            w[i * s] = v;
            up = v;
        }
    } else {
        double fm2 = in[(n - 2) * s], fm1 = in[(n - 1) * s], f0 = in[0], fp1 = in[s];
        double nxt = in[2 * s];
        auto prow = [&](int i, bool acc) {
            const double fp2 = nxt;
            int j = i + 3;
            if (j >= n) j -= n;
            nxt = in[j * s];
            const DerivRowU r = ur[i];
            const double t = fma(r.c, fp2 - fm2, fp1 - fm1);
            const double v = t - r.mu * up;
            w[i * s] = v;
            if (acc) y0 += T.u0s[i] * v;
            up = v;
            fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
        };
        const int ku = T.ku < n ? T.ku : n;
        for (; i < ku; ++i) prow(i, true);
        for (; i < n; ++i) prow(i, false);
    }

    double fact = 0.0;
    if (T.periodic) fact = (y0 + T.sm1s * up) * T.sm2;
    double zn = 0.0;
    double w0 = w[(n - 1) * s];
    double w1 = w[(n - 2) * s];
    double w2 = w[(n - 3) * s];
    double w3 = w[(n - 4) * s];
    double o0 = out[(n - 1) * s];
    double o1 = out[(n - 2) * s];
    double o2 = out[(n - 3) * s];
    double o3 = out[(n - 4) * s];
    auto row = [&](int i, bool corr) {
        const double wi = w0, oi = o0;
        w0 = w1; w1 = w2; w2 = w3;
        o0 = o1; o1 = o2; o2 = o3;
        if (i - 4 >= 0) {
            w3 = w[(i - 4) * s];
            o3 = out[(i - 4) * s];
        }
        const DerivRowU r = ur[i];
        const double z = wi - r.gu * zn;
        zn = z;
        double acc = oi;
        if (corr) acc = oi - fact * T.zz[i];
        out[i * s] = fma(r.k, z, acc);
    };
    i = n - 1;
    if (T.periodic) {
        for (; i >= T.zhi; --i) row(i, true);
        for (; i >= T.zlo; --i) row(i, false);
        for (; i >= 0; --i) row(i, true);
    } else {
        for (; i >= 0; --i) row(i, false);
    }
}

// Body for one (virtual) block: bid = (x block, pencil row, field).
template <int EPI>
EMIX_DEV void deriv_yz_body(const DerivTable &T, const PencilFields &F, int nx, int nother, long s,
                            long os, uint3 bid, int tid, int bdim) {
    const int x = bid.x * bdim + tid;
    const int o = bid.y;
    if (x >= nx || o >= nother) return;
    const long base = x + (long)o * os;
    const int f = bid.z;
    const double *__restrict__ in = pick(F.in, f) + base;
    double *w = pick(F.w, f) + base;
    double *out = pick(F.out, f) + base;
    if constexpr (EPI == EPI_ACCUM) {
        deriv_yz_accum(T, in, w, out, s);
        return;
    }
    const int n = T.n;
    const DerivRow *__restrict__ rows = T.rows;

    // forward sweep; the input two rows ahead comes from a queue of four rows
    // loaded four iterations early (the loads' latency is longer than an
    // iteration of every resident warp)
    double wp = 0.0, y0 = 0.0;
    int i = 0;
    if (!T.periodic) {
        for (; i < T.nlo; ++i) {
            const double v = rhs_row(T, in, s, i) - rows[i].m * wp;
            w[i * s] = v;
            wp = v;
        }
        const int iend = n - T.nhi;
        if (i < iend) {
            double fm2 = in[(i - 2) * s], fm1 = in[(i - 1) * s], f0 = in[i * s], fp1 = in[(i + 1) * s];
            // q0..q3 = f(i+2) .. f(i+5) (rows past the end read as 0, unused)
            double q0 = in[(i + 2) * s];
            double q1 = i + 3 < n ? in[(i + 3) * s] : 0.0;
            double q2 = i + 4 < n ? in[(i + 4) * s] : 0.0;
            double q3 = i + 5 < n ? in[(i + 5) * s] : 0.0;
            for (; i < iend; ++i) {
                const double fp2 = q0;
                q0 = q1; q1 = q2; q2 = q3;
                if (i + 6 < n) q3 = in[(i + 6) * s];
                const DerivRow r = rows[i];
                const double v = r.A * (fp1 - fm1) + r.B * (fp2 - fm2) - r.m * wp;
                w[i * s] = v;
                wp = v;
                fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
            }
        }
        for (; i < n; ++i) {
            const double v = rhs_row(T, in, s, i) - rows[i].m * wp;
            w[i * s] = v;
            wp = v;
        }
    } else {
        double fm2 = in[(n - 2) * s], fm1 = in[(n - 1) * s], f0 = in[0], fp1 = in[s];
        double nxt = in[2 * s];
        // rows [0, ku) also accumulate y0 (branch-free runs)
        auto prow = [&](int i, bool acc) {
            const double fp2 = nxt;
            int j = i + 3;
            if (j >= n) j -= n;
            nxt = in[j * s];
            const DerivRow r = rows[i];
            const double v = r.A * (fp1 - fm1) + r.B * (fp2 - fm2) - r.m * wp;
            w[i * s] = v;
            if (acc) y0 += T.u0[i] * v;
            wp = v;
            fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
        };
        const int ku = T.ku < n ? T.ku : n;
        for (; i < ku; ++i) prow(i, true);
        for (; i < n; ++i) prow(i, false);
    }

    // backward sweep; w from a queue of four rows loaded four iterations
    // early (pencils have at least 6 rows)
    double fact = 0.0;
    if (T.periodic) fact = (y0 + T.sm1 * wp) * T.sm2;
    double yn = 0.0;
    // w0..w3 = w(i) .. w(i-3)
    double w0 = w[(n - 1) * s];
    double w1 = w[(n - 2) * s];
    double w2 = w[(n - 3) * s];
    double w3 = w[(n - 4) * s];
    // one row; the cyclic correction only where zz is nonzero
    auto row = [&](int i, bool corr) {
        const double wi = w0;
        w0 = w1; w1 = w2; w2 = w3;
        if (i - 4 >= 0) w3 = w[(i - 4) * s];
        const double y = wi - rows[i].g * yn;
        yn = y;
        double xv = y;
        if (corr) xv = y - fact * T.zz[i];
        out[i * s] = xv;
    };
    // branch-free runs: the correction rows [zhi, n) and [0, zlo) of the
    // cyclic operator, none for the closed one
    i = n - 1;
    if (T.periodic) {
        for (; i >= T.zhi; --i) row(i, true);
        for (; i >= T.zlo; --i) row(i, false);
        for (; i >= 0; --i) row(i, true);
    } else {
        for (; i >= 0; --i) row(i, false);
    }
}

// grid: (ceil(nx/blockDim.x), nother, nf); blockIdx.z = field
template <int EPI>
__global__ void __launch_bounds__(128)
k_deriv_yz(DerivTable T, PencilFields F, int nx, int nother, long s, long os) {
    deriv_yz_body<EPI>(T, F, nx, nother, s, os, blockIdx, threadIdx.x, blockDim.x);
}

// Two y/z derivatives of the same kind in one launch: fields [0, nfa) along
// the first table's axis, the rest along the second's.  The velocity
// gradients' y and z pencils then fill the GPU as one grid of 6 fields, not
// two grids of 3 whose last waves leave most SMs idle.
// grid: (ceil(nx/blockDim.x), max(na, nb), nfa + nfb)
__global__ void __launch_bounds__(128)
k_deriv_yz_pair(DerivTable Ta, DerivTable Tb, PencilFields F, int nfa, int nx, int na, long sa,
                long osa, int nb, long sb, long osb);

// ---------------------------------------------------------------------------
// x pencils: a warp owns 32 consecutive pencils (flattened (j,k)).  Rows are
// staged 32 at a time (plus a 2-row look-ahead) through a per-warp shared tile
// with coalesced loads; each lane then walks its own pencil through the tile
// with the same register sliding window as the y/z kernel, writes w back into
// the tile, and the tile is stored coalesced.  The backward sweep streams the
// chunks in reverse the same way.
// grid: (ceil(npencil / (32*warps_per_block)), 1, nf); block 32*warps
// ---------------------------------------------------------------------------
constexpr int kXRows = 34;          // 32 rows + 2 look-ahead
constexpr int kXLd = kXRows + 1;    // padded leading dimension (odd: no bank conflicts)
constexpr int kXTile = 32 * kXLd;

// warps per block (4, 2 or 1) of an x-pencil launch over np pencils of nf
// fields: 4, unless that gives fewer than 8 blocks per SM (small grids); then
// the count that gives the most loaded SM the fewest warps (its blocks,
// ceil(blocks / SMs), times the warps), the larger on a tie
inline int x_warps(long np, int nf) {
    const long sms = device_sms();
    auto blocks = [&](int w) { return (np + 32L * w - 1) / (32L * w) * nf; };
    if (blocks(4) >= 8 * sms) return 4;
    int best = 4;
    long load = (blocks(4) + sms - 1) / sms * 4;
    for (int w : {2, 1}) {
        const long l = (blocks(w) + sms - 1) / sms * w;
        if (l < load) { best = w; load = l; }
    }
    return best;
}

// Body for one (virtual) block of `nwarps` warps: bid = (pencil group, -, field).
template <int EPI>
EMIX_DEV void deriv_x_body(const DerivTable &T, const PencilFields &F, long npencil, uint3 bid,
                           int tid, int nwarps, double *smem) {
    const int warp = tid >> 5, lane = tid & 31;
    double *tile = smem + warp * kXTile;
    const long p0 = ((long)bid.x * nwarps + warp) * 32;
    if (p0 >= npencil) return;  // whole warp
    const int npw = (int)min((long)32, npencil - p0);
    const int f = bid.z;
    const int n = T.n;
    const double *__restrict__ in = pick(F.in, f) + p0 * n;
    double *w = pick(F.w, f) + p0 * n;
    double *out = pick(F.out, f) + p0 * n;
    const DerivRow *__restrict__ rows = T.rows;
    double *t = tile + lane * kXLd;      // this lane's pencil in the tile
    const bool mine = lane < npw;

    // registers of the walk (lane = pencil)
    double wp = 0.0, y0 = 0.0;
    double fm2 = 0.0, fm1 = 0.0, f0 = 0.0, fp1 = 0.0;
    double head0 = 0.0, head1 = 0.0, head2 = 0.0, head3 = 0.0;   // f_0..f_3 (closures, wrap)
    double tail0 = 0.0, tail1 = 0.0, tail2 = 0.0, tail3 = 0.0;   // f_{n-1}..f_{n-4}
    if (T.periodic && mine) {
        fm2 = in[(long)lane * n + n - 2];
        fm1 = in[(long)lane * n + n - 1];
    }
    for (int c0 = 0; c0 < n; c0 += 32) {
        const int cl = min(32, n - c0);             // rows completed in this chunk
        const int ld = min(kXRows, n - c0);         // rows loaded (with look-ahead)
        // coalesced load: row r of pencil q -> tile[q][r]
        for (int q = 0; q < npw; ++q) {
            const double *src = in + (long)q * n + c0;
            if (lane < ld) tile[q * kXLd + lane] = src[lane];
            if (lane + 32 < ld) tile[q * kXLd + lane + 32] = src[lane + 32];
        }
        __syncwarp();
        if (mine) {
            int r = 0;
            if (c0 == 0) {
                head0 = t[0]; head1 = t[1]; head2 = t[2]; head3 = t[3];
                if (T.periodic) {
                    f0 = head0; fp1 = head1;   // fm2, fm1 hold f_{n-2}, f_{n-1}
                } else {
                    // the table builder guarantees nlo == 2: rows 0 and 1 are
                    // closures on f_0..f_3, and the window of row 2 is f_0..f_3
                    fm2 = head0; fm1 = head1; f0 = head2; fp1 = head3;
                    for (; r < T.nlo; ++r) {
                        const double *c = T.clo + 4 * r;
                        const double v = c[0] * head0 + c[1] * head1 + c[2] * head2 + c[3] * head3 -
                                         rows[r].m * wp;
                        t[r] = v;
                        wp = v;
                    }
                }
            }
            // one interior row (fp2 given); y0 accumulated on request
            auto irow = [&](int r, double fp2, bool acc) {
                const int i = c0 + r;
                const DerivRow rw = rows[i];
                const double v = rw.A * (fp1 - fm1) + rw.B * (fp2 - fm2) - rw.m * wp;
                if (acc) y0 += T.u0[i] * v;
                fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
                t[r] = v;
                wp = v;
            };
            // branch-free runs of rows
            if (!T.periodic) {
                const int rint = min(cl, n - T.nhi - c0);   // rows before the closures
                // unrolled: the walk through the tile reads shared memory only,
                // and later rows' stencils overlap the recurrence
#pragma unroll 4
                for (; r < rint; ++r) irow(r, t[r + 2], false);
                for (; r < cl; ++r) {
                    const int i = c0 + r;
                    // closures on f_{n-1}..f_{n-4} (nhi == 2): at row n-2 the
                    // window holds exactly those four values
                    if (i == n - T.nhi) { tail0 = fp1; tail1 = f0; tail2 = fm1; tail3 = fm2; }
                    const double *c = T.chi + 4 * (n - 1 - i);
                    const double v = c[0] * tail0 + c[1] * tail1 + c[2] * tail2 + c[3] * tail3 -
                                     rows[i].m * wp;
                    t[r] = v;
                    wp = v;
                }
            } else {
                const int rku = max(r, min(cl, T.ku - c0));     // rows i < ku: accumulate y0
                const int rnw = max(rku, min(cl, n - 2 - c0));  // rows i + 2 < n: no wrap
                for (; r < rku; ++r) {
                    const int i = c0 + r;
                    irow(r, (i + 2 < n) ? t[r + 2] : (i + 2 == n ? head0 : head1), true);
                }
                for (; r < rnw; ++r) irow(r, t[r + 2], false);
                for (; r < cl; ++r) irow(r, c0 + r + 2 == n ? head0 : head1, false);
            }
        }
        __syncwarp();
        for (int q = 0; q < npw; ++q)
            if (lane < cl) w[(long)q * n + c0 + lane] = tile[q * kXLd + lane];
        __syncwarp();
    }

    double fact = 0.0;
    if (T.periodic) fact = (y0 + T.sm1 * wp) * T.sm2;
    double yn = 0.0;
    for (int c0 = ((n - 1) / 32) * 32; c0 >= 0; c0 -= 32) {
        const int cl = min(32, n - c0);
        for (int q = 0; q < npw; ++q)
            if (lane < cl) tile[q * kXLd + lane] = w[(long)q * n + c0 + lane];
        __syncwarp();
        if (mine) {
            if (!T.periodic) {
#pragma unroll 4
                for (int r = cl - 1; r >= 0; --r) {
                    const double y = t[r] - rows[c0 + r].g * yn;
                    yn = y;
                    t[r] = y;
                }
            } else {
                for (int r = cl - 1; r >= 0; --r) {
                    const int i = c0 + r;
                    const double y = t[r] - rows[i].g * yn;
                    yn = y;
                    double xv = y;
                    if (i < T.zlo || i >= T.zhi) xv = y - fact * T.zz[i];
                    t[r] = xv;
                }
            }
        }
        __syncwarp();
        for (int q = 0; q < npw; ++q) {
            if (lane < cl) {
                double v = tile[q * kXLd + lane];
                double *o = out + (long)q * n + c0 + lane;
                if (EPI == EPI_ACCUM) v += *o;
                *o = v;
            }
        }
        __syncwarp();
    }
}

template <int EPI>
__global__ void __launch_bounds__(128)
k_deriv_x(DerivTable T, PencilFields F, long npencil) {
    extern __shared__ double smem[];
    deriv_x_body<EPI>(T, F, npencil, blockIdx, threadIdx.x, blockDim.x >> 5, smem);
}

// Launch helper: derivative of nf fields along axis; w may equal out when
// epi == EPI_STORE.  in must not alias w/out.
int launch_deriv(const DerivTable &T, int axis, int epi, int nf, const double *const *in,
                 double *const *w, double *const *out, int nx, int ny, int nz,
                 cudaStream_t st);

// Stored y and z derivatives in one launch (k_deriv_yz_pair): nfa fields
// along axis 1 (in/out [0, nfa)), nfb along axis 2 (the next nfb); w = out.
// The outputs must not alias each other or the inputs.
int launch_deriv_yz_pair(const DerivTable &Ty, const DerivTable &Tz, int nfa, int nfb,
                         const double *const *in, double *const *out, int nx, int ny, int nz,
                         cudaStream_t st);

} // namespace emix
