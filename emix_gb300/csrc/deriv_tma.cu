// deriv_tma.cu -- the y/z pencil sweeps with their rows staged by TMA tiled
// copies (k_deriv_yz_tma; deriv_tma.cuh), and the counters of their bounded
// waits.
//
// Per row the arithmetic is the load kernels' (deriv.cuh): accumulating,
// deriv_yz_accum's forward sweep u_i = fma(c_i, f_{i+2} - f_{i-2},
// f_{i+1} - f_{i-1}) - mu_i u_{i-1} on the scaled unknowns, backward
// z_i = u_i - gu_i z_{i+1}, out_i += k_i z_i; storing, deriv_yz_body's
// w_i = A_i (f_{i+1} - f_{i-1}) + B_i (f_{i+2} - f_{i-2}) - m_i w_{i-1},
// x_i = w_i - g_i x_{i+1}; closures by their explicit four-point rows.
// Only where the rows come from differs.  The reference transposes the field and walks each pencil
// serially (src/Schemes/derivCompact.cu:8-37,146-215).
#include "deriv_tma.cuh"
#include "tma.cuh"

#include <cstring>

namespace emix {
namespace {


// blocks that gave up waiting for a copy; copies left out (test hook)
__device__ int g_pencil_tma_timeouts = 0;
__device__ int g_pencil_tma_drop = 0;

EMIX_DEV void expect_bytes(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}

EMIX_DEV void copy_rows(const CUtensorMap *map, unsigned dst, unsigned bar, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];"
                 :: "r"(dst), "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
                 : "memory");
}

// The ring of one block: kPtS shared buffers of two boxes each, one mbarrier
// per buffer.  Copy number q goes to buffer q % kPtS and completes phase
// (q / kPtS) & 1 of its barrier.  Thread 0 issues and waits; every thread
// keeps the same counts of copies issued and of waits.
template <int B>
struct PencilRing {
    static constexpr unsigned kBytes = B * kPtR * 8;   // one box
    static constexpr int kBuf = 2 * kPtR * B;          // doubles per buffer
    double *buf;
    unsigned long long *bar;
    int *s_ok;
    bool go;          // false: the copies are left out (test hook)
    int issued = 0;   // copies issued so far
    int waits = 0;    // waits so far

    EMIX_DEV void init() {
        if (threadIdx.x == 0) {
            for (int b = 0; b < kPtS; ++b)
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar[b])), "r"(1) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
    }
    EMIX_DEV double *slot(int q) const { return buf + (q % kPtS) * kBuf; }
    // thread 0: copy q, the box of map m at (x0, c1, c2) into the buffer's
    // lower half and, with m2, the box of m2 at (x0, d1, d2) into its upper half
    EMIX_DEV void copy(int q, const CUtensorMap *m, int x0, int c1, int c2, const CUtensorMap *m2, int d1,
                       int d2) {
        const unsigned b = smem_u32(&bar[q % kPtS]);
        expect_bytes(b, m2 ? 2 * kBytes : kBytes);
        copy_rows(m, smem_u32(slot(q)), b, x0, c1, c2);
        if (m2) copy_rows(m2, smem_u32(slot(q) + kPtR * B), b, x0, d1, d2);
    }
    // copies q0 .. q0 + cnt - 1 into buffers no thread reads any more (after
    // a block-wide barrier)
    template <class F>
    EMIX_DEV void start(int q0, int cnt, F &&issue) {
        if (!go) return;
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            for (int q = q0; q < q0 + cnt; ++q) issue(q);
        }
        issued += cnt;
    }
    // copy q into the buffer every thread has finished reading (the caller
    // has passed a wait since its last read)
    template <class F>
    EMIX_DEV void refill(int q, F &&issue) {
        if (!go) return;
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q);
        }
        ++issued;
    }
    // copy q landed (a block-wide barrier); s_ok by the parity of the wait's
    // count, so the next wait cannot overwrite a flag still being read
    EMIX_DEV bool wait(int q) {
        const int k = waits++ & 1;
        if (threadIdx.x == 0) s_ok[k] = mbar_wait(smem_u32(&bar[q % kPtS]), (unsigned)((q / kPtS) & 1));
        __syncthreads();
        return s_ok[k] != 0;
    }
    // copy q did not arrive: count the block, let the copies in flight land
    // (bounded) before the block's shared memory goes
    EMIX_DEV void give_up(int q) {
        if (threadIdx.x == 0) {
            atomicAdd(&g_pencil_tma_timeouts, 1);
            for (int p = q; p < issued; ++p) mbar_wait(smem_u32(&bar[p % kPtS]), (unsigned)((p / kPtS) & 1));
        }
    }
};

// box coordinates of the rows from `row` along `axis` of the block's pencils
EMIX_DEV void box_origin(int axis, int o, int row, int &c1, int &c2) {
    if (axis == 1) { c1 = row; c2 = o; } else { c1 = o; c2 = row; }
}

// One block's pencils (B consecutive x, one per thread) of one field along
// `axis`: table T, input in (read directly only for the cyclic wrap),
// forward-sweep buffer w, output out (EPI_STORE: w = out), rows brought
// through the ring R.  Copy numbers run over both sweeps: the forward sweep's
// copy of chunk c (rows 4c .. 4c+3) is number c, the backward sweep's copy of
// chunk C-1-q is number C+q.  CYC: the cyclic operator (the load kernels'
// deriv_yz_accum / deriv_yz_body periodic path, row for row): every row a
// stencil row, the window wrapping round the pencil, rows [0, ku) summing
// the Sherman-Morrison y0, the correction fact zz_i on rows outside
// [zlo, zhi) of the backward sweep.
template <int B, int EPI, bool CYC>
EMIX_DEV void tma_pencils(const CUtensorMap *mi, const CUtensorMap *mw, const CUtensorMap *mo,
                          const DerivTable &T, const double *in, double *w, double *out, bool live, int x0,
                          int o, int axis, long s, PencilRing<B> &R) {
    constexpr int kBuf = PencilRing<B>::kBuf;
    const int tid = threadIdx.x;
    const int n = T.n, C = (n + kPtR - 1) / kPtR;
    const double *buf = R.buf;
    auto issue_in = [&](int q) {   // forward copy q = chunk q
        int c1, c2;
        box_origin(axis, o, q * kPtR, c1, c2);
        R.copy(q, mi, x0, c1, c2, nullptr, 0, 0);
    };
    // backward copy q = chunk C-1-(q-C): w, and the target when accumulating
    auto issue_wo = [&](int q) {
        int c1, c2;
        box_origin(axis, o, (C - 1 - (q - C)) * kPtR, c1, c2);
        R.copy(q, mw, x0, c1, c2, EPI == EPI_ACCUM ? mo : nullptr, c1, c2);
    };
    R.init();
    const int first = C < kPtS ? C : kPtS;
    R.start(0, first, issue_in);

    // ---- forward sweep ----
    if (!R.wait(0)) { R.give_up(0); return; }
    const double h0 = buf[tid], h1 = buf[B + tid], h2 = buf[2 * B + tid], h3 = buf[3 * B + tid];
    double up = 0.0, fact = 0.0;
    if constexpr (CYC) {
        // f_{n-2}, f_{n-1} by plain loads, f_n = f_0 and f_{n+1} = f_1 from
        // the first chunk
        double fm2 = in[(n - 2) * s], fm1 = in[(n - 1) * s], f0 = h0, fp1 = h1;
        const int ku = T.ku < n ? T.ku : n;
        double y0 = 0.0;
        int cur = 0;
        for (int i = 0; i < n; ++i) {
            const int j = i + 2;
            double fp2;
            if (j < n) {
                const int c = j / kPtR;
                if (c != cur) {
                    if (!R.wait(c)) { R.give_up(c); return; }
                    if (cur + kPtS < C) R.refill(cur + kPtS, issue_in);
                    cur = c;
                }
                fp2 = buf[(c % kPtS) * kBuf + (j - c * kPtR) * B + tid];
            } else {
                fp2 = j == n ? h0 : h1;
            }
            double v;
            if (EPI == EPI_ACCUM) {
                const DerivRowU r = T.urows[i];
                const double t = fma(r.c, fp2 - fm2, fp1 - fm1);
                v = t - r.mu * up;
                if (i < ku) y0 += T.u0s[i] * v;
            } else {
                const DerivRow r = T.rows[i];
                v = r.A * (fp1 - fm1) + r.B * (fp2 - fm2) - r.m * up;
                if (i < ku) y0 += T.u0[i] * v;
            }
            if (live) w[i * s] = v;
            up = v;
            fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
        }
        fact = (y0 + (EPI == EPI_ACCUM ? T.sm1s : T.sm1) * up) * T.sm2;
    } else {
    // closure rows 0, 1 on f_0..f_3 (the table builder guarantees nlo == 2)
    for (int i = 0; i < T.nlo; ++i) {
        const double *c = T.clo + 4 * i;
        const double m = EPI == EPI_ACCUM ? T.urows[i].mu : T.rows[i].m;
        const double v = (c[0] * h0 + c[1] * h1 + c[2] * h2 + c[3] * h3) - m * up;
        if (live) w[i * s] = v;
        up = v;
    }
    double fm2 = h0, fm1 = h1, f0 = h2, fp1 = h3;
    const int iend = n - T.nhi;
    int cur = 0;   // the chunk the window reads from
    for (int i = T.nlo; i < iend; ++i) {
        const int j = i + 2, c = j / kPtR;
        if (c != cur) {
            // chunk `cur` is read by every thread: its buffer takes the copy
            // kPtS chunks ahead
            if (!R.wait(c)) { R.give_up(c); return; }
            if (cur + kPtS < C) R.refill(cur + kPtS, issue_in);
            cur = c;
        }
        const double fp2 = buf[(c % kPtS) * kBuf + (j - c * kPtR) * B + tid];
        double v;
        if (EPI == EPI_ACCUM) {
            const DerivRowU r = T.urows[i];
            const double t = fma(r.c, fp2 - fm2, fp1 - fm1);
            v = t - r.mu * up;
        } else {
            const DerivRow r = T.rows[i];
            v = r.A * (fp1 - fm1) + r.B * (fp2 - fm2) - r.m * up;
        }
        if (live) w[i * s] = v;
        up = v;
        fm2 = fm1; fm1 = f0; f0 = fp1; fp1 = fp2;
    }
    // closure rows n-2, n-1 on f_{n-1}..f_{n-4}, which the window now holds
    const double t0 = fp1, t1 = f0, t2 = fm1, t3 = fm2;
    for (int i = iend; i < n; ++i) {
        const double *c = T.chi + 4 * (n - 1 - i);
        const double m = EPI == EPI_ACCUM ? T.urows[i].mu : T.rows[i].m;
        const double v = (c[0] * t0 + c[1] * t1 + c[2] * t2 + c[3] * t3) - m * up;
        if (live) w[i * s] = v;
        up = v;
    }
    }
    // the stores of w must be visible to the copy unit's reads below
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();

    // ---- backward sweep: chunks from the top ----
    R.start(C, first, issue_wo);
    double zn = 0.0;
    for (int q = 0; q < C; ++q) {
        const int c = C - 1 - q, seq = C + q;
        if (!R.wait(seq)) { R.give_up(seq); return; }
        if (q >= 1 && q - 1 + kPtS < C) R.refill(seq - 1 + kPtS, issue_wo);
        const double *Wb = R.slot(seq), *Ob = Wb + kPtR * B;
        const int ihi = min(n - 1, c * kPtR + kPtR - 1);
        for (int i = ihi; i >= c * kPtR; --i) {
            const int rr = i - c * kPtR;
            const double wi = Wb[rr * B + tid];
            if (EPI == EPI_ACCUM) {
                const double oi = Ob[rr * B + tid];
                const DerivRowU r = T.urows[i];
                const double z = wi - r.gu * zn;
                zn = z;
                double acc = oi;
                if (CYC && (i >= T.zhi || i < T.zlo)) acc = oi - fact * T.zz[i];
                if (live) out[i * s] = fma(r.k, z, acc);
            } else {
                const double y = wi - T.rows[i].g * zn;
                zn = y;
                double xv = y;
                if (CYC && (i >= T.zhi || i < T.zlo)) xv = y - fact * T.zz[i];
                if (live) out[i * s] = xv;
            }
        }
    }
}

// D^T = (1/h) B^T A^{-T} of one block's pencils, the arithmetic of the load
// kernel k_deriv_t (adjoint_deriv.cu) row for row: the forward sweep of A^T,
// y_i = fma(-m_i, y_{i-1}, in_i ib_i), on rows of `in` from the ring into w;
// the backward sweep z_i = w_i - g_i z_{i+1} on rows of w from the ring, with
// the window zq[t] = z_{i+t} from which out_j, j = i + 3, is finished (the
// interior rows by the antisymmetric stencil, the closure rows by B^T's
// 7-point rows).  Accumulating, the targets out_j of a chunk come with its w
// rows as a second box three rows further along (rows past the end read as
// zero and are not written); rows 0..2, finished after the last chunk, by
// plain loads.
template <int B, int ACC>
EMIX_DEV void tma_pencils_t(const CUtensorMap *mi, const CUtensorMap *mw, const CUtensorMap *mo,
                            const DerivTTable &T, double *w, double *out, bool live, int x0, int o, int axis,
                            long s, PencilRing<B> &R) {
    const int tid = threadIdx.x;
    const int n = T.n, C = (n + kPtR - 1) / kPtR;
    auto issue_in = [&](int q) {
        int c1, c2;
        box_origin(axis, o, q * kPtR, c1, c2);
        R.copy(q, mi, x0, c1, c2, nullptr, 0, 0);
    };
    auto issue_wo = [&](int q) {
        const int row = (C - 1 - (q - C)) * kPtR;
        int c1, c2, d1, d2;
        box_origin(axis, o, row, c1, c2);
        box_origin(axis, o, row + 3, d1, d2);
        R.copy(q, mw, x0, c1, c2, ACC ? mo : nullptr, d1, d2);
    };
    R.init();
    const int first = C < kPtS ? C : kPtS;
    R.start(0, first, issue_in);

    // ---- forward sweep of A^T ----
    double y = 0.0;
    for (int c = 0; c < C; ++c) {
        if (!R.wait(c)) { R.give_up(c); return; }
        if (c >= 1 && c - 1 + kPtS < C) R.refill(c - 1 + kPtS, issue_in);
        const double *Ib = R.slot(c) + tid;
        const int i0 = c * kPtR;
        if (i0 + kPtR <= n) {
            // a whole chunk: its four rows read at once
            const DerivTRow r0 = T.rows[i0], r1 = T.rows[i0 + 1], r2 = T.rows[i0 + 2], r3 = T.rows[i0 + 3];
            const double a0 = Ib[0] * r0.ib, a1 = Ib[B] * r1.ib, a2 = Ib[2 * B] * r2.ib, a3 = Ib[3 * B] * r3.ib;
            y = fma(-r0.m, y, a0);
            if (live) w[i0 * s] = y;
            y = fma(-r1.m, y, a1);
            if (live) w[(i0 + 1) * s] = y;
            y = fma(-r2.m, y, a2);
            if (live) w[(i0 + 2) * s] = y;
            y = fma(-r3.m, y, a3);
            if (live) w[(i0 + 3) * s] = y;
        } else {
            for (int i = i0; i < n; ++i) {
                const DerivTRow r = T.rows[i];
                y = fma(-r.m, y, Ib[(i - i0) * B] * r.ib);
                if (live) w[i * s] = y;
            }
        }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();

    // ---- backward sweep and B^T ----
    R.start(C, first, issue_wo);
    double zq[7];
#pragma unroll
    for (int t = 0; t < 7; ++t) zq[t] = 0.0;
    double z = 0.0;
    const bool fast = T.jlo <= T.jhi;
    // z_i into the window
    auto push = [&](int i, double wi) {
#pragma unroll
        for (int t = 6; t > 0; --t) zq[t] = zq[t - 1];
        z = (i == n - 1) ? wi : fma(-T.rows[i].g, z, wi);
        zq[0] = z;
    };
    // out_j of an interior row (the antisymmetric stencil); old: its value
    auto interior = [&](double old) {
        return ACC ? fma(T.ta, zq[2] - zq[4], fma(T.tb, zq[1] - zq[5], old))
                   : fma(T.ta, zq[2] - zq[4], T.tb * (zq[1] - zq[5]));
    };
    auto finish = [&](int j, double old) {   // out_j from the window
        double v;
        if (fast && j >= T.jlo && j <= T.jhi) {
            v = interior(old);
        } else {
            const double *b = T.bt + 7 * (long)j;
            v = b[0] * zq[0];
#pragma unroll
            for (int t = 1; t < 7; ++t) v = fma(b[t], zq[t], v);
            if (ACC) v = old + v;
        }
        if (live) out[j * s] = v;
    };
    for (int q = 0; q < C; ++q) {
        const int c = C - 1 - q, seq = C + q;
        if (!R.wait(seq)) { R.give_up(seq); return; }
        if (q >= 1 && q - 1 + kPtS < C) R.refill(seq - 1 + kPtS, issue_wo);
        const double *Wb = R.slot(seq) + tid, *Ob = Wb + kPtR * B;
        const int i0 = c * kPtR;
        if (fast && i0 + kPtR <= n - 1 && i0 + 3 >= T.jlo && i0 + kPtR + 2 <= T.jhi) {
            // a whole chunk of interior rows j = i + 3, none the last row
            const double w3 = Wb[3 * B], w2 = Wb[2 * B], w1 = Wb[B], w0 = Wb[0];
            double o3 = 0.0, o2 = 0.0, o1 = 0.0, o0 = 0.0;
            if (ACC) { o3 = Ob[3 * B]; o2 = Ob[2 * B]; o1 = Ob[B]; o0 = Ob[0]; }
            const double g3 = T.rows[i0 + 3].g, g2 = T.rows[i0 + 2].g, g1 = T.rows[i0 + 1].g,
                         g0 = T.rows[i0].g;
            auto row = [&](int i, double g, double wi, double old) {
#pragma unroll
                for (int t = 6; t > 0; --t) zq[t] = zq[t - 1];
                z = fma(-g, z, wi);
                zq[0] = z;
                const double v = interior(old);
                if (live) out[(i + 3) * s] = v;
            };
            row(i0 + 3, g3, w3, o3);
            row(i0 + 2, g2, w2, o2);
            row(i0 + 1, g1, w1, o1);
            row(i0, g0, w0, o0);
        } else {
            for (int i = min(n - 1, i0 + kPtR - 1); i >= i0; --i) {
                const int rr = i - i0;
                push(i, Wb[rr * B]);
                if (i + 3 < n) finish(i + 3, ACC ? Ob[rr * B] : 0.0);
            }
        }
    }
    // rows 2, 1, 0 (i = -1, -2, -3): zeros enter the window
    for (int j = 2; j >= 0; --j) {
#pragma unroll
        for (int t = 6; t > 0; --t) zq[t] = zq[t - 1];
        zq[0] = 0.0;
        if (j < n) finish(j, ACC && live ? out[j * s] : 0.0);
    }
}

// grid (ceil(nx / B), max of the fields' other extents, nf), B threads.
// Fields [0, nfa) run with table Ta, the rest with Tb, each along its map's
// axis.
template <int B, int EPI, bool CYC>
__global__ void __launch_bounds__(B)
k_deriv_yz_tma(const __grid_constant__ PencilMaps M, const DerivTable Ta, const DerivTable Tb,
               const PencilFields F, int nfa, int nx, int ny, int nz) {
    __shared__ __align__(128) double buf[kPtS * 2 * kPtR * B];
    __shared__ __align__(8) unsigned long long bar[kPtS];
    __shared__ int s_ok[2];
    const int f = blockIdx.z, o = blockIdx.y, axis = M.axis[f];
    const int nother = axis == 1 ? nz : ny;
    if (o >= nother) return;   // the whole block, before any barrier
    const long s = axis == 1 ? (long)nx : (long)nx * ny;
    const long os = axis == 1 ? (long)nx * ny : (long)nx;
    const int x0 = blockIdx.x * B, x = x0 + (int)threadIdx.x;
    const bool live = x < nx;
    const long off = (long)(live ? x : 0) + (long)o * os;
    const double *in = pick(F.in, f) + off;
    double *w = pick(F.w, f) + off;
    double *out = pick(F.out, f) + off;
    PencilRing<B> R{buf, bar, s_ok, g_pencil_tma_drop == 0};
    if (f < nfa)
        tma_pencils<B, EPI, CYC>(&M.in[f], &M.w[f], &M.out[f], Ta, in, w, out, live, x0, o, axis, s, R);
    else
        tma_pencils<B, EPI, CYC>(&M.in[f], &M.w[f], &M.out[f], Tb, in, w, out, live, x0, o, axis, s, R);
}

// D^T of nf fields along their maps' axes (one table), the same grid
template <int B, int ACC>
__global__ void __launch_bounds__(B)
k_deriv_t_yz_tma(const __grid_constant__ PencilMaps M, const DerivTTable T, const PencilFields F, int nx,
                 int ny, int nz) {
    __shared__ __align__(128) double buf[kPtS * 2 * kPtR * B];
    __shared__ __align__(8) unsigned long long bar[kPtS];
    __shared__ int s_ok[2];
    const int f = blockIdx.z, o = blockIdx.y, axis = M.axis[f];
    const int nother = axis == 1 ? nz : ny;
    if (o >= nother) return;   // the whole block, before any barrier
    const long s = axis == 1 ? (long)nx : (long)nx * ny;
    const long os = axis == 1 ? (long)nx * ny : (long)nx;
    const int x0 = blockIdx.x * B, x = x0 + (int)threadIdx.x;
    const bool live = x < nx;
    const long off = (long)(live ? x : 0) + (long)o * os;
    PencilRing<B> R{buf, bar, s_ok, g_pencil_tma_drop == 0};
    tma_pencils_t<B, ACC>(&M.in[f], &M.w[f], &M.out[f], T, pick(F.w, f) + off, pick(F.out, f) + off, live, x0,
                          o, axis, s, R);
}

} // namespace

bool pencil_tma_maps(PencilMaps *M, const int *axis, int nf, const double *const *in, double *const *w,
                     double *const *out, int nx, int ny, int nz) {
    if (nf < 1 || nf > kMaxFields || (nx & 1) != 0) return false;
    PFN_cuTensorMapEncodeTiled_v12000 fn = tma_encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t stride[2] = {(cuuint64_t)nx * 8, (cuuint64_t)nx * ny * 8};
    // block width: the one of 128, 64, 32 pencils that idles the fewest lanes
    int width = 128, waste = ((nx + 127) / 128) * 128 - nx;
    for (int b : {64, 32}) {
        const int wv = ((nx + b - 1) / b) * b - nx;
        if (wv < waste) { width = b; waste = wv; }
    }
    // a launch of fewer than 8 blocks per SM (small grids) is spread evenly
    // instead: the width that gives the most loaded SM the fewest pencil
    // slots (its blocks, ceil(blocks / SMs), times the width), the wider on
    // a tie
    int nother = 0;
    for (int f = 0; f < nf; ++f) nother = max(nother, axis[f] == 1 ? nz : ny);
    const long sms = device_sms();
    if ((long)((nx + width - 1) / width) * nother * nf < 8 * sms) {
        long best = 0;
        for (int b : {128, 64, 32}) {
            const long blocks = (long)((nx + b - 1) / b) * nother * nf;
            const long slots = (blocks + sms - 1) / sms * b;
            if (b == 128 || slots < best) { width = b; best = slots; }
        }
    }
    const cuuint32_t estride[3] = {1, 1, 1};
    std::memset(M, 0, sizeof *M);
    for (int f = 0; f < nf; ++f) {
        if (axis[f] != 1 && axis[f] != 2) return false;
        const cuuint32_t box[3] = {(cuuint32_t)width, axis[f] == 1 ? (cuuint32_t)kPtR : 1u,
                                   axis[f] == 2 ? (cuuint32_t)kPtR : 1u};
        auto enc = [&](CUtensorMap *m, const double *p) {
            if ((reinterpret_cast<uintptr_t>(p) & 15) != 0) return false;
            return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(p), dim, stride, box, estride,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        };
        if (!enc(&M->in[f], in[f]) || !enc(&M->w[f], w[f]) || !enc(&M->out[f], out[f])) return false;
        M->axis[f] = axis[f];
    }
    M->width = width;
    return true;
}

int launch_deriv_yz_tma(const DerivTable &Ta, const DerivTable &Tb, const PencilMaps &M, int epi, int nfa, int nf,
                        const double *const *in, double *const *w, double *const *out, int nx, int ny, int nz,
                        cudaStream_t st) {
    if (nf < 1 || nf > kMaxFields || nfa < 0 || nfa > nf || (epi != EPI_STORE && epi != EPI_ACCUM)) return EMIX_ERR_ARG;
    // one launch is all closed or all cyclic tables
    const bool cyc = (nfa > 0 ? Ta : Tb).periodic != 0;
    int nother = 0;
    for (int f = 0; f < nf; ++f) {
        const DerivTable &T = f < nfa ? Ta : Tb;
        const int ax = M.axis[f];
        if ((ax != 1 && ax != 2) || (T.periodic != 0) != cyc || (!cyc && (T.nlo != 2 || T.nhi != 2)) ||
            T.n != (ax == 1 ? ny : nz))
            return EMIX_ERR_ARG;
        nother = max(nother, ax == 1 ? nz : ny);
    }
    if (nother > 65535) return EMIX_ERR_ARG;
    PencilFields F{};
    for (int f = 0; f < nf; ++f) {
        F.in[f] = in[f];
        F.w[f] = w[f];
        F.out[f] = out[f];
    }
    const int B = M.width;
    const dim3 grid((nx + B - 1) / B, nother, nf);
#define EMIX_TMA_LAUNCH(BW, CY)                                                                     \
    if (B == BW && cyc == CY) {                                                                     \
        if (epi == EPI_ACCUM)                                                                       \
            k_deriv_yz_tma<BW, EPI_ACCUM, CY><<<grid, BW, 0, st>>>(M, Ta, Tb, F, nfa, nx, ny, nz);  \
        else                                                                                        \
            k_deriv_yz_tma<BW, EPI_STORE, CY><<<grid, BW, 0, st>>>(M, Ta, Tb, F, nfa, nx, ny, nz);  \
        EMIX_CUDA_TRY(cudaGetLastError());                                                          \
        return EMIX_OK;                                                                             \
    }
    EMIX_TMA_LAUNCH(128, false)
    EMIX_TMA_LAUNCH(64, false)
    EMIX_TMA_LAUNCH(32, false)
    EMIX_TMA_LAUNCH(128, true)
    EMIX_TMA_LAUNCH(64, true)
    EMIX_TMA_LAUNCH(32, true)
#undef EMIX_TMA_LAUNCH
    return EMIX_ERR_ARG;
}

int launch_deriv_t_yz_tma(const DerivTTable &T, const PencilMaps &M, int acc, int nf, const double *const *in,
                          double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st) {
    if (nf < 1 || nf > kMaxFields || (acc != 0 && acc != 1) || T.periodic) return EMIX_ERR_ARG;
    int nother = 0;
    for (int f = 0; f < nf; ++f) {
        const int ax = M.axis[f];
        if ((ax != 1 && ax != 2) || T.n != (ax == 1 ? ny : nz)) return EMIX_ERR_ARG;
        nother = max(nother, ax == 1 ? nz : ny);
    }
    if (nother > 65535) return EMIX_ERR_ARG;
    PencilFields F{};
    for (int f = 0; f < nf; ++f) {
        F.in[f] = in[f];
        F.w[f] = w[f];
        F.out[f] = out[f];
    }
    const int B = M.width;
    const dim3 grid((nx + B - 1) / B, nother, nf);
#define EMIX_TMA_LAUNCH(BW)                                                                         \
    if (B == BW) {                                                                                  \
        if (acc)                                                                                    \
            k_deriv_t_yz_tma<BW, 1><<<grid, BW, 0, st>>>(M, T, F, nx, ny, nz);                      \
        else                                                                                        \
            k_deriv_t_yz_tma<BW, 0><<<grid, BW, 0, st>>>(M, T, F, nx, ny, nz);                      \
        EMIX_CUDA_TRY(cudaGetLastError());                                                          \
        return EMIX_OK;                                                                             \
    }
    EMIX_TMA_LAUNCH(128)
    EMIX_TMA_LAUNCH(64)
    EMIX_TMA_LAUNCH(32)
#undef EMIX_TMA_LAUNCH
    return EMIX_ERR_ARG;
}

} // namespace emix

using namespace emix;

extern "C" int emix_pencil_tma_timeouts(int *count) {
    if (!count) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaMemcpyFromSymbol(count, g_pencil_tma_timeouts, sizeof(int)));
    return EMIX_OK;
}

extern "C" int emix_pencil_tma_test_drop(int on) {
    if (on != 0 && on != 1) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaMemcpyToSymbol(g_pencil_tma_drop, &on, sizeof(int)));
    EMIX_CUDA_TRY(cudaDeviceSynchronize());
    return EMIX_OK;
}
