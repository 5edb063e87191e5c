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

// One block's pencils (B consecutive x, one per thread) of one field along
// `axis`: table T, forward-sweep buffer w, output out (EPI_STORE: w = out),
// rows brought through the shared ring `buf` ([kPtS][2][kPtR * B]) on the
// barriers `bar`.  Copy sequence numbers run over both sweeps: the forward
// sweep's copy of chunk c (rows 4c .. 4c+3) is number c, the backward
// sweep's copy of chunk C-1-q is number C+q; number q uses buffer q % kPtS at
// phase (q / kPtS) & 1.
template <int B, int EPI>
EMIX_DEV void tma_pencils(const CUtensorMap *mi, const CUtensorMap *mw, const CUtensorMap *mo,
                          const DerivTable &T, double *w, double *out, bool live, int x0, int o, int axis,
                          long s, double *buf, unsigned long long *bar, int *s_ok) {
    constexpr unsigned kBytes = B * kPtR * 8;   // one copy
    constexpr int kBuf = 2 * kPtR * B;          // doubles per ring buffer
    const int tid = threadIdx.x;
    const int n = T.n, C = (n + kPtR - 1) / kPtR;
    const bool go = g_pencil_tma_drop == 0;
    // box origin of chunk c: x0, and the chunk's first row along the axis
    auto origin = [&](int c, int &c1, int &c2) {
        if (axis == 1) { c1 = c * kPtR; c2 = o; } else { c1 = o; c2 = c * kPtR; }
    };
    auto issue_in = [&](int q) {   // forward copy q = chunk q
        const int b = q % kPtS;
        int c1, c2;
        origin(q, c1, c2);
        expect_bytes(smem_u32(&bar[b]), kBytes);
        copy_rows(mi, smem_u32(buf + b * kBuf), smem_u32(&bar[b]), x0, c1, c2);
    };
    // backward copy q = chunk C-1-(q-C): w, and the target when accumulating
    auto issue_wo = [&](int q) {
        const int b = q % kPtS;
        int c1, c2;
        origin(C - 1 - (q - C), c1, c2);
        expect_bytes(smem_u32(&bar[b]), EPI == EPI_ACCUM ? 2 * kBytes : kBytes);
        copy_rows(mw, smem_u32(buf + b * kBuf), smem_u32(&bar[b]), x0, c1, c2);
        if (EPI == EPI_ACCUM) copy_rows(mo, smem_u32(buf + b * kBuf + kPtR * B), smem_u32(&bar[b]), x0, c1, c2);
    };
    int issued = 0;   // copies issued so far (the same count in every thread)
    int waits = 0;    // waits so far (the same count in every thread)
    // s_ok by the parity of the wait's count: the next wait cannot overwrite
    // a flag still being read
    auto wait_copy = [&](int q) -> bool {
        const int k = waits++ & 1;
        if (tid == 0) s_ok[k] = mbar_wait(smem_u32(&bar[q % kPtS]), (unsigned)((q / kPtS) & 1));
        __syncthreads();
        return s_ok[k] != 0;
    };
    // copy q did not arrive: count the block, let the copies in flight land
    // (bounded) before the block's shared memory goes, leave the pencils
    auto give_up = [&](int q) {
        if (tid == 0) {
            atomicAdd(&g_pencil_tma_timeouts, 1);
            for (int p = q; p < issued; ++p) mbar_wait(smem_u32(&bar[p % kPtS]), (unsigned)((p / kPtS) & 1));
        }
    };

    if (tid == 0) {
        for (int b = 0; b < kPtS; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(&bar[b])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    const int first = C < kPtS ? C : kPtS;
    if (go) {
        if (tid == 0)
            for (int q = 0; q < first; ++q) issue_in(q);
        issued = first;
    }

    // ---- forward sweep ----
    if (!wait_copy(0)) { give_up(0); return; }
    const double h0 = buf[tid], h1 = buf[B + tid], h2 = buf[2 * B + tid], h3 = buf[3 * B + tid];
    double up = 0.0;
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
            if (!wait_copy(c)) { give_up(c); return; }
            if (go && cur + kPtS < C) {
                if (tid == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue_in(cur + kPtS);
                }
                ++issued;
            }
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
    // the stores of w must be visible to the copy unit's reads below
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();

    // ---- backward sweep: chunks from the top ----
    if (go) {
        if (tid == 0)
            for (int q = 0; q < first; ++q) issue_wo(C + q);
        issued += first;
    }
    double zn = 0.0;
    for (int q = 0; q < C; ++q) {
        const int c = C - 1 - q, seq = C + q;
        if (!wait_copy(seq)) { give_up(seq); return; }
        if (q >= 1 && go && q - 1 + kPtS < C) {
            if (tid == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_wo(seq - 1 + kPtS);
            }
            ++issued;
        }
        const double *Wb = buf + (seq % kPtS) * kBuf, *Ob = Wb + kPtR * B;
        const int ihi = min(n - 1, c * kPtR + kPtR - 1);
        for (int i = ihi; i >= c * kPtR; --i) {
            const int rr = i - c * kPtR;
            const double wi = Wb[rr * B + tid];
            if (EPI == EPI_ACCUM) {
                const double oi = Ob[rr * B + tid];
                const DerivRowU r = T.urows[i];
                const double z = wi - r.gu * zn;
                zn = z;
                if (live) out[i * s] = fma(r.k, z, oi);
            } else {
                const double y = wi - T.rows[i].g * zn;
                zn = y;
                if (live) out[i * s] = y;
            }
        }
    }
}

// grid (ceil(nx / B), max of the fields' other extents, nf), B threads.
// Fields [0, nfa) run with table Ta, the rest with Tb, each along its map's
// axis.
template <int B, int EPI>
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
    double *w = pick(F.w, f) + off;
    double *out = pick(F.out, f) + off;
    if (f < nfa)
        tma_pencils<B, EPI>(&M.in[f], &M.w[f], &M.out[f], Ta, w, out, live, x0, o, axis, s, buf, bar, s_ok);
    else
        tma_pencils<B, EPI>(&M.in[f], &M.w[f], &M.out[f], Tb, w, out, live, x0, o, axis, s, buf, bar, s_ok);
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
    int nother = 0;
    for (int f = 0; f < nf; ++f) {
        const DerivTable &T = f < nfa ? Ta : Tb;
        const int ax = M.axis[f];
        if ((ax != 1 && ax != 2) || T.periodic || T.nlo != 2 || T.nhi != 2 || T.n != (ax == 1 ? ny : nz))
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
#define EMIX_TMA_LAUNCH(BW)                                                                         \
    if (B == BW) {                                                                                  \
        if (epi == EPI_ACCUM)                                                                       \
            k_deriv_yz_tma<BW, EPI_ACCUM><<<grid, BW, 0, st>>>(M, Ta, Tb, F, nfa, nx, ny, nz);      \
        else                                                                                        \
            k_deriv_yz_tma<BW, EPI_STORE><<<grid, BW, 0, st>>>(M, Ta, Tb, F, nfa, nx, ny, nz);      \
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
