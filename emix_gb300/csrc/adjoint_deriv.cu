// adjoint_deriv.cu -- D^T, the transpose of the compact first derivative
// D = (1/h) A^{-1} B of every scheme: D^T = (1/h) B^T A^{-T}.
//
// One thread per pencil: lanes along x for the y and z pencils; for the x
// pencils (contiguous rows) 32-row chunks staged through shared memory.  Forward sweep of
// A^T into the scratch w, backward sweep with a 7-value register window of z
// from which out_j = sum_k B^T[j][k] z_{j+k-3} is finished as soon as its last
// z is known (4 operations on the interior rows, where B^T is the
// antisymmetric 5-point stencil).  The cyclic scheme is anti-self-adjoint (D^T = -D) and uses the
// forward kernels with a negated table.  Given tensor maps, the y and z
// passes run k_deriv_t_yz_tma (deriv_tma.cu), the same arithmetic on rows
// staged by TMA.
#include "adjoint.cuh"

namespace emix {

namespace {

template <int ACC>
__global__ void __launch_bounds__(128) k_deriv_t(DerivTTable T, PencilFields F, int axis, int nx,
                                                 int ny, int nz) {
    const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long base, s;
    int L;
    if (axis == 0) {
        if (p >= (long)ny * nz) return;
        base = p * nx; s = 1; L = nx;
    } else if (axis == 1) {
        if (p >= (long)nx * nz) return;
        base = (p % nx) + (p / nx) * (long)nx * ny; s = nx; L = ny;
    } else {
        if (p >= (long)nx * ny) return;
        base = p; s = (long)nx * ny; L = nz;
    }
    const int f = blockIdx.y;
    const double *in = pick(F.in, f) + base;
    double *w = pick(F.w, f) + base;
    double *out = pick(F.out, f) + base;
    const DerivTRow *R = T.rows;
    const double *BT = T.bt;
    // forward: y_i = r_i ib_i - m_i y_{i-1}
    double y = 0.0;
    for (int i = 0; i < L; ++i) {
        const DerivTRow r = R[i];
        y = fma(-r.m, y, in[i * s] * r.ib);
        w[i * s] = y;
    }
    // backward: z_i = y_i - g_i z_{i+1}; zq[t] = z_{i+t}; out_j, j = i + 3,
    // once z_i is known.  Three branch-free runs of j: the closure rows at the
    // top, the interior rows (4 operations on the antisymmetric stencil), the
    // closure rows at the bottom.
    double zq[7];
#pragma unroll
    for (int t = 0; t < 7; ++t) zq[t] = 0.0;
    double z = 0.0;
    auto advance = [&](int i) {
#pragma unroll
        for (int t = 6; t > 0; --t) zq[t] = zq[t - 1];
        if (i >= 0) {
            const double wi = w[i * s];
            z = (i == L - 1) ? wi : fma(-R[i].g, z, wi);
            zq[0] = z;
        } else {
            zq[0] = 0.0;
        }
    };
    auto put = [&](int j, double o) {
        if (ACC) out[j * s] += o;
        else out[j * s] = o;
    };
    auto general = [&](int j) {
        const double *b = BT + 7 * (long)j;
        double o = b[0] * zq[0];
#pragma unroll
        for (int t = 1; t < 7; ++t) o = fma(b[t], zq[t], o);
        put(j, o);
    };
    const bool fast = T.jlo <= T.jhi;
    const int jtop = fast ? T.jhi : -1;   // rows above jtop: closure rows
    const int jbot = fast ? T.jlo : 0;    // rows below jbot: closure rows
    int i = L - 1;
    for (; i >= -3 && i + 3 > jtop; --i) {
        advance(i);
        if (i + 3 < L) general(i + 3);
    }
    if (fast) {
        for (; i + 3 >= jbot; --i) {
            advance(i);
            // accumulated: the add folds into the stencil's second FMA
            const long js = (long)(i + 3) * s;
            if (ACC) out[js] = fma(T.ta, zq[2] - zq[4], fma(T.tb, zq[1] - zq[5], out[js]));
            else out[js] = fma(T.ta, zq[2] - zq[4], T.tb * (zq[1] - zq[5]));
        }
    }
    for (; i >= -3; --i) {
        advance(i);
        general(i + 3);
    }
}

// x pencils (contiguous rows): a warp owns 32 pencils and stages 32-row
// chunks through a per-warp [32][kXLd] shared tile, loaded and stored with
// coalesced row accesses; each lane then walks its own pencil through the tile
// (as k_deriv_x does for D).  In the backward walk the output row j = i + 3 is
// written into the tile slot of w row j, which the descending walk has already
// consumed (slots up to 34 for the 3 rows past a 32-row chunk).
template <int ACC>
__global__ void __launch_bounds__(128) k_deriv_t_x(DerivTTable T, PencilFields F, long np) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *tile = smem + warp * kXTile;
    const long p0 = ((long)blockIdx.x * (blockDim.x >> 5) + warp) * 32;
    if (p0 >= np) return;   // whole warp
    const int npw = (int)min((long)32, np - p0);
    const int f = blockIdx.y;
    const int n = T.n;
    const double *in = pick(F.in, f) + p0 * n;
    double *w = pick(F.w, f) + p0 * n;
    double *out = pick(F.out, f) + p0 * n;
    const DerivTRow *R = T.rows;
    const double *BT = T.bt;
    double *t = tile + lane * kXLd;
    const bool mine = lane < npw;

    // forward: y_i = in_i ib_i - m_i y_{i-1}, chunk by chunk into w
    double y = 0.0;
    for (int c0 = 0; c0 < n; c0 += 32) {
        const int cl = min(32, n - c0);
        for (int q = 0; q < npw; ++q)
            if (lane < cl) tile[q * kXLd + lane] = in[(long)q * n + c0 + lane];
        __syncwarp();
        if (mine) {
            for (int r = 0; r < cl; ++r) {
                const DerivTRow rw = R[c0 + r];
                y = fma(-rw.m, y, t[r] * rw.ib);
                t[r] = y;
            }
        }
        __syncwarp();
        for (int q = 0; q < npw; ++q)
            if (lane < cl) w[(long)q * n + c0 + lane] = tile[q * kXLd + lane];
        __syncwarp();
    }

    // backward: z_i = w_i - g_i z_{i+1}; zq[t] = z_{i+t}; out_j, j = i + 3
    double zq[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) zq[k] = 0.0;
    double z = 0.0;
    const bool fast = T.jlo <= T.jhi;
    const int jtop = fast ? T.jhi : -1, jbot = fast ? T.jlo : 0;
    for (int c0 = ((n - 1) / 32) * 32; c0 >= 0; c0 -= 32) {
        const int cl = min(32, n - c0);
        for (int q = 0; q < npw; ++q)
            if (lane < cl) tile[q * kXLd + lane] = w[(long)q * n + c0 + lane];
        __syncwarp();
        if (mine) {
            auto advance = [&](int i) {
#pragma unroll
                for (int k = 6; k > 0; --k) zq[k] = zq[k - 1];
                if (i >= 0) {
                    const double wi = t[i - c0];
                    z = (i == n - 1) ? wi : fma(-R[i].g, z, wi);
                    zq[0] = z;
                } else {
                    zq[0] = 0.0;
                }
            };
            auto general = [&](int j) {
                const double *b = BT + 7 * (long)j;
                double o = b[0] * zq[0];
#pragma unroll
                for (int k = 1; k < 7; ++k) o = fma(b[k], zq[k], o);
                t[j - c0] = o;
            };
            const int iend = c0 == 0 ? -3 : c0;   // the last chunk also finishes rows 0..2
            int i = c0 + cl - 1;
            // three branch-free runs of j = i + 3: closure rows at the top, the
            // interior (4 operations), closure rows at the bottom
            for (; i >= iend && i + 3 > jtop; --i) {
                advance(i);
                if (i + 3 < n) general(i + 3);
            }
            if (fast) {
                for (; i >= iend && i + 3 >= jbot; --i) {
                    advance(i);
                    t[i + 3 - c0] = fma(T.ta, zq[2] - zq[4], T.tb * (zq[1] - zq[5]));
                }
            }
            for (; i >= iend; --i) {
                advance(i);
                general(i + 3);
            }
        }
        __syncwarp();
        // out rows [c0 + 3, c0 + cl + 3) (from row 0 in the last chunk), below n
        const int js = c0 == 0 ? 0 : c0 + 3, je = min(c0 + cl + 3, n);
        if (ACC) {
            // the targets of eight pencils loaded before any is stored, so
            // their loads are in flight together
            const int j = js + lane;
            const bool in1 = j < je;
            for (int q0 = 0; q0 < npw; q0 += 8) {
                double old[8];
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    old[k] = in1 && q0 + k < npw ? out[(long)(q0 + k) * n + j] : 0.0;
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (in1 && q0 + k < npw)
                        out[(long)(q0 + k) * n + j] = tile[(q0 + k) * kXLd + j - c0] + old[k];
            }
            // the last chunk's rows past the first 32 of its range
            for (int q = 0; q < npw; ++q)
                for (int jj = j + 32; jj < je; jj += 32) {
                    double *o = out + (long)q * n + jj;
                    *o = tile[q * kXLd + jj - c0] + *o;
                }
        } else {
            for (int q = 0; q < npw; ++q)
                for (int j = js + lane; j < je; j += 32) out[(long)q * n + j] = tile[q * kXLd + j - c0];
        }
        __syncwarp();
    }
}

} // namespace

int launch_deriv_t(const DerivTTable &T, int axis, int acc, int nf, const double *const *in,
                   double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st,
                   const PencilMaps *maps) {
    if (nf < 1 || nf > kMaxFields || axis < 0 || axis > 2) return EMIX_ERR_ARG;
    if (maps && axis != 0 && !T.periodic)
        return launch_deriv_t_yz_tma(T, *maps, acc, nf, in, w, out, nx, ny, nz, st);
    if (T.periodic) {
        if (!acc) return launch_deriv(T.neg, axis, EPI_STORE, nf, in, w, out, nx, ny, nz, st);
        return launch_deriv(T.neg, axis, EPI_ACCUM, nf, in, w, out, nx, ny, nz, st);
    }
    PencilFields F{};
    for (int f = 0; f < nf; ++f) {
        F.in[f] = in[f];
        F.w[f] = w[f];
        F.out[f] = out[f];
    }
    const long np = axis == 0 ? (long)ny * nz : (axis == 1 ? (long)nx * nz : (long)nx * ny);
    dim3 grid((unsigned)((np + 127) / 128), nf);
    if (axis == 0) {
        // warps of 32 pencils (four per block, fewer for small launches,
        // x_warps), one staging tile per warp
        const int warps = x_warps(np, nf);
        const dim3 gx((unsigned)((np + 32 * warps - 1) / (32 * warps)), nf);
        const size_t shm = warps * kXTile * sizeof(double);
        if (acc) k_deriv_t_x<1><<<gx, 32 * warps, shm, st>>>(T, F, np);
        else k_deriv_t_x<0><<<gx, 32 * warps, shm, st>>>(T, F, np);
    } else if (acc) {
        k_deriv_t<1><<<grid, 128, 0, st>>>(T, F, axis, nx, ny, nz);
    } else {
        k_deriv_t<0><<<grid, 128, 0, st>>>(T, F, axis, nx, ny, nz);
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

using namespace emix;

extern "C" {

namespace {

int deriv_t_dev(int scheme, int axis, int nf, double *out, const double *in, double h, int nx, int ny, int nz,
                int accumulate, void *stream, bool tma) {
    const int dims[3] = {nx, ny, nz};
    if (axis < 0 || axis > 2 || nf < 1 || nf > kMaxFields || !out || !in || !(h > 0) || nx < 1 ||
        ny < 1 || nz < 1 || (accumulate != 0 && accumulate != 1))
        return EMIX_ERR_ARG;
    DerivTTable T;
    int rc = get_deriv_t_table(scheme, dims[axis], h, &T);
    if (rc) return rc;
    if (tma && (axis == 0 || T.periodic)) return EMIX_ERR_ARG;
    const long n = (long)nx * ny * nz;
    double *scr;
    rc = device_scratch((size_t)nf * n * sizeof(double), &scr);
    if (rc) return rc;
    const double *ins[kMaxFields];
    double *ws[kMaxFields], *outs[kMaxFields];
    int axes[kMaxFields];
    for (int f = 0; f < nf; ++f) {
        ins[f] = in + f * n;
        ws[f] = scr + f * n;
        outs[f] = out + f * n;
        axes[f] = axis;
    }
    PencilMaps M;
    if (tma && !pencil_tma_maps(&M, axes, nf, ins, ws, outs, nx, ny, nz)) return EMIX_ERR_ARG;
    return launch_deriv_t(T, axis, accumulate, nf, ins, ws, outs, nx, ny, nz, (cudaStream_t)stream,
                          tma ? &M : nullptr);
}

} // namespace

int emix_deriv_t_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                     int nx, int ny, int nz, int accumulate, void *stream) {
    return deriv_t_dev(scheme, axis, nf, out, in, h, nx, ny, nz, accumulate, stream, false);
}

int emix_deriv_t_tma_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                         int nx, int ny, int nz, int accumulate, void *stream) {
    return deriv_t_dev(scheme, axis, nf, out, in, h, nx, ny, nz, accumulate, stream, true);
}

} // extern "C"
