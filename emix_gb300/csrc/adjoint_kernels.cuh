// adjoint_kernels.cuh -- the adjoint kernels of one RK3 substep and of the
// tank objective, as argument structs plus kernels (adjoint.cu launches them).
#pragma once

#include "adjoint_cells.cuh"

namespace emix {

// sum of v over the block into *out (one atomic per block)
EMIX_DEV void block_sum_add(double v, double *out) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.0) atomicAdd(out, v);
    }
    __syncthreads();
}

// sum of v over the block into out[blockIdx.x] (no atomics: the partial sums
// are added in a fixed order by k_sum_partials, so the total is reproducible)
EMIX_DEV void block_sum_store(double v, double *out) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) out[blockIdx.x] = v;
    }
}

// out[0] = sum of the np partial sums, in a fixed order (one block of 1024)
__global__ void k_sum_partials(const double *part, int np, double *out) {
    __shared__ double s[1024];
    double v = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) v += part[i];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = s[0];
}

// ---- RK update: (convert + impeller)^T at every cell into T5 --------------
struct RkAdjArgs {
    RkArgs a;              // the forward substep's arguments (tape pointers)
    const double *lo;      // 5: adjoint of the substep's um output
    const double *lu;      // 3 or null: adjoint of its u output
    const double *lp;      // 1 or null: adjoint of its pres output
    double *T5;            // 5: adjoint of the values entering the impeller
    double *red;           // [0]: d/d omega
};

__global__ void __launch_bounds__(256) k_adj_rk_a(RkAdjArgs A) {
    const RkArgs &a = A.a;
    const long n = a.n;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    double lom = 0.0;
    for (long q0 = blockIdx.x * (long)blockDim.x; q0 < n; q0 += (long)gridDim.x * blockDim.x) {
        const long q = q0 + threadIdx.x;
        if (q < n) {
            double v[5];
            const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((long)nx * ny));
            if (a.walls && (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k >= nz - 2))
                wall_x(a, i, j, k, v);
            else
                rk_combine(a, q, v);
            double lo[5], lu[3] = {0.0, 0.0, 0.0}, lv[5];
            for (int m = 0; m < 5; ++m) lo[m] = A.lo[m * n + q];
            if (A.lu)
                for (int d = 0; d < 3; ++d) lu[d] = A.lu[d * n + q];
            const double lp = A.lp ? A.lp[q] : 0.0;
            convert_adj(a, q, v, lo, lu, lp, lv, &lom);
            for (int m = 0; m < 5; ++m) A.T5[m * n + q] = lv[m];
        }
    }
    block_sum_add(lom, A.red);
}

// the walls: each wall cell's adjoint goes to the cell its value was copied from
__global__ void k_adj_rk_b(RkAdjArgs A) {
    const RkArgs &a = A.a;
    const long n = a.n;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long nf = rk_face_count(nx, ny, nz);
    const long pz = (long)nx * ny, py = (long)nx * (nz - 3);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nf; q += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (q < 3 * pz) {
            const int pl = (int)(q / pz);
            const long r = q - pl * pz;
            i = (int)(r % nx); j = (int)(r / nx); k = pl == 0 ? 0 : nz - 3 + pl;
        } else if (q < 3 * pz + 2 * py) {
            const long r0 = q - 3 * pz;
            const int pl = (int)(r0 / py);
            const long r = r0 - pl * py;
            i = (int)(r % nx); k = 1 + (int)(r / nx); j = pl == 0 ? 0 : ny - 1;
        } else {
            const long px = (long)(ny - 2) * (nz - 3);
            const long r0 = q - 3 * pz - 2 * py;
            const int pl = (int)(r0 / px);
            const long r = r0 - pl * px;
            j = 1 + (int)(r % (ny - 2)); k = 1 + (int)(r / (ny - 2)); i = pl == 0 ? 0 : nx - 1;
        }
        const long f = i + (long)nx * (j + (long)ny * k);
        for (int c = 0; c < 5; ++c) {
            const double l = A.T5[c * n + f];
            const long src = wall_source(a, i, j, k, c);
            if (src >= 0 && l != 0.0) atomicAdd(&A.T5[c * n + src], l);
            A.T5[c * n + f] = 0.0;
        }
    }
}

// the RK combination: lum0 += ca lv, lumc = cb lv (or += into lum0), lR = cr j11 lv
struct RkCombAdjArgs {
    const double *T5, *jbn;
    double *lum0, *lumc, *lR;
    double ca, cb, cr;
    long n;
};

__global__ void k_adj_rk_c(RkCombAdjArgs A) {
    const long n = A.n;
    EMIX_FOR_CELLS(q, n) {
        const double j11 = A.jbn[10 * n + q];
        for (int m = 0; m < 5; ++m) {
            const double l = A.T5[m * n + q];
            A.lum0[m * n + q] += A.ca * l;
            if (A.lumc) A.lumc[m * n + q] = A.cb * l;
            A.lR[m * n + q] = A.cr * j11 * l;
        }
    }
}

// ---- fluxes -----------------------------------------------------------------
struct FluxAdjArgs {
    const double *lF;                 // 15 fields
    const double *umc, *u, *vis, *dvel, *jbn, *jx, *jy, *jz;
    double *lumc;                     // 5 fields, fields 1..4 accumulated
    double *lu, *lp, *ldvel, *lvis;   // stored
    long n;
};

__global__ void __launch_bounds__(256) k_adj_flux(FluxAdjArgs A) {
    const long n = A.n;
    EMIX_FOR_CELLS(q, n) {
        double lF[15], um[4], u[3], dv[9], lum[4] = {0, 0, 0, 0}, lu[3] = {0, 0, 0}, ldv[9];
        for (int c = 0; c < 15; ++c) lF[c] = A.lF[c * n + q];
        for (int c = 0; c < 4; ++c) um[c] = A.umc[(c + 1) * n + q];
        for (int c = 0; c < 3; ++c) u[c] = A.u[c * n + q];
        for (int c = 0; c < 9; ++c) dv[c] = A.dvel[c * n + q];
        double lp = 0.0, lvs = 0.0;
        flux_adj(um, u, A.vis[q], dv, A.jbn[q], A.jbn[4 * n + q], A.jbn[8 * n + q], A.jx[q], A.jy[q],
                 A.jz[q], lF, lum, lu, lp, ldv, lvs);
        for (int c = 0; c < 4; ++c) A.lumc[(c + 1) * n + q] += lum[c];
        for (int c = 0; c < 3; ++c) A.lu[c * n + q] = lu[c];
        A.lp[q] = lp;
        for (int c = 0; c < 9; ++c) A.ldvel[c * n + q] = ldv[c];
        A.lvis[q] = lvs;
    }
}

// ---- Smagorinsky ------------------------------------------------------------
struct SmagAdjArgs {
    const double *dvel, *jbn, *dxyz, *lvis;
    double cs;
    double *ldvel, *red;   // red[1]: d/d Cs
    long n;
};

__global__ void __launch_bounds__(256) k_adj_smag(SmagAdjArgs A) {
    const long n = A.n;
    double lcs = 0.0;
    for (long q0 = blockIdx.x * (long)blockDim.x; q0 < n; q0 += (long)gridDim.x * blockDim.x) {
        const long q = q0 + threadIdx.x;
        if (q < n) {
            // the targets loaded with the inputs, not after the arithmetic
            double dv[9], ldv[9], old[9];
            for (int c = 0; c < 9; ++c) {
                dv[c] = A.dvel[c * n + q];
                old[c] = A.ldvel[c * n + q];
                ldv[c] = 0.0;
            }
            lcs += smag_adj(dv, A.jbn[q], A.jbn[4 * n + q], A.jbn[8 * n + q], A.cs, A.dxyz[q], A.lvis[q],
                            ldv);
            for (int c = 0; c < 9; ++c)
                if (ldv[c] != 0.0) A.ldvel[c * n + q] = old[c] + ldv[c];
        }
    }
    block_sum_add(lcs, A.red + 1);
}

// dst += src over cnt values
__global__ void k_add_into(double *dst, const double *src, long cnt) {
    EMIX_FOR_CELLS(q, cnt) dst[q] += src[q];
}

// ---- primitive variables at the start of the step -----------------------------
__global__ void k_adj_prim(const double *um0, const double *lu, const double *lp, double inv_m2,
                           double *lum0, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double um[4] = {um0[q], um0[n + q], um0[2 * n + q], um0[3 * n + q]};
        const double l3[3] = {lu[q], lu[n + q], lu[2 * n + q]};
        double lum[4] = {0, 0, 0, 0};
        prim_adj(um, inv_m2, l3, lp[q], lum);
        for (int c = 0; c < 4; ++c) lum0[c * n + q] += lum[c];
    }
}

} // namespace emix
