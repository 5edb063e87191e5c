// extrapolate.cu -- the legacy advect_CUDA: pressure extrapolated into the
// solid object by the upwind extrapolation equation
//
//     d(ext)/dtau + S (grad phiS) . grad(ext) = 0,   S = [phiS > 0]
//
// advanced by 10 TVD-RK3 pseudo-steps of dtau = deltamin/2 on a grid padded
// with 5 mirrored ghost layers (src/LevelSet/lsTransportEc.cu:24-197,
// src/LevelSet/interface.cu:341-436, src/LevelSet/extrapol.cu:5-212).
//
// Kernels:
//   k_ext_setup   once per call: the direction field so*dphi of
//                 DevFirstOrder_LS (extrapol.cu:100-153) folded with the
//                 centre metric into one coefficient per axis, plus a byte of
//                 upwind directions.  Reads sobject and the metric at mirrored
//                 indices, so neither is padded in memory.
//   k_ext_stage   one TVD stage: the right-hand side of extrapolKernel
//                 (extrapol.cu:5-98) with the RunGK_*S combination
//                 (extrapol.cu:155-212) fused; ping-pongs between buffers so
//                 the stencil reads never meet a write.
//
// Boundary rules on the padded grid follow the reference: DevFirstOrder_LS
// takes factor 1 on every boundary cell, extrapolKernel's centre value id2 is
// the neighbour named by the last applicable of its six boundary rules.
// The reference's mirror kernels assume a cubic padded grid and its launch
// grids cover only multiples of (10, 10, 5) cells; this implementation
// mirrors and updates every cell for any size with nx, ny, nz >= 5.
#include "common.cuh"
#include "weno.cuh"

#include <cstdint>
#include <cstdio>

namespace emix {

int device_scratch(size_t bytes, double **out);

namespace {

constexpr int kExtG = 5;               // ghost layers (lsTransportEc.cu:37)
constexpr int kExtBX = 32, kExtBY = 8;  // stage kernel block

struct ExtSetupArgs {
    const double *sobject, *j0, *j4, *j8;   // unpadded, read at mirrored indices
    double sx, sy, sz;                       // 1/deltaX ... as the kernels receive them
    int nx, ny, nz, g, flag;
    double *coef;                            // 3 planes of ng
    uint8_t *dir;                            // 2 bits per axis: 1 downwind, 2 upwind
    long ng;
};

struct ExtStageArgs {
    const double *src;   // field the right-hand side is taken of
    const double *e0;    // field at the start of the pseudo-step
    const double *coef;
    const uint8_t *dir;
    double *out;
    int nxg, nyg, nzg;
    long ng;
    double dt;
    int stage;
};

__device__ __forceinline__ long mirror_index(int X, int Y, int Z, int g, int nx, int ny, int nz) {
    return mirror(X, g, nx) + (long)nx * (mirror(Y, g, ny) + (long)ny * mirror(Z, g, nz));
}

__global__ void k_ext_setup(ExtSetupArgs a) {
    const int g = a.g, nx = a.nx, ny = a.ny, nz = a.nz;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < a.ng; q += (long)gridDim.x * blockDim.x) {
        const int X = (int)(q % nxg), Y = (int)((q / nxg) % nyg), Z = (int)(q / ((long)nxg * nyg));
        // DevFirstOrder_LS neighbours and factor (extrapol.cu:130-139)
        int xm = X - 1, xp = X + 1, ym = Y - 1, yp = Y + 1, zm = Z - 1, zp = Z + 1;
        double factor = 0.5;
        if (X == 0) { xm = X; factor = 1.0; }
        if (Y == 0) { ym = Y; factor = 1.0; }
        if (Z == 0) { zm = Z; factor = 1.0; }
        if (X == nxg - 1) { xp = X; factor = 1.0; }
        if (Y == nyg - 1) { yp = Y; factor = 1.0; }
        if (Z == nzg - 1) { zp = Z; factor = 1.0; }
        const double *S = a.sobject;
        const long c = mirror_index(X, Y, Z, g, nx, ny, nz);
        const double s0 = S[c];
        const double J[3] = {a.j0[c], a.j4[c], a.j8[c]};
        const double sc[3] = {a.sx, a.sy, a.sz};
        const double dS[3] = {
            S[mirror_index(xp, Y, Z, g, nx, ny, nz)] - S[mirror_index(xm, Y, Z, g, nx, ny, nz)],
            S[mirror_index(X, yp, Z, g, nx, ny, nz)] - S[mirror_index(X, ym, Z, g, nx, ny, nz)],
            S[mirror_index(X, Y, zp, g, nx, ny, nz)] - S[mirror_index(X, Y, zm, g, nx, ny, nz)]};
        // side to extrapolate into (extrapol.cu:56-62)
        const double so = a.flag > 0 ? (double)(s0 > 0.0) : -1.0 * (double)(s0 <= 0.0);
        unsigned bits = 0;
        for (int d = 0; d < 3; ++d) {
            const double a_d = sc[d] * J[d];               // deltaX*jbn of the differences
            const double p_d = so * (factor * sc[d] * J[d] * dS[d]);
            a.coef[d * a.ng + q] = a_d * p_d;
            bits |= (p_d > 0.0 ? 1u : (p_d < 0.0 ? 2u : 0u)) << (2 * d);
        }
        a.dir[q] = (uint8_t)bits;
    }
}

__global__ void __launch_bounds__(kExtBX *kExtBY) k_ext_stage(ExtStageArgs a) {
    const int X = blockIdx.x * kExtBX + threadIdx.x;
    const int Y = blockIdx.y * kExtBY + threadIdx.y;
    const int Z = blockIdx.z;
    if (X >= a.nxg || Y >= a.nyg) return;
    const long sxy = (long)a.nxg * a.nyg;
    const long id = X + (long)a.nxg * Y + sxy * Z;
    // extrapolKernel neighbours and centre id2 (extrapol.cu:45-52)
    long ip = id + 1, im = id - 1, jp = id + a.nxg, jm = id - a.nxg, kp = id + sxy, km = id - sxy;
    long id2 = id;
    if (X == 0) { id2 = ip; im = id; }
    if (Y == 0) { id2 = jp; jm = id; }
    if (Z == 0) { id2 = kp; km = id; }
    if (X == a.nxg - 1) { id2 = im; ip = id; }
    if (Y == a.nyg - 1) { id2 = jm; jp = id; }
    if (Z == a.nzg - 1) { id2 = km; kp = id; }
    const unsigned bits = a.dir[id];
    const double *E = a.src;
    const double ec = E[id2];
    double r = 0.0;
    if (bits & 3u) r = a.coef[id] * ((bits & 1u) ? ec - E[im] : E[ip] - ec);
    if ((bits >> 2) & 3u) r += a.coef[a.ng + id] * (((bits >> 2) & 1u) ? ec - E[jm] : E[jp] - ec);
    if ((bits >> 4) & 3u) r += a.coef[2 * a.ng + id] * (((bits >> 4) & 1u) ? ec - E[km] : E[kp] - ec);
    const double e0 = a.e0[id];
    double o;
    if (a.stage == 1) o = e0 - a.dt * r;
    else if (a.stage == 2) o = 0.75 * e0 + 0.25 * (E[id] - a.dt * r);
    else o = (e0 + 2.0 * (E[id] - a.dt * r)) / 3.0;
    a.out[id] = o;
}

int grid1(long n) { return grid_cap(n, 16); }

} // namespace

// ext (unpadded, in/out) extrapolated across phiS > 0 (flag > 0) or phiS <= 0
// (flag <= 0) by `iters` TVD-RK3 pseudo-steps of dtext on the grid padded with
// kExtG mirrored layers; jbn holds the 11 metric components (1, 5, 9 read).
int extrapolate_impl(double *ext, const double *phiS, const double *jbn, double deltaX,
                     double deltaY, double deltaZ, int nx, int ny, int nz, double dtext, int flag,
                     int iters, cudaStream_t st) {
    const int g = kExtG;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    const long n = (long)nx * ny * nz, ng = (long)nxg * nyg * nzg;
    double *scr;
    // E, A, B, 3 coefficient planes, direction bytes
    const size_t bytes = (size_t)6 * ng * sizeof(double) + (size_t)ng + 256;
    int rc = device_scratch(bytes, &scr);
    if (rc) return rc;
    double *E = scr, *A = scr + ng, *B = scr + 2 * ng, *coef = scr + 3 * ng;
    uint8_t *dir = reinterpret_cast<uint8_t *>(scr + 6 * ng);

    PadArgs pa{E, ext, g, 1.0, nx, ny, nz, ng};
    k_ghost_pad<<<grid1(ng), 256, 0, st>>>(pa);
    ExtSetupArgs sa{phiS, jbn, jbn + 4 * n, jbn + 8 * n, 1.0 / deltaX, 1.0 / deltaY, 1.0 / deltaZ,
                    nx, ny, nz, g, flag, coef, dir, ng};
    k_ext_setup<<<grid1(ng), 256, 0, st>>>(sa);
    const dim3 blk(kExtBX, kExtBY), grd((nxg + kExtBX - 1) / kExtBX, (nyg + kExtBY - 1) / kExtBY, nzg);
    for (int it = 0; it < iters; ++it) {
        ExtStageArgs s1{E, E, coef, dir, A, nxg, nyg, nzg, ng, dtext, 1};
        k_ext_stage<<<grd, blk, 0, st>>>(s1);
        ExtStageArgs s2{A, E, coef, dir, B, nxg, nyg, nzg, ng, dtext, 2};
        k_ext_stage<<<grd, blk, 0, st>>>(s2);
        ExtStageArgs s3{B, E, coef, dir, E, nxg, nyg, nzg, ng, dtext, 3};
        k_ext_stage<<<grd, blk, 0, st>>>(s3);
    }
    k_ghost_unpad<<<grid1(n), 256, 0, st>>>(ext, E, g, nx, ny, nz);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

using namespace emix;

namespace {

bool ext_args_ok(const void *p, const void *j, const void *s, double dx, double dy, double dz,
                 int nx, int ny, int nz) {
    return p && j && s && nx >= kExtG && ny >= kExtG && nz >= kExtG && dx > 0 && dy > 0 && dz > 0;
}

} // namespace

extern "C" {

int emix_extrapolate_dev(double *ext, const double *phiS, const double *jbn, double deltaX,
                         double deltaY, double deltaZ, int nx, int ny, int nz, double dtext,
                         int flag, int iters, void *stream) {
    if (!ext_args_ok(ext, jbn, phiS, deltaX, deltaY, deltaZ, nx, ny, nz) || iters < 0 || !(dtext >= 0))
        return EMIX_ERR_ARG;
    return extrapolate_impl(ext, phiS, jbn, deltaX, deltaY, deltaZ, nx, ny, nz, dtext, flag, iters,
                            (cudaStream_t)stream);
}

int emix_advect_extrapolate_dev(double *press, const double *jbn, const double *sobject,
                                double deltaX, double deltaY, double deltaZ, int nx, int ny, int nz,
                                double deltamin, void *stream) {
    if (!ext_args_ok(press, jbn, sobject, deltaX, deltaY, deltaZ, nx, ny, nz) || !(deltamin >= 0))
        return EMIX_ERR_ARG;
    // dtext = deltamin*0.5, Flag = 1, 10 pseudo-steps (lsTransportEc.cu:161-162,
    // interface.cu:386)
    return extrapolate_impl(press, sobject, jbn, deltaX, deltaY, deltaZ, nx, ny, nz, deltamin * 0.5, 1,
                            10, (cudaStream_t)stream);
}

int emix_advect_extrapolate(double *press, const double *jbn, const double *sobject, double deltaX,
                            double deltaY, double deltaZ, int nx, int ny, int nz, double deltamin) {
    if (!ext_args_ok(press, jbn, sobject, deltaX, deltaY, deltaZ, nx, ny, nz) || !(deltamin >= 0))
        return EMIX_ERR_ARG;
    const size_t n = (size_t)nx * ny * nz;
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 13 * n * sizeof(double));
    if (e != cudaSuccess) {
        set_last_error(e, "emix_advect_extrapolate cudaMalloc", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    double *dp = d, *dj = d + n, *ds = d + 12 * n;
    int rc = EMIX_OK;
    e = cudaMemcpy(dp, press, n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dj, jbn, 11 * n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ds, sobject, n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        rc = emix_advect_extrapolate_dev(dp, dj, ds, deltaX, deltaY, deltaZ, nx, ny, nz, deltamin, nullptr);
        if (rc == EMIX_OK) e = cudaMemcpy(press, dp, n * sizeof(double), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) {
        set_last_error(e, "emix_advect_extrapolate", __FILE__, __LINE__);
        rc = EMIX_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}

// The reference's symbol (src/LevelSet/lsTransportEc.cu:24-35, Fortran
// interface include/LevelSet/interfaceAdvect.h:3-16): host buffers in and
// out, synchronous, on the current device (the reference forces device 1).
// Errors are printed and the call returns; it never exits the process.
void advect_CUDA(double *press, double *jbn, double *sobject, double deltaX, double deltaY,
                 double deltaZ, int Nx, int Ny, int Nz, double deltamin) {
    int rc = emix_advect_extrapolate(press, jbn, sobject, deltaX, deltaY, deltaZ, Nx, Ny, Nz, deltamin);
    if (rc != EMIX_OK) fprintf(stderr, "advect_CUDA: error %d: %s\n", rc, emix_last_error());
}

} // extern "C"
