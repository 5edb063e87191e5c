// weno.cu -- WENO5 level-set stage kernel, ghost padding and the
// cuAdvectLsJB-equivalent entry points.
#include "weno.cuh"

namespace emix {

int device_scratch(size_t bytes, double **out);

__global__ void k_weno_scales(const double *__restrict__ jbn, double *__restrict__ wce, double sx,
                              double sy, double sz, long n) {
    double2 *ce = reinterpret_cast<double2 *>(wce);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double c[3] = {jbn[q] * sx, jbn[4 * n + q] * sy, jbn[8 * n + q] * sz};
        for (int d = 0; d < 3; ++d) ce[d * n + q] = make_double2(c[d], kWenoEps4 / (c[d] * c[d]));
    }
}

__global__ void k_ghost_pad(PadArgs a) {
    const long end = a.qend > 0 ? a.qend : a.ng;
    for (long q = a.qbeg + blockIdx.x * (long)blockDim.x + threadIdx.x; q < end; q += (long)gridDim.x * blockDim.x)
        pad_cell(a, q);
}

__global__ void k_ghost_unpad(double *__restrict__ val, const double *__restrict__ ghost, int g,
                              int nx, int ny, int nz) {
    const int nxg = nx + 2 * g, nyg = ny + 2 * g;
    const long n = (long)nx * ny * nz;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nx);
        const int j = (int)((q / nx) % ny);
        const int k = (int)(q / ((long)nx * ny));
        val[q] = ghost[(i + g) + (long)nxg * ((j + g) + (long)nyg * (k + g))];
    }
}

int launch_weno_stage(const WenoArgs &a_in, cudaStream_t st, const CUtensorMap *tmap) {
    WenoArgs a = a_in;
    const int dims[3] = {a.nxg, a.nyg, a.nzg};
    for (int d = 0; d < 3; ++d) {
        if (a.rn[d] <= 0) { a.r0[d] = 0; a.rn[d] = dims[d]; }   // default: whole padded grid
        if (a.r0[d] < 0 || a.r0[d] + a.rn[d] > dims[d]) return EMIX_ERR_ARG;
    }
    return launch_weno_march(a, st, tmap);
}

namespace {
int pad_grid(long n) { return grid_cap(n, 8); }

int weno_advect_impl(double *phi, const double *vel, const double *jbn, double hx, double hy,
                     double hz, double dt, int nxg, int nyg, int nzg, int ref_bugs,
                     cudaStream_t st, double *scratch) {
    const long ng = (long)nxg * nyg * nzg;
    double *p1 = scratch, *p2 = scratch + ng;
    WenoArgs a{};
    a.vel = vel; a.jbn = jbn; a.reflect = 0; a.out_interior = 0;
    a.nxg = nxg; a.nyg = nyg; a.nzg = nzg; a.g = 0;
    a.sx = 1.0 / hx; a.sy = 1.0 / hy; a.sz = 1.0 / hz;
    a.dt = dt; a.ref_bugs = ref_bugs;
    a.phi = phi; a.phi0 = phi; a.out = p1; a.stage = 1;
    int rc = launch_weno_stage(a, st);
    if (rc) return rc;
    a.phi = p1; a.out = p2; a.stage = 2;
    rc = launch_weno_stage(a, st);
    if (rc) return rc;
    a.phi = p2; a.out = phi; a.stage = 3;
    return launch_weno_stage(a, st);
}

bool weno_dims_ok(int nxg, int nyg, int nzg) {
    // the stage kernel's grid: 16 x 16 columns, y tiles in gridDim.y
    return nxg >= 6 && nyg >= 6 && nzg >= 6 && (nyg + 15) / 16 <= 65535;
}
} // namespace

} // namespace emix

using namespace emix;

extern "C" {

int emix_weno5_advect_dev(double *phi, const double *vel, const double *jbn, double hx, double hy,
                          double hz, double dt, int nxg, int nyg, int nzg, int ref_bugs,
                          void *stream) {
    if (!phi || !vel || !jbn || !weno_dims_ok(nxg, nyg, nzg) || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    const long ng = (long)nxg * nyg * nzg;
    double *scr;
    int rc = device_scratch(2 * ng * sizeof(double), &scr);
    if (rc) return rc;
    return weno_advect_impl(phi, vel, jbn, hx, hy, hz, dt, nxg, nyg, nzg, ref_bugs,
                            (cudaStream_t)stream, scr);
}

int emix_weno5_advect(double *phi, const double *vel, const double *jbn, double hx, double hy,
                      double hz, double dt, int nxg, int nyg, int nzg, int ref_bugs) {
    if (!phi || !vel || !jbn || !weno_dims_ok(nxg, nyg, nzg) || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    const long ng = (long)nxg * nyg * nzg;
    // phi, vel (3), jbn (11), scratch (2)
    double *d = nullptr;
    if (cudaMalloc(&d, 17 * ng * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("cudaMalloc failed in emix_weno5_advect");
        return EMIX_ERR_ALLOC;
    }
    int rc = EMIX_OK;
    cudaError_t e = cudaMemcpy(d, phi, ng * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + ng, vel, 3 * ng * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + 4 * ng, jbn, 11 * ng * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        rc = weno_advect_impl(d, d + ng, d + 4 * ng, hx, hy, hz, dt, nxg, nyg, nzg, ref_bugs, 0,
                              d + 15 * ng);
        if (rc == EMIX_OK) e = cudaMemcpy(phi, d, ng * sizeof(double), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) {
        set_last_error(e, "emix_weno5_advect copy", __FILE__, __LINE__);
        rc = EMIX_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}

int emix_ghost_pad_dev(double *ghost, const double *val, int g, double direction, int nx, int ny,
                       int nz, void *stream) {
    if (!ghost || !val || g < 0 || g > nx || g > ny || g > nz || nx < 1 || ny < 1 || nz < 1)
        return EMIX_ERR_ARG;
    const long ng = (long)(nx + 2 * g) * (ny + 2 * g) * (nz + 2 * g);
    PadArgs pa{ghost, val, g, direction, nx, ny, nz, ng};
    k_ghost_pad<<<pad_grid(ng), 256, 0, (cudaStream_t)stream>>>(pa);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

int emix_ghost_unpad_dev(double *val, const double *ghost, int g, int nx, int ny, int nz,
                         void *stream) {
    if (!ghost || !val || g < 0 || nx < 1 || ny < 1 || nz < 1) return EMIX_ERR_ARG;
    k_ghost_unpad<<<pad_grid((long)nx * ny * nz), 256, 0, (cudaStream_t)stream>>>(val, ghost, g, nx,
                                                                                  ny, nz);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // extern "C"
