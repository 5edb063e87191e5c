// boundary.cu -- wall boundary conditions, the CFL reduction and the grid
// metrics on the device.
//
//   frontera_z_val / frontera_y_val / frontera_x_val
//       src/MSVSingle/frontera_z.f90:219-262, frontera_y.f90:220-247,
//       frontera_x.f90:223-255 (applied in that order after each RK substep,
//       solver/rungek_ico.f90:98-100)
//   TSTEP / INITSTEP   src/MSVSingle/tstep_incomp.f90:1-174
//   JACOBEANO          solver/jacob_malla.f90:1-171
#include "boundary.cuh"
#include "deriv.cuh"

#include <cmath>

namespace emix {

int device_scratch(size_t bytes, double **out);

__global__ void k_bc(BcArgs a) {
    const long np = bc_count(a);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < np; q += (long)gridDim.x * blockDim.x)
        bc_cell(a, q);
}

namespace {

// inverse of the smaller neighbour spacing per axis (INITSTEP), and the CFL
// number of TSTEP: max_d dx_d^-1 (|u_d| + sqrt(cs^2 + u_d^2))
__global__ void k_cfl(const double *__restrict__ u, const double *__restrict__ xyz, double cs,
                      int nx, int ny, int nz, unsigned long long *__restrict__ out) {
    const long n = (long)nx * ny * nz;
    double m = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((long)nx * ny));
        const long st[3] = {1, nx, (long)nx * ny};
        const int idx[3] = {i, j, k}, dim[3] = {nx, ny, nz};
        for (int d = 0; d < 3; ++d) {
            const double *X = xyz + d * n;
            double h;
            if (idx[d] == 0) h = X[q + st[d]] - X[q];
            else if (idx[d] == dim[d] - 1) h = X[q] - X[q - st[d]];
            else h = fmin(X[q] - X[q - st[d]], X[q + st[d]] - X[q]);
            const double a = fabs(u[d * n + q]);
            const double c = (1.0 / h) * (a + sqrt(cs * cs + a * a));
            m = fmax(m, c);
        }
    }
    // non-negative doubles order like their bit patterns
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// det, 1/det and the inverse metric from the nine derivatives, in place
// (jacob_malla.f90:125-169); flags a vanishing Jacobian (|det| <= 1e-20)
__global__ void k_metric_invert(double *__restrict__ jbn, long n, int *__restrict__ bad) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        double j[10];
        for (int c = 1; c <= 9; ++c) j[c] = jbn[(c - 1) * n + q];
        const double det = j[1] * j[5] * j[9] - j[1] * j[6] * j[8] + j[2] * j[6] * j[7] -
                           j[2] * j[4] * j[9] + j[3] * j[4] * j[8] - j[3] * j[5] * j[7];
        if (fabs(det) <= 1.e-20) atomicExch(bad, 1);
        const double inv = 1. / det;
        const double t1 = j[5] * j[9] - j[6] * j[8], t4 = j[3] * j[8] - j[2] * j[9],
                     t7 = j[2] * j[6] - j[3] * j[5], t2 = j[6] * j[7] - j[4] * j[9],
                     t5 = j[1] * j[9] - j[3] * j[7], t8 = j[3] * j[4] - j[1] * j[6],
                     t3 = j[4] * j[8] - j[5] * j[7], t6 = j[2] * j[7] - j[1] * j[8],
                     t9 = j[1] * j[5] - j[2] * j[4];
        jbn[9 * n + q] = det;
        jbn[10 * n + q] = inv;
        jbn[q] = t1 * inv;
        jbn[n + q] = -t2 * inv;
        jbn[2 * n + q] = t3 * inv;
        jbn[3 * n + q] = -t4 * inv;
        jbn[4 * n + q] = t5 * inv;
        jbn[5 * n + q] = -t6 * inv;
        jbn[6 * n + q] = t7 * inv;
        jbn[7 * n + q] = -t8 * inv;
        jbn[8 * n + q] = t9 * inv;
    }
}

int grid1d(long n) { return grid_cap(n, 8); }

} // namespace

int launch_bc_walls(double *um1, int nx, int ny, int nz, cudaStream_t st) {
    for (int axis = 2; axis >= 0; --axis) {   // z, y, x as in rungek_ico.f90:98-100
        BcArgs a{um1, axis, nx, ny, nz, (long)nx * ny * nz};
        k_bc<<<grid1d(bc_count(a)), 256, 0, st>>>(a);
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

using namespace emix;

extern "C" {

int emix_bc_walls_dev(double *um, int nx, int ny, int nz, void *stream) {
    if (!um || nx < 5 || ny < 5 || nz < 5) return EMIX_ERR_ARG;
    return launch_bc_walls(um, nx, ny, nz, (cudaStream_t)stream);
}

int emix_cfl_dev(const double *u, const double *xyz, double mach, int nx, int ny, int nz,
                 double *cfla, void *stream) {
    if (!u || !xyz || !cfla || nx < 2 || ny < 2 || nz < 2 || !(mach > 0)) return EMIX_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    double *scr;
    int rc = device_scratch(sizeof(double), &scr);
    if (rc) return rc;
    EMIX_CUDA_TRY(cudaMemsetAsync(scr, 0, sizeof(double), st));
    const double cs = sqrt(1. / mach);   // src/MSVSingle/source_incomp.f90:11
    k_cfl<<<grid1d((long)nx * ny * nz), 256, 0, st>>>(u, xyz, cs, nx, ny, nz,
                                                      reinterpret_cast<unsigned long long *>(scr));
    EMIX_CUDA_TRY(cudaGetLastError());
    EMIX_CUDA_TRY(cudaMemcpyAsync(cfla, scr, sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    return EMIX_OK;
}

int emix_tstep_dt(double cfla, double olddt, double cfl, double *dt) {
    // dt = olddt/cflm*cfl with cflm = olddt*cfla, then the up/down smoothing
    // of TSTEP (tstep_incomp.f90:138-153; up = 0.5, down = 1.2 from INITSTEP)
    if (!dt || !(cfla > 0) || !(olddt > 0) || !(cfl > 0)) return EMIX_ERR_ARG;
    const double up = 0.5, down = 1.2;
    const double cflm = olddt * cfla;
    double d = olddt / cflm * cfl;
    const double diff = d - olddt;
    d = olddt + 0.5 * (up + down) * diff + 0.5 * (up - down) * fabs(diff);
    *dt = d;
    return EMIX_OK;
}

int emix_metrics_dev(const double *xyz, double *jbn, int scheme, double hx, double hy, double hz,
                     int nx, int ny, int nz, void *stream) {
    if (!xyz || !jbn || nx < 6 || ny < 6 || nz < 6 || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long n = (long)nx * ny * nz;
    const int dims[3] = {nx, ny, nz};
    const double h[3] = {hx, hy, hz};
    // d/dxi of x,y,z -> jbn(1),(4),(7); d/deta -> (2),(5),(8); d/dzeta -> (3),(6),(9)
    for (int ax = 0; ax < 3; ++ax) {
        DerivTable T;
        int rc = get_deriv_table(scheme, dims[ax], h[ax], &T);
        if (rc) return rc;
        const double *in[3] = {xyz, xyz + n, xyz + 2 * n};
        double *out[3] = {jbn + ax * n, jbn + (3 + ax) * n, jbn + (6 + ax) * n};
        rc = launch_deriv(T, ax, EPI_STORE, 3, in, out, out, nx, ny, nz, st);
        if (rc) return rc;
    }
    int *bad;
    double *scr;
    int rc = device_scratch(sizeof(double), &scr);
    if (rc) return rc;
    bad = reinterpret_cast<int *>(scr);
    EMIX_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
    k_metric_invert<<<grid1d(n), 256, 0, st>>>(jbn, n, bad);
    EMIX_CUDA_TRY(cudaGetLastError());
    int hbad = 0;
    EMIX_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    if (hbad) {
        set_last_message("emix_metrics_dev: vanishing Jacobian (|det| <= 1e-20), as JACOBEANO stops");
        return EMIX_ERR_ARG;
    }
    return EMIX_OK;
}

} // extern "C"
