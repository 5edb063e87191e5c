// pointwise.cu -- cell-local kernels (fluxes, SGS viscosity, RK update) and
// their status-returning entry points.
#include "pointwise.cuh"

#include <cmath>

namespace emix {

int device_scratch(size_t bytes, double **out);

__global__ void k_flux_one(int neq, double *__restrict__ e, double *__restrict__ f,
                           double *__restrict__ g, double *__restrict__ ev,
                           double *__restrict__ fv, double *__restrict__ gv,
                           const double *__restrict__ um, const double *__restrict__ u,
                           const double *__restrict__ pres, const double *__restrict__ dvel,
                           const double *__restrict__ jbn, const double *__restrict__ vis, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double um2 = um[n + q], um3 = um[2 * n + q], um4 = um[3 * n + q];
        const double j1 = jbn[q], j5 = jbn[4 * n + q], j9 = jbn[8 * n + q];
        const double *dv = dvel + q;
        double p1, p2;
        switch (neq) {
        case 1:  // flujos_compact.f90:21-40
            e[q] = -um2; f[q] = -um3; g[q] = -um4;
            ev[q] = 0.0; fv[q] = 0.0; gv[q] = 0.0;
            break;
        case 2: {  // :43-84
            const double u1 = u[q], p = pres[q], vs = vis[q];
            e[q] = -um2 * u1 - p; f[q] = -um3 * u1; g[q] = -um4 * u1;
            ev[q] = vs * (2.0 * (j1 * dv[0]));
            p1 = j1 * dv[n]; p2 = j5 * dv[3 * n];
            fv[q] = vs * (p1 + p2);
            p1 = j1 * dv[2 * n]; p2 = j9 * dv[6 * n];
            gv[q] = vs * (p1 + p2);
            break;
        }
        case 3: {  // :88-128
            const double u2 = u[n + q], p = pres[q], vs = vis[q];
            e[q] = -um2 * u2; f[q] = -um3 * u2 - p; g[q] = -um4 * u2;
            p1 = j1 * dv[n]; p2 = j5 * dv[3 * n];
            ev[q] = vs * (p1 + p2);
            fv[q] = vs * (2.0 * (j5 * dv[4 * n]));
            p1 = j9 * dv[7 * n]; p2 = j5 * dv[5 * n];
            gv[q] = vs * (p1 + p2);
            break;
        }
        case 4: {  // :133-173
            const double u3 = u[2 * n + q], p = pres[q], vs = vis[q];
            e[q] = -um2 * u3; f[q] = -um3 * u3; g[q] = -um4 * u3 - p;
            p1 = j1 * dv[2 * n]; p2 = j9 * dv[6 * n];
            ev[q] = vs * (p1 + p2);
            p1 = j9 * dv[7 * n]; p2 = j5 * dv[5 * n];
            fv[q] = vs * (p1 + p2);
            gv[q] = vs * (2.0 * (j9 * dv[8 * n]));
            break;
        }
        default: {  // :176-214
            const double um5 = um[4 * n + q];
            e[q] = -u[q] * um5; f[q] = -u[n + q] * um5; g[q] = -u[2 * n + q] * um5;
            ev[q] = 0.0; fv[q] = 0.0; gv[q] = 0.0;
            break;
        }
        }
    }
}

__global__ void k_sgs_setup(const double *__restrict__ xyz, double *__restrict__ dxyz,
                            double *__restrict__ ratios, int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    const double *X = xyz, *Y = xyz + n, *Z = xyz + 2 * n;
    EMIX_FOR_CELLS(q, n) {
        const int i = (int)(q % nx);
        const int j = (int)((q / nx) % ny);
        const int k = (int)(q / ((long)nx * ny));
        const long sy = nx, sz = (long)nx * ny;
        double dxm, dxp, dym, dyp, dzm, dzp;
        if (i > 0 && i < nx - 1) { dxm = X[q] - X[q - 1]; dxp = X[q + 1] - X[q]; }
        else if (i == 0) { dxp = X[q + 1] - X[q]; dxm = dxp; }
        else { dxm = X[q] - X[q - 1]; dxp = dxm; }
        if (j > 0 && j < ny - 1) { dym = Y[q] - Y[q - sy]; dyp = Y[q + sy] - Y[q]; }
        else if (j == 0) { dyp = Y[q + sy] - Y[q]; dym = dyp; }
        else { dym = Y[q] - Y[q - sy]; dyp = dym; }
        if (k > 0 && k < nz - 1) { dzm = Z[q] - Z[q - sz]; dzp = Z[q + sz] - Z[q]; }
        else if (k == 0) { dzp = Z[q + sz] - Z[q]; dzm = dzp; }
        else { dzm = Z[q] - Z[q - sz]; dzp = dzm; }
        // the reference's **(1/3) (sgdm_incomp.f90:89,97-108) as cube roots
        const double d = cbrt(fmax(dxm, dxp) * fmax(dym, dyp) * fmax(dzm, dzp));
        dxyz[q] = d;
        ratios[q] = cbrt(d / dxp);
        ratios[n + q] = cbrt(d / dxm);
        ratios[2 * n + q] = cbrt(d / dyp);
        ratios[3 * n + q] = cbrt(d / dym);
        ratios[4 * n + q] = cbrt(d / dzp);
        ratios[5 * n + q] = cbrt(d / dzm);
    }
}

__global__ void k_prim(PrimArgs a) {
    const long end = a.qend > 0 ? a.qend : a.n;
    for (long q = a.qbeg + blockIdx.x * (long)blockDim.x + threadIdx.x; q < end; q += (long)gridDim.x * blockDim.x)
        prim_cell(a, q);
}
__global__ void __launch_bounds__(256, 2) k_flux_all(FluxArgs a) { EMIX_FOR_CELLS(q, a.n) flux_cell(a, q); }
__global__ void k_sgs_smag(SmagArgs a) { EMIX_FOR_CELLS(q, a.n) smag_cell(a, q); }
__global__ void __launch_bounds__(256, 2) k_smag_flux(SmagArgs s, FluxArgs f) {
    EMIX_FOR_CELLS(q, f.n) smag_flux_cell(s, f, q);
}
__global__ void k_sgs_sf(SfArgs a) { EMIX_FOR_CELLS(q, a.n) sf_cell(a, q); }
__global__ void k_vort(VortArgs a) { EMIX_FOR_CELLS(q, a.n) vort_cell(a, q); }
__global__ void k_selective(SelArgs a) { EMIX_FOR_CELLS(q, a.n) select_cell(a, q); }
__global__ void k_rk_post(RkArgs a) {
    const long end = a.qend > 0 ? a.qend : rk_count(a);
    for (long q = a.qbeg + blockIdx.x * (long)blockDim.x + threadIdx.x; q < end; q += (long)gridDim.x * blockDim.x)
        rk_cell(a, q);
}

} // namespace emix

using namespace emix;

extern "C" {

int emix_flux_dev(int neq, double *e, double *f, double *g, double *ev, double *fv, double *gv,
                  const double *um, const double *u, const double *pres, const double *dvel,
                  const double *jbn, const double *vis, int nx, int ny, int nz, void *stream) {
    if (neq < 1 || neq > 5 || !e || !f || !g || !ev || !fv || !gv || !um || !u || !pres || !dvel ||
        !jbn || !vis || nx < 1 || ny < 1 || nz < 1)
        return EMIX_ERR_ARG;
    const long n = (long)ncell(nx, ny, nz);
    k_flux_one<<<cells_grid(n), 256, 0, (cudaStream_t)stream>>>(neq, e, f, g, ev, fv, gv, um, u, pres,
                                                                dvel, jbn, vis, n);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

int emix_sgs_setup_dev(const double *xyz, double *dxyzsgd, double *ratios, int nx, int ny, int nz,
                       void *stream) {
    if (!xyz || !dxyzsgd || !ratios || nx < 2 || ny < 2 || nz < 2) return EMIX_ERR_ARG;
    k_sgs_setup<<<cells_grid((long)ncell(nx, ny, nz)), 256, 0, (cudaStream_t)stream>>>(
        xyz, dxyzsgd, ratios, nx, ny, nz);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

int emix_sgs_viscosity_dev(int model, double coef, double c4, const double *u, const double *dvel,
                           const double *jbn, const double *dxyzsgd, const double *ratios,
                           double *amut, double *vis, int nx, int ny, int nz, void *stream) {
    if (!dvel || !jbn || !dxyzsgd || !vis || nx < 2 || ny < 2 || nz < 2) return EMIX_ERR_ARG;
    const long n = (long)ncell(nx, ny, nz);
    cudaStream_t st = (cudaStream_t)stream;
    if (model == EMIX_SGS_NONE || model == EMIX_SGS_SMAGORINSKY) {
        SmagArgs sa{dvel, jbn, dxyzsgd, model == EMIX_SGS_NONE ? 0.0 : coef, c4, amut, vis, n};
        k_sgs_smag<<<cells_grid(n), 256, 0, st>>>(sa);
        EMIX_CUDA_TRY(cudaGetLastError());
        return EMIX_OK;
    }
    if (model != EMIX_SGS_STRUCTURE || !u || !ratios) return EMIX_ERR_ARG;
    double *scr;
    const size_t need = (size_t)(amut ? 3 : 4) * n * sizeof(double);
    int rc = device_scratch(need, &scr);
    if (rc) return rc;
    double *w = scr;
    double *am = amut ? amut : scr + 3 * n;
    SfArgs fa{u, ratios, dxyzsgd, coef, am, nx, ny, nz, n};
    VortArgs va{dvel, jbn, w, n};
    const double cutoff = cos(20.0 * atan(1.0) / 45.0);   // sgdm_incomp.f90:18
    SelArgs la{w, am, vis, cutoff, c4, nx, ny, nz, n};
    k_sgs_sf<<<cells_grid(n), 256, 0, st>>>(fa);
    k_vort<<<cells_grid(n), 256, 0, st>>>(va);
    k_selective<<<cells_grid(n), 256, 0, st>>>(la);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // extern "C"
