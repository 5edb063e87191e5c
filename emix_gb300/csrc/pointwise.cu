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

__global__ void __launch_bounds__(256, 2) k_flux_all(FluxArgs a) {
    const long n = a.n;
    EMIX_FOR_CELLS(q, n) {
        const double r = a.um[q];
        (void)r;
        const double um2 = a.um[n + q], um3 = a.um[2 * n + q], um4 = a.um[3 * n + q],
                     um5 = a.um[4 * n + q];
        const double u1 = a.u[q], u2 = a.u[n + q], u3 = a.u[2 * n + q];
        const double p = a.pres[q], vs = a.vis[q];
        const double j1 = a.jbn[q], j5 = a.jbn[4 * n + q], j9 = a.jbn[8 * n + q];
        const double *dv = a.dvel + q;
        const double JX = a.jx[q], JY = a.jy[q], JZ = a.jz[q];
        // strain pieces shared by the viscous fluxes of equations 2..4
        const double sxx = j1 * dv[0], syy = j5 * dv[4 * n], szz = j9 * dv[8 * n];
        const double sxy = j1 * dv[n] + j5 * dv[3 * n];        // p1+p2 of :68-70 and :102-104
        const double sxz = j1 * dv[2 * n] + j9 * dv[6 * n];    // :79-81 and :147-149
        const double syz = j9 * dv[7 * n] + j5 * dv[5 * n];    // :123-125 and :157-159
        const double vxy = vs * sxy, vxz = vs * sxz, vyz = vs * syz;
        // equation 1
        a.F[0][q] = JX * (-um2);
        a.F[1][q] = JY * (-um3);
        a.F[2][q] = JZ * (-um4);
        // equation 2
        a.F[3][q] = JX * ((-um2 * u1 - p) + vs * (2.0 * sxx));
        a.F[4][q] = JY * (-um3 * u1 + vxy);
        a.F[5][q] = JZ * (-um4 * u1 + vxz);
        // equation 3
        a.F[6][q] = JX * (-um2 * u2 + vxy);
        a.F[7][q] = JY * ((-um3 * u2 - p) + vs * (2.0 * syy));
        a.F[8][q] = JZ * (-um4 * u2 + vyz);
        // equation 4
        a.F[9][q] = JX * (-um2 * u3 + vxz);
        a.F[10][q] = JY * (-um3 * u3 + vyz);
        a.F[11][q] = JZ * ((-um4 * u3 - p) + vs * (2.0 * szz));
        // equation 5
        a.F[12][q] = JX * (-u1 * um5);
        a.F[13][q] = JY * (-u2 * um5);
        a.F[14][q] = JZ * (-u3 * um5);
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
        const double d = pow(fmax(dxm, dxp) * fmax(dym, dyp) * fmax(dzm, dzp), 1.0 / 3.0);
        dxyz[q] = d;
        ratios[q] = pow(d / dxp, 1.0 / 3.0);
        ratios[n + q] = pow(d / dxm, 1.0 / 3.0);
        ratios[2 * n + q] = pow(d / dyp, 1.0 / 3.0);
        ratios[3 * n + q] = pow(d / dym, 1.0 / 3.0);
        ratios[4 * n + q] = pow(d / dzp, 1.0 / 3.0);
        ratios[5 * n + q] = pow(d / dzm, 1.0 / 3.0);
    }
}

__global__ void k_sgs_smag(const double *__restrict__ dvel, const double *__restrict__ jbn,
                           const double *__restrict__ dxyz, double cs, double c4,
                           double *__restrict__ amut, double *__restrict__ vis, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double j1 = jbn[q], j5 = jbn[4 * n + q], j9 = jbn[8 * n + q];
        const double *dv = dvel + q;
        const double ux = j1 * dv[0], vx = j1 * dv[n], wx = j1 * dv[2 * n];
        const double uy = j5 * dv[3 * n], vy = j5 * dv[4 * n], wy = j5 * dv[5 * n];
        const double uz = j9 * dv[6 * n], vz = j9 * dv[7 * n], wz = j9 * dv[8 * n];
        const double s12 = 0.5 * (uy + vx), s13 = 0.5 * (uz + wx), s23 = 0.5 * (vz + wy);
        const double ss = ux * ux + vy * vy + wz * wz + 2.0 * (s12 * s12 + s13 * s13 + s23 * s23);
        const double cd = cs * dxyz[q];
        const double a = cd * cd * sqrt(2.0 * ss);
        if (amut) amut[q] = a;
        vis[q] = c4 * 1.0 + a;
    }
}

__global__ void k_sgs_sf(const double *__restrict__ u, const double *__restrict__ ratios,
                         const double *__restrict__ dxyz, double amu0,
                         double *__restrict__ amut, int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    const double *U = u, *V = u + n, *W = u + 2 * n;
    const long sy = nx, sz = (long)nx * ny;
    EMIX_FOR_CELLS(q, n) {
        const int i = (int)(q % nx);
        const int j = (int)((q / nx) % ny);
        const int k = (int)(q / sz);
        double a, b, c, s;
        long p, m;
        // the six one-sided increments in the order of f_structura
        p = i < nx - 1 ? q + 1 : q; m = i < nx - 1 ? q : q - 1;
        double r = ratios[q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = a * a + b * b + c * c;
        if (i > 0) { p = q - 1; m = q; } else { p = q + 1; m = q; }
        r = ratios[n + q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = s + a * a + b * b + c * c;
        if (j < ny - 1) { p = q + sy; m = q; } else { p = q; m = q - sy; }
        r = ratios[2 * n + q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = s + a * a + b * b + c * c;
        if (j > 0) { p = q - sy; m = q; } else { p = q; m = q + sy; }
        r = ratios[3 * n + q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = s + a * a + b * b + c * c;
        if (k < nz - 1) { p = q + sz; m = q; } else { p = q; m = q - sz; }
        r = ratios[4 * n + q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = s + a * a + b * b + c * c;
        if (k > 0) { p = q - sz; m = q; } else { p = q; m = q + sz; }
        r = ratios[5 * n + q];
        a = (U[p] - U[m]) * r; b = (V[p] - V[m]) * r; c = (W[p] - W[m]) * r;
        s = s + a * a + b * b + c * c;
        s = s * (1.0 / 6.0);
        amut[q] = amu0 * sqrt(s) * dxyz[q];
    }
}

__global__ void k_vort(const double *__restrict__ dvel, const double *__restrict__ jbn,
                       double *__restrict__ w, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double j1 = jbn[q], j5 = jbn[4 * n + q], j9 = jbn[8 * n + q];
        const double *dv = dvel + q;
        w[q] = j5 * dv[7 * n] - j9 * dv[5 * n];
        w[n + q] = j9 * dv[2 * n] - j1 * dv[6 * n];
        w[2 * n + q] = j1 * dv[3 * n] - j5 * dv[n];
    }
}

__global__ void k_selective(const double *__restrict__ w, double *__restrict__ amut,
                            double *__restrict__ vis, double cutoff, double c4,
                            int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    const double *wx = w, *wy = w + n, *wz = w + 2 * n;
    const long sy = nx, sz = (long)nx * ny;
    EMIX_FOR_CELLS(q, n) {
        const int i = (int)(q % nx);
        const int j = (int)((q / nx) % ny);
        const int k = (int)(q / sz);
        const long a1 = i < nx - 1 ? q + 1 : q, a2 = i > 0 ? q - 1 : q;
        const long a3 = k < nz - 1 ? q + sz : q, a4 = k > 0 ? q - sz : q;
        const long a5 = j < ny - 1 ? q + sy : q, a6 = j > 0 ? q - sy : q;
        const double wxn = wx[a1] + wx[a2] + wx[a3] + wx[a4] + wx[a5] + wx[a6];
        const double wyn = wy[a1] + wy[a2] + wy[a3] + wy[a4] + wy[a5] + wy[a6];
        const double wzn = wz[a1] + wz[a2] + wz[a3] + wz[a4] + wz[a5] + wz[a6];
        const double x = wx[q], y = wy[q], z = wz[q];
        double wn = x * x + y * y + z * z;
        wn = sqrt(wn * (wxn * wxn + wyn * wyn + wzn * wzn));
        const double s1 = (x * wxn + y * wyn + z * wzn) / wn;
        double a = amut[q];
        if (s1 > cutoff) a = 0.0;
        amut[q] = a;
        vis[q] = c4 * 1.0 + a;
    }
}

__global__ void k_prim(const double *__restrict__ um, double *__restrict__ u,
                       double *__restrict__ pres, double inv_m2, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double r = um[q];
        const double rr = 1.0 / r;
        pres[q] = r * inv_m2;
        u[q] = um[n + q] * rr;
        u[n + q] = um[2 * n + q] * rr;
        u[2 * n + q] = um[3 * n + q] * rr;
    }
}

__global__ void k_rk_post(RkArgs a) {
    const long n = a.n;
    const double dt = a.dt;
    EMIX_FOR_CELLS(q, n) {
        const double j11 = a.jbn[10 * n + q];
        double v[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const double rs = j11 * a.R[m * n + q];
            const double u0 = a.um0[m * n + q];
            if (a.stage == 1) {          // rungek_ico.f90:89-90
                v[m] = u0 + dt * rs;
            } else if (a.stage == 2) {   // :153-154
                v[m] = 0.75 * u0 + 0.25 * a.um[m * n + q] + (0.25 * dt) * rs;
            } else {                     // :217-220
                v[m] = (1.0 / 3.0) * u0 + (2.0 / 3.0) * a.um[m * n + q] + ((2.0 / 3.0) * dt) * rs;
            }
        }
        // varc_to_varnc + clip + mask + varc_to_varnc (:104-124)
        const double r = v[0];
        const double rr = 1.0 / r;
        const double mk = a.mask[q];
        double uu[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double x = v[d + 1] * rr;
            x = fmin(6.0, x);
            x = fmax(-6.0, x);
            const double mom = x * r * mk;
            uu[d] = mom * rr;
        }
        const double p = r * a.inv_m2;
        // rebuild after the level-set call site (:127-138)
        const double r1 = p * a.mach * a.mach;
        a.out[q] = r1;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a.out[(d + 1) * n + q] = uu[d] * r1;
            a.u[d * n + q] = uu[d];
        }
        a.out[4 * n + q] = v[4];
        a.pres[q] = p;
    }
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
        k_sgs_smag<<<cells_grid(n), 256, 0, st>>>(dvel, jbn, dxyzsgd,
                                                  model == EMIX_SGS_NONE ? 0.0 : coef, c4, amut, vis, n);
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
    k_sgs_sf<<<cells_grid(n), 256, 0, st>>>(u, ratios, dxyzsgd, coef, am, nx, ny, nz);
    k_vort<<<cells_grid(n), 256, 0, st>>>(dvel, jbn, w, n);
    const double cutoff = cos(20.0 * atan(1.0) / 45.0);   // sgdm_incomp.f90:18
    k_selective<<<cells_grid(n), 256, 0, st>>>(w, am, vis, cutoff, c4, nx, ny, nz);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // extern "C"
