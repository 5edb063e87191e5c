/*
 * oracle.cpp -- CPU restatement of the eMix3d per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA kernels and the timed
 * CPU baseline.  Nothing in the product library links or calls this file.
 *
 * Each function follows the reference (jramirezcr/eMix3d) file:line named in
 * its comment, in the same arithmetic order.  OpenMP only splits independent
 * pencils / planes, so results do not depend on the thread count.
 *
 * Parity pinning: the reference ships no tests, golden vectors or fixtures
 * and its Fortran CPU path cannot be compiled here.  Scheme C, cuDivergence,
 * the WENO5 step and the ghost padding are pinned against outputs of the
 * reference's own CUDA kernels (tests/golden/reference_cuda.npz); the
 * Fortran-only parts are pinned by analytic known-answer tests only (parity
 * unpinned against the reference for those).
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline size_t lin(int i, int j, int k, int nx, int ny) {
    return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k);
}

/* Thomas solve as written in derivnper (solver/derivada.f90:111-122,
 * src/MSVSingle/derivada_incomp.f90:315-326) and cuDerivCS
 * (src/Schemes/derivCompact.cu:199-212).  Arrays are 0-based here. */
void thomas(int n, const double *a, const double *b, const double *c,
            const double *r, double *u, double *gam) {
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int l = 1; l < n; ++l) {
        gam[l] = c[l - 1] / bet;
        bet = b[l] - a[l] * gam[l];
        u[l] = (r[l] - a[l] * u[l - 1]) / bet;
    }
    for (int l = n - 2; l >= 0; --l) u[l] = u[l] - gam[l + 1] * u[l + 1];
}

/* Variant A: inideriv + derivnper, solver/derivada.f90:2-93,95-125.
 * delta multiplies the stencil (the Fortran passes deltax = nx-1 = 1/h). */
void deriv_A(int n, double *u, double delta, double *r, double *gam,
             double *a, double *b, double *c) {
    const double ars = 3. / 4., ars1 = -17. / 6., brs1 = 3. / 2., crs1 = 1.5;
    for (int l = 0; l < n; ++l) { b[l] = 1.0; a[l] = 1. / 4.; c[l] = 1. / 4.; }
    a[0] = 0.0; a[n - 1] = 3.0;
    c[0] = 3.0; c[n - 1] = 0.0;
    for (int l = 1; l < n - 1; ++l) r[l] = delta * (ars * (u[l + 1] - u[l - 1]));
    r[0] = delta * (ars1 * u[0] + brs1 * u[1] + crs1 * u[2] - 1. / 6. * u[3]);
    r[n - 1] = delta * (-ars1 * u[n - 1] - brs1 * u[n - 2] - crs1 * u[n - 3] + 1. / 6. * u[n - 4]);
    thomas(n, a, b, c, r, u, gam);
}

/* Variant B coefficients: src/MSVSingle/derivada_incomp.f90:130-218. */
void coef_B(int n, double *a, double *b, double *c) {
    for (int l = 0; l < n; ++l) b[l] = 1.0;
    a[0] = 0.0; a[1] = 0.25; a[n - 2] = 0.25; a[n - 1] = 2.0;
    for (int l = 2; l < n - 2; ++l) a[l] = 1.0 / 3.0;
    c[0] = 2.0; c[1] = 0.25; c[n - 2] = 0.25; c[n - 1] = 0.0;
    for (int l = 2; l < n - 2; ++l) c[l] = 1.0 / 3.0;
}

/* Variant B non-periodic: derivnper, src/MSVSingle/derivada_incomp.f90:297-329. */
void deriv_B(int n, double *u, double delta, double *r, double *gam,
             double *a, double *b, double *c) {
    const double ars = 7. / 9., brs = 1. / 36., ars1 = -2.5, brs1 = 2., crs1 = 0.5, ars2 = 0.75;
    coef_B(n, a, b, c);
    for (int l = 2; l < n - 2; ++l)
        r[l] = delta * (ars * (u[l + 1] - u[l - 1]) + brs * (u[l + 2] - u[l - 2]));
    r[0] = delta * (ars1 * u[0] + brs1 * u[1] + crs1 * u[2]);
    r[n - 1] = delta * (-ars1 * u[n - 1] - brs1 * u[n - 2] - crs1 * u[n - 3]);
    r[1] = delta * (ars2 * (u[2] - u[0]));
    r[n - 2] = delta * (ars2 * (u[n - 1] - u[n - 3]));
    thomas(n, a, b, c, r, u, gam);
}

/* Variant B periodic: derivper (cyclic, Sherman-Morrison),
 * src/MSVSingle/derivada_incomp.f90:221-294, coefficients :192-206. */
void deriv_Bper(int n, double *u, double delta, double *r, double *gam,
                double *a, double *b, double *c, double *bb, double *x, double *z) {
    const double ars = 7. / 9., brs = 1. / 36.;
    for (int l = 0; l < n; ++l) { b[l] = 1.0; a[l] = 1.0 / 3.0; c[l] = 1.0 / 3.0; }
    for (int l = 2; l < n - 2; ++l)
        r[l] = delta * (ars * (u[l + 1] - u[l - 1]) + brs * (u[l + 2] - u[l - 2]));
    r[0] = delta * (ars * (u[1] - u[n - 1]) + brs * (u[2] - u[n - 2]));
    r[n - 1] = delta * (ars * (u[0] - u[n - 2]) + brs * (u[1] - u[n - 3]));
    r[1] = delta * (ars * (u[2] - u[0]) + brs * (u[3] - u[n - 1]));
    r[n - 2] = delta * (ars * (u[n - 1] - u[n - 3]) + brs * (u[0] - u[n - 4]));
    const double alpha = a[0], beta = c[n - 1], gamma = -b[0];
    bb[0] = b[0] - gamma;
    bb[n - 1] = b[n - 1] - alpha * beta / gamma;
    for (int l = 1; l < n - 1; ++l) bb[l] = b[l];
    thomas(n, a, bb, c, r, x, gam);
    for (int l = 0; l < n; ++l) u[l] = 0.0;
    u[0] = gamma;
    u[n - 1] = alpha;
    thomas(n, a, bb, c, u, z, gam);
    const double fact = (x[0] + beta * x[n - 1] / gamma) / (1. + z[0] + beta * z[n - 1] / gamma);
    for (int l = 0; l < n; ++l) u[l] = x[l] - fact * z[l];
}

/* Variant C: getC6RHS + cuDerivCS, src/Schemes/derivCompact.cu:81-215.
 * The kernel is passed delta = h and scales by (1.0/delta). */
void deriv_C(int n, double *f, double delta, double *r, double *gam,
             double *a, double *b, double *c) {
    const double ars = 14.0 / (9.0 * 2.0), brs = 1.0 / (9.0 * 4.0),
                 ars1 = -17.0 / 6.0, brs1 = 3.0 / 2.0, crs1 = 3.0 / 2.0, drs1 = -1.0 / 6.0,
                 ars2 = -3.0 / 4.0, brs2 = 0.0, crs2 = 3.0 / 4.0, drs2 = 0.0;
    const double s = 1.0 / delta;
    for (int i = 2; i < n - 2; ++i)
        r[i] = s * (ars * (f[i + 1] - f[i - 1]) + (brs * (f[i + 2] - f[i - 2])));
    r[0] = s * (ars1 * f[0] + brs1 * f[1] + crs1 * f[2] + drs1 * f[3]);
    r[1] = s * (ars2 * f[0] + brs2 * f[1] + crs2 * f[2] + drs2 * f[3]);
    r[n - 1] = s * (-ars1 * f[n - 1] - brs1 * f[n - 2] - crs1 * f[n - 3] - drs1 * f[n - 4]);
    r[n - 2] = s * (-ars2 * f[n - 1] - brs2 * f[n - 2] - crs2 * f[n - 3] - drs2 * f[n - 4]);
    /* diagonals as staged in shared memory, derivCompact.cu:162-190 */
    for (int i = 0; i < n; ++i) { a[i] = 1.0 / 3.0; b[i] = 1.0; c[i] = 1.0 / 3.0; }
    a[0] = 0.0; a[1] = 1.0 / 4.0; a[n - 1] = 3.0; a[n - 2] = 1.0 / 4.0;
    c[0] = 3.0; c[1] = 1.0 / 4.0; c[n - 1] = 0.0; c[n - 2] = 1.0 / 4.0;
    thomas(n, a, b, c, r, f, gam);
}

struct Work {
    std::vector<double> buf;
    double *r, *gam, *a, *b, *c, *bb, *x, *z, *p;
    explicit Work(int n) : buf((size_t)9 * n) {
        double *q = buf.data();
        r = q; gam = q + n; a = q + 2 * n; b = q + 3 * n; c = q + 4 * n;
        bb = q + 5 * n; x = q + 6 * n; z = q + 7 * n; p = q + 8 * n;
    }
};

/* One pencil in place; h is the computational spacing. */
void pencil(int scheme, int n, double *u, double h, Work &w) {
    switch (scheme) {
    case ORC_SCHEME_A: deriv_A(n, u, 1.0 / h, w.r, w.gam, w.a, w.b, w.c); break;
    case ORC_SCHEME_B: deriv_B(n, u, 1.0 / h, w.r, w.gam, w.a, w.b, w.c); break;
    case ORC_SCHEME_BPER: deriv_Bper(n, u, 1.0 / h, w.r, w.gam, w.a, w.b, w.c, w.bb, w.x, w.z); break;
    default: deriv_C(n, u, h, w.r, w.gam, w.a, w.b, w.c); break;
    }
}

bool scheme_ok(int s) { return s >= ORC_SCHEME_A && s <= ORC_SCHEME_C; }

/* --- WENO5 pieces, src/LevelSet/lsTools.cu ------------------------------ */

/* Dev1thO_Downwind, lsTools.cu:53-95: backward differences times 1/h; at
 * index 0 the difference phi(1)-phi(0) is used. */
void dev1_downwind(double *dphi, const double *phi, double sx, double sy, double sz,
                   int nx, int ny, int nz) {
    const size_t off = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t id = lin(i, j, k, nx, ny);
                size_t im = id - 1, jm = id - nx, km = id - (size_t)nx * ny;
                size_t ix = id, iy = id, iz = id;
                if (i == 0) { im = id; ix = lin(1, j, k, nx, ny); }
                if (j == 0) { jm = id; iy = lin(i, 1, k, nx, ny); }
                if (k == 0) { km = id; iz = lin(i, j, 1, nx, ny); }
                dphi[id] = sx * (phi[ix] - phi[im]);
                dphi[off + id] = sy * (phi[iy] - phi[jm]);
                dphi[2 * off + id] = sz * (phi[iz] - phi[km]);
            }
}

/* PhiDevPlusParameterJB, lsTools.cu:587-673 (left-biased, phi^-).  With
 * ref_bugs the z-top neighbour id_kp2 = id_jm1 of lsTools.cu:636 is kept;
 * otherwise id_kp2 = id_km1, mirroring the x and y branches. */
void weno_plus(double *out, const double *dphi, const double *jbn,
               int nx, int ny, int nz, int ref_bugs) {
    const size_t off = (size_t)nx * ny * nz;
    const long NX = nx, NXY = (long)nx * ny;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long id = (long)lin(i, j, k, nx, ny);
                long im1 = id - 1, ip1 = id + 1, jm1 = id - NX, jp1 = id + NX,
                     km1 = id - NXY, kp1 = id + NXY, im2 = id - 2, ip2 = id + 2,
                     jm2 = id - 2 * NX, jp2 = id + 2 * NX, km2 = id - 2 * NXY, kp2 = id + 2 * NXY;
                if (i == 0) { im1 = id; im2 = ip1; }
                if (i == 1) { im2 = im1; }
                if (i == nx - 1) { ip1 = id; ip2 = im1; }
                if (i == nx - 2) { ip2 = ip1; }
                if (j == 0) { jm1 = id; jm2 = jp1; }
                if (j == 1) { jm2 = jm1; }
                if (j == ny - 1) { jp1 = id; jp2 = jm1; }
                if (j == ny - 2) { jp2 = jp1; }
                if (k == 0) { km1 = id; km2 = kp1; }
                if (k == 1) { km2 = km1; }
                if (k == nz - 1) { kp1 = id; kp2 = ref_bugs ? jm1 : km1; }
                if (k == nz - 2) { kp2 = kp1; }
                double jx = jbn[id], jy = jbn[id + 4 * off], jz = jbn[id + 8 * off];
                const double *dx = dphi, *dy = dphi + off, *dz = dphi + 2 * off;
                out[id] = orc_phi_x_weno(dx[im2] * jx, dx[im1] * jx, dx[id] * jx, dx[ip1] * jx, dx[ip2] * jx);
                out[id + off] = orc_phi_x_weno(dy[jm2] * jy, dy[jm1] * jy, dy[id] * jy, dy[jp1] * jy, dy[jp2] * jy);
                out[id + 2 * off] = orc_phi_x_weno(dz[km2] * jz, dz[km1] * jz, dz[id] * jz, dz[kp1] * jz, dz[kp2] * jz);
            }
}

/* PhiDevMinusParameterJB, lsTools.cu:676-770 (right-biased, phi^+). */
void weno_minus(double *out, const double *dphi, const double *jbn,
                int nx, int ny, int nz) {
    const size_t off = (size_t)nx * ny * nz;
    const long NX = nx, NXY = (long)nx * ny;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long id = (long)lin(i, j, k, nx, ny);
                long im1 = id - 1, im2 = id - 2, ip1 = id + 1, jm1 = id - NX, jm2 = id - 2 * NX,
                     jp1 = id + NX, km1 = id - NXY, km2 = id - 2 * NXY, kp1 = id + NXY,
                     ip2 = id + 2, jp2 = id + 2 * NX, kp2 = id + 2 * NXY,
                     ip3 = id + 3, jp3 = id + 3 * NX, kp3 = id + 3 * NXY;
                if (i == 0) { im1 = id; }
                if (i == nx - 1) { ip1 = id; ip2 = im1; ip3 = im2; }
                if (i == nx - 2) { ip2 = ip1; ip3 = id; }
                if (i == nx - 3) { ip3 = ip2; }
                if (j == 0) { jm1 = id; }
                if (j == ny - 1) { jp1 = id; jp2 = jm1; jp3 = jm2; }
                if (j == ny - 2) { jp2 = jp1; jp3 = id; }
                if (j == ny - 3) { jp3 = jp2; }
                if (k == 0) { km1 = id; }
                if (k == nz - 1) { kp1 = id; kp2 = km1; kp3 = km2; }
                if (k == nz - 2) { kp2 = kp1; kp3 = id; }
                if (k == nz - 3) { kp3 = kp2; }
                double jx = jbn[id], jy = jbn[id + 4 * off], jz = jbn[id + 8 * off];
                const double *dx = dphi, *dy = dphi + off, *dz = dphi + 2 * off;
                out[id] = orc_phi_x_weno(dx[ip3] * jx, dx[ip2] * jx, dx[ip1] * jx, dx[id] * jx, dx[im1] * jx);
                out[id + off] = orc_phi_x_weno(dy[jp3] * jy, dy[jp2] * jy, dy[jp1] * jy, dy[id] * jy, dy[jm1] * jy);
                out[id + 2 * off] = orc_phi_x_weno(dz[kp3] * jz, dz[kp2] * jz, dz[kp1] * jz, dz[id] * jz, dz[km1] * jz);
            }
}

/* advect_RS_WENO, lsTools.cu:361-417. */
void advect_rs(double *rs, const double *vel, const double *pp, const double *pm, size_t n) {
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        size_t id = (size_t)q;
        double acc[3];
        for (int d = 0; d < 3; ++d) {
            double v = vel[id + d * n];
            double rsign = (double)(v > 0.0) - (double)(v < 0.0);
            acc[d] = 0.5 * (rsign + 1.0) * v * pp[id + d * n]
                   + 0.5 * std::fabs(rsign - 1.0) * v * pm[id + d * n];
        }
        rs[id] = acc[0] + acc[1] + acc[2];
    }
}

} // namespace

extern "C" {

static int g_threads = 0;

void orc_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_deriv_pencil(int scheme, int n, double *u, double h) {
    if (!scheme_ok(scheme) || n < 5 || !u || !(h > 0.0)) return 1;
    Work w(n);
    pencil(scheme, n, u, h, w);
    return 0;
}

int orc_deriv3d(int scheme, int axis, int nx, int ny, int nz, double h,
                const double *in, double *out) {
    if (!scheme_ok(scheme) || axis < 0 || axis > 2 || !in || !out || !(h > 0.0)) return 1;
    const int n = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (n < 5 || nx < 1 || ny < 1 || nz < 1) return 1;
    if (axis == 0) {            /* deriv_vel.f90:17-27 */
#pragma omp parallel
        {
            Work w(n);
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j) {
                    for (int i = 0; i < nx; ++i) w.p[i] = in[lin(i, j, k, nx, ny)];
                    pencil(scheme, n, w.p, h, w);
                    for (int i = 0; i < nx; ++i) out[lin(i, j, k, nx, ny)] = w.p[i];
                }
        }
    } else if (axis == 1) {     /* deriv_vel.f90:53-63 */
#pragma omp parallel
        {
            Work w(n);
#pragma omp for collapse(2) schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int i = 0; i < nx; ++i) {
                    for (int j = 0; j < ny; ++j) w.p[j] = in[lin(i, j, k, nx, ny)];
                    pencil(scheme, n, w.p, h, w);
                    for (int j = 0; j < ny; ++j) out[lin(i, j, k, nx, ny)] = w.p[j];
                }
        }
    } else {                    /* deriv_vel.f90:89-99 */
#pragma omp parallel
        {
            Work w(n);
#pragma omp for collapse(2) schedule(static)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    for (int k = 0; k < nz; ++k) w.p[k] = in[lin(i, j, k, nx, ny)];
                    pencil(scheme, n, w.p, h, w);
                    for (int k = 0; k < nz; ++k) out[lin(i, j, k, nx, ny)] = w.p[k];
                }
        }
    }
    return 0;
}

int orc_cudaDeriv(const int *schemes, double *dvel, double *dtemp,
                  const double *vel, const double *temp,
                  double hx, double hy, double hz, int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    const double h[3] = {hx, hy, hz};
    int rc = 0;
    /* output order of solver/cuDeriv.cu:629-644: d/dx (u,v,w), d/dy (u,v,w),
     * d/dz (u,v,w); then dT/dx, dT/dy, dT/dz. */
    for (int ax = 0; ax < 3; ++ax)
        for (int c = 0; c < 3; ++c)
            rc |= orc_deriv3d(schemes[ax], ax, nx, ny, nz, h[ax], vel + c * n, dvel + (3 * ax + c) * n);
    for (int ax = 0; ax < 3; ++ax)
        rc |= orc_deriv3d(schemes[ax], ax, nx, ny, nz, h[ax], temp, dtemp + ax * n);
    return rc;
}

int orc_cuDivergence(const int *schemes, double *rs, double *rsv,
                     const double *e, const double *f, const double *g,
                     const double *ev, const double *fv, const double *gv,
                     const double *jbn, double hx, double hy, double hz,
                     int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> w(12 * n);
    double *pe = &w[0], *pf = &w[n], *pg = &w[2 * n], *pev = &w[3 * n], *pfv = &w[4 * n], *pgv = &w[5 * n];
    double *de = &w[6 * n], *df = &w[7 * n], *dg = &w[8 * n], *dev = &w[9 * n], *dfv = &w[10 * n], *dgv = &w[11 * n];
    const double *j1 = jbn, *j5 = jbn + 4 * n, *j9 = jbn + 8 * n, *j10 = jbn + 9 * n, *j11 = jbn + 10 * n;
    /* projection, solver/divergencia.f90:225-243 */
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        pe[q] = j10[q] * (j1[q] * e[q]);
        pf[q] = j10[q] * (j5[q] * f[q]);
        pg[q] = j10[q] * (j9[q] * g[q]);
        pev[q] = j10[q] * (j1[q] * ev[q]);
        pfv[q] = j10[q] * (j5[q] * fv[q]);
        pgv[q] = j10[q] * (j9[q] * gv[q]);
    }
    int rc = 0;
    rc |= orc_deriv3d(schemes[0], 0, nx, ny, nz, hx, pe, de);
    rc |= orc_deriv3d(schemes[0], 0, nx, ny, nz, hx, pev, dev);
    rc |= orc_deriv3d(schemes[1], 1, nx, ny, nz, hy, pf, df);
    rc |= orc_deriv3d(schemes[1], 1, nx, ny, nz, hy, pfv, dfv);
    rc |= orc_deriv3d(schemes[2], 2, nx, ny, nz, hz, pg, dg);
    rc |= orc_deriv3d(schemes[2], 2, nx, ny, nz, hz, pgv, dgv);
    /* solver/divergencia.f90:346-354 */
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        rs[q] = j11[q] * (de[q] + df[q] + dg[q]);
        rsv[q] = j11[q] * (dev[q] + dfv[q] + dgv[q]);
    }
    return rc;
}

int orc_flujos(int neq, int nx, int ny, int nz,
               double *e, double *f, double *g,
               double *ev, double *fv, double *gv,
               const double *um, const double *u, const double *pres,
               const double *dvel, const double *jbn, const double *vis) {
    if (neq < 1 || neq > 5) return 1;
    const size_t n = (size_t)nx * ny * nz;
    const double *um2 = um + n, *um3 = um + 2 * n, *um4 = um + 3 * n, *um5 = um + 4 * n;
    const double *u1 = u, *u2 = u + n, *u3 = u + 2 * n;
    const double *j1 = jbn, *j5 = jbn + 4 * n, *j9 = jbn + 8 * n;
#define DV(c) (dvel + (size_t)((c) - 1) * n)
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        double p0, p1, p2;
        switch (neq) {
        case 1: /* flujos_compact.f90:21-40 */
            e[q] = -um2[q]; f[q] = -um3[q]; g[q] = -um4[q];
            ev[q] = 0.0; fv[q] = 0.0; gv[q] = 0.0;
            break;
        case 2: /* :43-84 */
            e[q] = -um2[q] * u1[q] - pres[q];
            f[q] = -um3[q] * u1[q];
            g[q] = -um4[q] * u1[q];
            p0 = j1[q] * DV(1)[q];
            ev[q] = vis[q] * (2.0 * p0);
            p1 = j1[q] * DV(2)[q]; p2 = j5[q] * DV(4)[q];
            fv[q] = vis[q] * (p1 + p2);
            p1 = j1[q] * DV(3)[q]; p2 = j9[q] * DV(7)[q];
            gv[q] = vis[q] * (p1 + p2);
            break;
        case 3: /* :88-128 */
            e[q] = -um2[q] * u2[q];
            f[q] = -um3[q] * u2[q] - pres[q];
            g[q] = -um4[q] * u2[q];
            p1 = j1[q] * DV(2)[q]; p2 = j5[q] * DV(4)[q];
            ev[q] = vis[q] * (p1 + p2);
            p1 = j5[q] * DV(5)[q];
            fv[q] = vis[q] * (2.0 * p1);
            p1 = j9[q] * DV(8)[q]; p2 = j5[q] * DV(6)[q];
            gv[q] = vis[q] * (p1 + p2);
            break;
        case 4: /* :133-173 */
            e[q] = -um2[q] * u3[q];
            f[q] = -um3[q] * u3[q];
            g[q] = -um4[q] * u3[q] - pres[q];
            p1 = j1[q] * DV(3)[q]; p2 = j9[q] * DV(7)[q];
            ev[q] = vis[q] * (p1 + p2);
            p1 = j9[q] * DV(8)[q]; p2 = j5[q] * DV(6)[q];
            fv[q] = vis[q] * (p1 + p2);
            p2 = j9[q] * DV(9)[q];
            gv[q] = vis[q] * (2.0 * p2);
            break;
        default: /* :176-214 */
            e[q] = -u1[q] * um5[q];
            f[q] = -u2[q] * um5[q];
            g[q] = -u3[q] * um5[q];
            ev[q] = 0.0; fv[q] = 0.0; gv[q] = 0.0;
            break;
        }
    }
#undef DV
    return 0;
}

int orc_inisgdm(int nx, int ny, int nz, const double *xyz, double *dxyzsgd, double *ratios) {
    if (nx < 2 || ny < 2 || nz < 2) return 1;
    const size_t n = (size_t)nx * ny * nz;
    const double *X = xyz, *Y = xyz + n, *Z = xyz + 2 * n;
    double *dxp = ratios, *dxm = ratios + n, *dyp = ratios + 2 * n, *dym = ratios + 3 * n,
           *dzp = ratios + 4 * n, *dzm = ratios + 5 * n;
    /* spacings, solver/sgdm_incomp.f90:20-69 */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t id = lin(i, j, k, nx, ny);
                if (i > 0 && i < nx - 1) {
                    dxm[id] = X[id] - X[id - 1];
                    dxp[id] = X[id + 1] - X[id];
                } else if (i == 0) {
                    dxp[id] = X[id + 1] - X[id];
                    dxm[id] = X[id + 1] - X[id];
                } else {
                    dxm[id] = X[id] - X[id - 1];
                    dxp[id] = X[id] - X[id - 1];
                }
                size_t sy = nx;
                if (j > 0 && j < ny - 1) {
                    dym[id] = Y[id] - Y[id - sy];
                    dyp[id] = Y[id + sy] - Y[id];
                } else if (j == 0) {
                    dyp[id] = Y[id + sy] - Y[id];
                    dym[id] = Y[id + sy] - Y[id];
                } else {
                    dym[id] = Y[id] - Y[id - sy];
                    dyp[id] = Y[id] - Y[id - sy];
                }
                size_t sz = (size_t)nx * ny;
                if (k > 0 && k < nz - 1) {
                    dzm[id] = Z[id] - Z[id - sz];
                    dzp[id] = Z[id + sz] - Z[id];
                } else if (k == 0) {
                    dzp[id] = Z[id + sz] - Z[id];
                    dzm[id] = Z[id + sz] - Z[id];
                } else {
                    dzm[id] = Z[id] - Z[id - sz];
                    dzp[id] = Z[id] - Z[id - sz];
                }
            }
    /* :75-108 */
    for (size_t id = 0; id < n; ++id) {
        double dzmax = std::fmax(dzm[id], dzp[id]);
        double dymax = std::fmax(dym[id], dyp[id]);
        double dxmax = std::fmax(dxm[id], dxp[id]);
        dxyzsgd[id] = std::pow(dxmax * dymax * dzmax, 1. / 3.);
    }
    for (size_t id = 0; id < n; ++id) {
        dxp[id] = std::pow(dxyzsgd[id] / dxp[id], 1.0 / 3.0);
        dxm[id] = std::pow(dxyzsgd[id] / dxm[id], 1.0 / 3.0);
        dyp[id] = std::pow(dxyzsgd[id] / dyp[id], 1.0 / 3.0);
        dym[id] = std::pow(dxyzsgd[id] / dym[id], 1.0 / 3.0);
        dzp[id] = std::pow(dxyzsgd[id] / dzp[id], 1.0 / 3.0);
        dzm[id] = std::pow(dxyzsgd[id] / dzm[id], 1.0 / 3.0);
    }
    return 0;
}

int orc_sgs_sf(int nx, int ny, int nz, const double *u, const double *dvel,
               const double *jbn, const double *dxyzsgd, const double *ratios,
               double amu0, double *amut) {
    if (nx < 2 || ny < 2 || nz < 2) return 1;
    const size_t n = (size_t)nx * ny * nz;
    const double *U = u, *V = u + n, *W = u + 2 * n;
    const double *dxp = ratios, *dxm = ratios + n, *dyp = ratios + 2 * n, *dym = ratios + 3 * n,
                 *dzp = ratios + 4 * n, *dzm = ratios + 5 * n;
    const size_t sy = nx, sz = (size_t)nx * ny;
    /* f_structura, solver/sgdm_incomp.f90:166-298: six one-sided squared
     * increments, accumulated in the reference's loop order. */
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t id = lin(i, j, k, nx, ny);
                double a, b, c, s;
                /* x+ (:180-197): assignment */
                size_t p = (i < nx - 1) ? id + 1 : id, m = (i < nx - 1) ? id : id - 1;
                a = (U[p] - U[m]) * dxp[id]; b = (V[p] - V[m]) * dxp[id]; c = (W[p] - W[m]) * dxp[id];
                s = a * a + b * b + c * c;
                /* x- (:198-215) */
                if (i > 0) { p = id - 1; m = id; } else { p = id + 1; m = id; }
                a = (U[p] - U[m]) * dxm[id]; b = (V[p] - V[m]) * dxm[id]; c = (W[p] - W[m]) * dxm[id];
                s = s + a * a + b * b + c * c;
                /* y+ (:217-234) */
                if (j < ny - 1) { p = id + sy; m = id; } else { p = id; m = id - sy; }
                a = (U[p] - U[m]) * dyp[id]; b = (V[p] - V[m]) * dyp[id]; c = (W[p] - W[m]) * dyp[id];
                s = s + a * a + b * b + c * c;
                /* y- (:235-252): at j=1 the reference uses u(1)-u(2) */
                if (j > 0) { p = id - sy; m = id; } else { p = id; m = id + sy; }
                a = (U[p] - U[m]) * dym[id]; b = (V[p] - V[m]) * dym[id]; c = (W[p] - W[m]) * dym[id];
                s = s + a * a + b * b + c * c;
                /* z+ (:255-272) */
                if (k < nz - 1) { p = id + sz; m = id; } else { p = id; m = id - sz; }
                a = (U[p] - U[m]) * dzp[id]; b = (V[p] - V[m]) * dzp[id]; c = (W[p] - W[m]) * dzp[id];
                s = s + a * a + b * b + c * c;
                /* z- (:273-290) */
                if (k > 0) { p = id - sz; m = id; } else { p = id; m = id + sz; }
                a = (U[p] - U[m]) * dzm[id]; b = (V[p] - V[m]) * dzm[id]; c = (W[p] - W[m]) * dzm[id];
                s = s + a * a + b * b + c * c;
                s = s / 6.e0;                       /* :292-298 */
                amut[id] = amu0 * std::sqrt(s) * dxyzsgd[id];   /* viscosidad_t :131-137 */
            }
    /* VORT, :330-341 */
    std::vector<double> wv(3 * n);
    double *wx = &wv[0], *wy = &wv[n], *wz = &wv[2 * n];
    const double *j1 = jbn, *j5 = jbn + 4 * n, *j9 = jbn + 8 * n;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        wx[q] = j5[q] * dvel[7 * n + q] - j9[q] * dvel[5 * n + q];
        wy[q] = j9[q] * dvel[2 * n + q] - j1[q] * dvel[6 * n + q];
        wz[q] = j1[q] * dvel[3 * n + q] - j5[q] * dvel[1 * n + q];
    }
    /* SELECTIVO, :346-395; cutoff = cos(20 degrees) (:18) */
    const double cutoff = std::cos(20.0 * std::atan(1.0) / 45.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1, kp = k + 1, km = k - 1;
                if (i == nx - 1) ip = nx - 1;
                if (i == 0) im = 0;
                if (j == ny - 1) jp = ny - 1;
                if (j == 0) jm = 0;
                if (k == nz - 1) kp = nz - 1;
                if (k == 0) km = 0;
                size_t id = lin(i, j, k, nx, ny);
                size_t a1 = lin(ip, j, k, nx, ny), a2 = lin(im, j, k, nx, ny), a3 = lin(i, j, kp, nx, ny),
                       a4 = lin(i, j, km, nx, ny), a5 = lin(i, jp, k, nx, ny), a6 = lin(i, jm, k, nx, ny);
                double wxn = wx[a1] + wx[a2] + wx[a3] + wx[a4] + wx[a5] + wx[a6];
                double wyn = wy[a1] + wy[a2] + wy[a3] + wy[a4] + wy[a5] + wy[a6];
                double wzn = wz[a1] + wz[a2] + wz[a3] + wz[a4] + wz[a5] + wz[a6];
                double wn = wx[id] * wx[id] + wy[id] * wy[id] + wz[id] * wz[id];
                wn = std::sqrt(wn * (wxn * wxn + wyn * wyn + wzn * wzn));
                double ps1 = wx[id] * wxn, ps2 = wy[id] * wyn, ps3 = wz[id] * wzn;
                double s1 = (ps1 + ps2 + ps3) / wn;
                if (s1 > cutoff) amut[id] = 0.0;
            }
    return 0;
}

int orc_sgs_smag(int nx, int ny, int nz, const double *dvel, const double *jbn,
                 const double *dxyzsgd, double cs, double *amut) {
    const size_t n = (size_t)nx * ny * nz;
    const double *j1 = jbn, *j5 = jbn + 4 * n, *j9 = jbn + 8 * n;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        double ux = j1[q] * dvel[q], vx = j1[q] * dvel[n + q], wx = j1[q] * dvel[2 * n + q];
        double uy = j5[q] * dvel[3 * n + q], vy = j5[q] * dvel[4 * n + q], wy = j5[q] * dvel[5 * n + q];
        double uz = j9[q] * dvel[6 * n + q], vz = j9[q] * dvel[7 * n + q], wz = j9[q] * dvel[8 * n + q];
        double s12 = 0.5 * (uy + vx), s13 = 0.5 * (uz + wx), s23 = 0.5 * (vz + wy);
        double ss = ux * ux + vy * vy + wz * wz + 2.0 * (s12 * s12 + s13 * s13 + s23 * s23);
        double cd = cs * dxyzsgd[q];
        amut[q] = cd * cd * std::sqrt(2.0 * ss);
    }
    return 0;
}

int orc_viscosidad(int n, const double *amut, double c4, double *vis) {
    for (int q = 0; q < n; ++q) {
        double v = 1.0;
        vis[q] = c4 * v + amut[q];
    }
    return 0;
}

double orc_phi_x_weno(double beta1, double beta2, double beta3, double beta4, double beta5) {
    /* Phi_x_WENO, src/LevelSet/lsTools.cu:9-50 */
    double s_b1 = (13.0 / 12.0) * (beta1 - 2.0 * beta2 + beta3) * (beta1 - 2.0 * beta2 + beta3)
                + (0.25) * (beta1 - 4.0 * beta2 + 3.0 * beta3) * (beta1 - 4.0 * beta2 + 3.0 * beta3);
    double s_b2 = (13.0 / 12.0) * (beta2 - 2.0 * beta3 + beta4) * (beta2 - 2.0 * beta3 + beta4)
                + (0.25) * (beta2 - beta4) * (beta2 - beta4);
    double s_b3 = (13.0 / 12.0) * (beta3 - 2.0 * beta4 + beta5) * (beta3 - 2.0 * beta4 + beta5)
                + (0.25) * (3.0 * beta3 - 4.0 * beta4 + beta5) * (3.0 * beta3 - 4.0 * beta4 + beta5);
    double alpha_1 = 0.1 / ((s_b1 + 1.0e-6) * (s_b1 + 1.0e-6));
    double alpha_2 = 0.6 / ((s_b2 + 1.0e-6) * (s_b2 + 1.0e-6));
    double alpha_3 = 0.3 / ((s_b3 + 1.0e-6) * (s_b3 + 1.0e-6));
    double omega_1 = alpha_1 / (alpha_1 + alpha_2 + alpha_3);
    double omega_2 = alpha_2 / (alpha_1 + alpha_2 + alpha_3);
    double omega_3 = alpha_3 / (alpha_1 + alpha_2 + alpha_3);
    return ((omega_1 * (2.0 * beta1 - 7.0 * beta2 + 11.0 * beta3)
             + omega_2 * (-1.0 * beta2 + 5.0 * beta3 + 2.0 * beta4)
             + omega_3 * (2.0 * beta3 + 5.0 * beta4 - beta5)) * (1.0 / 6.0));
}

int orc_to_ghost(double *ghost, const double *val, int g, int nx, int ny, int nz) {
    /* cuSwapToGhost, src/LevelSet/lsTools.cu:772-796 */
    const int nxg = nx + 2 * g, nyg = ny + 2 * g;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                ghost[lin(i + g, j + g, k + g, nxg, nyg)] = val[lin(i, j, k, nx, ny)];
    return 0;
}

int orc_from_ghost(double *val, const double *ghost, int g, int nx, int ny, int nz) {
    /* cuSwapFromGhost, src/LevelSet/lsTools.cu:798-822 */
    const int nxg = nx + 2 * g, nyg = ny + 2 * g;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                val[lin(i, j, k, nx, ny)] = ghost[lin(i + g, j + g, k + g, nxg, nyg)];
    return 0;
}

int orc_mirror_ghost(double *G, int g, int nx, int ny, int nz, double dir) {
    /* cuGhostCellsMirror3dZ/Y/X, src/LevelSet/lsTools.cu:482-585, applied in
     * the Z, Y, X order of lsTransportEc.cu:119-127, each over the full
     * ghosted extent of the other two axes. */
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    for (int y = 0; y < nyg; ++y)
        for (int x = 0; x < nxg; ++x)
            for (int d = 0; d < g; ++d) {
                G[lin(x, y, g - d - 1, nxg, nyg)] = G[lin(x, y, g + d, nxg, nyg)] * dir;
                G[lin(x, y, nz + d + g, nxg, nyg)] = G[lin(x, y, nz - d - 1 + g, nxg, nyg)] * dir;
            }
    for (int z = 0; z < nzg; ++z)
        for (int x = 0; x < nxg; ++x)
            for (int d = 0; d < g; ++d) {
                G[lin(x, g - d - 1, z, nxg, nyg)] = G[lin(x, g + d, z, nxg, nyg)] * dir;
                G[lin(x, ny + d + g, z, nxg, nyg)] = G[lin(x, ny - d - 1 + g, z, nxg, nyg)] * dir;
            }
    for (int z = 0; z < nzg; ++z)
        for (int y = 0; y < nyg; ++y)
            for (int d = 0; d < g; ++d) {
                G[lin(g - d - 1, y, z, nxg, nyg)] = G[lin(g + d, y, z, nxg, nyg)] * dir;
                G[lin(nx + d + g, y, z, nxg, nyg)] = G[lin(nx - d - 1 + g, y, z, nxg, nyg)] * dir;
            }
    return 0;
}

int orc_weno_rhs(double *rs, const double *phi, const double *vel, const double *jbn,
                 double hx, double hy, double hz, int nx, int ny, int nz, int ref_bugs) {
    if (nx < 4 || ny < 4 || nz < 4) return 1;
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> d(3 * n), pp(3 * n), pm(3 * n);
    dev1_downwind(d.data(), phi, 1.0 / hx, 1.0 / hy, 1.0 / hz, nx, ny, nz);
    weno_plus(pp.data(), d.data(), jbn, nx, ny, nz, ref_bugs);
    weno_minus(pm.data(), d.data(), jbn, nx, ny, nz);
    advect_rs(rs, vel, pp.data(), pm.data(), n);
    return 0;
}

int orc_weno_advect(double *phi, const double *vel, const double *jbn,
                    double hx, double hy, double hz, double dt,
                    int nx, int ny, int nz, int ref_bugs) {
    /* cuAdvectLsJB, src/LevelSet/lsTransportEc.cu:201-418, with RunGK_*
     * from src/LevelSet/extrapol.cu:155-212. */
    if (nx < 4 || ny < 4 || nz < 4) return 1;
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> rs(n), tmp(n);
    orc_weno_rhs(rs.data(), phi, vel, jbn, hx, hy, hz, nx, ny, nz, ref_bugs);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) tmp[q] = phi[q] - dt * rs[q];
    orc_weno_rhs(rs.data(), tmp.data(), vel, jbn, hx, hy, hz, nx, ny, nz, ref_bugs);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) tmp[q] = 0.75 * phi[q] + 0.25 * (tmp[q] - dt * rs[q]);
    orc_weno_rhs(rs.data(), tmp.data(), vel, jbn, hx, hy, hz, nx, ny, nz, ref_bugs);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) phi[q] = (phi[q] + 2.0 * (tmp[q] - dt * rs[q])) / 3.0;
    return 0;
}

/* DevFirstOrder_LS (src/LevelSet/extrapol.cu:100-153): central differences of
 * the solid level set times the centre metric, with the factor 1 (one-sided
 * difference) on every boundary cell of the grid, whichever axis it borders. */
static void dev_first_order_ls(double *dphi, const double *phiS, const double *j0, const double *j4,
                               const double *j8, double sx, double sy, double sz,
                               int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t id = lin(i, j, k, nx, ny);
                size_t ip = id + 1, im = id - 1, jp = id + nx, jm = id - nx,
                       kp = id + (size_t)nx * ny, km = id - (size_t)nx * ny;
                double factor = 0.5;
                if (i == 0) { im = id; factor = 1.0; }
                if (j == 0) { jm = id; factor = 1.0; }
                if (k == 0) { km = id; factor = 1.0; }
                if (i == nx - 1) { ip = id; factor = 1.0; }
                if (j == ny - 1) { jp = id; factor = 1.0; }
                if (k == nz - 1) { kp = id; factor = 1.0; }
                dphi[id] = factor * sx * j0[id] * (phiS[ip] - phiS[im]);
                dphi[n + id] = factor * sy * j4[id] * (phiS[jp] - phiS[jm]);
                dphi[2 * n + id] = factor * sz * j8[id] * (phiS[kp] - phiS[km]);
            }
}

/* extrapolKernel (src/LevelSet/extrapol.cu:5-98): upwind right-hand side of
 * the extrapolation equation, rs = sum_d (so dphi_d) D_d ext, where D_d is the
 * one-sided difference on the upwind side of so*dphi_d.  On boundary cells the
 * centre value is replaced by a neighbour (id2), the last applicable of the
 * six boundary rules winning, as the reference writes them. */
static void extrapol_rhs(double *rs, const double *ext, const double *phiS, const double *j0,
                         const double *j4, const double *j8, const double *dphi, double sx,
                         double sy, double sz, int nx, int ny, int nz, int flag) {
    const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t id = lin(i, j, k, nx, ny);
                size_t ip = id + 1, im = id - 1, jp = id + nx, jm = id - nx,
                       kp = id + (size_t)nx * ny, km = id - (size_t)nx * ny;
                size_t id2 = id;
                if (i == 0) { id2 = ip; im = id; }
                if (j == 0) { id2 = jp; jm = id; }
                if (k == 0) { id2 = kp; km = id; }
                if (i == nx - 1) { id2 = im; ip = id; }
                if (j == ny - 1) { id2 = jm; jp = id; }
                if (k == nz - 1) { id2 = km; kp = id; }
                const double so = flag > 0 ? (double)(phiS[id] > 0.0) : -1.0 * (double)(phiS[id] <= 0.0);
                const double px = so * dphi[id], py = so * dphi[n + id], pz = so * dphi[2 * n + id];
                const double xd = sx * j0[id] * (ext[id2] - ext[im]);
                const double yd = sy * j4[id] * (ext[id2] - ext[jm]);
                const double zd = sz * j8[id] * (ext[id2] - ext[km]);
                const double xu = sx * j0[id] * (ext[ip] - ext[id2]);
                const double yu = sy * j4[id] * (ext[jp] - ext[id2]);
                const double zu = sz * j8[id] * (ext[kp] - ext[id2]);
                double m = (double)(px > 0.0) - (double)(px < 0.0);
                double r = (0.5 * (m + 1.0) * xd + 0.5 * std::fabs(m - 1.0) * xu) * px;
                m = (double)(py > 0.0) - (double)(py < 0.0);
                r += (0.5 * (m + 1.0) * yd + 0.5 * std::fabs(m - 1.0) * yu) * py;
                m = (double)(pz > 0.0) - (double)(pz < 0.0);
                r += (0.5 * (m + 1.0) * zd + 0.5 * std::fabs(m - 1.0) * zu) * pz;
                rs[id] = r;
            }
}

int orc_extrapolation(double *ext, const double *phiS, const double *j0, const double *j4,
                      const double *j8, double sx, double sy, double sz, int nx, int ny, int nz,
                      double dtext, int flag, int iters) {
    /* cuExtrapolation (src/LevelSet/interface.cu:341-436): the gradient of the
     * solid level set once, then `iters` TVD-RK3 pseudo-steps (10 in the
     * reference) of the extrapolation equation with RunGK_First/Second/ThirdS
     * (src/LevelSet/extrapol.cu:155-212). */
    if (nx < 2 || ny < 2 || nz < 2 || iters < 0) return 1;
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> dphi(3 * n), rs(n), d(n);
    dev_first_order_ls(dphi.data(), phiS, j0, j4, j8, sx, sy, sz, nx, ny, nz);
    for (int it = 0; it < iters; ++it) {
        extrapol_rhs(rs.data(), ext, phiS, j0, j4, j8, dphi.data(), sx, sy, sz, nx, ny, nz, flag);
        for (size_t q = 0; q < n; ++q) d[q] = ext[q] - dtext * rs[q];
        extrapol_rhs(rs.data(), d.data(), phiS, j0, j4, j8, dphi.data(), sx, sy, sz, nx, ny, nz, flag);
        for (size_t q = 0; q < n; ++q) d[q] = 0.75 * ext[q] + 0.25 * (d[q] - dtext * rs[q]);
        extrapol_rhs(rs.data(), d.data(), phiS, j0, j4, j8, dphi.data(), sx, sy, sz, nx, ny, nz, flag);
        for (size_t q = 0; q < n; ++q) ext[q] = (ext[q] + 2.0 * (d[q] - dtext * rs[q])) / 3.0;
    }
    return 0;
}

int orc_advect_extrapolate(double *press, const double *jbn, const double *sobject,
                           double deltaX, double deltaY, double deltaZ, int nx, int ny, int nz,
                           double deltamin) {
    /* advect_CUDA as linked (src/LevelSet/lsTransportEc.cu:24-197): pad
     * pressure, the solid level set and the metric components 1, 5, 9 with 5
     * mirrored ghost layers (:91-157), extrapolate the pressure across the
     * solid with dtext = deltamin/2 and Flag = 1 (:161-162), then copy the
     * interior back (:164-168).  The kernels get 1/deltaX (interface.cu:372-377). */
    const int g = 5;
    if (nx < g || ny < g || nz < g) return 1;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    const size_t n = (size_t)nx * ny * nz, ng = (size_t)nxg * nyg * nzg;
    std::vector<double> P(ng, 0.0), S(ng, 0.0), J(3 * ng, 0.0);
    orc_to_ghost(P.data(), press, g, nx, ny, nz);
    orc_mirror_ghost(P.data(), g, nx, ny, nz, 1.0);
    orc_to_ghost(S.data(), sobject, g, nx, ny, nz);
    orc_mirror_ghost(S.data(), g, nx, ny, nz, 1.0);
    for (int c = 0; c < 3; ++c) {
        orc_to_ghost(&J[c * ng], jbn + (size_t)(4 * c) * n, g, nx, ny, nz);
        orc_mirror_ghost(&J[c * ng], g, nx, ny, nz, 1.0);
    }
    int rc = orc_extrapolation(P.data(), S.data(), &J[0], &J[ng], &J[2 * ng], 1.0 / deltaX,
                               1.0 / deltaY, 1.0 / deltaZ, nxg, nyg, nzg, deltamin * 0.5, 1, 10);
    if (rc) return rc;
    orc_from_ghost(press, P.data(), g, nx, ny, nz);
    return 0;
}

/* inifiltro (src/MSVSingle/filtro_incomp.f90:1-162): the tridiagonal rows of
 * the compact filter for a pencil of n points.  b = 1; with zrows = 0 the
 * non-periodic rows (a = c = cfilt for 1-based rows 6..n-5, 0 elsewhere:
 * cfilt2..cfilt5 are 0 in both branches of :17-31), with zrows = 1 the
 * periodic rows (a = c = cfilt everywhere), which filtrado passes for z. */
static void filter_rows(int n, double cfilt, int zrows, double *a, double *b, double *c) {
    for (int l = 0; l < n; ++l) {
        b[l] = 1.0;
        const bool in = zrows || (l >= 5 && l <= n - 6);
        a[l] = in ? cfilt : 0.0;
        c[l] = in ? cfilt : 0.0;
    }
}

int orc_filtronper(int n, double *u, double cfilt, int zrows) {
    /* filtronper (src/MSVSingle/filtro_incomp.f90:307-362) with the
     * right-hand-side constants of inifiltro (:140-145) */
    if (n < 11) return 1;
    const double arsf = (193. + 126. * cfilt) / 256., brsf = (105. + 302. * cfilt) / 256.,
                 crsf = (-15. + 30. * cfilt) / 64., drsf = (45. - 90. * cfilt) / 512.,
                 ersf = (-5. + 10. * cfilt) / 256., frsf = (1. - 2 * cfilt) / 512.;
    std::vector<double> a(n), b(n), c(n), r(n), gam(n);
    filter_rows(n, cfilt, zrows, a.data(), b.data(), c.data());
    for (int l = 5; l <= n - 6; ++l)
        r[l] = 0.5 * (arsf * (u[l] + u[l]) + brsf * (u[l + 1] + u[l - 1]) + crsf * (u[l + 2] + u[l - 2]) +
                      drsf * (u[l + 3] + u[l - 3]) + ersf * (u[l + 4] + u[l - 4]) +
                      frsf * (u[l + 5] + u[l - 5]));
    for (int l = 0; l < 5; ++l) {   /* SIN FILTRO rows (:336-345) */
        r[l] = u[l];
        r[n - 1 - l] = u[n - 1 - l];
    }
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int l = 1; l < n; ++l) {
        gam[l] = c[l - 1] / bet;
        bet = b[l] - a[l] * gam[l];
        u[l] = (r[l] - a[l] * u[l - 1]) / bet;
    }
    for (int l = n - 2; l >= 0; --l) u[l] = u[l] - gam[l + 1] * u[l + 1];
    return 0;
}

int orc_filtrado(double *um, const double *jbn, double cfilt, int nx, int ny, int nz) {
    /* filtrado with itf = 1, the only value it is called with
     * (solver/rungek_ico.f90:269-276; src/MSVSingle/herramientas_incomp2.f90:
     * 227-410): for each of the 5 equations, x then y then z, each pencil
     * scaled by jbn(10) before and by jbn(11) after; z with the periodic rows
     * azpf/bzpf/czpf (:281-289, 361-371). */
    if (nx < 11 || ny < 11 || nz < 11) return 1;
    const size_t n = (size_t)nx * ny * nz;
    const double *J10 = jbn + 9 * n, *J11 = jbn + 10 * n;
    for (int m = 0; m < 5; ++m) {
        double *f = um + (size_t)m * n;
#pragma omp parallel
        {
            std::vector<double> du(nx), dv(ny), dw(nz);
#pragma omp for schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j) {
                    for (int i = 0; i < nx; ++i) du[i] = f[lin(i, j, k, nx, ny)] * J10[lin(i, j, k, nx, ny)];
                    orc_filtronper(nx, du.data(), cfilt, 0);
                    for (int i = 0; i < nx; ++i) f[lin(i, j, k, nx, ny)] = du[i] * J11[lin(i, j, k, nx, ny)];
                }
#pragma omp for schedule(static)
            for (int k = 0; k < nz; ++k)
                for (int i = 0; i < nx; ++i) {
                    for (int j = 0; j < ny; ++j) dv[j] = f[lin(i, j, k, nx, ny)] * J10[lin(i, j, k, nx, ny)];
                    orc_filtronper(ny, dv.data(), cfilt, 0);
                    for (int j = 0; j < ny; ++j) f[lin(i, j, k, nx, ny)] = dv[j] * J11[lin(i, j, k, nx, ny)];
                }
#pragma omp for schedule(static)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    for (int k = 0; k < nz; ++k) dw[k] = f[lin(i, j, k, nx, ny)] * J10[lin(i, j, k, nx, ny)];
                    orc_filtronper(nz, dw.data(), cfilt, 1);
                    for (int k = 0; k < nz; ++k) f[lin(i, j, k, nx, ny)] = dw[k] * J11[lin(i, j, k, nx, ny)];
                }
        }
    }
    return 0;
}

/* makeAspa (src/Geometry/rush_ruth_me.f90:519-593) for every blade, then
 * addMaskCil for the hub and the shaft (src/Geometry/rotating.f90:110-140):
 * the impeller mask of one cell at time t. */
static double impeller_mask_cell(const orc_impeller *imp, double x, double y, double z, double t) {
    double m = 1.0;
    const double two_pi = 2.0 * 3.14159265358979323846;
    for (int b = 0; b < imp->nblades; ++b) {
        const double th = imp->theta0 + imp->omega * t + b * (two_pi / imp->nblades);
        const double c = std::cos(th), sn = std::sin(th);
        /* planes of a blade rotated by th: A1..A4 = (0,1), (0,-1), (1,0), (-1,0) */
        const double A1p = 0.0 * c - 1.0 * sn, B1p = 0.0 * sn + 1.0 * c;
        const double A2p = 0.0 * c - (-1.0) * sn, B2p = 0.0 * sn + (-1.0) * c;
        const double A3p = 1.0 * c - 0.0 * sn, B3p = 1.0 * sn + 0.0 * c;
        const double A4p = -1.0 * c - 0.0 * sn, B4p = -1.0 * sn + 0.0 * c;
        const double pl1 = A1p * x + B1p * y + (-imp->half_thick);
        const double pl2 = A2p * x + B2p * y + (-imp->half_thick);
        const double pl3 = A3p * x + B3p * y + (-imp->r2);
        const double pl4 = A4p * x + B4p * y + imp->r1;
        if (pl1 <= 0.0 && pl2 <= 0.0 && pl3 <= 0.0 && pl4 <= 0.0 && z >= imp->z1 && z <= imp->z2) m = 0.0;
    }
    const double radio = std::sqrt(x * x + y * y);
    if (radio >= 0.0 && radio <= imp->hub_r && z >= imp->hub_z1 && z <= imp->hub_z2) m = 0.0;
    if (radio >= 0.0 && radio <= imp->shaft_r && z >= imp->shaft_z0 && z <= imp->shaft_z1) m = 0.0;
    return m;
}

/* the body velocity of addAngularVel (rotating.f90:163-186): the polar angle
 * from atan(|y/x|) with the reference's constants for pi, then
 * (-omega r sin, omega r cos) */
static void impeller_velocity(double omega, double x, double y, double *ue, double *ve) {
    const double radio = std::sqrt(x * x + y * y);
    double th;
    if (x != 0.0) th = std::atan(std::fabs(y / x));
    else th = 3.1415926 / 2.;
    if (x < 0.0 && y > 0.0) th = 3.141592 - th;
    else if (x < 0.0 && y <= 0.0) th = th + 3.141592;
    else if (x >= 0.0 && y < 0.0) th = 2.0 * 3.141592 - th;
    *ue = -1.0 * omega * radio * std::sin(th);
    *ve = omega * radio * std::cos(th);
}

/* The blade-edge interpolation of rushton (rush_ruth_me.f90:97-185) with
 * getInterpolData (:302-517) and getMatrix (:243-299), blade by blade: the
 * cells next to a blade in the (x, y) plane of the first z layer take, in
 * the blade band, the velocity of the plane through the blade-surface point
 * (rigid rotation there) and two neighbour cells on the outer side; cells are
 * visited in the reference's k, j, i order, so a cell may read a neighbour
 * updated before it.  The interpolated mask of :116-128 only feeds the
 * impellermask output and is left out. */
static void impeller_interp(double *um, const double *xyz, const orc_impeller *imp, double t,
                            int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    const double *X = xyz, *Y = xyz + n, *Z = xyz + 2 * n;
    const double dx = (X[lin(nx - 1, 0, 0, nx, ny)] - X[lin(0, 0, 0, nx, ny)]) / (double)(nx - 1);
    const double dy = (Y[lin(0, ny - 1, 0, nx, ny)] - Y[lin(0, 0, 0, nx, ny)]) / (double)(ny - 1);
    const double dz = (Z[lin(0, 0, nz - 1, nx, ny)] - Z[lin(0, 0, 0, nx, ny)]) / (double)(nz - 1);
    const double rango = std::sqrt(dx * dx + dy * dy + dz * dz);
    const double two_pi = 2.0 * 3.14159265358979323846, pi = 2.0 * std::acos(0.0);
    const size_t n2 = (size_t)nx * ny;
    std::vector<double> m2(n2), M(9 * n2), P1(2 * n2);
    std::vector<int> flag(n2), i1(n2), j1(n2), i2(n2), j2(n2);
    for (int b = 0; b < imp->nblades; ++b) {
        const double th = imp->theta0 + imp->omega * t + b * (two_pi / imp->nblades);
        const double c = std::cos(th), sn = std::sin(th);
        const double A[4] = {0.0 * c - 1.0 * sn, 0.0 * c - (-1.0) * sn, 1.0 * c - 0.0 * sn, -1.0 * c - 0.0 * sn};
        const double B[4] = {0.0 * sn + 1.0 * c, 0.0 * sn + (-1.0) * c, 1.0 * sn + 0.0 * c, -1.0 * sn + 0.0 * c};
        const double D[4] = {-imp->half_thick, -imp->half_thick, -imp->r2, imp->r1};
        auto plane = [&](int q, double x, double y) { return A[q] * x + B[q] * y + D[q]; };
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t id = lin(i, j, 0, nx, ny);
                bool in = true;
                for (int q = 0; q < 4; ++q) in = in && plane(q, X[id], Y[id]) <= 0.0;
                m2[j * nx + i] = in ? 0.0 : 1.0;
                flag[j * nx + i] = 1;
            }
        for (int j = 1; j < ny - 1; ++j)
            for (int i = 1; i < nx - 1; ++i) {
                const size_t q = (size_t)j * nx + i;
                if (m2[q] == 1.0 && (m2[q + 1] == 0.0 || m2[q - 1] == 0.0 || m2[q + nx] == 0.0 ||
                                     m2[q - nx] == 0.0))
                    flag[q] = -1;
            }
        double Ag = 0.0, Bg = 0.0, Dg = 0.0;
        bool have = false;
        for (int j = 1; j < ny - 1; ++j)
            for (int i = 1; i < nx - 1; ++i) {
                const size_t q = (size_t)j * nx + i;
                if (flag[q] != -1) continue;
                const size_t id = lin(i, j, 0, nx, ny);
                const double x = X[id], y = Y[id];
                for (int pq = 0; pq < 4; ++pq) {
                    const double v = plane(pq, x, y);
                    if (v >= 0.0 && v <= rango) { Ag = A[pq]; Bg = B[pq]; Dg = D[pq]; have = true; break; }
                }
                if (!have) { flag[q] = 1; continue; }   /* no plane yet: left alone */
                const double tt = -(Dg + x * Ag + y * Bg) / (Ag * Ag + Bg * Bg);
                const double angle = std::acos(Ag) / std::sqrt(Ag * Ag + Bg * Bg);
                const int sA = Ag >= 0.0 ? 1 : -1, sB = Bg >= 0.0 ? 1 : -1;
                int a1i, a1j, a2i, a2j;
                if ((angle >= pi / 6.0 && angle <= pi / 3.0) || (angle >= 2.0 * pi / 3.0 && angle <= 5.0 * pi / 6.0)) {
                    a1i = i + sA; a1j = j; a2i = i; a2j = j + sB;
                } else if (angle <= pi / 6.0 || angle >= 5.0 * pi / 6.0) {
                    a1i = i + sA; a1j = j; a2i = i + sA; a2j = j + sB;
                } else {
                    a1i = i; a1j = j + sB; a2i = i + sA; a2j = j + sB;
                }
                i1[q] = a1i; j1[q] = a1j; i2[q] = a2i; j2[q] = a2j;
                const double p1x = x + tt * Ag, p1y = y + tt * Bg;
                const size_t e1 = lin(a1i, a1j, 0, nx, ny), e2 = lin(a2i, a2j, 0, nx, ny);
                const double p2x = X[e1], p2y = Y[e1], p3x = X[e2], p3y = Y[e2];
                P1[2 * q] = p1x; P1[2 * q + 1] = p1y;
                /* getMatrix (:262-296) */
                const double det = p2x * p3y - p3x * p2y + p1x * p2y - p1x * p3y + p3x * p1y - p2x * p1y;
                double *m = &M[9 * q];
                m[0] = (p2x * p3y - p3x * p2y) / det;
                m[1] = (p3x * p1y - p1x * p3y) / det;
                m[2] = (p1x * p2y - p2x * p1y) / det;
                m[3] = (p2y - p3y) / det;
                m[4] = (p3y - p1y) / det;
                m[5] = (p1y - p2y) / det;
                m[6] = (p3x - p2x) / det;
                m[7] = (p1x - p3x) / det;
                m[8] = (p2x - p1x) / det;
            }
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t q = (size_t)j * nx + i;
                    const size_t id = lin(i, j, k, nx, ny);
                    if (flag[q] != -1 || !(Z[id] >= imp->z1 && Z[id] <= imp->z2)) continue;
                    double ux, vy;
                    impeller_velocity(imp->omega, P1[2 * q], P1[2 * q + 1], &ux, &vy);
                    const size_t e1 = lin(i1[q], j1[q], k, nx, ny), e2 = lin(i2[q], j2[q], k, nx, ny);
                    const double *m = &M[9 * q];
                    for (int d = 1; d <= 2; ++d) {
                        const double ub = d == 1 ? ux : vy;
                        const double ua = um[d * n + e1] / um[e1], uc = um[d * n + e2] / um[e2];
                        const double cb1 = m[0] * ub + m[1] * ua + m[2] * uc;
                        const double cb2 = m[3] * ub + m[4] * ua + m[5] * uc;
                        const double cb3 = m[6] * ub + m[7] * ua + m[8] * uc;
                        um[d * n + id] = (cb1 + X[id] * cb2 + Y[id] * cb3) * um[id];
                    }
                }
    }
}

int orc_impeller_force(double *um, const double *xyz, const orc_impeller *imp, double t,
                       int nx, int ny, int nz, double *mask_out) {
    const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        const double x = xyz[q], y = xyz[n + q], z = xyz[2 * n + q];
        const double m = impeller_mask_cell(imp, x, y, z, t);
        double ue = 0.0, ve = 0.0;
        if (m != 1.0) impeller_velocity(imp->omega, x, y, &ue, &ve);
        const double r = um[q];
        um[n + q] = ((1.0 - m) * ue + m * (um[n + q] / r)) * r;
        um[2 * n + q] = ((1.0 - m) * ve + m * (um[2 * n + q] / r)) * r;
        um[3 * n + q] = m * um[3 * n + q];
        if (mask_out) mask_out[q] = m;
    }
    if (imp->interp) impeller_interp(um, xyz, imp, t, nx, ny, nz);
    return 0;
}

/* reini_RS_WENOJB (src/LevelSet/lsTools.cu:824-902): the Godunov
 * approximation of |grad phi| from the left-biased (pp) and right-biased (pm)
 * WENO5 derivatives, upwinded by the sign of phi0, and
 * rs = S(phi0) (|grad phi| - 1) with S = phi0 / sqrt(phi0^2 + dmin^2). */
static void reini_rs(double *rs, const double *pp, const double *pm, const double *phi0,
                     const double *dmins, size_t n) {
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)n; ++q) {
        const size_t id = (size_t)q;
        const double ta = (double)(phi0[id] > 0.0) - (double)(phi0[id] < 0.0);
        double r[3];
        for (int d = 0; d < 3; ++d) {
            const double a = pp[id + d * n], b = pm[id + d * n];
            double pmax = std::max(a, 0.0) * std::max(a, 0.0);
            double pmin = std::min(b, 0.0) * std::min(b, 0.0);
            r[d] = 0.5 * (ta + 1.0) * std::max(pmax, pmin);
            pmax = std::max(b, 0.0) * std::max(b, 0.0);
            pmin = std::min(a, 0.0) * std::min(a, 0.0);
            r[d] += 0.5 * std::fabs(ta - 1.0) * std::max(pmax, pmin);
        }
        const double grad = std::sqrt(r[0] + r[1] + r[2]);
        const double so = phi0[id] / std::sqrt(phi0[id] * phi0[id] + dmins[id] * dmins[id]);
        rs[id] = 1.0 * so * (grad - 1.0);
    }
}

int orc_reinit(double *phi, const double *jbn, const double *dmins, double dX, double dY, double dZ,
               int nxg, int nyg, int nzg, int g, double deltamin, int iters, int ref_bugs) {
    /* cuReinitLsJB (src/LevelSet/lsTransportEc.cu:420-676): on the padded
     * grid, per iteration: mirror the ghost layers, phi0 = phi, then three
     * TVD-RK3 stages of d(phi)/dtau = -S(phi0)(|grad phi| - 1) with
     * dtau = deltamin/2; the kernels get 1/deltaX as their scale. */
    const int nx = nxg - 2 * g, ny = nyg - 2 * g, nz = nzg - 2 * g;
    if (nx < 1 || ny < 1 || nz < 1 || nxg < 4 || nyg < 4 || nzg < 4 || iters < 0) return 1;
    const size_t n = (size_t)nxg * nyg * nzg;
    const double dt = 0.5 * deltamin;
    std::vector<double> d(3 * n), pp(3 * n), pm(3 * n), rs(n), phi0(n), tmp(n);
    auto rhs = [&](const double *f) {
        dev1_downwind(d.data(), f, 1.0 / dX, 1.0 / dY, 1.0 / dZ, nxg, nyg, nzg);
        weno_plus(pp.data(), d.data(), jbn, nxg, nyg, nzg, ref_bugs);
        weno_minus(pm.data(), d.data(), jbn, nxg, nyg, nzg);
        reini_rs(rs.data(), pp.data(), pm.data(), phi0.data(), dmins, n);
    };
    for (int it = 0; it < iters; ++it) {
        orc_mirror_ghost(phi, g, nx, ny, nz, 1.0);
        std::memcpy(phi0.data(), phi, n * sizeof(double));
        rhs(phi);
        for (size_t q = 0; q < n; ++q) tmp[q] = phi[q] - dt * rs[q];
        rhs(tmp.data());
        for (size_t q = 0; q < n; ++q) tmp[q] = 0.75 * phi[q] + 0.25 * (tmp[q] - dt * rs[q]);
        rhs(tmp.data());
        for (size_t q = 0; q < n; ++q) phi[q] = (phi[q] + 2.0 * (tmp[q] - dt * rs[q])) / 3.0;
    }
    return 0;
}

int orc_bc_walls(double *um, int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    double *U[5] = {um, um + n, um + 2 * n, um + 3 * n, um + 4 * n};
    /* frontera_z_val (src/MSVSingle/frontera_z.f90:231-259) */
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            size_t k0 = lin(i, j, 0, nx, ny), k1 = lin(i, j, 1, nx, ny);
            size_t kn = lin(i, j, nz - 1, nx, ny), kn1 = lin(i, j, nz - 2, nx, ny), kn2 = lin(i, j, nz - 3, nx, ny);
            U[0][k0] = U[0][k1];
            U[1][k0] = U[1][k1];
            U[2][k0] = U[2][k1];
            U[3][k0] = 0.0;
            U[4][k0] = U[4][k1];
            U[0][kn] = 1.0;
            U[0][kn1] = 1.0;
            U[1][kn] = U[1][kn2];
            U[1][kn1] = U[1][kn2];
            U[2][kn] = U[2][kn2];
            U[2][kn1] = U[2][kn2];
            U[3][kn] = 0.0;
            U[3][kn1] = 0.0;
            U[4][kn] = U[4][kn2];
            U[4][kn1] = U[4][kn2];
        }
    /* frontera_y_val (frontera_y.f90:231-244) */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            size_t a = lin(i, 0, k, nx, ny), a1 = lin(i, 1, k, nx, ny);
            size_t b = lin(i, ny - 1, k, nx, ny), b1 = lin(i, ny - 2, k, nx, ny);
            U[0][a] = U[0][a1];
            U[0][b] = U[0][b1];
            U[1][a] = 0.0; U[1][b] = 0.0;
            U[2][a] = 0.0; U[2][b] = 0.0;
            U[3][a] = 0.0; U[3][b] = 0.0;
            U[4][a] = U[4][a1];
            U[4][b] = U[4][b1];
        }
    /* frontera_x_val (frontera_x.f90:238-252) */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            size_t a = lin(0, j, k, nx, ny), b = lin(nx - 1, j, k, nx, ny);
            U[1][a] = 0.0; U[2][a] = 0.0; U[3][a] = 0.0;
            U[4][a] = U[4][a + 1];
            U[0][a] = U[0][a + 1];
            U[1][b] = 0.0; U[2][b] = 0.0; U[3][b] = 0.0;
            U[4][b] = U[4][b - 1];
            U[0][b] = U[0][b - 1];
        }
    return 0;
}

double orc_cfl(const double *u, const double *xyz, double mach, int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    const double cs = std::sqrt(1. / mach);   /* source_incomp.f90:11 */
    const int dims[3] = {nx, ny, nz};
    const size_t st[3] = {1, (size_t)nx, (size_t)nx * ny};
    double cfla = 0.;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t q = lin(i, j, k, nx, ny);
                const int idx[3] = {i, j, k};
                double c[3];
                for (int d = 0; d < 3; ++d) {
                    /* INITSTEP spacings (tstep_incomp.f90:11-70), inverted (:74-80) */
                    const double *X = xyz + d * n;
                    double h;
                    if (idx[d] == 0) h = X[q + st[d]] - X[q];
                    else if (idx[d] == dims[d] - 1) h = X[q] - X[q - st[d]];
                    else h = std::fmin(X[q] - X[q - st[d]], X[q + st[d]] - X[q]);
                    double a = std::fabs(u[d * n + q]);
                    a = a + std::sqrt(cs * cs + a * a);   /* tstep_incomp.f90:118-123 */
                    c[d] = (1. / h) * a;
                }
                cfla = std::fmax(cfla, std::fmax(c[0], std::fmax(c[1], c[2])));
            }
    return cfla;
}

int orc_jacobeano(const double *xyz, double *jbn, int scheme, double hx, double hy, double hz,
                  int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    const double h[3] = {hx, hy, hz};
    /* jacob_malla.f90:10-123: d/dxi -> (1),(4),(7), d/deta -> (2),(5),(8), d/dzeta -> (3),(6),(9) */
    for (int ax = 0; ax < 3; ++ax)
        for (int c = 0; c < 3; ++c)
            if (orc_deriv3d(scheme, ax, nx, ny, nz, h[ax], xyz + c * n, jbn + (3 * c + ax) * n)) return 1;
    for (size_t q = 0; q < n; ++q) {
        double j[10];
        for (int c = 1; c <= 9; ++c) j[c] = jbn[(c - 1) * n + q];
        const double det = j[1] * j[5] * j[9] - j[1] * j[6] * j[8] + j[2] * j[6] * j[7] -
                           j[2] * j[4] * j[9] + j[3] * j[4] * j[8] - j[3] * j[5] * j[7];
        if (std::fabs(det) <= 1.e-20) return 2;   /* :136-139 */
        const double inv = 1. / det;
        const double t1 = j[5] * j[9] - j[6] * j[8], t4 = j[3] * j[8] - j[2] * j[9],
                     t7 = j[2] * j[6] - j[3] * j[5], t2 = j[6] * j[7] - j[4] * j[9],
                     t5 = j[1] * j[9] - j[3] * j[7], t8 = j[3] * j[4] - j[1] * j[6],
                     t3 = j[4] * j[8] - j[5] * j[7], t6 = j[2] * j[7] - j[1] * j[8],
                     t9 = j[1] * j[5] - j[2] * j[4];
        jbn[9 * n + q] = det;
        jbn[10 * n + q] = inv;
        jbn[q] = t1 * inv; jbn[n + q] = -t2 * inv; jbn[2 * n + q] = t3 * inv;
        jbn[3 * n + q] = -t4 * inv; jbn[4 * n + q] = t5 * inv; jbn[5 * n + q] = -t6 * inv;
        jbn[6 * n + q] = t7 * inv; jbn[7 * n + q] = -t8 * inv; jbn[8 * n + q] = t9 * inv;
    }
    return 0;
}

int orc_step(const orc_step_params *p, double *um0, double *phi,
             const double *jbn, const double *mask,
             const double *dxyzsgd, const double *ratios) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 6 || ny < 6 || nz < 6) return 1;
    for (int a = 0; a < 3; ++a) if (!scheme_ok(p->scheme[a])) return 1;
    const size_t n = (size_t)nx * ny * nz;
    const double M = p->mach, dt = p->dt;
    std::vector<double> um(5 * n), um1(5 * n), u(3 * n), pres(n), temp(n), dvel(9 * n), dtemp(3 * n),
        amut(n), vis(n), fl(6 * n), rs(n), rsv(n);
    /* the state handed in is um0; the primitive variables follow from it as
     * in varc_to_varnc (src/MSVSingle/herramientas_incomp2.f90:16-27) */
    for (size_t q = 0; q < n; ++q) {
        temp[q] = um0[4 * n + q];
        pres[q] = um0[q] / (M * M);
        u[q] = um0[n + q] / um0[q];
        u[n + q] = um0[2 * n + q] / um0[q];
        u[2 * n + q] = um0[3 * n + q] / um0[q];
    }
    const int g = p->ls_ghost;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    const size_t ng = (size_t)nxg * nyg * nzg;
    std::vector<double> phig0, phiA, phiB, velg, jbng, rsg;
    if (p->level_set) {
        phig0.assign(ng, 0.0); phiA.assign(ng, 0.0); phiB.assign(ng, 0.0);
        velg.assign(3 * ng, 0.0); jbng.assign(11 * ng, 0.0); rsg.assign(ng, 0.0);
        for (int c : {0, 4, 8}) {
            orc_to_ghost(&jbng[c * ng], jbn + c * n, g, nx, ny, nz);
            orc_mirror_ghost(&jbng[c * ng], g, nx, ny, nz, 1.0);
        }
        /* padded and mirrored as advect_CUDA does (lsTransportEc.cu:91-127) */
        orc_to_ghost(phig0.data(), phi, g, nx, ny, nz);
        orc_mirror_ghost(phig0.data(), g, nx, ny, nz, 1.0);
    }
    std::memcpy(um.data(), um0, 5 * n * sizeof(double));   /* rungek_ico.f90:68-76 */
    for (int s = 1; s <= 3; ++s) {
        /* level set: TVD-RK3 stage s of cuAdvectLsJB (lsTransportEc.cu:201-418,
         * extrapol.cu:155-212) with the velocity of this substep, so that the
         * level set advances with the flow in one SSP-RK3 step */
        if (p->level_set) {
            for (int d = 0; d < 3; ++d) {
                orc_to_ghost(&velg[d * ng], &u[d * n], g, nx, ny, nz);
                orc_mirror_ghost(&velg[d * ng], g, nx, ny, nz, 1.0);
            }
            const double *cur = s == 1 ? phig0.data() : (s == 2 ? phiA.data() : phiB.data());
            orc_weno_rhs(rsg.data(), cur, velg.data(), jbng.data(), p->h[0], p->h[1], p->h[2],
                         nxg, nyg, nzg, p->ref_bugs);
            for (size_t q = 0; q < ng; ++q) {
                if (s == 1) phiA[q] = phig0[q] - dt * rsg[q];
                else if (s == 2) phiB[q] = 0.75 * phig0[q] + 0.25 * (phiA[q] - dt * rsg[q]);
                else phiA[q] = (phig0[q] + 2.0 * (phiB[q] - dt * rsg[q])) / 3.0;
            }
            if (s == 3) orc_from_ghost(phi, phiA.data(), g, nx, ny, nz);
        }
        orc_cudaDeriv(p->scheme, dvel.data(), dtemp.data(), u.data(), temp.data(),
                      p->h[0], p->h[1], p->h[2], nx, ny, nz);
        if (p->sgs_model == 2)
            orc_sgs_sf(nx, ny, nz, u.data(), dvel.data(), jbn, dxyzsgd, ratios, p->amu0, amut.data());
        else if (p->sgs_model == 1)
            orc_sgs_smag(nx, ny, nz, dvel.data(), jbn, dxyzsgd, p->cs, amut.data());
        else
            std::fill(amut.begin(), amut.end(), 0.0);
        orc_viscosidad((int)n, amut.data(), p->c4, vis.data());
        for (int m = 1; m <= 5; ++m) {
            double *e = &fl[0], *f = &fl[n], *gg = &fl[2 * n], *ev = &fl[3 * n], *fv = &fl[4 * n], *gv = &fl[5 * n];
            orc_flujos(m, nx, ny, nz, e, f, gg, ev, fv, gv, um.data(), u.data(), pres.data(),
                       dvel.data(), jbn, vis.data());
            orc_cuDivergence(p->scheme, rs.data(), rsv.data(), e, f, gg, ev, fv, gv, jbn,
                             p->h[0], p->h[1], p->h[2], nx, ny, nz);
            double *o = &um1[(m - 1) * n];
            const double *a0 = um0 + (m - 1) * n, *a = &um[(m - 1) * n];
            for (size_t q = 0; q < n; ++q) {
                if (s == 1)      /* rungek_ico.f90:89-90 */
                    o[q] = a0[q] + dt * (rs[q] + rsv[q]);
                else if (s == 2) /* :153-154 */
                    o[q] = 0.75 * a0[q] + 0.25 * a[q] + 0.25 * dt * (rs[q] + rsv[q]);
                else             /* :217-220 */
                    o[q] = (1.0 / 3.0) * a0[q] + (2.0 / 3.0) * a[q] + (2.0 / 3.0) * dt * (rs[q] + rsv[q]);
            }
        }
        if (p->bc_walls) orc_bc_walls(um1.data(), nx, ny, nz);   /* rungek_ico.f90:98-100 */
        /* rushton(s) at dto, dto + dt/2, dto + dt (rungek_ico.f90:102;
         * rush_ruth_me.f90:52-54) */
        if (p->imp.on) {
            if (!p->xyz) return 1;
            const double ts = p->time + (s == 1 ? 0.0 : (s == 2 ? 0.5 * dt : dt));
            orc_impeller_force(um1.data(), p->xyz, &p->imp, ts, nx, ny, nz, nullptr);
        }
        /* varc_to_varnc, clip to [-6,6], mask, varc_to_varnc
         * (rungek_ico.f90:104-124, herramientas_incomp2.f90:16-27) */
        for (size_t q = 0; q < n; ++q) {
            double r = um1[q];
            temp[q] = um1[4 * n + q];
            pres[q] = r / (M * M);
            for (int d = 0; d < 3; ++d) {
                double v = um1[(d + 1) * n + q] / r;
                v = std::fmin(6.0, v);
                v = std::fmax(-6.0, v);
                um1[(d + 1) * n + q] = v * r * mask[q];
            }
            pres[q] = um1[q] / (M * M);
            for (int d = 0; d < 3; ++d) u[d * n + q] = um1[(d + 1) * n + q] / um1[q];
            temp[q] = um1[4 * n + q];
        }
        /* rebuild the conserved variables after the advectLevelSet call site,
         * rungek_ico.f90:127-138 */
        for (size_t q = 0; q < n; ++q) {
            um1[q] = pres[q] * M * M;
            um1[n + q] = u[q] * um1[q];
            um1[2 * n + q] = u[n + q] * um1[q];
            um1[3 * n + q] = u[2 * n + q] * um1[q];
        }
        std::memcpy(um.data(), um1.data(), 5 * n * sizeof(double));
    }
    /* the compact filter every filter_every-th step, counting from the first
     * (itf = 1, 10, 19, ...: rungek_ico.f90:269-276) */
    if (p->filter_every > 0 && p->step_index % p->filter_every == 0)
        if (orc_filtrado(um1.data(), jbn, p->cfilt, nx, ny, nz)) return 1;
    std::memcpy(um0, um1.data(), 5 * n * sizeof(double));   /* rungek_ico.f90:278 */
    return 0;
}

} // extern "C"
