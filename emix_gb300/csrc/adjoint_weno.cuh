// adjoint_weno.cuh -- adjoint of one level-set TVD stage (weno_march_body in
// weno_march.cuh), of the mirrored padding, and of the tank objective.
#pragma once

#include "adjoint_kernels.cuh"

namespace emix {

struct WenoAdjArgs {
    const double *phi;       // the stage's input (padded)
    const double *lout;      // adjoint of its output: padded (stages 1, 2) or interior (stage 3)
    double *lphi0;           // adjoint of phi_0 (padded), accumulated (stages 2, 3)
    double *lphiin;          // adjoint of the input (padded), accumulated
    double *lD;              // 3 padded fields: adjoint of the backward differences (atomic)
    double *lu;              // 3 interior fields: adjoint of the velocity (atomic)
    const double *vel, *wce;      // wce: (C, E) pairs as in WenoArgs
    int nxg, nyg, nzg, g;
    int r0[3], rn[3];
    double dt;
    int stage;
};

// backward difference D(p) = phi(p) - phi(p-1), D(0) = phi(1) - phi(0)
EMIX_DEV double bdiff(const double *phi, long base, long s, int p) {
    return p == 0 ? phi[base + s] - phi[base] : phi[base + p * s] - phi[base + (p - 1) * s];
}

__global__ void __launch_bounds__(256) k_adj_weno(WenoAdjArgs A) {
    const int nxg = A.nxg, nyg = A.nyg, nzg = A.nzg, g = A.g;
    const int nx = nxg - 2 * g, ny = nyg - 2 * g, nz = nzg - 2 * g;
    const long ng = (long)nxg * nyg * nzg, nv = (long)nx * ny * nz;
    const long cnt = (long)A.rn[0] * A.rn[1] * A.rn[2];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < cnt; t += (long)gridDim.x * blockDim.x) {
        const int X = A.r0[0] + (int)(t % A.rn[0]);
        const int Y = A.r0[1] + (int)((t / A.rn[0]) % A.rn[1]);
        const int Z = A.r0[2] + (int)(t / ((long)A.rn[0] * A.rn[1]));
        const long id = X + (long)nxg * (Y + (long)nyg * Z);
        double lo;
        if (A.stage == 3) {
            const int I = X - g, J = Y - g, K = Z - g;
            if (I < 0 || I >= nx || J < 0 || J >= ny || K < 0 || K >= nz) continue;
            lo = A.lout[I + (long)nx * (J + (long)ny * K)];
        } else {
            lo = A.lout[id];
        }
        if (lo == 0.0) continue;
        // stage 1: phi_s - dt rs; 2: 0.75 phi_0 + 0.25 (phi_s - dt rs);
        // 3: (phi_0 + 2 (phi_s - dt rs)) / 3   (extrapol.cu:155-212)
        double lrs;
        if (A.stage == 1) {
            A.lphiin[id] += lo;
            lrs = -A.dt * lo;
        } else if (A.stage == 2) {
            A.lphi0[id] += 0.75 * lo;
            A.lphiin[id] += 0.25 * lo;
            lrs = -0.25 * A.dt * lo;
        } else {
            A.lphi0[id] += lo / 3.0;
            A.lphiin[id] += 2.0 * lo / 3.0;
            lrs = -(2.0 / 3.0) * A.dt * lo;
        }
        const long iv = mirror(X, g, nx) + (long)nx * (mirror(Y, g, ny) + (long)ny * mirror(Z, g, nz));
        const int c3[3] = {X, Y, Z};
        const int L3[3] = {nxg, nyg, nzg};
        const long s3[3] = {1, nxg, (long)nxg * nyg};
        for (int d = 0; d < 3; ++d) {
            const double ud = A.vel[d * nv + iv];
            const double2 ce = weno_scale(A.wce, d, nv, iv);
            const double mx = ce.x, ex = ce.y;
            int p[5];
            if (__double_as_longlong(ud) >= 0) stencil_left(c3[d], L3[d], p);
            else stencil_right(c3[d], L3[d], p);
            const long base = id - c3[d] * s3[d];
            double v[5], gr[5];
            for (int k = 0; k < 5; ++k) v[k] = bdiff(A.phi, base, s3[d], p[k]);
            const double W = weno5_grad(v[0], v[1], v[2], v[3], v[4], ex, gr);
            atomicAdd(&A.lu[d * nv + iv], lrs * mx * W);
            const double f = lrs * ud * mx;
            for (int k = 0; k < 5; ++k)
                if (gr[k] != 0.0) atomicAdd(&A.lD[d * ng + base + p[k] * s3[d]], f * gr[k]);
        }
    }
}

// the differences' adjoint onto phi: D(p) = phi(p) - phi(p-1), D(0) = phi(1) - phi(0)
__global__ void k_adj_weno_dphi(const double *lD, double *lphi, int nxg, int nyg, int nzg) {
    const long ng = (long)nxg * nyg * nzg;
    const int L3[3] = {nxg, nyg, nzg};
    const long s3[3] = {1, nxg, (long)nxg * nyg};
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < ng; q += (long)gridDim.x * blockDim.x) {
        const int c3[3] = {(int)(q % nxg), (int)((q / nxg) % nyg), (int)(q / ((long)nxg * nyg))};
        double acc = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double *D = lD + d * ng;
            const int c = c3[d];
            const long s = s3[d];
            acc += c >= 1 ? D[q] : -D[q];
            if (c + 1 <= L3[d] - 1) acc -= D[q + s];
            if (c == 1) acc += D[q - s];
        }
        if (acc != 0.0) lphi[q] += acc;
    }
}

// transpose of the mirrored padding: each interior cell gathers the adjoint
// of every padded cell that mirrors it
__global__ void k_adj_unpad(const double *lpad, double *lint, int g, int nx, int ny, int nz) {
    const long n = (long)nx * ny * nz;
    const int nxg = nx + 2 * g, nyg = ny + 2 * g;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int c3[3] = {(int)(q % nx), (int)((q / nx) % ny), (int)(q / ((long)nx * ny))};
        const int n3[3] = {nx, ny, nz};
        int img[3][3], cnt[3];
        for (int d = 0; d < 3; ++d) {
            const int i = c3[d], m = n3[d];
            cnt[d] = 0;
            img[d][cnt[d]++] = i + g;
            if (i < g) img[d][cnt[d]++] = g - 1 - i;
            if (i >= m - g) img[d][cnt[d]++] = 2 * m + g - 1 - i;
        }
        double acc = 0.0;
        for (int a = 0; a < cnt[0]; ++a)
            for (int b = 0; b < cnt[1]; ++b)
                for (int c = 0; c < cnt[2]; ++c)
                    acc += lpad[img[0][a] + (long)nxg * (img[1][b] + (long)nyg * img[2][c])];
        lint[q] += acc;
    }
}

// ---- tank objective -----------------------------------------------------------
//   J = w_ke sum_{r_in <= r <= r_out} dV |u|^2/2 + w_if sum dV delta_eps(phi) |grad phi|
// with dV = jbn(10) hx hy hz, u = um(2..4)/um(1), grad phi from central
// differences (one-sided at the walls) times the diagonal metric, and the
// cosine smoothed delta of width eps.
struct ObjArgs {
    const double *um, *phi, *xyz, *jbn;
    double h[3];
    double r_in, r_out, eps, w_ke, w_if;
    int nx, ny, nz;
    double *red;           // per-block partial sums of J (gridDim.x of them)
    double *lum, *lphi;    // adjoints (lum stored, lphi accumulated atomically); may be null
};

__global__ void __launch_bounds__(256) k_objective(ObjArgs A) {
    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const long n = (long)nx * ny * nz;
    const double pi = 3.14159265358979323846;
    double jsum = 0.0;
    for (long q0 = blockIdx.x * (long)blockDim.x; q0 < n; q0 += (long)gridDim.x * blockDim.x) {
        const long q = q0 + threadIdx.x;
        if (q >= n) continue;
        const double dV = A.jbn[9 * n + q] * A.h[0] * A.h[1] * A.h[2];
        // kinetic energy in the annulus
        const double x = A.xyz[q], y = A.xyz[n + q];
        const double rr = sqrt(x * x + y * y);
        const double w = (rr >= A.r_in && rr <= A.r_out) ? A.w_ke * dV : 0.0;
        const double r = A.um[q];
        const double u1 = A.um[n + q] / r, u2 = A.um[2 * n + q] / r, u3 = A.um[3 * n + q] / r;
        const double uu = u1 * u1 + u2 * u2 + u3 * u3;
        jsum += 0.5 * w * uu;
        if (A.lum) {
            A.lum[q] = -w * uu / r;
            A.lum[n + q] = w * u1 / r;
            A.lum[2 * n + q] = w * u2 / r;
            A.lum[3 * n + q] = w * u3 / r;
            A.lum[4 * n + q] = 0.0;
        }
        // interface area
        const double ph = A.phi[q];
        if (fabs(ph) >= A.eps) continue;
        const int c3[3] = {(int)(q % nx), (int)((q / nx) % ny), (int)(q / ((long)nx * ny))};
        const int n3[3] = {nx, ny, nz};
        const long s3[3] = {1, nx, (long)nx * ny};
        const double jd[3] = {A.jbn[q], A.jbn[4 * n + q], A.jbn[8 * n + q]};
        double gd[3], cp[3], cm[3];
        long ip[3], im[3];
        for (int d = 0; d < 3; ++d) {
            const int c = c3[d];
            ip[d] = c < n3[d] - 1 ? q + s3[d] : q;
            im[d] = c > 0 ? q - s3[d] : q;
            const double inv = (c > 0 && c < n3[d] - 1) ? 0.5 / A.h[d] : 1.0 / A.h[d];
            cp[d] = jd[d] * inv;
            cm[d] = -jd[d] * inv;
            gd[d] = cp[d] * A.phi[ip[d]] + cm[d] * A.phi[im[d]];
        }
        const double gn = sqrt(gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2] + 1e-300);
        const double arg = pi * ph / A.eps;
        const double del = (1.0 + cos(arg)) / (2.0 * A.eps);
        jsum += A.w_if * dV * del * gn;
        if (A.lphi) {
            const double ddel = -pi * sin(arg) / (2.0 * A.eps * A.eps);
            atomicAdd(&A.lphi[q], A.w_if * dV * ddel * gn);
            const double f = A.w_if * dV * del / gn;
            for (int d = 0; d < 3; ++d) {
                atomicAdd(&A.lphi[ip[d]], f * gd[d] * cp[d]);
                atomicAdd(&A.lphi[im[d]], f * gd[d] * cm[d]);
            }
        }
    }
    block_sum_store(jsum, A.red);
}

} // namespace emix
