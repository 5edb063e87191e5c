// adjoint_cells.cuh -- cell-local reverse-mode bodies of the RK3 substep.
//
// Each body takes the adjoint of a forward body's outputs and returns (or
// accumulates) the adjoint of its inputs, differentiating the forward
// arithmetic as written in pointwise.cuh / weno.cuh / impeller.cuh:
//   prim     u = um(2..4)/um(1), pres = um(1)/M^2
//   flux     the 15 projected fluxes of flujos (inviscid + viscous)
//   smag     vis = c4 + (Cs Delta)^2 sqrt(2 S:S)
//   convert  clip to [-6, 6], mask, rebuild (rungek_ico.f90:104-138)
//   impeller rigid rotation inside the impeller (linear in omega)
//   weno5    the WENO5 reconstruction with its nonlinear weights
#pragma once

#include "pointwise.cuh"
#include "weno.cuh"

namespace emix {

// ---- WENO5: value and gradient with respect to the five differences ------
// Same arithmetic as weno5() (weno.cuh), reverse-differentiated by hand:
//   W = v3 + N / (12 S),  N = sum w_k r_k,  S = sum w_k,
//   w_1 = t2 t3, w_2 = 6 t1 t3, w_3 = 3 t1 t2,  t_k = (sigma_k + eps)^2,
//   sigma_k = (13/3) d_k^2 + e_k^2,  r_1 = d_1 + 3 e_1, r_2 = d_2 - 3 e_2,
//   r_3 = d_3 - 3 e_3.
EMIX_DEV double weno5_grad(double v1, double v2, double v3, double v4, double v5, double eps4,
                           double g[5]) {
    constexpr double c13 = 13.0 / 3.0;
    const double d1 = v1 - 2.0 * v2 + v3, e1 = v1 - 4.0 * v2 + 3.0 * v3;
    const double d2 = v2 - 2.0 * v3 + v4, e2 = v2 - v4;
    const double d3 = v3 - 2.0 * v4 + v5, e3 = 3.0 * v3 - 4.0 * v4 + v5;
    const double s1 = c13 * d1 * d1 + e1 * e1 + eps4;
    const double s2 = c13 * d2 * d2 + e2 * e2 + eps4;
    const double s3 = c13 * d3 * d3 + e3 * e3 + eps4;
    const double t1 = s1 * s1, t2 = s2 * s2, t3 = s3 * s3;
    const double w1 = t2 * t3, w2 = 6.0 * t1 * t3, w3 = 3.0 * t1 * t2;
    const double r1 = d1 + 3.0 * e1, r2 = d2 - 3.0 * e2, r3 = d3 - 3.0 * e3;
    const double S = w1 + w2 + w3;
    const double N = w1 * r1 + w2 * r2 + w3 * r3;
    const double iS = rcp_fast(S);
    const double q = iS * (1.0 / 12.0);
    const double W = v3 + N * q;
    // dW = dv3 + q (sum w_k dr_k + sum dw_k (r_k - N/S))
    const double NS = N * iS;
    const double a1 = q * (r1 - NS), a2 = q * (r2 - NS), a3 = q * (r3 - NS);
    // dw: dt1 (6 t3 a2 + 3 t2 a3) + dt2 (t3 a1 + 3 t1 a3) + dt3 (t2 a1 + 6 t1 a2)
    const double lt1 = 6.0 * t3 * a2 + 3.0 * t2 * a3;
    const double lt2 = t3 * a1 + 3.0 * t1 * a3;
    const double lt3 = t2 * a1 + 6.0 * t1 * a2;
    // t_k = s_k^2: ds_k = 2 s_k lt_k; s_k: dd_k 2 c13 d_k, de_k 2 e_k
    const double ls1 = 2.0 * s1 * lt1, ls2 = 2.0 * s2 * lt2, ls3 = 2.0 * s3 * lt3;
    const double ld1 = ls1 * 2.0 * c13 * d1 + q * w1, le1 = ls1 * 2.0 * e1 + 3.0 * q * w1;
    const double ld2 = ls2 * 2.0 * c13 * d2 + q * w2, le2 = ls2 * 2.0 * e2 - 3.0 * q * w2;
    const double ld3 = ls3 * 2.0 * c13 * d3 + q * w3, le3 = ls3 * 2.0 * e3 - 3.0 * q * w3;
    g[0] = ld1 + le1;
    g[1] = -2.0 * ld1 - 4.0 * le1 + ld2 + le2;
    g[2] = 1.0 + ld1 + 3.0 * le1 - 2.0 * ld2 + ld3 + 3.0 * le3;
    g[3] = ld2 - le2 - 2.0 * ld3 - 4.0 * le3;
    g[4] = ld3 + le3;
    return W;
}

// ---- primitive variables ---------------------------------------------------
EMIX_DEV void prim_adj(const double um[4], double inv_m2, const double lu[3], double lp,
                       double lum[4]) {
    const double r = um[0], rr = rcp_fast(r);
    double l0 = lp * inv_m2;
    for (int d = 0; d < 3; ++d) {
        lum[d + 1] += lu[d] * rr;
        l0 -= lu[d] * um[d + 1] * rr * rr;
    }
    lum[0] += l0;
}

// ---- fluxes: lF (15) -> lum(2..5), lu (3), lp, ldvel (9), lvis ---------------
// um = fields 2..5 of the conserved state (rho u, rho v, rho w, T)
EMIX_DEV void flux_adj(const double um[4], const double u[3], double vs, const double dv[9],
                       double j1, double j5, double j9, double JX, double JY, double JZ,
                       const double lF[15], double lum[4], double lu[3], double &lp,
                       double ldv[9], double &lvs) {
    const double um2 = um[0], um3 = um[1], um4 = um[2], um5 = um[3];
    const double u1 = u[0], u2 = u[1], u3 = u[2];
    const double sxx = j1 * dv[0], syy = j5 * dv[4], szz = j9 * dv[8];
    const double sxy = j1 * dv[1] + j5 * dv[3];
    const double sxz = j1 * dv[2] + j9 * dv[6];
    const double syz = j9 * dv[7] + j5 * dv[5];
    const double x0 = lF[0] * JX, y0 = lF[1] * JY, z0 = lF[2] * JZ;
    const double a1 = lF[3] * JX, b1 = lF[4] * JY, c1 = lF[5] * JZ;
    const double a2 = lF[6] * JX, b2 = lF[7] * JY, c2 = lF[8] * JZ;
    const double a3 = lF[9] * JX, b3 = lF[10] * JY, c3 = lF[11] * JZ;
    const double a4 = lF[12] * JX, b4 = lF[13] * JY, c4 = lF[14] * JZ;
    lum[0] += -x0 - a1 * u1 - a2 * u2 - a3 * u3;
    lum[1] += -y0 - b1 * u1 - b2 * u2 - b3 * u3;
    lum[2] += -z0 - c1 * u1 - c2 * u2 - c3 * u3;
    lum[3] += -(a4 * u1 + b4 * u2 + c4 * u3);
    lu[0] += -(a1 * um2 + b1 * um3 + c1 * um4) - a4 * um5;
    lu[1] += -(a2 * um2 + b2 * um3 + c2 * um4) - b4 * um5;
    lu[2] += -(a3 * um2 + b3 * um3 + c3 * um4) - c4 * um5;
    lp += -(a1 + b2 + c3);
    lvs = a1 * 2.0 * sxx + b2 * 2.0 * syy + c3 * 2.0 * szz + (b1 + a2) * sxy + (c1 + a3) * sxz +
          (c2 + b3) * syz;
    const double lsxx = 2.0 * vs * a1, lsyy = 2.0 * vs * b2, lszz = 2.0 * vs * c3;
    const double lsxy = vs * (b1 + a2), lsxz = vs * (c1 + a3), lsyz = vs * (c2 + b3);
    ldv[0] = j1 * lsxx;
    ldv[4] = j5 * lsyy;
    ldv[8] = j9 * lszz;
    ldv[1] = j1 * lsxy;
    ldv[3] = j5 * lsxy;
    ldv[2] = j1 * lsxz;
    ldv[6] = j9 * lsxz;
    ldv[7] = j9 * lsyz;
    ldv[5] = j5 * lsyz;
}

// ---- Smagorinsky: lvis -> ldvel (+=), returns d vis / d Cs * lvis ----------
EMIX_DEV double smag_adj(const double dv[9], double j1, double j5, double j9, double cs,
                         double delta, double lvis, double ldv[9]) {
    const double ux = j1 * dv[0], vx = j1 * dv[1], wx = j1 * dv[2];
    const double uy = j5 * dv[3], vy = j5 * dv[4], wy = j5 * dv[5];
    const double uz = j9 * dv[6], vz = j9 * dv[7], wz = j9 * dv[8];
    const double s12 = 0.5 * (uy + vx), s13 = 0.5 * (uz + wx), s23 = 0.5 * (vz + wy);
    const double ss = ux * ux + vy * vy + wz * wz + 2.0 * (s12 * s12 + s13 * s13 + s23 * s23);
    const double root = sqrt_fast(2.0 * ss);
    const double cd = cs * delta;
    if (root > 0.0) {
        const double lss = lvis * cd * cd * rcp_fast(root);
        const double l12 = 2.0 * lss * s12, l13 = 2.0 * lss * s13, l23 = 2.0 * lss * s23;
        ldv[0] += j1 * 2.0 * ux * lss;
        ldv[4] += j5 * 2.0 * vy * lss;
        ldv[8] += j9 * 2.0 * wz * lss;
        ldv[3] += j5 * l12;   // uy
        ldv[1] += j1 * l12;   // vx
        ldv[6] += j9 * l13;   // uz
        ldv[2] += j1 * l13;   // wx
        ldv[7] += j9 * l23;   // vz
        ldv[5] += j5 * l23;   // wy
    }
    return lvis * 2.0 * cs * delta * delta * root;
}

// ---- RK conversions and impeller -------------------------------------------
// v: values entering the impeller (after the walls); lo (5), lu (3), lp: the
// adjoints of the substep's outputs um1, u, pres.  Returns lv (5) of v and
// adds d/d omega to *lomega.
EMIX_DEV void convert_adj(const RkArgs &a, long q, const double v_in[5], const double lo[5],
                          const double lu[3], double lp, double lv[5], double *lomega) {
    double v[5] = {v_in[0], v_in[1], v_in[2], v_in[3], v_in[4]};
    double m = 1.0, ue1 = 0.0, ve1 = 0.0;
    if (a.imp.on && a.impflag[q]) {
        const long n = a.n;
        const double x = a.xyz[q], y = a.xyz[n + q], z = a.xyz[2 * n + q];
        m = impeller_mask(a.imp, a.clock + 2 + 2 * (a.stage - 1) * kImpMaxBlades, x, y, z);
        if (m != 1.0) {
            const double2 uv = impeller_velocity(1.0, x, y);
            ue1 = uv.x;
            ve1 = uv.y;
            v[1] = a.imp.omega * ue1 * v[0];
            v[2] = a.imp.omega * ve1 * v[0];
            v[3] = 0.0;
        }
    }
    // conversions at v
    const double r = v[0], rr = rcp_fast(r), mk = a.mask[q];
    double lr = lo[0] + lp * a.inv_m2;
    for (int d = 0; d < 3; ++d) {
        const double c = v[d + 1] * rr;
        const double gd = (c > -6.0 && c < 6.0) ? 1.0 : 0.0;
        const double cl = fmax(-6.0, fmin(6.0, c));
        lr += lo[d + 1] * mk * (cl - gd * c) - lu[d] * gd * mk * c * rr;
        lv[d + 1] = lo[d + 1] * gd * mk + lu[d] * gd * mk * rr;
    }
    lv[4] = lo[4];
    lv[0] = lr;
    if (m != 1.0) {
        // inside: v1 = omega ue1 r, v2 = omega ve1 r, v3 = 0
        lv[0] += a.imp.omega * (lv[1] * ue1 + lv[2] * ve1);
        *lomega += r * (lv[1] * ue1 + lv[2] * ve1);
        lv[1] = 0.0;
        lv[2] = 0.0;
        lv[3] = 0.0;
    }
}

// the cell whose combined value field c of wall cell (i,j,k) takes after
// frontera_z, _y, _x (wall_z/y/x in pointwise.cuh), or -1 when a constant
EMIX_DEV long wall_source(const RkArgs &a, int i, int j, int k, int c) {
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (i == 0 || i == nx - 1) {
        if (c >= 1 && c <= 3) return -1;
        i = i == 0 ? 1 : nx - 2;
    }
    if (j == 0 || j == ny - 1) {
        if (c >= 1 && c <= 3) return -1;
        j = j == 0 ? 1 : ny - 2;
    }
    if (k == 0) {
        if (c == 3) return -1;
        k = 1;
    } else if (k >= nz - 2) {
        if (c == 0 || c == 3) return -1;
        k = nz - 3;
    }
    return i + (long)nx * (j + (long)ny * k);
}

} // namespace emix
