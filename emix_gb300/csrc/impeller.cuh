// impeller.cuh -- the rotating impeller as a volumetric forcing: the linked
// rushton(sub_step) without its blade-edge interpolation
// (src/Geometry/rush_ruth_me.f90:2-108; makeAspa :519-593; addMaskCil and
// addAngularVel, src/Geometry/rotating.f90:110-205).
//
// Per cell: the impeller mask m (0 inside a blade, the hub disc or the shaft,
// 1 elsewhere) at the substep's time, then
//   um2 = ((1-m) ue + m um2/um1) um1,  um3 likewise with ve,  um4 = m um4,
// with (ue, ve) the rigid rotation at the cell.  The blade angles of the three
// substeps of a step are computed once per step on the device (k_imp_clock)
// from t = t0 + k dt, so graph replays advance the impeller.
//
// The plane tests and the angle arithmetic use explicitly rounded operations
// (no contraction) so the mask is decided exactly as written.
#pragma once

#include "common.cuh"

namespace emix {

constexpr int kImpMaxBlades = 16;
// clock buffer: [0] t0, [1] steps taken, then per substep s and blade b the
// pair (cos, sin) of the blade angle at index 2 + 2 (s kImpMaxBlades + b)
constexpr int kImpClockLen = 2 + 2 * 3 * kImpMaxBlades;

struct ImpGeom {
    int on, nblades;
    double omega, theta0;
    double r1, r2, z1, z2, half_thick;
    double hub_r, hub_z1, hub_z2;
    double shaft_r, shaft_z0, shaft_z1;
};

struct ImpClockArgs {
    double *clock;
    double dt;
    ImpGeom g;
};

// mask of one cell; cs = the (cos, sin) pairs of this substep's blades
EMIX_DEV double impeller_mask(const ImpGeom &g, const double *cs, double x, double y, double z) {
    double m = 1.0;
    if (z >= g.z1 && z <= g.z2) {
        for (int b = 0; b < g.nblades; ++b) {
            const double c = cs[2 * b], sn = cs[2 * b + 1];
            const double cx = __dmul_rn(c, x), cy = __dmul_rn(c, y);
            const double sx = __dmul_rn(sn, x), sy = __dmul_rn(sn, y);
            const double pl1 = __dadd_rn(__dadd_rn(-sx, cy), -g.half_thick);
            const double pl2 = __dadd_rn(__dadd_rn(sx, -cy), -g.half_thick);
            const double pl3 = __dadd_rn(__dadd_rn(cx, sy), -g.r2);
            const double pl4 = __dadd_rn(__dadd_rn(-cx, -sy), g.r1);
            if (pl1 <= 0.0 && pl2 <= 0.0 && pl3 <= 0.0 && pl4 <= 0.0) m = 0.0;
        }
    }
    const bool hub = z >= g.hub_z1 && z <= g.hub_z2;
    const bool shaft = z >= g.shaft_z0 && z <= g.shaft_z1;
    if (hub || shaft) {
        // radio <= R decided on sqrt(x^2 + y^2) as written; the square is only
        // a filter (with a margin far above rounding) that skips the root
        const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
        const double R = fmax(hub ? g.hub_r : 0.0, shaft ? g.shaft_r : 0.0) * (1.0 + 1e-12);
        if (r2 <= R * R) {
            const double radio = sqrt(r2);
            if (hub && radio <= g.hub_r) m = 0.0;
            if (shaft && radio <= g.shaft_r) m = 0.0;
        }
    }
    return m;
}

// body velocity of addAngularVel (rotating.f90:163-186), with its polar angle
// from atan(|y/x|) and its constants for pi
// (kept out of line: it runs only inside the impeller and is heavy)
static __device__ __noinline__ double2 impeller_velocity(double omega, double x, double y) {
    const double radio = sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
    double th;
    if (x != 0.0) th = atan(fabs(y / x));
    else th = 3.1415926 / 2.;
    if (x < 0.0 && y > 0.0) th = 3.141592 - th;
    else if (x < 0.0 && y <= 0.0) th = th + 3.141592;
    else if (x >= 0.0 && y < 0.0) th = 2.0 * 3.141592 - th;
    return make_double2(-1.0 * omega * radio * sin(th), omega * radio * cos(th));
}

// the forcing on the conserved values v[5] of one cell
EMIX_DEV void impeller_force_cell(const ImpGeom &g, const double *cs, double x, double y, double z,
                                  double v[5], double *mask_out) {
    const double m = impeller_mask(g, cs, x, y, z);
    if (mask_out) *mask_out = m;
    // outside the impeller the forcing is the identity (up to the reference's
    // u/rho*rho round trip, which is left out)
    if (m == 1.0) return;
    const double2 uv = impeller_velocity(g.omega, x, y);
    const double ue = uv.x, ve = uv.y;
    const double r = v[0];
    v[1] = ((1.0 - m) * ue + m * (v[1] / r)) * r;
    v[2] = ((1.0 - m) * ve + m * (v[2] / r)) * r;
    v[3] = m * v[3];
}

// t = t0 + k dt at the start of the step; the substeps are at t, t + dt/2,
// t + dt (rush_ruth_me.f90:52-54); then k += 1.  One thread.
EMIX_DEV void imp_clock_tick(const ImpClockArgs &a) {
    const double t0 = a.clock[0], k = a.clock[1];
    const double t = __dadd_rn(t0, __dmul_rn(k, a.dt));
    const int nb = a.g.nblades;
    const double two_pi = 2.0 * 3.14159265358979323846;
    for (int s = 0; s < 3; ++s) {
        const double ts = __dadd_rn(t, s == 0 ? 0.0 : (s == 1 ? 0.5 * a.dt : a.dt));
        for (int b = 0; b < nb; ++b) {
            const double th = __dadd_rn(__dadd_rn(a.g.theta0, __dmul_rn(a.g.omega, ts)),
                                        __dmul_rn((double)b, two_pi / nb));
            double sn, c;
            sincos(th, &sn, &c);
            a.clock[2 + 2 * (s * kImpMaxBlades + b)] = c;
            a.clock[3 + 2 * (s * kImpMaxBlades + b)] = sn;
        }
    }
    a.clock[1] = k + 1.0;
}

__global__ void k_imp_clock(ImpClockArgs a);

// the blade-edge interpolation (impeller_interp.cu)
struct ImpInterpArgs {
    ImpGeom g;
    const double *xyz, *clock, *mask;
    double *out, *u;        // the substep's um output and u output, updated in place
    int nx, ny, nz;
    long n;
    double rango;           // grid diagonal (getInterpolData :357-361)
    int stage, phase;       // phase 0: geometry, 1: lists, 2: apply
    unsigned char *status;  // per blade and plane cell
    signed char *face;
    double *geo;            // 11 per blade and plane cell: matrix, surface point
    int *nb;                // 2 per blade and plane cell: neighbour cells
    int *list, *count;
};
__global__ void k_interp_geom(ImpInterpArgs a);
__global__ void k_interp_list(ImpInterpArgs a);
__global__ void k_interp_apply(ImpInterpArgs a);

// 1 where some blade angle could put the cell inside the impeller (blade
// band within reach of a blade corner, hub disc, shaft), 0 elsewhere: the RK
// kernel tests only flagged cells.  The margin 1e-9 is far above rounding.
__global__ void k_imp_flags(const double *xyz, ImpGeom g, long n, unsigned char *flag);

} // namespace emix
