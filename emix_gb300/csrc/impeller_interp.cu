// impeller_interp.cu -- the blade-edge interpolation of rushton(sub_step)
// (src/Geometry/rush_ruth_me.f90:97-185 with getInterpolData :302-517 and
// getMatrix :243-299).
//
// For every blade, the cells next to it in the (x, y) plane of the first z
// layer get the velocity of the plane through three points: the nearest point
// on a blade face (moving with the blade) and two neighbour cells on the outer
// side.  The reference visits the cells blade by blade in k, j, i order and a
// cell may read a neighbour updated before it, so the update keeps that order:
//   k_interp_geom   (parallel)  per blade and plane cell: flag, face, points,
//                               the 3x3 interpolation matrix
//   k_interp_list   (a block per blade)  the flagged cells in j, i order; a
//                               cell without a face within reach takes the
//                               face of the flagged cell before it, as the
//                               reference's loop does
//   k_interp_apply  (a thread per z layer) blades in order, cells in list
//                               order, in place on the substep's output
// It runs after the RK update of the substep; the reference interpolates
// before the conversions, which on these cells (no clip, mask 1) differ from
// the values used here by rounding only.
#include "plan.cuh"

namespace emix {

namespace {

struct Plane4 {
    double A[4], B[4], D[4];
};

EMIX_DEV Plane4 blade_planes(const ImpGeom &g, const double *cs, int b) {
    const double c = cs[2 * b], sn = cs[2 * b + 1];
    Plane4 P;
    P.A[0] = -sn; P.B[0] = c;  P.D[0] = -g.half_thick;
    P.A[1] = sn;  P.B[1] = -c; P.D[1] = -g.half_thick;
    P.A[2] = c;   P.B[2] = sn; P.D[2] = -g.r2;
    P.A[3] = -c;  P.B[3] = -sn; P.D[3] = g.r1;
    return P;
}

EMIX_DEV double pl(const Plane4 &P, int q, double x, double y) {
    return __dadd_rn(__dadd_rn(__dmul_rn(P.A[q], x), __dmul_rn(P.B[q], y)), P.D[q]);
}

EMIX_DEV bool inside2d(const Plane4 &P, double x, double y) {
    return pl(P, 0, x, y) <= 0.0 && pl(P, 1, x, y) <= 0.0 && pl(P, 2, x, y) <= 0.0 && pl(P, 3, x, y) <= 0.0;
}

// geometry of flagged cell (i, j) with face pq: neighbours and matrix
EMIX_DEV void cell_geometry(const ImpInterpArgs &a, const Plane4 &P, int pq, int i, int j, double *geo,
                            int *nb) {
    const int nx = a.nx;
    const double *X = a.xyz, *Y = a.xyz + a.n;
    const long id = i + (long)nx * j;
    const double x = X[id], y = Y[id];
    const double Ag = P.A[pq], Bg = P.B[pq], Dg = P.D[pq];
    const double tt = -(Dg + x * Ag + y * Bg) / (Ag * Ag + Bg * Bg);
    const double pi = 2.0 * acos(0.0);
    const double angle = acos(Ag) / sqrt(Ag * Ag + Bg * Bg);
    const int sA = Ag >= 0.0 ? 1 : -1, sB = Bg >= 0.0 ? 1 : -1;
    int a1i, a1j, a2i, a2j;
    if ((angle >= pi / 6.0 && angle <= pi / 3.0) || (angle >= 2.0 * pi / 3.0 && angle <= 5.0 * pi / 6.0)) {
        a1i = i + sA; a1j = j; a2i = i; a2j = j + sB;
    } else if (angle <= pi / 6.0 || angle >= 5.0 * pi / 6.0) {
        a1i = i + sA; a1j = j; a2i = i + sA; a2j = j + sB;
    } else {
        a1i = i; a1j = j + sB; a2i = i + sA; a2j = j + sB;
    }
    const long e1 = a1i + (long)nx * a1j, e2 = a2i + (long)nx * a2j;
    const double p1x = x + tt * Ag, p1y = y + tt * Bg;
    const double p2x = X[e1], p2y = Y[e1], p3x = X[e2], p3y = Y[e2];
    const double det = p2x * p3y - p3x * p2y + p1x * p2y - p1x * p3y + p3x * p1y - p2x * p1y;
    geo[0] = (p2x * p3y - p3x * p2y) / det;
    geo[1] = (p3x * p1y - p1x * p3y) / det;
    geo[2] = (p1x * p2y - p2x * p1y) / det;
    geo[3] = (p2y - p3y) / det;
    geo[4] = (p3y - p1y) / det;
    geo[5] = (p1y - p2y) / det;
    geo[6] = (p3x - p2x) / det;
    geo[7] = (p1x - p3x) / det;
    geo[8] = (p2x - p1x) / det;
    geo[9] = p1x;
    geo[10] = p1y;
    nb[0] = (int)e1;
    nb[1] = (int)e2;
}

} // namespace

__global__ void k_interp_geom(ImpInterpArgs a) {
    const int nx = a.nx, ny = a.ny;
    const long n2 = (long)nx * ny;
    const double *X = a.xyz, *Y = a.xyz + a.n;
    const double *cs = a.clock + 2 + 2 * (a.stage - 1) * kImpMaxBlades;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < a.g.nblades * n2;
         t += (long)gridDim.x * blockDim.x) {
        const int b = (int)(t / n2);
        const long q = t - b * n2;
        const int i = (int)(q % nx), j = (int)(q / nx);
        const Plane4 P = blade_planes(a.g, cs, b);
        int st = 0;
        if (i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1 && !inside2d(P, X[q], Y[q]) &&
            (inside2d(P, X[q + 1], Y[q + 1]) || inside2d(P, X[q - 1], Y[q - 1]) ||
             inside2d(P, X[q + nx], Y[q + nx]) || inside2d(P, X[q - nx], Y[q - nx]))) {
            st = 2;   // flagged, face not found yet
            for (int pq = 0; pq < 4; ++pq) {
                const double v = pl(P, pq, X[q], Y[q]);
                if (v >= 0.0 && v <= a.rango) {
                    cell_geometry(a, P, pq, i, j, a.geo + (b * n2 + q) * 11, a.nb + 2 * (b * n2 + q));
                    a.face[b * n2 + q] = (signed char)pq;
                    st = 1;
                    break;
                }
            }
        }
        a.status[b * n2 + q] = (unsigned char)st;
    }
}

// one block per blade: the flagged cells in q = i + nx j order, and the faces
// of cells that found none
__global__ void __launch_bounds__(1024) k_interp_list(ImpInterpArgs a) {
    const int b = blockIdx.x;
    const long n2 = (long)a.nx * a.ny;
    const unsigned char *st = a.status + b * n2;
    int *list = a.list + b * n2;
    __shared__ int base;
    __shared__ int warp_tot[32];
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (long c0 = 0; c0 < n2; c0 += blockDim.x) {
        const long q = c0 + threadIdx.x;
        const int f = (q < n2 && st[q] != 0) ? 1 : 0;
        // block-wide exclusive scan of f
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int v = f;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) warp_tot[wid] = v;
        __syncthreads();
        if (wid == 0) {
            int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += u;
            }
            warp_tot[lane] = w;   // inclusive over warps
        }
        __syncthreads();
        const int excl = v - f + (wid > 0 ? warp_tot[wid - 1] : 0);
        if (f) list[base + excl] = (int)q;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) base += excl + f;
        __syncthreads();
    }
    const int cnt = base;
    if (threadIdx.x == 0) a.count[b] = cnt;
    // cells without a face of their own take the face of the last earlier
    // flagged cell that has one (the reference's loop keeps Agen, Bgen, Dgen)
    const double *cs = a.clock + 2 + 2 * (a.stage - 1) * kImpMaxBlades;
    const Plane4 P = blade_planes(a.g, cs, b);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int q = list[e];
        if (a.status[b * n2 + q] != 2) continue;
        int pq = -1;
        for (int f = e - 1; f >= 0; --f) {
            const int qf = list[f];
            if (a.status[b * n2 + qf] == 1) { pq = a.face[b * n2 + qf]; break; }
        }
        if (pq >= 0) cell_geometry(a, P, pq, q % a.nx, q / a.nx, a.geo + (b * n2 + q) * 11,
                                   a.nb + 2 * (b * n2 + q));
        a.face[b * n2 + q] = (signed char)pq;   // -1: left alone
    }
}

// one thread per z layer: blades in order, cells in list order
__global__ void k_interp_apply(ImpInterpArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nz) return;
    const long n = a.n, n2 = (long)a.nx * a.ny;
    const double *X = a.xyz, *Y = a.xyz + n, *Z = a.xyz + 2 * n;
    double *um = a.out;
    for (int b = 0; b < a.g.nblades; ++b) {
        const int cnt = a.count[b];
        for (int e = 0; e < cnt; ++e) {
            const int q = a.list[b * n2 + e];
            if (a.face[b * n2 + q] < 0) continue;
            const long id = q + n2 * k;
            const double z = Z[id];
            if (!(z >= a.g.z1 && z <= a.g.z2)) continue;
            const double *m = a.geo + (b * n2 + q) * 11;
            const int *nb = a.nb + 2 * (b * n2 + q);
            const double2 uv = impeller_velocity(a.g.omega, m[9], m[10]);
            const long e1 = nb[0] + n2 * k, e2 = nb[1] + n2 * k;
            const double r = um[id], mk = a.mask[id];
            for (int d = 1; d <= 2; ++d) {
                const double ub = d == 1 ? uv.x : uv.y;
                const double ua = um[d * n + e1] / um[e1], uc = um[d * n + e2] / um[e2];
                const double cb1 = m[0] * ub + m[1] * ua + m[2] * uc;
                const double cb2 = m[3] * ub + m[4] * ua + m[5] * uc;
                const double cb3 = m[6] * ub + m[7] * ua + m[8] * uc;
                double vel = cb1 + X[id] * cb2 + Y[id] * cb3;
                // the conversions of the substep (clip, mask, rebuild)
                vel = fmax(-6.0, fmin(6.0, vel)) * mk;
                um[d * n + id] = vel * r;
                a.u[(d - 1) * n + id] = vel;
            }
        }
    }
}

} // namespace emix
