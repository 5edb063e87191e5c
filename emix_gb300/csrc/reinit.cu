// reinit.cu -- Sussman reinitialisation of the level set, the device form of
// cuReinitLsJB (src/LevelSet/lsTransportEc.cu:420-676) with the right-hand
// side reini_RS_WENOJB (src/LevelSet/lsTools.cu:824-902):
//
//   per iteration: mirror the ghost layers of phi, phi0 = phi, then three
//   TVD-RK3 stages of  d(phi)/dtau = -S(phi0) (|grad phi| - 1),
//   S = phi0 / sqrt(phi0^2 + dmin^2),  dtau = deltamin / 2,
//   |grad phi| by the Godunov upwinding of the left- and right-biased WENO5
//   derivatives (PhiDevPlus/MinusParameterJB, lsTools.cu:587-770).
//
// One fused kernel per stage: both WENO5 reconstructions of each direction
// (away from the padded grid's edges from six shared differences, their
// second differences and four shared scaled third differences, weno5s), the
// Godunov combination, the speed and the stage update; stages ping-pong
// between two scratch fields so that stencil reads never meet a write.
#include "weno_march.cuh"

namespace emix {

namespace {

struct ReinitArgs {
    const double *src;    // field the derivatives are taken of
    const double *phi;    // iteration start (the TVD combination's phi_n)
    const double *phi0;   // sign field
    const double *jbn;    // padded, 11 components (1, 5, 9 read)
    const double *dmins;  // padded smoothing widths
    double *out;
    int nxg, nyg, nzg;
    double sx, sy, sz, dt;
    int stage, ref_bugs;
};

// max(x, 0) and max(-x, 0) by the sign bit; x*x of the larger of two
// non-negative doubles (their bit patterns order as integers)
EMIX_DEV double pos_part(double x) { return __double_as_longlong(x) > 0 ? x : 0.0; }
EMIX_DEV double neg_mag(double x) { return __double_as_longlong(x) < 0 ? -x : 0.0; }
EMIX_DEV double sq_of_larger(double a, double b) {
    const double m = __double_as_longlong(a) >= __double_as_longlong(b) ? a : b;
    return m * m;
}

EMIX_DEV double bd(const double *f, long base, long s, int p) {
    return p == 0 ? f[base + s] - f[base] : f[base + p * s] - f[base + (p - 1) * s];
}

__global__ void __launch_bounds__(256) k_reinit_stage(ReinitArgs a) {
    const int nxg = a.nxg, nyg = a.nyg, nzg = a.nzg;
    const long sxy = (long)nxg * nyg, ng = sxy * nzg;
    for (long id = blockIdx.x * (long)blockDim.x + threadIdx.x; id < ng; id += (long)gridDim.x * blockDim.x) {
        const int c3[3] = {(int)(id % nxg), (int)((id / nxg) % nyg), (int)(id / sxy)};
        const int L3[3] = {nxg, nyg, nzg};
        const long s3[3] = {1, nxg, sxy};
        const double sc[3] = {a.sx, a.sy, a.sz};
        const double p0 = a.phi0[id];
        const int tsg = (p0 > 0.0) - (p0 < 0.0);   // sign of phi0
        double r = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double C = sc[d] * a.jbn[4 * d * ng + id];
            const double eps = kWenoEps4 * rcp_fast(C * C);
            const long base = id - c3[d] * s3[d];
            const int c = c3[d];
            double am, bp;
            if (c >= 2 && c <= L3[d] - 4) {
                // both reconstructions from the six differences D(c-2..c+3)
                // and their five second differences (weno5a)
                double v[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) v[k] = bd(a.src, base, s3[d], c - 2 + k);
                const double A0 = v[1] - v[0], A1 = v[2] - v[1], A2 = v[3] - v[2], A3 = v[4] - v[3],
                             A4 = v[5] - v[4];
                // the four third differences both sides share, scaled for weno5s
                const double S1 = kSqrt13_3 * (A1 - A0), S2 = kSqrt13_3 * (A2 - A1),
                             S3 = kSqrt13_3 * (A3 - A2), S4 = kSqrt13_3 * (A4 - A3);
                am = C * weno5s(v[2], A0, A1, A2, A3, S1, S2, S3, eps, 6.0);    // phi^-: D(c), A(c-1..c+2)
                bp = C * weno5s(v[3], A4, A3, A2, A1, S4, S3, S2, eps, -6.0);   // phi^+: D(c+1), -A(c+3..c)
            } else {
                int p[5];
                // left-biased (phi^-)
                stencil_left(c, L3[d], p);
                double v5 = bd(a.src, base, s3[d], p[4]);
                if (d == 2 && a.ref_bugs && c == nzg - 1) {
                    // lsTools.cu:636: id_kp2 = id_jm1 at the top layer
                    const long ib = c3[1] == 0 ? id : id - nxg;
                    v5 = a.src[ib] - a.src[ib - sxy];
                }
                am = C * weno5(bd(a.src, base, s3[d], p[0]), bd(a.src, base, s3[d], p[1]),
                               bd(a.src, base, s3[d], p[2]), bd(a.src, base, s3[d], p[3]), v5, eps);
                // right-biased (phi^+)
                stencil_right(c, L3[d], p);
                bp = C * weno5(bd(a.src, base, s3[d], p[0]), bd(a.src, base, s3[d], p[1]),
                               bd(a.src, base, s3[d], p[2]), bd(a.src, base, s3[d], p[3]),
                               bd(a.src, base, s3[d], p[4]), eps);
            }
            // Godunov: phi0 > 0 takes max(max(a-, 0)^2, min(b+, 0)^2), phi0 < 0
            // max(max(b+, 0)^2, min(a-, 0)^2), phi0 = 0 their mean; the larger
            // of two non-negative magnitudes squared, the magnitudes picked by
            // sign and compared as integers (squaring is monotone)
            const double g1 = sq_of_larger(pos_part(am), neg_mag(bp));
            const double g2 = sq_of_larger(pos_part(bp), neg_mag(am));
            r += tsg > 0 ? g1 : (tsg < 0 ? g2 : fma(0.5, g2, 0.5 * g1));
        }
        const double dm = a.dmins[id];
        const double rs = (p0 * rsqrt_fast(fma(p0, p0, dm * dm))) * (sqrt_fast(r) - 1.0);
        const double t = a.src[id] - a.dt * rs;
        double o;
        if (a.stage == 1) o = t;
        else if (a.stage == 2) o = 0.75 * a.phi[id] + 0.25 * t;
        else o = fma(2.0, t, a.phi[id]) * (1.0 / 3.0);
        a.out[id] = o;
    }
}

// ghost layers of a padded field from its own interior (mirror images)
__global__ void k_mirror_inplace(double *f, int g, int nx, int ny, int nz) {
    const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
    const long ng = (long)nxg * nyg * nzg;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < ng; q += (long)gridDim.x * blockDim.x) {
        const int X = (int)(q % nxg), Y = (int)((q / nxg) % nyg), Z = (int)(q / ((long)nxg * nyg));
        if (X >= g && X < nx + g && Y >= g && Y < ny + g && Z >= g && Z < nz + g) continue;
        const long src = (mirror(X, g, nx) + g) + (long)nxg * ((mirror(Y, g, ny) + g) + (long)nyg * (mirror(Z, g, nz) + g));
        f[q] = f[src];
    }
}

int grid_r(long n) { return grid_cap(n, 8); }

} // namespace

int reinit_impl(double *phi, const double *jbn, const double *dmins, double dX, double dY, double dZ,
                int nxg, int nyg, int nzg, int g, double deltamin, int iters, int ref_bugs,
                cudaStream_t st) {
    const long ng = (long)nxg * nyg * nzg;
    double *scr;
    int rc = device_scratch((size_t)3 * ng * sizeof(double), &scr);
    if (rc) return rc;
    double *phi0 = scr, *A = scr + ng, *B = scr + 2 * ng;
    const int nx = nxg - 2 * g, ny = nyg - 2 * g, nz = nzg - 2 * g;
    ReinitArgs a{};
    a.phi = phi; a.phi0 = phi0; a.jbn = jbn; a.dmins = dmins;
    a.nxg = nxg; a.nyg = nyg; a.nzg = nzg;
    a.sx = 1.0 / dX; a.sy = 1.0 / dY; a.sz = 1.0 / dZ; a.dt = 0.5 * deltamin; a.ref_bugs = ref_bugs;
    for (int it = 0; it < iters; ++it) {
        if (g > 0) k_mirror_inplace<<<grid_r(ng), 256, 0, st>>>(phi, g, nx, ny, nz);
        EMIX_CUDA_TRY(cudaMemcpyAsync(phi0, phi, ng * sizeof(double), cudaMemcpyDeviceToDevice, st));
        a.src = phi; a.out = A; a.stage = 1;
        k_reinit_stage<<<grid_r(ng), 256, 0, st>>>(a);
        a.src = A; a.out = B; a.stage = 2;
        k_reinit_stage<<<grid_r(ng), 256, 0, st>>>(a);
        a.src = B; a.out = phi; a.stage = 3;
        k_reinit_stage<<<grid_r(ng), 256, 0, st>>>(a);
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

using namespace emix;

extern "C" {

int emix_reinit_dev(double *phi, const double *jbn, const double *dmins, double deltaX, double deltaY,
                    double deltaZ, int nxg, int nyg, int nzg, int gcells, double deltamin, int iters,
                    int ref_bugs, void *stream) {
    if (!phi || !jbn || !dmins || gcells < 0 || nxg - 2 * gcells < 1 || nyg - 2 * gcells < 1 ||
        nzg - 2 * gcells < 1 || nxg < 4 || nyg < 4 || nzg < 4 || iters < 0 || !(deltaX > 0) ||
        !(deltaY > 0) || !(deltaZ > 0) || (ref_bugs != 0 && ref_bugs != 1))
        return EMIX_ERR_ARG;
    return reinit_impl(phi, jbn, dmins, deltaX, deltaY, deltaZ, nxg, nyg, nzg, gcells, deltamin, iters,
                       ref_bugs, (cudaStream_t)stream);
}

} // extern "C"
