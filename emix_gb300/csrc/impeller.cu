// impeller.cu -- the impeller clock (blade angles of a step's three substeps)
// and a standalone form of the impeller forcing.
#include "impeller.cuh"

namespace emix {

__global__ void k_imp_clock(ImpClockArgs a) {
    if (blockIdx.x == 0 && threadIdx.x == 0) imp_clock_tick(a);
}

__global__ void k_imp_flags(const double *xyz, ImpGeom g, long n, unsigned char *flag) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double x = xyz[q], y = xyz[n + q], z = xyz[2 * n + q];
        const double r2 = x * x + y * y;
        const double m = 1.0 + 1e-9;
        const double rb = (g.r2 * g.r2 + g.half_thick * g.half_thick) * m * m;
        bool c = false;
        if (z >= g.z1 && z <= g.z2 && r2 <= rb) c = true;
        if (z >= g.hub_z1 && z <= g.hub_z2 && r2 <= g.hub_r * g.hub_r * m * m) c = true;
        if (z >= g.shaft_z0 && z <= g.shaft_z1 && r2 <= g.shaft_r * g.shaft_r * m * m) c = true;
        flag[q] = c ? 1 : 0;
    }
}

namespace {

__global__ void k_impeller_force(double *um, const double *xyz, ImpGeom g, const double *cs, long n,
                                 double *mask) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        double v[5] = {um[q], um[n + q], um[2 * n + q], um[3 * n + q], 0.0};
        double m;
        impeller_force_cell(g, cs, xyz[q], xyz[n + q], xyz[2 * n + q], v, &m);
        um[n + q] = v[1];
        um[2 * n + q] = v[2];
        um[3 * n + q] = v[3];
        if (mask) mask[q] = m;
    }
}

} // namespace

bool impeller_ok(const ImpGeom &g) {
    return !g.on || (g.nblades >= 0 && g.nblades <= kImpMaxBlades);
}

} // namespace emix

using namespace emix;

extern "C" {

int emix_impeller_force_dev(double *um, const double *xyz, const emix_impeller *imp, double t,
                            int nx, int ny, int nz, double *mask, void *stream) {
    if (!um || !xyz || !imp || nx < 1 || ny < 1 || nz < 1) return EMIX_ERR_ARG;
    ImpGeom g{1, imp->nblades, imp->omega, imp->theta0, imp->r1, imp->r2, imp->z1, imp->z2,
              imp->half_thick, imp->hub_r, imp->hub_z1, imp->hub_z2, imp->shaft_r, imp->shaft_z0,
              imp->shaft_z1};
    if (!impeller_ok(g)) return EMIX_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    // blade angles at t through the clock kernel (k = 0, dt = 0, t0 = t)
    double *clk = nullptr;
    EMIX_CUDA_TRY(cudaMallocAsync(&clk, kImpClockLen * sizeof(double), st));
    const double head[2] = {t, 0.0};
    cudaError_t e = cudaMemcpyAsync(clk, head, sizeof head, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        ImpClockArgs ca{clk, 0.0, g};
        k_imp_clock<<<1, 32, 0, st>>>(ca);
        const long n = (long)nx * ny * nz;
        k_impeller_force<<<grid_cap(n, 8), 256, 0, st>>>(um, xyz, g, clk + 2, n, mask);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(clk, st);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(e, "emix_impeller_force_dev", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    return EMIX_OK;
}

} // extern "C"
