// deriv_ops.cu -- derivative-based operators and the reference's drop-in
// symbols cudaDeriv / cuDivergence.
//
// The reference allocates every temporary and copies every field over the
// host link on each call (solver/cuDeriv.cu:545-644,
// solver/cuDivergence.cu:124-187).  Here the device-pointer forms allocate
// nothing but cached scratch, and the host-pointer forms keep a grow-only
// device workspace per device so repeated calls pay only the copies.
#include "deriv.cuh"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

namespace emix {

// ---- error state --------------------------------------------------------
namespace {
thread_local std::string t_last_error;
}

void set_last_error(cudaError_t e, const char *what, const char *file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    t_last_error = buf;
}

void set_last_message(const char *msg) { t_last_error = msg ? msg : ""; }

const char *last_error() { return t_last_error.c_str(); }

// ---- launch helper ------------------------------------------------------
// Block width of the y/z pencil kernels: the one of 128, 64, 32 threads that
// leaves the fewest idle lanes in the last block of a row (ties to the wider),
// e.g. 64 for nx = 192 where 128 would idle a quarter of the threads.
std::atomic<int> g_yz_block{0};   // emix_pencil_set_yz_block: 0 = by the rule below

int yz_block(int nx) {
    const int forced = g_yz_block.load(std::memory_order_relaxed);
    if (forced) return forced;
    int best = 128, waste = ((nx + 127) / 128) * 128 - nx;
    for (int bs : {64, 32}) {
        const int w = ((nx + bs - 1) / bs) * bs - nx;
        if (w < waste) { best = bs; waste = w; }
    }
    return best;
}

int launch_deriv(const DerivTable &T, int axis, int epi, int nf, const double *const *in,
                 double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st) {
    if (nf < 1 || nf > kMaxFields) return EMIX_ERR_ARG;
    const int n = axis == 0 ? nx : (axis == 1 ? ny : nz);
    if (T.n != n) return EMIX_ERR_ARG;
    PencilFields F{};
    for (int f = 0; f < nf; ++f) {
        F.in[f] = in[f];
        F.w[f] = w[f];
        F.out[f] = out[f];
    }
    if (axis == 0) {
        const long np = (long)ny * nz;
        const int warps = x_warps(np, nf);
        const long blocks = (np + 32 * warps - 1) / (32 * warps);
        const size_t shm = (size_t)warps * kXTile * sizeof(double);
        dim3 grid((unsigned)blocks, 1, nf);
        if (epi == EPI_STORE)
            k_deriv_x<EPI_STORE><<<grid, 32 * warps, shm, st>>>(T, F, np);
        else
            k_deriv_x<EPI_ACCUM><<<grid, 32 * warps, shm, st>>>(T, F, np);
    } else {
        const int bs = yz_block(nx);
        const int nother = axis == 1 ? nz : ny;
        const long s = axis == 1 ? (long)nx : (long)nx * ny;
        const long os = axis == 1 ? (long)nx * ny : (long)nx;
        if (nother > 65535) return EMIX_ERR_ARG;
        dim3 grid((nx + bs - 1) / bs, nother, nf);
        if (epi == EPI_STORE)
            k_deriv_yz<EPI_STORE><<<grid, bs, 0, st>>>(T, F, nx, nother, s, os);
        else
            k_deriv_yz<EPI_ACCUM><<<grid, bs, 0, st>>>(T, F, nx, nother, s, os);
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

__global__ void __launch_bounds__(128)
k_deriv_yz_pair(DerivTable Ta, DerivTable Tb, PencilFields F, int nfa, int nx, int na, long sa,
                long osa, int nb, long sb, long osb) {
    if ((int)blockIdx.z < nfa)
        deriv_yz_body<EPI_STORE>(Ta, F, nx, na, sa, osa, blockIdx, threadIdx.x, blockDim.x);
    else
        deriv_yz_body<EPI_STORE>(Tb, F, nx, nb, sb, osb, blockIdx, threadIdx.x, blockDim.x);
}

int launch_deriv_yz_pair(const DerivTable &Ty, const DerivTable &Tz, int nfa, int nfb,
                         const double *const *in, double *const *out, int nx, int ny, int nz,
                         cudaStream_t st) {
    if (nfa < 1 || nfb < 1 || nfa + nfb > kMaxFields || Ty.n != ny || Tz.n != nz) return EMIX_ERR_ARG;
    if (ny > 65535 || nz > 65535) return EMIX_ERR_ARG;
    PencilFields F{};
    for (int f = 0; f < nfa + nfb; ++f) {
        F.in[f] = in[f];
        F.w[f] = out[f];
        F.out[f] = out[f];
    }
    const int bs = yz_block(nx);
    // axis 1: pencils (x, z); axis 2: pencils (x, y)
    dim3 grid((nx + bs - 1) / bs, ny > nz ? ny : nz, nfa + nfb);
    k_deriv_yz_pair<<<grid, bs, 0, st>>>(Ty, Tz, F, nfa, nx, nz, (long)nx, (long)nx * ny, ny,
                                         (long)nx * ny, (long)nx);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

namespace {

bool dims_ok(int nx, int ny, int nz) {
    return nx >= 6 && ny >= 6 && nz >= 6 && nx <= kTableMaxN && ny <= kTableMaxN && nz <= kTableMaxN &&
           ny <= 65535 && nz <= 65535;
}

bool scheme_ok(int s) { return s >= EMIX_SCHEME_A && s <= EMIX_SCHEME_C; }

// flux projection e <- jbn10*(jbn1*e) ... (solver/divergencia.f90:225-243;
// solver/cuDivergence.cu:4-19 multiplies in the other order)
__global__ void k_project(double *__restrict__ pe, double *__restrict__ pf, double *__restrict__ pg,
                          double *__restrict__ pev, double *__restrict__ pfv, double *__restrict__ pgv,
                          const double *__restrict__ e, const double *__restrict__ f,
                          const double *__restrict__ g, const double *__restrict__ ev,
                          const double *__restrict__ fv, const double *__restrict__ gv,
                          const double *__restrict__ jbn, long n) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double j10 = jbn[9 * n + q];
        const double j1 = jbn[q], j5 = jbn[4 * n + q], j9 = jbn[8 * n + q];
        pe[q] = j10 * (j1 * e[q]);
        pf[q] = j10 * (j5 * f[q]);
        pg[q] = j10 * (j9 * g[q]);
        pev[q] = j10 * (j1 * ev[q]);
        pfv[q] = j10 * (j5 * fv[q]);
        pgv[q] = j10 * (j9 * gv[q]);
    }
}

// rs = jbn11 * (sum of the three derivatives), solver/divergencia.f90:346-354
__global__ void k_scale_jbn11(double *__restrict__ rs, double *__restrict__ rsv,
                              const double *__restrict__ jbn, long n) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const double j11 = jbn[10 * n + q];
        rs[q] = j11 * rs[q];
        rsv[q] = j11 * rsv[q];
    }
}

int grid_for(long n) { return grid_cap(n, 16); }

// grow-only scratch per device for the device-pointer operators
struct Scratch {
    std::mutex mu;
    double *p[8] = {nullptr};
    size_t cap[8] = {0};
};
Scratch g_scratch;

int scratch_get(int dev, size_t bytes, double **out) {
    if (dev < 0 || dev >= 8) return EMIX_ERR_ARG;
    if (g_scratch.cap[dev] < bytes) {
        if (g_scratch.p[dev]) cudaFree(g_scratch.p[dev]);
        g_scratch.p[dev] = nullptr;
        g_scratch.cap[dev] = 0;
        if (cudaMalloc(&g_scratch.p[dev], bytes) != cudaSuccess) {
            cudaGetLastError();
            set_last_message("cudaMalloc of operator scratch failed");
            return EMIX_ERR_ALLOC;
        }
        g_scratch.cap[dev] = bytes;
    }
    *out = g_scratch.p[dev];
    return EMIX_OK;
}

} // namespace

int cudaDeriv_dev_impl(const int schemes[3], double *dvel, double *dtemp, const double *vel,
                       const double *temp, const double h[3], int nx, int ny, int nz,
                       cudaStream_t st) {
    const size_t n = ncell(nx, ny, nz);
    const int dims[3] = {nx, ny, nz};
    const bool wt = temp != nullptr && dtemp != nullptr;
    for (int ax = 0; ax < 3; ++ax) {
        DerivTable T;
        int rc = get_deriv_table(schemes[ax], dims[ax], h[ax], &T);
        if (rc) return rc;
        const double *in[4] = {vel, vel + n, vel + 2 * n, temp};
        double *out[4] = {dvel + (3 * ax) * n, dvel + (3 * ax + 1) * n, dvel + (3 * ax + 2) * n,
                          wt ? dtemp + ax * n : nullptr};
        rc = launch_deriv(T, ax, EPI_STORE, wt ? 4 : 3, in, out, out, nx, ny, nz, st);
        if (rc) return rc;
    }
    return EMIX_OK;
}

int cuDivergence_dev_impl(const int schemes[3], double *rs, double *rsv, const double *e,
                          const double *f, const double *g, const double *ev, const double *fv,
                          const double *gv, const double *jbn, const double h[3], int nx, int ny,
                          int nz, cudaStream_t st, double *scratch /* 8 fields */) {
    const size_t n = ncell(nx, ny, nz);
    double *P = scratch;            // 6 projected fluxes
    double *W = scratch + 6 * n;    // 2 forward-sweep buffers for the accumulating passes
    k_project<<<grid_for((long)n), 256, 0, st>>>(P, P + n, P + 2 * n, P + 3 * n, P + 4 * n, P + 5 * n,
                                                 e, f, g, ev, fv, gv, jbn, (long)n);
    EMIX_CUDA_TRY(cudaGetLastError());
    const int dims[3] = {nx, ny, nz};
    for (int ax = 0; ax < 3; ++ax) {
        DerivTable T;
        int rc = get_deriv_table(schemes[ax], dims[ax], h[ax], &T);
        if (rc) return rc;
        const double *in[2] = {P + ax * n, P + (3 + ax) * n};
        double *out[2] = {rs, rsv};
        double *wb[2] = {W, W + n};
        if (ax == 0)
            rc = launch_deriv(T, ax, EPI_STORE, 2, in, out, out, nx, ny, nz, st);
        else
            rc = launch_deriv(T, ax, EPI_ACCUM, 2, in, wb, out, nx, ny, nz, st);
        if (rc) return rc;
    }
    k_scale_jbn11<<<grid_for((long)n), 256, 0, st>>>(rs, rsv, jbn, (long)n);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

// ---- host-pointer workspace for the synchronous entry points -----------------
namespace {
struct HostWs {
    std::mutex mu;
    double *buf[8] = {nullptr};
    size_t cap[8] = {0};
    cudaStream_t st[8] = {nullptr};
};
HostWs g_ws;
int g_legacy_scheme = EMIX_SCHEME_C;

int ws_get(size_t bytes, double **out, cudaStream_t *st) {
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 8) return EMIX_ERR_ARG;
    if (!g_ws.st[dev]) EMIX_CUDA_TRY(cudaStreamCreateWithFlags(&g_ws.st[dev], cudaStreamNonBlocking));
    if (g_ws.cap[dev] < bytes) {
        if (g_ws.buf[dev]) cudaFree(g_ws.buf[dev]);
        g_ws.buf[dev] = nullptr;
        g_ws.cap[dev] = 0;
        if (cudaMalloc(&g_ws.buf[dev], bytes) != cudaSuccess) {
            cudaGetLastError();
            set_last_message("cudaMalloc of the host-call workspace failed");
            return EMIX_ERR_ALLOC;
        }
        g_ws.cap[dev] = bytes;
    }
    *out = g_ws.buf[dev];
    *st = g_ws.st[dev];
    return EMIX_OK;
}
} // namespace

// SM count per device ordinal, queried on first use (0 = not yet known)
std::atomic<int> g_sms[64];

int device_sms() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1;
    }
    int v = g_sms[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) {
        cudaGetLastError();
        return 1;
    }
    g_sms[dev].store(v, std::memory_order_relaxed);
    return v;
}

// One grow-only scratch buffer per device, shared by every call of the
// device-pointer operators on that device: calls that overlap on the GPU
// (different streams or threads) race on it.
int device_scratch(size_t bytes, double **out) {
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_scratch.mu);
    return scratch_get(dev, bytes, out);
}

} // namespace emix

using namespace emix;

extern "C" {

const char *emix_last_error(void) { return emix::last_error(); }

const char *emix_version(void) { return "emix_gb300 0.1.0 (sm_103a, FP64)"; }

int emix_pencil_set_yz_block(int threads) {
    if (threads != 0 && threads != 32 && threads != 64 && threads != 128) return EMIX_ERR_ARG;
    g_yz_block.store(threads, std::memory_order_relaxed);
    return EMIX_OK;
}

int emix_set_legacy_scheme(int scheme) {
    if (!scheme_ok(scheme)) return EMIX_ERR_ARG;
    g_legacy_scheme = scheme;
    return EMIX_OK;
}

int emix_deriv_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                   int nx, int ny, int nz, void *stream) {
    if (!scheme_ok(scheme) || axis < 0 || axis > 2 || nf < 1 || nf > kMaxFields || !out || !in ||
        !(h > 0.0) || !dims_ok(nx, ny, nz))
        return EMIX_ERR_ARG;
    const int dims[3] = {nx, ny, nz};
    DerivTable T;
    int rc = get_deriv_table(scheme, dims[axis], h, &T);
    if (rc) return rc;
    const size_t n = ncell(nx, ny, nz);
    const double *ip[kMaxFields];
    double *op[kMaxFields];
    for (int f = 0; f < nf; ++f) {
        ip[f] = in + f * n;
        op[f] = out + f * n;
    }
    return launch_deriv(T, axis, EPI_STORE, nf, ip, op, op, nx, ny, nz, (cudaStream_t)stream);
}

int emix_cudaDeriv_dev(const int schemes[3], double *dVel, double *dTemp, const double *vel,
                       const double *temp, double hx, double hy, double hz, int nx, int ny, int nz,
                       void *stream) {
    if (!schemes || !dVel || !vel || !dims_ok(nx, ny, nz) || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (!scheme_ok(schemes[a])) return EMIX_ERR_ARG;
    const double h[3] = {hx, hy, hz};
    return cudaDeriv_dev_impl(schemes, dVel, dTemp, vel, temp, h, nx, ny, nz, (cudaStream_t)stream);
}

int emix_cudaDeriv(const int schemes[3], double *dVel, double *dTemp, const double *vel,
                   const double *temp, double hx, double hy, double hz, int nx, int ny, int nz) {
    if (!schemes || !dVel || !dTemp || !vel || !temp || !dims_ok(nx, ny, nz) || !(hx > 0) ||
        !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (!scheme_ok(schemes[a])) return EMIX_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_ws.mu);
    const size_t n = ncell(nx, ny, nz);
    double *d;
    cudaStream_t st;
    int rc = ws_get(16 * n * sizeof(double), &d, &st);
    if (rc) return rc;
    double *dv = d, *dtp = d + 3 * n, *ddv = d + 4 * n, *ddt = d + 13 * n;
    EMIX_CUDA_TRY(cudaMemcpyAsync(dv, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(dtp, temp, n * sizeof(double), cudaMemcpyHostToDevice, st));
    const double h[3] = {hx, hy, hz};
    rc = cudaDeriv_dev_impl(schemes, ddv, ddt, dv, dtp, h, nx, ny, nz, st);
    if (rc) return rc;
    EMIX_CUDA_TRY(cudaMemcpyAsync(dVel, ddv, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(dTemp, ddt, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    return EMIX_OK;
}

int emix_cuDivergence_dev(const int schemes[3], double *rs, double *rsv, const double *e,
                          const double *f, const double *g, const double *ev, const double *fv,
                          const double *gv, const double *jbn, double hx, double hy, double hz,
                          int nx, int ny, int nz, void *stream) {
    if (!schemes || !rs || !rsv || !e || !f || !g || !ev || !fv || !gv || !jbn ||
        !dims_ok(nx, ny, nz) || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (!scheme_ok(schemes[a])) return EMIX_ERR_ARG;
    const size_t n = ncell(nx, ny, nz);
    double *scr;
    int rc = device_scratch(8 * n * sizeof(double), &scr);
    if (rc) return rc;
    const double h[3] = {hx, hy, hz};
    return cuDivergence_dev_impl(schemes, rs, rsv, e, f, g, ev, fv, gv, jbn, h, nx, ny, nz,
                                 (cudaStream_t)stream, scr);
}

int emix_cuDivergence(const int schemes[3], double *rs, double *rsv, const double *e,
                      const double *f, const double *g, const double *ev, const double *fv,
                      const double *gv, const double *jbn, double hx, double hy, double hz,
                      int nx, int ny, int nz) {
    if (!schemes || !rs || !rsv || !e || !f || !g || !ev || !fv || !gv || !jbn ||
        !dims_ok(nx, ny, nz) || !(hx > 0) || !(hy > 0) || !(hz > 0))
        return EMIX_ERR_ARG;
    for (int a = 0; a < 3; ++a)
        if (!scheme_ok(schemes[a])) return EMIX_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_ws.mu);
    const size_t n = ncell(nx, ny, nz);
    double *d;
    cudaStream_t st;
    // inputs 6 + jbn 11 + outputs 2 + scratch 8
    int rc = ws_get(27 * n * sizeof(double), &d, &st);
    if (rc) return rc;
    double *de = d, *dj = d + 6 * n, *drs = d + 17 * n, *drsv = d + 18 * n, *scr = d + 19 * n;
    const double *src[6] = {e, f, g, ev, fv, gv};
    for (int q = 0; q < 6; ++q)
        EMIX_CUDA_TRY(cudaMemcpyAsync(de + q * n, src[q], n * sizeof(double), cudaMemcpyHostToDevice, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(dj, jbn, 11 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    const double h[3] = {hx, hy, hz};
    rc = cuDivergence_dev_impl(schemes, drs, drsv, de, de + n, de + 2 * n, de + 3 * n, de + 4 * n,
                               de + 5 * n, dj, h, nx, ny, nz, st, scr);
    if (rc) return rc;
    EMIX_CUDA_TRY(cudaMemcpyAsync(rs, drs, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(rsv, drsv, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    return EMIX_OK;
}

void cudaDeriv(double *dVel, double *dTemp, double *vel, double *temp, double *amut,
               double *dxyzsgd, double *jbn, double deltaX, double deltaY, double deltaZ, int Nx,
               int Ny, int Nz) {
    (void)amut; (void)dxyzsgd; (void)jbn;
    const int s[3] = {g_legacy_scheme, g_legacy_scheme, g_legacy_scheme};
    int rc = emix_cudaDeriv(s, dVel, dTemp, vel, temp, deltaX, deltaY, deltaZ, Nx, Ny, Nz);
    if (rc) fprintf(stderr, "cudaDeriv: error %d: %s\n", rc, emix_last_error());
}

void cuDivergence(double *rs, double *rsv, double *e, double *f, double *g, double *ev, double *fv,
                  double *gv, double *jbn, double deltaX, double deltaY, double deltaZ, int Nx,
                  int Ny, int Nz) {
    const int s[3] = {g_legacy_scheme, g_legacy_scheme, g_legacy_scheme};
    int rc = emix_cuDivergence(s, rs, rsv, e, f, g, ev, fv, gv, jbn, deltaX, deltaY, deltaZ, Nx,
                               Ny, Nz);
    if (rc) fprintf(stderr, "cuDivergence: error %d: %s\n", rc, emix_last_error());
}

} // extern "C"
