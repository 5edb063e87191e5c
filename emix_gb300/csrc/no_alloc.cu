// no_alloc.cu -- WENO5 level-set advection that allocates no device memory.
//
// emix_weno5_advect_dev needs two padded stage fields of scratch and takes
// them from a grow-only buffer that it cudaMallocs on demand.  Some callers
// cannot let a library allocate: cudaMalloc and cudaFree can block on the
// whole device and take driver locks, which a caller stepping a solver in a
// latency-bound loop cannot afford, and a process whose device memory is
// already reserved by another allocator (a framework's caching allocator, a
// host code with a fixed memory budget) may see cudaMalloc fail although its
// own pool has room.  This variant takes its scratch from a fixed array
// compiled into the library instead.
//
// Limit: nxg*nyg*nzg <= kNoAllocMaxCells (1,048,576 padded cells, e.g. 101^3);
// the array holds two such fields, 16 MiB.  The array is part of this file's
// device module, which CUDA loads lazily: the first call on a device loads it
// (reserving the 16 MiB there until the process exits) together with the
// stage kernels, and so does take device memory once.  Make that first call
// at set-up, outside any latency-bound loop and before any stream capture;
// every later call allocates nothing.  The array is shared by all calls: a
// call overwrites what the previous call left in it, and calls that overlap on
// the GPU (different streams or threads) race on it.
#include "weno.cuh"

namespace emix {
namespace {

constexpr long kNoAllocMaxCells = 1L << 20;

// Two padded stage fields.  Host code must not use this name as a device
// address (in host code it denotes a host-side shadow); the address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_weno_stage_scratch[2 * kNoAllocMaxCells];

// The array's device address on the current device, looked up on every call
// (a host-side lookup once the module is loaded; a cached address would go
// stale if the device's context were torn down and created again).
int scratch_address(double **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_weno_stage_scratch);
    if (e != cudaSuccess || p == nullptr) {
        set_last_error(e, "cudaGetSymbolAddress(g_weno_stage_scratch)", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    *out = static_cast<double *>(p);
    return EMIX_OK;
}

} // namespace
} // namespace emix

using namespace emix;

extern "C" int emix_weno5_advect_dev_noalloc(double *phi, const double *vel, const double *jbn,
                                             double hx, double hy, double hz, double dt,
                                             int nxg, int nyg, int nzg, int ref_bugs,
                                             void *stream) {
    if (!phi || !vel || !jbn || nxg < 6 || nyg < 6 || nzg < 6 || !(hx > 0) || !(hy > 0) ||
        !(hz > 0) || (nyg + 15) / 16 > 65535)
        return EMIX_ERR_ARG;
    const long ng = (long)nxg * nyg * nzg;
    if (ng > kNoAllocMaxCells) {
        set_last_message("emix_weno5_advect_dev_noalloc: nxg*nyg*nzg exceeds the 1048576-cell "
                         "limit of the static scratch; use emix_weno5_advect_dev");
        return EMIX_ERR_ARG;
    }
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    // both stage fields are written in full before they are read, so nothing
    // needs clearing between calls
    double *p1 = scratch, *p2 = scratch + ng;
    cudaStream_t st = (cudaStream_t)stream;
    WenoArgs a{};
    a.vel = vel; a.jbn = jbn; a.reflect = 0; a.out_interior = 0;
    a.nxg = nxg; a.nyg = nyg; a.nzg = nzg; a.g = 0;
    a.sx = 1.0 / hx; a.sy = 1.0 / hy; a.sz = 1.0 / hz;
    a.dt = dt; a.ref_bugs = ref_bugs;
    a.phi = phi; a.phi0 = phi; a.out = p1; a.stage = 1;
    if ((rc = launch_weno_stage(a, st))) return rc;
    a.phi = p1; a.out = p2; a.stage = 2;
    if ((rc = launch_weno_stage(a, st))) return rc;
    a.phi = p2; a.out = phi; a.stage = 3;
    return launch_weno_stage(a, st);
}
