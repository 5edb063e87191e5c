// weno_march.cu -- launch of the z-marching level-set TVD stage
// (weno_march_body_t, weno_march.cuh) on one grid: with the plane tiles
// brought by TMA tiled copies where the copy unit's alignment rules hold,
// by register-staged loads otherwise.
#include "weno_march.cuh"


#include <atomic>
#include <cstring>
#include <mutex>

namespace emix {

namespace {

__global__ void __launch_bounds__(kNT, 4) k_weno_march(WenoArgs a) {
    weno_march_body_t<false>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.z, nullptr);
}

__global__ void __launch_bounds__(kNT, 4) k_weno_march_tma(const __grid_constant__ CUtensorMap tmap,
                                                           const WenoArgs a) {
    weno_march_body_t<true>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.z, &tmap);
}


// resident blocks per SM x SMs of a stage kernel on the current device
// (queried once per kernel and device ordinal)
template <class K>
int resident_blocks(K kernel, std::atomic<int> (&cache)[64]) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return device_sms() * 4;
    }
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kNT, 0) != cudaSuccess) {
        cudaGetLastError();
        return device_sms() * 4;
    }
    v = device_sms() * (per > 0 ? per : 1);
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

std::atomic<int> g_res_plain[64], g_res_tma[64];

} // namespace

PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

bool weno_tma_map(CUtensorMap *m, const WenoArgs &a) {
    const int nxg = a.nxg, nyg = a.nyg, nzg = a.nzg;
    if ((reinterpret_cast<uintptr_t>(a.phi) & 15) != 0 || (nxg & 1) != 0 || nxg < kTW || nyg < kTY)
        return false;
    PFN_cuTensorMapEncodeTiled_v12000 fn = tma_encode_fn();
    if (!fn) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)nxg, (cuuint64_t)nyg, (cuuint64_t)nzg};
    const cuuint64_t stride[2] = {(cuuint64_t)nxg * 8, (cuuint64_t)nxg * nyg * 8};
    const cuuint32_t box[3] = {(cuuint32_t)kTW, (cuuint32_t)kTY, 1};
    const cuuint32_t estride[3] = {1, 1, 1};
    std::memset(m, 0, sizeof *m);
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(a.phi), dim, stride, box,
                          estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

int launch_weno_march(const WenoArgs &a, cudaStream_t st, const CUtensorMap *tmap) {
    const int gx = (a.rn[0] + kMX - 1) / kMX, gy = (a.rn[1] + kMY - 1) / kMY;
    if (gy > 65535) return EMIX_ERR_ARG;
    const int resident = tmap ? resident_blocks(k_weno_march_tma, g_res_tma) : resident_blocks(k_weno_march, g_res_plain);
    // z chunks: the count whose block total fills the last wave best, chunks
    // of at least 8 planes, the smaller count on a tie
    const long cols = (long)gx * gy;
    long best = 1;
    double best_eff = 0.0;
    const long maxgz = a.rn[2] / 8 < 1 ? 1 : (a.rn[2] / 8 > 65535 ? 65535 : a.rn[2] / 8);
    for (long gz = 1; gz <= maxgz && gz <= 64; ++gz) {
        const long T = cols * gz;
        const long waves = (T + resident - 1) / resident;
        const double eff = (double)T / ((double)waves * resident);
        if (eff > best_eff + 1e-3) { best_eff = eff; best = gz; }
    }
    const dim3 grid(gx, gy, (unsigned)best);
    if (tmap) k_weno_march_tma<<<grid, kNT, 0, st>>>(*tmap, a);
    else k_weno_march<<<grid, kNT, 0, st>>>(a);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

extern "C" int emix_weno_tma_timeouts(int *count) {
    if (!count) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaMemcpyFromSymbol(count, emix::g_weno_tma_timeouts, sizeof(int)));
    return EMIX_OK;
}

extern "C" int emix_weno_tma_test_drop(int on) {
    if (on != 0 && on != 1) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaMemcpyToSymbol(emix::g_weno_tma_drop, &on, sizeof(int)));
    EMIX_CUDA_TRY(cudaDeviceSynchronize());
    return EMIX_OK;
}
