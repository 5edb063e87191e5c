// weno_march.cu -- launch of the z-marching level-set TVD stage
// (weno_march_body, weno_march.cuh) on one grid.
#include "weno_march.cuh"

namespace emix {

namespace {

__global__ void __launch_bounds__(kNT, 4) k_weno_march(WenoArgs a) {
    weno_march_body(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.z);
}

} // namespace

int launch_weno_march(const WenoArgs &a, cudaStream_t st) {
    const int gx = (a.rn[0] + kMX - 1) / kMX, gy = (a.rn[1] + kMY - 1) / kMY;
    if (gy > 65535) return EMIX_ERR_ARG;
    // resident blocks of the device (queried once)
    static int resident = 0;
    if (resident == 0) {
        int dev = 0, sms = 0, per = 0;
        EMIX_CUDA_TRY(cudaGetDevice(&dev));
        EMIX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        EMIX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_weno_march, kNT, 0));
        resident = sms * (per > 0 ? per : 1);
    }
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
    k_weno_march<<<dim3(gx, gy, (unsigned)best), kNT, 0, st>>>(a);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix
