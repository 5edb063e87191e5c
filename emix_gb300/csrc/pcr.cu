// pcr.cu -- single-grid launch of the PCR + Thomas y/z derivative
// (pcr_yz_warp, pcr.cuh) and its entry point emix_deriv_pcr_dev.
#include "pcr.cuh"

namespace emix {
namespace {

// grid (ceil(nx / pcr_block_x<S>()), nother, nf); 4 warps per block
template <int S, int EPI>
__global__ void __launch_bounds__(128)
k_deriv_pcr(PcrTable P, PencilFields F, int nx, int nother, long s, long os) {
    const int warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * pcr_block_x<S>() + warp * (32 >> S);
    pcr_yz_warp<S, pcr_rows<S>(), EPI>(P, F, nx, nother, s, os, x0, blockIdx.y, blockIdx.z);
}

template <int S>
void launch_s(const PcrTable &P, int epi, int nf, const PencilFields &F, int nx, int nother, long s, long os,
              cudaStream_t st) {
    const dim3 grid((nx + pcr_block_x<S>() - 1) / pcr_block_x<S>(), nother, nf);
    if (epi == EPI_STORE) k_deriv_pcr<S, EPI_STORE><<<grid, 128, 0, st>>>(P, F, nx, nother, s, os);
    else k_deriv_pcr<S, EPI_ACCUM><<<grid, 128, 0, st>>>(P, F, nx, nother, s, os);
}

} // namespace

int launch_deriv_pcr(const PcrTable &P, int axis, int epi, int nf, const double *const *in,
                     double *const *out, int nx, int ny, int nz, cudaStream_t st) {
    if ((axis != 1 && axis != 2) || nf < 1 || nf > kMaxFields || P.n != (axis == 1 ? ny : nz)) return EMIX_ERR_ARG;
    const int nother = axis == 1 ? nz : ny;
    if (nother > 65535) return EMIX_ERR_ARG;
    const long s = axis == 1 ? (long)nx : (long)nx * ny;
    const long os = axis == 1 ? (long)nx * ny : (long)nx;
    PencilFields F{};
    for (int f = 0; f < nf; ++f) {
        F.in[f] = in[f];
        F.w[f] = out[f];
        F.out[f] = out[f];
    }
    switch (P.steps) {
    case 2: launch_s<2>(P, epi, nf, F, nx, nother, s, os, st); break;
    case 3: launch_s<3>(P, epi, nf, F, nx, nother, s, os, st); break;
    case 4: launch_s<4>(P, epi, nf, F, nx, nother, s, os, st); break;
    case 5: launch_s<5>(P, epi, nf, F, nx, nother, s, os, st); break;
    default: return EMIX_ERR_ARG;
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

} // namespace emix

using namespace emix;

extern "C" int emix_deriv_pcr_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                                  int steps, int nx, int ny, int nz, void *stream) {
    if (scheme < EMIX_SCHEME_A || scheme > EMIX_SCHEME_C || (axis != 1 && axis != 2) || nf < 1 ||
        nf > kMaxFields || !out || !in || !(h > 0.0) || steps < 2 || steps > kPcrMaxSteps || nx < 1 ||
        ny < 6 || nz < 6)
        return EMIX_ERR_ARG;
    const int n = axis == 1 ? ny : nz;
    if (n > kPcrMaxN) {
        set_last_message("emix_deriv_pcr_dev: pencils longer than 160 rows are not supported");
        return EMIX_ERR_ARG;
    }
    PcrTable P;
    int rc = get_pcr_table(scheme, n, h, steps, &P);
    if (rc) return rc;
    const long cells = (long)nx * ny * nz;
    const double *ins[kMaxFields];
    double *outs[kMaxFields];
    for (int f = 0; f < nf; ++f) {
        ins[f] = in + f * cells;
        outs[f] = out + f * cells;
    }
    return launch_deriv_pcr(P, axis, EPI_STORE, nf, ins, outs, nx, ny, nz, (cudaStream_t)stream);
}
