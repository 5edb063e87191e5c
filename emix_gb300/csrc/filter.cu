// filter.cu -- the compact filter `filtrado` (src/MSVSingle/
// herramientas_incomp2.f90:227-410 with filtronper, src/MSVSingle/
// filtro_incomp.f90:307-362, and the rows and constants of inifiltro, :1-162).
//
// Per pencil of n points: r = the 11-point filter stencil of J*f on rows
// 6..n-5 (1-based), r = J*f on the five rows at either end; solve the
// tridiagonal system (b = 1, a = c = cfilt on the filtered rows; on every row
// for z, which gets the periodic row arrays azpf/czpf); f = result / J.
// Applied to the 5 conserved fields along x, then y, then z (itf = 1, the only
// value RUNGEK passes).
//
// Kernel: one thread per pencil, lanes along x for the y and z pencils
// (coalesced), along y for the x pencils (each lane walks its own line; the
// lines stay in L1 across the walk).  The forward sweep computes the stencil
// from an 11-value register window of the original values, so the
// forward-eliminated values can overwrite the field in place; the backward
// sweep finishes in place.  Thomas factors (1/bet, gam) are precomputed on
// the host per (n, cfilt, row kind): 16 FP64 operations per point, no divide.
#include "common.cuh"

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace emix {

struct FiltRow {
    double a;    // sub-diagonal a(l)
    double ib;   // 1 / bet(l)
    double g;    // gam(l+1), 0 on the last row
};

struct FilterArgs {
    double *f;                  // nf fields of n, filtered in place
    const double *jac, *ijac;   // jbn(10) = J, jbn(11) = 1/J
    const FiltRow *rows;
    double ca, cb, cc, cd, ce, cf;   // arsf, brsf/2, crsf/2, drsf/2, ersf/2, frsf/2
    int axis, nx, ny, nz;
    long n;
};

namespace {

struct FiltKey {
    int dev, n, zrows;
    unsigned long long cbits;
    bool operator<(const FiltKey &o) const {
        return std::tie(dev, n, zrows, cbits) < std::tie(o.dev, o.n, o.zrows, o.cbits);
    }
};

std::mutex g_filt_mu;
std::map<FiltKey, FiltRow *> g_filt_tables;

// Thomas factors of inifiltro's rows (the same recurrences as filtronper)
void filter_rows_host(int n, double cfilt, int zrows, std::vector<FiltRow> &R) {
    std::vector<double> a(n), c(n), gam(n + 1, 0.0), ib(n);
    for (int l = 0; l < n; ++l) {
        const bool in = zrows || (l >= 5 && l <= n - 6);
        a[l] = in ? cfilt : 0.0;
        c[l] = in ? cfilt : 0.0;
    }
    double bet = 1.0;
    ib[0] = 1.0 / bet;
    for (int l = 1; l < n; ++l) {
        gam[l] = c[l - 1] / bet;
        bet = 1.0 - a[l] * gam[l];
        ib[l] = 1.0 / bet;
    }
    R.resize(n);
    for (int l = 0; l < n; ++l) R[l] = FiltRow{l == 0 ? 0.0 : a[l], ib[l], l + 1 < n ? gam[l + 1] : 0.0};
}

int get_filter_rows(int n, double cfilt, int zrows, const FiltRow **out) {
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    FiltKey key{dev, n, zrows, 0};
    std::memcpy(&key.cbits, &cfilt, sizeof cfilt);
    std::lock_guard<std::mutex> lock(g_filt_mu);
    auto it = g_filt_tables.find(key);
    if (it != g_filt_tables.end()) {
        *out = it->second;
        return EMIX_OK;
    }
    std::vector<FiltRow> R;
    filter_rows_host(n, cfilt, zrows, R);
    FiltRow *d = nullptr;
    EMIX_CUDA_TRY(cudaMalloc(&d, n * sizeof(FiltRow)));
    cudaError_t e = cudaMemcpy(d, R.data(), n * sizeof(FiltRow), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        set_last_error(e, "filter table copy", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    g_filt_tables[key] = d;
    *out = d;
    return EMIX_OK;
}

__global__ void __launch_bounds__(128) k_filter(FilterArgs a) {
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long base, s;
    int L;
    if (a.axis == 0) {
        if (p >= (long)ny * nz) return;
        base = p * nx; s = 1; L = nx;
    } else if (a.axis == 1) {
        if (p >= (long)nx * nz) return;
        const long i = p % nx, k = p / nx;
        base = i + k * (long)nx * ny; s = nx; L = ny;
    } else {
        if (p >= (long)nx * ny) return;
        base = p; s = (long)nx * ny; L = nz;
    }
    double *f = a.f + blockIdx.y * a.n + base;
    const double *J = a.jac + base, *IJ = a.ijac + base;
    const FiltRow *R = a.rows;
    // w[5 + d] = J f at row l + d
    double w[11];
#pragma unroll
    for (int d = 0; d < 11; ++d) {
        const int l = d - 5;
        w[d] = (l >= 0 && l < L) ? f[l * s] * J[l * s] : 0.0;
    }
    double y = 0.0;
    // one row: the 11-point right-hand side on the interior rows, the value
    // itself on the five rows at each end (branch-free runs of rows)
    auto row = [&](int l, bool interior) {
        double r;
        if (interior)
            r = a.ca * w[5] + a.cb * (w[6] + w[4]) + a.cc * (w[7] + w[3]) + a.cd * (w[8] + w[2]) +
                a.ce * (w[9] + w[1]) + a.cf * (w[10] + w[0]);
        else
            r = w[5];
        const FiltRow q = R[l];
        y = (r - q.a * y) * q.ib;
        f[l * s] = y;
#pragma unroll
        for (int d = 0; d < 10; ++d) w[d] = w[d + 1];
        const int ln = l + 6;
        w[10] = ln < L ? f[ln * s] * J[ln * s] : 0.0;
    };
    const int lo = L < 5 ? L : 5, hi = L - 5 > lo ? L - 5 : lo;
    int l = 0;
    for (; l < lo; ++l) row(l, false);
    for (; l < hi; ++l) row(l, true);
    for (; l < L; ++l) row(l, false);
    double x = y;
    f[(long)(L - 1) * s] = x * IJ[(long)(L - 1) * s];
    for (int l = L - 2; l >= 0; --l) {
        x = f[l * s] - R[l].g * x;
        f[l * s] = x * IJ[l * s];
    }
}

} // namespace

// One filter pass along `axis` over nf fields (in place), rows of kind zrows.
int launch_filter(double *f, int nf, const double *jbn, double cfilt, int axis, int zrows, int nx,
                  int ny, int nz, cudaStream_t st) {
    const int dims[3] = {nx, ny, nz};
    const FiltRow *rows;
    int rc = get_filter_rows(dims[axis], cfilt, zrows, &rows);
    if (rc) return rc;
    const long n = (long)nx * ny * nz;
    FilterArgs a;
    a.f = f; a.jac = jbn + 9 * n; a.ijac = jbn + 10 * n; a.rows = rows;
    // inifiltro :140-145; the stencil's 0.5 folded into the pair weights
    a.ca = (193. + 126. * cfilt) / 256.;
    a.cb = 0.5 * ((105. + 302. * cfilt) / 256.);
    a.cc = 0.5 * ((-15. + 30. * cfilt) / 64.);
    a.cd = 0.5 * ((45. - 90. * cfilt) / 512.);
    a.ce = 0.5 * ((-5. + 10. * cfilt) / 256.);
    a.cf = 0.5 * ((1. - 2 * cfilt) / 512.);
    a.axis = axis; a.nx = nx; a.ny = ny; a.nz = nz; a.n = n;
    const long np = axis == 0 ? (long)ny * nz : (axis == 1 ? (long)nx * nz : (long)nx * ny);
    dim3 grid((unsigned)((np + 127) / 128), nf);
    k_filter<<<grid, 128, 0, st>>>(a);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

// filtrado with itf = 1: x, y (non-periodic rows), z (periodic rows)
int launch_filtrado(double *um, const double *jbn, double cfilt, int nx, int ny, int nz,
                    cudaStream_t st) {
    for (int axis = 0; axis < 3; ++axis) {
        int rc = launch_filter(um, 5, jbn, cfilt, axis, axis == 2 ? 1 : 0, nx, ny, nz, st);
        if (rc) return rc;
    }
    return EMIX_OK;
}

// host-side preparation of the tables (before any stream capture)
int prepare_filtrado(double cfilt, int nx, int ny, int nz) {
    const FiltRow *r;
    int rc = get_filter_rows(nx, cfilt, 0, &r);
    if (!rc) rc = get_filter_rows(ny, cfilt, 0, &r);
    if (!rc) rc = get_filter_rows(nz, cfilt, 1, &r);
    return rc;
}

} // namespace emix

using namespace emix;

extern "C" {

int emix_filter_dev(double *f, int nf, const double *jbn, double cfilt, int axis, int zrows, int nx,
                    int ny, int nz, void *stream) {
    const int dims[3] = {nx, ny, nz};
    if (!f || !jbn || nf < 1 || nf > 65535 || axis < 0 || axis > 2 || (zrows != 0 && zrows != 1) ||
        nx < 1 || ny < 1 || nz < 1 || dims[axis] < 11 || dims[axis] > kTableMaxN)
        return EMIX_ERR_ARG;
    return launch_filter(f, nf, jbn, cfilt, axis, zrows, nx, ny, nz, (cudaStream_t)stream);
}

int emix_filtrado_dev(double *um, const double *jbn, double cfilt, int nx, int ny, int nz,
                      void *stream) {
    if (!um || !jbn || nx < 11 || ny < 11 || nz < 11 || nx > kTableMaxN || ny > kTableMaxN ||
        nz > kTableMaxN)
        return EMIX_ERR_ARG;
    return launch_filtrado(um, jbn, cfilt, nx, ny, nz, (cudaStream_t)stream);
}

} // extern "C"
