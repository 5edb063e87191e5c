// ref_harness.cu -- runs the reference's own CUDA kernels (compiled unmodified
// into oracle/_ref/*.cubin by oracle/ref/build_ref.sh) on seeded inputs, to
// pin the CPU oracle against the reference itself.  TEST INFRASTRUCTURE ONLY.
//
// The launch sequences restate the reference's host drivers:
//   deriv  : cu::cs::dFdX/dFdY/dFdZ       src/Schemes/derivCompact.cu:222-409
//   div    : cuDivergence                 solver/cuDivergence.cu:107-189
//   weno   : cuAdvectLsJB                 src/LevelSet/lsTransportEc.cu:201-418
//   pad    : cuSwapToGhost + mirrors      src/LevelSet/lsTransportEc.cu:91-127
//   extrap : advect_CUDA as linked        src/LevelSet/lsTransportEc.cu:24-197
//            with cuExtrapolation         src/LevelSet/interface.cu:341-436
//   reinit : cuReinitLsJB                 src/LevelSet/lsTransportEc.cu:420-676
// with two deliberate differences: the z grid of the level-set kernels is
// NzG/5 (the reference writes NxG/5, :232), and grids are only used where they
// tile the arrays exactly (the level-set kernels have no bounds checks).
//
// usage:
//   ref_harness deriv <nx> <ny> <nz> <axis> <h> in.bin out.bin
//   ref_harness div <nx> <ny> <nz> <hx> <hy> <hz> e f g ev fv gv jbn rs rsv   (.bin paths)
//   ref_harness weno <nxg> <nyg> <nzg> <hx> <hy> <hz> <dt> phi vel jbn out
//   ref_harness pad <nx> <ny> <nz> <g> val out
//   ref_harness extrap <nx> <ny> <nz> <dX> <dY> <dZ> <deltamin> press jbn sobject out
//   ref_harness reinit <nxg> <nyg> <nzg> <g> <dX> <dY> <dZ> <deltamin> <iters> phi jbn dmins out
#include <cuda.h>
#include <cxxabi.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "arraydev_layout.h"

#define CK(x)                                                                                \
    do {                                                                                     \
        CUresult r_ = (x);                                                                   \
        if (r_ != CUDA_SUCCESS) {                                                            \
            const char *s_ = nullptr;                                                        \
            cuGetErrorString(r_, &s_);                                                       \
            fprintf(stderr, "%s failed: %s (line %d)\n", #x, s_ ? s_ : "?", __LINE__);       \
            exit(2);                                                                         \
        }                                                                                    \
    } while (0)

static std::string g_dir = "oracle/_ref";
static std::vector<CUmodule> g_mods;

static void load_modules() {
    const char *names[] = {"ref_cuDeriv.cubin", "ref_cuDivergence.cubin", "ref_lsTools.cubin",
                           "ref_extrapol.cubin"};
    for (const char *n : names) {
        CUmodule m;
        std::string p = g_dir + "/" + n;
        CK(cuModuleLoad(&m, p.c_str()));
        g_mods.push_back(m);
    }
}

// Find a kernel whose demangled (or plain) name contains `key`.
static CUfunction find_kernel(const char *key) {
    for (CUmodule m : g_mods) {
        unsigned int cnt = 0;
        CK(cuModuleGetFunctionCount(&cnt, m));
        std::vector<CUfunction> fs(cnt);
        CK(cuModuleEnumerateFunctions(fs.data(), cnt, m));
        for (CUfunction f : fs) {
            const char *name = nullptr;
            CK(cuFuncGetName(&name, f));
            int st = 0;
            char *dem = abi::__cxa_demangle(name, nullptr, nullptr, &st);
            std::string s = (st == 0 && dem) ? dem : name;
            free(dem);
            if (s.find(key) != std::string::npos) return f;
        }
    }
    fprintf(stderr, "kernel %s not found\n", key);
    exit(3);
}

// Kernel parameter blob laid out as the reference's ArrayDev3D<double>.
struct Arr {
    alignas(8) unsigned char b[REF_ARRAYDEV3D_SIZE];
};

static Arr arr(CUdeviceptr p, int nx, int ny, int nz) {
    Arr a;
    memset(a.b, 0, sizeof a.b);
    memcpy(a.b + REF_OFF_DDATA, &p, sizeof p);
    int dim = nx * ny * nz;
    memcpy(a.b + REF_OFF_DIMSIZE, &dim, sizeof dim);
    memcpy(a.b + REF_OFF_NX, &nx, sizeof nx);
    memcpy(a.b + REF_OFF_NY, &ny, sizeof ny);
    memcpy(a.b + REF_OFF_NZ, &nz, sizeof nz);
    return a;
}

static int cdiv(int a, int b) { return (a + b - 1) / b; }

static void launch(CUfunction f, int gx, int gy, int gz, int bx, int by, int bz, unsigned smem,
                   void **args) {
    CK(cuLaunchKernel(f, gx, gy, gz, bx, by, bz, smem, 0, args, nullptr));
}

static std::vector<double> read_bin(const char *path, size_t n) {
    std::vector<double> v(n);
    FILE *fp = fopen(path, "rb");
    if (!fp || fread(v.data(), sizeof(double), n, fp) != n) {
        fprintf(stderr, "cannot read %zu doubles from %s\n", n, path);
        exit(4);
    }
    fclose(fp);
    return v;
}

static void write_bin(const char *path, const std::vector<double> &v) {
    FILE *fp = fopen(path, "wb");
    if (!fp || fwrite(v.data(), sizeof(double), v.size(), fp) != v.size()) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(4);
    }
    fclose(fp);
}

static CUdeviceptr dalloc(size_t n) {
    CUdeviceptr p;
    CK(cuMemAlloc(&p, n * sizeof(double)));
    CK(cuMemsetD8(p, 0, n * sizeof(double)));
    return p;
}

static CUdeviceptr upload(const std::vector<double> &v) {
    CUdeviceptr p = dalloc(v.size());
    CK(cuMemcpyHtoD(p, v.data(), v.size() * sizeof(double)));
    return p;
}

static std::vector<double> download(CUdeviceptr p, size_t n) {
    std::vector<double> v(n);
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(v.data(), p, n * sizeof(double)));
    return v;
}

// cu::cs::dFdX / dFdY / dFdZ (derivCompact.cu:222-409), variant C.
static void ref_deriv(CUdeviceptr out, CUdeviceptr f, double delta, int nx, int ny, int nz, int axis) {
    static CUfunction kRHS = find_kernel("getC6RHS<double>");
    static CUfunction kCS = find_kernel("cuDerivCS<double>");
    static CUfunction kTJ = find_kernel("transposeArrayJ<double>");
    static CUfunction kTK = find_kernel("transposeArrayK<double>");
    const size_t n = (size_t)nx * ny * nz;
    CUdeviceptr rhs = dalloc(n), trash = dalloc(n), ftrans = dalloc(n);
    if (axis == 0) {
        Arr A_rhs = arr(rhs, nx, ny, nz), A_f = arr(f, nx, ny, nz), A_out = arr(out, nx, ny, nz),
            A_tr = arr(trash, nx, ny, nz);
        void *a1[] = {&A_rhs, &A_f, &delta};
        launch(kRHS, cdiv(nx, 8), cdiv(ny, 8), cdiv(nz, 4), 8, 8, 4, 0, a1);
        void *a2[] = {&A_out, &A_rhs, &A_tr};
        launch(kCS, cdiv(ny, 16), cdiv(nz, 16), 1, 16, 16, 1, 3 * nx * 8, a2);
    } else if (axis == 1) {
        const int gx = cdiv(ny, 8), gy = cdiv(nx, 8), gz = cdiv(nz, 4);
        Arr A_ft = arr(ftrans, ny, nx, nz), A_f = arr(f, nx, ny, nz), A_rhs = arr(rhs, ny, nx, nz),
            A_tr = arr(trash, ny, nx, nz), A_out = arr(out, nx, ny, nz);
        void *a0[] = {&A_ft, &A_f};
        launch(kTJ, gx, gy, gz, 8, 8, 4, 0, a0);
        void *a1[] = {&A_rhs, &A_ft, &delta};
        launch(kRHS, gx, gy, gz, 8, 8, 4, 0, a1);
        void *a2[] = {&A_ft, &A_rhs, &A_tr};
        launch(kCS, cdiv(nx, 16), cdiv(nz, 16), 1, 16, 16, 1, 3 * ny * 8, a2);
        void *a3[] = {&A_out, &A_ft};
        launch(kTJ, gy, gx, gz, 8, 8, 4, 0, a3);
    } else {
        const int gx = cdiv(nz, 8), gy = cdiv(ny, 8), gz = cdiv(nx, 4);
        Arr A_ft = arr(ftrans, nz, ny, nx), A_f = arr(f, nx, ny, nz), A_rhs = arr(rhs, nz, ny, nx),
            A_tr = arr(trash, nz, ny, nx), A_out = arr(out, nx, ny, nz);
        void *a0[] = {&A_ft, &A_f};
        launch(kTK, gx, gy, gz, 8, 8, 4, 0, a0);
        void *a1[] = {&A_rhs, &A_ft, &delta};
        launch(kRHS, gx, gy, gz, 8, 8, 4, 0, a1);
        void *a2[] = {&A_ft, &A_rhs, &A_tr};
        launch(kCS, cdiv(ny, 16), cdiv(nx, 16), 1, 16, 16, 1, 3 * nz * 8, a2);
        void *a3[] = {&A_out, &A_ft};
        launch(kTK, gz, gy, gx, 4, 8, 8, 0, a3);
    }
    CK(cuCtxSynchronize());
    cuMemFree(rhs);
    cuMemFree(trash);
    cuMemFree(ftrans);
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: see header\n");
        return 1;
    }
    const char *dir = getenv("EMIX_REF_DIR");
    if (dir) g_dir = dir;
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    load_modules();
    const std::string mode = argv[1];

    if (mode == "deriv" && argc == 9) {
        int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]), axis = atoi(argv[5]);
        double h = atof(argv[6]);
        size_t n = (size_t)nx * ny * nz;
        CUdeviceptr f = upload(read_bin(argv[7], n)), out = dalloc(n);
        ref_deriv(out, f, h, nx, ny, nz, axis);
        write_bin(argv[8], download(out, n));
    } else if (mode == "div" && argc == 17) {
        int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
        double hx = atof(argv[5]), hy = atof(argv[6]), hz = atof(argv[7]);
        size_t n = (size_t)nx * ny * nz;
        CUdeviceptr F[6];
        for (int q = 0; q < 6; ++q) F[q] = upload(read_bin(argv[8 + q], n));
        std::vector<double> jbn = read_bin(argv[14], 11 * n);
        CUdeviceptr J = upload(jbn);
        CUdeviceptr j0 = J, j4 = J + 4 * n * 8, j8 = J + 8 * n * 8, jdet = J + 9 * n * 8,
                    j10 = J + 10 * n * 8;
        CUfunction kP = find_kernel("kernProyectDataJBN<double>");
        CUfunction kD = find_kernel("kernGetDiv<double>");
        const int gx = cdiv(nx, 8), gy = cdiv(ny, 8), gz = cdiv(nz, 4);
        CUdeviceptr jc[6] = {j0, j4, j8, j0, j4, j8};
        for (int q = 0; q < 6; ++q) {   // cuDivergence.cu:166-172
            Arr a = arr(F[q], nx, ny, nz), b = arr(jdet, nx, ny, nz), c = arr(jc[q], nx, ny, nz);
            void *args[] = {&a, &b, &c};
            launch(kP, gx, gy, gz, 8, 8, 4, 0, args);
        }
        CUdeviceptr D[6];
        for (int q = 0; q < 6; ++q) D[q] = dalloc(n);
        ref_deriv(D[0], F[0], hx, nx, ny, nz, 0);   // :174-181
        ref_deriv(D[3], F[3], hx, nx, ny, nz, 0);
        ref_deriv(D[1], F[1], hy, nx, ny, nz, 1);
        ref_deriv(D[4], F[4], hy, nx, ny, nz, 1);
        ref_deriv(D[2], F[2], hz, nx, ny, nz, 2);
        ref_deriv(D[5], F[5], hz, nx, ny, nz, 2);
        CUdeviceptr rs = dalloc(n), rsv = dalloc(n);
        {   // :183-184
            Arr o = arr(rs, nx, ny, nz), jj = arr(j10, nx, ny, nz), a = arr(D[0], nx, ny, nz),
                b = arr(D[1], nx, ny, nz), c = arr(D[2], nx, ny, nz);
            void *args[] = {&o, &jj, &a, &b, &c};
            launch(kD, gx, gy, gz, 8, 8, 4, 0, args);
            Arr o2 = arr(rsv, nx, ny, nz), a2 = arr(D[3], nx, ny, nz), b2 = arr(D[4], nx, ny, nz),
                c2 = arr(D[5], nx, ny, nz);
            void *args2[] = {&o2, &jj, &a2, &b2, &c2};
            launch(kD, gx, gy, gz, 8, 8, 4, 0, args2);
        }
        write_bin(argv[15], download(rs, n));
        write_bin(argv[16], download(rsv, n));
    } else if (mode == "weno" && argc == 13) {
        unsigned nxg = atoi(argv[2]), nyg = atoi(argv[3]), nzg = atoi(argv[4]);
        double hx = atof(argv[5]), hy = atof(argv[6]), hz = atof(argv[7]), dt = atof(argv[8]);
        if (nxg % 10 || nyg % 10 || nzg % 5) {
            fprintf(stderr, "weno: padded sizes must tile the (10,10,5) blocks exactly\n");
            return 5;
        }
        size_t ng = (size_t)nxg * nyg * nzg;
        CUdeviceptr phi = upload(read_bin(argv[9], ng)), vel = upload(read_bin(argv[10], 3 * ng)),
                    jbn = upload(read_bin(argv[11], 11 * ng));
        CUdeviceptr dPhi = dalloc(3 * ng), pP = dalloc(3 * ng), pM = dalloc(3 * ng), rs = dalloc(ng),
                    tmp = dalloc(ng);
        CUfunction kD = find_kernel("Dev1thO_Downwind"), kP = find_kernel("PhiDevPlusParameterJB"),
                   kM = find_kernel("PhiDevMinusParameterJB"), kR = find_kernel("advect_RS_WENO"),
                   k1 = find_kernel("RunGK_FirstS"), k2 = find_kernel("RunGK_SecondS"),
                   k3 = find_kernel("RunGK_ThirdS");
        const int gx = nxg / 10, gy = nyg / 10, gz = nzg / 5;
        double sx = 1.0 / hx, sy = 1.0 / hy, sz = 1.0 / hz;
        int ix = nxg, iy = nyg, iz = nzg;
        for (int stage = 1; stage <= 3; ++stage) {
            CUdeviceptr src = stage == 1 ? phi : tmp;
            void *ad[] = {&dPhi, &src, &sx, &sy, &sz, &nxg, &nyg, &nzg};
            launch(kD, gx, gy, gz, 10, 10, 5, 0, ad);
            void *ap[] = {&pP, &dPhi, &jbn, &nxg, &nyg, &nzg};
            void *am[] = {&pM, &dPhi, &jbn, &nxg, &nyg, &nzg};
            launch(kP, gx, gy, gz, 10, 10, 5, 0, ap);
            launch(kM, gx, gy, gz, 10, 10, 5, 0, am);
            void *ar[] = {&rs, &vel, &pP, &pM, &nxg, &nyg, &nzg};
            launch(kR, gx, gy, gz, 10, 10, 5, 0, ar);
            if (stage == 1) {
                void *a[] = {&tmp, &phi, &dt, &rs, &ix, &iy, &iz};
                launch(k1, gx, gy, gz, 10, 10, 5, 0, a);
            } else if (stage == 2) {
                void *a[] = {&tmp, &phi, &tmp, &dt, &rs, &ix, &iy, &iz};
                launch(k2, gx, gy, gz, 10, 10, 5, 0, a);
            } else {
                void *a[] = {&phi, &phi, &tmp, &dt, &rs, &ix, &iy, &iz};
                launch(k3, gx, gy, gz, 10, 10, 5, 0, a);
            }
        }
        write_bin(argv[12], download(phi, ng));
    } else if (mode == "pad" && argc == 8) {
        int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]), g = atoi(argv[5]);
        const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
        if (nx % 10 || ny % 10 || nz % 5 || nxg % 10 || nyg % 10 || nxg != nyg || nyg != nzg) {
            fprintf(stderr, "pad: sizes must tile the reference grids exactly (cubic padded grid)\n");
            return 5;
        }
        size_t n = (size_t)nx * ny * nz, ng = (size_t)nxg * nyg * nzg;
        CUdeviceptr val = upload(read_bin(argv[6], n)), G = dalloc(ng);
        CUfunction kS = find_kernel("cuSwapToGhost"), kZ = find_kernel("cuGhostCellsMirror3dZ"),
                   kY = find_kernel("cuGhostCellsMirror3dY"), kX = find_kernel("cuGhostCellsMirror3dX");
        void *as[] = {&G, &val, &g, &nx, &ny, &nz};
        launch(kS, nx / 10, ny / 10, nz / 5, 10, 10, 5, 0, as);
        double dir = 1.0;
        void *am[] = {&G, &g, &nx, &ny, &nz, &dir};
        launch(kZ, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
        launch(kY, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
        launch(kX, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
        write_bin(argv[7], download(G, ng));
    } else if (mode == "extrap" && argc == 13) {
        int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
        double dX = atof(argv[5]), dY = atof(argv[6]), dZ = atof(argv[7]), dmin = atof(argv[8]);
        int g = 5;
        const int nxg = nx + 2 * g, nyg = ny + 2 * g, nzg = nz + 2 * g;
        if (nx % 10 || ny % 10 || nz % 5 || nxg != nyg || nyg != nzg) {
            fprintf(stderr, "extrap: sizes must tile the reference grids exactly (cubic padded grid)\n");
            return 5;
        }
        size_t n = (size_t)nx * ny * nz, ng = (size_t)nxg * nyg * nzg;
        CUdeviceptr pW = upload(read_bin(argv[9], n)), jW = upload(read_bin(argv[10], 11 * n)),
                    sW = upload(read_bin(argv[11], n));
        CUdeviceptr pG = dalloc(ng), sG = dalloc(ng), jG = dalloc(11 * ng);
        CUfunction kS = find_kernel("cuSwapToGhost"), kF = find_kernel("cuSwapFromGhost"),
                   kZ = find_kernel("cuGhostCellsMirror3dZ"), kY = find_kernel("cuGhostCellsMirror3dY"),
                   kX = find_kernel("cuGhostCellsMirror3dX"), kD = find_kernel("DevFirstOrder_LS"),
                   kE = find_kernel("extrapolKernel"), k1 = find_kernel("RunGK_FirstS"),
                   k2 = find_kernel("RunGK_SecondS"), k3 = find_kernel("RunGK_ThirdS");
        // lsTransportEc.cu:99-157: pad, then mirror (press and sobject Z,Y,X; jbn X,Y,Z)
        auto swap_to = [&](CUdeviceptr G, CUdeviceptr W) {
            void *a[] = {&G, &W, &g, &nx, &ny, &nz};
            launch(kS, nx / 10, ny / 10, nz / 5, 10, 10, 5, 0, a);
        };
        swap_to(pG, pW);
        for (int c : {0, 4, 8}) swap_to(jG + c * ng * sizeof(double), jW + c * n * sizeof(double));
        swap_to(sG, sW);
        double dir = 1.0;
        auto mirror = [&](CUfunction k, CUdeviceptr G) {
            void *a[] = {&G, &g, &nx, &ny, &nz, &dir};
            launch(k, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, a);
        };
        for (CUdeviceptr G : {pG, sG}) { mirror(kZ, G); mirror(kY, G); mirror(kX, G); }
        for (int c : {0, 4, 8}) {
            CUdeviceptr G = jG + c * ng * sizeof(double);
            mirror(kX, G); mirror(kY, G); mirror(kZ, G);
        }
        // cuExtrapolation(d_press, d_sobject, d_jbn, dX, dY, dZ, NxG, NyG, NzG, deltamin*0.5, 1)
        CUdeviceptr dPhi = dalloc(3 * ng), rs = dalloc(ng), d = dalloc(ng);
        const int gx = nxg / 10, gy = nyg / 10, gz = nzg / 5;
        double sx = 1.0 / dX, sy = 1.0 / dY, sz = 1.0 / dZ, dtext = dmin * 0.5;
        unsigned ux = nxg, uy = nyg, uz = nzg;
        int ix = nxg, iy = nyg, iz = nzg, flag = 1;
        void *ad[] = {&dPhi, &sG, &jG, &sx, &sy, &sz, &ux, &uy, &uz};
        launch(kD, gx, gy, gz, 10, 10, 5, 0, ad);
        for (int it = 1; it <= 10; ++it) {
            void *e1[] = {&rs, &pG, &sG, &jG, &dPhi, &sx, &sy, &sz, &ux, &uy, &uz, &flag};
            launch(kE, gx, gy, gz, 10, 10, 5, 0, e1);
            void *r1[] = {&d, &pG, &dtext, &rs, &ix, &iy, &iz};
            launch(k1, gx, gy, gz, 10, 10, 5, 0, r1);
            void *e2[] = {&rs, &d, &sG, &jG, &dPhi, &sx, &sy, &sz, &ux, &uy, &uz, &flag};
            launch(kE, gx, gy, gz, 10, 10, 5, 0, e2);
            void *r2[] = {&d, &pG, &d, &dtext, &rs, &ix, &iy, &iz};
            launch(k2, gx, gy, gz, 10, 10, 5, 0, r2);
            launch(kE, gx, gy, gz, 10, 10, 5, 0, e2);
            void *r3[] = {&pG, &pG, &d, &dtext, &rs, &ix, &iy, &iz};
            launch(k3, gx, gy, gz, 10, 10, 5, 0, r3);
        }
        void *af[] = {&pW, &pG, &g, &nx, &ny, &nz};
        launch(kF, nx / 10, ny / 10, nz / 5, 10, 10, 5, 0, af);
        write_bin(argv[12], download(pW, n));
    } else if (mode == "reinit" && argc == 15) {
        unsigned nxg = atoi(argv[2]), nyg = atoi(argv[3]), nzg = atoi(argv[4]);
        int g = atoi(argv[5]);
        double dX = atof(argv[6]), dY = atof(argv[7]), dZ = atof(argv[8]), dmin = atof(argv[9]);
        int iters = atoi(argv[10]);
        if (nxg % 10 || nyg % 10 || nzg % 5 || nxg != nyg || nyg != nzg || (int)nxg <= 2 * g) {
            fprintf(stderr, "reinit: sizes must tile the reference grids exactly (cubic padded grid)\n");
            return 5;
        }
        size_t ng = (size_t)nxg * nyg * nzg;
        CUdeviceptr phi = upload(read_bin(argv[11], ng)), jbn = upload(read_bin(argv[12], 11 * ng)),
                    dmins = upload(read_bin(argv[13], ng));
        CUdeviceptr dPhi = dalloc(3 * ng), pP = dalloc(3 * ng), pM = dalloc(3 * ng), rs = dalloc(ng),
                    phi0 = dalloc(ng), tmp = dalloc(ng);
        CUfunction kD = find_kernel("Dev1thO_Downwind"), kP = find_kernel("PhiDevPlusParameterJB"),
                   kM = find_kernel("PhiDevMinusParameterJB"), kR = find_kernel("reini_RS_WENOJB"),
                   k1 = find_kernel("RunGK_FirstS"), k2 = find_kernel("RunGK_SecondS"),
                   k3 = find_kernel("RunGK_ThirdS"), kZ = find_kernel("cuGhostCellsMirror3dZ"),
                   kY = find_kernel("cuGhostCellsMirror3dY"), kX = find_kernel("cuGhostCellsMirror3dX");
        const int gx = nxg / 10, gy = nyg / 10, gz = nzg / 5;
        double sx = 1.0 / dX, sy = 1.0 / dY, sz = 1.0 / dZ, dt = 0.5 * dmin, dir = 1.0;
        int ix = nxg, iy = nyg, iz = nzg, nxi = nxg - 2 * g, nyi = nyg - 2 * g, nzi = nzg - 2 * g;
        auto rhs = [&](CUdeviceptr f, bool plus_first) {
            void *ad[] = {&dPhi, &f, &sx, &sy, &sz, &nxg, &nyg, &nzg};
            launch(kD, gx, gy, gz, 10, 10, 5, 0, ad);
            void *ap[] = {&pP, &dPhi, &jbn, &nxg, &nyg, &nzg};
            void *am[] = {&pM, &dPhi, &jbn, &nxg, &nyg, &nzg};
            if (plus_first) {
                launch(kP, gx, gy, gz, 10, 10, 5, 0, ap);
                launch(kM, gx, gy, gz, 10, 10, 5, 0, am);
            } else {
                launch(kM, gx, gy, gz, 10, 10, 5, 0, am);
                launch(kP, gx, gy, gz, 10, 10, 5, 0, ap);
            }
            void *ar[] = {&rs, &f, &dmins, &pP, &pM, &phi0, &nxg, &nyg, &nzg};
            launch(kR, gx, gy, gz, 10, 10, 5, 0, ar);
        };
        for (int it = 0; it < iters; ++it) {
            // lsTransportEc.cu:476-489: mirror Z, Y, X, then phi0 = phi
            void *am[] = {&phi, &g, &nxi, &nyi, &nzi, &dir};
            launch(kZ, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
            launch(kY, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
            launch(kX, nxg / 10, nyg / 10, 1, 10, 10, 1, 0, am);
            CK(cuMemcpyDtoD(phi0, phi, ng * sizeof(double)));
            rhs(phi, true);
            void *a1[] = {&tmp, &phi, &dt, &rs, &ix, &iy, &iz};
            launch(k1, gx, gy, gz, 10, 10, 5, 0, a1);
            rhs(tmp, false);
            void *a2[] = {&tmp, &phi, &tmp, &dt, &rs, &ix, &iy, &iz};
            launch(k2, gx, gy, gz, 10, 10, 5, 0, a2);
            rhs(tmp, false);
            void *a3[] = {&phi, &phi, &tmp, &dt, &rs, &ix, &iy, &iz};
            launch(k3, gx, gy, gz, 10, 10, 5, 0, a3);
        }
        write_bin(argv[14], download(phi, ng));
    } else {
        fprintf(stderr, "bad arguments for mode %s\n", mode.c_str());
        return 1;
    }
    CK(cuCtxSynchronize());
    printf("ok %s\n", mode.c_str());
    return 0;
}
