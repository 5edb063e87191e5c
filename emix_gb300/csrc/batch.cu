// batch.cu -- many independent grids of uneven size advanced together.
//
// A batch owns one context per grid (each with its own arena, tables and
// plan).  Position k of every plan is the same kernel kind, so a batched step
// issues one launch per position over a work list of (grid, virtual block)
// items covering every grid's launch of that position: pointwise positions as
// persistent kernels whose CTAs walk the list, pencil and level-set positions
// with one CTA per item.  Small grids, which alone fill a fraction of the GPU
// and are bound by launch overhead, then share the machine.  The step is
// captured in a CUDA graph.  The work-list granularity (pencils per y/z block,
// cells per pointwise item, resident CTAs per SM of the persistent kernels)
// is chosen by a timing autotuner.
#include "ctx.cuh"
#include "pcr.cuh"
#include "weno_march.cuh"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

// the single-grid context (step.cu)
struct emix_ctx;
namespace emix {
const std::vector<Launch> &ctx_plan(emix_ctx *c);
int ctx_ready(emix_ctx *c);
} // namespace emix

namespace emix {
namespace {

// grid owning virtual block vb: largest g with start[g] <= vb
EMIX_DEV int find_grid(const long *__restrict__ start, int ngrid, long vb) {
    int lo = 0, hi = ngrid - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= vb) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct Shape {
    int gx, gy, gz, aux;
};

// pointwise bodies over `cpb` x 256 cells per virtual block
struct PrimOp { using A = PrimArgs; static EMIX_DEV void cell(const A &a, long q) { prim_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct PadOp { using A = PadArgs; static EMIX_DEV void cell(const A &a, long q) { pad_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.ng; } };
struct SmagOp { using A = SmagArgs; static EMIX_DEV void cell(const A &a, long q) { smag_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct SfOp { using A = SfArgs; static EMIX_DEV void cell(const A &a, long q) { sf_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct VortOp { using A = VortArgs; static EMIX_DEV void cell(const A &a, long q) { vort_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct SelOp { using A = SelArgs; static EMIX_DEV void cell(const A &a, long q) { select_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct FluxOp { using A = FluxArgs; static EMIX_DEV void cell(const A &a, long q) { flux_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return a.n; } };
struct BcOp { using A = BcArgs; static EMIX_DEV void cell(const A &a, long q) { bc_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return bc_count(a); } };
struct ClockOp { using A = ImpClockArgs; static EMIX_DEV void cell(const A &a, long q) { if (q == 0) imp_clock_tick(a); } static EMIX_DEV long cnt(const A &) { return 1; } };
struct RkOp { using A = RkArgs; static EMIX_DEV void cell(const A &a, long q) { rk_cell(a, q); } static EMIX_DEV long cnt(const A &a) { return rk_count(a); } };

template <class Op>
__global__ void __launch_bounds__(256, 2)
k_batch_cells(const typename Op::A *__restrict__ args, const long *__restrict__ start, int ngrid,
              int cpb) {
    const long total = start[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int g = find_grid(start, ngrid, vb);
        const typename Op::A &a = args[g];
        const long n = Op::cnt(a);
        const long q0 = (vb - start[g]) * 256L * cpb + threadIdx.x;
        for (int k = 0; k < cpb; ++k) {
            const long q = q0 + 256L * k;
            if (q < n) Op::cell(a, q);
        }
    }
}

// the z-marching stage body over (grid, column tile, z chunk) items
__global__ void __launch_bounds__(kNT, 4)
k_batch_weno(const WenoArgs *__restrict__ args, const long *__restrict__ start,
             const Shape *__restrict__ shape, int ngrid) {
    const long total = start[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int g = find_grid(start, ngrid, vb);
        const long local = vb - start[g];
        const Shape sh = shape[g];
        weno_march_body(args[g], (int)(local % sh.gx), (int)((local / sh.gx) % sh.gy),
                        (int)(local / ((long)sh.gx * sh.gy)), sh.gz);
        __syncthreads();   // the tiles are refilled by the next item
    }
}

template <int EPI>
__global__ void __launch_bounds__(128)
k_batch_deriv_x(const DerivArgs *__restrict__ args, const long *__restrict__ start,
                const Shape *__restrict__ shape, int ngrid) {
    extern __shared__ double smem[];
    const long total = start[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int g = find_grid(start, ngrid, vb);
        const long local = vb - start[g];
        const Shape sh = shape[g];
        const DerivArgs &a = args[g];
        const uint3 bid = make_uint3((unsigned)(local % sh.gx), 0u, (unsigned)(local / sh.gx));
        deriv_x_body<EPI>(a.T, a.F, (long)a.ny * a.nz, bid, threadIdx.x, blockDim.x >> 5, smem);
    }
}

// item vb of a y/z pencil position
template <int EPI>
EMIX_DEV void batch_yz_item(const DerivArgs *__restrict__ args, const long *__restrict__ start,
                            const Shape *__restrict__ shape, int ngrid, long vb) {
    const int g = find_grid(start, ngrid, vb);
    const long local = vb - start[g];
    const Shape sh = shape[g];
    const DerivArgs &a = args[g];
    const uint3 bid = make_uint3((unsigned)(local % sh.gx), (unsigned)((local / sh.gx) % sh.gy),
                                 (unsigned)(local / ((long)sh.gx * sh.gy)));
    const int nx = a.nx;
    const int nother = a.axis == 1 ? a.nz : a.ny;
    const long s = a.axis == 1 ? (long)nx : (long)nx * a.ny;
    const long os = a.axis == 1 ? (long)nx * a.ny : (long)nx;
    deriv_yz_body<EPI>(a.T, a.F, nx, nother, s, os, bid, threadIdx.x, blockDim.x);
}

template <int EPI>
__global__ void __launch_bounds__(128)
k_batch_deriv_yz(const DerivArgs *__restrict__ args, const long *__restrict__ start,
                 const Shape *__restrict__ shape, int ngrid) {
    const long total = start[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) batch_yz_item<EPI>(args, start, shape, ngrid, vb);
}

// a y/z position by PCR + Thomas (S steps): item = (x block of
// pcr_block_x<S>() pencils, other coordinate, field), one warp per 32 / 2^S
// pencils
template <int S, int EPI>
__global__ void __launch_bounds__(128)
k_batch_deriv_pcr(const DerivArgs *__restrict__ args, const PcrTable *__restrict__ pargs,
                  const long *__restrict__ start, const Shape *__restrict__ shape, int ngrid) {
    const long total = start[ngrid];
    const int warp = threadIdx.x >> 5;
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int g = find_grid(start, ngrid, vb);
        const long local = vb - start[g];
        const Shape sh = shape[g];
        const DerivArgs &a = args[g];
        const int bx = (int)(local % sh.gx), by = (int)((local / sh.gx) % sh.gy),
                  bz = (int)(local / ((long)sh.gx * sh.gy));
        const int nx = a.nx;
        const int nother = a.axis == 1 ? a.nz : a.ny;
        const long s = a.axis == 1 ? (long)nx : (long)nx * a.ny;
        const long os = a.axis == 1 ? (long)nx * a.ny : (long)nx;
        pcr_yz_warp<S, pcr_rows<S>(), EPI>(pargs[g], a.F, nx, nother, s, os,
                                           bx * pcr_block_x<S>() + warp * (32 >> S), by, bz);
    }
}

// two y/z positions (the gradients' y and z) over one work list
__global__ void __launch_bounds__(128)
k_batch_deriv_yz_pair(const DerivArgs *__restrict__ aa, const long *__restrict__ sa,
                      const Shape *__restrict__ ha, const DerivArgs *__restrict__ ab,
                      const long *__restrict__ sb, const Shape *__restrict__ hb, int ngrid) {
    const long ta = sa[ngrid], total = ta + sb[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        if (vb < ta) batch_yz_item<EPI_STORE>(aa, sa, ha, ngrid, vb);
        else batch_yz_item<EPI_STORE>(ab, sb, hb, ngrid, vb - ta);
    }
}

// Smagorinsky and the fluxes of a cell from one set of strain pieces, over
// the fluxes' work list (the same cells as the Smagorinsky position's)
__global__ void __launch_bounds__(256, 2)
k_batch_smag_flux(const SmagArgs *__restrict__ sargs, const FluxArgs *__restrict__ fargs,
                  const long *__restrict__ start, int ngrid, int cpb) {
    const long total = start[ngrid];
    for (long vb = blockIdx.x; vb < total; vb += gridDim.x) {
        const int g = find_grid(start, ngrid, vb);
        const FluxArgs &f = fargs[g];
        const long q0 = (vb - start[g]) * 256L * cpb + threadIdx.x;
        for (int k = 0; k < cpb; ++k) {
            const long q = q0 + 256L * k;
            if (q < f.n) smag_flux_cell(sargs[g], f, q);
        }
    }
}

} // namespace

// Launch configuration shared by all positions of a batch.
struct BatchTune {
    int cpb;       // cells per thread in pointwise items (x 256 per item)
    int yz_bs;     // threads per y/z pencil block
    int ctas_sm;   // resident CTAs per SM for the persistent grids
    int pcr;       // PCR steps of the y/z positions (0: one Thomas sweep per pencil)
};

struct BatchPos {
    int kind, cls, epi;
    int fuse;          // runs with the next position as one launch (plan_fuse_next, every grid)
    void *args;        // device array of ngrid argument structs
    long *start;       // device prefix sums of virtual blocks, ngrid + 1
    Shape *shape;      // device per-grid virtual launch shapes
    long total;
    PcrTable *pcr;     // y/z positions under tune.pcr > 0: device array of ngrid PCR tables
    int pcr_steps;     // PCR steps of this position (0: Thomas)
};

} // namespace emix

using namespace emix;

struct emix_batch {
    std::vector<emix_ctx *> grids;
    cudaStream_t stream = nullptr, own = nullptr;
    std::vector<BatchPos> pos;
    void *dmem = nullptr;           // one device allocation for all position tables
    BatchTune tune{4, 64, 4, 0};
    bool built = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int sms = 1;       // SMs of the device, set at creation
    // concurrency inside a step (emix_batch_set_overlap): bit 0 the level-set
    // positions, bit 1 the x-gradient positions on the second stream
    int overlap = 3;
    static constexpr int kForks = 6;   // per step: 3 level-set + 3 x-gradient positions
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev[kForks] = {}, join_ev[kForks] = {};
    // ms per step the last autotune measured: [0] the best Thomas shapes,
    // [k] the same with k PCR steps in the y/z positions (-1: not measured)
    double pcr_ms[kPcrMaxSteps + 1] = {-1.0, -1.0, -1.0, -1.0, -1.0, -1.0};
};

namespace {

size_t args_size(int kind) {
    switch (kind) {
    case LK_PRIM: return sizeof(PrimArgs);
    case LK_PAD: return sizeof(PadArgs);
    case LK_WENO: return sizeof(WenoArgs);
    case LK_DERIV_X: case LK_DERIV_YZ: return sizeof(DerivArgs);
    case LK_SMAG: return sizeof(SmagArgs);
    case LK_SF: return sizeof(SfArgs);
    case LK_VORT: return sizeof(VortArgs);
    case LK_SELECT: return sizeof(SelArgs);
    case LK_FLUX: return sizeof(FluxArgs);
    case LK_RK: return sizeof(RkArgs);
    case LK_BC: return sizeof(BcArgs);
    case LK_CLOCK: return sizeof(ImpClockArgs);
    default: return 0;
    }
}

const void *args_ptr(const Launch &L) {
    switch (L.kind) {
    case LK_PRIM: return &L.prim;
    case LK_PAD: return &L.pad;
    case LK_WENO: return &L.weno;
    case LK_DERIV_X: case LK_DERIV_YZ: return &L.deriv;
    case LK_SMAG: return &L.smag;
    case LK_SF: return &L.sf;
    case LK_VORT: return &L.vort;
    case LK_SELECT: return &L.sel;
    case LK_FLUX: return &L.flux;
    case LK_RK: return &L.rk;
    case LK_BC: return &L.bc;
    case LK_CLOCK: return &L.clock;
    default: return nullptr;
    }
}

long point_count(const Launch &L) {
    switch (L.kind) {
    case LK_PRIM: return L.prim.n;
    case LK_PAD: return L.pad.ng;
    case LK_SMAG: return L.smag.n;
    case LK_SF: return L.sf.n;
    case LK_VORT: return L.vort.n;
    case LK_SELECT: return L.sel.n;
    case LK_FLUX: return L.flux.n;
    case LK_RK: return rk_count(L.rk);
    case LK_BC: return bc_count(L.bc);
    case LK_CLOCK: return 1;
    default: return 0;
    }
}

// virtual launch shape of one grid's launch under the tuning `t`
Shape shape_of(const Launch &L, const BatchTune &t) {
    Shape s{1, 1, 1, 0};
    if (L.kind == LK_WENO) {
        // 16 x 16 columns in z chunks of at most 32 planes
        s.gx = (L.weno.rn[0] + kMX - 1) / kMX;
        s.gy = (L.weno.rn[1] + kMY - 1) / kMY;
        s.gz = (L.weno.rn[2] + 31) / 32;
    } else if (L.kind == LK_DERIV_X) {
        const long np = (long)L.deriv.ny * L.deriv.nz;
        s.gx = (int)((np + 127) / 128);
        s.gz = L.deriv.nf;
    } else if (L.kind == LK_DERIV_YZ && t.pcr > 0) {
        const int bxp = 4 * (32 >> t.pcr);
        s.gx = (L.deriv.nx + bxp - 1) / bxp;
        s.gy = L.deriv.axis == 1 ? L.deriv.nz : L.deriv.ny;
        s.gz = L.deriv.nf;
    } else if (L.kind == LK_DERIV_YZ) {
        s.gx = (L.deriv.nx + t.yz_bs - 1) / t.yz_bs;
        s.gy = L.deriv.axis == 1 ? L.deriv.nz : L.deriv.ny;
        s.gz = L.deriv.nf;
    } else {
        const long per = 256L * t.cpb;
        s.gx = (int)((point_count(L) + per - 1) / per);
    }
    return s;
}

int build(emix_batch *b) {
    const int G = (int)b->grids.size();
    std::vector<const std::vector<Launch> *> plans(G);
    for (int g = 0; g < G; ++g) {
        if (!ctx_ready(b->grids[g])) {
            set_last_message("emix_batch_step: static fields of a grid not set");
            return EMIX_ERR_ARG;
        }
        plans[g] = &ctx_plan(b->grids[g]);
        if (plans[g]->size() != plans[0]->size()) {
            set_last_message("emix_batch: grids must share level-set and SGS options");
            return EMIX_ERR_ARG;
        }
    }
    const size_t np = plans[0]->size();
    // host image of every position's tables, laid out back to back
    std::vector<unsigned char> host;
    std::vector<size_t> off_args(np), off_start(np), off_shape(np), off_pcr(np, 0);
    std::vector<long> totals(np);
    std::vector<int> pcr_on(np, 0);
    auto align = [&](size_t a) { host.resize((host.size() + a - 1) / a * a); };
    for (size_t k = 0; k < np; ++k) {
        const Launch &L0 = (*plans[0])[k];
        const size_t as = args_size(L0.kind);
        align(256);
        off_args[k] = host.size();
        host.resize(host.size() + as * G);
        std::vector<long> start(G + 1, 0);
        std::vector<Shape> sh(G);
        // y/z positions run by PCR + Thomas when the tuning asks for it and
        // every grid's pencils fit (at most kPcrMaxN rows)
        BatchTune tk = b->tune;
        if (L0.kind == LK_DERIV_YZ && tk.pcr > 0) {
            for (int g = 0; g < G; ++g) {
                const Launch &L = (*plans[g])[k];
                if ((L.deriv.axis == 1 ? L.deriv.ny : L.deriv.nz) > kPcrMaxN) tk.pcr = 0;
            }
        } else {
            tk.pcr = 0;
        }
        pcr_on[k] = tk.pcr;
        for (int g = 0; g < G; ++g) {
            const Launch &L = (*plans[g])[k];
            if (L.kind != L0.kind || (L.kind == LK_DERIV_X || L.kind == LK_DERIV_YZ ? L.deriv.epi != L0.deriv.epi : false)) {
                set_last_message("emix_batch: plans of the grids differ");
                return EMIX_ERR_ARG;
            }
            std::memcpy(host.data() + off_args[k] + as * g, args_ptr(L), as);
            sh[g] = shape_of(L, tk);
            start[g + 1] = start[g] + (long)sh[g].gx * sh[g].gy * sh[g].gz;
        }
        totals[k] = start[G];
        align(256);
        off_start[k] = host.size();
        host.resize(host.size() + sizeof(long) * (G + 1));
        std::memcpy(host.data() + off_start[k], start.data(), sizeof(long) * (G + 1));
        align(256);
        off_shape[k] = host.size();
        host.resize(host.size() + sizeof(Shape) * G);
        std::memcpy(host.data() + off_shape[k], sh.data(), sizeof(Shape) * G);
        if (pcr_on[k]) {
            std::vector<PcrTable> pt(G);
            for (int g = 0; g < G; ++g) {
                const Launch &L = (*plans[g])[k];
                const int ax = L.deriv.axis;
                const emix_params &gp = b->grids[g]->p;
                int rc = get_pcr_table(gp.scheme[ax], ax == 1 ? L.deriv.ny : L.deriv.nz, gp.h[ax], pcr_on[k],
                                       &pt[g]);
                if (rc) return rc;
            }
            align(256);
            off_pcr[k] = host.size();
            host.resize(host.size() + sizeof(PcrTable) * G);
            std::memcpy(host.data() + off_pcr[k], pt.data(), sizeof(PcrTable) * G);
        }
    }
    if (b->dmem) cudaFree(b->dmem);
    b->dmem = nullptr;
    if (cudaMalloc(&b->dmem, host.size()) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("cudaMalloc of the batch tables failed");
        return EMIX_ERR_ALLOC;
    }
    EMIX_CUDA_TRY(cudaMemcpy(b->dmem, host.data(), host.size(), cudaMemcpyHostToDevice));
    b->pos.assign(np, BatchPos{});
    unsigned char *base = static_cast<unsigned char *>(b->dmem);
    for (size_t k = 0; k < np; ++k) {
        const Launch &L0 = (*plans[0])[k];
        BatchPos &P = b->pos[k];
        P.kind = L0.kind;
        P.cls = L0.cls;
        P.epi = (L0.kind == LK_DERIV_X || L0.kind == LK_DERIV_YZ) ? L0.deriv.epi : 0;
        P.args = base + off_args[k];
        P.start = reinterpret_cast<long *>(base + off_start[k]);
        P.shape = reinterpret_cast<Shape *>(base + off_shape[k]);
        P.total = totals[k];
        P.pcr = pcr_on[k] ? reinterpret_cast<PcrTable *>(base + off_pcr[k]) : nullptr;
        P.fuse = plan_fuse_next(*plans[0], k);
        for (int g = 1; g < G && P.fuse; ++g)
            if (plan_fuse_next(*plans[g], k) != P.fuse) P.fuse = 0;
        // the gradients' y and z pair runs as one Thomas launch only
        if (P.fuse == 1 && (pcr_on[k] || (k + 1 < np && pcr_on[k + 1]))) P.fuse = 0;
    }
    for (size_t k = 0; k < np; ++k) b->pos[k].pcr_steps = pcr_on[k];
    b->built = true;
    return EMIX_OK;
}

// one CTA per work item: the pencil walks and the stage's z marches are long
// and latency-bound, so the hardware scheduler keeps as many of them resident
// as registers and shared memory allow (a persistent grid of a few CTAs per SM
// would cap the resident warps)
int all_items(long total) {
    const long c = total < 1 ? 1 : (total > 2147483647L ? 2147483647L : total);
    return (int)c;
}

// CTAs of a pointwise position: a persistent grid of ctas_sm per SM, or (0)
// one CTA per item
int ctas(const emix_batch *b, long total) {
    if (b->tune.ctas_sm == 0) return all_items(total);
    long c = (long)b->sms * b->tune.ctas_sm;
    if (c > total) c = total;
    return (int)(c < 1 ? 1 : c);
}

// position k on stream st (with the next one where they run as one launch);
// *used: the positions it covered
int launch_pos(emix_batch *b, size_t k, cudaStream_t st, size_t *used) {
    const int G = (int)b->grids.size();
    const size_t npos = b->pos.size();
    *used = 1;
    {
        const BatchPos &P = b->pos[k];
        if (P.fuse && k + 1 < npos) {
            const BatchPos &Q = b->pos[k + 1];
            if (P.fuse == 1)
                k_batch_deriv_yz_pair<<<all_items(P.total + Q.total), b->tune.yz_bs, 0, st>>>(
                    (const DerivArgs *)P.args, P.start, P.shape, (const DerivArgs *)Q.args, Q.start, Q.shape, G);
            else
                k_batch_smag_flux<<<ctas(b, Q.total), 256, 0, st>>>((const SmagArgs *)P.args,
                                                                   (const FluxArgs *)Q.args, Q.start, G,
                                                                   b->tune.cpb);
            *used = 2;
            EMIX_CUDA_TRY(cudaGetLastError());
            return EMIX_OK;
        }
        const int nb = ctas(b, P.total);
        switch (P.kind) {
        case LK_PRIM: k_batch_cells<PrimOp><<<nb, 256, 0, st>>>((const PrimArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_PAD: k_batch_cells<PadOp><<<nb, 256, 0, st>>>((const PadArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_SMAG: k_batch_cells<SmagOp><<<nb, 256, 0, st>>>((const SmagArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_SF: k_batch_cells<SfOp><<<nb, 256, 0, st>>>((const SfArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_VORT: k_batch_cells<VortOp><<<nb, 256, 0, st>>>((const VortArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_SELECT: k_batch_cells<SelOp><<<nb, 256, 0, st>>>((const SelArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_FLUX: k_batch_cells<FluxOp><<<nb, 256, 0, st>>>((const FluxArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_RK: k_batch_cells<RkOp><<<nb, 256, 0, st>>>((const RkArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_BC: k_batch_cells<BcOp><<<nb, 256, 0, st>>>((const BcArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_CLOCK: k_batch_cells<ClockOp><<<nb, 256, 0, st>>>((const ImpClockArgs *)P.args, P.start, G, b->tune.cpb); break;
        case LK_WENO:
            k_batch_weno<<<all_items(P.total), kNT, 0, st>>>((const WenoArgs *)P.args, P.start, P.shape, G);
            break;
        case LK_DERIV_X: {
            const size_t shm = 4 * kXTile * sizeof(double);
            if (P.epi == EPI_STORE)
                k_batch_deriv_x<EPI_STORE><<<all_items(P.total), 128, shm, st>>>((const DerivArgs *)P.args, P.start, P.shape, G);
            else
                k_batch_deriv_x<EPI_ACCUM><<<all_items(P.total), 128, shm, st>>>((const DerivArgs *)P.args, P.start, P.shape, G);
            break;
        }
        case LK_DERIV_YZ:
            if (P.pcr) {
                const DerivArgs *da = (const DerivArgs *)P.args;
                const int nbk = all_items(P.total);
#define EMIX_PCR_CASE(S)                                                                                 \
    case S:                                                                                              \
        if (P.epi == EPI_STORE)                                                                          \
            k_batch_deriv_pcr<S, EPI_STORE><<<nbk, 128, 0, st>>>(da, P.pcr, P.start, P.shape, G);         \
        else                                                                                             \
            k_batch_deriv_pcr<S, EPI_ACCUM><<<nbk, 128, 0, st>>>(da, P.pcr, P.start, P.shape, G);         \
        break;
                switch (P.pcr_steps) {
                    EMIX_PCR_CASE(2)
                    EMIX_PCR_CASE(3)
                    EMIX_PCR_CASE(4)
                    EMIX_PCR_CASE(5)
                default:
                    return EMIX_ERR_ARG;
                }
#undef EMIX_PCR_CASE
                break;
            }
            if (P.epi == EPI_STORE)
                k_batch_deriv_yz<EPI_STORE><<<all_items(P.total), b->tune.yz_bs, 0, st>>>((const DerivArgs *)P.args, P.start, P.shape, G);
            else
                k_batch_deriv_yz<EPI_ACCUM><<<all_items(P.total), b->tune.yz_bs, 0, st>>>((const DerivArgs *)P.args, P.start, P.shape, G);
            break;
        default:
            return EMIX_ERR_ARG;
        }
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

// one step: the positions in order on the batch's stream; with the second
// stream, the level-set positions there joined before the next RK update
// (which overwrites the velocity they read), the x-gradient positions joined
// before the first position after the gradients' y and z
int issue(emix_batch *b) {
    cudaStream_t st = b->stream;
    const bool fork = (b->overlap & 1) && b->side, gfork = (b->overlap & 2) && b->side;
    const size_t npos = b->pos.size();
    int ne = 0;   // events used
    int wjoin = -1, gjoin = -1;   // pending joins (event index)
    for (size_t k = 0; k < npos;) {
        const BatchPos &P = b->pos[k];
        const bool w = fork && P.kind == LK_WENO, gx = gfork && P.kind == LK_DERIV_X && P.cls == CLS_GRADX;
        if (gjoin >= 0 && P.cls != CLS_GRADY && P.cls != CLS_GRADZ) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, b->join_ev[gjoin], 0));
            gjoin = -1;
        }
        if (wjoin >= 0 && P.kind == LK_RK) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, b->join_ev[wjoin], 0));
            wjoin = -1;
        }
        size_t used = 1;
        if ((w || gx) && ne < emix_batch::kForks) {
            EMIX_CUDA_TRY(cudaEventRecord(b->fork_ev[ne], st));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(b->side, b->fork_ev[ne], 0));
            if (int rc = launch_pos(b, k, b->side, &used)) return rc;
            EMIX_CUDA_TRY(cudaEventRecord(b->join_ev[ne], b->side));
            (w ? wjoin : gjoin) = ne++;
        } else if (int rc = launch_pos(b, k, st, &used)) {
            return rc;
        }
        k += used;
    }
    if (wjoin >= 0) EMIX_CUDA_TRY(cudaStreamWaitEvent(st, b->join_ev[wjoin], 0));
    if (gjoin >= 0) EMIX_CUDA_TRY(cudaStreamWaitEvent(st, b->join_ev[gjoin], 0));
    return EMIX_OK;
}

void drop_graph(emix_batch *b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
}

void destroy_side(emix_batch *b) {
    for (int e = 0; e < emix_batch::kForks; ++e) {
        if (b->fork_ev[e]) cudaEventDestroy(b->fork_ev[e]);
        if (b->join_ev[e]) cudaEventDestroy(b->join_ev[e]);
        b->fork_ev[e] = b->join_ev[e] = nullptr;
    }
    if (b->side) cudaStreamDestroy(b->side);
    b->side = nullptr;
}

int step_impl(emix_batch *b, int nsteps, int use_graph) {
    if (!b->built) {
        int rc = build(b);
        if (rc) return rc;
    }
    if (!use_graph) {
        for (int s = 0; s < nsteps; ++s) {
            int rc = issue(b);
            if (rc) return rc;
        }
        return EMIX_OK;
    }
    if (!b->gexec) {
        EMIX_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc = issue(b);
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &gr);
        if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
        if (e != cudaSuccess) { set_last_error(e, "cudaStreamEndCapture", __FILE__, __LINE__); return EMIX_ERR_CUDA; }
        b->graph = gr;
        e = cudaGraphInstantiate(&b->gexec, gr, 0);
        if (e != cudaSuccess) {
            drop_graph(b);
            set_last_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
            return EMIX_ERR_CUDA;
        }
    }
    for (int s = 0; s < nsteps; ++s) EMIX_CUDA_TRY(cudaGraphLaunch(b->gexec, b->stream));
    return EMIX_OK;
}

} // namespace

extern "C" {

int emix_batch_create(int ngrid, const emix_params *params, emix_batch **out) {
    if (!out || !params || ngrid < 1) return EMIX_ERR_ARG;
    *out = nullptr;
    for (int g = 0; g < ngrid; ++g)
        if (params[g].imp.on && params[g].imp.interp) {
            set_last_message("emix_batch_create: the impeller's blade-edge interpolation is not batched");
            return EMIX_ERR_ARG;
        }
    for (int g = 0; g < ngrid; ++g)
        if (params[g].filter_every != 0) {
            set_last_message("emix_batch_create: the compact filter is not batched (filter_every must be 0)");
            return EMIX_ERR_ARG;
        }
    for (int g = 1; g < ngrid; ++g)
        if (params[g].level_set != params[0].level_set || params[g].sgs_model != params[0].sgs_model ||
            params[g].bc_walls != params[0].bc_walls ||
            (params[0].level_set && params[g].ls_ghost != params[0].ls_ghost))
            return EMIX_ERR_ARG;
    emix_batch *b = new (std::nothrow) emix_batch();
    if (!b) return EMIX_ERR_ALLOC;
    b->sms = device_sms();
    for (int g = 0; g < ngrid; ++g) {
        emix_ctx *c = nullptr;
        int rc = emix_ctx_create(&params[g], &c);
        if (rc) {
            for (emix_ctx *x : b->grids) emix_ctx_destroy(x);
            delete b;
            return rc;
        }
        b->grids.push_back(c);
    }
    if (cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        for (emix_ctx *x : b->grids) emix_ctx_destroy(x);
        delete b;
        return EMIX_ERR_CUDA;
    }
    b->stream = b->own;
    for (emix_ctx *c : b->grids) emix_ctx_set_stream(c, b->stream);
    // the second stream of the step's concurrency (without it, one stream)
    bool ok = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) == cudaSuccess;
    for (int e = 0; e < emix_batch::kForks && ok; ++e)
        ok = cudaEventCreateWithFlags(&b->fork_ev[e], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->join_ev[e], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        destroy_side(b);
    }
    *out = b;
    return EMIX_OK;
}

int emix_batch_destroy(emix_batch *b) {
    if (!b) return EMIX_ERR_ARG;
    cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (emix_ctx *c : b->grids) emix_ctx_destroy(c);
    if (b->dmem) cudaFree(b->dmem);
    destroy_side(b);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return EMIX_OK;
}

int emix_batch_grid(emix_batch *b, int g, emix_ctx **ctx) {
    if (!b || !ctx || g < 0 || g >= (int)b->grids.size()) return EMIX_ERR_ARG;
    *ctx = b->grids[g];
    return EMIX_OK;
}

int emix_batch_set_stream(emix_batch *b, void *stream) {
    if (!b) return EMIX_ERR_ARG;
    b->stream = stream ? (cudaStream_t)stream : b->own;
    for (emix_ctx *c : b->grids) emix_ctx_set_stream(c, b->stream);
    drop_graph(b);
    return EMIX_OK;
}

int emix_batch_step(emix_batch *b, int nsteps, int use_graph) {
    if (!b || nsteps < 0) return EMIX_ERR_ARG;
    return step_impl(b, nsteps, use_graph);
}

int emix_batch_step_per_grid(emix_batch *b, int nsteps, int use_graph) {
    if (!b || nsteps < 0) return EMIX_ERR_ARG;
    for (int s = 0; s < nsteps; ++s)
        for (emix_ctx *c : b->grids) {
            int rc = emix_step(c, 1, use_graph);
            if (rc) return rc;
        }
    return EMIX_OK;
}

int emix_batch_set_tuning(emix_batch *b, int cells_per_thread, int yz_block, int ctas_per_sm) {
    if (!b || cells_per_thread < 1 || cells_per_thread > 64 || ctas_per_sm < 0 || ctas_per_sm > 64 ||
        (yz_block != 32 && yz_block != 64 && yz_block != 128))
        return EMIX_ERR_ARG;
    b->tune = BatchTune{cells_per_thread, yz_block, ctas_per_sm, b->tune.pcr};
    b->built = false;
    drop_graph(b);
    return EMIX_OK;
}

int emix_batch_get_tuning(emix_batch *b, int *cells_per_thread, int *yz_block, int *ctas_per_sm) {
    if (!b) return EMIX_ERR_ARG;
    if (cells_per_thread) *cells_per_thread = b->tune.cpb;
    if (yz_block) *yz_block = b->tune.yz_bs;
    if (ctas_per_sm) *ctas_per_sm = b->tune.ctas_sm;
    return EMIX_OK;
}

int emix_batch_set_overlap(emix_batch *b, int mode) {
    if (!b || mode < 0 || mode > 3) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->overlap = mode;
    drop_graph(b);
    return EMIX_OK;
}

int emix_batch_set_pcr(emix_batch *b, int steps) {
    if (!b || (steps != 0 && (steps < 2 || steps > kPcrMaxSteps))) return EMIX_ERR_ARG;
    b->tune.pcr = steps;
    b->built = false;
    drop_graph(b);
    return EMIX_OK;
}

int emix_batch_get_pcr(emix_batch *b, int *steps) {
    if (!b || !steps) return EMIX_ERR_ARG;
    *steps = b->tune.pcr;
    return EMIX_OK;
}

int emix_batch_pcr_positions(emix_batch *b, int *count) {
    if (!b || !count) return EMIX_ERR_ARG;
    if (!b->built) {
        int rc = build(b);
        if (rc) return rc;
    }
    int c = 0;
    for (const BatchPos &P : b->pos) c += P.pcr_steps > 0 ? 1 : 0;
    *count = c;
    return EMIX_OK;
}

int emix_batch_autotune(emix_batch *b, int nsteps, double *best_ms) {
    // Times every candidate launch configuration on the real batch (the state
    // advances; callers re-upload their initial state afterwards) and keeps
    // the fastest.
    if (!b || nsteps < 1) return EMIX_ERR_ARG;
    const int cpbs[] = {1, 4};
    const int bss[] = {32, 64, 128};
    const int ctass[] = {0, 2, 4, 8};
    BatchTune best = b->tune;
    float best_t = 1e30f;
    cudaEvent_t e0, e1;
    EMIX_CUDA_TRY(cudaEventCreate(&e0));
    EMIX_CUDA_TRY(cudaEventCreate(&e1));
    int rc = EMIX_OK;
    for (double &m : b->pcr_ms) m = -1.0;
    // ms per step of the current tuning
    auto timed = [&](float *ms) -> int {
        int r = step_impl(b, 1, 0);   // build + warm
        if (r) return r;
        cudaEventRecord(e0, b->stream);
        if ((r = step_impl(b, nsteps, 0))) return r;
        cudaEventRecord(e1, b->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) return EMIX_ERR_CUDA;
        cudaEventElapsedTime(ms, e0, e1);
        *ms /= nsteps;
        return EMIX_OK;
    };
    // the launch shapes with one Thomas sweep per pencil, then the PCR depth
    // of the y/z positions on the best of those
    b->tune.pcr = 0;
    for (int cpb : cpbs)
        for (int bs : bss)
            for (int cs : ctass) {
                if ((rc = emix_batch_set_tuning(b, cpb, bs, cs))) goto done;
                float ms = 0.f;
                if ((rc = timed(&ms))) goto done;
                if (ms < best_t) { best_t = ms; best = b->tune; }
            }
    b->pcr_ms[0] = best_t;
    for (int sp = 2; sp <= kPcrMaxSteps; ++sp) {
        if ((rc = emix_batch_set_tuning(b, best.cpb, best.yz_bs, best.ctas_sm))) goto done;
        if ((rc = emix_batch_set_pcr(b, sp))) goto done;
        float ms = 0.f;
        if ((rc = timed(&ms))) goto done;
        b->pcr_ms[sp] = ms;
        if (ms < best_t) { best_t = ms; best = b->tune; }
    }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    b->tune.pcr = best.pcr;
    rc = emix_batch_set_tuning(b, best.cpb, best.yz_bs, best.ctas_sm);
    if (best_ms) *best_ms = best_t;
    return rc;
}

int emix_batch_autotune_pcr_ms(emix_batch *b, double *ms) {
    if (!b || !ms) return EMIX_ERR_ARG;
    for (int k = 0; k <= kPcrMaxSteps; ++k) ms[k] = b->pcr_ms[k];
    return EMIX_OK;
}

} // extern "C"
