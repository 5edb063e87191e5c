// adjoint.cu -- reverse-mode gradient of a tank objective through the RK3
// step: dJ/d(omega, Cs) for the impeller angular velocity and the
// Smagorinsky constant.
//
// Forward: nsteps graph-replayed steps of the context, saving the state
// (um0, phi and the impeller clock) every `every` steps (checkpoints), then J.
// Reverse: per segment of `every` steps (last first), the states of the
// segment are recomputed from its checkpoint; per step (last first), the step
// is recomputed once more with a tape of every substep's inputs (u, pres,
// dvel, vis, divergence R, the substep's um), then the step's adjoint runs.
// With every = 0, where HBM holds every step's tape, the forward pass tapes
// each step as it runs and the reverse sweep recomputes nothing.  The step's
// adjoint runs substep by substep in reverse:
//   RK update (conversions, impeller, walls, combination) -> divergence (D^T)
//   -> fluxes -> Smagorinsky -> gradients (D^T) -> level-set stage (WENO5)
// and finally the primitive variables and the transposed ghost padding.
#include "adjoint.cuh"
#include "adjoint_weno.cuh"
#include "ctx.cuh"

#include <cstring>
#include <new>
#include <vector>

// the inputs of one step's substeps that its adjoint reads; in the mode that
// keeps every step's tape (every = 0) also the level-set stages' padded
// inputs and the impeller clock, which the context overwrites step by step
struct Tape {
    double *um0 = nullptr, *u[3] = {}, *p[3] = {}, *dvel[3] = {}, *vis[3] = {}, *R[3] = {}, *umc[3] = {};
    double *phig[3] = {};   // keep mode: stage inputs (else the context's buffers)
    double *clock = nullptr; // keep mode: the step's impeller clock (kImpClockLen)
};

struct emix_adj {
    emix_ctx *c = nullptr;
    int nsteps = 0, every = 1;
    bool keep = false;               // every = 0: every step's tape kept, no recomputation
    emix_objective obj{};
    double *arena = nullptr;
    size_t bytes = 0;
    double *cp = nullptr;            // checkpoints: (nsteps/every + 1) x 6n
    double *cp_clock = nullptr;      // impeller clock (t0, k) of each checkpoint (device)
    double *seg = nullptr;           // states of one segment: every x 6n
    double *seg_clock = nullptr;
    double *final_state = nullptr;   // 6n, restored after the reverse sweep
    double *final_clock = nullptr;   // 2
    // tape of the step being differentiated (tapes[k] in the keep mode)
    Tape *tape = nullptr;
    std::vector<Tape> tapes;
    double *final_clock_full = nullptr;   // keep mode: the clock after the last step
    // adjoint fields
    double *Lum0, *LA, *LB, *LU0, *LU1, *LP0, *LP1, *LR, *LF, *Ldvel, *Lvis, *T5, *W;
    double *Lphi, *Lphi_prev, *Lphig0, *LphiA, *LphiB, *LD;
    double *LuW;                     // the level-set stage's velocity adjoint (second stream)
    double *red;                     // [0] dJ/domega, [1] dJ/dCs, [2] J
    emix::DerivTTable TT[3];
    double J = 0.0;
    // tensor maps of the reverse sweep's y/z D^T passes (rows by TMA while the
    // context's pencil_tma is on): the divergence's per axis, the gradients'
    // per axis and target (LU0, LU1); ok where the copy unit's rules hold
    emix::PencilMaps tdiv[2], tgrad[2][2];
    bool tdiv_ok[2] = {false, false}, tgrad_ok[2][2] = {{false, false}, {false, false}};
    // the taped forward's second-stream work (emix_adj_set_overlap)
    int overlap = 1;
    cudaEvent_t ev_fork = nullptr, ev_a = nullptr, ev_b = nullptr;
    // the reverse sweep's level-set adjoints on the second stream
    cudaEvent_t ev_wfork = nullptr, ev_wdone = nullptr, ev_wfree = nullptr;
};

namespace emix {
namespace {

int grid_n(long n) { return grid_cap(n, 8); }

bool has_clock(const emix_ctx *c) { return c->clock != nullptr; }

// state of the context <-> a 6n buffer (um0, phi) plus the clock head (2
// values), all on the device and in stream order
int save_state(emix_adj *a, double *dst, double *clk) {
    emix_ctx *c = a->c;
    const long n = c->n;
    cudaStream_t st = c->stream;
    EMIX_CUDA_TRY(cudaMemcpyAsync(dst, c->um0, 5 * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(dst + 5 * n, c->phi, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (has_clock(c))
        EMIX_CUDA_TRY(cudaMemcpyAsync(clk, c->clock, 2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return EMIX_OK;
}

int load_state(emix_adj *a, const double *src, const double *clk) {
    emix_ctx *c = a->c;
    const long n = c->n;
    cudaStream_t st = c->stream;
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->um0, src, 5 * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->phi, src + 5 * n, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (has_clock(c))
        EMIX_CUDA_TRY(cudaMemcpyAsync(c->clock, clk, 2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return EMIX_OK;
}

int copy(double *dst, const double *src, long cnt, cudaStream_t st) {
    EMIX_CUDA_TRY(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return EMIX_OK;
}

int zero(double *p, long cnt, cudaStream_t st) {
    EMIX_CUDA_TRY(cudaMemsetAsync(p, 0, cnt * sizeof(double), st));
    return EMIX_OK;
}

} // namespace
} // namespace emix

namespace emix {
namespace {

// one step with its tape (the launches of the plan, eager, with copies of
// each substep's inputs).  With the context's second stream (a->overlap) the
// tape copies and the level-set stages run there, overlapped with the flow's
// kernels: each copy forks after the record that produced its source; the
// substep's inputs (um0, u, pres, um, the stage's padded phi) and its
// level-set stage join before its RK update, which overwrites u, pres and um;
// the gradients, viscosity and divergence join before the next substep's
// gradients, which overwrite the first of them, or at the step's end.
int taped_step(emix_adj *a) {
    emix_ctx *c = a->c;
    const long n = c->n;
    cudaStream_t st = c->stream;
    const bool two = a->overlap && c->side && a->ev_fork;
    cudaStream_t sd = two ? c->side : st;
    bool pend_a = false, pend_b = false;
    // fork the second stream after what the compute stream has issued so far
    auto fork = [&]() -> int {
        if (two) {
            EMIX_CUDA_TRY(cudaEventRecord(a->ev_fork, st));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, a->ev_fork, 0));
        }
        return EMIX_OK;
    };
    auto done = [&](cudaEvent_t ev, bool &pend) -> int {
        if (two) {
            EMIX_CUDA_TRY(cudaEventRecord(ev, sd));
            pend = true;
        }
        return EMIX_OK;
    };
    auto join = [&](cudaEvent_t ev, bool &pend) -> int {
        if (pend) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, ev, 0));
            pend = false;
        }
        return EMIX_OK;
    };
    Tape &T = *a->tape;
    int rc;
    if ((rc = fork()) || (rc = copy(T.um0, c->um0, 5 * n, sd)) || (rc = done(a->ev_a, pend_a))) return rc;
    int s = 0;
    const std::vector<Launch> &P = c->plan;
    for (size_t k = 0; k < P.size(); ++k) {
        const Launch &L = P[k];
        if (L.kind == LK_RK && (rc = join(a->ev_a, pend_a))) return rc;
        if (L.kind == LK_DERIV_X && L.cls == CLS_GRADX && (rc = join(a->ev_b, pend_b))) return rc;
        if (L.kind == LK_WENO) {
            ++s;
            if ((rc = fork())) return rc;
            if ((rc = copy(T.u[s - 1], c->u, 3 * n, sd))) return rc;
            if ((rc = copy(T.p[s - 1], c->pres, n, sd))) return rc;
            if (s >= 2 && (rc = copy(T.umc[s - 1], c->um, 5 * n, sd))) return rc;
            if (T.phig[s - 1] && (rc = copy(T.phig[s - 1], L.weno.phi, c->ng, sd))) return rc;
            if ((rc = launch_single(L, sd)) || (rc = done(a->ev_a, pend_a))) return rc;
            continue;
        }
        // the records the step runs as one launch run as one here too (the
        // same values bit for bit); the tape copies follow the pair
        const int fuse = c->fuse ? plan_fuse_next(P, k) : 0;
        const Launch *last = &L;
        if (fuse) {
            if ((rc = launch_fused_pair(P, k, st))) return rc;
            last = &P[++k];
        } else if ((rc = launch_single(L, st))) {
            return rc;
        }
        if (L.kind == LK_CLOCK && T.clock && (rc = copy(T.clock, c->clock, kImpClockLen, st))) return rc;
        if (s >= 1) {
            double *dst = nullptr;
            const double *src = nullptr;
            long cnt = 0;
            if (last->cls == CLS_GRADZ) { dst = T.dvel[s - 1]; src = c->dvel; cnt = 9 * n; }
            if (L.kind == LK_SMAG) { dst = T.vis[s - 1]; src = c->vis; cnt = n; }
            if (last->cls == CLS_DIVZ) { dst = T.R[s - 1]; src = c->R; cnt = 5 * n; }
            if (dst && ((rc = fork()) || (rc = copy(dst, src, cnt, sd)) || (rc = done(a->ev_b, pend_b))))
                return rc;
        }
    }
    if ((rc = join(a->ev_a, pend_a)) || (rc = join(a->ev_b, pend_b))) return rc;
    return s == 3 ? EMIX_OK : EMIX_ERR_ARG;
}

// the forward arguments of substep s's RK launch (the non-wall one) and of
// its level-set stage
const Launch *plan_rk(emix_ctx *c, int s) {
    int k = 0;
    for (const Launch &L : c->plan)
        if (L.kind == LK_RK && !L.rk.faces && ++k == s) return &L;
    return nullptr;
}

const Launch *plan_weno(emix_ctx *c, int s) {
    int k = 0;
    for (const Launch &L : c->plan)
        if (L.kind == LK_WENO && ++k == s) return &L;
    return nullptr;
}

// D^T along y or z of nf fields with rows by TMA: while the context's
// pencil_tma is on and the pass has fewer pencils than about one resident
// wave of the device (1024 per SM): there the one-thread-per-pencil loads
// leave too few warps to hide their latency and the staged rows win; at
// larger sizes the loads are as fast and the ring's waits cost more.
bool tma_rows(const emix_adj *a, int ax, int nf) {
    const emix_params &p = a->c->p;
    const long np = (long)p.nx * (ax == 1 ? p.nz : p.ny);
    return a->c->pencil_tma && np * nf < 1024L * device_sms();
}

// adjoint of the taped step: in a->LA (um0 of the next step) and a->Lphi
// (phi of the next step); out a->Lum0 and a->Lphi_prev (this step's start)
int step_adjoint(emix_adj *a) {
    emix_ctx *c = a->c;
    const emix_params &p = c->p;
    const long n = c->n, ng = c->ng;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    cudaStream_t st = c->stream;
    int rc;
    if ((rc = zero(a->Lum0, 5 * n, st)) || (rc = zero(a->Lphig0, ng, st)) ||
        (rc = zero(a->LphiA, ng, st)) || (rc = zero(a->LphiB, ng, st)))
        return rc;
    // With the context's second stream (a->overlap) the level-set stages'
    // adjoints run there, concurrently with the flow's: they chain only
    // through the phi adjoints and the tape, and stage s's velocity adjoint
    // goes to LuW, added to the substep's LuIn on the compute stream once both
    // are done (the next stage waits for that add before reusing LuW).
    const bool two = a->overlap && c->side && a->ev_wfork;
    cudaStream_t sw = two ? c->side : st;
    if (two) {
        EMIX_CUDA_TRY(cudaEventRecord(a->ev_wfork, st));
        EMIX_CUDA_TRY(cudaStreamWaitEvent(sw, a->ev_wfork, 0));
    }
    double *Lo = a->LA, *Lnext = a->LB;          // adjoint of the substep's um output / input
    double *LuOut = nullptr, *LpOut = nullptr;   // adjoint of its u / pres outputs
    double *LuIn = a->LU0, *LpIn = a->LP0;
    const Tape &T = *a->tape;
    for (int s = 3; s >= 1; --s) {
        const Launch *Lrk = plan_rk(c, s), *Lw = plan_weno(c, s);
        if (!Lrk || !Lw) return EMIX_ERR_ARG;
        const double *umc = s == 1 ? T.um0 : T.umc[s - 1];
        // level-set stage s's adjoint: on sw before the flow's (two streams),
        // else after it on the compute stream, where the flux adjoint has
        // stored LuIn and the gradients' D^T have accumulated into it
        auto level_set_stage = [&]() -> int {
            if (two && s < 3) EMIX_CUDA_TRY(cudaStreamWaitEvent(sw, a->ev_wfree, 0));
            int r;
            if ((r = zero(a->LD, 3 * ng, sw))) return r;
            if (two && (r = zero(a->LuW, 3 * n, sw))) return r;
            const WenoArgs &wa = Lw->weno;
            WenoAdjArgs G{};
            G.phi = T.phig[s - 1] ? T.phig[s - 1] : wa.phi;
            G.lout = s == 3 ? a->Lphi : (s == 2 ? a->LphiB : a->LphiA);
            G.lphi0 = a->Lphig0;
            G.lphiin = s == 1 ? a->Lphig0 : (s == 2 ? a->LphiA : a->LphiB);
            G.lD = a->LD; G.lu = two ? a->LuW : LuIn; G.vel = T.u[s - 1]; G.wce = wa.wce;
            G.nxg = wa.nxg; G.nyg = wa.nyg; G.nzg = wa.nzg; G.g = wa.g;
            for (int d = 0; d < 3; ++d) { G.r0[d] = wa.r0[d]; G.rn[d] = wa.rn[d]; }
            G.dt = wa.dt; G.stage = s;
            k_adj_weno<<<grid_n((long)wa.rn[0] * wa.rn[1] * wa.rn[2]), 256, 0, sw>>>(G);
            k_adj_weno_dphi<<<grid_n(ng), 256, 0, sw>>>(a->LD, G.lphiin, wa.nxg, wa.nyg, wa.nzg);
            EMIX_CUDA_TRY(cudaGetLastError());
            if (two) EMIX_CUDA_TRY(cudaEventRecord(a->ev_wdone, sw));
            return EMIX_OK;
        };
        if (two && (rc = level_set_stage())) return rc;
        // RK update
        RkAdjArgs A{};
        A.a = Lrk->rk;
        A.a.R = T.R[s - 1];
        A.a.um0 = T.um0;
        A.a.um = umc;
        A.lo = Lo; A.lu = LuOut; A.lp = LpOut; A.T5 = a->T5; A.red = a->red;
        k_adj_rk_a<<<grid_n(n), 256, 0, st>>>(A);
        if (p.bc_walls) k_adj_rk_b<<<grid_n(rk_face_count(nx, ny, nz)), 256, 0, st>>>(A);
        RkCombAdjArgs C{};
        C.T5 = a->T5; C.jbn = c->jbn; C.lum0 = a->Lum0; C.lR = a->LR; C.n = n;
        C.lumc = s >= 2 ? Lnext : nullptr;
        C.ca = s == 1 ? 1.0 : (s == 2 ? 0.75 : 1.0 / 3.0);
        C.cb = s == 1 ? 0.0 : (s == 2 ? 0.25 : 2.0 / 3.0);
        C.cr = (s == 1 ? 1.0 : (s == 2 ? 0.25 : 2.0 / 3.0)) * p.dt;
        k_adj_rk_c<<<grid_n(n), 256, 0, st>>>(C);
        // divergence: LF[3m + ax] = D_ax^T LR[m]
        for (int ax = 0; ax < 3; ++ax) {
            const double *in[5];
            double *w[5], *out[5];
            for (int m = 0; m < 5; ++m) {
                in[m] = a->LR + m * n;
                w[m] = a->W + m * n;
                out[m] = a->LF + (3 * m + ax) * n;
            }
            const PencilMaps *pm = ax && tma_rows(a, ax, 5) && a->tdiv_ok[ax - 1] ? &a->tdiv[ax - 1] : nullptr;
            if ((rc = launch_deriv_t(a->TT[ax], ax, 0, 5, in, w, out, nx, ny, nz, st, pm))) return rc;
        }
        // fluxes
        FluxAdjArgs F{};
        F.lF = a->LF; F.umc = umc; F.u = T.u[s - 1]; F.vis = T.vis[s - 1];
        F.dvel = T.dvel[s - 1]; F.jbn = c->jbn; F.jx = c->jx; F.jy = c->jy; F.jz = c->jz;
        F.lumc = s >= 2 ? Lnext : a->Lum0;
        F.lu = LuIn; F.lp = LpIn; F.ldvel = a->Ldvel; F.lvis = a->Lvis; F.n = n;
        k_adj_flux<<<grid_n(n), 256, 0, st>>>(F);
        // Smagorinsky
        SmagAdjArgs S{};
        S.dvel = T.dvel[s - 1]; S.jbn = c->jbn; S.dxyz = c->dxyz; S.lvis = a->Lvis;
        S.cs = p.sgs_model == EMIX_SGS_NONE ? 0.0 : p.cs; S.ldvel = a->Ldvel; S.red = a->red; S.n = n;
        k_adj_smag<<<grid_n(n), 256, 0, st>>>(S);
        // velocity gradients: LuIn[c] += D_ax^T Ldvel[3 ax + c]
        for (int ax = 0; ax < 3; ++ax) {
            const double *in[3];
            double *w[3], *out[3];
            for (int q = 0; q < 3; ++q) {
                in[q] = a->Ldvel + (3 * ax + q) * n;
                w[q] = a->W + q * n;
                out[q] = LuIn + q * n;
            }
            const int v = LuIn == a->LU0 ? 0 : 1;
            const PencilMaps *pm =
                ax && tma_rows(a, ax, 3) && a->tgrad_ok[ax - 1][v] ? &a->tgrad[ax - 1][v] : nullptr;
            if ((rc = launch_deriv_t(a->TT[ax], ax, 1, 3, in, w, out, nx, ny, nz, st, pm))) return rc;
        }
        if (!two && (rc = level_set_stage())) return rc;
        if (two) {
            // the level-set stage's adjoint has run beside this substep's
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, a->ev_wdone, 0));
            k_add_into<<<grid_n(3 * n), 256, 0, st>>>(LuIn, a->LuW, 3 * n);
            EMIX_CUDA_TRY(cudaGetLastError());
            EMIX_CUDA_TRY(cudaEventRecord(a->ev_wfree, st));
        }
        // hand over to substep s-1
        LuOut = LuIn; LpOut = LpIn;
        LuIn = LuIn == a->LU0 ? a->LU1 : a->LU0;
        LpIn = LpIn == a->LP0 ? a->LP1 : a->LP0;
        double *t = Lo; Lo = Lnext; Lnext = t;
    }
    // primitive variables of substep 1 (u, pres from um0); LuOut holds their adjoint
    k_adj_prim<<<grid_n(n), 256, 0, st>>>(T.um0, LuOut, LpOut, 1.0 / (p.mach * p.mach), a->Lum0, n);
    if ((rc = zero(a->Lphi_prev, n, st))) return rc;
    k_adj_unpad<<<grid_n(n), 256, 0, st>>>(a->Lphig0, a->Lphi_prev, p.ls_ghost, nx, ny, nz);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}

int objective(emix_adj *a, bool adjoint, double *J) {
    emix_ctx *c = a->c;
    const emix_params &p = c->p;
    const long n = c->n;
    cudaStream_t st = c->stream;
    int rc;
    ObjArgs O{};
    O.um = c->um0; O.phi = c->phi; O.xyz = c->xyz; O.jbn = c->jbn;
    for (int d = 0; d < 3; ++d) O.h[d] = p.h[d];
    O.r_in = a->obj.r_in; O.r_out = a->obj.r_out; O.eps = a->obj.eps;
    O.w_ke = a->obj.w_ke; O.w_if = a->obj.w_if;
    O.nx = p.nx; O.ny = p.ny; O.nz = p.nz; O.red = a->red + 8;
    if (adjoint) {
        O.lum = a->LA;
        O.lphi = a->Lphi;
        if ((rc = zero(a->Lphi, n, st))) return rc;
    }
    const int nb = grid_n(n);
    k_objective<<<nb, 256, 0, st>>>(O);
    k_sum_partials<<<1, 1024, 0, st>>>(a->red + 8, nb, a->red + 2);
    EMIX_CUDA_TRY(cudaGetLastError());
    EMIX_CUDA_TRY(cudaMemcpyAsync(J, a->red + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    return EMIX_OK;
}

} // namespace
} // namespace emix

using namespace emix;

namespace {

double *take(double *&q, long cnt) {
    double *r = q;
    q += cnt;
    return r;
}

void destroy_events(emix_adj *a) {
    for (cudaEvent_t *e : {&a->ev_fork, &a->ev_a, &a->ev_b, &a->ev_wfork, &a->ev_wdone, &a->ev_wfree}) {
        if (*e) cudaEventDestroy(*e);
        *e = nullptr;
    }
}

// forward steps of one segment: from state `from` (clock clk), storing the
// state before each step into `store` (when not null)
int run_steps(emix_adj *a, int nsteps, double *store, double *store_clk, int first) {
    emix_ctx *c = a->c;
    const long n = c->n;
    for (int k = 0; k < nsteps; ++k) {
        if (store) {
            int rc = save_state(a, store + (long)(first + k) * 6 * n, store_clk + 2 * (first + k));
            if (rc) return rc;
        }
        int rc = emix_step(c, 1, 1);
        if (rc) return rc;
    }
    return EMIX_OK;
}

} // namespace

extern "C" {

int emix_adj_create(emix_ctx *c, int nsteps, int every, const emix_objective *obj, emix_adj **out) {
    if (!c || !out || !obj || nsteps < 1 || every < 0 || every > nsteps) return EMIX_ERR_ARG;
    *out = nullptr;
    const emix_params &p = c->p;
    if (!c->static_set || !p.level_set || p.sgs_model == EMIX_SGS_STRUCTURE || !p.imp.on ||
        p.imp.interp || p.filter_every != 0 || p.ref_bugs != 0) {
        set_last_message("emix_adj_create: the adjoint covers the tank step (level set on, "
                         "Smagorinsky or no SGS, impeller on without the blade-edge "
                         "interpolation, no filter, ref_bugs 0)");
        return EMIX_ERR_ARG;
    }
    emix_adj *a = new (std::nothrow) emix_adj();
    if (!a) return EMIX_ERR_ALLOC;
    a->c = c;
    a->nsteps = nsteps;
    a->keep = every == 0;
    a->every = a->keep ? 1 : every;
    a->obj = *obj;
    const int dims[3] = {p.nx, p.ny, p.nz};
    for (int d = 0; d < 3; ++d) {
        int rc = get_deriv_t_table(p.scheme[d], dims[d], p.h[d], &a->TT[d]);
        if (rc) { delete a; return rc; }
    }
    const long n = c->n, ng = c->ng;
    const bool keep = a->keep;
    const int ncp = keep ? 0 : (nsteps + every - 1) / every;
    const int nseg = keep ? 0 : every;
    const int ntape = keep ? nsteps : 1;
    const long tape_cnt = 5 * n + 3 * (3 + 1 + 9 + 1 + 5) * n + 2 * 5 * n      // 72 fields
                          + (keep ? 3 * ng + kImpClockLen : 0);
    const long cnt = (long)ncp * 6 * n + (long)nseg * 6 * n + 6 * n        // checkpoints, segment, final
                     + (long)ntape * tape_cnt + (keep ? kImpClockLen : 0)  // tapes, final clock
                     + 5 * n * 3 + 3 * n * 2 + n * 2 + 5 * n + 15 * n + 9 * n + n + 5 * n + 6 * n
                     + 2 * n + 3 * ng + 3 * ng + 3 * n + 8 + 2048
                     + 2 * (long)ncp + 2 * (long)nseg + 2;                 // checkpoint clocks
    a->bytes = (size_t)cnt * sizeof(double);
    if (cudaMalloc(&a->arena, a->bytes) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("cudaMalloc of the adjoint arena failed");
        delete a;
        return EMIX_ERR_ALLOC;
    }
    double *q = a->arena;
    a->cp = take(q, (long)ncp * 6 * n);
    a->seg = take(q, (long)nseg * 6 * n);
    a->final_state = take(q, 6 * n);
    a->tapes.resize(ntape);
    for (Tape &T : a->tapes) {
        T.um0 = take(q, 5 * n);
        for (int s = 0; s < 3; ++s) {
            T.u[s] = take(q, 3 * n);
            T.p[s] = take(q, n);
            T.dvel[s] = take(q, 9 * n);
            T.vis[s] = take(q, n);
            T.R[s] = take(q, 5 * n);
            T.umc[s] = s >= 1 ? take(q, 5 * n) : nullptr;
        }
        if (keep) {
            for (int s = 0; s < 3; ++s) T.phig[s] = take(q, ng);
            T.clock = take(q, kImpClockLen);
        }
    }
    a->tape = &a->tapes[0];
    a->final_clock_full = keep ? take(q, kImpClockLen) : nullptr;
    a->Lum0 = take(q, 5 * n); a->LA = take(q, 5 * n); a->LB = take(q, 5 * n);
    a->LU0 = take(q, 3 * n); a->LU1 = take(q, 3 * n);
    a->LP0 = take(q, n); a->LP1 = take(q, n);
    a->LR = take(q, 5 * n); a->LF = take(q, 15 * n); a->Ldvel = take(q, 9 * n); a->Lvis = take(q, n);
    a->T5 = take(q, 5 * n); a->W = take(q, 6 * n);
    a->Lphi = take(q, n); a->Lphi_prev = take(q, n);
    a->Lphig0 = take(q, ng); a->LphiA = take(q, ng); a->LphiB = take(q, ng);
    a->LD = take(q, 3 * ng);
    a->LuW = take(q, 3 * n);
    a->red = take(q, 8 + 2048);   // [0] dJ/domega, [1] dJ/dCs, [2] J, then J's block partials
    a->cp_clock = take(q, 2 * (long)ncp);
    a->seg_clock = take(q, 2 * (long)nseg);
    a->final_clock = take(q, 2);
    for (int ax = 1; ax <= 2; ++ax) {
        const int axes[5] = {ax, ax, ax, ax, ax};
        if (a->TT[ax].periodic) continue;
        const double *in[5];
        double *w[5], *o[5];
        for (int m = 0; m < 5; ++m) {
            in[m] = a->LR + m * n;
            w[m] = a->W + m * n;
            o[m] = a->LF + (3 * m + ax) * n;
        }
        a->tdiv_ok[ax - 1] = pencil_tma_maps(&a->tdiv[ax - 1], axes, 5, in, w, o, p.nx, p.ny, p.nz);
        for (int v = 0; v < 2; ++v) {
            double *lu = v == 0 ? a->LU0 : a->LU1;
            for (int q = 0; q < 3; ++q) {
                in[q] = a->Ldvel + (3 * ax + q) * n;
                w[q] = a->W + q * n;
                o[q] = lu + q * n;
            }
            a->tgrad_ok[ax - 1][v] = pencil_tma_maps(&a->tgrad[ax - 1][v], axes, 3, in, w, o, p.nx, p.ny, p.nz);
        }
    }
    if (c->side &&
        (cudaEventCreateWithFlags(&a->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&a->ev_a, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&a->ev_b, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&a->ev_wfork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&a->ev_wdone, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&a->ev_wfree, cudaEventDisableTiming) != cudaSuccess)) {
        // without the events both passes run on the compute stream alone
        cudaGetLastError();
        destroy_events(a);
    }
    *out = a;
    return EMIX_OK;
}

int emix_adj_destroy(emix_adj *a) {
    if (!a) return EMIX_ERR_ARG;
    cudaStreamSynchronize(a->c->stream);
    destroy_events(a);
    cudaFree(a->arena);
    delete a;
    return EMIX_OK;
}

int emix_adj_set_overlap(emix_adj *a, int on) {
    if (!a || on < 0 || on > 1) return EMIX_ERR_ARG;
    a->overlap = on;
    return EMIX_OK;
}

int emix_adj_device_bytes(emix_adj *a, size_t *bytes) {
    if (!a || !bytes) return EMIX_ERR_ARG;
    *bytes = a->bytes;
    return EMIX_OK;
}

int emix_adj_forward(emix_adj *a, double *J) {
    if (!a || !J) return EMIX_ERR_ARG;
    int rc;
    if (a->keep) {
        // every step taped as it runs: the reverse sweep recomputes nothing
        emix_ctx *c = a->c;
        for (int k = 0; k < a->nsteps; ++k) {
            a->tape = &a->tapes[k];
            if ((rc = taped_step(a))) return rc;
            ++c->step_index;   // as emix_step counts its steps
        }
        if ((rc = copy(a->final_clock_full, c->clock, kImpClockLen, c->stream))) return rc;
        if ((rc = save_state(a, a->final_state, a->final_clock))) return rc;
        if ((rc = objective(a, false, J))) return rc;
        a->J = *J;
        return EMIX_OK;
    }
    // checkpoints every `every` steps from the context's current state
    for (int k = 0; k < a->nsteps; k += a->every) {
        const int cpi = k / a->every;
        if ((rc = save_state(a, a->cp + (long)cpi * 6 * a->c->n, a->cp_clock + 2 * cpi))) return rc;
        const int m = k + a->every <= a->nsteps ? a->every : a->nsteps - k;
        if ((rc = run_steps(a, m, nullptr, nullptr, 0))) return rc;
    }
    if ((rc = save_state(a, a->final_state, a->final_clock))) return rc;
    if ((rc = objective(a, false, J))) return rc;
    a->J = *J;
    return EMIX_OK;
}

int emix_adj_backward(emix_adj *a, double *dJ) {
    if (!a || !dJ) return EMIX_ERR_ARG;
    emix_ctx *c = a->c;
    const long n = c->n;
    int rc;
    const long step_index = c->step_index;   // the recomputations below advance it
    if ((rc = zero(a->red, 2, c->stream))) return rc;
    // adjoint of J at the final state: a->LA (um0), a->Lphi (phi)
    if ((rc = load_state(a, a->final_state, a->final_clock))) return rc;
    double J;
    if ((rc = objective(a, true, &J))) return rc;
    if (a->keep) {
        // the tapes of the forward pass; each step's impeller clock restored
        for (int k = a->nsteps - 1; k >= 0; --k) {
            a->tape = &a->tapes[k];
            if ((rc = copy(c->clock, a->tapes[k].clock, kImpClockLen, c->stream))) return rc;
            if ((rc = step_adjoint(a))) return rc;
            double *t = a->LA; a->LA = a->Lum0; a->Lum0 = t;
            t = a->Lphi; a->Lphi = a->Lphi_prev; a->Lphi_prev = t;
        }
        if ((rc = copy(c->clock, a->final_clock_full, kImpClockLen, c->stream))) return rc;
    }
    const int ncp = a->keep ? 0 : (a->nsteps + a->every - 1) / a->every;
    for (int cpi = ncp - 1; cpi >= 0; --cpi) {
        const int first = cpi * a->every;
        const int m = first + a->every <= a->nsteps ? a->every : a->nsteps - first;
        // states before each step of the segment
        if ((rc = load_state(a, a->cp + (long)cpi * 6 * n, a->cp_clock + 2 * cpi))) return rc;
        if ((rc = run_steps(a, m - 1, a->seg, a->seg_clock, 0))) return rc;
        if ((rc = save_state(a, a->seg + (long)(m - 1) * 6 * n, a->seg_clock + 2 * (m - 1)))) return rc;
        for (int k = m - 1; k >= 0; --k) {
            if ((rc = load_state(a, a->seg + (long)k * 6 * n, a->seg_clock + 2 * k))) return rc;
            if ((rc = taped_step(a))) return rc;
            if ((rc = step_adjoint(a))) return rc;
            // the step's input adjoint becomes the previous step's output adjoint
            double *t = a->LA; a->LA = a->Lum0; a->Lum0 = t;
            t = a->Lphi; a->Lphi = a->Lphi_prev; a->Lphi_prev = t;
        }
    }
    double h[3];
    EMIX_CUDA_TRY(cudaMemcpyAsync(h, a->red, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    dJ[0] = h[0];
    dJ[1] = h[1];
    // leave the context at the final state of the forward pass
    if ((rc = load_state(a, a->final_state, a->final_clock))) return rc;
    c->step_index = step_index;
    return EMIX_OK;
}

int emix_adj_state_gradient(emix_adj *a, double *lum, double *lphi) {
    // adjoint of the initial state (valid after emix_adj_backward), device pointers
    if (!a || !lum || !lphi) return EMIX_ERR_ARG;
    const long n = a->c->n;
    EMIX_CUDA_TRY(cudaMemcpyAsync(lum, a->LA, 5 * n * sizeof(double), cudaMemcpyDeviceToDevice, a->c->stream));
    EMIX_CUDA_TRY(cudaMemcpyAsync(lphi, a->Lphi, n * sizeof(double), cudaMemcpyDeviceToDevice, a->c->stream));
    EMIX_CUDA_TRY(cudaStreamSynchronize(a->c->stream));
    return EMIX_OK;
}

int emix_ctx_set_forcing(emix_ctx *c, double omega, double cs) {
    if (!c) return EMIX_ERR_ARG;
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->p.imp.omega = omega;
    c->p.cs = cs;
    ctx_rebuild_plan(c);
    return EMIX_OK;
}

} // extern "C"
