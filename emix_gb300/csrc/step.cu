// step.cu -- device-resident RK3 step (solver/rungek_ico.f90:61-313).
//
// A context owns every field of one grid in one device allocation.  A step
// is a fixed sequence of launches on the context stream (optionally replayed
// from a captured CUDA graph):
//
//   prim (u, p from um0) ; pad phi into the ghosted grid
//   for substep s = 1, 2, 3:
//     level-set stage s  (WENO5, SSP-RK3 weights of substep s, velocity u^{s-1})
//     velocity gradients  x, y, z                (cudaDeriv without dT: unused)
//     SGS viscosity       vis = c4 + amut        (viscosidad_t + viscosidad)
//     fluxes              15 fields, 5 equations x 3 directions, inviscid+viscous
//     flux divergence     R_m = d/dxi E_m + d/deta F_m + d/dzeta G_m
//     RK update + conversions (clip, mask, rebuild um1)
//
// The level set is advanced as part of the same SSP-RK3 step (one TVD stage
// per flow substep, each with the velocity the flow stage uses); with a
// frozen velocity this is exactly one cuAdvectLsJB step.
#include "ctx.cuh"

#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace emix {
int launch_deriv(const DerivTable &T, int axis, int epi, int nf, const double *const *in,
                 double *const *w, double *const *out, int nx, int ny, int nz, cudaStream_t st);

__global__ void k_metric_products(const double *__restrict__ jbn, double *__restrict__ jx,
                                  double *__restrict__ jy, double *__restrict__ jz, long n) {
    EMIX_FOR_CELLS(q, n) {
        const double j10 = jbn[9 * n + q];
        jx[q] = j10 * jbn[q];
        jy[q] = j10 * jbn[4 * n + q];
        jz[q] = j10 * jbn[8 * n + q];
    }
}
int launch_single(const Launch &L, cudaStream_t st) {
    switch (L.kind) {
    case LK_PRIM:
        k_prim<<<cells_grid(L.prim.n), 256, 0, st>>>(L.prim);
        break;
    case LK_PAD:
        k_ghost_pad<<<cells_grid(L.pad.qend > 0 ? L.pad.qend - L.pad.qbeg : L.pad.ng), 256, 0, st>>>(L.pad);
        break;
    case LK_WENO:
        return launch_weno_stage(L.weno, st, L.tmap);
    case LK_DERIV_X:
    case LK_DERIV_YZ:
        if (L.pmaps)
            return launch_deriv_yz_tma(L.deriv.T, L.deriv.T, *L.pmaps, L.deriv.epi, L.deriv.nf, L.deriv.nf,
                                       L.deriv.F.in, L.deriv.F.w, L.deriv.F.out, L.deriv.nx, L.deriv.ny,
                                       L.deriv.nz, st);
        return launch_deriv(L.deriv.T, L.deriv.axis, L.deriv.epi, L.deriv.nf, L.deriv.F.in, L.deriv.F.w,
                            L.deriv.F.out, L.deriv.nx, L.deriv.ny, L.deriv.nz, st);
    case LK_SMAG:
        k_sgs_smag<<<cells_grid(L.smag.n), 256, 0, st>>>(L.smag);
        break;
    case LK_SF:
        k_sgs_sf<<<cells_grid(L.sf.n), 256, 0, st>>>(L.sf);
        break;
    case LK_VORT:
        k_vort<<<cells_grid(L.vort.n), 256, 0, st>>>(L.vort);
        break;
    case LK_SELECT:
        k_selective<<<cells_grid(L.sel.n), 256, 0, st>>>(L.sel);
        break;
    case LK_FLUX:
        k_flux_all<<<cells_grid(L.flux.n), 256, 0, st>>>(L.flux);
        break;
    case LK_RK:
        k_rk_post<<<cells_grid(rk_count(L.rk)), 256, 0, st>>>(L.rk);
        break;
    case LK_BC:
        k_bc<<<cells_grid(bc_count(L.bc)), 256, 0, st>>>(L.bc);
        break;
    case LK_CLOCK:
        k_imp_clock<<<1, 32, 0, st>>>(L.clock);
        break;
    case LK_INTERP:
        if (L.interp.phase == 0)
            k_interp_geom<<<cells_grid((long)L.interp.g.nblades * L.interp.nx * L.interp.ny), 256, 0, st>>>(L.interp);
        else if (L.interp.phase == 1)
            k_interp_list<<<L.interp.g.nblades, 1024, 0, st>>>(L.interp);
        else
            k_interp_apply<<<(L.interp.nz + 63) / 64, 64, 0, st>>>(L.interp);
        break;
    default:
        return EMIX_ERR_ARG;
    }
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}
} // namespace emix

using namespace emix;



static const char *kClassNames[] = {
    "prim", "ghost_pad", "weno_stage", "grad_x", "grad_y", "grad_z", "sgs", "flux",
    "div_x", "div_y", "div_z", "rk_post", "filter", "grad_yz", "sgs_flux"};

namespace emix {
const std::vector<Launch> &ctx_plan(emix_ctx *c) { return c->plan; }
int ctx_ready(emix_ctx *c) { return c->static_set ? 1 : 0; }
} // namespace emix

namespace {

struct ProfScope {
    emix_ctx *c;
    int slot;
    ProfScope(emix_ctx *c_, int cls) : c(c_), slot(-1) {
        if (c->prof && c->prof_n < 64) {
            slot = c->prof_n++;
            c->prof_cls[slot] = cls;
            cudaEventRecord(c->prof_ev[2 * slot], c->stream);
        }
    }
    ~ProfScope() {
        if (slot >= 0) cudaEventRecord(c->prof_ev[2 * slot + 1], c->stream);
    }
};

Launch make(int kind, int cls) {
    Launch L;
    std::memset(&L, 0, sizeof L);
    L.kind = kind;
    L.cls = cls;
    return L;
}

Launch deriv_launch(const DerivTable &T, int axis, int epi, int nf, const double *const *in,
                    double *const *w, double *const *out, int nx, int ny, int nz, int cls) {
    Launch L = make(axis == 0 ? LK_DERIV_X : LK_DERIV_YZ, cls);
    L.deriv.T = T;
    for (int f = 0; f < nf; ++f) {
        L.deriv.F.in[f] = in[f];
        L.deriv.F.w[f] = w[f];
        L.deriv.F.out[f] = out[f];
    }
    L.deriv.axis = axis; L.deriv.epi = epi; L.deriv.nf = nf;
    L.deriv.nx = nx; L.deriv.ny = ny; L.deriv.nz = nz;
    return L;
}

// The launches of one RK3 step, in order.
// The cyclic scheme's rows by TMA where a launch carries at least 2^16
// pencils (nx x nother x fields): 128^3 periodic 380.7 -> 398.1 Mcell-RK3-
// steps/s with them, 64^3 (20 K pencils a launch) 234.0 -> 208.9, so the
// small launches keep their loads
bool cyclic_tma_pays(int nx, int nother, int nf) { return (long)nx * nother * nf >= 65536; }

void build_plan(emix_ctx *c) {
    const emix_params &p = c->p;
    const long n = c->n;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const double inv_m2 = 1.0 / (p.mach * p.mach);
    std::vector<Launch> &P = c->plan;
    P.clear();
    const ImpGeom ig{p.imp.on, p.imp.nblades, p.imp.omega, p.imp.theta0, p.imp.r1, p.imp.r2,
                     p.imp.z1, p.imp.z2, p.imp.half_thick, p.imp.hub_r, p.imp.hub_z1, p.imp.hub_z2,
                     p.imp.shaft_r, p.imp.shaft_z0, p.imp.shaft_z1};
    if (ig.on) {
        // blade angles of this step's substeps, then advance the clock
        Launch L = make(LK_CLOCK, CLS_RK);
        L.clock = ImpClockArgs{c->clock, p.dt, ig};
        P.push_back(L);
    }
    {
        Launch L = make(LK_PRIM, CLS_PRIM);
        L.prim = PrimArgs{c->um0, c->u, c->pres, inv_m2, n};
        P.push_back(L);
    }
    if (p.level_set) {
        Launch L = make(LK_PAD, CLS_PAD);
        L.pad = PadArgs{c->phig0, c->phi, p.ls_ghost, 1.0, nx, ny, nz, c->ng};
        P.push_back(L);
    }
    for (int s = 1; s <= 3; ++s) {
        const double *umcur = s == 1 ? c->um0 : c->um;
        if (p.level_set) {
            Launch L = make(LK_WENO, CLS_WENO);
            WenoArgs &a = L.weno;
            const int g = p.ls_ghost;
            a.phi = s == 1 ? c->phig0 : (s == 2 ? c->phigA : c->phigB);
            a.phi0 = c->phig0;
            a.out = s == 1 ? c->phigA : (s == 2 ? c->phigB : c->phi);
            a.out_interior = s == 3 ? 1 : 0;
            a.vel = c->u;
            a.jbn = c->jbn;
            a.reflect = 1;
            a.nxg = nx + 2 * g; a.nyg = ny + 2 * g; a.nzg = nz + 2 * g; a.g = g;
            a.sx = 1.0 / p.h[0]; a.sy = 1.0 / p.h[1]; a.sz = 1.0 / p.h[2];
            a.dt = p.dt; a.stage = s; a.ref_bugs = p.ref_bugs;
            a.wce = c->wenoCE;
            // stage 3 writes only the interior, so stage 2 is needed only within
            // the 3-cell reach of the WENO5 stencil around it, and stage 3 only on
            // the interior (stage 1 covers the whole padded grid)
            const int dims[3] = {nx, ny, nz};
            const int gd[3] = {a.nxg, a.nyg, a.nzg};
            for (int d = 0; d < 3; ++d) {
                a.r0[d] = 0; a.rn[d] = gd[d];
                if (s == 2) { a.r0[d] = g - 3; a.rn[d] = dims[d] + 6; }
                if (s == 3) { a.r0[d] = g; a.rn[d] = dims[d]; }
            }
            if (c->tma && weno_tma_map(&c->weno_tmap[s - 1], a)) L.tmap = &c->weno_tmap[s - 1];
            P.push_back(L);
        }
        // velocity gradients (cudaDeriv; dT/dx_i feeds nothing on this path:
        // the m=5 viscous fluxes are zero, flujos_compact.f90:187-214)
        // (the y and z records run as one launch in a single-grid step)
        for (int ax = 0; ax < 3; ++ax) {
            const double *in[3] = {c->u, c->u + n, c->u + 2 * n};
            double *out[3] = {c->dvel + 3 * ax * n, c->dvel + (3 * ax + 1) * n, c->dvel + (3 * ax + 2) * n};
            P.push_back(deriv_launch(c->T[ax], ax, EPI_STORE, 3, in, out, out, nx, ny, nz, CLS_GRADX + ax));
            if (ax == 1) P.back().deriv.pair = 1;
        }
        {
            // the y and z records as one launch with its rows by TMA, where
            // the copy unit's rules hold (both tables closed or both cyclic)
            const double *in[6] = {c->u, c->u + n, c->u + 2 * n, c->u, c->u + n, c->u + 2 * n};
            double *out[6] = {c->dvel + 3 * n, c->dvel + 4 * n, c->dvel + 5 * n,
                              c->dvel + 6 * n, c->dvel + 7 * n, c->dvel + 8 * n};
            const int axes[6] = {1, 1, 1, 2, 2, 2};
            PencilMaps *pm = &c->pmaps[6 + (s - 1)];
            if (c->pencil_tma && c->T[1].periodic == c->T[2].periodic &&
                (!c->T[1].periodic || cyclic_tma_pays(nx, std::max(ny, nz), 6)) &&
                pencil_tma_maps(pm, axes, 6, in, out, out, nx, ny, nz))
                P[P.size() - 2].pair_pmaps = pm;
        }
        // SGS viscosity
        if (p.sgs_model == EMIX_SGS_STRUCTURE) {
            const double cutoff = cos(20.0 * atan(1.0) / 45.0);
            Launch a = make(LK_SF, CLS_SGS), b = make(LK_VORT, CLS_SGS), d = make(LK_SELECT, CLS_SGS);
            a.sf = SfArgs{c->u, c->ratios, c->dxyz, p.amu0, c->amut, nx, ny, nz, n};
            b.vort = VortArgs{c->dvel, c->jbn, c->vort, n};
            d.sel = SelArgs{c->vort, c->amut, c->vis, cutoff, p.c4, nx, ny, nz, n};
            P.push_back(a);
            P.push_back(b);
            P.push_back(d);
        } else {
            Launch L = make(LK_SMAG, CLS_SGS);
            L.smag = SmagArgs{c->dvel, c->jbn, c->dxyz, p.sgs_model == EMIX_SGS_NONE ? 0.0 : p.cs, p.c4,
                              nullptr, c->vis, n};
            P.push_back(L);
        }
        // fluxes
        {
            Launch L = make(LK_FLUX, CLS_FLUX);
            FluxArgs &fa = L.flux;
            for (int q = 0; q < 15; ++q) fa.F[q] = c->flux + q * n;
            fa.um = umcur; fa.u = c->u; fa.pres = c->pres; fa.dvel = c->dvel; fa.vis = c->vis;
            fa.jbn = c->jbn; fa.jx = c->jx; fa.jy = c->jy; fa.jz = c->jz; fa.n = n;
            P.push_back(L);
        }
        // divergence: R_m = sum over directions of the compact derivative
        for (int ax = 0; ax < 3; ++ax) {
            const double *in[5];
            double *out[5], *wb[5];
            for (int m = 0; m < 5; ++m) {
                in[m] = c->flux + (3 * m + ax) * n;
                out[m] = c->R + m * n;
                wb[m] = c->W + m * n;
            }
            if (ax == 0) {
                P.push_back(deriv_launch(c->T[ax], ax, EPI_STORE, 5, in, out, out, nx, ny, nz, CLS_DIVX));
            } else {
                P.push_back(deriv_launch(c->T[ax], ax, EPI_ACCUM, 5, in, wb, out, nx, ny, nz, CLS_DIVX + ax));
                // rows by TMA where the copy unit's rules hold
                PencilMaps *pm = &c->pmaps[2 * (s - 1) + (ax - 1)];
                const int axes[5] = {ax, ax, ax, ax, ax};
                if (c->pencil_tma && (!c->T[ax].periodic || cyclic_tma_pays(nx, ax == 1 ? nz : ny, 5)) &&
                    pencil_tma_maps(pm, axes, 5, in, wb, out, nx, ny, nz))
                    P.back().pmaps = pm;
            }
        }
        // RK update and conversions; with walls the boundary conditions go
        // between the RK combination and the conversions (rungek_ico.f90:98-104):
        // the wall cells first, in a launch of their own that recomputes the
        // RK values the wall rules copy, then every other cell
        {
            Launch L = make(LK_RK, CLS_RK);
            RkArgs &ra = L.rk;
            ra.R = c->R; ra.um0 = c->um0; ra.um = c->um;
            ra.out = s == 3 ? c->um0 : c->um;
            ra.u = c->u; ra.pres = c->pres; ra.jbn = c->jbn; ra.mask = c->mask;
            ra.dt = p.dt; ra.mach = p.mach; ra.inv_m2 = inv_m2; ra.stage = s; ra.n = n;
            ra.nx = nx; ra.ny = ny; ra.nz = nz;
            ra.walls = p.bc_walls;
            ra.faces = 0;
            ra.imp = ig;
            ra.xyz = c->xyz;
            ra.clock = c->clock;
            ra.impflag = c->impflag;
            if (p.bc_walls) {
                Launch F = L;
                F.rk.faces = 1;
                P.push_back(F);
            }
            P.push_back(L);
            if (ig.on && p.imp.interp) {
                // the blade-edge interpolation of rushton(s) on the substep's output
                Launch I = make(LK_INTERP, CLS_RK);
                ImpInterpArgs &ia = I.interp;
                ia.g = ig; ia.xyz = c->xyz; ia.clock = c->clock; ia.mask = c->mask;
                ia.out = ra.out; ia.u = c->u; ia.nx = nx; ia.ny = ny; ia.nz = nz; ia.n = n;
                ia.rango = c->rango; ia.stage = s;
                ia.status = c->ip_status; ia.face = c->ip_face; ia.geo = c->ip_geo; ia.nb = c->ip_nb;
                ia.list = c->ip_list; ia.count = c->ip_count;
                for (int ph = 0; ph < 3; ++ph) {
                    ia.phase = ph;
                    P.push_back(I);
                }
            }
        }
    }
}

bool filter_due(const emix_ctx *c) {
    return c->p.filter_every > 0 && c->step_index % c->p.filter_every == 0;
}

} // namespace

namespace emix {
// Records k and k+1 of a plan that run as one launch: the gradients' y and z
// records (1), Smagorinsky and the fluxes that read its viscosity (2); 0
// otherwise.  The records stay separate in the plan: the fused kernels run
// the same per-cell functions (the same values bit for bit), and the records
// keep each operator's arguments for the adjoint's reverse sweep.
int plan_fuse_next(const std::vector<Launch> &P, size_t k) {
    if (k + 1 >= P.size()) return 0;
    const Launch &L = P[k], &M = P[k + 1];
    if (L.kind == LK_DERIV_YZ && L.deriv.pair && M.kind == LK_DERIV_YZ && L.deriv.epi == EPI_STORE &&
        M.deriv.epi == EPI_STORE && L.deriv.nf + M.deriv.nf <= kMaxFields)
        return 1;
    if (L.kind == LK_SMAG && M.kind == LK_FLUX && M.flux.vis == L.smag.vis && M.flux.dvel == L.smag.dvel &&
        M.flux.jbn == L.smag.jbn && M.flux.n == L.smag.n)
        return 2;
    return 0;
}

int launch_fused_pair(const std::vector<Launch> &P, size_t k, cudaStream_t st) {
    const Launch &L = P[k];
    if (plan_fuse_next(P, k) == 1) {
        // the gradients' y and z records as one launch
        const DerivArgs &a = L.deriv, &b = P[k + 1].deriv;
        const double *in[kMaxFields];
        double *out[kMaxFields];
        for (int f = 0; f < a.nf; ++f) { in[f] = a.F.in[f]; out[f] = a.F.out[f]; }
        for (int f = 0; f < b.nf; ++f) { in[a.nf + f] = b.F.in[f]; out[a.nf + f] = b.F.out[f]; }
        if (L.pair_pmaps)
            return launch_deriv_yz_tma(a.T, b.T, *L.pair_pmaps, EPI_STORE, a.nf, a.nf + b.nf, in, out, out, a.nx,
                                       a.ny, a.nz, st);
        return launch_deriv_yz_pair(a.T, b.T, a.nf, b.nf, in, out, a.nx, a.ny, a.nz, st);
    }
    const FluxArgs &fa = P[k + 1].flux;
    k_smag_flux<<<cells_grid(fa.n), 256, 0, st>>>(L.smag, fa);
    EMIX_CUDA_TRY(cudaGetLastError());
    return EMIX_OK;
}
} // namespace emix

namespace {

int fused_with_next(const emix_ctx *c, size_t k) { return c->fuse ? plan_fuse_next(c->plan, k) : 0; }

int launch_fused(emix_ctx *c, size_t k, cudaStream_t st) { return launch_fused_pair(c->plan, k, st); }

int issue_step(emix_ctx *c) {
    const bool fork = (c->overlap & 1) && c->side && !c->prof;
    const bool gfork = (c->overlap & 2) && c->side && !c->prof;
    int s = 0, gs = 0;
    bool joined = true, gjoined = true;
    const size_t np = c->plan.size();
    int launches = 0;
    for (size_t k = 0; k < np; ++k) {
        const Launch &L = c->plan[k];
        if (gfork && L.kind == LK_DERIV_X && L.cls == CLS_GRADX && gs < 3) {
            EMIX_CUDA_TRY(cudaEventRecord(c->gfork_ev[gs], c->stream));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(c->side, c->gfork_ev[gs], 0));
            int rc = launch_single(L, c->side);
            if (rc) return rc;
            EMIX_CUDA_TRY(cudaEventRecord(c->gjoin_ev[gs], c->side));
            gjoined = false;
            ++gs;
            ++launches;
            continue;
        }
        if (!gjoined && L.cls != CLS_GRADY && L.cls != CLS_GRADZ) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->gjoin_ev[gs - 1], 0));
            gjoined = true;
        }
        const int fuse = fused_with_next(c, k);
        if (fuse) {
            ProfScope ps(c, fuse == 1 ? CLS_GRADYZ : CLS_SGSFLUX);
            int rc = launch_fused(c, k, c->stream);
            if (rc) return rc;
            ++k;
            ++launches;
            continue;
        }
        if (fork && L.kind == LK_WENO) {
            EMIX_CUDA_TRY(cudaEventRecord(c->fork_ev[s], c->stream));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(c->side, c->fork_ev[s], 0));
            int rc = launch_single(L, c->side);
            if (rc) return rc;
            EMIX_CUDA_TRY(cudaEventRecord(c->join_ev[s], c->side));
            joined = false;
            ++s;
            ++launches;
            continue;
        }
        if (fork && !joined && L.kind == LK_RK) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join_ev[s - 1], 0));
            joined = true;
        }
        ProfScope ps(c, L.cls);
        int rc = launch_single(L, c->stream);
        if (rc) return rc;
        ++launches;
    }
    if (fork && !joined) EMIX_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join_ev[s - 1], 0));
    if (!gjoined) EMIX_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->gjoin_ev[gs - 1], 0));
    c->launches = launches;
    return EMIX_OK;
}

bool params_ok(const emix_params *p) {
    if (!p) return false;
    if (p->nx < 6 || p->ny < 6 || p->nz < 6 || p->nx > kTableMaxN || p->ny > kTableMaxN ||
        p->nz > kTableMaxN || p->ny > 65535 || p->nz > 65535)
        return false;
    for (int a = 0; a < 3; ++a) {
        if (p->scheme[a] < EMIX_SCHEME_A || p->scheme[a] > EMIX_SCHEME_C) return false;
        if (!(p->h[a] > 0.0)) return false;
    }
    if (p->sgs_model < EMIX_SGS_NONE || p->sgs_model > EMIX_SGS_STRUCTURE) return false;
    if (p->bc_walls != 0 && p->bc_walls != 1) return false;
    if (p->filter_every < 0 || (p->filter_every > 0 && (p->nx < 11 || p->ny < 11 || p->nz < 11)))
        return false;
    if (p->imp.on && p->imp.interp != 0 && p->imp.interp != 1) return false;
    if ((p->imp.on != 0 && p->imp.on != 1) ||
        (p->imp.on && (p->imp.nblades < 0 || p->imp.nblades > kImpMaxBlades)))
        return false;
    if (!(p->mach > 0.0) || !(p->dt > 0.0)) return false;
    if (p->level_set && (p->ls_ghost < 3 || p->ls_ghost > p->nx || p->ls_ghost > p->ny ||
                         p->ls_ghost > p->nz))
        return false;
    return true;
}

void drop_graph(emix_ctx *c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    if (c->fgexec) cudaGraphExecDestroy(c->fgexec);
    if (c->fgraph) cudaGraphDestroy(c->fgraph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->fgexec = nullptr;
    c->fgraph = nullptr;
}

int issue_filter(emix_ctx *c) {
    return launch_filtrado(c->um0, c->jbn, c->p.cfilt, c->p.nx, c->p.ny, c->p.nz, c->stream);
}

// capture `issue` on the context stream into an executable graph
template <class F>
int capture(emix_ctx *c, F issue, cudaGraph_t *g, cudaGraphExec_t *ge) {
    EMIX_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = issue();
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
    if (e != cudaSuccess) { set_last_error(e, "cudaStreamEndCapture", __FILE__, __LINE__); return EMIX_ERR_CUDA; }
    e = cudaGraphInstantiate(ge, gr, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(gr);
        set_last_error(e, "cudaGraphInstantiate", __FILE__, __LINE__);
        return EMIX_ERR_CUDA;
    }
    *g = gr;
    return EMIX_OK;
}

// Plan positions of the records the host-buffer step issues in its own way.
struct HostPlan {
    long prim = -1, pad = -1, weno[4] = {-1, -1, -1, -1}, rkf3 = -1, rk3 = -1;
};

bool find_host_plan(const emix_ctx *c, HostPlan &h) {
    const std::vector<Launch> &P = c->plan;
    const long np = (long)P.size();
    for (long k = 0; k < np; ++k) {
        const Launch &L = P[k];
        if (L.kind == LK_PRIM) h.prim = k;
        else if (L.kind == LK_PAD) h.pad = k;
        else if (L.kind == LK_WENO && L.weno.stage >= 1 && L.weno.stage <= 3) h.weno[L.weno.stage] = k;
        else if (L.kind == LK_RK && L.rk.stage == 3) (L.rk.faces ? h.rkf3 : h.rk3) = k;
    }
    // the padding and the first level-set stage directly after the primitive
    // variables, the last RK update last
    return h.prim >= 0 && h.pad == h.prim + 1 && h.weno[1] == h.pad + 1 && h.weno[3] >= 0 && h.rk3 == np - 1;
}

// The host-buffer step's overlapped form applies: a level-set context with
// its second stream free, the plan of this library's single-grid step, no
// blade-edge interpolation after the RK update, planes deep enough for the
// upload slabs (the ghost planes mirror within ls_ghost planes of a face).
bool host_pipeline_ok(const emix_ctx *c) {
    HostPlan h;
    return c->p.level_set && c->side && !(c->p.imp.on && c->p.imp.interp) &&
           c->p.nz / c->p.ls_ghost >= 1 && find_host_plan(c, h);
}

// One step of emix_step_host, issued directly (not from the graph), with its
// host copies on the side stream overlapped with it.
//   um_in, phi_in (uploads): phi first, then um by z-slabs; as each slab
//     lands, the primitive variables of its cells and the first level-set
//     stage on the padded planes whose velocity it holds run on it (the
//     stage fills the GPU even on a slab; pencil launches would not).
//   um_out, phi_out (copies back): the last level-set stage moves after the
//     last RK update (it reads the velocity of the substep before, copied
//     aside first, since the update overwrites it); the update runs by
//     z-slabs, each slab of um copied back while the rest of the step runs,
//     then the stage by z-slabs of the interior, each slab of phi copied back.
// The launches compute exactly what issue_step's do.  A step after which the
// filter is due copies back after the filter instead.
int step_host_one(emix_ctx *c, const double *um_in, const double *phi_in, double *um_out,
                  double *phi_out) {
    HostPlan h;
    if (!find_host_plan(c, h)) return EMIX_ERR_ARG;
    const emix_params &p = c->p;
    const long n = c->n, plane = (long)p.nx * p.ny;
    const int nz = p.nz, g = p.ls_ghost;
    const bool up = um_in != nullptr;
    const bool due = filter_due(c);
    const bool down = um_out != nullptr && !due;
    cudaStream_t st = c->stream, sd = c->side;
    constexpr int SI = emix_ctx::kE2eSlabsIn, S = emix_ctx::kE2eSlabs;
    // events: [0] start, [1] unused, [2, 2+SI) phi and um slabs in, then S
    // um slabs final, then S phi slabs final, then SI slabs padded, then the
    // two slab streams done
    cudaEvent_t *ev = c->e2e_ev, *ev_in = ev + 2, *ev_um = ev + 2 + SI, *ev_phi = ev + 2 + SI + S;
    cudaEvent_t *ev_pad = ev + 2 + SI + 2 * S, *ev_slab = ev_pad + SI;
    auto zcut = [nz](int b, int parts) { return (int)((long)nz * b / parts); };
    const size_t db = sizeof(double);

    // the side stream's copies follow whatever the context stream holds
    EMIX_CUDA_TRY(cudaEventRecord(ev[0], st));
    EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, ev[0], 0));
    // upload slabs (phi, then um) at least ls_ghost planes deep (the ghost
    // planes mirror within ls_ghost planes of a face); the first half as deep
    // as the others, since nothing computes before it lands
    const int su = up ? ((nz / g + 1) / 2 < SI ? (nz / g + 1) / 2 : SI) : 0;
    auto zin = [nz, su](int b) { return b == 0 ? 0 : (int)((long)nz * (2 * b - 1) / (2 * su - 1)); };
    for (int b = 0; b < su; ++b) {
        const long q0 = plane * zin(b), q1 = plane * zin(b + 1);
        EMIX_CUDA_TRY(cudaMemcpyAsync(c->phi + q0, phi_in + q0, (size_t)(q1 - q0) * db, cudaMemcpyHostToDevice, sd));
        for (int m = 0; m < 5; ++m)
            EMIX_CUDA_TRY(cudaMemcpyAsync(c->um0 + m * n + q0, um_in + m * n + q0, (size_t)(q1 - q0) * db,
                                          cudaMemcpyHostToDevice, sd));
        EMIX_CUDA_TRY(cudaEventRecord(ev_in[b], sd));
    }

    int launches = 0;
    const bool fork = (c->overlap & 1) && !c->prof, gfork = (c->overlap & 2) && !c->prof;
    int fs = 0, gs = 0;
    bool joined = true, gjoined = true;
    const long np = (long)c->plan.size();
    for (long k = 0; k < np; ++k) {
        const Launch &L = c->plan[k];
        if (up && (k == h.pad || k == h.weno[1])) continue;   // issued with the slabs
        if (up && k == h.prim) {
            // per slab: the primitive variables, the padded planes that mirror
            // into the slab (with the ghost planes of the end slabs), and the
            // first level-set stage on the previous slab's padded planes,
            // whose WENO5 reach (3 planes) ends within this slab's
            const long pg = (long)(p.nx + 2 * g) * (p.ny + 2 * g);
            auto padded = [&](int b, int &za, int &zb) {
                za = b == 0 ? 0 : g + zin(b);
                zb = b == su - 1 ? nz + 2 * g : g + zin(b + 1);
            };
            // the stage's slabs alternate between two streams, each after
            // the padding of the slab above it (and so after everything the
            // context stream issued before), and join the context stream
            // after the last
            auto stage1 = [&](int b, cudaEvent_t after) -> int {
                Launch Wl = c->plan[h.weno[1]];
                int za, zb;
                padded(b, za, zb);
                Wl.weno.r0[2] = za;
                Wl.weno.rn[2] = zb - za;
                cudaStream_t x = c->slab_st[b & 1];
                EMIX_CUDA_TRY(cudaStreamWaitEvent(x, after, 0));
                return launch_single(Wl, x);
            };
            for (int b = 0; b < su; ++b) {
                EMIX_CUDA_TRY(cudaStreamWaitEvent(st, ev_in[b], 0));
                Launch Pq = L;
                Pq.prim.qbeg = plane * zin(b);
                Pq.prim.qend = plane * zin(b + 1);
                int rc = launch_single(Pq, st);
                Launch Pd = c->plan[h.pad];
                int za, zb;
                padded(b, za, zb);
                Pd.pad.qbeg = pg * za;
                Pd.pad.qend = pg * zb;
                if (!rc) rc = launch_single(Pd, st);
                if (rc) return rc;
                EMIX_CUDA_TRY(cudaEventRecord(ev_pad[b], st));
                if (b >= 1 && (rc = stage1(b - 1, ev_pad[b]))) return rc;
                launches += 2 + (b >= 1);
            }
            if (int rc = stage1(su - 1, ev_pad[su - 1])) return rc;
            ++launches;
            for (int x = 0; x < 2; ++x) {
                EMIX_CUDA_TRY(cudaEventRecord(ev_slab[x], c->slab_st[x]));
                EMIX_CUDA_TRY(cudaStreamWaitEvent(st, ev_slab[x], 0));
            }
            continue;
        }
        if (down && k == h.weno[3]) continue;   // issued after the last RK update
        // the graph-replayed step's concurrency (issue_step) for the records
        // issued here one by one: the x gradients and the level-set stages
        // not sliced with the copies run on the second stream, joined before
        // the records that overwrite what they read
        if (gfork && L.kind == LK_DERIV_X && L.cls == CLS_GRADX && gs < 3) {
            EMIX_CUDA_TRY(cudaEventRecord(c->gfork_ev[gs], st));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, c->gfork_ev[gs], 0));
            if (int rc = launch_single(L, sd)) return rc;
            EMIX_CUDA_TRY(cudaEventRecord(c->gjoin_ev[gs], sd));
            gjoined = false;
            ++gs;
            ++launches;
            continue;
        }
        if (!gjoined && L.cls != CLS_GRADY && L.cls != CLS_GRADZ) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, c->gjoin_ev[gs - 1], 0));
            gjoined = true;
        }
        if (fork && L.kind == LK_WENO && fs < 3) {
            EMIX_CUDA_TRY(cudaEventRecord(c->fork_ev[fs], st));
            EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, c->fork_ev[fs], 0));
            if (int rc = launch_single(L, sd)) return rc;
            EMIX_CUDA_TRY(cudaEventRecord(c->join_ev[fs], sd));
            joined = false;
            ++fs;
            ++launches;
            continue;
        }
        if (!joined && L.kind == LK_RK) {
            EMIX_CUDA_TRY(cudaStreamWaitEvent(st, c->join_ev[fs - 1], 0));
            joined = true;
        }
        if (down && k == (h.rkf3 >= 0 ? h.rkf3 : h.rk3))
            // the velocity the last level-set stage reads, kept in W (free
            // after the last divergence) before the update overwrites it
            EMIX_CUDA_TRY(cudaMemcpyAsync(c->W, c->u, (size_t)3 * n * db, cudaMemcpyDeviceToDevice, st));
        if (down && k == h.rk3) {
            for (int b = 0; b < S; ++b) {
                const long q0 = plane * zcut(b, S), q1 = plane * zcut(b + 1, S);
                if (q1 <= q0) continue;
                RkArgs ra = L.rk;
                ra.qbeg = q0;
                ra.qend = q1;
                k_rk_post<<<cells_grid(q1 - q0), 256, 0, st>>>(ra);
                EMIX_CUDA_TRY(cudaGetLastError());
                ++launches;
                EMIX_CUDA_TRY(cudaEventRecord(ev_um[b], st));
                EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, ev_um[b], 0));
                for (int m = 0; m < 5; ++m)
                    EMIX_CUDA_TRY(cudaMemcpyAsync(um_out + m * n + q0, L.rk.out + m * n + q0,
                                                  (size_t)(q1 - q0) * db, cudaMemcpyDeviceToHost, sd));
            }
            Launch Wl = c->plan[h.weno[3]];
            Wl.weno.vel = c->W;
            for (int b = 0; b < S; ++b) {
                const int z0 = zcut(b, S), z1 = zcut(b + 1, S);
                if (z1 <= z0) continue;
                Wl.weno.r0[2] = g + z0;
                Wl.weno.rn[2] = z1 - z0;
                int rc = launch_single(Wl, st);
                if (rc) return rc;
                ++launches;
                EMIX_CUDA_TRY(cudaEventRecord(ev_phi[b], st));
                EMIX_CUDA_TRY(cudaStreamWaitEvent(sd, ev_phi[b], 0));
                EMIX_CUDA_TRY(cudaMemcpyAsync(phi_out + plane * z0, c->phi + plane * z0,
                                              (size_t)(z1 - z0) * plane * db, cudaMemcpyDeviceToHost, sd));
            }
            continue;
        }
        const int fuse = fused_with_next(c, (size_t)k);
        int rc = fuse ? launch_fused(c, (size_t)k, st) : launch_single(L, st);
        if (rc) return rc;
        k += fuse ? 1 : 0;
        ++launches;
    }
    if (!joined) EMIX_CUDA_TRY(cudaStreamWaitEvent(st, c->join_ev[fs - 1], 0));
    if (!gjoined) EMIX_CUDA_TRY(cudaStreamWaitEvent(st, c->gjoin_ev[gs - 1], 0));
    c->launches = launches;
    if (due) {
        int rc = c->fgexec ? (cudaGraphLaunch(c->fgexec, st) == cudaSuccess ? EMIX_OK : EMIX_ERR_CUDA)
                           : issue_filter(c);
        if (rc) return rc;
    }
    ++c->step_index;
    if (um_out && !down) {
        EMIX_CUDA_TRY(cudaMemcpyAsync(um_out, c->um0, 5 * n * db, cudaMemcpyDeviceToHost, st));
        EMIX_CUDA_TRY(cudaMemcpyAsync(phi_out, c->phi, n * db, cudaMemcpyDeviceToHost, st));
    }
    return EMIX_OK;
}

} // namespace

namespace emix {
void ctx_rebuild_plan(emix_ctx *c) {
    drop_graph(c);
    build_plan(c);
}
int ctx_issue_step(emix_ctx *c) { return issue_step(c); }
} // namespace emix

extern "C" {

int emix_ctx_create(const emix_params *p, emix_ctx **out) {
    if (!out || !params_ok(p)) return EMIX_ERR_ARG;
    *out = nullptr;
    emix_ctx *c = new (std::nothrow) emix_ctx();
    if (!c) return EMIX_ERR_ALLOC;
    c->p = *p;
    EMIX_CUDA_TRY(cudaGetDevice(&c->dev));
    const long n = (long)ncell(p->nx, p->ny, p->nz);
    const int g = p->level_set ? p->ls_ghost : 0;
    const long ng = p->level_set ? (long)(p->nx + 2 * g) * (p->ny + 2 * g) * (p->nz + 2 * g) : 0;
    c->n = n;
    c->ng = ng;
    const int dims[3] = {p->nx, p->ny, p->nz};
    for (int a = 0; a < 3; ++a) {
        int rc = get_deriv_table(p->scheme[a], dims[a], p->h[a], &c->T[a]);
        if (rc) { delete c; return rc; }
    }
    if (p->filter_every > 0) {
        int rc = prepare_filtrado(p->cfilt, p->nx, p->ny, p->nz);
        if (rc) { delete c; return rc; }
    }
    const bool sf = p->sgs_model == EMIX_SGS_STRUCTURE;
    const long nfield = 5 + 5 + 3 + 1 + 9 + 1 + 15 + 5 + 5 + 11 + 3 + 1 + 1 + (p->level_set ? 7 : 0) +
                        (sf ? 1 + 3 + 6 : 0);
    const bool imp = p->imp.on != 0;
    const long nb2 = imp && p->imp.interp ? (long)p->imp.nblades * p->nx * p->ny : 0;
    const size_t ip_words = nb2 ? 11 * nb2 + 2 * ((nb2 + 7) / 8) + nb2 + (nb2 + 1) / 2 + kImpMaxBlades : 0;
    const size_t bytes = ((size_t)(nfield + (imp ? 3 : 0)) * n + 3 * (size_t)ng +
                          (imp ? kImpClockLen + (n + 7) / 8 : 0) + ip_words + 1) * sizeof(double);
    if (cudaMalloc(&c->arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("cudaMalloc of the context arena failed");
        delete c;
        return EMIX_ERR_ALLOC;
    }
    c->arena_bytes = bytes;
    double *q = c->arena;
    auto take = [&](long cnt) { double *r = q; q += cnt; return r; };
    c->um0 = take(5 * n); c->um = take(5 * n); c->u = take(3 * n); c->pres = take(n);
    c->dvel = take(9 * n); c->vis = take(n); c->flux = take(15 * n); c->R = take(5 * n);
    c->W = take(5 * n); c->jbn = take(11 * n); c->jx = take(n); c->jy = take(n); c->jz = take(n);
    c->mask = take(n); c->dxyz = take(n);
    c->phi = p->level_set ? take(n) : nullptr;
    if ((q - c->arena) & 1) ++q;   // 16-byte pairs
    c->wenoCE = p->level_set ? take(6 * n) : nullptr;
    c->amut = sf ? take(n) : nullptr;
    c->vort = sf ? take(3 * n) : nullptr;
    c->ratios = sf ? take(6 * n) : nullptr;
    c->phig0 = p->level_set ? take(ng) : nullptr;
    c->phigA = p->level_set ? take(ng) : nullptr;
    c->phigB = p->level_set ? take(ng) : nullptr;
    c->xyz = imp ? take(3 * n) : nullptr;
    c->clock = imp ? take(kImpClockLen) : nullptr;
    c->impflag = imp ? reinterpret_cast<unsigned char *>(take((n + 7) / 8)) : nullptr;
    if (imp && p->imp.interp) {
        const long nb2 = (long)p->imp.nblades * p->nx * p->ny;
        c->ip_geo = take(11 * nb2);
        c->ip_status = reinterpret_cast<unsigned char *>(take((nb2 + 7) / 8));
        c->ip_face = reinterpret_cast<signed char *>(take((nb2 + 7) / 8));
        c->ip_nb = reinterpret_cast<int *>(take(nb2));
        c->ip_list = reinterpret_cast<int *>(take((nb2 + 1) / 2));
        c->ip_count = reinterpret_cast<int *>(take(kImpMaxBlades));
    }
    if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->arena);
        delete c;
        set_last_message("cudaStreamCreate failed");
        return EMIX_ERR_CUDA;
    }
    c->stream = c->own;
    if (p->level_set) {
        if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            c->side = nullptr;
        }
        for (int k = 0; k < 3 && c->side; ++k)
            if (cudaEventCreateWithFlags(&c->fork_ev[k], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->join_ev[k], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->gfork_ev[k], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->gjoin_ev[k], cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                if (c->side) cudaStreamDestroy(c->side);
                c->side = nullptr;
            }
    }
    // both concurrency modes on where the second stream exists (measured
    // 474.3 -> 479.0 Mcell-RK3-steps/s at 256^3: they fill launch tails)
    c->overlap = c->side ? 3 : 0;
    if (cudaMemsetAsync(c->arena, 0, bytes, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(c->own);
        cudaFree(c->arena);
        delete c;
        set_last_message("clearing the context arena failed");
        return EMIX_ERR_CUDA;
    }
    if (imp) {
        const double head[2] = {p->t0, 0.0};
        if (cudaMemcpy(c->clock, head, sizeof head, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            cudaStreamDestroy(c->own);
            cudaFree(c->arena);
            delete c;
            set_last_message("setting the impeller clock failed");
            return EMIX_ERR_CUDA;
        }
    }
    build_plan(c);
    *out = c;
    return EMIX_OK;
}

int emix_ctx_destroy(emix_ctx *c) {
    if (!c) return EMIX_ERR_ARG;
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    for (cudaEvent_t &e : c->prof_ev)
        if (e) cudaEventDestroy(e);
    if (c->own) cudaStreamDestroy(c->own);
    for (int k = 0; k < 3; ++k) {
        if (c->fork_ev[k]) cudaEventDestroy(c->fork_ev[k]);
        if (c->join_ev[k]) cudaEventDestroy(c->join_ev[k]);
        if (c->gfork_ev[k]) cudaEventDestroy(c->gfork_ev[k]);
        if (c->gjoin_ev[k]) cudaEventDestroy(c->gjoin_ev[k]);
    }
    for (cudaEvent_t e : c->e2e_ev) {
        if (e) cudaEventDestroy(e);
    }
    for (cudaStream_t x : c->slab_st)
        if (x) cudaStreamDestroy(x);
    if (c->side) cudaStreamDestroy(c->side);
    cudaFree(c->arena);
    delete c;
    return EMIX_OK;
}

int emix_ctx_set_tma(emix_ctx *c, int on) {
    if (!c || (on != 0 && on != 1)) return EMIX_ERR_ARG;
    c->tma = on == 1;
    ctx_rebuild_plan(c);
    return EMIX_OK;
}

int emix_ctx_tma_stages(emix_ctx *c) {
    if (!c) return -1;
    int k = 0;
    for (const Launch &L : c->plan) k += (L.kind == LK_WENO && L.tmap) ? 1 : 0;
    return k;
}

int emix_ctx_set_pencil_tma(emix_ctx *c, int on) {
    if (!c || (on != 0 && on != 1)) return EMIX_ERR_ARG;
    c->pencil_tma = on == 1;
    ctx_rebuild_plan(c);
    return EMIX_OK;
}

int emix_ctx_pencil_tma_launches(emix_ctx *c) {
    if (!c) return -1;
    int k = 0;
    const size_t np = c->plan.size();
    for (size_t q = 0; q < np; ++q) {
        const Launch &L = c->plan[q];
        if (L.kind != LK_DERIV_YZ) continue;
        if (L.pmaps) ++k;
        if (L.pair_pmaps && fused_with_next(c, q) == 1) ++k;
    }
    return k;
}

int emix_ctx_set_overlap(emix_ctx *c, int on) {
    if (!c || on < 0 || on > 3) return EMIX_ERR_ARG;
    c->overlap = on;
    drop_graph(c);
    return EMIX_OK;
}

int emix_ctx_set_fusion(emix_ctx *c, int on) {
    if (!c || (on != 0 && on != 1)) return EMIX_ERR_ARG;
    c->fuse = on == 1;
    drop_graph(c);
    return EMIX_OK;
}

int emix_ctx_set_stream(emix_ctx *c, void *stream) {
    if (!c) return EMIX_ERR_ARG;
    c->stream = stream ? (cudaStream_t)stream : c->own;
    drop_graph(c);
    return EMIX_OK;
}

int emix_ctx_set_static(emix_ctx *c, const double *jbn, const double *mask, const double *xyz) {
    if (!c || !jbn || !mask || !xyz) return EMIX_ERR_ARG;
    const long n = c->n;
    const emix_params &p = c->p;
    cudaStream_t st = c->stream;
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->jbn, jbn, 11 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->mask, mask, n * sizeof(double), cudaMemcpyHostToDevice, st));
    // coordinates go through the flux buffer (free at this point)
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->flux, xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    if (c->xyz && p.imp.interp) {
        // grid diagonal of getInterpolData (rush_ruth_me.f90:357-361)
        const int nx = p.nx, ny = p.ny, nz = p.nz;
        const long nxy = (long)nx * ny;
        const double dx = (xyz[nx - 1] - xyz[0]) / (double)(nx - 1);
        const double dy = (xyz[n + (long)nx * (ny - 1)] - xyz[n]) / (double)(ny - 1);
        const double dz = (xyz[2 * n + nxy * (nz - 1)] - xyz[2 * n]) / (double)(nz - 1);
        c->rango = sqrt(dx * dx + dy * dy + dz * dz);
        ctx_rebuild_plan(c);
    }
    if (c->xyz) {
        EMIX_CUDA_TRY(cudaMemcpyAsync(c->xyz, c->flux, 3 * n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        const ImpGeom ig{p.imp.on, p.imp.nblades, p.imp.omega, p.imp.theta0, p.imp.r1, p.imp.r2,
                         p.imp.z1, p.imp.z2, p.imp.half_thick, p.imp.hub_r, p.imp.hub_z1,
                         p.imp.hub_z2, p.imp.shaft_r, p.imp.shaft_z0, p.imp.shaft_z1};
        k_imp_flags<<<cells_grid(n), 256, 0, st>>>(c->xyz, ig, n, c->impflag);
    }
    double *ratios = c->ratios ? c->ratios : c->flux + 3 * n;
    k_sgs_setup<<<cells_grid(n), 256, 0, st>>>(c->flux, c->dxyz, ratios, p.nx, p.ny, p.nz);
    k_metric_products<<<cells_grid(n), 256, 0, st>>>(c->jbn, c->jx, c->jy, c->jz, n);
    if (p.level_set)
        k_weno_scales<<<cells_grid(n), 256, 0, st>>>(c->jbn, c->wenoCE, 1.0 / p.h[0], 1.0 / p.h[1],
                                                     1.0 / p.h[2], n);
    EMIX_CUDA_TRY(cudaGetLastError());
    EMIX_CUDA_TRY(cudaStreamSynchronize(st));
    c->static_set = true;
    return EMIX_OK;
}

int emix_ctx_upload(emix_ctx *c, const double *um, const double *phi) {
    if (!c || !um) return EMIX_ERR_ARG;
    const long n = c->n;
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->um0, um, 5 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (c->p.level_set) {
        if (!phi) return EMIX_ERR_ARG;
        EMIX_CUDA_TRY(cudaMemcpyAsync(c->phi, phi, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return EMIX_OK;
}

int emix_ctx_download(emix_ctx *c, double *um, double *phi) {
    if (!c || !um) return EMIX_ERR_ARG;
    const long n = c->n;
    EMIX_CUDA_TRY(cudaMemcpyAsync(um, c->um0, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (c->p.level_set && phi)
        EMIX_CUDA_TRY(cudaMemcpyAsync(phi, c->phi, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return EMIX_OK;
}

int emix_ctx_state(emix_ctx *c, double **um, double **phi) {
    if (!c) return EMIX_ERR_ARG;
    if (um) *um = c->um0;
    if (phi) *phi = c->phi;
    return EMIX_OK;
}

int emix_step(emix_ctx *c, int nsteps, int use_graph) {
    if (!c || nsteps < 0) return EMIX_ERR_ARG;
    if (!c->static_set) {
        set_last_message("emix_step: static fields not set (emix_ctx_set_static)");
        return EMIX_ERR_ARG;
    }
    if (use_graph && !c->gexec) {
        int rc = capture(c, [&] { return issue_step(c); }, &c->graph, &c->gexec);
        if (rc) { drop_graph(c); return rc; }
    }
    if (use_graph && c->p.filter_every > 0 && !c->fgexec) {
        int rc = capture(c, [&] { return issue_filter(c); }, &c->fgraph, &c->fgexec);
        if (rc) { drop_graph(c); return rc; }
    }
    for (int s = 0; s < nsteps; ++s) {
        if (use_graph) {
            EMIX_CUDA_TRY(cudaGraphLaunch(c->gexec, c->stream));
        } else {
            int rc = issue_step(c);
            if (rc) return rc;
        }
        // filtrado after the step's last substep (rungek_ico.f90:269-278)
        if (filter_due(c)) {
            if (use_graph) {
                EMIX_CUDA_TRY(cudaGraphLaunch(c->fgexec, c->stream));
            } else {
                int rc = issue_filter(c);
                if (rc) return rc;
            }
        }
        ++c->step_index;
    }
    return EMIX_OK;
}

int emix_ctx_get_step_index(emix_ctx *c, long *index) {
    if (!c || !index) return EMIX_ERR_ARG;
    *index = c->step_index;
    return EMIX_OK;
}

int emix_ctx_set_time(emix_ctx *c, double t0) {
    if (!c || !c->clock) return EMIX_ERR_ARG;
    const double head[2] = {t0, 0.0};
    EMIX_CUDA_TRY(cudaMemcpyAsync(c->clock, head, sizeof head, cudaMemcpyHostToDevice, c->stream));
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return EMIX_OK;
}

int emix_ctx_get_time(emix_ctx *c, double *t) {
    if (!c || !t || !c->clock) return EMIX_ERR_ARG;
    double head[2];
    EMIX_CUDA_TRY(cudaMemcpyAsync(head, c->clock, sizeof head, cudaMemcpyDeviceToHost, c->stream));
    EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *t = head[0] + head[1] * c->p.dt;
    return EMIX_OK;
}

int emix_ctx_set_step_index(emix_ctx *c, long index) {
    if (!c || index < 0) return EMIX_ERR_ARG;
    c->step_index = index;
    return EMIX_OK;
}

// emix_step_host without its check of the level-set stage's bounded waits
static int step_host_run(emix_ctx *c, double *um, double *phi, int nsteps) {
    const long n = c->n;
    if (!host_pipeline_ok(c) || nsteps < 1) {
        // plain form: upload, steps, copies back, all on the context stream
        EMIX_CUDA_TRY(cudaMemcpyAsync(c->um0, um, 5 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        if (c->p.level_set)
            EMIX_CUDA_TRY(cudaMemcpyAsync(c->phi, phi, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        int rc = emix_step(c, nsteps, 1);
        if (rc) return rc;
        EMIX_CUDA_TRY(cudaMemcpyAsync(um, c->um0, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (c->p.level_set)
            EMIX_CUDA_TRY(cudaMemcpyAsync(phi, c->phi, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
        return EMIX_OK;
    }
    for (cudaEvent_t &e : c->e2e_ev)
        if (!e) EMIX_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaStream_t &x : c->slab_st)
        if (!x) EMIX_CUDA_TRY(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    // the first step takes the uploads, the last the copies back, the steps
    // between (if any) replay the graph
    int rc;
    if (nsteps == 1) {
        rc = step_host_one(c, um, phi, um, phi);
    } else {
        rc = step_host_one(c, um, phi, nullptr, nullptr);
        if (!rc && nsteps > 2) rc = emix_step(c, nsteps - 2, 1);
        if (!rc) rc = step_host_one(c, nullptr, nullptr, um, phi);
    }
    cudaError_t e1 = cudaStreamSynchronize(c->stream);
    cudaError_t e2 = cudaStreamSynchronize(c->side);
    if (rc) return rc;
    EMIX_CUDA_TRY(e1);
    EMIX_CUDA_TRY(e2);
    return EMIX_OK;
}

int emix_step_host(emix_ctx *c, double *um, double *phi, int nsteps) {
    if (!c || !um || nsteps < 0) return EMIX_ERR_ARG;
    if (c->p.level_set && !phi) return EMIX_ERR_ARG;
    // a block whose bounded TMA waits ran out (a level-set stage block, or a
    // divergence pencil block) leaves its cells unwritten: the timeout
    // counters are read before and after the steps, and a rise is returned as
    // an error
    const bool tma_stages = emix_ctx_tma_stages(c) > 0;
    const bool tma_pencils = emix_ctx_pencil_tma_launches(c) > 0;
    int tmo0 = 0, pto0 = 0;
    if (tma_stages) {
        int rc = emix_weno_tma_timeouts(&tmo0);
        if (rc) return rc;
    }
    if (tma_pencils) {
        int rc = emix_pencil_tma_timeouts(&pto0);
        if (rc) return rc;
    }
    int rc = step_host_run(c, um, phi, nsteps);
    if (rc) return rc;
    if (tma_stages) {
        int tmo1 = 0;
        rc = emix_weno_tma_timeouts(&tmo1);
        if (rc) return rc;
        if (tmo1 != tmo0) {
            set_last_message("emix_step_host: level-set stage blocks gave up waiting for their TMA "
                             "plane copies; phi is incomplete");
            return EMIX_ERR_TIMEOUT;
        }
    }
    if (tma_pencils) {
        int pto1 = 0;
        rc = emix_pencil_tma_timeouts(&pto1);
        if (rc) return rc;
        if (pto1 != pto0) {
            set_last_message("emix_step_host: divergence pencil blocks gave up waiting for their TMA "
                             "row copies; um is incomplete");
            return EMIX_ERR_TIMEOUT;
        }
    }
    return EMIX_OK;
}

int emix_ctx_launches_per_step(emix_ctx *c) {
    if (!c) return -1;
    // every record is one launch, except the pairs that run as one
    int k = 0;
    const size_t np = c->plan.size();
    for (size_t q = 0; q < np; ++q) {
        if (fused_with_next(c, q)) ++q;
        ++k;
    }
    return k;
}

long long emix_ctx_device_bytes(emix_ctx *c) { return c ? (long long)c->arena_bytes : -1; }

const char *emix_profile_class_name(int cls) {
    return (cls >= 0 && cls < CLS_COUNT) ? kClassNames[cls] : "";
}

int emix_profile_class_count(void) { return CLS_COUNT; }

int emix_ctx_profile(emix_ctx *c, int nsteps, double *ms, int *launches) {
    if (!c || nsteps < 1 || !ms || !launches) return EMIX_ERR_ARG;
    if (!c->static_set) return EMIX_ERR_ARG;
    for (int k = 0; k < CLS_COUNT; ++k) { ms[k] = 0.0; launches[k] = 0; }
    for (cudaEvent_t &e : c->prof_ev)
        if (!e) EMIX_CUDA_TRY(cudaEventCreate(&e));
    for (int s = 0; s < nsteps; ++s) {
        c->prof = true;
        c->prof_n = 0;
        int rc = issue_step(c);
        if (!rc && filter_due(c)) {
            ProfScope ps(c, CLS_FILTER);
            rc = issue_filter(c);
        }
        c->prof = false;
        if (rc) return rc;
        ++c->step_index;
        EMIX_CUDA_TRY(cudaStreamSynchronize(c->stream));
        for (int q = 0; q < c->prof_n; ++q) {
            float t = 0.f;
            EMIX_CUDA_TRY(cudaEventElapsedTime(&t, c->prof_ev[2 * q], c->prof_ev[2 * q + 1]));
            ms[c->prof_cls[q]] += t;
            launches[c->prof_cls[q]] += 1;
        }
    }
    return EMIX_OK;
}

} // extern "C"
