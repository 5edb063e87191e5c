// ctx.cuh -- the device-resident context of one grid (emix_ctx), shared by
// the step (step.cu) and its adjoint (adjoint.cu).
#pragma once

#include "plan.cuh"

#include <vector>

struct emix_ctx {
    emix_params p{};
    int dev = 0;
    long n = 0, ng = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own = nullptr;
    double *arena = nullptr;
    size_t arena_bytes = 0;
    double *um0, *um, *u, *pres, *dvel, *vis, *amut, *vort, *flux, *R, *W, *jbn, *jx, *jy, *jz,
        *mask, *dxyz, *ratios, *phi, *phig0, *phigA, *phigB, *wenoC, *wenoE, *xyz, *clock;
    unsigned char *impflag = nullptr;
    // blade-edge interpolation of the impeller (imp.interp)
    double *ip_geo = nullptr;
    unsigned char *ip_status = nullptr;
    signed char *ip_face = nullptr;
    int *ip_nb = nullptr, *ip_list = nullptr, *ip_count = nullptr;
    double rango = 0.0;
    emix::DerivTable T[3];
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t fgraph = nullptr;          // the filter (filtrado), when on
    cudaGraphExec_t fgexec = nullptr;
    long step_index = 0;
    bool static_set = false;
    int launches = 0;
    // optional per-launch timing (emix_ctx_profile): events around every launch
    bool prof = false;
    int prof_n = 0;
    cudaEvent_t prof_ev[2 * 64] = {};
    int prof_cls[64] = {};
    std::vector<emix::Launch> plan;   // one RK3 step
};

namespace emix {
// step.cu: rebuild the launch plan after a parameter change (drops the
// captured graphs), and issue one step's launches on the context stream
void ctx_rebuild_plan(emix_ctx *c);
int ctx_issue_step(emix_ctx *c);
} // namespace emix
