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
        *mask, *dxyz, *ratios, *phi, *phig0, *phigA, *phigB, *wenoCE, *xyz, *clock;
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
    // the level-set stages run on a second stream, concurrently with the
    // flow's kernels of the same substep (fork before the stage, join before
    // the RK update that overwrites the velocity the stage reads), and so do
    // the x gradients beside the y and z gradients: both fill the launch tails
    // of the other stream's FP64-bound kernels (emix_ctx_set_overlap; on by
    // default for level-set contexts)
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev[3] = {}, join_ev[3] = {};
    // bit 1: the level-set stages on `side`; bit 2: each substep's x
    // gradients on `side`, concurrent with its y and z gradients (joined
    // before the first launch that reads them)
    int overlap = 0;
    cudaEvent_t gfork_ev[3] = {}, gjoin_ev[3] = {};
    // pairs of records run as one launch (plan_fuse_next; emix_ctx_set_fusion)
    bool fuse = true;
    // the level-set stages' plane tiles by TMA (emix_ctx_set_tma; on by
    // default where the copy unit's alignment rules hold), one map per stage
    bool tma = true;
    CUtensorMap weno_tmap[3];
    // the divergence's y and z passes and the gradients' fused y + z launch
    // with their rows by TMA (emix_ctx_set_pencil_tma): maps per substep,
    // [2s + a] the divergence along axis a + 1, [6 + s] the gradients
    bool pencil_tma = true;
    emix::PencilMaps pmaps[9];
    // emix_step_host's own issue of its first and last steps
    // (issue_step_host, step.cu): the uploads and the copies back on `side`,
    // overlapped with the step by z-slabs; the events it orders them with
    static constexpr int kE2eSlabsIn = 8, kE2eSlabs = 4;
    static constexpr int kE2eEvents = 2 + kE2eSlabsIn + 2 * kE2eSlabs + kE2eSlabsIn + 2;
    cudaEvent_t e2e_ev[kE2eEvents] = {};
    // the first level-set stage's slabs alternate between these two streams,
    // so that one slab's last wave overlaps the next slab's first
    cudaStream_t slab_st[2] = {};
};

namespace emix {
// step.cu: rebuild the launch plan after a parameter change (drops the
// captured graphs), and issue one step's launches on the context stream
void ctx_rebuild_plan(emix_ctx *c);
int ctx_issue_step(emix_ctx *c);
} // namespace emix
