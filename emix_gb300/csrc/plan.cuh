// plan.cuh -- a step as a list of kernel-argument records.
//
// A context builds its RK3 step once as a plan: one record per launch, with
// every pointer and constant the kernel needs.  A single grid executes the
// plan with ordinary launches (launch_single).  A batch of grids executes
// position k of all plans as one persistent launch over every grid's work
// (batch.cu), which is possible because the kernel bodies take explicit block
// indices.
#pragma once

#include "boundary.cuh"
#include "deriv.cuh"
#include "deriv_tma.cuh"
#include "pointwise.cuh"
#include "weno.cuh"

#include <vector>

namespace emix {

enum LaunchKind {
    LK_PRIM, LK_PAD, LK_WENO, LK_DERIV_X, LK_DERIV_YZ, LK_SMAG, LK_SF, LK_VORT, LK_SELECT,
    LK_FLUX, LK_RK, LK_BC, LK_CLOCK, LK_INTERP, LK_COUNT
};

// profile classes (emix_ctx_profile)
enum {
    CLS_PRIM, CLS_PAD, CLS_WENO, CLS_GRADX, CLS_GRADY, CLS_GRADZ, CLS_SGS, CLS_FLUX,
    CLS_DIVX, CLS_DIVY, CLS_DIVZ, CLS_RK, CLS_FILTER, CLS_GRADYZ, CLS_SGSFLUX, CLS_COUNT
};

struct DerivArgs {
    DerivTable T;
    PencilFields F;
    int axis, epi, nf, nx, ny, nz;
    int pair;   // single-grid step: run with the next record (the z launch) as one launch
};

struct Launch {
    int kind;
    int cls;
    union {
        PrimArgs prim;
        PadArgs pad;
        WenoArgs weno;
        DerivArgs deriv;
        SmagArgs smag;
        SfArgs sf;
        VortArgs vort;
        SelArgs sel;
        FluxArgs flux;
        RkArgs rk;
        BcArgs bc;
        ImpClockArgs clock;
        ImpInterpArgs interp;
    };
    const CUtensorMap *tmap;   // LK_WENO: plane tiles by TMA (null: register-staged loads)
    const PencilMaps *pmaps;   // LK_DERIV_YZ accumulating: rows by TMA (null: loads)
    const PencilMaps *pair_pmaps;   // the gradients' y record: the fused y + z launch by TMA
};

int launch_single(const Launch &L, cudaStream_t st);

// records k and k+1 of a plan that run as one launch (step.cu): 1 the
// gradients' y and z records, 2 Smagorinsky and the fluxes; 0 none
int plan_fuse_next(const std::vector<Launch> &P, size_t k);

// records k and k+1 as the one launch plan_fuse_next pairs them into (the
// gradient pair by TMA rows where the y record carries its maps)
int launch_fused_pair(const std::vector<Launch> &P, size_t k, cudaStream_t st);

// compact filter (filter.cu): filtrado on um[5] in place; the tables are
// prepared on the host before any stream capture
int launch_filtrado(double *um, const double *jbn, double cfilt, int nx, int ny, int nz,
                    cudaStream_t st);
int prepare_filtrado(double cfilt, int nx, int ny, int nz);

} // namespace emix
