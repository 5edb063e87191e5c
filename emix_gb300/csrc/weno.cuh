// weno.cuh -- WENO5 level-set advection (one TVD-RK3 stage per launch).
//
// Semantics follow the reference's never-called driver cuAdvectLsJB
// (src/LevelSet/lsTransportEc.cu:201-418): Dev1thO_Downwind -> the
// left/right-biased Jiang-Peng reconstructions PhiDevPlusParameterJB /
// PhiDevMinusParameterJB (src/LevelSet/lsTools.cu:587-770) -> the upwind
// selection of advect_RS_WENO (:361-417) -> RunGK_First/Second/ThirdS
// (src/LevelSet/extrapol.cu:155-212), all on the ghost-padded grid, with the
// reference's index rules at the padded-grid edges.
//
// One fused kernel per stage instead of five launches and ten field passes:
// each block stages the backward differences of its tile (plus the stencil
// halo) in shared memory once per direction, and each cell evaluates only
// the upwind reconstruction its velocity selects (the other one is
// multiplied by zero in the reference).
#pragma once

#include "common.cuh"

namespace emix {

struct WenoArgs {
    const double *phi;   // padded field read with the stencil
    const double *phi0;  // padded field read at the cell (stages 2 and 3)
    double *out;         // padded output, or unpadded interior when out_interior
    const double *vel;   // 3 components
    const double *jbn;   // components 0, 4, 8 read
    int reflect;         // 1: vel/jbn are unpadded and read at mirrored indices
    int out_interior;
    int nxg, nyg, nzg;   // padded dimensions
    int g;               // ghost layers (used when reflect or out_interior)
    double sx, sy, sz;   // 1/h per axis
    double dt;
    int stage;           // 1, 2, 3
    int ref_bugs;
};

constexpr int kWX = 32, kWY = 4, kWZ = 2;

__global__ void __launch_bounds__(kWX *kWY *kWZ) k_weno_stage(WenoArgs a);

// Padding with mirrored ghost cells: cuSwapToGhost followed by
// cuGhostCellsMirror3dZ/Y/X (src/LevelSet/lsTools.cu:482-585,772-796).
__global__ void k_ghost_pad(double *__restrict__ ghost, const double *__restrict__ val, int g,
                            double dir, int nx, int ny, int nz);
__global__ void k_ghost_unpad(double *__restrict__ val, const double *__restrict__ ghost, int g,
                              int nx, int ny, int nz);

int launch_weno_stage(const WenoArgs &a, cudaStream_t st);

} // namespace emix
