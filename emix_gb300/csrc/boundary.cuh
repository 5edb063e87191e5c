// boundary.cuh -- wall boundary conditions of the reference's RK substep as
// plane kernels: frontera_z_val, frontera_y_val, frontera_x_val
// (src/MSVSingle/frontera_z.f90:219-262, frontera_y.f90:220-247,
// frontera_x.f90:223-255), applied in that order to um1 after the RK
// combination (solver/rungek_ico.f90:98-100).
#pragma once

#include "common.cuh"

namespace emix {

struct BcArgs {
    double *um;     // 5 fields
    int axis;       // 2 = z walls, 1 = y walls, 0 = x walls
    int nx, ny, nz;
    long n;
};

__host__ __device__ inline long bc_count(const BcArgs &a) {
    return a.axis == 2 ? (long)a.nx * a.ny : (a.axis == 1 ? (long)a.nx * a.nz : (long)a.ny * a.nz);
}

EMIX_DEV void bc_cell(const BcArgs &a, long q) {
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long n = a.n;
    double *U[5] = {a.um, a.um + n, a.um + 2 * n, a.um + 3 * n, a.um + 4 * n};
    if (a.axis == 2) {
        // z = 1: copy from z = 2, um(4) = 0; z = nz-1, nz: um(1) = 1, copy from
        // nz-2 (um(2), um(3), um(5)), um(4) = 0
        const long lo = q, lo1 = q + (long)nx * ny;
        const long hi = q + (long)(nz - 1) * nx * ny, hi1 = q + (long)(nz - 2) * nx * ny,
                   hi2 = q + (long)(nz - 3) * nx * ny;
        U[0][lo] = U[0][lo1];
        U[1][lo] = U[1][lo1];
        U[2][lo] = U[2][lo1];
        U[3][lo] = 0.0;
        U[4][lo] = U[4][lo1];
        U[0][hi] = 1.0;
        U[0][hi1] = 1.0;
        U[1][hi] = U[1][hi2];
        U[1][hi1] = U[1][hi2];
        U[2][hi] = U[2][hi2];
        U[2][hi1] = U[2][hi2];
        U[3][hi] = 0.0;
        U[3][hi1] = 0.0;
        U[4][hi] = U[4][hi2];
        U[4][hi1] = U[4][hi2];
    } else if (a.axis == 1) {
        // y walls: um(1), um(5) copied from the neighbour plane, momentum 0
        const int i = (int)(q % nx), k = (int)(q / nx);
        const long lo = i + (long)nx * ny * k, hi = lo + (long)nx * (ny - 1);
        U[0][lo] = U[0][lo + nx];
        U[0][hi] = U[0][hi - nx];
        U[1][lo] = 0.0; U[1][hi] = 0.0;
        U[2][lo] = 0.0; U[2][hi] = 0.0;
        U[3][lo] = 0.0; U[3][hi] = 0.0;
        U[4][lo] = U[4][lo + nx];
        U[4][hi] = U[4][hi - nx];
    } else {
        // x walls: momentum 0, um(5) and um(1) copied from the neighbour plane
        const long lo = (long)nx * q, hi = lo + nx - 1;
        U[1][lo] = 0.0; U[2][lo] = 0.0; U[3][lo] = 0.0;
        U[4][lo] = U[4][lo + 1];
        U[0][lo] = U[0][lo + 1];
        U[1][hi] = 0.0; U[2][hi] = 0.0; U[3][hi] = 0.0;
        U[4][hi] = U[4][hi - 1];
        U[0][hi] = U[0][hi - 1];
    }
}

__global__ void k_bc(BcArgs a);

int launch_bc_walls(double *um1, int nx, int ny, int nz, cudaStream_t st);

} // namespace emix
