// pointwise.cuh -- cell-local kernels of the RK3 substep: fluxes, SGS
// viscosity, RK update and the variable conversions.
#pragma once

#include "common.cuh"

namespace emix {

// Loop over cells with a grid-stride loop (grids are sized to the GPU).
#define EMIX_FOR_CELLS(q, n) \
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (n); q += (long)gridDim.x * blockDim.x)

inline int cells_grid(long n, int bs = 256) {
    long b = (n + bs - 1) / bs;
    const long cap = 152L * 8;   // 8 resident blocks per SM on 152 SMs
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

// ---- flujos(neq), solver/flujos_compact.f90:21-217 -------------------------
__global__ void k_flux_one(int neq, double *__restrict__ e, double *__restrict__ f,
                           double *__restrict__ g, double *__restrict__ ev,
                           double *__restrict__ fv, double *__restrict__ gv,
                           const double *__restrict__ um, const double *__restrict__ u,
                           const double *__restrict__ pres, const double *__restrict__ dvel,
                           const double *__restrict__ jbn, const double *__restrict__ vis, long n);

// Fused flux of all five equations for the RK3 step, inviscid plus viscous,
// already projected by J*dxi/dx (x), J*deta/dy (y), J*dzeta/dz (z):
//   F[3*m + d] = Jd * (inviscid_{m,d} + viscous_{m,d}),  m = 0..4, d = 0..2.
// jx/jy/jz are the static products jbn10*jbn1, jbn10*jbn5, jbn10*jbn9.
struct FluxArgs {
    double *F[15];
    const double *um;    // 5 fields
    const double *u;     // 3 fields
    const double *pres;
    const double *dvel;  // 9 fields
    const double *vis;
    const double *jbn;   // 11 fields (components 0, 4, 8 read)
    const double *jx, *jy, *jz;
    long n;
};
__global__ void k_flux_all(FluxArgs a);

// ---- SGS ---------------------------------------------------------------------
// INISGDM (solver/sgdm_incomp.f90:20-108)
__global__ void k_sgs_setup(const double *__restrict__ xyz, double *__restrict__ dxyz,
                            double *__restrict__ ratios, int nx, int ny, int nz);

// Smagorinsky: amut = (Cs*Delta)^2 sqrt(2 S_ij S_ij), vis = c4 + amut
__global__ void k_sgs_smag(const double *__restrict__ dvel, const double *__restrict__ jbn,
                           const double *__restrict__ dxyz, double cs, double c4,
                           double *__restrict__ amut, double *__restrict__ vis, long n);

// structure function (f_structura + amu0*sqrt*Delta), solver/sgdm_incomp.f90:131-137,166-298
__global__ void k_sgs_sf(const double *__restrict__ u, const double *__restrict__ ratios,
                         const double *__restrict__ dxyz, double amu0,
                         double *__restrict__ amut, int nx, int ny, int nz);
// VORT, :330-341
__global__ void k_vort(const double *__restrict__ dvel, const double *__restrict__ jbn,
                       double *__restrict__ w, long n);
// SELECTIVO (:346-395) and viscosidad (vis = c4 + amut)
__global__ void k_selective(const double *__restrict__ w, double *__restrict__ amut,
                            double *__restrict__ vis, double cutoff, double c4,
                            int nx, int ny, int nz);

// ---- RK3 step pieces -----------------------------------------------------------
// primitive variables from um: u = um(2..4)/um(1), pres = um(1)/Mach^2
__global__ void k_prim(const double *__restrict__ um, double *__restrict__ u,
                       double *__restrict__ pres, double inv_m2, long n);

// rs = jbn11*R; RK stage s; varc_to_varnc, clip to [-6,6], mask, varc_to_varnc;
// rebuild um1(1) = pres*Mach*Mach, um1(2..4) = u*um1(1)
// (solver/rungek_ico.f90:83-138,150-198,210-267)
struct RkArgs {
    const double *R;      // 5 fields
    const double *um0;    // 5
    const double *um;     // 5 (previous substep)
    double *out;          // 5 (may alias um or um0: read-before-write per cell)
    double *u;            // 3
    double *pres;
    const double *jbn;
    const double *mask;
    double dt, mach, inv_m2;
    int stage;
    long n;
};
__global__ void k_rk_post(RkArgs a);

} // namespace emix
