/*
 * oracle.h -- CPU restatement of the eMix3d per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in emix_gb300/csrc; only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py load it.  The product path never
 * calls it.
 *
 * Every function restates one piece of the reference (jramirezcr/eMix3d) and
 * names the file:line it follows.  Arithmetic is written in the same order
 * as the reference so that results agree to rounding; the build uses
 * -ffp-contract=off so x86 and Arm hosts give identical results.
 *
 * Layout: Fortran column-major, i fastest, linear index i + nx*(j + ny*k)
 * (src/Engine/cuArray.cu:123).  Multi-component arrays stack components
 * with stride nx*ny*nz (solver/cuDeriv.cu:588-590).
 *
 * Parity pinning: the reference has no tests, golden vectors or fixtures,
 * and its Fortran CPU path cannot be compiled here (no Fortran compiler).
 * Scheme C, cuDivergence, the WENO5 TVD-RK3 step, the ghost padding and the
 * pressure extrapolation of advect_CUDA are pinned against outputs of the reference's own CUDA kernels run on a GPU
 * (tests/golden/reference_cuda.npz); the Fortran-only parts (schemes A, B and
 * cyclic B, flujos, the SGS models, the RK loop) are pinned by analytic
 * known-answer tests only -- parity against the reference's own outputs is
 * unpinned for those.
 */
#ifndef EMIX_ORACLE_H
#define EMIX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Compact-scheme variants (one per coefficient table in the reference). */
enum {
    ORC_SCHEME_A = 0,      /* solver/derivada.f90:2-125 (Pade-4, alpha=1/4, alpha_1=3)   */
    ORC_SCHEME_B = 1,      /* src/MSVSingle/derivada_incomp.f90:130-218,297-329 (Lele-6) */
    ORC_SCHEME_BPER = 2,   /* src/MSVSingle/derivada_incomp.f90:221-294 (cyclic Lele-6)  */
    ORC_SCHEME_C = 3       /* src/Schemes/derivCompact.cu:81-215 (production GPU)       */
};

/* One pencil, in place.  h is the grid spacing in computational space. */
int orc_deriv_pencil(int scheme, int n, double *u, double h);

/* Derivative of a 3-D field along axis (0=x,1=y,2=z); gather/derivnper/scatter
 * as solver/deriv_vel.f90:17-161. */
int orc_deriv3d(int scheme, int axis, int nx, int ny, int nz, double h,
                const double *in, double *out);

/* cudaDeriv contract (solver/cuDeriv.cu:529-654): 9 velocity and 3
 * temperature derivatives in computational coordinates. */
int orc_cudaDeriv(const int *schemes, double *dvel, double *dtemp,
                  const double *vel, const double *temp,
                  double hx, double hy, double hz, int nx, int ny, int nz);

/* cuDivergence contract (solver/cuDivergence.cu:107-189 and
 * solver/divergencia.f90:225-354).  Inputs are not modified. */
int orc_cuDivergence(const int *schemes, double *rs, double *rsv,
                     const double *e, const double *f, const double *g,
                     const double *ev, const double *fv, const double *gv,
                     const double *jbn, double hx, double hy, double hz,
                     int nx, int ny, int nz);

/* flujos(neq) (solver/flujos_compact.f90:21-217).  neq in 1..5. */
int orc_flujos(int neq, int nx, int ny, int nz,
               double *e, double *f, double *g,
               double *ev, double *fv, double *gv,
               const double *um, const double *u, const double *pres,
               const double *dvel, const double *jbn, const double *vis);

/* INISGDM (solver/sgdm_incomp.f90:2-114): filter width and the six
 * one-sided spacing ratios from grid coordinates xyz (3 components). */
int orc_inisgdm(int nx, int ny, int nz, const double *xyz,
                double *dxyzsgd, double *ratios /* 6: xp,xm,yp,ym,zp,zm */);

/* viscosidad_t with the selective structure-function model
 * (solver/sgdm_incomp.f90:117-162,166-315,319-343,346-395). */
int orc_sgs_sf(int nx, int ny, int nz, const double *u, const double *dvel,
               const double *jbn, const double *dxyzsgd, const double *ratios,
               double amu0, double *amut);

/* Smagorinsky eddy viscosity from the physical gradient jbn(1|5|9)*dvel:
 * nu_t = (Cs*Delta)^2 * sqrt(2 S_ij S_ij).  Not in the reference. */
int orc_sgs_smag(int nx, int ny, int nz, const double *dvel, const double *jbn,
                 const double *dxyzsgd, double cs, double *amut);

/* viscosidad (src/MSVSingle/viscosidad_incomp.f90:12-20): vis = c4 + amut. */
int orc_viscosidad(int n, const double *amut, double c4, double *vis);

/* Level set: ghost padding and mirroring (src/LevelSet/lsTools.cu:482-585,
 * 772-822), and one WENO5 TVD-RK3 advection step on ghosted arrays
 * (src/LevelSet/lsTransportEc.cu:201-418). */
int orc_to_ghost(double *ghost, const double *val, int g, int nx, int ny, int nz);
int orc_mirror_ghost(double *ghost, int g, int nx, int ny, int nz, double direction);
int orc_from_ghost(double *val, const double *ghost, int g, int nx, int ny, int nz);
int orc_weno_rhs(double *rs, const double *phi, const double *vel, const double *jbn,
                 double hx, double hy, double hz, int nxg, int nyg, int nzg,
                 int ref_bugs);
int orc_weno_advect(double *phi, const double *vel, const double *jbn,
                    double hx, double hy, double hz, double dt,
                    int nxg, int nyg, int nzg, int ref_bugs);
double orc_phi_x_weno(double b1, double b2, double b3, double b4, double b5);

/* A rotating Rushton-type impeller as a volumetric forcing, the linked
 * rushton(sub_step) without its blade-edge interpolation
 * (src/Geometry/rush_ruth_me.f90:2-108 with makeAspa :519-593, and
 * addMaskCil / addAngularVel, src/Geometry/rotating.f90:110-205): a mask that
 * is 0 inside nblades rectangular blades (blade b at angle
 * theta0 + omega*t + b*2*pi/nblades, radial extent [r1, r2], half-thickness
 * half_thick, z in [z1, z2]), a hub disc (radius hub_r, z in
 * [hub_z1, hub_z2]) and a shaft (radius shaft_r, z in [shaft_z0, shaft_z1]),
 * and 1 elsewhere; inside it the velocity is that of the rotating body. */
typedef struct {
    int on;
    int nblades;
    double omega, theta0;
    double r1, r2, z1, z2, half_thick;
    double hub_r, hub_z1, hub_z2;
    double shaft_r, shaft_z0, shaft_z1;
    int interp;           /* 1: also the blade-edge interpolation (:97-185, getInterpolData) */
} orc_impeller;

/* Parameters of one RK3 step (solver/rungek_ico.f90:61-313). */
typedef struct {
    int nx, ny, nz;
    int scheme[3];        /* per axis: ORC_SCHEME_* */
    double h[3];          /* computational spacing per axis */
    int sgs_model;        /* 0 none, 1 Smagorinsky, 2 selective structure function */
    double cs;            /* Smagorinsky constant */
    double amu0;          /* structure-function constant (0.1781 in the reference) */
    double c4;            /* 1/Re */
    double mach;
    double dt;
    int level_set;        /* 1: advance the level set with the flow: one WENO5 TVD stage per substep */
    int ls_ghost;         /* ghost layers for the level set (5 in the reference) */
    int ref_bugs;         /* 1: reproduce the reference's z-top WENO index */
    int bc_walls;         /* 1: frontera_z/y/x_val after each RK combination */
    int filter_every;     /* > 0: filtrado at the end of steps with step_index % filter_every == 0 (9 in the reference) */
    double cfilt;         /* filter parameter alpha (cfilt of data.in) */
    long step_index;      /* steps taken before this one */
    orc_impeller imp;     /* rotating impeller forcing after the walls */
    double time;          /* time at the start of this step (dto) */
    const double *xyz;    /* grid coordinates (3 fields), read when imp.on */
} orc_step_params;

/* One RK3 step.  State in/out: um (5 fields) and phi (1 field, may be NULL
 * when level_set == 0).  Static inputs: jbn (11), mask, dxyzsgd, ratios (6,
 * only for the structure-function model). */
int orc_step(const orc_step_params *p, double *um, double *phi,
             const double *jbn, const double *mask,
             const double *dxyzsgd, const double *ratios);

/* frontera_z_val, frontera_y_val, frontera_x_val in that order on um[5]
 * (src/MSVSingle/frontera_z.f90:219-262, frontera_y.f90:220-247,
 * frontera_x.f90:223-255). */
int orc_bc_walls(double *um, int nx, int ny, int nz);

/* CFL number of TSTEP with the spacings of INITSTEP
 * (src/MSVSingle/tstep_incomp.f90:1-136). */
double orc_cfl(const double *u, const double *xyz, double mach, int nx, int ny, int nz);

/* JACOBEANO (solver/jacob_malla.f90:1-171) with the given scheme and spacing. */
int orc_jacobeano(const double *xyz, double *jbn, int scheme, double hx, double hy, double hz,
                  int nx, int ny, int nz);

/* cuExtrapolation (src/LevelSet/interface.cu:341-436) on an (already padded)
 * grid: ext is extrapolated across the region phiS > 0 (flag > 0) or
 * phiS <= 0 (flag <= 0); j0, j4, j8 are metric components 1, 5, 9; sx, sy, sz
 * the inverse spacings the kernels receive; iters TVD-RK3 pseudo-steps. */
int orc_extrapolation(double *ext, const double *phiS, const double *j0, const double *j4,
                      const double *j8, double sx, double sy, double sz, int nx, int ny, int nz,
                      double dtext, int flag, int iters);

/* advect_CUDA as linked (src/LevelSet/lsTransportEc.cu:24-197): pressure
 * extrapolation into the solid object sobject, with 5 mirrored ghost layers;
 * press in/out, jbn 11 components (1, 5, 9 read). */
int orc_advect_extrapolate(double *press, const double *jbn, const double *sobject,
                           double deltaX, double deltaY, double deltaZ, int nx, int ny, int nz,
                           double deltamin);

/* filtronper (src/MSVSingle/filtro_incomp.f90:307-362) on one pencil, in
 * place, with the rows of inifiltro for cfilt (zrows = 1: the periodic rows
 * that filtrado passes for z). */
int orc_filtronper(int n, double *u, double cfilt, int zrows);

/* filtrado as RUNGEK calls it (itf = 1; herramientas_incomp2.f90:227-410) on
 * um[5] in place. */
int orc_filtrado(double *um, const double *jbn, double cfilt, int nx, int ny, int nz);

/* The impeller forcing at time t on um[5] in place (rush_ruth_me.f90:52-95);
 * mask_out (may be NULL) receives the impeller mask. */
int orc_impeller_force(double *um, const double *xyz, const orc_impeller *imp, double t,
                       int nx, int ny, int nz, double *mask_out);

/* cuReinitLsJB (src/LevelSet/lsTransportEc.cu:420-676): `iters` Sussman
 * reinitialisation iterations of the padded level set phi (in/out) with the
 * padded metric jbn (11 components), per-cell smoothing widths dmins, ghost
 * width g, pseudo time step deltamin/2; ref_bugs keeps the z-top index of
 * PhiDevPlusParameterJB. */
int orc_reinit(double *phi, const double *jbn, const double *dmins, double dX, double dY, double dZ,
               int nxg, int nyg, int nzg, int g, double deltamin, int iters, int ref_bugs);

/* Number of OpenMP threads the oracle uses (0 = library default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
