/*
 * emix_gb300.h -- C ABI of the GB300-native eMix3d hot path.
 *
 * The library (libemix_gb300.so) replaces the CUDA side of the reference's
 * Fortran -> C boundary.  Plain pointers and sizes only; no C++ or torch
 * types.  Fields are Fortran column-major (i fastest, index
 * i + nx*(j + ny*k)); multi-component arrays stack components with stride
 * nx*ny*nz.  All arithmetic is IEEE FP64.
 *
 * Two families of entry points:
 *   - the reference's own symbols (cudaDeriv, cuDivergence) with byte-identical
 *     signatures: host pointers, synchronous, void return; on error they print
 *     a message and return (they never exit or trap);
 *   - emix_* functions that return an int status (EMIX_OK == 0) and come in
 *     host-pointer and device-pointer ("_dev") forms.
 *
 * Every entry point runs on the calling thread's current CUDA device.
 */
#ifndef EMIX_GB300_H
#define EMIX_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    EMIX_OK = 0,
    EMIX_ERR_ARG = 1,          /* bad size, null pointer, unknown option      */
    EMIX_ERR_CUDA = 2,         /* a CUDA runtime call failed                  */
    EMIX_ERR_ALLOC = 3,        /* device or pinned allocation failed          */
    EMIX_ERR_UNSUPPORTED = 4,  /* option not built                            */
    EMIX_ERR_TIMEOUT = 5       /* a bounded device wait gave up               */
};

/* ---- compact first-derivative schemes ----------------------------------- */
enum {
    EMIX_SCHEME_A = 0,     /* Pade-4 interior, alpha_1 = 3 closure: solver/derivada.f90:2-125           */
    EMIX_SCHEME_B = 1,     /* Lele-6 interior, 3rd/4th-order closure: src/MSVSingle/derivada_incomp.f90:130-218,297-329 */
    EMIX_SCHEME_BPER = 2,  /* cyclic Lele-6 (Sherman-Morrison): src/MSVSingle/derivada_incomp.f90:221-294 */
    EMIX_SCHEME_C = 3      /* Lele-6 interior, alpha_1 = 3 closure: src/Schemes/derivCompact.cu:81-215 */
};

/* ---- SGS models --------------------------------------------------------- */
enum {
    EMIX_SGS_NONE = 0,
    EMIX_SGS_SMAGORINSKY = 1,   /* nu_t = (Cs*Delta)^2 sqrt(2 S_ij S_ij); not in the reference        */
    EMIX_SGS_STRUCTURE = 2      /* selective structure function: solver/sgdm_incomp.f90:117-395      */
};

/* Message describing the last error on the calling thread ("" if none). */
const char *emix_last_error(void);

/* Library version string. */
const char *emix_version(void);

/* ========================================================================
 * Reference symbols (drop-in)
 * ======================================================================== */

/* Replaces cudaDeriv, solver/cuDeriv.cu:529-539 (Fortran interface
 * solver/deriv_vel_cuda.f90:19-39).  Outputs dVel[9] in the order d/dx(u,v,w),
 * d/dy(u,v,w), d/dz(u,v,w) and dTemp[3] = dT/dx, dT/dy, dT/dz, in
 * computational coordinates.  deltaX/Y/Z are the grid spacings h (the
 * kernel scales by 1/h).  amut, dxyzsgd and jbn are accepted and unused, as in
 * the reference.  Scheme: the one set by emix_set_legacy_scheme (default
 * EMIX_SCHEME_C, the reference's production GPU scheme). */
void cudaDeriv(double *dVel, double *dTemp, double *vel, double *temp,
               double *amut, double *dxyzsgd, double *jbn,
               double deltaX, double deltaY, double deltaZ,
               int Nx, int Ny, int Nz);

/* Replaces cuDivergence, solver/cuDivergence.cu:107-119 (Fortran interface
 * solver/divergencia_cuda.f90:21-42).  rs  = jbn11*(d/dxi(jbn10*jbn1*e) +
 * d/deta(jbn10*jbn5*f) + d/dzeta(jbn10*jbn9*g)), rsv the same for ev,fv,gv.
 * jbn holds 11 components; the inputs are not modified. */
void cuDivergence(double *rs, double *rsv, double *e, double *f, double *g,
                  double *ev, double *fv, double *gv, double *jbn,
                  double deltaX, double deltaY, double deltaZ,
                  int Nx, int Ny, int Nz);

/* Scheme used by the two symbols above (EMIX_SCHEME_*).  Returns status. */
int emix_set_legacy_scheme(int scheme);

/* ========================================================================
 * Status-returning operators
 * ======================================================================== */

/* Compact derivative of nf fields along axis (0=x, 1=y, 2=z), device
 * pointers.  in and out hold nf fields each (stride nx*ny*nz) and must not
 * overlap.  Replaces cu::cs::dFdX/dFdY/dFdZ, src/Schemes/derivCompact.cu:222-409,
 * generalised to every scheme of the reference. */
int emix_deriv_dev(int scheme, int axis, int nf, double *out, const double *in,
                   double h, int nx, int ny, int nz, void *stream);

/* emix_deriv_dev along y (axis 1) or z (axis 2) by parallel cyclic
 * reduction + Thomas instead of one serial Thomas sweep per pencil
 * (src/Schemes/derivCompact.cu:146-215 solves each pencil serially): steps =
 * 2..5 PCR steps split each pencil over 2^steps lanes of a warp (partners
 * exchanged by warp shuffles), each lane then solving its 2^-steps share by
 * Thomas.  Pencils of at most 160 rows (EMIX_ERR_ARG otherwise).  The same
 * operator as emix_deriv_dev to rounding.  Device pointers. */
int emix_deriv_pcr_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                       int steps, int nx, int ny, int nz, void *stream);

/* cudaDeriv with status, explicit per-axis schemes, host pointers. */
int emix_cudaDeriv(const int schemes[3], double *dVel, double *dTemp,
                   const double *vel, const double *temp,
                   double hx, double hy, double hz, int nx, int ny, int nz);

/* Same, device pointers, asynchronous on stream.  dTemp/temp may be NULL
 * (the temperature derivatives are then skipped). */
int emix_cudaDeriv_dev(const int schemes[3], double *dVel, double *dTemp,
                       const double *vel, const double *temp,
                       double hx, double hy, double hz, int nx, int ny, int nz,
                       void *stream);

/* cuDivergence with status, explicit schemes, host pointers. */
int emix_cuDivergence(const int schemes[3], double *rs, double *rsv,
                      const double *e, const double *f, const double *g,
                      const double *ev, const double *fv, const double *gv,
                      const double *jbn, double hx, double hy, double hz,
                      int nx, int ny, int nz);

/* Same, device pointers. */
int emix_cuDivergence_dev(const int schemes[3], double *rs, double *rsv,
                          const double *e, const double *f, const double *g,
                          const double *ev, const double *fv, const double *gv,
                          const double *jbn, double hx, double hy, double hz,
                          int nx, int ny, int nz, void *stream);

/* flujos(neq), solver/flujos_compact.f90:1-220: inviscid and viscous fluxes
 * of equation neq (1..5) into e,f,g,ev,fv,gv.  um[5], u[3], pres, dvel[9],
 * jbn[11], vis.  Device pointers. */
int emix_flux_dev(int neq, double *e, double *f, double *g,
                  double *ev, double *fv, double *gv,
                  const double *um, const double *u, const double *pres,
                  const double *dvel, const double *jbn, const double *vis,
                  int nx, int ny, int nz, void *stream);

/* INISGDM, solver/sgdm_incomp.f90:2-114: filter width dxyzsgd and the six
 * spacing ratios (order xp, xm, yp, ym, zp, zm) from grid coordinates
 * xyz[3].  Device pointers. */
int emix_sgs_setup_dev(const double *xyz, double *dxyzsgd, double *ratios,
                       int nx, int ny, int nz, void *stream);

/* viscosidad_t + viscosidad (solver/sgdm_incomp.f90:117-162,
 * src/MSVSingle/viscosidad_incomp.f90:12-20): eddy viscosity amut and
 * vis = c4 + amut.  model = EMIX_SGS_*; coef = Cs (Smagorinsky) or amu0
 * (structure function).  u[3], dvel[9], jbn[11], dxyzsgd, ratios[6] (only
 * read by the structure-function model).  amut may be NULL.  Device
 * pointers. */
int emix_sgs_viscosity_dev(int model, double coef, double c4,
                           const double *u, const double *dvel, const double *jbn,
                           const double *dxyzsgd, const double *ratios,
                           double *amut, double *vis,
                           int nx, int ny, int nz, void *stream);

/* One WENO5 TVD-RK3 step of phi_t + vel . grad(phi) = 0 on ghost-padded
 * arrays, as cuAdvectLsJB (src/LevelSet/lsTransportEc.cu:201-418): phi
 * (nxg*nyg*nzg, updated in place), vel[3] and jbn[11] (components 0, 4 and 8
 * read) all on the padded grid; hx,hy,hz are the spacings h.  ref_bugs = 1
 * keeps the reference's z-top neighbour index (lsTools.cu:636).  Device
 * pointers; the scratch (two padded stage fields) comes from a grow-only
 * device buffer of the library, allocated on the first call that needs more;
 * calls that overlap on the GPU race on it. */
int emix_weno5_advect_dev(double *phi, const double *vel, const double *jbn,
                          double hx, double hy, double hz, double dt,
                          int nxg, int nyg, int nzg, int ref_bugs, void *stream);

/* Same, host pointers, synchronous. */
int emix_weno5_advect(double *phi, const double *vel, const double *jbn,
                      double hx, double hy, double hz, double dt,
                      int nxg, int nyg, int nzg, int ref_bugs);

/* Same step as emix_weno5_advect_dev without allocating device memory; it
 * has no counterpart in the reference.  For callers that cannot let a library
 * call cudaMalloc (it can block the device, and fails when another allocator
 * already holds the memory).  The two padded stage fields come from a 16 MiB
 * array compiled into the library, so nxg*nyg*nzg must not exceed 1048576
 * (EMIX_ERR_ARG otherwise).  CUDA loads the library's device code lazily, so
 * the first call on a device loads the array's module (reserving its 16 MiB
 * on that device until the process exits) and the stage kernels: that first
 * call does take device memory once.  Make it at set-up, outside any
 * latency-bound loop and before any stream capture; later calls allocate
 * nothing.  All calls share the array: calls that overlap on the GPU race on
 * it. */
int emix_weno5_advect_dev_noalloc(double *phi, const double *vel, const double *jbn,
                                  double hx, double hy, double hz, double dt,
                                  int nxg, int nyg, int nzg, int ref_bugs, void *stream);

/* Ghost padding (cuSwapToGhost + cuGhostCellsMirror3dZ/Y/X,
 * src/LevelSet/lsTools.cu:482-585,772-796) and unpadding (cuSwapFromGhost,
 * :798-822).  ghost is (nx+2g)(ny+2g)(nz+2g).  Device pointers. */
int emix_ghost_pad_dev(double *ghost, const double *val, int g, double direction,
                       int nx, int ny, int nz, void *stream);
int emix_ghost_unpad_dev(double *val, const double *ghost, int g,
                         int nx, int ny, int nz, void *stream);

/* ========================================================================
 * Pressure extrapolation into the solid (the linked advect_CUDA)
 * ======================================================================== */

/* The reference's symbol advect_CUDA (src/LevelSet/lsTransportEc.cu:24-35;
 * Fortran interface include/LevelSet/interfaceAdvect.h:3-16, called from
 * solver/advectLS.f90:19 with deltaX = h).  As linked, it extrapolates the
 * pressure into the solid object sobject > 0: 5 mirrored ghost layers, the
 * direction field of DevFirstOrder_LS, 10 TVD-RK3 pseudo-steps of
 * deltamin/2 (src/LevelSet/interface.cu:341-436).  Host buffers, synchronous,
 * current device; errors are printed and the call returns. */
void advect_CUDA(double *press, double *jbn, double *sobject,
                 double deltaX, double deltaY, double deltaZ,
                 int Nx, int Ny, int Nz, double deltamin);

/* advect_CUDA with a status code (host buffers, synchronous). */
int emix_advect_extrapolate(double *press, const double *jbn, const double *sobject,
                            double deltaX, double deltaY, double deltaZ,
                            int nx, int ny, int nz, double deltamin);

/* advect_CUDA on device pointers, queued on `stream`.  Uses the library's
 * per-device scratch (6 padded fields): calls that overlap on one device race. */
int emix_advect_extrapolate_dev(double *press, const double *jbn, const double *sobject,
                                double deltaX, double deltaY, double deltaZ,
                                int nx, int ny, int nz, double deltamin, void *stream);

/* cuExtrapolation (src/LevelSet/interface.cu:341-436) on the grid padded with
 * 5 mirrored layers: ext extrapolated across phiS > 0 (flag > 0) or
 * phiS <= 0 (flag <= 0) by `iters` TVD-RK3 pseudo-steps of dtext; the kernels
 * use 1/deltaX as the reference's do.  Device pointers; jbn 11 components
 * (1, 5, 9 read).  Same scratch caveat as above. */
int emix_extrapolate_dev(double *ext, const double *phiS, const double *jbn,
                         double deltaX, double deltaY, double deltaZ,
                         int nx, int ny, int nz, double dtext, int flag, int iters,
                         void *stream);

/* ========================================================================
 * Adjoint building blocks
 * ======================================================================== */

/* out = D^T in (accumulate = 0) or out += D^T in (1): the transpose of the
 * compact first derivative emix_deriv_dev computes (no counterpart in the
 * reference; the adjoint of cudaDeriv / cuDivergence).  Device pointers;
 * uses the library's per-device scratch. */
int emix_deriv_t_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                     int nx, int ny, int nz, int accumulate, void *stream);

/* emix_deriv_t_dev along y or z (axis 1, 2) with the rows staged by TMA
 * tiled copies, as the adjoint's reverse sweep runs it: the same values bit
 * for bit.  EMIX_ERR_ARG where the copy unit's rules do not hold (axis 0,
 * the cyclic scheme, nx odd, a pointer not 16-byte aligned). */
int emix_deriv_t_tma_dev(int scheme, int axis, int nf, double *out, const double *in, double h,
                         int nx, int ny, int nz, int accumulate, void *stream);

/* Sussman reinitialisation of a padded level set: the device form of
 * cuReinitLsJB (src/LevelSet/lsTransportEc.cu:420-676, with
 * reini_RS_WENOJB, src/LevelSet/lsTools.cu:824-902).  phi (in/out), jbn
 * (11 components) and dmins are arrays of the padded grid nxg x nyg x nzg with
 * gcells ghost layers, mirrored at the start of every iteration; iters
 * iterations (10 in the reference) of three TVD-RK3 stages of deltamin/2; the
 * kernels use 1/deltaX.  ref_bugs keeps the z-top index of
 * PhiDevPlusParameterJB.  Uses the library's per-device scratch. */
int emix_reinit_dev(double *phi, const double *jbn, const double *dmins, double deltaX, double deltaY,
                    double deltaZ, int nxg, int nyg, int nzg, int gcells, double deltamin, int iters,
                    int ref_bugs, void *stream);

/* ========================================================================
 * Compact filter
 * ======================================================================== */

/* filtrado as RUNGEK calls it (itf = 1: x, then y, then z;
 * src/MSVSingle/herramientas_incomp2.f90:227-410), with filtronper
 * (src/MSVSingle/filtro_incomp.f90:307-362) on every pencil: each pencil of
 * um[0..4] is scaled by jbn(10), filtered, scaled by jbn(11).  z uses the
 * periodic row arrays, as filtrado passes them.  In place, device pointers,
 * every dimension >= 11. */
int emix_filtrado_dev(double *um, const double *jbn, double cfilt,
                      int nx, int ny, int nz, void *stream);

/* One filter pass along `axis` over nf fields in place; zrows = 1 selects the
 * periodic rows (a = c = cfilt on every row), 0 the non-periodic ones. */
int emix_filter_dev(double *f, int nf, const double *jbn, double cfilt, int axis, int zrows,
                    int nx, int ny, int nz, void *stream);

/* ========================================================================
 * Boundary conditions, time step and metrics
 * ======================================================================== */

/* frontera_z_val, frontera_y_val, frontera_x_val in that order on um[5]
 * (src/MSVSingle/frontera_z.f90:219-262, frontera_y.f90:220-247,
 * frontera_x.f90:223-255).  Device pointers. */
int emix_bc_walls_dev(double *um, int nx, int ny, int nz, void *stream);

/* CFL number of TSTEP (src/MSVSingle/tstep_incomp.f90:99-136): the maximum
 * over cells and axes of (|u_d| + sqrt(cs^2 + u_d^2)) / dx_d with dx_d the
 * smaller neighbour spacing (INITSTEP) and cs = sqrt(1/Mach).  u[3], xyz[3]
 * device pointers; *cfla is written on the host (synchronous). */
int emix_cfl_dev(const double *u, const double *xyz, double mach, int nx, int ny, int nz,
                 double *cfla, void *stream);

/* New time step from the CFL number as TSTEP (:138-153): dt = cfl/cfla,
 * smoothed against olddt with up = 0.5, down = 1.2. */
int emix_tstep_dt(double cfla, double olddt, double cfl, double *dt);

/* JACOBEANO (solver/jacob_malla.f90:1-171): jbn[11] from grid coordinates
 * xyz[3] with the compact derivative of `scheme` (the reference uses
 * EMIX_SCHEME_A) and spacings h.  Synchronous; EMIX_ERR_ARG when the
 * Jacobian vanishes somewhere (|det| <= 1e-20). */
int emix_metrics_dev(const double *xyz, double *jbn, int scheme, double hx, double hy, double hz,
                     int nx, int ny, int nz, void *stream);

/* ========================================================================
 * Device-resident RK3 step (solver/rungek_ico.f90:61-313)
 * ======================================================================== */

/* A rotating impeller applied as a volumetric forcing after the walls in
 * every substep: the linked rushton(sub_step) without its blade-edge
 * interpolation (src/Geometry/rush_ruth_me.f90:2-108, makeAspa :519-593;
 * addMaskCil, addAngularVel: src/Geometry/rotating.f90:110-205).  Blade b at
 * angle theta0 + omega*t + b*2*pi/nblades is the box r1 <= along <= r2,
 * |across| <= half_thick, z1 <= z <= z2; the hub disc has radius hub_r over
 * [hub_z1, hub_z2], the shaft radius shaft_r over [shaft_z0, shaft_z1].
 * Inside, the velocity is set to the rigid rotation (-omega*y, omega*x).
 * The reference's impeller is omega = -2*pi, theta0 = -pi/6 (:58-61). */
typedef struct emix_impeller {
    int on;             /* 0: no impeller forcing                                  */
    int nblades;        /* <= 16                                                   */
    double omega, theta0;
    double r1, r2, z1, z2, half_thick;
    double hub_r, hub_z1, hub_z2;
    double shaft_r, shaft_z0, shaft_z1;
    int interp;         /* 1: also the blade-edge interpolation of the velocity
                           (rush_ruth_me.f90:97-185 with getInterpolData)       */
} emix_impeller;

typedef struct emix_params {
    int nx, ny, nz;
    int scheme[3];      /* per axis, EMIX_SCHEME_*                                */
    double h[3];        /* computational spacing per axis                          */
    int sgs_model;      /* EMIX_SGS_*                                              */
    double cs;          /* Smagorinsky constant                                    */
    double amu0;        /* structure-function constant (0.1781 in the reference)   */
    double c4;          /* 1/Re                                                    */
    double mach;        /* um(1) = p*Mach^2                                        */
    double dt;
    int level_set;      /* 1: advance the level set with the flow (WENO5, SSP-RK3) */
    int ls_ghost;       /* ghost layers of the level-set grid (5 in the reference) */
    int ref_bugs;       /* 1: keep the reference's z-top WENO neighbour index      */
    int bc_walls;       /* 1: apply frontera_z/y/x_val after each RK combination   */
    int filter_every;   /* > 0: compact filter (filtrado) after every filter_every-th
                           step, counting from the first (9 in the reference,
                           solver/rungek_ico.f90:269-276); 0: off               */
    double cfilt;       /* filter parameter alpha (cfilt of data.in)              */
    emix_impeller imp;  /* rotating impeller forcing (imp.on = 0: none)           */
    double t0;          /* time at the start of the first step (the impeller's clock) */
} emix_params;

/* The impeller forcing at time t on um[5] (device pointers, in place);
 * mask (may be NULL) receives the impeller mask.  Synchronous. */
int emix_impeller_force_dev(double *um, const double *xyz, const emix_impeller *imp, double t,
                            int nx, int ny, int nz, double *mask, void *stream);

typedef struct emix_ctx emix_ctx;

/* Create a context holding every field of one grid in device memory. */
int emix_ctx_create(const emix_params *p, emix_ctx **out);
int emix_ctx_destroy(emix_ctx *ctx);

/* Stream the context launches on (NULL = the context's own stream). */
int emix_ctx_set_stream(emix_ctx *ctx, void *stream);

/* Concurrency inside a step, a bit mask (0 = one stream; 3, both bits, is
 * the default of level-set contexts, 0 of the others):
 * bit 1 (value 1): each level-set stage runs on a second stream of the
 * context, concurrently with the flow's kernels of its substep (joined before
 * the RK update); bit 2 (value 2): each substep's x gradients run on the
 * second stream concurrently with its y and z gradients (joined before the
 * first launch that reads them).  Results are the same bit for bit in every
 * mode (only level-set contexts have the second stream).  On the 256^3 tank
 * both bits together gain 1% (the concurrent launches fill each other's last
 * waves). */
int emix_ctx_set_overlap(emix_ctx *ctx, int on);

/* 1 (default): the gradients' y and z passes run as one launch, and so do
 * the Smagorinsky viscosity and the fluxes; 0: every operator in a launch of
 * its own.  The values are the same bit for bit (for checks). */
int emix_ctx_set_fusion(emix_ctx *ctx, int on);

/* 1 (default): the level-set stages bring their phi plane tiles into shared
 * memory with TMA tiled copies (one 3-D tensor map per stage) wherever the
 * copy unit's rules hold (padded x extent even, at least 24 x 22 cells);
 * 0: register-staged loads.  Results are bitwise the same either way.
 * emix_ctx_tma_stages gives how many of the step's stages use the copies. */
int emix_ctx_set_tma(emix_ctx *ctx, int on);
int emix_ctx_tma_stages(emix_ctx *ctx);

/* Stage blocks (since the library was loaded, on the current device) that
 * gave up waiting for a plane copy after about 0.3 s and left their cells
 * unwritten; 0 in every correct run. */
int emix_weno_tma_timeouts(int *count);

/* 1: the flux divergence's y and z passes (the accumulating pencil sweeps)
 * bring the rows they read into shared memory by TMA tiled copies (4 rows x
 * 128 pencils per copy, a ring of three), where the copy unit's rules hold
 * (closed schemes, nx even, 16-byte aligned fields); 0: the threads load
 * them.  The values are the same either way.  emix_ctx_pencil_tma_launches
 * gives how many of the step's launches use the copies.  The reference
 * transposes each field and walks each pencil serially
 * (src/Schemes/derivCompact.cu:8-37,146-215). */
int emix_ctx_set_pencil_tma(emix_ctx *ctx, int on);
int emix_ctx_pencil_tma_launches(emix_ctx *ctx);

/* Pencil blocks (since the library was loaded, on the current device) that
 * gave up waiting for a row copy after about 0.3 s and left their pencils
 * unwritten; 0 in every correct run. */
int emix_pencil_tma_timeouts(int *count);

/* Test hook for those bounded waits: 1 makes the TMA pencil launches issue
 * no copies (current device), so every block gives up after its wait, counts
 * itself and leaves its pencils; 0 restores normal operation.  Never set in a
 * production run. */
int emix_pencil_tma_test_drop(int on);

/* Test hook for the bounded waits: 1 makes the TMA level-set stages issue no
 * plane copies (current device), so every stage block gives up after its
 * waits (about a second), counts itself and leaves its cells unwritten; the
 * context stays usable.  0 restores normal operation.  Never set in a
 * production run. */
int emix_weno_tma_test_drop(int on);

/* Static inputs from host memory: jbn[11], mask, grid coordinates xyz[3]
 * (used to build the SGS filter width, as INISGDM). */
int emix_ctx_set_static(emix_ctx *ctx, const double *jbn, const double *mask,
                        const double *xyz);

/* State transfer, host memory: um[5] (p*Mach^2, rho*u, rho*v, rho*w, T) and
 * phi (may be NULL when the level set is off). */
int emix_ctx_upload(emix_ctx *ctx, const double *um, const double *phi);
int emix_ctx_download(emix_ctx *ctx, double *um, double *phi);

/* Device pointers of the state (um: 5 fields, phi: 1 field). */
int emix_ctx_state(emix_ctx *ctx, double **um, double **phi);

/* Advance nsteps RK3 steps on the device, asynchronously on the context
 * stream.  use_graph = 1 replays a captured CUDA graph of one step (and one
 * of the filter, when it is on). */
int emix_step(emix_ctx *ctx, int nsteps, int use_graph);

/* Steps taken by the context so far (starts at 0; the filter runs after the
 * steps whose index is a multiple of filter_every).  Settable for restarts. */
int emix_ctx_get_step_index(emix_ctx *ctx, long *index);
int emix_ctx_set_step_index(emix_ctx *ctx, long index);

/* The impeller's clock: time of the next step = t0 + k*dt with k the steps
 * taken since the clock was last set (emix_ctx_set_time sets t0 and k = 0). */
int emix_ctx_set_time(emix_ctx *ctx, double t0);
int emix_ctx_get_time(emix_ctx *ctx, double *t);

/* End-to-end form: copy um/phi from host, advance nsteps, copy back;
 * synchronous.  The uploads (phi and um by z-slabs, on a second stream)
 * overlap the first step's primitive variables, ghost padding and first
 * level-set stage; the copies back overlap the last step where its results
 * are final early (phi after the last level-set stage, um by z-slabs of the
 * last RK update); page-locked host buffers let them run asynchronously.  The
 * values are those of emix_step, bit for bit.  Returns EMIX_ERR_TIMEOUT when
 * a level-set stage block or a y/z pencil block gave up waiting for its TMA
 * copies during the call (its cells are then unwritten).  emix_step and the
 * other device-pointer forms return before their kernels finish: their
 * callers poll emix_weno_tma_timeouts and emix_pencil_tma_timeouts instead. */
int emix_step_host(emix_ctx *ctx, double *um, double *phi, int nsteps);

/* Number of kernel launches one step issues (for accounting; the records
 * that run as one launch counted once). */
int emix_ctx_launches_per_step(emix_ctx *ctx);

/* Bytes of device memory the context holds. */
long long emix_ctx_device_bytes(emix_ctx *ctx);

/* Per-kernel timing: run nsteps steps (no graph) with CUDA events around
 * every launch on the context stream; ms[k] and launches[k] receive the
 * summed duration and launch count of kernel class k
 * (k < emix_profile_class_count(), named by emix_profile_class_name). */
int emix_ctx_profile(emix_ctx *ctx, int nsteps, double *ms, int *launches);
int emix_profile_class_count(void);
const char *emix_profile_class_name(int cls);

/* ========================================================================
 * Batched ensemble: many independent grids of uneven size in one launch
 * per kernel position (no counterpart in the reference, which advances one
 * grid per process)
 * ======================================================================== */

typedef struct emix_batch emix_batch;

/* One context per params[g]; all grids must share level_set, ls_ghost and
 * sgs_model (their steps then issue the same kernel sequence). */
int emix_batch_create(int ngrid, const emix_params *params, emix_batch **out);
int emix_batch_destroy(emix_batch *b);

/* Member context g, for emix_ctx_set_static / _upload / _download / _state. */
int emix_batch_grid(emix_batch *b, int g, emix_ctx **ctx);

int emix_batch_set_stream(emix_batch *b, void *stream);

/* Advance every grid nsteps RK3 steps: one persistent launch per kernel
 * position over the work of all grids; use_graph = 1 replays a captured
 * graph of one batched step. */
int emix_batch_step(emix_batch *b, int nsteps, int use_graph);

/* The same steps issued grid by grid (each grid's own launches), the
 * comparison point for the batched form. */
int emix_batch_step_per_grid(emix_batch *b, int nsteps, int use_graph);

/* Work-list granularity of the batched launches: cells per thread of the
 * pointwise items (x256 per item), threads per y/z pencil block (32, 64 or
 * 128) and resident CTAs per SM of the persistent pointwise grids (0: one
 * CTA per pointwise item instead of a persistent grid). */
int emix_batch_set_tuning(emix_batch *b, int cells_per_thread, int yz_block, int ctas_per_sm);
int emix_batch_get_tuning(emix_batch *b, int *cells_per_thread, int *yz_block, int *ctas_per_sm);

/* y/z pencil positions of the batched step by parallel cyclic reduction +
 * Thomas (emix_deriv_pcr_dev) with steps = 2..5 PCR steps, or 0 (default)
 * by one Thomas sweep per pencil.  A position whose pencils exceed 160 rows
 * in any grid keeps the Thomas sweep; emix_batch_pcr_positions counts the
 * positions that run by PCR.  The gradients' y and z positions then run as
 * two launches. */
int emix_batch_set_pcr(emix_batch *b, int steps);

/* Concurrency inside a batched step, as emix_ctx_set_overlap: bit 0 the
 * level-set positions, bit 1 the x-gradient positions on a second stream
 * (3, the default: both; 0: one stream).  The same values bit for bit in
 * every mode. */
int emix_batch_set_overlap(emix_batch *b, int mode);
int emix_batch_get_pcr(emix_batch *b, int *steps);
int emix_batch_pcr_positions(emix_batch *b, int *count);

/* Autotuner: times every candidate launch shape (cells per pointwise item,
 * y/z block width, resident CTAs per SM) over nsteps batched steps with one
 * Thomas sweep per pencil, then the best of them with 2..5 PCR steps in the
 * y/z positions, and keeps the fastest (advances the state; re-upload it
 * afterwards).  best_ms (may be NULL) receives the best ms per step. */
int emix_batch_autotune(emix_batch *b, int nsteps, double *best_ms);

/* ms per step the last emix_batch_autotune measured: ms[0] the best shape
 * with Thomas sweeps, ms[k] (k = 2..5) the same shape with k PCR steps; -1
 * where not measured.  ms holds 6 values. */
int emix_batch_autotune_pcr_ms(emix_batch *b, double *ms);

/* Diagnostic: measured FP64 fused-multiply-add throughput of the current
 * device in lane operations per second (a short dependent-chain kernel). */
int emix_fp64_peak(double *lane_ops_per_s);

/* Diagnostic with no counterpart in the reference: the block width (32, 64
 * or 128 threads, one pencil each) of the single-grid y/z pencil launches
 * issued afterwards; 0 (default) picks the width that idles the fewest lanes
 * of the last block of a row.  Process-wide; graphs keep the width they were
 * captured with. */
int emix_pencil_set_yz_block(int threads);

/* Diagnostic with no counterpart in the reference: the kernels' own
 * reciprocal and square-root routines (third-order steps from
 * single-precision seeds) beside CUDA's 1.0/x, sqrt(x) and 1.0/sqrt(x) on the
 * same n arguments x, in one kernel.  out[6*n]: component k = 0..5 holds
 * rcp_fast, 1.0/x, sqrt_fast, sqrt, rsqrt_fast, 1.0/sqrt.  Device pointers,
 * asynchronous on stream. */
int emix_math_selftest_dev(const double *x, double *out, long n, void *stream);

/* ========================================================================
 * Gradient of a tank objective through the RK3 step (hand-written adjoint;
 * no counterpart in the reference)
 * ======================================================================== */

/* J = w_ke * sum_{r_in <= r <= r_out} dV |u|^2 / 2
 *   + w_if * sum dV delta_eps(phi) |grad phi|
 * over the state after the forward steps; r = sqrt(x^2 + y^2), dV =
 * jbn(10) hx hy hz, delta_eps the cosine-smoothed delta of half-width eps,
 * grad phi by central differences (one-sided at the walls) times the diagonal
 * metric. */
typedef struct emix_objective {
    double r_in, r_out, eps, w_ke, w_if;
} emix_objective;

typedef struct emix_adj emix_adj;

/* An adjoint of `nsteps` steps of ctx with a checkpoint every `every` steps
 * (1 = every step; larger values trade recomputation for memory; the reverse
 * sweep recomputes each step once with its tape).  every = 0: the forward
 * pass keeps every step's tape (72 fields, the level-set stages' 3 padded
 * inputs and the impeller clock per step) and the reverse sweep recomputes
 * nothing, for runs whose tapes fit in HBM.  Covers the tank step: level set
 * on, Smagorinsky (or no SGS), impeller on, no filter. */
int emix_adj_create(emix_ctx *ctx, int nsteps, int every, const emix_objective *obj,
                    emix_adj **adj);
int emix_adj_destroy(emix_adj *adj);
int emix_adj_device_bytes(emix_adj *adj, size_t *bytes);

/* 1 (default): the taped forward steps copy their tapes and run the
 * level-set stages on the context's second stream, overlapped with the
 * flow's kernels; 0: everything on the compute stream.  The same values bit
 * for bit either way. */
int emix_adj_set_overlap(emix_adj *adj, int on);

/* Run nsteps from the context's current state, keeping checkpoints; J out. */
int emix_adj_forward(emix_adj *adj, double *J);

/* Reverse sweep after emix_adj_forward: dJ[0] = dJ/d(impeller omega),
 * dJ[1] = dJ/dCs.  Leaves the context at the forward pass's final state. */
int emix_adj_backward(emix_adj *adj, double *dJ);

/* dJ/d(initial um[5]) and dJ/d(initial phi), device pointers (after backward). */
int emix_adj_state_gradient(emix_adj *adj, double *lum, double *lphi);

/* Change the impeller angular velocity and the Smagorinsky constant of a
 * context (the plan is rebuilt; captured graphs are dropped). */
int emix_ctx_set_forcing(emix_ctx *ctx, double omega, double cs);

/* ========================================================================
 * Checkpoint files of the reference (Fortran unformatted sequential records:
 * 4-byte length markers around each record, 4-byte integers, 8-byte reals;
 * records of 2^31 bytes or more as signed subrecords).  Host buffers.
 * ======================================================================== */

/* field_SS.NNN of GRAVA (solver/gravar_incomp.f90:19-34): nd | nx ny nz |
 * u | v | w | temp | pres; u holds the three velocity fields. */
int emix_write_field(const char *path, int nd, int nx, int ny, int nz, const double *u,
                     const double *temp, const double *pres);
/* leer_campos (solver/leer_incomp.f90:65-95): fails on a different nd or size. */
int emix_read_field(const char *path, int nd, int nx, int ny, int nz, double *u, double *temp,
                    double *pres);
/* time_SS.NNN: dto, it (gravar_incomp.f90:36-40). */
int emix_write_time(const char *path, double dto, int it);
int emix_read_time(const char *path, double *dto, int *it);
/* One record of n reals (impellermask_SS.NNN, gravar_incomp.f90:42-46). */
int emix_write_array(const char *path, const double *a, long n);
int emix_read_array(const char *path, double *a, long n);
/* sobject.field: nx ny nz | sobject (leer_incomp.f90:99-106). */
int emix_read_sobject(const char *path, int nx, int ny, int nz, double *sobject);

#ifdef __cplusplus
}
#endif
#endif /* EMIX_GB300_H */
