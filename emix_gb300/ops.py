"""Python mirror of the reference's operator interface over the C ABI.

Function names and argument meaning follow the reference's Fortran -> C
boundary (``cudaDeriv``, ``cuDivergence``; solver/deriv_vel_cuda.f90:19-39,
solver/divergencia_cuda.f90:21-42) and its level-set driver
(``cuAdvectLsJB``, src/LevelSet/lsTransportEc.cu:201-418).  Host arrays are
numpy float64, C-ordered as ``(ncomp, nz, ny, nx)`` -- the same bytes as the
Fortran ``(nx, ny, nz, ncomp)`` arrays.  Device forms take torch CUDA tensors
and launch on torch's current stream.  Errors raise :class:`EmixError`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import EmixError, EmixParams, check, i3  # noqa: F401
from .fields import SCHEME_A, SCHEME_B, SCHEME_BPER, SCHEME_C  # noqa: F401

SGS_NONE, SGS_SMAGORINSKY, SGS_STRUCTURE = 0, 1, 2


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous float64")
        return a.ctypes.data
    if a is None:
        return None
    # torch tensor
    if str(a.dtype) != "torch.float64" or not a.is_contiguous():
        raise ValueError("tensors must be contiguous float64")
    return a.data_ptr()


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dims(a):
    nz, ny, nx = a.shape[-3:]
    return nx, ny, nz


def _schemes(s):
    if isinstance(s, int):
        s = (s, s, s)
    return i3(*s)


# --------------------------------------------------------------------------
# host-pointer forms
# --------------------------------------------------------------------------
def cudaDeriv(vel: np.ndarray, temp: np.ndarray, h, schemes=SCHEME_C):
    """Velocity and temperature gradients in computational coordinates.

    vel (3, nz, ny, nx), temp (nz, ny, nx), h = (hx, hy, hz).  Returns
    dvel (9, ...) ordered d/dx(u,v,w), d/dy(u,v,w), d/dz(u,v,w) and
    dtemp (3, ...), as solver/cuDeriv.cu:629-644."""
    lib = _lib.load()
    nx, ny, nz = _dims(temp)
    dvel = np.empty((9, nz, ny, nx))
    dtemp = np.empty((3, nz, ny, nx))
    rc = lib.emix_cudaDeriv(_schemes(schemes), _ptr(dvel), _ptr(dtemp), _ptr(vel), _ptr(temp),
                            h[0], h[1], h[2], nx, ny, nz)
    check(rc, "emix_cudaDeriv")
    return dvel, dtemp


def cudaDeriv_legacy(dvel, dtemp, vel, temp, amut, dxyzsgd, jbn, dx, dy, dz, nx, ny, nz):
    """The reference symbol itself (void, prints on error)."""
    lib = _lib.load()
    lib.cudaDeriv(_ptr(dvel), _ptr(dtemp), _ptr(vel), _ptr(temp), _ptr(amut), _ptr(dxyzsgd),
                  _ptr(jbn), dx, dy, dz, nx, ny, nz)


def cuDivergence(e, f, g, ev, fv, gv, jbn, h, schemes=SCHEME_C):
    """rs, rsv of solver/cuDivergence.cu:107-189 (host arrays)."""
    lib = _lib.load()
    nx, ny, nz = _dims(e)
    rs = np.empty((nz, ny, nx))
    rsv = np.empty((nz, ny, nx))
    rc = lib.emix_cuDivergence(_schemes(schemes), _ptr(rs), _ptr(rsv), _ptr(e), _ptr(f), _ptr(g),
                               _ptr(ev), _ptr(fv), _ptr(gv), _ptr(jbn), h[0], h[1], h[2],
                               nx, ny, nz)
    check(rc, "emix_cuDivergence")
    return rs, rsv


def cuDivergence_legacy(rs, rsv, e, f, g, ev, fv, gv, jbn, dx, dy, dz, nx, ny, nz):
    lib = _lib.load()
    lib.cuDivergence(_ptr(rs), _ptr(rsv), _ptr(e), _ptr(f), _ptr(g), _ptr(ev), _ptr(fv),
                     _ptr(gv), _ptr(jbn), dx, dy, dz, nx, ny, nz)


def set_legacy_scheme(scheme: int):
    check(_lib.load().emix_set_legacy_scheme(scheme), "emix_set_legacy_scheme")


def weno5_advect(phi: np.ndarray, vel: np.ndarray, jbn: np.ndarray, h, dt: float,
                 ref_bugs: int = 0) -> np.ndarray:
    """One WENO5 TVD-RK3 step on ghost-padded host arrays (cuAdvectLsJB).
    Returns the new phi; the input is not modified."""
    lib = _lib.load()
    nx, ny, nz = _dims(phi)
    out = np.array(phi, dtype=np.float64, copy=True, order="C")
    rc = lib.emix_weno5_advect(_ptr(out), _ptr(vel), _ptr(jbn), h[0], h[1], h[2], dt,
                               nx, ny, nz, ref_bugs)
    check(rc, "emix_weno5_advect")
    return out


def advect_extrapolate(press: np.ndarray, jbn: np.ndarray, sobject: np.ndarray, delta,
                       deltamin: float) -> np.ndarray:
    """advect_CUDA as the reference links it: the pressure extrapolated into
    the solid object (sobject > 0).  delta = (deltaX, deltaY, deltaZ) as the
    Fortran passes them (the spacings h).  Returns the new pressure."""
    lib = _lib.load()
    nx, ny, nz = _dims(press)
    out = np.array(press, dtype=np.float64, copy=True, order="C")
    rc = lib.emix_advect_extrapolate(_ptr(out), _ptr(np.ascontiguousarray(jbn)),
                                     _ptr(np.ascontiguousarray(sobject)), delta[0], delta[1],
                                     delta[2], nx, ny, nz, deltamin)
    check(rc, "emix_advect_extrapolate")
    return out


def advect_CUDA_legacy(press: np.ndarray, jbn: np.ndarray, sobject: np.ndarray, delta,
                       deltamin: float) -> None:
    """The reference's void symbol advect_CUDA, in place on press."""
    lib = _lib.load()
    nx, ny, nz = _dims(press)
    assert press.dtype == np.float64 and press.flags["C_CONTIGUOUS"]
    lib.advect_CUDA(_ptr(press), _ptr(np.ascontiguousarray(jbn)), _ptr(np.ascontiguousarray(sobject)),
                    delta[0], delta[1], delta[2], nx, ny, nz, deltamin)


# --------------------------------------------------------------------------
# device forms (torch tensors)
# --------------------------------------------------------------------------
def deriv_dev(x, axis: int, h: float, scheme=SCHEME_C):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(x)
    nf = 1 if x.dim() == 3 else x.shape[0]
    out = torch.empty_like(x)
    check(lib.emix_deriv_dev(scheme, axis, nf, _ptr(out), _ptr(x), h, nx, ny, nz, _stream()),
          "emix_deriv_dev")
    return out


def deriv_pcr_dev(x, axis: int, h: float, steps: int, scheme=SCHEME_C):
    """deriv_dev along y or z by parallel cyclic reduction (steps 2..5) +
    Thomas (emix_deriv_pcr_dev)."""
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(x)
    nf = 1 if x.dim() == 3 else x.shape[0]
    out = torch.empty_like(x)
    check(lib.emix_deriv_pcr_dev(scheme, axis, nf, _ptr(out), _ptr(x), h, steps, nx, ny, nz, _stream()),
          "emix_deriv_pcr_dev")
    return out


def cudaDeriv_dev(vel, temp, h, schemes=SCHEME_C):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(vel)
    dvel = torch.empty((9, nz, ny, nx), dtype=torch.float64, device=vel.device)
    dtemp = None if temp is None else torch.empty((3, nz, ny, nx), dtype=torch.float64,
                                                  device=vel.device)
    check(lib.emix_cudaDeriv_dev(_schemes(schemes), _ptr(dvel), _ptr(dtemp), _ptr(vel),
                                 _ptr(temp), h[0], h[1], h[2], nx, ny, nz, _stream()),
          "emix_cudaDeriv_dev")
    return dvel, dtemp


def cuDivergence_dev(e, f, g, ev, fv, gv, jbn, h, schemes=SCHEME_C):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(e)
    rs = torch.empty_like(e)
    rsv = torch.empty_like(e)
    check(lib.emix_cuDivergence_dev(_schemes(schemes), _ptr(rs), _ptr(rsv), _ptr(e), _ptr(f),
                                    _ptr(g), _ptr(ev), _ptr(fv), _ptr(gv), _ptr(jbn),
                                    h[0], h[1], h[2], nx, ny, nz, _stream()),
          "emix_cuDivergence_dev")
    return rs, rsv


def flux_dev(neq, um, u, pres, dvel, jbn, vis):
    """flujos(neq): returns (e, f, g, ev, fv, gv) as device tensors."""
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(pres)
    out = [torch.empty_like(pres) for _ in range(6)]
    check(lib.emix_flux_dev(neq, *[_ptr(o) for o in out], _ptr(um), _ptr(u), _ptr(pres),
                            _ptr(dvel), _ptr(jbn), _ptr(vis), nx, ny, nz, _stream()),
          "emix_flux_dev")
    return tuple(out)


def sgs_setup_dev(xyz):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(xyz)
    dxyz = torch.empty(xyz.shape[1:], dtype=torch.float64, device=xyz.device)
    ratios = torch.empty((6,) + tuple(xyz.shape[1:]), dtype=torch.float64, device=xyz.device)
    check(lib.emix_sgs_setup_dev(_ptr(xyz), _ptr(dxyz), _ptr(ratios), nx, ny, nz, _stream()),
          "emix_sgs_setup_dev")
    return dxyz, ratios


def sgs_viscosity_dev(model, coef, c4, u, dvel, jbn, dxyzsgd, ratios=None):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(dxyzsgd)
    amut = torch.empty_like(dxyzsgd)
    vis = torch.empty_like(dxyzsgd)
    check(lib.emix_sgs_viscosity_dev(model, coef, c4, _ptr(u), _ptr(dvel), _ptr(jbn),
                                     _ptr(dxyzsgd), _ptr(ratios), _ptr(amut), _ptr(vis),
                                     nx, ny, nz, _stream()),
          "emix_sgs_viscosity_dev")
    return amut, vis


def weno5_advect_dev(phi, vel, jbn, h, dt, ref_bugs=0):
    """In-place WENO5 TVD-RK3 step on padded device tensors."""
    lib = _lib.load()
    nx, ny, nz = _dims(phi)
    check(lib.emix_weno5_advect_dev(_ptr(phi), _ptr(vel), _ptr(jbn), h[0], h[1], h[2], dt,
                                    nx, ny, nz, ref_bugs, _stream()),
          "emix_weno5_advect_dev")
    return phi


def impeller_force_dev(um, xyz, imp, t):
    """The impeller forcing at time t on device tensors (um in place); returns the mask."""
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(um)
    c = _lib.EmixImpeller()
    c.on = 1
    for f, _ in _lib.EmixImpeller._fields_[1:]:
        setattr(c, f, getattr(imp, f))
    mask = torch.empty_like(um[0])
    check(lib.emix_impeller_force_dev(_ptr(um), _ptr(xyz), C.byref(c), t, nx, ny, nz, _ptr(mask),
                                      _stream()), "emix_impeller_force_dev")
    return mask


def deriv_t_dev(y, axis: int, h: float, scheme=SCHEME_C, out=None, tma=False):
    """D^T y along `axis` (the transpose of deriv_dev); out += D^T y when out
    is given.  tma: the y/z form with its rows staged by TMA (the adjoint's)."""
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(y)
    nf = 1 if y.dim() == 3 else y.shape[0]
    acc = out is not None
    if out is None:
        out = torch.empty_like(y)
    fn, name = ((lib.emix_deriv_t_tma_dev, "emix_deriv_t_tma_dev") if tma
                else (lib.emix_deriv_t_dev, "emix_deriv_t_dev"))
    check(fn(scheme, axis, nf, _ptr(out), _ptr(y), h, nx, ny, nz, int(acc), _stream()), name)
    return out


def reinit_dev(phi, jbn, dmins, delta, g, deltamin, iters=10, ref_bugs=0):
    """Sussman reinitialisation (cuReinitLsJB) of a padded level set, in place."""
    lib = _lib.load()
    nx, ny, nz = _dims(phi)
    check(lib.emix_reinit_dev(_ptr(phi), _ptr(jbn), _ptr(dmins), delta[0], delta[1], delta[2],
                              nx, ny, nz, g, deltamin, iters, ref_bugs, _stream()), "emix_reinit_dev")
    return phi


def filtrado_dev(um, jbn, cfilt):
    """filtrado (x, y, z compact filter of the 5 fields) in place on device tensors."""
    lib = _lib.load()
    nx, ny, nz = _dims(um)
    check(lib.emix_filtrado_dev(_ptr(um), _ptr(jbn), cfilt, nx, ny, nz, _stream()), "emix_filtrado_dev")
    return um


def filter_dev(f, jbn, cfilt, axis, zrows=0):
    """One filter pass along `axis` over the fields of f (3-D or stacked 4-D), in place."""
    lib = _lib.load()
    nx, ny, nz = _dims(f)
    nf = 1 if f.dim() == 3 else f.shape[0]
    check(lib.emix_filter_dev(_ptr(f), nf, _ptr(jbn), cfilt, axis, zrows, nx, ny, nz, _stream()),
          "emix_filter_dev")
    return f


def advect_extrapolate_dev(press, jbn, sobject, delta, deltamin):
    """advect_CUDA on device tensors, in place on press."""
    lib = _lib.load()
    nx, ny, nz = _dims(press)
    check(lib.emix_advect_extrapolate_dev(_ptr(press), _ptr(jbn), _ptr(sobject), delta[0], delta[1],
                                          delta[2], nx, ny, nz, deltamin, _stream()),
          "emix_advect_extrapolate_dev")
    return press


def extrapolate_dev(ext, phiS, jbn, delta, dtext, flag=1, iters=10):
    """cuExtrapolation on the 5-layer mirrored padding of device tensors, in
    place on ext."""
    lib = _lib.load()
    nx, ny, nz = _dims(ext)
    check(lib.emix_extrapolate_dev(_ptr(ext), _ptr(phiS), _ptr(jbn), delta[0], delta[1], delta[2],
                                   nx, ny, nz, dtext, flag, iters, _stream()),
          "emix_extrapolate_dev")
    return ext


def weno5_advect_dev_noalloc(phi, vel, jbn, h, dt, ref_bugs=0):
    """In-place WENO5 TVD-RK3 step on padded device tensors that allocates no
    device memory: the stage scratch is a fixed 16 MiB array inside the
    library, so the padded grid may hold at most 1048576 cells.  For callers
    that cannot let a library call cudaMalloc.  Calls that overlap on the GPU
    share (and race on) that array."""
    lib = _lib.load()
    nx, ny, nz = _dims(phi)
    check(lib.emix_weno5_advect_dev_noalloc(_ptr(phi), _ptr(vel), _ptr(jbn), h[0], h[1], h[2], dt,
                                            nx, ny, nz, ref_bugs, _stream()),
          "emix_weno5_advect_dev_noalloc")
    return phi


def bc_walls_dev(um):
    """frontera_z/y/x_val in place on a (5, nz, ny, nx) device tensor."""
    lib = _lib.load()
    nx, ny, nz = _dims(um)
    check(lib.emix_bc_walls_dev(_ptr(um), nx, ny, nz, _stream()), "emix_bc_walls_dev")
    return um


def cfl_dev(u, xyz, mach):
    """CFL number of TSTEP (maximum over cells), from device tensors."""
    lib = _lib.load()
    nx, ny, nz = _dims(u)
    out = C.c_double()
    check(lib.emix_cfl_dev(_ptr(u), _ptr(xyz), mach, nx, ny, nz, C.byref(out), _stream()),
          "emix_cfl_dev")
    return out.value


def tstep_dt(cfla, olddt, cfl=0.3):
    out = C.c_double()
    check(_lib.load().emix_tstep_dt(cfla, olddt, cfl, C.byref(out)), "emix_tstep_dt")
    return out.value


def metrics_dev(xyz, h, scheme=SCHEME_A):
    """JACOBEANO: jbn (11, nz, ny, nx) from coordinates (3, nz, ny, nx) on the device."""
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(xyz)
    jbn = torch.empty((11, nz, ny, nx), dtype=torch.float64, device=xyz.device)
    check(lib.emix_metrics_dev(_ptr(xyz), _ptr(jbn), scheme, h[0], h[1], h[2], nx, ny, nz,
                               _stream()), "emix_metrics_dev")
    return jbn


def ghost_pad_dev(val, g, direction=1.0):
    import torch
    lib = _lib.load()
    nx, ny, nz = _dims(val)
    out = torch.empty((nz + 2 * g, ny + 2 * g, nx + 2 * g), dtype=torch.float64, device=val.device)
    check(lib.emix_ghost_pad_dev(_ptr(out), _ptr(val), g, direction, nx, ny, nz, _stream()),
          "emix_ghost_pad_dev")
    return out


def ghost_unpad_dev(ghost, g):
    import torch
    lib = _lib.load()
    nzg, nyg, nxg = ghost.shape
    nx, ny, nz = nxg - 2 * g, nyg - 2 * g, nzg - 2 * g
    out = torch.empty((nz, ny, nx), dtype=torch.float64, device=ghost.device)
    check(lib.emix_ghost_unpad_dev(_ptr(out), _ptr(ghost), g, nx, ny, nz, _stream()),
          "emix_ghost_unpad_dev")
    return out


def pencil_tma_timeouts() -> int:
    """Pencil blocks that gave up waiting for a TMA row copy (0 in a correct run)."""
    out = C.c_int()
    check(_lib.load().emix_pencil_tma_timeouts(C.byref(out)), "emix_pencil_tma_timeouts")
    return out.value


def weno_tma_timeouts() -> int:
    """Level-set stage blocks that gave up waiting for a TMA plane copy (0 in a correct run)."""
    out = C.c_int()
    check(_lib.load().emix_weno_tma_timeouts(C.byref(out)), "emix_weno_tma_timeouts")
    return out.value


def fp64_peak() -> float:
    """Measured FP64 FMA lane-operations per second of the current device."""
    v = C.c_double()
    check(_lib.load().emix_fp64_peak(C.byref(v)), "emix_fp64_peak")
    return v.value


# --------------------------------------------------------------------------
# device-resident RK3 step
# --------------------------------------------------------------------------
class Context:
    """One grid resident in device memory; wraps ``emix_ctx``."""

    def __init__(self, workload=None, *, params: EmixParams | None = None, level_set=True,
                 ref_bugs=0, ls_ghost=5, bc_walls=0, filter_every=0, cfilt=0.0):
        lib = _lib.load()
        if params is None:
            params = _params_of(workload, level_set, ref_bugs, ls_ghost, bc_walls, filter_every, cfilt)
        self.params = params
        self._h = C.c_void_p()
        check(lib.emix_ctx_create(C.byref(params), C.byref(self._h)), "emix_ctx_create")
        self.lib = lib
        if workload is not None:
            self.set_static(workload.jbn, workload.mask, workload.grid.coords())
            self.upload(workload.um, workload.phi if level_set else None)

    @property
    def shape(self):
        p = self.params
        return (p.nz, p.ny, p.nx)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        check(self.lib.emix_ctx_set_stream(self._h, C.c_void_p(stream_ptr)), "emix_ctx_set_stream")

    def set_static(self, jbn, mask, xyz):
        jbn = np.ascontiguousarray(jbn, dtype=np.float64)
        mask = np.ascontiguousarray(mask, dtype=np.float64)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        check(self.lib.emix_ctx_set_static(self._h, _ptr(jbn), _ptr(mask), _ptr(xyz)),
              "emix_ctx_set_static")

    def upload(self, um, phi=None):
        um = np.ascontiguousarray(um, dtype=np.float64)
        phi = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        check(self.lib.emix_ctx_upload(self._h, _ptr(um), _ptr(phi)), "emix_ctx_upload")

    def download(self):
        p = self.params
        um = np.empty((5, p.nz, p.ny, p.nx))
        phi = np.empty((p.nz, p.ny, p.nx)) if p.level_set else None
        check(self.lib.emix_ctx_download(self._h, _ptr(um), _ptr(phi)), "emix_ctx_download")
        return um, phi

    def state_ptrs(self):
        a, b = C.c_void_p(), C.c_void_p()
        check(self.lib.emix_ctx_state(self._h, C.byref(a), C.byref(b)), "emix_ctx_state")
        return a.value, b.value

    def step(self, nsteps=1, use_graph=False):
        check(self.lib.emix_step(self._h, nsteps, 1 if use_graph else 0), "emix_step")

    def set_overlap(self, on):
        """Concurrency inside a step: False/0 one stream; True/1 the level-set
        stages on a second stream; 2 the x gradients on it; 3 both."""
        mode = int(on) if not isinstance(on, bool) else (1 if on else 0)
        check(self.lib.emix_ctx_set_overlap(self._h, mode), "emix_ctx_set_overlap")

    def set_fusion(self, on: bool):
        """Run the gradients' y and z passes, and Smagorinsky with the fluxes,
        as one launch each (default) or every operator alone; the values are
        bitwise the same."""
        check(self.lib.emix_ctx_set_fusion(self._h, 1 if on else 0), "emix_ctx_set_fusion")

    def set_tma(self, on: bool):
        """Plane tiles of the level-set stages by TMA copies (default) or by
        register-staged loads; the results are bitwise the same."""
        check(self.lib.emix_ctx_set_tma(self._h, 1 if on else 0), "emix_ctx_set_tma")

    def tma_stages(self) -> int:
        return int(self.lib.emix_ctx_tma_stages(self._h))

    def set_pencil_tma(self, on: bool):
        """The divergence's y/z passes with their rows staged by TMA (same values)."""
        check(self.lib.emix_ctx_set_pencil_tma(self._h, 1 if on else 0), "emix_ctx_set_pencil_tma")

    def pencil_tma_launches(self) -> int:
        return int(self.lib.emix_ctx_pencil_tma_launches(self._h))

    @property
    def time(self) -> float:
        v = C.c_double()
        check(self.lib.emix_ctx_get_time(self._h, C.byref(v)), "emix_ctx_get_time")
        return v.value

    @time.setter
    def time(self, t0: float):
        check(self.lib.emix_ctx_set_time(self._h, float(t0)), "emix_ctx_set_time")

    @property
    def step_index(self) -> int:
        v = C.c_long()
        check(self.lib.emix_ctx_get_step_index(self._h, C.byref(v)), "emix_ctx_get_step_index")
        return v.value

    @step_index.setter
    def step_index(self, index: int):
        check(self.lib.emix_ctx_set_step_index(self._h, int(index)), "emix_ctx_set_step_index")

    def step_host(self, um, phi, nsteps=1):
        check(self.lib.emix_step_host(self._h, _ptr(um), _ptr(phi), nsteps), "emix_step_host")

    def profile(self, nsteps=1):
        """Per-kernel-class device time: {name: (total_ms, launches)} over nsteps
        steps, from CUDA events on the context stream."""
        k = self.lib.emix_profile_class_count()
        ms = (C.c_double * k)()
        nl = (C.c_int * k)()
        check(self.lib.emix_ctx_profile(self._h, nsteps, ms, nl), "emix_ctx_profile")
        return {self.lib.emix_profile_class_name(i).decode(): (ms[i], nl[i]) for i in range(k)}

    def launches_per_step(self):
        return self.lib.emix_ctx_launches_per_step(self._h)

    def device_bytes(self):
        return self.lib.emix_ctx_device_bytes(self._h)

    def close(self):
        if self._h:
            self.lib.emix_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _params_of(w, level_set=True, ref_bugs=0, ls_ghost=5, bc_walls=0, filter_every=0,
               cfilt=0.0) -> EmixParams:
    g = w.grid
    p = EmixParams()
    p.nx, p.ny, p.nz = g.nx, g.ny, g.nz
    for a in range(3):
        p.scheme[a] = w.schemes[a]
        p.h[a] = g.h(a)
    p.sgs_model = w.sgs_model
    p.cs = w.cs
    p.amu0 = w.amu0
    p.c4 = 1.0 / w.reynolds
    p.mach = w.mach
    p.dt = w.dt
    p.level_set = 1 if level_set else 0
    p.ls_ghost = ls_ghost
    p.ref_bugs = ref_bugs
    p.bc_walls = bc_walls
    p.filter_every = filter_every
    p.cfilt = cfilt
    imp = getattr(w, "impeller", None)
    if imp is not None:
        p.imp.on = 1
        for f, _ in _lib.EmixImpeller._fields_[1:]:
            setattr(p.imp, f, getattr(imp, f))
    p.t0 = getattr(w, "t0", 0.0)
    return p


class Batch:
    """Independent grids of uneven size advanced together (``emix_batch``)."""

    def __init__(self, workloads, level_set=True, ref_bugs=0, ls_ghost=5, bc_walls=0):
        lib = _lib.load()
        self.lib = lib
        self.workloads = list(workloads)
        arr = (EmixParams * len(self.workloads))(
            *[_params_of(w, level_set, ref_bugs, ls_ghost, bc_walls) for w in self.workloads])
        self._h = C.c_void_p()
        check(lib.emix_batch_create(len(self.workloads), arr, C.byref(self._h)), "emix_batch_create")
        self.level_set = level_set
        self.ctx = []
        for g, w in enumerate(self.workloads):
            h = C.c_void_p()
            check(lib.emix_batch_grid(self._h, g, C.byref(h)), "emix_batch_grid")
            self.ctx.append(h)
            jbn = np.ascontiguousarray(w.jbn)
            mask = np.ascontiguousarray(w.mask)
            xyz = np.ascontiguousarray(w.grid.coords())
            check(lib.emix_ctx_set_static(h, _ptr(jbn), _ptr(mask), _ptr(xyz)), "emix_ctx_set_static")
        self.upload()

    @property
    def ncell(self):
        return sum(w.grid.ncell for w in self.workloads)

    def upload(self):
        """Initial state of every grid, and the impeller clocks back to t0."""
        for h, w in zip(self.ctx, self.workloads):
            um = np.ascontiguousarray(w.um)
            phi = np.ascontiguousarray(w.phi) if self.level_set else None
            check(self.lib.emix_ctx_upload(h, _ptr(um), _ptr(phi)), "emix_ctx_upload")
            if getattr(w, "impeller", None) is not None:
                check(self.lib.emix_ctx_set_time(h, getattr(w, "t0", 0.0)), "emix_ctx_set_time")

    def download(self, g):
        w = self.workloads[g]
        nz, ny, nx = w.grid.shape
        um = np.empty((5, nz, ny, nx))
        phi = np.empty((nz, ny, nx)) if self.level_set else None
        check(self.lib.emix_ctx_download(self.ctx[g], _ptr(um), _ptr(phi)), "emix_ctx_download")
        return um, phi

    def set_stream(self, stream_ptr):
        check(self.lib.emix_batch_set_stream(self._h, C.c_void_p(stream_ptr)), "emix_batch_set_stream")

    def step(self, nsteps=1, use_graph=False):
        check(self.lib.emix_batch_step(self._h, nsteps, 1 if use_graph else 0), "emix_batch_step")

    def step_per_grid(self, nsteps=1, use_graph=False):
        check(self.lib.emix_batch_step_per_grid(self._h, nsteps, 1 if use_graph else 0),
              "emix_batch_step_per_grid")

    def set_tuning(self, cells_per_thread, yz_block, ctas_per_sm):
        check(self.lib.emix_batch_set_tuning(self._h, cells_per_thread, yz_block, ctas_per_sm),
              "emix_batch_set_tuning")

    def tuning(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(self.lib.emix_batch_get_tuning(self._h, C.byref(a), C.byref(b), C.byref(c)),
              "emix_batch_get_tuning")
        return a.value, b.value, c.value

    def autotune(self, nsteps=2):
        ms = C.c_double()
        check(self.lib.emix_batch_autotune(self._h, nsteps, C.byref(ms)), "emix_batch_autotune")
        self.upload()
        return ms.value

    def set_overlap(self, mode: int):
        """Concurrency inside a batched step: 0 one stream, bit 0 the level-set
        positions, bit 1 the x-gradient positions on a second stream (3: both)."""
        check(self.lib.emix_batch_set_overlap(self._h, int(mode)), "emix_batch_set_overlap")

    def set_pcr(self, steps: int):
        """PCR steps (2..5) of the y/z pencil positions, 0 for Thomas sweeps."""
        check(self.lib.emix_batch_set_pcr(self._h, steps), "emix_batch_set_pcr")

    def pcr(self) -> int:
        v = C.c_int()
        check(self.lib.emix_batch_get_pcr(self._h, C.byref(v)), "emix_batch_get_pcr")
        return v.value

    def pcr_positions(self) -> int:
        v = C.c_int()
        check(self.lib.emix_batch_pcr_positions(self._h, C.byref(v)), "emix_batch_pcr_positions")
        return v.value

    def autotune_pcr_ms(self):
        """{steps: ms per step} the last autotune measured (0: Thomas)."""
        ms = (C.c_double * 6)()
        check(self.lib.emix_batch_autotune_pcr_ms(self._h, ms), "emix_batch_autotune_pcr_ms")
        return {k: ms[k] for k in (0, 2, 3, 4, 5) if ms[k] >= 0}

    def close(self):
        if self._h:
            self.lib.emix_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



# --------------------------------------------------------------------------
# gradient of the tank objective (hand-written adjoint of the RK3 step)
# --------------------------------------------------------------------------
def tank_objective(workload, r_in=0.2, r_out=0.5, radius=1.0, w_ke=1.0, w_if=1.0):
    """Kinetic energy in the annulus r_in R <= r <= r_out R plus the smoothed
    interface area of the level set (delta half-width 1.5 x the largest
    spacing)."""
    g = workload.grid
    dmax = max(g.length[a] * g.h(a) for a in range(3))
    o = _lib.EmixObjective()
    o.r_in, o.r_out, o.eps = r_in * radius, r_out * radius, 1.5 * dmax
    o.w_ke, o.w_if = w_ke, w_if
    return o


class Adjoint:
    """Forward steps with checkpoints and the reverse sweep (``emix_adj``);
    every = 0 keeps every step's tape from the forward pass (no recomputation),
    for runs whose tapes fit in HBM."""

    def __init__(self, ctx: "Context", nsteps: int, every: int = 1, objective=None):
        self.lib = _lib.load()
        self.ctx = ctx
        self.objective = objective
        self._h = C.c_void_p()
        check(self.lib.emix_adj_create(ctx.handle, nsteps, every, C.byref(objective),
                                       C.byref(self._h)), "emix_adj_create")

    def forward(self) -> float:
        J = C.c_double()
        check(self.lib.emix_adj_forward(self._h, C.byref(J)), "emix_adj_forward")
        return J.value

    def backward(self):
        dJ = (C.c_double * 2)()
        check(self.lib.emix_adj_backward(self._h, dJ), "emix_adj_backward")
        return dJ[0], dJ[1]

    def state_gradient(self):
        import torch
        nz, ny, nx = self.ctx.shape
        lum = torch.empty((5, nz, ny, nx), dtype=torch.float64, device="cuda")
        lphi = torch.empty((nz, ny, nx), dtype=torch.float64, device="cuda")
        check(self.lib.emix_adj_state_gradient(self._h, _ptr(lum), _ptr(lphi)),
              "emix_adj_state_gradient")
        return lum, lphi

    def set_overlap(self, on: bool):
        """Tape copies and level-set stages of the taped forward on the
        context's second stream (default) or on the compute stream."""
        check(self.lib.emix_adj_set_overlap(self._h, int(bool(on))), "emix_adj_set_overlap")

    def device_bytes(self) -> int:
        b = C.c_size_t()
        check(self.lib.emix_adj_device_bytes(self._h, C.byref(b)), "emix_adj_device_bytes")
        return b.value

    def close(self):
        if self._h:
            self.lib.emix_adj_destroy(self._h)
            self._h = C.c_void_p()


class TankGradient:
    """J(omega, Cs) of a tank run as a torch.autograd.Function: the forward
    runs nsteps RK3 steps from the workload's initial state with the given
    impeller angular velocity and Smagorinsky constant; the backward is the
    hand-written adjoint."""

    def __init__(self, workload, nsteps, every=1, objective=None, **ctx_kw):
        self.workload = workload
        self.ctx = Context(workload, **ctx_kw)
        try:
            self.adj = Adjoint(self.ctx, nsteps, every, objective or tank_objective(workload))
        except Exception:
            # the adjoint's arena did not fit: release the context's before raising
            self.ctx.close()
            raise

    def run(self, omega: float, cs: float) -> float:
        w = self.workload
        check(self.ctx.lib.emix_ctx_set_forcing(self.ctx.handle, float(omega), float(cs)),
              "emix_ctx_set_forcing")
        self.ctx.upload(w.um, w.phi)
        self.ctx.time = getattr(w, "t0", 0.0)
        return self.adj.forward()

    def function(self):
        import torch
        runner = self

        class _J(torch.autograd.Function):
            @staticmethod
            def forward(fctx, theta):
                J = runner.run(float(theta[0]), float(theta[1]))
                return torch.tensor(J, dtype=torch.float64)

            @staticmethod
            def backward(fctx, grad):
                d = runner.adj.backward()
                return grad * torch.tensor(d, dtype=torch.float64)

        return _J.apply

    def close(self):
        self.adj.close()
        self.ctx.close()


# --------------------------------------------------------------------------
# the reference's checkpoint files (GRAVA / leer_campos)
# --------------------------------------------------------------------------
def _primitive(um, mach):
    r = um[0]
    u = np.ascontiguousarray(um[1:4] / r)
    return u, np.ascontiguousarray(um[4]), np.ascontiguousarray(r / (mach * mach))


def write_checkpoint(directory, serie, sample, um, mach, dto, it, impellermask=None, nd=5):
    """GRAVA's files for the state um (5 conserved fields): field_SS.NNN with
    u, v, w, temp, pres (varc_to_varnc), time_SS.NNN and, when given,
    impellermask_SS.NNN.  Returns the field file's path."""
    import os
    lib = _lib.load()
    nz, ny, nx = um.shape[-3:]
    u, temp, pres = _primitive(np.asarray(um, dtype=np.float64), mach)
    tag = f"{serie:02d}.{sample:03d}"
    fpath = os.path.join(directory, f"field_{tag}")
    check(lib.emix_write_field(fpath.encode(), nd, nx, ny, nz, _ptr(u), _ptr(temp), _ptr(pres)),
          "emix_write_field")
    check(lib.emix_write_time(os.path.join(directory, f"time_{tag}").encode(), float(dto), int(it)),
          "emix_write_time")
    if impellermask is not None:
        m = np.ascontiguousarray(impellermask, dtype=np.float64)
        check(lib.emix_write_array(os.path.join(directory, f"impellermask_{tag}").encode(), _ptr(m),
                                   m.size), "emix_write_array")
    return fpath


def read_field(path, shape, mach, nd=5):
    """leer_campos: the field file at `path` for a grid of shape (nz, ny, nx),
    converted back to the conserved state (varnc_to_varc)."""
    lib = _lib.load()
    nz, ny, nx = shape
    u = np.empty((3, nz, ny, nx))
    temp = np.empty((nz, ny, nx))
    pres = np.empty((nz, ny, nx))
    check(lib.emix_read_field(str(path).encode(), nd, nx, ny, nz, _ptr(u), _ptr(temp), _ptr(pres)),
          "emix_read_field")
    r = pres * mach * mach
    return np.stack([r, u[0] * r, u[1] * r, u[2] * r, temp])


def read_time(path):
    lib = _lib.load()
    d, i = C.c_double(), C.c_int()
    check(lib.emix_read_time(str(path).encode(), C.byref(d), C.byref(i)), "emix_read_time")
    return d.value, i.value
