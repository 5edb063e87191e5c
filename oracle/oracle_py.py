"""ctypes binding of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product library never
imports it.  See oracle.h for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

SCHEME_A, SCHEME_B, SCHEME_BPER, SCHEME_C = 0, 1, 2, 3
vp = C.c_void_p
i3 = C.c_int * 3


class Impeller(C.Structure):
    _fields_ = [
        ("on", C.c_int), ("nblades", C.c_int), ("omega", C.c_double), ("theta0", C.c_double),
        ("r1", C.c_double), ("r2", C.c_double), ("z1", C.c_double), ("z2", C.c_double),
        ("half_thick", C.c_double), ("hub_r", C.c_double), ("hub_z1", C.c_double),
        ("hub_z2", C.c_double), ("shaft_r", C.c_double), ("shaft_z0", C.c_double),
        ("shaft_z1", C.c_double), ("interp", C.c_int),
    ]


class StepParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("scheme", C.c_int * 3), ("h", C.c_double * 3),
        ("sgs_model", C.c_int), ("cs", C.c_double), ("amu0", C.c_double), ("c4", C.c_double),
        ("mach", C.c_double), ("dt", C.c_double),
        ("level_set", C.c_int), ("ls_ghost", C.c_int), ("ref_bugs", C.c_int),
        ("bc_walls", C.c_int), ("filter_every", C.c_int), ("cfilt", C.c_double),
        ("step_index", C.c_long), ("imp", Impeller), ("time", C.c_double), ("xyz", vp),
    ]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    src = HERE / "oracle.cpp"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        build()
    lib = C.CDLL(str(LIB))
    sig = {
        "orc_deriv_pencil": [C.c_int, C.c_int, vp, C.c_double],
        "orc_deriv3d": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, vp, vp],
        "orc_cudaDeriv": [i3, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                          C.c_int, C.c_int, C.c_int],
        "orc_cuDivergence": [i3] + [vp] * 9 + [C.c_double] * 3 + [C.c_int] * 3,
        "orc_flujos": [C.c_int, C.c_int, C.c_int, C.c_int] + [vp] * 12,
        "orc_inisgdm": [C.c_int, C.c_int, C.c_int, vp, vp, vp],
        "orc_sgs_sf": [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.c_double, vp],
        "orc_sgs_smag": [C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_double, vp],
        "orc_viscosidad": [C.c_int, vp, C.c_double, vp],
        "orc_to_ghost": [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int],
        "orc_mirror_ghost": [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double],
        "orc_from_ghost": [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int],
        "orc_weno_rhs": [vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                         C.c_int, C.c_int, C.c_int, C.c_int],
        "orc_weno_advect": [vp, vp, vp, C.c_double, C.c_double, C.c_double, C.c_double,
                            C.c_int, C.c_int, C.c_int, C.c_int],
        "orc_step": [C.POINTER(StepParams), vp, vp, vp, vp, vp, vp],
        "orc_bc_walls": [vp, C.c_int, C.c_int, C.c_int],
        "orc_jacobeano": [vp, vp, C.c_int, C.c_double, C.c_double, C.c_double,
                          C.c_int, C.c_int, C.c_int],
        "orc_extrapolation": [vp, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                              C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int],
        "orc_advect_extrapolate": [vp, vp, vp, C.c_double, C.c_double, C.c_double,
                                   C.c_int, C.c_int, C.c_int, C.c_double],
        "orc_filtronper": [C.c_int, vp, C.c_double, C.c_int],
        "orc_impeller_force": [vp, vp, C.POINTER(Impeller), C.c_double, C.c_int, C.c_int, C.c_int, vp],
        "orc_filtrado": [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int],
        "orc_reinit": [vp, vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                       C.c_int, C.c_double, C.c_int, C.c_int],
        "orc_set_threads": [C.c_int],
        "orc_get_threads": [],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.orc_cfl.argtypes = [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int]
    lib.orc_cfl.restype = C.c_double
    lib.orc_phi_x_weno.argtypes = [C.c_double] * 5
    lib.orc_phi_x_weno.restype = C.c_double
    lib.orc_set_threads.restype = None
    _lib = lib
    return lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "need C-contiguous float64"
    return a.ctypes.data


def _dims(a):
    nz, ny, nx = a.shape[-3:]
    return nx, ny, nz


def _ok(rc, name):
    if rc != 0:
        raise RuntimeError(f"{name} returned {rc}")


def set_threads(n: int):
    load().orc_set_threads(int(n))


def get_threads() -> int:
    return load().orc_get_threads()


def deriv_pencil(scheme, u, h):
    u = np.array(u, dtype=np.float64, copy=True)
    _ok(load().orc_deriv_pencil(scheme, u.size, _p(u), h), "orc_deriv_pencil")
    return u


def deriv3d(scheme, axis, f, h):
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty_like(f)
    nx, ny, nz = _dims(f)
    _ok(load().orc_deriv3d(scheme, axis, nx, ny, nz, h, _p(f), _p(out)), "orc_deriv3d")
    return out


def cudaDeriv(schemes, vel, temp, h):
    nx, ny, nz = _dims(temp)
    dvel = np.empty((9, nz, ny, nx))
    dtemp = np.empty((3, nz, ny, nx))
    s = schemes if not isinstance(schemes, int) else (schemes,) * 3
    _ok(load().orc_cudaDeriv(i3(*s), _p(dvel), _p(dtemp), _p(np.ascontiguousarray(vel)),
                             _p(np.ascontiguousarray(temp)), h[0], h[1], h[2], nx, ny, nz),
        "orc_cudaDeriv")
    return dvel, dtemp


def cuDivergence(schemes, e, f, g, ev, fv, gv, jbn, h):
    nx, ny, nz = _dims(e)
    rs = np.empty((nz, ny, nx))
    rsv = np.empty((nz, ny, nx))
    s = schemes if not isinstance(schemes, int) else (schemes,) * 3
    arrs = [np.ascontiguousarray(a) for a in (e, f, g, ev, fv, gv, jbn)]
    _ok(load().orc_cuDivergence(i3(*s), _p(rs), _p(rsv), *[_p(a) for a in arrs],
                                h[0], h[1], h[2], nx, ny, nz), "orc_cuDivergence")
    return rs, rsv


def flujos(neq, um, u, pres, dvel, jbn, vis):
    nx, ny, nz = _dims(pres)
    out = [np.empty((nz, ny, nx)) for _ in range(6)]
    _ok(load().orc_flujos(neq, nx, ny, nz, *[_p(o) for o in out], _p(um), _p(u), _p(pres),
                          _p(dvel), _p(jbn), _p(vis)), "orc_flujos")
    return tuple(out)


def inisgdm(xyz):
    nx, ny, nz = _dims(xyz)
    d = np.empty((nz, ny, nx))
    r = np.empty((6, nz, ny, nx))
    _ok(load().orc_inisgdm(nx, ny, nz, _p(np.ascontiguousarray(xyz)), _p(d), _p(r)),
        "orc_inisgdm")
    return d, r


def sgs_sf(u, dvel, jbn, dxyz, ratios, amu0=0.1781):
    nx, ny, nz = _dims(dxyz)
    a = np.empty((nz, ny, nx))
    _ok(load().orc_sgs_sf(nx, ny, nz, _p(u), _p(dvel), _p(jbn), _p(dxyz), _p(ratios), amu0,
                          _p(a)), "orc_sgs_sf")
    return a


def sgs_smag(dvel, jbn, dxyz, cs=0.1):
    nx, ny, nz = _dims(dxyz)
    a = np.empty((nz, ny, nx))
    _ok(load().orc_sgs_smag(nx, ny, nz, _p(dvel), _p(jbn), _p(dxyz), cs, _p(a)), "orc_sgs_smag")
    return a


def viscosidad(amut, c4):
    v = np.empty_like(amut)
    _ok(load().orc_viscosidad(amut.size, _p(amut), c4, _p(v)), "orc_viscosidad")
    return v


def ghost_pad(val, g, direction=1.0):
    nx, ny, nz = _dims(val)
    out = np.zeros((nz + 2 * g, ny + 2 * g, nx + 2 * g))
    lib = load()
    lib.orc_to_ghost(_p(out), _p(np.ascontiguousarray(val)), g, nx, ny, nz)
    lib.orc_mirror_ghost(_p(out), g, nx, ny, nz, direction)
    return out


def ghost_unpad(ghost, g):
    nzg, nyg, nxg = ghost.shape
    out = np.empty((nzg - 2 * g, nyg - 2 * g, nxg - 2 * g))
    load().orc_from_ghost(_p(out), _p(ghost), g, nxg - 2 * g, nyg - 2 * g, nzg - 2 * g)
    return out


def phi_x_weno(b1, b2, b3, b4, b5):
    return load().orc_phi_x_weno(b1, b2, b3, b4, b5)


def weno_rhs(phi, vel, jbn, h, ref_bugs=0):
    nx, ny, nz = _dims(phi)
    rs = np.empty_like(phi)
    _ok(load().orc_weno_rhs(_p(rs), _p(phi), _p(vel), _p(jbn), h[0], h[1], h[2], nx, ny, nz,
                            ref_bugs), "orc_weno_rhs")
    return rs


def weno_advect(phi, vel, jbn, h, dt, ref_bugs=0):
    phi = np.array(phi, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(phi)
    _ok(load().orc_weno_advect(_p(phi), _p(np.ascontiguousarray(vel)), _p(np.ascontiguousarray(jbn)),
                               h[0], h[1], h[2], dt, nx, ny, nz, ref_bugs), "orc_weno_advect")
    return phi


def extrapolation(ext, phiS, j0, j4, j8, s, dtext, flag=1, iters=10):
    """cuExtrapolation on a given (padded) grid; returns the extrapolated field."""
    ext = np.array(ext, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(ext)
    c = np.ascontiguousarray
    _ok(load().orc_extrapolation(_p(ext), _p(c(phiS)), _p(c(j0)), _p(c(j4)), _p(c(j8)), s[0], s[1],
                                 s[2], nx, ny, nz, dtext, flag, iters), "orc_extrapolation")
    return ext


def advect_extrapolate(press, jbn, sobject, delta, deltamin):
    """advect_CUDA as linked: pressure extrapolated into the solid object."""
    press = np.array(press, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(press)
    c = np.ascontiguousarray
    _ok(load().orc_advect_extrapolate(_p(press), _p(c(jbn)), _p(c(sobject)), delta[0], delta[1],
                                      delta[2], nx, ny, nz, deltamin), "orc_advect_extrapolate")
    return press


def reinit(phi, jbn, dmins, delta, g, deltamin, iters=10, ref_bugs=0):
    """cuReinitLsJB on padded arrays; returns the reinitialised phi."""
    phi = np.array(phi, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(phi)
    c = np.ascontiguousarray
    _ok(load().orc_reinit(_p(phi), _p(c(jbn)), _p(c(dmins)), delta[0], delta[1], delta[2], nx, ny, nz,
                          g, deltamin, iters, ref_bugs), "orc_reinit")
    return phi


def bc_walls(um):
    um = np.array(um, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(um)
    _ok(load().orc_bc_walls(_p(um), nx, ny, nz), "orc_bc_walls")
    return um


def cfl(u, xyz, mach):
    nx, ny, nz = _dims(xyz)
    return load().orc_cfl(_p(np.ascontiguousarray(u)), _p(np.ascontiguousarray(xyz)), mach, nx, ny, nz)


def jacobeano(xyz, scheme, h):
    nx, ny, nz = _dims(xyz)
    jbn = np.empty((11, nz, ny, nx))
    _ok(load().orc_jacobeano(_p(np.ascontiguousarray(xyz)), _p(jbn), scheme, h[0], h[1], h[2],
                             nx, ny, nz), "orc_jacobeano")
    return jbn


def impeller_force(um, xyz, imp, t):
    """The impeller forcing at time t; returns (um, mask)."""
    um = np.array(um, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(um)
    mask = np.empty(um.shape[1:])
    c = Impeller()
    c.on = 1
    for f, _ in Impeller._fields_[1:]:
        setattr(c, f, getattr(imp, f))
    _ok(load().orc_impeller_force(_p(um), _p(np.ascontiguousarray(xyz)), C.byref(c), t, nx, ny, nz,
                                  _p(mask)), "orc_impeller_force")
    return um, mask


def filtronper(u, cfilt, zrows=0):
    u = np.array(u, dtype=np.float64, copy=True)
    _ok(load().orc_filtronper(len(u), _p(u), cfilt, zrows), "orc_filtronper")
    return u


def filtrado(um, jbn, cfilt):
    um = np.array(um, dtype=np.float64, copy=True)
    nx, ny, nz = _dims(um)
    _ok(load().orc_filtrado(_p(um), _p(np.ascontiguousarray(jbn)), cfilt, nx, ny, nz), "orc_filtrado")
    return um


def step_params(workload, level_set=True, ref_bugs=0, ls_ghost=5, bc_walls=0, filter_every=0,
                cfilt=0.0):
    w = workload
    p = StepParams()
    p.nx, p.ny, p.nz = w.grid.nx, w.grid.ny, w.grid.nz
    for a in range(3):
        p.scheme[a] = w.schemes[a]
        p.h[a] = w.grid.h(a)
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
    p.step_index = 0
    imp = getattr(w, "impeller", None)
    if imp is not None:
        p.imp.on = 1
        for f, _ in Impeller._fields_[1:]:
            setattr(p.imp, f, getattr(imp, f))
        p._xyz = np.ascontiguousarray(w.grid.coords())   # kept alive with the params
        p.xyz = p._xyz.ctypes.data
    p.time = getattr(w, "t0", 0.0)
    return p


def step(params: StepParams, um, phi, jbn, mask, dxyz, ratios=None, nsteps=1):
    um = np.array(um, dtype=np.float64, copy=True)
    phi = None if phi is None else np.array(phi, dtype=np.float64, copy=True)
    lib = load()
    t0 = params.time
    for it in range(nsteps):
        params.step_index = it
        params.time = t0 + it * params.dt
        _ok(lib.orc_step(C.byref(params), _p(um), _p(phi), _p(np.ascontiguousarray(jbn)),
                         _p(np.ascontiguousarray(mask)), _p(np.ascontiguousarray(dxyz)),
                         _p(None if ratios is None else np.ascontiguousarray(ratios))),
            "orc_step")
    return um, phi
