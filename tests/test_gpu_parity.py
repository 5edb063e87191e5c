"""Parity of every CUDA operator with the CPU oracle on seeded inputs.

All comparisons are normwise relative L-infinity per field, tolerance 1e-12
(FP64 throughout; the kernels use precomputed Thomas factors and fused
multiply-adds, so results agree with the oracle to rounding, not bitwise).
The calls go through the C ABI of libemix_gb300.so.
"""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import TOL, assert_close, relerr

pytestmark = pytest.mark.gpu

SCHEMES = [F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C]
SIZES = [(24, 20, 28), (33, 17, 12), (6, 7, 9)]


def _torch():
    import torch
    return torch


def dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    _torch().cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("shape", SIZES)
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_deriv_axis(emix, oracle, scheme, shape, axis):
    nx, ny, nz = shape
    w = F.random_box(nx, ny, nz, seed=11, periodic=(scheme == F.SCHEME_BPER))
    f = np.ascontiguousarray(w.um[1:4])
    h = w.grid.h(axis)
    got = host(emix.deriv_dev(dev(f), axis, h, scheme))
    for c in range(3):
        ref = oracle.deriv3d(scheme, axis, f[c], h)
        assert_close(got[c], ref, what=f"scheme {scheme} axis {axis} comp {c}")


@pytest.mark.parametrize("scheme", SCHEMES)
def test_cudaDeriv_host(emix, oracle, scheme):
    w = F.random_box(20, 18, 22, seed=3, periodic=(scheme == F.SCHEME_BPER))
    vel = np.ascontiguousarray(w.um[1:4] / w.um[0])
    temp = np.ascontiguousarray(w.um[4])
    h = tuple(w.grid.h(a) for a in range(3))
    dvel, dtemp = emix.cudaDeriv(vel, temp, h, scheme)
    rdvel, rdtemp = oracle.cudaDeriv(scheme, vel, temp, h)
    for c in range(9):
        assert_close(dvel[c], rdvel[c], what=f"dvel[{c}]")
    for c in range(3):
        assert_close(dtemp[c], rdtemp[c], what=f"dtemp[{c}]")


def test_cudaDeriv_reference_symbol(emix, oracle):
    """The reference's own symbol, Fortran argument order, default scheme C."""
    nx, ny, nz = 16, 14, 18
    w = F.random_box(nx, ny, nz, seed=4)
    vel = np.ascontiguousarray(w.um[1:4] / w.um[0])
    temp = np.ascontiguousarray(w.um[4])
    jbn = np.ascontiguousarray(w.jbn)
    amut = np.zeros((nz, ny, nx))
    dxyz = np.zeros((nz, ny, nx))
    dvel = np.zeros((9, nz, ny, nx))
    dtemp = np.zeros((3, nz, ny, nx))
    h = [w.grid.h(a) for a in range(3)]
    emix.set_legacy_scheme(F.SCHEME_C)
    emix.cudaDeriv_legacy(dvel, dtemp, vel, temp, amut, dxyz, jbn, h[0], h[1], h[2], nx, ny, nz)
    rdvel, rdtemp = oracle.cudaDeriv(F.SCHEME_C, vel, temp, h)
    assert_close(dvel, rdvel, what="dvel")
    assert_close(dtemp, rdtemp, what="dtemp")


@pytest.mark.parametrize("scheme", [F.SCHEME_B, F.SCHEME_C, F.SCHEME_BPER])
def test_cuDivergence(emix, oracle, scheme):
    w = F.random_box(18, 16, 20, seed=7, periodic=(scheme == F.SCHEME_BPER))
    rng = [F.uniform(21, q, w.grid.shape) for q in range(6)]
    e, f, g, ev, fv, gv = [np.ascontiguousarray(r) for r in rng]
    jbn = np.ascontiguousarray(w.jbn)
    h = tuple(w.grid.h(a) for a in range(3))
    rs, rsv = emix.cuDivergence(e, f, g, ev, fv, gv, jbn, h, scheme)
    r_rs, r_rsv = oracle.cuDivergence(scheme, e, f, g, ev, fv, gv, jbn, h)
    assert_close(rs, r_rs, what="rs")
    assert_close(rsv, r_rsv, what="rsv")
    # device form
    d = [dev(a) for a in (e, f, g, ev, fv, gv, jbn)]
    drs, drsv = emix.cuDivergence_dev(*d, h, scheme)
    assert_close(host(drs), r_rs, what="rs (device)")
    assert_close(host(drsv), r_rsv, what="rsv (device)")


def test_cuDivergence_reference_symbol(emix, oracle):
    nx, ny, nz = 12, 15, 13
    w = F.random_box(nx, ny, nz, seed=8)
    e, f, g, ev, fv, gv = [np.ascontiguousarray(F.uniform(5, q, w.grid.shape)) for q in range(6)]
    jbn = np.ascontiguousarray(w.jbn)
    h = [w.grid.h(a) for a in range(3)]
    keep = [a.copy() for a in (e, f, g, ev, fv, gv)]
    rs = np.zeros((nz, ny, nx))
    rsv = np.zeros((nz, ny, nx))
    emix.set_legacy_scheme(F.SCHEME_C)
    emix.cuDivergence_legacy(rs, rsv, e, f, g, ev, fv, gv, jbn, h[0], h[1], h[2], nx, ny, nz)
    r_rs, r_rsv = oracle.cuDivergence(F.SCHEME_C, e, f, g, ev, fv, gv, jbn, h)
    assert_close(rs, r_rs, what="rs")
    assert_close(rsv, r_rsv, what="rsv")
    for a, b in zip(keep, (e, f, g, ev, fv, gv)):
        assert np.array_equal(a, b), "inputs must not be modified"


@pytest.mark.parametrize("neq", [1, 2, 3, 4, 5])
def test_flux(emix, oracle, neq):
    w = F.random_box(14, 12, 10, seed=9)
    n = w.grid.shape
    um = np.ascontiguousarray(w.um)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    pres = np.ascontiguousarray(w.um[0] / w.mach ** 2)
    dvel = np.ascontiguousarray(np.stack([F.uniform(31, q, n) for q in range(9)]))
    vis = np.ascontiguousarray(1e-3 + 1e-4 * (1 + F.uniform(32, 0, n)))
    jbn = np.ascontiguousarray(w.jbn)
    got = emix.flux_dev(neq, dev(um), dev(u), dev(pres), dev(dvel), dev(jbn), dev(vis))
    ref = oracle.flujos(neq, um, u, pres, dvel, jbn, vis)
    for q in range(6):
        assert_close(host(got[q]), ref[q], what=f"flux {q}")


def _stretched_coords(nx, ny, nz):
    g = F.Grid(nx, ny, nz, (1.0, 1.2, 0.8))
    x, y, z = (g.coords1d(a) for a in range(3))
    x = x + 0.03 * np.sin(2 * np.pi * x)
    y = y ** 1.2
    z = z + 0.02 * z * z
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.ascontiguousarray(np.stack([X, Y, Z]))


def test_sgs_setup(emix, oracle):
    xyz = _stretched_coords(13, 11, 9)
    d, r = emix.sgs_setup_dev(dev(xyz))
    rd, rr = oracle.inisgdm(xyz)
    assert_close(host(d), rd, what="dxyzsgd")
    for q in range(6):
        assert_close(host(r)[q], rr[q], what=f"ratio {q}")


@pytest.mark.parametrize("model", [1, 2])
def test_sgs_viscosity(emix, oracle, model):
    w = F.random_box(16, 14, 12, seed=12)
    xyz = _stretched_coords(16, 14, 12)
    dxyz, ratios = oracle.inisgdm(xyz)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    h = tuple(w.grid.h(a) for a in range(3))
    dvel, _ = oracle.cudaDeriv(F.SCHEME_B, u, np.ascontiguousarray(w.um[4]), h)
    jbn = np.ascontiguousarray(w.jbn)
    c4 = 1e-3
    if model == 1:
        ref = oracle.sgs_smag(dvel, jbn, dxyz, 0.1)
        amut, vis = emix.sgs_viscosity_dev(1, 0.1, c4, dev(u), dev(dvel), dev(jbn), dev(dxyz))
    else:
        ref = oracle.sgs_sf(u, dvel, jbn, dxyz, ratios, 0.1781)
        amut, vis = emix.sgs_viscosity_dev(2, 0.1781, c4, dev(u), dev(dvel), dev(jbn), dev(dxyz),
                                           dev(ratios))
        assert np.any(ref == 0.0) or True
    assert_close(host(amut), ref, what="amut")
    assert_close(host(vis), oracle.viscosidad(ref, c4), what="vis")


@pytest.mark.parametrize("g", [3, 5])
def test_ghost_pad(emix, oracle, g):
    w = F.random_box(9, 8, 7, seed=13)
    val = np.ascontiguousarray(w.phi)
    got = host(emix.ghost_pad_dev(dev(val), g, 1.0))
    ref = oracle.ghost_pad(val, g, 1.0)
    assert np.array_equal(got, ref)
    got_m = host(emix.ghost_pad_dev(dev(val), g, -1.0))
    assert np.array_equal(got_m, oracle.ghost_pad(val, g, -1.0))
    back = host(emix.ghost_unpad_dev(dev(ref), g))
    assert np.array_equal(back, val)


def _ls_case(nx, ny, nz, seed, g=5):
    w = F.random_box(nx, ny, nz, seed=seed)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    # sign changes in every direction exercise both upwind reconstructions
    u[0] -= 0.3
    u[2] *= -1.0
    phig = np.ascontiguousarray(np.zeros((nz + 2 * g, ny + 2 * g, nx + 2 * g)))
    from oracle import oracle_py as O
    phig = O.ghost_pad(np.ascontiguousarray(w.phi), g)
    velg = np.ascontiguousarray(np.stack([O.ghost_pad(np.ascontiguousarray(u[c]), g) for c in range(3)]))
    jbng = np.zeros((11,) + phig.shape)
    for c in (0, 4, 8):
        jbng[c] = O.ghost_pad(np.ascontiguousarray(w.jbn[c]), g)
    h = tuple(w.grid.h(a) for a in range(3))
    return phig, velg, np.ascontiguousarray(jbng), h, 0.3 * min(h)


@pytest.mark.parametrize("ref_bugs", [0, 1])
@pytest.mark.parametrize("shape", [(10, 9, 11), (20, 20, 20)])
def test_weno5_advect(emix, oracle, ref_bugs, shape):
    phig, velg, jbng, h, dt = _ls_case(*shape, seed=14)
    ref = oracle.weno_advect(phig, velg, jbng, h, dt, ref_bugs)
    got = emix.weno5_advect(phig, velg, jbng, h, dt, ref_bugs)
    assert_close(got, ref, what="phi (host entry)")
    t = dev(phig)
    emix.weno5_advect_dev(t, dev(velg), dev(jbng), h, dt, ref_bugs)
    assert_close(host(t), ref, what="phi (device entry)")


def test_weno5_ref_bugs_differs_only_at_top(emix, oracle):
    phig, velg, jbng, h, dt = _ls_case(12, 12, 12, seed=15)
    velg[2] = np.abs(velg[2]) + 0.1      # left-biased z reconstruction everywhere
    velg = np.ascontiguousarray(velg)
    a = emix.weno5_advect(phig, velg, jbng, h, dt, 0)
    b = emix.weno5_advect(phig, velg, jbng, h, dt, 1)
    diff = np.abs(a - b).max(axis=(1, 2))
    nzg = phig.shape[0]
    assert np.all(diff[: nzg - 7] == 0.0)
    assert diff[nzg - 1] > 0.0


def _step_case(kind):
    if kind == "periodic_smag":
        w = F.random_box(16, 18, 14, seed=21, periodic=True)
        w.sgs_model = 1
    elif kind == "walls_sf":
        w = F.random_box(14, 16, 18, seed=22, periodic=False)
        w.sgs_model = 2
    elif kind == "walls_C_smag":
        w = F.random_box(16, 14, 16, seed=23, periodic=False, scheme=F.SCHEME_C)
        w.sgs_model = 1
    else:
        w = F.random_box(12, 12, 12, seed=24, periodic=False, scheme=F.SCHEME_A)
        w.sgs_model = 0
    w.mask = F.uniform(25, 0, w.grid.shape) > -0.9   # a few masked cells
    w.mask = w.mask.astype(np.float64)
    return w


@pytest.mark.parametrize("kind", ["periodic_smag", "walls_sf", "walls_C_smag", "walls_A_none"])
@pytest.mark.parametrize("level_set", [True, False])
def test_step(emix, oracle, kind, level_set):
    w = _step_case(kind)
    ctx = emix.Context(w, level_set=level_set)
    ctx.step(2, use_graph=False)
    um, phi = ctx.download()
    p = oracle.step_params(w, level_set=level_set)
    dxyz, ratios = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi if level_set else None, w.jbn, w.mask, dxyz,
                            ratios, nsteps=2)
    for m in range(5):
        assert_close(um[m], rum[m], what=f"um[{m}]")
    if level_set:
        assert_close(phi, rphi, what="phi")
    # graph replay gives the same result as direct launches
    ctx.upload(w.um, w.phi if level_set else None)
    ctx.step(2, use_graph=True)
    um2, phi2 = ctx.download()
    assert np.array_equal(um2, um)
    if level_set:
        assert np.array_equal(phi2, phi)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 3])
def test_overlapped_streams_give_the_same_bits(emix, mode):
    """The level-set stages (mode 1), the x gradients (mode 2) or both on a
    second stream, and the context's one stream (the default), give
    identical results."""
    w = F.stirred_tank(n=24, impeller=True)
    a = emix.Context(w, bc_walls=1)
    b = emix.Context(w, bc_walls=1)
    a.set_overlap(mode)
    b.set_overlap(0)
    for use_graph in (False, True):
        a.upload(w.um, w.phi); a.time = 0.0
        b.upload(w.um, w.phi); b.time = 0.0
        a.step(3, use_graph=use_graph)
        b.step(3, use_graph=use_graph)
        ua, pa = a.download()
        ub, pb = b.download()
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
    a.close()
    b.close()


def _ulp_nudged(x, seed):
    """x with every value moved by one ulp up or down (seeded)."""
    d = np.random.default_rng(seed).integers(0, 2, size=x.shape).astype(bool)
    return np.where(d, np.nextafter(x, np.inf), np.nextafter(x, -np.inf))


@pytest.mark.gpu
def test_taylor_green_64_ten_steps(emix, oracle):
    """The 64^3 periodic Taylor-Green box with the sphere level set, as the
    reference's CPU-runnable configuration is set up (cyclic scheme B,
    Smagorinsky Cs = 0.1, Re = 1000, CFL 0.3), 10 full RK3 steps through the
    device context against the same 10 steps of the oracle.

    Every field is held to 1e-12 unless the problem itself cannot resolve it:
    the oracle is also run from inputs moved by one ulp, and a field whose own
    spread under that perturbation exceeds 1e-12 is held to twice that spread.
    This is the w-momentum, whose largest value is the 1e-3 noise while its
    equation carries O(1) terms: one ulp of input moves it by about 2e-12
    after one step and 5e-12 after ten, so no FP64 evaluation order can
    match another to 1e-12 there."""
    w = F.taylor_green(64)
    ctx = emix.Context(w, level_set=True)
    ctx.step(10, use_graph=True)
    um, phi = ctx.download()
    ctx.close()
    p = oracle.step_params(w, level_set=True)
    dxyz, ratios = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, dxyz, ratios, nsteps=10)
    sum_, sphi = oracle.step(p, _ulp_nudged(w.um, 5), _ulp_nudged(w.phi, 6), w.jbn, w.mask, dxyz,
                             ratios, nsteps=10)
    for m in range(5):
        spread = relerr(sum_[m], rum[m])
        tol = TOL if spread <= TOL else 2.0 * spread
        if m != 3:
            assert tol == TOL, f"um[{m}]: spread {spread:.2e} under one ulp of input"
        assert_close(um[m], rum[m], tol=tol, what=f"um[{m}] (one-ulp spread {spread:.2e})")
    assert relerr(sphi, rphi) <= TOL
    assert_close(phi, rphi, what="phi")


@pytest.mark.gpu
@pytest.mark.parametrize("n,nz", [(24, 24), (30, 21), (23, 26)])
def test_tma_plane_tiles_give_the_same_bits(emix, n, nz):
    """The level-set stages with their phi plane tiles brought by TMA tiled
    copies and with register-staged loads give identical results; odd padded
    x extents (n = 23: 33 cells) fall back to the loads by themselves."""
    timeouts = emix.weno_tma_timeouts()
    w = F.stirred_tank(n=n, nz=nz, impeller=True)
    a = emix.Context(w, bc_walls=1)
    b = emix.Context(w, bc_walls=1)
    b.set_tma(False)
    assert b.tma_stages() == 0
    assert a.tma_stages() == (3 if (n + 10) % 2 == 0 else 0)
    for use_graph in (False, True):
        a.upload(w.um, w.phi); a.time = 0.0
        b.upload(w.um, w.phi); b.time = 0.0
        a.step(3, use_graph=use_graph)
        b.step(3, use_graph=use_graph)
        ua, pa = a.download()
        ub, pb = b.download()
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
    a.close()
    b.close()
    assert emix.weno_tma_timeouts() == timeouts


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_longest_pencils(emix, oracle, scheme, axis):
    """Pencils of the longest supported length (4096 rows; the x pencils walk
    128 staging chunks) against the oracle, D^T against D by the dot-product
    identity, and one row more rejected with EMIX_ERR_ARG."""
    shape = [6, 7, 6]                  # the other axes at the minimum of 6 cells
    shape[axis] = 4096
    nx, ny, nz = shape
    w = F.random_box(nx, ny, nz, seed=12, periodic=(scheme == F.SCHEME_BPER))
    f = np.ascontiguousarray(w.um[1:3])
    h = w.grid.h(axis)
    got = host(emix.deriv_dev(dev(f), axis, h, scheme))
    for c in range(2):
        ref = oracle.deriv3d(scheme, axis, f[c], h)
        assert_close(got[c], ref, what=f"scheme {scheme} axis {axis} comp {c}")
    y = np.ascontiguousarray(w.um[3:5])
    dty = host(emix.deriv_t_dev(dev(y), axis, h, scheme))
    lhs, rhs = float((got * y).sum()), float((f * dty).sum())
    assert abs(lhs - rhs) <= 1e-12 * (np.abs(got).sum() * np.abs(y).max())
    shape[axis] = 4097
    too_long = np.zeros((1, shape[2], shape[1], shape[0]))
    with pytest.raises(Exception):
        emix.deriv_dev(dev(too_long), axis, h, scheme)
