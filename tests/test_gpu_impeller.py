"""Rotating impeller forcing (rushton(sub_step) without the blade-edge
interpolation): the oracle against its definition, the device forcing and the
step with the impeller against the oracle."""
import math

import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close


def _tank(n=24, omega=1.7):
    w = F.stirred_tank(n=n, impeller=True, impeller_omega=omega)
    # a coarse grid: make the blades thick enough to hold cells
    w.impeller.half_thick = 3.0 * w.impeller.half_thick
    return w


def test_oracle_impeller_sets_body_rotation(oracle):
    w = _tank()
    xyz = w.grid.coords()
    um, m = oracle.impeller_force(w.um, xyz, w.impeller, 0.3)
    inside = m == 0.0
    assert inside.sum() > 20 and (~inside).sum() > 0
    om = w.impeller.omega
    r = um[0]
    # rigid rotation inside, up to the reference's 7-digit pi in the polar angle
    assert_close((um[1] / r)[inside], (-om * xyz[1])[inside], tol=3e-6, what="u inside")
    assert_close((um[2] / r)[inside], (om * xyz[0])[inside], tol=3e-6, what="v inside")
    assert np.all(um[3][inside] == 0.0)
    # outside, only the round trip u/rho*rho
    assert_close(um[1][~inside], w.um[1][~inside], tol=1e-15, what="outside")


def test_oracle_impeller_mask_rotates(oracle):
    """A blade turned by one blade spacing is the next blade: the mask at
    t + 2 pi / (nblades |omega|) equals the mask at t."""
    w = _tank(32, omega=2.0)
    xyz = w.grid.coords()
    imp = w.impeller
    _, m0 = oracle.impeller_force(w.um, xyz, imp, 0.1)
    _, m1 = oracle.impeller_force(w.um, xyz, imp, 0.1 + 2 * math.pi / (imp.nblades * abs(imp.omega)))
    # rounding of the angle can move cells that sit on a blade face
    assert np.mean(m0 != m1) < 2e-3
    _, m2 = oracle.impeller_force(w.um, xyz, imp, 0.1 + 0.5 * math.pi / (imp.nblades * abs(imp.omega)))
    assert np.mean(m0 != m2) > 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("t", [0.0, 0.37, 2.9])
def test_impeller_force_matches_oracle(emix, oracle, t):
    import torch
    w = _tank(28)
    xyz = np.ascontiguousarray(w.grid.coords())
    ref, mref = oracle.impeller_force(w.um, xyz, w.impeller, t)
    um = torch.from_numpy(np.ascontiguousarray(w.um)).cuda()
    m = emix.impeller_force_dev(um, torch.from_numpy(xyz).cuda(), w.impeller, t)
    torch.cuda.synchronize()
    assert np.array_equal(m.cpu().numpy(), mref)
    got = um.cpu().numpy()
    for c in range(4):
        assert_close(got[c], ref[c], what=f"um[{c}]")


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_step_with_impeller_matches_oracle(emix, oracle, use_graph):
    w = _tank(24)
    w.t0 = 0.25
    p = oracle.step_params(w, level_set=True, bc_walls=1)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=3)
    ctx = emix.Context(w, bc_walls=1)
    ctx.step(3, use_graph=use_graph)
    um, phi = ctx.download()
    for m in range(5):
        assert_close(um[m], rum[m], what=f"um[{m}]")
    assert_close(phi, rphi, what="phi")
    assert abs(ctx.time - (0.25 + 3 * w.dt)) <= 1e-15
    # restarting the clock repeats the forcing
    ctx.upload(w.um, w.phi)
    ctx.time = 0.25
    ctx.step(3, use_graph=use_graph)
    assert_close(ctx.download()[0], rum, what="after set_time")
    ctx.close()


@pytest.mark.gpu
def test_batched_impeller_equals_per_grid(emix):
    ws = [_tank(n, omega=om) for n, om in ((16, 0.7), (24, 1.9), (20, 1.2))]
    for w in ws:
        w.dt = min(x.dt for x in ws)
    b = emix.Batch(ws, bc_walls=1)
    b.step_per_grid(2)
    ref = [b.download(g)[0] for g in range(len(ws))]
    b.upload()
    b.step(2, use_graph=True)
    for g in range(len(ws)):
        assert_close(b.download(g)[0], ref[g], tol=1e-13, what=f"grid {g}")
    b.close()


def test_oracle_interpolation_keeps_a_rigid_rotation(oracle):
    """The interpolation fits a plane through the blade-surface point (moving
    rigidly) and two outer neighbours: on a flow that is the same rigid
    rotation everywhere it changes nothing (up to the reference's 7-digit pi)."""
    w = _tank(32, omega=1.4)
    X, Y, Z = w.grid.coords()
    om = w.impeller.omega
    um = w.um.copy()
    um[1] = -om * Y * um[0]
    um[2] = om * X * um[0]
    a, _ = oracle.impeller_force(um, w.grid.coords(), w.impeller, 0.05)
    w.impeller.interp = 1
    b, _ = oracle.impeller_force(um, w.grid.coords(), w.impeller, 0.05)
    changed = np.abs(b - a).max(axis=0) > 0
    assert changed.sum() > 10
    assert_close(b[1] / b[0], -om * Y, tol=3e-6, what="u")
    assert_close(b[2] / b[0], om * X, tol=3e-6, what="v")


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_step_with_impeller_interpolation_matches_oracle(emix, oracle, use_graph):
    w = _tank(28, omega=1.6)
    w.impeller.interp = 1
    w.t0 = 0.1
    p = oracle.step_params(w, level_set=True, bc_walls=1)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=2)
    # the interpolation changes the result
    w0 = _tank(28, omega=1.6)
    w0.t0 = 0.1
    p0 = oracle.step_params(w0, level_set=True, bc_walls=1)
    rum0, _ = oracle.step(p0, w0.um, w0.phi, w0.jbn, w0.mask, d, r, nsteps=2)
    assert np.abs(rum - rum0).max() > 1e-6
    ctx = emix.Context(w, bc_walls=1)
    ctx.step(2, use_graph=use_graph)
    um, phi = ctx.download()
    for m in range(5):
        assert_close(um[m], rum[m], what=f"um[{m}]")
    assert_close(phi, rphi, what="phi")
    ctx.close()
