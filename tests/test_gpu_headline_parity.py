"""Parity at the benchmark's own sizes: the 256^3 stirred tank (walls,
rotating impeller, Lele-6 with 3rd/4th-order closures, Smagorinsky, WENO5
level set) stepped once through the host-buffer entry point emix_step_host,
exactly as bench.py times it, and the 128^3 tank of the gradient workload
over its 8 steps through the graph-replayed device context, both against the
oracle's steps (the RK loop of solver/rungek_ico.f90:61-313 restated) at
1e-12 normwise relative L-inf per field.
"""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _oracle_steps(oracle, w, nsteps):
    p = oracle.step_params(w, level_set=True, bc_walls=1)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    return oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=nsteps)


def test_tank_256_one_step_through_the_host_entry_point(emix, oracle):
    w = F.stirred_tank(n=256, impeller=True)
    ctx = emix.Context(w, level_set=True, ls_ghost=5, bc_walls=1)
    um = np.ascontiguousarray(w.um.copy())
    phi = np.ascontiguousarray(w.phi.copy())
    ctx.step_host(um, phi, 1)
    ctx.close()
    rum, rphi = _oracle_steps(oracle, w, 1)
    for m in range(5):
        assert_close(um[m], rum[m], what=f"256^3 tank, one step: um[{m}]")
    assert_close(phi, rphi, what="256^3 tank, one step: phi")


def test_tank_128_eight_steps(emix, oracle):
    w = F.stirred_tank(n=128, impeller=True)
    ctx = emix.Context(w, level_set=True, ls_ghost=5, bc_walls=1)
    ctx.step(8, use_graph=True)
    um, phi = ctx.download()
    ctx.close()
    rum, rphi = _oracle_steps(oracle, w, 8)
    for m in range(5):
        assert_close(um[m], rum[m], what=f"128^3 tank, 8 steps: um[{m}]")
    assert_close(phi, rphi, what="128^3 tank, 8 steps: phi")
