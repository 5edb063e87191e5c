"""Wall boundary conditions, CFL reduction and grid metrics on the device
against the CPU oracle, and the step with walls."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("shape", [(9, 8, 7), (20, 17, 13)])
def test_bc_walls(emix, oracle, shape):
    w = F.random_box(*shape, seed=51)
    um = np.ascontiguousarray(w.um)
    got = host(emix.bc_walls_dev(dev(um)))
    assert np.array_equal(got, oracle.bc_walls(um))


def test_cfl(emix, oracle):
    w = F.stirred_tank(n=24)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    xyz = np.ascontiguousarray(w.grid.coords())
    # stretch one axis so the neighbour-spacing minimum matters
    xyz[2] = xyz[2] ** 1.3
    got = emix.cfl_dev(dev(u), dev(xyz), w.mach)
    ref = oracle.cfl(u, xyz, w.mach)
    assert got == ref
    dt = emix.tstep_dt(got, 1e-3, 0.3)
    cflm = 1e-3 * got
    d = 1e-3 / cflm * 0.3
    diff = d - 1e-3
    assert abs(dt - (1e-3 + 0.85 * diff - 0.35 * abs(diff))) <= 1e-18


@pytest.mark.parametrize("scheme", [F.SCHEME_A, F.SCHEME_C])
def test_metrics(emix, oracle, scheme):
    g = F.Grid(14, 12, 10, (1.0, 1.2, 0.8))
    x, y, z = (g.coords1d(a) for a in range(3))
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    xyz = np.ascontiguousarray(np.stack([X + 0.05 * np.sin(3 * Y), Y + 0.04 * np.cos(2 * Z) * X,
                                         Z + 0.03 * X * Y]))
    h = (g.h(0), g.h(1), g.h(2))
    got = host(emix.metrics_dev(dev(xyz), h, scheme))
    ref = oracle.jacobeano(xyz, scheme, h)
    # the inverse metric as a 3x3 matrix field, normwise: single entries that
    # are a cancellation of small products (here jbn[6]) carry rounding at the
    # matrix's scale, not their own
    assert_close(got[:9], ref[:9], what="jbn[0:9]")
    for c in (9, 10):
        assert_close(got[c], ref[c], what=f"jbn[{c}]")


def test_metrics_singular(emix):
    g = F.Grid(8, 8, 8)
    xyz = np.ascontiguousarray(np.zeros((3,) + g.shape))
    with pytest.raises(emix.EmixError):
        emix.metrics_dev(dev(xyz), (0.1, 0.1, 0.1))


@pytest.mark.parametrize("sgs", [1, 2])
def test_step_with_walls(emix, oracle, sgs):
    w = F.random_box(14, 12, 16, seed=52)
    w.sgs_model = sgs
    ctx = emix.Context(w, level_set=True, bc_walls=1)
    ctx.step(2)
    um, phi = ctx.download()
    p = oracle.step_params(w, bc_walls=1)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=2)
    for m in range(5):
        assert_close(um[m], rum[m], what=f"um[{m}]")
    assert_close(phi, rphi, what="phi")
    ctx.close()


def test_batch_with_walls(emix):
    ws = F.ensemble(ngrids=3, seed=12, sizes=(16, 24))
    b = emix.Batch(ws, bc_walls=1)
    b.step_per_grid(1)
    ref = [b.download(g)[0] for g in range(3)]
    b.upload()
    b.step(1, use_graph=True)
    for g in range(3):
        assert_close(b.download(g)[0], ref[g], tol=1e-13, what=f"grid {g}")
    b.close()
