"""Pressure extrapolation into the solid (the linked advect_CUDA) on the
device against the CPU oracle, on sizes the reference's own launch grids do
not tile (and non-cubic padded grids), with both extrapolation sides."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close


def _case(shape, seed):
    nx, ny, nz = shape
    sh = (nz, ny, nx)
    z, y, x = np.meshgrid(np.linspace(0, 1, nz), np.linspace(0, 1, ny), np.linspace(0, 1, nx),
                          indexing="ij")
    sobj = 0.3 - np.sqrt((x - 0.5) ** 2 + (y - 0.4) ** 2 + (z - 0.55) ** 2)
    press = np.cos(2 * x) * np.sin(3 * y + z) + 0.01 * F.uniform(seed, 0, sh)
    jbn = np.zeros((11,) + sh)
    for c in (0, 4, 8):
        jbn[c] = 1.0 + 0.1 * F.uniform(seed, 1 + c, sh)
    delta = (1.0 / (nx - 1), 1.0 / (ny - 1), 1.0 / (nz - 1))
    return (np.ascontiguousarray(press), np.ascontiguousarray(jbn), np.ascontiguousarray(sobj), delta,
            0.8 * min(delta))


def test_oracle_extrapolation_keeps_fluid_side(oracle):
    """With no solid cell (sobject <= 0 everywhere) the direction field is zero
    and every pseudo-step returns the pressure up to rounding."""
    press, jbn, sobj, delta, dmin = _case((12, 10, 9), 71)
    out = oracle.advect_extrapolate(press, jbn, -np.abs(sobj) - 0.01, delta, dmin)
    assert_close(out, press, tol=1e-15, what="press")


def test_oracle_extrapolation_moves_only_near_solid(oracle):
    press, jbn, sobj, delta, dmin = _case((16, 14, 12), 72)
    out = oracle.advect_extrapolate(press, jbn, sobj, delta, dmin)
    changed = np.abs(out - press) > 1e-13
    assert changed.any()
    # information travels one cell per stage from the solid side
    assert not changed[sobj < -0.2].any()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(13, 9, 11), (24, 20, 16), (20, 20, 20)])
def test_advect_extrapolate_matches_oracle(emix, oracle, shape):
    press, jbn, sobj, delta, dmin = _case(shape, 73)
    ref = oracle.advect_extrapolate(press, jbn, sobj, delta, dmin)
    got = emix.advect_extrapolate(press, jbn, sobj, delta, dmin)
    assert_close(got, ref, what="press")
    assert_close(got - press, ref - press, tol=1e-11, what="change of press")


@pytest.mark.gpu
@pytest.mark.parametrize("flag,iters", [(1, 3), (-1, 10), (1, 0)])
def test_extrapolate_dev_matches_oracle(emix, oracle, flag, iters):
    import torch
    press, jbn, sobj, delta, dmin = _case((18, 15, 12), 74)
    g = 5
    P = oracle.ghost_pad(press, g)
    S = oracle.ghost_pad(sobj, g)
    J = [oracle.ghost_pad(jbn[c], g) for c in (0, 4, 8)]
    ref = oracle.ghost_unpad(
        oracle.extrapolation(P, S, *J, tuple(1.0 / d for d in delta), 0.3 * dmin, flag, iters), g)
    t = torch.from_numpy(press.copy()).cuda()
    emix.extrapolate_dev(t, torch.from_numpy(sobj).cuda(), torch.from_numpy(jbn).cuda(), delta,
                         0.3 * dmin, flag, iters)
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    assert_close(got, ref, what="ext")
    if iters == 0:
        assert np.array_equal(got, press)


@pytest.mark.gpu
def test_advect_extrapolate_rejects_bad_sizes(emix):
    press, jbn, sobj, delta, dmin = _case((8, 8, 8), 75)
    with pytest.raises(emix.EmixError):
        emix.advect_extrapolate(press[:4], jbn[:, :4], sobj[:4], delta, dmin)
