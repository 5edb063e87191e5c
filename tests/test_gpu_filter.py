"""Compact filter (filtrado / filtronper): the oracle against the filter's
defining properties, the device filter against the oracle, and the step with
the filter every few steps."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close


def test_filter_rhs_weights_preserve_constants(oracle):
    """The interior stencil sums to 1 + 2*alpha, the tridiagonal rows to the
    same, and the unfiltered end rows have a = c = 0: constants pass through
    x/y pencils unchanged."""
    for cf in (0.3, 0.45, 0.49):
        u = np.full(40, 2.5)
        assert_close(oracle.filtronper(u, cf, 0), u, tol=1e-14, what=f"alpha {cf}")


def test_filter_z_rows_change_the_end_values(oracle):
    """z gets the periodic row arrays (a = c = alpha on every row) with the
    non-periodic right-hand side, so even a constant is altered near the ends
    (herramientas_incomp2.f90 passes azpf/bzpf/czpf for z)."""
    u = np.full(60, 1.0)
    out = oracle.filtronper(u, 0.3, 1)
    assert abs(out[0] - 1.0) > 1e-3
    assert_close(out[25:35], u[25:35], tol=1e-6, what="interior")


def test_filter_removes_odd_even_mode(oracle):
    """The 10th-order stencil weights annihilate (-1)^l in the interior."""
    n = 80
    u = (-1.0) ** np.arange(n)
    out = oracle.filtronper(u, 0.4, 0)
    assert np.max(np.abs(out[25:n - 25])) < 1e-6
    # the five end rows are not filtered
    assert out[0] != 0.0


def test_filter_low_wavenumbers_pass(oracle):
    n = 96
    x = np.arange(n) * (2 * np.pi / 48)
    u = np.sin(x)
    out = oracle.filtronper(u, 0.49, 0)
    assert_close(out[10:n - 10], u[10:n - 10], tol=1e-6, what="smooth mode")


def _state(shape, seed):
    nx, ny, nz = shape
    sh = (nz, ny, nx)
    um = np.stack([1.0 + 0.1 * F.uniform(seed, m, sh) for m in range(5)])
    jbn = np.zeros((11,) + sh)
    for c in range(9):
        jbn[c] = F.uniform(seed, 10 + c, sh)
    jbn[9] = 1.0 + 0.2 * F.uniform(seed, 30, sh)
    jbn[10] = 1.0 / jbn[9]
    return np.ascontiguousarray(um), np.ascontiguousarray(jbn)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,cf", [((16, 13, 12), 0.45), ((24, 20, 18), 0.49), ((11, 11, 11), 0.3)])
def test_filtrado_matches_oracle(emix, oracle, shape, cf):
    import torch
    um, jbn = _state(shape, 81)
    ref = oracle.filtrado(um, jbn, cf)
    t = torch.from_numpy(um.copy()).cuda()
    emix.filtrado_dev(t, torch.from_numpy(jbn).cuda(), cf)
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    for m in range(5):
        assert_close(got[m], ref[m], what=f"um[{m}]")
    # the filter changes the field (not an identity pass)
    assert np.max(np.abs(ref - um)) > 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("axis,zrows", [(0, 0), (1, 0), (2, 1), (2, 0), (0, 1)])
def test_filter_pass_matches_oracle(emix, oracle, axis, zrows):
    import torch
    um, jbn = _state((14, 12, 13), 82)
    f = um[:2].copy()
    ref = f.copy()
    n = f.shape[1:]
    for m in range(2):
        g = ref[m] * jbn[9]
        g = np.moveaxis(g, 2 - axis, -1).copy()
        for idx in np.ndindex(g.shape[:-1]):
            g[idx] = oracle.filtronper(g[idx], 0.47, zrows)
        ref[m] = np.moveaxis(g, -1, 2 - axis) * jbn[10]
    t = torch.from_numpy(f).cuda()
    emix.filter_dev(t, torch.from_numpy(jbn).cuda(), 0.47, axis, zrows)
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    assert got.shape[1:] == n
    assert_close(got, ref, what=f"axis {axis} zrows {zrows}")


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_step_with_filter_matches_oracle(emix, oracle, use_graph):
    w = F.random_box(16, 14, 12, seed=83)
    p = oracle.step_params(w, level_set=True, filter_every=2, cfilt=0.45)
    d, r = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rum, rphi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, d, r, nsteps=3)
    ctx = emix.Context(w, filter_every=2, cfilt=0.45)
    ctx.step(3, use_graph=use_graph)
    assert ctx.step_index == 3
    um, phi = ctx.download()
    for m in range(5):
        assert_close(um[m], rum[m], what=f"um[{m}]")
    assert_close(phi, rphi, what="phi")
    ctx.close()


@pytest.mark.gpu
def test_step_index_selects_filtered_steps(emix):
    w = F.random_box(12, 12, 12, seed=84)
    a = emix.Context(w, filter_every=3, cfilt=0.45)
    b = emix.Context(w, filter_every=3, cfilt=0.45)
    b.step_index = 1          # not a filtered step
    c = emix.Context(w)       # no filter
    for x in (a, b, c):
        x.step(1)
    ua, ub, uc = a.download()[0], b.download()[0], c.download()[0]
    assert np.array_equal(ub, uc)
    assert not np.array_equal(ua, uc)
    for x in (a, b, c):
        x.close()


@pytest.mark.gpu
def test_batch_rejects_filter(emix):
    ws = F.ensemble(ngrids=2, seed=3, sizes=(16,))
    from emix_gb300 import _lib
    import ctypes as C
    ps = (_lib.EmixParams * 2)(*[emix._params_of(w, filter_every=9, cfilt=0.45) for w in ws])
    h = C.c_void_p()
    rc = _lib.load().emix_batch_create(2, ps, C.byref(h))
    assert rc != 0
