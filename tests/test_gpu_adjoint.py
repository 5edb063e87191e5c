"""Adjoint of the RK3 step: each transposed operator against the forward one
(dot-product identities <A x, y> = <x, A^T y>), then gradients of the tank
objective against central finite differences of the forward step."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _dot(a, b):
    return float((a * b).sum())


@pytest.mark.parametrize("scheme", [F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_deriv_transpose_dot_product(emix, oracle, scheme, axis):
    import torch
    shape = (3, 11, 13, 12)            # (fields, nz, ny, nx)
    x = F.uniform(91, axis, shape)
    y = F.uniform(92, axis, shape)
    n = (12, 13, 11)[axis]
    h = 1.0 / (n - 1) if scheme != F.SCHEME_BPER else 1.0 / n
    dx = emix.deriv_dev(_dev(x), axis, h, scheme).cpu().numpy()
    dty = emix.deriv_t_dev(_dev(y), axis, h, scheme).cpu().numpy()
    lhs, rhs = _dot(dx, y), _dot(x, dty)
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + np.abs(dx).sum() * np.abs(y).max())
    # against the dense transpose of the oracle's operator on one pencil
    cols = []
    for k in range(n):
        shp = [1, 1, 1]
        shp[2 - axis] = n
        f = np.zeros(shp)
        f.reshape(-1)[k] = 1.0
        cols.append(oracle.deriv3d(scheme, axis, f, h).reshape(-1))
    Dm = np.stack(cols, axis=1)
    take = [0, 0, 0]
    take[2 - axis] = slice(None)
    yp = y[0][tuple(take)]
    got = dty[0][tuple(take)]
    assert_close(got, Dm.T @ yp, tol=1e-12, what="pencil")
    # accumulate form
    acc = _dev(x)
    emix.deriv_t_dev(_dev(y), axis, h, scheme, out=acc)
    assert_close(acc.cpu().numpy(), x + dty, tol=1e-14, what="accumulate")
    torch.cuda.synchronize()


@pytest.mark.parametrize("scheme", [F.SCHEME_A, F.SCHEME_B, F.SCHEME_C])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_deriv_transpose_long_pencils(emix, oracle, scheme, axis):
    """Pencils of 70 rows (x pencils cross two 32-row staging chunks and end
    in a partial one; 35 pencils leave a partial warp): every pencil of D^T y
    against the dense transpose of the oracle's operator, both forms."""
    shape = [2, 5, 7, 6]               # (fields, nz, ny, nx)
    shape[3 - axis] = 70
    shape = tuple(shape)
    y = F.uniform(95, axis, shape)
    x = F.uniform(96, axis, shape)
    n = 70
    h = 1.0 / (n - 1)
    cols = []
    for k in range(n):
        shp = [1, 1, 1]
        shp[2 - axis] = n
        f = np.zeros(shp)
        f.reshape(-1)[k] = 1.0
        cols.append(oracle.deriv3d(scheme, axis, f, h).reshape(-1))
    Dm = np.stack(cols, axis=1)
    ax = 3 - axis
    want = np.moveaxis(np.tensordot(Dm.T, np.moveaxis(y, ax, 0), axes=1), 0, ax)
    got = emix.deriv_t_dev(_dev(y), axis, h, scheme).cpu().numpy()
    assert_close(got, want, tol=1e-12, what="D^T")
    acc = _dev(x)
    emix.deriv_t_dev(_dev(y), axis, h, scheme, out=acc)
    assert_close(acc.cpu().numpy(), x + want, tol=1e-12, what="accumulate")


def _tank_case(n=20, steps=2):
    w = F.stirred_tank(n=n, impeller=True, impeller_omega=1.3, height=2.0)
    # the free surface inside the box so the interface term is active
    X, Y, Z = w.grid.coords()
    w.phi = np.ascontiguousarray(Z - 1.0 + 0.05 * np.sin(3 * X) * np.cos(2 * Y))
    return w


def _runner(emix, w, steps, every=1):
    return emix.TankGradient(w, steps, every, bc_walls=1)


@pytest.mark.parametrize("every", [0, 1, 2])
def test_parameter_gradient_matches_finite_differences(emix, every):
    w = _tank_case()
    r = _runner(emix, w, 3, every)
    om, cs = 1.3, 0.1
    J = r.run(om, cs)
    g_om, g_cs = r.adj.backward()
    assert np.isfinite(J) and J > 0
    def cfd(k, p0, h):
        args_p = [om, cs]; args_p[k] = p0 + h
        args_m = [om, cs]; args_m[k] = p0 - h
        return (r.run(*args_p) - r.run(*args_m)) / (2 * h)

    for k, (p0, g) in enumerate(((om, g_om), (cs, g_cs))):
        assert g != 0.0
        # Richardson-extrapolated central differences (error O(h^4)): the
        # gradient to 1e-6; plain h = 1e-6 differences to their rounding limit
        h = 1e-3 * abs(p0)
        fd = (4.0 * cfd(k, p0, 0.5 * h) - cfd(k, p0, h)) / 3.0
        assert abs(g - fd) <= 1e-6 * abs(fd), (k, g, fd)
        h6 = 1e-6 * max(abs(p0), 1.0)
        fd6 = cfd(k, p0, h6)
        assert abs(g - fd6) <= 1e-6 * abs(fd) + 20 * 2.2e-16 * abs(J) / h6, (k, g, fd6)
    r.close()


def test_kept_tapes_give_the_recomputed_gradient(emix):
    """every = 0 (every step's tape kept from the forward pass, nothing
    recomputed) against checkpoints every step with recomputation: the same
    J, dJ/d(omega, Cs) and initial-state adjoint, and the context left at the
    same final state."""
    import torch
    w = _tank_case()
    out = []
    for every in (0, 1):
        r = _runner(emix, w, 3, every)
        J = r.run(1.3, 0.1)
        g = r.adj.backward()
        lum, lphi = r.adj.state_gradient()
        um, phi = r.ctx.download()
        out.append((J, g, lum.cpu().numpy(), lphi.cpu().numpy(), um, phi, r.ctx.step_index))
        r.close()
    (J0, g0, l0, p0, u0, f0, k0), (J1, g1, l1, p1, u1, f1, k1) = out
    assert J0 == J1 and k0 == k1
    assert abs(g0[0] - g1[0]) <= 1e-14 * abs(g1[0]) and abs(g0[1] - g1[1]) <= 1e-14 * abs(g1[1])
    assert_close(l0, l1, tol=1e-13, what="lum")
    assert_close(p0, p1, tol=1e-13, what="lphi")
    assert np.array_equal(u0, u1) and np.array_equal(f0, f1)
    torch.cuda.synchronize()


@pytest.mark.parametrize("every", [0, 1])
def test_taped_forward_overlap_is_neutral(emix, every):
    """The taped forward with its tape copies and level-set stages on the
    second stream (the default) against everything on the compute stream:
    bit for bit the same J and final state, and the same dJ/d(omega, Cs) and
    initial-state adjoint to the rounding of the reverse sweep's atomic
    scatters (a tape copy joined too late, or a stage read before it was
    written, would show far above that)."""
    w = _tank_case(n=36)
    out = []
    for on in (1, 0):
        r = _runner(emix, w, 3, every)
        r.adj.set_overlap(on)
        J = r.run(1.3, 0.1)
        g = r.adj.backward()
        lum, lphi = r.adj.state_gradient()
        um, phi = r.ctx.download()
        out.append((J, g, lum.cpu().numpy(), lphi.cpu().numpy(), um, phi))
        r.close()
    (J0, g0, l0, p0, u0, f0), (J1, g1, l1, p1, u1, f1) = out
    assert J0 == J1
    assert np.array_equal(u0, u1) and np.array_equal(f0, f1)
    assert abs(g0[0] - g1[0]) <= 1e-14 * abs(g1[0]) and abs(g0[1] - g1[1]) <= 1e-14 * abs(g1[1])
    assert_close(l0, l1, tol=1e-13, what="lum")
    assert_close(p0, p1, tol=1e-13, what="lphi")


def test_state_gradient_matches_directional_derivative(emix):
    import torch
    w = _tank_case(18)
    r = _runner(emix, w, 2)
    J = r.run(1.3, 0.1)
    r.adj.backward()
    lum, lphi = r.adj.state_gradient()
    lum, lphi = lum.cpu().numpy(), lphi.cpu().numpy()
    um0, phi0 = w.um.copy(), w.phi.copy()
    sh = phi0.shape
    dum = np.stack([1e-2 * F.uniform(93, m, sh) for m in range(5)]) * np.abs(um0).max(axis=(1, 2, 3))[:, None, None, None]
    dphi = 1e-2 * F.uniform(94, 0, sh)
    def dd(du, dp, eps):
        vals = []
        for sgn in (1, -1):
            w.um = np.ascontiguousarray(um0 + sgn * eps * du)
            w.phi = np.ascontiguousarray(phi0 + sgn * eps * dp)
            vals.append(r.run(1.3, 0.1))
        return (vals[0] - vals[1]) / (2 * eps)

    # central differences in the asymptotic range of each direction (the
    # interface term's smoothed delta needs the smaller step)
    for du, dp, eps in ((dum, 0 * dphi, 1e-4), (0 * dum, dphi, 1e-5)):
        pred = float((lum * du).sum() + (lphi * dp).sum())
        fd = dd(du, dp, eps)
        assert pred != 0.0
        assert abs(pred - fd) <= 1e-6 * abs(fd), (pred, fd)
    w.um, w.phi = um0, phi0
    r.close()


def test_autograd_function(emix):
    import torch
    w = _tank_case(16)
    r = _runner(emix, w, 2)
    f = r.function()
    theta = torch.tensor([1.3, 0.1], dtype=torch.float64, requires_grad=True)
    J = f(theta)
    J.backward()
    g = theta.grad.numpy()
    J2 = r.run(1.3, 0.1)
    assert float(J.detach()) == J2
    g2 = r.adj.backward()
    assert np.allclose(g, g2, rtol=1e-12, atol=0)
    r.close()
