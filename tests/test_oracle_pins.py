"""Known-answer pins for the CPU oracle (no GPU).

The reference ships no tests, fixtures or golden vectors and its Fortran
cannot be compiled here, so the oracle is pinned against mathematics:
each compact scheme against a dense solve of the exact system the reference
builds, the modified wavenumber of the cyclic Lele scheme, polynomial
exactness of every closure, and the WENO5 reconstruction against its linear
limit and its convergence order.
"""
import math

import numpy as np
import pytest

from emix_gb300 import fields as F


def dense_system(scheme, n, h):
    """Tridiagonal matrix and RHS-stencil matrix as the reference builds them."""
    A = np.zeros((n, n))
    Bm = np.zeros((n, n))
    s = 1.0 / h
    if scheme == F.SCHEME_BPER:
        ars, brs = 7 / 9, 1 / 36
        for i in range(n):
            A[i, i] = 1.0
            A[i, (i - 1) % n] = 1 / 3
            A[i, (i + 1) % n] = 1 / 3
            Bm[i, (i + 1) % n] += ars * s
            Bm[i, (i - 1) % n] -= ars * s
            Bm[i, (i + 2) % n] += brs * s
            Bm[i, (i - 2) % n] -= brs * s
        return A, Bm
    if scheme == F.SCHEME_A:      # solver/derivada.f90
        a = [0.0] + [0.25] * (n - 2) + [3.0]
        c = [3.0] + [0.25] * (n - 2) + [0.0]
        ars, brs = 0.75, 0.0
        lo = {0: [-17 / 6, 1.5, 1.5, -1 / 6]}
        hi = {0: [17 / 6, -1.5, -1.5, 1 / 6]}
        first, last = 1, n - 1
    elif scheme == F.SCHEME_B:    # src/MSVSingle/derivada_incomp.f90
        a = [0.0, 0.25] + [1 / 3] * (n - 4) + [0.25, 2.0]
        c = [2.0, 0.25] + [1 / 3] * (n - 4) + [0.25, 0.0]
        ars, brs = 7 / 9, 1 / 36
        lo = {0: [-2.5, 2.0, 0.5, 0.0], 1: [-0.75, 0.0, 0.75, 0.0]}
        hi = {0: [2.5, -2.0, -0.5, 0.0], 1: [0.75, 0.0, -0.75, 0.0]}
        first, last = 2, n - 2
    else:                          # src/Schemes/derivCompact.cu
        a = [0.0, 0.25] + [1 / 3] * (n - 4) + [0.25, 3.0]
        c = [3.0, 0.25] + [1 / 3] * (n - 4) + [0.25, 0.0]
        ars, brs = 7 / 9, 1 / 36
        lo = {0: [-17 / 6, 1.5, 1.5, -1 / 6], 1: [-0.75, 0.0, 0.75, 0.0]}
        hi = {0: [17 / 6, -1.5, -1.5, 1 / 6], 1: [0.75, 0.0, -0.75, 0.0]}
        first, last = 2, n - 2
    for i in range(n):
        A[i, i] = 1.0
        if i > 0:
            A[i, i - 1] = a[i]
        if i < n - 1:
            A[i, i + 1] = c[i]
    for i in range(first, last):
        Bm[i, i + 1] += ars * s
        Bm[i, i - 1] -= ars * s
        if brs:
            Bm[i, i + 2] += brs * s
            Bm[i, i - 2] -= brs * s
    for r, co in lo.items():
        Bm[r, :4] = np.array(co) * s
    for r, co in hi.items():
        Bm[n - 1 - r, n - 1] += co[0] * s
        Bm[n - 1 - r, n - 2] += co[1] * s
        Bm[n - 1 - r, n - 3] += co[2] * s
        Bm[n - 1 - r, n - 4] += co[3] * s
    return A, Bm


@pytest.mark.parametrize("scheme", [F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C])
@pytest.mark.parametrize("n", [7, 16, 33, 64])
def test_pencil_matches_dense_solve(oracle, scheme, n):
    h = 1.0 / (n if scheme == F.SCHEME_BPER else n - 1)
    u = F.uniform(3, n, (n,))
    A, Bm = dense_system(scheme, n, h)
    ref = np.linalg.solve(A, Bm @ u)
    got = oracle.deriv_pencil(scheme, u, h)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_modified_wavenumber_lele6(oracle):
    n = 32
    L = 2 * math.pi
    h = L / n
    x = np.arange(n) * h
    for k in range(1, n // 2):
        kh = k * h
        kp = (14 / 9 * math.sin(kh) + 1 / 18 * math.sin(2 * kh)) / (1 + 2 / 3 * math.cos(kh)) / h
        got = oracle.deriv_pencil(F.SCHEME_BPER, np.sin(k * x), h)
        assert np.max(np.abs(got - kp * np.cos(k * x))) <= 1e-12 * max(1.0, kp)


@pytest.mark.parametrize("scheme,degree", [(F.SCHEME_A, 4), (F.SCHEME_B, 3), (F.SCHEME_C, 4)])
def test_polynomial_exactness(oracle, scheme, degree):
    n = 21
    h = 1.0 / (n - 1)
    x = np.arange(n) * h
    for p in range(0, degree + 1):
        got = oracle.deriv_pencil(scheme, x ** p, h)
        ref = p * x ** (p - 1) if p > 0 else np.zeros(n)
        assert np.max(np.abs(got - ref)) <= 1e-11, (scheme, p)
    # one degree more is not exact
    got = oracle.deriv_pencil(scheme, x ** (degree + 1), h)
    assert np.max(np.abs(got - (degree + 1) * x ** degree)) > 1e-9


def test_lele6_interior_order(oracle):
    """Away from the closures the B scheme is 6th order."""
    errs = []
    for n in (41, 81):
        h = 1.0 / (n - 1)
        x = np.arange(n) * h
        d = oracle.deriv_pencil(F.SCHEME_BPER, np.sin(2 * math.pi * x[:-1] * 1.0), 1.0 / (n - 1))
        errs.append(np.max(np.abs(d - 2 * math.pi * np.cos(2 * math.pi * x[:-1]))))
    assert math.log2(errs[0] / errs[1]) > 5.5


def test_deriv3d_axes_match_pencils(oracle):
    w = F.random_box(9, 8, 7, seed=2)
    f = np.ascontiguousarray(w.um[1])
    for axis in range(3):
        d = oracle.deriv3d(F.SCHEME_C, axis, f, 0.1)
        g = np.moveaxis(f, 2 - axis, -1)
        ref = np.apply_along_axis(lambda p: oracle.deriv_pencil(F.SCHEME_C, p, 0.1), -1, g)
        assert np.array_equal(d, np.moveaxis(ref, -1, 2 - axis))


def test_weno_consistency_and_linear_limit(oracle):
    # constant differences reproduce the constant
    for v in (0.0, 1.0, -3.5, 1e3):
        assert abs(oracle.phi_x_weno(v, v, v, v, v) - v) <= 1e-15 * max(1.0, abs(v))
    # smooth data: nonlinear weights tend to 0.1/0.6/0.3 -> linear 5th-order value
    x = np.linspace(0.0, 0.004, 5)
    v = 1.0 + 0.3 * x + 0.05 * x ** 2
    lin = (2 * v[0] - 13 * v[1] + 47 * v[2] + 27 * v[3] - 3 * v[4]) / 60
    assert abs(oracle.phi_x_weno(*v) - lin) < 1e-12
    # a jump in the leftmost difference: the weight of stencil 1 collapses
    got = oracle.phi_x_weno(10.0, 1.0, 1.0, 1.0, 1.0)
    assert abs(got - 1.0) < 1e-6


def test_weno_convergence_order(oracle):
    """WENO5 upwind gradient of a smooth profile converges at ~5th order."""
    errs = []
    for n in (24, 48):
        g = 5
        L = 1.0
        h = L / n
        nxg = n + 2 * g
        x = (np.arange(nxg) - g) * h
        phi1 = np.sin(2 * math.pi * x / L)
        phi = np.ascontiguousarray(np.broadcast_to(phi1, (8, 8, nxg)).copy())
        vel = np.zeros((3,) + phi.shape)
        vel[0] = 1.0
        jbn = np.zeros((11,) + phi.shape)
        jbn[0] = jbn[4] = jbn[8] = 1.0
        rs = oracle.weno_rhs(phi, np.ascontiguousarray(vel), np.ascontiguousarray(jbn), (h, h, h))
        ref = 2 * math.pi / L * np.cos(2 * math.pi * x / L)
        inner = slice(g, nxg - g)
        errs.append(np.max(np.abs(rs[4, 4, inner] - ref[inner])))
    assert math.log2(errs[0] / errs[1]) > 4.5


def test_mirror_ghost(oracle):
    val = F.uniform(1, 0, (4, 5, 6))
    g = 3
    G = oracle.ghost_pad(np.ascontiguousarray(val), g, 1.0)
    nz, ny, nx = val.shape

    def m(I, n):
        I = I - g
        return -I - 1 if I < 0 else (2 * n - 1 - I if I >= n else I)
    for Z in (0, 2, nz + g, nz + 2 * g - 1):
        for Y in (1, g, ny + g + 1):
            for X in (0, g + 2, nx + 2 * g - 1):
                assert G[Z, Y, X] == val[m(Z, nz), m(Y, ny), m(X, nx)]
    Gm = oracle.ghost_pad(np.ascontiguousarray(val), g, -1.0)
    assert Gm[0, 0, 0] == -val[m(0, nz), m(0, ny), m(0, nx)]      # three reflections
    assert Gm[g, g, 0] == -val[0, 0, m(0, nx)]                      # one reflection
    assert Gm[0, 0, g] == val[m(0, nz), m(0, ny), 0]                 # two reflections
    assert np.array_equal(oracle.ghost_unpad(G, g), val)


def test_sgs_uniform_grid_values(oracle):
    g = F.Grid(6, 7, 8, (0.5, 0.7, 0.8))
    d, r = oracle.inisgdm(np.ascontiguousarray(g.coords()))
    dx = [g.length[a] * g.h(a) for a in range(3)]
    delta = (dx[0] * dx[1] * dx[2]) ** (1 / 3)
    assert np.allclose(d, delta, rtol=1e-14)
    for q, a in enumerate([0, 0, 1, 1, 2, 2]):
        assert np.allclose(r[q], (delta / dx[a]) ** (1 / 3), rtol=1e-14)


def test_smagorinsky_pure_shear(oracle):
    """u = S*y: |S| = S, nu_t = (Cs*Delta)^2 * S."""
    g = F.Grid(8, 8, 8, (1.0, 1.0, 1.0))
    dvel = np.zeros((9,) + g.shape)
    S = 2.5
    dvel[3] = S                         # du/deta with deta/dy = 1
    jbn = g.jbn()
    dxyz = np.full(g.shape, 0.01)
    a = oracle.sgs_smag(np.ascontiguousarray(dvel), np.ascontiguousarray(jbn), dxyz, 0.1)
    assert np.allclose(a, (0.1 * 0.01) ** 2 * S, rtol=1e-14)


def test_step_conserves_uniform_state(oracle):
    """A uniform state at rest on a periodic box is a fixed point of the step."""
    w = F.random_box(8, 8, 8, seed=1, periodic=True)
    w.um[0] = 1.0
    w.um[1:4] = 0.0
    w.um[4] = 1.0
    w.phi[:] = 0.25
    p = oracle.step_params(w)
    dxyz, ratios = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    um, phi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, dxyz, ratios)
    assert np.allclose(um, w.um, atol=1e-13)
    assert np.allclose(phi, 0.25, atol=1e-13)


def test_thread_count_invariance(oracle):
    w = F.random_box(10, 9, 8, seed=4)
    p = oracle.step_params(w)
    dxyz, ratios = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    oracle.set_threads(1)
    a, pa = oracle.step(p, w.um, w.phi, w.jbn, w.mask, dxyz, ratios)
    oracle.set_threads(4)
    b, pb = oracle.step(p, w.um, w.phi, w.jbn, w.mask, dxyz, ratios)
    oracle.set_threads(0)
    assert np.array_equal(a, b) and np.array_equal(pa, pb)


def test_taylor_green_w_momentum_is_conditioned_beyond_1e12(oracle):
    """The conditioning behind the 64^3 Taylor-Green parity test: one RK3
    step of the oracle from inputs moved by one ulp (seeded directions)
    already differs from the unmoved step by more than 1e-12 (normwise
    relative) in the w-momentum, whose largest value is the 1e-3 noise, while
    the other fields stay near 1e-14."""
    w = F.taylor_green(64)
    p = oracle.step_params(w, level_set=True)
    dxyz, ratios = oracle.inisgdm(np.ascontiguousarray(w.grid.coords()))
    rng = np.random.default_rng(5)

    def nudged(x):
        d = rng.integers(0, 2, size=x.shape).astype(bool)
        return np.where(d, np.nextafter(x, np.inf), np.nextafter(x, -np.inf))

    a_um, a_phi = oracle.step(p, w.um, w.phi, w.jbn, w.mask, dxyz, ratios, nsteps=1)
    b_um, b_phi = oracle.step(p, nudged(w.um), nudged(w.phi), w.jbn, w.mask, dxyz, ratios, nsteps=1)
    rel = [float(np.max(np.abs(b_um[m] - a_um[m])) / np.max(np.abs(a_um[m]))) for m in range(5)]
    assert rel[3] > 1e-12
    assert max(rel[0], rel[1], rel[2], rel[4]) < 1e-13
    assert float(np.max(np.abs(b_phi - a_phi)) / np.max(np.abs(a_phi))) < 1e-14
