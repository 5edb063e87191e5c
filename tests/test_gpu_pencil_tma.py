"""The flux divergence's y and z passes and the velocity gradients' fused y
and z launch (closed and cyclic schemes) with their rows staged by TMA tiled
copies
(emix_ctx_set_pencil_tma, on by default) against the same passes with
loads: the same values bit for bit (the same arithmetic in the same order) in
the graph-replayed and eager steps, the host-buffer step and the taped
forward; the transposed passes of the adjoint's reverse sweep
(emix_deriv_t_tma_dev) against their load kernel, bit for bit; the fall-back
where the copy unit's rules do not hold; and the bounded waits (copies
dropped by a test hook: every block gives up, counts itself, the host-buffer
step reports EMIX_ERR_TIMEOUT, and the context recovers)."""
import numpy as np
import pytest

from emix_gb300 import fields as F

pytestmark = pytest.mark.gpu


def _pair(w, **kw):
    from emix_gb300 import ops
    a = ops.Context(w, **kw)
    b = ops.Context(w, **kw)
    a.set_pencil_tma(True)
    b.set_pencil_tma(False)
    return a, b


# blocks of 32 (small launches spread evenly), 64, 32, 32, and 128 (a launch
# of more than 8 blocks per SM: the width that idles the fewest lanes)
@pytest.mark.parametrize("shape", [(24, 24), (40, 26), (130, 20), (128, 10), (256, 24)])
def test_tma_rows_give_the_same_bits(emix, shape):
    n, nz = shape
    timeouts = emix.pencil_tma_timeouts()
    w = F.stirred_tank(n=n, nz=nz, impeller=True)
    a, b = _pair(w, bc_walls=1)
    # per substep: divergence y, divergence z, gradients y + z
    assert a.pencil_tma_launches() == 9 and b.pencil_tma_launches() == 0
    for use_graph in (True, False):
        for c in (a, b):
            c.upload(w.um, w.phi)
            c.time = 0.0
            c.step(3, use_graph=use_graph)
        ua, pa = a.download()
        ub, pb = b.download()
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
    hu = [np.ascontiguousarray(w.um.copy()) for _ in range(2)]
    hp = [np.ascontiguousarray(w.phi.copy()) for _ in range(2)]
    for c, u, p in ((a, hu[0], hp[0]), (b, hu[1], hp[1])):
        c.upload(w.um, w.phi)
        c.time = 0.0
        c.step_host(u, p, 2)
    assert np.array_equal(hu[0], hu[1]) and np.array_equal(hp[0], hp[1])
    a.close()
    b.close()
    assert emix.pencil_tma_timeouts() == timeouts


@pytest.mark.parametrize("case", ["tgv128", "box256x64x64"])
def test_cyclic_tma_rows_give_the_same_bits(emix, case):
    """The cyclic scheme (periodic boxes) with rows staged by TMA (launches of
    at least 2^16 pencils): the wrap rows, the Sherman-Morrison sum and
    correction as in the load kernels, bit for bit, in graph-replayed and
    eager steps."""
    if case == "tgv128":
        w = F.taylor_green(128)
    else:
        w = F.random_box(256, 64, 64, periodic=True)
    timeouts = emix.pencil_tma_timeouts()
    a, b = _pair(w, level_set=False)
    assert a.pencil_tma_launches() == 9 and b.pencil_tma_launches() == 0
    for use_graph in (True, False):
        for c in (a, b):
            c.upload(w.um, w.phi)
            c.step(3, use_graph=use_graph)
        assert np.array_equal(a.download()[0], b.download()[0])
    a.close()
    b.close()
    assert emix.pencil_tma_timeouts() == timeouts


def test_tma_rows_fall_back_where_the_rules_do_not_hold(emix):
    from emix_gb300 import ops
    odd = ops.Context(F.stirred_tank(n=23, nz=20, impeller=True), bc_walls=1)
    odd.set_pencil_tma(True)
    assert odd.pencil_tma_launches() == 0     # nx odd: rows not 16-byte aligned
    odd.close()
    small = ops.Context(F.taylor_green(24))
    small.set_pencil_tma(True)
    assert small.pencil_tma_launches() == 0   # cyclic launches of fewer than 2^16 pencils
    small.close()
    wm = F.random_box(256, 64, 64)
    wm.schemes = (F.SCHEME_C, F.SCHEME_BPER, F.SCHEME_C)
    mixed = ops.Context(wm)
    mixed.set_pencil_tma(True)
    # y cyclic, z closed: the divergence's y and z passes by TMA, the fused
    # gradient pair (one launch of both tables) keeps its loads
    assert mixed.pencil_tma_launches() == 6
    mixed.close()


def test_taped_forward_with_tma_rows(emix):
    from emix_gb300 import ops
    w = F.stirred_tank(n=24, impeller=True, impeller_omega=1.3)
    res = []
    for on in (True, False):
        r = ops.TankGradient(w, 2, 0, bc_walls=1)
        r.ctx.set_pencil_tma(on)
        J = r.run(1.3, 0.1)
        res.append((J, r.ctx.download()))
        r.close()
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1][0], res[1][1][0])


def test_dropped_row_copies_time_out_and_the_context_recovers(emix):
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    w = F.stirred_tank(n=24, impeller=True)
    a, b = _pair(w, bc_walls=1)
    before = emix.pencil_tma_timeouts()
    um = np.ascontiguousarray(w.um.copy())
    phi = np.ascontiguousarray(w.phi.copy())
    _lib.check(lib.emix_pencil_tma_test_drop(1), "emix_pencil_tma_test_drop")
    try:
        with pytest.raises(RuntimeError, match="TMA"):
            a.step_host(um, phi, 1)
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.emix_pencil_tma_test_drop(0), "emix_pencil_tma_test_drop")
    assert emix.pencil_tma_timeouts() > before
    after = emix.pencil_tma_timeouts()
    for c in (a, b):
        c.upload(w.um, w.phi)
        c.time = 0.0
        c.step(2)
    ua, pa = a.download()
    ub, pb = b.download()
    assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
    assert emix.pencil_tma_timeouts() == after
    a.close()
    b.close()


# (nf, nz, ny, nx): pencils of 26 and 9 rows (a partial last chunk, whose
# accumulation box runs past the end), 130 and 64 rows, in blocks of 32; and
# launches of more than 8 blocks per SM along y, in blocks of 128 and 64
@pytest.mark.parametrize("shape", [(5, 9, 26, 40), (3, 130, 13, 20), (2, 64, 6, 128), (1, 10, 9, 24),
                                   (1, 640, 8, 256), (1, 416, 10, 192)])
@pytest.mark.parametrize("scheme", [F.SCHEME_A, F.SCHEME_B, F.SCHEME_C])
def test_transposed_passes_with_tma_rows_give_the_same_bits(emix, shape, scheme):
    """D^T along y and z (the adjoint's reverse-sweep passes) with rows staged
    by TMA against the load kernel: the same values bit for bit, storing and
    accumulating."""
    import torch
    timeouts = emix.pencil_tma_timeouts()
    nf, nz, ny, nx = shape
    for axis in (1, 2):
        n = (nx, ny, nz)[axis]
        h = 1.0 / (n - 1)
        y = torch.from_numpy(F.uniform(97, axis, shape)).cuda()
        x = torch.from_numpy(F.uniform(98, axis, shape)).cuda()
        a = emix.deriv_t_dev(y, axis, h, scheme, tma=True)
        b = emix.deriv_t_dev(y, axis, h, scheme)
        assert torch.equal(a, b), (axis, "store")
        a = x.clone()
        b = x.clone()
        emix.deriv_t_dev(y, axis, h, scheme, out=a, tma=True)
        emix.deriv_t_dev(y, axis, h, scheme, out=b)
        assert torch.equal(a, b), (axis, "accumulate")
    torch.cuda.synchronize()
    assert emix.pencil_tma_timeouts() == timeouts


def test_transposed_passes_refuse_where_the_rules_do_not_hold(emix):
    import torch
    from emix_gb300 import _lib
    y = torch.zeros((4, 6, 7), dtype=torch.float64, device="cuda")    # nx = 7: rows not 16-byte aligned
    with pytest.raises(_lib.EmixError):
        emix.deriv_t_dev(y, 1, 0.1, F.SCHEME_C, tma=True)
    y = torch.zeros((4, 6, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.EmixError):
        emix.deriv_t_dev(y, 0, 0.1, F.SCHEME_C, tma=True)                # x pencils: the load kernel's
    with pytest.raises(_lib.EmixError):
        emix.deriv_t_dev(y, 1, 1.0 / 6, F.SCHEME_BPER, tma=True)        # the cyclic scheme: D^T = -D


def test_transposed_pass_with_dropped_copies_times_out(emix):
    """Copies left out by the test hook: every block gives up after its
    bounded wait, counts itself and writes nothing; the next pass is exact."""
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    y = torch.from_numpy(F.uniform(99, 1, (12, 20, 32))).cuda()
    before = emix.pencil_tma_timeouts()
    out = torch.full_like(y, 7.0)
    _lib.check(lib.emix_pencil_tma_test_drop(1), "emix_pencil_tma_test_drop")
    try:
        emix.deriv_t_dev(y, 1, 0.05, F.SCHEME_C, out=out, tma=True)
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.emix_pencil_tma_test_drop(0), "emix_pencil_tma_test_drop")
    assert emix.pencil_tma_timeouts() == before + 12     # one block of 32 pencils per z plane
    assert bool((out == 7.0).all())
    a = emix.deriv_t_dev(y, 1, 0.05, F.SCHEME_C, tma=True)
    b = emix.deriv_t_dev(y, 1, 0.05, F.SCHEME_C)
    assert torch.equal(a, b)
    assert emix.pencil_tma_timeouts() == before + 12
