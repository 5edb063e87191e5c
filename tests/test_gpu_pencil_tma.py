"""The flux divergence's y and z passes and the velocity gradients' fused y
and z launch with their rows staged by TMA tiled copies
(emix_ctx_set_pencil_tma, on by default) against the same passes with
loads: the
same values bit for bit (the same arithmetic in the same order) in the
graph-replayed and eager steps, the host-buffer step and the taped forward;
the fall-back where the copy unit's rules do not hold; and the bounded waits
(copies dropped by a test hook: every block gives up, counts itself, the
host-buffer step reports EMIX_ERR_TIMEOUT, and the context recovers)."""
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


@pytest.mark.parametrize("shape", [(24, 24), (40, 26), (130, 20), (128, 10)])   # blocks of 32, 64, 32, 128
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


def test_tma_rows_fall_back_where_the_rules_do_not_hold(emix):
    from emix_gb300 import ops
    odd = ops.Context(F.stirred_tank(n=23, nz=20, impeller=True), bc_walls=1)
    odd.set_pencil_tma(True)
    assert odd.pencil_tma_launches() == 0     # nx odd: rows not 16-byte aligned
    odd.close()
    per = ops.Context(F.taylor_green(16))
    per.set_pencil_tma(True)
    assert per.pencil_tma_launches() == 0     # the cyclic scheme keeps its loads
    per.close()


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
