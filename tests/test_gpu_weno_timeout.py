"""The level-set stage's bounded waits for its TMA plane copies: with the
copies dropped (a test hook), every stage block gives up after its waits,
counts itself and returns, and the context stays usable afterwards."""
import numpy as np
import pytest

from emix_gb300 import fields as F

pytestmark = pytest.mark.gpu


def test_dropped_plane_copies_time_out_and_the_context_recovers(emix):
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    w = F.stirred_tank(n=24, impeller=True)
    a = emix.Context(w, bc_walls=1)
    b = emix.Context(w, bc_walls=1)
    b.set_tma(False)
    assert a.tma_stages() == 3
    before = emix.weno_tma_timeouts()
    _lib.check(lib.emix_weno_tma_test_drop(1), "emix_weno_tma_test_drop")
    try:
        a.step(1)
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.emix_weno_tma_test_drop(0), "emix_weno_tma_test_drop")
    assert emix.weno_tma_timeouts() > before
    # the same context, copies restored: bitwise the register-staged result
    after = emix.weno_tma_timeouts()
    a.upload(w.um, w.phi); a.time = 0.0
    b.upload(w.um, w.phi); b.time = 0.0
    a.step(2)
    b.step(2)
    ua, pa = a.download()
    ub, pb = b.download()
    assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
    assert emix.weno_tma_timeouts() == after
    a.close()
    b.close()


def test_step_host_reports_dropped_plane_copies_as_an_error(emix):
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    w = F.stirred_tank(n=24, impeller=True)
    a = emix.Context(w, bc_walls=1)
    assert a.tma_stages() == 3
    um = np.ascontiguousarray(w.um.copy())
    phi = np.ascontiguousarray(w.phi.copy())
    _lib.check(lib.emix_weno_tma_test_drop(1), "emix_weno_tma_test_drop")
    try:
        with pytest.raises(RuntimeError, match="TMA"):
            a.step_host(um, phi, 1)
        torch.cuda.synchronize()
    finally:
        _lib.check(lib.emix_weno_tma_test_drop(0), "emix_weno_tma_test_drop")
    # copies restored: the same call succeeds
    um = np.ascontiguousarray(w.um.copy())
    phi = np.ascontiguousarray(w.phi.copy())
    a.upload(w.um, w.phi); a.time = 0.0
    a.step_host(um, phi, 1)
    assert np.isfinite(um).all() and np.isfinite(phi).all()
    a.close()
