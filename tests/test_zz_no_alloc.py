"""WENO5 level-set advection through the entry point that allocates no device
memory (emix_weno5_advect_dev_noalloc), checked against the allocating entry
point emix_weno5_advect_dev on two calls in a row.

The no-alloc entry point is for callers that cannot let a library call
cudaMalloc (it can block the whole device, and it fails when another
allocator already holds the memory); its scratch is a fixed 16 MiB array in
the library, which caps the padded grid at 1048576 cells.  This file is
collected last so that a failure here leaves every other test already run.
"""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import TOL, assert_close

pytestmark = pytest.mark.gpu


def _padded_case(nx, ny, nz, seed, g=5):
    from oracle import oracle_py as O
    w = F.random_box(nx, ny, nz, seed=seed)
    u = np.ascontiguousarray(w.um[1:4] / w.um[0])
    u[0] -= 0.3
    u[2] *= -1.0
    phig = O.ghost_pad(np.ascontiguousarray(w.phi), g)
    velg = np.ascontiguousarray(np.stack([O.ghost_pad(np.ascontiguousarray(u[c]), g)
                                          for c in range(3)]))
    jbng = np.zeros((11,) + phig.shape)
    for c in (0, 4, 8):
        jbng[c] = O.ghost_pad(np.ascontiguousarray(w.jbn[c]), g)
    h = tuple(w.grid.h(a) for a in range(3))
    return phig, velg, np.ascontiguousarray(jbng), h, 0.3 * min(h)


def _device(*arrays):
    import torch
    return [torch.from_numpy(a).cuda() for a in arrays]


def test_noalloc_matches_allocating_entry_on_two_calls(emix):
    import torch
    # the first call on a device loads the library's lazily loaded device code
    # (the static array's module and the stage kernels), which reserves device
    # memory once: a set-up call on the smallest grid comes first, so that both
    # checked calls must leave the free device memory unchanged
    phig, velg, jbng, h, dt = _padded_case(6, 6, 6, seed=40)
    p0, v0, j0 = _device(phig, velg, jbng)
    emix.weno5_advect_dev_noalloc(p0, v0, j0, h, dt, 0)
    torch.cuda.synchronize()
    cases = [(_padded_case(20, 18, 22, seed=41), 0), (_padded_case(30, 26, 24, seed=42), 1)]
    for call, ((phig, velg, jbng, h, dt), bugs) in enumerate(cases):
        phi_new, vel, jbn = _device(phig, velg, jbng)
        phi_ref = torch.from_numpy(phig).cuda()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        emix.weno5_advect_dev_noalloc(phi_new, vel, jbn, h, dt, bugs)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        emix.weno5_advect_dev(phi_ref, vel, jbn, h, dt, bugs)
        torch.cuda.synchronize()
        assert_close(phi_new.cpu().numpy(), phi_ref.cpu().numpy(), tol=TOL, what=f"call {call + 1}")
        assert free_after == free_before, f"call {call + 1}: the no-alloc entry point changed device memory use"


def test_noalloc_rejects_grids_beyond_the_static_limit(emix):
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    t = torch.zeros(8, device="cuda", dtype=torch.float64)
    p = t.data_ptr()
    rc = lib.emix_weno5_advect_dev_noalloc(p, p, p, 0.1, 0.1, 0.1, 0.01, 128, 128, 65, 0, None)
    assert rc == 1
    assert b"1048576" in lib.emix_last_error()
