"""Level-set reinitialisation (cuReinitLsJB): the oracle against its
defining property, the device form against the oracle."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import assert_close


def _case(nxg, nyg, nzg, seed, scale=2.5):
    z, y, x = np.meshgrid(np.linspace(0, 1, nzg), np.linspace(0, 1, nyg), np.linspace(0, 1, nxg),
                          indexing="ij")
    d = np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2) - 0.25
    phi = scale * d * (1.0 + 0.3 * np.sin(5 * x)) + 1e-3 * F.uniform(seed, 0, d.shape)
    jbn = np.zeros((11,) + d.shape)
    for c in (0, 4, 8):
        jbn[c] = 1.0 + 0.05 * F.uniform(seed, 1 + c, d.shape)
    h = (1.0 / (nxg - 1), 1.0 / (nyg - 1), 1.0 / (nzg - 1))
    dm = np.full(d.shape, min(h))
    return np.ascontiguousarray(phi), np.ascontiguousarray(jbn), dm, h, d


def test_oracle_reinit_restores_unit_gradient(oracle):
    phi, jbn, dm, h, d = _case(30, 30, 30, 1)
    jbn[0] = jbn[4] = jbn[8] = 1.0
    out = oracle.reinit(phi, jbn, dm, h, 5, min(h), iters=20)
    g0 = np.sqrt(sum(q * q for q in np.gradient(phi, *h[::-1])))
    g1 = np.sqrt(sum(q * q for q in np.gradient(out, *h[::-1])))
    band = np.abs(d) < 0.1
    assert abs(np.mean(g1[band]) - 1.0) < 0.06 < abs(np.mean(g0[band]) - 1.0)
    # the zero level set stays put (to a fraction of a cell)
    assert np.max(np.abs(out[np.abs(d) < 0.02])) < 0.5 * min(h) * 3


@pytest.mark.gpu
@pytest.mark.parametrize("shape,ref_bugs,iters", [((30, 30, 30), 0, 10), ((26, 22, 19), 0, 4),
                                                  ((30, 30, 25), 1, 3)])
def test_reinit_matches_oracle(emix, oracle, shape, ref_bugs, iters):
    import torch
    phi, jbn, dm, h, _ = _case(*shape, seed=2)
    ref = oracle.reinit(phi, jbn, dm, h, 5, min(h), iters=iters, ref_bugs=ref_bugs)
    t = torch.from_numpy(phi.copy()).cuda()
    emix.reinit_dev(t, torch.from_numpy(jbn).cuda(), torch.from_numpy(dm).cuda(), h, 5, min(h),
                    iters=iters, ref_bugs=ref_bugs)
    torch.cuda.synchronize()
    assert_close(t.cpu().numpy(), ref, what="phi")
