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
