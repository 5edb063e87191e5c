"""The y/z compact derivative by parallel cyclic reduction + Thomas
(emix_deriv_pcr_dev, 2..5 PCR steps) against the oracle's serial solve
(solver/derivada.f90, src/MSVSingle/derivada_incomp.f90,
src/Schemes/derivCompact.cu:146-215 restated) at 1e-12, and against the
library's Thomas kernels, for every scheme, both axes and pencil lengths from
the shortest to the longest the PCR form takes (160 rows; 161 rejected)."""
import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import TOL, assert_close

pytestmark = pytest.mark.gpu

SCHEMES = [F.SCHEME_A, F.SCHEME_B, F.SCHEME_BPER, F.SCHEME_C]


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("axis", [1, 2])
@pytest.mark.parametrize("steps", [2, 3, 4, 5])
def test_pcr_matches_oracle(emix, oracle, scheme, axis, steps):
    for shape in ((19, 48, 33), (40, 23, 64), (9, 6, 7)):
        nx, ny, nz = shape
        w = F.random_box(nx, ny, nz, seed=31, periodic=(scheme == F.SCHEME_BPER))
        f = np.ascontiguousarray(w.um[1:4])
        h = w.grid.h(axis)
        got = _host(emix.deriv_pcr_dev(_dev(f), axis, h, steps, scheme))
        thomas = _host(emix.deriv_dev(_dev(f), axis, h, scheme))
        for c in range(3):
            ref = oracle.deriv3d(scheme, axis, f[c], h)
            assert_close(got[c], ref, what=f"scheme {scheme} axis {axis} steps {steps} {shape} comp {c}")
            assert_close(got[c], thomas[c], tol=1e-13, what=f"against Thomas, {shape} comp {c}")


@pytest.mark.parametrize("scheme", SCHEMES)
def test_pcr_longest_pencils_and_limit(emix, oracle, scheme):
    w = F.random_box(12, 160, 160, seed=32, periodic=(scheme == F.SCHEME_BPER))
    f = np.ascontiguousarray(w.um[1:3])
    for axis in (1, 2):
        h = w.grid.h(axis)
        for steps in (2, 5):
            got = _host(emix.deriv_pcr_dev(_dev(f), axis, h, steps, scheme))
            for c in range(2):
                assert_close(got[c], oracle.deriv3d(scheme, axis, f[c], h),
                             what=f"160 rows, axis {axis}, steps {steps}, comp {c}")
    too_long = np.zeros((1, 161, 6, 8))
    with pytest.raises(Exception, match="160"):
        emix.deriv_pcr_dev(_dev(too_long), 2, 0.1, 3, scheme)
