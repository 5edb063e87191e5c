"""Shared helpers for the parity tests."""
import numpy as np

# normwise relative L-infinity tolerance for FP64 parity against the oracle
TOL = 1e-12


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = float(np.max(np.abs(b)))
    num = float(np.max(np.abs(a - b)))
    if den == 0.0:
        return num
    return num / den


def assert_close(a, b, tol=TOL, what=""):
    e = relerr(a, b)
    assert np.all(np.isfinite(np.asarray(a))), f"{what}: non-finite values"
    assert e <= tol, f"{what}: relative L-inf error {e:.3e} > {tol:.1e}"
    return e
