"""The kernels' own reciprocal and square-root routines (rcp_fast, sqrt_fast,
rsqrt_fast: third-order steps from single-precision seeds, with CUDA's
operators as the slow path outside the exponent range the steps handle)
against CUDA's 1.0/x, sqrt(x) and 1.0/sqrt(x), computed in the same kernel on
the same arguments (emix_math_selftest_dev).

Arguments: 10^7 random bit patterns (every sign, biased exponent and
mantissa, so zeros, subnormals, infinities and NaNs included) plus every
exponent edge where the routines switch paths.  On the fast path the result
is within one ulp of the correctly rounded value: CUDA's 1.0/x and sqrt(x)
are correctly rounded themselves, while 1.0/sqrt(x) rounds twice (the root,
then the quotient), so the reciprocal root is compared with 1/sqrt(x) in
extended precision (numpy.longdouble) rounded once to double, and with CUDA's
1.0/sqrt(x) within two ulps.  On the slow path each routine returns CUDA's
operator itself, bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_RANDOM = 10_000_000


def _arguments():
    rng = np.random.default_rng(20261204)
    bits = rng.integers(0, 2**63, size=N_RANDOM, dtype=np.int64).astype(np.uint64)
    bits |= rng.integers(0, 2, size=N_RANDOM, dtype=np.uint64) << np.uint64(63)
    edges = []
    mant = [0, 1, 2**51, 2**52 - 1, 0x5555555555555, 0xAAAAAAAAAAAAA]
    for e in (0, 1, 2, 3, 1022, 1023, 1024, 2042, 2043, 2044, 2045, 2046, 2047):
        for m in mant:
            for s in (0, 1):
                edges.append((s << 63) | (e << 52) | m)
    x = np.concatenate([bits, np.array(edges, dtype=np.uint64)]).view(np.float64)
    return np.ascontiguousarray(x)


def _ulps(a, b):
    """ulp distance of same-sign finite values (bit patterns are sign-magnitude)."""
    ia = a.view(np.int64) & np.int64(0x7FFFFFFFFFFFFFFF)
    ib = b.view(np.int64) & np.int64(0x7FFFFFFFFFFFFFFF)
    return np.abs(ia - ib)


def _same_bits(a, b):
    return (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))


def test_fast_reciprocal_and_roots_against_cuda(emix):
    import torch
    from emix_gb300 import _lib
    lib = _lib.load()
    x = _arguments()
    n = x.size
    xd = torch.from_numpy(x).cuda()
    out = torch.empty(6 * n, dtype=torch.float64, device="cuda")
    _lib.check(lib.emix_math_selftest_dev(xd.data_ptr(), out.data_ptr(), n, None),
               "emix_math_selftest_dev")
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(6, n)
    ebits = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    neg = (x.view(np.uint64) >> np.uint64(63)) == 1

    report = {}
    for name, fast, ref, lo, hi, allow_neg in (("rcp", o[0], o[1], 2, 2043, True),
                                               ("sqrt", o[2], o[3], 2, 2045, False),
                                               ("rsqrt", o[4], o[5], 2, 2045, False)):
        on = (ebits >= lo) & (ebits <= hi)
        if not allow_neg:
            on &= ~neg
        slow = ~on
        assert on.sum() > N_RANDOM // 3 and slow.sum() > 1000
        assert np.all(np.isfinite(fast[on])) and np.all(np.isfinite(ref[on]))
        assert np.all(np.signbit(fast[on]) == np.signbit(ref[on])), f"{name}: sign"
        if name == "rsqrt":
            xs = x[on].astype(np.longdouble)
            exact = (np.longdouble(1) / np.sqrt(xs)).astype(np.float64)
            uc = _ulps(fast[on], ref[on])
            assert uc.max() <= 2, f"rsqrt: {uc.max()} ulp from CUDA's 1.0/sqrt on the fast path"
            u = _ulps(fast[on], exact)
        else:
            u = _ulps(fast[on], ref[on])
        report[name] = (int(u.max()), float(np.mean(u != 0)))
        assert u.max() <= 1, f"{name}: {u.max()} ulp from the correctly rounded value on the fast path"
        same = _same_bits(fast[slow], ref[slow])
        assert same.all(), f"{name}: slow path differs from CUDA's operator"
    print("max ulp, fraction not bitwise equal:", report)
