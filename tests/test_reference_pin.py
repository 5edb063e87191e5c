"""The CPU oracle against outputs of the reference's own CUDA kernels.

tests/golden/reference_cuda.npz holds outputs of the reference's kernels
(compiled unmodified from its sources, run on a GB300 by
tests/golden/make_reference_golden.py): the variant-C compact derivative
(cu::cs::dFdX/Y/Z), cuDivergence, one cuAdvectLsJB WENO5 TVD-RK3 step (with
the reference's own z-top neighbour index), the advect_CUDA ghost padding and
advect_CUDA itself (pressure extrapolation into the solid).
The oracle must match them to 1e-12 (normwise relative L-inf), the padding
bitwise.  The GPU test at the end checks the CUDA library against the same
vectors.
"""
from pathlib import Path

import numpy as np
import pytest

from emix_gb300 import fields as F
from helpers import TOL, assert_close

GOLD = Path(__file__).resolve().parent / "golden" / "reference_cuda.npz"


@pytest.fixture(scope="module")
def gold():
    """Reference outputs plus the regenerated inputs (same seeds)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_reference_golden",
                                                  GOLD.parent / "make_reference_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = dict(np.load(GOLD))
    for name, f in mg.deriv_cases():
        g[f"{name}_in"] = f
    fl, jbn = mg.div_case()
    for q, a in enumerate(fl):
        g[f"div_in{q}"] = a
    g["div_jbn"] = jbn
    g["weno_phi"], g["weno_vel"], g["weno_jbn"], _, _ = mg.weno_case()
    g["pad_in"] = mg.pad_case()
    g["extrap_press"], g["extrap_jbn"], g["extrap_sobj"], g["extrap_delta"], g["extrap_dmin"] = \
        mg.extrap_case()
    (g["reinit_phi"], g["reinit_jbn"], g["reinit_dm"], g["reinit_h"], g["reinit_dmin"],
     g["reinit_iters"]) = mg.reinit_case()
    return g


def test_oracle_deriv_matches_reference_kernels(oracle, gold):
    for name in ("deriv0", "deriv1"):
        f = gold[f"{name}_in"]
        for axis in range(3):
            h = float(gold[f"{name}_h{axis}"])
            assert_close(oracle.deriv3d(F.SCHEME_C, axis, f, h), gold[f"{name}_a{axis}"], tol=TOL,
                         what=f"{name} axis {axis}")


def test_oracle_divergence_matches_reference_kernels(oracle, gold):
    fl = [gold[f"div_in{q}"] for q in range(6)]
    rs, rsv = oracle.cuDivergence(F.SCHEME_C, *fl, gold["div_jbn"], tuple(gold["div_h"]))
    assert_close(rs, gold["div_rs"], tol=TOL, what="rs")
    assert_close(rsv, gold["div_rsv"], tol=TOL, what="rsv")


def test_oracle_weno_matches_reference_kernels(oracle, gold):
    out = oracle.weno_advect(gold["weno_phi"], gold["weno_vel"], gold["weno_jbn"],
                             tuple(gold["weno_h"]), float(gold["weno_dt"]), ref_bugs=1)
    assert_close(out, gold["weno_out"], tol=TOL, what="phi after one step")


def test_oracle_padding_matches_reference_kernels(oracle, gold):
    assert np.array_equal(oracle.ghost_pad(gold["pad_in"], 5, 1.0), gold["pad_out"])


def test_oracle_extrapolation_matches_reference_kernels(oracle, gold):
    if "extrap_out" not in gold:
        pytest.skip("no advect_CUDA vectors in this golden file")
    out = oracle.advect_extrapolate(gold["extrap_press"], gold["extrap_jbn"], gold["extrap_sobj"],
                                    gold["extrap_delta"], gold["extrap_dmin"])
    # the extrapolation moves only the solid side, so compare the change too
    assert_close(out, gold["extrap_out"], tol=TOL, what="press")
    assert_close(out - gold["extrap_press"], gold["extrap_out"] - gold["extrap_press"], tol=1e-11,
                 what="change of press")


def test_oracle_reinit_matches_reference_kernels(oracle, gold):
    if "reinit_out" not in gold:
        pytest.skip("no cuReinitLsJB vectors in this golden file")
    out = oracle.reinit(gold["reinit_phi"], gold["reinit_jbn"], gold["reinit_dm"], gold["reinit_h"], 5,
                        gold["reinit_dmin"], iters=gold["reinit_iters"], ref_bugs=1)
    assert_close(out, gold["reinit_out"], tol=TOL, what="phi")


@pytest.mark.gpu
def test_cuda_reinit_matches_reference_kernels(emix, gold):
    import torch
    if "reinit_out" not in gold:
        pytest.skip("no cuReinitLsJB vectors in this golden file")
    t = torch.from_numpy(gold["reinit_phi"].copy()).cuda()
    emix.reinit_dev(t, torch.from_numpy(gold["reinit_jbn"]).cuda(), torch.from_numpy(gold["reinit_dm"]).cuda(),
                    gold["reinit_h"], 5, gold["reinit_dmin"], iters=gold["reinit_iters"], ref_bugs=1)
    torch.cuda.synchronize()
    assert_close(t.cpu().numpy(), gold["reinit_out"], tol=TOL, what="phi")


@pytest.mark.gpu
def test_cuda_extrapolation_matches_reference_kernels(emix, gold):
    if "extrap_out" not in gold:
        pytest.skip("no advect_CUDA vectors in this golden file")
    out = emix.advect_extrapolate(gold["extrap_press"], gold["extrap_jbn"], gold["extrap_sobj"],
                                  gold["extrap_delta"], gold["extrap_dmin"])
    assert_close(out, gold["extrap_out"], tol=TOL, what="press")
    assert_close(out - gold["extrap_press"], gold["extrap_out"] - gold["extrap_press"], tol=1e-11,
                 what="change of press")
    legacy = np.array(gold["extrap_press"], copy=True)
    emix.advect_CUDA_legacy(legacy, gold["extrap_jbn"], gold["extrap_sobj"], gold["extrap_delta"],
                            gold["extrap_dmin"])
    assert np.array_equal(legacy, out)


@pytest.mark.gpu
def test_cuda_library_matches_reference_kernels(emix, gold):
    import torch
    for name in ("deriv0", "deriv1"):
        f = gold[f"{name}_in"]
        for axis in range(3):
            h = float(gold[f"{name}_h{axis}"])
            got = emix.deriv_dev(torch.from_numpy(f).cuda(), axis, h, F.SCHEME_C).cpu().numpy()
            assert_close(got, gold[f"{name}_a{axis}"], tol=TOL, what=f"{name} axis {axis}")
    fl = [np.ascontiguousarray(gold[f"div_in{q}"]) for q in range(6)]
    rs, rsv = emix.cuDivergence(*fl, np.ascontiguousarray(gold["div_jbn"]), tuple(gold["div_h"]),
                                F.SCHEME_C)
    assert_close(rs, gold["div_rs"], tol=TOL, what="rs")
    assert_close(rsv, gold["div_rsv"], tol=TOL, what="rsv")
    out = emix.weno5_advect(np.ascontiguousarray(gold["weno_phi"]), np.ascontiguousarray(gold["weno_vel"]),
                            np.ascontiguousarray(gold["weno_jbn"]), tuple(gold["weno_h"]),
                            float(gold["weno_dt"]), 1)
    assert_close(out, gold["weno_out"], tol=TOL, what="phi after one step")
    pad = emix.ghost_pad_dev(torch.from_numpy(np.ascontiguousarray(gold["pad_in"])).cuda(), 5)
    assert np.array_equal(pad.cpu().numpy(), gold["pad_out"])
