"""The C ABI library loads on a CPU-only host and exports every entry point
that include/emix_gb300.h declares; argument checks fail with EMIX_ERR_ARG
before any CUDA call."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "emix_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \t\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))


@pytest.fixture(scope="module")
def lib():
    from emix_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        import emix_gb300.build as b
        b.build()
    return _lib.load()


def test_header_lists_the_reference_symbols():
    names = declared_functions()
    for n in ("cudaDeriv", "cuDivergence", "emix_step", "emix_weno5_advect_dev", "emix_ctx_create"):
        assert n in names
    assert len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_prototypes_cover_header(lib):
    from emix_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.PROTOTYPES)


def test_version(lib):
    assert b"sm_103a" in lib.emix_version()


def test_argument_errors_without_gpu(lib):
    from emix_gb300._lib import EmixParams, i3
    ERR_ARG = 1
    n = 4   # below the minimum pencil length
    a = np.zeros(64)
    p = a.ctypes.data
    assert lib.emix_cudaDeriv(i3(3, 3, 3), p, p, p, p, 0.1, 0.1, 0.1, n, 8, 8) == ERR_ARG
    assert lib.emix_cudaDeriv(i3(9, 3, 3), p, p, p, p, 0.1, 0.1, 0.1, 8, 8, 8) == ERR_ARG
    assert lib.emix_cudaDeriv(i3(3, 3, 3), p, p, p, p, -0.1, 0.1, 0.1, 8, 8, 8) == ERR_ARG
    assert lib.emix_deriv_dev(3, 3, 1, p, p, 0.1, 8, 8, 8, None) == ERR_ARG
    assert lib.emix_deriv_dev(3, 0, 7, p, p, 0.1, 8, 8, 8, None) == ERR_ARG
    assert lib.emix_cuDivergence(i3(3, 3, 3), None, p, p, p, p, p, p, p, p, 0.1, 0.1, 0.1,
                                 8, 8, 8) == ERR_ARG
    assert lib.emix_flux_dev(6, *([p] * 12), 8, 8, 8, None) == ERR_ARG
    assert lib.emix_weno5_advect(p, p, p, 0.1, 0.1, 0.1, 0.01, 5, 8, 8, 0) == ERR_ARG
    assert lib.emix_sgs_viscosity_dev(2, 0.1, 1e-3, None, p, p, p, None, None, p, 8, 8, 8,
                                      None) == ERR_ARG
    prm = EmixParams()
    prm.nx = prm.ny = prm.nz = 8
    for a_ in range(3):
        prm.scheme[a_] = 3
        prm.h[a_] = 0.1
    prm.mach = 0.1
    prm.dt = 0.0           # invalid
    h = C.c_void_p()
    assert lib.emix_ctx_create(C.byref(prm), C.byref(h)) == ERR_ARG
    prm.dt = 1e-3
    prm.level_set = 1
    prm.ls_ghost = 2       # fewer ghost layers than the WENO5 stencil needs
    assert lib.emix_ctx_create(C.byref(prm), C.byref(h)) == ERR_ARG
    assert lib.emix_step(None, 1, 0) == ERR_ARG
    # the adjoint's and the batch's stream switches, the TMA form of D^T and
    # the pencil copies' test hook: argument checks before any CUDA call
    assert lib.emix_adj_set_overlap(None, 1) == ERR_ARG
    assert lib.emix_batch_set_overlap(None, 3) == ERR_ARG
    assert lib.emix_deriv_t_tma_dev(3, 1, 7, p, p, 0.1, 8, 8, 8, 0, None) == ERR_ARG
    assert lib.emix_deriv_t_tma_dev(3, 1, 1, p, p, 0.1, 8, 8, 8, 2, None) == ERR_ARG
    assert lib.emix_deriv_t_tma_dev(3, 1, 1, p, p, -0.1, 8, 8, 8, 0, None) == ERR_ARG
    assert lib.emix_pencil_tma_test_drop(2) == ERR_ARG
    assert lib.emix_weno_tma_test_drop(2) == ERR_ARG
