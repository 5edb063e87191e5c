"""ctypes binding of libemix_gb300.so (the C ABI declared in include/emix_gb300.h).

The library is the product: there is no Python or CPU fallback.  Importing
this module loads the in-tree shared library and raises if it is missing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libemix_gb300.so"

EMIX_OK = 0
EMIX_ERR_ALLOC = 3
STATUS_NAMES = {0: "EMIX_OK", 1: "EMIX_ERR_ARG", 2: "EMIX_ERR_CUDA", 3: "EMIX_ERR_ALLOC",
                4: "EMIX_ERR_UNSUPPORTED", 5: "EMIX_ERR_TIMEOUT"}

dp = C.POINTER(C.c_double)
vp = C.c_void_p
i3 = C.c_int * 3


class EmixError(RuntimeError):
    def __init__(self, rc: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(rc, rc)}: {msg}")
        self.rc = rc


class EmixImpeller(C.Structure):
    _fields_ = [
        ("on", C.c_int), ("nblades", C.c_int), ("omega", C.c_double), ("theta0", C.c_double),
        ("r1", C.c_double), ("r2", C.c_double), ("z1", C.c_double), ("z2", C.c_double),
        ("half_thick", C.c_double), ("hub_r", C.c_double), ("hub_z1", C.c_double),
        ("hub_z2", C.c_double), ("shaft_r", C.c_double), ("shaft_z0", C.c_double),
        ("shaft_z1", C.c_double), ("interp", C.c_int),
    ]


class EmixObjective(C.Structure):
    _fields_ = [("r_in", C.c_double), ("r_out", C.c_double), ("eps", C.c_double),
                ("w_ke", C.c_double), ("w_if", C.c_double)]


class EmixParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("scheme", C.c_int * 3),
        ("h", C.c_double * 3),
        ("sgs_model", C.c_int),
        ("cs", C.c_double), ("amu0", C.c_double), ("c4", C.c_double),
        ("mach", C.c_double), ("dt", C.c_double),
        ("level_set", C.c_int), ("ls_ghost", C.c_int), ("ref_bugs", C.c_int),
        ("bc_walls", C.c_int), ("filter_every", C.c_int), ("cfilt", C.c_double),
        ("imp", EmixImpeller), ("t0", C.c_double),
    ]


# name -> (restype, argtypes); the order follows include/emix_gb300.h
PROTOTYPES = {
    "emix_last_error": (C.c_char_p, []),
    "emix_version": (C.c_char_p, []),
    "cudaDeriv": (None, [vp, vp, vp, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                         C.c_int, C.c_int, C.c_int]),
    "cuDivergence": (None, [vp] * 9 + [C.c_double] * 3 + [C.c_int] * 3),
    "emix_set_legacy_scheme": (C.c_int, [C.c_int]),
    "emix_deriv_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, C.c_double,
                                 C.c_int, C.c_int, C.c_int, vp]),
    "emix_deriv_pcr_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, C.c_double, C.c_int,
                                     C.c_int, C.c_int, C.c_int, vp]),
    "emix_cudaDeriv": (C.c_int, [i3, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.c_int, C.c_int]),
    "emix_cudaDeriv_dev": (C.c_int, [i3, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                                     C.c_int, C.c_int, C.c_int, vp]),
    "emix_cuDivergence": (C.c_int, [i3] + [vp] * 9 + [C.c_double] * 3 + [C.c_int] * 3),
    "emix_cuDivergence_dev": (C.c_int, [i3] + [vp] * 9 + [C.c_double] * 3 + [C.c_int] * 3 + [vp]),
    "emix_flux_dev": (C.c_int, [C.c_int] + [vp] * 12 + [C.c_int] * 3 + [vp]),
    "emix_sgs_setup_dev": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp]),
    "emix_sgs_viscosity_dev": (C.c_int, [C.c_int, C.c_double, C.c_double] + [vp] * 7 +
                               [C.c_int] * 3 + [vp]),
    "emix_weno5_advect_dev": (C.c_int, [vp, vp, vp] + [C.c_double] * 4 + [C.c_int] * 4 + [vp]),
    "emix_weno5_advect": (C.c_int, [vp, vp, vp] + [C.c_double] * 4 + [C.c_int] * 4),
    "emix_impeller_force_dev": (C.c_int, [vp, vp, C.POINTER(EmixImpeller), C.c_double, C.c_int,
                                          C.c_int, C.c_int, vp, vp]),
    "emix_deriv_t_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, C.c_double, C.c_int, C.c_int,
                                   C.c_int, C.c_int, vp]),
    "emix_deriv_t_tma_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, C.c_double, C.c_int, C.c_int,
                                       C.c_int, C.c_int, vp]),
    "emix_adj_create": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(EmixObjective), C.POINTER(vp)]),
    "emix_adj_destroy": (C.c_int, [vp]),
    "emix_adj_device_bytes": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
    "emix_adj_set_overlap": (C.c_int, [vp, C.c_int]),
    "emix_adj_forward": (C.c_int, [vp, C.POINTER(C.c_double)]),
    "emix_adj_backward": (C.c_int, [vp, C.POINTER(C.c_double)]),
    "emix_adj_state_gradient": (C.c_int, [vp, vp, vp]),
    "emix_ctx_set_forcing": (C.c_int, [vp, C.c_double, C.c_double]),
    "emix_reinit_dev": (C.c_int, [vp, vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                  C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, vp]),
    "emix_write_field": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp]),
    "emix_read_field": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp]),
    "emix_write_time": (C.c_int, [C.c_char_p, C.c_double, C.c_int]),
    "emix_read_time": (C.c_int, [C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "emix_write_array": (C.c_int, [C.c_char_p, vp, C.c_long]),
    "emix_read_array": (C.c_int, [C.c_char_p, vp, C.c_long]),
    "emix_read_sobject": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, vp]),
    "emix_filtrado_dev": (C.c_int, [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, vp]),
    "emix_filter_dev": (C.c_int, [vp, C.c_int, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, vp]),
    "advect_CUDA": (None, [vp, vp, vp] + [C.c_double] * 3 + [C.c_int] * 3 + [C.c_double]),
    "emix_advect_extrapolate": (C.c_int, [vp, vp, vp] + [C.c_double] * 3 + [C.c_int] * 3 +
                                [C.c_double]),
    "emix_advect_extrapolate_dev": (C.c_int, [vp, vp, vp] + [C.c_double] * 3 + [C.c_int] * 3 +
                                    [C.c_double, vp]),
    "emix_extrapolate_dev": (C.c_int, [vp, vp, vp] + [C.c_double] * 3 + [C.c_int] * 3 +
                             [C.c_double, C.c_int, C.c_int, vp]),
    "emix_weno5_advect_dev_noalloc": (C.c_int, [vp, vp, vp] + [C.c_double] * 4 + [C.c_int] * 4
                                      + [vp]),
    "emix_ghost_pad_dev": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, vp]),
    "emix_ghost_unpad_dev": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]),
    "emix_ctx_create": (C.c_int, [C.POINTER(EmixParams), C.POINTER(vp)]),
    "emix_ctx_destroy": (C.c_int, [vp]),
    "emix_ctx_set_stream": (C.c_int, [vp, vp]),
    "emix_ctx_set_static": (C.c_int, [vp, vp, vp, vp]),
    "emix_ctx_upload": (C.c_int, [vp, vp, vp]),
    "emix_ctx_download": (C.c_int, [vp, vp, vp]),
    "emix_ctx_state": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "emix_step": (C.c_int, [vp, C.c_int, C.c_int]),
    "emix_ctx_set_overlap": (C.c_int, [vp, C.c_int]),
    "emix_ctx_set_fusion": (C.c_int, [vp, C.c_int]),
    "emix_ctx_set_tma": (C.c_int, [vp, C.c_int]),
    "emix_ctx_tma_stages": (C.c_int, [vp]),
    "emix_weno_tma_timeouts": (C.c_int, [C.POINTER(C.c_int)]),
    "emix_weno_tma_test_drop": (C.c_int, [C.c_int]),
    "emix_ctx_set_pencil_tma": (C.c_int, [vp, C.c_int]),
    "emix_ctx_pencil_tma_launches": (C.c_int, [vp]),
    "emix_pencil_tma_timeouts": (C.c_int, [C.POINTER(C.c_int)]),
    "emix_pencil_tma_test_drop": (C.c_int, [C.c_int]),
    "emix_ctx_get_step_index": (C.c_int, [vp, C.POINTER(C.c_long)]),
    "emix_ctx_set_step_index": (C.c_int, [vp, C.c_long]),
    "emix_ctx_set_time": (C.c_int, [vp, C.c_double]),
    "emix_ctx_get_time": (C.c_int, [vp, C.POINTER(C.c_double)]),
    "emix_step_host": (C.c_int, [vp, vp, vp, C.c_int]),
    "emix_ctx_launches_per_step": (C.c_int, [vp]),
    "emix_ctx_device_bytes": (C.c_longlong, [vp]),
    "emix_ctx_profile": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "emix_profile_class_count": (C.c_int, []),
    "emix_profile_class_name": (C.c_char_p, [C.c_int]),
    "emix_fp64_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "emix_pencil_set_yz_block": (C.c_int, [C.c_int]),
    "emix_math_selftest_dev": (C.c_int, [vp, vp, C.c_long, vp]),
    "emix_bc_walls_dev": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp]),
    "emix_cfl_dev": (C.c_int, [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int,
                               C.POINTER(C.c_double), vp]),
    "emix_tstep_dt": (C.c_int, [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "emix_metrics_dev": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_int, C.c_int, C.c_int, vp]),
    "emix_batch_create": (C.c_int, [C.c_int, C.POINTER(EmixParams), C.POINTER(vp)]),
    "emix_batch_destroy": (C.c_int, [vp]),
    "emix_batch_grid": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
    "emix_batch_set_stream": (C.c_int, [vp, vp]),
    "emix_batch_step": (C.c_int, [vp, C.c_int, C.c_int]),
    "emix_batch_step_per_grid": (C.c_int, [vp, C.c_int, C.c_int]),
    "emix_batch_set_tuning": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
    "emix_batch_get_tuning": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    "emix_batch_autotune": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
    "emix_batch_set_pcr": (C.c_int, [vp, C.c_int]),
    "emix_batch_set_overlap": (C.c_int, [vp, C.c_int]),
    "emix_batch_get_pcr": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "emix_batch_pcr_positions": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "emix_batch_autotune_pcr_ms": (C.c_int, [vp, C.POINTER(C.c_double)]),
}

_lib = None


def load(path: Path | str | None = None):
    """Load the library once; raises ``RuntimeError`` if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, where: str):
    if rc != EMIX_OK:
        msg = load().emix_last_error()
        raise EmixError(rc, where, msg.decode() if msg else "")
