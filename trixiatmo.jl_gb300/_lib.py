"""ctypes binding of the C ABI in include/trixiatmo_gpu.h.

This is the same binding a Julia `ccall` shim makes; it loads the in-tree
``_build/libtrixiatmo_gpu.so`` and raises if the library is missing — there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

TAG_OK = 0
TAG_E_INVALID = 1
TAG_E_CUDA = 2
TAG_E_NO_DEVICE = 3
TAG_E_STATE = 4
TAG_E_IO = 5

TAG_SOLVAR_CONS2CONS = 0
TAG_SOLVAR_CONS2PRIM = 1
TAG_SOLVAR_CONTRAVARIANT2GLOBAL = 2
TAG_SOLVAR_CONS2PRIM_AND_VORTICITY = 3
TAG_H5_INT64 = 0
TAG_H5_FLOAT64 = 1
TAG_H5_STRING = 2

TAG_S_NAN = 0x1
TAG_S_NEG_DENSITY = 0x2
TAG_S_NEG_PRESSURE = 0x4
TAG_S_NEWTON_MAXIT = 0x8

TAG_EQ_EULER_ENERGY_2D = 1
TAG_EQ_EULER_ENERGY_3D = 2
TAG_EQ_RAINY_2D = 3
TAG_VF_EC_RAIN = 2
TAG_VF_WEAK_FORM = 3
TAG_SF_LAX_FRIEDRICHS = 2
TAG_SRC_RAINY = 1
TAG_SRC_RAINY_CONVERGENCE = 2
TAG_BC_SIMPLE_SLIP_WALL = 3
TAG_BC_DIRICHLET = 4
TAG_EQ_MOIST_EULER_2D = 4
TAG_VF_CHANDRASHEKAR = 4
TAG_SF_CHANDRASHEKAR = 3
TAG_SRC_GEOPOTENTIAL = 3
TAG_SRC_MOIST_BUBBLE = 4
TAG_SRC_MOIST_CONVERGENCE_DRY = 5
TAG_SRC_MOIST_CONVERGENCE = 6
TAG_SRC_MOIST_GRAVITY_WAVE = 7
TAG_SRC_RAINY_NO_PHASE_CHANGE = 8
TAG_SRC_MOUNTAIN_WAVE = 9
TAG_EQ_COVARIANT_SWE = 5
TAG_EQ_POTENTIAL_TEMPERATURE_2D = 6
TAG_EQ_POTENTIAL_TEMPERATURE_3D = 7
TAG_EQ_INTERNAL_ENERGY_2D = 8
TAG_VF_IE_ETEC = 10
TAG_VF_PT_KG = 11
TAG_SF_IE_ES = 7
TAG_SF_PT_EC = 8
TAG_VF_PT_TEC = 7
TAG_VF_PT_EC = 8
TAG_VF_PT_ETEC = 9
TAG_VF_COV_CENTRAL = 5
TAG_VF_COV_EC = 6
TAG_SF_COV_EC = 4
TAG_SF_COV_EC_LLF = 5
TAG_SF_COV_CENTRAL = 6
TAG_RK_CK2N54 = 0
TAG_RK_SSPRK43 = 1
TAG_RK_SSPRK33 = 2
TAG_AQ_STATE = 0
TAG_AQ_ENTROPY = 1
TAG_AQ_ENERGY_TOTAL = 2
TAG_AQ_ENTROPY_TIMEDERIVATIVE = 3
MLP_PARAMS = 1293
MLP_TRAINABLE = 1281
TAG_VF_RANOCHA_WARUSZEWSKI = 1
TAG_SF_LMARS = 1
TAG_BC_SLIP_WALL_STRUCTURED = 1
TAG_BC_SLIP_WALL_NORMAL = 2

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class TagConfig(ctypes.Structure):
    _fields_ = [
        ("equations", ctypes.c_int32),
        ("volume_flux", ctypes.c_int32),
        ("surface_flux", ctypes.c_int32),
        ("polydeg", ctypes.c_int32),
        ("nelements", ctypes.c_int32),
        ("ninterfaces", ctypes.c_int32),
        ("nboundaries", ctypes.c_int32),
        ("nmembers", ctypes.c_int32),
        ("derivative_split", _dp),
        ("weights", _dp),
        ("contravariant_vectors", _dp),
        ("inverse_jacobian", _dp),
        ("node_coordinates", _dp),
        ("interface_elements", _ip),
        ("interface_faces", _ip),
        ("interface_flip", _ip),
        ("boundary_elements", _ip),
        ("boundary_faces", _ip),
        ("boundary_kinds", _ip),
        ("element_member", _ip),
        ("params", ctypes.c_double * 8),
        ("aux_node_vars", _dp),
    ]


class NewtonStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_int64), ("updates", ctypes.c_int64),
                ("fallbacks", ctypes.c_int64), ("not_converged", ctypes.c_int64)]


class AdaptiveStats(ctypes.Structure):
    _fields_ = [("accepted", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("dt_first", ctypes.c_double), ("dt_last", ctypes.c_double)]


_fp = ctypes.POINTER(ctypes.c_float)

# exported symbol -> (restype, argtypes)
class H5Attribute(ctypes.Structure):
    """tag_h5_attribute"""
    _fields_ = [("name", ctypes.c_char_p), ("type", ctypes.c_int32), ("i", ctypes.c_int64),
                ("d", ctypes.c_double), ("s", ctypes.c_char_p)]


class H5Dataset(ctypes.Structure):
    """tag_h5_dataset"""
    _fields_ = [("name", ctypes.c_char_p), ("data", _dp), ("count", ctypes.c_int64),
                ("var_name", ctypes.c_char_p)]


SIGNATURES = {
    "tag_create": (ctypes.c_int, [ctypes.POINTER(TagConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "tag_create_ensemble": (ctypes.c_int, [ctypes.POINTER(TagConfig), ctypes.c_int32,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "tag_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tag_ndofs_total": (ctypes.c_int64, [ctypes.c_void_p]),
    "tag_rhs": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int32]),
    "tag_set_state": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_get_state": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_state_device_ptr": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_dp)]),
    "tag_max_dt": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_max_dt_members": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_time_kernels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp]),
    "tag_rk_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                    ctypes.c_double, _dp]),
    "tag_rk_adaptive": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_int32,
                                        ctypes.c_int64, ctypes.c_void_p]),
    "tag_get_cta_threads": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "tag_set_tile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "tag_set_time_integrator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "tag_set_boundary_values": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_set_source": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, ctypes.c_int32]),
    "tag_analyze_integral": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_double, _dp]),
    "tag_analysis_nodes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), _dp]),
    "tag_analyze_errors": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp]),
    "tag_lgl_basis": (ctypes.c_int, [ctypes.c_int32, _dp, _dp]),
    "tag_cov_metric_terms": (ctypes.c_int, [_dp, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_int32, ctypes.c_int32, _dp, _dp, _dp, _dp]),
    "tag_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.c_int32]),
    "tag_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "tag_set_elements_per_block": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "tag_get_elements_per_block": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "tag_fp64_peak": (ctypes.c_int, [_dp]),
    "tag_shell_geometry": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int32, _dp, _dp, _dp,
                                          ctypes.c_int32, ctypes.c_double, ctypes.c_double, _dp,
                                          _dp, _dp]),
    "tag_eval_means": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                                      ctypes.c_double, _dp, _dp, _dp, _dp]),
    "tag_last_error": (ctypes.c_char_p, []),
    "tag_set_newton": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_int32, ctypes.c_int32]),
    "tag_newton_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _ip,
                                        ctypes.POINTER(NewtonStats)]),
    "tag_newton_solve_states": (ctypes.c_int, [_dp, ctypes.c_int64, ctypes.c_int32,
                                               ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                               _fp, _ip, ctypes.POINTER(NewtonStats)]),
    "tag_set_mlp": (ctypes.c_int, [ctypes.c_void_p, _fp]),
    "tag_set_newton_start": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "tag_newton_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.c_int32]),
    "tag_mlp_forward": (ctypes.c_int, [_fp, _fp, ctypes.c_int64, _fp]),
    "tag_mlp_loss_grad": (ctypes.c_int, [_fp, _fp, _fp, ctypes.c_int64, _fp, _fp]),
    "tag_mlp_train": (ctypes.c_int, [_fp, _fp, _fp, ctypes.c_int64, ctypes.c_int32,
                                     ctypes.c_int32, ctypes.c_float, ctypes.c_uint64, _fp]),
    "tag_rhs_noalloc": (ctypes.c_int, [ctypes.POINTER(TagConfig), _dp, _dp, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_uint32)]),
    "tag_set_state_sink": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tag_solution_variables": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                              _ip, ctypes.POINTER(ctypes.c_int64), _dp]),
    "tag_h5_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(H5Attribute), ctypes.c_int32,
                                    ctypes.POINTER(H5Dataset), ctypes.c_int32]),
}

_lib = None


class TagError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"trixiatmo_gpu error {code}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library; raises if it cannot be found or built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError(f"libtrixiatmo_gpu.so not built: {_build.LIB}")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int):
    if rc != TAG_OK:
        msg = load().tag_last_error()
        raise TagError(rc, msg.decode() if msg else "")
    return rc
