"""ctypes binding of libdnsmc.so (include/dnsmc.h).

The library is built in-tree by dnsmc_gb300.build (or __graft_entry__.build);
importing this module never falls back to anything else: a missing library is
an ImportError-like RuntimeError with the build command in the message.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

c_int_p = ctypes.POINTER(ctypes.c_int)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_uint32_p = ctypes.POINTER(ctypes.c_uint32)
c_int32_p = ctypes.POINTER(ctypes.c_int32)

OK = 0
ERR_ARG, ERR_STATE, ERR_CUDA, ERR_IO, ERR_TIMEOUT, ERR_NOMEM, ERR_TABLE, ERR_NODEVICE = 1, 2, 3, 4, 5, 6, 7, 8
STATUS_STEP_CAP, STATUS_NONFINITE, STATUS_BAD_FIELD, STATUS_COPY_TIMEOUT = 0x1, 0x2, 0x4, 0x8
RESULT_F64, RESULT_F32 = 0, 1
MODEL_CK, MODEL_GREY_BANDS, MODEL_PARTICLE, MODEL_GREY, MODEL_TABLE = 0, 1, 2, 3, 4
LAYOUT_DENSE, LAYOUT_FORTRAN = 0, 1
SAMPLER_IID, SAMPLER_RQMC = 0, 1
CV_BINS = 64  # DNSMC_CV_BINS: bins per hemisphere of the control variate's surrogate table


class Config(ctypes.Structure):
    """Mirror of dnsmc_config."""
    _fields_ = [
        ("imax", ctypes.c_int), ("jmax", ctypes.c_int), ("kmax", ctypes.c_int),
        ("p_row", ctypes.c_int),
        ("Lx", ctypes.c_float), ("Ly", ctypes.c_float), ("Lz", ctypes.c_float),
        ("stretched_x", ctypes.c_int),
        ("nvar", ctypes.c_int), ("photmax", ctypes.c_int),
        ("T_west", ctypes.c_float), ("T_east", ctypes.c_float),
        ("eps_west", ctypes.c_float), ("eps_east", ctypes.c_float),
        ("toll", ctypes.c_float), ("max_steps", ctypes.c_int), ("grid_num", ctypes.c_int),
        ("model", ctypes.c_int), ("kappa", ctypes.c_float), ("n_groups", ctypes.c_int),
        ("seed", ctypes.c_uint64), ("sampler", ctypes.c_int), ("local_sampling", ctypes.c_int),
        ("control_variate", ctypes.c_int), ("cv_moments", ctypes.c_int),
        ("block_threads", ctypes.c_int), ("tile_a", ctypes.c_int), ("mg_steps", ctypes.c_int),
    ]


class TableDesc(ctypes.Structure):
    """Mirror of dnsmc_table_desc."""
    _fields_ = [
        ("nbands", ctypes.c_int), ("nq", ctypes.c_int), ("nT", ctypes.c_int), ("nX", ctypes.c_int),
        ("T0", ctypes.c_float), ("dT", ctypes.c_float), ("X0", ctypes.c_float), ("dX", ctypes.c_float),
        ("k", c_float_p), ("wvc", c_float_p), ("dnu", c_float_p), ("wq", c_float_p), ("Ib", c_float_p),
        ("prob", c_float_p), ("probg", c_float_p), ("kP", c_float_p),
    ]


class LblDesc(ctypes.Structure):
    """Mirror of dnsmc_lbl_desc."""
    _fields_ = [
        ("nT", ctypes.c_int), ("nX", ctypes.c_int), ("npts", ctypes.c_longlong),
        ("wv0", ctypes.c_double), ("dwv", ctypes.c_double), ("kappa", ctypes.POINTER(ctypes.c_double)),
        ("nbands", ctypes.c_int), ("first", ctypes.POINTER(ctypes.c_longlong)), ("count", ctypes.POINTER(ctypes.c_int)),
        ("wv_left", ctypes.POINTER(ctypes.c_double)), ("wv_right", ctypes.POINTER(ctypes.c_double)),
        ("nq", ctypes.c_int), ("gq", ctypes.POINTER(ctypes.c_double)), ("n_pwrk", ctypes.c_int),
    ]


class CvNetConfig(ctypes.Structure):
    """Mirror of dnsmc_cvnet_config."""
    _fields_ = [
        ("n_groups", ctypes.c_int), ("T_center", ctypes.c_float), ("T_scale", ctypes.c_float),
        ("x_center", ctypes.c_float), ("x_scale", ctypes.c_float), ("lr", ctypes.c_float),
        ("adam_beta1", ctypes.c_float), ("adam_beta2", ctypes.c_float), ("adam_eps", ctypes.c_float),
        ("ridge", ctypes.c_float), ("batch", ctypes.c_int), ("seed", ctypes.c_uint64),
    ]


CVNET_NFEAT, CVNET_NOUT, CVNET_NLABEL = 67, 64, 8
CVNET_BETA, CVNET_RAYS = 1, 2

# name -> (restype, argtypes); every symbol include/dnsmc.h declares
SIGNATURES = {
    "dnsmc_set_default_config": (None, [ctypes.POINTER(Config)]),
    "dnsmc_config_from_env": (ctypes.c_int, [ctypes.POINTER(Config)]),
    "dnsmc_last_error": (ctypes.c_char_p, []),
    "dnsmc_version": (ctypes.c_char_p, []),
    "dnsmc_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)]),
    "dnsmc_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dnsmc_load_tables_ref": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int]),
    "dnsmc_use_grey_band_tables": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                  ctypes.c_float]),
    "dnsmc_set_table": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(TableDesc)]),
    "dnsmc_get_table_info": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_float_p,
                                            c_float_p, c_float_p, c_float_p]),
    "dnsmc_get_table": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p,
                                       c_float_p]),
    "dnsmc_set_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, c_float_p, ctypes.c_int]),
    "dnsmc_set_fields_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "dnsmc_set_region": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_int] * 6),
    "dnsmc_set_rays": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p]),
    "dnsmc_packet_count": (ctypes.c_int, [ctypes.c_void_p, c_int_p]),
    "dnsmc_packet_shape": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p]),
    "dnsmc_set_rays_per_item": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_int_p]),
    "dnsmc_get_item_steps": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dnsmc_get_rays_per_item": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p]),
    "dnsmc_get_cv_beta": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "dnsmc_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dnsmc_set_graph": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dnsmc_get_coarse_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, c_float_p]),
    "dnsmc_get_graph_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "dnsmc_set_rays_adaptive": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_int]),
    "dnsmc_set_particles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_float_p, c_float_p, ctypes.c_float]),
    "dnsmc_set_particle_field": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_int]),
    "dnsmc_cvnet_default_config": (None, [ctypes.POINTER(CvNetConfig)]),
    "dnsmc_cvnet_create": (ctypes.c_int, [ctypes.POINTER(CvNetConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "dnsmc_cvnet_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dnsmc_cvnet_param_count": (ctypes.c_longlong, []),
    "dnsmc_cvnet_get_params": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p]),
    "dnsmc_cvnet_set_params": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p]),
    "dnsmc_cvnet_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dnsmc_cvnet_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "dnsmc_cvnet_features": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_float_p]),
    "dnsmc_cvnet_add_training_data": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dnsmc_cvnet_clear_training_data": (ctypes.c_int, [ctypes.c_void_p]),
    "dnsmc_cvnet_training_rows": (ctypes.c_longlong, [ctypes.c_void_p]),
    "dnsmc_cvnet_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p]),
    "dnsmc_cvnet_eval": (ctypes.c_int, [ctypes.c_void_p, c_float_p, ctypes.c_longlong, c_float_p]),
    "dnsmc_cvnet_gradient": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p, ctypes.c_int, ctypes.c_longlong,
                                            c_float_p, c_double_p]),
    "dnsmc_cvnet_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int]),
    "dnsmc_solve_async": (ctypes.c_int, [ctypes.c_void_p]),
    "dnsmc_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "dnsmc_get_results": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "dnsmc_save_table": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dnsmc_get_launch_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_longlong)]),
    "dnsmc_ck_from_lbl": (ctypes.c_int, [ctypes.POINTER(LblDesc), c_float_p, c_double_p]),
    "dnsmc_load_table": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dnsmc_set_result_type": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dnsmc_get_results_float": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p]),
    "dnsmc_get_group_results": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "dnsmc_status": (ctypes.c_int, [ctypes.c_void_p, c_uint32_p]),
    "dnsmc_get_counters": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p, c_double_p]),
    "dnsmc_get_timing": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "dnsmc_get_tmax": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "dnsmc_get_sampling": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_float_p, c_int_p,
                                          c_int_p, c_int_p, c_float_p, c_float_p]),
    "dnsmc_prepare_sampling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_float]),
    "dnsmc_set_cv_beta": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "dnsmc_get_cv_data": (ctypes.c_int, [ctypes.c_void_p, c_int_p, c_float_p, c_float_p, c_double_p, c_double_p]),
    "dnsmc_get_cv_table": (ctypes.c_int, [ctypes.c_void_p, c_float_p]),
    "dnsmc_get_cv_moments": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "dnsmc_get_geometry": (ctypes.c_int, [ctypes.c_void_p, c_float_p, c_float_p, c_float_p]),
    "dnsmc_trace_ray": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, c_int32_p, c_int_p, c_uint32_p]),
    "dnsmc_solve_grey_noalloc": (ctypes.c_int, [ctypes.POINTER(Config), c_float_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mc_gpu_": (None, [c_float_p, c_int_p]),
    "get_results_": (None, [c_float_p, c_float_p]),
    "dnsmc_dropin_configure": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p]),
    "dnsmc_dropin_release": (ctypes.c_int, []),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load the in-tree libdnsmc.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m dnsmc_gb300.build` "
                           "(the solver has no fallback implementation)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class DnsmcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dnsmc error {code}: {msg}")
        self.code = code


def launch_count() -> int:
    """Kernels the library has launched in this process (dnsmc_get_launch_count)."""
    n = ctypes.c_longlong()
    check(load().dnsmc_get_launch_count(ctypes.byref(n)))
    return n.value


def check(rc: int) -> None:
    if rc != OK:
        raise DnsmcError(rc, load().dnsmc_last_error().decode(errors="replace"))
