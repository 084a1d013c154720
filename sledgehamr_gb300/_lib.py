"""ctypes binding of libsledgehamr_gb300.so (include/sledgehamr_gb300.h).

The library is the only compute path of this package: loading fails loudly
when it has not been built (run ``python -c "import __graft_entry__ as g;
g.build()"`` or ``python sledgehamr_gb300/build.py``).
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsledgehamr_gb300.so")

SH_OK = 0
SH_ERR_ARG = -1
SH_ERR_PROJECT = -2
SH_ERR_CUDA = -3
SH_ERR_NOMEM = -4
SH_ERR_UNSUPPORTED = -5
SH_ERR_TIMEOUT = -6
SH_ERR_NONFINITE = -7

SH_TAG_STATIC_MAX_CELLS = 1 << 22

SH_FAMILY_AXION_LAP1 = 1
SH_FAMILY_AXION_LAP2 = 2
SH_FAMILY_FOPT_GW = 3
SH_PREC_FP64 = 0
SH_PREC_FP32_KAHAN = 1
SH_PREC_FP32 = 2

SH_OUT_COMPONENT = 0
SH_OUT_COMPONENT_SQ = 1
SH_OUT_A_PRIME2 = 2
SH_OUT_A_PRIME_SCREENED = 3
SH_OUT_R_PRIME2 = 4

SH_NEW = 0
SH_OLD = 1
SH_ADVANCE_NO_SWAP = 1

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
llp = C.POINTER(C.c_longlong)
vp = C.c_void_p


class ShBox(C.Structure):
    _fields_ = [("lo", C.c_int * 3), ("hi", C.c_int * 3)]


class ShAmrConfig(C.Structure):
    _fields_ = [("project", C.c_int), ("with_gw", C.c_int), ("integrator", C.c_int),
                ("nghost", C.c_int), ("N0", C.c_int), ("max_level", C.c_int),
                ("blocking_factor", C.c_int), ("max_grid_size", C.c_int),
                ("n_error_buf", C.c_int), ("record_regrids", C.c_int),
                ("L", C.c_double), ("cfl", C.c_double), ("t_start", C.c_double),
                ("regrid_dt", C.c_double), ("string_width_threshold", C.c_double),
                ("string_lambda", C.c_double), ("te_crit", C.c_double * 32),
                ("params", C.c_double * 32), ("nparams", C.c_int),
                ("gw_params", C.c_double * 16), ("ngw", C.c_int), ("clustering", C.c_int),
                ("grid_eff", C.c_double), ("params_tag", C.c_double * 32),
                ("nparams_tag", C.c_int), ("params_mod", C.c_double * 32),
                ("nparams_mod", C.c_int), ("params_mod_norm0", C.c_int),
                ("check_finite", C.c_int), ("max_local_regrids", C.c_int),
                ("volume_threshold_strong", C.c_double), ("volume_threshold_weak", C.c_double),
                ("precision", C.c_int)]


class ShRequest(C.Structure):
    _fields_ = [("N", C.c_int), ("dx", C.c_double), ("dt", C.c_double), ("t_end", C.c_double),
                ("params", C.c_double * 4), ("nbubbles", C.c_int), ("xyz", C.c_void_p),
                ("profile", C.c_void_p), ("nbins", C.c_int), ("inv_dx", C.c_double),
                ("Lcut", C.c_double), ("zero_padding", C.c_int), ("projection_type", C.c_int),
                ("unbinned", C.c_int), ("max_level", C.c_int), ("blocking_factor", C.c_int),
                ("max_grid_size", C.c_int), ("te_crit", C.c_double * 2),
                ("regrid_dt", C.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "sh_ctx_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
    "sh_ctx_destroy": (C.c_int, [vp]),
    "sh_ctx_last_error": (C.c_char_p, [vp]),
    "sh_ctx_set_stream": (C.c_int, [vp, vp]),
    "sh_ctx_stream": (vp, [vp]),
    "sh_ctx_synchronize": (C.c_int, [vp]),
    "sh_ctx_kernel_launches": (C.c_longlong, [vp]),
    "sh_ctx_profile": (C.c_int, [vp, C.c_int]),
    "sh_ctx_profile_read": (C.c_int, [vp, C.c_char_p, dp, llp]),
    "sh_project_count": (C.c_int, []),
    "sh_project_name": (C.c_char_p, [C.c_int]),
    "sh_project_find": (C.c_int, [C.c_char_p, ip]),
    "sh_project_ncomp": (C.c_int, [C.c_int, C.c_int, ip, ip]),
    "sh_project_comp_name": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_char_p)]),
    "sh_level_project": (C.c_int, [vp, ip, ip]),
    "sh_h5_create": (C.c_int, [C.POINTER(vp)]),
    "sh_h5_destroy": (C.c_int, [vp]),
    "sh_h5_last_error": (C.c_char_p, [vp]),
    "sh_h5_add": (C.c_int, [vp, C.c_char_p, C.c_int, vp, C.c_longlong]),
    "sh_h5_count": (C.c_int, [vp, llp]),
    "sh_h5_write": (C.c_int, [vp, C.c_char_p]),
    "sh_output_level": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]),
    "sh_output_slices": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, vp]),
    "sh_output_level_host": (C.c_int, [C.POINTER(ShBox), C.c_int, C.c_int, vp,
                                       C.POINTER(C.c_char_p), C.c_double, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.c_int, vp]),
    "sh_output_slices_host": (C.c_int, [C.POINTER(ShBox), C.c_int, C.c_int, vp,
                                        C.POINTER(C.c_char_p), C.c_double, C.c_int, C.c_int,
                                        C.c_int, vp, vp]),
    "sh_level_create": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, C.POINTER(ShBox), C.c_int,
                                  C.c_int, C.POINTER(vp)]),
    "sh_level_create_prec": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, C.POINTER(ShBox), C.c_int,
                                       C.c_int, C.c_int, C.POINTER(vp)]),
    "sh_level_precision": (C.c_int, [vp, ip]),
    "sh_level_destroy": (C.c_int, [vp, vp]),
    "sh_level_info": (C.c_int, [vp, ip, ip, llp]),
    "sh_level_time": (C.c_int, [vp, C.c_int, dp, ip]),
    "sh_level_set_time": (C.c_int, [vp, C.c_int, C.c_double, C.c_int]),
    "sh_level_boxes": (C.c_int, [vp, C.POINTER(ShBox), C.c_int, ip]),
    "sh_level_set_index": (C.c_int, [vp, C.c_int]),
    "sh_ensemble_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, C.POINTER(vp)]),
    "sh_ensemble_destroy": (C.c_int, [vp]),
    "sh_ensemble_last_error": (C.c_char_p, [vp]),
    "sh_ensemble_info": (C.c_int, [vp, ip, ip, ip, ip, llp, llp, ip]),
    "sh_ensemble_kernel_launches": (C.c_longlong, [vp]),
    "sh_ensemble_set_time": (C.c_int, [vp, C.c_double]),
    "sh_ensemble_time": (C.c_int, [vp, dp]),
    "sh_ensemble_write": (C.c_int, [vp, C.c_int, vp]),
    "sh_ensemble_read": (C.c_int, [vp, C.c_int, vp]),
    "sh_ensemble_set_graph": (C.c_int, [vp, C.c_int]),
    "sh_ensemble_step": (C.c_int, [vp, C.c_double, C.c_int]),
    "sh_ensemble_tune": (C.c_int, [vp, C.c_int, C.c_double, ip]),
    "sh_ensemble_energy": (C.c_int, [vp, vp]),
    "sh_ensemble_string_count": (C.c_int, [vp, vp]),
    "sh_ensemble_create_pool": (C.c_int, [vp, C.c_int, C.c_int, C.c_longlong, C.POINTER(vp)]),
    "sh_ensemble_admit": (C.c_int, [vp, C.c_int, C.c_double, vp, C.c_double, ip]),
    "sh_ensemble_release": (C.c_int, [vp, C.c_int]),
    "sh_ensemble_pool_info": (C.c_int, [vp, llp, llp, llp, ip]),
    "sh_server_create": (C.c_int, [vp, C.c_int, C.c_longlong, C.POINTER(vp)]),
    "sh_server_destroy": (C.c_int, [vp]),
    "sh_server_last_error": (C.c_char_p, [vp]),
    "sh_server_submit": (C.c_int, [vp, C.POINTER(ShRequest), llp]),
    "sh_server_step": (C.c_int, [vp, ip, ip, ip]),
    "sh_server_status": (C.c_int, [vp, C.c_longlong, ip, vp]),
    "sh_server_result": (C.c_int, [vp, C.c_longlong, vp, vp, C.c_int, ip]),
    "sh_server_info": (C.c_int, [vp, ip, ip, llp, llp, llp]),
    "sh_level_domain": (C.c_int, [vp, vp, vp]),
    "sh_scalar_spectrum": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_double, vp, vp, C.c_int, ip]),
    "sh_projection": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]),
    "sh_ensemble_add_bubbles": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_double,
                                          C.c_double]),
    "sh_level_add_bubbles": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp,
                                       C.c_int, C.c_double, C.c_double, C.c_double]),
    "sh_ensemble_set_spectrum_precision": (C.c_int, [vp, C.c_int]),
    "sh_ensemble_gw_spectrum": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp,
                                          C.c_int, ip]),
    "sh_amr_config_defaults": (C.c_int, [C.POINTER(ShAmrConfig)]),
    "sh_amr_create": (C.c_int, [vp, C.POINTER(ShAmrConfig), vp, C.POINTER(vp)]),
    "sh_amr_destroy": (C.c_int, [vp, vp]),
    "sh_amr_step": (C.c_int, [vp, vp, C.c_int]),
    "sh_amr_info": (C.c_int, [vp, ip, llp, ip]),
    "sh_amr_set_tag_params": (C.c_int, [vp, vp, C.c_int, vp, C.c_int]),
    "sh_amr_set_timer_sync": (C.c_int, [vp, C.c_int]),
    "sh_amr_timer": (C.c_int, [vp, C.c_int, C.POINTER(C.c_char_p), dp, llp]),
    "sh_amr_level": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
    "sh_amr_set_trace": (C.c_int, [vp, C.c_int]),
    "sh_amr_checkpoint": (C.c_int, [vp, vp, C.c_char_p]),
    "sh_amr_restart": (C.c_int, [vp, C.POINTER(ShAmrConfig), C.c_char_p, C.POINTER(vp)]),
    "sh_amr_trace": (C.c_int, [vp, C.c_char_p, C.c_longlong, llp]),
    "sh_amr_regrid_record": (C.c_int, [vp, C.c_int, ip, dp, C.POINTER(ShBox), C.c_int, ip, vp,
                                       C.c_longlong, llp, C.POINTER(ShBox), C.c_int, ip]),
    "sh_level_write": (C.c_int, [vp, vp, C.c_int, C.c_int, vp]),
    "sh_level_read": (C.c_int, [vp, vp, C.c_int, C.c_int, vp]),
    "sh_level_reduce": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "sh_level_write_device": (C.c_int, [vp, vp, C.c_int, C.c_int, vp]),
    "sh_level_read_device": (C.c_int, [vp, vp, C.c_int, C.c_int, vp]),
    "sh_level_fill_patch": (C.c_int, [vp, vp, C.c_int]),
    "sh_level_set_coarse": (C.c_int, [vp, vp, vp]),
    "sh_level_fill_from": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double]),
    "sh_level_advance": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, C.c_double, C.c_double, vp,
                                   C.c_int, vp, C.c_int, C.c_int, vp, C.c_int]),
    "sh_level_rhs": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                               vp, C.c_int, vp, C.c_int, C.c_int, vp, vp]),
    "sh_average_down": (C.c_int, [vp, vp, C.c_int, vp, C.c_int]),
    "sh_average_down_te": (C.c_int, [vp, vp, vp]),
    "sh_tag_blocks": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                                vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, llp]),
    "sh_tag": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, vp, vp,
                         C.c_int, vp, C.c_int, vp, vp, vp, C.c_longlong, llp]),
    "sh_tag_static": (C.c_int, [vp, vp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                                vp, vp, C.c_int, vp, C.c_int, vp, vp, vp, C.c_longlong, llp]),
    "sh_spectrum_bins": (C.c_int, [C.c_int, vp, C.c_int, ip]),
    "sh_index_to_k": (C.c_int, [C.c_int, C.c_int, vp]),
    "sh_gw_spectrum": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int, ip]),
    "sh_probe_fp64_fma_rate": (C.c_int, [C.c_int, dp]),
    "sh_probe_wait_timeout": (C.c_int, [C.c_int, ip]),
    "sh_ensemble_set_staging": (C.c_int, [vp, C.c_int]),
    "sh_ensemble_staging": (C.c_int, [vp, ip]),
    "sh_level_check_finite": (C.c_int, [vp, vp, C.c_int, llp]),
    "sh_level_string_tags": (C.c_int, [vp, vp, C.c_double, C.c_int, C.c_double, C.c_double, vp,
                                       C.c_int, llp]),
    "sh_string_xi": (C.c_int, [C.c_longlong, C.c_double, C.c_double, C.c_double, dp]),
    "sh_evolve_periodic": (C.c_int, [vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_double,
                                     C.c_double, C.c_double, C.c_int, vp, C.c_int, vp, C.c_int,
                                     C.c_int, vp]),
}

_lib = None


def load() -> C.CDLL:
    """Loads the library once; raises if it is missing (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python sledgehamr_gb300/build.py)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
