"""ctypes binding of libgbx.so (the C ABI declared in include/gbx.h)."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbx.so")

_i = ctypes.c_int
_d = ctypes.c_double
_p = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); every symbol declared in include/gbx.h
SIGNATURES = {
    "gbx_last_error": (ctypes.c_char_p, []),
    "gbx_version": (ctypes.c_char_p, []),
    "gbx_transpose": (_i, [_p, _p, _p, _i, _p, _p]),
    "gbx_transpose_blocks": (_i, [_p, _p, _i, _p, _i, _p, _p]),
    "gbx_dltc_transpose": (_i, [_p, _p, _p, _p, _i, _p, _p]),
    "gbx_local_contraction": (_i, [_i, _i, _i, _p, _p, _p, _i, _i, _d, _p]),
    "gbx_local_contraction_noalloc": (_i, [_i, _i, _i, _p, _p, _p, _i, _i, _d, _p]),
    "gbx_dltc_compute": (_i, [_p, _p, _p, _i, _i, _i, _p]),
    "gbx_create_big_matrix": (_i, [_i, _p, _p, _i, _p, _p, _i, _i, _i, _p, _ip, _ip, _p]),
    "gbx_rrr_unique_tiles": (_i, [_i, ctypes.c_char_p, _p, _p, _i, _ip, _p]),
    "gbx_rrr_initialize": (_i, [_i, _p, _p, _i, ctypes.c_int64, _p, _p]),
    "gbx_create_big_matrix_nl": (_i, [_i, _p, _p, _i, _p, _i, _p, _i, _i, _i, _p, _p, _i, _p, _ip, _ip, _p]),
    "gbx_revert_big_matrix": (_i, [_i, _p, _p, _i, _p, _i, _i, _i, _p, _p, _p]),
    "gbx_plan_create": (_i, [_p, _p, _p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _i, _i, _i,
                             ctypes.POINTER(_p)]),
    "gbx_execute": (_i, [_p, _p, _p, _p, _d, _p]),
    "gbx_plan_flops": (_d, [_p]),
    "gbx_plan_destroy": (_i, [_p]),
    "gbx_grouped_gemm_f64": (_i, [_p, _i, _p]),
    "gbx_group_create": (_i, [_p, _i, _i, _i, ctypes.POINTER(_p)]),
    "gbx_group_execute": (_i, [_p, _i, _p]),
    "gbx_group_autotune": (_i, [_p, _i, _p]),
    "gbx_group_info": (_i, [_p, _p, _p, ctypes.POINTER(_d)]),
    "gbx_group_destroy": (_i, [_p]),
    "gbx_server_create": (_i, [_p, ctypes.POINTER(_p)]),
    "gbx_server_add_job": (_i, [_p, _p, ctypes.POINTER(_i), ctypes.POINTER(_d)]),
    "gbx_server_submit": (_i, [_p, _i, _d]),
    "gbx_server_run": (_i, [_p, _d]),
    "gbx_server_results": (_i, [_p, _p, ctypes.POINTER(_i)]),
    "gbx_server_stats": (_i, [_p, _p]),
    "gbx_server_destroy": (_i, [_p]),
    "gbx_split_gemm": (_i, [_p, _p, _p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _i, _p]),
    "gbx_split_set_width": (_i, [_i]),
    "gbx_wait_selftest": (_i, [ctypes.c_longlong, _p]),
    "gbx_cc_default_config": (None, [_p]),
    "gbx_cc_footprint": (_i, [_p, ctypes.POINTER(_d), ctypes.POINTER(_d), ctypes.POINTER(_d)]),
    "gbx_cc_capture": (_i, [_p]),
    "gbx_cc_plan_info": (_i, [_p, _i, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "gbx_cc_check": (_i, [_p]),
    "gbx_cc_create": (_i, [_p, _p, ctypes.POINTER(_p)]),
    "gbx_cc_enqueue": (_i, [_p, _i, _p]),
    "gbx_cc_iterate": (_i, [_p, _i, _p, _p]),
    "gbx_cc_energies": (_i, [_p, _p, _ip]),
    "gbx_cc_stats_get": (_i, [_p, _p]),
    "gbx_cc_get_orbitals": (_i, [_p, _p, _p]),
    "gbx_cc_get_amplitudes": (_i, [_p, _p, _p, _p]),
    "gbx_cc_destroy": (_i, [_p]),
    "gbx_cc_gemm_shapes": (_i, [_p, _p, _ip]),
    "gbx_cc_amplitude_elems": (_i, [_p, _p, _p]),
    "gbx_cc_set_amplitudes": (_i, [_p, _p, _p, _p]),
    "gbx_cc_read_energy": (_i, [_p, _p, _p]),
    "gbx_cc_save_amplitudes": (_i, [_p, _p, _p, _p]),
    "gbx_cc_profile": (_i, [_p, _i, _p, _p, _p, _p, _p, _p, _i, _ip, _p]),
    "gbx_cc_time_gemm": (_i, [_p, _i, _i, _p, _p, _p, _p, _p]),
    "gbx_cc_contraction_error": (_i, [_p, _i, _p, _p, _p]),
    "gbx_cc_program_info": (_i, [_p, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "gbx_cc_program_selftest": (_i, [ctypes.c_longlong, _p]),
    "gbx_dltc_mul_orders": (_i, [_i, _p, _i, _p, _p, _p, _p, _p, _p, _p]),
    "gbx_dltc_task_mul": (_i, [_d, _i, _p, _p, _i, _p, _p, _i, _p, _p, _p, _p, _p, _i, _p]),
    "gbx_dltc_task_sum": (_i, [_d, _i, _p, _p, _i, _p, _p, _p, _p, _p, _p]),
    "gbx_dltc_table": (_i, [_i, _p, _p, _p, _p, _p, _i]),
    "gbx_dltc_program_create": (_i, [_i, _p, _i, ctypes.POINTER(_p)]),
    "gbx_dltc_program_tensor": (_i, [_p, _i, _p, _p]),
    "gbx_dltc_program_run": (_i, [_p, _i, _i, _p]),
    "gbx_dltc_program_check": (_i, [_p]),
    "gbx_dltc_program_flops": (_d, [_p]),
    "gbx_dltc_program_destroy": (_i, [_p]),
}

_lib = None


class GbxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gbx error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libgbx.so; raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbx.so is not built: run `python -m dtcf_gb300.build` (path %s)" % LIB_PATH)
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(rc):
    if rc != 0:
        raise GbxError(rc, lib().gbx_last_error().decode())
    return rc
