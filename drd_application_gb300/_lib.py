"""Loads libdrd_gb300.so and declares its C-ABI for ctypes.

There is no fallback: if the library is missing or fails to load, every entry point of
this package raises.  Build it with drd_application_gb300.build.build().
"""
import ctypes as C
import os

from . import abi
from .build import lib_path

_LIB = None

# Every symbol include/drd_gb300.h declares, with its ctypes signature.
_dp = C.POINTER(C.c_double)
_ctx = C.c_void_p
_st = C.POINTER(abi.drd_status)
SIGNATURES = {
    "drd_abi_version": (C.c_int, []),
    "drd_create": (C.c_int, [C.POINTER(abi.drd_params), C.POINTER(C.c_void_p)]),
    "drd_destroy": (C.c_int, [_ctx]),
    "drd_set_params": (C.c_int, [_ctx, C.POINTER(abi.drd_params)]),
    "drd_last_error": (C.c_char_p, [_ctx]),
    "drd_set_coefs": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, _dp, _dp]),
    "drd_set_tp_fields": (C.c_int, [_ctx, _dp, _dp, _dp, _dp]),
    "drd_set_ch_blend": (C.c_int, [_ctx, _dp]),
    "drd_host_register": (C.c_int, [C.c_void_p, C.c_int64]),
    "drd_host_unregister": (C.c_int, [C.c_void_p]),
    "drd_ch_blend_probe": (C.c_int, [_ctx, C.c_int, C.c_uint64, C.c_int, _dp]),
    "drd_interpolate_coef": (C.c_int, [_ctx, _dp, _dp, _dp, _dp]),
    "drd_two_phase_coef": (C.c_int, [_ctx, _dp, _dp, _dp, _dp]),
    "drd_batch_create": (C.c_int, [C.c_int, C.POINTER(abi.drd_batch_problem), C.c_int, C.POINTER(C.c_void_p)]),
    "drd_batch_run": (C.c_int, [C.c_void_p, _dp]),
    "drd_batch_result": (C.c_int, [C.c_void_p, C.c_int, _dp, _st]),
    "drd_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp]),
    "drd_batch_destroy": (C.c_int, [C.c_void_p]),
    "drd_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "drd_batch_length": (C.c_long, [C.c_int, C.c_int, C.c_int]),
    "drd_reinint_by_phsolve": (C.c_int, [_ctx, _dp, _dp, _dp]),
    "drd_dissipation": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.POINTER(abi.drd_diagnostics)]),
    "drd_write_fort23": (C.c_int, [C.c_char_p, C.c_double, C.POINTER(abi.drd_diagnostics)]),
    "drd_write_fort22": (C.c_int, [C.c_char_p, C.c_int, C.c_double, C.POINTER(abi.drd_diagnostics)]),
    "drd_phsolve_ori": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp, _st]),
    "drd_finit_wall": (C.c_int, [_ctx, _dp, C.c_int, _dp, _dp, _dp]),
    "drd_particle_params_default": (C.c_int, [C.POINTER(abi.drd_particle_params), C.c_double, C.c_double]),
    "drd_particle_initialize": (C.c_int, [C.POINTER(abi.drd_particle_params), C.c_double, C.c_double, _dp]),
    "drd_particles_set": (C.c_int, [_ctx, C.POINTER(abi.drd_particle_params), _dp, _dp]),
    "drd_particles_get": (C.c_int, [_ctx, _dp, _dp]),
    "drd_force_caculation_vel": (C.c_int, [_ctx, C.c_double, C.c_double, _dp, _dp]),
    "drd_update_position_vel": (C.c_int, [_ctx, _dp, _dp, C.c_double]),
    "drd_interpolate_coef_particles": (C.c_int, [_ctx, _dp, _dp, _dp]),
    "drd_phsolve": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp, _st]),
    "drd_ph_mu_solve": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp, _st]),
    "drd_velosolve_combined": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp, _dp,
                                         _dp, _st]),
    "drd_velosolve_2_combined": (C.c_int, [_ctx, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
                                           _dp, _dp, _dp, _dp, _dp, _dp, _st]),
    "drd_presolve_2": (C.c_int, [_ctx, _dp, _dp, C.c_double, _dp, _st]),
    "drd_mass": (C.c_int, [_ctx, _dp, _dp]),
    "drd_state_upload": (C.c_int, [_ctx, C.c_int, _dp]),
    "drd_state_download": (C.c_int, [_ctx, C.c_int, _dp]),
    "drd_state_device_ptr": (C.c_int, [_ctx, C.c_int, C.POINTER(_dp)]),
    "drd_step": (C.c_int, [_ctx, C.c_int, C.c_double, C.POINTER(abi.drd_step_stats)]),
    "drd_steps_async": (C.c_int, [_ctx, C.c_int, C.c_double, C.c_int]),
    "drd_synchronize": (C.c_int, [_ctx]),
    "drd_read_deck": (C.c_int, [C.c_char_p, C.POINTER(abi.drd_deck), C.c_char_p, C.c_int]),
    "drd_params_from_deck": (C.c_int, [C.POINTER(abi.drd_deck), C.c_int, C.c_int, C.c_int,
                                       C.POINTER(abi.drd_params)]),
    "drd_output": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 7 + [C.c_double]),
    "drd_input": (C.c_int, [C.c_char_p, C.c_int, C.c_int] + [_dp] * 7),
    "drd_read_time": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp]),
    "drd_output_particles": (C.c_int, [C.c_char_p, C.c_int, _dp]),
    "drd_checkpoint_async": (C.c_int, [_ctx, C.c_char_p, C.c_double]),
    "drd_checkpoint_wait": (C.c_int, [_ctx]),
    "drd_presolve_2_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                         C.c_double, C.c_void_p, C.c_void_p]),
    "drd_op_apply": (C.c_int, [_ctx, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    "drd_op_length": (C.c_long, [_ctx, C.c_int]),
    "drd_solve": (C.c_int, [_ctx, C.c_int, C.c_int, _dp, _dp, C.POINTER(abi.drd_status)]),
    "drd_barrier_selftest": (C.c_int, [_ctx, C.c_int, C.POINTER(C.c_int)]),
    "drd_kernel_bench": (C.c_int, [_ctx, C.c_int, C.c_int, _dp, _dp, _dp]),
    "drd_flush_l2": (C.c_int, [_ctx, C.c_int64]),
    "drd_kernel_launches": (C.c_int64, [_ctx]),
    "drd_persistent_solver": (C.c_int, [_ctx, C.c_char_p, C.c_int]),
    "drd_persist_profile": (C.c_int, [_ctx, C.POINTER(C.c_int64), C.c_int]),
    "drd_stream": (C.c_void_p, [_ctx]),
    "drd_unet_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]),
    "drd_unet_destroy": (C.c_int, [C.c_void_p]),
    "drd_unet_param_count": (C.c_int64, [C.c_void_p]),
    "drd_unet_last_error": (C.c_char_p, [C.c_void_p]),
    "drd_unet_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "drd_unet_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "drd_unet_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "drd_unet_gradients": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "drd_unet_train_step": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]),
    "drd_unet_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
}


def load(path=None):
    """Load (once) and return the CUDA library with its signatures declared."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    path = path or lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first "
                           "(python -m drd_application_gb300.build); there is no CPU fallback")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.drd_abi_version() != abi.DRD_ABI_VERSION:
        raise RuntimeError("libdrd_gb300.so ABI version does not match drd_application_gb300.abi")
    if path == lib_path():
        _LIB = lib
    return lib
