"""ctypes binding of libvec_gpu.so (the C-ABI of include/vec.h).

There is no CPU fallback: if the CUDA library is missing, loading fails
with an error naming the file.
"""
import ctypes as C
import os

from .params import VecClosureReport, VecDiag, VecParams, VecScalars, VecSnapshot

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libvec_gpu.so")

# exported symbols of include/vec.h with their ctypes signatures
_vp = C.c_void_p
_dp = C.c_void_p   # double* (host numpy data pointer or device pointer)
SIGNATURES = {
    "vec_params_default": (C.c_int, [C.POINTER(VecParams)]),
    "vec_params_read_input": (C.c_int, [C.c_char_p, C.POINTER(VecParams)]),
    "vec_create": (C.c_int, [C.POINTER(VecParams), C.POINTER(_vp)]),
    "vec_destroy": (C.c_int, [_vp]),
    "vec_last_error": (C.c_char_p, []),
    "vec_stream": (_vp, [_vp]),
    "vec_sync": (C.c_int, [_vp]),
    "vec_set_field": (C.c_int, [_vp, C.c_int, _dp]),
    "vec_get_field": (C.c_int, [_vp, C.c_int, _dp]),
    "vec_set_mean": (C.c_int, [_vp, C.c_int, _dp]),
    "vec_get_mean": (C.c_int, [_vp, C.c_int, _dp]),
    "vec_set_bzbar": (C.c_int, [_vp, C.c_double]),
    "vec_get_bzbar": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "vec_get_scalars": (C.c_int, [_vp, C.POINTER(VecScalars)]),
    "vec_set_scalars": (C.c_int, [_vp, C.POINTER(VecScalars)]),
    "vec_static": (C.c_int, [_vp]),
    "vec_mag_init": (C.c_int, [_vp]),
    "vec_calcdt": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "vec_d1bydx": (C.c_int, [_vp, _dp, _dp]),
    "vec_d1bydy": (C.c_int, [_vp, _dp, _dp]),
    "vec_d2bydx": (C.c_int, [_vp, _dp, _dp, _dp]),
    "vec_d2bydy": (C.c_int, [_vp, _dp, _dp, _dp]),
    "vec_dealias": (C.c_int, [_vp, _dp]),
    "vec_forwardfft": (C.c_int, [_vp, _dp, _dp]),
    "vec_inversefft": (C.c_int, [_vp, _dp, _dp]),
    "vec_d1bydz": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "vec_d1upbydz": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "vec_d2bydz": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "vec_d1bydz1d": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "vec_d2bydz1d": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "vec_hydro_deriv": (C.c_int, [_vp]),
    "vec_mag_deriv": (C.c_int, [_vp]),
    "vec_bandj": (C.c_int, [_vp]),
    "vec_magdealias": (C.c_int, [_vp]),
    "vec_boundary": (C.c_int, [_vp]),
    "vec_mag_boundary": (C.c_int, [_vp]),
    "vec_ab3_update": (C.c_int, [_vp]),
    "vec_diag": (C.c_int, [_vp, C.POINTER(VecDiag)]),
    "vec_step": (C.c_int, [_vp, C.c_int]),
    "vec_last_diag": (C.c_int, [_vp, C.POINTER(VecDiag)]),
    "vec_profile": (C.c_int, [_vp, C.c_int]),
    "vec_profile_count": (C.c_int, [_vp]),
    "vec_profile_get": (C.c_int, [_vp, C.c_int, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]),
    "vec_profile_reset": (C.c_int, [_vp]),
    "vec_launch_count": (C.c_longlong, [_vp]),
    "vec_use_graphs": (C.c_int, [_vp, C.c_int]),
    "vec_ensemble_create": (C.c_int, [C.POINTER(VecParams), C.c_int, C.POINTER(_vp)]),
    "vec_ensemble_destroy": (C.c_int, [_vp]),
    "vec_ensemble_size": (C.c_int, [_vp]),
    "vec_ensemble_member": (_vp, [_vp, C.c_int]),
    "vec_ensemble_start": (C.c_int, [_vp]),
    "vec_ensemble_step": (C.c_int, [_vp, C.c_int]),
    "vec_ensemble_sync": (C.c_int, [_vp]),
    "vec_ensemble_tune": (C.c_int, [_vp, C.c_int, C.c_char_p]),
    "vec_tunables": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "vec_set_tunables": (C.c_int, [_vp, C.c_int, C.c_int]),
    "vec_line_f32": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]),
    "vec_selftest_wait": (C.c_int, [_vp, C.c_longlong]),
    "vec_measure_fp64": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "vec_net_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(_vp)]),
    "vec_net_destroy": (C.c_int, [_vp]),
    "vec_net_nparams": (C.c_longlong, [_vp]),
    "vec_net_get_params": (C.c_int, [_vp, _dp]),
    "vec_net_set_params": (C.c_int, [_vp, _dp]),
    "vec_net_get_grads": (C.c_int, [_vp, _dp]),
    "vec_net_forward": (C.c_int, [_vp, _dp, _dp]),
    "vec_net_backward": (C.c_int, [_vp, _dp, C.POINTER(C.c_double)]),
    "vec_net_adam": (C.c_int, [_vp, C.c_float]),
    "vec_net_launch_count": (C.c_longlong, [_vp]),
    "vec_net_time": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_double),
                               C.POINTER(C.c_double)]),
    "vec_closure_create": (C.c_int, [C.POINTER(VecParams), C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(_vp)]),
    "vec_closure_destroy": (C.c_int, [_vp]),
    "vec_closure_net": (_vp, [_vp]),
    "vec_closure_npairs": (C.c_int, [_vp]),
    "vec_box_filter": (C.c_int, [_vp, _vp, _vp]),
    "vec_closure_add_pair": (C.c_int, [_vp, _vp, _vp]),
    "vec_closure_get_pair": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "vec_closure_fit_norm": (C.c_int, [_vp, C.c_int]),
    "vec_closure_get_norm": (C.c_int, [_vp, _dp]),
    "vec_closure_set_norm": (C.c_int, [_vp, _dp]),
    "vec_closure_train": (C.c_int, [_vp, C.c_int, C.c_float, C.c_int, C.c_ulonglong, _dp]),
    "vec_closure_eval": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "vec_closure_attach": (C.c_int, [_vp, _vp, C.c_int]),
    "vec_closure_infer": (C.c_int, [_vp, _vp]),
    "vec_closure_step": (C.c_int, [_vp, _vp, C.c_int]),
    "vec_closure_run": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int,
                                  C.POINTER(VecClosureReport)]),
    "vec_closure_set_output": (C.c_int, [_vp, C.c_float, C.c_float]),
    "vec_top_nusselt": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "vec_expand": (C.c_int, [_vp, _vp, _dp, _dp]),
    "vec_upsample": (C.c_int, [_vp, _vp]),
    "vec_nc_write": (C.c_int, [C.c_char_p, C.POINTER(VecSnapshot), C.c_int]),
    "vec_nc_write_fmt": (C.c_int, [C.c_char_p, C.POINTER(VecSnapshot), C.c_int, C.c_int]),
    "vec_nc_read": (C.c_int, [C.c_char_p, C.POINTER(VecSnapshot)]),
    "vec_write_snapshot": (C.c_int, [_vp, C.c_char_p, C.c_int, C.c_char_p]),
    "vec_read_restart": (C.c_int, [_vp, C.c_char_p]),
    "vec_calcdt_noalloc": (C.c_int, [C.POINTER(VecParams)] + [_dp] * 9 + [_vp]),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load():
    """Load libvec_gpu.so (loading needs no GPU; calls that compute do)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"CUDA library {LIB_PATH} is missing: run `python -m fug30v0kxc_gb300.build` "
                "(or __graft_entry__.build()) first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
