"""Loader of the in-tree GB300 library and its ctypes prototypes."""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsem2d_gb300.so")
_lib = None

vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
PP = C.POINTER(C.c_void_p)

# (name, restype, argtypes) of every exported function; include/*.h is the
# authority, the tests check this table against the headers
PROTOTYPES = [
    # sem2d_gpu.h
    ("sem2d_gpu_version", C.c_int, []),
    ("sem2d_gpu_device_count", C.c_int, []),
    ("sem2d_gpu_create", C.c_int, [C.POINTER(abi.ProblemDesc), PP]),
    ("sem2d_gpu_create_batch", C.c_int, [C.POINTER(abi.ProblemDesc), C.c_int, PP]),
    ("sem2d_gpu_batch_open", C.c_int, [PP]),
    ("sem2d_gpu_batch_add", C.c_int, [vp, C.POINTER(abi.ProblemDesc)]),
    ("sem2d_gpu_batch_add_many", C.c_int, [vp, C.POINTER(abi.ProblemDesc), C.c_int]),
    ("sem2d_gpu_batch_close", C.c_int, [vp]),
    ("sem2d_gpu_batch_size", C.c_int, [vp]),
    ("sem2d_gpu_batch_member", C.c_void_p, [vp, C.c_int]),
    ("sem2d_gpu_checkpoint_every", C.c_int, [vp, C.c_int]),
    ("sem2d_gpu_adjoint", C.c_int, [vp, dp, dp, dp, dp]),
    ("sem2d_gpu_step", C.c_int, [vp, C.c_int]),
    ("sem2d_gpu_step_timed", C.c_int, [vp, C.c_int, dp]),
    ("sem2d_gpu_stream", C.c_void_p, [vp]),
    ("sem2d_gpu_sync", C.c_int, [vp]),
    ("sem2d_gpu_current_step", C.c_int, [vp]),
    ("sem2d_gpu_get_fields", C.c_int, [vp, dp, dp, dp]),
    ("sem2d_gpu_get_seismograms", C.c_int, [vp, dp]),
    ("sem2d_gpu_get_fault", C.c_int, [vp, dp]),
    ("sem2d_gpu_get_fault_potency", C.c_int, [vp, dp]),
    ("sem2d_gpu_get_strain_stress", C.c_int, [vp, dp, dp]),
    ("sem2d_gpu_get_fault_state", C.c_int, [vp, dp, dp, dp, dp, dp]),
    ("sem2d_gpu_get_info", C.c_int, [vp, ip, dp, dp]),
    ("sem2d_gpu_reset", C.c_int, [vp]),
    ("sem2d_gpu_kernel_launches", C.c_longlong, [vp]),
    ("sem2d_gpu_tile_shape", C.c_int, [vp, ip, ip]),
    ("sem2d_gpu_destroy", C.c_int, [vp]),
    ("sem2d_gpu_last_error", C.c_char_p, [vp]),
    ("sem2d_gpu_step_noalloc", C.c_int, [C.POINTER(abi.LatticeArgs), C.c_int, vp]),
    # sem2d_host.h
    ("sem2d_grid_build", C.c_int, [C.POINTER(abi.Deck), PP]),
    ("sem2d_grid_sizes", C.c_int, [vp, ip, ip, ip]),
    ("sem2d_grid_ibool", C.c_int, [vp, ip]),
    ("sem2d_grid_coord", C.c_int, [vp, dp]),
    ("sem2d_grid_tags", C.c_int, [vp, ip]),
    ("sem2d_grid_boundary", C.c_int, [vp, C.c_int, ip, ip]),
    ("sem2d_grid_gll", C.c_int, [vp, dp, dp, dp]),
    ("sem2d_grid_destroy", None, [vp]),
    ("sem2d_problem_build", C.c_int, [vp, C.POINTER(abi.Deck), PP]),
    ("sem2d_problem_get_desc", C.c_int, [vp, C.POINTER(abi.ProblemDesc)]),
    ("sem2d_problem_time", C.c_int, [vp, dp, ip, dp]),
    ("sem2d_problem_rec_coord", C.c_int, [vp, dp]),
    ("sem2d_problem_fault_coord", C.c_int, [vp, dp]),
    ("sem2d_problem_destroy", None, [vp]),
    ("sem2d_host_last_error", C.c_char_p, []),
    ("sem2d_abi_struct_sizes", C.c_int, [ip, ip]),
    ("sem2d_abi_field_offsets", C.c_int, [C.c_int, C.POINTER(C.c_longlong), C.c_int]),
    ("sem2d_stf_eval", C.c_int, [C.POINTER(abi.Stf), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("sem2d_tune_cache_path", C.c_int, [C.c_char_p, C.c_int]),
    ("sem2d_tune_key", C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_char_p, C.c_int]),
    ("sem2d_tune_lookup", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(abi.TuneEntry)]),
    ("sem2d_tune_record", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(abi.TuneEntry)]),
    ("sem2d_tune_select", C.c_int, [C.POINTER(abi.TuneEntry), C.c_int, C.c_double]),
]


def lib(build_if_missing=True):
    """The loaded library (compiled first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError("libsem2d_gb300.so is not built (run sem2dpack_gb300.build)")
            from . import build
            build.build()
        L = C.CDLL(LIB_PATH)
        for name, res, args in PROTOTYPES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib
