"""ctypes binding of the helmgpu C ABI (include/helmgpu.h).

This is the same binding a Julia ``ccall`` shim or any other FFI would make:
plain structs, pointers and sizes.  Loading fails loudly when the compiled
library is absent -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhelmgpu.so"

HZ_OK = 0
HZ_NOT_CONVERGED = 1
HZ_ERR_ARG = -1
HZ_ERR_CUDA = -2
HZ_ERR_ALLOC = -3
HZ_ERR_NUMERIC = -4
HZ_ERR_STATE = -5
HZ_ERR_NO_DEVICE = -6

HZ_MEM_HOST = 0
HZ_MEM_DEVICE = 1
HZ_PREC_FP64 = 0
HZ_PREC_MIXED = 1
HZ_OUTER_FP64 = 0
HZ_OUTER_EMULATED = 1
HZ_KRYLOV_FGMRES = 0
HZ_KRYLOV_BICGSTAB = 1
HZ_COARSE_GALERKIN = 0
HZ_COARSE_REDISCRETIZE = 1
HZ_RELAX_JAC = 0
HZ_RELAX_JAC_GMRES = 1
HZ_OP_H = 0
HZ_OP_SH = 1
HZ_NOALLOC_MAX_COLS = 4096
HZ_NET_CONV_WARP_MMA = 0
HZ_NET_CONV_TCGEN05 = 1
HZ_NET_CONV_AUTO = 2


class hz_problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("n", C.c_int64 * 3),
        ("h", C.c_double * 3),
        ("omega_re", C.c_double),
        ("omega_im", C.c_double),
        ("m", C.POINTER(C.c_double)),
        ("gamma", C.POINTER(C.c_double)),
        ("neumann_on_top", C.c_int32),
        ("sommerfeld", C.c_int32),
        ("order_neumann_bc", C.c_int32),
    ]


class hz_options(C.Structure):
    _fields_ = [
        ("levels", C.c_int32),
        ("max_outer", C.c_int32),
        ("rel_tol", C.c_double),
        ("relax_pre", C.c_int32),
        ("relax_post", C.c_int32),
        ("relax_param", C.c_double),
        ("cycle", C.c_int32),
        ("krylov", C.c_int32),
        ("inner", C.c_int32),
        ("shift", C.c_double),
        ("precision", C.c_int32),
        ("coarse_op", C.c_int32),
        ("verbose", C.c_int32),
        ("profile", C.c_int32),
        ("device", C.c_int32),
        ("outer_arith", C.c_int32),
        ("cuda_graph", C.c_int32),
        ("autotune", C.c_int32),
        ("relax_type", C.c_int32),
        ("relax_from", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


class hz_stats(C.Structure):
    _fields_ = [
        ("outer", C.c_int32),
        ("n_prec", C.c_int32),
        ("max_col_iters", C.c_int32),
        ("converged_cols", C.c_int32),
        ("max_relres", C.c_double),
        ("setup_time", C.c_double),
        ("solve_time", C.c_double),
        ("kernel_launches", C.c_int64),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
    ]


_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol include/helmgpu.h declares
SIGNATURES = {
    "hz_version": (C.c_int32, []),
    "hz_last_error": (C.c_char_p, [_vp]),
    "hz_default_options": (None, [C.POINTER(hz_options)]),
    "hz_create": (C.c_int, [C.POINTER(hz_problem), C.POINTER(hz_options), C.POINTER(_vp)]),
    "hz_destroy": (C.c_int, [_vp]),
    "hz_solve": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(hz_stats)]),
    "hz_column_stats": (C.c_int, [_vp, _dp, C.POINTER(C.c_int32), C.c_int32]),
    "hz_apply": (C.c_int, [_vp, C.c_int32, C.c_int32, _vp, _vp, C.c_int64, C.c_int32, C.c_int32]),
    "hz_apply_noalloc": (C.c_int, [_vp, C.c_int32, C.c_int32, _vp, _vp, C.c_int64, C.c_int32]),
    "hz_clear": (C.c_int, [_vp]),
    "hz_copy": (C.c_int, [_vp, C.POINTER(_vp)]),
    "hz_stream": (_vp, [_vp]),
    "hz_kernel_times": (C.c_int, [_vp, C.c_int32, C.c_char_p, C.c_int32, _i64p, _i64p, _dp, _dp]),
    "hz_reset_kernel_times": (C.c_int, [_vp]),
    "hz_set_profile": (C.c_int, [_vp, C.c_int32]),
    "hz_set_cuda_graph": (C.c_int, [_vp, C.c_int32]),
    "hz_net_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(_vp)]),
    "hz_net_destroy": (C.c_int, [_vp]),
    "hz_net_num_params": (C.c_int64, []),
    "hz_net_layer_shape": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "hz_net_get_weights": (C.c_int, [_vp, _vp]),
    "hz_net_set_weights": (C.c_int, [_vp, _vp]),
    "hz_net_forward": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int32, C.c_int32]),
    "hz_net_gradient": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int32, C.c_int32, _dp, _vp]),
    "hz_net_train": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_double,
                               C.c_int32, _dp]),
    "hz_net3d_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(_vp)]),
    "hz_net3d_num_params": (C.c_int64, []),
    "hz_net3d_layer_shape": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "hz_net_dim": (C.c_int, [_vp]),
    "hz_net_set_conv_path": (C.c_int, [_vp, C.c_int32]),
    "hz_net3d_forward": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32]),
    "hz_net3d_gradient": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32, _dp,
                                    _vp]),
    "hz_net3d_train": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                 C.c_double, C.c_int32, _dp]),
    "hz_kernel_flops": (C.c_int, [_vp, C.c_int32, _dp]),
    "hz_tune_info": (C.c_int, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "hz_net_save": (C.c_int, [_vp, C.c_char_p]),
    "hz_net_load": (C.c_int, [_vp, C.c_char_p]),
    "hz_net_file_info": (C.c_int, [C.c_char_p, _i64p, _i64p]),
    "hz_net_set_profile": (C.c_int, [_vp, C.c_int32]),
    "hz_net_kernel_times": (C.c_int, [_vp, C.c_int32, C.c_char_p, C.c_int32, _i64p, _i64p, _dp, _dp, _dp]),
    "hz_net_reset_kernel_times": (C.c_int, [_vp]),
    "hz_attach_net": (C.c_int, [_vp, _vp, C.c_int32, C.c_double]),
    "hz_learned_stats": (C.c_int, [_vp, _i64p, C.POINTER(C.c_int32)]),
    "hz_collect_pairs": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                   _vp, _vp, _dp, _dp, _i64p]),
    "hz_max_frequency": (C.c_double, [_dp, C.c_int64, _dp, C.c_int32]),
    "hz_abl": (C.c_int, [C.c_int32, _i64p, C.c_int32, _i64p, C.c_double, _dp]),
    "hz_sommerfeld": (C.c_int, [C.c_int32, _i64p, _dp, _dp, C.c_double, C.c_int32, C.c_int32, _dp]),
    "hz_helmholtz_mass": (C.c_int, [C.POINTER(hz_problem), _dp]),
    "hz_point_source": (C.c_int, [C.c_int32, _i64p, _dp, _i64p, _dp]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libhelmgpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"helmgpu library not built: {p} is missing (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class HelmgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"helmgpu error {code}: {msg}")
        self.code = code


def check(code: int, handle=None) -> int:
    if code < 0:
        lib = load()
        msg = lib.hz_last_error(handle)
        raise HelmgpuError(code, msg.decode() if msg else "")
    return code
