"""ctypes binding of the C ABI (include/mlpcg_gb300.h).

The shared library is the only compute path of this package: when it cannot
be loaded, every op raises (there is no CPU fallback).  ``load()`` builds it
in-tree with nvcc when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

F32, BF16, F64 = 0, 1, 2
_lock = threading.Lock()
_lib = None

_vp, _i, _i64, _sz, _fp, _u8p = C.c_void_p, C.c_int, C.c_int64, C.c_size_t, C.c_void_p, C.c_void_p

# name -> (restype, argtypes)
_PROTOS = {
    "mlpcg_last_error": (C.c_char_p, []),
    "mlpcg_abi_version": (_i, []),
    "mlpcg_stencil_gen": (_i, [_fp, _i, _i, _i, _i, _fp, _fp, _vp, _i, _i64, _vp]),
    "mlpcg_stencil_apply": (_i, [_vp, _i, _i64, _vp, _i, _i, _vp, _i, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_stencil_coeff_grad": (_i, [_fp, _fp, _i, _fp, _i64, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_stencil_wgrad_workspace": (_sz, [_i, _i, _i]),
    "mlpcg_stencil_wgrad": (_i, [_fp, _i64, _fp, _i, _i, _i, _i, _fp, _fp, _vp, _sz, _vp]),
    "mlpcg_stencil_image_grad": (_i, [_fp, _i64, _fp, _fp, _i, _i, _i, _vp]),
    "mlpcg_sm_block_3d_workspace": (_sz, [_i, _i, _i]),
    "mlpcg_sm_block_3d_forward": (_i, [_fp, _i, _fp, _i, _fp, _fp, _fp, _i, _i, _i, _i, _i, _vp, _sz, _vp]),
    "mlpcg_sm_block_3d_backward": (_i, [_fp, _fp, _i, _fp, _i, _fp, _fp, _fp, _fp, _fp, _fp,
                                        _i, _i, _i, _i, _i, _vp, _sz, _vp]),
    "mlpcg_sm_linear_3d_workspace": (_sz, [_i, _i, _i]),
    "mlpcg_sm_linear_3d_forward": (_i, [_fp, _i, _i, _i, _fp, _fp, _i, _fp, _fp, _vp, _sz, _vp]),
    "mlpcg_sm_linear_3d_backward": (_i, [_fp, _fp, _fp, _fp, _vp]),
    "mlpcg_sm_linear_3d_image_grad": (_i, [_fp, _fp, _fp, _i, _i, _i, _vp]),
    "mlpcg_avg_pool2": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_avg_pool2_adjoint": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_upsample2": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_upsample2_adjoint": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_axpby": (_i, [_fp, _vp, _fp, _vp, _vp, _i, _i64, _vp]),
    "mlpcg_laplacian_apply": (_i, [_u8p, _vp, _vp, _i, _i, _i, _i, _vp]),
    "mlpcg_precond_create": (_i, [_i, _i, _i, _i, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_precond_create_spd": (_i, [_i, _i, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_precond_create_kind": (_i, [_i, _i, _i, _i, _i, _i, _i, _i, _vp]),
    "mlpcg_precond_check": (_i, [_vp, _vp, _vp]),
    "mlpcg_precond_set_copy_stall": (_i, [_vp, _i, _vp]),
    "mlpcg_precond_coarse_cluster": (_i, [_vp, _vp, _vp]),
    "mlpcg_precond_set_coarse_cluster": (_i, [_vp, _i]),
    "mlpcg_precond_set_small_levels": (_i, [_vp, _i]),
    "mlpcg_precond_class_counts": (_i, [_vp, _i, _vp, _vp, _vp]),
    "mlpcg_precond_class_counts_transposed": (_i, [_vp, _i, _vp, _vp, _vp]),
    "mlpcg_precond_workspace": (_sz, [_vp]),
    "mlpcg_precond_destroy": (None, [_vp]),
    "mlpcg_precond_setup": (_i, [_vp, _vp, _sz, _fp, _fp, _vp]),
    "mlpcg_precond_apply": (_i, [_vp, _fp, _fp, _fp, _vp]),
    "mlpcg_precond_coefficients": (_i, [_vp, _fp, _vp]),
    "mlpcg_precond_apply_stages": (_i, [_vp, _i, _i, _fp, _fp, _fp, _vp]),
    "mlpcg_precond_level_info": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "mlpcg_solver_create": (_i, [_i, _i, _i, _vp, _i, _i, C.c_double, _i, _vp]),
    "mlpcg_solver_workspace": (_sz, [_vp]),
    "mlpcg_solver_destroy": (None, [_vp]),
    "mlpcg_solver_bind": (_i, [_vp, _vp, _sz, _u8p, _vp, _vp]),
    "mlpcg_solver_solve": (_i, [_vp, _i, _vp]),
    "mlpcg_solver_solve_zero_guess": (_i, [_vp, _i, _vp]),
    "mlpcg_solver_result": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "mlpcg_solver_set_schedule": (_i, [_vp, _i]),
    "mlpcg_solver_set_copy_stall": (_i, [_vp, _i]),
    "mlpcg_solver_set_dependent_launch": (_i, [_vp, _i]),
    "mlpcg_solver_dependent_edges": (_i, [_vp, _vp]),
    "mlpcg_solver_set_fused_dots": (_i, [_vp, _i]),
    "mlpcg_solver_fused_dots": (_i, [_vp, _vp]),
    "mlpcg_solver_get_schedule": (_i, [_vp, _vp]),
    "mlpcg_batch_create": (_i, [_vp, _i, _vp]),
    "mlpcg_batch_solve": (_i, [_vp, _vp]),
    "mlpcg_batch_destroy": (None, [_vp]),
    "mlpcg_flags_to_image": (_i, [_u8p, _fp, _i64, _vp]),
    "mlpcg_fluid_order_entries": (_sz, [_i64]),
    "mlpcg_fluid_order": (_i, [_u8p, _i64, _vp, _vp]),
    "mlpcg_scatter_fluid": (_i, [_fp, _i64, _u8p, _vp, _i64, _fp, _vp]),
    "mlpcg_gather_fluid": (_i, [_fp, _u8p, _vp, _i64, _fp, _i64, _vp]),
    "mlpcg_host_mapped": (_i, [_vp, _vp]),
    "mlpcg_dot_workspace": (_sz, [_i64]),
    "mlpcg_dot": (_i, [_vp, _vp, _i, _i64, _vp, _vp, _sz, _vp]),
    "mlpcg_dot_noalloc": (_i, [_vp, _vp, _i, _i64, _vp, _vp]),
}


class MLPCGError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


def load():
    """Return the loaded ctypes library (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.LIB_PATH
            if not path.exists() or os.environ.get("MLPCG_REBUILD"):
                path = _build.build()
            lib = C.CDLL(str(path), mode=C.RTLD_LOCAL)
            for name, (res, args) in _PROTOS.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def call(name: str, *args) -> None:
    """Invoke ``name`` and raise MLPCGError with the library's message on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.mlpcg_last_error().decode(errors="replace")
        raise MLPCGError(f"{name} failed with status {rc}: {msg}")


def query(name: str, *args):
    return getattr(load(), name)(*args)


def exported_symbols():
    return sorted(_PROTOS)
