"""ctypes binding of libswm_gb300.so (the C-ABI of include/swm_gpu.h).

The library is built in-tree by cubedsphere_sbp_swm_gb300.build; loading
fails loudly when it is missing (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

SWM_OK = 0
SWM_E_INVALID = -1
SWM_E_UNSUPPORTED = -2
SWM_E_CUDA = -3
SWM_E_NOMEM = -4
SWM_E_DEVICE = -5
SWM_E_IO = -6

SWM_FP64_PLAIN = 0
SWM_FP32_FUSED = 1

# staggering of a context and its meshes (swm_ctx_grid, swm_mesh_dims)
SWM_GRID_AH = 0
SWM_GRID_C = 1
SWM_MESH_P, SWM_MESH_U, SWM_MESH_V, SWM_MESH_Q = 0, 1, 2, 3

# largest N that swm_sync_scalar_static accepts
SWM_SYNC_STATIC_MAX_N = 1024

# every entry point of include/swm_gpu.h
EXPORTS = (
    "swm_ctx_create", "swm_ctx_create_named", "swm_ctx_destroy", "swm_last_error",
    "swm_ctx_synchronize", "swm_ctx_stream", "swm_ctx_npts", "swm_set_orography",
    "swm_state_create", "swm_state_create_similar", "swm_state_free", "swm_state_upload",
    "swm_state_download", "swm_state_upload_async", "swm_state_download_async", "swm_assign_s1",
    "swm_assign_s1v1", "swm_assign_s1v1s2v2",
    "swm_update_s1v1", "swm_update_s1v1s2v2", "swm_dot", "swm_norm2", "swm_apply",
    "swm_apply_unfused", "swm_rk4_step", "swm_diagnostics", "swm_field_create",
    "swm_field_free", "swm_field_upload", "swm_field_download", "swm_op_co2contra",
    "swm_op_massflux", "swm_op_ke", "swm_op_grad", "swm_op_div", "swm_op_curl",
    "swm_op_coriolis", "swm_op_grad_perp", "swm_op_contra2co", "swm_op_grad_a2_ecs", "swm_halo_ecs_o",
    "swm_op_div_a2_ecs", "swm_halo_ecs_a_vec", "swm_op_grad_c2_ecs", "swm_halo_ecs_xy", "swm_laplace_ch",
    "swm_sync_scalar", "swm_sync_vector_cov", "swm_quadrature_mass",
    "swm_timing_enable", "swm_timing_read", "swm_sync_scalar_static",
    "swm_ensemble_create", "swm_ensemble_destroy", "swm_ensemble_last_error", "swm_ensemble_size",
    "swm_ensemble_member", "swm_ensemble_upload", "swm_ensemble_download",
    "swm_ensemble_diagnostics", "swm_ensemble_step", "swm_ensemble_synchronize",
    "swm_ensemble_stream", "swm_ensemble_set_shape", "swm_ensemble_get_shape", "swm_ensemble_tune",
    "swm_apply_tl", "swm_apply_ad", "swm_rk4_tl", "swm_rk4_ad", "swm_adjoint_create",
    "swm_adjoint_destroy", "swm_adjoint_forward", "swm_adjoint_backward", "swm_adjoint_counts",
    "swm_state_upload_device", "swm_state_download_device", "swm_quadrature_weights",
    "swm_diffusion_set", "swm_apply_diffusion", "swm_diffusion_step", "swm_model_step",
    "swm_laplace", "swm_latlon_create", "swm_latlon_destroy", "swm_latlon_regrid_field",
    "swm_latlon_regrid_vector", "swm_latlon_regrid_state", "swm_latlon_write", "swm_paneled_write",
    "swm_tune_stage", "swm_get_stage_shape", "swm_set_stage_shape", "swm_work_split", "swm_ensemble_set_width",
    "swm_ensemble_get_width", "swm_state_save", "swm_state_load", "swm_ctx_grid", "swm_mesh_dims",
    "swm_field_create_mesh",
)


class SwmConfig(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("sbp_order", ctypes.c_int),
        ("radius", ctypes.c_double),
        ("grav", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("rotation_axis", ctypes.c_double * 3),
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
    ]


class SwmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
_D = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libswm_gb300.so, compiling it first when it is absent or stale."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise OSError(f"libswm_gb300.so not found at {path}: build the CUDA library first")
    L = ctypes.CDLL(path)
    I, D, VP, C = ctypes.c_int, ctypes.c_double, _VP, ctypes.c_char_p
    PP = ctypes.POINTER(ctypes.c_void_p)

    def sig(name, res, *args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    sig("swm_ctx_create", I, ctypes.POINTER(SwmConfig), PP)
    sig("swm_ctx_create_named", I, ctypes.POINTER(SwmConfig), C, C, C, C, C, C, C, C, PP)
    sig("swm_ctx_destroy", None, VP)
    sig("swm_last_error", C, VP)
    sig("swm_ctx_synchronize", I, VP)
    sig("swm_ctx_stream", VP, VP)
    sig("swm_ctx_npts", ctypes.c_size_t, VP)
    sig("swm_set_orography", I, VP, _D)
    sig("swm_state_create", I, VP, PP)
    sig("swm_state_create_similar", I, VP, VP, PP)
    sig("swm_state_free", None, VP)
    sig("swm_state_upload", I, VP, VP, _D, _D, _D)
    sig("swm_state_download", I, VP, VP, _D, _D, _D)
    sig("swm_state_upload_async", I, VP, VP, _D, _D, _D)
    sig("swm_state_download_async", I, VP, VP, _D, _D, _D)
    sig("swm_assign_s1", I, VP, VP, D)
    sig("swm_assign_s1v1", I, VP, VP, D, VP)
    sig("swm_assign_s1v1s2v2", I, VP, VP, D, VP, D, VP)
    sig("swm_update_s1v1", I, VP, VP, D, VP)
    sig("swm_update_s1v1s2v2", I, VP, VP, D, VP, D, VP)
    sig("swm_dot", I, VP, VP, VP, _D)
    sig("swm_norm2", I, VP, VP, _D)
    sig("swm_apply", I, VP, VP, VP)
    sig("swm_apply_unfused", I, VP, VP, VP)
    sig("swm_rk4_step", I, VP, VP, D, I)
    sig("swm_diffusion_set", I, VP, C, D, C, D)
    sig("swm_apply_diffusion", I, VP, VP, VP)
    sig("swm_diffusion_step", I, VP, VP, D, I)
    sig("swm_model_step", I, VP, VP, D, I)
    sig("swm_laplace", I, VP, VP, VP, I)
    sig("swm_latlon_create", I, VP, I, I, C, C, PP)
    sig("swm_latlon_destroy", None, VP)
    sig("swm_latlon_regrid_field", I, VP, VP, VP, _D)
    sig("swm_latlon_regrid_vector", I, VP, VP, VP, VP, _D, _D)
    sig("swm_latlon_regrid_state", I, VP, VP, VP, _D, _D, _D)
    sig("swm_latlon_write", I, VP, VP, VP, C, C, C, I)
    sig("swm_paneled_write", I, VP, VP, I, C, I)
    sig("swm_tune_stage", I, VP, VP, D, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I),
        ctypes.POINTER(I), _D)
    sig("swm_get_stage_shape", I, VP, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I),
        ctypes.POINTER(I), ctypes.POINTER(I))
    sig("swm_set_stage_shape", I, VP, I, I, I, I)
    sig("swm_work_split", I, I, I, I, I, I, ctypes.POINTER(I), I, ctypes.POINTER(I))
    sig("swm_ensemble_set_width", I, VP, I)
    sig("swm_ensemble_get_width", I, VP, ctypes.POINTER(I))
    sig("swm_state_save", I, VP, VP, C, D)
    sig("swm_state_load", I, VP, VP, C, _D)
    sig("swm_diagnostics", I, VP, VP, _D)
    sig("swm_field_create", I, VP, PP)
    sig("swm_field_create_mesh", I, VP, I, PP)
    sig("swm_ctx_grid", I, VP)
    sig("swm_mesh_dims", I, VP, I, ctypes.POINTER(I), ctypes.POINTER(I))
    sig("swm_field_free", None, VP)
    sig("swm_field_upload", I, VP, VP, _D)
    sig("swm_field_download", I, VP, VP, _D)
    sig("swm_op_co2contra", I, VP, VP, VP, VP, VP)
    sig("swm_op_massflux", I, VP, VP, VP, VP, VP, VP)
    sig("swm_op_ke", I, VP, VP, VP, VP, VP, VP)
    sig("swm_op_grad", I, VP, VP, VP, VP)
    sig("swm_op_div", I, VP, VP, VP, VP)
    sig("swm_op_curl", I, VP, VP, VP, VP)
    sig("swm_op_coriolis", I, VP, VP, VP, VP, VP, VP, VP)
    sig("swm_op_grad_perp", I, VP, VP, VP, VP)
    sig("swm_op_contra2co", I, VP, VP, VP, VP, VP)
    sig("swm_op_grad_a2_ecs", I, VP, VP, VP, VP)
    sig("swm_halo_ecs_o", I, VP, VP, I, _D)
    sig("swm_op_div_a2_ecs", I, VP, VP, VP, VP)
    sig("swm_op_grad_c2_ecs", I, VP, VP, VP, VP)
    sig("swm_halo_ecs_xy", I, VP, VP, I, _D)
    sig("swm_laplace_ch", I, VP, VP, VP, I)
    sig("swm_halo_ecs_a_vec", I, VP, VP, VP, I, _D, _D)
    sig("swm_sync_scalar", I, VP, VP)
    sig("swm_sync_vector_cov", I, VP, VP, VP)
    sig("swm_quadrature_mass", I, VP, VP, _D)
    sig("swm_timing_enable", I, VP, I)
    sig("swm_timing_read", I, VP, _D, ctypes.POINTER(ctypes.c_long), _D,
        ctypes.POINTER(ctypes.c_long))
    sig("swm_sync_scalar_static", I, VP, VP)
    IP = ctypes.POINTER(ctypes.c_int)
    sig("swm_ensemble_create", I, ctypes.POINTER(SwmConfig), I, IP, _D, PP)
    sig("swm_ensemble_destroy", None, VP)
    sig("swm_ensemble_last_error", C, VP)
    sig("swm_ensemble_size", I, VP)
    sig("swm_ensemble_member", I, VP, I, PP, PP)
    sig("swm_ensemble_upload", I, VP, I, _D, _D, _D)
    sig("swm_ensemble_download", I, VP, I, _D, _D, _D)
    sig("swm_ensemble_diagnostics", I, VP, I, _D)
    sig("swm_ensemble_step", I, VP, I)
    sig("swm_ensemble_synchronize", I, VP)
    sig("swm_ensemble_stream", VP, VP)
    sig("swm_ensemble_set_shape", I, VP, I, I)
    sig("swm_ensemble_get_shape", I, VP, IP, IP, IP)
    sig("swm_ensemble_tune", I, VP, I, IP, IP, _D)
    LP = ctypes.POINTER(ctypes.c_long)
    sig("swm_apply_tl", I, VP, VP, VP, VP)
    sig("swm_apply_ad", I, VP, VP, VP, VP)
    sig("swm_rk4_tl", I, VP, VP, VP, D)
    sig("swm_rk4_ad", I, VP, VP, VP, D)
    sig("swm_adjoint_create", I, VP, I, I, D, PP)
    sig("swm_adjoint_destroy", None, VP)
    sig("swm_adjoint_forward", I, VP, VP, VP)
    sig("swm_adjoint_backward", I, VP, VP)
    sig("swm_adjoint_counts", I, VP, LP, LP, LP)
    sig("swm_state_upload_device", I, VP, VP, VP, VP, VP)
    sig("swm_state_download_device", I, VP, VP, VP, VP, VP)
    sig("swm_quadrature_weights", I, VP, _D)
    _lib = L
    return L


def check(rc: int, ctx=None) -> None:
    if rc != SWM_OK:
        msg = load().swm_last_error(ctx)
        raise SwmError(rc, msg.decode() if msg else "")


def check_ensemble(rc: int, ens=None) -> None:
    if rc != SWM_OK:
        msg = load().swm_ensemble_last_error(ens)
        raise SwmError(rc, msg.decode() if msg else "")
