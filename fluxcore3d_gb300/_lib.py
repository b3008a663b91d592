"""ctypes binding of libfluxcore3d_gb300.so.

The library is the only compute backend.  `lib()` raises when it is missing or
when CUDA is unavailable; there is no CPU or torch fallback behind it.
Tensors cross the boundary as raw device pointers (`tensor.data_ptr()`) and
the launching stream as `torch.cuda.current_stream().cuda_stream`.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

_LIB = None
_LOAD_ERROR: str | None = None

c_float_p = C.POINTER(C.c_float)
vp = C.c_void_p
i32 = C.c_int
i64 = C.c_longlong
f32 = C.c_float
f64 = C.c_double


class PlaneBC(C.Structure):
    """Mirror of fc_plane_bc."""
    _fields_ = [("axis", C.c_int32), ("plane_idx", C.c_int32), ("interior_idx", C.c_int32),
                ("bc_type", C.c_int32), ("u_in_lat", C.c_float), ("rho_out_lat", C.c_float),
                ("sign", C.c_int32), ("pad", C.c_int32)]


class StepArgs(C.Structure):
    """Mirror of fc_lbm_step_args (include/fluxcore3d_gb300.h)."""

    _fields_ = [
        ("storage", C.c_int32),
        ("collision", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("periodic", C.c_int32 * 3),
        ("pop_in", vp),
        ("pop_out", vp),
        ("f32", vp),
        ("rho", vp),
        ("u", vp),
        ("v", vp),
        ("w", vp),
        ("cell_flags", vp),
        ("link_off", vp),
        ("link_hdr", vp),
        ("link_w", vp),
        ("n_links", i64),
        ("sponge", vp),
        ("sponge_axis", C.c_int32),
        ("has_links", C.c_int32),
        ("omega", f32),
        ("omega_plus", f32),
        ("omega_minus", f32),
        ("S", f32 * 19),
        ("Cs_dx2", f32),
        ("omega0", f32),
        ("dev_err", vp),
        ("link_cells", vp),
        ("n_link_cells", i64),
        ("phase_mask", C.c_int32),
        ("separate_link_pass", C.c_int32),
        ("cells_per_thread", C.c_int32),
        ("staging", C.c_int32),
        ("link_val", C.c_void_p),
        ("n_link_val", C.c_int64),
        ("tile_links", C.c_void_p),
        ("n_tile_links", C.c_int64),
        ("link_pos", C.c_void_p),
        ("n_link_pos", C.c_int64),
        ("link_src", C.c_void_p),
        ("n_link_src", C.c_int64),
        ("skip_link_gather", C.c_int32),
        ("tracer_in", vp),
        ("tracer_out", vp),
        ("tracer_u", vp),
        ("tracer_v", vp),
        ("tracer_w", vp),
        ("tracer_solid", vp),
        ("tracer_dissipation", f32),
        ("tile_order", C.c_int32),
        ("gather_order", C.c_int32),
    ]


ABI_VERSION = 2   # FC_ABI_VERSION of the header these mirrors follow


# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple] = {
    "fc_abi_version": (i32, []),
    "fc_lbm_step_args_size": (i64, []),
    # lattice, per-operation
    "fc_lbm_macro_collide_bgk": (i32, [vp, vp, vp, vp, vp, vp, vp, f32, i64, vp]),
    "fc_lbm_macro_collide_trt": (i32, [vp, vp, vp, vp, vp, vp, vp, f32, f32, i64, vp]),
    "fc_lbm_macro_collide_mrt": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, i64, vp]),
    "fc_lbm_macro_collide_mrt_smag": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, f32, f32, i64, vp]),
    "fc_lbm_stream_pull": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, vp]),
    "fc_lbm_sponge": (i32, [vp, vp, vp, vp, vp, vp, i64, vp]),
    "fc_lbm_ibb": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, i64, vp, vp]),
    "fc_lbm_reset_solid": (i32, [vp, vp, i64, vp]),
    "fc_lbm_zou_he_bc": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, f32, f32, i32, vp]),
    "fc_lbm_convective_workspace_bytes": (i64, [i32, i32]),
    "fc_lbm_convective_bc": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, f32, i32, i32, vp, i64, vp]),
    "fc_lbm_convective_noalloc_max_plane": (i64, []),
    "fc_lbm_convective_bc_noalloc": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, f32, i32, i32, vp]),
    # lattice, FP64 run of the plain method
    "fc_lbm64_macro_collide": (i32, [i32, vp, vp, vp, vp, vp, vp, vp, f32, f32, f32, vp, f32, f32, i64, vp]),
    "fc_lbm64_stream_pull": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, vp]),
    "fc_lbm64_sponge": (i32, [vp, vp, vp, vp, vp, vp, i64, vp]),
    "fc_lbm64_ibb": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, i64, vp, vp]),
    "fc_lbm64_reset_solid": (i32, [vp, vp, i64, vp]),
    "fc_lbm64_zou_he_bc": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, f64, f64, i32, vp]),
    "fc_lbm64_convective_bc": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, f64, i32, i32, vp, i64, vp]),
    # lattice, fused
    "fc_lbm_fused_step": (i32, [C.POINTER(StepArgs), vp]),
    "fc_lbm_link_gather": (i32, [C.POINTER(StepArgs), vp, C.c_int64, i32, vp]),
    "fc_lbm_planes_zou_he_collide": (i32, [C.POINTER(StepArgs), C.POINTER(PlaneBC), i32, vp]),
    "fc_lbm_wait_selftest": (i32, [C.c_uint, i32, vp, vp]),
    "fc_lbm_tile_links": (C.c_int64, [C.POINTER(StepArgs), vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, vp]),
    "fc_lbm_collide_from_f32": (i32, [C.POINTER(StepArgs), i32, i32, vp]),
    "fc_lbm_materialize": (i32, [C.POINTER(StepArgs), vp]),
    "fc_lbm_pin_solid": (i32, [C.POINTER(StepArgs), vp]),
    # multigrid
    "fc_mg_mop": (i32, [vp] * 9 + [f32, i32, i32, i32, i32, i32, vp]),
    "fc_mg_jacobi": (i32, [vp, vp, vp, vp, i64, vp]),
    "fc_mg_apply_L": (i32, [vp] * 9 + [f32, i32, i32, i32, i32, i32, vp]),
    "fc_mg_smooth": (i32, [vp] * 11 + [f32, i32, i32, i32, i32, i32, vp]),
    "fc_mg_smooth_first2": (i32, [vp] * 10 + [f32, i32, i32, i32, i32, i32, vp]),
    "fc_mg_smooth_small": (i32, [vp] * 10 + [f32, i32, i32, i32, i32, i32, i32, i32, vp]),
    "fc_mg_smooth_from_zero": (i32, [vp, vp, vp, i64, vp]),
    "fc_mg_residual_restrict": (i32, [vp] * 10 + [f32, i32, i32, i32, i32, i32, vp, i32, i32, i32, vp]),
    "fc_mg_prolong_correct": (i32, [vp, vp, vp, i32, i32, i32, i32, i32, i32, f32, vp]),
    "fc_mg_reduce_workspace_bytes": (i64, [i64]),
    "fc_mg_residual_norm2": (i32, [vp] * 10 + [f32, i32, i32, i32, i32, i32, vp, vp, i64, vp, vp]),
    "fc_mg_build_coeffs": (i32, [vp] * 5 + [i32, i32, i32, i32, i32, f32, f32] + [vp] * 7 + [vp]),
    "fc_mg_restrict_mean": (i32, [vp, i32, i32, i32, vp, i32, vp]),
    "fc_mg_inv_diag": (i32, [vp, vp, vp, f32, f32, i64, vp]),
    "fc_mg_coarse_dense_bytes": (i64, [i32, i32, i32]),
    "fc_mg_coarse_dense_build": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, f32, i32, i32, i32, i32, i32, vp, i64, vp]),
    "fc_mg_coarse_dense_apply": (i32, [vp, vp, vp, vp, i32, vp]),
    # krylov
    "fc_vec_workspace_bytes": (i64, [i64]),
    "fc_vec_dot": (i32, [i32, vp, vp, i64, vp, vp, i64, vp, vp]),
    "fc_vec_axpby": (i32, [i32, vp, vp, i64, f64, vp, vp, f64, vp, vp]),
    "fc_vec_convert": (i32, [i32, vp, vp, i64, vp, f64, vp]),
    "fc_vec_dot2_workspace_bytes": (C.c_int64, [C.c_int64]),
    "fc_vec_dot2": (i32, [i32, vp, vp, vp, C.c_int64, vp, C.c_int64, vp, vp]),
    "fc_bicgstab_p": (i32, [i32, vp, vp, vp, C.c_int64, vp, vp]),
    "fc_bicgstab_xr": (i32, [i32, vp, vp, vp, vp, C.c_int64, vp, i32, vp, C.c_int64, vp]),
    "fc_mg_mop_f64": (i32, [vp] * 8 + [f64, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
    "fc_mg_mop_f32": (i32, [vp] * 8 + [f32, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
    "fc_mg_mop_transpose_f32": (i32, [vp] * 7 + [f32, i32, i32, i32, i32, i32, vp, vp, vp]),
    # thermal
    "fc_thermal_rhs": (i32, [vp] * 7 + [f32, i64, vp]),
    "fc_thermal_reconstruct": (i32, [vp, vp, vp, i32, i32, i32, i32, i32, vp]),
    "fc_thermal_workspace_bytes": (i64, [i64]),
    "fc_thermal_convergence_metrics": (i32, [vp, vp, vp, i64, vp, i64, vp, vp]),
    "fc_thermal_physics_check": (i32, [vp, vp, f32, f32, i64, vp]),
    "fc_thermal_steady_residual": (i32, [vp] * 10 + [f32, i32, i32, i32, i32, i32, vp, i64, vp, vp]),
    # tcgen05 convolutions
    "fc_conv3d_fwd": (i32, [vp, vp, vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
    "fc_conv3d_dgrad_workspace_bytes": (i64, [i32, i32]),
    "fc_conv3d_dgrad": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, vp, i64, vp, vp, vp, vp]),
    "fc_conv3d_wgrad_workspace_bytes": (i64, [i32, i32, i32, i32, i32, i32, i32]),
    "fc_conv3d_wgrad": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, i64, vp, vp, vp]),
    # network glue
    "fc_nn_pack_input": (i32, [vp, vp, vp, i64, i64, f32, f32, vp, vp]),
    "fc_nn_avgpool2": (i32, [vp, i32, i32, i32, i32, i32, vp, vp]),
    "fc_nn_avgpool2_bwd": (i32, [vp, i32, i32, i32, i32, i32, vp, vp]),
    "fc_nn_upsample_concat": (i32, [vp, i32, vp, i32, i32, i32, i32, i32, vp, vp]),
    "fc_nn_upsample_concat_bwd": (i32, [vp, i32, i32, i32, i32, i32, i32, vp, vp, vp]),
    "fc_nn_act_bwd": (i32, [vp, vp, vp, i32, i64, vp, vp, vp]),
    "fc_nn_take_channel0": (i32, [vp, i32, vp, i64, i64, vp, vp, vp]),
    "fc_nn_mse_workspace_bytes": (i64, [i64]),
    "fc_nn_mse_grad": (i32, [vp, i32, vp, vp, i64, vp, vp, i64, vp]),
    "fc_nn_adam": (i32, [vp, vp, vp, vp, vp, i64, i32, i32, f32, f32, f32, f32, i32, f32, vp]),
    # geometry set-up
    "fc_geom_edt_workspace_bytes": (i64, [i32, i32, i32]),
    "fc_geom_signed_edt": (i32, [vp, i32, i32, i32, f64, vp, vp, i64, vp]),
    "fc_ibb_links_workspace_bytes": (i64, [i32, i32, i32]),
    "fc_ibb_count_links": (i32, [vp, i32, i32, i32, vp, i64, vp, vp]),
    "fc_ibb_build_links": (i32, [vp, i32, i32, i32, vp, i64, i64, vp, vp, vp, vp, vp, vp, vp]),
    "fc_ibb_q_from_sdf": (i32, [vp, i32, i32, i32, f32, f32, f32, f64, i32, vp, vp, i64, vp, vp, vp, vp, vp, vp]),
    "fc_ibb_weights_from_q": (i32, [vp, i64, vp, vp, vp, vp]),
    # snapshot / checkpoint I/O
    "fc_snapshot_pack": (i32, [vp, vp, vp, vp, vp, i64, i32, vp, vp]),
    "fc_columns_gather": (i32, [vp, i32, i64, vp, i64, vp, vp, vp]),
    "fc_columns_scatter": (i32, [vp, i32, i64, vp, i64, vp, vp, vp]),
    # STL voxelization, body stamping
    "fc_vox_prepared_floats": (i64, [i64]),
    "fc_vox_prepare_triangles": (i32, [vp, i64, f32, vp, vp]),
    "fc_vox_parity_z": (i32, [vp, i64, i32, i32, i32, f64, f64, f64, f64, f64, f64, vp, vp]),
    "fc_geom_stamp_body": (i32, [vp, i32, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp, vp, f32, f32, vp, vp,
                                 vp]),
    # FP64 conservation integrals
    "fc_lbm_mass_workspace_bytes": (i64, []),
    "fc_lbm_mass": (i32, [vp, i32, vp, i64, vp, i64, vp, vp]),
    "fc_mg_heat_balance_workspace_bytes": (i64, [i64]),
    "fc_mg_heat_balance": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, i32, i32, i32, i32, vp, i64, vp, vp]),
    # passive tracer
    "fc_tracer_step": (i32, [vp, vp, vp, vp, vp, vp, i32, i32, i32, f32, vp]),
    "fc_tracer_inject": (i32, [vp, vp, i64, vp]),
}

STATUS_TEXT = {1: "bad argument", 2: "CUDA launch failure", 3: "unsupported combination",
               4: "size exceeds the fixed capacity of this entry point"}


def lib_path() -> str:
    return _build.LIB_PATH


def _load():
    global _LIB, _LOAD_ERROR
    if _LIB is not None or _LOAD_ERROR is not None:
        return
    path = lib_path()
    if not os.path.exists(path):
        _LOAD_ERROR = f"{path} is not built (run fluxcore3d_gb300._build.build())"
        return
    try:
        L = C.CDLL(path)
    except OSError as e:  # pragma: no cover - depends on the machine
        _LOAD_ERROR = f"cannot load {path}: {e}"
        return
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    size_fn = getattr(L, "fc_lbm_step_args_size", None)
    if L.fc_abi_version() != ABI_VERSION or size_fn is None or size_fn() != C.sizeof(StepArgs):
        _LOAD_ERROR = (f"{path} was built from another version of the interface "
                       f"(ABI {L.fc_abi_version()}, expected {ABI_VERSION}): rebuild it")
        return
    _LIB = L


def load_error() -> str | None:
    _load()
    return _LOAD_ERROR


def lib():
    """The loaded library; raises RuntimeError if it cannot be used."""
    _load()
    if _LIB is None:
        raise RuntimeError(f"fluxcore3d_gb300 native library unavailable: {_LOAD_ERROR}")
    return _LIB


def exported_symbols() -> list[str]:
    """Names from SIGNATURES that the loaded library actually exports."""
    L = lib()
    return [n for n in SIGNATURES if hasattr(L, n)]


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed: {STATUS_TEXT.get(rc, f'status {rc}')}")


def call(name: str, *args) -> int:
    fn = getattr(lib(), name)
    rc = fn(*args)
    if fn.restype is i32:
        check(rc, name)
    return rc
