"""ctypes binding of the C ABI declared in ``include/tensorf_gb300.h``.

The library is loaded from this package directory (built in-tree by ``_build.py``).
There is no fallback: if the shared library is missing or a CUDA device is absent the
calls fail loudly.
"""
from __future__ import annotations

import ctypes
import pathlib
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_int64, c_size_t, c_uint64, c_void_p

PKG_DIR = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libtensorf_gb300.so"

ABI_VERSION = 3  # TVM_ABI_VERSION of include/tensorf_gb300.h
TVM_OK = 0
ERROR_NAMES = {
    -1: "TVM_ERR_INVALID",
    -2: "TVM_ERR_SHAPE",
    -3: "TVM_ERR_DTYPE",
    -4: "TVM_ERR_ALIGN",
    -5: "TVM_ERR_UNSUPPORTED",
    -6: "TVM_ERR_LAUNCH",
    -7: "TVM_ERR_NONFINITE",
    -8: "TVM_ERR_TIMEOUT",
    -9: "TVM_ERR_WORKSPACE",
}
TVM_F32, TVM_BF16, TVM_F64 = 0, 1, 2
TVM_MLP_DEFAULT, TVM_MLP_SIMT_F32 = 0, 1
TVM_MODE_RGB, TVM_MODE_DIST_MEDIAN, TVM_MODE_DIST_MEAN = 0, 1, 2
TVM_SAMPLER_BBOX, TVM_SAMPLER_CONTRACT, TVM_SAMPLER_PROPOSAL = 0, 1, 2


class VmField(ctypes.Structure):
    _fields_ = [("grid_dim", c_int32), ("channels", c_int32), ("dtype", c_int32), ("_pad", c_int32),
                ("lines", c_void_p), ("planes", c_void_p)]


class ModelDesc(ctypes.Structure):
    _fields_ = [("grid_dim", c_int32), ("density_channels", c_int32), ("appearance_channels", c_int32),
                ("feature_n_freqs", c_int32), ("viewdir_n_freqs", c_int32), ("squash_dim", c_int32),
                ("units", c_int32), ("dtype", c_int32), ("mlp_math", c_int32), ("proposal_grid", c_int32),
                ("proposal_rank", c_int32), ("proposal_units", c_int32), ("num_cameras", c_int32)]


class ParamLayout(ctypes.Structure):
    _fields_ = [(n, c_int64) for n in (
        "density_lines", "density_planes", "appearance_lines", "appearance_planes",
        "mlp_w0", "mlp_w1", "mlp_b1", "mlp_w2", "mlp_b2", "mlp_w3", "mlp_b3",
        "proposal_lines", "proposal_planes", "proposal_w1", "proposal_b1", "proposal_w2", "proposal_b2",
        "mlp_begin", "total",
        "shadow_density_lines", "shadow_density_planes", "shadow_appearance_lines",
        "shadow_appearance_planes", "shadow_proposal_lines", "shadow_proposal_planes",
        "shadow_total")] + [("encoded_dim", c_int32), ("_pad", c_int32), ("mlp_embed", c_int64)]


class Rays(ctypes.Structure):
    _fields_ = [("count", c_int64), ("origins", c_void_p), ("directions", c_void_p), ("camera_indices", c_void_p)]


class RenderDesc(ctypes.Structure):
    _fields_ = [("density_samples", c_int32), ("appearance_samples", c_int32), ("mode", c_int32),
                ("sampler", c_int32), ("density_shift", c_float), ("_pad0", c_float),
                ("aabb", c_float * 6), ("schedule", c_void_p), ("jitter", c_void_p),
                ("jitter_per_ray", c_int32), ("gumbel_per_ray", c_int32), ("gumbel", c_void_p),
                ("proposal_samples", c_int32), ("contract", c_int32), ("proposal_jitter", c_void_p),
                ("proposal_shift", c_float), ("proposal_loss_weight", c_float)]


class AdamDesc(ctypes.Structure):
    _fields_ = [("lr_tensor", c_float), ("lr_mlp", c_float), ("b1", c_float), ("b2", c_float),
                ("eps", c_float), ("lr_decay", c_float), ("count", c_int32), ("defer_fields", c_int32),
                ("grad_sq", c_void_p), ("device_step", c_void_p), ("pending_count", c_int32),
                ("pending_lr_decay", c_float)]


class NoiseJob(ctypes.Structure):
    _fields_ = [("dst", c_void_p), ("n", c_int64), ("mul", c_uint64), ("add", c_uint64), ("kind", c_int32),
                ("_pad", c_int32)]


NOISE_BATCH_MAX = 4

# name -> (restype, argtypes)
_SIGNATURES = {
    "tvm_abi_version": (c_int32, []),
    "tvm_last_error_message": (c_char_p, []),
    "tvm_kernel_launches": (c_uint64, []),
    "tvm_set_phase_events": (c_int32, [POINTER(c_void_p), c_int32]),
    "tvm_get_param_layout": (c_int32, [POINTER(ModelDesc), POINTER(ParamLayout)]),
    "tvm_vm_to_channel_last": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p]),
    "tvm_vm_to_channel_first": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tvm_vm_features_fwd": (c_int32, [POINTER(VmField), c_void_p, c_int64, c_void_p, c_void_p]),
    "tvm_vm_features_bwd": (c_int32, [POINTER(VmField), c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tvm_sample_points": (c_int32, [POINTER(Rays), POINTER(RenderDesc), c_void_p, c_void_p, c_void_p, c_void_p]),
    "tvm_composite_fwd": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_void_p]),
    "tvm_composite_bwd": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tvm_topk_select": (c_int32, [c_void_p, c_void_p, c_int32, c_int64, c_int32, c_int32, c_void_p, c_void_p]),
    "tvm_mlp_workspace_size": (c_size_t, [POINTER(ModelDesc), c_int64]),
    "tvm_mlp_fwd": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                              c_void_p, c_size_t, c_void_p]),
    "tvm_mlp_bwd": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "tvm_mlp_fwd_static_scratch": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                            c_void_p]),
    "tvm_proposal_fwd": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, POINTER(Rays), POINTER(RenderDesc),
                                   c_void_p, c_void_p, c_void_p]),
    "tvm_proposal_resample": (c_int32, [POINTER(Rays), POINTER(RenderDesc), c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p]),
    "tvm_proposal_loss": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_int32, c_int32, c_float, c_void_p,
                                    c_void_p, c_void_p]),
    "tvm_proposal_bwd": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, POINTER(Rays),
                                   POINTER(RenderDesc), c_void_p, c_void_p, c_void_p]),
    "tvm_loss_f64_workspace_size": (c_size_t, [POINTER(ModelDesc), POINTER(RenderDesc), c_int64]),
    "tvm_loss_f64": (c_int32, [POINTER(ModelDesc), c_void_p, POINTER(Rays), c_void_p, POINTER(RenderDesc), c_int64,
                               ctypes.c_double, c_void_p, c_void_p, c_size_t, c_void_p]),
    "tvm_resize_field": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tvm_gemm": (c_int32, [c_int32, c_int32, c_int32, c_int64, c_int32, c_int64, c_void_p, c_int64, c_void_p,
                           c_int64, c_void_p, c_int64, c_int32, c_void_p]),
    "tvm_device_status": (c_int32, [POINTER(c_int32), c_void_p]),
    "tvm_render_workspace_size": (c_size_t, [POINTER(ModelDesc), POINTER(RenderDesc), c_int64]),
    "tvm_render_fwd": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, POINTER(Rays), POINTER(RenderDesc),
                                 c_void_p, c_void_p, c_size_t, c_void_p]),
    "tvm_train_workspace_size": (c_size_t, [POINTER(ModelDesc), POINTER(RenderDesc), c_int64]),
    "tvm_train_step": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 POINTER(AdamDesc), POINTER(Rays), c_void_p, POINTER(RenderDesc), c_void_p,
                                 c_void_p, c_size_t, c_void_p]),
    "tvm_loss_and_grad": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, POINTER(Rays), c_void_p,
                                    POINTER(RenderDesc), c_void_p, c_void_p, c_size_t, c_void_p]),
    "tvm_adam_step": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_void_p, POINTER(AdamDesc),
                                c_void_p, c_void_p]),
    "tvm_set_step_scalars": (c_int32, [c_void_p, c_int32, c_float, c_uint64, c_int32, c_float, c_void_p]),
    "tvm_apply_pending_fields": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                           POINTER(AdamDesc), c_void_p]),
    "tvm_noise_fill_keyed": (c_int32, [c_void_p, c_int64, c_uint64, c_void_p, c_uint64, c_uint64, c_int32, c_void_p]),
    "tvm_noise_fill_keyed_batch": (c_int32, [POINTER(NoiseJob), c_int32, c_uint64, c_void_p, c_void_p]),
    "tvm_refresh_shadow": (c_int32, [POINTER(ModelDesc), c_void_p, c_void_p, c_void_p]),
    "tvm_l2_probe": (c_int32, [c_int32, c_void_p, c_size_t, c_int32, c_void_p]),
    "tvm_noise_fill": (c_int32, [c_void_p, c_int64, c_uint64, c_uint64, c_int32, c_void_p]),
    "tvm_camera_rays": (c_int32, [POINTER(c_double), POINTER(c_double), POINTER(c_double), c_int32, c_int32,
                                  c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "tvm_sphere_scene_render": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_double, c_void_p,
                                          POINTER(Rays), c_int32, c_void_p, c_void_p]),
}


class TvmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


_LIB = None


def load() -> ctypes.CDLL:
    """Load the in-tree shared library (once) and declare every signature."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH.name} is not built; run __graft_entry__.build() (or "
                           f"python {PKG_DIR / '_build.py'}) first")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.tvm_abi_version() != ABI_VERSION:
        raise RuntimeError("ABI version mismatch")
    _LIB = lib
    return lib


def exported_symbols():
    return list(_SIGNATURES)


def check(status: int) -> None:
    if status != TVM_OK:
        msg = load().tvm_last_error_message()
        raise TvmError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
