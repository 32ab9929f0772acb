"""The GB300 kernels as jax.ffi custom calls, with jax.custom_vjp gradients, for the
reference's own JAX code.

tensorf-jax calls these seams inside ``jax.jit`` (tensorf/training.py:101-205):

* ``TensorVM.interpolate`` (tensorf/tensor_vm.py:42-89) -> :func:`vm_interpolate`
* ``compute_segment_probabilities`` (tensorf/render.py:300-347) ->
  :func:`compute_segment_probabilities`
* ``FeatureMlp.__call__`` (tensorf/networks.py:45-121) -> :func:`feature_mlp`
* ``render_rays`` for one chunk of a bounded scene (tensorf/render.py:105-279) ->
  :func:`render_rays_chunk` (forward only, as ``render_rays_batched`` uses it)

Each wrapper registers a handler of ``libtvm_jax_ffi.so`` (built from
``csrc/jax/tvm_jax_ffi.cc`` by :func:`build`) and calls it with ``jax.ffi.ffi_call``.
Field tensors are passed channel-last (``tvm_vm_to_channel_last`` layout); the MLP
takes the flat parameter buffer of ``tvm_get_param_layout``. Scratch memory is an
extra u8 result buffer sized by the library, so XLA's allocator owns it.

Needs jax >= 0.4.31 with CUDA. JAX is not part of this image, so nothing else in
tensorf_gb300 imports this module, and ``_build.build()`` compiles the shim only where
``jax.ffi`` exists.
"""
from __future__ import annotations

import ctypes
import pathlib
from functools import partial

PKG_DIR = pathlib.Path(__file__).resolve().parent
SHIM_LIB = PKG_DIR / "libtvm_jax_ffi.so"

# Every handler symbol the shim defines; registered under the same name.
HANDLERS = (
    "tvm_vm_features_fwd_ffi",
    "tvm_vm_features_bwd_ffi",
    "tvm_composite_fwd_ffi",
    "tvm_composite_bwd_ffi",
    "tvm_mlp_fwd_ffi",
    "tvm_mlp_fwd_static_ffi",
    "tvm_mlp_bwd_ffi",
    "tvm_render_fwd_ffi",
)


def build(verbose: bool = False) -> pathlib.Path:
    """Compile libtvm_jax_ffi.so against jax's FFI headers and libtensorf_gb300.so."""
    from . import _build

    return _build.build_jax_shim(verbose)


_REGISTERED = False


def register() -> None:
    """Register every handler with XLA for the CUDA platform (once)."""
    global _REGISTERED
    if _REGISTERED:
        return
    import jax.ffi

    from . import _lib

    _lib.load()  # the kernels' library first, so the shim's dependency resolves in-tree
    so = ctypes.cdll.LoadLibrary(str(SHIM_LIB))
    for name in HANDLERS:
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(so, name)), platform="CUDA")
    _REGISTERED = True


def _model_attrs(spec):
    import numpy as np

    return dict(grid=np.int32(spec.grid_dim), density_channels=np.int32(spec.density_feat_dim),
                appearance_channels=np.int32(spec.appearance_feat_dim),
                feature_n_freqs=np.int32(spec.feature_n_freqs), viewdir_n_freqs=np.int32(spec.viewdir_n_freqs))


def _mlp_workspace_bytes(spec, n: int) -> int:
    from . import _lib

    md = spec.desc()
    return int(_lib.load().tvm_mlp_workspace_size(ctypes.byref(md), int(n)))


# ---- TensorVM.interpolate ---------------------------------------------------------------
def _vm_call(lines, planes, ijk):
    import jax
    import jax.numpy as jnp
    import numpy as np

    register()
    C = lines.shape[-1]
    out = jax.ShapeDtypeStruct((3 * C, ijk.shape[1]), jnp.float32)
    return jax.ffi.ffi_call("tvm_vm_features_fwd_ffi", out)(lines, planes, ijk, grid=np.int32(lines.shape[1]),
                                                            channels=np.int32(C))


def _make_vm_interpolate():
    import jax
    import jax.numpy as jnp
    import numpy as np

    @jax.custom_vjp
    def vm_interpolate(lines, planes, ijk):
        """(3C, n) features of channel-last lines [3][G][C] / planes [3][G][G][C] at
        ijk (3, n) in [-1, 1] (TensorVM.interpolate, tensor_vm.py:42-89)."""
        return _vm_call(lines, planes, ijk)

    def fwd(lines, planes, ijk):
        return _vm_call(lines, planes, ijk), (lines, planes, ijk)

    def bwd(res, g):
        lines, planes, ijk = res
        C = lines.shape[-1]
        gl, gp = jax.ffi.ffi_call("tvm_vm_features_bwd_ffi",
                                  (jax.ShapeDtypeStruct(lines.shape, jnp.float32),
                                   jax.ShapeDtypeStruct(planes.shape, jnp.float32)))(
            lines, planes, ijk, g, grid=np.int32(lines.shape[1]), channels=np.int32(C))
        return gl, gp, jnp.zeros_like(ijk)

    vm_interpolate.defvjp(fwd, bwd)
    return vm_interpolate


# ---- compute_segment_probabilities ------------------------------------------------------------
def _make_segment_probabilities():
    import jax
    import jax.numpy as jnp
    import numpy as np

    def call(sigmas, step_sizes):
        register()
        sd = jax.ShapeDtypeStruct(sigmas.shape, jnp.float32)
        return jax.ffi.ffi_call("tvm_composite_fwd_ffi", (sd, sd))(sigmas, step_sizes,
                                                                   samples=np.int32(sigmas.shape[-1]))

    @jax.custom_vjp
    def compute_segment_probabilities(sigmas, step_sizes):
        """(p_exits, p_terminates), each shaped like sigmas (render.py:300-347)."""
        return call(sigmas, step_sizes)

    def fwd(sigmas, step_sizes):
        return call(sigmas, step_sizes), (sigmas, step_sizes)

    def bwd(res, g):
        sigmas, step_sizes = res
        g_pe, g_pt = g
        gs = jax.ffi.ffi_call("tvm_composite_bwd_ffi", jax.ShapeDtypeStruct(sigmas.shape, jnp.float32))(
            sigmas, step_sizes, g_pe, g_pt, samples=np.int32(sigmas.shape[-1]))
        return gs, jnp.zeros_like(step_sizes)

    compute_segment_probabilities.defvjp(fwd, bwd)
    return compute_segment_probabilities


# ---- FeatureMlp ----------------------------------------------------------------------------------
def _make_feature_mlp():
    import jax
    import jax.numpy as jnp
    import numpy as np

    def call(spec, params, features, viewdirs):
        register()
        n = features.shape[0]
        outs = (jax.ShapeDtypeStruct((n, 3), jnp.float32),
                jax.ShapeDtypeStruct((_mlp_workspace_bytes(spec, n),), jnp.uint8))
        rgb, _ = jax.ffi.ffi_call("tvm_mlp_fwd_ffi", outs)(params, features, viewdirs, **_model_attrs(spec),
                                                             dtype=np.int32(spec.desc().dtype))
        return rgb

    @partial(jax.custom_vjp, nondiff_argnums=(0,))
    def feature_mlp(spec, params, features, viewdirs):
        """rgb (n, 3) of FeatureMlp (networks.py:45-121) from the flat parameter buffer,
        features (n, 3C) and view directions (n, 3)."""
        return call(spec, params, features, viewdirs)

    def fwd(spec, params, features, viewdirs):
        return call(spec, params, features, viewdirs), (params, features, viewdirs)

    def bwd(spec, res, g):
        params, features, viewdirs = res
        n = features.shape[0]
        outs = (jax.ShapeDtypeStruct(features.shape, jnp.float32), jax.ShapeDtypeStruct(params.shape, jnp.float32),
                jax.ShapeDtypeStruct((_mlp_workspace_bytes(spec, n),), jnp.uint8))
        gf, gp, _ = jax.ffi.ffi_call("tvm_mlp_bwd_ffi", outs)(params, features, viewdirs, g, **_model_attrs(spec),
                                                               dtype=np.int32(spec.desc().dtype))
        return gp, gf, jnp.zeros_like(viewdirs)

    feature_mlp.defvjp(fwd, bwd)
    return feature_mlp


def feature_mlp_static(spec, params, features, viewdirs):
    """The FeatureMlp forward on the library's static scratch (no workspace buffer from
    XLA): for handlers that must not take device memory from XLA's allocator."""
    import jax
    import jax.numpy as jnp
    import numpy as np

    register()
    out = jax.ShapeDtypeStruct((features.shape[0], 3), jnp.float32)
    return jax.ffi.ffi_call("tvm_mlp_fwd_static_ffi", out)(params, features, viewdirs, **_model_attrs(spec),
                                                           dtype=np.int32(spec.desc().dtype))


# ---- render_rays ------------------------------------------------------------------------------------
def render_rays_chunk(spec, params, origins, directions, jitter, gumbel, *, density_samples: int,
                      appearance_samples: int, mode: int = 0, density_shift: float = 10.0,
                      aabb=(-1.0, 1.0)):
    """render_rays (render.py:105-279) for one chunk of rays of a bounded scene with a
    cubic aabb, FP32 model: rgb (R, 3) for mode 0, distances (R,) otherwise. ``jitter``
    (N,) and ``gumbel`` (N,) are the reference's draws from its PRNG keys."""
    import jax
    import jax.numpy as jnp
    import numpy as np

    from . import _lib

    register()
    R = origins.shape[0]
    desc = _lib.RenderDesc()
    desc.density_samples, desc.appearance_samples, desc.mode = density_samples, appearance_samples, mode
    desc.sampler = _lib.TVM_SAMPLER_BBOX
    for a in range(3):
        desc.aabb[a], desc.aabb[3 + a] = aabb[0], aabb[1]
    desc.gumbel = 1  # any non-NULL value: the size query checks that RGB mode will get a Gumbel array
    md = spec.desc()
    ws = int(_lib.load().tvm_render_workspace_size(ctypes.byref(md), ctypes.byref(desc), R))
    out_shape = (R, 3) if mode == 0 else (R,)
    outs = (jax.ShapeDtypeStruct(out_shape, jnp.float32), jax.ShapeDtypeStruct((ws,), jnp.uint8))
    out, _ = jax.ffi.ffi_call("tvm_render_fwd_ffi", outs)(
        params, origins, directions, jitter, gumbel, **_model_attrs(spec), density_samples=np.int32(density_samples),
        appearance_samples=np.int32(appearance_samples), mode=np.int32(mode), density_shift=np.float32(density_shift),
        aabb_min=np.float32(aabb[0]), aabb_max=np.float32(aabb[1]))
    return out


vm_interpolate = _make_vm_interpolate()
compute_segment_probabilities = _make_segment_probabilities()
feature_mlp = _make_feature_mlp()
