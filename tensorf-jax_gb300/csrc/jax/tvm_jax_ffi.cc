// XLA FFI handlers over the C ABI, so that tensorf-jax's own Python code can call the
// GB300 kernels from inside jax.jit (jax.ffi.ffi_call) with jax.custom_vjp gradients.
//
// One handler per seam of the reference:
//   TensorVM.interpolate            tensorf/tensor_vm.py:42-89   tvm_vm_features_{fwd,bwd}
//   compute_segment_probabilities   tensorf/render.py:300-347    tvm_composite_{fwd,bwd}
//   FeatureMlp.__call__             tensorf/networks.py:45-121   tvm_mlp_{fwd,bwd}, tvm_mlp_fwd_static_scratch
//   render_rays (one chunk)         tensorf/render.py:105-279    tvm_render_fwd
// Each handler only unpacks XLA's buffers and attributes into the C ABI's plain
// pointers and sizes; every check and launch is the library's. XLA owns every buffer:
// the scratch a call needs is an extra result buffer (a u8 array sized by the matching
// *_workspace_size call, which tensorf_gb300/jax_ops.py requests), except for the
// static-scratch MLP forward, which needs none. Gradient results are zeroed here
// first because the C ABI accumulates into them.
//
// Build (where jaxlib >= 0.4.31 provides the FFI headers; JAX is not part of this
// image, so build() skips it when jax.ffi is missing):
//   g++ -std=c++17 -O2 -shared -fPIC -I"$(python -c 'import jax.ffi; print(jax.ffi.include_dir())')"
//       -I include -I /usr/local/cuda/include tvm_jax_ffi.cc -L<pkg> -ltensorf_gb300 -o libtvm_jax_ffi.so
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "tensorf_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(int status, const char* what) {
  if (status == TVM_OK) return ffi::Error::Success();
  return ffi::Error(status == TVM_ERR_LAUNCH ? ffi::ErrorCode::kInternal : ffi::ErrorCode::kInvalidArgument,
                    std::string(what) + ": " + tvm_last_error_message());
}

ffi::Error zero(cudaStream_t s, void* p, size_t bytes, const char* what) {
  if (bytes == 0) return ffi::Error::Success();
  if (cudaMemsetAsync(p, 0, bytes, s) != cudaSuccess)
    return ffi::Error(ffi::ErrorCode::kInternal, std::string(what) + ": cudaMemsetAsync failed");
  return ffi::Error::Success();
}

// The FeatureMlp / model attributes every MLP and render handler takes.
tvm_model_desc model_desc(int32_t grid, int32_t density_channels, int32_t appearance_channels, int32_t feature_n_freqs,
                          int32_t viewdir_n_freqs, int32_t dtype) {
  tvm_model_desc m{};
  m.grid_dim = grid;
  m.density_channels = density_channels;
  m.appearance_channels = appearance_channels;
  m.feature_n_freqs = feature_n_freqs;
  m.viewdir_n_freqs = viewdir_n_freqs;
  m.squash_dim = 27;
  m.units = 128;
  m.dtype = dtype;
  m.mlp_math = TVM_MLP_DEFAULT;
  return m;
}

// ---- TensorVM.interpolate -----------------------------------------------------------
// lines [3][G][C], planes [3][G][G][C] (channel-last f32), ijk (3, n) -> out (3C, n).
ffi::Error VmFeaturesFwd(cudaStream_t s, ffi::Buffer<ffi::F32> lines, ffi::Buffer<ffi::F32> planes,
                         ffi::Buffer<ffi::F32> ijk, ffi::ResultBuffer<ffi::F32> out, int32_t grid, int32_t channels) {
  tvm_vm_field f{grid, channels, TVM_F32, 0, lines.typed_data(), planes.typed_data()};
  const int64_t n = static_cast<int64_t>(ijk.element_count() / 3);
  return status_error(tvm_vm_features_fwd(&f, ijk.typed_data(), n, out->typed_data(), s), "tvm_vm_features_fwd");
}

ffi::Error VmFeaturesBwd(cudaStream_t s, ffi::Buffer<ffi::F32> lines, ffi::Buffer<ffi::F32> planes,
                         ffi::Buffer<ffi::F32> ijk, ffi::Buffer<ffi::F32> grad_out,
                         ffi::ResultBuffer<ffi::F32> grad_lines, ffi::ResultBuffer<ffi::F32> grad_planes,
                         int32_t grid, int32_t channels) {
  tvm_vm_field f{grid, channels, TVM_F32, 0, lines.typed_data(), planes.typed_data()};
  const int64_t n = static_cast<int64_t>(ijk.element_count() / 3);
  ffi::Error e = zero(s, grad_lines->typed_data(), grad_lines->size_bytes(), "grad_lines");
  if (e.failure()) return e;
  e = zero(s, grad_planes->typed_data(), grad_planes->size_bytes(), "grad_planes");
  if (e.failure()) return e;
  return status_error(tvm_vm_features_bwd(&f, ijk.typed_data(), n, grad_out.typed_data(), grad_lines->typed_data(),
                                          grad_planes->typed_data(), s),
                      "tvm_vm_features_bwd");
}

// ---- compute_segment_probabilities -----------------------------------------------------
ffi::Error CompositeFwd(cudaStream_t s, ffi::Buffer<ffi::F32> sigmas, ffi::Buffer<ffi::F32> steps,
                        ffi::ResultBuffer<ffi::F32> p_exits, ffi::ResultBuffer<ffi::F32> p_terminates,
                        int32_t samples) {
  const int64_t rays = static_cast<int64_t>(sigmas.element_count()) / samples;
  return status_error(tvm_composite_fwd(sigmas.typed_data(), steps.typed_data(), rays, samples, p_exits->typed_data(),
                                        p_terminates->typed_data(), s),
                      "tvm_composite_fwd");
}

ffi::Error CompositeBwd(cudaStream_t s, ffi::Buffer<ffi::F32> sigmas, ffi::Buffer<ffi::F32> steps,
                        ffi::Buffer<ffi::F32> grad_p_exits, ffi::Buffer<ffi::F32> grad_p_terminates,
                        ffi::ResultBuffer<ffi::F32> grad_sigmas, int32_t samples) {
  const int64_t rays = static_cast<int64_t>(sigmas.element_count()) / samples;
  return status_error(tvm_composite_bwd(sigmas.typed_data(), steps.typed_data(), rays, samples,
                                        grad_p_exits.typed_data(), grad_p_terminates.typed_data(),
                                        grad_sigmas->typed_data(), s),
                      "tvm_composite_bwd");
}

// ---- FeatureMlp --------------------------------------------------------------------------
// params: the flat parameter buffer of tvm_get_param_layout (f32); features (n, 3C),
// viewdirs (n, 3) -> rgb (n, 3); workspace: u8[tvm_mlp_workspace_size].
ffi::Error MlpFwd(cudaStream_t s, ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> features,
                  ffi::Buffer<ffi::F32> viewdirs, ffi::ResultBuffer<ffi::F32> rgb, ffi::ResultBuffer<ffi::U8> workspace,
                  int32_t grid, int32_t density_channels, int32_t appearance_channels, int32_t feature_n_freqs,
                  int32_t viewdir_n_freqs, int32_t dtype) {
  const tvm_model_desc m =
      model_desc(grid, density_channels, appearance_channels, feature_n_freqs, viewdir_n_freqs, dtype);
  const int64_t n = static_cast<int64_t>(viewdirs.element_count() / 3);
  return status_error(tvm_mlp_fwd(&m, params.typed_data(), features.typed_data(), viewdirs.typed_data(), nullptr,
                                  n, rgb->typed_data(), workspace->typed_data(), workspace->size_bytes(), s),
                      "tvm_mlp_fwd");
}

// The same forward with no scratch buffer from XLA: the library's static array.
ffi::Error MlpFwdStatic(cudaStream_t s, ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> features,
                        ffi::Buffer<ffi::F32> viewdirs, ffi::ResultBuffer<ffi::F32> rgb, int32_t grid,
                        int32_t density_channels, int32_t appearance_channels, int32_t feature_n_freqs,
                        int32_t viewdir_n_freqs, int32_t dtype) {
  const tvm_model_desc m =
      model_desc(grid, density_channels, appearance_channels, feature_n_freqs, viewdir_n_freqs, dtype);
  const int64_t n = static_cast<int64_t>(viewdirs.element_count() / 3);
  return status_error(tvm_mlp_fwd_static_scratch(&m, params.typed_data(), features.typed_data(),
                                                 viewdirs.typed_data(), n, rgb->typed_data(), s),
                      "tvm_mlp_fwd_static_scratch");
}

// grad_rgb (n, 3) -> grad_features (n, 3C) and grad_params (flat layout, zeroed here).
ffi::Error MlpBwd(cudaStream_t s, ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> features,
                  ffi::Buffer<ffi::F32> viewdirs, ffi::Buffer<ffi::F32> grad_rgb,
                  ffi::ResultBuffer<ffi::F32> grad_features, ffi::ResultBuffer<ffi::F32> grad_params,
                  ffi::ResultBuffer<ffi::U8> workspace, int32_t grid, int32_t density_channels,
                  int32_t appearance_channels, int32_t feature_n_freqs, int32_t viewdir_n_freqs, int32_t dtype) {
  const tvm_model_desc m =
      model_desc(grid, density_channels, appearance_channels, feature_n_freqs, viewdir_n_freqs, dtype);
  const int64_t n = static_cast<int64_t>(viewdirs.element_count() / 3);
  ffi::Error e = zero(s, grad_params->typed_data(), grad_params->size_bytes(), "grad_params");
  if (e.failure()) return e;
  return status_error(tvm_mlp_bwd(&m, params.typed_data(), features.typed_data(), viewdirs.typed_data(), nullptr,
                                  n, grad_rgb.typed_data(), grad_features->typed_data(), grad_params->typed_data(),
                                  workspace->typed_data(), workspace->size_bytes(), s),
                      "tvm_mlp_bwd");
}

// ---- render_rays, one chunk (bounded scene, RGB or distance mode) ------------------------------
// origins, directions (R, 3); jitter (N,) and gumbel (N,) replay the reference's draws.
ffi::Error RenderFwd(cudaStream_t s, ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> origins,
                     ffi::Buffer<ffi::F32> directions, ffi::Buffer<ffi::F32> jitter, ffi::Buffer<ffi::F32> gumbel,
                     ffi::ResultBuffer<ffi::F32> out, ffi::ResultBuffer<ffi::U8> workspace, int32_t grid,
                     int32_t density_channels, int32_t appearance_channels, int32_t feature_n_freqs,
                     int32_t viewdir_n_freqs, int32_t density_samples, int32_t appearance_samples, int32_t mode,
                     float density_shift, float aabb_min, float aabb_max) {
  const tvm_model_desc m =
      model_desc(grid, density_channels, appearance_channels, feature_n_freqs, viewdir_n_freqs, TVM_F32);
  tvm_render_desc c{};
  c.density_samples = density_samples;
  c.appearance_samples = appearance_samples;
  c.mode = mode;
  c.sampler = TVM_SAMPLER_BBOX;
  c.density_shift = density_shift;
  for (int a = 0; a < 3; ++a) {
    c.aabb[a] = aabb_min;
    c.aabb[3 + a] = aabb_max;
  }
  c.jitter = jitter.typed_data();
  c.gumbel = gumbel.typed_data();
  tvm_rays rays{static_cast<int64_t>(origins.element_count() / 3), origins.typed_data(), directions.typed_data()};
  return status_error(tvm_render_fwd(&m, params.typed_data(), nullptr, &rays, &c, out->typed_data(),
                                     workspace->typed_data(), workspace->size_bytes(), s),
                      "tvm_render_fwd");
}

}  // namespace

#define TVM_MODEL_ATTRS(b)                                                                                  \
  (b).Attr<int32_t>("grid").Attr<int32_t>("density_channels").Attr<int32_t>("appearance_channels")           \
      .Attr<int32_t>("feature_n_freqs").Attr<int32_t>("viewdir_n_freqs")

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_vm_features_fwd_ffi, VmFeaturesFwd,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Attr<int32_t>("grid")
                                  .Attr<int32_t>("channels"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_vm_features_bwd_ffi, VmFeaturesBwd,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Attr<int32_t>("grid")
                                  .Attr<int32_t>("channels"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_composite_fwd_ffi, CompositeFwd,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Attr<int32_t>("samples"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_composite_bwd_ffi, CompositeBwd,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Attr<int32_t>("samples"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_mlp_fwd_ffi, MlpFwd,
                              TVM_MODEL_ATTRS(ffi::Ffi::Bind()
                                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::U8>>())
                                  .Attr<int32_t>("dtype"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_mlp_fwd_static_ffi, MlpFwdStatic,
                              TVM_MODEL_ATTRS(ffi::Ffi::Bind()
                                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::F32>>())
                                  .Attr<int32_t>("dtype"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_mlp_bwd_ffi, MlpBwd,
                              TVM_MODEL_ATTRS(ffi::Ffi::Bind()
                                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::U8>>())
                                  .Attr<int32_t>("dtype"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(tvm_render_fwd_ffi, RenderFwd,
                              TVM_MODEL_ATTRS(ffi::Ffi::Bind()
                                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Arg<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::F32>>()
                                                  .Ret<ffi::Buffer<ffi::U8>>())
                                  .Attr<int32_t>("density_samples")
                                  .Attr<int32_t>("appearance_samples")
                                  .Attr<int32_t>("mode")
                                  .Attr<float>("density_shift")
                                  .Attr<float>("aabb_min")
                                  .Attr<float>("aabb_max"));
