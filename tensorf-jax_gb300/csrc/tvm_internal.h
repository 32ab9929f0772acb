// Internal launchers shared between the translation units of the library.
#pragma once

#include <cuda_runtime.h>

#include "tvm_common.cuh"
#include "tvm_sampler.cuh"

namespace tvm {

// ---- per-device launch set-up (tvm_api.cu) ----
// SM count of the current device (looked up once per device).
int device_sms();
// Raise fn's dynamic shared-memory limit to at least `bytes` on the current device.
// Kernel attributes are per device, so this is done once per (device, kernel); safe to
// call from several host threads.
int ensure_smem_limit(const void* fn, int bytes, const char* what);

// Field view with a typed storage pointer (dtype decides the cast).
struct FieldView {
  int G, C, dtype;
  const void* lines;
  const void* planes;
};

// ---- VM feature kernels (tvm_vm.cu) ----
int launch_vm_features_fwd(const FieldView& f, const float* coords, int64_t n, float* out,
                           cudaStream_t st);
int launch_vm_features_bwd(const FieldView& f, const float* coords, int64_t n,
                           const float* grad_out, float* glines, float* gplanes, cudaStream_t st);
int launch_density_fwd(const FieldView& f, float shift, const float* origins, const float* dirs,
                       int64_t R, const SamplerArgs& s, float* sigma, cudaStream_t st);
int launch_density_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins,
                       const float* dirs, int64_t R, const SamplerArgs& s, const float* gsum,
                       cudaStream_t st);
int launch_appearance_fwd(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                          const SamplerArgs& s, const int32_t* sel_idx, int k, float* X0,
                          cudaStream_t st);
// FeatureMlp input tiles of BF16 models: X0 stored as the fused MLP kernels' A-operand
// images, one per 128 rows: 144 bf16 features per row in the tcgen05 K-major canonical
// layout (core matrices of 8 rows x 16 bytes, K-chunks 128 bytes apart, 8-row groups
// 2304 bytes apart). One bulk copy moves a tile into shared memory. Rows past the last
// are zero.
constexpr int X0T_ROWS = 128, X0T_FEAT = 144, X0T_SBO = (X0T_FEAT / 8) * 128;
constexpr int64_t X0T_TILE_BYTES = (int64_t)X0T_ROWS * X0T_FEAT * 2;
inline int64_t x0t_bytes(int64_t M) { return ((M + X0T_ROWS - 1) / X0T_ROWS) * X0T_TILE_BYTES; }
// appearance_fwd writing tiles (bf16 fields with 48 channels per pair only).
int launch_appearance_fwd_tiles(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                                const SamplerArgs& s, const int32_t* sel_idx, int k, uint8_t* X0t,
                                cudaStream_t st);
int launch_appearance_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins,
                          const float* dirs, int64_t R, const SamplerArgs& s,
                          const int32_t* sel_idx, int k, const float* dX0, cudaStream_t st);
int launch_points(const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                  float* points, float* ts, float* steps, cudaStream_t st);
int launch_to_channel_last(int G, int C, const float* vec, const float* mat, int dtype, void* lines,
                           void* planes, cudaStream_t st);
int launch_resize_field(int M, int N, int C, const float* src_lines, const float* src_planes, float* dst_lines,
                        float* dst_planes, cudaStream_t st);
int launch_to_channel_first(int G, int C, const float* lines, const float* planes, float* vec,
                            float* mat, cudaStream_t st);

// ---- compositing kernels (tvm_composite.cu) ----
int launch_segment_fwd(const float* sigmas, const float* steps, int64_t R, int N, float* p_exits,
                       float* p_term, cudaStream_t st);
int launch_segment_bwd(const float* sigmas, const float* steps, int64_t R, int N, const float* g_pe,
                       const float* g_pt, float* g_sigma, cudaStream_t st);
int launch_topk(const float* p, const float* gumbel, int gumbel_per_ray, int64_t R, int N, int k,
                int32_t* idx, cudaStream_t st);
// Fused: sigma (R,N) -> selection (RGB) or distance (DIST modes). p_last = the exit
// probability of the last sample, q_last = 1 - p_last computed without cancellation.
int launch_composite_select(const float* sigma, const float* origins, const float* dirs, int64_t R,
                            const SamplerArgs& s, int mode, int k, const float* gumbel,
                            int gumbel_per_ray, int32_t* sel_idx, float* w_sel, float* p_last,
                            float* q_last, float* wsum, float* dist_out, float* w_dense, cudaStream_t st);
// Dense backward with explicit step sizes into dL/d(pre-softplus sum).
int launch_segment_bwd_sum(const float* sigmas, const float* steps, int64_t R, int N, const float* g_pt,
                           float* g_sum, cudaStream_t st);
// Fused: per-ray colour, loss and the gradients entering the MLP and the compositing.
int launch_color_loss(const float* rgb_sel, const float* w_sel, const float* p_last, const float* q_last,
                      const float* wsum, int64_t R, int k, const float* target, float* color_out,
                      float* loss, float* dZ3, float* gw_sel, float* gP, cudaStream_t st);
int launch_composite_bwd(const float* sigma, const float* origins, const float* dirs, int64_t R,
                         const SamplerArgs& s, int k, const int32_t* sel_idx, const float* gw_sel,
                         const float* gP, float* gsum, cudaStream_t st);

// ---- MLP (tvm_mlp.cu) ----
struct MlpDims {
  int feat;    // 3*C_a
  int squash;  // 27
  int enc;     // encoded width (150 at n=2)
  int units;   // 128
  int nf, nv;  // fourier frequencies
  int math;    // 0: tcgen05 bf16, 1: tcgen05 split-tf32 (FP32-accurate), 2: FP32 SIMT
  int cams;    // camera embeddings (FiLM after layer 2); 0 = none
};
struct MlpWeights {
  const float *w0, *w1, *b1, *w2, *b2, *w3, *b3;
  const float* embed;  // (cams, units) or null
};
struct MlpGrads {
  float *w0, *w1, *b1, *w2, *b2, *w3, *b3;
  float* embed;
};
size_t mlp_workspace_bytes(const MlpDims& d, int64_t M);      // forward + backward
size_t mlp_fwd_workspace_bytes(const MlpDims& d, int64_t M);  // forward only (a prefix of the above)
// rgb = FeatureMlp(X0, viewdir, camera). Viewdir of row m is dirs[(m / rows_per_dir) * 3 ...],
// its camera cams[m / rows_per_dir] (cams is read only when d.cams > 0).
// max_ctas: the fused BF16 kernels' grid cap (launch_mlp_fwd_fused), 0 for one CTA per SM.
// X0t: the input as tiles (launch_appearance_fwd_tiles) instead of X0; fused path only.
// prepacked: the fused kernels' weight images are already at mlp_fused_wpack(ws)
// (launch_mlp_pack_fused), packed since the weights last changed.
int mlp_forward(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs, const int32_t* cams,
                int rows_per_dir, int64_t M, float* rgb, Workspace& ws, cudaStream_t st, int max_ctas = 0,
                const uint8_t* X0t = nullptr, bool prepacked = false);
// Where mlp_forward on this workspace state keeps the fused kernels' weight images.
uint8_t* mlp_fused_wpack(Workspace ws);
// Needs the preceding mlp_forward on the same workspace: its kept row-major activations
// (layered path), or its packed bf16 weights (fused path, which recomputes the forward
// from X0 and the view directions).
// dZ3: gradient wrt the pre-sigmoid output (M,3). dX0 may be null.
int mlp_backward(const MlpDims& d, const MlpWeights& w, const MlpGrads& g, const float* X0, const float* dirs,
                 const int32_t* cams, int rows_per_dir, int64_t M, const float* dZ3, float* dX0, Workspace& ws,
                 cudaStream_t st, int max_ctas = 0, const uint8_t* X0t = nullptr);
int gemm_any(int math, bool at, bool bt, int64_t M, int N, int64_t K, const float* A, int64_t lda,
             const float* B, int64_t ldb, float* D, int64_t ldd, bool accumulate, cudaStream_t st);
int device_status(int32_t* out, cudaStream_t st);  // copy + clear the tensor-core status word
int fused_status(int32_t* out, cudaStream_t st);   // same for the fused MLP kernel
int prop_status(int32_t* out, cudaStream_t st);    // same for the tensor-core proposal backward
bool mlp_fused_supported(const MlpDims& d);
// wpack: mlp_fused_pack_bytes() of scratch (16-byte aligned) for the packed weights.
size_t mlp_fused_pack_bytes();
// max_ctas > 0 caps the persistent grid (fewer CTAs each take more tiles), leaving the
// other SMs to kernels that run beside it on other streams; 0: one CTA per SM.
// X0t: input tiles instead of the row-major X0 (which is then not read).
int launch_mlp_fwd_fused(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs, int rows_per_dir,
                         int64_t M, float* rgb, uint8_t* wpack, cudaStream_t st, int max_ctas = 0,
                         const uint8_t* X0t = nullptr, bool prepacked = false);
// The fused kernels' bf16 weight images into wpack (what launch_mlp_fwd_fused does first
// unless prepacked).
int launch_mlp_pack_fused(const MlpWeights& w, uint8_t* wpack, cudaStream_t st);
// Fused BF16 backward: recomputes the forward per tile, accumulates all weight and
// bias gradients into g, writes dX0 (M, 144) when non-null. wpack: the images packed by
// launch_mlp_fwd_fused.
int launch_mlp_bwd_fused(const MlpWeights& w, const MlpGrads& g, const float* X0, const float* dirs,
                         int rows_per_dir, int64_t M, const float* dZ3, float* dX0, const uint8_t* wpack,
                         cudaStream_t st, int max_ctas = 0, const uint8_t* X0t = nullptr);
int launch_sigmoid_bwd(const float* rgb, const float* grad_rgb, int64_t M, float* dZ3,
                       cudaStream_t st);


// ---- proposal network (tvm_proposal.cu) ----
// The proposal MLP evaluated inside the feature kernel (H may be null: inference).
struct PropMlp {
  int units;
  const float *w1, *b1, *w2, *b2;
  float shift;
  float* H;
  float* sigma;                    // forward: sigma out (may be NULL)
  const float* sigma_in = nullptr;  // backward: if set, dz holds dL/dsigma of these sigmas
};
int launch_prop_features(const FieldView& f, const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                         const float* edges, const float* jitter, float* X, float* delta, const PropMlp* mlp,
                         cudaStream_t st);
// Fused proposal backward from dz = dL/d(pre-softplus) (or dL/dsigma with
// mlp.sigma_in): field scatter and MLP weight gradients (all accumulate).
int launch_prop_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins, const float* dirs,
                    int64_t R, const SamplerArgs& s, const float* edges, const float* jitter, const float* dz,
                    const PropMlp& mlp, float* gw1, float* gb1, float* gw2, float* gb2, cudaStream_t st);
// Resampling of the proposal weights wprop (R, Np), or (sig set) of the weights of the
// bin densities sig and lengths len, which are then written to w_out.
int launch_resample(const float* wprop, const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                    const float* edges, int Nm, const float* jitter, float* t_out, float* d_out, int32_t* bins,
                    cudaStream_t st, const float* sig = nullptr, const float* len = nullptr, float* w_out = nullptr);
int launch_prop_loss(const float* wmain, const float* wprop, const int32_t* bins, int64_t R, int Np, int Nm,
                     float scale, float* loss, float* gprop, cudaStream_t st);

// ---- FP64 loss for finite-difference checks (tvm_fdcheck.cu) ----
size_t loss_f64_scratch_bytes(const tvm_model_desc& m, int encoded_dim, int64_t R, int N);
int launch_loss_f64(const tvm_param_layout& L, const tvm_model_desc& m, const float* params, int64_t pidx,
                    double delta, const tvm_rays& rays, const float* colors, const tvm_render_desc& c,
                    double* scratch, double* loss, cudaStream_t st);

// ---- Adam (tvm_adam.cu) ----
// blocks_per_sm caps the grid-stride grid: a full 8 when Adam has the GPU to itself,
// fewer when it runs beside other kernels on a side stream and must leave them room.
// pending: with a device_step, read the pending update's scalars (and do nothing when
// its count is 0).
int launch_adam(float* params, float* grads, float* mu, float* nu, int64_t n, int64_t mlp_begin,
                const tvm_adam_desc& a, __nv_bfloat16* shadow, int64_t shadow_n, cudaStream_t st,
                int blocks_per_sm = 8, bool pending = false);
// Adam over the elements [lo, hi) of the flat buffers only (lo a segment start); the
// learning-rate group and the shadow follow the element's place in the whole layout.
int launch_adam_range(float* params, float* grads, float* mu, float* nu, int64_t lo, int64_t hi, int64_t mlp_begin,
                      const tvm_adam_desc& d, __nv_bfloat16* shadow, int64_t shadow_n, cudaStream_t st,
                      int blocks_per_sm = 8, bool pending = false);
int launch_shadow(const float* src, __nv_bfloat16* dst, int64_t n, cudaStream_t st);
int launch_set_step_scalars(tvm_step_scalars* step, const tvm_step_scalars& v, cudaStream_t st);

}  // namespace tvm
