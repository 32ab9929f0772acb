/*
 * tensorf_gb300.h -- C ABI of the GB300 (sm_103a) TensoRF-VM render-and-train path.
 *
 * Every entry point:
 *   - takes caller-owned DEVICE pointers (plain pointers, element counts), a POD
 *     descriptor where the shape is more than a couple of integers, and a
 *     cudaStream_t passed as `void*` (NULL = legacy default stream);
 *   - validates shapes, dtypes, alignment and null pointers on the host and returns
 *     a negative TVM_ERR_* code before launching anything when they are wrong, with
 *     a message readable through tvm_last_error_message() (per calling thread);
 *   - allocates nothing: scratch comes from a caller buffer sized by the matching
 *     *_workspace_size() call (tvm_mlp_fwd_static_scratch instead uses a static array
 *     inside the library);
 *   - keeps no global mutable state besides the per-thread error message, the device
 *     status words and that static array, so calls on distinct streams from distinct
 *     threads are independent, except overlapping tvm_mlp_fwd_static_scratch calls.
 *
 * Layouts (device memory). Field tensors are CHANNEL-LAST:
 *   lines  [3][G][C]     element (m, x, c)        at (m*G + x)*C + c
 *   planes [3][G][G][C]  element (m, row, col, c) at ((m*G + row)*G + col)*C + c
 * The reference stores TensorVMSingle.vector as (3, C, G) and .matrix as (3, C, G, G)
 * (tensorf/tensor_vm.py:129-138); tvm_vm_to_channel_last() converts. Pair m reads its
 * line at coordinate P_m[0] and its plane at (row, col) = (P_m[1], P_m[2]) with
 * P_0 = (0,1,2), P_1 = (2,0,1), P_2 = (1,2,0) (tensor_vm.py:50-52).
 *
 * Randomness is an INPUT: sample jitter and the Gumbel noise of the weighted
 * appearance-sample choice are arrays the caller passes (or fills with
 * tvm_noise_fill), so results are bit-reproducible and the reference's own draws can
 * be replayed.
 */
#ifndef TENSORF_GB300_H_
#define TENSORF_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TVM_ABI_VERSION 3

/* Symbols of this library are exported with default visibility. */
#ifndef TVM_API
#define TVM_API __attribute__((visibility("default")))
#endif

/* Status codes. */
#define TVM_OK 0
#define TVM_ERR_INVALID (-1)     /* null pointer or bad scalar argument */
#define TVM_ERR_SHAPE (-2)       /* sizes out of the supported range */
#define TVM_ERR_DTYPE (-3)       /* unsupported dtype / dtype combination */
#define TVM_ERR_ALIGN (-4)       /* pointer not aligned as the layout requires */
#define TVM_ERR_UNSUPPORTED (-5) /* valid request the library does not implement */
#define TVM_ERR_LAUNCH (-6)      /* CUDA launch or runtime error */
#define TVM_ERR_NONFINITE (-7)   /* non-finite value detected */
#define TVM_ERR_TIMEOUT (-8)     /* a bounded device wait gave up */
#define TVM_ERR_WORKSPACE (-9)   /* workspace too small */

/* Storage dtypes. */
#define TVM_F32 0
#define TVM_BF16 1
#define TVM_F64 2

/* Render modes (tensorf/render.py:18-23). */
#define TVM_MODE_RGB 0
#define TVM_MODE_DIST_MEDIAN 1
#define TVM_MODE_DIST_MEAN 2

/* Samplers. */
#define TVM_SAMPLER_BBOX 0     /* render.py:175-186, 350-434 */
#define TVM_SAMPLER_CONTRACT 1 /* render.py:122-173 (schedule supplied by caller) */
#define TVM_SAMPLER_PROPOSAL 2 /* proposal-guided: samples resampled from a proposal network */
#define TVM_SAMPLER_EXPLICIT 3 /* internal: per-sample distances and lengths given */

/* One VM-decomposed tensor (TensorVM, tensor_vm.py:14-40). */
typedef struct {
  int32_t grid_dim; /* G */
  int32_t channels; /* C per vector-matrix pair: 8, 16, 24, 32 or 48 */
  int32_t dtype;    /* TVM_F32 / TVM_BF16 / TVM_F64 */
  int32_t _pad;
  const void* lines;  /* [3][G][C] */
  const void* planes; /* [3][G][G][C] */
} tvm_vm_field;

/* Model description: the two VM tensors and the FeatureMlp (networks.py:38-121). */
typedef struct {
  int32_t grid_dim;            /* G */
  int32_t density_channels;    /* C_d (density_feat_dim) */
  int32_t appearance_channels; /* C_a (appearance_feat_dim) */
  int32_t feature_n_freqs;     /* fourier frequencies of the squashed features */
  int32_t viewdir_n_freqs;     /* fourier frequencies of the view direction */
  int32_t squash_dim;          /* FeatureMlp.feature_squash_dim, 27 */
  int32_t units;               /* FeatureMlp.units, 128 */
  int32_t dtype;               /* arithmetic/storage mode: TVM_F32, TVM_BF16, TVM_F64 */
  int32_t mlp_math;            /* TVM_MLP_DEFAULT or TVM_MLP_SIMT_F32 (TVM_F32 models only) */
  int32_t proposal_grid;       /* proposal VM grid (e.g. 64); 0 = no proposal network */
  int32_t proposal_rank;       /* proposal components per pair: 4 */
  int32_t proposal_units;      /* proposal MLP hidden width (16 -> units -> 1): 64 */
  int32_t num_cameras;         /* FeatureMlp.num_cameras: FiLM camera embeddings (networks.py:103-111);
                                  0 = none. Needs an even `units`. */
} tvm_model_desc;

/* MLP arithmetic. DEFAULT: TVM_F32 models run the dense layers on tcgen05 tensor
 * cores with a 3-pass split-tf32 product (hi*hi + hi*lo + lo*hi, ~22 significant bits
 * per input, fp32 accumulation), TVM_BF16 models with one bf16 pass. SIMT_F32: plain
 * FP32 FMA on the CUDA cores. */
#define TVM_MLP_DEFAULT 0
#define TVM_MLP_SIMT_F32 1

/* Offsets (in elements of the master dtype: float, or double for TVM_F64) of every
 * parameter segment inside one flat parameter buffer. Grad, Adam mu and nu buffers
 * use the same layout. Segments are 64-element aligned. MLP kernels are (in, out)
 * row-major like flax's Dense kernels. */
typedef struct {
  int64_t density_lines, density_planes;
  int64_t appearance_lines, appearance_planes;
  int64_t mlp_w0, mlp_w1, mlp_b1, mlp_w2, mlp_b2, mlp_w3, mlp_b3;
  int64_t proposal_lines, proposal_planes;                  /* tensor lr group */
  int64_t proposal_w1, proposal_b1, proposal_w2, proposal_b2; /* MLP lr group */
  int64_t mlp_begin; /* first MLP element: [0, mlp_begin) is the tensor lr group */
  int64_t total;
  /* BF16 mode: element offsets of the bf16 shadow copies of the field tensors inside
   * the shadow buffer; 0 otherwise. */
  int64_t shadow_density_lines, shadow_density_planes;
  int64_t shadow_appearance_lines, shadow_appearance_planes;
  int64_t shadow_proposal_lines, shadow_proposal_planes;
  int64_t shadow_total;
  int32_t encoded_dim; /* MLP input width after the fourier encoding (150 for n=2) */
  int32_t _pad;
  int64_t mlp_embed;   /* camera embedding table (num_cameras, units) of the FeatureMlp's
                          nn.Embed (MLP lr group); 0 when num_cameras == 0 */
} tvm_param_layout;

/* A batch of rays (cameras.Rays3D, cameras.py:10-20), device pointers. */
typedef struct {
  int64_t count;          /* R */
  const float* origins;   /* (R, 3) */
  const float* directions;/* (R, 3) */
  const int32_t* camera_indices; /* (R,) camera of each ray, for models with num_cameras > 0
                                    (indices are clamped into [0, num_cameras)); else unused */
} tvm_rays;

/* Per-call render configuration (render.RenderConfig, render.py:26-36, plus the
 * inputs the reference derives from PRNG keys). */
typedef struct {
  int32_t density_samples;    /* N */
  int32_t appearance_samples; /* k */
  int32_t mode;               /* TVM_MODE_* */
  int32_t sampler;            /* TVM_SAMPLER_* */
  float density_shift;        /* added before softplus; the reference uses +10.0 (render.py:207) */
  float _pad0;
  float aabb[6];              /* min xyz, max xyz (TrainState.aabb, training.py:96) */
  const float* schedule;      /* CONTRACT: (N,) fixed t schedule; BBOX: unused */
  const float* jitter;        /* BBOX: (N,) shared by all rays (render.py:177-186) or
                                 NULL for no jitter; CONTRACT: (R, N) per sample */
  int32_t jitter_per_ray;     /* BBOX only: 1 if jitter is (R, N) instead of (N,) */
  int32_t gumbel_per_ray;     /* 1 if gumbel is (R, N), 0 if (N,) shared (reference) */
  const float* gumbel;        /* Gumbel noise of jax.random.choice (render.py:461-469) */
  /* PROPOSAL sampler: Np proposal bins per ray (uniform over the aabb segment, or the
   * caller's Np+1 edges in `schedule` when `contract` is set), N main samples resampled
   * from the proposal histogram; `jitter` is then (R, N), one per main interval. */
  int32_t proposal_samples;      /* Np */
  int32_t contract;              /* 1: unbounded scene, L-inf contraction to [-2,2]^3 */
  const float* proposal_jitter;  /* (R, Np) uniforms, one per proposal bin */
  float proposal_shift;          /* added before the proposal softplus */
  float proposal_loss_weight;    /* weight of the proposal bound loss (training) */
} tvm_render_desc;

/* The per-step scalars in device memory, for training steps recorded once as a CUDA
 * graph and replayed: the host writes the next step's values with tvm_set_step_scalars
 * on the replay stream before each replay, and the recorded kernels read them. */
typedef struct {
  int32_t count;         /* Adam step count after increment: 1 on the first update */
  float lr_decay;        /* multiplier from the exponential decay (training.py:158-181) */
  uint64_t noise_stream; /* stream id of the step's noise key (see tvm_noise_fill_keyed) */
  int32_t pending_count; /* the field update the previous step left pending (tvm_adam_desc.
                            defer_fields): its count, or 0 for none */
  float pending_lr_decay;/* and its learning-rate decay */
} tvm_step_scalars;

/* Adam hyper-parameters (training.py:207-243; optax.scale_by_adam). */
typedef struct {
  float lr_tensor;  /* 0.02 */
  float lr_mlp;     /* 1e-3 */
  float b1, b2, eps;/* 0.9, 0.99, 1e-8 */
  float lr_decay;   /* multiplier from the exponential decay (training.py:158-181) */
  int32_t count;    /* step count after increment: 1 on the first update */
  int32_t defer_fields; /* tvm_train_step only. 1: leave this step's update of the density and
                       appearance fields (their parameters, moments and the gradients it
                       would consume and zero) pending; the next tvm_train_step applies it
                       first, beside its own start, or tvm_apply_pending_fields does.
                       Nothing reads those segments in between, so the result is the same
                       as updating at once. The fields' gradients are then not counted in
                       grad_sq. */
  float* grad_sq;   /* optional device float, or NULL: overwritten with the sum of the squared
                       gradients the update consumed, the square of optax.global_norm(grads)
                       that training_step logs as grad_norm (training.py:190-196) */
  const tvm_step_scalars* device_step; /* optional device struct, or NULL: when set, the
                       update reads count, lr_decay and the pending update's scalars from it
                       when it runs (the host fields are then not used), so a recorded step
                       can be replayed */
  int32_t pending_count;   /* tvm_train_step with device_step NULL: the count of a field
                              update the previous call left pending, or 0 for none */
  float pending_lr_decay;  /* and its learning-rate decay */
} tvm_adam_desc;

/* ---- library ---------------------------------------------------------------------- */
TVM_API int tvm_abi_version(void);
TVM_API const char* tvm_last_error_message(void);
/* Number of kernels this library has launched from the calling thread. */
TVM_API uint64_t tvm_kernel_launches(void);
/* Measurement hook: when `events` (n cudaEvent_t created by the caller) is set for the
 * calling thread, tvm_train_step / tvm_loss_and_grad / tvm_render_fwd run the whole pass
 * on the caller's stream, in phase order (no side streams, full grids), and record
 * events[i] there at the boundary before phase i and events[12] after the last one
 * (phases: 0 proposal network forward + resampling, 1 density fwd, 2 composite+select,
 * 3 appearance gather, 4 MLP fwd, 5 colour+loss, 6 MLP bwd, 7 appearance scatter,
 * 8 composite bwd, 9 density scatter, 10 proposal bound loss + backward, 11 Adam: in
 * tvm_train_step, one update over every segment whose update is not deferred). A field
 * update left pending by the previous step runs before phase 0. Unused trailing phases
 * record nothing. NULL disables. */
TVM_API int tvm_set_phase_events(void* const* events, int32_t n);

/* ---- parameter layout ---------------------------------------------------------- */
/* Fill *out for the model. Replaces the pytree structure of render.LearnableParams
 * (render.py:39-46) with one flat buffer. */
TVM_API int tvm_get_param_layout(const tvm_model_desc* model, tvm_param_layout* out);

/* Reference channel-first (3, C, G) / (3, C, G, G) float32 -> channel-last lines /
 * planes in `dtype` (tensor_vm.py:129-138). dst_* are device buffers. */
TVM_API int tvm_vm_to_channel_last(int32_t grid_dim, int32_t channels, const float* vector_cf,
                           const float* matrix_cf, int32_t dtype, void* lines, void* planes,
                           void* stream);
/* Inverse of the above for float32 channel-last buffers (gradients, parameters). */
TVM_API int tvm_vm_to_channel_first(int32_t grid_dim, int32_t channels, const float* lines,
                            const float* planes, float* vector_cf, float* matrix_cf, void* stream);

/* TensorVMSingle.resize (tensor_vm.py:182-198) for all three pairs of one tensor:
 * float32 channel-last lines [3][old][C] / planes [3][old][old][C] -> [3][new][C] /
 * [3][new][new][C], resampled like resize_with_aligned_corners (tensor_vm.py:202-223):
 * jax.image.scale_and_translate, linear kernel, antialias, aligned corners. Used on the
 * parameters and on both Adam moments when training upsamples the grid
 * (TrainState.resize_grid, training.py:245-276). dst must not alias src. */
TVM_API int tvm_resize_field(int32_t old_grid, int32_t new_grid, int32_t channels, const float* src_lines,
                             const float* src_planes, float* dst_lines, float* dst_planes, void* stream);

/* ---- (a) VM feature evaluation: TensorVM.interpolate (tensor_vm.py:42-89) --------- */
/* coords (3, n) float32 in [-1, 1]; out (3C, n) float32, mode-major like the
 * reference. */
TVM_API int tvm_vm_features_fwd(const tvm_vm_field* field, const float* coords, int64_t n, float* out,
                        void* stream);
/* grad_out (3C, n) -> ACCUMULATES into grad_lines [3][G][C] and grad_planes
 * [3][G][G][C] (float32, channel-last). Backward of map_coordinates(order=1,
 * mode="nearest") (tensor_vm.py:226-250): clamped corners receive the weights of the
 * unclamped coordinate. */
TVM_API int tvm_vm_features_bwd(const tvm_vm_field* field, const float* coords, int64_t n,
                        const float* grad_out, float* grad_lines, float* grad_planes,
                        void* stream);

/* ---- (b) ray samplers --------------------------------------------------------------- */
/* sample_points_along_ray_within_bbox vmapped over rays (render.py:350-434, 177-186)
 * or the contracted sampler (render.py:122-173), followed by the [-1, 1]
 * normalisation (render.py:192-196). points (3, R, N) normalised; ts (R, N);
 * step_sizes (R, N). Any output may be NULL. */
TVM_API int tvm_sample_points(const tvm_rays* rays, const tvm_render_desc* cfg, float* points,
                      float* ts, float* step_sizes, void* stream);

/* ---- (c) compositing and selection -------------------------------------------------- */
/* compute_segment_probabilities (render.py:300-347): sigmas, step_sizes (R, N) ->
 * p_exits, p_terminates (R, N). */
TVM_API int tvm_composite_fwd(const float* sigmas, const float* step_sizes, int64_t rays,
                      int32_t samples, float* p_exits, float* p_terminates, void* stream);
/* Backward of the above: grad_p_exits, grad_p_terminates (R, N) (either may be NULL)
 * -> grad_sigmas (R, N) (overwritten). */
TVM_API int tvm_composite_bwd(const float* sigmas, const float* step_sizes, int64_t rays,
                      int32_t samples, const float* grad_p_exits, const float* grad_p_terminates,
                      float* grad_sigmas, void* stream);
/* Weighted choice without replacement (render.py:459-470): per row, the k indices
 * with the largest log(p) + gumbel, largest first, equal keys -> lower index first.
 * p (R, N); gumbel (N,) shared or (R, N) if gumbel_per_ray; indices (R, k) int32. */
TVM_API int tvm_topk_select(const float* p, const float* gumbel, int32_t gumbel_per_ray, int64_t rays,
                    int32_t samples, int32_t k, int32_t* indices, void* stream);

/* ---- (d) FeatureMlp (networks.py:45-121) --------------------------------------------- */
/* features (n, 3*C_a), viewdirs (n, 3) -> rgb (n, 3). params: flat buffer in the
 * tvm_param_layout layout, 16-byte aligned (master dtype float32; TVM_BF16 models use bf16 tensor
 * cores, TVM_F32 models float32 arithmetic). camera_indices (n,): camera of each row
 * for models with num_cameras > 0 (networks.py:103-111), else NULL. workspace:
 * tvm_mlp_workspace_size(). Models with camera embeddings run the layered GEMMs with a
 * separate FiLM pass (the fused and pipelined kernels take models without them). */
TVM_API size_t tvm_mlp_workspace_size(const tvm_model_desc* model, int64_t n);
TVM_API int tvm_mlp_fwd(const tvm_model_desc* model, const void* params, const float* features,
                const float* viewdirs, const int32_t* camera_indices, int64_t n, float* rgb, void* workspace,
                size_t workspace_bytes, void* stream);
/* grad_rgb (n, 3) -> grad_features (n, 3*C_a) (overwritten, may be NULL) and
 * ACCUMULATES the MLP weight gradients into grads (flat layout). */
TVM_API int tvm_mlp_bwd(const tvm_model_desc* model, const void* params, const float* features,
                const float* viewdirs, const int32_t* camera_indices, int64_t n, const float* grad_rgb,
                float* grad_features, void* grads, void* workspace, size_t workspace_bytes, void* stream);

/* FeatureMlp forward without a caller workspace. This function has no counterpart in
 * the reference. It computes the same rgb as tvm_mlp_fwd, with the same kernels, but
 * it allocates nothing and takes no workspace. Its scratch is one static device array
 * of TVM_MLP_STATIC_SCRATCH_BYTES inside the library, shared by every call on a
 * device.
 *
 * It is for callers that can neither allocate nor pass scratch:
 *   - a handler run by another framework's executor, such as an XLA FFI custom call.
 *     XLA reserves most of device memory up front, and a handler only receives the
 *     buffers its call declares.
 *   - code that must not stall other streams, because cudaFree synchronises the
 *     device.
 *
 * Limit: n is at most the number of rows whose forward scratch (the part of the
 * tvm_mlp_fwd workspace the forward writes) fits the array. For the default TVM_F32
 * model (144 features, 27 squash, 2/2 frequencies, 128 units) that is 20,164 rows. A
 * TVM_BF16 model with those dimensions runs the fused kernel: it needs only the
 * 87,040-byte packed weights, so n is not limited. Larger n returns TVM_ERR_SHAPE
 * before any launch, and the message gives the maximum for the model. It takes no
 * camera indices: models with camera embeddings return TVM_ERR_UNSUPPORTED.
 *
 * Alignment: params must be 16-byte aligned (TVM_ERR_ALIGN otherwise). TVM_F32
 * models accept any features pointer; TVM_BF16 models read features with 16-byte
 * loads and return TVM_ERR_ALIGN when it is not 16-byte aligned, as tvm_mlp_fwd does.
 *
 * Set-up: the first call with a device current looks up the array's device address
 * for that device. That lookup may load the library's module and reserve the array.
 * Make that first call before any stream capture. The address is kept for the life
 * of the process: do not call this function on a device after cudaDeviceReset.
 *
 * Calls whose GPU work overlaps race on the shared array: different streams, or
 * different threads, with no ordering between them. Order them on one stream or with
 * events. Nothing in the array has to start at zero. */
#define TVM_MLP_STATIC_SCRATCH_BYTES (32u << 20)
TVM_API int tvm_mlp_fwd_static_scratch(const tvm_model_desc* model, const void* params,
                                       const float* features, const float* viewdirs, int64_t n,
                                       float* rgb, void* stream);

/* Plain GEMM on the tensor-core path used by the MLP (exposed for testing):
 * D[M x N] (+)= A(m,k) * B(k,n), A(m,k) = a_trans ? A[k*lda + m] : A[m*lda + k],
 * B(k,n) = b_trans ? B[n*ldb + k] : B[k*ldb + n]; all float32 in memory. math: 0 =
 * tcgen05 bf16, 1 = tcgen05 split-tf32 (FP32-accurate), 2 = FP32 SIMT. accumulate:
 * 0 overwrites D, 1 adds into D atomically (K is then split across CTAs). */
TVM_API int tvm_gemm(int32_t math, int32_t a_trans, int32_t b_trans, int64_t M, int32_t N, int64_t K,
                     const float* A, int64_t lda, const float* B, int64_t ldb, float* D, int64_t ldd,
                     int32_t accumulate, void* stream);
/* Copy the device status word into *out (host) and clear it: bit 0 = a bounded
 * tensor-core wait gave up (results of that call are invalid). */
TVM_API int tvm_device_status(int32_t* out, void* stream);

/* ---- (e) proposal network ------------------------------------------------------------ */
/* The stages of TVM_SAMPLER_PROPOSAL that tvm_render_fwd and tvm_train_step run fused.
 * The reference has no proposal network (it samples uniformly; render.py:126 suggests
 * one); these seams stand beside its sampler seam (render.py:122-186), and a caller that
 * binds them composes: fwd -> tvm_composite_fwd (p_terminates = the proposal weights) ->
 * resample -> main field; in training the main weights -> loss -> tvm_composite_bwd ->
 * bwd. cfg: sampler TVM_SAMPLER_PROPOSAL with proposal_samples (Np), proposal_jitter,
 * proposal_shift, aabb, contract and (contract) the Np+1 edges in schedule. */
/* Proposal forward: per ray, Np bins (uniform over the ray's aabb segment, or the
 * caller's edges with contraction), one jittered point per bin, its 12 VM features
 * plus [x, y, z, max|x|] through the 16 -> units -> 1 MLP, softplus(z + shift).
 * sigmas, deltas (bin lengths): (R, Np). */
TVM_API int tvm_proposal_fwd(const tvm_model_desc* model, const void* params, const void* shadow,
                             const tvm_rays* rays, const tvm_render_desc* cfg, float* sigmas, float* deltas,
                             void* stream);
/* Resampling: proposal weights (R, Np) -> N = cfg->density_samples main intervals at the
 * quantiles i/N of w + (0.01 sum w + 1e-4) / Np, one point each at cfg->jitter (R, N):
 * ts, deltas (R, N) and bins (R, N+1) int32, the proposal bin of each interval edge. */
TVM_API int tvm_proposal_resample(const tvm_rays* rays, const tvm_render_desc* cfg, const float* weights,
                                  float* ts, float* deltas, int32_t* bins, void* stream);
/* Bound loss: scale * sum_i max(0, w_i - bound_i)^2 / (w_i + 1e-7), bound_i the proposal
 * mass over bins [bins_i, bins_i+1] (the fused step uses scale = loss_weight / R).
 * main_weights (R, N) (no gradient), proposal_weights (R, Np), bins (R, N+1).
 * loss: one device float, ACCUMULATED (may be NULL); grad_proposal_weights (R, Np)
 * overwritten. */
TVM_API int tvm_proposal_loss(const float* main_weights, const float* proposal_weights, const int32_t* bins,
                              int64_t rays, int32_t proposal_samples, int32_t samples, float scale, float* loss,
                              float* grad_proposal_weights, void* stream);
/* Proposal backward: grad_sigmas (R, Np) of the sigmas tvm_proposal_fwd returned ->
 * ACCUMULATES into the proposal segments of grads (field lines and planes, w1, b1, w2,
 * b2). Recomputes the features from the same rays, cfg and proposal_jitter. */
TVM_API int tvm_proposal_bwd(const tvm_model_desc* model, const void* params, const void* shadow, void* grads,
                             const tvm_rays* rays, const tvm_render_desc* cfg, const float* sigmas,
                             const float* grad_sigmas, void* stream);

/* ---- fused render_rays / training_step ---------------------------------------------- */
/* render_rays (render.py:105-279) for one chunk of rays. out: (R, 3) for RGB, (R,) for
 * distances. params: flat master buffer; shadow: bf16 copies (TVM_BF16 models) or
 * NULL. */
TVM_API size_t tvm_render_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg,
                                 int64_t rays);
TVM_API int tvm_render_fwd(const tvm_model_desc* model, const void* params, const void* shadow,
                   const tvm_rays* rays, const tvm_render_desc* cfg, float* out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* TrainState.training_step (training.py:101-205): render (RGB mode), MSE loss against
 * colors (R, 3), backward, Adam update of params/mu/nu (flat layout), refresh of the
 * bf16 shadow (TVM_BF16), grads zeroed for the next step. loss_out: device float,
 * written with the MSE. grads must be zero on entry (they are left zero), except for
 * the field segments of a pending update (adam->pending_count or device_step), which
 * this call applies first: on a side stream, with the forward's density and appearance
 * kernels waiting for it. adam->defer_fields leaves this step's field update pending. */
TVM_API size_t tvm_train_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg,
                                int64_t rays);
TVM_API int tvm_train_step(const tvm_model_desc* model, void* params, void* shadow, void* grads,
                   void* adam_mu, void* adam_nu, const tvm_adam_desc* adam, const tvm_rays* rays,
                   const float* colors, const tvm_render_desc* cfg, float* loss_out,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Side streams. With a proposal network (TVM_SAMPLER_PROPOSAL), tvm_train_step and
 * tvm_loss_and_grad run the proposal's bound loss and backward on a second stream,
 * forked from `stream` after the forward compositing. tvm_train_step also applies Adam
 * segment by segment as each segment's gradient becomes final: the appearance field and
 * the FeatureMlp on a third stream while `stream` runs the density backward, the
 * proposal network on the second, the density field on `stream`. Both side streams
 * belong to the calling thread and device, run at the lowest priority and are created
 * on first use (with four events); all their work is joined back into `stream` before
 * the call's work there ends, so work a caller orders after the call on `stream` sees
 * every gradient and every update. */

/* Loss and gradients only (no Adam): used by gradient checks. grads ACCUMULATE. */
TVM_API int tvm_loss_and_grad(const tvm_model_desc* model, const void* params, const void* shadow,
                      void* grads, const tvm_rays* rays, const float* colors,
                      const tvm_render_desc* cfg, float* loss_out, void* workspace,
                      size_t workspace_bytes, void* stream);

/* FP64 evaluation of the training loss for finite-difference checks of the FP32
 * gradients, done on the device. It follows render_rays (render.py:105-279, RGB mode)
 * and the MSE of training_step (training.py:121-134) in double precision. Optionally
 * params[perturb_index] + perturb_delta replaces one parameter (-1: none). It supports
 * TVM_F32 models without camera embeddings, the bounded sampler, and k == N <= 1024: every sample reaches the
 * appearance path, so the loss has no selection discontinuity. *loss_out (device
 * double) is overwritten. This is a check path, not tuned for speed. */
TVM_API size_t tvm_loss_f64_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg,
                                           int64_t rays);
TVM_API int tvm_loss_f64(const tvm_model_desc* model, const void* params, const tvm_rays* rays,
                         const float* colors, const tvm_render_desc* cfg, int64_t perturb_index,
                         double perturb_delta, double* loss_out, void* workspace,
                         size_t workspace_bytes, void* stream);

/* Fused Adam over the flat buffers (training.py:184-203, 213-243). n = layout.total.
 * Elements [0, mlp_begin) use lr_tensor, the rest lr_mlp. Zeroes grads. If shadow is
 * non-NULL (TVM_BF16) the field segments are rounded into it. */
TVM_API int tvm_adam_step(const tvm_model_desc* model, void* params, void* grads, void* mu, void* nu,
                  const tvm_adam_desc* adam, void* shadow, void* stream);
/* Write a step's scalars into a device tvm_step_scalars, ordered on `stream` (one
 * single-thread kernel: the values travel as launch arguments, so the host may reuse its
 * variables at once). No counterpart in the reference, whose jitted step takes its
 * optimizer state and key as traced arrays. */
TVM_API int tvm_set_step_scalars(tvm_step_scalars* device_step, int32_t count, float lr_decay,
                                 uint64_t noise_stream, int32_t pending_count, float pending_lr_decay,
                                 void* stream);
/* Apply a field update that tvm_train_step left pending (defer_fields): Adam over the
 * density and appearance field segments with adam->pending_count and
 * adam->pending_lr_decay, their gradients zeroed, their bf16 shadow refreshed. */
TVM_API int tvm_apply_pending_fields(const tvm_model_desc* model, void* params, void* shadow, void* grads,
                                     void* mu, void* nu, const tvm_adam_desc* adam, void* stream);
/* Round the field segments of params into the bf16 shadow (after init / load). */
TVM_API int tvm_refresh_shadow(const tvm_model_desc* model, const void* params, void* shadow,
                       void* stream);

/* ---- measurement ------------------------------------------------------------------------ */
/* L2 bandwidth probe (no counterpart in the reference: it measures the roofline
 * denominator of the gather and scatter kernels, whose fields stay in L2). Streams
 * `passes` full passes over `buf` (`bytes`, a multiple of 16, small enough to stay in
 * L2): kind 0 reads it with 16-byte loads that bypass L1, kind 1 adds 1.0 to every
 * float with 16-byte float4 reductions (it changes the buffer). The caller times the
 * launch on `stream`; bytes moved = passes * bytes. */
TVM_API int tvm_l2_probe(int32_t kind, void* buf, size_t bytes, int32_t passes, void* stream);

/* ---- data generation ---------------------------------------------------------------- */
/* Counter-based noise: dst[i] = U[0,1) (kind 0) or standard Gumbel (kind 1) from
 * (seed, stream_id, i). */
TVM_API int tvm_noise_fill(float* dst, int64_t n, uint64_t seed, uint64_t stream_id, int32_t kind,
                   void* stream);
/* tvm_noise_fill with the stream id read on the device when the kernel runs:
 * stream_id = step->noise_stream * mul + add (mod 2^64). A key split k -> (2k+1, 2k+2)
 * is a (mul, add) pair, so the draws of a recorded step follow the key the host writes
 * into `step` before each replay. */
TVM_API int tvm_noise_fill_keyed(float* dst, int64_t n, uint64_t seed, const tvm_step_scalars* step,
                                 uint64_t mul, uint64_t add, int32_t kind, void* stream);
/* Up to TVM_NOISE_BATCH_MAX tvm_noise_fill_keyed draws of one seed in one launch (a
 * training step's jitter, proposal jitter and Gumbel noise): each job is filled exactly as
 * tvm_noise_fill_keyed fills it. */
#define TVM_NOISE_BATCH_MAX 4
typedef struct {
  float* dst;
  int64_t n;
  uint64_t mul, add;
  int32_t kind; /* 0 uniform [0, 1), 1 Gumbel */
  int32_t _pad;
} tvm_noise_job;
TVM_API int tvm_noise_fill_keyed_batch(const tvm_noise_job* jobs, int32_t njobs, uint64_t seed,
                                       const tvm_step_scalars* step, void* stream);
/* Pinhole rays of one camera (cameras.py:100-143): K (3x3 row-major), R_wc (3x3),
 * t_wc (3): origins/directions (H*W, 3) float32, pixel (v, u) row-major. The
 * pixel subset `pixels` (n indices into H*W) may be NULL for the full frame. */
TVM_API int tvm_camera_rays(const double* K, const double* R_world_camera, const double* t_world_camera,
                    int32_t width, int32_t height, const int64_t* pixels, int64_t n,
                    float* origins, float* directions, void* stream);
/* FP64 quadrature of a field of constant-density spheres (analytic training target):
 * centers (S,3), radii (S,), colors (S,3) float64; colors_out (R, 3) float32. The
 * quadrature spans each ray's aabb segment with n_samples midpoint samples and a
 * white background. */
TVM_API int tvm_sphere_scene_render(const double* centers, const double* radii, const double* colors,
                            int32_t spheres, double density, const float* aabb,
                            const tvm_rays* rays, int32_t n_samples, float* colors_out,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TENSORF_GB300_H_ */
