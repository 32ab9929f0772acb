// C ABI entry points: argument validation, parameter layout, the per-seam functions
// and the fused render_rays / training_step orchestration.
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "tvm_internal.h"

namespace tvm {

static thread_local char g_err[512] = "";
static thread_local uint64_t g_launches = 0;
static thread_local cudaEvent_t g_events[32];
static thread_local int g_n_events = 0;

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void phase_mark(int phase, cudaStream_t st) {
  if (phase >= 0 && phase < g_n_events) cudaEventRecord(g_events[phase], st);
}

int check_launch(const char* what) {
  ++g_launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return TVM_ERR_LAUNCH;
  }
  return TVM_OK;
}

// Per-device launch set-up. Both tables are keyed by device ordinal: a kernel's
// shared-memory limit and the SM count belong to one device, and a process may drive
// several.
static std::mutex g_setup_mu;

static int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  return dev;
}

int device_sms() {
  static std::vector<int> sms;
  const int dev = current_device();
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if ((int)sms.size() <= dev) sms.resize(dev + 1, 0);
  if (sms[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = n > 0 ? n : 1;
  }
  return sms[dev];
}

int ensure_smem_limit(const void* fn, int bytes, const char* what) {
  static std::map<std::pair<int, const void*>, int> raised;  // (device, kernel) -> bytes
  const int dev = current_device();
  std::lock_guard<std::mutex> lock(g_setup_mu);
  int& have = raised[{dev, fn}];
  if (have >= bytes) return TVM_OK;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "%s: shared-memory attribute (%d bytes): %s", what, bytes,
              cudaGetErrorString(e));
  have = bytes;
  return TVM_OK;
}

// Two more streams per calling thread and device, each with a fork and a join event:
//  - `stream` (lowest priority): the proposal network's backward and update, which
//    depend only on the forward, run there beside the main field's backward;
//  - `branch` (highest priority): the appearance branch of the backward (FeatureMlp
//    backward, appearance scatter, their update), the longer of the two chains that
//    follow the loss, runs there while the caller's stream runs the density branch; at
//    the start of a training step, the field update the previous step left pending runs
//    there too, beside the proposal forward, and the density and appearance gathers wait
//    for its two halves.
struct SideStream {
  cudaStream_t stream = nullptr, branch = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, fork2 = nullptr, join2 = nullptr;
  cudaEvent_t fork3 = nullptr, density_ready = nullptr, appearance_ready = nullptr;
  cudaEvent_t fork4 = nullptr, packed = nullptr;
};

static int side_stream(SideStream*& out) {
  static thread_local std::vector<SideStream> per_device;
  const int dev = current_device();
  if ((int)per_device.size() <= dev) per_device.resize(dev + 1);
  SideStream& s = per_device[dev];
  if (s.stream == nullptr) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s.stream, cudaStreamNonBlocking, least);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s.branch, cudaStreamNonBlocking, greatest);
    for (cudaEvent_t* ev : {&s.fork, &s.join, &s.fork2, &s.join2, &s.fork3, &s.density_ready, &s.appearance_ready,
                            &s.fork4, &s.packed})
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "side stream: %s", cudaGetErrorString(e));
  }
  out = &s;
  return TVM_OK;
}

static int64_t seg(int64_t& off, int64_t n) {
  const int64_t at = off;
  off = round_up(off + n, 64);
  return at;
}

static int encoded_dim(const tvm_model_desc& m) {
  return m.squash_dim + 3 + 2 * m.feature_n_freqs * m.squash_dim + 2 * m.viewdir_n_freqs * 3;
}

static bool channels_ok(int c) { return c == 8 || c == 16 || c == 24 || c == 32 || c == 48; }

static int validate_model(const tvm_model_desc* m) {
  TVM_REQUIRE(m != nullptr, TVM_ERR_INVALID, "model descriptor is NULL");
  TVM_REQUIRE(m->grid_dim >= 2 && m->grid_dim <= 4096, TVM_ERR_SHAPE, "grid_dim=%d outside [2, 4096]",
              m->grid_dim);
  TVM_REQUIRE(channels_ok(m->density_channels), TVM_ERR_UNSUPPORTED,
              "density_channels=%d not compiled (8, 16, 24, 32, 48)", m->density_channels);
  TVM_REQUIRE(channels_ok(m->appearance_channels), TVM_ERR_UNSUPPORTED,
              "appearance_channels=%d not compiled (8, 16, 24, 32, 48)", m->appearance_channels);
  TVM_REQUIRE(m->feature_n_freqs >= 0 && m->feature_n_freqs <= 16 && m->viewdir_n_freqs >= 0 &&
                  m->viewdir_n_freqs <= 16,
              TVM_ERR_SHAPE, "fourier frequencies must be in [0, 16]");
  TVM_REQUIRE(m->squash_dim >= 1 && m->squash_dim <= 64 && m->units >= 1 && m->units <= 1024,
              TVM_ERR_SHAPE, "squash_dim / units out of range");
  TVM_REQUIRE(m->dtype == TVM_F32 || m->dtype == TVM_BF16, TVM_ERR_DTYPE,
              "model dtype %d not supported (TVM_F32, TVM_BF16)", m->dtype);
  TVM_REQUIRE(m->mlp_math == TVM_MLP_DEFAULT || (m->mlp_math == TVM_MLP_SIMT_F32 && m->dtype == TVM_F32),
              TVM_ERR_INVALID, "mlp_math=%d invalid for dtype %d", m->mlp_math, m->dtype);
  TVM_REQUIRE(m->num_cameras >= 0 && m->num_cameras <= (1 << 24), TVM_ERR_SHAPE, "num_cameras=%d outside [0, 2^24]",
              m->num_cameras);
  TVM_REQUIRE(m->num_cameras == 0 || m->units % 2 == 0, TVM_ERR_SHAPE,
              "camera embeddings condition half of the units: units=%d must be even", m->units);
  if (m->proposal_grid != 0) {
    TVM_REQUIRE(m->proposal_grid >= 2 && m->proposal_grid <= 1024, TVM_ERR_SHAPE, "proposal_grid=%d outside [2, 1024]",
                m->proposal_grid);
    TVM_REQUIRE(m->proposal_rank == 4, TVM_ERR_UNSUPPORTED, "proposal_rank must be 4");
    TVM_REQUIRE(m->proposal_units >= 4 && m->proposal_units <= 128 && m->proposal_units % 4 == 0, TVM_ERR_SHAPE,
                "proposal_units must be a multiple of 4 in [4, 128]");
  }
  return TVM_OK;
}

static void make_layout(const tvm_model_desc& m, tvm_param_layout& L) {
  memset(&L, 0, sizeof(L));
  const int64_t G = m.grid_dim;
  const int64_t Cd = m.density_channels, Ca = m.appearance_channels;
  const int enc = encoded_dim(m);
  int64_t off = 0;
  L.density_lines = seg(off, 3 * G * Cd);
  L.density_planes = seg(off, 3 * G * G * Cd);
  L.appearance_lines = seg(off, 3 * G * Ca);
  L.appearance_planes = seg(off, 3 * G * G * Ca);
  const int64_t Gp = m.proposal_grid, Cp = m.proposal_rank;
  if (Gp > 0) {
    L.proposal_lines = seg(off, 3 * Gp * Cp);
    L.proposal_planes = seg(off, 3 * Gp * Gp * Cp);
  }
  L.mlp_begin = off;
  L.mlp_w0 = seg(off, 3 * Ca * m.squash_dim);
  L.mlp_w1 = seg(off, (int64_t)enc * m.units);
  L.mlp_b1 = seg(off, m.units);
  L.mlp_w2 = seg(off, (int64_t)m.units * m.units);
  L.mlp_b2 = seg(off, m.units);
  L.mlp_w3 = seg(off, (int64_t)m.units * 3);
  L.mlp_b3 = seg(off, 3);
  if (m.num_cameras > 0) L.mlp_embed = seg(off, (int64_t)m.num_cameras * m.units);
  if (Gp > 0) {
    L.proposal_w1 = seg(off, 16LL * m.proposal_units);
    L.proposal_b1 = seg(off, m.proposal_units);
    L.proposal_w2 = seg(off, m.proposal_units);
    L.proposal_b2 = seg(off, 1);
  }
  L.total = off;
  if (m.dtype == TVM_BF16) {
    L.shadow_density_lines = L.density_lines;
    L.shadow_density_planes = L.density_planes;
    L.shadow_appearance_lines = L.appearance_lines;
    L.shadow_appearance_planes = L.appearance_planes;
    L.shadow_proposal_lines = L.proposal_lines;
    L.shadow_proposal_planes = L.proposal_planes;
    L.shadow_total = L.mlp_begin;
  }
  L.encoded_dim = enc;
}

static int validate_rays(const tvm_rays* rays, const tvm_model_desc* m = nullptr) {
  TVM_REQUIRE(rays != nullptr, TVM_ERR_INVALID, "rays is NULL");
  TVM_REQUIRE(m == nullptr || m->num_cameras == 0 || rays->count == 0 || rays->camera_indices != nullptr,
              TVM_ERR_INVALID, "a model with camera embeddings needs the rays' camera_indices");
  TVM_REQUIRE(rays->count >= 0 && rays->count <= (1LL << 31), TVM_ERR_SHAPE, "ray count %lld out of range",
              (long long)rays->count);
  TVM_REQUIRE(rays->count == 0 || (rays->origins && rays->directions), TVM_ERR_INVALID,
              "ray origins/directions are NULL");
  return TVM_OK;
}

static int validate_render(const tvm_render_desc* c, int64_t R, bool need_select,
                           const tvm_model_desc* m = nullptr) {
  TVM_REQUIRE(c != nullptr, TVM_ERR_INVALID, "render descriptor is NULL");
  if (c->sampler == TVM_SAMPLER_PROPOSAL) {
    TVM_REQUIRE(m == nullptr || m->proposal_grid > 0, TVM_ERR_INVALID,
                "proposal sampler needs a model with a proposal network");
    TVM_REQUIRE(c->proposal_samples >= 2 && c->proposal_samples <= 512, TVM_ERR_SHAPE,
                "proposal_samples=%d outside [2, 512]", c->proposal_samples);
    TVM_REQUIRE(c->density_samples <= 512, TVM_ERR_SHAPE, "proposal-guided density_samples must be <= 512");
    TVM_REQUIRE(c->proposal_jitter != nullptr && c->jitter != nullptr, TVM_ERR_INVALID,
                "proposal sampler needs proposal_jitter (R, Np) and jitter (R, N)");
    TVM_REQUIRE(!c->contract || c->schedule != nullptr, TVM_ERR_INVALID,
                "unbounded proposal sampling needs the Np+1 bin edges in schedule");
  }
  TVM_REQUIRE(c->density_samples >= 1 && c->density_samples <= 8192, TVM_ERR_SHAPE,
              "density_samples=%d outside [1, 8192]", c->density_samples);
  TVM_REQUIRE(c->sampler == TVM_SAMPLER_BBOX || c->sampler == TVM_SAMPLER_CONTRACT ||
                  c->sampler == TVM_SAMPLER_PROPOSAL,
              TVM_ERR_INVALID, "unknown sampler %d", c->sampler);
  TVM_REQUIRE(c->mode == TVM_MODE_RGB || c->mode == TVM_MODE_DIST_MEAN || c->mode == TVM_MODE_DIST_MEDIAN,
              TVM_ERR_INVALID, "unknown mode %d", c->mode);
  for (int a = 0; a < 3; ++a)
    TVM_REQUIRE(c->aabb[a] < c->aabb[3 + a], TVM_ERR_INVALID, "aabb min must be < max on every axis");
  if (c->sampler == TVM_SAMPLER_CONTRACT) {
    TVM_REQUIRE(c->density_samples >= 2, TVM_ERR_SHAPE, "contracted sampler needs >= 2 samples");
    TVM_REQUIRE(c->schedule != nullptr && c->jitter != nullptr, TVM_ERR_INVALID,
                "contracted sampler needs schedule (N,) and jitter (R, N)");
  }
  if (need_select && c->mode == TVM_MODE_RGB) {
    TVM_REQUIRE(c->appearance_samples >= 1 && c->appearance_samples <= c->density_samples &&
                    c->appearance_samples <= 1024,
                TVM_ERR_SHAPE, "appearance_samples=%d must be in [1, min(N, 1024)]", c->appearance_samples);
    TVM_REQUIRE(c->gumbel != nullptr, TVM_ERR_INVALID, "RGB mode needs the Gumbel noise array");
  }
  TVM_REQUIRE(R * (int64_t)c->density_samples < (1LL << 40), TVM_ERR_SHAPE, "R*N too large");
  return TVM_OK;
}

static SamplerArgs sampler_args(const tvm_render_desc& c) {
  SamplerArgs s;
  s.sampler = c.sampler;
  s.N = c.density_samples;
  for (int a = 0; a < 6; ++a) s.aabb[a] = c.aabb[a];
  s.schedule = c.schedule;
  s.jitter = c.jitter;
  s.jitter_per_ray = c.jitter_per_ray;
  return s;
}

static MlpDims mlp_dims(const tvm_model_desc& m) {
  MlpDims d;
  d.feat = 3 * m.appearance_channels;
  d.squash = m.squash_dim;
  d.enc = encoded_dim(m);
  d.units = m.units;
  d.nf = m.feature_n_freqs;
  d.nv = m.viewdir_n_freqs;
  d.math = (m.dtype == TVM_BF16) ? 0 : (m.mlp_math == TVM_MLP_SIMT_F32 ? 2 : 1);
  d.cams = m.num_cameras;
  return d;
}

static MlpWeights mlp_weights(const tvm_param_layout& L, const float* p) {
  return MlpWeights{p + L.mlp_w0, p + L.mlp_w1, p + L.mlp_b1, p + L.mlp_w2,
                    p + L.mlp_b2, p + L.mlp_w3, p + L.mlp_b3, L.mlp_embed ? p + L.mlp_embed : nullptr};
}
static MlpGrads mlp_grads(const tvm_param_layout& L, float* g) {
  return MlpGrads{g + L.mlp_w0, g + L.mlp_w1, g + L.mlp_b1, g + L.mlp_w2,
                  g + L.mlp_b2, g + L.mlp_w3, g + L.mlp_b3, L.mlp_embed ? g + L.mlp_embed : nullptr};
}

// Fields read by the gathers: bf16 shadow in BF16 mode, the FP32 master otherwise.
static FieldView density_field(const tvm_model_desc& m, const tvm_param_layout& L, const float* p,
                               const void* shadow) {
  if (m.dtype == TVM_BF16 && shadow) {
    const __nv_bfloat16* s = static_cast<const __nv_bfloat16*>(shadow);
    return FieldView{m.grid_dim, m.density_channels, TVM_BF16, s + L.shadow_density_lines,
                     s + L.shadow_density_planes};
  }
  return FieldView{m.grid_dim, m.density_channels, TVM_F32, p + L.density_lines, p + L.density_planes};
}
static FieldView appearance_field(const tvm_model_desc& m, const tvm_param_layout& L, const float* p,
                                  const void* shadow) {
  if (m.dtype == TVM_BF16 && shadow) {
    const __nv_bfloat16* s = static_cast<const __nv_bfloat16*>(shadow);
    return FieldView{m.grid_dim, m.appearance_channels, TVM_BF16, s + L.shadow_appearance_lines,
                     s + L.shadow_appearance_planes};
  }
  return FieldView{m.grid_dim, m.appearance_channels, TVM_F32, p + L.appearance_lines,
                   p + L.appearance_planes};
}

// Buffers of one render / train pass, carved from the workspace in a fixed order.
struct PassBufs {
  float* sigma;
  int32_t* sel;
  float *w_sel, *p_last, *q_last, *wsum, *X0, *rgb, *dZ3, *gw, *gP, *gsum, *dX0;
  uint8_t* X0t;  // the FeatureMlp input as tiles (BF16 models on the fused kernels), else X0
  // proposal-guided sampling
  float *sig_p, *delta_p, *w_p, *t_main, *d_main, *w_dense, *g_wp, *dz_p, *loss_p;
  int32_t* bins;
};

// BF16 models whose FeatureMlp runs on the fused kernels take its input as tiles
// (launch_appearance_fwd_tiles): bf16 in the kernels' operand layout, one bulk copy each.
static bool uses_input_tiles(const tvm_model_desc& m, const tvm_render_desc& c) {
  return m.dtype == TVM_BF16 && c.mode == TVM_MODE_RGB && mlp_fused_supported(mlp_dims(m));
}

static PassBufs carve_pass(const tvm_model_desc& m, const tvm_render_desc& c, int64_t R,
                           bool backward, Workspace& ws) {
  PassBufs b{};
  const int64_t N = c.density_samples;
  const int64_t k = (c.mode == TVM_MODE_RGB) ? c.appearance_samples : 0;
  const int64_t M = R * k;
  const int64_t F = 3LL * m.appearance_channels;
  b.sigma = ws.take<float>(R * N);
  b.sel = ws.take<int32_t>(M);
  b.w_sel = ws.take<float>(M);
  b.p_last = ws.take<float>(R);
  b.q_last = ws.take<float>(R);
  b.wsum = ws.take<float>(R);
  if (uses_input_tiles(m, c))
    b.X0t = ws.take<uint8_t>(x0t_bytes(M));
  else
    b.X0 = ws.take<float>(M * F);
  b.rgb = ws.take<float>(M * 3);
  if (backward) {
    b.dZ3 = ws.take<float>(M * 3);
    b.gw = ws.take<float>(M);
    b.gP = ws.take<float>(R);
    b.gsum = ws.take<float>(R * N);
    b.dX0 = ws.take<float>(M * F);
  }
  if (c.sampler == TVM_SAMPLER_PROPOSAL) {
    const int64_t S = R * c.proposal_samples;
    b.sig_p = ws.take<float>(S);
    b.delta_p = ws.take<float>(S);
    b.w_p = ws.take<float>(S);
    b.t_main = ws.take<float>(R * N);
    b.d_main = ws.take<float>(R * N);
    b.bins = ws.take<int32_t>(R * (N + 1));
    if (backward) {
      b.w_dense = ws.take<float>(R * N);
      b.g_wp = ws.take<float>(S);
      b.dz_p = ws.take<float>(S);
      b.loss_p = ws.take<float>(1);
    }
  }
  return b;
}

static size_t pass_bytes(const tvm_model_desc& m, const tvm_render_desc& c, int64_t R, bool backward) {
  Workspace ws{nullptr, 0, 0, true};
  carve_pass(m, c, R, backward, ws);
  const int64_t k = (c.mode == TVM_MODE_RGB) ? c.appearance_samples : 0;
  return ws.used + 256 + mlp_workspace_bytes(mlp_dims(m), R * k) + 256;
}

static FieldView proposal_field(const tvm_model_desc& m, const tvm_param_layout& L, const float* p,
                                const void* shadow) {
  if (m.dtype == TVM_BF16 && shadow) {
    const __nv_bfloat16* s = static_cast<const __nv_bfloat16*>(shadow);
    return FieldView{m.proposal_grid, m.proposal_rank, TVM_BF16, s + L.shadow_proposal_lines,
                     s + L.shadow_proposal_planes};
  }
  return FieldView{m.proposal_grid, m.proposal_rank, TVM_F32, p + L.proposal_lines, p + L.proposal_planes};
}

// Sampler of the proposal bins: bounded scenes use the aabb segment (Np uniform bins),
// unbounded ones the caller's edges with contraction.
static SamplerArgs proposal_sampler(const tvm_render_desc& c) {
  SamplerArgs s{};
  s.sampler = c.contract ? TVM_SAMPLER_EXPLICIT : TVM_SAMPLER_BBOX;
  s.contract = c.contract;
  s.N = c.proposal_samples;
  for (int a = 0; a < 6; ++a) s.aabb[a] = c.aabb[a];
  return s;
}

// Adam of a training step, applied segment by segment inside run_pass as each
// segment's gradient becomes final.
struct AdamPlan {
  float *params, *mu, *nu;
  tvm_adam_desc desc;
  __nv_bfloat16* shadow;  // BF16 models: the field shadow, refreshed with the update
  int64_t shadow_n;
  bool pending;           // apply the previous step's pending field update first
  bool defer;             // leave this step's field update pending
};

// The density and appearance fields' segments of the flat layout: [0, fields_end).
static int64_t fields_end(const tvm_model_desc& m, const tvm_param_layout& L) {
  return m.proposal_grid > 0 ? L.proposal_lines : L.mlp_begin;
}

// The scalars of a pending field update: the caller's pending count and decay, or (a
// replayed step) those the kernels read from device_step.
static tvm_adam_desc pending_desc(const tvm_adam_desc& d) {
  tvm_adam_desc p = d;
  p.count = d.pending_count;
  p.lr_decay = d.pending_lr_decay;
  p.grad_sq = nullptr;  // the previous step's gradients: not this step's norm
  p.defer_fields = 0;
  return p;
}

// render_rays forward, and (if grads != null) the loss and backward of training_step,
// and (if adam != null) the step's Adam update.
static int run_pass(const tvm_model_desc& m, const float* params, const void* shadow, float* grads,
                    const tvm_rays& rays, const float* colors, const tvm_render_desc& c,
                    float* loss, float* out, void* workspace, size_t ws_bytes, cudaStream_t st,
                    const AdamPlan* adam = nullptr) {
  tvm_param_layout L;
  make_layout(m, L);
  const bool backward = grads != nullptr;
  const int64_t R = rays.count;
  Workspace ws{static_cast<char*>(workspace), ws_bytes, 0, false};
  PassBufs b = carve_pass(m, c, R, backward, ws);
  TVM_REQUIRE(ws.ok(), TVM_ERR_WORKSPACE, "workspace too small (%zu bytes)", ws_bytes);
  if (R == 0) return TVM_OK;
  const MlpDims d = mlp_dims(m);
  SamplerArgs s = sampler_args(c);
  const bool proposal = c.sampler == TVM_SAMPLER_PROPOSAL;
  const SamplerArgs sp = proposal ? proposal_sampler(c) : SamplerArgs{};
  const float* edges = (proposal && c.contract) ? c.schedule : nullptr;
  // The field update the previous step left pending (tvm_adam_desc.defer_fields). Nothing
  // before the density gathers reads the field segments, so it runs beside the start of
  // this pass on the branch stream: density first, then appearance, each half signalled
  // to the gathers that read it. With phase events set it runs here, before phase 0.
  SideStream* pend_side = nullptr;
  if (backward && adam && adam->pending) {
    const tvm_adam_desc pd = pending_desc(adam->desc);
    const int64_t a0 = L.appearance_lines, a1 = fields_end(m, L);
    if (g_n_events == 0) {
      TVM_TRY(side_stream(pend_side));
      cudaError_t e = cudaEventRecord(pend_side->fork3, st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(pend_side->branch, pend_side->fork3, 0);
      TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "pending update fork: %s", cudaGetErrorString(e));
      const cudaStream_t ps = pend_side->branch;
      TVM_TRY(launch_adam_range(adam->params, grads, adam->mu, adam->nu, 0, a0, L.mlp_begin, pd, adam->shadow,
                                adam->shadow_n, ps, 8, true));
      e = cudaEventRecord(pend_side->density_ready, ps);
      TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "pending update: %s", cudaGetErrorString(e));
      TVM_TRY(launch_adam_range(adam->params, grads, adam->mu, adam->nu, a0, a1, L.mlp_begin, pd, adam->shadow,
                                adam->shadow_n, ps, 8, true));
      e = cudaEventRecord(pend_side->appearance_ready, ps);
      TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "pending update: %s", cudaGetErrorString(e));
    } else {
      TVM_TRY(launch_adam_range(adam->params, grads, adam->mu, adam->nu, 0, a1, L.mlp_begin, pd, adam->shadow,
                                adam->shadow_n, st, 8, true));
    }
  }
  // The fused BF16 MLP's weight images depend only on the MLP weights, final since the
  // last update: off the pass's critical path, they are packed on the side stream beside
  // its start, where mlp_forward would otherwise pack them just before the forward.
  const MlpWeights w = mlp_weights(L, params);
  SideStream* pack_side = nullptr;
  if (g_n_events == 0 && b.X0t) {
    TVM_TRY(side_stream(pack_side));
    cudaError_t e = cudaEventRecord(pack_side->fork4, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(pack_side->stream, pack_side->fork4, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "weight packing fork: %s", cudaGetErrorString(e));
    TVM_TRY(launch_mlp_pack_fused(w, mlp_fused_wpack(Workspace{static_cast<char*>(workspace), ws_bytes, ws.used, false}),
                                  pack_side->stream));
    e = cudaEventRecord(pack_side->packed, pack_side->stream);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "weight packing: %s", cudaGetErrorString(e));
  }
  phase_mark(0, st);
  if (proposal) {
    // Proposal network forward, then resampling into explicit main samples.
    // Features and the 16-U-1 MLP in one kernel (the proposal backward recomputes them).
    const FieldView fp = proposal_field(m, L, params, shadow);
    const PropMlp pm{m.proposal_units, params + L.proposal_w1, params + L.proposal_b1, params + L.proposal_w2,
                     params + L.proposal_b2, c.proposal_shift, nullptr, b.sig_p};
    TVM_TRY(launch_prop_features(fp, rays.origins, rays.directions, R, sp, edges, c.proposal_jitter, nullptr,
                                 b.delta_p, &pm, st));
    // The proposal weights (kept in w_p for the bound loss) and the resampling, one launch.
    TVM_TRY(launch_resample(nullptr, rays.origins, rays.directions, R, sp, edges, c.density_samples, c.jitter,
                            b.t_main, b.d_main, b.bins, st, b.sig_p, b.delta_p, b.w_p));
    s = SamplerArgs{};
    s.sampler = TVM_SAMPLER_EXPLICIT;
    s.N = c.density_samples;
    for (int a = 0; a < 6; ++a) s.aabb[a] = c.aabb[a];
    s.ts = b.t_main;
    s.deltas = b.d_main;
    s.contract = c.contract;
  }
  const FieldView fd = density_field(m, L, params, shadow);
  const FieldView fa = appearance_field(m, L, params, shadow);
  const int k = c.appearance_samples;

  phase_mark(1, st);
  if (pend_side) {  // the density gathers read the pending update's result
    cudaError_t e = cudaStreamWaitEvent(st, pend_side->density_ready, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "pending update join: %s", cudaGetErrorString(e));
  }
  TVM_TRY(launch_density_fwd(fd, c.density_shift, rays.origins, rays.directions, R, s, b.sigma, st));
  phase_mark(2, st);
  if (c.mode != TVM_MODE_RGB) {
    TVM_TRY(launch_composite_select(b.sigma, rays.origins, rays.directions, R, s, c.mode, 0, nullptr, 0,
                                    nullptr, nullptr, nullptr, nullptr, nullptr, out, nullptr, st));
    phase_mark(3, st);
    return TVM_OK;
  }
  TVM_TRY(launch_composite_select(b.sigma, rays.origins, rays.directions, R, s, c.mode, k, c.gumbel,
                                  c.gumbel_per_ray, b.sel, b.w_sel, b.p_last, b.q_last, b.wsum, nullptr,
                                  (proposal && backward) ? b.w_dense : nullptr, st));
  // With phase events set, the whole pass runs on the caller's stream in phase order, so
  // each phase is the span of its own kernels. Otherwise work that depends on neither
  // branch of the main chain runs beside it on side streams.
  const bool overlap = g_n_events == 0;
  SideStream* side = nullptr;
  if (overlap && backward) TVM_TRY(side_stream(side));
  auto fork_to = [&](cudaStream_t to, cudaEvent_t ev) {
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "stream fork: %s", cudaGetErrorString(e));
    return TVM_OK;
  };
  auto branch_done = [&](cudaStream_t from, cudaEvent_t ev) {
    cudaError_t e = cudaEventRecord(ev, from);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "stream join: %s", cudaGetErrorString(e));
    return TVM_OK;
  };
  auto join = [&](cudaEvent_t ev) {
    cudaError_t e = cudaStreamWaitEvent(st, ev, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "stream join: %s", cudaGetErrorString(e));
    return TVM_OK;
  };
  // Updates beside other kernels use a persistent grid of a few blocks per SM, which
  // leaves the SMs to the kernels they run beside: two while a step's field scatters have
  // a million or more density samples to work through, four below that, where those
  // kernels are short and leave the SMs idle between them.
  const int side_blocks_per_sm = R * (int64_t)c.density_samples >= (1 << 20) ? 2 : 4;
  auto adam_seg = [&](int64_t lo, int64_t hi, cudaStream_t s_) {
    return launch_adam_range(adam->params, grads, adam->mu, adam->nu, lo, hi, L.mlp_begin, adam->desc, adam->shadow,
                             adam->shadow_n, s_, s_ == st ? 8 : side_blocks_per_sm);
  };
  const bool has_prop = m.proposal_grid > 0;
  // Proposal bound loss on the main weights, then the proposal network's backward and its
  // update: they need only the forward's outputs and touch only the proposal's segments.
  auto proposal_backward = [&](cudaStream_t s_) {
    cudaError_t e = cudaMemsetAsync(b.loss_p, 0, sizeof(float), s_);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "proposal loss: %s", cudaGetErrorString(e));
    TVM_TRY(launch_prop_loss(b.w_dense, b.w_p, b.bins, R, c.proposal_samples, c.density_samples,
                             c.proposal_loss_weight / (float)R, b.loss_p, b.g_wp, s_));
    TVM_TRY(launch_segment_bwd_sum(b.sig_p, b.delta_p, R, c.proposal_samples, b.g_wp, b.dz_p, s_));
    const FieldView fp = proposal_field(m, L, params, shadow);
    const PropMlp pm{m.proposal_units, params + L.proposal_w1, params + L.proposal_b1, params + L.proposal_w2,
                     params + L.proposal_b2, c.proposal_shift, nullptr, nullptr};
    TVM_TRY(launch_prop_bwd(fp, grads + L.proposal_lines, grads + L.proposal_planes, rays.origins, rays.directions,
                            R, sp, edges, c.proposal_jitter, b.dz_p, pm, grads + L.proposal_w1,
                            grads + L.proposal_b1, grads + L.proposal_w2, grads + L.proposal_b2, s_));
    if (adam && overlap) {  // the proposal's own parameters: fields, then its MLP
      TVM_TRY(adam_seg(L.proposal_lines, L.mlp_begin, s_));
      TVM_TRY(adam_seg(L.proposal_w1, L.total, s_));
    }
    return TVM_OK;
  };
  const bool prop_forked = overlap && proposal && backward;
  if (prop_forked) {
    TVM_TRY(fork_to(side->stream, side->fork));
    TVM_TRY(proposal_backward(side->stream));
    TVM_TRY(branch_done(side->stream, side->join));
  }
  phase_mark(3, st);
  if (pend_side) {  // the appearance gathers read the pending update's result
    cudaError_t e = cudaStreamWaitEvent(st, pend_side->appearance_ready, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "pending update join: %s", cudaGetErrorString(e));
  }
  if (b.X0t)
    TVM_TRY(launch_appearance_fwd_tiles(fa, rays.origins, rays.directions, R, s, b.sel, k, b.X0t, st));
  else
    TVM_TRY(launch_appearance_fwd(fa, rays.origins, rays.directions, R, s, b.sel, k, b.X0, st));
  phase_mark(4, st);
  const size_t mlp_off = ws.used;
  if (pack_side) {
    cudaError_t e = cudaStreamWaitEvent(st, pack_side->packed, 0);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "weight packing join: %s", cudaGetErrorString(e));
  }
  // The fused BF16 MLP kernels fill every SM's shared memory and TMEM, so nothing runs
  // beside them on an SM they hold. Where other streams have work at the same time (the
  // proposal backward beside the forward; the density branch beside the backward) they
  // take half the SMs, each CTA working through more tiles: same-box A/B, BF16 step
  // 1.445 -> 1.399 ms and proposal step 0.366 -> 0.352 ms. Their time alone gets longer,
  // so a pass on one stream keeps the whole GPU for them.
  const int shared_ctas = device_sms() / 2;
  TVM_TRY(mlp_forward(d, w, b.X0, rays.directions, rays.camera_indices, k, R * k, b.rgb, ws, st,
                      overlap && prop_forked ? shared_ctas : 0, b.X0t, pack_side != nullptr));
  phase_mark(5, st);
  if (!backward) {
    TVM_TRY(launch_color_loss(b.rgb, b.w_sel, b.p_last, b.q_last, b.wsum, R, k, nullptr, out, nullptr, nullptr,
                              nullptr, nullptr, st));
    phase_mark(6, st);
    return TVM_OK;
  }
  TVM_TRY(launch_color_loss(b.rgb, b.w_sel, b.p_last, b.q_last, b.wsum, R, k, colors, out, loss, b.dZ3, b.gw,
                            b.gP, st));
  phase_mark(6, st);
  // Two independent branches follow the loss. The appearance branch (FeatureMlp backward,
  // appearance scatter, then the update of both) reads the rgb gradient dZ3; the density
  // branch (compositing backward, density scatter, then the density field's update)
  // reads the weight gradients gw / gP. They write disjoint gradient segments and
  // workspace buffers, so the appearance branch, the longer one, runs on a high-priority
  // side stream while the density branch runs on the caller's stream.
  cudaStream_t ab = st;
  if (overlap) {
    TVM_TRY(fork_to(side->branch, side->fork2));
    ab = side->branch;
  }
  Workspace ws2{static_cast<char*>(workspace), ws_bytes, mlp_off, false};
  TVM_TRY(mlp_backward(d, w, mlp_grads(L, grads), b.X0, rays.directions, rays.camera_indices, k, R * k, b.dZ3,
                       b.dX0, ws2, ab, overlap ? shared_ctas : 0, b.X0t));
  phase_mark(7, st);
  TVM_TRY(launch_appearance_bwd(fa, grads + L.appearance_lines, grads + L.appearance_planes,
                                rays.origins, rays.directions, R, s, b.sel, k, b.dX0, ab));
  const bool defer = adam && adam->defer;  // the field segments' update is left pending
  if (overlap) {
    if (adam) {
      if (!defer) TVM_TRY(adam_seg(L.appearance_lines, fields_end(m, L), ab));
      TVM_TRY(adam_seg(L.mlp_begin, has_prop ? L.proposal_w1 : L.total, ab));
    }
    TVM_TRY(branch_done(ab, side->join2));
  }
  phase_mark(8, st);
  TVM_TRY(launch_composite_bwd(b.sigma, rays.origins, rays.directions, R, s, k, b.sel, b.gw, b.gP,
                               b.gsum, st));
  phase_mark(9, st);
  TVM_TRY(launch_density_bwd(fd, grads + L.density_lines, grads + L.density_planes, rays.origins,
                             rays.directions, R, s, b.gsum, st));
  phase_mark(10, st);
  if (proposal && !overlap) TVM_TRY(proposal_backward(st));
  phase_mark(11, st);
  if (adam) {
    if (overlap) {  // the density field
      if (!defer) TVM_TRY(adam_seg(L.density_lines, L.appearance_lines, st));
    } else {
      TVM_TRY(adam_seg(defer ? fields_end(m, L) : 0, L.total, st));
    }
  }
  if (overlap) {  // the caller's stream resumes once both side streams are done
    TVM_TRY(join(side->join2));
    if (prop_forked) TVM_TRY(join(side->join));
  }
  return TVM_OK;
}

}  // namespace tvm

using namespace tvm;

extern "C" {

int tvm_abi_version(void) { return TVM_ABI_VERSION; }

uint64_t tvm_kernel_launches(void) { return g_launches; }

int tvm_set_phase_events(void* const* events, int32_t n) {
  TVM_REQUIRE(n >= 0 && n <= 32, TVM_ERR_SHAPE, "at most 32 phase events");
  TVM_REQUIRE(n == 0 || events != nullptr, TVM_ERR_INVALID, "events is NULL");
  for (int i = 0; i < n; ++i) g_events[i] = static_cast<cudaEvent_t>(events[i]);
  g_n_events = n;
  return TVM_OK;
}

const char* tvm_last_error_message(void) { return g_err; }

int tvm_get_param_layout(const tvm_model_desc* model, tvm_param_layout* out) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(out != nullptr, TVM_ERR_INVALID, "out is NULL");
  make_layout(*model, *out);
  return TVM_OK;
}

int tvm_vm_to_channel_last(int32_t grid_dim, int32_t channels, const float* vector_cf,
                           const float* matrix_cf, int32_t dtype, void* lines, void* planes,
                           void* stream) {
  TVM_REQUIRE(grid_dim >= 2 && channels >= 1, TVM_ERR_SHAPE, "bad grid_dim/channels");
  TVM_REQUIRE(vector_cf && matrix_cf && lines && planes, TVM_ERR_INVALID, "NULL pointer");
  return launch_to_channel_last(grid_dim, channels, vector_cf, matrix_cf, dtype, lines, planes,
                                as_stream(stream));
}

int tvm_vm_to_channel_first(int32_t grid_dim, int32_t channels, const float* lines,
                            const float* planes, float* vector_cf, float* matrix_cf, void* stream) {
  TVM_REQUIRE(grid_dim >= 2 && channels >= 1, TVM_ERR_SHAPE, "bad grid_dim/channels");
  TVM_REQUIRE(vector_cf && matrix_cf && lines && planes, TVM_ERR_INVALID, "NULL pointer");
  return launch_to_channel_first(grid_dim, channels, lines, planes, vector_cf, matrix_cf,
                                 as_stream(stream));
}

static int validate_field(const tvm_vm_field* f) {
  TVM_REQUIRE(f != nullptr, TVM_ERR_INVALID, "field is NULL");
  TVM_REQUIRE(f->grid_dim >= 2 && f->grid_dim <= 4096, TVM_ERR_SHAPE, "grid_dim=%d outside [2, 4096]",
              f->grid_dim);
  TVM_REQUIRE(channels_ok(f->channels), TVM_ERR_UNSUPPORTED, "channels=%d not compiled (8, 16, 24, 32, 48)",
              f->channels);
  TVM_REQUIRE(f->dtype == TVM_F32 || f->dtype == TVM_BF16, TVM_ERR_DTYPE, "field dtype %d", f->dtype);
  TVM_REQUIRE(f->lines && f->planes, TVM_ERR_INVALID, "field lines/planes NULL");
  TVM_REQUIRE(aligned(f->lines, 16) && aligned(f->planes, 16), TVM_ERR_ALIGN,
              "field buffers must be 16-byte aligned");
  return TVM_OK;
}

static FieldView view_of(const tvm_vm_field* f) {
  return FieldView{f->grid_dim, f->channels, f->dtype, f->lines, f->planes};
}

int tvm_vm_features_fwd(const tvm_vm_field* field, const float* coords, int64_t n, float* out,
                        void* stream) {
  TVM_TRY(validate_field(field));
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(n == 0 || (coords && out), TVM_ERR_INVALID, "coords/out NULL");
  return launch_vm_features_fwd(view_of(field), coords, n, out, as_stream(stream));
}

int tvm_vm_features_bwd(const tvm_vm_field* field, const float* coords, int64_t n,
                        const float* grad_out, float* grad_lines, float* grad_planes, void* stream) {
  TVM_TRY(validate_field(field));
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(n == 0 || (coords && grad_out && grad_lines && grad_planes), TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(grad_lines, 16) && aligned(grad_planes, 16), TVM_ERR_ALIGN,
              "gradient buffers must be 16-byte aligned");
  return launch_vm_features_bwd(view_of(field), coords, n, grad_out, grad_lines, grad_planes,
                                as_stream(stream));
}

int tvm_sample_points(const tvm_rays* rays, const tvm_render_desc* cfg, float* points, float* ts,
                      float* step_sizes, void* stream) {
  TVM_TRY(validate_rays(rays));
  TVM_TRY(validate_render(cfg, rays->count, false));
  TVM_REQUIRE(cfg->sampler != TVM_SAMPLER_PROPOSAL, TVM_ERR_UNSUPPORTED,
              "tvm_sample_points covers the bbox and contracted samplers");
  return launch_points(rays->origins, rays->directions, rays->count, sampler_args(*cfg), points, ts,
                       step_sizes, as_stream(stream));
}

int tvm_composite_fwd(const float* sigmas, const float* step_sizes, int64_t rays, int32_t samples,
                      float* p_exits, float* p_terminates, void* stream) {
  TVM_REQUIRE(rays >= 0 && samples >= 1, TVM_ERR_SHAPE, "rays >= 0 and samples >= 1 required");
  TVM_REQUIRE(rays == 0 || (sigmas && step_sizes), TVM_ERR_INVALID, "NULL pointer");
  return launch_segment_fwd(sigmas, step_sizes, rays, samples, p_exits, p_terminates, as_stream(stream));
}

int tvm_composite_bwd(const float* sigmas, const float* step_sizes, int64_t rays, int32_t samples,
                      const float* grad_p_exits, const float* grad_p_terminates, float* grad_sigmas,
                      void* stream) {
  TVM_REQUIRE(rays >= 0 && samples >= 1 && samples <= 8192, TVM_ERR_SHAPE, "samples outside [1, 8192]");
  TVM_REQUIRE(rays == 0 || (sigmas && step_sizes && grad_sigmas), TVM_ERR_INVALID, "NULL pointer");
  return launch_segment_bwd(sigmas, step_sizes, rays, samples, grad_p_exits, grad_p_terminates,
                            grad_sigmas, as_stream(stream));
}

int tvm_topk_select(const float* p, const float* gumbel, int32_t gumbel_per_ray, int64_t rays,
                    int32_t samples, int32_t k, int32_t* indices, void* stream) {
  TVM_REQUIRE(rays >= 0 && samples >= 1 && samples <= 8192, TVM_ERR_SHAPE, "samples outside [1, 8192]");
  TVM_REQUIRE(k >= 1 && k <= samples && k <= 1024, TVM_ERR_SHAPE, "k=%d must be in [1, min(N, 1024)]", k);
  TVM_REQUIRE(rays == 0 || (p && gumbel && indices), TVM_ERR_INVALID, "NULL pointer");
  return launch_topk(p, gumbel, gumbel_per_ray, rays, samples, k, indices, as_stream(stream));
}

size_t tvm_mlp_workspace_size(const tvm_model_desc* model, int64_t n) {
  if (validate_model(model) != TVM_OK || n < 0) return 0;
  // Forward activations plus the rgb / pre-sigmoid gradient tvm_mlp_bwd recomputes.
  return mlp_workspace_bytes(mlp_dims(*model), n) + (size_t)n * 6 * sizeof(float) + 1024;
}

int tvm_mlp_fwd(const tvm_model_desc* model, const void* params, const float* features,
                const float* viewdirs, const int32_t* camera_indices, int64_t n, float* rgb, void* workspace,
                size_t workspace_bytes, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(n == 0 || (params && features && viewdirs && rgb && workspace), TVM_ERR_INVALID,
              "NULL pointer");
  TVM_REQUIRE(aligned(params, 16), TVM_ERR_ALIGN, "params must be 16-byte aligned");
  TVM_REQUIRE(n == 0 || model->num_cameras == 0 || camera_indices, TVM_ERR_INVALID,
              "a model with camera embeddings needs camera_indices");
  tvm_param_layout L;
  make_layout(*model, L);
  Workspace ws{static_cast<char*>(workspace), workspace_bytes, 0, false};
  return mlp_forward(mlp_dims(*model), mlp_weights(L, static_cast<const float*>(params)), features,
                     viewdirs, camera_indices, 1, n, rgb, ws, as_stream(stream));
}

int tvm_mlp_bwd(const tvm_model_desc* model, const void* params, const float* features,
                const float* viewdirs, const int32_t* camera_indices, int64_t n, const float* grad_rgb,
                float* grad_features, void* grads, void* workspace, size_t workspace_bytes, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(n == 0 || (params && features && viewdirs && grad_rgb && grads && workspace),
              TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(params, 16) && aligned(grads, 16), TVM_ERR_ALIGN, "params and grads must be 16-byte aligned");
  TVM_REQUIRE(n == 0 || model->num_cameras == 0 || camera_indices, TVM_ERR_INVALID,
              "a model with camera embeddings needs camera_indices");
  if (n == 0) return TVM_OK;
  tvm_param_layout L;
  make_layout(*model, L);
  const MlpDims d = mlp_dims(*model);
  const MlpWeights w = mlp_weights(L, static_cast<const float*>(params));
  cudaStream_t st = as_stream(stream);
  // Recompute the forward (activations are not kept across ABI calls), then backward.
  Workspace ws{static_cast<char*>(workspace), workspace_bytes, 0, false};
  float* rgb = ws.take<float>(n * 3);
  float* dz = ws.take<float>(n * 3);
  const size_t off = ws.used;
  TVM_REQUIRE(ws.ok(), TVM_ERR_WORKSPACE, "workspace too small");
  TVM_TRY(mlp_forward(d, w, features, viewdirs, camera_indices, 1, n, rgb, ws, st));
  TVM_TRY(launch_sigmoid_bwd(rgb, grad_rgb, n, dz, st));
  Workspace ws2{static_cast<char*>(workspace), workspace_bytes, off, false};
  return mlp_backward(d, w, mlp_grads(L, static_cast<float*>(grads)), features, viewdirs, camera_indices, 1, n, dz,
                      grad_features, ws2, st);
}

size_t tvm_render_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg, int64_t rays) {
  if (validate_model(model) != TVM_OK || validate_render(cfg, rays, true, model) != TVM_OK || rays < 0) return 0;
  return pass_bytes(*model, *cfg, rays, false);
}

size_t tvm_train_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg, int64_t rays) {
  if (validate_model(model) != TVM_OK || validate_render(cfg, rays, true, model) != TVM_OK || rays < 0) return 0;
  return pass_bytes(*model, *cfg, rays, true);
}

static int validate_params(const tvm_model_desc* m, const void* params, const void* shadow) {
  TVM_REQUIRE(params != nullptr, TVM_ERR_INVALID, "params is NULL");
  TVM_REQUIRE(aligned(params, 16), TVM_ERR_ALIGN, "params must be 16-byte aligned");
  if (m->dtype == TVM_BF16) {
    TVM_REQUIRE(shadow != nullptr, TVM_ERR_INVALID, "BF16 model needs the bf16 shadow buffer");
    TVM_REQUIRE(aligned(shadow, 16), TVM_ERR_ALIGN, "shadow must be 16-byte aligned");
  }
  return TVM_OK;
}

// ---- proposal seams: the stages of the fused pass's proposal-guided sampling, one
// call each (bins -> sigma and lengths, weights -> main samples, bound loss, backward).
static int validate_proposal(const tvm_model_desc* m, const tvm_rays* rays, const tvm_render_desc* c) {
  TVM_TRY(validate_model(m));
  TVM_TRY(validate_rays(rays));
  TVM_REQUIRE(c != nullptr, TVM_ERR_INVALID, "render descriptor is NULL");
  TVM_REQUIRE(m->proposal_grid > 0, TVM_ERR_INVALID, "the model has no proposal network");
  TVM_REQUIRE(c->sampler == TVM_SAMPLER_PROPOSAL, TVM_ERR_INVALID, "the descriptor's sampler must be TVM_SAMPLER_PROPOSAL");
  TVM_REQUIRE(c->proposal_samples >= 2 && c->proposal_samples <= 512, TVM_ERR_SHAPE,
              "proposal_samples=%d outside [2, 512]", c->proposal_samples);
  TVM_REQUIRE(rays->count == 0 || c->proposal_jitter != nullptr, TVM_ERR_INVALID, "proposal_jitter (R, Np) is NULL");
  TVM_REQUIRE(!c->contract || c->schedule != nullptr, TVM_ERR_INVALID,
              "unbounded proposal sampling needs the Np+1 bin edges in schedule");
  for (int a = 0; a < 3; ++a)
    TVM_REQUIRE(c->aabb[a] < c->aabb[3 + a], TVM_ERR_INVALID, "aabb min must be < max on every axis");
  return TVM_OK;
}

int tvm_proposal_fwd(const tvm_model_desc* model, const void* params, const void* shadow, const tvm_rays* rays,
                     const tvm_render_desc* cfg, float* sigmas, float* deltas, void* stream) {
  TVM_TRY(validate_proposal(model, rays, cfg));
  TVM_TRY(validate_params(model, params, shadow));
  const int64_t R = rays->count;
  TVM_REQUIRE(R == 0 || (sigmas && deltas), TVM_ERR_INVALID, "sigmas/deltas NULL");
  tvm_param_layout L;
  make_layout(*model, L);
  const float* p = static_cast<const float*>(params);
  const PropMlp pm{model->proposal_units, p + L.proposal_w1, p + L.proposal_b1, p + L.proposal_w2,
                   p + L.proposal_b2, cfg->proposal_shift, nullptr, sigmas};
  return launch_prop_features(proposal_field(*model, L, p, shadow), rays->origins, rays->directions, R,
                              proposal_sampler(*cfg), cfg->contract ? cfg->schedule : nullptr, cfg->proposal_jitter,
                              nullptr, deltas, &pm, as_stream(stream));
}

int tvm_proposal_resample(const tvm_rays* rays, const tvm_render_desc* cfg, const float* weights, float* ts,
                          float* deltas, int32_t* bins, void* stream) {
  TVM_TRY(validate_rays(rays));
  TVM_REQUIRE(cfg != nullptr, TVM_ERR_INVALID, "render descriptor is NULL");
  TVM_REQUIRE(cfg->sampler == TVM_SAMPLER_PROPOSAL, TVM_ERR_INVALID, "the descriptor's sampler must be TVM_SAMPLER_PROPOSAL");
  TVM_REQUIRE(cfg->proposal_samples >= 2 && cfg->proposal_samples <= 512, TVM_ERR_SHAPE,
              "proposal_samples=%d outside [2, 512]", cfg->proposal_samples);
  TVM_REQUIRE(cfg->density_samples >= 1 && cfg->density_samples <= 512, TVM_ERR_SHAPE,
              "density_samples=%d outside [1, 512]", cfg->density_samples);
  TVM_REQUIRE(!cfg->contract || cfg->schedule != nullptr, TVM_ERR_INVALID,
              "unbounded proposal sampling needs the Np+1 bin edges in schedule");
  const int64_t R = rays->count;
  TVM_REQUIRE(R == 0 || (weights && cfg->jitter && ts && deltas && bins), TVM_ERR_INVALID,
              "weights, jitter (R, N) and the outputs must be set");
  for (int a = 0; a < 3; ++a)
    TVM_REQUIRE(cfg->aabb[a] < cfg->aabb[3 + a], TVM_ERR_INVALID, "aabb min must be < max on every axis");
  return launch_resample(weights, rays->origins, rays->directions, R, proposal_sampler(*cfg),
                         cfg->contract ? cfg->schedule : nullptr, cfg->density_samples, cfg->jitter, ts, deltas, bins,
                         as_stream(stream));
}

int tvm_proposal_loss(const float* main_weights, const float* proposal_weights, const int32_t* bins, int64_t rays,
                      int32_t proposal_samples, int32_t samples, float scale, float* loss,
                      float* grad_proposal_weights, void* stream) {
  TVM_REQUIRE(rays >= 0 && rays <= (1LL << 31), TVM_ERR_SHAPE, "ray count out of range");
  TVM_REQUIRE(proposal_samples >= 2 && proposal_samples <= 512 && samples >= 1 && samples <= 512, TVM_ERR_SHAPE,
              "proposal_samples in [2, 512] and samples in [1, 512] required");
  TVM_REQUIRE(rays == 0 || (main_weights && proposal_weights && bins && grad_proposal_weights), TVM_ERR_INVALID,
              "NULL pointer");
  return launch_prop_loss(main_weights, proposal_weights, bins, rays, proposal_samples, samples, scale, loss,
                          grad_proposal_weights, as_stream(stream));
}

int tvm_proposal_bwd(const tvm_model_desc* model, const void* params, const void* shadow, void* grads,
                     const tvm_rays* rays, const tvm_render_desc* cfg, const float* sigmas,
                     const float* grad_sigmas, void* stream) {
  TVM_TRY(validate_proposal(model, rays, cfg));
  TVM_TRY(validate_params(model, params, shadow));
  const int64_t R = rays->count;
  TVM_REQUIRE(R == 0 || (sigmas && grad_sigmas), TVM_ERR_INVALID, "sigmas/grad_sigmas NULL");
  TVM_REQUIRE(grads && aligned(grads, 16), TVM_ERR_ALIGN, "grads NULL or not 16-byte aligned");
  tvm_param_layout L;
  make_layout(*model, L);
  const float* p = static_cast<const float*>(params);
  float* g = static_cast<float*>(grads);
  PropMlp pm{model->proposal_units, p + L.proposal_w1, p + L.proposal_b1, p + L.proposal_w2,
             p + L.proposal_b2, cfg->proposal_shift, nullptr, nullptr};
  pm.sigma_in = sigmas;
  return launch_prop_bwd(proposal_field(*model, L, p, shadow), g + L.proposal_lines, g + L.proposal_planes,
                         rays->origins, rays->directions, R, proposal_sampler(*cfg),
                         cfg->contract ? cfg->schedule : nullptr, cfg->proposal_jitter, grad_sigmas, pm,
                         g + L.proposal_w1, g + L.proposal_b1, g + L.proposal_w2, g + L.proposal_b2,
                         as_stream(stream));
}

int tvm_render_fwd(const tvm_model_desc* model, const void* params, const void* shadow,
                   const tvm_rays* rays, const tvm_render_desc* cfg, float* out, void* workspace,
                   size_t workspace_bytes, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_TRY(validate_rays(rays, model));
  TVM_TRY(validate_render(cfg, rays->count, true, model));
  TVM_TRY(validate_params(model, params, shadow));
  TVM_REQUIRE(rays->count == 0 || (out && workspace), TVM_ERR_INVALID, "out/workspace NULL");
  return run_pass(*model, static_cast<const float*>(params), shadow, nullptr, *rays, nullptr, *cfg,
                  nullptr, out, workspace, workspace_bytes, as_stream(stream));
}

int tvm_loss_and_grad(const tvm_model_desc* model, const void* params, const void* shadow, void* grads,
                      const tvm_rays* rays, const float* colors, const tvm_render_desc* cfg,
                      float* loss_out, void* workspace, size_t workspace_bytes, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_TRY(validate_rays(rays, model));
  TVM_TRY(validate_render(cfg, rays->count, true, model));
  TVM_TRY(validate_params(model, params, shadow));
  TVM_REQUIRE(cfg->mode == TVM_MODE_RGB, TVM_ERR_INVALID, "training needs RGB mode");
  TVM_REQUIRE(grads && aligned(grads, 16), TVM_ERR_ALIGN, "grads NULL or not 16-byte aligned");
  TVM_REQUIRE(rays->count == 0 || (colors && loss_out && workspace), TVM_ERR_INVALID, "NULL pointer");
  cudaStream_t st = as_stream(stream);
  if (loss_out) {
    cudaError_t e = cudaMemsetAsync(loss_out, 0, sizeof(float), st);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
  }
  return run_pass(*model, static_cast<const float*>(params), shadow, static_cast<float*>(grads), *rays,
                  colors, *cfg, loss_out, nullptr, workspace, workspace_bytes, st);
}

int tvm_adam_step(const tvm_model_desc* model, void* params, void* grads, void* mu, void* nu,
                  const tvm_adam_desc* adam, void* shadow, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(params && grads && mu && nu && adam, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(params, 16) && aligned(grads, 16) && aligned(mu, 16) && aligned(nu, 16),
              TVM_ERR_ALIGN, "Adam buffers must be 16-byte aligned");
  TVM_REQUIRE(adam->device_step || adam->count >= 1, TVM_ERR_INVALID, "Adam count must be >= 1");
  TVM_REQUIRE(!adam->device_step || aligned(adam->device_step, 8), TVM_ERR_ALIGN, "device_step must be 8-byte aligned");
  tvm_param_layout L;
  make_layout(*model, L);
  cudaStream_t st = as_stream(stream);
  const bool bf16 = shadow && model->dtype == TVM_BF16;
  TVM_REQUIRE(!bf16 || aligned(shadow, 8), TVM_ERR_ALIGN, "shadow must be 8-byte aligned");
  if (adam->grad_sq) {
    cudaError_t e = cudaMemsetAsync(adam->grad_sq, 0, sizeof(float), st);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
  }
  return launch_adam(static_cast<float*>(params), static_cast<float*>(grads), static_cast<float*>(mu),
                     static_cast<float*>(nu), L.total, L.mlp_begin, *adam,
                     bf16 ? static_cast<__nv_bfloat16*>(shadow) : nullptr, bf16 ? L.shadow_total : 0, st);
}

int tvm_set_step_scalars(tvm_step_scalars* device_step, int32_t count, float lr_decay, uint64_t noise_stream,
                         int32_t pending_count, float pending_lr_decay, void* stream) {
  TVM_REQUIRE(device_step != nullptr, TVM_ERR_INVALID, "device_step is NULL");
  TVM_REQUIRE(aligned(device_step, 8), TVM_ERR_ALIGN, "device_step must be 8-byte aligned");
  TVM_REQUIRE(count >= 1, TVM_ERR_INVALID, "Adam count must be >= 1");
  TVM_REQUIRE(pending_count >= 0, TVM_ERR_INVALID, "pending count must be >= 0");
  tvm_step_scalars v;
  memset(&v, 0, sizeof(v));
  v.count = count;
  v.lr_decay = lr_decay;
  v.noise_stream = noise_stream;
  v.pending_count = pending_count;
  v.pending_lr_decay = pending_lr_decay;
  return launch_set_step_scalars(device_step, v, as_stream(stream));
}

int tvm_apply_pending_fields(const tvm_model_desc* model, void* params, void* shadow, void* grads, void* mu, void* nu,
                             const tvm_adam_desc* adam, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(params && grads && mu && nu && adam, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(params, 16) && aligned(grads, 16) && aligned(mu, 16) && aligned(nu, 16),
              TVM_ERR_ALIGN, "Adam buffers must be 16-byte aligned");
  TVM_REQUIRE(adam->pending_count >= 1, TVM_ERR_INVALID, "no pending update (pending_count must be >= 1)");
  tvm_param_layout L;
  make_layout(*model, L);
  const bool bf16 = shadow && model->dtype == TVM_BF16;
  TVM_REQUIRE(!bf16 || aligned(shadow, 8), TVM_ERR_ALIGN, "shadow must be 8-byte aligned");
  tvm_adam_desc d = pending_desc(*adam);
  d.device_step = nullptr;
  return launch_adam_range(static_cast<float*>(params), static_cast<float*>(grads), static_cast<float*>(mu),
                           static_cast<float*>(nu), 0, fields_end(*model, L), L.mlp_begin, d,
                           bf16 ? static_cast<__nv_bfloat16*>(shadow) : nullptr, bf16 ? L.shadow_total : 0,
                           as_stream(stream));
}

int tvm_refresh_shadow(const tvm_model_desc* model, const void* params, void* shadow, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(model->dtype == TVM_BF16, TVM_ERR_DTYPE, "shadow exists only for TVM_BF16 models");
  TVM_REQUIRE(params && shadow, TVM_ERR_INVALID, "NULL pointer");
  tvm_param_layout L;
  make_layout(*model, L);
  return launch_shadow(static_cast<const float*>(params), static_cast<__nv_bfloat16*>(shadow),
                       L.shadow_total, as_stream(stream));
}

int tvm_gemm(int32_t math, int32_t a_trans, int32_t b_trans, int64_t M, int32_t N, int64_t K, const float* A,
             int64_t lda, const float* B, int64_t ldb, float* D, int64_t ldd, int32_t accumulate, void* stream) {
  TVM_REQUIRE(math >= 0 && math <= 2, TVM_ERR_INVALID, "math must be 0, 1 or 2");
  TVM_REQUIRE(M >= 0 && N >= 0 && K >= 0 && M < (1LL << 31) && K < (1LL << 40), TVM_ERR_SHAPE, "bad sizes");
  if (M == 0 || N == 0) return TVM_OK;
  TVM_REQUIRE(A && B && D, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(ldd >= N && lda >= 1 && ldb >= 1, TVM_ERR_SHAPE, "bad leading dimensions");
  if (K == 0 && !accumulate) {
    cudaError_t e = cudaMemset2DAsync(D, ldd * sizeof(float), 0, N * sizeof(float), M, as_stream(stream));
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
    return TVM_OK;
  }
  return gemm_any(math, a_trans != 0, b_trans != 0, M, N, K, A, lda, B, ldb, D, ldd, accumulate != 0,
                  as_stream(stream));
}

static int validate_loss_f64(const tvm_model_desc* model, const tvm_render_desc* cfg, int64_t R) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(model->dtype == TVM_F32, TVM_ERR_DTYPE, "the FP64 loss checks TVM_F32 models");
  TVM_REQUIRE(model->num_cameras == 0, TVM_ERR_UNSUPPORTED, "the FP64 loss covers models without camera embeddings");
  TVM_TRY(validate_render(cfg, R, false, model));
  TVM_REQUIRE(cfg->sampler == TVM_SAMPLER_BBOX && cfg->mode == TVM_MODE_RGB, TVM_ERR_UNSUPPORTED,
              "the FP64 loss supports the bounded sampler in RGB mode");
  TVM_REQUIRE(cfg->appearance_samples == cfg->density_samples && cfg->density_samples <= 1024, TVM_ERR_UNSUPPORTED,
              "the FP64 loss needs k == N <= 1024 (every sample reaches the appearance path)");
  return TVM_OK;
}

size_t tvm_loss_f64_workspace_size(const tvm_model_desc* model, const tvm_render_desc* cfg, int64_t rays) {
  if (validate_loss_f64(model, cfg, rays) != TVM_OK) return 0;
  tvm_param_layout L;
  make_layout(*model, L);
  return loss_f64_scratch_bytes(*model, L.encoded_dim, rays, cfg->density_samples) + 256;
}

int tvm_loss_f64(const tvm_model_desc* model, const void* params, const tvm_rays* rays, const float* colors,
                 const tvm_render_desc* cfg, int64_t perturb_index, double perturb_delta, double* loss_out,
                 void* workspace, size_t workspace_bytes, void* stream) {
  TVM_TRY(validate_rays(rays, model));
  TVM_TRY(validate_loss_f64(model, cfg, rays->count));
  TVM_REQUIRE(params && loss_out && (rays->count == 0 || colors), TVM_ERR_INVALID, "NULL pointer");
  tvm_param_layout L;
  make_layout(*model, L);
  TVM_REQUIRE(perturb_index >= -1 && perturb_index < L.total, TVM_ERR_INVALID, "perturb_index %lld out of range",
              (long long)perturb_index);
  const size_t need = loss_f64_scratch_bytes(*model, L.encoded_dim, rays->count, cfg->density_samples);
  TVM_REQUIRE(workspace_bytes >= need && (need == 0 || workspace), TVM_ERR_WORKSPACE,
              "workspace too small (%zu < %zu bytes)", workspace_bytes, need);
  TVM_REQUIRE(aligned(workspace, 8) && aligned(loss_out, 8), TVM_ERR_ALIGN, "workspace and loss_out: 8-byte aligned");
  return launch_loss_f64(L, *model, static_cast<const float*>(params), perturb_index, perturb_delta, *rays, colors,
                         *cfg, static_cast<double*>(workspace), loss_out, as_stream(stream));
}

int tvm_resize_field(int32_t old_grid, int32_t new_grid, int32_t channels, const float* src_lines,
                     const float* src_planes, float* dst_lines, float* dst_planes, void* stream) {
  TVM_REQUIRE(old_grid >= 2 && old_grid <= 4096 && new_grid >= 2 && new_grid <= 4096, TVM_ERR_SHAPE,
              "grid sizes %d -> %d outside [2, 4096]", old_grid, new_grid);
  TVM_REQUIRE(channels >= 1 && channels <= 1024, TVM_ERR_SHAPE, "channels=%d outside [1, 1024]", channels);
  TVM_REQUIRE(src_lines && src_planes && dst_lines && dst_planes, TVM_ERR_INVALID, "NULL pointer");
  return launch_resize_field(old_grid, new_grid, channels, src_lines, src_planes, dst_lines, dst_planes,
                             as_stream(stream));
}

int tvm_device_status(int32_t* out, void* stream) {
  TVM_REQUIRE(out != nullptr, TVM_ERR_INVALID, "out is NULL");
  return device_status(out, as_stream(stream));
}

int tvm_train_step(const tvm_model_desc* model, void* params, void* shadow, void* grads, void* adam_mu,
                   void* adam_nu, const tvm_adam_desc* adam, const tvm_rays* rays, const float* colors,
                   const tvm_render_desc* cfg, float* loss_out, void* workspace, size_t workspace_bytes,
                   void* stream) {
  // The checks of tvm_loss_and_grad and tvm_adam_step, then one pass that applies Adam
  // segment by segment as the gradients become final (same result as the two calls).
  TVM_TRY(validate_model(model));
  TVM_TRY(validate_rays(rays, model));
  TVM_TRY(validate_render(cfg, rays->count, true, model));
  TVM_TRY(validate_params(model, params, shadow));
  TVM_REQUIRE(cfg->mode == TVM_MODE_RGB, TVM_ERR_INVALID, "training needs RGB mode");
  TVM_REQUIRE(grads && aligned(grads, 16), TVM_ERR_ALIGN, "grads NULL or not 16-byte aligned");
  TVM_REQUIRE(rays->count == 0 || (colors && loss_out && workspace), TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(adam_mu && adam_nu && adam, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(adam_mu, 16) && aligned(adam_nu, 16), TVM_ERR_ALIGN, "Adam buffers must be 16-byte aligned");
  TVM_REQUIRE(adam->device_step || adam->count >= 1, TVM_ERR_INVALID, "Adam count must be >= 1");
  TVM_REQUIRE(!adam->device_step || aligned(adam->device_step, 8), TVM_ERR_ALIGN, "device_step must be 8-byte aligned");
  cudaStream_t st = as_stream(stream);
  tvm_param_layout L;
  make_layout(*model, L);
  TVM_REQUIRE(adam->pending_count >= 0, TVM_ERR_INVALID, "pending count must be >= 0");
  const bool bf16 = shadow && model->dtype == TVM_BF16;
  const AdamPlan plan{static_cast<float*>(params), static_cast<float*>(adam_mu), static_cast<float*>(adam_nu), *adam,
                      bf16 ? static_cast<__nv_bfloat16*>(shadow) : nullptr, bf16 ? L.shadow_total : 0,
                      adam->device_step != nullptr || adam->pending_count > 0, adam->defer_fields != 0};
  if (rays->count == 0) {  // no rays: a plain Adam step on zero gradients
    if (plan.pending)
      TVM_TRY(launch_adam_range(plan.params, static_cast<float*>(grads), plan.mu, plan.nu, 0, fields_end(*model, L),
                                L.mlp_begin, pending_desc(*adam), plan.shadow, plan.shadow_n, st, 8, true));
    if (adam->grad_sq) {
      cudaError_t e = cudaMemsetAsync(adam->grad_sq, 0, sizeof(float), st);
      TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
    }
    TVM_TRY(launch_adam_range(plan.params, static_cast<float*>(grads), plan.mu, plan.nu,
                              plan.defer ? fields_end(*model, L) : 0, L.total, L.mlp_begin, *adam, plan.shadow,
                              plan.shadow_n, st));
    phase_mark(12, st);
    return TVM_OK;
  }
  for (float* z : {loss_out, adam->grad_sq}) {
    if (!z) continue;
    cudaError_t e = cudaMemsetAsync(z, 0, sizeof(float), st);
    TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
  }
  TVM_TRY(run_pass(*model, static_cast<const float*>(params), shadow, static_cast<float*>(grads), *rays, colors, *cfg,
                   loss_out, nullptr, workspace, workspace_bytes, st, &plan));
  phase_mark(12, st);
  return TVM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// FeatureMlp forward on library-owned scratch (tvm_mlp_fwd_static_scratch).
//
// Some callers cannot hand this library a workspace or let it allocate one:
//   - a handler run by another framework's executor, e.g. an XLA FFI custom call:
//     XLA's allocator reserves most of device memory up front (so a cudaMalloc of
//     our own can fail), and a handler only receives the buffers its call declares;
//   - code that must not stall other streams: cudaFree synchronises the device.
// For them the MLP forward's scratch (the layered path's activation buffers, or the
// fused path's packed bf16 weights, laid out exactly as for tvm_mlp_fwd) lives in one
// static device array owned by this file.
//
// The array holds TVM_MLP_STATIC_SCRATCH_BYTES (32 MiB), and a call may use it for the
// forward's buffers only (mlp_fwd_workspace_bytes), not the backward's. Its device
// address is looked up once per device, by the first call made with that device
// current (cudaGetSymbolAddress, which may load this module and so reserve the array);
// that first call should come before any stream capture. Later calls only launch
// kernels. The address is kept for the life of the process, so the entry point must
// not be used on a device after cudaDeviceReset there.
//
// Every call on a device shares the one array, so calls whose GPU work overlaps
// (different streams, or different host threads, without an ordering between them)
// race on it and give wrong results; order them on one stream or with events.
// Nothing in the array has to start at zero: each call writes every scratch byte it
// reads before reading it, so the array is never cleared.
// ---------------------------------------------------------------------------------
namespace tvm {

constexpr size_t kMlpStaticScratchBytes = size_t(32) << 20;
constexpr int kMaxStaticScratchDevices = 64;

static __device__ __align__(256) unsigned char g_mlp_static_scratch[kMlpStaticScratchBytes];

static std::mutex g_static_scratch_mu;
static void* g_static_scratch_ptr[kMaxStaticScratchDevices] = {};

// Device address of g_mlp_static_scratch for the current device (set-up on first use).
static int static_scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  TVM_REQUIRE(e == cudaSuccess, TVM_ERR_LAUNCH, "cudaGetDevice: %s", cudaGetErrorString(e));
  TVM_REQUIRE(dev >= 0 && dev < kMaxStaticScratchDevices, TVM_ERR_UNSUPPORTED,
              "device %d: static scratch supports devices 0..%d", dev, kMaxStaticScratchDevices - 1);
  std::lock_guard<std::mutex> lock(g_static_scratch_mu);
  if (g_static_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_mlp_static_scratch);
    TVM_REQUIRE(e == cudaSuccess && p != nullptr, TVM_ERR_LAUNCH, "cudaGetSymbolAddress(static scratch): %s",
                cudaGetErrorString(e));
    g_static_scratch_ptr[dev] = p;
  }
  *out = g_static_scratch_ptr[dev];
  return TVM_OK;
}

// Largest row count whose forward scratch fits the static array (monotone in n).
static int64_t static_scratch_max_rows(const MlpDims& d) {
  int64_t lo = 0, hi = int64_t(1) << 32;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    if (mlp_fwd_workspace_bytes(d, mid) <= kMlpStaticScratchBytes) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace tvm

extern "C" {

int tvm_mlp_fwd_static_scratch(const tvm_model_desc* model, const void* params, const float* features,
                               const float* viewdirs, int64_t n, float* rgb, void* stream) {
  TVM_TRY(validate_model(model));
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(model->num_cameras == 0, TVM_ERR_UNSUPPORTED,
              "the static-scratch forward takes models without camera embeddings");
  const MlpDims d = mlp_dims(*model);
  const size_t need = mlp_fwd_workspace_bytes(d, n);
  TVM_REQUIRE(need <= kMlpStaticScratchBytes, TVM_ERR_SHAPE,
              "n=%lld rows need %zu bytes of MLP scratch; the static scratch holds %zu bytes, "
              "at most %lld rows for this model",
              (long long)n, need, kMlpStaticScratchBytes, (long long)static_scratch_max_rows(d));
  if (n == 0) return TVM_OK;
  TVM_REQUIRE(params && features && viewdirs && rgb, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(params, 16), TVM_ERR_ALIGN, "params must be 16-byte aligned");
  void* scratch = nullptr;
  TVM_TRY(static_scratch_address(&scratch));
  tvm_param_layout L;
  make_layout(*model, L);
  Workspace ws{static_cast<char*>(scratch), kMlpStaticScratchBytes, 0, false};
  return mlp_forward(d, mlp_weights(L, static_cast<const float*>(params)), features, viewdirs, nullptr, 1, n, rgb, ws,
                     as_stream(stream));
}

}  // extern "C"
