// Fused Adam over the flat parameter buffer.
//
// Reference: training.py:184-203 and _make_optimizer (training.py:207-243):
// optax.chain(scale_by_adam(b1=0.9, b2=0.99, eps=1e-8, eps_root=0),
// masked(scale(-lr_mlp)), masked(scale(-lr_tensor))) followed by the learning-rate
// decay multiplier and apply_updates. One pass streams param, grad, mu, nu (4 reads,
// 3 writes + the zeroed grad): 32 B per parameter, HBM-bound, plus 2 B for the bf16
// shadow of the field segments in BF16 mode. float4 lanes, grid sized to the 152 SMs.
// Every value is touched once per step, so loads and stores carry the evict-first
// (streaming) cache hint: in a training step Adam runs beside the density scatter, whose
// field must stay in L2, and its half gigabyte would otherwise push that field out.
#include <algorithm>

#include "tvm_internal.h"

namespace tvm {

struct AdamScalars {
  float b1, b2, omb1, omb2, rbc1, rbc2, eps, lr_t, lr_m, decay;
  float* grad_sq;  // accumulates the sum of g^2 when non-null
  const tvm_step_scalars* step;  // when non-null: count and decay are read from it
  int pending;                   // read the pending update's scalars from `step` instead
};

// optax.bias_correction: 1 / (1 - decay**count) in float32.
__host__ __device__ __forceinline__ float bias_correction_rcp(float decay, int count) {
  return 1.0f / (1.0f - powf(decay, (float)count));
}

// mu_hat = mu / (1 - b1^t) and nu_hat = nu / (1 - b2^t) as products with the
// host-side reciprocals (at most one rounding apart from the quotients).
__device__ __forceinline__ float adam_one(float p, float g, float& m, float& v, float lr,
                                          const AdamScalars& a) {
  m = a.omb1 * g + a.b1 * m;
  v = a.omb2 * (g * g) + a.b2 * v;
  const float mh = m * a.rbc1;
  const float vh = v * a.rbc2;
  const float u = mh / (sqrtf(vh + 0.0f) + a.eps);
  return p + a.decay * (-lr * u);
}

// shadow (may be null): bf16 copy of the updated elements [0, shadow_n). With
// a.grad_sq, every warp adds the squares of the gradients it consumed to it.
__global__ void __launch_bounds__(256) adam_kernel(float* __restrict__ p, float* __restrict__ g,
                                                   float* __restrict__ m, float* __restrict__ v, int64_t n,
                                                   int64_t mlp_begin, __nv_bfloat16* __restrict__ shadow,
                                                   int64_t shadow_n, AdamScalars a) {
  if (a.step != nullptr) {  // a replayed step: this update's scalars from device memory
    const int count = a.pending ? a.step->pending_count : a.step->count;
    if (count <= 0) return;  // no pending update (the host applied it already)
    a.decay = a.pending ? a.step->pending_lr_decay : a.step->lr_decay;
    a.rbc1 = bias_correction_rcp(a.b1, count);
    a.rbc2 = bias_correction_rcp(a.b2, count);
  }
  const int64_t n4 = n / 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float sq = 0.f;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
    float4 pp = __ldcs(reinterpret_cast<const float4*>(p) + q);
    const float4 gg = __ldcs(reinterpret_cast<const float4*>(g) + q);
    sq += (gg.x * gg.x + gg.y * gg.y) + (gg.z * gg.z + gg.w * gg.w);
    float4 mm = __ldcs(reinterpret_cast<const float4*>(m) + q);
    float4 vv = __ldcs(reinterpret_cast<const float4*>(v) + q);
    const int64_t e = q * 4;
    const float lr = (e < mlp_begin) ? a.lr_t : a.lr_m;  // mlp_begin is a multiple of 64
    pp.x = adam_one(pp.x, gg.x, mm.x, vv.x, lr, a);
    pp.y = adam_one(pp.y, gg.y, mm.y, vv.y, lr, a);
    pp.z = adam_one(pp.z, gg.z, mm.z, vv.z, lr, a);
    pp.w = adam_one(pp.w, gg.w, mm.w, vv.w, lr, a);
    __stcs(reinterpret_cast<float4*>(p) + q, pp);
    __stcs(reinterpret_cast<float4*>(m) + q, mm);
    __stcs(reinterpret_cast<float4*>(v) + q, vv);
    // The gradient is consumed: zeroed for the next step's accumulation. Elements no
    // sample reached (most of the fields in a proposal-guided step) are zero already;
    // skipping their store saves 16 of the 136 bytes four elements move.
    if (gg.x != 0.f || gg.y != 0.f || gg.z != 0.f || gg.w != 0.f)
      __stcs(reinterpret_cast<float4*>(g) + q, make_float4(0.f, 0.f, 0.f, 0.f));
    if (shadow != nullptr && e < shadow_n) {
      __nv_bfloat162 lo = __floats2bfloat162_rn(pp.x, pp.y), hi = __floats2bfloat162_rn(pp.z, pp.w);
      __stcs(reinterpret_cast<uint2*>(shadow) + q,
             make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi)));
    }
  }
  for (int64_t e = n4 * 4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    float mm = m[e], vv = v[e];
    sq += g[e] * g[e];
    p[e] = adam_one(p[e], g[e], mm, vv, (e < mlp_begin) ? a.lr_t : a.lr_m, a);
    m[e] = mm;
    v[e] = vv;
    g[e] = 0.f;
    if (shadow != nullptr && e < shadow_n) shadow[e] = __float2bfloat16_rn(p[e]);
  }
  if (a.grad_sq != nullptr) {  // every thread of the block reaches this point
    // One reduction per block into the single word: per-warp reductions to one address
    // serialise in L2.
    __shared__ float warp_sq[8];
    sq = warp_sum(sq);
    if ((threadIdx.x & 31) == 0) warp_sq[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_sq[w];
      if (t != 0.f) atomicAdd(a.grad_sq, t);
    }
  }
}

__global__ void shadow_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst,
                              int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
    dst[e] = __float2bfloat16_rn(src[e]);
}

int launch_adam(float* params, float* grads, float* mu, float* nu, int64_t n, int64_t mlp_begin,
                const tvm_adam_desc& d, __nv_bfloat16* shadow, int64_t shadow_n, cudaStream_t st, int blocks_per_sm,
                bool pending) {
  if (n == 0) return TVM_OK;
  AdamScalars a;
  a.b1 = d.b1;
  a.b2 = d.b2;
  a.omb1 = (float)(1.0 - (double)d.b1);
  a.omb2 = (float)(1.0 - (double)d.b2);
  a.rbc1 = bias_correction_rcp(d.b1, d.count);
  a.rbc2 = bias_correction_rcp(d.b2, d.count);
  a.eps = d.eps;
  a.lr_t = d.lr_tensor;
  a.lr_m = d.lr_mlp;
  a.decay = d.lr_decay;
  a.grad_sq = d.grad_sq;
  a.step = d.device_step;
  a.pending = pending ? 1 : 0;
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n / 4 + 1, 256), (int64_t)blocks_per_sm * device_sms());
  adam_kernel<<<blocks, 256, 0, st>>>(params, grads, mu, nu, n, mlp_begin, shadow, shadow_n, a);
  return check_launch("adam");
}

int launch_adam_range(float* params, float* grads, float* mu, float* nu, int64_t lo, int64_t hi, int64_t mlp_begin,
                      const tvm_adam_desc& d, __nv_bfloat16* shadow, int64_t shadow_n, cudaStream_t st,
                      int blocks_per_sm, bool pending) {
  if (hi <= lo) return TVM_OK;
  // lo is a segment start (a multiple of 64 elements), so the offset buffers keep their
  // 16-byte alignment and the kernel's float4 lanes stay whole.
  const bool sh = shadow != nullptr && lo < shadow_n;
  return launch_adam(params + lo, grads + lo, mu + lo, nu + lo, hi - lo, mlp_begin - lo, d, sh ? shadow + lo : nullptr,
                     sh ? shadow_n - lo : 0, st, blocks_per_sm, pending);
}

__global__ void set_step_scalars_kernel(tvm_step_scalars* step, tvm_step_scalars v) { *step = v; }

int launch_set_step_scalars(tvm_step_scalars* step, const tvm_step_scalars& v, cudaStream_t st) {
  set_step_scalars_kernel<<<1, 1, 0, st>>>(step, v);
  return check_launch("set_step_scalars");
}

int launch_shadow(const float* src, __nv_bfloat16* dst, int64_t n, cudaStream_t st) {
  if (n == 0) return TVM_OK;
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 8);
  shadow_kernel<<<blocks, 256, 0, st>>>(src, dst, n);
  return check_launch("shadow");
}

}  // namespace tvm
