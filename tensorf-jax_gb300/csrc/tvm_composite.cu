// Compositing, appearance-sample selection and the compositing backward.
//
// Reference: compute_segment_probabilities (render.py:300-347), the weighted choice
// of appearance samples (render.py:459-470), the unbiasing coefficient and RGB
// composite with white background (render.py:232-246, 518-548), the distance modes
// (render.py:248-276) and the MSE loss of training_step (training.py:140).
//
// GB300 mapping: one warp owns one ray. Samples are taken 32 at a time, the
// log-transmittance cumsum is a warp shuffle scan with a carry, so transmittance stays
// in FP32 log space until the exp. The selection is exact: keys log(w)+g are mapped to
// order-preserving uint32, a 32-step MSB-first radix select finds the k-th largest key
// (count via __reduce_add_sync), winners are compacted in index order with ballots, and
// a bitonic sort in shared memory over (key desc, index asc) yields lax.top_k's order
// and tie-break. The backward runs the scan forward once more, then a reverse
// (suffix) scan for the sum over later samples.
#include <algorithm>

#include "tvm_internal.h"

namespace tvm {

__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// Exact top-k of N uint32 keys held in shared memory by one warp. Writes k packed
// entries (key << 32 | ~index) to list[0..k), sorted by key descending then index
// ascending (by_key), or in increasing index order (!by_key, no sort); list has P >= k
// slots (P a power of two).
__device__ void warp_topk(const uint32_t* keys, int N, int k, uint64_t* list, int P, int lane, bool by_key = true) {
  uint32_t T = 0;
  for (int b = 31; b >= 0; --b) {
    const uint32_t cand = T | (1u << b);
    unsigned cnt = 0;
    for (int i = lane; i < N; i += 32) cnt += (keys[i] >= cand) ? 1u : 0u;
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (cnt >= (unsigned)k) T = cand;
  }
  unsigned gt = 0;
  for (int i = lane; i < N; i += 32) gt += (keys[i] > T) ? 1u : 0u;
  gt = __reduce_add_sync(0xffffffffu, gt);
  const int need_eq = k - (int)gt;
  int sel_base = 0, eq_base = 0;
  for (int base = 0; base < N; base += 32) {
    const int i = base + lane;
    const uint32_t key = (i < N) ? keys[i] : 0u;
    const bool is_gt = (i < N) && key > T;
    const bool is_eq = (i < N) && key == T;
    const unsigned eqm = __ballot_sync(0xffffffffu, is_eq);
    const int eq_rank = eq_base + __popc(eqm & lanemask_lt(lane));
    const bool sel = is_gt || (is_eq && eq_rank < need_eq);
    const unsigned selm = __ballot_sync(0xffffffffu, sel);
    if (sel) {
      const int pos = sel_base + __popc(selm & lanemask_lt(lane));
      list[pos] = ((uint64_t)key << 32) | (uint64_t)(0xFFFFFFFFu - (uint32_t)i);
    }
    sel_base += __popc(selm);
    eq_base += __popc(eqm);
  }
  __syncwarp();
  if (!by_key) return;  // list[0, k) is already in increasing sample order
  for (int j = k + lane; j < P; j += 32) list[j] = 0ull;
  __syncwarp();
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < (P >> 1); t += 32) {
        const int lo = 2 * stride * (t / stride) + (t % stride);
        const int hi = lo + stride;
        const bool desc = (lo & size) == 0;
        const uint64_t a = list[lo], c = list[hi];
        if (desc ? (a < c) : (a > c)) {
          list[lo] = c;
          list[hi] = a;
        }
      }
      __syncwarp();
    }
  }
}

__device__ __forceinline__ int entry_index(uint64_t e) {
  return (int)(0xFFFFFFFFu - (uint32_t)(e & 0xFFFFFFFFull));
}

static inline int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// ---------------------------------------------------------------------------------
// Seam: compute_segment_probabilities forward.
// ---------------------------------------------------------------------------------
__global__ void segment_fwd_kernel(const float* __restrict__ sigmas, const float* __restrict__ steps,
                                   int64_t R, int N, float* __restrict__ p_exits,
                                   float* __restrict__ p_term) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= R) return;
  float carry = 0.f;
  for (int base = 0; base < N; base += 32) {
    const int i = base + lane;
    const bool valid = i < N;
    const float sv = valid ? -__ldg(sigmas + r * N + i) * __ldg(steps + r * N + i) : 0.f;
    const float incl = warp_inclusive_scan(sv, lane) + carry;
    const float prev = __shfl_up_sync(0xffffffffu, incl, 1);
    const float excl = (lane == 0) ? carry : prev;
    if (valid) {
      if (p_exits) p_exits[r * N + i] = expf(incl);
      if (p_term) p_term[r * N + i] = -expm1f(sv) * expf(excl);
    }
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
}

// ---------------------------------------------------------------------------------
// Backward of the compositing. With s_i = -sigma_i * delta_i, S_i = sum_{j<=i} s_j,
// w_i = (1 - e^{s_i}) e^{S_{i-1}}, p_exit_i = e^{S_i}:
//   dL/ds_i = -gw_i e^{S_i} + sum_{j>i} gw_j w_j + sum_{j>=i} gpe_j e^{S_j}.
// SPARSE: gw comes as (sel_idx, gw_sel) rows of k, gpe only at the last sample (gP).
// Output: dL/dsigma (OUT_SUM=false) or dL/d(pre-softplus sum) (OUT_SUM=true, times
// sigmoid(x) = 1 - e^{-sigma}).
// ---------------------------------------------------------------------------------
template <bool SPARSE, bool OUT_SUM>
__global__ void composite_bwd_kernel(const float* __restrict__ sigma, const float* __restrict__ steps,
                                     const float* __restrict__ origins, const float* __restrict__ dirs,
                                     int64_t R, SamplerArgs s, const float* __restrict__ g_pe,
                                     const float* __restrict__ g_pt, int k,
                                     const int32_t* __restrict__ sel_idx,
                                     const float* __restrict__ gw_sel, const float* __restrict__ gP,
                                     float* __restrict__ out) {
  extern __shared__ float smem_f[];
  const int N = s.N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* S = smem_f + (size_t)warp * 3 * N;
  float* A = S + N;
  float* GW = A + N;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= R) return;
  RayGeom g;
  if (!steps) g = load_ray(origins, dirs, r, s);
  auto delta_of = [&](int i) -> float {
    if (steps) return __ldg(steps + r * N + i);
    float t, d;
    sample_t(g, s, r, i, t, d);
    return d;
  };
  if (SPARSE) {
    for (int i = lane; i < N; i += 32) GW[i] = 0.f;
    __syncwarp();
    for (int j = lane; j < k; j += 32) GW[__ldg(sel_idx + r * k + j)] = __ldg(gw_sel + r * k + j);
    __syncwarp();
  }
  float carry = 0.f;
  for (int base = 0; base < N; base += 32) {
    const int i = base + lane;
    const bool valid = i < N;
    const float sv = valid ? -__ldg(sigma + r * N + i) * delta_of(i) : 0.f;
    const float incl = warp_inclusive_scan(sv, lane) + carry;
    const float prev = __shfl_up_sync(0xffffffffu, incl, 1);
    const float excl = (lane == 0) ? carry : prev;
    if (valid) {
      const float w = -expm1f(sv) * expf(excl);
      const float gw = SPARSE ? GW[i] : (g_pt ? __ldg(g_pt + r * N + i) : 0.f);
      float e = gw * w;
      if (!SPARSE && g_pe) e += __ldg(g_pe + r * N + i) * expf(incl);
      S[i] = incl;
      A[i] = e;
      if (!SPARSE) GW[i] = gw;
    }
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
  const float p_last = expf(carry);
  const float gpl = (SPARSE && gP) ? __ldg(gP + r) * p_last : 0.f;
  __syncwarp();
  float carry2 = 0.f;  // sum of e_j over samples after the current chunk
  const int last_base = ((N - 1) / 32) * 32;
  for (int base = last_base; base >= 0; base -= 32) {
    const int i = base + lane;
    const bool valid = i < N;
    const float e = valid ? A[i] : 0.f;
    const float incl = warp_inclusive_suffix(e, lane) + carry2;
    const float nxt = __shfl_down_sync(0xffffffffu, incl, 1);
    const float strict = (lane == 31) ? carry2 : nxt;  // sum_{j>i} e_j
    if (valid) {
      const float eS = expf(S[i]);
      float dlds = -GW[i] * eS + strict + gpl;
      if (!SPARSE && g_pe) dlds += __ldg(g_pe + r * N + i) * eS;  // the j == i term
      const float sg = __ldg(sigma + r * N + i);
      float gsg = dlds * (-delta_of(i));
      if (OUT_SUM) gsg = gsg * (-expm1f(-sg));
      out[r * N + i] = gsg;
    }
    carry2 = __shfl_sync(0xffffffffu, incl, 0);
  }
}

// ---------------------------------------------------------------------------------
// Seam: weighted choice without replacement = top-k of log(p) + gumbel.
// ---------------------------------------------------------------------------------
__global__ void topk_kernel(const float* __restrict__ p, const float* __restrict__ gumbel,
                            int gumbel_per_ray, int64_t R, int N, int k, int P,
                            int32_t* __restrict__ idx) {
  extern __shared__ unsigned char smem_b[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t per_warp = (size_t)N * 8 + (size_t)P * 8;
  uint32_t* keys = reinterpret_cast<uint32_t*>(smem_b + warp * per_warp);
  uint64_t* list = reinterpret_cast<uint64_t*>(smem_b + warp * per_warp + (size_t)N * 8);
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= R) return;
  for (int i = lane; i < N; i += 32) {
    const float gn = __ldg(gumbel + (gumbel_per_ray ? r * N + i : i));
    keys[i] = float_key_bits(logf(__ldg(p + r * N + i)) + gn);
  }
  __syncwarp();
  warp_topk(keys, N, k, list, P, lane);
  for (int j = lane; j < k; j += 32) idx[r * k + j] = entry_index(list[j]);
}

// ---------------------------------------------------------------------------------
// Fused forward compositing: sigma (R,N) -> (RGB) selection of k appearance samples,
// their weights, p_exit of the last sample and the sum of selected weights;
// (DIST_MEAN / DIST_MEDIAN) the distance.
// ---------------------------------------------------------------------------------
__global__ void composite_select_kernel(const float* __restrict__ sigma,
                                        const float* __restrict__ origins,
                                        const float* __restrict__ dirs, int64_t R, SamplerArgs s,
                                        int mode, int k, int P, const float* __restrict__ gumbel,
                                        int gumbel_per_ray, int32_t* __restrict__ sel_idx,
                                        float* __restrict__ w_sel, float* __restrict__ p_last_out,
                                        float* __restrict__ q_last_out, float* __restrict__ wsum_out,
                                        float* __restrict__ dist_out, float* __restrict__ w_dense) {
  extern __shared__ unsigned char smem_b[];
  const int N = s.N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t per_warp = (size_t)N * 8 + (size_t)P * 8;
  uint32_t* keys = reinterpret_cast<uint32_t*>(smem_b + warp * per_warp);
  float* wbuf = reinterpret_cast<float*>(keys + N);
  uint64_t* list = reinterpret_cast<uint64_t*>(smem_b + warp * per_warp + (size_t)N * 8);
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= R) return;
  RayGeom g = load_ray(origins, dirs, r, s);
  float carry = 0.f, dmean = 0.f, dmed = INFINITY, t_last = 0.f;
  bool found = false;
  for (int base = 0; base < N; base += 32) {
    const int i = base + lane;
    const bool valid = i < N;
    float t = 0.f, delta = 0.f;
    if (valid) sample_t(g, s, r, i, t, delta);
    const float sv = valid ? -__ldg(sigma + r * N + i) * delta : 0.f;
    const float incl = warp_inclusive_scan(sv, lane) + carry;
    const float prev = __shfl_up_sync(0xffffffffu, incl, 1);
    const float excl = (lane == 0) ? carry : prev;
    const float w = -expm1f(sv) * expf(excl);
    if (w_dense && valid) w_dense[r * N + i] = w;
    if (mode == TVM_MODE_RGB) {
      if (valid) {
        wbuf[i] = w;
        const float gn = __ldg(gumbel + (gumbel_per_ray ? r * N + i : i));
        keys[i] = float_key_bits(logf(w) + gn);
      }
    } else if (mode == TVM_MODE_DIST_MEAN) {
      if (valid) dmean += w * t;
      if (i == N - 1) t_last = t;
    } else {
      const unsigned b = __ballot_sync(0xffffffffu, valid && (1.0f - expf(incl)) > 0.5f);
      if (!found && b != 0u) {
        dmed = __shfl_sync(0xffffffffu, t, __ffs(b) - 1);
        found = true;
      }
    }
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
  const float p_last = expf(carry);
  if (mode == TVM_MODE_DIST_MEAN) {
    dmean = warp_sum(dmean);
    t_last = __shfl_sync(0xffffffffu, t_last, (N - 1) & 31);
    if (lane == 0) dist_out[r] = dmean + p_last * t_last;
    return;
  }
  if (mode == TVM_MODE_DIST_MEDIAN) {
    if (lane == 0) dist_out[r] = dmed;
    return;
  }
  __syncwarp();
  // Selected samples in increasing sample order (the set of jax.random.choice; the
  // order only fixes the row order of the appearance path, and the colour is summed in
  // sample order as the reference's scatter into (R, N) does).
  warp_topk(keys, N, k, list, P, lane, false);
  float ws = 0.f;
  for (int j = lane; j < k; j += 32) {
    const int i = entry_index(list[j]);
    const float w = wbuf[i];
    sel_idx[r * k + j] = i;
    w_sel[r * k + j] = w;
    ws += w;
  }
  ws = warp_sum(ws);
  if (lane == 0) {
    p_last_out[r] = p_last;
    q_last_out[r] = -expm1f(carry);  // 1 - p_last without cancellation
    wsum_out[r] = ws;
  }
}

// ---------------------------------------------------------------------------------
// Colour, loss and gradients (render.py:232-246, 529-546; training.py:140).
// C = unbias * sum_j w_j rgb_j + p_last (white background),
// unbias = (1 - p_last + 1e-8) / (sum_j w_j + 1e-8).
// ---------------------------------------------------------------------------------
__global__ void color_loss_kernel(const float* __restrict__ rgb_sel, const float* __restrict__ w_sel,
                                  const float* __restrict__ p_last_in, const float* __restrict__ q_last_in,
                                  const float* __restrict__ wsum_in, int64_t R, int k,
                                  const float* __restrict__ target, float* __restrict__ color_out,
                                  float* __restrict__ loss, float* __restrict__ dZ3,
                                  float* __restrict__ gw_sel, float* __restrict__ gP) {
  __shared__ float block_loss[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  float my_loss = 0.f;
  if (r < R) {
    float acc[3] = {0.f, 0.f, 0.f};
    for (int j = lane; j < k; j += 32) {
      const float w = __ldg(w_sel + r * k + j);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += w * __ldg(rgb_sel + (r * k + j) * 3 + c);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] = warp_sum(acc[c]);
    const float p_last = __ldg(p_last_in + r);
    const float wsum = __ldg(wsum_in + r);
    const float unbias = (__ldg(q_last_in + r) + 1e-8f) / (wsum + 1e-8f);  // q_last = 1 - p_last
    float col[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) col[c] = acc[c] * unbias + p_last * 1.0f;
    if (color_out && lane == 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) color_out[r * 3 + c] = col[c];
    }
    if (target) {
      const float inv = 1.0f / (3.0f * (float)R);
      float gC[3], A = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float diff = col[c] - __ldg(target + r * 3 + c);
        my_loss += diff * diff;
        gC[c] = 2.0f * diff * inv;
        A += gC[c] * acc[c];
      }
      my_loss *= inv;
      const float den = wsum + 1e-8f;
      for (int j = lane; j < k; j += 32) {
        const float w = __ldg(w_sel + r * k + j);
        float rg = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float v = __ldg(rgb_sel + (r * k + j) * 3 + c);
          rg += v * gC[c];
          dZ3[(r * k + j) * 3 + c] = gC[c] * w * unbias * (v * (1.0f - v));
        }
        gw_sel[r * k + j] = unbias * rg - A * unbias / den;
      }
      if (lane == 0) gP[r] = (gC[0] + gC[1] + gC[2]) - A / den;
    }
  }
  if (loss) {
    if (lane == 0) block_loss[warp] = my_loss;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += block_loss[q];
      atomicAdd(loss, t);
    }
  }
}

// ---------------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------------
static int warps_for_smem(size_t per_warp, int max_warps = 8) {
  const size_t budget = 96 * 1024;
  int w = (int)std::min<size_t>((size_t)max_warps, budget / std::max<size_t>(per_warp, 1));
  return std::max(w, 1);
}

static int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024) return ensure_smem_limit(fn, (int)bytes, "compositing");
  return TVM_OK;
}

int launch_segment_fwd(const float* sigmas, const float* steps, int64_t R, int N, float* p_exits,
                       float* p_term, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  segment_fwd_kernel<<<(unsigned)ceil_div(R, 8), 256, 0, st>>>(sigmas, steps, R, N, p_exits, p_term);
  return check_launch("segment_fwd");
}

int launch_segment_bwd(const float* sigmas, const float* steps, int64_t R, int N, const float* g_pe,
                       const float* g_pt, float* g_sigma, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const size_t per_warp = (size_t)N * 3 * sizeof(float);
  const int warps = warps_for_smem(per_warp);
  const size_t smem = per_warp * warps;
  TVM_TRY(set_smem((const void*)composite_bwd_kernel<false, false>, smem));
  SamplerArgs s{};
  s.N = N;
  composite_bwd_kernel<false, false><<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(
      sigmas, steps, nullptr, nullptr, R, s, g_pe, g_pt, 0, nullptr, nullptr, nullptr, g_sigma);
  return check_launch("segment_bwd");
}

int launch_segment_bwd_sum(const float* sigmas, const float* steps, int64_t R, int N, const float* g_pt,
                           float* g_sum, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const size_t per_warp = (size_t)N * 3 * sizeof(float);
  const int warps = warps_for_smem(per_warp);
  const size_t smem = per_warp * warps;
  TVM_TRY(set_smem((const void*)composite_bwd_kernel<false, true>, smem));
  SamplerArgs s{};
  s.N = N;
  composite_bwd_kernel<false, true><<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(
      sigmas, steps, nullptr, nullptr, R, s, nullptr, g_pt, 0, nullptr, nullptr, nullptr, g_sum);
  return check_launch("segment_bwd_sum");
}

int launch_topk(const float* p, const float* gumbel, int gumbel_per_ray, int64_t R, int N, int k,
                int32_t* idx, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const int P = next_pow2(k);
  const size_t per_warp = (size_t)N * 8 + (size_t)P * 8;
  const int warps = warps_for_smem(per_warp);
  const size_t smem = per_warp * warps;
  TVM_TRY(set_smem((const void*)topk_kernel, smem));
  topk_kernel<<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(p, gumbel, gumbel_per_ray, R,
                                                                       N, k, P, idx);
  return check_launch("topk");
}

int launch_composite_select(const float* sigma, const float* origins, const float* dirs, int64_t R,
                            const SamplerArgs& s, int mode, int k, const float* gumbel,
                            int gumbel_per_ray, int32_t* sel_idx, float* w_sel, float* p_last,
                            float* q_last, float* wsum, float* dist_out, float* w_dense, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const int P = (mode == TVM_MODE_RGB) ? next_pow2(k) : 1;
  const size_t per_warp = (size_t)s.N * 8 + (size_t)P * 8;
  const int warps = warps_for_smem(per_warp);
  const size_t smem = per_warp * warps;
  TVM_TRY(set_smem((const void*)composite_select_kernel, smem));
  composite_select_kernel<<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(
      sigma, origins, dirs, R, s, mode, k, P, gumbel, gumbel_per_ray, sel_idx, w_sel, p_last, q_last, wsum,
      dist_out, w_dense);
  return check_launch("composite_select");
}

int launch_color_loss(const float* rgb_sel, const float* w_sel, const float* p_last, const float* q_last,
                      const float* wsum, int64_t R, int k, const float* target, float* color_out,
                      float* loss, float* dZ3, float* gw_sel, float* gP, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  color_loss_kernel<<<(unsigned)ceil_div(R, 8), 256, 0, st>>>(rgb_sel, w_sel, p_last, q_last, wsum, R, k,
                                                               target, color_out, loss, dZ3, gw_sel,
                                                               gP);
  return check_launch("color_loss");
}

int launch_composite_bwd(const float* sigma, const float* origins, const float* dirs, int64_t R,
                         const SamplerArgs& s, int k, const int32_t* sel_idx, const float* gw_sel,
                         const float* gP, float* gsum, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const size_t per_warp = (size_t)s.N * 3 * sizeof(float);
  const int warps = warps_for_smem(per_warp);
  const size_t smem = per_warp * warps;
  TVM_TRY(set_smem((const void*)composite_bwd_kernel<true, true>, smem));
  composite_bwd_kernel<true, true><<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(
      sigma, nullptr, origins, dirs, R, s, nullptr, nullptr, k, sel_idx, gw_sel, gP, gsum);
  return check_launch("composite_bwd");
}

}  // namespace tvm
