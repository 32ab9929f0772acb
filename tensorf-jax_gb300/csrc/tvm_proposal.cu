// Proposal network: a density-only VM tensor (rank 4 per pair, small grid) plus a
// 16 -> 64 -> 1 MLP that predicts where along each ray the full field is worth
// evaluating. The reference has no such component (render.py:126 notes that "an
// occupancy grid or proposal network would really help us here"); the design follows
// the proposal sampling of mip-NeRF 360 (Barron et al., 2022):
//
//  * proposal bins: Np bins per ray over the aabb segment (bounded scenes) or over
//    caller-given edges (unbounded scenes), one jittered sample per bin;
//  * proposal density sigma^ = softplus(MLP([12 VM features, x, y, z, |x|_inf]) + shift),
//    weights w^ by the same log-space compositing as the main field;
//  * resampling: N+1 edges at the quantiles i/N of the bin histogram (w^ plus a 1%
//    uniform floor), one jittered main sample per resulting interval;
//  * training: the main field's weights w_i (no gradient) must not exceed the
//    proposal mass over the bins their interval overlaps,
//    L = lambda/R * sum_i max(0, w_i - bound_i)^2 / (w_i + 1e-7), gradient into w^ only.
//
// The 16 -> U -> 1 MLP is evaluated inside the per-sample feature kernel. Its backward
// runs fused with the field scatter: on tcgen05 for BF16 models with U = 64 (bf16
// operands, as the rest of that mode), in FP32 SIMT otherwise.
#include "tvm_internal.h"
#include "tvm_tc.cuh"

namespace tvm {

constexpr int PROP_C = 4;      // components per pair
constexpr int PROP_IN = 16;    // MLP input width

// Bin edge j (0..Np) of a ray: t_min + j * step over its aabb segment (step = segment
// length / Np, as the bounded sampler computes it), or the caller's edges.
__device__ __forceinline__ float prop_edge(const RayGeom& g, const float* edges, int j) {
  return edges ? __ldg(edges + j) : g.t_min + (float)j * g.step;
}

template <typename T>
__device__ __forceinline__ void load4(const T* p, float (&v)[4]);
template <>
__device__ __forceinline__ void load4<float>(const float* p, float (&v)[4]) {
  const float4 q = __ldg(reinterpret_cast<const float4*>(p));
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <>
__device__ __forceinline__ void load4<__nv_bfloat16>(const __nv_bfloat16* p, float (&v)[4]) {
  const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
  const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.x));
  const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.y));
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

struct PropPair {
  Tap tl, tr, tc;
  float L[4], P[4];
};

template <typename T>
__device__ __forceinline__ void prop_pair(const T* lines, const T* planes, int G, int m, float ul, float ur, float uc,
                                          PropPair& e) {
  e.tl = make_tap(ul, G);
  e.tr = make_tap(ur, G);
  e.tc = make_tap(uc, G);
  const T* lb = lines + (int64_t)m * G * PROP_C;
  const T* pb = planes + (int64_t)m * G * G * PROP_C;
  float l0[4], l1[4], p00[4], p01[4], p10[4], p11[4];
  load4<T>(lb + e.tl.i0 * PROP_C, l0);
  load4<T>(lb + e.tl.i1 * PROP_C, l1);
  load4<T>(pb + ((int64_t)e.tr.i0 * G + e.tc.i0) * PROP_C, p00);
  load4<T>(pb + ((int64_t)e.tr.i0 * G + e.tc.i1) * PROP_C, p01);
  load4<T>(pb + ((int64_t)e.tr.i1 * G + e.tc.i0) * PROP_C, p10);
  load4<T>(pb + ((int64_t)e.tr.i1 * G + e.tc.i1) * PROP_C, p11);
  const float w00 = e.tr.w0 * e.tc.w0, w01 = e.tr.w0 * e.tc.w1, w10 = e.tr.w1 * e.tc.w0, w11 = e.tr.w1 * e.tc.w1;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    e.L[c] = e.tl.w0 * l0[c] + e.tl.w1 * l1[c];
    e.P[c] = w00 * p00[c] + w01 * p01[c] + w10 * p10[c] + w11 * p11[c];
  }
}

// Geometry of proposal sample (r, j): world distance, bin length, normalised point.
__device__ __forceinline__ void prop_sample(const RayGeom& g, const SamplerArgs& s, const float* edges, int Np,
                                            const float* jitter, int64_t r, int j, float& t, float& len,
                                            float (&x)[3]) {
  const float e0 = prop_edge(g, edges, j);
  const float e1 = prop_edge(g, edges, j + 1);
  len = e1 - e0;
  t = e0 + __ldg(jitter + r * Np + j) * len;
  sample_point(g, s, t, x);
}

// Features X[s] = [12 VM features (pair-major), x, y, z, |x|_inf], bin length, and
// (with weights) the whole MLP in registers: h = relu(X W1 + b1), sigma = softplus(h W2
// + b2 + shift). The weights sit in shared memory and every thread reads the same
// element at the same time (broadcast); each thread carries PROP_SPT samples (blockDim
// apart) through the MLP, so every weight it loads serves all of them. X and h are
// written only when the backward needs them.
constexpr int PROP_SPT = 2;
template <typename T>
__device__ __forceinline__ void prop_sample_features(const T* __restrict__ lines, const T* __restrict__ planes, int G,
                                                     const float* __restrict__ origins, const float* __restrict__ dirs,
                                                     const SamplerArgs& s, const float* __restrict__ edges,
                                                     const float* __restrict__ jitter, int64_t smp,
                                                     float (&out)[PROP_IN], float& len) {
  const int Np = s.N;
  const int64_t r = smp / Np;
  const int j = (int)(smp - r * Np);
  RayGeom g = load_ray(origins, dirs, r, s);
  float t, x[3];
  prop_sample(g, s, edges, Np, jitter, r, j, t, len, x);
  float u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = grid_coord(x[a], G);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PropPair e;
    prop_pair<T>(lines, planes, G, m, u[a], u[b], u[c], e);
#pragma unroll
    for (int q = 0; q < 4; ++q) out[m * 4 + q] = e.L[q] * e.P[q];
  }
  out[12] = x[0];
  out[13] = x[1];
  out[14] = x[2];
  out[15] = fmaxf(fabsf(x[0]), fmaxf(fabsf(x[1]), fabsf(x[2])));
}

template <typename T>
__global__ void __launch_bounds__(128) prop_features_kernel(
    const T* __restrict__ lines, const T* __restrict__ planes, int G, const float* __restrict__ origins,
    const float* __restrict__ dirs, int64_t R, SamplerArgs s, const float* __restrict__ edges,
    const float* __restrict__ jitter, float* __restrict__ X, float* __restrict__ delta, int units,
    const float* __restrict__ w1, const float* __restrict__ b1, const float* __restrict__ w2,
    const float* __restrict__ b2, float shift, float* __restrict__ H, float* __restrict__ sigma) {
  extern __shared__ __align__(16) float sw[];  // w1 transposed [units][16], b1 [units], w2 [units]
  const bool mlp = w1 != nullptr;
  if (mlp) {
    for (int e = threadIdx.x; e < 18 * units; e += blockDim.x) {
      float v;
      if (e < 16 * units) {
        const int u = e / 16, i = e % 16;
        v = __ldg(w1 + i * units + u);
      } else {
        v = e < 17 * units ? __ldg(b1 + e - 16 * units) : __ldg(w2 + e - 17 * units);
      }
      sw[e] = v;
    }
    __syncthreads();
  }
  const int64_t n = R * s.N;
  const int64_t smp0 = (int64_t)blockIdx.x * (PROP_SPT * blockDim.x) + threadIdx.x;
  if (smp0 >= n) return;
  int64_t smps[PROP_SPT];
  bool has[PROP_SPT];
  float out[PROP_SPT][PROP_IN];
#pragma unroll
  for (int k = 0; k < PROP_SPT; ++k) {
    smps[k] = smp0 + (int64_t)k * blockDim.x;
    has[k] = smps[k] < n;
    if (!has[k]) {
#pragma unroll
      for (int i = 0; i < PROP_IN; ++i) out[k][i] = 0.f;
      continue;
    }
    float len;
    prop_sample_features<T>(lines, planes, G, origins, dirs, s, edges, jitter, smps[k], out[k], len);
    if (X) {
      float4* dst = reinterpret_cast<float4*>(X + smps[k] * PROP_IN);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        dst[q] = make_float4(out[k][4 * q], out[k][4 * q + 1], out[k][4 * q + 2], out[k][4 * q + 3]);
    }
    delta[smps[k]] = len;
  }
  if (!mlp) return;
  const float4* sw1 = reinterpret_cast<const float4*>(sw);  // row u: 16 weights
  const float* sb1 = sw + 16 * units;
  const float* sw2 = sw + 17 * units;
  float z[PROP_SPT];
#pragma unroll
  for (int k = 0; k < PROP_SPT; ++k) z[k] = __ldg(b2);
  for (int u = 0; u < units; ++u) {
    float h[PROP_SPT];
#pragma unroll
    for (int k = 0; k < PROP_SPT; ++k) h[k] = sb1[u];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 w = sw1[u * 4 + q];
#pragma unroll
      for (int k = 0; k < PROP_SPT; ++k) {
        h[k] = fmaf(out[k][4 * q], w.x, h[k]);
        h[k] = fmaf(out[k][4 * q + 1], w.y, h[k]);
        h[k] = fmaf(out[k][4 * q + 2], w.z, h[k]);
        h[k] = fmaf(out[k][4 * q + 3], w.w, h[k]);
      }
    }
    const float w2u = sw2[u];
#pragma unroll
    for (int k = 0; k < PROP_SPT; ++k) {
      h[k] = fmaxf(h[k], 0.0f);
      if (H && has[k]) H[smps[k] * units + u] = h[k];
      z[k] = fmaf(h[k], w2u, z[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < PROP_SPT; ++k)
    if (has[k]) sigma[smps[k]] = softplus_f(z[k] + shift);
}

// Fused proposal backward, one thread per sample, 128 samples per block: recompute the
// features X (16) and hidden units h (U) in registers, dz -> dh = dz * w2 * [h > 0] ->
// dX = dh W1^T -> scatter dX[0:12) into the proposal field gradients. The weight
// gradients dW1 = sum_s X_s dh_s^T, db1 = sum dh, dW2 = sum h dz, db2 = sum dz are
// reduced over the block in shared memory, then added to global memory with one atomic
// per weight per block.
constexpr int PBWD_THREADS = 128;

// dL/dz of sample i, z the proposal MLP's output before the shift and softplus: dz_in
// holds it, or (sig_in set) dz_in holds dL/dsigma, scaled by dsigma/dz = sigmoid(z +
// shift) = 1 - exp(-sigma) for sigma = softplus(z + shift).
__device__ __forceinline__ float load_dz(const float* __restrict__ dz_in, const float* __restrict__ sig_in,
                                         int64_t i) {
  const float g = __ldg(dz_in + i);
  return sig_in ? g * -expm1f(-__ldg(sig_in + i)) : g;
}

template <typename T>
__global__ void __launch_bounds__(PBWD_THREADS) prop_bwd_kernel(
    const T* __restrict__ lines, const T* __restrict__ planes, int G, float* __restrict__ glines,
    float* __restrict__ gplanes, const float* __restrict__ origins, const float* __restrict__ dirs, int64_t R,
    SamplerArgs s, const float* __restrict__ edges, const float* __restrict__ jitter, const float* __restrict__ dz_in,
    const float* __restrict__ sig_in, int units, const float* __restrict__ w1, const float* __restrict__ b1, const float* __restrict__ w2,
    float* __restrict__ gw1, float* __restrict__ gb1, float* __restrict__ gw2, float* __restrict__ gb2) {
  extern __shared__ __align__(16) float sm[];
  float* sw1 = sm;                          // transposed [U][16]
  float* sb1 = sw1 + 16 * units;            // [U]
  float* sw2 = sb1 + units;                 // [U]
  const int ld = units + 4;                 // row pitch: float4-aligned, 4-way store conflicts at most
  float* sX = sw2 + units;                  // [128][16]
  float* sdh = sX + PBWD_THREADS * 16;      // [128][U+4]
  float* sh = sdh + PBWD_THREADS * ld;      // [128][U+4]
  float* sdz = sh + PBWD_THREADS * ld;      // [128]
  const int tid = threadIdx.x;
  for (int e = tid; e < 18 * units; e += PBWD_THREADS) {
    float v;
    if (e < 16 * units) {
      const int u = e / 16, i = e % 16;
      v = __ldg(w1 + i * units + u);
    } else {
      v = e < 17 * units ? __ldg(b1 + e - 16 * units) : __ldg(w2 + e - 17 * units);
    }
    sm[e] = v;
  }
  __syncthreads();
  const int Np = s.N;
  const int64_t smp = (int64_t)blockIdx.x * PBWD_THREADS + tid;
  const bool valid = smp < R * Np;
  float dz = valid ? load_dz(dz_in, sig_in, smp) : 0.f;
  // A sample with dz = 0 adds nothing to any gradient (dh = 0, so dX, dW1, dW2 and db1
  // rows are all zero): its gathers and scatter are skipped.
  const bool live = valid && dz != 0.f;
  float X[PROP_IN];
#pragma unroll
  for (int i = 0; i < PROP_IN; ++i) X[i] = 0.f;
  PropPair e3[3];
  if (live) {
    const int64_t r = smp / Np;
    const int j = (int)(smp - r * Np);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, len, x[3];
    prop_sample(g, s, edges, Np, jitter, r, j, t, len, x);
    float u3[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) u3[a] = grid_coord(x[a], G);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      int a, b, c;
      mode_perm(m, a, b, c);
      prop_pair<T>(lines, planes, G, m, u3[a], u3[b], u3[c], e3[m]);
#pragma unroll
      for (int q = 0; q < 4; ++q) X[m * 4 + q] = e3[m].L[q] * e3[m].P[q];
    }
    X[12] = x[0];
    X[13] = x[1];
    X[14] = x[2];
    X[15] = fmaxf(fabsf(x[0]), fmaxf(fabsf(x[1]), fabsf(x[2])));
  }
  // Recompute h, form dh and dX.
  float dX[PROP_IN];
#pragma unroll
  for (int i = 0; i < PROP_IN; ++i) dX[i] = 0.f;
  const float4* sw1v = reinterpret_cast<const float4*>(sw1);
  for (int u = 0; u < units; ++u) {
    float4 w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = sw1v[u * 4 + q];
    float h = sb1[u];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      h = fmaf(X[4 * q], w[q].x, h);
      h = fmaf(X[4 * q + 1], w[q].y, h);
      h = fmaf(X[4 * q + 2], w[q].z, h);
      h = fmaf(X[4 * q + 3], w[q].w, h);
    }
    h = fmaxf(h, 0.f);
    const float dh = (h > 0.f) ? dz * sw2[u] : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      dX[4 * q] = fmaf(dh, w[q].x, dX[4 * q]);
      dX[4 * q + 1] = fmaf(dh, w[q].y, dX[4 * q + 1]);
      dX[4 * q + 2] = fmaf(dh, w[q].z, dX[4 * q + 2]);
      dX[4 * q + 3] = fmaf(dh, w[q].w, dX[4 * q + 3]);
    }
    sdh[tid * ld + u] = dh;
    sh[tid * ld + u] = h;
  }
#pragma unroll
  for (int i = 0; i < PROP_IN; ++i) sX[tid * 16 + i] = X[i];
  sdz[tid] = dz;
  // Field gradient scatter.
  bool any = false;
#pragma unroll
  for (int q = 0; q < 12; ++q) any |= (dX[q] != 0.0f);
  if (live && any) {
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const PropPair& e = e3[m];
      float* lb = glines + (int64_t)m * G * PROP_C;
      float* pb = gplanes + (int64_t)m * G * G * PROP_C;
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.P[q] * e.tl.w0;
      atomicAdd(reinterpret_cast<float4*>(lb + e.tl.i0 * PROP_C), make_float4(v[0], v[1], v[2], v[3]));
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.P[q] * e.tl.w1;
      atomicAdd(reinterpret_cast<float4*>(lb + e.tl.i1 * PROP_C), make_float4(v[0], v[1], v[2], v[3]));
      const float w[4] = {e.tr.w0 * e.tc.w0, e.tr.w0 * e.tc.w1, e.tr.w1 * e.tc.w0, e.tr.w1 * e.tc.w1};
      const int rows[4] = {e.tr.i0, e.tr.i0, e.tr.i1, e.tr.i1};
      const int cols[4] = {e.tc.i0, e.tc.i1, e.tc.i0, e.tc.i1};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.L[q] * w[k];
        atomicAdd(reinterpret_cast<float4*>(pb + ((int64_t)rows[k] * G + cols[k]) * PROP_C),
                  make_float4(v[0], v[1], v[2], v[3]));
      }
    }
  }
  __syncthreads();
  // Block reduction of the weight gradients. dW1 (16 x U): thread t owns feature
  // i = t % 16 and units [8*(t/16), +8) (+ 64 per extra pass when U > 64), 8 FMAs per
  // sample from one X load and two 16-byte dh loads. Then dW2, db1 and db2.
  for (int u0 = (tid / 16) * 8; u0 < units; u0 += (PBWD_THREADS / 16) * 8) {
    const int i = tid % 16;
    float acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = 0.f;
    if (u0 + 8 <= units) {
      for (int q = 0; q < PBWD_THREADS; ++q) {
        const float xv = sX[q * 16 + i];
        const float4 d0 = *reinterpret_cast<const float4*>(sdh + q * ld + u0);
        const float4 d1 = *reinterpret_cast<const float4*>(sdh + q * ld + u0 + 4);
        acc[0] = fmaf(xv, d0.x, acc[0]); acc[1] = fmaf(xv, d0.y, acc[1]);
        acc[2] = fmaf(xv, d0.z, acc[2]); acc[3] = fmaf(xv, d0.w, acc[3]);
        acc[4] = fmaf(xv, d1.x, acc[4]); acc[5] = fmaf(xv, d1.y, acc[5]);
        acc[6] = fmaf(xv, d1.z, acc[6]); acc[7] = fmaf(xv, d1.w, acc[7]);
      }
    } else {
      for (int q = 0; q < PBWD_THREADS; ++q) {
        const float xv = sX[q * 16 + i];
        for (int e = 0; e < 8 && u0 + e < units; ++e) acc[e] = fmaf(xv, sdh[q * ld + u0 + e], acc[e]);
      }
    }
    for (int e = 0; e < 8 && u0 + e < units; ++e)
      if (acc[e] != 0.f) atomicAdd(gw1 + i * units + u0 + e, acc[e]);
  }
  for (int e = tid; e < 2 * units + 1; e += PBWD_THREADS) {
    float acc = 0.f;
    if (e < units) {
      for (int q = 0; q < PBWD_THREADS; ++q) acc = fmaf(sh[q * ld + e], sdz[q], acc);
      if (acc != 0.f) atomicAdd(gw2 + e, acc);
    } else if (e < 2 * units) {
      for (int q = 0; q < PBWD_THREADS; ++q) acc += sdh[q * ld + e - units];
      if (acc != 0.f) atomicAdd(gb1 + e - units, acc);
    } else {
      for (int q = 0; q < PBWD_THREADS; ++q) acc += sdz[q];
      if (acc != 0.f) atomicAdd(gb2, acc);
    }
  }
}

// Resampling, one warp per ray: histogram q_j = w^_j + (0.01 * sum w^ + 1e-4) / Np over
// the Np bins, main edges at the quantiles i/N (i = 0..N) by linear interpolation
// inside the bin, one main sample per interval at edge_i + jitter * length.
// WEIGHTS: the proposal weights are computed here from the bin densities and lengths,
// with segment_fwd_kernel's arithmetic, and written to wprop (one launch fewer on the
// pass's critical path); otherwise wprop is read.
template <bool WEIGHTS>
__global__ void resample_kernel(float* __restrict__ wprop, const float* __restrict__ sig,
                                const float* __restrict__ len, const float* __restrict__ origins,
                                const float* __restrict__ dirs, int64_t R, SamplerArgs s, const float* __restrict__ edges,
                                int Nm, const float* __restrict__ jitter, float* __restrict__ t_out,
                                float* __restrict__ d_out, int32_t* __restrict__ bins) {
  extern __shared__ float smem_f[];
  const int Np = s.N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* cdf = smem_f + warp * (2 * (Np + 1) + (Nm + 1));  // cdf[0..Np], edge[0..Np], sedge[0..Nm]
  float* edge = cdf + (Np + 1);
  float* sedge = edge + (Np + 1);
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= R) return;
  RayGeom g = load_ray(origins, dirs, r, s);
  // cdf[j + 1] holds bin j's weight until the scan below replaces it.
  float tot = 0.f;
  if (WEIGHTS) {
    float carry_s = 0.f;
    for (int base = 0; base < Np; base += 32) {
      const int j = base + lane;
      const bool valid = j < Np;
      const float sv = valid ? -__ldg(sig + r * Np + j) * __ldg(len + r * Np + j) : 0.f;
      const float incl = warp_inclusive_scan(sv, lane) + carry_s;
      const float prev = __shfl_up_sync(0xffffffffu, incl, 1);
      const float excl = (lane == 0) ? carry_s : prev;
      if (valid) {
        const float w = -expm1f(sv) * expf(excl);
        wprop[r * Np + j] = w;
        cdf[j + 1] = w;
        tot += w;
      }
      carry_s = __shfl_sync(0xffffffffu, incl, 31);
    }
  } else {
    for (int j = lane; j < Np; j += 32) {
      cdf[j + 1] = __ldg(wprop + r * Np + j);
      tot += cdf[j + 1];
    }
  }
  tot = warp_sum(tot);
  const float floor_w = (0.01f * tot + 1e-4f) / (float)Np;
  float carry = 0.f;
  __syncwarp();
  if (lane == 0) cdf[0] = 0.f;
  for (int base = 0; base < Np; base += 32) {
    const int j = base + lane;
    const float q = (j < Np) ? cdf[j + 1] + floor_w : 0.f;
    const float incl = warp_inclusive_scan(q, lane) + carry;
    if (j < Np) cdf[j + 1] = incl;
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
  for (int j = lane; j <= Np; j += 32) edge[j] = prop_edge(g, edges, j);
  __syncwarp();
  const float Q = carry;
  for (int i = lane; i <= Nm; i += 32) {
    int bin;
    float e;
    if (i == 0) {
      bin = 0;
      e = edge[0];
    } else if (i == Nm) {
      bin = Np - 1;
      e = edge[Np];
    } else {
      const float target = Q * ((float)i / (float)Nm);
      int lo = 0, hi = Np - 1;  // largest bin with cdf[bin] <= target
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cdf[mid] <= target) lo = mid; else hi = mid - 1;
      }
      bin = lo;
      const float q = cdf[bin + 1] - cdf[bin];
      const float f = q > 0.f ? fminf(fmaxf((target - cdf[bin]) / q, 0.f), 1.f) : 0.f;
      e = edge[bin] + f * (edge[bin + 1] - edge[bin]);
    }
    sedge[i] = e;
    bins[r * (Nm + 1) + i] = bin;
  }
  __syncwarp();
  for (int i = lane; i < Nm; i += 32) {
    const float a = sedge[i], b = fmaxf(sedge[i + 1], a);
    const float len = b - a;
    t_out[r * Nm + i] = a + __ldg(jitter + r * Nm + i) * len;
    d_out[r * Nm + i] = len;
  }
}

// Proposal bound loss and its gradient wrt w^ (one warp per ray). Each interval's bound
// is summed directly over its bins: a difference of two prefix sums would lose the small
// bounds of empty space to FP32 cancellation (the prefix reaches the ray's total mass).
// The intervals tile the bins in order, so the direct sums read about Np + Nm values.
__global__ void prop_loss_kernel(const float* __restrict__ wmain, const float* __restrict__ wprop,
                                 const int32_t* __restrict__ bins, int64_t R, int Np, int Nm, float scale,
                                 float* __restrict__ loss, float* __restrict__ gprop) {
  extern __shared__ float smem_f[];
  __shared__ float block_loss[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* W = smem_f + warp * 2 * (Np + 2);
  float* diff = W + (Np + 2);
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (r >= R) {  // a whole warp past the last ray: it adds nothing to the block's loss
    if (lane == 0) block_loss[warp] = 0.f;
    __syncthreads();
    return;
  }
  for (int j = lane; j < Np; j += 32) W[j] = __ldg(wprop + r * Np + j);
  for (int j = lane; j < Np + 2; j += 32) diff[j] = 0.f;
  __syncwarp();
  float my_loss = 0.f;
  for (int i = lane; i < Nm; i += 32) {
    // Clamped into the ray's bins (the resampler's indices always are; a caller's may not).
    const int lo = min(max(__ldg(bins + r * (Nm + 1) + i), 0), Np - 1);
    const int hi = min(max(__ldg(bins + r * (Nm + 1) + i + 1), lo), Np - 1);
    float bound = 0.f;
    for (int j = lo; j <= hi; ++j) bound += W[j];
    const float w = __ldg(wmain + r * Nm + i);
    const float dd = fmaxf(w - bound, 0.f);
    const float inv = 1.0f / (w + 1e-7f);
    my_loss += dd * dd * inv;
    const float gi = -2.0f * dd * inv * scale;
    if (gi != 0.f) {
      atomicAdd(&diff[lo], gi);
      atomicAdd(&diff[hi + 1], -gi);
    }
  }
  // One reduction per block into the single loss word: per-warp reductions to one
  // address serialise in L2.
  my_loss = warp_sum(my_loss);
  if (lane == 0) block_loss[warp] = my_loss * scale;
  __syncthreads();
  if (threadIdx.x == 0 && loss) {
    float t = 0.f;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += block_loss[q];
    atomicAdd(loss, t);
  }
  __syncwarp();
  float carry = 0.f;
  for (int base = 0; base < Np; base += 32) {
    const int j = base + lane;
    const float v = (j < Np) ? diff[j] : 0.f;
    const float incl = warp_inclusive_scan(v, lane) + carry;
    if (j < Np) gprop[r * Np + j] = incl;
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
}

// ---------------------------------------------------------------------------------
static int launch_prop_fwd_tc(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                              const SamplerArgs& s, const float* edges, const float* jitter, float* delta,
                              const PropMlp& mlp, cudaStream_t st);

int launch_prop_features(const FieldView& f, const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                         const float* edges, const float* jitter, float* X, float* delta, const PropMlp* mlp,
                         cudaStream_t st) {
  const int64_t n = R * s.N;
  if (n == 0) return TVM_OK;
  if (f.dtype == TVM_BF16 && mlp && mlp->units == 64 && !X && !mlp->H && mlp->sigma)
    return launch_prop_fwd_tc(f, origins, dirs, R, s, edges, jitter, delta, *mlp, st);  // BF16: tensor cores
  const unsigned blocks = (unsigned)ceil_div(n, 128 * PROP_SPT);  // 128 threads, PROP_SPT samples each
  const int units = mlp ? mlp->units : 0;
  const size_t smem = mlp ? (size_t)18 * units * sizeof(float) : 0;
  const float *w1 = mlp ? mlp->w1 : nullptr, *b1 = mlp ? mlp->b1 : nullptr, *w2 = mlp ? mlp->w2 : nullptr,
              *b2 = mlp ? mlp->b2 : nullptr;
  float* H = mlp ? mlp->H : nullptr;
  float* sig = mlp ? mlp->sigma : nullptr;
  const float shift = mlp ? mlp->shift : 0.f;
  if (f.dtype == TVM_BF16)
    prop_features_kernel<__nv_bfloat16><<<blocks, 128, smem, st>>>(
        (const __nv_bfloat16*)f.lines, (const __nv_bfloat16*)f.planes, f.G, origins, dirs, R, s, edges, jitter, X,
        delta, units, w1, b1, w2, b2, shift, H, sig);
  else
    prop_features_kernel<float><<<blocks, 128, smem, st>>>((const float*)f.lines, (const float*)f.planes, f.G, origins,
                                                           dirs, R, s, edges, jitter, X, delta, units, w1, b1, w2, b2,
                                                           shift, H, sig);
  return check_launch("prop_features");
}

// ---------------------------------------------------------------------------------
// Tensor-core proposal backward for BF16 models with 64 hidden units. Persistent CTAs
// of 128 threads, one 128-sample tile at a time (thread = sample = TMEM lane):
//   gather X (16, bf16 A tile)            -> MMA  H = X W1              (TMEM, 64 cols)
//   h = relu(H + b1), dh = dz w2 [h > 0]  -> bf16 tiles H, dH (units padded to 128)
//   MMA dX = dH W1^T (16 cols) | dW1^T += dH^T X | [dW2, db1] += H^T [dz, 0] + dH^T [0, 1]
//   dX[0:12) -> float4 scatter into the proposal field gradients.
// The weight-gradient products contract over the tile's samples and read the H / dH /
// X / Z tiles as MN-major operands. They accumulate in TMEM across the CTA's tiles and
// reach global memory once per CTA. bf16 operands, fp32 accumulation: the BF16 mode's
// arithmetic.
// ---------------------------------------------------------------------------------
static __device__ int g_prop_status;  // sticky: bit 0 = a bounded tensor-core wait gave up

namespace ptc {

constexpr int THREADS = 128;
constexpr int U = 64;
constexpr uint32_t WAIT_LIMIT = 1u << 24;
// Shared-memory map (bytes). Tiles are [rows][width] bf16, K-major canonical, SBO =
// (width / 8) * 128.
constexpr int SBO_16 = 256, SBO_128 = 2048;
constexpr int OFF_W1 = 0;                       // [64 units][16 inputs]: 2 KB
constexpr int OFF_X = OFF_W1 + U * 16 * 2;      // [128][16]
constexpr int OFF_Z1 = OFF_X + 128 * 16 * 2;    // [128][16], column 0 = dz
constexpr int OFF_Z2 = OFF_Z1 + 128 * 16 * 2;   // [128][16], column 1 = 1
constexpr int OFF_H = OFF_Z2 + 128 * 16 * 2;    // [128][128], columns 64.. stay 0
constexpr int OFF_DH = OFF_H + 128 * 128 * 2;   // [128][128], columns 64.. stay 0
constexpr int OFF_BAR = OFF_DH + 128 * 128 * 2;
constexpr int SMEM = OFF_BAR + 64;              // ~78 KB: at most 2 CTAs per SM, 2 x 128 TMEM columns
// TMEM columns.
constexpr uint32_t T_H = 0, T_DX = 64, T_W1 = 80, T_W2 = 96, NCOLS = 128;

__device__ __forceinline__ int coff(int row, int kchunk, int sbo) { return (row >> 3) * sbo + kchunk * 128 + (row & 7) * 16; }
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
struct Op {
  uint32_t addr, lbo, sbo, step;
};
__device__ __forceinline__ Op kmaj(uint32_t addr, uint32_t sbo) { return Op{addr, 128u, sbo, 256u}; }
// MN-major view of a natural tile whose rows are the K index (LBO = K-direction core
// stride, SBO = MN-direction core stride, no swizzle).
__device__ __forceinline__ Op mnmaj(uint32_t addr, uint32_t row_group_stride) {
  return Op{addr, row_group_stride, 128u, 2u * row_group_stride};
}
__host__ __device__ constexpr uint32_t idesc_t(int M, int N, bool a_mn, bool b_mn) {
  return tc::idesc(M, N, 1u) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}
__device__ __forceinline__ void mma_run(uint32_t d, Op a, Op b, int ksteps, uint32_t idesc, bool accumulate) {
#pragma unroll 1
  for (int s = 0; s < ksteps; ++s) {
    tc::mma_bf16(d, tc::sdesc(a.addr + s * a.step, a.lbo, a.sbo), tc::sdesc(b.addr + s * b.step, b.lbo, b.sbo),
                 idesc, (accumulate || s > 0) ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(THREADS) prop_bwd_tc_kernel(
    const __nv_bfloat16* __restrict__ lines, const __nv_bfloat16* __restrict__ planes, int G,
    float* __restrict__ glines, float* __restrict__ gplanes, const float* __restrict__ origins,
    const float* __restrict__ dirs, int64_t R, SamplerArgs s, const float* __restrict__ edges,
    const float* __restrict__ jitter, const float* __restrict__ dz_in, const float* __restrict__ sig_in,
    const float* __restrict__ w1, const float* __restrict__ b1, const float* __restrict__ w2, float* __restrict__ gw1, float* __restrict__ gb1,
    float* __restrict__ gw2, float* __restrict__ gb2) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + OFF_BAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  if (warp == 0) tc::tmem_alloc(tslot, NCOLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  // W1 image (B operand [unit][input]), constant columns of Z2, zero halves of H / dH.
  for (int c = tid; c < U * 2; c += THREADS) {
    const int u = c >> 1, kc = c & 1;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = __ldg(w1 + (kc * 8 + e) * U + u);
    *reinterpret_cast<uint4*>(smem + OFF_W1 + coff(u, kc, SBO_16)) =
        make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
  }
  {
    const int r = tid;
    *reinterpret_cast<uint4*>(smem + OFF_Z2 + coff(r, 0, SBO_16)) = make_uint4(pack2(0.f, 1.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(smem + OFF_Z2 + coff(r, 1, SBO_16)) = make_uint4(0u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(smem + OFF_Z1 + coff(r, 1, SBO_16)) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int kc = 8; kc < 16; ++kc) {
      *reinterpret_cast<uint4*>(smem + OFF_H + coff(r, kc, SBO_128)) = make_uint4(0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4*>(smem + OFF_DH + coff(r, kc, SBO_128)) = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t sb = tc::smem_u32(smem);
  uint32_t phase = 0;
  int ok = 1;
  bool first = true;
  float db2 = 0.f;
  auto run = [&](auto&& issue_fn) -> bool {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      issue_fn();
      tc::mma_commit(mbar);
    }
    const int done = tc::mbar_wait(mbar, phase, WAIT_LIMIT) ? 1 : 0;
    phase ^= 1u;
    const int all = __syncthreads_and(done);
    tc::fence_after_sync();
    return all != 0;
  };

  const int Np = s.N;
  const int64_t nsmp = R * Np;
  const int64_t ntiles = (nsmp + THREADS - 1) / THREADS;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t smp = tile * THREADS + tid;
    const bool valid = smp < nsmp;
    const float dz = valid ? load_dz(dz_in, sig_in, smp) : 0.f;
    db2 += dz;
    // A sample with dz = 0 adds nothing to any gradient (its dH row is zero): it keeps a
    // zero row in the tile and skips its gathers and scatter.
    const bool live = valid && dz != 0.f;
    float X[PROP_IN];
#pragma unroll
    for (int i = 0; i < PROP_IN; ++i) X[i] = 0.f;
    PropPair e3[3];
    if (live) {
      const int64_t r = smp / Np;
      const int j = (int)(smp - r * Np);
      RayGeom g = load_ray(origins, dirs, r, s);
      float t, len, x[3];
      prop_sample(g, s, edges, Np, jitter, r, j, t, len, x);
      float u3[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) u3[a] = grid_coord(x[a], G);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        int a, b, c;
        mode_perm(m, a, b, c);
        prop_pair<__nv_bfloat16>(lines, planes, G, m, u3[a], u3[b], u3[c], e3[m]);
#pragma unroll
        for (int q = 0; q < 4; ++q) X[m * 4 + q] = e3[m].L[q] * e3[m].P[q];
      }
      X[12] = x[0];
      X[13] = x[1];
      X[14] = x[2];
      X[15] = fmaxf(fabsf(x[0]), fmaxf(fabsf(x[1]), fabsf(x[2])));
    }
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
      *reinterpret_cast<uint4*>(smem + OFF_X + coff(tid, kc, SBO_16)) =
          make_uint4(pack2(X[8 * kc], X[8 * kc + 1]), pack2(X[8 * kc + 2], X[8 * kc + 3]),
                     pack2(X[8 * kc + 4], X[8 * kc + 5]), pack2(X[8 * kc + 6], X[8 * kc + 7]));
    }
    *reinterpret_cast<uint4*>(smem + OFF_Z1 + coff(tid, 0, SBO_16)) = make_uint4(pack2(dz, 0.f), 0u, 0u, 0u);
    // H = X W1.
    if (!run([&] { mma_run(tmem + T_H, kmaj(sb + OFF_X, SBO_16), kmaj(sb + OFF_W1, SBO_16), 1,
                           idesc_t(128, U, false, false), false); })) { ok = 0; break; }
#pragma unroll
    for (int ch = 0; ch < U / 16; ++ch) {
      float v[16];
      tc::tmem_ld16(tmem + T_H + lane_off + ch * 16, v);
      float dh[16];
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int u = ch * 16 + e;
        v[e] = fmaxf(v[e] + __ldg(b1 + u), 0.f);
        dh[e] = v[e] > 0.f ? dz * __ldg(w2 + u) : 0.f;
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        *reinterpret_cast<uint4*>(smem + OFF_H + coff(tid, ch * 2 + q, SBO_128)) =
            make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                       pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
        *reinterpret_cast<uint4*>(smem + OFF_DH + coff(tid, ch * 2 + q, SBO_128)) =
            make_uint4(pack2(dh[8 * q], dh[8 * q + 1]), pack2(dh[8 * q + 2], dh[8 * q + 3]),
                       pack2(dh[8 * q + 4], dh[8 * q + 5]), pack2(dh[8 * q + 6], dh[8 * q + 7]));
      }
    }
    // dX = dH W1^T; dW1^T += dH^T X; [dW2, db1] += H^T Z1 + dH^T Z2.
    if (!run([&] {
          mma_run(tmem + T_DX, kmaj(sb + OFF_DH, SBO_128), mnmaj(sb + OFF_W1, SBO_16), U / 16,
                  idesc_t(128, 16, false, true), false);
          mma_run(tmem + T_W1, mnmaj(sb + OFF_DH, SBO_128), mnmaj(sb + OFF_X, SBO_16), THREADS / 16,
                  idesc_t(128, 16, true, true), !first);
          mma_run(tmem + T_W2, mnmaj(sb + OFF_H, SBO_128), mnmaj(sb + OFF_Z1, SBO_16), THREADS / 16,
                  idesc_t(128, 16, true, true), !first);
          mma_run(tmem + T_W2, mnmaj(sb + OFF_DH, SBO_128), mnmaj(sb + OFF_Z2, SBO_16), THREADS / 16,
                  idesc_t(128, 16, true, true), true);
        })) { ok = 0; break; }
    float dX[16];
    tc::tmem_ld16(tmem + T_DX + lane_off, dX);
    bool any = false;
#pragma unroll
    for (int q = 0; q < 12; ++q) any |= (dX[q] != 0.0f);
    if (live && any) {
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const PropPair& e = e3[m];
        float* lb = glines + (int64_t)m * G * PROP_C;
        float* pb = gplanes + (int64_t)m * G * G * PROP_C;
        float v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.P[q] * e.tl.w0;
        atomicAdd(reinterpret_cast<float4*>(lb + e.tl.i0 * PROP_C), make_float4(v[0], v[1], v[2], v[3]));
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.P[q] * e.tl.w1;
        atomicAdd(reinterpret_cast<float4*>(lb + e.tl.i1 * PROP_C), make_float4(v[0], v[1], v[2], v[3]));
        const float w[4] = {e.tr.w0 * e.tc.w0, e.tr.w0 * e.tc.w1, e.tr.w1 * e.tc.w0, e.tr.w1 * e.tc.w1};
        const int rows[4] = {e.tr.i0, e.tr.i0, e.tr.i1, e.tr.i1};
        const int cols[4] = {e.tc.i0, e.tc.i1, e.tc.i0, e.tc.i1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = dX[m * 4 + q] * e.L[q] * w[k];
          atomicAdd(reinterpret_cast<float4*>(pb + ((int64_t)rows[k] * G + cols[k]) * PROP_C),
                    make_float4(v[0], v[1], v[2], v[3]));
        }
      }
    }
    first = false;
  }
  if (ok && !first) {
    // TMEM lane u (< 64): dW1^T row u = dW1[:, u]; [dW2, db1] row u.
    float v[16];
    tc::tmem_ld16(tmem + T_W1 + lane_off, v);
    if (tid < U) {
#pragma unroll
      for (int i = 0; i < PROP_IN; ++i) atomicAdd(gw1 + i * U + tid, v[i]);
    }
    tc::tmem_ld16(tmem + T_W2 + lane_off, v);
    if (tid < U) {
      atomicAdd(gw2 + tid, v[0]);
      atomicAdd(gb1 + tid, v[1]);
    }
    float sdz = db2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sdz += __shfl_xor_sync(0xffffffffu, sdz, o);
    if ((tid & 31) == 0) atomicAdd(gb2, sdz);
  }
  if (!ok) {
    if (tid == 0) atomicOr(&g_prop_status, 1);
    tc::mbar_wait(mbar, phase ^ 1u, WAIT_LIMIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, NCOLS);
  }
}

// Tensor-core proposal forward for BF16 models with 64 hidden units. Persistent CTAs of
// 128 threads, one 128-sample tile at a time (thread = sample = TMEM lane): the 16
// features go to a bf16 A tile, one MMA gives H = X W1 (TMEM, 64 fp32 columns), and the
// epilogue forms z = b2 + sum_u relu(H_u + b1_u) w2_u and sigma = softplus(z + shift).
// X and W1 are the bf16 operands of the tensor-core backward, so the forward's hidden
// units are the ones the backward recomputes. A few KB of shared memory and 64 TMEM
// columns per CTA let four CTAs share an SM: some gather while others wait for their
// product.
constexpr int FWD_BAR = OFF_X + 128 * 16 * 2;  // W1 image and X tile, then the barrier
constexpr int FWD_SMEM = FWD_BAR + 64;
constexpr uint32_t FWD_NCOLS = 64;
constexpr int FWD_CTAS_PER_SM = 4;

__global__ void __launch_bounds__(THREADS) prop_fwd_tc_kernel(
    const __nv_bfloat16* __restrict__ lines, const __nv_bfloat16* __restrict__ planes, int G,
    const float* __restrict__ origins, const float* __restrict__ dirs, int64_t R, SamplerArgs s,
    const float* __restrict__ edges, const float* __restrict__ jitter, float* __restrict__ delta,
    const float* __restrict__ w1, const float* __restrict__ b1, const float* __restrict__ w2,
    const float* __restrict__ b2, float shift, float* __restrict__ sigma) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + FWD_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + FWD_BAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  if (warp == 0) tc::tmem_alloc(tslot, FWD_NCOLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  for (int c = tid; c < U * 2; c += THREADS) {  // W1 image (B operand [unit][input])
    const int u = c >> 1, kc = c & 1;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = __ldg(w1 + (kc * 8 + e) * U + u);
    *reinterpret_cast<uint4*>(smem + OFF_W1 + coff(u, kc, SBO_16)) =
        make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t sb = tc::smem_u32(smem);
  const float4* b14 = reinterpret_cast<const float4*>(b1);
  const float4* w24 = reinterpret_cast<const float4*>(w2);
  const float bias2 = __ldg(b2);
  uint32_t phase = 0;
  int ok = 1;
  const int64_t nsmp = R * s.N;
  const int64_t ntiles = (nsmp + THREADS - 1) / THREADS;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t smp = tile * THREADS + tid;
    const bool valid = smp < nsmp;
    float X[PROP_IN];
#pragma unroll
    for (int i = 0; i < PROP_IN; ++i) X[i] = 0.f;
    if (valid) {
      float len;
      prop_sample_features<__nv_bfloat16>(lines, planes, G, origins, dirs, s, edges, jitter, smp, X, len);
      delta[smp] = len;
    }
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
      *reinterpret_cast<uint4*>(smem + OFF_X + coff(tid, kc, SBO_16)) =
          make_uint4(pack2(X[8 * kc], X[8 * kc + 1]), pack2(X[8 * kc + 2], X[8 * kc + 3]),
                     pack2(X[8 * kc + 4], X[8 * kc + 5]), pack2(X[8 * kc + 6], X[8 * kc + 7]));
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      mma_run(tmem, kmaj(sb + OFF_X, SBO_16), kmaj(sb + OFF_W1, SBO_16), 1, idesc_t(128, U, false, false), false);
      tc::mma_commit(mbar);
    }
    const int done = tc::mbar_wait(mbar, phase, WAIT_LIMIT) ? 1 : 0;
    phase ^= 1u;
    if (!__syncthreads_and(done)) {
      ok = 0;
      break;
    }
    tc::fence_after_sync();
    float h[U];
    tc::tmem_ld64(tmem + lane_off, h);
    float z = bias2;
#pragma unroll
    for (int q = 0; q < U / 4; ++q) {
      const float4 b = __ldg(b14 + q), w = __ldg(w24 + q);
      z = fmaf(fmaxf(h[4 * q] + b.x, 0.f), w.x, z);
      z = fmaf(fmaxf(h[4 * q + 1] + b.y, 0.f), w.y, z);
      z = fmaf(fmaxf(h[4 * q + 2] + b.z, 0.f), w.z, z);
      z = fmaf(fmaxf(h[4 * q + 3] + b.w, 0.f), w.w, z);
    }
    if (valid) sigma[smp] = softplus_f(z + shift);
  }
  if (!ok) {
    if (tid == 0) atomicOr(&g_prop_status, 1);
    tc::mbar_wait(mbar, phase ^ 1u, WAIT_LIMIT);  // the product in flight, before TMEM is freed
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, FWD_NCOLS);
  }
}

}  // namespace ptc

static int launch_prop_fwd_tc(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                              const SamplerArgs& s, const float* edges, const float* jitter, float* delta,
                              const PropMlp& mlp, cudaStream_t st) {
  if (!aligned(mlp.b1, 16) || !aligned(mlp.w2, 16)) {
    set_error("proposal forward: b1 and w2 must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  const int64_t tiles = ceil_div(R * s.N, (int64_t)ptc::THREADS);
  const unsigned grid =
      (unsigned)std::min<int64_t>(tiles, (int64_t)ptc::FWD_CTAS_PER_SM * std::max(device_sms(), 1));
  ptc::prop_fwd_tc_kernel<<<grid, ptc::THREADS, ptc::FWD_SMEM, st>>>(
      (const __nv_bfloat16*)f.lines, (const __nv_bfloat16*)f.planes, f.G, origins, dirs, R, s, edges, jitter, delta,
      mlp.w1, mlp.b1, mlp.w2, mlp.b2, mlp.shift, mlp.sigma);
  return check_launch("prop_fwd_tc");
}

int prop_status(int32_t* out, cudaStream_t st) {
  int32_t v = 0;
  const int32_t zero = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_prop_status, sizeof(int32_t), 0, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(g_prop_status, &zero, sizeof(int32_t), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_error("prop_status: %s", cudaGetErrorString(e));
    return TVM_ERR_LAUNCH;
  }
  *out = v;
  return TVM_OK;
}

int launch_prop_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins, const float* dirs,
                    int64_t R, const SamplerArgs& s, const float* edges, const float* jitter, const float* dz,
                    const PropMlp& mlp, float* gw1, float* gb1, float* gw2, float* gb2, cudaStream_t st) {
  const int64_t n = R * s.N;
  if (n == 0) return TVM_OK;
  const int U = mlp.units;
  if (f.dtype == TVM_BF16 && U == ptc::U) {
    TVM_TRY(ensure_smem_limit((const void*)ptc::prop_bwd_tc_kernel, ptc::SMEM, "proposal backward"));
    const int sms = device_sms();
    const int64_t tiles = ceil_div(n, ptc::THREADS);
    // One CTA per SM although two fit: the kernel runs beside the main field's backward on
    // a side stream, and the room it leaves there is worth more than its own speed
    // (same-box A/B of the proposal step: -2 us).
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, std::max(sms, 1));
    ptc::prop_bwd_tc_kernel<<<grid, ptc::THREADS, ptc::SMEM, st>>>(
        (const __nv_bfloat16*)f.lines, (const __nv_bfloat16*)f.planes, f.G, glines, gplanes, origins, dirs, R, s, edges,
        jitter, dz, mlp.sigma_in, mlp.w1, mlp.b1, mlp.w2, gw1, gb1, gw2, gb2);
    return check_launch("prop_bwd_tc");
  }
  const size_t smem = ((size_t)18 * U + PBWD_THREADS * 16 + 2 * PBWD_THREADS * (U + 4) + PBWD_THREADS) * sizeof(float);
  const unsigned blocks = (unsigned)ceil_div(n, PBWD_THREADS);
  if (f.dtype == TVM_BF16) {
    auto fn = prop_bwd_kernel<__nv_bfloat16>;
    TVM_TRY(ensure_smem_limit((const void*)fn, (int)smem, "proposal backward"));
    fn<<<blocks, PBWD_THREADS, smem, st>>>((const __nv_bfloat16*)f.lines, (const __nv_bfloat16*)f.planes, f.G, glines,
                                           gplanes, origins, dirs, R, s, edges, jitter, dz, mlp.sigma_in, U, mlp.w1, mlp.b1, mlp.w2,
                                           gw1, gb1, gw2, gb2);
  } else {
    auto fn = prop_bwd_kernel<float>;
    TVM_TRY(ensure_smem_limit((const void*)fn, (int)smem, "proposal backward"));
    fn<<<blocks, PBWD_THREADS, smem, st>>>((const float*)f.lines, (const float*)f.planes, f.G, glines, gplanes,
                                           origins, dirs, R, s, edges, jitter, dz, mlp.sigma_in, U, mlp.w1, mlp.b1,
                                           mlp.w2, gw1, gb1, gw2, gb2);
  }
  return check_launch("prop_bwd");
}

int launch_resample(const float* wprop, const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                    const float* edges, int Nm, const float* jitter, float* t_out, float* d_out, int32_t* bins,
                    cudaStream_t st, const float* sig, const float* len, float* w_out) {
  if (R == 0) return TVM_OK;
  const int warps = 4;
  const size_t smem = (size_t)warps * (2 * (s.N + 1) + (Nm + 1)) * sizeof(float);
  const unsigned grid = (unsigned)ceil_div(R, warps);
  if (sig)
    resample_kernel<true><<<grid, warps * 32, smem, st>>>(w_out, sig, len, origins, dirs, R, s, edges, Nm, jitter, t_out,
                                                          d_out, bins);
  else
    resample_kernel<false><<<grid, warps * 32, smem, st>>>(const_cast<float*>(wprop), nullptr, nullptr, origins, dirs,
                                                           R, s, edges, Nm, jitter, t_out, d_out, bins);
  return check_launch("resample");
}

int launch_prop_loss(const float* wmain, const float* wprop, const int32_t* bins, int64_t R, int Np, int Nm,
                     float scale, float* loss, float* gprop, cudaStream_t st) {
  if (R == 0) return TVM_OK;
  const int warps = 8;
  const size_t smem = (size_t)warps * 2 * (Np + 2) * sizeof(float);
  prop_loss_kernel<<<(unsigned)ceil_div(R, warps), warps * 32, smem, st>>>(wmain, wprop, bins, R, Np, Nm, scale, loss,
                                                                           gprop);
  return check_launch("prop_loss");
}

}  // namespace tvm
