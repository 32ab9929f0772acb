// VM (vector-matrix) feature evaluation and its backward scatter.
//
// Reference: TensorVM.interpolate / TensorVMSingle.interpolate /
// linear_interpolation_with_channel_axis (tensorf/tensor_vm.py:42-89, 140-167,
// 226-250). Pair m of a tensor contributes feat[m*C + c] = line_m[c](u_a) *
// plane_m[c](u_b, u_c): a linear lookup along one axis times a bilinear lookup on the
// other two, with map_coordinates(order=1, mode="nearest") semantics.
//
// GB300 mapping: fields live channel-last ([G][C] rows per line, [G][G][C] per plane)
// so every tap of a sample is C contiguous elements. Four lanes (a quad) own one
// sample; lane q reads channels [q*C/4, (q+1)*C/4) of every tap with 16-byte vector
// loads (float4, or uint4/uint2 of bf16), so a quad fetches whole 32-byte sectors and
// a warp keeps 8 samples -- 144 independent 16-byte loads for density -- in flight.
// The fields (17 MB density + 52 MB appearance in FP32 at G=300) stay resident in
// the 126 MB L2; the kernels are bound by L2 gather bandwidth. Gradients go back with
// 16-byte vector reductions (float4 atomicAdd, sm_90+) into FP32 buffers with the same
// channel-last layout, so a quad's reduction covers whole sectors too.
#include "tvm_internal.h"

namespace tvm {

template <typename T, int CPL>
struct PairEval {
  Tap tl, tr, tc;
  float L[CPL], P[CPL];
};

// Evaluate pair m at grid coordinates (ul; ur, uc) for channels [ch0, ch0+CPL).
template <typename T, int CPL>
__device__ __forceinline__ void vm_pair_eval(const T* __restrict__ lines, const T* __restrict__ planes,
                                             int G, int C, int m, float ul, float ur, float uc,
                                             int ch0, PairEval<T, CPL>& e) {
  e.tl = make_tap(ul, G);
  e.tr = make_tap(ur, G);
  e.tc = make_tap(uc, G);
  const T* lb = lines + (int64_t)m * G * C + ch0;
  const T* pb = planes + (int64_t)m * G * G * C + ch0;
  float l0[CPL], l1[CPL], p00[CPL], p01[CPL], p10[CPL], p11[CPL];
  load_chunk<CPL>(lb + (int64_t)e.tl.i0 * C, l0);
  load_chunk<CPL>(lb + (int64_t)e.tl.i1 * C, l1);
  load_chunk<CPL>(pb + ((int64_t)e.tr.i0 * G + e.tc.i0) * C, p00);
  load_chunk<CPL>(pb + ((int64_t)e.tr.i0 * G + e.tc.i1) * C, p01);
  load_chunk<CPL>(pb + ((int64_t)e.tr.i1 * G + e.tc.i0) * C, p10);
  load_chunk<CPL>(pb + ((int64_t)e.tr.i1 * G + e.tc.i1) * C, p11);
  // Corner weights are (row weight) * (column weight), summed in the corner order of
  // jax's itertools.product loop: (0,0), (0,1), (1,0), (1,1).
  const float w00 = e.tr.w0 * e.tc.w0, w01 = e.tr.w0 * e.tc.w1;
  const float w10 = e.tr.w1 * e.tc.w0, w11 = e.tr.w1 * e.tc.w1;
#pragma unroll
  for (int j = 0; j < CPL; ++j) {
    e.L[j] = e.tl.w0 * l0[j] + e.tl.w1 * l1[j];
    e.P[j] = w00 * p00[j] + w01 * p01[j] + w10 * p10[j] + w11 * p11[j];
  }
}

// Scatter the gradient of pair m: d line tap += g * w_tap * P, d plane corner +=
// g * w_corner * L (per channel g).
template <typename T, int CPL>
__device__ __forceinline__ void vm_pair_scatter(float* __restrict__ glines, float* __restrict__ gplanes,
                                                int G, int C, int m, int ch0,
                                                const PairEval<T, CPL>& e, const float (&g)[CPL]) {
  float* lb = glines + (int64_t)m * G * C + ch0;
  float* pb = gplanes + (int64_t)m * G * G * C + ch0;
  float gl[CPL], gp[CPL];
#pragma unroll
  for (int j = 0; j < CPL; ++j) gl[j] = g[j] * e.P[j] * e.tl.w0;
  red_chunk<CPL>(lb + (int64_t)e.tl.i0 * C, gl);
#pragma unroll
  for (int j = 0; j < CPL; ++j) gl[j] = g[j] * e.P[j] * e.tl.w1;
  red_chunk<CPL>(lb + (int64_t)e.tl.i1 * C, gl);
  const float w[4] = {e.tr.w0 * e.tc.w0, e.tr.w0 * e.tc.w1, e.tr.w1 * e.tc.w0, e.tr.w1 * e.tc.w1};
  const int rows[4] = {e.tr.i0, e.tr.i0, e.tr.i1, e.tr.i1};
  const int cols[4] = {e.tc.i0, e.tc.i1, e.tc.i0, e.tc.i1};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int j = 0; j < CPL; ++j) gp[j] = g[j] * e.L[j] * w[q];
    red_chunk<CPL>(pb + ((int64_t)rows[q] * G + cols[q]) * C, gp);
  }
}

// One tap slot's reductions for the 8 samples (quads) of a warp. Along a ray every tap
// index is monotone, so quads of consecutive samples that land on the same texel form a
// contiguous run: the run's values are summed in registers (a segmented reduction over
// quads with shuffles of 4, 8 and 16 lanes) and its first quad issues one reduction.
// key: the texel (>= 0), or -1 for a quad with nothing to add. All 32 lanes call this.
template <int CPL>
__device__ __forceinline__ void warp_red_chunk(float* __restrict__ base, int key, int C, float (&v)[CPL]) {
  const unsigned lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(0xffffffffu, key, 4);  // the previous quad's key, same channels
  const bool head = lane < 4 || prev != key;
  const unsigned heads = __ballot_sync(0xffffffffu, head) & 0x11111111u;  // one bit per quad
  if (heads != 0x11111111u) {  // some quad continues a run (the same for the whole warp)
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
      float u[CPL];
#pragma unroll
      for (int j = 0; j < CPL; ++j) u[j] = __shfl_down_sync(0xffffffffu, v[j], o);
      // lane + o belongs to this run when no quad in (lane, lane + o] starts a run
      if (lane + o < 32 && ((heads >> (lane + 1)) & ((1u << o) - 1u)) == 0u) {
#pragma unroll
        for (int j = 0; j < CPL; ++j) v[j] += u[j];
      }
    }
  }
  if (head && key >= 0) red_chunk<CPL>(base + (int64_t)key * C, v);
}

// vm_pair_scatter for the consecutive samples of a warp, each tap slot merged over the
// warp's quads (warp_red_chunk). active: this quad's sample has a gradient to add.
template <typename T, int CPL>
__device__ __forceinline__ void vm_pair_scatter_warp(float* __restrict__ glines, float* __restrict__ gplanes,
                                                     int G, int C, int m, int ch0, bool active,
                                                     const PairEval<T, CPL>& e, const float (&g)[CPL]) {
  float* lb = glines + (int64_t)m * G * C + ch0;
  float* pb = gplanes + (int64_t)m * G * G * C + ch0;
  float v[CPL];
#pragma unroll
  for (int j = 0; j < CPL; ++j) v[j] = g[j] * e.P[j] * e.tl.w0;
  warp_red_chunk<CPL>(lb, active ? e.tl.i0 : -1, C, v);
#pragma unroll
  for (int j = 0; j < CPL; ++j) v[j] = g[j] * e.P[j] * e.tl.w1;
  warp_red_chunk<CPL>(lb, active ? e.tl.i1 : -1, C, v);
  const float w[4] = {e.tr.w0 * e.tc.w0, e.tr.w0 * e.tc.w1, e.tr.w1 * e.tc.w0, e.tr.w1 * e.tc.w1};
  const int rows[4] = {e.tr.i0, e.tr.i0, e.tr.i1, e.tr.i1};
  const int cols[4] = {e.tc.i0, e.tc.i1, e.tc.i0, e.tc.i1};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int j = 0; j < CPL; ++j) v[j] = g[j] * e.L[j] * w[q];
    warp_red_chunk<CPL>(pb, active ? rows[q] * G + cols[q] : -1, C, v);
  }
}

// Scatter of two samples' gradients for pair m (sample b optional): b's taps that land
// on one of a's taps are added into a's values first, so a texel shared by consecutive
// samples of a ray gets one reduction instead of two. (Consecutive samples of a ray are
// less than one voxel apart at the configured sample counts, so most of their taps
// coincide.)
template <typename T, int CPL>
__device__ __forceinline__ void vm_pair_scatter2(float* __restrict__ glines, float* __restrict__ gplanes, int G,
                                                 int C, int m, int ch0, const PairEval<T, CPL>& a,
                                                 const float (&ga)[CPL], bool has_b, const PairEval<T, CPL>& b,
                                                 const float (&gb)[CPL]) {
  float* lb = glines + (int64_t)m * G * C + ch0;
  float* pb = gplanes + (int64_t)m * G * G * C + ch0;
  float l0[CPL], l1[CPL];
#pragma unroll
  for (int j = 0; j < CPL; ++j) {
    l0[j] = ga[j] * a.P[j] * a.tl.w0;
    l1[j] = ga[j] * a.P[j] * a.tl.w1;
  }
  const float wa[4] = {a.tr.w0 * a.tc.w0, a.tr.w0 * a.tc.w1, a.tr.w1 * a.tc.w0, a.tr.w1 * a.tc.w1};
  const int ra[4] = {a.tr.i0, a.tr.i0, a.tr.i1, a.tr.i1};
  const int ca[4] = {a.tc.i0, a.tc.i1, a.tc.i0, a.tc.i1};
  float pv[4][CPL];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int j = 0; j < CPL; ++j) pv[q][j] = ga[j] * a.L[j] * wa[q];
  }
  if (has_b) {
    const int lidx[2] = {b.tl.i0, b.tl.i1};
    const float lw[2] = {b.tl.w0, b.tl.w1};
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      float v[CPL];
#pragma unroll
      for (int j = 0; j < CPL; ++j) v[j] = gb[j] * b.P[j] * lw[t];
      if (lidx[t] == a.tl.i0) {
#pragma unroll
        for (int j = 0; j < CPL; ++j) l0[j] += v[j];
      } else if (lidx[t] == a.tl.i1) {
#pragma unroll
        for (int j = 0; j < CPL; ++j) l1[j] += v[j];
      } else {
        red_chunk<CPL>(lb + (int64_t)lidx[t] * C, v);
      }
    }
    const float wb[4] = {b.tr.w0 * b.tc.w0, b.tr.w0 * b.tc.w1, b.tr.w1 * b.tc.w0, b.tr.w1 * b.tc.w1};
    const int rb[4] = {b.tr.i0, b.tr.i0, b.tr.i1, b.tr.i1};
    const int cb[4] = {b.tc.i0, b.tc.i1, b.tc.i0, b.tc.i1};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      float v[CPL];
#pragma unroll
      for (int j = 0; j < CPL; ++j) v[j] = gb[j] * b.L[j] * wb[t];
      int hit = -1;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (hit < 0 && rb[t] == ra[q] && cb[t] == ca[q]) hit = q;
      if (hit >= 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q == hit) {
#pragma unroll
            for (int j = 0; j < CPL; ++j) pv[q][j] += v[j];
          }
        }
      } else {
        red_chunk<CPL>(pb + ((int64_t)rb[t] * G + cb[t]) * C, v);
      }
    }
  }
  red_chunk<CPL>(lb + (int64_t)a.tl.i0 * C, l0);
  red_chunk<CPL>(lb + (int64_t)a.tl.i1 * C, l1);
#pragma unroll
  for (int q = 0; q < 4; ++q) red_chunk<CPL>(pb + ((int64_t)ra[q] * G + ca[q]) * C, pv[q]);
}

__device__ __forceinline__ unsigned quad_mask() { return 0xFu << (threadIdx.x & 28); }

__device__ __forceinline__ float quad_sum(float v) {
  const unsigned qm = quad_mask();
  v += __shfl_xor_sync(qm, v, 1);
  v += __shfl_xor_sync(qm, v, 2);
  return v;
}

// ---------------------------------------------------------------------------------
// Seam: TensorVM.interpolate with explicit coordinates.
// ---------------------------------------------------------------------------------
template <typename T, int C>
__global__ void __launch_bounds__(256) vm_features_fwd_kernel(const T* __restrict__ lines,
                                                             const T* __restrict__ planes, int G,
                                                             const float* __restrict__ coords,
                                                             int64_t n, float* __restrict__ out) {
  constexpr int CPL = C / 4;
  const int64_t smp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  if (smp >= n) return;
  float u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = grid_coord(__ldg(coords + a * n + smp), G);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> e;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
#pragma unroll
    for (int j = 0; j < CPL; ++j) out[(int64_t)(m * C + sub * CPL + j) * n + smp] = e.L[j] * e.P[j];
  }
}

template <typename T, int C>
__global__ void __launch_bounds__(256) vm_features_bwd_kernel(const T* __restrict__ lines,
                                                             const T* __restrict__ planes, int G,
                                                             const float* __restrict__ coords,
                                                             int64_t n, const float* __restrict__ gout,
                                                             float* __restrict__ glines,
                                                             float* __restrict__ gplanes) {
  constexpr int CPL = C / 4;
  const int64_t smp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  if (smp >= n) return;
  float u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = grid_coord(__ldg(coords + a * n + smp), G);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> e;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
    float g[CPL];
#pragma unroll
    for (int j = 0; j < CPL; ++j) g[j] = __ldg(gout + (int64_t)(m * C + sub * CPL + j) * n + smp);
    vm_pair_scatter<T, CPL>(glines, gplanes, G, C, m, sub * CPL, e, g);
  }
}

// ---------------------------------------------------------------------------------
// Fused density: sampler -> density VM -> sum -> softplus (render.py:177-207).
// ---------------------------------------------------------------------------------
template <typename T, int C>
__global__ void __launch_bounds__(256) density_fwd_kernel(const T* __restrict__ lines,
                                                         const T* __restrict__ planes, int G,
                                                         float shift,
                                                         const float* __restrict__ origins,
                                                         const float* __restrict__ dirs,
                                                         int64_t total, SamplerArgs s,
                                                         float* __restrict__ sigma) {
  constexpr int CPL = C / 4;
  const int64_t smp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  if (smp >= total) return;
  const int64_t r = smp / s.N;
  const int i = (int)(smp - r * s.N);
  RayGeom g = load_ray(origins, dirs, r, s);
  float t, delta, x[3], u[3];
  sample_t(g, s, r, i, t, delta);
  sample_point(g, s, t, x);
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = grid_coord(x[a], G);
  float acc = 0.f;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> e;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
#pragma unroll
    for (int j = 0; j < CPL; ++j) acc += e.L[j] * e.P[j];
  }
  acc = quad_sum(acc);
  if (sub == 0) sigma[smp] = softplus_f(acc + shift);
}

template <typename T, int C>
__global__ void __launch_bounds__(256) density_bwd_kernel(const T* __restrict__ lines,
                                                         const T* __restrict__ planes, int G,
                                                         float* __restrict__ glines,
                                                         float* __restrict__ gplanes,
                                                         const float* __restrict__ origins,
                                                         const float* __restrict__ dirs,
                                                         int64_t total, SamplerArgs s,
                                                         const float* __restrict__ gsum) {
  // The warp's 8 samples are consecutive along a ray: their reductions are merged per
  // texel (vm_pair_scatter_warp), so every lane stays to the end.
  constexpr int CPL = C / 4;
  const int64_t smp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  const float gs = smp < total ? __ldg(gsum + smp) : 0.0f;
  const bool active = gs != 0.0f;
  if (__all_sync(0xffffffffu, !active)) return;  // nothing to scatter in this warp
  float u[3] = {0.f, 0.f, 0.f};
  if (active) {
    const int64_t r = smp / s.N;
    const int i = (int)(smp - r * s.N);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = grid_coord(x[a], G);
  }
  float gv[CPL];
#pragma unroll
  for (int j = 0; j < CPL; ++j) gv[j] = gs;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> e;
    if (active) {
      vm_pair_eval<T, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
    } else {
      e = PairEval<T, CPL>{};
    }
    vm_pair_scatter_warp<T, CPL>(glines, gplanes, G, C, m, sub * CPL, active, e, gv);
  }
}

template <typename T, int C>
__global__ void __launch_bounds__(256, 3) density_bwd2_kernel(const T* __restrict__ lines,
                                                         const T* __restrict__ planes, int G,
                                                         float* __restrict__ glines,
                                                         float* __restrict__ gplanes,
                                                         const float* __restrict__ origins,
                                                         const float* __restrict__ dirs,
                                                         int64_t total, SamplerArgs s,
                                                         const float* __restrict__ gsum) {
  // A quad owns samples 2p and 2p + 1 (consecutive along a ray unless 2p + 1 starts the
  // next ray, which is still correct, only merges less). Capped at 80 registers for
  // three resident blocks: the kernel waits on gathers, and the few spills cost less.
  constexpr int CPL = C / 4;
  const int64_t pair = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  const int64_t sa = 2 * pair, sbi = sa + 1;
  if (sa >= total) return;
  const float gsa = __ldg(gsum + sa);
  const float gsb = sbi < total ? __ldg(gsum + sbi) : 0.0f;
  if (gsa == 0.0f && gsb == 0.0f) return;  // the whole quad agrees: nothing to scatter
  float ua[3], ub[3];
  {
    const int64_t r = sa / s.N;
    const int i = (int)(sa - r * s.N);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) ua[a] = grid_coord(x[a], G);
  }
  const bool has_b = gsb != 0.0f;
  if (has_b) {
    const int64_t r = sbi / s.N;
    const int i = (int)(sbi - r * s.N);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) ub[a] = grid_coord(x[a], G);
  }
  float ga[CPL], gb[CPL];
#pragma unroll
  for (int j = 0; j < CPL; ++j) {
    ga[j] = gsa;
    gb[j] = gsb;
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> ea, eb;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, ua[a], ua[b], ua[c], sub * CPL, ea);
    if (has_b) vm_pair_eval<T, CPL>(lines, planes, G, C, m, ub[a], ub[b], ub[c], sub * CPL, eb);
    vm_pair_scatter2<T, CPL>(glines, gplanes, G, C, m, sub * CPL, ea, ga, has_b, eb, gb);
  }
}

// ---------------------------------------------------------------------------------
// Fused appearance gather for the selected samples (render.py:472-486): row
// m = r*k + j uses sample sel_idx[m] of ray r; X0[m] = 3C features, mode-major.
// ---------------------------------------------------------------------------------
template <typename T, int C>
__global__ void __launch_bounds__(256) appearance_fwd_kernel(const T* __restrict__ lines,
                                                            const T* __restrict__ planes, int G,
                                                            const float* __restrict__ origins,
                                                            const float* __restrict__ dirs,
                                                            int64_t rows, int k, SamplerArgs s,
                                                            const int32_t* __restrict__ sel_idx,
                                                            float* __restrict__ X0) {
  constexpr int CPL = C / 4;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  if (row >= rows) return;
  const int64_t r = row / k;
  const int i = __ldg(sel_idx + row);
  RayGeom g = load_ray(origins, dirs, r, s);
  float t, delta, x[3], u[3];
  sample_t(g, s, r, i, t, delta);
  sample_point(g, s, t, x);
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = grid_coord(x[a], G);
  float* dst = X0 + row * (3 * C) + sub * CPL;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> e;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
    float v[CPL];
#pragma unroll
    for (int j = 0; j < CPL; ++j) v[j] = e.L[j] * e.P[j];
    store_streaming<CPL>(dst + m * C, v);
  }
}

// The same features written as FeatureMlp input tiles (bf16, 48 channels per pair): lane
// sub of a row's quad holds channels [12 sub, 12 sub + 12) of every pair, stored as three
// 8-byte pieces at their canonical positions. The quads of the padded rows past the last
// selected sample write zeros, so a tile is whole.
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

__global__ void __launch_bounds__(256) appearance_fwd_tiles_kernel(const __nv_bfloat16* __restrict__ lines,
                                                                  const __nv_bfloat16* __restrict__ planes, int G,
                                                                  const float* __restrict__ origins,
                                                                  const float* __restrict__ dirs, int64_t rows,
                                                                  int64_t rows_padded, int k, SamplerArgs s,
                                                                  const int32_t* __restrict__ sel_idx,
                                                                  uint8_t* __restrict__ X0t) {
  constexpr int C = 48, CPL = C / 4;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  if (row >= rows_padded) return;
  float v[3][CPL];
  if (row < rows) {
    const int64_t r = row / k;
    const int i = __ldg(sel_idx + row);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3], u[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = grid_coord(x[a], G);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      int a, b, c;
      mode_perm(m, a, b, c);
      PairEval<__nv_bfloat16, CPL> e;
      vm_pair_eval<__nv_bfloat16, CPL>(lines, planes, G, C, m, u[a], u[b], u[c], sub * CPL, e);
#pragma unroll
      for (int j = 0; j < CPL; ++j) v[m][j] = e.L[j] * e.P[j];
    }
  } else {
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int j = 0; j < CPL; ++j) v[m][j] = 0.f;
  }
  const int rr = (int)(row & (X0T_ROWS - 1));
  uint8_t* base = X0t + (row / X0T_ROWS) * X0T_TILE_BYTES + (rr >> 3) * X0T_SBO + (rr & 7) * 16;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
#pragma unroll
    for (int p = 0; p < CPL / 4; ++p) {
      const int kk = m * C + sub * CPL + 4 * p;  // a multiple of 4: half a K-chunk
      __stcs(reinterpret_cast<uint2*>(base + (kk >> 3) * 128 + (kk & 7) * 2),
             make_uint2(pack_bf16x2(v[m][4 * p], v[m][4 * p + 1]), pack_bf16x2(v[m][4 * p + 2], v[m][4 * p + 3])));
    }
  }
}

template <typename T, int C>
__global__ void __launch_bounds__(256) appearance_bwd_kernel(const T* __restrict__ lines,
                                                            const T* __restrict__ planes, int G,
                                                            float* __restrict__ glines,
                                                            float* __restrict__ gplanes,
                                                            const float* __restrict__ origins,
                                                            const float* __restrict__ dirs,
                                                            int64_t rows, int k, SamplerArgs s,
                                                            const int32_t* __restrict__ sel_idx,
                                                            const float* __restrict__ dX0) {
  // One quad per (pair m, row), pair-major: with few selected samples (k < 32) there are
  // few rows, and three quads per row keep three times as many warps in flight. A ray's
  // selected samples are consecutive rows in sample order, so a warp's 8 quads are mostly
  // neighbours along one ray for the same pair: their reductions are merged per texel
  // (vm_pair_scatter_warp), and every lane stays to the end.
  constexpr int CPL = C / 4;
  const int64_t quad = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  const int m = (int)(quad / rows < 3 ? quad / rows : 2);
  const int64_t row = quad - (int64_t)m * rows;
  const bool active = quad < 3 * rows;
  if (__all_sync(0xffffffffu, !active)) return;
  int a, b, c;
  mode_perm(m, a, b, c);
  PairEval<T, CPL> e;
  float gv[CPL];
  if (active) {
    const int64_t r = row / k;
    const int i = __ldg(sel_idx + row);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3], u[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int q = 0; q < 3; ++q) u[q] = grid_coord(x[q], G);
    // the pair's axes, selected without indexing the array by a runtime value
    auto pick = [&](int q) { return q == 0 ? u[0] : (q == 1 ? u[1] : u[2]); };
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, pick(a), pick(b), pick(c), sub * CPL, e);
    load_streaming<CPL>(dX0 + row * (3 * C) + m * C + sub * CPL, gv);
  } else {
    e = PairEval<T, CPL>{};
#pragma unroll
    for (int j = 0; j < CPL; ++j) gv[j] = 0.0f;
  }
  vm_pair_scatter_warp<T, CPL>(glines, gplanes, G, C, m, sub * CPL, active, e, gv);
}

template <typename T, int C>
__global__ void __launch_bounds__(256) appearance_bwd2_kernel(const T* __restrict__ lines,
                                                            const T* __restrict__ planes, int G,
                                                            float* __restrict__ glines,
                                                            float* __restrict__ gplanes,
                                                            const float* __restrict__ origins,
                                                            const float* __restrict__ dirs,
                                                            int64_t rows, int k, SamplerArgs s,
                                                            const int32_t* __restrict__ sel_idx,
                                                            const float* __restrict__ dX0) {
  // A quad owns rows 2p and 2p + 1: the selected samples of a ray are stored in
  // increasing sample order, so consecutive rows are neighbours along the ray.
  constexpr int CPL = C / 4;
  const int64_t pair = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  const int sub = threadIdx.x & 3;
  const int64_t ra_ = 2 * pair, rb_ = ra_ + 1;
  if (ra_ >= rows) return;
  const bool has_b = rb_ < rows;
  float ua[3], ub[3];
  {
    const int64_t r = ra_ / k;
    const int i = __ldg(sel_idx + ra_);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) ua[a] = grid_coord(x[a], G);
  }
  if (has_b) {
    const int64_t r = rb_ / k;
    const int i = __ldg(sel_idx + rb_);
    RayGeom g = load_ray(origins, dirs, r, s);
    float t, delta, x[3];
    sample_t(g, s, r, i, t, delta);
    sample_point(g, s, t, x);
#pragma unroll
    for (int a = 0; a < 3; ++a) ub[a] = grid_coord(x[a], G);
  }
  const float* srca = dX0 + ra_ * (3 * C) + sub * CPL;
  const float* srcb = dX0 + rb_ * (3 * C) + sub * CPL;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    PairEval<T, CPL> ea, eb;
    vm_pair_eval<T, CPL>(lines, planes, G, C, m, ua[a], ua[b], ua[c], sub * CPL, ea);
    float ga[CPL], gb[CPL];
    load_streaming<CPL>(srca + m * C, ga);
    if (has_b) {
      load_streaming<CPL>(srcb + m * C, gb);
    } else {
#pragma unroll
      for (int j = 0; j < CPL; ++j) gb[j] = 0.0f;
    }
    if (has_b) vm_pair_eval<T, CPL>(lines, planes, G, C, m, ub[a], ub[b], ub[c], sub * CPL, eb);
    vm_pair_scatter2<T, CPL>(glines, gplanes, G, C, m, sub * CPL, ea, ga, has_b, eb, gb);
  }
}

// ---------------------------------------------------------------------------------
// Sampler seam and layout conversion.
// ---------------------------------------------------------------------------------
__global__ void points_kernel(const float* __restrict__ origins, const float* __restrict__ dirs,
                              int64_t total, SamplerArgs s, float* __restrict__ points,
                              float* __restrict__ ts, float* __restrict__ steps) {
  const int64_t smp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (smp >= total) return;
  const int64_t r = smp / s.N;
  const int i = (int)(smp - r * s.N);
  RayGeom g = load_ray(origins, dirs, r, s);
  float t, delta, x[3];
  sample_t(g, s, r, i, t, delta);
  sample_point(g, s, t, x);
  if (points) {
#pragma unroll
    for (int a = 0; a < 3; ++a) points[a * total + smp] = x[a];
  }
  if (ts) ts[smp] = t;
  if (steps) steps[smp] = delta;
}

template <typename T>
__device__ __forceinline__ T cvt_from_f(float v);
template <>
__device__ __forceinline__ float cvt_from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 cvt_from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// (3, C, G) -> [3][G][C] and (3, C, G, G) -> [3][G][G][C].
template <typename T>
__global__ void to_channel_last_kernel(int G, int C, const float* __restrict__ vec,
                                       const float* __restrict__ mat, T* __restrict__ lines,
                                       T* __restrict__ planes) {
  const int64_t nl = 3LL * G * C, np = 3LL * G * G * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nl + np;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nl) {
      int64_t c = e % C, x = (e / C) % G, m = e / ((int64_t)C * G);
      lines[e] = cvt_from_f<T>(vec[(m * C + c) * G + x]);
    } else {
      int64_t q = e - nl;
      int64_t c = q % C, col = (q / C) % G, row = (q / ((int64_t)C * G)) % G,
              m = q / ((int64_t)C * G * G);
      planes[q] = cvt_from_f<T>(mat[((m * C + c) * G + row) * G + col]);
    }
  }
}

__global__ void to_channel_first_kernel(int G, int C, const float* __restrict__ lines,
                                        const float* __restrict__ planes, float* __restrict__ vec,
                                        float* __restrict__ mat) {
  const int64_t nl = 3LL * G * C, np = 3LL * G * G * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nl + np;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nl) {
      int64_t c = e % C, x = (e / C) % G, m = e / ((int64_t)C * G);
      vec[(m * C + c) * G + x] = lines[e];
    } else {
      int64_t q = e - nl;
      int64_t c = q % C, col = (q / C) % G, row = (q / ((int64_t)C * G)) % G,
              m = q / ((int64_t)C * G * G);
      mat[((m * C + c) * G + row) * G + col] = planes[q];
    }
  }
}

// ---------------------------------------------------------------------------------
// Dispatch.
// ---------------------------------------------------------------------------------
#define TVM_DISPATCH_C(C_, ...)                                                   \
  switch (C_) {                                                                   \
    case 8: { constexpr int CC = 8; __VA_ARGS__; break; }                         \
    case 16: { constexpr int CC = 16; __VA_ARGS__; break; }                       \
    case 24: { constexpr int CC = 24; __VA_ARGS__; break; }                       \
    case 32: { constexpr int CC = 32; __VA_ARGS__; break; }                       \
    case 48: { constexpr int CC = 48; __VA_ARGS__; break; }                       \
    default:                                                                      \
      set_error("channels=%d not compiled (supported: 8, 16, 24, 32, 48)", (int)(C_)); \
      return TVM_ERR_UNSUPPORTED;                                                 \
  }

#define TVM_DISPATCH_FIELD(f, ...)                                                           \
  do {                                                                                       \
    if ((f).dtype == TVM_F32) {                                                              \
      using TT = float;                                                                      \
      const TT* L_ = static_cast<const TT*>((f).lines);                                      \
      const TT* P_ = static_cast<const TT*>((f).planes);                                     \
      TVM_DISPATCH_C((f).C, __VA_ARGS__);                                                    \
    } else if ((f).dtype == TVM_BF16) {                                                      \
      using TT = __nv_bfloat16;                                                              \
      const TT* L_ = static_cast<const TT*>((f).lines);                                      \
      const TT* P_ = static_cast<const TT*>((f).planes);                                     \
      TVM_DISPATCH_C((f).C, __VA_ARGS__);                                                    \
    } else {                                                                                 \
      set_error("field dtype %d not supported", (f).dtype);                                  \
      return TVM_ERR_DTYPE;                                                                  \
    }                                                                                        \
  } while (0)

static inline unsigned quad_blocks(int64_t items) { return (unsigned)ceil_div(items * 4, 256); }

int launch_vm_features_fwd(const FieldView& f, const float* coords, int64_t n, float* out,
                           cudaStream_t st) {
  if (n == 0) return TVM_OK;
  TVM_DISPATCH_FIELD(f, (vm_features_fwd_kernel<TT, CC><<<quad_blocks(n), 256, 0, st>>>(
                             L_, P_, f.G, coords, n, out)));
  return check_launch("vm_features_fwd");
}

int launch_vm_features_bwd(const FieldView& f, const float* coords, int64_t n,
                           const float* grad_out, float* glines, float* gplanes, cudaStream_t st) {
  if (n == 0) return TVM_OK;
  TVM_DISPATCH_FIELD(f, (vm_features_bwd_kernel<TT, CC><<<quad_blocks(n), 256, 0, st>>>(
                             L_, P_, f.G, coords, n, grad_out, glines, gplanes)));
  return check_launch("vm_features_bwd");
}

int launch_density_fwd(const FieldView& f, float shift, const float* origins, const float* dirs,
                       int64_t R, const SamplerArgs& s, float* sigma, cudaStream_t st) {
  const int64_t total = R * s.N;
  if (total == 0) return TVM_OK;
  TVM_DISPATCH_FIELD(f, (density_fwd_kernel<TT, CC><<<quad_blocks(total), 256, 0, st>>>(
                             L_, P_, f.G, shift, origins, dirs, total, s, sigma)));
  return check_launch("density_fwd");
}

// Two samples per quad with merged reductions pay off when samples are dense along the
// rays (512 uniform samples, 64 selected); with few samples per ray the single-sample
// kernels keep more warps resident, which matters more.
constexpr int kPairScatterMinSamples = 128;
constexpr int kPairScatterMinSelected = 32;

int launch_density_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins,
                       const float* dirs, int64_t R, const SamplerArgs& s, const float* gsum,
                       cudaStream_t st) {
  const int64_t total = R * s.N;
  if (total == 0) return TVM_OK;
  if (s.N >= kPairScatterMinSamples) {
    TVM_DISPATCH_FIELD(f, (density_bwd2_kernel<TT, CC><<<quad_blocks((total + 1) / 2), 256, 0, st>>>(
                               L_, P_, f.G, glines, gplanes, origins, dirs, total, s, gsum)));
  } else {
    TVM_DISPATCH_FIELD(f, (density_bwd_kernel<TT, CC><<<quad_blocks(total), 256, 0, st>>>(
                               L_, P_, f.G, glines, gplanes, origins, dirs, total, s, gsum)));
  }
  return check_launch("density_bwd");
}

int launch_appearance_fwd(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                          const SamplerArgs& s, const int32_t* sel_idx, int k, float* X0,
                          cudaStream_t st) {
  const int64_t rows = R * k;
  if (rows == 0) return TVM_OK;
  TVM_DISPATCH_FIELD(f, (appearance_fwd_kernel<TT, CC><<<quad_blocks(rows), 256, 0, st>>>(
                             L_, P_, f.G, origins, dirs, rows, k, s, sel_idx, X0)));
  return check_launch("appearance_fwd");
}

int launch_appearance_fwd_tiles(const FieldView& f, const float* origins, const float* dirs, int64_t R,
                                const SamplerArgs& s, const int32_t* sel_idx, int k, uint8_t* X0t,
                                cudaStream_t st) {
  if (f.dtype != TVM_BF16 || f.C * 3 != X0T_FEAT) {
    set_error("appearance input tiles need a bf16 field of 48 channels per pair");
    return TVM_ERR_UNSUPPORTED;
  }
  if (!aligned(X0t, 16)) {
    set_error("appearance input tiles must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  const int64_t rows = R * k;
  if (rows == 0) return TVM_OK;
  const int64_t rows_padded = ceil_div(rows, (int64_t)X0T_ROWS) * X0T_ROWS;
  appearance_fwd_tiles_kernel<<<quad_blocks(rows_padded), 256, 0, st>>>(
      static_cast<const __nv_bfloat16*>(f.lines), static_cast<const __nv_bfloat16*>(f.planes), f.G, origins, dirs,
      rows, rows_padded, k, s, sel_idx, X0t);
  return check_launch("appearance_fwd_tiles");
}

int launch_appearance_bwd(const FieldView& f, float* glines, float* gplanes, const float* origins,
                          const float* dirs, int64_t R, const SamplerArgs& s,
                          const int32_t* sel_idx, int k, const float* dX0, cudaStream_t st) {
  const int64_t rows = R * k;
  if (rows == 0) return TVM_OK;
  if (k >= kPairScatterMinSelected) {
    TVM_DISPATCH_FIELD(f, (appearance_bwd2_kernel<TT, CC><<<quad_blocks((rows + 1) / 2), 256, 0, st>>>(
                               L_, P_, f.G, glines, gplanes, origins, dirs, rows, k, s, sel_idx, dX0)));
  } else {
    TVM_DISPATCH_FIELD(f, (appearance_bwd_kernel<TT, CC><<<quad_blocks(3 * rows), 256, 0, st>>>(
                               L_, P_, f.G, glines, gplanes, origins, dirs, rows, k, s, sel_idx, dX0)));
  }
  return check_launch("appearance_bwd");
}

int launch_points(const float* origins, const float* dirs, int64_t R, const SamplerArgs& s,
                  float* points, float* ts, float* steps, cudaStream_t st) {
  const int64_t total = R * s.N;
  if (total == 0) return TVM_OK;
  points_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, st>>>(origins, dirs, total, s, points,
                                                                 ts, steps);
  return check_launch("sample_points");
}

// ---------------------------------------------------------------------------------
// Grid resize: TensorVMSingle.resize (tensor_vm.py:182-198) via
// resize_with_aligned_corners (tensor_vm.py:202-223), i.e. jax.image.scale_and_translate
// with the linear (triangle) kernel, antialias on, scale s = (N-1)/(M-1) and translation
// 0.5 - s/2 on every resized axis. Output index o samples input position
// f = (o + 0.5)/s - t/s - 0.5 = o (M-1)/(N-1); the weights max(0, 1 - |f - i| / k) with
// k = max(1/s, 1) (wider only when downsampling) are normalised by their sum, and zero
// when f lies outside [-0.5, M - 0.5]. Float32 arithmetic, as jax runs it.
// ---------------------------------------------------------------------------------
struct ResizeAxis {
  int M;            // input size
  float inv_scale;  // 1 / s
  float tinv;       // translation / s
  float kscale;     // kernel width
};

constexpr int RESIZE_MAXTAPS = 64;  // host rejects kernels wider than this

__device__ int resize_taps(const ResizeAxis& ax, int o, int (&idx)[RESIZE_MAXTAPS], float (&w)[RESIZE_MAXTAPS]) {
  const float f = ((float)o + 0.5f) * ax.inv_scale - ax.tinv - 0.5f;
  if (!(f >= -0.5f && f <= (float)ax.M - 0.5f)) return 0;
  int lo = (int)ceilf(f - ax.kscale), hi = (int)floorf(f + ax.kscale);
  lo = max(lo, 0);
  hi = min(hi, ax.M - 1);
  int n = 0;
  float tot = 0.f;
  for (int i = lo; i <= hi && n < RESIZE_MAXTAPS; ++i) {
    const float x = fabsf(f - (float)i) / ax.kscale;
    const float wi = fmaxf(0.f, 1.f - x);
    if (wi > 0.f) {
      idx[n] = i;
      w[n] = wi;
      tot += wi;
      ++n;
    }
  }
  if (!(fabsf(tot) > 1000.f * 1.1920929e-7f)) return 0;
  for (int k = 0; k < n; ++k) w[k] = w[k] / tot;
  return n;
}

// lines [3][M][C] -> [3][N][C]; one thread per output (pair, position, channel).
__global__ void resize_lines_kernel(const float* __restrict__ src, float* __restrict__ dst, int N, int C,
                                    ResizeAxis ax) {
  const int64_t total = 3LL * N * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const int o = (int)((e / C) % N);
    const int m = (int)(e / ((int64_t)C * N));
    int idx[RESIZE_MAXTAPS];
    float w[RESIZE_MAXTAPS];
    const int n = resize_taps(ax, o, idx, w);
    float acc = 0.f;
    for (int k = 0; k < n; ++k) acc += w[k] * __ldg(src + ((int64_t)m * ax.M + idx[k]) * C + c);
    dst[e] = acc;
  }
}

// planes [3][M][M][C] -> [3][N][N][C], separable: rows first, then columns (the order
// scale_and_translate contracts its spatial axes in).
__global__ void resize_planes_kernel(const float* __restrict__ src, float* __restrict__ dst, int N, int C,
                                     ResizeAxis ax) {
  const int64_t total = 3LL * N * N * C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const int q = (int)((e / C) % N);
    const int r = (int)((e / ((int64_t)C * N)) % N);
    const int m = (int)(e / ((int64_t)C * N * N));
    int ri[RESIZE_MAXTAPS], qi[RESIZE_MAXTAPS];
    float rw[RESIZE_MAXTAPS], qw[RESIZE_MAXTAPS];
    const int nr = resize_taps(ax, r, ri, rw);
    const int nq = resize_taps(ax, q, qi, qw);
    float acc = 0.f;
    for (int b = 0; b < nq; ++b) {
      float col = 0.f;
      for (int a = 0; a < nr; ++a)
        col += rw[a] * __ldg(src + (((int64_t)m * ax.M + ri[a]) * ax.M + qi[b]) * C + c);
      acc += qw[b] * col;
    }
    dst[e] = acc;
  }
}

int launch_resize_field(int M, int N, int C, const float* src_lines, const float* src_planes, float* dst_lines,
                        float* dst_planes, cudaStream_t st) {
  ResizeAxis ax;
  ax.M = M;
  // jax: scale = float32((N - 1) / (M - 1)), translation = -(scale / 2 - 0.5),
  // inv_scale = 1 / scale, sample_f = (o + 0.5) * inv_scale - translation * inv_scale - 0.5.
  const float scale = (float)((N - 1.0) / (M - 1.0));
  const float translation = -(scale / 2.0f - 0.5f);
  ax.inv_scale = 1.0f / scale;
  ax.tinv = translation * ax.inv_scale;
  ax.kscale = ax.inv_scale > 1.0f ? ax.inv_scale : 1.0f;
  if (2.0f * ax.kscale + 2.0f > (float)RESIZE_MAXTAPS) {
    set_error("resize from %d to %d: the antialiasing kernel spans more than %d taps", M, N, RESIZE_MAXTAPS);
    return TVM_ERR_UNSUPPORTED;
  }
  const int64_t nl = 3LL * N * C, np = 3LL * N * N * C;
  resize_lines_kernel<<<(unsigned)std::min<int64_t>(ceil_div(nl, 256), 152 * 16), 256, 0, st>>>(src_lines, dst_lines,
                                                                                                N, C, ax);
  TVM_TRY(check_launch("resize_lines"));
  resize_planes_kernel<<<(unsigned)std::min<int64_t>(ceil_div(np, 256), 152 * 16), 256, 0, st>>>(src_planes,
                                                                                                 dst_planes, N, C, ax);
  return check_launch("resize_planes");
}

int launch_to_channel_last(int G, int C, const float* vec, const float* mat, int dtype, void* lines,
                           void* planes, cudaStream_t st) {
  const int64_t n = 3LL * G * C * (G + 1);
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 16);
  if (dtype == TVM_F32) {
    to_channel_last_kernel<float><<<blocks, 256, 0, st>>>(G, C, vec, mat, (float*)lines,
                                                          (float*)planes);
  } else if (dtype == TVM_BF16) {
    to_channel_last_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(
        G, C, vec, mat, (__nv_bfloat16*)lines, (__nv_bfloat16*)planes);
  } else {
    set_error("to_channel_last: dtype %d not supported", dtype);
    return TVM_ERR_DTYPE;
  }
  return check_launch("to_channel_last");
}

int launch_to_channel_first(int G, int C, const float* lines, const float* planes, float* vec,
                            float* mat, cudaStream_t st) {
  const int64_t n = 3LL * G * C * (G + 1);
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 16);
  to_channel_first_kernel<<<blocks, 256, 0, st>>>(G, C, lines, planes, vec, mat);
  return check_launch("to_channel_first");
}

}  // namespace tvm
