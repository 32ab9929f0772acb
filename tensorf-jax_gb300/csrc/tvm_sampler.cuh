// Ray-sample generation on the device: the bounded-scene sampler
// (render.py:350-434 vmapped at 177-186) and the contracted-scene sampler
// (render.py:122-173), plus the [-1,1] normalisation (render.py:192-196).
#pragma once

#include "tvm_common.cuh"

namespace tvm {

struct SamplerArgs {
  int sampler;  // TVM_SAMPLER_*
  int N;        // samples per ray
  float aabb[6];
  const float* schedule;  // CONTRACT: (N,)
  const float* jitter;    // BBOX: (N,) or (R,N) or NULL; CONTRACT: (R,N)
  int jitter_per_ray;     // BBOX only
  const float* ts;        // EXPLICIT: (R,N) sample distances
  const float* deltas;    // EXPLICIT: (R,N) segment lengths
  int contract;           // EXPLICIT: contract points to [-2,2]^3 before normalising
};

struct RayGeom {
  float o[3], d[3];
  float t_min, step;  // BBOX segment (render.py:369)
};

__device__ __forceinline__ RayGeom load_ray(const float* origins, const float* dirs, int64_t r,
                                             const SamplerArgs& s) {
  RayGeom g;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    g.o[a] = __ldg(origins + 3 * r + a);
    g.d[a] = __ldg(dirs + 3 * r + a);
  }
  g.t_min = 0.f;
  g.step = 0.f;
  if (s.sampler == TVM_SAMPLER_BBOX) {
    // ray_segment_from_bounding_box (render.py:399-434), min_segment_length=1e-3.
    float mx = -INFINITY, mn = INFINITY;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float den = g.d[a] + 1e-8f;
      float t0 = (s.aabb[a] - g.o[a]) / den;
      float t1 = (s.aabb[3 + a] - g.o[a]) / den;
      mx = fmaxf(mx, fminf(t0, t1));
      mn = fminf(mn, fmaxf(t0, t1));
    }
    float t_min = fmaxf(0.0f, mx);
    float t_max = mn;
    float t_max_c = fmaxf(t_max, t_min + 1e-3f);
    bool valid = t_min < t_max;
    float lo = valid ? t_min : 0.0f;
    float hi = valid ? t_max_c : 1e-3f;
    g.t_min = lo;
    g.step = (hi - lo) / (float)s.N;
  }
  return g;
}

// Distance t and segment length delta of sample i of ray r.
__device__ __forceinline__ void sample_t(const RayGeom& g, const SamplerArgs& s, int64_t r, int i,
                                         float& t, float& delta) {
  if (s.sampler == TVM_SAMPLER_BBOX) {
    float tt = (float)i;
    if (s.jitter != nullptr) tt = tt + __ldg(s.jitter + (s.jitter_per_ray ? r * s.N + i : i));
    tt = tt * g.step;
    t = g.t_min + tt;
    delta = g.step;
  } else if (s.sampler == TVM_SAMPLER_EXPLICIT) {
    t = __ldg(s.ts + r * s.N + i);
    delta = __ldg(s.deltas + r * s.N + i);
  } else {
    // Fixed schedule, step = roll(ts,-1) - ts with the last copied from the one
    // before (render.py:154-155), jitter per sample (render.py:158-161).
    float base = __ldg(s.schedule + i);
    float st = (i + 1 < s.N) ? __ldg(s.schedule + i + 1) - base
                             : base - __ldg(s.schedule + i - 1);
    t = base + st * __ldg(s.jitter + r * s.N + i);
    delta = st;
  }
}

// World point of distance t, contracted if needed, then normalised to [-1,1] by the
// aabb (render.py:164-171, 192-196).
__device__ __forceinline__ void sample_point(const RayGeom& g, const SamplerArgs& s, float t,
                                             float (&x)[3]) {
  float p[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) p[a] = g.o[a] + g.d[a] * t;
  if (s.sampler == TVM_SAMPLER_CONTRACT || (s.sampler == TVM_SAMPLER_EXPLICIT && s.contract)) {
    float nrm = fmaxf(fabsf(p[0]), fmaxf(fabsf(p[1]), fabsf(p[2])));
    if (!(nrm <= 1.0f)) {
      float sc = 2.0f - 1.0f / nrm;
#pragma unroll
      for (int a = 0; a < 3; ++a) p[a] = sc * p[a] / nrm;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) x[a] = ((p[a] - s.aabb[a]) / (s.aabb[3 + a] - s.aabb[a]) - 0.5f) * 2.0f;
}

}  // namespace tvm
