// Shared device/host helpers of the TensoRF-VM sm_103a kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <stdint.h>

#include "tensorf_gb300.h"

namespace tvm {

// ---------------------------------------------------------------------------------
// Host-side error reporting (per calling thread).
// ---------------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int check_launch(const char* what);  // TVM_OK or TVM_ERR_LAUNCH after a launch (counts it)
void phase_mark(int phase, cudaStream_t st);  // records the phase event if hooks are set

#define TVM_REQUIRE(cond, code, ...)  \
  do {                                \
    if (!(cond)) {                    \
      ::tvm::set_error(__VA_ARGS__);  \
      return (code);                  \
    }                                 \
  } while (0)

#define TVM_TRY(expr)          \
  do {                         \
    int _st = (expr);          \
    if (_st != TVM_OK) return _st; \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// Bump allocator over a caller-provided workspace.
struct Workspace {
  char* base;
  size_t size;
  size_t used;
  bool dry;  // sizing pass: base may be null
  template <typename T>
  T* take(int64_t count) {
    size_t off = (used + 255) & ~size_t(255);
    used = off + size_t(count) * sizeof(T);
    if (dry) return nullptr;
    return reinterpret_cast<T*>(base + off);
  }
  bool ok() const { return dry || used <= size; }
};

// ---------------------------------------------------------------------------------
// Device helpers.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }

// Load CPL consecutive storage elements into float registers with the widest
// naturally aligned vector loads (the caller guarantees alignment to the chunk
// size: chunk offsets are multiples of CPL and CPL*sizeof(T) divides the vector
// width used). Read-only path: parameters do not change inside a kernel.
template <int CPL>
__device__ __forceinline__ void load_chunk(const float* p, float (&v)[CPL]) {
  if constexpr (CPL % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 4; ++j) {
      float4 q = __ldg(reinterpret_cast<const float4*>(p) + j);
      v[4 * j + 0] = q.x;
      v[4 * j + 1] = q.y;
      v[4 * j + 2] = q.z;
      v[4 * j + 3] = q.w;
    }
  } else if constexpr (CPL % 2 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
      float2 q = __ldg(reinterpret_cast<const float2*>(p) + j);
      v[2 * j + 0] = q.x;
      v[2 * j + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < CPL; ++j) v[j] = __ldg(p + j);
  }
}

template <int CPL>
__device__ __forceinline__ void load_chunk(const __nv_bfloat16* p, float (&v)[CPL]) {
  if constexpr (CPL % 8 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 8; ++j) {
      uint4 q = __ldg(reinterpret_cast<const uint4*>(p) + j);
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float2 f = __bfloat1622float2(h[e]);
        v[8 * j + 2 * e] = f.x;
        v[8 * j + 2 * e + 1] = f.y;
      }
    }
  } else if constexpr (CPL % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 4; ++j) {
      uint2 q = __ldg(reinterpret_cast<const uint2*>(p) + j);
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        float2 f = __bfloat1622float2(h[e]);
        v[4 * j + 2 * e] = f.x;
        v[4 * j + 2 * e + 1] = f.y;
      }
    }
  } else if constexpr (CPL % 2 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
      unsigned int q = __ldg(reinterpret_cast<const unsigned int*>(p) + j);
      float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q));
      v[2 * j] = f.x;
      v[2 * j + 1] = f.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < CPL; ++j) v[j] = __bfloat162float(p[j]);
  }
}

// Vector atomic add of CPL floats into global memory: 16-byte reds (sm_90+ float4
// atomicAdd) where the chunk allows, else 8-byte or scalar ones.
template <int CPL>
__device__ __forceinline__ void red_chunk(float* p, const float (&v)[CPL]) {
  if constexpr (CPL % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 4; ++j)
      atomicAdd(reinterpret_cast<float4*>(p) + j,
                make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]));
  } else if constexpr (CPL % 2 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j)
      atomicAdd(reinterpret_cast<float2*>(p) + j, make_float2(v[2 * j], v[2 * j + 1]));
  } else {
#pragma unroll
    for (int j = 0; j < CPL; ++j) atomicAdd(p + j, v[j]);
  }
}

// A lane's CPL consecutive floats of a buffer that is written once and read once
// (appearance features, their gradients), moved with the evict-first cache hint so the
// stream does not push the fields out of L2. p is 16-byte aligned when CPL % 4 == 0, else
// 8-byte aligned.
template <int CPL>
__device__ __forceinline__ void store_streaming(float* p, const float (&v)[CPL]) {
  if constexpr (CPL % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 4; ++j)
      __stcs(reinterpret_cast<float4*>(p) + j, make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]));
  } else {
    static_assert(CPL % 2 == 0, "lanes hold an even number of channels");
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) __stcs(reinterpret_cast<float2*>(p) + j, make_float2(v[2 * j], v[2 * j + 1]));
  }
}

template <int CPL>
__device__ __forceinline__ void load_streaming(const float* p, float (&v)[CPL]) {
  if constexpr (CPL % 4 == 0) {
#pragma unroll
    for (int j = 0; j < CPL / 4; ++j) {
      const float4 q = __ldcs(reinterpret_cast<const float4*>(p) + j);
      v[4 * j] = q.x;
      v[4 * j + 1] = q.y;
      v[4 * j + 2] = q.z;
      v[4 * j + 3] = q.w;
    }
  } else {
    static_assert(CPL % 2 == 0, "lanes hold an even number of channels");
#pragma unroll
    for (int j = 0; j < CPL / 2; ++j) {
      const float2 q = __ldcs(reinterpret_cast<const float2*>(p) + j);
      v[2 * j] = q.x;
      v[2 * j + 1] = q.y;
    }
  }
}

// Linear-interpolation taps of map_coordinates(order=1, mode="nearest")
// (tensor_vm.py:226-250): weights from the unclamped coordinate, both corner indices
// clamped into [0, G-1]. The float->int conversion is done on a clamped copy so
// huge or non-finite coordinates still give in-range indices.
struct Tap {
  int i0, i1;
  float w0, w1;
};

__device__ __forceinline__ Tap make_tap(float u, int G) {
  float fl = floorf(u);
  Tap t;
  t.w1 = u - fl;
  t.w0 = 1.0f - t.w1;
  float flc = fminf(fmaxf(fl, -1.0f), (float)G);
  int i = (int)flc;
  t.i0 = min(max(i, 0), G - 1);
  t.i1 = min(max(i + 1, 0), G - 1);
  return t;
}

// [-1,1] -> [0, G-1] (tensor_vm.py:149-153), same operation order.
__device__ __forceinline__ float grid_coord(float x, int G) {
  float u = (x + 1.0f) / 2.0f;
  return u * ((float)G - 1.0f);
}

// jax.nn.softplus(x) = logaddexp(x, 0).
__device__ __forceinline__ float softplus_f(float x) {
  return fmaxf(x, 0.0f) + log1pf(expf(-fabsf(x)));
}

// Order-preserving map of a float key to an unsigned int (larger float -> larger
// uint), used by the exact top-k.
__device__ __forceinline__ uint32_t float_key_bits(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Inclusive prefix sum across the warp (lane order).
__device__ __forceinline__ float warp_inclusive_scan(float v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    float n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Inclusive suffix sum across the warp (lane order reversed).
__device__ __forceinline__ float warp_inclusive_suffix(float v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    float n = __shfl_down_sync(0xffffffffu, v, o);
    if (lane + o < 32) v += n;
  }
  return v;
}

// Coordinate permutation of pair m (tensor_vm.py:50-52): line coordinate, plane row,
// plane column.
__device__ __forceinline__ void mode_perm(int m, int& a, int& b, int& c) {
  a = (m == 0) ? 0 : (m == 1 ? 2 : 1);
  b = (m == 0) ? 1 : (m == 1 ? 0 : 2);
  c = (m == 0) ? 2 : (m == 1 ? 1 : 0);
}

}  // namespace tvm
