// Data generation on the device: counter-based noise, pinhole camera rays
// (cameras.py:100-143) and the FP64 quadrature of the analytic sphere scene used as
// the training target.
#include <algorithm>

#include "tvm_internal.h"

namespace tvm {

// SplitMix64 finaliser (Steele, Lea, Flood 2014) over (seed, stream, index).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Elements [i0, n) step `stride` of the draw (seed, stream id sid): uniform [0, 1) or
// Gumbel from 24 random bits of each element's hash.
__device__ __forceinline__ void noise_range(float* __restrict__ dst, int64_t n, uint64_t seed, uint64_t sid, int kind,
                                            int64_t i0, int64_t stride) {
  const uint64_t key = mix64(seed ^ mix64(sid + 0x9E3779B97F4A7C15ull));
  for (int64_t i = i0; i < n; i += stride) {
    const uint64_t h = mix64(key + (uint64_t)i * 0xD1B54A32D192ED03ull);
    const uint32_t bits = (uint32_t)(h >> 40);  // 24 random bits
    if (kind == 0) {
      dst[i] = (float)bits * (1.0f / 16777216.0f);  // [0, 1)
    } else {
      const float u = ((float)bits + 0.5f) * (1.0f / 16777216.0f);  // (0, 1)
      dst[i] = -logf(-logf(u));
    }
  }
}

// step (optional): the stream id is step->noise_stream * mul + add, read when it runs.
__global__ void noise_kernel(float* __restrict__ dst, int64_t n, uint64_t seed, uint64_t sid, int kind,
                             const tvm_step_scalars* __restrict__ step, uint64_t mul) {
  if (step != nullptr) sid = step->noise_stream * mul + sid;
  noise_range(dst, n, seed, sid, kind, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
              (int64_t)gridDim.x * blockDim.x);
}

// Several keyed draws, one per blockIdx.y.
struct NoiseBatch {
  tvm_noise_job job[TVM_NOISE_BATCH_MAX];
};
__global__ void noise_batch_kernel(NoiseBatch b, uint64_t seed, const tvm_step_scalars* __restrict__ step) {
  const tvm_noise_job& j = b.job[blockIdx.y];
  noise_range(j.dst, j.n, seed, step->noise_stream * j.mul + j.add, j.kind,
              (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

struct Cam {
  double Kinv[9];
  double R[9];
  double t[3];
};

__global__ void camera_rays_kernel(Cam cam, int width, int height, const int64_t* __restrict__ pixels,
                                   int64_t n, float* __restrict__ origins, float* __restrict__ dirs) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int64_t pix = pixels ? pixels[e] : e;
  const double u = (double)(pix % width), v = (double)(pix / width);
  double c[3], d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) c[a] = cam.Kinv[3 * a] * u + cam.Kinv[3 * a + 1] * v + cam.Kinv[3 * a + 2];
#pragma unroll
  for (int a = 0; a < 3; ++a) d[a] = cam.R[3 * a] * c[0] + cam.R[3 * a + 1] * c[1] + cam.R[3 * a + 2] * c[2];
  const double nrm = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + 1e-8;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dirs[3 * e + a] = (float)(d[a] / nrm);
    origins[3 * e + a] = (float)cam.t[a];
  }
}

// One warp per ray: n_samples midpoint samples over the ray's aabb segment, sigma =
// density * #spheres containing the point, colour = mean colour of those spheres,
// transmittance by an FP64 warp scan of -sigma*dt. White background.
__global__ void sphere_scene_kernel(const double* __restrict__ centers, const double* __restrict__ radii,
                                    const double* __restrict__ colors, int S, double density,
                                    const float* __restrict__ aabb_in, const float* __restrict__ origins,
                                    const float* __restrict__ dirs, int64_t R, int ns,
                                    float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= R) return;
  double o[3], d[3], aabb[6];
  for (int a = 0; a < 3; ++a) {
    o[a] = origins[3 * r + a];
    d[a] = dirs[3 * r + a];
  }
  for (int a = 0; a < 6; ++a) aabb[a] = aabb_in[a];
  double mx = -INFINITY, mn = INFINITY;
  for (int a = 0; a < 3; ++a) {
    const double den = d[a] + 1e-8;
    const double t0 = (aabb[a] - o[a]) / den, t1 = (aabb[3 + a] - o[a]) / den;
    mx = fmax(mx, fmin(t0, t1));
    mn = fmin(mn, fmax(t0, t1));
  }
  const double t_min = fmax(0.0, mx);
  const double t_max = fmax(mn, t_min + 1e-3);
  const bool valid = t_min < mn;
  const double lo = valid ? t_min : 0.0, hi = valid ? t_max : 1e-3;
  const double dt = (hi - lo) / ns;
  double carry = 0.0, acc[3] = {0.0, 0.0, 0.0};
  for (int base = 0; base < ns; base += 32) {
    const int i = base + lane;
    double sv = 0.0, col[3] = {0.0, 0.0, 0.0};
    if (i < ns) {
      const double t = lo + (i + 0.5) * dt;
      double p[3];
      for (int a = 0; a < 3; ++a) p[a] = o[a] + t * d[a];
      int cnt = 0;
      for (int q = 0; q < S; ++q) {
        const double dx = p[0] - centers[3 * q], dy = p[1] - centers[3 * q + 1], dz = p[2] - centers[3 * q + 2];
        if (sqrt(dx * dx + dy * dy + dz * dz) < radii[q]) {
          ++cnt;
          for (int a = 0; a < 3; ++a) col[a] += colors[3 * q + a];
        }
      }
      if (cnt > 0)
        for (int a = 0; a < 3; ++a) col[a] /= cnt;
      sv = -density * cnt * dt;
    }
    double incl = sv;
    for (int off = 1; off < 32; off <<= 1) {
      const double nb = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += nb;
    }
    incl += carry;
    const double prev = __shfl_up_sync(0xffffffffu, incl, 1);
    const double excl = (lane == 0) ? carry : prev;
    const double w = (1.0 - exp(sv)) * exp(excl);
    for (int a = 0; a < 3; ++a) acc[a] += w * col[a];
    carry = __shfl_sync(0xffffffffu, incl, 31);
  }
  for (int a = 0; a < 3; ++a) {
    for (int off = 16; off > 0; off >>= 1) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], off);
  }
  if (lane == 0) {
    const double bg = exp(carry);
    for (int a = 0; a < 3; ++a) out[3 * r + a] = (float)(acc[a] + bg);
  }
}

}  // namespace tvm

using namespace tvm;

extern "C" {

int tvm_noise_fill(float* dst, int64_t n, uint64_t seed, uint64_t stream_id, int32_t kind, void* stream) {
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(kind == 0 || kind == 1, TVM_ERR_INVALID, "kind must be 0 (uniform) or 1 (gumbel)");
  if (n == 0) return TVM_OK;
  TVM_REQUIRE(dst != nullptr, TVM_ERR_INVALID, "dst is NULL");
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 16);
  noise_kernel<<<blocks, 256, 0, as_stream(stream)>>>(dst, n, seed, stream_id, kind, nullptr, 0);
  return check_launch("noise_fill");
}

int tvm_noise_fill_keyed_batch(const tvm_noise_job* jobs, int32_t njobs, uint64_t seed, const tvm_step_scalars* step,
                               void* stream) {
  TVM_REQUIRE(njobs >= 0 && njobs <= TVM_NOISE_BATCH_MAX, TVM_ERR_SHAPE, "njobs=%d outside [0, %d]", njobs,
              TVM_NOISE_BATCH_MAX);
  if (njobs == 0) return TVM_OK;
  TVM_REQUIRE(jobs != nullptr && step != nullptr, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(step, 8), TVM_ERR_ALIGN, "step must be 8-byte aligned");
  NoiseBatch b{};
  int64_t most = 0;
  for (int q = 0; q < njobs; ++q) {
    TVM_REQUIRE(jobs[q].n >= 0, TVM_ERR_SHAPE, "job %d: n < 0", q);
    TVM_REQUIRE(jobs[q].kind == 0 || jobs[q].kind == 1, TVM_ERR_INVALID, "job %d: kind must be 0 or 1", q);
    TVM_REQUIRE(jobs[q].n == 0 || jobs[q].dst != nullptr, TVM_ERR_INVALID, "job %d: dst is NULL", q);
    b.job[q] = jobs[q];
    most = std::max(most, jobs[q].n);
  }
  if (most == 0) return TVM_OK;
  const dim3 grid((unsigned)std::min<int64_t>(ceil_div(most, 256), 152 * 16), (unsigned)njobs);
  noise_batch_kernel<<<grid, 256, 0, as_stream(stream)>>>(b, seed, step);
  return check_launch("noise_fill_batch");
}

int tvm_noise_fill_keyed(float* dst, int64_t n, uint64_t seed, const tvm_step_scalars* step, uint64_t mul,
                         uint64_t add, int32_t kind, void* stream) {
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  TVM_REQUIRE(kind == 0 || kind == 1, TVM_ERR_INVALID, "kind must be 0 (uniform) or 1 (gumbel)");
  if (n == 0) return TVM_OK;
  TVM_REQUIRE(dst != nullptr && step != nullptr, TVM_ERR_INVALID, "NULL pointer");
  TVM_REQUIRE(aligned(step, 8), TVM_ERR_ALIGN, "step must be 8-byte aligned");
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 16);
  noise_kernel<<<blocks, 256, 0, as_stream(stream)>>>(dst, n, seed, add, kind, step, mul);
  return check_launch("noise_fill");
}

static bool invert3(const double* m, double* o) {
  const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                     m[2] * (m[3] * m[7] - m[4] * m[6]);
  if (det == 0.0) return false;
  const double id = 1.0 / det;
  o[0] = (m[4] * m[8] - m[5] * m[7]) * id;
  o[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  o[3] = (m[5] * m[6] - m[3] * m[8]) * id;
  o[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  o[6] = (m[3] * m[7] - m[4] * m[6]) * id;
  o[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
  return true;
}

int tvm_camera_rays(const double* K, const double* R_world_camera, const double* t_world_camera,
                    int32_t width, int32_t height, const int64_t* pixels, int64_t n, float* origins,
                    float* directions, void* stream) {
  TVM_REQUIRE(K && R_world_camera && t_world_camera, TVM_ERR_INVALID, "camera pointers NULL (host)");
  TVM_REQUIRE(width >= 1 && height >= 1, TVM_ERR_SHAPE, "bad image size");
  if (!pixels) n = (int64_t)width * height;
  TVM_REQUIRE(n >= 0, TVM_ERR_SHAPE, "n < 0");
  if (n == 0) return TVM_OK;
  TVM_REQUIRE(origins && directions, TVM_ERR_INVALID, "outputs NULL");
  Cam cam;
  TVM_REQUIRE(invert3(K, cam.Kinv), TVM_ERR_INVALID, "K is singular");
  for (int i = 0; i < 9; ++i) cam.R[i] = R_world_camera[i];
  for (int i = 0; i < 3; ++i) cam.t[i] = t_world_camera[i];
  camera_rays_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, as_stream(stream)>>>(cam, width, height, pixels, n,
                                                                                 origins, directions);
  return check_launch("camera_rays");
}

int tvm_sphere_scene_render(const double* centers, const double* radii, const double* colors, int32_t spheres,
                            double density, const float* aabb, const tvm_rays* rays, int32_t n_samples,
                            float* colors_out, void* stream) {
  TVM_REQUIRE(rays != nullptr, TVM_ERR_INVALID, "rays NULL");
  TVM_REQUIRE(spheres >= 0 && n_samples >= 1, TVM_ERR_SHAPE, "bad sizes");
  if (rays->count == 0) return TVM_OK;
  TVM_REQUIRE(centers && radii && colors && aabb && rays->origins && rays->directions && colors_out,
              TVM_ERR_INVALID, "NULL pointer");
  sphere_scene_kernel<<<(unsigned)ceil_div(rays->count, 8), 256, 0, as_stream(stream)>>>(
      centers, radii, colors, spheres, density, aabb, rays->origins, rays->directions, rays->count, n_samples,
      colors_out);
  return check_launch("sphere_scene");
}

}  // extern "C"
