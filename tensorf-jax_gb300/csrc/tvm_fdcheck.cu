// FP64 evaluation of the training loss, for finite-difference checks of the FP32
// gradients on the device. Not on the hot path: one warp per ray, the whole forward
// (bounded sampler, both VM tensors, compositing, FeatureMlp, MSE) in double
// precision, with one parameter optionally perturbed by a double-precision delta.
// Every density sample reaches the appearance path (k = N), so the loss is a smooth
// function of the parameters (no sample selection).
//
// Follows render.py:105-279 (render_rays with RenderMode.RGB), render.py:300-347
// (segment probabilities), render.py:350-434 (bounded sampler), tensor_vm.py:42-89,
// 140-167, 226-250 (VM interpolation) and networks.py:13-121 (FeatureMlp).
#include "tvm_internal.h"

namespace tvm {
namespace fd64 {

struct Params {
  const float* p;
  int64_t idx;   // perturbed element, or -1
  double delta;
  __device__ __forceinline__ double operator()(int64_t i) const {
    const double v = (double)__ldg(p + i);
    return i == idx ? v + delta : v;
  }
};

struct Field {
  int64_t lines, planes;  // element offsets in the flat buffer
  int C;
};

__device__ __forceinline__ void tap64(double u, int G, int& i0, int& i1, double& w0, double& w1) {
  const double fl = floor(u);
  w1 = u - fl;
  w0 = 1.0 - w1;
  const double flc = fmin(fmax(fl, -1.0), (double)G);
  const int i = (int)flc;
  i0 = min(max(i, 0), G - 1);
  i1 = min(max(i + 1, 0), G - 1);
}

// feat[m*C + c] for grid coordinates u (3), or the sum over all of them.
__device__ void vm64(const Params& P, const Field& f, int G, const double (&u)[3], double* feat, double* sum) {
  double acc = 0.0;
  for (int m = 0; m < 3; ++m) {
    int a, b, c;
    mode_perm(m, a, b, c);
    int l0, l1, r0, r1, c0, c1;
    double lw0, lw1, rw0, rw1, cw0, cw1;
    tap64(u[a], G, l0, l1, lw0, lw1);
    tap64(u[b], G, r0, r1, rw0, rw1);
    tap64(u[c], G, c0, c1, cw0, cw1);
    const int64_t lb = f.lines + (int64_t)m * G * f.C, pb = f.planes + (int64_t)m * G * G * f.C;
    for (int ch = 0; ch < f.C; ++ch) {
      const double L = lw0 * P(lb + (int64_t)l0 * f.C + ch) + lw1 * P(lb + (int64_t)l1 * f.C + ch);
      const double Pl = rw0 * cw0 * P(pb + ((int64_t)r0 * G + c0) * f.C + ch) +
                        rw0 * cw1 * P(pb + ((int64_t)r0 * G + c1) * f.C + ch) +
                        rw1 * cw0 * P(pb + ((int64_t)r1 * G + c0) * f.C + ch) +
                        rw1 * cw1 * P(pb + ((int64_t)r1 * G + c1) * f.C + ch);
      if (feat) feat[m * f.C + ch] = L * Pl;
      acc += L * Pl;
    }
  }
  if (sum) *sum = acc;
}

struct Mlp {
  int64_t w0, w1, b1, w2, b2, w3, b3;
  int feat, squash, enc, units, nf, nv;
};

// rgb = FeatureMlp(x0, d) in double. x1 scratch: enc, h scratch: 2 * units.
__device__ void mlp64(const Params& P, const Mlp& M, const double* x0, const double (&d)[3], double* x1, double* h,
                      double (&rgb)[3]) {
  const double kHalfPi = 1.5707963267948966;
  for (int j = 0; j < M.squash; ++j) {
    double s = 0.0;
    for (int i = 0; i < M.feat; ++i) s += x0[i] * P(M.w0 + (int64_t)i * M.squash + j);
    x1[j] = s;
  }
  for (int a = 0; a < 3; ++a) x1[M.squash + a] = d[a];
  // [sin(2^f v)]_f then [sin(2^f v + pi/2)]_f per coordinate (networks.py:13-35).
  int col = M.squash + 3;
  for (int j = 0; j < M.squash; ++j) {
    for (int q = 0; q < 2 * M.nf; ++q) {
      const double x = x1[j] * (double)(1 << (q % M.nf));
      x1[col++] = sin(q < M.nf ? x : x + kHalfPi);
    }
  }
  for (int a = 0; a < 3; ++a) {
    for (int q = 0; q < 2 * M.nv; ++q) {
      const double x = d[a] * (double)(1 << (q % M.nv));
      x1[col++] = sin(q < M.nv ? x : x + kHalfPi);
    }
  }
  double* h1 = h;
  double* h2 = h + M.units;
  for (int u = 0; u < M.units; ++u) {
    double s = P(M.b1 + u);
    for (int i = 0; i < M.enc; ++i) s += x1[i] * P(M.w1 + (int64_t)i * M.units + u);
    h1[u] = fmax(s, 0.0);
  }
  for (int u = 0; u < M.units; ++u) {
    double s = P(M.b2 + u);
    for (int i = 0; i < M.units; ++i) s += h1[i] * P(M.w2 + (int64_t)i * M.units + u);
    h2[u] = fmax(s, 0.0);
  }
  for (int c = 0; c < 3; ++c) {
    double s = P(M.b3 + c);
    for (int i = 0; i < M.units; ++i) s += h2[i] * P(M.w3 + (int64_t)i * 3 + c);
    rgb[c] = 1.0 / (1.0 + exp(-s));
  }
}

struct Args {
  Params P;
  Field dens, app;
  Mlp mlp;
  int G, N;
  double aabb[6];
  double shift;
  const float *origins, *dirs, *colors, *jitter;
  int jitter_per_ray;
  int64_t R;
  double* scratch;  // per sample: (3C_a + enc + 2 units) doubles, R * N samples
  double* loss;     // accumulates sum of squared errors / (3R)
};

// One warp per ray. Lanes evaluate samples; lane 0 composites.
__global__ void __launch_bounds__(32) loss_f64_kernel(Args a) {
  extern __shared__ double sh[];  // sigma[N], rgb[N][3]
  const int64_t r = blockIdx.x;
  const int lane = threadIdx.x;
  double o[3], d[3];
  for (int k = 0; k < 3; ++k) {
    o[k] = (double)__ldg(a.origins + 3 * r + k);
    d[k] = (double)__ldg(a.dirs + 3 * r + k);
  }
  // ray_segment_from_bounding_box (render.py:399-434) with min_segment_length 1e-3.
  double mx = -INFINITY, mn = INFINITY;
  for (int k = 0; k < 3; ++k) {
    const double den = d[k] + 1e-8;
    const double t0 = (a.aabb[k] - o[k]) / den, t1 = (a.aabb[3 + k] - o[k]) / den;
    mx = fmax(mx, fmin(t0, t1));
    mn = fmin(mn, fmax(t0, t1));
  }
  const double t_min = fmax(0.0, mx), t_max = mn;
  const bool valid = t_min < t_max;
  const double lo = valid ? t_min : 0.0, hi = valid ? fmax(t_max, t_min + 1e-3) : 1e-3;
  const double step = (hi - lo) / a.N;
  const int stride_s = 3 * a.app.C + a.mlp.enc + 2 * a.mlp.units;
  for (int i = lane; i < a.N; i += 32) {
    double tt = (double)i;
    if (a.jitter) tt += (double)__ldg(a.jitter + (a.jitter_per_ray ? r * a.N + i : i));
    const double t = lo + tt * step;
    double u[3];
    for (int k = 0; k < 3; ++k) {
      const double p = o[k] + d[k] * t;
      const double x = ((p - a.aabb[k]) / (a.aabb[3 + k] - a.aabb[k]) - 0.5) * 2.0;
      u[k] = (x + 1.0) / 2.0 * (double)(a.G - 1);
    }
    double dsum;
    vm64(a.P, a.dens, a.G, u, nullptr, &dsum);
    const double z = dsum + a.shift;
    sh[i] = fmax(z, 0.0) + log1p(exp(-fabs(z)));
    double* s = a.scratch + (r * a.N + i) * stride_s;
    vm64(a.P, a.app, a.G, u, s, nullptr);
    double rgb[3];
    mlp64(a.P, a.mlp, s, d, s + 3 * a.app.C, s + 3 * a.app.C + a.mlp.enc, rgb);
    for (int c = 0; c < 3; ++c) sh[a.N + 3 * i + c] = rgb[c];
  }
  __syncwarp();
  if (lane == 0) {
    // compute_segment_probabilities (render.py:300-347), then the RGB composite with
    // every sample selected (render.py:511-546, white background).
    double logT = 0.0, wsum = 0.0, col[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < a.N; ++i) {
      const double sgm = -sh[i] * step;
      const double w = (1.0 - exp(sgm)) * exp(logT);
      logT += sgm;
      wsum += w;
      for (int c = 0; c < 3; ++c) col[c] += w * sh[a.N + 3 * i + c];
    }
    const double p_last = exp(logT);
    const double unbias = (1.0 - p_last + 1e-8) / (wsum + 1e-8);
    double se = 0.0;
    for (int c = 0; c < 3; ++c) {
      const double e = col[c] * unbias + p_last - (double)__ldg(a.colors + 3 * r + c);
      se += e * e;
    }
    atomicAdd(a.loss, se / (3.0 * (double)a.R));
  }
}

}  // namespace fd64

int launch_loss_f64(const tvm_param_layout& L, const tvm_model_desc& m, const float* params, int64_t pidx,
                    double delta, const tvm_rays& rays, const float* colors, const tvm_render_desc& c,
                    double* scratch, double* loss, cudaStream_t st) {
  fd64::Args a{};
  a.P = fd64::Params{params, pidx, delta};
  a.dens = fd64::Field{L.density_lines, L.density_planes, m.density_channels};
  a.app = fd64::Field{L.appearance_lines, L.appearance_planes, m.appearance_channels};
  a.mlp = fd64::Mlp{L.mlp_w0, L.mlp_w1, L.mlp_b1, L.mlp_w2, L.mlp_b2, L.mlp_w3, L.mlp_b3,
                    3 * m.appearance_channels, m.squash_dim, L.encoded_dim, m.units, m.feature_n_freqs,
                    m.viewdir_n_freqs};
  a.G = m.grid_dim;
  a.N = c.density_samples;
  for (int k = 0; k < 6; ++k) a.aabb[k] = (double)c.aabb[k];
  a.shift = (double)c.density_shift;
  a.origins = rays.origins;
  a.dirs = rays.directions;
  a.colors = colors;
  a.jitter = c.jitter;
  a.jitter_per_ray = c.jitter_per_ray;
  a.R = rays.count;
  a.scratch = scratch;
  a.loss = loss;
  cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(double), st);
  if (e != cudaSuccess) {
    set_error("memset: %s", cudaGetErrorString(e));
    return TVM_ERR_LAUNCH;
  }
  if (rays.count == 0) return TVM_OK;
  const size_t smem = (size_t)a.N * 4 * sizeof(double);
  fd64::loss_f64_kernel<<<(unsigned)rays.count, 32, smem, st>>>(a);
  return check_launch("loss_f64");
}

size_t loss_f64_scratch_bytes(const tvm_model_desc& m, int encoded_dim, int64_t R, int N) {
  return (size_t)R * N * (3 * m.appearance_channels + encoded_dim + 2 * m.units) * sizeof(double);
}

}  // namespace tvm
