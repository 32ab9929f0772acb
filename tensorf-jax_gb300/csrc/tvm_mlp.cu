// FeatureMlp (networks.py:38-121) in FP32: the plain-precision path.
//
//   H0 = X0 @ W0                      (3C -> 27, no bias; the folded basis matrix)
//   X1 = [H0, d, PE(H0), PE(d)]       (networks.py:68-76; PE per networks.py:13-35)
//   H1 = relu(X1 @ W1 + b1), H2 = relu(H1 @ W2 + b2), rgb = sigmoid(H2 @ W3 + b3)
//
// Layered design: each dense layer is one tiled FP32 SIMT GEMM (64x64 tile, 16-deep
// k-slices staged in shared memory, 4x4 outputs per thread) with its bias / ReLU /
// sigmoid / ReLU-mask epilogue fused; the Fourier encoding and its backward are
// elementwise kernels. Weight gradients are split-K GEMMs X^T @ dY over row chunks
// with one atomic per output per chunk. Activations (H0..H2) are kept in the
// workspace for the backward.
#include <algorithm>
#include <type_traits>

#include "tvm_internal.h"
#include "tvm_tcgemm.cuh"

namespace tvm {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;
constexpr float kHalfPi = 1.57079632679489661923f;

// Epilogues. operator() handles one element; vec4 four consecutive columns of one row
// (n..n+3, clipped at N), with one 16-byte access when the address allows it.
template <class E>
__device__ __forceinline__ void vec4_scalar(const E& e, int64_t m, int n, const float (&v)[4], int N) {
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (n + j < N) e(m, n + j, v[j]);
}
__device__ __forceinline__ bool vec_ok(const float* p, int n, int N) {
  return n + 3 < N && (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

struct EpiStore {
  float* C;
  int ldc;
  __device__ void operator()(int64_t m, int n, float v) const { C[m * ldc + n] = v; }
  __device__ void vec4(int64_t m, int n, const float (&v)[4], int N) const {
    float* p = C + m * ldc + n;
    if (vec_ok(p, n, N)) *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else vec4_scalar(*this, m, n, v, N);
  }
};
// act: 0 none, 1 relu, 2 sigmoid
struct EpiBiasAct {
  float* C;
  int ldc;
  const float* bias;
  int act;
  __device__ float f(int n, float v) const {
    if (bias) v = v + __ldg(bias + n);
    if (act == 1) v = fmaxf(v, 0.0f);
    if (act == 2) v = 1.0f / (1.0f + expf(-v));
    return v;
  }
  __device__ void operator()(int64_t m, int n, float v) const { C[m * ldc + n] = f(n, v); }
  __device__ void vec4(int64_t m, int n, const float (&v)[4], int N) const {
    float* p = C + m * ldc + n;
    if (vec_ok(p, n, N)) *reinterpret_cast<float4*>(p) = make_float4(f(n, v[0]), f(n + 1, v[1]), f(n + 2, v[2]), f(n + 3, v[3]));
    else vec4_scalar(*this, m, n, v, N);
  }
};
// C = v * (H > 0): backward through a ReLU whose output is H.
struct EpiReluMask {
  float* C;
  int ldc;
  const float* H;
  int ldh;
  __device__ void operator()(int64_t m, int n, float v) const {
    C[m * ldc + n] = (__ldg(H + m * ldh + n) > 0.0f) ? v : 0.0f;
  }
  __device__ void vec4(int64_t m, int n, const float (&v)[4], int N) const {
    float* p = C + m * ldc + n;
    const float* h = H + m * ldh + n;
    if (vec_ok(p, n, N) && (reinterpret_cast<uintptr_t>(h) & 15) == 0) {
      const float4 hv = __ldg(reinterpret_cast<const float4*>(h));
      *reinterpret_cast<float4*>(p) = make_float4(hv.x > 0.f ? v[0] : 0.f, hv.y > 0.f ? v[1] : 0.f,
                                                  hv.z > 0.f ? v[2] : 0.f, hv.w > 0.f ? v[3] : 0.f);
    } else {
      vec4_scalar(*this, m, n, v, N);
    }
  }
};
struct EpiAtomic {
  float* C;
  int ldc;
  __device__ void operator()(int64_t m, int n, float v) const { atomicAdd(C + m * ldc + n, v); }
  __device__ void vec4(int64_t m, int n, const float (&v)[4], int N) const {
    float* p = C + m * ldc + n;
    if (vec_ok(p, n, N)) atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    else vec4_scalar(*this, m, n, v, N);
  }
};
}  // namespace

// C(m,n) = sum_k A(m,k) B(k,n) for k in this CTA's split [z*kc, (z+1)*kc).
// A(m,k) = A[m*lda + k] (AT=false) or A[k*lda + m] (AT=true).
// B(k,n) = B[k*ldb + n] (BT=false) or B[n*ldb + k] (BT=true).
template <bool AT, bool BT, class Epi>
__global__ void __launch_bounds__(256) sgemm_kernel(int64_t M, int N, int64_t K,
                                                   const float* __restrict__ A, int64_t lda,
                                                   const float* __restrict__ B, int64_t ldb,
                                                   int64_t kc, Epi epi) {
  __shared__ __align__(16) float As[BK][BM + 4];
  __shared__ __align__(16) float Bs[BK][BN + 4];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * BM;
  const int n0 = blockIdx.x * BN;
  const int64_t kbeg = (int64_t)blockIdx.z * kc;
  const int64_t kend = std::min<int64_t>(K, kbeg + kc);
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int e = tid; e < BM * BK; e += 256) {
      int mm, kk;
      if (!AT) { mm = e / BK; kk = e % BK; } else { kk = e / BM; mm = e % BM; }
      const int64_t gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < kend) v = AT ? __ldg(A + gk * lda + gm) : __ldg(A + gm * lda + gk);
      As[kk][mm] = v;
    }
#pragma unroll
    for (int e = tid; e < BK * BN; e += 256) {
      int kk, nn;
      if (!BT) { kk = e / BN; nn = e % BN; } else { nn = e / BK; kk = e % BK; }
      const int64_t gk = k0 + kk;
      const int gn = n0 + nn;
      float v = 0.f;
      if (gn < N && gk < kend) v = BT ? __ldg(B + (int64_t)gn * ldb + gk) : __ldg(B + gk * ldb + gn);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w};
      const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n < N) epi(m, n, acc[i][j]);
    }
  }
}

template <bool AT, bool BT, class Epi>
static int gemm(int64_t M, int N, int64_t K, const float* A, int64_t lda, const float* B,
                int64_t ldb, Epi epi, cudaStream_t st, int64_t kc = 0) {
  if (M == 0 || N == 0) return TVM_OK;
  if (kc <= 0) kc = K;
  const int64_t splits = ceil_div(K, kc);
  dim3 grid((unsigned)ceil_div(N, BN), (unsigned)ceil_div(M, BM), (unsigned)splits);
  sgemm_kernel<AT, BT, Epi><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, kc, epi);
  return check_launch("sgemm");
}

// One dense product with the model's arithmetic: SIMT FP32, tcgen05 bf16 or tcgen05
// split-bf16.
// kc < 0 asks for a split-K reduction sized for the GPU (the epilogue accumulates).
template <bool AT, bool BT, class Epi>
static int mm(int math, int64_t M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
              Epi epi, cudaStream_t st, int64_t kc = 0) {
  if (kc < 0) kc = (math == 2) ? 4096 : splitk_chunk(M, K);
  if (math == 2) return gemm<AT, BT>(M, N, K, A, lda, B, ldb, epi, st, kc);
  if (math == 1) return tc_gemm<AT, BT, tcg::FMT_TF32, true>(M, N, K, A, lda, B, ldb, epi, st, kc);
  return tc_gemm<AT, BT, tcg::FMT_BF16, false>(M, N, K, A, lda, B, ldb, epi, st, kc);
}

// X1[m][sq..enc) from X1[m][0..sq) (= H0) and the view direction
// (networks.py:68-76). A block owns 32 rows: their H0 and directions go to shared
// memory, then consecutive threads write consecutive columns of a row.
constexpr int PE_ROWS = 32;
__global__ void __launch_bounds__(256) pe_fwd_kernel(float* __restrict__ X1, int ld, int64_t M, int sq, int enc,
                                                    int nf, int nv, const float* __restrict__ dirs,
                                                    int rows_per_dir) {
  __shared__ float h[PE_ROWS][65];
  __shared__ float dv[PE_ROWS][3];
  const int64_t m0 = (int64_t)blockIdx.x * PE_ROWS;
  const int nrows = (int)(M - m0 < PE_ROWS ? M - m0 : PE_ROWS);
  for (int e = threadIdx.x; e < nrows * sq; e += blockDim.x) {
    const int r = e / sq, j = e - r * sq;
    h[r][j] = X1[(m0 + r) * ld + j];
  }
  for (int e = threadIdx.x; e < nrows * 3; e += blockDim.x) {
    const int r = e / 3, a = e - r * 3;
    dv[r][a] = __ldg(dirs + ((m0 + r) / rows_per_dir) * 3 + a);
  }
  __syncthreads();
  // One thread per (row, encoded coordinate): one sincosf, the higher frequencies by
  // the double-angle identities (sin 2x = 2 s c, cos 2x = c^2 - s^2) for up to 4
  // frequencies, direct sincosf beyond. sin(x + pi/2) is written as cos(x).
  const int f_end = sq + 3 + sq * 2 * nf;
  for (int e = threadIdx.x; e < nrows * (sq + 3); e += blockDim.x) {
    const int r = e / (sq + 3), j = e - r * (sq + 3);
    float* row = X1 + (m0 + r) * ld;
    float x;
    int n, col;
    if (j < sq) {
      x = h[r][j];
      n = nf;
      col = sq + 3 + j * 2 * nf;
    } else {
      x = dv[r][j - sq];
      row[j] = x;
      n = nv;
      col = f_end + (j - sq) * 2 * nv;
    }
    float sn, cs;
    sincosf(x, &sn, &cs);
    for (int f = 0; f < n; ++f) {
      if (f > 0) {
        if (n <= 4) {
          const float s2 = 2.0f * sn * cs, c2 = cs * cs - sn * sn;
          sn = s2;
          cs = c2;
        } else {
          sincosf(x * (float)(1 << f), &sn, &cs);
        }
      }
      row[col + f] = sn;
      row[col + n + f] = cs;
    }
  }
}

// dH0[m][j] = dX1[m][j] + sum_f dX1[m][PE(j,f)] * d PE / d h (one thread per (m, j)),
// h = X1[m][j].
__global__ void __launch_bounds__(256) pe_bwd_kernel(const float* __restrict__ dX1, int ld,
                                                    const float* __restrict__ X1, int64_t M, int sq, int nf,
                                                    float* __restrict__ dH0) {
  const int64_t m0 = (int64_t)blockIdx.x * PE_ROWS;
  const int nrows = (int)(M - m0 < PE_ROWS ? M - m0 : PE_ROWS);
  for (int e = threadIdx.x; e < nrows * sq; e += blockDim.x) {
    const int r = e / sq, j = e - r * sq;
    const int64_t m = m0 + r;
    const float hv = __ldg(X1 + m * ld + j);
    float g = __ldg(dX1 + m * ld + j);
    const float* pe = dX1 + m * ld + sq + 3 + j * 2 * nf;
    for (int f = 0; f < nf; ++f) {
      const float sc = (float)(1 << f);
      const float x = hv * sc;
      g += __ldg(pe + f) * cosf(x) * sc;
      g += __ldg(pe + nf + f) * cosf(x + kHalfPi) * sc;
    }
    dH0[m * sq + j] = g;
  }
}

// out[n] += sum over rows of Y[m][n].
__global__ void colsum_kernel(const float* __restrict__ Y, int ld, int64_t M, int N, int64_t chunk,
                              float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int64_t m0 = (int64_t)blockIdx.y * chunk;
  const int64_t m1 = std::min<int64_t>(M, m0 + chunk);
  float s = 0.f;
  for (int64_t m = m0; m < m1; ++m) s += __ldg(Y + m * ld + n);
  atomicAdd(out + n, s);
}

__global__ void sigmoid_bwd_kernel(const float* __restrict__ rgb, const float* __restrict__ g,
                                   int64_t n, float* __restrict__ dz) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float v = __ldg(rgb + e);
  dz[e] = __ldg(g + e) * (v * (1.0f - v));
}

static int ld_x1(const MlpDims& d) { return (int)round_up(d.enc, 4); }

// Workspace carve-out shared by forward and backward (same order).
struct MlpBufs {
  float *X1, *H1, *H2, *dH2, *dH1, *dX1, *dH0;
  uint8_t* wpack;
};
static MlpBufs carve(const MlpDims& d, int64_t M, Workspace& ws) {
  MlpBufs b{};
  if (mlp_fused_supported(d)) {  // the fused kernels keep every activation on chip
    b.wpack = ws.take<uint8_t>((int64_t)mlp_fused_pack_bytes());
    return b;
  }
  b.X1 = ws.take<float>(M * ld_x1(d));
  b.H1 = ws.take<float>(M * d.units);
  b.H2 = ws.take<float>(M * d.units);
  b.dH2 = ws.take<float>(M * d.units);
  b.dH1 = ws.take<float>(M * d.units);
  b.dX1 = ws.take<float>(M * ld_x1(d));
  b.dH0 = ws.take<float>(M * d.squash);
  return b;
}

size_t mlp_workspace_bytes(const MlpDims& d, int64_t M) {
  Workspace ws{nullptr, 0, 0, true};
  carve(d, M, ws);
  return ws.used + 256;
}


int mlp_forward(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs,
                int rows_per_dir, int64_t M, float* rgb, Workspace& ws, cudaStream_t st) {
  MlpBufs b = carve(d, M, ws);
  if (!ws.ok()) {
    set_error("mlp workspace too small");
    return TVM_ERR_WORKSPACE;
  }
  const int l1 = ld_x1(d);
  if (mlp_fused_supported(d)) {
    // BF16: all four layers in one tcgen05 kernel. Nothing is kept for the backward,
    // which recomputes the activations from X0 (only the packed weights are reused).
    return launch_mlp_fwd_fused(d, w, X0, dirs, rows_per_dir, M, rgb, b.wpack, st);
  }
  TVM_TRY((mm<false, false>(d.math, M, d.squash, d.feat, X0, d.feat, w.w0, d.squash, EpiStore{b.X1, l1}, st)));
  pe_fwd_kernel<<<(unsigned)ceil_div(M, PE_ROWS), 256, 0, st>>>(b.X1, l1, M, d.squash, d.enc, d.nf, d.nv, dirs,
                                                                 rows_per_dir);
  TVM_TRY(check_launch("pe_fwd"));
  TVM_TRY((mm<false, false>(d.math, M, d.units, d.enc, b.X1, l1, w.w1, d.units,
                              EpiBiasAct{b.H1, d.units, w.b1, 1}, st)));
  TVM_TRY((mm<false, false>(d.math, M, d.units, d.units, b.H1, d.units, w.w2, d.units,
                              EpiBiasAct{b.H2, d.units, w.b2, 1}, st)));
  TVM_TRY((mm<false, false>(d.math, M, 3, d.units, b.H2, d.units, w.w3, 3, EpiBiasAct{rgb, 3, w.b3, 2}, st)));
  return TVM_OK;
}

int mlp_backward(const MlpDims& d, const MlpWeights& w, const MlpGrads& g, const float* X0, const float* dirs,
                 int rows_per_dir, int64_t M, const float* dZ3, float* dX0, Workspace& ws, cudaStream_t st) {
  MlpBufs b = carve(d, M, ws);
  if (!ws.ok()) {
    set_error("mlp workspace too small");
    return TVM_ERR_WORKSPACE;
  }
  if (mlp_fused_supported(d)) {
    return launch_mlp_bwd_fused(w, g, X0, dirs, rows_per_dir, M, dZ3, dX0, b.wpack, st);
  }
  const int l1 = ld_x1(d);
  const int64_t kc = -1;  // weight gradients: split-K over the rows, sized per GEMM
  {
    // Layer 3: dH2 = (dZ3 @ W3^T) * [H2 > 0]; dW3 = H2^T dZ3; db3 = sum dZ3.
    TVM_TRY((mm<false, true>(d.math, M, d.units, 3, dZ3, 3, w.w3, 3, EpiReluMask{b.dH2, d.units, b.H2, d.units}, st)));
    TVM_TRY((mm<true, false>(d.math, d.units, 3, M, b.H2, d.units, dZ3, 3, EpiAtomic{g.w3, 3}, st, kc)));
    // Layer 2.
    TVM_TRY((mm<false, true>(d.math, M, d.units, d.units, b.dH2, d.units, w.w2, d.units,
                             EpiReluMask{b.dH1, d.units, b.H1, d.units}, st)));
    TVM_TRY((mm<true, false>(d.math, d.units, d.units, M, b.H1, d.units, b.dH2, d.units, EpiAtomic{g.w2, d.units}, st, kc)));
    // Layer 1.
    TVM_TRY((mm<false, true>(d.math, M, d.enc, d.units, b.dH1, d.units, w.w1, d.units, EpiStore{b.dX1, l1}, st)));
    TVM_TRY((mm<true, false>(d.math, d.enc, d.units, M, b.X1, l1, b.dH1, d.units, EpiAtomic{g.w1, d.units}, st, kc)));
  }
  // Bias gradients.
  {
    const int64_t cs = 128;  // rows per colsum block: M/128 blocks keep every SM busy
    dim3 grid3(1, (unsigned)ceil_div(M, cs));
    colsum_kernel<<<grid3, 32, 0, st>>>(dZ3, 3, M, 3, cs, g.b3);
    TVM_TRY(check_launch("colsum"));
    dim3 gridu((unsigned)ceil_div(d.units, 128), (unsigned)ceil_div(M, cs));
    colsum_kernel<<<gridu, 128, 0, st>>>(b.dH2, d.units, M, d.units, cs, g.b2);
    TVM_TRY(check_launch("colsum"));
    colsum_kernel<<<gridu, 128, 0, st>>>(b.dH1, d.units, M, d.units, cs, g.b1);
    TVM_TRY(check_launch("colsum"));
  }
  // Fourier encoding backward, then layer 0.
  pe_bwd_kernel<<<(unsigned)ceil_div(M, PE_ROWS), 256, 0, st>>>(b.dX1, l1, b.X1, M, d.squash, d.nf, b.dH0);
  TVM_TRY(check_launch("pe_bwd"));
  TVM_TRY((mm<true, false>(d.math, d.feat, d.squash, M, X0, d.feat, b.dH0, d.squash, EpiAtomic{g.w0, d.squash}, st, kc)));
  if (dX0) {
    TVM_TRY((mm<false, true>(d.math, M, d.feat, d.squash, b.dH0, d.squash, w.w0, d.squash, EpiStore{dX0, d.feat}, st)));
  }
  return TVM_OK;
}

int launch_sigmoid_bwd(const float* rgb, const float* grad_rgb, int64_t M, float* dZ3,
                       cudaStream_t st) {
  const int64_t n = M * 3;
  if (n == 0) return TVM_OK;
  sigmoid_bwd_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(rgb, grad_rgb, n, dZ3);
  return check_launch("sigmoid_bwd");
}

}  // namespace tvm

namespace tvm {

int device_status(int32_t* out, cudaStream_t st) {
  int32_t v = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_tc_status, sizeof(int32_t), 0, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    const int32_t zero = 0;
    e = cudaMemcpyToSymbolAsync(g_tc_status, &zero, sizeof(int32_t), 0, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_error("device_status: %s", cudaGetErrorString(e));
    return TVM_ERR_LAUNCH;
  }
  int32_t f = 0, q = 0;
  TVM_TRY(fused_status(&f, st));
  TVM_TRY(prop_status(&q, st));
  *out = v | f | q;
  return TVM_OK;
}

int gemm_any(int math, bool at, bool bt, int64_t M, int N, int64_t K, const float* A, int64_t lda,
             const float* B, int64_t ldb, float* D, int64_t ldd, bool accumulate, cudaStream_t st) {
  const int ldc = (int)ldd;
  const int64_t kc = accumulate ? -1 : 0;
#define TVM_GEMM_CASE(AT_, BT_)                                                                     \
  if (at == AT_ && bt == BT_) {                                                                     \
    if (accumulate) return mm<AT_, BT_>(math, M, N, K, A, lda, B, ldb, EpiAtomic{D, ldc}, st, kc); \
    return mm<AT_, BT_>(math, M, N, K, A, lda, B, ldb, EpiStore{D, ldc}, st);                    \
  }
  TVM_GEMM_CASE(false, false)
  TVM_GEMM_CASE(false, true)
  TVM_GEMM_CASE(true, false)
  TVM_GEMM_CASE(true, true)
#undef TVM_GEMM_CASE
  return TVM_ERR_INVALID;
}

}  // namespace tvm

namespace tvm {

}  // namespace tvm
