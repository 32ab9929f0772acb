// FeatureMlp (networks.py:38-121) for the FP32 and the generic paths.
//
//   H0 = X0 @ W0                      (3C -> 27, no bias; the folded basis matrix)
//   X1 = [H0, d, PE(H0), PE(d)]       (networks.py:68-76; PE per networks.py:13-35)
//   H1 = relu(X1 @ W1 + b1), H2 = relu(H1 @ W2 + b2), rgb = sigmoid(H2 @ W3 + b3)
//
// Three implementations, chosen by the model:
//   - BF16 models with the reference widths: the fused tcgen05 kernels of
//     tvm_mlpfused.cu (no activations kept);
//   - FP32 models with the reference widths (27 squash features, 2 frequencies, 128
//     units): split-tf32 products on the persistent pipelined GEMM of tvm_pgemm.cuh with
//     the encoding, layer 3, ReLU masks and bias sums fused into its epilogues, a
//     one-pass layer-3 backward, and split-K tcgen05 weight gradients;
//   - any other widths: layered products (tcgen05 bf16 / split-tf32 GEMMs of
//     tvm_tcgemm.cuh, or FP32 SIMT), elementwise encoding kernels and column sums.
// Activations needed by the backward are kept in the caller's workspace.
#include <algorithm>
#include <type_traits>

#include <cudaTypedefs.h>

#include "tvm_internal.h"
#include "tvm_tcgemm.cuh"
#include "tvm_pgemm.cuh"

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
  static constexpr bool kColumns = false;
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
  static constexpr bool kColumns = false;
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
  static constexpr bool kColumns = false;
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
  static constexpr bool kColumns = false;
  float* C;
  int ldc;
  __device__ void operator()(int64_t m, int n, float v) const { atomicAdd(C + m * ldc + n, v); }
  __device__ void vec4(int64_t m, int n, const float (&v)[4], int N) const {
    float* p = C + m * ldc + n;
    if (vec_ok(p, n, N)) atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    else vec4_scalar(*this, m, n, v, N);
  }
};
// C[n * ldc + m] += v: accumulates the transpose of the product (a weight gradient
// computed as dY^T X, so that each activation is read once). vec4_col gets rows
// m..m+3 of column n (clipped at M).
struct EpiAtomicT {
  static constexpr bool kColumns = true;
  float* C;
  int ldc;
  __device__ void operator()(int64_t m, int n, float v) const { atomicAdd(C + (int64_t)n * ldc + m, v); }
  __device__ void vec4_col(int64_t m, int n, const float (&v)[4], int64_t M) const {
    float* p = C + (int64_t)n * ldc + m;
    if (m + 3 < M && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
      atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (m + j < M) atomicAdd(p + j, v[j]);
    }
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

// ---------------------------------------------------------------------------------
// FP32 (split-tf32) path on the persistent pipelined GEMM (tvm_pgemm.cuh), for the
// reference FeatureMlp widths: 27 squash features, 2 encoding frequencies for features
// and directions (encoded width 150), 128 hidden units.
//
//   forward:  X1 = [H0, d, PE(H0), PE(d)] with H0 = X0 W0      (L0 GEMM, encoding in its epilogue)
//             H1 = relu(X1 W1 + b1)                              (L1 GEMM)
//             H2 = relu(H1 W2 + b2), rgb = sigmoid(H2 W3 + b3)   (L2 GEMM, layer 3 in its epilogue)
//   backward: dH2, dW3, db3, db2 from H2 and dZ3                 (l3_bwd_kernel, one pass)
//             dH1 = (dH2 W2^T) * [H1 > 0], db1 = colsum dH1      (GEMM, mask + column sums in its epilogue)
//             dH0 = PE^T(dH1 W1^T)                               (GEMM, encoding backward in its epilogue)
//             dX0 = dH0 W0^T                                     (GEMM)
//             dW2 = H1^T dH2, dW1 = X1^T dH1, dW0 = X0^T dH0     (split-K tc_gemm)
// ---------------------------------------------------------------------------------
static bool pmlp_supported(const MlpDims& d) {
  return d.math == 1 && d.cams == 0 && d.squash == pg::SQ && d.enc == pg::ENC && d.nf == 2 && d.nv == 2 && d.units == 128 &&
         d.feat % 4 == 0 && d.feat >= 4 && d.feat <= 160;
}
static int pmlp_nt_dx0(const MlpDims& d) { return d.feat <= 64 ? 64 : d.feat <= 144 ? 144 : 160; }
constexpr int PMLP_NT_DX1 = 144;  // dX1 columns the encoding backward reads: [h | d | PE(h)] = 138

// Byte sizes of the six packed weight images (forward: L0, L1, L2; backward: dH1, dX1, dX0).
struct PmlpImages {
  int bytes[6];
  int total() const { return bytes[0] + bytes[1] + bytes[2] + bytes[3] + bytes[4] + bytes[5]; }
};
static PmlpImages pmlp_images(const MlpDims& d) {
  PmlpImages im;
  im.bytes[0] = pg::image_bytes(d.feat, 32);
  im.bytes[1] = pg::image_bytes(pg::ENC, 128);
  im.bytes[2] = pg::image_bytes(128, 128);
  im.bytes[3] = pg::image_bytes(128, 128);
  im.bytes[4] = pg::image_bytes(128, PMLP_NT_DX1);
  im.bytes[5] = pg::image_bytes(pg::SQ, pmlp_nt_dx0(d));
  return im;
}

static int pack_images(const pg::PackJob* jobs, int count, cudaStream_t st) {
  pg::PackList list{};
  int most = 0;
  for (int i = 0; i < count; ++i) {
    list.job[i] = jobs[i];
    most = std::max(most, jobs[i].kp * jobs[i].np);
  }
  list.count = count;
  dim3 grid((unsigned)ceil_div(most, 256), (unsigned)count);
  pg::pack_kernel<<<grid, 256, 0, st>>>(list);
  return check_launch("pgemm pack");
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Row-major fp32 matrix (cols wide, rows high, row pitch ld elements) as a 2-D tensor map
// with a box of bx columns x by rows and the given shared-memory swizzle; reads past the
// edges return zero.
static int make_map(CUtensorMap* m, const float* base, int64_t cols, int64_t rows, int64_t ld, int bx, int by,
                    CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE) {
  auto enc = tensor_map_encoder();
  TVM_REQUIRE(enc != nullptr, TVM_ERR_LAUNCH, "cuTensorMapEncodeTiled is unavailable");
  TVM_REQUIRE(aligned(base, 16) && (ld * 4) % 16 == 0 && cols > 0 && rows > 0, TVM_ERR_ALIGN,
              "tensor map: base %p / pitch %lld not 16-byte aligned", (const void*)base, (long long)(ld * 4));
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TVM_REQUIRE(r == CUDA_SUCCESS, TVM_ERR_LAUNCH, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return TVM_OK;
}

// ocols: the output width the TMA-stored epilogues write (ea.out with row pitch ea.ldo).
template <int KIND, int NT>
static int pgemm(int64_t M, int N, int K, const float* A, int64_t lda, const uint8_t* bimg, const pg::EpiArgs& ea,
                 cudaStream_t st, int ocols = 0) {
  if (M == 0) return TVM_OK;
  const bool tma_out = KIND == pg::EPI_BIAS_RELU || KIND == pg::EPI_BIAS_RELU_L3 || KIND == pg::EPI_MASK_COLSUM ||
                       KIND == pg::EPI_PE_FWD ||
                       (KIND == pg::EPI_STORE && aligned(ea.out, 16) && ea.ldo % 4 == 0);
  TVM_REQUIRE(aligned(bimg, 16) && N <= NT && K > 0 && M <= INT32_MAX &&
                  ((KIND != pg::EPI_BIAS_RELU && KIND != pg::EPI_BIAS_RELU_L3 && KIND != pg::EPI_MASK_COLSUM) ||
                   N == NT),
              TVM_ERR_INVALID, "pgemm: unsupported operands (K=%d, lda=%lld, N=%d)", K, (long long)lda, N);
  CUtensorMap tmA, tmO;
  TVM_TRY(make_map(&tmA, A, K, M, lda, pg::BK, pg::BM, CU_TENSOR_MAP_SWIZZLE_128B));
  if (tma_out) {
    TVM_TRY(make_map(&tmO, ea.out, ocols > 0 ? ocols : N, M, ea.ldo, pg::OUT_BOX_COLS, pg::OUT_BOX_ROWS));
  } else {
    tmO = tmA;
  }
  // Shared memory left after the B images goes to store blocks (up to 4 per epilogue warp
  // while at least 4 TMA stages still fit) and then to the TMA ring.
  constexpr int EF = pg::epi_smem_floats<KIND, NT>();
  const int base = pg::smem_base_bytes<NT>(K, EF);
  const int avail = pg::SMEM_LIMIT - base;
  int nsb = 0;
  if (tma_out) {
    nsb = 1;
    for (int cand : {4, 2})
      if (avail - cand * pg::EPI_WARPS * pg::OUT_BOX_FLOATS * 4 >= 4 * pg::TILE_BYTES) {
        nsb = cand;
        break;
      }
  }
  const int stage = nsb * pg::EPI_WARPS * pg::OUT_BOX_FLOATS * 4;
  const int slots = std::min(pg::MAX_SLOTS, (avail - stage) / pg::TILE_BYTES);
  TVM_REQUIRE(slots >= 2, TVM_ERR_UNSUPPORTED, "pgemm: K=%d, N=%d leaves %d pipeline slots", K, NT, slots);
  const int bytes = std::max(base + slots * pg::TILE_BYTES + stage, pg::MIN_SMEM);
  auto fn = pg::pgemm_kernel<KIND, NT>;
  TVM_TRY(ensure_smem_limit((const void*)fn, pg::SMEM_LIMIT, "pgemm"));
  const int64_t tiles = ceil_div(M, pg::BM);
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, device_sms());
  fn<<<grid, pg::THREADS, bytes, st>>>(M, N, K, tmA, tmO, bimg, slots, nsb, ea);
  return check_launch("pgemm");
}

// Layer 3 of the backward in one pass over H2 (networks.py:112-121, sigmoid folded
// into dZ3): dH2 = (dZ3 W3^T) * [H2 > 0], dW3 += H2^T dZ3, db3 += sum dZ3,
// db2 += sum dH2. A warp takes four consecutive rows at a time (grid-stride), lane l
// columns 4l..4l+3 of the 128 units; partial sums stay in registers, are reduced
// over the block in shared memory and added once per block.
constexpr int L3_THREADS = 512;
__global__ void __launch_bounds__(L3_THREADS) l3_bwd_kernel(int64_t M, const float* __restrict__ H2,
                                                           const float* __restrict__ dZ3,
                                                           const float* __restrict__ W3, float* __restrict__ dH2,
                                                           float* __restrict__ gW3, float* __restrict__ gb3,
                                                           float* __restrict__ gb2) {
  __shared__ float sW[128 * 3], sB2[128], sB3[4];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 128 * 3; i += L3_THREADS) sW[i] = 0.0f;
  if (tid < 128) sB2[tid] = 0.0f;
  if (tid < 4) sB3[tid] = 0.0f;
  float w[4][3], aw[4][3], ab2[4], ab3[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    ab2[c] = 0.0f;
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      w[c][o] = __ldg(W3 + (4 * lane + c) * 3 + o);
      aw[c][o] = 0.0f;
    }
  }
  __syncthreads();
  const int64_t nwarps = (int64_t)gridDim.x * (L3_THREADS / 32);
  for (int64_t m0 = ((int64_t)blockIdx.x * (L3_THREADS / 32) + warp) * 4; m0 < M; m0 += nwarps * 4) {
    float4 h[4];
    float z[4][3];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int64_t m = m0 + r;
      if (m < M) {
        h[r] = __ldg(reinterpret_cast<const float4*>(H2 + m * 128) + lane);
#pragma unroll
        for (int o = 0; o < 3; ++o) z[r][o] = __ldg(dZ3 + m * 3 + o);
      } else {
        h[r] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int o = 0; o < 3; ++o) z[r][o] = 0.0f;
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float hv[4] = {h[r].x, h[r].y, h[r].z, h[r].w};
      float dv[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float g = z[r][0] * w[c][0] + z[r][1] * w[c][1] + z[r][2] * w[c][2];
        dv[c] = hv[c] > 0.0f ? g : 0.0f;
        ab2[c] += dv[c];
#pragma unroll
        for (int o = 0; o < 3; ++o) aw[c][o] = fmaf(hv[c], z[r][o], aw[c][o]);
      }
#pragma unroll
      for (int o = 0; o < 3; ++o) ab3[o] += z[r][o];
      if (m0 + r < M)
        *reinterpret_cast<float4*>(dH2 + (m0 + r) * 128 + 4 * lane) = make_float4(dv[0], dv[1], dv[2], dv[3]);
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    atomicAdd(&sB2[4 * lane + c], ab2[c]);
#pragma unroll
    for (int o = 0; o < 3; ++o) atomicAdd(&sW[(4 * lane + c) * 3 + o], aw[c][o]);
  }
  if (lane == 0) {
#pragma unroll
    for (int o = 0; o < 3; ++o) atomicAdd(&sB3[o], ab3[o]);
  }
  __syncthreads();
  for (int i = tid; i < 128 * 3; i += L3_THREADS) atomicAdd(gW3 + i, sW[i]);
  if (tid < 128) atomicAdd(gb2 + tid, sB2[tid]);
  if (tid < 3) atomicAdd(gb3 + tid, sB3[tid]);
}

// FiLM camera conditioning after layer 2 (networks.py:103-111): with the row's embedding
// e = embed[camera], units j >= U/2 become e[j - U/2] * h_j + e[j]; the lower half passes
// through. H2f = FiLM(H2), one thread per (row, unit). Camera indices are clamped into
// [0, cams).
__device__ __forceinline__ int film_camera(const int32_t* cams, int64_t row, int rows_per_dir, int ncam) {
  return min(max(__ldg(cams + row / rows_per_dir), 0), ncam - 1);
}

__global__ void film_fwd_kernel(int64_t M, int U, const float* __restrict__ H2, const float* __restrict__ emb,
                                const int32_t* __restrict__ cams, int rows_per_dir, int ncam,
                                float* __restrict__ H2f) {
  const int64_t n = M * U;
  const int half = U / 2;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / U;
    const int j = (int)(e - row * U);
    const float h = H2[e];
    if (j < half) {
      H2f[e] = h;
    } else {
      const float* c = emb + (int64_t)film_camera(cams, row, rows_per_dir, ncam) * U;
      H2f[e] = __ldg(c + j - half) * h + __ldg(c + j);
    }
  }
}

// FiLM backward, in place on dH: dH2f (gradient of the conditioned units) -> dH2, the
// gradient of layer 2's pre-activation (the ReLU mask from H2 applied), and the embedding
// gradient d e[j - U/2] += dH2f_j * h_j, d e[j] += dH2f_j. A block walks FILM_ROWS
// consecutive rows per unit; rows of one ray share its camera, so each thread adds its
// sums to the embedding gradient only when the camera changes.
constexpr int FILM_ROWS = 64;

__global__ void film_bwd_kernel(int64_t M, int U, const float* __restrict__ H2, const float* __restrict__ emb,
                                const int32_t* __restrict__ cams, int rows_per_dir, int ncam, float* __restrict__ dH,
                                float* __restrict__ gemb) {
  const int64_t r0 = (int64_t)blockIdx.x * FILM_ROWS;
  const int64_t r1 = min(M, r0 + FILM_ROWS);
  const int half = U / 2;
  for (int j = threadIdx.x; j < U; j += blockDim.x) {
    int cur = -1;
    float acc_scale = 0.f, acc_shift = 0.f;
    for (int64_t r = r0; r < r1; ++r) {
      const float h = H2[r * U + j];
      float g = dH[r * U + j];
      if (j >= half) {
        const int cam = film_camera(cams, r, rows_per_dir, ncam);
        if (cam != cur) {
          if (cur >= 0) {
            atomicAdd(gemb + (int64_t)cur * U + j - half, acc_scale);
            atomicAdd(gemb + (int64_t)cur * U + j, acc_shift);
          }
          cur = cam;
          acc_scale = acc_shift = 0.f;
        }
        acc_scale += g * h;
        acc_shift += g;
        g *= __ldg(emb + (int64_t)cam * U + j - half);
      }
      dH[r * U + j] = h > 0.f ? g : 0.f;
    }
    if (cur >= 0) {
      atomicAdd(gemb + (int64_t)cur * U + j - half, acc_scale);
      atomicAdd(gemb + (int64_t)cur * U + j, acc_shift);
    }
  }
}

// Workspace carve-out shared by forward and backward. The buffers the forward writes
// come first, so a forward-only carve is a prefix of the full one and a forward
// followed by a backward on the same workspace sees the same addresses.
struct MlpBufs {
  float *X1, *H1, *H2, *dH2, *dH1, *dX1, *dH0;
  uint8_t* wpack;
  uint8_t* img[6];
  uint32_t* mask1;  // ReLU bits of H1 (4 words per row), for the dH1 product
  float* H2f;       // FiLM-conditioned H2 (models with camera embeddings)
};
static MlpBufs carve(const MlpDims& d, int64_t M, Workspace& ws, bool fwd_only) {
  MlpBufs b{};
  if (mlp_fused_supported(d)) {  // the fused kernels keep every activation on chip
    b.wpack = ws.take<uint8_t>((int64_t)mlp_fused_pack_bytes());
    return b;
  }
  if (pmlp_supported(d)) {
    const PmlpImages im = pmlp_images(d);
    for (int i = 0; i < 3; ++i) b.img[i] = ws.take<uint8_t>(im.bytes[i]);
    b.X1 = ws.take<float>(M * pg::LDX1);
    b.H1 = ws.take<float>(M * 128);
    b.H2 = ws.take<float>(M * 128);
    b.mask1 = ws.take<uint32_t>(M * 4);
    if (fwd_only) return b;
    for (int i = 3; i < 6; ++i) b.img[i] = ws.take<uint8_t>(im.bytes[i]);
    b.dH2 = ws.take<float>(M * 128);
    b.dH1 = ws.take<float>(M * 128);
    b.dH0 = ws.take<float>(M * pg::LDH0);
    return b;
  }
  b.X1 = ws.take<float>(M * ld_x1(d));
  b.H1 = ws.take<float>(M * d.units);
  b.H2 = ws.take<float>(M * d.units);
  if (d.cams > 0) b.H2f = ws.take<float>(M * d.units);
  if (fwd_only) return b;
  b.dH2 = ws.take<float>(M * d.units);
  b.dH1 = ws.take<float>(M * d.units);
  b.dX1 = ws.take<float>(M * ld_x1(d));
  b.dH0 = ws.take<float>(M * d.squash);
  return b;
}

size_t mlp_workspace_bytes(const MlpDims& d, int64_t M) {
  Workspace ws{nullptr, 0, 0, true};
  carve(d, M, ws, false);
  return ws.used + 256;
}

size_t mlp_fwd_workspace_bytes(const MlpDims& d, int64_t M) {
  Workspace ws{nullptr, 0, 0, true};
  carve(d, M, ws, true);
  return ws.used + 256;
}

uint8_t* mlp_fused_wpack(Workspace ws) { return ws.take<uint8_t>((int64_t)mlp_fused_pack_bytes()); }

int mlp_forward(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs, const int32_t* cams,
                int rows_per_dir, int64_t M, float* rgb, Workspace& ws, cudaStream_t st, int max_ctas,
                const uint8_t* X0t, bool prepacked) {
  MlpBufs b = carve(d, M, ws, true);
  if (!ws.ok()) {
    set_error("mlp workspace too small");
    return TVM_ERR_WORKSPACE;
  }
  const int l1 = ld_x1(d);
  if (mlp_fused_supported(d)) {
    // BF16: all four layers in one tcgen05 kernel. Nothing is kept for the backward,
    // which recomputes the activations from X0 (only the packed weights are reused).
    return launch_mlp_fwd_fused(d, w, X0, dirs, rows_per_dir, M, rgb, b.wpack, st, max_ctas, X0t, prepacked);
  }
  if (X0t) {
    set_error("mlp: input tiles need the fused BF16 kernels");
    return TVM_ERR_UNSUPPORTED;
  }
  if (pmlp_supported(d)) {
    const pg::PackJob jobs[3] = {{w.w0, d.squash, d.feat, d.squash, pg::kpad(d.feat), 32, 0, b.img[0]},
                                 {w.w1, 128, d.enc, 128, pg::kpad(pg::ENC), 128, 0, b.img[1]},
                                 {w.w2, 128, 128, 128, 128, 128, 0, b.img[2]}};
    TVM_TRY(pack_images(jobs, 3, st));
    if (aligned(X0, 16) && d.feat % 4 == 0) {
      pg::EpiArgs e0{};
      e0.out = b.X1;
      e0.ldo = pg::LDX1;
      e0.dirs = dirs;
      e0.rows_per_dir = rows_per_dir;
      TVM_TRY((pgemm<pg::EPI_PE_FWD, 32>(M, d.squash, d.feat, X0, d.feat, b.img[0], e0, st, pg::ENC)));
    } else {  // features the tensor unit cannot address: layered L0 and encoding
      TVM_TRY((mm<false, false>(d.math, M, d.squash, d.feat, X0, d.feat, w.w0, d.squash, EpiStore{b.X1, pg::LDX1},
                                st)));
      pe_fwd_kernel<<<(unsigned)ceil_div(M, PE_ROWS), 256, 0, st>>>(b.X1, pg::LDX1, M, d.squash, d.enc, d.nf, d.nv,
                                                                     dirs, rows_per_dir);
      TVM_TRY(check_launch("pe_fwd"));
    }
    pg::EpiArgs e1{};
    e1.out = b.H1;
    e1.ldo = 128;
    e1.bias = w.b1;
    e1.mask = b.mask1;
    TVM_TRY((pgemm<pg::EPI_BIAS_RELU, 128>(M, 128, d.enc, b.X1, pg::LDX1, b.img[1], e1, st)));
    pg::EpiArgs e2{};
    e2.out = b.H2;
    e2.ldo = 128;
    e2.bias = w.b2;
    e2.w3 = w.w3;
    e2.b3 = w.b3;
    e2.rgb = rgb;
    return pgemm<pg::EPI_BIAS_RELU_L3, 128>(M, 128, 128, b.H1, 128, b.img[2], e2, st);
  }
  TVM_TRY((mm<false, false>(d.math, M, d.squash, d.feat, X0, d.feat, w.w0, d.squash, EpiStore{b.X1, l1}, st)));
  pe_fwd_kernel<<<(unsigned)ceil_div(M, PE_ROWS), 256, 0, st>>>(b.X1, l1, M, d.squash, d.enc, d.nf, d.nv, dirs,
                                                                 rows_per_dir);
  TVM_TRY(check_launch("pe_fwd"));
  TVM_TRY((mm<false, false>(d.math, M, d.units, d.enc, b.X1, l1, w.w1, d.units,
                              EpiBiasAct{b.H1, d.units, w.b1, 1}, st)));
  TVM_TRY((mm<false, false>(d.math, M, d.units, d.units, b.H1, d.units, w.w2, d.units,
                              EpiBiasAct{b.H2, d.units, w.b2, 1}, st)));
  const float* h2 = b.H2;
  if (d.cams > 0) {
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(M * d.units, 256), 8 * device_sms());
    film_fwd_kernel<<<blocks, 256, 0, st>>>(M, d.units, b.H2, w.embed, cams, rows_per_dir, d.cams, b.H2f);
    TVM_TRY(check_launch("film_fwd"));
    h2 = b.H2f;
  }
  TVM_TRY((mm<false, false>(d.math, M, 3, d.units, h2, d.units, w.w3, 3, EpiBiasAct{rgb, 3, w.b3, 2}, st)));
  return TVM_OK;
}

int mlp_backward(const MlpDims& d, const MlpWeights& w, const MlpGrads& g, const float* X0, const float* dirs,
                 const int32_t* cams, int rows_per_dir, int64_t M, const float* dZ3, float* dX0, Workspace& ws,
                 cudaStream_t st, int max_ctas, const uint8_t* X0t) {
  MlpBufs b = carve(d, M, ws, false);
  if (!ws.ok()) {
    set_error("mlp workspace too small");
    return TVM_ERR_WORKSPACE;
  }
  if (mlp_fused_supported(d)) {
    return launch_mlp_bwd_fused(w, g, X0, dirs, rows_per_dir, M, dZ3, dX0, b.wpack, st, max_ctas, X0t);
  }
  if (X0t) {
    set_error("mlp: input tiles need the fused BF16 kernels");
    return TVM_ERR_UNSUPPORTED;
  }
  const int l1 = ld_x1(d);
  const int64_t kc = -1;  // weight gradients: split-K over the rows, sized per GEMM
  if (pmlp_supported(d)) {
    const int ntx = pmlp_nt_dx0(d);
    const pg::PackJob jobs[3] = {{w.w2, 128, 128, 128, 128, 128, 1, b.img[3]},
                                 {w.w1, 128, 128, pg::PED, 128, PMLP_NT_DX1, 1, b.img[4]},
                                 {w.w0, d.squash, d.squash, d.feat, pg::kpad(pg::SQ), ntx, 1, b.img[5]}};
    TVM_TRY(pack_images(jobs, 3, st));
    if (M > 0) {
      const unsigned blocks = (unsigned)std::min<int64_t>(2 * device_sms(), ceil_div(M, 4 * (L3_THREADS / 32)));
      l3_bwd_kernel<<<blocks, L3_THREADS, 0, st>>>(M, b.H2, dZ3, w.w3, b.dH2, g.w3, g.b3, g.b2);
      TVM_TRY(check_launch("l3_bwd"));
    }
    pg::EpiArgs e1{};
    e1.out = b.dH1;
    e1.ldo = 128;
    e1.mask = b.mask1;
    e1.colsum = g.b1;
    TVM_TRY((pgemm<pg::EPI_MASK_COLSUM, 128>(M, 128, 128, b.dH2, 128, b.img[3], e1, st)));
    TVM_TRY((mm<true, false>(d.math, 128, 128, M, b.H1, 128, b.dH2, 128, EpiAtomic{g.w2, 128}, st, kc)));
    // dW1 = X1^T dH1 is computed transposed (dH1^T X1: the output width is the M of one
    // 128-row tile, so each activation is read once).
    pg::EpiArgs e0{};
    e0.out = b.dH0;
    e0.H = b.X1;
    e0.ldh = pg::LDX1;
    TVM_TRY((pgemm<pg::EPI_PE_BWD, PMLP_NT_DX1>(M, pg::PED, 128, b.dH1, 128, b.img[4], e0, st)));
    TVM_TRY((mm<true, false>(d.math, 128, d.enc, M, b.dH1, 128, b.X1, pg::LDX1, EpiAtomicT{g.w1, 128}, st, kc)));
    TVM_TRY((mm<true, false>(d.math, d.feat, d.squash, M, X0, d.feat, b.dH0, pg::LDH0, EpiAtomic{g.w0, d.squash},
                             st, kc)));
    if (dX0) {
      pg::EpiArgs ex{};
      ex.out = dX0;
      ex.ldo = d.feat;
      if (ntx == 64) {
        TVM_TRY((pgemm<pg::EPI_STORE, 64>(M, d.feat, pg::SQ, b.dH0, pg::LDH0, b.img[5], ex, st)));
      } else if (ntx == 144) {
        TVM_TRY((pgemm<pg::EPI_STORE, 144>(M, d.feat, pg::SQ, b.dH0, pg::LDH0, b.img[5], ex, st)));
      } else {
        TVM_TRY((pgemm<pg::EPI_STORE, 160>(M, d.feat, pg::SQ, b.dH0, pg::LDH0, b.img[5], ex, st)));
      }
    }
    return TVM_OK;
  }
  {
    // Layer 3: dH2 = (dZ3 @ W3^T) * [H2 > 0]; dW3 = H2^T dZ3; db3 = sum dZ3. With camera
    // embeddings layer 3 reads the conditioned H2f, and the FiLM backward turns its
    // gradient into dH2 (mask included) and the embedding gradient.
    if (d.cams > 0) {
      TVM_TRY((mm<false, true>(d.math, M, d.units, 3, dZ3, 3, w.w3, 3, EpiStore{b.dH2, d.units}, st)));
      TVM_TRY((mm<true, false>(d.math, d.units, 3, M, b.H2f, d.units, dZ3, 3, EpiAtomic{g.w3, 3}, st, kc)));
      film_bwd_kernel<<<(unsigned)ceil_div(M, FILM_ROWS), 128, 0, st>>>(M, d.units, b.H2, w.embed, cams, rows_per_dir,
                                                                       d.cams, b.dH2, g.embed);
      TVM_TRY(check_launch("film_bwd"));
    } else {
      TVM_TRY((mm<false, true>(d.math, M, d.units, 3, dZ3, 3, w.w3, 3, EpiReluMask{b.dH2, d.units, b.H2, d.units},
                               st)));
      TVM_TRY((mm<true, false>(d.math, d.units, 3, M, b.H2, d.units, dZ3, 3, EpiAtomic{g.w3, 3}, st, kc)));
    }
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
