// Generic tcgen05 GEMM: D[M x N] = A[M x K] * B[K x N] on the 5th-generation tensor
// cores, fp32 accumulation in TMEM, fused per-element epilogue.
//
// Operands are read from global memory (fp32 or bf16, either orientation) and staged
// into shared memory in the K-major, no-swizzle canonical layout, converted to the MMA
// input format on the way:
//   FMT_BF16  kind::f16,  bf16 inputs, 8 elements per 16-byte chunk, MMA K = 16;
//   FMT_TF32  kind::tf32, tf32 inputs, 4 elements per 16-byte chunk, MMA K = 8.
// SPLIT stages each operand as a hi/lo pair (hi = round(x), lo = round(x - hi)) and
// issues three MMAs per k-step (hi*hi + hi*lo + lo*hi). With tf32 that carries ~22
// significant bits of every input: FP32-level accuracy on the tensor cores.
//
// Tile: 128 rows of D per CTA (one TMEM lane per row) and all N <= NT columns in one
// TMEM accumulator; K in stages of 64 (row-major A) or 128 bytes (transposed A) per row. 256 threads stage; thread 0 issues
// the MMAs and commits to an mbarrier; the global loads of stage s+1 are issued into
// registers before waiting for the MMAs of stage s. TMEM is read back by warps w and
// w+4 (TMEM sub-partition w % 4), each half of the columns. Split-K over gridDim.z.
#pragma once

#include "tvm_tc.cuh"

namespace tvm {

__device__ int g_tc_status;  // sticky: bit 0 = an mbarrier wait gave up

namespace tcg {

constexpr int BM = 128;
constexpr int THREADS = 256;
constexpr int KCH = 8;           // default 16-byte chunks per row per stage (128 bytes)
constexpr int PAD = 8192;        // slack after the operand tiles
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr int FMT_BF16 = 0, FMT_TF32 = 1;

__host__ __device__ constexpr uint32_t ncols_for(int nt) { return nt <= 32 ? 32 : nt <= 64 ? 64 : nt <= 128 ? 128 : 256; }
__host__ __device__ constexpr int epc(int fmt) { return fmt == FMT_BF16 ? 8 : 4; }

template <typename T>
__device__ __forceinline__ float ld1(const T* p);
template <>
__device__ __forceinline__ float ld1<float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ld1<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// Loads one stage (rows [r0, r0+R) x k in [k0, k0 + 8*EPC)) of X into registers and
// writes it to the canonical tile. X(r, k) = KCONTIG ? X[r*ld + k] : X[k*ld + r]; rows
// >= rlim and k >= kend read as zero.
template <int R, bool KCONTIG, typename T, int FMT, int KC = KCH>
struct Stager {
  static constexpr int EPC = epc(FMT);
  static constexpr int CHUNKS = R * KC;
  static constexpr int PER = (CHUNKS + THREADS - 1) / THREADS;
  float v[PER][EPC];

  // KCONTIG: a warp covers 8 rows x 4 chunks, so each 16-byte shared store of the warp
  // fills whole 128-byte core matrices (no bank conflicts) while each row still reads 64
  // contiguous bytes of global memory. Otherwise consecutive lanes take consecutive rows.
  static_assert(!KCONTIG || (R % 8 == 0 && KC % 4 == 0), "row / chunk grouping");
  __device__ __forceinline__ static void chunk_rc(int c, int& r, int& kc) {
    if (KCONTIG) {
      const int grp = c >> 5, lane = c & 31;
      r = 8 * (grp % (R / 8)) + (lane & 7);
      kc = 4 * (grp / (R / 8)) + (lane >> 3);
    } else {
      kc = c / R;
      r = c % R;
    }
  }

  __device__ __forceinline__ void load(const T* __restrict__ X, int64_t ld, int64_t r0, int64_t rlim, int64_t k0,
                                       int64_t kend, int tid) {
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int c = tid + i * THREADS;
      if (c >= CHUNKS) break;
      int r, kc;
      chunk_rc(c, r, kc);
      const int64_t gr = r0 + r;
      const int64_t gk = k0 + kc * EPC;
      if (KCONTIG && gr < rlim && gk + EPC <= kend) {
        const T* p = X + gr * ld + gk;
        if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
          if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int q = 0; q < EPC / 4; ++q) {
              const float4 f = __ldg(reinterpret_cast<const float4*>(p) + q);
              v[i][4 * q] = f.x;
              v[i][4 * q + 1] = f.y;
              v[i][4 * q + 2] = f.z;
              v[i][4 * q + 3] = f.w;
            }
          } else {
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int q = 0; q < EPC / 2; ++q) {
              const float2 f = __bfloat1622float2(h[q]);
              v[i][2 * q] = f.x;
              v[i][2 * q + 1] = f.y;
            }
          }
          continue;
        }
      }
#pragma unroll
      for (int j = 0; j < EPC; ++j) {
        const int64_t k = gk + j;
        v[i][j] = (gr < rlim && k < kend) ? ld1<T>(X + (KCONTIG ? gr * ld + k : k * ld + gr)) : 0.0f;
      }
    }
  }

  template <bool SPLIT>
  __device__ __forceinline__ void store(uint8_t* hi, uint8_t* lo, int tid) const {
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int c = tid + i * THREADS;
      if (c >= CHUNKS) break;
      int r, kc;
      chunk_rc(c, r, kc);
      uint32_t h[4], l[4];
      if (FMT == FMT_BF16) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          __nv_bfloat162 hb = __floats2bfloat162_rn(v[i][2 * j], v[i][2 * j + 1]);
          h[j] = *reinterpret_cast<uint32_t*>(&hb);
          if (SPLIT) {
            const float2 hf = __bfloat1622float2(hb);
            __nv_bfloat162 lb = __floats2bfloat162_rn(v[i][2 * j] - hf.x, v[i][2 * j + 1] - hf.y);
            l[j] = *reinterpret_cast<uint32_t*>(&lb);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          h[j] = tc::to_tf32(v[i][j]);
          if (SPLIT) l[j] = tc::to_tf32(v[i][j] - __uint_as_float(h[j]));
        }
      }
      const int off = (r >> 3) * (KC * 128) + kc * 128 + (r & 7) * 16;
      *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
      if (SPLIT) *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
};

template <int NT, bool SPLIT, int KC = KCH>
struct Smem {
  static constexpr int A_BYTES = BM * KC * 16;
  static constexpr int B_BYTES = NT * KC * 16;
  static constexpr int NPASS = SPLIT ? 2 : 1;
  static constexpr int TILES = NPASS * (A_BYTES + B_BYTES);
  static constexpr int TOTAL = TILES + PAD + 64;
  // (CTAs per SM allowed by shared memory) * TMEM columns <= 512, so tcgen05.alloc
  // never waits for another CTA.
  static constexpr int MAX_CTAS = 512 / (int)ncols_for(NT);
  static constexpr int FLOOR = 232448 / (MAX_CTAS + 1) + 1024;
  static constexpr int BYTES = TOTAL > FLOOR ? TOTAL : FLOOR;
};

template <int NT, bool AT, bool BT, typename TA, typename TB, int FMT, bool SPLIT, class Epi, int KC>
__global__ void __launch_bounds__(THREADS) tc_gemm_kernel(int64_t M, int N, int64_t K, const TA* __restrict__ A,
                                                        int64_t lda, const TB* __restrict__ B, int64_t ldb,
                                                        int64_t kc, Epi epi) {
  using S = Smem<NT, SPLIT, KC>;
  constexpr int EPC = epc(FMT);
  constexpr int BK = KC * EPC;                  // K elements per stage
  constexpr int KSTEP = (FMT == FMT_BF16) ? 16 : 8;
  constexpr uint32_t NCOLS = ncols_for(NT);
  constexpr uint32_t IDESC = tc::idesc(BM, NT, FMT == FMT_BF16 ? 1u : 2u);
  constexpr uint32_t SBO = KC * 128;   // next 8-row group
  constexpr uint32_t LBO = 128;        // next core matrix along K
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sB_hi = smem;
  uint8_t* sB_lo = smem + S::B_BYTES;
  uint8_t* sA_hi = smem + S::NPASS * S::B_BYTES;
  uint8_t* sA_lo = sA_hi + S::A_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + S::TILES + PAD);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.y * BM;
  const int64_t n0 = (int64_t)blockIdx.x * NT;
  const int64_t kbeg = (int64_t)blockIdx.z * kc;
  const int64_t kend = kbeg + kc < K ? kbeg + kc : K;
  const int nst = kend > kbeg ? (int)((kend - kbeg + BK - 1) / BK) : 0;

  if (warp == 0) tc::tmem_alloc(tmem_slot, NCOLS);
  if (tid == 0) tc::mbar_init(mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const TB* Bn = BT ? B + n0 * ldb : B + n0;  // this CTA's column block
  const int64_t nlim = (int64_t)N - n0;
  Stager<BM, !AT, TA, FMT, KC> sa;
  Stager<NT, BT, TB, FMT, KC> sb;
  uint32_t phase = 0;
  int ok = 1;
  if (nst > 0) {
    sa.load(A, lda, m0, M, kbeg, kend, tid);
    sb.load(Bn, ldb, 0, nlim, kbeg, kend, tid);
  }
  for (int it = 0; it < nst; ++it) {
    if (it > 0) {  // the MMAs of the previous stage must be done before smem is reused
      const int done = tc::mbar_wait(mbar, phase, WAIT_LIMIT) ? 1 : 0;
      ok = __syncthreads_and(done);
      tc::fence_after_sync();
      if (!ok) break;
      phase ^= 1u;
    }
    sa.template store<SPLIT>(sA_hi, sA_lo, tid);
    sb.template store<SPLIT>(sB_hi, sB_lo, tid);
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t a_hi = tc::smem_u32(sA_hi), a_lo = tc::smem_u32(sA_lo);
      const uint32_t b_hi = tc::smem_u32(sB_hi), b_lo = tc::smem_u32(sB_lo);
#pragma unroll
      for (int s = 0; s < BK / KSTEP; ++s) {
        const uint64_t ah = tc::sdesc(a_hi + s * 256, LBO, SBO), bh = tc::sdesc(b_hi + s * 256, LBO, SBO);
        const uint32_t acc = (it > 0 || s > 0) ? 1u : 0u;
        if (FMT == FMT_BF16) {
          tc::mma_bf16(tmem, ah, bh, IDESC, acc);
        } else {
          tc::mma_tf32(tmem, ah, bh, IDESC, acc);
        }
        if (SPLIT) {
          const uint64_t al = tc::sdesc(a_lo + s * 256, LBO, SBO), bl = tc::sdesc(b_lo + s * 256, LBO, SBO);
          if (FMT == FMT_BF16) {
            tc::mma_bf16(tmem, ah, bl, IDESC, 1u);
            tc::mma_bf16(tmem, al, bh, IDESC, 1u);
          } else {
            tc::mma_tf32(tmem, ah, bl, IDESC, 1u);
            tc::mma_tf32(tmem, al, bh, IDESC, 1u);
          }
        }
      }
      tc::mma_commit(mbar);
    }
    if (it + 1 < nst) {  // next stage's global loads overlap the MMAs just issued
      sa.load(A, lda, m0, M, kbeg + (int64_t)(it + 1) * BK, kend, tid);
      sb.load(Bn, ldb, 0, nlim, kbeg + (int64_t)(it + 1) * BK, kend, tid);
    }
  }
  if (ok && nst > 0) {
    const int done = tc::mbar_wait(mbar, phase, WAIT_LIMIT) ? 1 : 0;
    ok = __syncthreads_and(done);
    tc::fence_after_sync();
  }

  if (ok && nst > 0) {
    // TMEM -> registers (thread t of warp w holds row 32*(w%4) + t) -> a per-warp
    // 32 x 16 shared buffer -> rows written four columns per thread, so each warp store
    // covers whole 32-byte sectors. The operand tiles are free once the last MMA is done.
    const int sub = warp & 3;
    float* buf = reinterpret_cast<float*>(smem) + warp * (32 * 17);
    constexpr int CH = (NT + 15) / 16;
    const int c_begin = (warp < 4) ? 0 : (CH + 1) / 2;
    const int c_end = (warp < 4) ? (CH + 1) / 2 : CH;
    for (int ch = c_begin; ch < c_end; ++ch) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)(ch * 16), v);
#pragma unroll
      for (int j = 0; j < 16; ++j) buf[lane * 17 + j] = v[j];
      __syncwarp();
      if constexpr (Epi::kColumns) {
        // Four consecutive rows of one column per thread (the epilogue writes D^T).
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int idx = q * 32 + lane;
          const int c = idx >> 3, r4 = (idx & 7) * 4;
          const int64_t row = m0 + sub * 32 + r4;
          const int64_t col = n0 + ch * 16 + c;
          if (row < M && col < N) {
            const float w4[4] = {buf[r4 * 17 + c], buf[(r4 + 1) * 17 + c], buf[(r4 + 2) * 17 + c],
                                 buf[(r4 + 3) * 17 + c]};
            epi.vec4_col(row, (int)col, w4, M);
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int idx = q * 32 + lane;
          const int r = idx >> 2, c4 = (idx & 3) * 4;
          const int64_t row = m0 + sub * 32 + r;
          const int64_t col = n0 + ch * 16 + c4;
          if (row < M && col < N) {
            const float w4[4] = {buf[r * 17 + c4], buf[r * 17 + c4 + 1], buf[r * 17 + c4 + 2], buf[r * 17 + c4 + 3]};
            epi.vec4(row, (int)col, w4, N);
          }
        }
      }
      __syncwarp();
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(&g_tc_status, 1);
    tc::mbar_wait(mbar, phase, WAIT_LIMIT);  // let in-flight MMAs drain before TMEM is freed
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, NCOLS);
  }
}

}  // namespace tcg

// Host wrapper with the operand conventions of the SIMT gemm():
// A(m,k) = AT ? A[k*lda + m] : A[m*lda + k]; B(k,n) = BT ? B[n*ldb + k] : B[k*ldb + n].
// kc > 0 splits K into chunks of kc across gridDim.z (the epilogue must accumulate).
template <bool AT, bool BT, int FMT, bool SPLIT, typename TA, typename TB, class Epi>
static int tc_gemm(int64_t M, int N, int64_t K, const TA* A, int64_t lda, const TB* B, int64_t ldb, Epi epi,
                   cudaStream_t st, int64_t kc = 0) {
  if (M == 0 || N == 0 || K == 0) return TVM_OK;
  if (kc <= 0) kc = K;
  const unsigned gz = (unsigned)ceil_div(K, kc);
  auto launch = [&](auto nt_tag) -> int {
    constexpr int NT = decltype(nt_tag)::value;
    // Row-major A streams 64-byte stages (smaller tiles, one more CTA per SM); the
    // transposed-A weight-gradient products keep 128-byte stages.
    constexpr int KC = AT ? 8 : 4;
    using S = tcg::Smem<NT, SPLIT, KC>;
    auto fn = tcg::tc_gemm_kernel<NT, AT, BT, TA, TB, FMT, SPLIT, Epi, KC>;
    TVM_TRY(ensure_smem_limit((const void*)fn, S::BYTES, "tc_gemm"));
    dim3 grid((unsigned)ceil_div(N, NT), (unsigned)ceil_div(M, tcg::BM), gz);
    fn<<<grid, tcg::THREADS, S::BYTES, st>>>(M, N, K, A, lda, B, ldb, kc, epi);
    return check_launch("tc_gemm");
  };
  if (N <= 16) return launch(std::integral_constant<int, 16>{});
  if (N <= 32) return launch(std::integral_constant<int, 32>{});
  if (N <= 128) return launch(std::integral_constant<int, 128>{});
  if (N <= 160) return launch(std::integral_constant<int, 160>{});
  return launch(std::integral_constant<int, 256>{});
}

// Split-K chunk for a K-long reduction onto an M x N output: one resident wave (152 SMs
// x 3 CTAs) of equal chunks, so no SM runs a tail wave and each CTA adds its partial
// tile to global memory once.
static inline int64_t splitk_chunk(int64_t M, int64_t K) {
  const int64_t mtiles = ceil_div(M, 128);
  const int64_t want = std::max<int64_t>(1, 456 / mtiles);
  return std::max<int64_t>(256, round_up(ceil_div(K, want), 32));
}

}  // namespace tvm
