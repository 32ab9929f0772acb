// Fused FeatureMlp forward for BF16 models on the tcgen05 tensor cores
// (networks.py:45-121, 2-frequency encodings: 144 -> 27 -> PE 150 -> 128 -> 128 -> 3).
//
// Persistent CTAs (one per SM, 256 threads). The four weight matrices are staged once
// per CTA into shared memory as bf16 B operands (K-major canonical layout, N padded to
// a multiple of 16, K to a multiple of 16). Per 128-row tile:
//   X0 (fp32, global) -> bf16 A tile -> MMA L0 (N=32, K=144) -> TMEM D0
//   tcgen05.ld D0 -> Fourier encoding in registers -> bf16 X1 tile (K=160)
//   MMA L1 (N=128, K=160) -> D1 -> +b1, ReLU -> bf16 H1 tile (reuses the X0 tile)
//   MMA L2 (N=128, K=128) -> D2 -> +b2, ReLU -> bf16 H2 tile (reuses the X1 tile)
//   MMA L3 (N=16,  K=128) -> D3 -> +b3, sigmoid -> rgb (global)
// Activations never leave the SM, except X1 / H1 / H2 in fp32 when a backward follows
// (the layered backward reads them). One elected thread issues the MMAs and commits to an
// mbarrier; every wait is bounded and reports through the device status word.
#include "tvm_internal.h"
#include "tvm_tc.cuh"

namespace tvm {

static __device__ int g_fused_status;  // sticky: bit 0 = a bounded wait gave up

namespace fmlp {

constexpr int BM = 128;
constexpr int THREADS = 256;
constexpr int F = 144;                 // 3 * 48 appearance features
constexpr int SQ = 27, SQP = 32;       // squash width, padded N of L0
constexpr int ENC = 150, ENCP = 160;   // encoded width, padded K of L1
constexpr int U = 128;                 // hidden units
constexpr int OUTP = 16;               // padded N of L3
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr float kHalfPi = 1.57079632679489661923f;

// Shared-memory map (bytes). SBO of a tile = (K / 8) * 128.
constexpr int SBO_F = (F / 8) * 128, SBO_E = (ENCP / 8) * 128, SBO_U = (U / 8) * 128;
constexpr int OFF_W0 = 0;                              // 32 x 144
constexpr int OFF_W1 = OFF_W0 + SQP * F * 2;           // 128 x 160
constexpr int OFF_W2 = OFF_W1 + U * ENCP * 2;          // 128 x 128
constexpr int OFF_W3 = OFF_W2 + U * U * 2;             // 16 x 128
constexpr int OFF_A0 = OFF_W3 + OUTP * U * 2;          // X0 (128 x 144) / H1 (128 x 128)
constexpr int OFF_A1 = OFF_A0 + BM * F * 2;            // X1 (128 x 160) / H2 (128 x 128)
constexpr int OFF_END = OFF_A1 + BM * ENCP * 2;
constexpr int PAD = 16384;                             // slack after the last tile
constexpr int OFF_BAR = OFF_END + PAD;
constexpr int SMEM = OFF_BAR + 64;
constexpr int WPACK_BYTES = OFF_A0;  // bf16 weight images W0..W3, laid out as in shared memory

__device__ __forceinline__ int coff(int row, int kchunk, int sbo) { return (row >> 3) * sbo + kchunk * 128 + (row & 7) * 16; }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// B operand from a row-major (in, out) fp32 weight: B(n, k) = W[k * ld + n], zero
// outside [0, nvalid) x [0, kvalid).
__device__ void stage_weight(uint8_t* dst, const float* __restrict__ W, int ld, int nrows, int kpad, int nvalid,
                             int kvalid, int tid, int nthreads) {
  const int kc_n = kpad / 8, sbo = kc_n * 128;
  for (int c = tid; c < nrows * kc_n; c += nthreads) {
    const int n = c % nrows, kc = c / nrows;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = kc * 8 + e;
      v[e] = (n < nvalid && k < kvalid) ? __ldg(W + (int64_t)k * ld + n) : 0.0f;
    }
    *reinterpret_cast<uint4*>(dst + coff(n, kc, sbo)) =
        make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
  }
}

__device__ __forceinline__ void issue(uint32_t tmem_d, uint32_t a, uint32_t b, int ksteps, uint32_t sbo_a,
                                      uint32_t sbo_b, uint32_t idesc) {
#pragma unroll 1
  for (int s = 0; s < ksteps; ++s) {
    const uint64_t ad = tc::sdesc(a + s * 256, 128, sbo_a);
    const uint64_t bd = tc::sdesc(b + s * 256, 128, sbo_b);
    tc::mma_bf16(tmem_d, ad, bd, idesc, s > 0 ? 1u : 0u);
  }
}

// Packs the four weight matrices into their shared-memory images (bf16, canonical
// layout) once per forward call; every CTA then fetches them with one bulk copy.
__global__ void pack_weights_kernel(uint8_t* __restrict__ out, const float* __restrict__ w0,
                                    const float* __restrict__ w1, const float* __restrict__ w2,
                                    const float* __restrict__ w3) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, n = gridDim.x * blockDim.x;
  stage_weight(out + OFF_W0, w0, SQ, SQP, F, SQ, F, tid, n);
  stage_weight(out + OFF_W1, w1, U, U, ENCP, U, ENC, tid, n);
  stage_weight(out + OFF_W2, w2, U, U, U, U, U, tid, n);
  stage_weight(out + OFF_W3, w3, 3, OUTP, U, 3, U, tid, n);
}

struct Args {
  int64_t M;
  const uint8_t* wpack;  // WPACK_BYTES of packed weights (16-byte aligned)
  const float* X0;     // (M, 144)
  const float* dirs;   // view direction of row m: dirs[(m / rows_per_dir) * 3 ...]
  int rows_per_dir;
  const float *w0, *w1, *b1, *w2, *b2, *w3, *b3;
  float* rgb;          // (M, 3)
  float* X1;           // optional feature-major fp32 copies for the backward:
  float* H1;           // X1 [ENC][M], H1 [U][M], H2 [U][M] (a warp's lanes hold
  float* H2;           // consecutive rows, so each store is one 128-byte line)
};

__global__ void __launch_bounds__(THREADS, 1) mlp_fwd_fused_kernel(Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + OFF_BAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = warp & 3, half = warp >> 2;

  uint64_t* wbar = mbar + 2;
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_init(wbar, 1);
  }
  __syncthreads();
  if (tid == 0) {  // one TMA bulk copy brings all weights in
    tc::mbar_expect_tx(wbar, WPACK_BYTES);
    tc::bulk_g2s(smem + OFF_W0, a.wpack, WPACK_BYTES, wbar);
  }
  int ok = tc::mbar_wait(wbar, 0, WAIT_LIMIT) ? 1 : 0;
  ok = __syncthreads_and(ok);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t D0 = tmem, D1 = tmem + 32, D2 = tmem + 160, D3 = tmem + 288;
  const uint32_t lane_off = (uint32_t)(sub * 32) << 16;
  const uint32_t sbase = tc::smem_u32(smem);
  uint32_t phase = 0;

  // Issue the MMAs of one layer from thread 0 and wait for them (all threads).
  auto layer = [&](uint32_t d, int a_off, int b_off, int ksteps, uint32_t sbo_a, uint32_t sbo_b, int n) -> bool {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      issue(d, sbase + a_off, sbase + b_off, ksteps, sbo_a, sbo_b, tc::idesc(BM, n, 1u));
      tc::mma_commit(mbar);
    }
    const int done = tc::mbar_wait(mbar, phase, WAIT_LIMIT) ? 1 : 0;
    phase ^= 1u;
    const int all = __syncthreads_and(done);
    tc::fence_after_sync();
    return all != 0;
  };

  const int64_t ntiles = (a.M + BM - 1) / BM;
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t m0 = tile * BM;
    // X0 tile: 128 rows x 18 chunks of 8 features.
    for (int c = tid; c < BM * (F / 8); c += THREADS) {
      const int r = c / (F / 8), kc = c % (F / 8);
      const int64_t row = m0 + r;
      float4 p = make_float4(0.f, 0.f, 0.f, 0.f), q = p;
      if (row < a.M) {
        const float4* src = reinterpret_cast<const float4*>(a.X0 + row * F + kc * 8);
        p = __ldg(src);
        q = __ldg(src + 1);
      }
      *reinterpret_cast<uint4*>(smem + OFF_A0 + coff(r, kc, SBO_F)) =
          make_uint4(pack2(p.x, p.y), pack2(p.z, p.w), pack2(q.x, q.y), pack2(q.z, q.w));
    }
    if (!layer(D0, OFF_A0, OFF_W0, F / 16, SBO_F, SBO_F, SQP)) { ok = 0; break; }

    // Fourier encoding (networks.py:13-35, 68-76), row r = 32*sub + lane. X1 columns:
    // [h (27) | d (3) | PE(h): 4 per feature | PE(d): 4 per axis | zero pad to 160], PE(v)
    // = [sin v, sin 2v, sin(v + pi/2), sin(2v + pi/2)] computed as [s, 2sc, c, c^2 - s^2]
    // from one sincos. Warp half 0 encodes features 0..13, half 1 features 14..26, the
    // direction and the padding. Each value is one 2-byte store at its canonical position.
    {
      const int r = sub * 32 + lane;
      const int64_t row = m0 + r;
      uint8_t* xrow = smem + OFF_A1 + (r >> 3) * SBO_E + (r & 7) * 16;
      auto put = [&](int col, float v) {
        *reinterpret_cast<__nv_bfloat16*>(xrow + (col >> 3) * 128 + (col & 7) * 2) = __float2bfloat16_rn(v);
        if (a.X1 && row < a.M) a.X1[(int64_t)col * a.M + row] = v;
      };
      auto pe4 = [&](int col, float v) {
        float sn, cs;
        __sincosf(v, &sn, &cs);
        put(col, sn);
        put(col + 1, 2.0f * sn * cs);
        put(col + 2, cs);
        put(col + 3, cs * cs - sn * sn);
      };
      float v16[16];
      if (half == 0) {
        tc::tmem_ld16(D0 + lane_off, v16);
#pragma unroll
        for (int j = 0; j < 14; ++j) {
          put(j, v16[j]);
          pe4(SQ + 3 + 4 * j, v16[j]);
        }
      } else {
        tc::tmem_ld16(D0 + lane_off, v16);  // columns 0..15: 14 and 15 are this half's
        const float h14 = v16[14], h15 = v16[15];
        tc::tmem_ld16(D0 + lane_off + 16, v16);
        put(14, h14);
        pe4(SQ + 3 + 4 * 14, h14);
        put(15, h15);
        pe4(SQ + 3 + 4 * 15, h15);
#pragma unroll
        for (int j = 16; j < SQ; ++j) {
          put(j, v16[j - 16]);
          pe4(SQ + 3 + 4 * j, v16[j - 16]);
        }
        float d[3] = {0.f, 0.f, 0.f};
        if (row < a.M) {
          const float* dp = a.dirs + (row / a.rows_per_dir) * 3;
          d[0] = __ldg(dp);
          d[1] = __ldg(dp + 1);
          d[2] = __ldg(dp + 2);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          put(SQ + q, d[q]);
          pe4(SQ + 3 + 4 * SQ + 4 * q, d[q]);
        }
#pragma unroll
        for (int c = ENC; c < ENCP; ++c)
          *reinterpret_cast<__nv_bfloat16*>(xrow + (c >> 3) * 128 + (c & 7) * 2) = __float2bfloat16_rn(0.f);
      }
    }
    if (!layer(D1, OFF_A1, OFF_W1, ENCP / 16, SBO_E, SBO_E, U)) { ok = 0; break; }

    // Hidden layers: +bias, ReLU, bf16 into the next A tile (and fp32 to global).
    auto hidden = [&](uint32_t Dsrc, const float* bias, int dst_off, float* gout) {
      const int r = sub * 32 + lane;
      const int64_t row = m0 + r;
      for (int ch = half * 4; ch < half * 4 + 4; ++ch) {
        float v[16];
        tc::tmem_ld16(Dsrc + lane_off + ch * 16, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j] + __ldg(bias + ch * 16 + j), 0.f);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          *reinterpret_cast<uint4*>(smem + dst_off + coff(r, ch * 2 + q, SBO_U)) =
              make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                         pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
        }
        if (gout && row < a.M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) gout[(int64_t)(ch * 16 + j) * a.M + row] = v[j];
        }
      }
    };
    hidden(D1, a.b1, OFF_A0, a.H1);
    if (!layer(D2, OFF_A0, OFF_W2, U / 16, SBO_U, SBO_U, U)) { ok = 0; break; }
    hidden(D2, a.b2, OFF_A1, a.H2);
    if (!layer(D3, OFF_A1, OFF_W3, U / 16, SBO_U, SBO_U, OUTP)) { ok = 0; break; }
    if (half == 0) {
      const int r = sub * 32 + lane;
      const int64_t row = m0 + r;
      float v[16];
      tc::tmem_ld16(D3 + lane_off, v);
      if (row < a.M) {
#pragma unroll
        for (int c = 0; c < 3; ++c) a.rgb[row * 3 + c] = 1.0f / (1.0f + expf(-(v[c] + __ldg(a.b3 + c))));
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (!ok) {
    if (tid == 0) atomicOr(&g_fused_status, 1);
    tc::mbar_wait(wbar, 0, WAIT_LIMIT);           // the weight copy, if it is still in flight
    tc::mbar_wait(mbar, phase ^ 1u, WAIT_LIMIT);  // drain the MMAs in flight before freeing TMEM
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

}  // namespace fmlp

int fused_status(int32_t* out, cudaStream_t st) {
  int32_t v = 0;
  const int32_t zero = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_fused_status, sizeof(int32_t), 0, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(g_fused_status, &zero, sizeof(int32_t), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_error("fused_status: %s", cudaGetErrorString(e));
    return TVM_ERR_LAUNCH;
  }
  *out = v;
  return TVM_OK;
}

bool mlp_fused_supported(const MlpDims& d) {
  return d.math == 0 && d.feat == fmlp::F && d.squash == fmlp::SQ && d.enc == fmlp::ENC && d.units == fmlp::U;
}

size_t mlp_fused_pack_bytes() { return fmlp::WPACK_BYTES; }

int launch_mlp_fwd_fused(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs, int rows_per_dir,
                         int64_t M, float* rgb, float* X1, float* H1, float* H2, uint8_t* wpack, cudaStream_t st) {
  if (M == 0) return TVM_OK;
  static int sms = 0;
  static bool attr = false;
  if (!attr) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(fmlp::mlp_fwd_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         fmlp::SMEM);
    if (e != cudaSuccess) {
      set_error("fused mlp smem attribute: %s", cudaGetErrorString(e));
      return TVM_ERR_LAUNCH;
    }
    attr = true;
  }
  if (!aligned(wpack, 16)) {
    set_error("packed weights must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  fmlp::pack_weights_kernel<<<64, 256, 0, st>>>(wpack, w.w0, w.w1, w.w2, w.w3);
  TVM_TRY(check_launch("pack_weights"));
  fmlp::Args a{M, wpack, X0, dirs, rows_per_dir, w.w0, w.w1, w.b1, w.w2, w.b2, w.w3, w.b3, rgb, X1, H1, H2};
  const int64_t ntiles = ceil_div(M, fmlp::BM);
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, std::max(sms, 1));
  fmlp::mlp_fwd_fused_kernel<<<grid, fmlp::THREADS, fmlp::SMEM, st>>>(a);
  return check_launch("mlp_fwd_fused");
}

}  // namespace tvm
