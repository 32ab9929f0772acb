// Fused FeatureMlp forward for BF16 models on the tcgen05 tensor cores
// (networks.py:45-121, 2-frequency encodings: 144 -> 27 -> PE 150 -> 128 -> 128 -> 3).
//
// Persistent CTAs (one per SM, 256 threads). The four weight matrices are staged once
// per CTA into shared memory as bf16 B operands (K-major canonical layout, N padded to
// a multiple of 16, K to a multiple of 16). Per 128-row tile:
//   X0 -> bf16 A tile (one bulk copy of an input tile, or fp32 rows through registers)
//      -> MMA L0 (N=32, K=144) -> TMEM D0
//   tcgen05.ld D0 -> Fourier encoding in registers -> bf16 X1 tile (K=160)
//   MMA L1 (N=128, K=160) -> D1 -> +b1, ReLU -> bf16 H1 tile (reuses the X0 tile)
//   MMA L2 (N=128, K=128) -> D2 -> +b2, ReLU -> bf16 H2 tile (reuses the X1 tile)
//   MMA L3 (N=16,  K=128) -> D3 -> +b3, sigmoid -> rgb (global)
// Activations never leave the SM (the fused backward recomputes them). One elected thread
// issues the MMAs and commits to an mbarrier; every wait is bounded and reports through
// the device status word.
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

// One 128-row tile of X0 (fp32, global) into a bf16 A tile (K-major canonical, SBO
// sbo) at dst; rows at or past M are zero. Each thread issues all of its loads before
// its first shared-memory store, so the tile costs one L2 round trip, not nine. The two
// halves (x0_fetch: loads into registers, x0_store: conversion and stores) also let a
// caller keep the next tile's loads in flight while it waits for an MMA.
constexpr int X0_PER_THREAD = BM * (F / 8) / THREADS;
static_assert(BM * (F / 8) % THREADS == 0, "whole chunks per thread");

__device__ __forceinline__ void x0_fetch(float4 (&p)[X0_PER_THREAD], float4 (&q)[X0_PER_THREAD], const float* X0,
                                         int64_t m0, int64_t M, int tid) {
#pragma unroll
  for (int i = 0; i < X0_PER_THREAD; ++i) {
    const int c = tid + i * THREADS;
    const int64_t row = m0 + c / (F / 8);
    p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    q[i] = p[i];
    if (row < M) {
      const float4* src = reinterpret_cast<const float4*>(X0 + row * F + (c % (F / 8)) * 8);
      p[i] = __ldg(src);
      q[i] = __ldg(src + 1);
    }
  }
}

__device__ __forceinline__ void x0_store(const float4 (&p)[X0_PER_THREAD], const float4 (&q)[X0_PER_THREAD],
                                         uint8_t* dst, int sbo, int tid) {
#pragma unroll
  for (int i = 0; i < X0_PER_THREAD; ++i) {
    const int c = tid + i * THREADS;
    *reinterpret_cast<uint4*>(dst + coff(c / (F / 8), c % (F / 8), sbo)) =
        make_uint4(pack2(p[i].x, p[i].y), pack2(p[i].z, p[i].w), pack2(q[i].x, q[i].y), pack2(q[i].z, q[i].w));
  }
}

__device__ __forceinline__ void load_x0_tile(uint8_t* dst, int sbo, const float* X0, int64_t m0, int64_t M,
                                             int tid) {
  constexpr int PER_THREAD = X0_PER_THREAD;
  float4 p[PER_THREAD], q[PER_THREAD];
#pragma unroll
  for (int i = 0; i < PER_THREAD; ++i) {
    const int c = tid + i * THREADS;
    const int64_t row = m0 + c / (F / 8);
    p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    q[i] = p[i];
    if (row < M) {
      const float4* src = reinterpret_cast<const float4*>(X0 + row * F + (c % (F / 8)) * 8);
      p[i] = __ldg(src);
      q[i] = __ldg(src + 1);
    }
  }
#pragma unroll
  for (int i = 0; i < PER_THREAD; ++i) {
    const int c = tid + i * THREADS;
    *reinterpret_cast<uint4*>(dst + coff(c / (F / 8), c % (F / 8), sbo)) =
        make_uint4(pack2(p[i].x, p[i].y), pack2(p[i].z, p[i].w), pack2(q[i].x, q[i].y), pack2(q[i].z, q[i].w));
  }
}

// Fourier encoding of one row (networks.py:13-35, 68-76) into its K-chunks of the X1
// tile. Columns: [h (27) | d (3) | PE(h): 4 per feature | PE(d): 4 per axis | `tail` at
// column 150 | zeros to 160], PE(v) = [sin v, sin 2v, sin(v + pi/2), sin(2v + pi/2)]
// computed as [s, 2sc, c, c^2 - s^2] from one sincos. v = [h0..h26, d0..d2]. Warp half
// HALF writes chunks 10*HALF .. 10*HALF + 9, each with one 16-byte store: 2-byte stores
// at the canonical positions of eight rows apart meet in the same banks.
__device__ __forceinline__ float enc_value(int c, const float (&v)[SQ + 3], const float (&sn)[SQ + 3],
                                           const float (&cs)[SQ + 3], float tail) {
  if (c < SQ + 3) return v[c];
  if (c < ENC) {
    const int f = (c - SQ - 3) >> 2, q = (c - SQ - 3) & 3;
    return q == 0 ? sn[f] : q == 1 ? 2.0f * sn[f] * cs[f] : q == 2 ? cs[f] : cs[f] * cs[f] - sn[f] * sn[f];
  }
  return c == ENC ? tail : 0.0f;
}

template <int HALF>
__device__ __forceinline__ void encode_row(uint8_t* xrow, const float (&v)[SQ + 3], float tail) {
  constexpr int K0 = HALF * (ENCP / 16);                          // first K-chunk of this half
  constexpr int F0 = (K0 * 8 - SQ - 3) > 0 ? (K0 * 8 - SQ - 3) / 4 : 0;
  constexpr int F1c = ((K0 + ENCP / 16) * 8 - SQ - 3 + 3) / 4;   // features whose PE these chunks hold
  constexpr int F1 = F1c < SQ + 3 ? F1c : SQ + 3;
  float sn[SQ + 3], cs[SQ + 3];
#pragma unroll
  for (int f = F0; f < F1; ++f) __sincosf(v[f], &sn[f], &cs[f]);
#pragma unroll
  for (int k = K0; k < K0 + ENCP / 16; ++k) {
    float e[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) e[i] = enc_value(8 * k + i, v, sn, cs, tail);
    *reinterpret_cast<uint4*>(xrow + k * 128) =
        make_uint4(pack2(e[0], e[1]), pack2(e[2], e[3]), pack2(e[4], e[5]), pack2(e[6], e[7]));
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

static_assert(X0T_ROWS == BM && X0T_FEAT == F && X0T_SBO == SBO_F, "input tiles are the A0 image");

struct Args {
  int64_t M;
  const uint8_t* wpack;  // WPACK_BYTES of packed weights (16-byte aligned)
  const float* X0;     // (M, 144), or
  const uint8_t* X0t;  // the same as input tiles (TILES kernels)
  const float* dirs;   // view direction of row m: dirs[(m / rows_per_dir) * 3 ...]
  int rows_per_dir;
  const float *w0, *w1, *b1, *w2, *b2, *w3, *b3;
  float* rgb;          // (M, 3)
};

// TILES: X0 arrives as input tiles, one bulk copy per tile into A0 (issued as soon as
// layer 2 has read H1 from A0, waited for before layer 0). Otherwise from the row-major
// fp32 X0 through registers.
template <bool TILES>
__global__ void __launch_bounds__(THREADS, 1) mlp_fwd_fused_kernel(Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + OFF_BAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = warp & 3, half = warp >> 2;

  uint64_t* wbar = mbar + 2;
  uint64_t* xbar = mbar + 3;  // input tile copies (TILES)
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_init(wbar, 1);
    tc::mbar_init(xbar, 1);
  }
  __syncthreads();
  const int64_t ntiles = (a.M + BM - 1) / BM;
  if (tid == 0) {  // one TMA bulk copy brings all weights in (and the first input tile)
    tc::mbar_expect_tx(wbar, WPACK_BYTES);
    tc::bulk_g2s(smem + OFF_W0, a.wpack, WPACK_BYTES, wbar);
    if (TILES && (int64_t)blockIdx.x < ntiles) {
      tc::mbar_expect_tx(xbar, (uint32_t)X0T_TILE_BYTES);
      tc::bulk_g2s(smem + OFF_A0, a.X0t + (int64_t)blockIdx.x * X0T_TILE_BYTES, (uint32_t)X0T_TILE_BYTES, xbar);
    }
  }
  // Row-major X0: the first tile (128 rows x 18 chunks of 8 features) is loaded while the
  // weights travel; each later one is fetched into registers during layer 1's epilogue
  // and layer 2's MMA and stored into the A0 tile once that MMA has read H1 from it.
  if (!TILES && (int64_t)blockIdx.x < ntiles)
    load_x0_tile(smem + OFF_A0, SBO_F, a.X0, (int64_t)blockIdx.x * BM, a.M, tid);
  bool x_pending = TILES && (int64_t)blockIdx.x < ntiles;  // a tile copy not yet waited for
  uint32_t xphase = 0;
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

  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t m0 = tile * BM;
    const int64_t next = tile + gridDim.x;
    {  // the tile after the next one travels to L2 while this tile computes
      const int64_t nt = next + gridDim.x, nm0 = nt * BM;
      if (nm0 < a.M) {
        const char* src = TILES ? reinterpret_cast<const char*>(a.X0t + nt * X0T_TILE_BYTES)
                                : reinterpret_cast<const char*>(a.X0 + nm0 * F);
        const int64_t nbytes = TILES ? X0T_TILE_BYTES : (a.M - nm0 < BM ? a.M - nm0 : BM) * F * 4;
        for (int64_t off = (int64_t)tid * 128; off < nbytes; off += THREADS * 128) tc::prefetch_l2(src + off);
      }
    }
    if (TILES) {  // this tile's input, copied in during the previous tile
      const int got = tc::mbar_wait(xbar, xphase, WAIT_LIMIT) ? 1 : 0;
      if (!__syncthreads_and(got)) { ok = 0; break; }
      xphase ^= 1u;
      x_pending = false;
    }
    // The row's view direction, read now so that its latency passes under layer 0.
    float dir[3] = {0.f, 0.f, 0.f};
    {
      const int64_t row = m0 + sub * 32 + lane;
      if (row < a.M) {
        const float* dp = a.dirs + (row / a.rows_per_dir) * 3;
        dir[0] = __ldg(dp);
        dir[1] = __ldg(dp + 1);
        dir[2] = __ldg(dp + 2);
      }
    }
    if (!layer(D0, OFF_A0, OFF_W0, F / 16, SBO_F, SBO_F, SQP)) { ok = 0; break; }

    // Fourier encoding of row r = 32*sub + lane into X1 (encode_row): both warp halves
    // read the row's 27 squashed features and its direction, and each writes ten K-chunks.
    {
      const int r = sub * 32 + lane;
      float v[SQ + 3], v16[16];
      tc::tmem_ld16(D0 + lane_off, v16);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = v16[j];
      tc::tmem_ld16(D0 + lane_off + 16, v16);
#pragma unroll
      for (int j = 16; j < SQ; ++j) v[j] = v16[j - 16];
      v[SQ] = dir[0];
      v[SQ + 1] = dir[1];
      v[SQ + 2] = dir[2];
      uint8_t* xrow = smem + OFF_A1 + (r >> 3) * SBO_E + (r & 7) * 16;
      if (half == 0)
        encode_row<0>(xrow, v, 0.f);
      else
        encode_row<1>(xrow, v, 0.f);
    }
    if (!layer(D1, OFF_A1, OFF_W1, ENCP / 16, SBO_E, SBO_E, U)) { ok = 0; break; }

    // Hidden layers: +bias, ReLU, bf16 into the next A tile. Warp half h takes columns
    // [64h, 64h + 64) of its rows: one TMEM load, float4 bias loads, 16-byte stores.
    auto hidden = [&](uint32_t Dsrc, const float* bias, int dst_off) {
      const int r = sub * 32 + lane;
      float v[64];
      tc::tmem_ld64(Dsrc + lane_off + half * 64, v);
      const float4* b4 = reinterpret_cast<const float4*>(bias + half * 64);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float4 b = __ldg(b4 + j);
        v[4 * j] = fmaxf(v[4 * j] + b.x, 0.f);
        v[4 * j + 1] = fmaxf(v[4 * j + 1] + b.y, 0.f);
        v[4 * j + 2] = fmaxf(v[4 * j + 2] + b.z, 0.f);
        v[4 * j + 3] = fmaxf(v[4 * j + 3] + b.w, 0.f);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        *reinterpret_cast<uint4*>(smem + dst_off + coff(r, half * 8 + q, SBO_U)) =
            make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                       pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
    };
    float4 xp[X0_PER_THREAD], xq[X0_PER_THREAD];  // row-major X0 only
    if constexpr (!TILES) {
      if (next < ntiles) x0_fetch(xp, xq, a.X0, next * BM, a.M, tid);  // in flight during hidden1, layer 2
    }
    hidden(D1, a.b1, OFF_A0);
    if (!layer(D2, OFF_A0, OFF_W2, U / 16, SBO_U, SBO_U, U)) { ok = 0; break; }
    if (next < ntiles) {  // layer 2 has read H1 from A0: the next tile's input goes there
      if constexpr (TILES) {
        if (tid == 0) {
          tc::mbar_expect_tx(xbar, (uint32_t)X0T_TILE_BYTES);
          tc::bulk_g2s(smem + OFF_A0, a.X0t + next * X0T_TILE_BYTES, (uint32_t)X0T_TILE_BYTES, xbar);
        }
        x_pending = true;
      } else {
        x0_store(xp, xq, smem + OFF_A0, SBO_F, tid);
      }
    }
    hidden(D2, a.b2, OFF_A1);
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
    tc::mbar_wait(wbar, 0, WAIT_LIMIT);             // the weight copy, if it is still in flight
    if (x_pending) tc::mbar_wait(xbar, xphase, WAIT_LIMIT);  // and an input tile copy
    tc::mbar_wait(mbar, phase ^ 1u, WAIT_LIMIT);    // drain the MMAs in flight before freeing TMEM
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}


// ---------------------------------------------------------------------------------
// Fused backward for BF16 models. Per 128-row tile, one persistent CTA per SM:
//   recompute  X0 -> L0 -> h -> Fourier encoding -> X1 -> L1 -> H1 -> L2 -> H2
//   (a) dH2 = (dZ W3^T) * [H2 > 0]          (b) dW3 += H2^T dZ
//   (c) dH1 = (dH2 W2^T) * [H1 > 0]          (d) dW2 += H1^T dH2   (e) db2 += dH2^T 1
//   (f) dX1 = dH1 W1^T -> encoding backward -> dH0                 (g) dW1 += X1^T dH1 (+ db1)
//   (h) dX0 = dH0 W0^T                       (i) dW0 += X0^T dH0
// The data-gradient products read activation tiles K-major as usual; the
// weight-gradient products contract over the tile's rows and read the SAME tiles as
// MN-major operands (transpose bits of the instruction descriptor), so no transposed
// copy is ever made. The four weight gradients (and db1, db2) accumulate in TMEM across
// all of a CTA's tiles and are added to the global gradients once at the end. Nothing
// but dX0 and the gradients goes back to global memory.
// ---------------------------------------------------------------------------------
namespace bwd {

// Natural tiles are [rows][width] bf16 in the K-major canonical layout with
// SBO = (width / 8) * 128. Shared-memory map (bytes):
constexpr int SBO_A = SBO_F;                // RA: 144 wide (X0, then H1 / dH1, then X0 again)
constexpr int SBO_B = SBO_E;                // RB: 160 wide (X1; dX0 staging at the end of a tile)
constexpr int SBO_C = SBO_U;                // RC: 128 wide (H2 / dH2)
constexpr int SBO_Z = 256;                  // RD, RE3: 16 wide (dZ, the constant e3 tile)
constexpr int SBO_H0 = 512;                 // RE: 32 wide (dH0)
constexpr int RA = WPACK_BYTES;             // after the forward's packed weight images
constexpr int RB = RA + BM * F * 2;
constexpr int RC = RB + BM * ENCP * 2;
constexpr int RD = RC + BM * U * 2;
constexpr int RE3 = RD + BM * 16 * 2;
constexpr int RE = RE3 + BM * 16 * 2;
constexpr int RF = RE + BM * SQP * 2;       // h (fp32, 128 x 27) for the encoding backward
constexpr int BAR = RF + BM * SQ * 4;
constexpr int SMEM = BAR + 64;
static_assert(SMEM <= 232448, "shared memory");

// TMEM columns: the per-tile chain (L0..L2 outputs, dH2, dH1, dX1, dX0) reuses
// [0, 144); the weight-gradient accumulators persist.
constexpr uint32_t T_CH = 0, T_W3 = 144, T_W2 = 160, T_W1 = 288, T_W0A = 448, T_W0B = 480;

// MN-major, no-swizzle canonical layout: LBO = byte distance between core matrices
// adjacent along K, SBO = along M/N. A natural tile read MN-major has K = its rows.
struct Op {
  uint32_t addr, lbo, sbo, step;  // step: start-address advance per 16-element K step
};
__device__ __forceinline__ Op kmaj(uint32_t addr, uint32_t sbo) { return Op{addr, 128u, sbo, 256u}; }
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

struct Args {
  int64_t M;
  const uint8_t* wpack;  // the forward's packed weight images (WPACK_BYTES)
  const float* X0;       // (M, 144), or
  const uint8_t* X0t;    // the same as input tiles (TILES kernels)
  const float* dirs;
  int rows_per_dir;
  const float *b1, *b2;
  const float* dZ3;      // (M, 3): gradient wrt the pre-sigmoid output
  float* dX0;            // (M, 144) overwritten, or null
  float *gw0, *gw1, *gb1, *gw2, *gb2, *gw3, *gb3;  // accumulate
};

// Encoding backward for features [J0, J0 + NJ) of row r: dh_j = dX1[j] + the
// derivatives of [sin h, sin 2h, cos h, cos 2h] (columns 30 + 4j .. 33 + 4j).
template <int J0, int NJ>
__device__ __forceinline__ void encoding_bwd(uint32_t taddr, const float* hrow, float (&dh)[14]) {
  float fc[NJ][4];
#pragma unroll
  for (int jj = 0; jj < NJ; ++jj) {
    float s1, c1;
    __sincosf(hrow[J0 + jj], &s1, &c1);
    fc[jj][0] = c1;
    fc[jj][1] = 2.0f * (c1 * c1 - s1 * s1);
    fc[jj][2] = -s1;
    fc[jj][3] = -4.0f * s1 * c1;
    dh[jj] = 0.0f;
  }
  constexpr int PE_LO = SQ + 3 + 4 * J0, PE_HI = PE_LO + 4 * NJ;  // encoding columns of these features
#pragma unroll
  for (int ch = 0; ch < 9; ++ch) {
    const int c0 = ch * 16;
    const bool direct = c0 < J0 + NJ && c0 + 16 > J0;
    const bool pe = c0 < PE_HI && c0 + 16 > PE_LO;
    if (!direct && !pe) continue;
    float v[16];
    tc::tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const int col = c0 + e;
      if (col >= J0 && col < J0 + NJ) dh[col - J0] += v[e];
      if (col >= PE_LO && col < PE_HI) {
        const int j = (col - PE_LO) >> 2, q = (col - PE_LO) & 3;
        dh[j] = fmaf(fc[j][q], v[e], dh[j]);
      }
    }
  }
}

// TILES: each tile's input arrives by bulk copies into RA, for layer 0 (issued when the
// previous tile's dW0 product has read RA) and again for dW0 (issued when dH1's products
// have read RA). Otherwise from the row-major fp32 X0 through registers, at those points.
template <bool TILES>
__global__ void __launch_bounds__(THREADS, 1) mlp_bwd_fused_kernel(Args a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + BAR);
  uint64_t* wbar = mbar + 1;
  uint64_t* xbar = mbar + 3;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + BAR + 16);
  float* hstash = reinterpret_cast<float*>(smem + RF);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = warp & 3, half = warp >> 2;
  const int r = sub * 32 + lane;  // tile row owned by this thread in the epilogues

  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_init(wbar, 1);
    tc::mbar_init(xbar, 1);
  }
  // Constant tile e3 (column 3 = 1): dH2^T e3 accumulates db2 into column 3 of dW3.
  for (int c = tid; c < BM * 2; c += THREADS) {
    const int row = c >> 1, kc = c & 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (kc == 0) v.y = pack2(0.0f, 1.0f);
    *reinterpret_cast<uint4*>(smem + RE3 + coff(row, kc, SBO_Z)) = v;
  }
  __syncthreads();
  const int64_t ntiles = (a.M + BM - 1) / BM;
  // Input tile copies into RA: issue_x0 (thread 0) and wait_x0 (everyone).
  bool x_pending = false;
  uint32_t xphase = 0;
  auto issue_x0 = [&](int64_t t) {
    if (tid == 0) {
      tc::mbar_expect_tx(xbar, (uint32_t)X0T_TILE_BYTES);
      tc::bulk_g2s(smem + RA, a.X0t + t * X0T_TILE_BYTES, (uint32_t)X0T_TILE_BYTES, xbar);
    }
    x_pending = true;
  };
  auto wait_x0 = [&]() -> bool {
    const int got = tc::mbar_wait(xbar, xphase, WAIT_LIMIT) ? 1 : 0;
    if (!__syncthreads_and(got)) return false;
    xphase ^= 1u;
    x_pending = false;
    return true;
  };
  if (tid == 0) {
    tc::mbar_expect_tx(wbar, WPACK_BYTES);
    tc::bulk_g2s(smem + OFF_W0, a.wpack, WPACK_BYTES, wbar);
  }
  if (TILES && (int64_t)blockIdx.x < ntiles) issue_x0(blockIdx.x);
  int ok = tc::mbar_wait(wbar, 0, WAIT_LIMIT) ? 1 : 0;
  ok = __syncthreads_and(ok);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t lane_off = (uint32_t)(sub * 32) << 16;
  const uint32_t sb = tc::smem_u32(smem);
  uint32_t phase = 0;
  float db3[3] = {0.f, 0.f, 0.f};
  bool first = true;

  // Thread 0 issues the MMAs of one step; everyone waits for them.
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
  auto load_x0 = [&](int64_t m0) {
    load_x0_tile(smem + RA, SBO_A, a.X0, m0, a.M, tid);
  };
  // +bias, ReLU, bf16 into a natural tile.
  // Warp half h takes columns [64h, 64h + 64) of its rows: one TMEM load, float4 bias
  // loads, 16-byte stores.
  auto hidden = [&](const float* bias, int dst, int sbo) {
    float v[64];
    tc::tmem_ld64(tmem + T_CH + lane_off + half * 64, v);
    const float4* b4 = reinterpret_cast<const float4*>(bias + half * 64);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float4 b = __ldg(b4 + j);
      v[4 * j] = fmaxf(v[4 * j] + b.x, 0.f);
      v[4 * j + 1] = fmaxf(v[4 * j + 1] + b.y, 0.f);
      v[4 * j + 2] = fmaxf(v[4 * j + 2] + b.z, 0.f);
      v[4 * j + 3] = fmaxf(v[4 * j + 3] + b.w, 0.f);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      *reinterpret_cast<uint4*>(smem + dst + coff(r, half * 8 + q, sbo)) =
          make_uint4(pack2(v[8 * q], v[8 * q + 1]), pack2(v[8 * q + 2], v[8 * q + 3]),
                     pack2(v[8 * q + 4], v[8 * q + 5]), pack2(v[8 * q + 6], v[8 * q + 7]));
  };
  // dH = D * [H > 0], written over H in place (H's tile is no longer read by any MMA).
  auto relu_bwd = [&](int reg, int sbo) {
    float v[64];
    tc::tmem_ld64(tmem + T_CH + lane_off + half * 64, v);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      uint4* p = reinterpret_cast<uint4*>(smem + reg + coff(r, half * 8 + q, sbo));
      uint4 hv = *p;
      const __nv_bfloat162* hb = reinterpret_cast<const __nv_bfloat162*>(&hv);
      uint32_t o[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 f = __bfloat1622float2(hb[e]);
        o[e] = pack2(f.x > 0.f ? v[8 * q + 2 * e] : 0.f, f.y > 0.f ? v[8 * q + 2 * e + 1] : 0.f);
      }
      *p = make_uint4(o[0], o[1], o[2], o[3]);
    }
  };

  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t m0 = tile * BM;
    if (TILES) {
      if (!wait_x0()) { ok = 0; break; }
    } else {
      load_x0(m0);
    }
    if (tid < BM) {  // dZ tile: columns 0..2, zero to 16
      const int64_t row = m0 + tid;
      float z0 = 0.f, z1 = 0.f, z2 = 0.f;
      if (row < a.M) {
        z0 = __ldg(a.dZ3 + row * 3);
        z1 = __ldg(a.dZ3 + row * 3 + 1);
        z2 = __ldg(a.dZ3 + row * 3 + 2);
        db3[0] += z0;
        db3[1] += z1;
        db3[2] += z2;
      }
      *reinterpret_cast<uint4*>(smem + RD + coff(tid, 0, SBO_Z)) = make_uint4(pack2(z0, z1), pack2(z2, 0.f), 0u, 0u);
      *reinterpret_cast<uint4*>(smem + RD + coff(tid, 1, SBO_Z)) = make_uint4(0u, 0u, 0u, 0u);
    }
    {  // the next tile's features and output gradients travel to L2 meanwhile
      const int64_t nm0 = (tile + gridDim.x) * BM;
      if (nm0 < a.M) {
        const int64_t nrows = a.M - nm0 < BM ? a.M - nm0 : BM;
        const char* src = TILES ? reinterpret_cast<const char*>(a.X0t + (tile + gridDim.x) * X0T_TILE_BYTES)
                                : reinterpret_cast<const char*>(a.X0 + nm0 * F);
        const int64_t nbytes = TILES ? X0T_TILE_BYTES : nrows * F * 4;
        for (int64_t off = (int64_t)tid * 128; off < nbytes; off += THREADS * 128) tc::prefetch_l2(src + off);
        if (tid * 128 < nrows * 12) tc::prefetch_l2(reinterpret_cast<const char*>(a.dZ3 + nm0 * 3) + tid * 128);
      }
    }
    // L0: h = X0 W0.
    if (!run([&] { mma_run(tmem + T_CH, kmaj(sb + RA, SBO_A), kmaj(sb + OFF_W0, SBO_F), F / 16,
                           idesc_t(BM, SQP, false, false), false); })) { ok = 0; break; }
    // Fourier encoding into X1 (as in the forward; column 150 = 1 makes dW1's product
    // also deliver db1), and h kept in fp32 for the encoding backward.
    {
      const int64_t row = m0 + r;
      float v[SQ + 3], v16[16];
      tc::tmem_ld16(tmem + T_CH + lane_off, v16);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = v16[j];
      tc::tmem_ld16(tmem + T_CH + lane_off + 16, v16);
#pragma unroll
      for (int j = 16; j < SQ; ++j) v[j] = v16[j - 16];
      v[SQ] = v[SQ + 1] = v[SQ + 2] = 0.f;
      if (row < a.M) {
        const float* dp = a.dirs + (row / a.rows_per_dir) * 3;
        v[SQ] = __ldg(dp);
        v[SQ + 1] = __ldg(dp + 1);
        v[SQ + 2] = __ldg(dp + 2);
      }
      uint8_t* xrow = smem + RB + (r >> 3) * SBO_B + (r & 7) * 16;
      if (half == 0) {
        encode_row<0>(xrow, v, 1.f);
#pragma unroll
        for (int j = 0; j < 14; ++j) hstash[r * SQ + j] = v[j];
      } else {
        encode_row<1>(xrow, v, 1.f);
#pragma unroll
        for (int j = 14; j < SQ; ++j) hstash[r * SQ + j] = v[j];
      }
    }
    // L1, L2 (the L1 product ignores column 150: W1's image is zero there).
    if (!run([&] { mma_run(tmem + T_CH, kmaj(sb + RB, SBO_B), kmaj(sb + OFF_W1, SBO_E), ENCP / 16,
                           idesc_t(BM, U, false, false), false); })) { ok = 0; break; }
    hidden(a.b1, RA, SBO_A);
    if (!run([&] { mma_run(tmem + T_CH, kmaj(sb + RA, SBO_A), kmaj(sb + OFF_W2, SBO_U), U / 16,
                           idesc_t(BM, U, false, false), false); })) { ok = 0; break; }
    hidden(a.b2, RC, SBO_C);
    // (a) dH2 pre-mask = dZ W3^T; (b) dW3 += H2^T dZ.
    if (!run([&] {
          mma_run(tmem + T_CH, kmaj(sb + RD, SBO_Z), mnmaj(sb + OFF_W3, SBO_U), 1, idesc_t(BM, U, false, true), false);
          mma_run(tmem + T_W3, mnmaj(sb + RC, SBO_C), mnmaj(sb + RD, SBO_Z), BM / 16, idesc_t(BM, 16, true, true),
                  !first);
        })) { ok = 0; break; }
    relu_bwd(RC, SBO_C);
    // (c) dH1 pre-mask = dH2 W2^T; (d) dW2^T += dH2^T H1; (e) db2 via dH2^T e3.
    if (!run([&] {
          mma_run(tmem + T_CH, kmaj(sb + RC, SBO_C), mnmaj(sb + OFF_W2, SBO_U), U / 16, idesc_t(BM, U, false, true),
                  false);
          mma_run(tmem + T_W2, mnmaj(sb + RC, SBO_C), mnmaj(sb + RA, SBO_A), BM / 16, idesc_t(BM, U, true, true),
                  !first);
          mma_run(tmem + T_W3, mnmaj(sb + RC, SBO_C), mnmaj(sb + RE3, SBO_Z), BM / 16, idesc_t(BM, 16, true, true),
                  true);
        })) { ok = 0; break; }
    relu_bwd(RA, SBO_A);
    // (f) dX1 = dH1 W1^T (144 columns: everything before the view-direction encoding);
    // (g) dW1^T += dH1^T X1 (column 150 of X1 is 1: db1).
    if (!run([&] {
          mma_run(tmem + T_CH, kmaj(sb + RA, SBO_A), mnmaj(sb + OFF_W1, SBO_E), U / 16, idesc_t(BM, F, false, true),
                  false);
          mma_run(tmem + T_W1, mnmaj(sb + RA, SBO_A), mnmaj(sb + RB, SBO_B), BM / 16, idesc_t(BM, ENCP, true, true),
                  !first);
        })) { ok = 0; break; }
    if (TILES) issue_x0(tile);  // RA is free: dW0 contracts X0 again
    {
      float dh[14];
      const float* hrow = hstash + r * SQ;
      uint8_t* drow = smem + RE + (r >> 3) * SBO_H0 + (r & 7) * 16;
      auto put = [&](int col, float v) {
        *reinterpret_cast<__nv_bfloat16*>(drow + (col >> 3) * 128 + (col & 7) * 2) = __float2bfloat16_rn(v);
      };
      if (half == 0) {
        encoding_bwd<0, 14>(tmem + T_CH + lane_off, hrow, dh);
#pragma unroll
        for (int j = 0; j < 14; ++j) put(j, dh[j]);
      } else {
        encoding_bwd<14, 13>(tmem + T_CH + lane_off, hrow, dh);
#pragma unroll
        for (int j = 0; j < 13; ++j) put(14 + j, dh[j]);
#pragma unroll
        for (int c = SQ; c < SQP; ++c) put(c, 0.0f);
      }
    }
    if (TILES) {
      if (!wait_x0()) { ok = 0; break; }
    } else {
      load_x0(m0);  // dW0 contracts X0 again; RA is free now
    }
    // (h) dX0 = dH0 W0^T; (i) dW0 += X0^T dH0 as two M = 128 products (features 0..127
    // and 16..143).
    if (!run([&] {
          if (a.dX0)
            mma_run(tmem + T_CH, kmaj(sb + RE, SBO_H0), mnmaj(sb + OFF_W0, SBO_F), SQP / 16,
                    idesc_t(BM, F, false, true), false);
          mma_run(tmem + T_W0A, mnmaj(sb + RA, SBO_A), mnmaj(sb + RE, SBO_H0), BM / 16,
                  idesc_t(BM, SQP, true, true), !first);
          mma_run(tmem + T_W0B, mnmaj(sb + RA + 256, SBO_A), mnmaj(sb + RE, SBO_H0), BM / 16,
                  idesc_t(BM, SQP, true, true), !first);
        })) { ok = 0; break; }
    // RA is free: the next tile's input travels while dX0 is stored.
    if (TILES && tile + gridDim.x < ntiles) issue_x0(tile + gridDim.x);
    if (a.dX0) {
      // TMEM -> per-warp 32 x 17 staging (in RB) -> 16-byte row stores.
      float* buf = reinterpret_cast<float*>(smem + RB) + warp * (32 * 17);
      const int ch_begin = half ? 5 : 0, ch_end = half ? 9 : 5;
      for (int ch = ch_begin; ch < ch_end; ++ch) {
        float v[16];
        tc::tmem_ld16(tmem + T_CH + lane_off + ch * 16, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) buf[lane * 17 + j] = v[j];
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int idx = q * 32 + lane;
          const int rr = idx >> 2, c4 = (idx & 3) * 4;
          const int64_t row = m0 + sub * 32 + rr;
          if (row < a.M) {
            *reinterpret_cast<float4*>(a.dX0 + row * F + ch * 16 + c4) =
                make_float4(buf[rr * 17 + c4], buf[rr * 17 + c4 + 1], buf[rr * 17 + c4 + 2], buf[rr * 17 + c4 + 3]);
          }
        }
        __syncwarp();
      }
    }
    first = false;
  }

  if (ok && !first) {
    // Weight gradients: TMEM lane = output row of each accumulator.
    float v[16];
    if (half == 0) {  // dW3 (lane = H2 feature, columns 0..2) and db2 (column 3)
      tc::tmem_ld16(tmem + T_W3 + lane_off, v);
#pragma unroll
      for (int n = 0; n < 3; ++n) atomicAdd(a.gw3 + r * 3 + n, v[n]);
      atomicAdd(a.gb2 + r, v[3]);
    } else {  // dW0, features 128..143 (lanes 112..127 of the second product)
#pragma unroll
      for (int ch = 0; ch < 2; ++ch) {
        tc::tmem_ld16(tmem + T_W0B + lane_off + ch * 16, v);
        if (r >= 112) {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (ch * 16 + j < SQ) atomicAdd(a.gw0 + (int64_t)(r + 16) * SQ + ch * 16 + j, v[j]);
        }
      }
    }
    if (half == 0) {  // dW0, features 0..127
#pragma unroll
      for (int ch = 0; ch < 2; ++ch) {
        tc::tmem_ld16(tmem + T_W0A + lane_off + ch * 16, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (ch * 16 + j < SQ) atomicAdd(a.gw0 + (int64_t)r * SQ + ch * 16 + j, v[j]);
      }
    }
    for (int ch = half * 4; ch < half * 4 + 4; ++ch) {  // dW2^T: lane = output unit, column = input
      tc::tmem_ld16(tmem + T_W2 + lane_off + ch * 16, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) atomicAdd(a.gw2 + (int64_t)(ch * 16 + j) * U + r, v[j]);
    }
    for (int ch = half * 5; ch < half * 5 + 5; ++ch) {  // dW1^T and db1 (input column 150)
      tc::tmem_ld16(tmem + T_W1 + lane_off + ch * 16, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int in = ch * 16 + j;
        if (in < ENC) atomicAdd(a.gw1 + (int64_t)in * U + r, v[j]);
        else if (in == ENC) atomicAdd(a.gb1 + r, v[j]);
      }
    }
    if (warp < 4) {
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        float s = db3[n];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(a.gb3 + n, s);
      }
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(&g_fused_status, 1);
    tc::mbar_wait(wbar, 0, WAIT_LIMIT);
    if (x_pending) tc::mbar_wait(xbar, xphase, WAIT_LIMIT);  // an input tile copy in flight
    tc::mbar_wait(mbar, phase ^ 1u, WAIT_LIMIT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

}  // namespace bwd

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
  return d.math == 0 && d.cams == 0 && d.feat == fmlp::F && d.squash == fmlp::SQ && d.enc == fmlp::ENC &&
         d.units == fmlp::U;
}

size_t mlp_fused_pack_bytes() { return fmlp::WPACK_BYTES; }

int launch_mlp_pack_fused(const MlpWeights& w, uint8_t* wpack, cudaStream_t st) {
  if (!aligned(wpack, 16)) {
    set_error("fused mlp: packed weights must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  fmlp::pack_weights_kernel<<<64, 256, 0, st>>>(wpack, w.w0, w.w1, w.w2, w.w3);
  return check_launch("pack_weights");
}

int launch_mlp_fwd_fused(const MlpDims& d, const MlpWeights& w, const float* X0, const float* dirs, int rows_per_dir,
                         int64_t M, float* rgb, uint8_t* wpack, cudaStream_t st, int max_ctas, const uint8_t* X0t,
                         bool prepacked) {
  if (M == 0) return TVM_OK;
  const bool tiles = X0t != nullptr;
  const void* kern = tiles ? (const void*)fmlp::mlp_fwd_fused_kernel<true> : (const void*)fmlp::mlp_fwd_fused_kernel<false>;
  TVM_TRY(ensure_smem_limit(kern, fmlp::SMEM, "fused mlp"));
  const int sms = device_sms();
  // Weights, features and biases are read with 16-byte loads or bulk copies.
  if (!aligned(wpack, 16) || !aligned(tiles ? (const void*)X0t : (const void*)X0, 16) || !aligned(w.b1, 16) ||
      !aligned(w.b2, 16)) {
    set_error("fused mlp: packed weights, features and biases must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  if (!prepacked) TVM_TRY(launch_mlp_pack_fused(w, wpack, st));
  fmlp::Args a{M, wpack, X0, X0t, dirs, rows_per_dir, w.w0, w.w1, w.b1, w.w2, w.b2, w.w3, w.b3, rgb};
  const int64_t ntiles = ceil_div(M, fmlp::BM);
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, std::max(max_ctas > 0 ? max_ctas : sms, 1));
  if (tiles)
    fmlp::mlp_fwd_fused_kernel<true><<<grid, fmlp::THREADS, fmlp::SMEM, st>>>(a);
  else
    fmlp::mlp_fwd_fused_kernel<false><<<grid, fmlp::THREADS, fmlp::SMEM, st>>>(a);
  return check_launch("mlp_fwd_fused");
}

int launch_mlp_bwd_fused(const MlpWeights& w, const MlpGrads& g, const float* X0, const float* dirs,
                         int rows_per_dir, int64_t M, const float* dZ3, float* dX0, const uint8_t* wpack,
                         cudaStream_t st, int max_ctas, const uint8_t* X0t) {
  if (M == 0) return TVM_OK;
  const bool tiles = X0t != nullptr;
  const void* kern =
      tiles ? (const void*)fmlp::bwd::mlp_bwd_fused_kernel<true> : (const void*)fmlp::bwd::mlp_bwd_fused_kernel<false>;
  TVM_TRY(ensure_smem_limit(kern, fmlp::bwd::SMEM, "fused mlp backward"));
  const int sms = device_sms();
  if (!aligned(wpack, 16) || !aligned(tiles ? (const void*)X0t : (const void*)X0, 16) || (dX0 && !aligned(dX0, 16)) ||
      !aligned(w.b1, 16) || !aligned(w.b2, 16)) {
    set_error("fused mlp backward: packed weights, features, biases and dX0 must be 16-byte aligned");
    return TVM_ERR_ALIGN;
  }
  fmlp::bwd::Args a{M, wpack, X0, X0t, dirs, rows_per_dir, w.b1, w.b2, dZ3, dX0,
                    g.w0, g.w1, g.b1, g.w2, g.b2, g.w3, g.b3};
  const int64_t ntiles = ceil_div(M, fmlp::BM);
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, std::max(max_ctas > 0 ? max_ctas : sms, 1));
  if (tiles)
    fmlp::bwd::mlp_bwd_fused_kernel<true><<<grid, fmlp::THREADS, fmlp::bwd::SMEM, st>>>(a);
  else
    fmlp::bwd::mlp_bwd_fused_kernel<false><<<grid, fmlp::THREADS, fmlp::bwd::SMEM, st>>>(a);
  return check_launch("mlp_bwd_fused");
}

}  // namespace tvm
