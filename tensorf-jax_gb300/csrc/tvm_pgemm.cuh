// Persistent, warp-specialised split-tf32 GEMM on the tcgen05 tensor cores for the
// FP32 FeatureMlp products with a row-major activation operand:
//
//   D[M x N] = A[M x K] * B[K x N],  A fp32 row-major (M up to R*k rows), B a weight.
//
// FP32 accuracy comes from three tf32 MMAs per product (hi*hi + hi*lo + lo*hi, hi =
// round(x), lo = round(x - hi)), which carries ~22 significant bits of every input.
//
// One CTA per SM walks 128-row tiles round-robin. Roles (320 threads):
//   warp 8      one thread loads each 128 x 32 stage of A (128-byte rows) with one 2-D
//               TMA copy in the 128-byte-swizzle layout, which is the K-major SWIZZLE_128B
//               operand layout of the MMA, into a shared-memory ring slot; rows past M
//               and columns past K arrive as zeros;
//   warps 0-3   converters: split the landed fp32 stage into tf32 hi (in place) and a lo
//               tile (a ring of two), then arrive on the slot's "full" mbarrier. They make
//               no global accesses, so the load/store unit stays free for the epilogue;
//   warp 9      one thread issues the MMAs of each stage into a TMEM accumulator and
//               commits to the slot's "empty" mbarrier (and, after a tile's last stage,
//               to the accumulator's "full" mbarrier);
//   warps 4-7   epilogue: warp 4+e reads TMEM lanes 32e..32e+31 (one row per thread)
//               with tcgen05.ld and applies the fused epilogue; plain row-major outputs
//               leave through 32 x 16 shared-memory blocks (a ring per warp) and 2-D TMA
//               stores. Two accumulators alternate, so the epilogue of tile t runs under
//               the MMAs of tile t+1.
// The B operand (hi and lo images, packed once per call by pack_kernel) stays resident
// in shared memory; bulk copies bring it in. Every wait is bounded: a wait that gives
// up sets bit 0 of g_tc_status and its role stops; the MMA thread drains its MMAs
// before TMEM is freed.
#pragma once

#include <cuda.h>

#include "tvm_tc.cuh"

namespace tvm {
namespace pg {

constexpr int BM = 128;
constexpr int BK = 32;                    // K elements per stage (one 128-byte swizzle row)
constexpr int KCH = BK / 4;               // 16-byte chunks per row per stage
constexpr int TILE_BYTES = BM * BK * 4;   // one stage tile (fp32 / tf32 hi, or tf32 lo)
constexpr int LO_SLOTS = 2;               // lo tiles: converted stages waiting for their MMAs
constexpr int SW_ATOM = 1024;             // 8 rows x 128 bytes: one 128-byte-swizzle atom
constexpr int CONV_WARPS = 4, EPI_WARPS = 4;
constexpr int CONV_THREADS = CONV_WARPS * 32;
constexpr int EPI_THREADS = EPI_WARPS * 32;
constexpr int EPI_WARP0 = CONV_WARPS;
constexpr int TMA_WARP = CONV_WARPS + EPI_WARPS;
constexpr int MMA_WARP = TMA_WARP + 1;
constexpr int THREADS = (MMA_WARP + 1) * 32;
constexpr int CHUNKS_PER_THREAD = BM * KCH / CONV_THREADS;  // 8
constexpr int MAX_SLOTS = 8;              // TMA ring depth (stages in flight)
constexpr int SMEM_LIMIT = 232448;        // opt-in dynamic shared memory per block
constexpr int MIN_SMEM = 120 * 1024;      // above half an SM: one CTA per SM (TMEM budget)
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr int OUT_BOX_COLS = 16, OUT_BOX_ROWS = 32;  // TMA store block of one epilogue warp
constexpr int OUT_BOX_FLOATS = OUT_BOX_COLS * OUT_BOX_ROWS;
constexpr int BAR_BYTES = 512;
static_assert(CHUNKS_PER_THREAD * CONV_THREADS == BM * KCH, "stage split");

__host__ __device__ constexpr int kpad(int K) { return (K + 7) / 8 * 8; }
__host__ __device__ constexpr int npad(int N) { return (N + 15) / 16 * 16; }
__host__ __device__ constexpr uint32_t acc_cols(int nt) { return nt <= 32 ? 32 : nt <= 64 ? 64 : nt <= 128 ? 128 : 256; }
// Bytes of one packed B image (hi, then lo) for K x N.
__host__ __device__ constexpr int image_bytes(int K, int N) { return 2 * npad(N) * kpad(K) * 4; }

// K-major SWIZZLE_128B operand: 8-row x 128-byte atoms (SBO = 1024 bytes between
// 8-row groups), swizzle mode 2 in bits 61-63 of the descriptor; the leading offset is
// unused for this layout (encoded as 1). A K step inside the atom advances the start
// address by its byte offset.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  return tc::sdesc(saddr, 16, SW_ATOM) | (2ull << 61);
}

// 2-D TMA copies (tensor maps built on the host with cuTensorMapEncodeTiled).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          tc::smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(tc::smem_u32(mbar))
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* tm, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(tm)),
               "r"(x), "r"(y), "r"(tc::smem_u32(src))
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void tma_store_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void tma_store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---------------------------------------------------------------------------------
// B images: B(k, n) = BT ? W[n * ldw + k] : W[k * ldw + n] for k < K, n < N, zero in
// the padding, split into tf32 hi / lo and laid out as the shared-memory operand:
// byte (n >> 3) * (KP * 32) + (k >> 2) * 128 + (n & 7) * 16 + (k & 3) * 4.
// ---------------------------------------------------------------------------------
// kp / np: the padded K and N of the kernel that reads the image (kp >= K, kp % 8 == 0,
// np >= N, np % 16 == 0).
struct PackJob {
  const float* W;
  int ldw, K, N, kp, np, bt;
  uint8_t* out;
};
struct PackList {
  PackJob job[4];
  int count;
};

__global__ void pack_kernel(PackList list) {
  const PackJob j = list.job[blockIdx.y];
  const int KP = j.kp;
  const int total = KP * j.np;
  float* hi = reinterpret_cast<float*>(j.out);
  float* lo = hi + total;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int n = e / KP, k = e - n * KP;
    float v = 0.0f;
    if (n < j.N && k < j.K) v = __ldg(j.bt ? j.W + (int64_t)n * j.ldw + k : j.W + (int64_t)k * j.ldw + n);
    const uint32_t h = tc::to_tf32(v);
    const uint32_t l = tc::to_tf32(v - __uint_as_float(h));
    const int off = (n >> 3) * (KP * 8) + (k >> 2) * 32 + (n & 7) * 4 + (k & 3);  // in floats
    hi[off] = __uint_as_float(h);
    lo[off] = __uint_as_float(l);
  }
}

// ---------------------------------------------------------------------------------
// Fused epilogues. Thread (warp 8+e, lane) owns row m0 + 32e + lane; taddr is its TMEM
// lane and the accumulator's first column. tcgen05.ld is warp-collective, so rows past
// M still load and only skip their stores.
// ---------------------------------------------------------------------------------
enum EpiKind : int {
  EPI_BIAS_RELU = 0,     // out = relu(acc + bias)                       (H1)
  EPI_BIAS_RELU_L3 = 1,  // out = relu(acc + bias); rgb = sigmoid(out W3 + b3)   (H2, rgb)
  EPI_PE_FWD = 2,        // X1 row = [h, d, PE(h), PE(d), 0 pad] from h = acc (N = 27)
  EPI_MASK_COLSUM = 3,   // out = acc * [H > 0] (H's ReLU bits); colsum += out    (dH1, db1)
  EPI_PE_BWD = 4,        // dH0 = acc[h] + d PE / d h . acc[PE(h)]        (dX1 -> dH0)
  EPI_STORE = 5,         // out = acc (TMA-stored when out is 16-byte aligned)   (dX0)
};

struct EpiArgs {
  float* out;
  int ldo;
  const float* bias;     // EPI_BIAS_RELU*: (N)
  const float* w3;       // EPI_BIAS_RELU_L3: (N, 3) row-major
  const float* b3;       // EPI_BIAS_RELU_L3: (3)
  float* rgb;            // EPI_BIAS_RELU_L3: (M, 3)
  const float* H;        // EPI_PE_BWD: X1 (M, ldh)
  int ldh;
  float* colsum;         // EPI_MASK_COLSUM: (N), accumulated
  uint32_t* mask;        // EPI_BIAS_RELU (optional, written) / EPI_MASK_COLSUM (read): (M, 4) ReLU bits
  const float* dirs;     // EPI_PE_FWD: view direction of row m at dirs[(m / rows_per_dir) * 3]
  int rows_per_dir;
};

// Feature-encoding widths of the fused epilogues (networks.py:13-35, 68-76 with
// 2 frequencies for features and directions): X1 = [h 27 | d 3 | PE(h) 108 | PE(d) 12].
constexpr int SQ = 27, ENC = 150, LDX1 = 152, LDH0 = 28;
constexpr int PEH = SQ + 3, PED = PEH + 4 * SQ;

__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}

// Sums 16 per-lane values over the warp's 32 lanes; lanes 2c and 2c+1 return column c.
__device__ __forceinline__ float warp_colsum16(float (&v)[16], int lane) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool up = lane & 16;
    const float send = up ? v[i] : v[i + 8];
    const float keep = up ? v[i + 8] : v[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  float b[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool up = lane & 8;
    const float send = up ? a[i] : a[i + 4];
    const float keep = up ? a[i + 4] : a[i];
    b[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  float c[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool up = lane & 4;
    const float send = up ? b[i] : b[i + 2];
    const float keep = up ? b[i + 2] : b[i];
    c[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  const bool up = lane & 2;
  const float send = up ? c[0] : c[1];
  const float keep = up ? c[1] : c[0];
  float d = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  return d + __shfl_xor_sync(0xffffffffu, d, 1);
}

// Writes this warp's 32 x 16 block (lane l holds row y + l, columns x..x+15) with one
// TMA store from the next of the warp's nsb shared-memory blocks; rows past M and
// columns past the map's width are dropped by the TMA unit. A block is rewritten once
// at most nsb - 1 later stores are still reading.
struct StoreRing {
  float* base;
  int nsb, next;
};
__device__ __forceinline__ void put_block(StoreRing& r, const float (&v)[16], const CUtensorMap* tm, int x, int y,
                                          int lane) {
  if (lane == 0) {
    if (r.nsb >= 4) asm volatile("cp.async.bulk.wait_group.read 3;" ::: "memory");
    else if (r.nsb >= 2) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
    else tma_store_wait_read();
  }
  __syncwarp();
  float* sb = r.base + r.next * OUT_BOX_FLOATS;
  r.next = r.next + 1 == r.nsb ? 0 : r.next + 1;
  float4* d = reinterpret_cast<float4*>(sb + lane * OUT_BOX_COLS);
#pragma unroll
  for (int q = 0; q < 4; ++q) d[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  tc::fence_proxy_async();
  __syncwarp();
  if (lane == 0) tma_store_2d(tm, x, y, sb);
}

template <int KIND, int NT>
struct Epilogue {
  static constexpr int NCH = NT / 16;
  float cs[KIND == EPI_MASK_COLSUM ? NCH : 1];  // per-lane column sums (colsum kind)

  __device__ void init() {
#pragma unroll
    for (int i = 0; i < (KIND == EPI_MASK_COLSUM ? NCH : 1); ++i) cs[i] = 0.0f;
  }

  // esm: the epilogue's constants in shared memory (W3 and b2 for the L3 kind); sb: the
  // warp's TMA store block; tm: the output tensor map; row0: the warp's first row.
  // pre: the row's prefetched global input (the ReLU bit mask, or X1's first 28 columns).
  __device__ void tile(const EpiArgs& a, int N, uint32_t taddr, int64_t row0, int64_t M, int lane, const float* esm,
                       StoreRing& sr, const CUtensorMap* tm, const float4 (&pre)[7]) {
    const int64_t row = row0 + lane;
    const bool valid = row < M;
    if constexpr (KIND == EPI_BIAS_RELU || KIND == EPI_BIAS_RELU_L3) {
      float z0 = 0.f, z1 = 0.f, z2 = 0.f;
      uint32_t bits[NCH / 2];
#pragma unroll
      for (int c = 0; c < NCH; c += 2) {
        float v[16], w[16];
        tc::tmem_ld16x2(taddr + c * 16, taddr + c * 16 + 16, v, w);
        uint32_t word = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = c * 16 + j;
          float x = (j < 16) ? v[j] : w[j - 16];
          x = fmaxf(x + (KIND == EPI_BIAS_RELU_L3 ? esm[3 * NT + n] : __ldg(a.bias + n)), 0.0f);
          word |= (x > 0.0f ? 1u : 0u) << j;
          if (j < 16) v[j] = x; else w[j - 16] = x;
          if constexpr (KIND == EPI_BIAS_RELU_L3) {
            z0 = fmaf(x, esm[3 * n], z0);
            z1 = fmaf(x, esm[3 * n + 1], z1);
            z2 = fmaf(x, esm[3 * n + 2], z2);
          }
        }
        bits[c / 2] = word;
        put_block(sr, v, tm, c * 16, (int)row0, lane);
        put_block(sr, w, tm, c * 16 + 16, (int)row0, lane);
      }
      if (a.mask && valid) {  // ReLU bits of the row (bit j of word c: column 32c + j > 0)
        static_assert(NCH == 8, "mask rows hold 128 columns");
        *reinterpret_cast<uint4*>(a.mask + row * 4) = make_uint4(bits[0], bits[1], bits[2], bits[3]);
      }
      if constexpr (KIND == EPI_BIAS_RELU_L3) {
        if (valid) {
          float* o = a.rgb + row * 3;
          o[0] = 1.0f / (1.0f + expf(-(z0 + esm[4 * NT])));
          o[1] = 1.0f / (1.0f + expf(-(z1 + esm[4 * NT + 1])));
          o[2] = 1.0f / (1.0f + expf(-(z2 + esm[4 * NT + 2])));
        }
      }
    } else if constexpr (KIND == EPI_PE_FWD) {
      // X1 row (networks.py:68-76): [h | d | PE(h_j) for j | PE(d_a) for a] with
      // PE(v) = [sin v, sin 2v, sin(v + pi/2), sin(2v + pi/2)] = [s, 2sc, c, c^2 - s^2].
      float x[SQ + 3];
      {
        float v[16], w[16];
        tc::tmem_ld16x2(taddr, taddr + 16, v, w);
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = v[j];
#pragma unroll
        for (int j = 16; j < SQ; ++j) x[j] = w[j - 16];
      }
      if (valid) {
        const float* dp = a.dirs + (row / a.rows_per_dir) * 3;
        x[SQ] = __ldg(dp);
        x[SQ + 1] = __ldg(dp + 1);
        x[SQ + 2] = __ldg(dp + 2);
      } else {
        x[SQ] = x[SQ + 1] = x[SQ + 2] = 0.0f;
      }
      float sn[SQ + 3], cn[SQ + 3];
#pragma unroll
      for (int j = 0; j < SQ + 3; ++j) sincosf(x[j], &sn[j], &cn[j]);
#pragma unroll
      for (int b = 0; b < (ENC + 15) / 16; ++b) {
        float blk[16];
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          const int col = b * 16 + jj;
          float val = 0.0f;
          if (col < PEH) {
            val = x[col];
          } else if (col < ENC) {
            const int j = (col - PEH) >> 2, t = (col - PEH) & 3;
            val = t == 0 ? sn[j] : t == 1 ? 2.0f * sn[j] * cn[j] : t == 2 ? cn[j] : cn[j] * cn[j] - sn[j] * sn[j];
          }
          blk[jj] = val;
        }
        put_block(sr, blk, tm, b * 16, (int)row0, lane);
      }
    } else if constexpr (KIND == EPI_MASK_COLSUM) {
      static_assert(NCH == 8, "mask rows hold 128 columns");
      const uint32_t bits[4] = {__float_as_uint(pre[0].x), __float_as_uint(pre[0].y), __float_as_uint(pre[0].z),
                                __float_as_uint(pre[0].w)};  // zero for rows past M
#pragma unroll
      for (int c = 0; c < NCH; c += 2) {
        float v[16], w[16];
        tc::tmem_ld16x2(taddr + c * 16, taddr + c * 16 + 16, v, w);
        const uint32_t word = bits[c / 2];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          v[j] = (word >> j) & 1u ? v[j] : 0.0f;
          w[j] = (word >> (16 + j)) & 1u ? w[j] : 0.0f;
        }
        put_block(sr, v, tm, c * 16, (int)row0, lane);
        put_block(sr, w, tm, c * 16 + 16, (int)row0, lane);
        cs[c] += warp_colsum16(v, lane);
        cs[c + 1] += warp_colsum16(w, lane);
      }
    } else if constexpr (KIND == EPI_PE_BWD) {
      // dH0[j] = dX1[j] + sum_f dX1[sin 2^f h_j] * 2^f cos(2^f h_j)
      //                 + dX1[sin(2^f h_j + pi/2)] * (-2^f sin(2^f h_j))   (networks.py:13-35)
      float hv[28];
#pragma unroll
      for (int q = 0; q < 7; ++q) {
        hv[4 * q] = pre[q].x;
        hv[4 * q + 1] = pre[q].y;
        hv[4 * q + 2] = pre[q].z;
        hv[4 * q + 3] = pre[q].w;
      }
      float s1[SQ], c1[SQ];
#pragma unroll
      for (int j = 0; j < SQ; ++j) sincosf(hv[j], &s1[j], &c1[j]);
      float dh[SQ];
#pragma unroll
      for (int j = 0; j < SQ; ++j) dh[j] = 0.0f;
      // Columns 0..143 in nine 16-column chunks; those past PED (direction terms) are unused.
#pragma unroll
      for (int c = 0; c < 9; c += 2) {
        float v[32];
        if (c + 1 < 9) {
          float x[16], y[16];
          tc::tmem_ld16x2(taddr + c * 16, taddr + c * 16 + 16, x, y);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            v[j] = x[j];
            v[16 + j] = y[j];
          }
        } else {
          float x[16];
          tc::tmem_ld16(taddr + c * 16, x);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            v[j] = x[j];
            v[16 + j] = 0.0f;
          }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = c * 16 + j;
          if (col < SQ) {
            dh[col] += v[j];
          } else if (col >= PEH && col < PED) {
            const int f = (col - PEH) >> 2, t = (col - PEH) & 3;
            const float s = s1[f], co = c1[f];
            float g;
            if (t == 0) g = co;                              // d sin h
            else if (t == 1) g = 2.0f * (co * co - s * s);   // d sin 2h = 2 cos 2h
            else if (t == 2) g = -s;                         // d cos h
            else g = -4.0f * s * co;                         // d cos 2h = -2 sin 2h
            dh[f] = fmaf(v[j], g, dh[f]);
          }
        }
      }
      if (valid) {
        float* o = a.out + row * LDH0;
#pragma unroll
        for (int q = 0; q < 6; ++q) st4(o + 4 * q, dh[4 * q], dh[4 * q + 1], dh[4 * q + 2], dh[4 * q + 3]);
        st4(o + 24, dh[24], dh[25], dh[26], 0.0f);
      }
    } else {  // EPI_STORE
      const bool ovec = ((reinterpret_cast<uintptr_t>(a.out) | (uintptr_t)(a.ldo * 4)) & 15) == 0;
      auto put16 = [&](int n0, const float (&x)[16]) {
        float* p = a.out + row * a.ldo + n0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int n = n0 + 4 * q;
          if (ovec && n + 3 < N) {
            st4(p + 4 * q, x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (n + e < N) p[4 * q + e] = x[4 * q + e];
          }
        }
      };
      // TMA stores when the host gave store blocks (an aligned output), else direct ones.
      const bool tma = sr.nsb > 0;
#pragma unroll
      for (int c = 0; c < NCH; c += 2) {
        float v[16], w[16];
        if (c + 1 < NCH) {
          tc::tmem_ld16x2(taddr + c * 16, taddr + c * 16 + 16, v, w);
          if (tma) {
            put_block(sr, v, tm, c * 16, (int)row0, lane);
            put_block(sr, w, tm, c * 16 + 16, (int)row0, lane);
          } else if (valid) {
            put16(c * 16, v);
            put16(c * 16 + 16, w);
          }
        } else {
          tc::tmem_ld16(taddr + c * 16, v);
          if (tma) put_block(sr, v, tm, c * 16, (int)row0, lane);
          else if (valid) put16(c * 16, v);
        }
      }
    }
  }

  __device__ void finish(const EpiArgs& a, int N, int lane) {
    if (lane == 0) tma_store_wait_all();
    if constexpr (KIND == EPI_MASK_COLSUM) {
      if ((lane & 1) == 0) {
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
          const int n = c * 16 + (lane >> 1);
          if (n < N) atomicAdd(a.colsum + n, cs[c]);
        }
      }
    }
  }
};

// Shared-memory floats the epilogue keeps: W3 (NT x 3) and the bias for the L3 kind.
template <int KIND, int NT>
__host__ __device__ constexpr int epi_smem_floats() {
  return KIND == EPI_BIAS_RELU_L3 ? 4 * NT + 4 : 0;
}

// Shared memory besides the TMA ring and the store blocks: alignment slack, B images,
// epilogue constants, the lo ring and the mbarriers.
template <int NT>
__host__ __device__ constexpr int smem_base_bytes(int K, int epi_floats) {
  return SW_ATOM + image_bytes(K, NT) + ((epi_floats * 4 + SW_ATOM - 1) & ~(SW_ATOM - 1)) + LO_SLOTS * TILE_BYTES +
         BAR_BYTES;
}

// tmA: A as a (K wide, M high) fp32 map with a 4 x 128 box. tmO: the output map with a
// 16 x 32 box (TMA-stored kinds). The A map's width is the K of the product: columns past
// it (row padding) read as zero. slots: TMA ring depth; nsb: store blocks per epilogue
// warp (1, 2 or 4; 0 for kinds that store directly).
template <int KIND, int NT>
__global__ void __launch_bounds__(THREADS, 1)
    pgemm_kernel(int64_t M, int N, int K, const __grid_constant__ CUtensorMap tmA,
                 const __grid_constant__ CUtensorMap tmO, const uint8_t* __restrict__ bimg, int slots, int nsb,
                 EpiArgs ea) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // The swizzled tiles need 1024-byte alignment in the shared window (1 KB is reserved).
  uint8_t* smem = smem_raw + ((SW_ATOM - (tc::smem_u32(smem_raw) & (SW_ATOM - 1))) & (SW_ATOM - 1));
  constexpr uint32_t NCOLS = acc_cols(NT);
  constexpr uint32_t IDESC = tc::idesc(BM, NT, 2u);
  constexpr int EF = epi_smem_floats<KIND, NT>();
  const int KP = kpad(K);
  const int img = image_bytes(K, NT);
  // Tiles read through swizzled descriptors start on 1024-byte atoms.
  uint8_t* sB = smem;                                                       // hi image, lo image
  float* sEpi = reinterpret_cast<float*>(smem + img);                       // epilogue constants
  uint8_t* sLo = smem + img + ((EF * 4 + SW_ATOM - 1) & ~(SW_ATOM - 1));    // LO_SLOTS lo tiles
  uint8_t* sRing = sLo + LO_SLOTS * TILE_BYTES;                             // slots fp32 / hi tiles
  float* sStage = reinterpret_cast<float*>(sRing + slots * TILE_BYTES);     // store blocks
  uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(sStage) + nsb * EPI_WARPS * OUT_BOX_FLOATS * 4);
  uint64_t* landed = bars;                   // [MAX_SLOTS] TMA bytes arrived
  uint64_t* full = bars + MAX_SLOTS;         // [MAX_SLOTS] hi/lo tiles ready
  uint64_t* empty = bars + 2 * MAX_SLOTS;    // [MAX_SLOTS] MMAs done with the slot
  uint64_t* lo_empty = bars + 3 * MAX_SLOTS; // [LO_SLOTS] MMAs done with the lo tile
  uint64_t* accf = lo_empty + LO_SLOTS;      // [2]
  uint64_t* acce = accf + 2;                 // [2]
  uint64_t* wbar = acce + 2;
  uint64_t* drain = wbar + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (M + BM - 1) / BM;
  const int my_tiles = ntiles > blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int KS = (K + BK - 1) / BK;
  const int64_t nq = (int64_t)my_tiles * KS;

  if (warp == 0) tc::tmem_alloc(tslot, 2 * NCOLS);
  if (tid == 0) {
    for (int s = 0; s < MAX_SLOTS; ++s) {
      tc::mbar_init(landed + s, 1);
      tc::mbar_init(full + s, CONV_THREADS);
      tc::mbar_init(empty + s, 1);
    }
    for (int s = 0; s < LO_SLOTS; ++s) tc::mbar_init(lo_empty + s, 1);
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(accf + b, 1);
      tc::mbar_init(acce + b, EPI_THREADS);
    }
    tc::mbar_init(wbar, 1);
    tc::mbar_init(drain, 1);
  }
  if (KIND == EPI_BIAS_RELU_L3) {
    for (int i = tid; i < 3 * NT; i += THREADS) sEpi[i] = (i < 3 * N) ? __ldg(ea.w3 + i) : 0.0f;
    for (int i = tid; i < NT; i += THREADS) sEpi[3 * NT + i] = (i < N) ? __ldg(ea.bias + i) : 0.0f;
    if (tid < 3) sEpi[4 * NT + tid] = __ldg(ea.b3 + tid);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  if (warp < CONV_WARPS) {
    // ---------------- converters: fp32 stage -> tf32 hi (in place) + lo ----------------
    for (int64_t q = 0; q < nq; ++q) {
      const int slot = (int)(q % slots), lj = (int)(q % LO_SLOTS);
      if (!tc::mbar_wait(landed + slot, (uint32_t)((q / slots) & 1), WAIT_LIMIT) ||
          (q >= LO_SLOTS && !tc::mbar_wait(lo_empty + lj, (uint32_t)((q / LO_SLOTS - 1) & 1), WAIT_LIMIT))) {
        atomicOr(&g_tc_status, 1);
        break;
      }
      uint8_t* hi = sRing + slot * TILE_BYTES;
      uint8_t* lo = sLo + lj * TILE_BYTES;
#pragma unroll
      for (int i = 0; i < CHUNKS_PER_THREAD; ++i) {
        const int off = (tid + i * CONV_THREADS) * 16;  // layout-agnostic: every chunk alike
        const float4 x = *reinterpret_cast<const float4*>(hi + off);
        const uint32_t h0 = tc::to_tf32(x.x), h1 = tc::to_tf32(x.y), h2 = tc::to_tf32(x.z), h3 = tc::to_tf32(x.w);
        const uint32_t l0 = tc::to_tf32(x.x - __uint_as_float(h0)), l1 = tc::to_tf32(x.y - __uint_as_float(h1));
        const uint32_t l2 = tc::to_tf32(x.z - __uint_as_float(h2)), l3 = tc::to_tf32(x.w - __uint_as_float(h3));
        *reinterpret_cast<uint4*>(hi + off) = make_uint4(h0, h1, h2, h3);
        *reinterpret_cast<uint4*>(lo + off) = make_uint4(l0, l1, l2, l3);
      }
      tc::fence_proxy_async();
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(full + slot)) : "memory");
    }
  } else if (warp < TMA_WARP) {
    // ---------------- epilogue ----------------
    const int e = warp - EPI_WARP0;  // TMEM sub-partition (warp % 4 == e)
    StoreRing sr{sStage + e * nsb * OUT_BOX_FLOATS, nsb, 0};
    Epilogue<KIND, NT> epi;
    epi.init();
    bool ok = true;
    for (int i = 0; i < my_tiles && ok; ++i) {
      const int b = i & 1;
      const int64_t row0 = ((int64_t)blockIdx.x + (int64_t)i * gridDim.x) * BM + 32 * e;
      const int64_t row = row0 + lane;
      // The row's global input is requested before the accumulator wait.
      float4 pre[7];
#pragma unroll
      for (int q = 0; q < 7; ++q) pre[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (KIND == EPI_MASK_COLSUM && row < M) pre[0] = __ldg(reinterpret_cast<const float4*>(ea.mask + row * 4));
      if (KIND == EPI_PE_BWD && row < M) {
#pragma unroll
        for (int q = 0; q < 7; ++q) pre[q] = __ldg(reinterpret_cast<const float4*>(ea.H + row * ea.ldh) + q);
      }
      ok = __all_sync(0xffffffffu, tc::mbar_wait(accf + b, (uint32_t)((i >> 1) & 1), WAIT_LIMIT));
      if (!ok) {
        if (lane == 0) atomicOr(&g_tc_status, 1);
        break;
      }
      tc::fence_after_sync();
      const uint32_t taddr = tmem + (uint32_t)(b * NCOLS) + ((uint32_t)(32 * e) << 16);
      epi.tile(ea, N, taddr, row0, M, lane, sEpi, sr, &tmO, pre);
      tc::fence_before_sync();
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(acce + b)) : "memory");
    }
    epi.finish(ea, N, lane);
  } else if (warp == TMA_WARP) {
    // ---------------- TMA loads of A ----------------
    if (lane == 0) {
      for (int64_t q = 0; q < nq; ++q) {
        const int slot = (int)(q % slots);
        const int64_t use = q / slots;
        if (use > 0 && !tc::mbar_wait(empty + slot, (uint32_t)((use - 1) & 1), WAIT_LIMIT)) {
          atomicOr(&g_tc_status, 1);
          break;
        }
        const int64_t tl = q / KS;
        const int ks = (int)(q - tl * KS);
        const int y = (int)(((int64_t)blockIdx.x + tl * gridDim.x) * BM);
        uint8_t* hi = sRing + slot * TILE_BYTES;
        tc::mbar_expect_tx(landed + slot, TILE_BYTES);
        tma_load_2d(hi, &tmA, ks * BK, y, landed + slot);
      }
      // No copy may still be writing shared memory when the CTA exits (the converters
      // wait for every stage unless a wait gave up).
      for (int64_t q = nq - slots > 0 ? nq - slots : 0; q < nq; ++q)
        if (!tc::mbar_wait(landed + (int)(q % slots), (uint32_t)((q / slots) & 1), WAIT_LIMIT)) atomicOr(&g_tc_status, 1);
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const int bytes = img;
    tc::mbar_expect_tx(wbar, (uint32_t)bytes);
    for (int off = 0; off < bytes; off += 32768) {
      const int n = bytes - off < 32768 ? bytes - off : 32768;
      tc::bulk_g2s(sB + off, bimg + off, (uint32_t)n, wbar);
    }
    bool ok = tc::mbar_wait(wbar, 0, WAIT_LIMIT);
    if (!ok) atomicOr(&g_tc_status, 1);
    const uint32_t b_hi = tc::smem_u32(sB), b_lo = b_hi + (uint32_t)(img / 2);
    const uint32_t sbo_b = (uint32_t)KP * 32;
    int64_t q = 0;
    for (int i = 0; i < my_tiles && ok; ++i) {
      const int b = i & 1;
      if (i >= 2 && !tc::mbar_wait(acce + b, (uint32_t)(((i >> 1) - 1) & 1), WAIT_LIMIT)) {
        atomicOr(&g_tc_status, 1);
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(b * NCOLS);
      for (int ks = 0; ks < KS; ++ks, ++q) {
        const int slot = (int)(q % slots), lj = (int)(q % LO_SLOTS);
        if (!tc::mbar_wait(full + slot, (uint32_t)((q / slots) & 1), WAIT_LIMIT)) {
          atomicOr(&g_tc_status, 1);
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t a_hi = tc::smem_u32(sRing + slot * TILE_BYTES), a_lo = tc::smem_u32(sLo + lj * TILE_BYTES);
        const int kleft = K - ks * BK;
        const int steps = (kleft >= BK ? BK : kleft + 7) / 8;
        for (int s = 0; s < steps; ++s) {
          // A: 128-byte-swizzled rows, K step s at byte 32 s of the atom; B: packed image.
          const uint32_t kb = (uint32_t)(ks * KCH + 2 * s) * 128;
          const uint64_t ah = sdesc_sw128(a_hi + 32 * s), al = sdesc_sw128(a_lo + 32 * s);
          const uint64_t bh = tc::sdesc(b_hi + kb, 128, sbo_b), bl = tc::sdesc(b_lo + kb, 128, sbo_b);
          tc::mma_tf32(d, ah, bh, IDESC, (ks > 0 || s > 0) ? 1u : 0u);
          tc::mma_tf32(d, ah, bl, IDESC, 1u);
          tc::mma_tf32(d, al, bh, IDESC, 1u);
        }
        tc::mma_commit(empty + slot);
        tc::mma_commit(lo_empty + lj);
      }
      if (!ok) break;
      tc::mma_commit(accf + b);
    }
    // Every MMA issued so far must finish before TMEM is released.
    tc::mma_commit(drain);
    if (!tc::mbar_wait(drain, 0, WAIT_LIMIT)) atomicOr(&g_tc_status, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * NCOLS);
  }
}

}  // namespace pg
}  // namespace tvm
