// Split-BF16 tensor-core DFT16 (precision-study variant of the FFT engine).
//
// A warp holds 32 independent 16-point vectors, one per lane (the radix-16
// butterflies of a Stockham stage).  Their DFTs are one real matrix product
//
//   Y (32 x 32) = X (32 x 32) . B (32 x 32),
//
// X row m = lane m's vector as (re, im) pairs, B[2n + p][2k + q] the real
// form of W = exp(DIR 2 pi i n k / 16):  [[Re W, Im W], [-Im W, Re W]].
// Each FP32 operand is split into a BF16 head and a BF16 tail,
// x = hi(x) + lo(x) + O(2^-16 |x|), and the product is taken as
// hi.hi + hi.lo + lo.hi with FP32 accumulation (the lo.lo term is below the
// representation error of the split).  The products run on the tensor cores
// with the warp-level mma.sync.m16n8k16 (bf16 inputs, f32 accumulators):
// 2 row tiles x 4 column tiles x 2 k-steps x 3 split terms = 48 MMAs.
//
// Operand layouts of m16n8k16 (PTX ISA, warp-level matrix fragments for
// .bf16): with g = lane / 4 and t = lane % 4,
//   A (16 x 16, row-major): a0 = (g, 2t..2t+1), a1 = (g+8, 2t..2t+1),
//                           a2 = (g, 2t+8..2t+9), a3 = (g+8, 2t+8..2t+9);
//   B (16 x 8, column):     b0 = (k 2t..2t+1, n g), b1 = (k 2t+8..2t+9, n g);
//   C/D (16 x 8, f32):      c0, c1 = (g, 2t..2t+1), c2, c3 = (g+8, 2t..2t+1);
// the lower 16 bits of a packed register hold the lower column/k index.
//
// Shared memory per block: the B fragments of both directions
// (kTcBfragWords words, filled once by tc_fill_bfrag) and one
// kTcScratchFloats staging tile per warp.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace sgpe {

constexpr int kTcRow = 36;                          // staging row stride (floats)
constexpr int kTcScratchFloats = 32 * kTcRow;       // per warp
constexpr int kTcBfragWords = 2 * 2 * 4 * 32 * 4;   // [dir][kt][nt][lane][b0hi, b1hi, b0lo, b1lo]

struct TcScratch {
  const uint32_t* bfrag;  // block-shared B fragments
  float* tile;            // this warp's staging tile
};

__device__ __forceinline__ uint32_t pack_bf16(float lo_col, float hi_col) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo_col, hi_col);  // .x -> low 16 bits
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Head and tail of the BF16 split of a pair of FP32 values, packed.
__device__ __forceinline__ void split_pair(float x0, float x1, uint32_t* hi, uint32_t* lo) {
  const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
  *hi = pack_bf16(__bfloat162float(h0), __bfloat162float(h1));
  *lo = pack_bf16(x0 - __bfloat162float(h0), x1 - __bfloat162float(h1));
}

// B[kk][c] of the real DFT16 matrix for direction dir (-1 forward, +1 inverse).
__device__ __forceinline__ float tc_bval(int kk, int c, int dir) {
  const int n = kk >> 1, p = kk & 1, k = c >> 1, q = c & 1;
  const int m = (n * k) & 15;
  double s, co;
  sincospi(double(m) / 8.0, &s, &co);  // angle 2 pi m / 16
  const double wr = co, wi = dir * s;
  const double v = p == 0 ? (q == 0 ? wr : wi) : (q == 0 ? -wi : wr);
  return float(v);
}

// B fragments of both directions into `bfrag` (kTcBfragWords words), the
// threads of the calling grid sharing the work (FP64 angles, rounded once
// to FP32, then split).  Run once per plan (sgpe_set_dft_mode).
__device__ __forceinline__ void tc_fill_bfrag(uint32_t* bfrag, int tid, int nthreads) {
  for (int i = tid; i < kTcBfragWords; i += nthreads) {
    const int reg = i & 3, lane = (i >> 2) & 31, nt = (i >> 7) & 3, kt = (i >> 9) & 1, d = (i >> 10) & 1;
    const int dir = d ? 1 : -1;
    const int g = lane >> 2, t = lane & 3;
    const int kk = kt * 16 + 2 * t + ((reg & 1) ? 8 : 0);
    const int c = nt * 8 + g;
    const float v0 = tc_bval(kk, c, dir), v1 = tc_bval(kk + 1, c, dir);
    uint32_t hi, lo;
    split_pair(v0, v1, &hi, &lo);
    bfrag[i] = (reg < 2) ? hi : lo;
  }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// In-place DFT16 of every lane's a[0..15] (natural order, direction DIR),
// warp-collective: all 32 lanes must call it together.
template <int DIR>
__device__ __forceinline__ void tc_dft16(float2 (&a)[16], const TcScratch& sc) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  float* tile = sc.tile;
  // stage X: row = lane, (re, im) interleaved
#pragma unroll
  for (int n = 0; n < 16; n += 2)
    *reinterpret_cast<float4*>(tile + lane * kTcRow + 2 * n) = make_float4(a[n].x, a[n].y, a[n + 1].x, a[n + 1].y);
  __syncwarp();
  uint32_t ahi[2][2][4], alo[2][2][4];  // [mt][kt][reg]
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const int r0 = mt * 16 + g, k0 = kt * 16 + 2 * t;
      const float2 x0 = *reinterpret_cast<const float2*>(tile + r0 * kTcRow + k0);
      const float2 x1 = *reinterpret_cast<const float2*>(tile + (r0 + 8) * kTcRow + k0);
      const float2 x2 = *reinterpret_cast<const float2*>(tile + r0 * kTcRow + k0 + 8);
      const float2 x3 = *reinterpret_cast<const float2*>(tile + (r0 + 8) * kTcRow + k0 + 8);
      split_pair(x0.x, x0.y, &ahi[mt][kt][0], &alo[mt][kt][0]);
      split_pair(x1.x, x1.y, &ahi[mt][kt][1], &alo[mt][kt][1]);
      split_pair(x2.x, x2.y, &ahi[mt][kt][2], &alo[mt][kt][2]);
      split_pair(x3.x, x3.y, &ahi[mt][kt][3], &alo[mt][kt][3]);
    }
  __syncwarp();  // every lane has read its fragments before the tile is overwritten
  const uint32_t* bf = sc.bfrag + (DIR > 0 ? 1024 : 0);
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const uint4 b = *reinterpret_cast<const uint4*>(bf + ((kt * 4 + nt) * 32 + lane) * 4);
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        mma_bf16(acc[mt], alo[mt][kt], b.x, b.y);   // lo . hi
        mma_bf16(acc[mt], ahi[mt][kt], b.z, b.w);   // hi . lo
        mma_bf16(acc[mt], ahi[mt][kt], b.x, b.y);   // hi . hi
      }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int r0 = mt * 16 + g, c0 = nt * 8 + 2 * t;
      *reinterpret_cast<float2*>(tile + r0 * kTcRow + c0) = make_float2(acc[mt][0], acc[mt][1]);
      *reinterpret_cast<float2*>(tile + (r0 + 8) * kTcRow + c0) = make_float2(acc[mt][2], acc[mt][3]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int n = 0; n < 16; n += 2) {
    const float4 y = *reinterpret_cast<const float4*>(tile + lane * kTcRow + 2 * n);
    a[n] = make_float2(y.x, y.y);
    a[n + 1] = make_float2(y.z, y.w);
  }
  __syncwarp();  // the tile is free for the next call
}

}  // namespace sgpe
