// umma_image.cuh — the tensor-core operand image of a mixture's L^-1
// (D <= 32): layout constants, and the device functions that write it, shared
// by the tensor-core kernel's image builder (k_umma.cu) and the fused EM
// update (k_em.cu), which rewrites one component's rows.
#pragma once
#include "pmcg_common.cuh"

namespace pmcg {

constexpr int kUmGC = 8;                      // components per group (256 operand rows)
constexpr int kUmHalf = 128 * 128;            // bytes of one 128-row x 32-float operand (16 KB)
constexpr int kUmOpBytes = 2 * kUmHalf;       // one 256-row operand (32 KB)
constexpr int kUmCopyBytes = 2 * kUmOpBytes;  // streamed per group: hi + lo (64 KB)
constexpr int kUmGroupStride = kUmCopyBytes + 1024;  // image stride per group: hi, lo, lc[8]

// Byte offset of element (row, col) (col < 32 floats) in a 128-byte-swizzled,
// K-major operand: 8-row atoms of 1024 bytes, 16-byte chunk c of row r stored
// at chunk c ^ (r mod 8).
__host__ __device__ __forceinline__ uint32_t sw128_off(int row, int col) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((col >> 2) ^ (row & 7)) & 7) << 4) + (col & 3) * 4);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ------------------------------------------------------------------ operand image
// Group g, component c (k = 8g + c), row i = 8 rb + r, column j: operand row
// n = 64 rb + 8 c + r holds W_k[i][:] split into TF32 hi and lo (zero for
// padding rows / columns / components). The shift s_n = -(L^-1 mu)_k[i],
// split into TF32 (hi, lo), sits in columns 24, 25 of rows that no K-step
// reads there: rows n < 64 min(KS, 3) of the hi operand (upper triangle, or
// unused when KS <= 3) and, for KS = 4, rows 192..255 in rows 0..63 of the lo
// operand. After the operands: the eight log-constants (-inf for padding).
__device__ __forceinline__ void umma_image_entry(const DevMixView &m, unsigned char *img, int g, int n, int j) {
  const int D = m.D, K = m.K, ldx = m.ldx;
  const int KS = (D + 7) >> 3;
  unsigned char *hi = img + (size_t)g * kUmGroupStride, *lo = hi + kUmOpBytes;
  const int rb = n >> 6, c = (n >> 3) & 7, r = n & 7, i = rb * 8 + r, k = g * kUmGC + c;
  float w = 0.f;
  if (k < K && i < D && j < D) w = m.W32[(size_t)k * D * ldx + (size_t)i * ldx + j];
  float h = tf32_round(w);
  float l = tf32_round(w - h);
  // shift entries (the slots are zero in the factor)
  if (j == 24 || j == 25) {
    const int nh = n;                                   // hi slot -> operand row nh
    const int nl = (KS == 4 && n < 64) ? n + 192 : -1;  // lo slot -> operand row nl
    auto shift = [&](int row, float &hv) {
      const int rrb = row >> 6, rc = (row >> 3) & 7, ri = rrb * 8 + (row & 7), rk = g * kUmGC + rc;
      const float sv = (rk < K && ri < D) ? -m.b32[(size_t)rk * D + ri] : 0.f;
      const float sh = tf32_round(sv);
      hv = (j == 24) ? sh : tf32_round(sv - sh);
    };
    if (nh < 64 * (KS < 3 ? KS : 3)) shift(nh, h);
    if (nl >= 0) shift(nl, l);
  }
  *reinterpret_cast<float *>(hi + sw128_off(n, j)) = h;
  *reinterpret_cast<float *>(lo + sw128_off(n, j)) = l;
}

// The 32 operand rows of component k (row n = 64 rb + 8 c + r of group k / 8,
// c = k mod 8) in both operands, shift slots included: every value of these
// rows belongs to component k alone.
__device__ __forceinline__ void umma_image_component(const DevMixView &m, unsigned char *img, int k) {
  const int g = k / kUmGC, c = k - g * kUmGC;
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int rr = e >> 5, j = e & 31;
    umma_image_entry(m, img, g, (rr >> 3) * 64 + c * 8 + (rr & 7), j);
  }
}

// The log-constants of every group (-inf for the padding components).
__device__ __forceinline__ void umma_image_lconst(const DevMixView &m, unsigned char *img) {
  const int G = (m.K + kUmGC - 1) / kUmGC;
  for (int e = threadIdx.x; e < G * kUmGC; e += blockDim.x) {
    const int g = e / kUmGC, c = e - g * kUmGC, k = e;
    reinterpret_cast<float *>(img + (size_t)g * kUmGroupStride + kUmCopyBytes)[c] = (k < m.K) ? m.lconst32[k] : -INFINITY;
  }
}

}  // namespace pmcg
