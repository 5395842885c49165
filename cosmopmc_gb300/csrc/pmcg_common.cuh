// pmcg_common.cuh — device helpers shared by the libpmcg kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define PMCG_PI 3.14159265358979323846
#define PMCG_LN2PI 1.83787706640934548356

// Philox4x32-10 (Salmon et al., SC'11): ten rounds of the published
// multiply/xor round function with a Weyl-sequence key schedule.
struct P4 { uint32_t x, y, z, w; };

// High word of a 32 x 32-bit product (the device's mul.hi; the same value on the host).
__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ P4 philox4x32_10(P4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t lo0 = 0xD2511F53u * c.x, hi0 = mulhi32(0xD2511F53u, c.x);
    uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = mulhi32(0xCD9E8D57u, c.z);
    P4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// 53-bit dyadic uniform in [0,1) from two words (same mapping as the oracle).
__host__ __device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}
// 24-bit uniform in [0,1) for the single-precision sampler.
__device__ __forceinline__ float u24(uint32_t a) { return (float)(a >> 8) * (1.0f / 16777216.0f); }

// Online log-sum-exp accumulator (max, sum exp(l-max)).
struct LSE {
  double m, s;
};
__device__ __forceinline__ void lse_add(double &m, double &s, double l) {
  if (l > m) { s = s * exp(m - l) + 1.0; m = l; }
  else if (l > -INFINITY) { s += exp(l - m); }
}

// Reduction record of the weight step: max, sum exp(l-m), sum exp(l-m)*l,
// sum exp(2(l-m)), count. Merged in a fixed tree order (deterministic).
struct WRed {
  double m, s, t, q;
  double n;
};
__device__ __forceinline__ WRed wred_empty() { WRed r; r.m = -INFINITY; r.s = r.t = r.q = 0.0; r.n = 0.0; return r; }
// FAST: the two rescaling factors e^{m_a - m}, e^{m_b - m} in single precision
// (single-precision runs); otherwise FP64.
template <bool FAST = false>
__device__ __forceinline__ WRed wred_merge(WRed a, WRed b) {
  if (b.m == -INFINITY) { a.n += b.n; return a; }
  if (a.m == -INFINITY) { b.n += a.n; return b; }
  WRed r;
  r.m = fmax(a.m, b.m);
  double ea = FAST ? (double)expf((float)(a.m - r.m)) : exp(a.m - r.m);
  double eb = FAST ? (double)expf((float)(b.m - r.m)) : exp(b.m - r.m);
  r.s = a.s * ea + b.s * eb;
  r.t = a.t * ea + b.t * eb;
  r.q = a.q * ea * ea + b.q * eb * eb;
  r.n = a.n + b.n;
  return r;
}
__device__ __forceinline__ WRed wred_shfl(WRed a, int off) {
  WRed b;
  b.m = __shfl_down_sync(0xffffffffu, a.m, off);
  b.s = __shfl_down_sync(0xffffffffu, a.s, off);
  b.t = __shfl_down_sync(0xffffffffu, a.t, off);
  b.q = __shfl_down_sync(0xffffffffu, a.q, off);
  b.n = __shfl_down_sync(0xffffffffu, a.n, off);
  return b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Index into a packed lower triangle, row-major (i >= j).
__host__ __device__ __forceinline__ int tri_idx(int i, int j) { return i * (i + 1) / 2 + j; }

// Device-side view of a mixture (proposal or Gaussian-mixture target).
struct DevMixView {
  int K, D, df, ldx;     // ldx: row stride of the single-precision sample rows
  const double *w;       // [K]
  const double *cw;      // [K] cumulative weights
  const double *mu;      // [K*D]
  const double *L;       // [K*D*D] lower Cholesky factor
  const double *Wt;      // [K*D*(D+1)/2] packed rows of L^-1
  const double *b;       // [K*D] L^-1 mu
  const double *lconst;  // [K] log w_k + normalising constant - log|L_k| (-inf for w_k == 0)
  const float *W32;      // [K*D*D] L^-1, row-major, zero above the diagonal
  const float *b32;      // [K*D]
  const float *lconst32; // [K]
  const float *L32;      // [K*D*ldx] L, rows padded to ldx, zero above the diagonal (single-precision draws)
  const float *mu32;     // [K*D]
  const unsigned char *bimg;  // tensor-core operand image of L^-1 (D <= 32), or null
  double cst;            // normalising constant of one component (depends on df and D only)
};

#define PMCG_CUDA_OK(expr) ((expr) == cudaSuccess)
