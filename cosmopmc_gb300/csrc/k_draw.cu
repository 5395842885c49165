// k_draw.cu — (a) proposal draws: component selection from a 53-bit uniform
// and the Cholesky transform of normal (or Student-t) variates.
// Replaces pmclib simulate_mix_mvdens (called at exec/cosmo_pmc.c:320).
#include "pmcg_kernels.h"

namespace pmcg {

// Box-Muller pair from one Philox block. FP64 path: two 53-bit uniforms (the
// oracle's mapping). FP32 path: the same 53-bit integers, 1-a and b, rounded
// once to float (integer conversions, no FP64 arithmetic), so its normals equal
// the FP64 ones to single precision, tails included.
template <typename Real>
__device__ __forceinline__ void box_muller(P4 o, Real &g0, Real &g1);

template <>
__device__ __forceinline__ void box_muller<double>(P4 o, double &g0, double &g1) {
  double a = u53(o.x, o.y), b = u53(o.z, o.w);
  double r = sqrt(-2.0 * log1p(-a));
  double sn, cs;
  sincospi(2.0 * b, &sn, &cs);
  g0 = r * cs;
  g1 = r * sn;
}
template <>
__device__ __forceinline__ void box_muller<float>(P4 o, float &g0, float &g1) {
  const unsigned long long A = ((unsigned long long)(o.x >> 5) << 26) | (unsigned long long)(o.y >> 6);
  const unsigned long long B = ((unsigned long long)(o.z >> 5) << 26) | (unsigned long long)(o.w >> 6);
  const float two53inv = 1.1102230246251565e-16f;  // 2^-53
  const float oma = __ull2float_rn((1ull << 53) - A) * two53inv;  // 1 - a in (0, 1]
  const float b = __ull2float_rn(B) * two53inv;
  float r = sqrtf(-2.0f * logf(oma));
  float sn, cs;
  sincospif(2.0f * b, &sn, &cs);
  g0 = r * cs;
  g1 = r * sn;
}

// One thread per sample; the block stages its rows in shared memory so the
// sample matrix is written with coalesced stores.
template <int MAXD, typename Real>
__global__ void __launch_bounds__(128) draw_kernel(DevMixView m, size_t N, uint32_t key0, uint32_t key1,
                                                   uint32_t call, const double *__restrict__ bmin,
                                                   const double *__restrict__ bmax, const double *__restrict__ pre_u,
                                                   const double *__restrict__ pre_z,
                                                   const double *__restrict__ pre_chi2, double *__restrict__ X64,
                                                   float *__restrict__ X32, int *__restrict__ idx,
                                                   short *__restrict__ flg, int *__restrict__ counts) {
  __shared__ double s_cw[kMaxK];
  __shared__ int s_cnt[kMaxK];
  extern __shared__ unsigned char s_raw[];
  Real *s_x = reinterpret_cast<Real *>(s_raw);

  const int K = m.K, D = m.D, df = m.df;
  const int ldo = (sizeof(Real) == 8) ? D : m.ldx;
  for (int k = threadIdx.x; k < K; k += blockDim.x) { s_cw[k] = m.cw[k]; s_cnt[k] = 0; }
  __syncthreads();

  const size_t n0 = (size_t)blockIdx.x * blockDim.x;
  const size_t n = n0 + threadIdx.x;
  if (n < N) {
    const uint32_t nlo = (uint32_t)n, nhi = (uint32_t)(n >> 32);
    double u;
    if (pre_u) {
      u = pre_u[n];
    } else {
      P4 c = {0u, nlo, nhi, call};
      P4 o = philox4x32_10(c, key0, key1);
      u = u53(o.x, o.y);
    }
    int k = -1;
    for (int j = 0; j < K; j++)
      if (u < s_cw[j]) { k = j; break; }
    if (k < 0)
      for (int j = K - 1; j >= 0; j--)
        if (m.w[j] > 0.0) { k = j; break; }
    if (k < 0) k = 0;

    const int nu = df > 0 ? df : 0;
    Real z[MAXD];
    Real c2 = (Real)0;
    if (pre_z) {
#pragma unroll
      for (int i = 0; i < MAXD; i++) z[i] = (i < D) ? (Real)pre_z[n * D + i] : (Real)0;
      c2 = pre_chi2 ? (Real)pre_chi2[n] : (Real)1;
    } else {
#pragma unroll
      for (int mm = 0; mm < MAXD / 2; mm++) {
        if (2 * mm < D) {
          P4 c = {1u + (uint32_t)mm, nlo, nhi, call};
          P4 o = philox4x32_10(c, key0, key1);
          Real g0, g1;
          box_muller<Real>(o, g0, g1);
          z[2 * mm] = g0;
          if (2 * mm + 1 < D) {
            z[2 * mm + 1] = g1;
          } else {
            z[2 * mm + 1] = (Real)0;
            if (nu > 0) c2 += g1 * g1;
          }
        } else {
          z[2 * mm] = (Real)0;
          z[2 * mm + 1] = (Real)0;
        }
      }
      const int jstart = (D % 2 == 0) ? D : D + 1;
      for (int j = jstart; j < D + nu; j += 2) {
        P4 c = {1u + (uint32_t)(j / 2), nlo, nhi, call};
        P4 o = philox4x32_10(c, key0, key1);
        Real g0, g1;
        box_muller<Real>(o, g0, g1);
        c2 += g0 * g0;
        if (j + 1 < D + nu) c2 += g1 * g1;
      }
    }
    const Real sc = (df > 0) ? (Real)sqrt((double)df / (double)c2) : (Real)1;
    // Factor and mean in the arithmetic type of the path (no per-element conversions).
    const Real *Lk = (sizeof(Real) == 8) ? (const Real *)(m.L + (size_t)k * D * D)
                                         : (const Real *)(m.L32 + (size_t)k * D * D);
    const Real *mk = (sizeof(Real) == 8) ? (const Real *)(m.mu + (size_t)k * D) : (const Real *)(m.mu32 + (size_t)k * D);
    int in = 1;
#pragma unroll
    for (int i = 0; i < MAXD; i++) {
      if (i < D) {
        Real acc = (Real)0;
#pragma unroll
        for (int j = 0; j <= i; j++) acc += __ldg(&Lk[i * D + j]) * z[j];
        Real xi = __ldg(&mk[i]) + sc * acc;
        s_x[threadIdx.x * ldo + i] = xi;
        if (bmin && ((double)xi < bmin[i] || (double)xi > bmax[i])) in = 0;
      }
    }
    for (int i = D; i < ldo; i++) s_x[threadIdx.x * ldo + i] = (Real)0;
    idx[n] = k;
    flg[n] = (short)in;
    atomicAdd(&s_cnt[k], 1);
  }
  __syncthreads();
  // coalesced copy of the block's rows
  const size_t rows = (N - n0 < (size_t)blockDim.x) ? (N - n0) : (size_t)blockDim.x;
  const size_t tot = rows * (size_t)ldo;
  if (sizeof(Real) == 8) {
    for (size_t e = threadIdx.x; e < tot; e += blockDim.x) X64[n0 * ldo + e] = (double)s_x[e];
  } else {
    for (size_t e = threadIdx.x; e < tot; e += blockDim.x) X32[n0 * ldo + e] = (float)s_x[e];
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (s_cnt[k]) atomicAdd(&counts[k], s_cnt[k]);
}

template <int MAXD, typename Real>
static cudaError_t draw_dispatch(const DevMixView &m, size_t N, uint64_t seed, uint32_t call, const double *bmin,
                                 const double *bmax, const double *pre_u, const double *pre_z,
                                 const double *pre_chi2, double *X64, float *X32, int *idx, short *flg,
                                 int *counts, cudaStream_t s) {
  const int bs = 128;
  const int ldo = (sizeof(Real) == 8) ? m.D : m.ldx;
  size_t smem = (size_t)bs * ldo * sizeof(Real);
  unsigned grid = (unsigned)((N + bs - 1) / bs);
  if (grid == 0) return cudaSuccess;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(draw_kernel<MAXD, Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  draw_kernel<MAXD, Real><<<grid, bs, smem, s>>>(m, N, (uint32_t)seed, (uint32_t)(seed >> 32), call, bmin, bmax,
                                                 pre_u, pre_z, pre_chi2, X64, X32, idx, flg, counts);
  return cudaGetLastError();
}

cudaError_t launch_draw(int precision, const DevMixView &m, size_t N, uint64_t seed, uint32_t call,
                        const double *bmin, const double *bmax, const double *pre_u, const double *pre_z,
                        const double *pre_chi2, double *X64, float *X32, int *idx, short *flg, int *counts,
                        cudaStream_t s) {
  if (m.D < 1 || m.D > kMaxD || m.K < 1 || m.K > kMaxK) return cudaErrorInvalidValue;
#define PMCG_DRAW(MD)                                                                                          \
  return precision == 0                                                                                        \
             ? draw_dispatch<MD, double>(m, N, seed, call, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx,  \
                                         flg, counts, s)                                                       \
             : draw_dispatch<MD, float>(m, N, seed, call, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx,   \
                                        flg, counts, s)
  if (m.D <= 8) { PMCG_DRAW(8); }
  if (m.D <= 16) { PMCG_DRAW(16); }
  if (m.D <= 32) { PMCG_DRAW(32); }
  PMCG_DRAW(64);
#undef PMCG_DRAW
}

__global__ void x32_to_x64_kernel(size_t N, int D, int ldx, const float *__restrict__ X32, double *__restrict__ X64) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t tot = N * (size_t)D;
  for (; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    size_t n = e / D;
    int i = (int)(e - n * D);
    X64[e] = (double)X32[n * ldx + i];
  }
}

cudaError_t launch_x32_to_x64(size_t N, int D, int ldx, const float *X32, double *X64, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  size_t tot = N * (size_t)D;
  unsigned grid = (unsigned)((tot + 255) / 256 < 4096 ? (tot + 255) / 256 : 4096);
  x32_to_x64_kernel<<<grid, 256, 0, s>>>(N, D, ldx, X32, X64);
  return cudaGetLastError();
}

__global__ void fill_f64_kernel(double *p, size_t n, double v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
cudaError_t launch_fill_f64(double *p, size_t n, double v, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unsigned grid = (unsigned)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
  fill_f64_kernel<<<grid, 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

}  // namespace pmcg

namespace pmcg {

__global__ void x64_to_x32_kernel(size_t N, int D, int ldx, const double *__restrict__ X64, float *__restrict__ X32) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t tot = N * (size_t)ldx;
  for (; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    size_t n = e / ldx;
    int i = (int)(e - n * ldx);
    X32[e] = (i < D) ? (float)X64[n * D + i] : 0.0f;
  }
}

cudaError_t launch_x64_to_x32(size_t N, int D, int ldx, const double *X64, float *X32, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  size_t tot = N * (size_t)ldx;
  unsigned grid = (unsigned)((tot + 255) / 256 < 4096 ? (tot + 255) / 256 : 4096);
  x64_to_x32_kernel<<<grid, 256, 0, s>>>(N, D, ldx, X64, X32);
  return cudaGetLastError();
}

// Draw counts per component from uploaded indices (integer atomics: exact).
__global__ void counts_kernel(size_t N, int K, const int *__restrict__ idx, int *__restrict__ counts) {
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    int k = idx[n];
    if (k >= 0 && k < K) atomicAdd(&counts[k], 1);
  }
}

cudaError_t launch_counts(size_t N, int K, const int *idx, int *counts, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * K, s);
  if (e != cudaSuccess || N == 0) return e;
  unsigned grid = (unsigned)((N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024);
  counts_kernel<<<grid, 256, 0, s>>>(N, K, idx, counts);
  return cudaGetLastError();
}

// Normalised weights uploaded by the caller -> log-weights (0 -> -inf).
__global__ void log_weights_kernel(size_t N, double *w, const short *flg) {
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x)
    w[n] = (flg[n] && w[n] > 0.0) ? log(w[n]) : -INFINITY;
}

cudaError_t launch_log_weights(size_t N, double *w, const short *flg, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  unsigned grid = (unsigned)((N + 255) / 256 < 1024 ? (N + 255) / 256 : 1024);
  log_weights_kernel<<<grid, 256, 0, s>>>(N, w, flg);
  return cudaGetLastError();
}

}  // namespace pmcg
