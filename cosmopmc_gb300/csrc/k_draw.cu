// k_draw.cu — (a) proposal draws: component selection from a 53-bit uniform
// and the Cholesky transform of normal (or Student-t) variates.
// Replaces pmclib simulate_mix_mvdens (called at exec/cosmo_pmc.c:320).
// The body (body_draw) is shared with the batch kernel.
#include "pmcg_bodies.cuh"

namespace pmcg {

template <int MAXD, typename Real>
__global__ void __launch_bounds__(128) draw_kernel(DevMixView m, size_t N, uint32_t key0, uint32_t key1,
                                                   uint32_t call, const double *__restrict__ bmin,
                                                   const double *__restrict__ bmax, const double *__restrict__ pre_u,
                                                   const double *__restrict__ pre_z,
                                                   const double *__restrict__ pre_chi2, double *__restrict__ X64,
                                                   float *__restrict__ X32, int *__restrict__ idx,
                                                   short *__restrict__ flg, int *__restrict__ counts) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  body_draw<MAXD, Real>(m, N, key0, key1, call, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx, flg, counts,
                        (size_t)blockIdx.x * blockDim.x, s_raw);
}

template <int MAXD, typename Real>
static cudaError_t draw_dispatch(const DevMixView &m, size_t N, uint64_t seed, uint32_t call, const double *bmin,
                                 const double *bmax, const double *pre_u, const double *pre_z,
                                 const double *pre_chi2, double *X64, float *X32, int *idx, short *flg,
                                 int *counts, cudaStream_t s) {
  const int bs = 128;
  const int ldo = (sizeof(Real) == 8) ? m.D : m.ldx;
  size_t smem = draw_smem<Real>(m.K, ldo, bs);
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

// ------------------------------------------------------------------ helpers
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

__global__ void fill_f64_kernel(double *p, size_t n, double v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
cudaError_t launch_fill_f64(double *p, size_t n, double v, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unsigned grid = (unsigned)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
  fill_f64_kernel<<<grid, 256, 0, s>>>(p, n, v);
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
