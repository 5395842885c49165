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
                                                   short *__restrict__ flg, int *__restrict__ counts,
                                                   const uint32_t *__restrict__ callp) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const uint32_t c = callp ? *callp : call;
  body_draw<MAXD, Real>(m, N, key0, key1, c, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx, flg, counts,
                        (size_t)blockIdx.x * blockDim.x, s_raw);
}

template <int MAXD, typename Real>
static cudaError_t draw_dispatch(const DevMixView &m, size_t N, uint64_t seed, uint32_t call, const double *bmin,
                                 const double *bmax, const double *pre_u, const double *pre_z,
                                 const double *pre_chi2, double *X64, float *X32, int *idx, short *flg,
                                 int *counts, cudaStream_t s, const uint32_t *callp) {
  const int bs = 128;
  const int ldo = (sizeof(Real) == 8) ? m.D : m.ldx;
  size_t smem = draw_smem<Real>(m.K, ldo, bs);
  unsigned grid = (unsigned)((N + bs - 1) / bs);
  if (grid == 0) return cudaSuccess;
  {
    cudaError_t e = allow_dyn_smem(draw_kernel<MAXD, Real>, smem);
    if (e != cudaSuccess) return e;
  }
  draw_kernel<MAXD, Real><<<grid, bs, smem, s>>>(m, N, (uint32_t)seed, (uint32_t)(seed >> 32), call, bmin, bmax,
                                                 pre_u, pre_z, pre_chi2, X64, X32, idx, flg, counts, callp);
  return cudaGetLastError();
}

cudaError_t launch_draw(int precision, const DevMixView &m, size_t N, uint64_t seed, uint32_t call,
                        const double *bmin, const double *bmax, const double *pre_u, const double *pre_z,
                        const double *pre_chi2, double *X64, float *X32, int *idx, short *flg, int *counts,
                        cudaStream_t s, const uint32_t *callp) {
  if (m.D < 1 || m.D > kMaxD || m.K < 1 || m.K > kMaxK) return cudaErrorInvalidValue;
#define PMCG_DRAW(MD)                                                                                          \
  return precision == 0                                                                                        \
             ? draw_dispatch<MD, double>(m, N, seed, call, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx,  \
                                         flg, counts, s, callp)                                                \
             : draw_dispatch<MD, float>(m, N, seed, call, bmin, bmax, pre_u, pre_z, pre_chi2, X64, X32, idx,   \
                                        flg, counts, s, callp)
  if (m.D <= 8) { PMCG_DRAW(8); }
  if (m.D <= 16) { PMCG_DRAW(16); }
  if (m.D <= 32) { PMCG_DRAW(32); }
  PMCG_DRAW(64);
#undef PMCG_DRAW
}

// ------------------------------------------------------------------ grouped draw
// Single-precision draws in three passes, so that the threads of a warp share
// one component's factor (broadcast reads) instead of gathering a different
// component's rows each: (1) component of every sample and the counts,
// (2) samples bucketed by component, (3) normals and transform in bucket
// order, rows written to the sample's own position. Every value equals the
// one-pass kernel's (same counters, same operations).

// Component k = min{k : u < C_k} (C non-decreasing), else the last component
// with positive weight. With u = A 2^-53 for the 53-bit integer A of the
// uniform, u < C_k <=> A < T_k = ceil(C_k 2^53) (C_k 2^53 is exact), so the
// binary search compares integers: the same pick as the FP64 comparison.
__device__ __forceinline__ int pick_component(const unsigned long long *s_T, const double *w, int K,
                                              unsigned long long A) {
  int lo = 0, hi = K;  // first index with A < T
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (A < s_T[mid]) hi = mid;
    else lo = mid + 1;
  }
  if (lo < K) return lo;
  for (int j = K - 1; j >= 0; j--)
    if (w[j] > 0.0) return j;
  return 0;
}

// Samples per block of the pick and bucket passes (kPickPer per thread): few
// blocks, so few global count / cursor atomics per component.
constexpr int kPickPer = 8;
constexpr int kPickBlock = 256 * kPickPer;

// Samples [n0, n1): component index, per-component counts (and, when ccounts
// is given, the counts of this range alone).
__global__ void __launch_bounds__(256) draw_pick_kernel(DevMixView m, size_t n0, size_t n1, uint32_t key0,
                                                        uint32_t key1, uint32_t call, const uint32_t *callp,
                                                        int *__restrict__ idx, int *__restrict__ counts,
                                                        int *__restrict__ ccounts) {
  extern __shared__ unsigned long long s_T[];
  if (callp) call = *callp;  // from device memory (iterations replayed as one graph)
  int *s_cnt = reinterpret_cast<int *>(s_T + m.K);
  for (int k = threadIdx.x; k < m.K; k += blockDim.x) {
    s_T[k] = (unsigned long long)ceil(m.cw[k] * 9007199254740992.0);
    s_cnt[k] = 0;
  }
  __syncthreads();
  const size_t b0 = n0 + (size_t)blockIdx.x * kPickBlock + threadIdx.x;
#pragma unroll
  for (int j = 0; j < kPickPer; j++) {
    const size_t n = b0 + (size_t)j * 256;
    if (n < n1) {
      P4 c = {0u, (uint32_t)n, (uint32_t)(n >> 32), call};
      P4 o = philox4x32_10(c, key0, key1);
      const unsigned long long A = ((unsigned long long)(o.x >> 5) << 26) | (unsigned long long)(o.y >> 6);
      const int k = pick_component(s_T, m.w, m.K, A);
      idx[n] = k;
      atomicAdd(&s_cnt[k], 1);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m.K; k += blockDim.x)
    if (s_cnt[k]) {
      atomicAdd(&counts[k], s_cnt[k]);
      if (ccounts) atomicAdd(&ccounts[k], s_cnt[k]);
    }
}

// Samples [n0, n1) bucketed by component: perm[off_k + r] = n with off_k the
// sum of the range's counts below k and r a block-local rank plus one
// reservation per (block, component); perm is indexed from the range start.
__global__ void __launch_bounds__(256) draw_bucket_kernel(size_t n0, size_t n1, int K, const int *__restrict__ idx,
                                                          const int *__restrict__ counts, int *__restrict__ cursor,
                                                          int *__restrict__ perm) {
  extern __shared__ int s_i[];
  int *s_off = s_i, *s_hist = s_i + K, *s_base = s_i + 2 * K;
  if (threadIdx.x == 0) {
    int o = 0;
    for (int k = 0; k < K; k++) { s_off[k] = o; o += counts[k]; }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) s_hist[k] = 0;
  __syncthreads();
  const size_t b0 = n0 + (size_t)blockIdx.x * kPickBlock + threadIdx.x;
  int kk[kPickPer], rr[kPickPer];
#pragma unroll
  for (int j = 0; j < kPickPer; j++) {
    const size_t n = b0 + (size_t)j * 256;
    kk[j] = 0; rr[j] = 0;
    if (n < n1) {
      kk[j] = idx[n];
      rr[j] = atomicAdd(&s_hist[kk[j]], 1);
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < K; j += blockDim.x)
    if (s_hist[j]) s_base[j] = s_off[j] + atomicAdd(&cursor[j], s_hist[j]);
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kPickPer; j++) {
    const size_t n = b0 + (size_t)j * 256;
    if (n < n1) perm[s_base[kk[j]] + rr[j]] = (int)n;
  }
}

// The cnt samples listed in perm (absolute sample indices), in list order.
// perm lists samples by component, so a block's samples nearly always share
// one: the rows of L_k and mu_k of the block's first sample are staged in
// shared memory (loads issued before the normals, so their latency overlaps
// the generator) and warps whose samples all belong to it read them there;
// any other warp reads its components from global memory.
// D <= 32: eight resident blocks (64 registers, a few spilled; measured 4%
// faster than six blocks at 74 registers); wider rows would spill heavily.
template <int MAXD>
__global__ void __launch_bounds__(128, MAXD <= 32 ? 8 : 1) draw_apply_kernel(DevMixView m, size_t cnt, uint32_t key0, uint32_t key1,
                                                         uint32_t call, const uint32_t *callp,
                                                         const double *__restrict__ bmin,
                                                         const double *__restrict__ bmax,
                                                         const int *__restrict__ perm, const int *__restrict__ idx,
                                                         float *__restrict__ X32, short *__restrict__ flg) {
  __shared__ __align__(16) float sL[MAXD * MAXD + MAXD];
  if (callp) call = *callp;
  const int D = m.D, ldx = m.ldx, df = m.df;
  const size_t p0 = (size_t)blockIdx.x * blockDim.x;  // < cnt: the grid covers cnt exactly
  const size_t p = p0 + threadIdx.x;
  const int kb = idx[perm[p0]];
  {
    const float4 *src = reinterpret_cast<const float4 *>(m.L32 + (size_t)kb * D * ldx);
    float4 *dst = reinterpret_cast<float4 *>(sL);
    for (int e = threadIdx.x; e < D * ldx / 4; e += blockDim.x) dst[e] = __ldg(src + e);
    for (int e = threadIdx.x; e < D; e += blockDim.x) sL[MAXD * MAXD + e] = __ldg(m.mu32 + (size_t)kb * D + e);
  }
  const bool live = p < cnt;
  const size_t n = live ? (size_t)perm[p] : 0;
  const int k = live ? idx[n] : kb;
  float z[MAXD];
  float c2 = 0.f;
  if (live) draw_normals<MAXD, float>(D, df > 0 ? df : 0, (uint32_t)n, (uint32_t)(n >> 32), call, key0, key1, z, c2);
  __syncthreads();
  const bool staged = __all_sync(0xffffffffu, k == kb);
  if (!live) return;
  const float sc = (df > 0) ? student_scale<float>(df, c2) : 1.f;
  float *row = X32 + n * ldx;
  const int in = staged ? draw_transform_store<MAXD, true>(D, ldx, sL, sL + MAXD * MAXD, z, sc, bmin, bmax, row)
                        : draw_transform_store<MAXD, false>(D, ldx, m.L32 + (size_t)k * D * ldx,
                                                            m.mu32 + (size_t)k * D, z, sc, bmin, bmax, row);
  flg[n] = (short)in;
}

cudaError_t launch_draw_grouped_range(const DevMixView &m, size_t N, size_t n0, size_t n1, uint64_t seed,
                                      uint32_t call, const double *bmin, const double *bmax, float *X32, int *idx,
                                      short *flg, int *counts, int *perm, int *cursor, cudaStream_t s,
                                      const uint32_t *callp) {
  if (m.D < 1 || m.D > kMaxD || m.K < 1 || m.K > kMaxK) return cudaErrorInvalidValue;
  if (N > (size_t)INT32_MAX || n0 > n1 || n1 > N) return cudaErrorInvalidValue;
  if (n1 == n0) return cudaSuccess;
  const bool whole = (n0 == 0 && n1 == N);
  int *ccounts = whole ? nullptr : cursor + m.K;  // the range's own counts (bucket offsets)
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const size_t cnt = n1 - n0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(cursor, 0, sizeof(int) * m.K * (whole ? 1 : 2), s)) != cudaSuccess) return e;
  const unsigned gp = (unsigned)((cnt + kPickBlock - 1) / kPickBlock);
  draw_pick_kernel<<<gp, 256, (size_t)m.K * 12, s>>>(m, n0, n1, k0, k1, call, callp, idx, counts, ccounts);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  draw_bucket_kernel<<<gp, 256, (size_t)m.K * 12, s>>>(n0, n1, m.K, idx, whole ? counts : ccounts, cursor,
                                                        perm + n0);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const unsigned g128 = (unsigned)((cnt + 127) / 128);
#define PMCG_APPLY(MD) \
  draw_apply_kernel<MD><<<g128, 128, 0, s>>>(m, cnt, k0, k1, call, callp, bmin, bmax, perm + n0, idx, X32, flg)
  if (m.ldx <= 8) PMCG_APPLY(8);
  else if (m.ldx <= 16) PMCG_APPLY(16);
  else if (m.ldx <= 32) PMCG_APPLY(32);
  else PMCG_APPLY(64);
#undef PMCG_APPLY
  return cudaGetLastError();
}

cudaError_t launch_draw_grouped(const DevMixView &m, size_t N, uint64_t seed, uint32_t call, const double *bmin,
                                const double *bmax, float *X32, int *idx, short *flg, int *counts, int *perm,
                                int *cursor, cudaStream_t s, const uint32_t *callp) {
  return launch_draw_grouped_range(m, N, 0, N, seed, call, bmin, bmax, X32, idx, flg, counts, perm, cursor, s,
                                   callp);
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

// Samples with a non-zero flag (warp ballots, one integer atomic per warp: exact).
__global__ void count_flags_kernel(size_t N, const short *__restrict__ flg, int *__restrict__ out) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  int c = 0;
  for (size_t n0 = (size_t)blockIdx.x * blockDim.x; n0 < N; n0 += stride) {
    const size_t n = n0 + threadIdx.x;
    c += __popc(__ballot_sync(0xffffffffu, n < N && flg[n] != 0));
  }
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

cudaError_t launch_count_flags(size_t N, const short *flg, int *out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int), s);
  if (e != cudaSuccess || N == 0) return e;
  size_t grid = (N + 255) / 256;
  if (grid > 1024) grid = 1024;
  count_flags_kernel<<<(unsigned)grid, 256, 0, s>>>(N, flg, out);
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
