// k_em.cu — (e) Rao-Blackwellised EM update of the proposal (Cappe et al.
// 2008), replacing pmclib update_prop_rb (exec/cosmo_pmc.c:247) including the
// burial of dead components (Manual/manual.tex:479-500).
//
// For component k with old mean c, per sample n (flg == 1):
//   v  = wbar_n * rho_nk = exp(logw_n - logSum - logq_n + lt_nk)
//   vt = v * tau_nk, tau = (nu+D)/(nu+Q_nk) for Student-t, 1 for Gaussian
// Statistics (the "E layout", E = 2 + D + D(D+1)/2 doubles):
//   [0] S0 = sum v, [1] St = sum vt, [2+i] S1_i = sum vt (x-c)_i,
//   [2+D+tri(i,j)] S2_ij = sum vt (x-c)_i (x-c)_j.
// Then mu' = c + S1/St, Sigma' = (S2 - St d d^T)/S0 with d = mu'-c, alpha' = S0.
// Each block covers one component and one contiguous chunk of samples and
// writes its partial statistics; the finalise kernel sums the chunks in a
// fixed order (deterministic), factorises Sigma' in FP64 and applies the
// dead-component rule.
#include "pmcg_kernels.h"

namespace pmcg {

constexpr int kMinCount = 20;  // MINCOUNT, Manual/manual.tex:483

__host__ __device__ inline int em_E(int D) { return 2 + D + D * (D + 1) / 2; }

// ------------------------------------------------------------------ FP64 statistics
constexpr int kTile64 = 32;

__global__ void __launch_bounds__(256) em_stats_f64_kernel(DevMixView m, size_t N, int S,
                                                           const double *__restrict__ X,
                                                           const double *__restrict__ logw,
                                                           const double *__restrict__ logq,
                                                           const double *__restrict__ lt,
                                                           const double *__restrict__ Qv, const DevStats *st,
                                                           double *__restrict__ part) {
  const int k = blockIdx.y, s = blockIdx.x, D = m.D, E = em_E(D);
  if (m.w[k] <= 0.0) return;  // buried: no statistics needed
  extern __shared__ double sm[];
  double *sx = sm;                        // kTile64 * D
  double *sv = sx + kTile64 * D;          // kTile64
  double *svt = sv + kTile64;             // kTile64
  const size_t chunk = (N + S - 1) / S;
  const size_t n0 = (size_t)s * chunk, n1 = (n0 + chunk < N) ? n0 + chunk : N;
  const double logSum = st->logSum;
  const double *ck = m.mu + (size_t)k * D;
  const double nu = (double)m.df;
  constexpr int kOwn = 10;  // up to 10 entries per thread (E <= 2560)
  double acc[kOwn];
  int ei[kOwn], ej[kOwn];
#pragma unroll
  for (int r = 0; r < kOwn; r++) {
    acc[r] = 0.0;
    int e = threadIdx.x + r * blockDim.x;
    ei[r] = -3; ej[r] = -3;
    if (e < E) {
      if (e == 0) { ei[r] = -2; }
      else if (e == 1) { ei[r] = -1; }
      else if (e < 2 + D) { ei[r] = e - 2; ej[r] = -1; }
      else {
        int t = e - 2 - D, i = 0;
        while (tri_idx(i + 1, 0) <= t) i++;
        ei[r] = i; ej[r] = t - tri_idx(i, 0);
      }
    }
  }
  for (size_t t0 = n0; t0 < n1; t0 += kTile64) {
    const int nt = (int)((n1 - t0 < (size_t)kTile64) ? (n1 - t0) : (size_t)kTile64);
    __syncthreads();
    if (threadIdx.x < kTile64) {
      double v = 0.0, vt = 0.0;
      if (threadIdx.x < nt) {
        size_t n = t0 + threadIdx.x;
        double lw = logw[n];
        if (lw > -INFINITY) {
          v = exp(lw - logSum - logq[n] + lt[(size_t)k * N + n]);
          vt = (m.df > 0) ? v * (nu + D) / (nu + Qv[(size_t)k * N + n]) : v;
        }
      }
      sv[threadIdx.x] = v;
      svt[threadIdx.x] = vt;
    }
    for (int e = threadIdx.x; e < kTile64 * D; e += blockDim.x) {
      int r = e / D, i = e - r * D;
      sx[e] = (r < nt) ? X[(t0 + r) * D + i] - ck[i] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kOwn; r++) {
      if (ei[r] == -3) continue;
      double a = acc[r];
      if (ei[r] == -2) { for (int q = 0; q < nt; q++) a += sv[q]; }
      else if (ei[r] == -1) { for (int q = 0; q < nt; q++) a += svt[q]; }
      else if (ej[r] == -1) { const int i = ei[r]; for (int q = 0; q < nt; q++) a = fma(svt[q], sx[q * D + i], a); }
      else {
        const int i = ei[r], j = ej[r];
        for (int q = 0; q < nt; q++) a = fma(svt[q] * sx[q * D + i], sx[q * D + j], a);
      }
      acc[r] = a;
    }
  }
  double *out = part + ((size_t)k * S + s) * E;
#pragma unroll
  for (int r = 0; r < kOwn; r++) {
    int e = threadIdx.x + r * blockDim.x;
    if (e < E) out[e] = acc[r];
  }
}

// ------------------------------------------------------------------ FP32 statistics
// Mixed path: the statistics are accumulated in each component's whitened
// frame a = L_k^-1 (x - mu_k) (entries O(1)), because a covariance of
// condition 1e6 cannot even be represented to its small eigenvalues in FP32
// in the raw frame. The finalise kernel maps them back in FP64:
// mu' = mu + L d_w, Sigma' = L Sigma_w L^T.
//
// Per tile of 64 samples: x rows are staged (row stride ldx+1: conflict-free
// column reads), then whitened with L^-1 staged transposed (float4 broadcasts,
// warps paired over i-blocks so every warp does the same number of steps).
// The augmented rows a = [a (padded to Dp), 1, 1/tau, 0, 0] with weight vt give,
// in the lower triangle of sum vt a a^T, S2 (whitened), S1 (row Dp), St (Dp,Dp)
// and S0 (Dp+1,Dp). Each thread owns one 4x4 block for one sample group; FP32
// sums are flushed into FP64 every kFlushTiles tiles.
constexpr int kTile32 = 64;
constexpr int kFlushTiles = 16;

__global__ void __launch_bounds__(256) em_stats_f32_kernel(DevMixView m, size_t N, int S,
                                                           const float *__restrict__ X,
                                                           const float *__restrict__ aw,
                                                           const float *__restrict__ lt,
                                                           const float *__restrict__ Qv,
                                                           double *__restrict__ part) {
  const int k = blockIdx.x, s = blockIdx.y, D = m.D, E = em_E(D);
  if (m.w[k] <= 0.0) return;
  const int Dp = m.ldx, Da = Dp + 4, nb = Da / 4, NB = nb * (nb + 1) / 2, nib = Dp / 4;
  const int ldt = Dp + 1;  // padded x-tile row stride
  const int G = blockDim.x / NB;
  extern __shared__ float4 smf4[];
  float *sWT = reinterpret_cast<float *>(smf4);   // [Dp][Dp]  (L^-1)^T
  float *sb = sWT + Dp * Dp;                      // [Dp]      L^-1 mu
  float *sa = sb + Dp;                            // [kTile32][Da] augmented whitened rows
  float *sx = sa + kTile32 * Da;                  // [kTile32][ldt] raw rows
  float *svt = sx + kTile32 * ldt;                // [kTile32]
  const size_t chunk = (N + S - 1) / S;
  const size_t n0 = (size_t)s * chunk, n1 = (n0 + chunk < N) ? n0 + chunk : N;
  const float nu = (float)m.df, rnd = 1.0f / ((float)m.df + (float)D);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;

  for (int e = tid; e < Dp * Dp; e += blockDim.x) {
    int i = e / Dp, j = e - i * Dp;  // sWT[j][i] = W[i][j]
    sWT[j * Dp + i] = (i < D) ? m.W32[(size_t)k * D * Dp + (size_t)i * Dp + j] : 0.f;
  }
  for (int i = tid; i < Dp; i += blockDim.x) sb[i] = (i < D) ? m.b32[(size_t)k * D + i] : 0.f;

  const int blk = tid % NB, grp = tid / NB;
  const bool active = grp < G;
  int bi = 0;
  while ((bi + 1) * (bi + 2) / 2 <= blk) bi++;
  const int bj = blk - bi * (bi + 1) / 2;

  float acc[16];
  double acc64[16];
#pragma unroll
  for (int e = 0; e < 16; e++) { acc[e] = 0.f; acc64[e] = 0.0; }
  int tiles = 0;
  for (size_t t0 = n0; t0 < n1; t0 += kTile32) {
    const int nt = (int)((n1 - t0 < (size_t)kTile32) ? (n1 - t0) : (size_t)kTile32);
    __syncthreads();
    if (tid < kTile32) {
      float vt = 0.f, itau = 1.f;
      if (tid < nt) {
        const size_t n = t0 + tid;
        const float v = expf(aw[n] + lt[(size_t)k * N + n]);  // aw = -inf where flg == 0
        if (m.df > 0) {
          itau = (nu + Qv[(size_t)k * N + n]) * rnd;
          vt = v / itau;
        } else {
          vt = v;
        }
      }
      svt[tid] = vt;
      float *row = sa + tid * Da;
      row[Dp] = 1.f;
      row[Dp + 1] = itau;
      row[Dp + 2] = 0.f;
      row[Dp + 3] = 0.f;
    }
    for (int e = tid; e < kTile32 * Dp; e += blockDim.x) {
      const int r = e / Dp, i = e - r * Dp;
      sx[r * ldt + i] = (r < nt) ? X[(t0 + r) * Dp + i] : 0.f;
    }
    __syncthreads();
    // whitening: unit u = (i-block ib, half h of the tile); warp w takes units
    // (w, 0) and (nib-1-w, 1) so the triangular lengths balance.
    for (int u = warp; u < 2 * nib; u += nwarp) {
      const int pair = u % nib, half = u / nib;
      const int ib = half == 0 ? pair : nib - 1 - pair;
      const int r = half * 32 + lane;
      float o0 = -sb[4 * ib], o1 = -sb[4 * ib + 1], o2 = -sb[4 * ib + 2], o3 = -sb[4 * ib + 3];
      const float *xr = sx + r * ldt;
      const int jmax = 4 * ib + 4;
      for (int j = 0; j < jmax; j++) {
        const float xv = xr[j];
        const float4 w4 = *reinterpret_cast<const float4 *>(sWT + j * Dp + 4 * ib);
        o0 = fmaf(w4.x, xv, o0); o1 = fmaf(w4.y, xv, o1); o2 = fmaf(w4.z, xv, o2); o3 = fmaf(w4.w, xv, o3);
      }
      float *ar = sa + r * Da + 4 * ib;
      const bool live = r < nt;
      ar[0] = live ? o0 : 0.f; ar[1] = live ? o1 : 0.f; ar[2] = live ? o2 : 0.f; ar[3] = live ? o3 : 0.f;
    }
    __syncthreads();
    if (active) {
      for (int q = grp; q < nt; q += G) {
        const float w = svt[q];
        float4 ai = *reinterpret_cast<const float4 *>(sa + q * Da + 4 * bi);
        const float4 aj = *reinterpret_cast<const float4 *>(sa + q * Da + 4 * bj);
        ai.x *= w; ai.y *= w; ai.z *= w; ai.w *= w;
        acc[0] = fmaf(ai.x, aj.x, acc[0]);   acc[1] = fmaf(ai.x, aj.y, acc[1]);
        acc[2] = fmaf(ai.x, aj.z, acc[2]);   acc[3] = fmaf(ai.x, aj.w, acc[3]);
        acc[4] = fmaf(ai.y, aj.x, acc[4]);   acc[5] = fmaf(ai.y, aj.y, acc[5]);
        acc[6] = fmaf(ai.y, aj.z, acc[6]);   acc[7] = fmaf(ai.y, aj.w, acc[7]);
        acc[8] = fmaf(ai.z, aj.x, acc[8]);   acc[9] = fmaf(ai.z, aj.y, acc[9]);
        acc[10] = fmaf(ai.z, aj.z, acc[10]); acc[11] = fmaf(ai.z, aj.w, acc[11]);
        acc[12] = fmaf(ai.w, aj.x, acc[12]); acc[13] = fmaf(ai.w, aj.y, acc[13]);
        acc[14] = fmaf(ai.w, aj.z, acc[14]); acc[15] = fmaf(ai.w, aj.w, acc[15]);
      }
    }
    if (++tiles == kFlushTiles) {
      tiles = 0;
#pragma unroll
      for (int e = 0; e < 16; e++) { acc64[e] += (double)acc[e]; acc[e] = 0.f; }
    }
  }
#pragma unroll
  for (int e = 0; e < 16; e++) acc64[e] += (double)acc[e];
  // reduce the sample groups in a fixed order
  __syncthreads();
  double *red = reinterpret_cast<double *>(smf4);  // G * NB * 16 doubles
  if (active) {
#pragma unroll
    for (int e = 0; e < 16; e++) red[((size_t)grp * NB + blk) * 16 + e] = acc64[e];
  }
  __syncthreads();
  double *out = part + ((size_t)k * S + s) * E;
  if (grp == 0) {
    for (int e = 0; e < 16; e++) {
      double t = red[(size_t)blk * 16 + e];
      for (int g = 1; g < G; g++) t += red[((size_t)g * NB + blk) * 16 + e];
      const int r = 4 * bi + e / 4, c = 4 * bj + e % 4;
      if (r < D && c <= r) out[2 + D + tri_idx(r, c)] = t;
      else if (r == Dp && c < D) out[2 + c] = t;
      else if (r == Dp && c == Dp) out[1] = t;
      else if (r == Dp + 1 && c == Dp) out[0] = t;
    }
  }
}

// Per-sample single-precision weight factor of the mixed EM:
// aw = log w - logSum - log q (-inf where flg == 0), one FP64 subtraction per sample.
__global__ void em_weight_factor_kernel(size_t N, const double *__restrict__ logw, const double *__restrict__ logq,
                                        const DevStats *__restrict__ st, float *__restrict__ aw) {
  const double ls = st->logSum;
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    const double l = logw[n];
    aw[n] = (l > -INFINITY) ? (float)(l - ls - logq[n]) : -INFINITY;
  }
}

size_t em_partials_size(int precision, int K, int D, int *S_out, size_t N) {
  int S = (8 * 152 + K - 1) / K;
  size_t maxS = (N + 2047) / 2048;
  if (maxS < 1) maxS = 1;
  if ((size_t)S > maxS) S = (int)maxS;
  if (S < 1) S = 1;
  *S_out = S;
  return (size_t)K * S * em_E(D) * sizeof(double);
}

// ------------------------------------------------------------------ finalise
// One block per component: fixed-order sum of the chunk partials, new mean
// and covariance, band limit, FP64 Cholesky; the dead rule buries the
// component (weight 0, parameters kept). With whitened statistics (mixed
// path) the moments are mapped back with the old factor: mu' = mu + L d,
// Sigma' = L Sigma_w L^T, all in FP64.
__global__ void em_finalize_kernel(DevMixView m, double *w, double *mu, double *L, size_t N, int S,
                                   const double *__restrict__ part, const int *__restrict__ counts,
                                   int band_limit, int whitened) {
  const int k = blockIdx.x, D = m.D, E = em_E(D);
  extern __shared__ double sh[];
  double *st = sh;             // E
  double *C = st + E;          // D*D
  double *Lo = C + D * D;      // D*D old factor (whitened only)
  double *T = Lo + D * D;      // D*D scratch (whitened only)
  __shared__ int s_dead;
  __shared__ double s_piv;
  if (m.w[k] <= 0.0) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    double t = 0.0;
    for (int s = 0; s < S; s++) t += part[((size_t)k * S + s) * E + e];
    st[e] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double S0 = st[0], St = st[1];
    s_dead = (counts[k] < kMinCount) || !(S0 >= 1.0 / (double)N) || !(St > 0.0) || !isfinite(S0) || !isfinite(St);
  }
  __syncthreads();
  if (s_dead) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  const double S0 = st[0], St = st[1];
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    int i = e / D, j = e - i * D;
    int a = i > j ? i : j, b = i > j ? j : i;
    double di = st[2 + i] / St, dj = st[2 + j] / St;
    C[e] = (st[2 + D + tri_idx(a, b)] - St * di * dj) / S0;
    if (whitened) Lo[e] = (j <= i) ? m.L[(size_t)k * D * D + e] : 0.0;
  }
  __syncthreads();
  if (whitened) {
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // T = Lo C
      int i = e / D, j = e - i * D;
      double t = 0.0;
      for (int q = 0; q <= i; q++) t += Lo[i * D + q] * C[q * D + j];
      T[e] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // C = T Lo^T
      int i = e / D, j = e - i * D;
      double t = 0.0;
      for (int q = 0; q <= j; q++) t += T[i * D + q] * Lo[j * D + q];
      C[e] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // symmetrise exactly
      int i = e / D, j = e - i * D;
      if (j < i) { double v = 0.5 * (C[i * D + j] + C[j * D + i]); T[e] = v; }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      int i = e / D, j = e - i * D;
      if (j < i) { C[i * D + j] = T[e]; C[j * D + i] = T[e]; }
    }
    __syncthreads();
  }
  if (band_limit > 0 && band_limit < D) {
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      int i = e / D, j = e - i * D;
      if ((i > j ? i - j : j - i) >= band_limit) C[e] = 0.0;
    }
    __syncthreads();
  }
  // in-place Cholesky, column by column
  for (int j = 0; j < D; j++) {
    if (threadIdx.x == 0) {
      double d = C[j * D + j];
      for (int q = 0; q < j; q++) d -= C[j * D + q] * C[j * D + q];
      if (!(d > 0.0) || !isfinite(d)) { s_dead = 1; d = 1.0; }
      s_piv = sqrt(d);
      C[j * D + j] = s_piv;
    }
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < D; i += blockDim.x) {
      double t = C[i * D + j];
      for (int q = 0; q < j; q++) t -= C[i * D + q] * C[j * D + q];
      C[i * D + j] = t / s_piv;
    }
    __syncthreads();
  }
  if (s_dead) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    double d;
    if (whitened) {
      d = 0.0;
      for (int q = 0; q <= i; q++) d += Lo[i * D + q] * (st[2 + q] / St);
    } else {
      d = st[2 + i] / St;
    }
    mu[(size_t)k * D + i] = m.mu[(size_t)k * D + i] + d;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    int i = e / D, j = e - i * D;
    L[(size_t)k * D * D + e] = (j <= i) ? C[e] : 0.0;
  }
  if (threadIdx.x == 0) w[k] = S0;
}

// Renormalise the surviving weights (fixed order), count the dead, ENC.
__global__ void em_renorm_kernel(int K, double *w, DevStats *st) {
  if (threadIdx.x != 0) return;
  double tot = 0.0;
  for (int k = 0; k < K; k++) tot += w[k];
  st->wsum = tot;
  if (!(tot > 0.0) || !isfinite(tot)) {
    st->status = -9005;  // PMCG_ENEGWEIGHT
    st->ndead = K;
    st->enc = 0.0;
    return;
  }
  double s2 = 0.0;
  int nd = 0;
  for (int k = 0; k < K; k++) {
    double v = w[k] / tot;
    w[k] = v;
    s2 += v * v;
    nd += (v == 0.0);
  }
  st->ndead = nd;
  st->enc = 1.0 / s2;
}

cudaError_t launch_em(int precision, DevMix &m, size_t N, const double *X64, const float *X32,
                      const double *logw, const double *logq, const double *lt64, const double *Q64,
                      const float *lt32, const float *Q32, const int *counts, double *partials, int S,
                      DevStats *st, int band_limit, float *aw32, cudaStream_t s) {
  DevMixView v = m.view();
  const int D = m.D, E = em_E(D);
  cudaError_t e;
  if (precision == 0) {
    if (E > 10 * 256) return cudaErrorInvalidValue;
    size_t smem = (size_t)(kTile64 * D + 2 * kTile64) * sizeof(double);
    em_stats_f64_kernel<<<dim3(S, m.K), 256, smem, s>>>(v, N, S, X64, logw, logq, lt64, Q64, st, partials);
  } else {
    const int Dp = m.ldx, Da = Dp + 4, nb = Da / 4, NB = nb * (nb + 1) / 2;
    if (NB > 256) return cudaErrorInvalidValue;
    const int G = 256 / NB;
    unsigned fgrid = (unsigned)((N + 255) / 256 < 2048 ? (N + 255) / 256 : 2048);
    em_weight_factor_kernel<<<fgrid, 256, 0, s>>>(N, logw, logq, st, aw32);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    size_t smem_tile = (size_t)(Dp * Dp + Dp + kTile32 * Da + kTile32 * (Dp + 1) + kTile32) * sizeof(float);
    size_t smem_red = (size_t)G * NB * 16 * sizeof(double);
    size_t smem = smem_tile > smem_red ? smem_tile : smem_red;
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(em_stats_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    // component-fastest grid: the blocks of one sample chunk run together and share it in L2
    em_stats_f32_kernel<<<dim3(m.K, S), 256, smem, s>>>(v, N, S, X32, aw32, lt32, Q32, partials);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int whitened = precision != 0;
  size_t fsmem = (size_t)(E + (whitened ? 3 : 1) * D * D) * sizeof(double);
  if (fsmem > 48 * 1024) {
    e = cudaFuncSetAttribute(em_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem);
    if (e != cudaSuccess) return e;
  }
  em_finalize_kernel<<<m.K, 128, fsmem, s>>>(v, m.w, m.mu, m.L, N, S, partials, counts, band_limit, whitened);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  em_renorm_kernel<<<1, 32, 0, s>>>(m.K, m.w, st);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return devmix_prepare(m, s);
}

}  // namespace pmcg
