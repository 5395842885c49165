// k_em.cu — (e) Rao-Blackwellised EM update of the proposal (Cappe et al.
// 2008), replacing pmclib update_prop_rb (exec/cosmo_pmc.c:247) including the
// burial of dead components (Manual/manual.tex:479-500).
//
// For component k with old mean c, per sample n (flg == 1):
//   v  = wbar_n * rho_nk = exp(logw_n - logSum - logq_n + lt_nk)
//   vt = v * tau_nk, tau = (nu+D)/(nu+Q_nk) for Student-t, 1 for Gaussian
// Statistics (the "E layout", E = 2 + D + D(D+1)/2 doubles):
//   [0] S0 = sum v, [1] St = sum vt, [2+i] S1_i = sum vt a_i,
//   [2+D+tri(i,j)] S2_ij = sum vt a_i a_j,
// with a = x - c (FP64 path) or a = L^-1 (x - c) (mixed path, whitened frame).
// Then d = S1/St, Sigma = (S2 - St d d^T)/S0, mu' = c + d (or c + L d and
// Sigma' = L Sigma L^T when whitened), alpha' = S0. Each block covers one
// component and one contiguous chunk of samples and writes its partial
// statistics; the finalise kernel sums the chunks in a fixed order
// (deterministic), factorises Sigma' in FP64 and applies the dead-component
// rule. The mixed, finalise and renormalise bodies are shared with the batch
// kernel (pmcg_bodies.cuh).
#include "pmcg_bodies.cuh"
#include "umma_image.cuh"

namespace pmcg {

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

// Three resident blocks per SM (80 registers, a few spilled): the kernel waits
// on gathers and barriers, and 24 warps hide more of that than 16 (measured:
// 37 us less at the mixture workload than at two blocks).
__global__ void __launch_bounds__(256, 3) em_stats_f32_kernel(DevMixView m, size_t N, int S,
                                                           const float *__restrict__ X,
                                                           const float *__restrict__ aw,
                                                           const float *__restrict__ lt,
                                                           const float *__restrict__ Qv,
                                                           double *__restrict__ part,
                                                           const uint32_t *__restrict__ mask) {
  extern __shared__ float4 smf4[];
  // component-fastest grid: the blocks of one sample chunk run together and share it in L2
  body_em_stats_f32(m, N, S, X, aw, lt, Qv, part, blockIdx.x, blockIdx.y, reinterpret_cast<unsigned char *>(smf4),
                    mask);
}

// The weight factor aw (as body_em_factor) and one bit per (component,
// sample): aw[n] + lt[k][n] > kEmLogMin, the listing test of the EM
// statistics. One streaming pass over lt (warp ballots, no atomics); each
// thread keeps its sample's factor in a register across the components.
__global__ void __launch_bounds__(256) em_factor_mask_kernel(size_t N, int K, const double *__restrict__ logw,
                                                             const double *__restrict__ logq,
                                                             const DevStats *__restrict__ st, float *__restrict__ aw,
                                                             const float *__restrict__ lt,
                                                             uint32_t *__restrict__ mask) {
  const double ls = st->logSum;
  const size_t W = (N + 31) / 32;
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < W * 32; n += (size_t)gridDim.x * blockDim.x) {
    float a = -INFINITY;
    if (n < N) {
      const double l = logw[n];
      a = (l > -INFINITY) ? (float)(l - ls - logq[n]) : -INFINITY;
      aw[n] = a;
    }
    const size_t wd = n / 32, nl = n < N ? n : N - 1;  // padding lanes read a valid sample
    const float *lp = lt + nl;
    uint32_t *mp = mask + wd;
    // 16 components' loads in flight while the previous 16 are tested
    float v[16], nv[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = (j < K) ? __ldg(lp + (size_t)j * N) : 0.f;
    lp += (size_t)16 * N;
#pragma unroll 1
    for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
      for (int j = 0; j < 16; j++) nv[j] = (k0 + 16 + j < K) ? __ldg(lp + (size_t)j * N) : 0.f;
      lp += (size_t)16 * N;
#pragma unroll
      for (int j = 0; j < 16; j++) {
        if (k0 + j < K) {
          const bool act = (n < N) && (a + v[j] > kEmLogMin);
          const unsigned bal = __ballot_sync(0xffffffffu, act);
          if ((threadIdx.x & 31) == 0) mp[(size_t)j * W] = bal;
        }
      }
      mp += (size_t)16 * W;
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = nv[j];
    }
  }
}

size_t em_mask_words(int K, size_t N) { return (size_t)K * ((N + 31) / 32); }

__global__ void em_weight_factor_kernel(size_t N, const double *__restrict__ logw, const double *__restrict__ logq,
                                        const DevStats *__restrict__ st, float *__restrict__ aw) {
  body_em_factor(N, logw, logq, st, aw, blockIdx.x);
}

// The EM update after the statistics, one block per component: the new weight,
// mean and factor (FP64), then for a live component its derived arrays (L^-1,
// L^-1 mu, single-precision copies) and its rows of the tensor operand image.
// The last block to finish (fence, then a counter; nothing waits) renormalises
// the weights and writes the constants and the image's log-constants, which
// depend on every weight. One launch instead of four dependent ones.
__global__ void __launch_bounds__(256) em_update_kernel(DevMix m, size_t N, int S, const double *__restrict__ part,
                                                        const int *__restrict__ counts, int band_limit,
                                                        int whitened, DevStats *st) {
  extern __shared__ double sh[];
  __shared__ int s_dead, s_last;
  __shared__ unsigned long long s_rmax;
  const DevMixView v = m.view();
  const int k = blockIdx.x;
  body_em_finalize(v, m.w, m.mu, m.L, N, S, part, counts, band_limit, whitened, k, st, sh, &s_dead);
  if (threadIdx.x == 0) s_rmax = 0ull;
  __syncthreads();
  if (st->status == 0 && m.w[k] > 0.0) {
    body_prepare_comp(v, m.logdetL, m.Wt, m.b, m.W32, m.b32, m.L32, m.mu32, k, sh, &s_rmax);
    __syncthreads();
    // single precision (the whitened update): a component narrower than single
    // precision resolves around its mean is numerically singular there, and is
    // buried like a component whose update is not positive definite (before the
    // renormalisation, which the last block does)
    if (whitened && __longlong_as_double((long long)s_rmax) > kF32RangeMax) {
      if (threadIdx.x == 0) {
        m.w[k] = 0.0;
        atomicAdd(&st->f32_range, 1);
      }
    } else if (m.bimg) {
      umma_image_component(v, m.bimg, k);
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(m.em_done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  body_em_renorm(m.K, m.w, st);
  __syncthreads();
  body_prepare_consts(v, m.logdetL, m.cw, m.lconst, m.lconst32);
  __syncthreads();
  if (m.bimg) umma_image_lconst(v, m.bimg);
  if (threadIdx.x == 0) *m.em_done = 0u;  // ready for the next update
}

int em_chunks(int K, size_t N) {
  // about 8 statistics blocks per SM (under 3 waves of 3 resident blocks); measured
  // against 2 and 16 per SM at the mixture workload. Chunks of at least 1024
  // samples: measured against 2048 and 512, the SN iteration at N = 10^4 takes
  // 0.139 / 0.147 / 0.140 ms and 256 batched runs 130 / 132 / 128 M samples/s
  int S = (8 * 152 + K - 1) / K;
  size_t maxS = (N + 1023) / 1024;
  if (maxS < 1) maxS = 1;
  if ((size_t)S > maxS) S = (int)maxS;
  if (S < 1) S = 1;
  return S;
}

size_t em_partials_size(int precision, int K, int D, int *S_out, size_t N) {
  (void)precision;
  const int S = em_chunks(K, N);
  *S_out = S;
  return (size_t)K * S * em_E(D) * sizeof(double);
}

cudaError_t launch_em(int precision, DevMix &m, size_t N, const double *X64, const float *X32,
                      const double *logw, const double *logq, const double *lt64, const double *Q64,
                      const float *lt32, const float *Q32, const int *counts, double *partials, int S,
                      DevStats *st, int band_limit, float *aw32, uint32_t *emmask, cudaStream_t s) {
  DevMixView v = m.view();
  const int D = m.D, E = em_E(D);
  cudaError_t e;
  if (precision == 0) {
    if (E > 10 * 256) return cudaErrorInvalidValue;
    size_t smem = (size_t)(kTile64 * D + 2 * kTile64) * sizeof(double);
    if ((e = allow_dyn_smem(em_stats_f64_kernel, smem)) != cudaSuccess) return e;
    em_stats_f64_kernel<<<dim3(S, m.K), 256, smem, s>>>(v, N, S, X64, logw, logq, lt64, Q64, st, partials);
  } else {
    const int Da = m.ldx + 4, nb = Da / 4, NB = nb * (nb + 1) / 2;
    if (NB > 256) return cudaErrorInvalidValue;
    if (emmask) {
      const size_t W = (N + 31) / 32;
      size_t gx = (W * 32 + 255) / 256;
      if (gx > 4864) gx = 4864;  // 32 blocks per SM (measured against 16: 1 us less)
      em_factor_mask_kernel<<<(unsigned)gx, 256, 0, s>>>(N, m.K, logw, logq, st, aw32, lt32, emmask);
    } else {
      em_weight_factor_kernel<<<(unsigned)((N + kTileW - 1) / kTileW), 256, 0, s>>>(N, logw, logq, st, aw32);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    size_t tb, rb;
    em32_layout(D, m.ldx, 256, &tb, &rb);
    size_t smem = tb > rb ? tb : rb;
    if ((e = allow_dyn_smem(em_stats_f32_kernel, smem)) != cudaSuccess) return e;
    em_stats_f32_kernel<<<dim3(m.K, S), 256, smem, s>>>(v, N, S, X32, aw32, lt32, Q32, partials, emmask);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int whitened = precision != 0;
  size_t usmem = finalize_smem(D, whitened);
  if (prepare_smem(D) > usmem) usmem = prepare_smem(D);
  // its static shared memory (the last block's weight and cumulative arrays)
  // counts against the default 48 KB too
  if ((e = allow_dyn_smem(em_update_kernel, usmem)) != cudaSuccess) return e;
  em_update_kernel<<<m.K, 256, usmem, s>>>(m, N, S, partials, counts, band_limit, whitened, st);
  return cudaGetLastError();
}

}  // namespace pmcg
