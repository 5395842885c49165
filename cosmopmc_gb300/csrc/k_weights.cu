// k_weights.cu — (d) importance log-weights, log-sum-exp normalisation,
// evidence, perplexity and ESS in one pass over the sample, all in FP64.
// Replaces pmclib generic_get_importance_weight_and_deduced_verb's weight
// arithmetic, normalize_importance_weight, evidence and perplexity_and_ess
// (exec/cosmo_pmc.c:46,62,343-345,378).
//
// Reduction record per block: (m, s, t, q, n) with m = max log-weight,
// s = sum e^{l-m}, t = sum e^{l-m} l, q = sum e^{2(l-m)}, n = count. Then
// logSum = m + ln s, H = logSum - t/s, sum wbar^2 = q/s^2. A fixed grid and a
// fixed merge order make the result bit-reproducible.
#include "pmcg_kernels.h"

namespace pmcg {

__device__ __forceinline__ void wred_add(WRed &r, double l) {
  if (l > r.m) {
    double e = exp(r.m - l);  // r.m == -inf gives 0
    r.s = r.s * e + 1.0;
    r.t = r.t * e + l;
    r.q = r.q * e * e + 1.0;
    r.m = l;
  } else {
    double e = exp(l - r.m);
    r.s += e;
    r.t += e * l;
    r.q += e * e;
  }
  r.n += 1.0;
}

__global__ void __launch_bounds__(256) weights_kernel(size_t N, double beta, const double *__restrict__ logpost,
                                                      const double *__restrict__ logq, short *__restrict__ flg,
                                                      double *__restrict__ logw, WRed *__restrict__ partials) {
  __shared__ WRed s_r[8];
  WRed r = wred_empty();
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    double l = -INFINITY;
    if (flg[n]) {
      l = beta * logpost[n] - (logq ? logq[n] : 0.0);
      if (!isfinite(l)) { l = -INFINITY; flg[n] = 0; }
    }
    logw[n] = l;
    if (l > -INFINITY) wred_add(r, l);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r = wred_merge(r, wred_shfl(r, o));
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_r[wid] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    WRed a = s_r[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) a = wred_merge(a, s_r[w]);
    partials[blockIdx.x] = a;
  }
}

// One block of 256 threads: each thread merges a strided subset of the partials,
// then a shuffle tree and a sequential pass over the 8 warps (fixed order).
__global__ void __launch_bounds__(256) weights_final_kernel(int nb, const WRed *__restrict__ partials, size_t N,
                                                            DevStats *st) {
  __shared__ WRed s_r[8];
  WRed a = wred_empty();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) a = wred_merge(a, partials[b]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = wred_merge(a, wred_shfl(a, o));
  if ((threadIdx.x & 31) == 0) s_r[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x != 0) return;
  a = s_r[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) a = wred_merge(a, s_r[w]);
  if (a.n == 0.0 || a.m == -INFINITY) {
    st->status = -9011;  // PMCG_ENOWEIGHT
    st->nok = 0.0;
    return;
  }
  st->status = 0;
  double ls = a.m + log(a.s);
  st->logSum = ls;
  st->maxW = a.m;
  st->H = ls - a.t / a.s;
  st->sumw2 = a.q / (a.s * a.s);
  st->nok = a.n;
  st->ln_evidence = ls - log((double)N);
  st->perplexity = exp(st->H) / (double)N;
  st->ess = 1.0 / st->sumw2;
}

cudaError_t launch_weights(size_t N, double beta, const double *logpost, const double *logq, short *flg,
                           double *logw, WRed *partials, DevStats *st, cudaStream_t s) {
  weights_kernel<<<kWeightBlocks, 256, 0, s>>>(N, beta, logpost, logq, flg, logw, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  weights_final_kernel<<<1, 256, 0, s>>>(kWeightBlocks, partials, N, st);
  return cudaGetLastError();
}

__global__ void normalise_kernel(size_t N, const double *__restrict__ logw, const short *__restrict__ flg,
                                 const DevStats *__restrict__ st, double *__restrict__ wbar) {
  const double ls = st->logSum;
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x)
    wbar[n] = flg[n] ? exp(logw[n] - ls) : 0.0;
}

cudaError_t launch_normalise(size_t N, const double *logw, const short *flg, const DevStats *st, double *wbar,
                             cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  unsigned grid = (unsigned)((N + 255) / 256 < 2048 ? (N + 255) / 256 : 2048);
  normalise_kernel<<<grid, 256, 0, s>>>(N, logw, flg, st, wbar);
  return cudaGetLastError();
}

}  // namespace pmcg
