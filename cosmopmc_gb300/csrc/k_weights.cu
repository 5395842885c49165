// k_weights.cu — (d) importance log-weights, log-sum-exp normalisation,
// evidence, perplexity and ESS in one pass over the sample, all in FP64.
// Replaces pmclib generic_get_importance_weight_and_deduced_verb's weight
// arithmetic, normalize_importance_weight, evidence and perplexity_and_ess
// (exec/cosmo_pmc.c:46,62,343-345,378).
//
// Reduction record per tile of kTileW samples: (m, s, t, q, n) with m = max
// log-weight, s = sum e^{l-m}, t = sum e^{l-m} l, q = sum e^{2(l-m)}, n = count.
// Then logSum = m + ln s, H = logSum - t/s, sum wbar^2 = q/s^2. The tile
// partition depends only on N and the merge order is fixed, so the result is
// bit-reproducible and identical inside a batch.
#include "pmcg_bodies.cuh"

namespace pmcg {

size_t weight_tiles(size_t N) { return N == 0 ? 1 : (N + kTileW - 1) / kTileW; }

template <bool FAST>
__global__ void __launch_bounds__(256) weights_kernel(size_t N, double beta, const double *__restrict__ logpost,
                                                      const double *__restrict__ logq, short *__restrict__ flg,
                                                      double *__restrict__ logw, WRed *__restrict__ partials) {
  __shared__ WRed s_r[8];
  body_weights_tile<FAST>(N, beta, logpost, logq, flg, logw, partials, blockIdx.x, s_r);
}

template <bool FAST>
__global__ void __launch_bounds__(256) weights_final_kernel(int nb, const WRed *__restrict__ partials, size_t N,
                                                            DevStats *st) {
  __shared__ WRed s_r[8];
  body_weights_final<FAST>(nb, partials, N, st, s_r);
}

cudaError_t launch_weights(size_t N, double beta, const double *logpost, const double *logq, short *flg,
                           double *logw, WRed *partials, DevStats *st, cudaStream_t s, int fast) {
  const unsigned nb = (unsigned)weight_tiles(N);
  if (fast) weights_kernel<true><<<nb, 256, 0, s>>>(N, beta, logpost, logq, flg, logw, partials);
  else weights_kernel<false><<<nb, 256, 0, s>>>(N, beta, logpost, logq, flg, logw, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (fast) weights_final_kernel<true><<<1, 256, 0, s>>>((int)nb, partials, N, st);
  else weights_final_kernel<false><<<1, 256, 0, s>>>((int)nb, partials, N, st);
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
