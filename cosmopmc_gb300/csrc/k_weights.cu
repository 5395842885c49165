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

// Tiles of kTileW samples; with done given, the last block to finish (fence,
// then a counter; nothing waits) merges every tile's record into the
// statistics, so the weight step is one launch.
template <bool FAST>
__global__ void __launch_bounds__(256) weights_kernel(size_t N, double beta, const double *betap,
                                                      const double *__restrict__ logpost,
                                                      const double *__restrict__ logq, short *__restrict__ flg,
                                                      double *__restrict__ logw, WRed *partials, DevStats *st,
                                                      unsigned *done) {
  __shared__ WRed s_r[8];
  __shared__ int s_last;
  if (betap) beta = *betap;  // from device memory (iterations replayed as one graph)
  body_weights_tile<FAST>(N, beta, logpost, logq, flg, logw, partials, blockIdx.x, s_r);
  if (!done) return;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  body_weights_final<FAST>((int)gridDim.x, partials, N, st, s_r);
  if (threadIdx.x == 0) *done = 0u;  // ready for the next weight step
}

template <bool FAST>
__global__ void __launch_bounds__(256) weights_final_kernel(int nb, const WRed *__restrict__ partials, size_t N,
                                                            DevStats *st) {
  __shared__ WRed s_r[8];
  body_weights_final<FAST>(nb, partials, N, st, s_r);
}

cudaError_t launch_weights(size_t N, double beta, const double *logpost, const double *logq, short *flg,
                           double *logw, WRed *partials, DevStats *st, cudaStream_t s, int fast,
                           const double *betap, unsigned *done) {
  const unsigned nb = (unsigned)weight_tiles(N);
  if (fast) weights_kernel<true><<<nb, 256, 0, s>>>(N, beta, betap, logpost, logq, flg, logw, partials, st, done);
  else weights_kernel<false><<<nb, 256, 0, s>>>(N, beta, betap, logpost, logq, flg, logw, partials, st, done);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || done) return e;
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

// ------------------------------------------------------------------ weighted moments
// (f) Weighted mean and covariance of a sample with its normalised weights
// (the post-processing means and covariances of exec/exec_helper.c:63-349 on
// the device). Block partial sums in a fixed order (deterministic); the mean
// in FP64; the centred second moments as single-precision products summed per
// 32-sample tile and accumulated in FP64.
namespace pmcg {

constexpr int kMomTile = 32;
constexpr int kMomPairs = 9;  // pairs per thread: ceil(64*65/2 / 256)

__global__ void __launch_bounds__(256) moments_mean_kernel(size_t N, int D, const double *__restrict__ X,
                                                           const double *__restrict__ wbar,
                                                           const short *__restrict__ flg, size_t chunk,
                                                           double *__restrict__ part) {
  __shared__ double red[256];
  const int G = blockDim.x / D, d = threadIdx.x % D, lane = threadIdx.x / D;
  const size_t n0 = (size_t)blockIdx.x * chunk, n1 = (n0 + chunk < N) ? n0 + chunk : N;
  double acc = 0.0;
  if (lane < G)
    for (size_t n = n0 + lane; n < n1; n += G)
      if (flg[n]) acc = fma(wbar[n], X[n * D + d], acc);
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < D) {
    double t = 0.0;
    for (int l = 0; l < G; l++) t += red[l * D + threadIdx.x];
    part[(size_t)blockIdx.x * D + threadIdx.x] = t;
  }
}

__global__ void moments_sum_kernel(int nb, int len, const double *__restrict__ part, double *__restrict__ out) {
  for (int e = threadIdx.x; e < len; e += blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < nb; b++) t += part[(size_t)b * len + e];
    out[e] = t;
  }
}

__global__ void __launch_bounds__(256) moments_cov_kernel(size_t N, int D, const double *__restrict__ X,
                                                          const double *__restrict__ wbar,
                                                          const short *__restrict__ flg,
                                                          const double *__restrict__ mean, size_t chunk,
                                                          double *__restrict__ part) {
  __shared__ float sc[kMomTile * 65];  // centred rows (stride D+1)
  __shared__ float sw[kMomTile];
  const int P = D * (D + 1) / 2, ld = D + 1;
  int pi[kMomPairs], pj[kMomPairs];
  double acc[kMomPairs];
#pragma unroll
  for (int r = 0; r < kMomPairs; r++) {
    const int p = threadIdx.x + r * blockDim.x;
    int i = 0;
    if (p < P) {
      i = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
      while ((i + 1) * (i + 2) / 2 <= p) i++;
      while (i * (i + 1) / 2 > p) i--;
    }
    pi[r] = i;
    pj[r] = p - i * (i + 1) / 2;
    acc[r] = 0.0;
  }
  const size_t n0 = (size_t)blockIdx.x * chunk, n1 = (n0 + chunk < N) ? n0 + chunk : N;
  for (size_t t0 = n0; t0 < n1; t0 += kMomTile) {
    __syncthreads();
    for (int e = threadIdx.x; e < kMomTile * D; e += blockDim.x) {
      const int r = e / D, d = e - r * D;
      const size_t n = t0 + r;
      sc[r * ld + d] = (n < n1) ? (float)(X[n * D + d] - mean[d]) : 0.f;
    }
    for (int r = threadIdx.x; r < kMomTile; r += blockDim.x) {
      const size_t n = t0 + r;
      sw[r] = (n < n1 && flg[n]) ? (float)wbar[n] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kMomPairs; r++) {
      if (threadIdx.x + r * blockDim.x < P) {
        float s = 0.f;
        for (int q = 0; q < kMomTile; q++) s = fmaf(sw[q] * sc[q * ld + pi[r]], sc[q * ld + pj[r]], s);
        acc[r] += (double)s;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kMomPairs; r++) {
    const int p = threadIdx.x + r * blockDim.x;
    if (p < P) part[(size_t)blockIdx.x * P + p] = acc[r];
  }
}

__global__ void moments_unpack_kernel(int D, const double *__restrict__ packed, double *__restrict__ cov) {
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    const int i = e / D, j = e - i * D, a = i > j ? i : j, b = i > j ? j : i;
    cov[e] = packed[a * (a + 1) / 2 + b];
  }
}

size_t moments_scratch_doubles(int D) {
  const int nb = 304;
  return (size_t)nb * (D + D * (D + 1) / 2) + D + D * (D + 1) / 2 + (size_t)D * D;
}

cudaError_t launch_moments(size_t N, int D, const double *X, const double *wbar, const short *flg, double *scratch,
                           double *mean_out, double *cov_out, cudaStream_t s) {
  if (N == 0 || D < 1 || D > kMaxD) return cudaErrorInvalidValue;
  const int nb = 304, P = D * (D + 1) / 2;
  const size_t chunk = (N + nb - 1) / nb;
  double *pmean = scratch, *pcov = pmean + (size_t)nb * D, *mean = pcov + (size_t)nb * P, *cpk = mean + D;
  (void)cpk;
  moments_mean_kernel<<<nb, 256, 0, s>>>(N, D, X, wbar, flg, chunk, pmean);
  moments_sum_kernel<<<1, 256, 0, s>>>(nb, D, pmean, mean);
  moments_cov_kernel<<<nb, 256, 0, s>>>(N, D, X, wbar, flg, mean, chunk, pcov);
  moments_sum_kernel<<<1, 256, 0, s>>>(nb, P, pcov, cpk);
  moments_unpack_kernel<<<1, 256, 0, s>>>(D, cpk, cov_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(mean_out, mean, sizeof(double) * D, cudaMemcpyDeviceToDevice, s);
}

}  // namespace pmcg
