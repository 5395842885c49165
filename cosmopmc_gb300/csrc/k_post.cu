// k_post.cu — weighted post-processing of a sample on the device: marginal
// median and one-sided confidence limits of every parameter, and weighted 1-D /
// 2-D histograms. Replaces the reference's mean_sigma_from_psim,
// median_from_psim and sigma_from_psim (exec/exec_helper.c:63-271) and
// create_1d_hist / create_2d_hist (wrappers/src/param.c:1229-1357), which run
// once per iteration on the host.
//
// Limits follow sigma_from_psim: samples sorted by the parameter, imean the
// first one at or above the centre (at most the last), the weights summed from
// imean outwards until the sum exceeds conf/2 (conf = 68.27, 95.45, 99.73 %);
// the limit is the distance from the centre to the sample after the last one
// summed, -1 when the sample ends first. The median is the value where the
// cumulative weight reaches 1/2 (the mean of the two samples around it when it
// passes 1/2). The sums are read from one FP64 inclusive scan of the sorted
// weights. The sort and the scan are Thrust's (CUDA toolkit): post-processing,
// off the iteration path.
#include <thrust/execution_policy.h>
#include <thrust/scan.h>
#include <thrust/sort.h>

#include <algorithm>
#include <vector>

#include "pmcg_bodies.cuh"

namespace pmcg {

// Order-preserving key of a double (non-NaN): larger value, larger key.
__device__ __forceinline__ unsigned long long post_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double post_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// Keys and weights of parameter a; samples with flg == 0 sort last with weight 0.
__global__ void post_pairs_kernel(size_t N, int D, int a, const double *__restrict__ X, const double *__restrict__ wbar,
                                  const short *__restrict__ flg, unsigned long long *key, double *w) {
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    const bool ok = flg[n] != 0;
    key[n] = ok ? post_key(X[n * D + a]) : ~0ull;
    w[n] = ok ? wbar[n] : 0.0;
  }
}

// First index i in [lo, hi) with C[i] > t (hi if none); C non-decreasing.
__device__ __forceinline__ long long first_above(const double *C, long long lo, long long hi, double t) {
  while (lo < hi) {
    const long long mid = (lo + hi) / 2;
    if (C[mid] > t) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}
// First index i in [lo, hi) with C[i] >= t (hi if none).
__device__ __forceinline__ long long first_at_least(const double *C, long long lo, long long hi, double t) {
  while (lo < hi) {
    const long long mid = (lo + hi) / 2;
    if (C[mid] >= t) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// One thread, over the sorted keys and the inclusive scan C of their weights:
// the centre (mean, or the median), then the three right and three left
// limits. With nv valid samples and imean the first at or above the centre
// (at most nv - 1), base = C[imean - 1]:
//  right, conf c: the sum w[imean..k] first exceeds c at the first k >= imean
//    with C[k] > base + c; the limit is sample k + 1 (-1 when k + 1 >= nv);
//  left: the sum w[k..imean-1] = base - C[k-1] first exceeds c at the largest
//    k <= imean - 1 with C[k-1] < base - c; the limit is sample k - 1 (-1 when
//    k - 1 < 0), i.e. m = min(p - 1, imean - 2) with p the first index with
//    C[p] >= base - c.
__global__ void post_summary_kernel(long long N, const unsigned long long *__restrict__ key,
                                    const double *__restrict__ C, int use_median, double mean, double *center_out,
                                    double *sigma_out, int *status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  // valid samples: the keys below the sentinel of flg == 0
  long long lo = 0, hi = N;
  while (lo < hi) {
    const long long mid = (lo + hi) / 2;
    if (key[mid] == ~0ull) hi = mid;
    else lo = mid + 1;
  }
  const long long nv = lo;
  if (nv < 1) { *status = 1; return; }
  auto par = [&](long long i) { return post_value(key[i]); };
  double center = mean;
  if (use_median) {
    const long long i = first_at_least(C, 0, nv, 0.5);
    if (i == nv) { *status = 2; return; }  // the weights do not reach 1/2
    center = (C[i] == 0.5 || i == 0) ? par(i) : 0.5 * (par(i) + par(i - 1));
  }
  lo = 0;
  hi = nv - 1;
  const unsigned long long kc = post_key(center);
  while (lo < hi) {
    const long long mid = (lo + hi) / 2;
    if (key[mid] >= kc) hi = mid;
    else lo = mid + 1;
  }
  const long long im = lo;
  const double base = im > 0 ? C[im - 1] : 0.0;
  const double conf[3] = {0.682689492137085897 / 2.0, 0.954499736103641585 / 2.0, 0.997300203936739810 / 2.0};
  for (int j = 0; j < 3; j++) {
    const long long k = first_above(C, im, nv, base + conf[j]);
    sigma_out[j] = (k + 1 < nv) ? par(k + 1) - center : -1.0;
    const long long p = first_at_least(C, 0, nv, base - conf[j]);
    const long long m = (p - 1 < im - 2) ? p - 1 : im - 2;
    sigma_out[3 + j] = (m >= 0) ? center - par(m) : -1.0;
  }
  *center_out = center;
  *status = 0;
}

// Bin j of [lo, hi] with nbin bins: e_j <= x < e_{j+1}, e_j = lo + j (hi - lo) / nbin,
// the last bin closed at hi; -1 outside.
__host__ __device__ inline double post_edge(double lo, double hi, int nbin, int j) {
  return (j == nbin) ? hi : lo + (hi - lo) * (double)j / (double)nbin;
}
__device__ __forceinline__ int post_bin(double x, double lo, double hi, int nbin) {
  if (!(x >= lo && x <= hi)) return -1;
  int j = (int)floor((x - lo) / (hi - lo) * (double)nbin);
  j = j < 0 ? 0 : (j > nbin - 1 ? nbin - 1 : j);
  if (x < post_edge(lo, hi, nbin, j)) j--;
  else if (j < nbin - 1 && x >= post_edge(lo, hi, nbin, j + 1)) j++;
  return j;
}

// 1-D: the bin masses of one parameter from its sorted keys and the scan C
// (threads over bins); scale multiplies every mass.
__global__ void post_hist1d_kernel(long long N, const unsigned long long *__restrict__ key,
                                   const double *__restrict__ C, int nbin, double lo, double hi, double scale,
                                   double *__restrict__ out) {
  auto first_key = [&](unsigned long long kv) {
    long long a = 0, b = N;
    while (a < b) {
      const long long mid = (a + b) / 2;
      if (key[mid] >= kv) b = mid;
      else a = mid + 1;
    }
    return a;
  };
  for (int j = threadIdx.x; j < nbin; j += blockDim.x) {
    const long long s0 = first_key(post_key(post_edge(lo, hi, nbin, j)));
    const long long s1 = (j == nbin - 1) ? first_key(post_key(hi) + 1ull) : first_key(post_key(post_edge(lo, hi, nbin, j + 1)));
    const double m = (s1 > s0) ? C[s1 - 1] - (s0 > 0 ? C[s0 - 1] : 0.0) : 0.0;
    out[j] = m * scale;
  }
}

// 2-D: joint bin index of (x_p, x_q) (sentinel outside or flg == 0).
__global__ void post_bin2_kernel(size_t N, int D, int p, int q, const double *__restrict__ X,
                                 const double *__restrict__ wbar, const short *__restrict__ flg, int nbin,
                                 double lop, double hip, double loq, double hiq, unsigned *key, double *w) {
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    unsigned k = 0xFFFFFFFFu;
    double v = 0.0;
    if (flg[n]) {
      const int bp = post_bin(X[n * D + p], lop, hip, nbin), bq = post_bin(X[n * D + q], loq, hiq, nbin);
      if (bp >= 0 && bq >= 0) { k = (unsigned)(bp * nbin + bq); v = wbar[n]; }
    }
    key[n] = k;
    w[n] = v;
  }
}

__global__ void post_hist2d_kernel(long long N, const unsigned *__restrict__ key, const double *__restrict__ C,
                                   int nb2, double scale, double *__restrict__ out) {
  auto first_key = [&](unsigned kv) {
    long long a = 0, b = N;
    while (a < b) {
      const long long mid = (a + b) / 2;
      if (key[mid] >= kv) b = mid;
      else a = mid + 1;
    }
    return a;
  };
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nb2; j += gridDim.x * blockDim.x) {
    const long long s0 = first_key((unsigned)j), s1 = first_key((unsigned)j + 1u);
    out[j] = ((s1 > s0) ? C[s1 - 1] - (s0 > 0 ? C[s0 - 1] : 0.0) : 0.0) * scale;
  }
}

size_t post_scratch_bytes(size_t N) { return N * (sizeof(unsigned long long) + 2 * sizeof(double)) + 256; }

cudaError_t launch_post_summary(size_t N, int D, const double *X, const double *wbar, const short *flg,
                                const double *mean, int use_median, void *scratch, double *center, double *sigma,
                                int *status, cudaStream_t s) {
  if (N == 0 || D < 1) return cudaErrorInvalidValue;
  unsigned long long *key = reinterpret_cast<unsigned long long *>(scratch);
  double *w = reinterpret_cast<double *>(key + N);
  double *C = w + N;
  std::vector<double> hmean(D);
  cudaError_t e = cudaMemcpyAsync(hmean.data(), mean, sizeof(double) * D, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  unsigned grid = (unsigned)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
  for (int a = 0; a < D; a++) {
    post_pairs_kernel<<<grid, 256, 0, s>>>(N, D, a, X, wbar, flg, key, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    thrust::stable_sort_by_key(thrust::cuda::par.on(s), key, key + N, w);
    thrust::inclusive_scan(thrust::cuda::par.on(s), w, w + N, C);
    post_summary_kernel<<<1, 32, 0, s>>>((long long)N, key, C, use_median, hmean[a], center + a, sigma + 6 * a,
                                         status + a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_post_hist1d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin,
                               const double *lo, const double *hi, double scale, void *scratch, double *hist,
                               cudaStream_t s) {
  if (N == 0 || D < 1 || nbin < 1) return cudaErrorInvalidValue;
  unsigned long long *key = reinterpret_cast<unsigned long long *>(scratch);
  double *w = reinterpret_cast<double *>(key + N);
  double *C = w + N;
  cudaError_t e;
  unsigned grid = (unsigned)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
  for (int a = 0; a < D; a++) {
    post_pairs_kernel<<<grid, 256, 0, s>>>(N, D, a, X, wbar, flg, key, w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    thrust::stable_sort_by_key(thrust::cuda::par.on(s), key, key + N, w);
    thrust::inclusive_scan(thrust::cuda::par.on(s), w, w + N, C);
    post_hist1d_kernel<<<1, 256, 0, s>>>((long long)N, key, C, nbin, lo[a], hi[a], scale, hist + (size_t)a * nbin);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_post_hist2d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin,
                               int p, int q, const double *lo, const double *hi, double scale, void *scratch,
                               double *hist, cudaStream_t s) {
  if (N == 0 || nbin < 1 || p < 0 || q < 0 || p >= D || q >= D || (long long)nbin * nbin >= 0xFFFFFFFFll)
    return cudaErrorInvalidValue;
  unsigned *key = reinterpret_cast<unsigned *>(scratch);
  double *w = reinterpret_cast<double *>(reinterpret_cast<char *>(scratch) + ((N * sizeof(unsigned) + 255) & ~(size_t)255));
  double *C = w + N;
  cudaError_t e;
  unsigned grid = (unsigned)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
  post_bin2_kernel<<<grid, 256, 0, s>>>(N, D, p, q, X, wbar, flg, nbin, lo[p], hi[p], lo[q], hi[q], key, w);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  thrust::stable_sort_by_key(thrust::cuda::par.on(s), key, key + N, w);
  thrust::inclusive_scan(thrust::cuda::par.on(s), w, w + N, C);
  const int nb2 = nbin * nbin;
  post_hist2d_kernel<<<(nb2 + 255) / 256 < 1024 ? (nb2 + 255) / 256 : 1024, 256, 0, s>>>((long long)N, key, C, nb2,
                                                                                        scale, hist);
  return cudaGetLastError();
}

}  // namespace pmcg

namespace pmcg {

// Weight clipping: keys ~order_key(log w) for counted samples (largest weight
// first), all ones for the others; a stable sort keeps equal weights in
// sample order, so ties go to the lower index.
__global__ void clip_keys_kernel(size_t N, const double *__restrict__ logw, const short *__restrict__ flg,
                                 unsigned long long *__restrict__ key, unsigned long long *__restrict__ idx) {
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
    key[n] = flg[n] ? ~dkey(logw[n]) : ~0ull;
    idx[n] = n;
  }
}

__global__ void clip_apply_kernel(int k, const unsigned long long *__restrict__ key,
                                  const unsigned long long *__restrict__ idx, short *__restrict__ flg, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k && key[i] != ~0ull) {
    flg[idx[i]] = 0;
    atomicAdd(count, 1);
  }
}

cudaError_t launch_clip_largest(size_t N, const double *logw, short *flg, int k, void *scratch, int *count,
                                cudaStream_t s) {
  if (N == 0 || k <= 0) return cudaMemsetAsync(count, 0, sizeof(int), s);
  if ((size_t)k > N) k = (int)N;
  unsigned long long *key = reinterpret_cast<unsigned long long *>(scratch);
  unsigned long long *idx = key + N;  // the first weight array of the post-processing scratch
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)std::min<size_t>((N + 255) / 256, 4096);
  clip_keys_kernel<<<grid, 256, 0, s>>>(N, logw, flg, key, idx);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  thrust::stable_sort_by_key(thrust::cuda::par.on(s), key, key + N, idx);
  clip_apply_kernel<<<(unsigned)((k + 255) / 256), 256, 0, s>>>(k, key, idx, flg, count);
  return cudaGetLastError();
}

}  // namespace pmcg
