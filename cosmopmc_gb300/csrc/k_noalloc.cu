// k_noalloc.cu — importance weights, evidence, perplexity and ESS without any
// allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: code that runs inside
// another framework's memory manager (the device memory belongs to that
// framework's pool), latency-bound serving loops where an allocation would
// implicitly synchronise the device, and host runtimes that forbid driver
// allocations after start-up. This entry point serves them: the caller passes
// the inputs and outputs, and the per-block partial sums live in a file-scope
// device array of fixed size that every GPU which loads the library holds until
// the process exits.
//
// The scratch holds one partial record per 2048 samples plus the final record,
// so a call accepts at most kNoAllocMaxSamples samples and rejects more with
// PMCG_EDIM. The first call on a device looks up the array's device address
// (cudaGetSymbolAddress, with that device current); make that first call before
// any stream capture. Every call is synchronous: it launches two kernels on the
// caller's stream, copies the final record into a host variable and waits for
// the stream, because the scalars are returned on the host. All calls share the
// array and every call overwrites the records it reads, so nothing carries over
// from the previous call — but calls whose kernels overlap on the GPU (other
// streams, other host threads) race on the array and must be serialised by the
// caller.
#include <mutex>

#include "../../include/pmcg.h"
#include "pmcg_internal.h"
#include "pmcg_kernels.h"

namespace pmcg {

constexpr int kNoAllocSamplesPerBlock = 2048;  // 256 threads x 8 samples
constexpr int kNoAllocMaxBlocks = 4096;
constexpr size_t kNoAllocMaxSamples = (size_t)kNoAllocSamplesPerBlock * kNoAllocMaxBlocks;  // 8,388,608

// kNoAllocMaxBlocks partial records + 1 final record (40 bytes each: ~160 KB).
static __device__ __align__(256) WRed g_noalloc_scratch[kNoAllocMaxBlocks + 1];

__device__ __forceinline__ void wred_push(WRed &r, double l) {
  if (l > r.m) {
    double e = exp(r.m - l);
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

// One block per 2048 samples; every block writes its partial record.
__global__ void __launch_bounds__(256) noalloc_weights_kernel(size_t N, double beta, const double *__restrict__ logpost,
                                                              const double *__restrict__ logq, short *__restrict__ flg,
                                                              double *__restrict__ logw, WRed *__restrict__ part) {
  __shared__ WRed s_r[8];
  WRed r = wred_empty();
  const size_t base = (size_t)blockIdx.x * kNoAllocSamplesPerBlock;
  for (int q = 0; q < kNoAllocSamplesPerBlock / 256; q++) {
    const size_t n = base + (size_t)q * blockDim.x + threadIdx.x;
    if (n >= N) break;
    double l = -INFINITY;
    if (flg[n]) {
      l = beta * logpost[n] - logq[n];
      if (!isfinite(l)) { l = -INFINITY; flg[n] = 0; }
    }
    logw[n] = l;
    if (l > -INFINITY) wred_push(r, l);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r = wred_merge(r, wred_shfl(r, o));
  if ((threadIdx.x & 31) == 0) s_r[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    WRed a = s_r[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) a = wred_merge(a, s_r[w]);
    part[blockIdx.x] = a;
  }
}

// Merges the nb partials (fixed order) into part[kNoAllocMaxBlocks].
__global__ void __launch_bounds__(256) noalloc_merge_kernel(int nb, WRed *part) {
  __shared__ WRed s_r[8];
  WRed a = wred_empty();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) a = wred_merge(a, part[b]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = wred_merge(a, wred_shfl(a, o));
  if ((threadIdx.x & 31) == 0) s_r[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    a = s_r[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) a = wred_merge(a, s_r[w]);
    part[kNoAllocMaxBlocks] = a;
  }
}

// Device address of the scratch array, looked up once per device.
static std::mutex g_noalloc_mu;
static WRed *g_noalloc_ptr[64] = {};

static WRed *noalloc_scratch(int dev, error **err) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (dev < 0 || dev >= 64) {
    set_error(err, PMCG_EARG, __LINE__, "device ordinal %d out of range", dev);
    return nullptr;
  }
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      set_error(err, PMCG_ECUDA, __LINE__, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return nullptr;
    }
    g_noalloc_ptr[dev] = (WRed *)p;
  }
  return g_noalloc_ptr[dev];
}

}  // namespace pmcg

using namespace pmcg;

extern "C" void pmcg_importance_weights_noalloc(size_t N, double beta, const double *logpost, const double *logq,
                                                short *flg, double *logw, pmcg_weight_stats *stats, void *stream,
                                                error **err) {
  if (N == 0 || !logpost || !logq || !flg || !logw || !stats) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_importance_weights_noalloc: null argument or zero samples");
    return;
  }
  if (N > kNoAllocMaxSamples) {
    set_error(err, PMCG_EDIM, __LINE__,
              "pmcg_importance_weights_noalloc: %zu samples exceed the fixed scratch limit of %zu", N,
              kNoAllocMaxSamples);
    return;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(err, PMCG_ECUDA, __LINE__, "cudaGetDevice: %s", cudaGetErrorString(e));
    return;
  }
  WRed *part = noalloc_scratch(dev, err);
  if (!part) return;
  // An error left on this thread by earlier, unrelated work is reported as
  // such (and cleared) instead of being taken for a failure of these launches.
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(err, PMCG_ECUDA, __LINE__, "CUDA error pending from earlier work on this thread: %s",
              cudaGetErrorString(e));
    return;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (int)((N + kNoAllocSamplesPerBlock - 1) / kNoAllocSamplesPerBlock);
  noalloc_weights_kernel<<<nb, 256, 0, s>>>(N, beta, logpost, logq, flg, logw, part);
  noalloc_merge_kernel<<<1, 256, 0, s>>>(nb, part);
  WRed a;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&a, part + kNoAllocMaxBlocks, sizeof(WRed), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(err, PMCG_ECUDA, __LINE__, "importance weights: %s", cudaGetErrorString(e));
    return;
  }
  if (a.n == 0.0 || !(a.m > -INFINITY)) {
    set_error(err, PMCG_ENOWEIGHT, __LINE__, "every sample has zero weight");
    return;
  }
  const double ls = a.m + log(a.s);
  stats->logSum = ls;
  stats->maxW = a.m;
  stats->ln_evidence = ls - log((double)N);
  stats->perplexity = exp(ls - a.t / a.s) / (double)N;
  stats->ess = (a.s * a.s) / a.q;
  stats->nok = (size_t)a.n;
}
