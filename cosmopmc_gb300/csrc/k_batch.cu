// k_batch.cu — many independent PMC runs, one persistent launch per iteration.
//
// A batch holds runs of uneven dimension, component count, sample count and
// likelihood (mixture, SN Ia or template target), all mixed precision. One
// iteration of every run is one cooperative kernel: twelve stages (draw, log q,
// log posterior, subset prior, weight tiles, weight merge, EM weight factor, EM
// statistics, EM finalise, mixture preparation, renormalise, constants),
// separated by grid barriers (a stage without work items is skipped). In each stage the blocks walk a flat list of work items
// (per-run tiles, components or runs); a block finds its run by a binary
// search over the stage's prefix table. The per-item work is the same body the
// single-run kernels execute, with the same tiling, so each run's results are
// bit-identical alone and inside any batch.
//
// The SN likelihood is the one body that needs more resident warps than the
// persistent kernel's two blocks per SM give: the SN runs' log-posterior items
// run in a grouped kernel of their own (one warp per sample, standalone shape)
// between the cooperative launch of the draw and log q stages and the one of
// the remaining stages.
//
// The launches, the upload of the per-iteration parameters (random-stream
// call, beta) and the download of every run's statistics are captured once in
// a CUDA graph. The grouped SN kernel's block size, the samples per thread of the
// log-density stages and the resident blocks per SM are picked by an autotuner
// that times the non-mutating stages (draw, log q, log posterior) and caches the
// choice per batch shape.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "pmcg_bodies.cuh"
#include "pmcg_engine.h"

namespace cg = cooperative_groups;

namespace pmcg {

enum BatchStage {
  kBDraw = 0, kBLogq, kBLogpost, kBPrior, kBWeights, kBWFinal, kBFactor, kBEmStats, kBEmFinal, kBPrepComp, kBRenorm,
  kBPrepConsts, kBStages
};

struct BatchDesc {
  DevMixView prop;
  int ptype;
  DevMixView target;
  SnDev sn;
  TplDev tpl;
  double logpr;
  int has_prior;
  PriorDev prior;
  size_t N;
  int S, CHp, CHt, maxd;
  uint32_t key0, key1;
  const double *bmin, *bmax;
  float *X32;
  int *idx, *counts;
  short *flg;
  double *logq, *logpost, *logw;
  float *lt32, *Q32, *aw32;
  WRed *wpart;
  double *empart;
  DevStats *st;
  double *w, *mu, *L, *Wt, *b, *logdetL, *cw, *lconst;
  float *W32, *b32, *lconst32, *L32, *mu32;
};

struct BatchDyn {
  double beta;
  uint32_t call;
  uint32_t pad;
};

__device__ __forceinline__ int find_run(const uint32_t *__restrict__ pre, int R, uint32_t item) {
  int lo = 0, hi = R;  // largest lo with pre[lo] <= item
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pre[mid] <= item) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int SPT>
__device__ __forceinline__ void batch_item(int stg, const BatchDesc &d, const BatchDyn &dy, uint32_t li,
                                           unsigned char *smem, WRed *s_r, int *s_dead,
                                           DevStats *stats_out, int r) {
  const int D = d.prop.D, K = d.prop.K, ldx = d.prop.ldx;
  switch (stg) {
    case kBDraw: {
      const size_t n0 = (size_t)li * blockDim.x;
      if (d.maxd <= 8)
        body_draw<8, float>(d.prop, d.N, d.key0, d.key1, dy.call, d.bmin, d.bmax, nullptr, nullptr, nullptr, nullptr,
                            d.X32, d.idx, d.flg, d.counts, n0, smem);
      else if (d.maxd <= 16)
        body_draw<16, float>(d.prop, d.N, d.key0, d.key1, dy.call, d.bmin, d.bmax, nullptr, nullptr, nullptr,
                             nullptr, d.X32, d.idx, d.flg, d.counts, n0, smem);
      else
        body_draw<32, float>(d.prop, d.N, d.key0, d.key1, dy.call, d.bmin, d.bmax, nullptr, nullptr, nullptr,
                             nullptr, d.X32, d.idx, d.flg, d.counts, n0, smem);
      break;
    }
    case kBLogq: {
      float *sw = reinterpret_cast<float *>(smem);
      if (d.maxd <= 8) body_mixlogpdf_f32<8, SPT>(d.prop, d.N, d.X32, d.logq, 0, 0.0, d.lt32, d.Q32, d.CHp, li, sw);
      else if (d.maxd <= 16)
        body_mixlogpdf_f32<16, SPT>(d.prop, d.N, d.X32, d.logq, 0, 0.0, d.lt32, d.Q32, d.CHp, li, sw);
      else body_mixlogpdf_f32<32, SPT>(d.prop, d.N, d.X32, d.logq, 0, 0.0, d.lt32, d.Q32, d.CHp, li, sw);
      break;
    }
    case kBLogpost: {
      if (d.ptype == kPluginMix) {
        float *sw = reinterpret_cast<float *>(smem);
        if (d.maxd <= 8)
          body_mixlogpdf_f32<8, SPT>(d.target, d.N, d.X32, d.logpost, 0, d.logpr, nullptr, nullptr, d.CHt, li, sw);
        else if (d.maxd <= 16)
          body_mixlogpdf_f32<16, SPT>(d.target, d.N, d.X32, d.logpost, 0, d.logpr, nullptr, nullptr, d.CHt, li, sw);
        else
          body_mixlogpdf_f32<32, SPT>(d.target, d.N, d.X32, d.logpost, 0, d.logpr, nullptr, nullptr, d.CHt, li, sw);
      } else if (d.ptype == kPluginSn) {
        const size_t n = (size_t)li * (blockDim.x >> 5) + (threadIdx.x >> 5);
        body_sn<true>(d.sn, d.N, D, nullptr, d.X32, ldx, d.logpost, d.flg, n, 1, d.logpr);
      } else {
        body_tpl<float>(d.tpl, d.N, nullptr, d.X32, ldx, d.logpost, d.flg, li, reinterpret_cast<float *>(smem), 1,
                        d.logpr);
      }
      break;
    }
    case kBPrior:
      body_prior_any<float>(d.prior, d.N, D, nullptr, d.X32, ldx, d.logpost, (size_t)li * blockDim.x + threadIdx.x);
      break;
    case kBWeights:
      body_weights_tile<true>(d.N, dy.beta, d.logpost, d.logq, d.flg, d.logw, d.wpart, li, s_r);
      break;
    case kBWFinal:
      body_weights_final<true>((int)((d.N + kTileW - 1) / kTileW), d.wpart, d.N, d.st, s_r);
      break;
    case kBFactor:
      body_em_factor(d.N, d.logw, d.logq, d.st, d.aw32, li);
      break;
    case kBEmStats:
      body_em_stats_f32(d.prop, d.N, d.S, d.X32, d.aw32, d.lt32, d.Q32, d.empart, (int)(li % K), (int)(li / K), smem);
      break;
    case kBEmFinal:
      body_em_finalize(d.prop, d.w, d.mu, d.L, d.N, d.S, d.empart, d.counts, D, 1, (int)li, d.st,
                       reinterpret_cast<double *>(smem), s_dead);
      break;
    case kBRenorm:
      body_em_renorm(K, d.w, d.st);
      break;
    case kBPrepComp: {
      __shared__ unsigned long long s_rmax;
      if (threadIdx.x == 0) s_rmax = 0ull;
      __syncthreads();
      body_prepare_comp(d.prop, d.logdetL, d.Wt, d.b, d.W32, d.b32, d.L32, d.mu32, (int)li,
                        reinterpret_cast<double *>(smem), &s_rmax);
      __syncthreads();
      // a component narrower than single precision resolves is buried before the
      // renormalisation stage, as in the single-run update
      if (threadIdx.x == 0 && d.st->status == 0 && d.w[li] > 0.0 &&
          __longlong_as_double((long long)s_rmax) > kF32RangeMax) {
        d.w[li] = 0.0;
        atomicAdd(&d.st->f32_range, 1);
      }
      break;
    }
    case kBPrepConsts:
      body_prepare_consts(d.prop, d.logdetL, d.cw, d.lconst, d.lconst32);
      for (int k = threadIdx.x; k < K; k += blockDim.x) d.counts[k] = 0;  // the next draw counts afresh
      __syncthreads();
      if (threadIdx.x == 0) stats_out[r] = *d.st;
      break;
    default:
      break;
  }
}

// Registers capped at 128 (two resident blocks per SM): the stages are mostly
// latency-bound, and 16 warps per SM hide more of it than 8 at up to 255
// registers; the spills (under 400 bytes, in the heaviest stage bodies) cost
// less (measured: the 256-run ragged batch 44.4 -> 32.7 ms per iteration).
template <int SPT>
__global__ void __launch_bounds__(256, 2) batch_kernel(const BatchDesc *__restrict__ descs,
                                                       const BatchDyn *__restrict__ dyn, int R,
                                                       const uint32_t *__restrict__ starts, int first, int last,
                                                       DevStats *stats_out) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ WRed s_r[8];
  __shared__ int s_dead;
  for (int stg = first; stg <= last; stg++) {
    const uint32_t *pre = starts + (size_t)stg * (R + 1);
    const uint32_t total = pre[R];
    if (total == 0) continue;  // a stage without work (the same for every block) needs no barrier
    for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
      const int r = find_run(pre, R, item);
      batch_item<SPT>(stg, descs[r], dyn[r], item - pre[r], smem, s_r, &s_dead, stats_out, r);
      __syncthreads();
    }
    if (stg < last) grid.sync();
  }
}

// The SN log-posterior of every SN run of the batch, one warp per sample, at
// the standalone SN kernel's shape (no register cap: many more resident warps
// than the persistent kernel's two 256-thread blocks per SM, which this
// latency-bound body needs); THREADS (64, 128 or 256) is picked by the
// autotuner. Launched between the cooperative launch of the draw and log q
// stages and the one of the remaining stages; the same body as the runs
// alone, so the same values whatever the block size.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) batch_sn_kernel(const BatchDesc *__restrict__ descs, int R,
                                                           const uint32_t *__restrict__ pre) {
  const uint32_t item = blockIdx.x;
  if (item >= pre[R]) return;
  const int r = find_run(pre, R, item);
  const SnDev sn = descs[r].sn;   // by value, as the standalone kernel's parameter
  const BatchDesc &d = descs[r];
  const size_t n = (size_t)(item - pre[r]) * (THREADS / 32) + (threadIdx.x >> 5);
  body_sn<true>(sn, d.N, d.prop.D, nullptr, d.X32, d.prop.ldx, d.logpost, d.flg, n, 1, d.logpr);
}

// Every run's draw counts set to zero (one block per run): the batch's draws add
// to them and its preparation stage zeroes them after each iteration.
__global__ void batch_zero_counts_kernel(const BatchDesc *__restrict__ descs, int R) {
  const int r = blockIdx.x;
  if (r >= R) return;
  const BatchDesc &d = descs[r];
  for (int k = threadIdx.x; k < d.prop.K; k += blockDim.x) d.counts[k] = 0;
}

// ------------------------------------------------------------------ host side
static size_t items_of(int stg, const BatchDesc &d, int spt, int threads) {
  const size_t N = d.N;
  const int K = d.prop.K;
  switch (stg) {
    case kBDraw: return (N + threads - 1) / threads;
    case kBLogq: return (N + (size_t)threads * spt - 1) / ((size_t)threads * spt);
    case kBLogpost:
      if (d.ptype == kPluginMix) return (N + (size_t)threads * spt - 1) / ((size_t)threads * spt);
      if (d.ptype == kPluginSn) return 0;   // batch_sn_kernel
      return (N + threads - 1) / threads;
    case kBPrior: return d.has_prior ? (N + threads - 1) / threads : 0;
    case kBWeights:
    case kBFactor: return (N + kTileW - 1) / kTileW;
    case kBEmStats: return (size_t)K * d.S;
    case kBEmFinal:
    case kBPrepComp: return (size_t)K;
    default: return 1;
  }
}

static size_t smem_of(const BatchDesc &d, int threads) {
  const int D = d.prop.D, K = d.prop.K, ldx = d.prop.ldx;
  size_t s = draw_smem<float>(K, ldx, threads);
  s = std::max(s, (size_t)d.CHp * mix_cs(D, ldx) * sizeof(float));
  if (d.ptype == kPluginMix) s = std::max(s, (size_t)d.CHt * mix_cs(D, ldx) * sizeof(float));
  if (d.ptype == kPluginTpl) s = std::max(s, tpl_smem<float>(d.tpl.P, threads));
  size_t tb, rb;
  em32_layout(D, ldx, threads, &tb, &rb);
  s = std::max(s, std::max(tb, rb));
  s = std::max(s, finalize_smem(D, 1));
  s = std::max(s, prepare_smem(D));
  return align16(s);
}

struct TuneKey {
  std::vector<long long> shape;
  bool operator<(const TuneKey &o) const { return shape < o.shape; }
};
static std::mutex g_tune_mu;
struct TuneChoice {
  int spt, bps, snt;   // samples per thread, blocks per SM, SN kernel threads per block
};
static std::map<TuneKey, TuneChoice> g_tune_cache;

}  // namespace pmcg

using namespace pmcg;

struct pmcg_batch {
  std::vector<pmcg_run *> runs;
  int R = 0;
  std::vector<BatchDesc> hdesc;
  BatchDesc *d_desc = nullptr;
  BatchDyn *d_dyn = nullptr, *h_dyn = nullptr;
  uint32_t *d_starts = nullptr;
  uint32_t *d_snpre = nullptr;   // prefix table of the SN kernel's items over the runs
  uint32_t sn_items = 0;
  DevStats *d_stats = nullptr, *h_stats = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int spt = 2, bps = 1, grid = 0, sms = 0, threads = 256;
  int snt = 128;          // threads per block of the grouped SN kernel
  size_t smem = 0;
  cudaGraphExec_t gexec = nullptr;
  bool graph = false;
  int cap = 0;              // runs the device and pinned arrays hold
  int iters_bound = 0;      // iterations since the runs were bound (the graph is captured at the second)
  float last_ms = 0.f;
  bool stage_timing = false, staged_last = false;
  cudaEvent_t sev[kBStages + 1] = {};
  float stage_ms[kBStages] = {};
};

namespace pmcg {

static bool bck(cudaError_t e, error **err, int line, const char *what) {
  if (e == cudaSuccess) return true;
  set_error(err, PMCG_ECUDA, line, "%s: %s", what, cudaGetErrorString(e));
  return false;
}
#define BCK(expr, what) bck((expr), err, __LINE__, (what))

template <int SPT>
static cudaError_t launch_batch(pmcg_batch *b, int first, int last) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(b->grid);
  cfg.blockDim = dim3(b->threads);
  cfg.dynamicSmemBytes = b->smem;
  cfg.stream = b->s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int R = b->R;
  return cudaLaunchKernelEx(&cfg, batch_kernel<SPT>, (const BatchDesc *)b->d_desc, (const BatchDyn *)b->d_dyn, R,
                            (const uint32_t *)b->d_starts, first, last, b->d_stats);
}

static cudaError_t launch_coop(pmcg_batch *b, int first, int last) {
  return b->spt == 1 ? launch_batch<1>(b, first, last) : launch_batch<2>(b, first, last);
}

// Stages first..last; the log-posterior stage's SN items run in the SN kernel.
// The grouped SN kernel at the batch's block size.
static cudaError_t launch_sn_group(pmcg_batch *b) {
  if (b->snt == 64) batch_sn_kernel<64><<<b->sn_items, 64, 0, b->s>>>(b->d_desc, b->R, b->d_snpre);
  else if (b->snt == 256) batch_sn_kernel<256><<<b->sn_items, 256, 0, b->s>>>(b->d_desc, b->R, b->d_snpre);
  else batch_sn_kernel<128><<<b->sn_items, 128, 0, b->s>>>(b->d_desc, b->R, b->d_snpre);
  return cudaGetLastError();
}

static cudaError_t launch_any(pmcg_batch *b, int first, int last) {
  if (b->sn_items == 0 || first > kBLogpost || last < kBLogpost) return launch_coop(b, first, last);
  cudaError_t e = cudaSuccess;
  if (first < kBLogpost && (e = launch_coop(b, first, kBLogpost - 1)) != cudaSuccess) return e;
  if ((e = launch_sn_group(b)) != cudaSuccess) return e;
  return launch_coop(b, kBLogpost, last);
}

// Prefix tables of all stages for the current samples-per-thread, and the grid.
static bool batch_configure(pmcg_batch *b, int spt, int bps, error **err) {
  b->spt = spt;
  std::vector<uint32_t> st((size_t)kBStages * (b->R + 1));
  for (int g = 0; g < kBStages; g++) {
    uint64_t acc = 0;
    for (int r = 0; r < b->R; r++) {
      st[(size_t)g * (b->R + 1) + r] = (uint32_t)acc;
      acc += items_of(g, b->hdesc[r], spt, b->threads);
    }
    if (acc > 0xFFFFFFF0ull) {
      set_error(err, PMCG_EDIM, __LINE__, "batch too large: %llu work items", (unsigned long long)acc);
      return false;
    }
    st[(size_t)g * (b->R + 1) + b->R] = (uint32_t)acc;
  }
  if (!BCK(cudaMemcpy(b->d_starts, st.data(), st.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "starts"))
    return false;
  {
    std::vector<uint32_t> sp(b->R + 1);
    uint64_t acc = 0;
    for (int r = 0; r < b->R; r++) {
      sp[r] = (uint32_t)acc;
      const BatchDesc &d = b->hdesc[r];
      const int wpb = b->snt / 32;    // samples (warps) per block
      if (d.ptype == kPluginSn) acc += (d.N + wpb - 1) / wpb;
    }
    if (acc > 0x7FFFFFF0ull) {
      set_error(err, PMCG_EDIM, __LINE__, "batch too large: %llu SN work items", (unsigned long long)acc);
      return false;
    }
    sp[b->R] = (uint32_t)acc;
    b->sn_items = (uint32_t)acc;
    if (!BCK(cudaMemcpy(b->d_snpre, sp.data(), sp.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "SN items"))
      return false;
  }
  size_t smem = 0;
  for (const BatchDesc &d : b->hdesc) smem = std::max(smem, smem_of(d, b->threads));
  b->smem = smem;
  const void *fn = spt == 1 ? (const void *)batch_kernel<1> : (const void *)batch_kernel<2>;
  if (!BCK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute"))
    return false;
  int occ = 0;
  if (!BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, b->threads, smem), "occupancy")) return false;
  if (occ < 1) {
    set_error(err, PMCG_EDIM, __LINE__, "batch kernel does not fit on an SM (%zu B shared memory)", smem);
    return false;
  }
  b->bps = std::max(1, std::min(bps, occ));
  b->grid = b->sms * b->bps;
  return true;
}

static void drop_graph(pmcg_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->graph = false;
}

// Capture upload + persistent launch + statistics download in one graph.
static void capture_graph(pmcg_batch *b) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return; }
  cudaError_t e1 = cudaMemcpyAsync(b->d_dyn, b->h_dyn, sizeof(BatchDyn) * b->R, cudaMemcpyHostToDevice, b->s);
  cudaError_t e2 = launch_any(b, 0, kBStages - 1);
  cudaError_t e3 = cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(DevStats) * b->R, cudaMemcpyDeviceToHost, b->s);
  cudaError_t e4 = cudaStreamEndCapture(b->s, &g);
  if (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess && e4 == cudaSuccess && g &&
      cudaGraphInstantiate(&b->gexec, g, 0) == cudaSuccess) {
    b->graph = true;
  } else {
    b->gexec = nullptr;
    b->graph = false;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
}

}  // namespace pmcg

namespace pmcg {
static void free_arrays(pmcg_batch *b) {
  if (b->d_desc) cudaFree(b->d_desc);
  if (b->d_dyn) cudaFree(b->d_dyn);
  if (b->h_dyn) cudaFreeHost(b->h_dyn);
  if (b->d_starts) cudaFree(b->d_starts);
  if (b->d_snpre) cudaFree(b->d_snpre);
  if (b->d_stats) cudaFree(b->d_stats);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  b->d_desc = nullptr; b->d_dyn = nullptr; b->h_dyn = nullptr; b->d_starts = nullptr; b->d_snpre = nullptr;
  b->d_stats = nullptr; b->h_stats = nullptr;
  b->cap = 0;
}

// Bind the runs: descriptors, capacity (kept across binds, grown when short),
// the runs' streams drained, their draw counts zeroed, the tuned configuration
// of this shape and the prefix tables. The graph is captured at the second
// iteration after a bind, so a batch rebound every iteration does not pay for
// captures it would use once.
static bool batch_bind(pmcg_batch *b, int nruns, pmcg_run *const *runs, error **err) {
  if (nruns < 1 || !runs) {
    set_error(err, PMCG_EARG, __LINE__, "batch: no runs");
    return false;
  }
  std::vector<BatchDesc> hd(nruns);
  for (int r = 0; r < nruns; r++) {
    pmcg_run *run = runs[r];
    if (!run || run->w.prec != PMCG_MIXED || run->w.D > 32 || !run->post || run->post->plugins.size() != 1) {
      set_error(err, PMCG_EUNSUPPORTED, __LINE__,
                "batch run %d: needs a mixed-precision run with D <= 32 and exactly one likelihood", r);
      return false;
    }
    if (run->launched) {
      set_error(err, PMCG_EARG, __LINE__, "batch run %d: an asynchronous iteration was not waited for", r);
      return false;
    }
    run->img_stale = true;                  // the batch's updates leave the operand image behind
    const Work &w = run->w;
    const Plugin &pl = run->post->plugins[0];
    BatchDesc &d = hd[r];
    memset(&d, 0, sizeof(d));
    d.prop = w.prop.view();
    d.ptype = pl.type;
    if (pl.type == kPluginMix) d.target = pl.mix.view();
    if (pl.type == kPluginSn) d.sn = pl.sn;
    if (pl.type == kPluginTpl) d.tpl = pl.tpl;
    d.logpr = run->post->logpr;
    d.has_prior = run->post->has_prior ? 1 : 0;
    d.prior = run->post->prior;
    d.N = w.N;
    d.S = w.S;
    d.CHp = mix_chunk(w.D, w.ldx, w.K);
    d.CHt = pl.type == kPluginMix ? mix_chunk(w.D, w.ldx, pl.mix.K) : 1;
    d.maxd = w.ldx <= 8 ? 8 : (w.ldx <= 16 ? 16 : 32);
    d.key0 = (uint32_t)run->seed;
    d.key1 = (uint32_t)(run->seed >> 32);
    d.bmin = run->box ? w.bmin : nullptr;
    d.bmax = run->box ? w.bmax : nullptr;
    d.X32 = w.X32; d.idx = w.idx; d.counts = w.counts; d.flg = w.flg;
    d.logq = w.logq; d.logpost = w.logpost; d.logw = w.logw;
    d.lt32 = w.lt32; d.Q32 = w.Q32; d.aw32 = w.aw32;
    d.wpart = w.wpart; d.empart = w.empart; d.st = w.dstats;
    d.w = w.prop.w; d.mu = w.prop.mu; d.L = w.prop.L; d.Wt = w.prop.Wt; d.b = w.prop.b;
    d.logdetL = w.prop.logdetL; d.cw = w.prop.cw; d.lconst = w.prop.lconst;
    d.W32 = w.prop.W32; d.b32 = w.prop.b32; d.lconst32 = w.prop.lconst32; d.L32 = w.prop.L32; d.mu32 = w.prop.mu32;
  }
  drop_graph(b);
  if (nruns > b->cap) {
    if (!BCK(cudaStreamSynchronize(b->s), "batch stream")) return false;
    free_arrays(b);
    const int cap = std::max(nruns, 16);
    bool ok = BCK(cudaMalloc(&b->d_desc, sizeof(BatchDesc) * cap), "descriptors") &&
              BCK(cudaMalloc(&b->d_dyn, sizeof(BatchDyn) * cap), "parameters") &&
              BCK(cudaMallocHost(&b->h_dyn, sizeof(BatchDyn) * cap), "parameters") &&
              BCK(cudaMalloc(&b->d_starts, sizeof(uint32_t) * kBStages * (cap + 1)), "prefix tables") &&
              BCK(cudaMalloc(&b->d_snpre, sizeof(uint32_t) * (cap + 1)), "prefix tables") &&
              BCK(cudaMalloc(&b->d_stats, sizeof(DevStats) * cap), "stats") &&
              BCK(cudaMallocHost(&b->h_stats, sizeof(DevStats) * cap), "stats");
    if (!ok) {
      free_arrays(b);
      return false;
    }
    b->cap = cap;
  }
  b->R = nruns;
  b->runs.assign(runs, runs + nruns);
  b->hdesc.swap(hd);
  // the runs' own streams may still have work queued (proposal uploads): drain
  // the busy ones (an idle stream answers the query at once)
  for (int r = 0; r < nruns; r++) {
    const cudaError_t q = cudaStreamQuery(runs[r]->w.s);
    if (q == cudaErrorNotReady) {
      if (!BCK(cudaStreamSynchronize(runs[r]->w.s), "run stream")) return false;
    } else if (!BCK(q, "run stream")) {
      return false;
    }
  }
  bool ok = BCK(cudaMemcpyAsync(b->d_desc, b->hdesc.data(), sizeof(BatchDesc) * nruns, cudaMemcpyHostToDevice, b->s),
                "descriptors");
  // The batch's draws add to the counts, which its preparation stage zeroes
  // after each iteration: start from zero (a fresh run's counts are
  // uninitialised; a run iterated alone holds that iteration's counts).
  if (ok) {
    batch_zero_counts_kernel<<<nruns, 128, 0, b->s>>>(b->d_desc, nruns);
    ok = BCK(cudaGetLastError(), "counts") && BCK(cudaStreamSynchronize(b->s), "descriptors");
  }
  // a tuned configuration for this shape, if any
  int spt = 2, bps = 1;
  b->snt = 128;
  {
    TuneKey key;
    for (const BatchDesc &d : b->hdesc) {
      key.shape.push_back(d.prop.D); key.shape.push_back(d.prop.K);
      key.shape.push_back((long long)d.N); key.shape.push_back(d.ptype);
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) { spt = it->second.spt; bps = it->second.bps; b->snt = it->second.snt; }
  }
  ok = ok && batch_configure(b, spt, bps, err);
  b->iters_bound = 0;
  return ok;
}
}  // namespace pmcg

extern "C" pmcg_batch *pmcg_batch_create(int nruns, pmcg_run *const *runs, error **err) {
  if (nruns < 1 || !runs) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_batch_create: no runs");
    return nullptr;
  }
  pmcg_batch *b = new pmcg_batch();
  int dev = 0;
  bool ok = BCK(cudaGetDevice(&dev), "device") &&
            BCK(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev), "SM count") &&
            BCK(cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking), "stream") &&
            BCK(cudaEventCreate(&b->e0), "event") && BCK(cudaEventCreate(&b->e1), "event") &&
            batch_bind(b, nruns, runs, err);
  if (!ok) {
    pmcg_batch_free(&b);
    return nullptr;
  }
  return b;
}

extern "C" void pmcg_batch_rebind(pmcg_batch *b, int nruns, pmcg_run *const *runs, error **err) {
  if (!b) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_batch_rebind: no batch");
    return;
  }
  if (!BCK(cudaStreamSynchronize(b->s), "batch stream")) return;
  batch_bind(b, nruns, runs, err);
}

extern "C" void pmcg_batch_iterate(pmcg_batch *b, const double *betas, pmcg_iter_stats *stats, error **err) {
  for (int r = 0; r < b->R; r++) {
    b->h_dyn[r].beta = betas ? betas[r] : 1.0;
    b->h_dyn[r].call = b->runs[r]->calls;
    b->h_dyn[r].pad = 0;
  }
  // the graph from the second iteration of a binding on (see batch_bind)
  if (!b->graph && !b->stage_timing && b->iters_bound >= 1) capture_graph(b);
  b->iters_bound++;
  bool ok = BCK(cudaEventRecord(b->e0, b->s), "event");
  b->staged_last = false;
  if (ok && b->stage_timing) {
    // the same stages, one launch each, events between them
    for (int g = 0; ok && g <= kBStages; g++)
      if (!b->sev[g]) ok = BCK(cudaEventCreate(&b->sev[g]), "event");
    ok = ok && BCK(cudaMemcpyAsync(b->d_dyn, b->h_dyn, sizeof(BatchDyn) * b->R, cudaMemcpyHostToDevice, b->s),
                   "parameters");
    for (int g = 0; ok && g < kBStages; g++)
      ok = BCK(cudaEventRecord(b->sev[g], b->s), "event") && BCK(launch_any(b, g, g), "batch stage");
    ok = ok && BCK(cudaEventRecord(b->sev[kBStages], b->s), "event") &&
         BCK(cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(DevStats) * b->R, cudaMemcpyDeviceToHost, b->s),
             "stats");
    b->staged_last = ok;
  } else if (ok && b->graph) {
    ok = BCK(cudaGraphLaunch(b->gexec, b->s), "batch graph");
  } else if (ok) {
    ok = BCK(cudaMemcpyAsync(b->d_dyn, b->h_dyn, sizeof(BatchDyn) * b->R, cudaMemcpyHostToDevice, b->s),
             "parameters") &&
         BCK(launch_any(b, 0, kBStages - 1), "batch kernel") &&
         BCK(cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(DevStats) * b->R, cudaMemcpyDeviceToHost, b->s), "stats");
  }
  ok = ok && BCK(cudaEventRecord(b->e1, b->s), "event") && BCK(cudaStreamSynchronize(b->s), "batch iteration");
  if (!ok) return;
  cudaEventElapsedTime(&b->last_ms, b->e0, b->e1);
  if (b->staged_last)
    for (int g = 0; g < kBStages; g++) cudaEventElapsedTime(&b->stage_ms[g], b->sev[g], b->sev[g + 1]);
  for (int r = 0; r < b->R; r++) {
    pmcg_run *run = b->runs[r];
    *run->w.hstats = b->h_stats[r];
    run->calls++;
    run->last_launches = 1;
    int status = b->h_stats[r].status;
    if (status == 0) {
      // runs in revive mode revive their dead components, as when iterated alone
      error *le = nullptr;
      if (!run_revive_dead(run, &le)) status = isError(le) ? getErrorValue(le) : PMCG_ECUDA;
      purgeError(&le);
    }
    if (stats) {
      const DevStats &h = b->h_stats[r];
      pmcg_iter_stats &o = stats[r];
      o.ln_evidence = h.ln_evidence; o.perplexity = h.perplexity; o.ess = h.ess; o.enc = h.enc;
      o.logSum = h.logSum; o.maxW = h.maxW; o.nok = (size_t)h.nok; o.ndead = h.ndead; o.status = status;
    }
  }
}

extern "C" void pmcg_batch_autotune(pmcg_batch *b, error **err) {
  const int spts[2] = {1, 2};
  const int bpss[3] = {1, 2, 4};
  float best = 1e30f;
  int bspt = b->spt, bbps = b->bps;
  // The grouped SN kernel's block size (its time does not depend on the other
  // two knobs): timed alone, three times per candidate, the last two kept. It
  // rewrites the SN runs' log-posteriors of the current sample (the same values).
  if (b->sn_items > 0) {
    const int snts[3] = {64, 128, 256};
    float sbest = 1e30f;
    int bsnt = b->snt;
    for (int ti = 0; ti < 3; ti++) {
      error *e = nullptr;
      b->snt = snts[ti];
      if (!batch_configure(b, b->spt, b->bps, &e)) { purgeError(&e); continue; }
      float tmin = 1e30f;
      for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(b->e0, b->s);
        cudaError_t ce = launch_sn_group(b);
        cudaEventRecord(b->e1, b->s);
        if (ce != cudaSuccess || cudaStreamSynchronize(b->s) != cudaSuccess) { tmin = 1e30f; cudaGetLastError(); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        if (rep > 0) tmin = std::min(tmin, ms);
      }
      if (tmin < sbest) { sbest = tmin; bsnt = snts[ti]; }
    }
    b->snt = bsnt;
  }
  // Time draw..log posterior (they only overwrite the sample buffers, which
  // the next iteration redraws): twice per candidate, keep the faster.
  for (int si = 0; si < 2; si++) {
    for (int bi = 0; bi < 3; bi++) {
      error *e = nullptr;
      if (!batch_configure(b, spts[si], bpss[bi], &e)) { purgeError(&e); continue; }
      if (b->bps != bpss[bi]) continue;  // occupancy clamp: already covered
      float tmin = 1e30f;
      for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(b->e0, b->s);
        cudaError_t ce = launch_any(b, kBDraw, kBLogpost);
        cudaEventRecord(b->e1, b->s);
        if (ce != cudaSuccess || cudaStreamSynchronize(b->s) != cudaSuccess) { tmin = 1e30f; cudaGetLastError(); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        if (rep > 0) tmin = std::min(tmin, ms);
      }
      if (tmin < best) { best = tmin; bspt = spts[si]; bbps = bpss[bi]; }
    }
  }
  if (!batch_configure(b, bspt, bbps, err)) return;
  {
    TuneKey key;
    for (const BatchDesc &d : b->hdesc) {
      key.shape.push_back(d.prop.D); key.shape.push_back(d.prop.K);
      key.shape.push_back((long long)d.N); key.shape.push_back(d.ptype);
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {b->spt, b->bps, b->snt};
  }
  capture_graph(b);
}

extern "C" void pmcg_batch_config(const pmcg_batch *b, int *samples_per_thread, int *blocks_per_sm, int *grid,
                                  int *graph) {
  if (samples_per_thread) *samples_per_thread = b->spt;
  if (blocks_per_sm) *blocks_per_sm = b->bps;
  if (grid) *grid = b->grid;
  if (graph) *graph = b->graph ? 1 : 0;
}

extern "C" double pmcg_batch_last_ms(const pmcg_batch *b) { return b->last_ms; }

extern "C" int pmcg_batch_sn_block(const pmcg_batch *b) { return b ? b->snt : 0; }

extern "C" void pmcg_batch_set_stage_timing(pmcg_batch *b, int on) {
  if (b) b->stage_timing = on != 0;
}

extern "C" int pmcg_batch_stage_ms(const pmcg_batch *b, double *ms) {
  static_assert(kBStages == PMCG_BATCH_STAGES, "stage count");
  if (!b || !ms || !b->staged_last) return -1;
  for (int g = 0; g < kBStages; g++) ms[g] = b->stage_ms[g];
  return 0;
}

extern "C" void pmcg_batch_free(pmcg_batch **pb) {
  if (!pb || !*pb) return;
  pmcg_batch *b = *pb;
  drop_graph(b);
  if (b->s) cudaStreamSynchronize(b->s);
  free_arrays(b);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  for (cudaEvent_t e : b->sev)
    if (e) cudaEventDestroy(e);
  if (b->s) cudaStreamDestroy(b->s);
  delete b;
  *pb = nullptr;
}
