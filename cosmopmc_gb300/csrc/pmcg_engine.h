// pmcg_engine.h — engine-internal state shared by pmcg_engine.cu (runs,
// drop-in mirrors, posteriors) and k_batch.cu (the batch kernel). Not part of
// the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pmcg.h"
#include "pmcg_internal.h"
#include "pmcg_kernels.h"

namespace pmcg {

// Carves one device allocation into 256-byte aligned arrays. First pass
// (base == nullptr) only measures.
struct Carver {
  char *base = nullptr;
  size_t off = 0;
  template <typename T>
  T *take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

enum PluginType { kPluginMix = 1, kPluginSn = 2, kPluginTpl = 3 };
struct Plugin {
  int type = 0;
  DevMix mix;
  SnDev sn;
  TplDev tpl;
};

// Buffers and scratch for one sample of N points (one run or one drop-in mirror).
struct Work {
  int K = 0, D = 0, df = -1, prec = 0, ldx = 0, S = 0;
  int tc = -1;   // tensor cores for this handle: 1 on, 0 off, -1 the process default
  size_t N = 0;
  cudaStream_t s = nullptr;
  DevMix prop;
  double *bmin = nullptr, *bmax = nullptr;
  double *X64 = nullptr;
  float *X32 = nullptr;
  int *idx = nullptr, *counts = nullptr;
  short *flg = nullptr;
  double *logq = nullptr, *logpost = nullptr, *logw = nullptr, *wbar = nullptr;
  double *lt64 = nullptr, *Q64 = nullptr;
  float *lt32 = nullptr, *Q32 = nullptr, *aw32 = nullptr;
  uint32_t *emmask = nullptr;  // EM listing bits (mixed path)
  int *perm = nullptr, *cursor = nullptr;  // draws bucketed by component (mixed path)
  WRed *wpart = nullptr;
  unsigned *wdone = nullptr;   // weight tiles finished (zero between weight steps)
  double *empart = nullptr;
  DevStats *dstats = nullptr, *hstats = nullptr;
  void *arena = nullptr;
  int launches = 0;
};

bool work_alloc(Work &w, int K, int D, int df, int prec, size_t N, error **err);
void work_free(Work &w);
// Device bytes work_alloc takes for this shape (admission control).
size_t work_bytes(int K, int D, int df, int prec, size_t N);

}  // namespace pmcg

struct pmcg_posterior {
  int npar = 0;
  double logpr = 0.0;          // constant per point: logpr_box + logpr_special
  double logpr_box = 0.0;      // flat box prior, -sum log(max - min)
  double logpr_special = 0.0;  // special prior (volume correction)
  int special = 0;
  std::vector<double> min, max;
  std::vector<pmcg::Plugin> plugins;
  bool has_prior = false;      // Gaussian / Student-t prior on a parameter subset
  pmcg::PriorDev prior;
  uint64_t stamp = 0;  // new at allocation and at every change (unique over the process)
};

// Per-iteration scalars read by the kernels of a captured iteration.
struct pmcg_iter_params {
  double beta;
  uint32_t call;
};

struct pmcg_run {
  pmcg::Work w;
  const pmcg_posterior *post = nullptr;
  bool box = false;
  uint64_t seed = 0;
  uint32_t calls = 0;
  int timing = 0;  // 1 per stage (direct launches), 2 whole iterations
  cudaEvent_t ev[PMCG_NSTAGE + 1] = {};
  double stage_ms[PMCG_NSTAGE] = {};
  double iter_ms = 0.0;
  int timed = 0;
  int last_launches = 0;
  // Single-precision runs replay one iteration as a CUDA graph: the kernels
  // read beta and the call counter from dpar, which the graph's first node
  // copies from the pinned hpar. Captured on first use; re-captured when the
  // tensor-core switch changes; graph_off after a failed capture.
  pmcg_iter_params *dpar = nullptr, *hpar = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_tc = -1, graph_launches = 0;
  bool graph_off = false;
  // An iteration in flight: a graph launched and not yet waited for
  // (pending_graph); pmcg_run_iterate_async's launch and its outcome.
  bool pending_graph = false;
  bool launched = false, launch_ok = false;
  // the proposal was updated by a batch, which keeps no tensor-core operand
  // image: rebuilt before the run's next iteration alone
  bool img_stale = false;
  error *launch_err = nullptr;
  // Dead components (sdead_comp, exec/cosmo_pmc.c:239-284): buried (default) or
  // revived after each update; the box on the host for the revival's shifts.
  int dead_mode = PMCG_DEAD_BURY;
  double fshift = 0.1;
  int nrevive = 1;
  std::vector<double> hmin, hmax;
};

namespace pmcg {
// The revival step of a run in PMCG_DEAD_REVIVE mode after a successful update
// (the run's statistics are in w.hstats); no-op in bury mode.
bool run_revive_dead(pmcg_run *r, error **err);
}  // namespace pmcg
