// pmcg_engine.cu — the PMC iteration engine behind the C ABI:
//  * device-resident runs (pmcg_run_*), one stream each;
//  * device posterior plugins (Gaussian mixture, SN Ia, dense template);
//  * the pmclib-named drop-in entry points, which keep a device mirror of
//    each pmc_simu they see (exec/cosmo_pmc.c:293-402 is the caller).
// Every per-sample computation runs in the CUDA kernels of k_*.cu; the host
// code here only moves data, sequences launches and reports errors.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "../../include/pmcg.h"
#include "pmcg_engine.h"

using pmcg::set_error;

namespace pmcg {

static bool ck(cudaError_t e, error **err, int line, const char *what) {
  if (e == cudaSuccess) return true;
  set_error(err, PMCG_ECUDA, line, "%s: %s", what, cudaGetErrorString(e));
  return false;
}
#define CK(expr, what) ck((expr), err, __LINE__, (what))

void work_free(Work &w) {
  devmix_free(w.prop);
  if (w.arena) cudaFree(w.arena);
  if (w.hstats) cudaFreeHost(w.hstats);
  if (w.s) cudaStreamDestroy(w.s);
  w = Work();
}

// Lays out the arrays of a Work in one allocation (c.base == nullptr: measure only).
static void work_layout(Work &w, Carver &c, size_t empart_bytes) {
  const size_t N = w.N;
  const int K = w.K, D = w.D, prec = w.prec;
  const bool t = w.df > 0;
  c.off = 0;
  w.bmin = c.take<double>(D);
  w.bmax = c.take<double>(D);
  w.X64 = c.take<double>(N * D);
  w.X32 = prec ? c.take<float>(N * w.ldx) : nullptr;
  w.idx = c.take<int>(N);
  w.counts = c.take<int>(K);
  w.flg = c.take<short>(N);
  w.logq = c.take<double>(N);
  w.logpost = c.take<double>(N);
  w.logw = c.take<double>(N);
  w.wbar = c.take<double>(N);
  w.lt64 = prec ? nullptr : c.take<double>(N * K);
  w.Q64 = (!prec && t) ? c.take<double>(N * K) : nullptr;
  w.lt32 = prec ? c.take<float>(N * K) : nullptr;
  w.Q32 = (prec && t) ? c.take<float>(N * K) : nullptr;
  w.aw32 = prec ? c.take<float>(N) : nullptr;
  w.emmask = prec ? c.take<uint32_t>(em_mask_words(K, N)) : nullptr;
  w.perm = prec ? c.take<int>(N) : nullptr;
  w.cursor = prec ? c.take<int>(2 * (size_t)K) : nullptr;
  w.wpart = c.take<WRed>(weight_tiles(N));
  w.wdone = c.take<unsigned>(1);
  w.empart = c.take<double>(empart_bytes / sizeof(double));
  w.dstats = c.take<DevStats>(1);
}

size_t work_bytes(int K, int D, int df, int prec, size_t N) {
  Work w;
  w.K = K; w.D = D; w.df = df; w.prec = prec; w.N = N; w.ldx = round4(D);
  int S;
  size_t empart_bytes = em_partials_size(prec, K, D, &S, N);
  Carver c;
  work_layout(w, c, empart_bytes);
  return c.off + 256 + devmix_bytes(K, D);  // + the proposal arena
}

bool work_alloc(Work &w, int K, int D, int df, int prec, size_t N, error **err) {
  if (D < 1 || D > kMaxD || K < 1 || K > kMaxK) {
    set_error(err, PMCG_EDIM, __LINE__, "unsupported shape K=%d D=%d (K<=%d, D<=%d)", K, D, kMaxK, kMaxD);
    return false;
  }
  w.K = K; w.D = D; w.df = df; w.prec = prec; w.N = N; w.ldx = round4(D);
  size_t empart_bytes = em_partials_size(prec, K, D, &w.S, N);
  Carver c;
  for (int pass = 0; pass < 2; pass++) {
    work_layout(w, c, empart_bytes);
    if (pass == 0) {
      if (!CK(cudaMalloc(&w.arena, c.off + 256), "device buffers")) return false;
      c.base = (char *)w.arena;
    }
  }
  if (!CK(cudaMallocHost(&w.hstats, sizeof(DevStats)), "pinned stats")) return false;
  if (!CK(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking), "stream")) return false;
  if (!CK(cudaMemsetAsync(w.dstats, 0, sizeof(DevStats), w.s), "stats") ||
      !CK(cudaMemsetAsync(w.counts, 0, sizeof(int) * K, w.s), "counts") ||
      !CK(cudaMemsetAsync(w.wdone, 0, sizeof(unsigned), w.s), "weight counter"))
    return false;
  if (!CK(devmix_alloc(w.prop, K, D, df), "proposal buffers")) return false;
  return true;
}
static bool upload_box(Work &w, const double *bmin, const double *bmax, error **err) {
  if (!bmin) return true;
  return CK(cudaMemcpyAsync(w.bmin, bmin, sizeof(double) * w.D, cudaMemcpyHostToDevice, w.s), "box") &&
         CK(cudaMemcpyAsync(w.bmax, bmax, sizeof(double) * w.D, cudaMemcpyHostToDevice, w.s), "box");
}

// Below this many samples the single-precision draw runs in one pass: the
// component-ordered draw's two extra kernels (pick, bucket) only pay off when
// there are enough samples per component to share a factor; the values are
// the same either way.
constexpr size_t kGroupedDrawMin = (size_t)1 << 15;

static bool stage_draw(Work &w, bool box, uint64_t seed, uint32_t call, error **err,
                       const uint32_t *callp = nullptr) {
  if (!CK(cudaMemsetAsync(w.counts, 0, sizeof(int) * w.K, w.s), "counts")) return false;
  if (w.prec == 1 && w.N >= kGroupedDrawMin) {
    w.launches += 3;
    return CK(launch_draw_grouped(w.prop.view(), w.N, seed, call, box ? w.bmin : nullptr, box ? w.bmax : nullptr,
                                  w.X32, w.idx, w.flg, w.counts, w.perm, w.cursor, w.s, callp),
              "draw kernels");
  }
  w.launches += 1;
  return CK(launch_draw(w.prec, w.prop.view(), w.N, seed, call, box ? w.bmin : nullptr, box ? w.bmax : nullptr,
                        nullptr, nullptr, nullptr, w.X64, w.X32, w.idx, w.flg, w.counts, w.s, callp),
            "draw kernel");
}

// The handle's tensor-core setting, else the process default.
static int tc_on(const Work &w) { return w.tc >= 0 ? w.tc : g_use_tensor_cores; }

// Single-precision mixture log-density on the tensor cores (tcgen05) when the
// switch is on and the mixture carries an operand image (D <= 32).
static bool use_tensor_cores(const Work &w, const DevMix &m) {
  return w.prec == 1 && tc_on(w) && m.bimg != nullptr && m.D <= 32;
}

static bool stage_logq(Work &w, error **err) {
  w.launches += 1;
  if (use_tensor_cores(w, w.prop))
    return CK(launch_umma_logq(w.prop.view(), w.prop.bimg, w.N, w.X32, w.logq, 0, 0.0, w.lt32, w.Q32,
                               &w.dstats->tc_err, w.s),
              "tensor-core mixture log-pdf kernel");
  return CK(launch_mixlogpdf(w.prec, w.prop.view(), w.N, w.X64, w.X32, w.logq, 0, 0.0, w.lt64, w.Q64, w.lt32,
                             w.Q32, w.s),
            "mixture log-pdf kernel");
}

// all_values: every sample's log-posterior is wanted (the batched posterior
// evaluation, importance_sample). Within an iteration the weight step reads it
// only where flg = 1, so a first likelihood that can write logpr + log L
// itself (SN Ia, a mixture, the tensor-core template) does, and the fill of
// logpr is left out (the same values where flg = 1).
static bool stage_logpost(Work &w, const pmcg_posterior *p, error **err, bool all_values = true) {
  if (p->npar != w.D) {
    set_error(err, PMCG_EDIM, __LINE__, "posterior has %d parameters, sample %d", p->npar, w.D);
    return false;
  }
  bool first_assigns = false;   // the first likelihood assigns
  if (!all_values && !p->plugins.empty()) {
    const Plugin &p0 = p->plugins[0];
    first_assigns = p0.type == kPluginSn || p0.type == kPluginMix ||
                 (p0.type == kPluginTpl && w.prec == 1 && tc_on(w) && p0.tpl.uimg);
  }
  if (!first_assigns) {
    w.launches += 1;
    if (!CK(launch_fill_f64(w.logpost, w.N, p->logpr, w.s), "fill")) return false;
  }
  bool first = true;
  for (const Plugin &pl : p->plugins) {
    const bool assign = first_assigns && first;
    first = false;
    w.launches += 1;
    if (pl.type == kPluginMix) {
      if (use_tensor_cores(w, pl.mix)) {
        if (!CK(launch_umma_logq(pl.mix.view(), pl.mix.bimg, w.N, w.X32, w.logpost, assign ? 0 : 1,
                                 assign ? p->logpr : 0.0, nullptr, nullptr, &w.dstats->tc_err, w.s),
                "tensor-core target mixture kernel"))
          return false;
      } else if (!CK(launch_mixlogpdf(w.prec, pl.mix.view(), w.N, w.X64, w.X32, w.logpost, assign ? 0 : 1,
                                      assign ? p->logpr : 0.0, nullptr, nullptr, nullptr, nullptr, w.s),
                     "target mixture kernel"))
        return false;
    } else if (pl.type == kPluginSn) {
      if (!CK(launch_sn(w.prec, pl.sn, w.N, w.D, w.X64, w.X32, w.ldx, w.logpost, w.flg, w.s, assign ? 1 : 0,
                        p->logpr),
              "SN kernel"))
        return false;
    } else if (pl.type == kPluginTpl) {
      if (w.prec == 1 && tc_on(w) && pl.tpl.uimg) {
        if (!CK(launch_tpl_umma(pl.tpl.uimg, pl.tpl.Dpar, w.N, w.X32, w.ldx, w.logpost, w.flg, &w.dstats->tc_err,
                                w.s, assign ? 1 : 0, p->logpr),
                "tensor-core template kernel"))
          return false;
      } else if (!CK(launch_tpl(w.prec, pl.tpl, w.N, w.X64, w.X32, w.ldx, w.logpost, w.flg, w.s), "template kernel")) {
        return false;
      }
    }
  }
  if (p->has_prior) {
    w.launches += 1;
    if (!CK(launch_prior(w.prec, p->prior, w.N, w.D, w.X64, w.X32, w.ldx, w.logpost, w.s), "prior kernel"))
      return false;
  }
  return true;
}

static bool stage_weights(Work &w, double beta, bool with_logq, error **err, const double *betap = nullptr) {
  w.launches += 1;
  return CK(launch_weights(w.N, beta, w.logpost, with_logq ? w.logq : nullptr, w.flg, w.logw, w.wpart, w.dstats,
                           w.s, w.prec == 1, betap, w.wdone),
            "weight kernel");
}

// The EM update of mixture `mix` (read as the old proposal, written with the new
// one) with the statistics `st` (read: the weight step's; written: the update's).
static bool stage_em_into(Work &w, DevMix &mix, DevStats *st, error **err) {
  // statistics and the fused update; mixed: + the weight factor with the listing bits
  w.launches += w.prec ? 3 : 2;
  return CK(launch_em(w.prec, mix, w.N, w.X64, w.X32, w.logw, w.logq, w.lt64, w.Q64, w.lt32, w.Q32, w.counts,
                      w.empart, w.S, st, w.D, w.aw32, w.emmask, w.s),
            "EM kernels");
}

static bool stage_em(Work &w, error **err) { return stage_em_into(w, w.prop, w.dstats, err); }

// Status of the statistics already copied to w.hstats.
static bool check_stats(Work &w, error **err) {
  if (w.hstats->tc_err != 0) {
    set_error(err, PMCG_ETIMEOUT, __LINE__, "tensor-core log-density: a pipeline wait expired");
    return false;
  }
  if (w.hstats->status != 0) {
    set_error(err, w.hstats->status, __LINE__,
              w.hstats->status == PMCG_ENOWEIGHT ? "every sample has zero weight" : "all component weights are zero");
    return false;
  }
  return true;
}

static bool fetch_stats(Work &w, error **err) {
  if (!CK(cudaMemcpyAsync(w.hstats, w.dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, w.s), "stats") ||
      !CK(cudaStreamSynchronize(w.s), "iteration"))
    return false;
  return check_stats(w, err);
}

// Single-precision runs: every live component must be wider than single
// precision resolves around its mean (max_i sum_j |(L^-1)_ij mu_j| at most
// kF32RangeMax, the device check of the EM update); else PMCG_EPRECISION.
static bool f32_range_ok(const std::vector<double> &w, const std::vector<double> &mu, const std::vector<double> &L,
                         int K, int D, error **err) {
  std::vector<double> Wr((size_t)D * D);
  for (int k = 0; k < K; k++) {
    if (!(w[k] > 0.0)) continue;
    const double *Lk = &L[(size_t)k * D * D], *mk = &mu[(size_t)k * D];
    double rmax = 0.0;
    for (int i = 0; i < D; i++) {   // row i of L^-1 by forward substitution
      double ra = 0.0;
      for (int j = i; j >= 0; j--) {
        double t = (i == j) ? 1.0 : 0.0;
        for (int q = j + 1; q <= i; q++) t -= Lk[(size_t)q * D + j] * Wr[(size_t)i * D + q];
        Wr[(size_t)i * D + j] = t / Lk[(size_t)j * D + j];
      }
      for (int j = 0; j <= i; j++) ra += std::fabs(Wr[(size_t)i * D + j]) * std::fabs(mk[j]);
      if (!(ra <= rmax)) rmax = ra;
    }
    if (!(rmax <= kF32RangeMax)) {
      set_error(err, PMCG_EPRECISION, __LINE__,
                "proposal component %d is narrower than single precision resolves around its mean "
                "(max_i sum_j |(L^-1)_ij mu_j| = %g); use a PMCG_FP64 run",
                k, rmax);
      return false;
    }
  }
  return true;
}

static bool upload_mix(DevMix &m, const mix_mvdens *mix, cudaStream_t s, error **err, bool f32 = false) {
  std::vector<double> w, mu, L;
  if (!flatten_mix(mix, w, mu, L, err)) return false;
  if (f32 && !f32_range_ok(w, mu, L, mix->ncomp, mix->ndim, err)) return false;
  return CK(devmix_upload(m, w.data(), mu.data(), L.data(), s), "mixture upload") &&
         CK(cudaStreamSynchronize(s), "mixture upload");
}

}  // namespace pmcg

using namespace pmcg;

// ===================================================================== posterior
// Device posteriors standing in for the caller's posterior callbacks, keyed by
// the callback's extra pointer.
static std::mutex g_reg_mu;
static std::unordered_map<const void *, const pmcg_posterior *> g_registered;

namespace pmcg {
const pmcg_posterior *registered_posterior(const void *extra) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  auto it = g_registered.find(extra);
  return it == g_registered.end() ? nullptr : it->second;
}
}  // namespace pmcg

extern "C" void pmcg_register_posterior(const void *extra, const pmcg_posterior *post) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  if (post) g_registered[extra] = post;
  else g_registered.erase(extra);
}

static std::atomic<uint64_t> g_post_stamp{0};
static void restamp(pmcg_posterior *p) { p->stamp = ++g_post_stamp; }

extern "C" pmcg_posterior *pmcg_posterior_alloc(int npar, const double *min, const double *max, error **err) {
  if (npar < 1 || npar > kMaxD) {
    set_error(err, PMCG_EDIM, __LINE__, "npar %d", npar);
    return nullptr;
  }
  pmcg_posterior *p = new pmcg_posterior();
  p->npar = npar;
  p->logpr = 0.0;
  if (min && max) {
    p->min.assign(min, min + npar);
    p->max.assign(max, max + npar);
    for (int j = 0; j < npar; j++) {
      if (!(max[j] > min[j])) {
        set_error(err, PMCG_EARG, __LINE__, "The minimum #%d (%g) is not smaller than the maximum (%g)", j, min[j],
                  max[j]);
        delete p;
        return nullptr;
      }
      p->logpr -= std::log(max[j] - min[j]);
    }
  }
  p->logpr_box = p->logpr;
  restamp(p);
  return p;
}

extern "C" void pmcg_posterior_free(pmcg_posterior **p) {
  if (!p || !*p) return;
  forget_posterior(*p);
  {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    for (auto it = g_registered.begin(); it != g_registered.end();) {
      if (it->second == *p) it = g_registered.erase(it);
      else ++it;
    }
  }
  for (Plugin &pl : (*p)->plugins) {
    devmix_free(pl.mix);
    if (pl.sn.arena) cudaFree(pl.sn.arena);
    if (pl.tpl.arena) cudaFree(pl.tpl.arena);
  }
  if ((*p)->prior.arena) cudaFree((*p)->prior.arena);
  delete *p;
  *p = nullptr;
}

extern "C" void pmcg_posterior_add_mixmvdens(pmcg_posterior *p, const mix_mvdens *target, error **err) {
  if (!p || !target || target->ndim != p->npar) {
    set_error(err, PMCG_EDIM, __LINE__, "target dimension does not match the posterior");
    return;
  }
  Plugin pl;
  pl.type = kPluginMix;
  int df = target->comp[0]->df;
  if (!CK(devmix_alloc(pl.mix, target->ncomp, target->ndim, df), "target buffers")) return;
  if (!upload_mix(pl.mix, target, 0, err)) { devmix_free(pl.mix); return; }
  p->plugins.push_back(pl);
  restamp(p);
}

// prior_log_pdf_special (wrappers/src/param.c:1055-1101): a constant per point,
// log of the box volume of the affected parameters minus log of the special
// prior's volume; applied once per point with the flat prior (:994-999).
extern "C" void pmcg_posterior_set_special(pmcg_posterior *p, int special, int ind_w0, int ind_w1, double a_acc,
                                           error **err) {
  if (!p) {
    set_error(err, PMCG_EARG, __LINE__, "null posterior");
    return;
  }
  double c = 0.0;
  const bool box = !p->min.empty();
  switch (special) {
    case PMCG_SPECIAL_NONE:
      break;
    case PMCG_SPECIAL_UNITY:
      // minus the default flat prior
      if (box)
        for (int i = 0; i < p->npar; i++) c += std::log(p->max[i] - p->min[i]);
      break;
    case PMCG_SPECIAL_DE_CONSERVATIVE: {
      if (ind_w0 < -1 || ind_w0 >= p->npar || ind_w1 < -1 || ind_w1 >= p->npar || (ind_w1 >= 0 && ind_w0 < 0) ||
          (ind_w1 >= 0 && !(a_acc < 1.0))) {
        set_error(err, PMCG_EARG, __LINE__, "de_conservative: parameter indices (%d, %d) or a_acc %g invalid",
                  ind_w0, ind_w1, a_acc);
        return;
      }
      if (ind_w0 < 0) break;  // no w0_de among the parameters: nothing added
      if (!box) {
        set_error(err, PMCG_EARG, __LINE__, "de_conservative needs the prior box of w0_de");
        return;
      }
      const double lo = p->min[ind_w0], hi = p->max[ind_w0];
      if (lo > -1.0 || hi < -1.0 / 3.0) {
        set_error(err, PMCG_EARG, __LINE__,
                  "Range of w0_de [%g;%g] should not be smaller than de_conservative prior [-1;-1/3]", lo, hi);
        return;
      }
      if (ind_w1 < 0) {
        c = std::log(hi - lo) - std::log(2.0 / 3.0);
      } else {
        const double t = 0.5 * (2.0 / 3.0) * (2.0 / 3.0);
        c = std::log(hi - lo) + std::log(p->max[ind_w1] - p->min[ind_w1]) - std::log(t / (1.0 - a_acc)) -
            std::log(t);
      }
      break;
    }
    default:
      set_error(err, PMCG_EARG, __LINE__, "Unknown special prior type %d", special);
      return;
  }
  p->special = special;
  p->logpr_special = c;
  p->logpr = p->logpr_box + c;
  restamp(p);
}

// The config prior with indprior (wrappers/src/param.c:1009-1026): the prior's
// coordinates are the flagged parameters in increasing order.
extern "C" void pmcg_posterior_add_mvdens_prior(pmcg_posterior *p, const mvdens *prior, const int *indprior,
                                                error **err) {
  if (!p || !prior || prior->ndim < 1) {
    set_error(err, PMCG_EARG, __LINE__, "invalid prior");
    return;
  }
  const int d = prior->ndim;
  std::vector<int> idx;
  for (int j = 0; j < p->npar; j++)
    if (!indprior || indprior[j] == 1) idx.push_back(j);
  if ((int)idx.size() != d) {
    set_error(err, PMCG_EDIM, __LINE__, "prior has %d dimensions, %d parameters are flagged", d, (int)idx.size());
    return;
  }
  // Cholesky factor (copy), its inverse (packed rows) and the constant
  std::vector<double> L((size_t)d * d, 0.0);
  double logdetL = 0.0;
  if (prior->chol) {
    for (int i = 0; i < d; i++)
      for (int j = 0; j <= i; j++) L[(size_t)i * d + j] = prior->std[(size_t)i * d + j];
    for (int i = 0; i < d; i++) logdetL += std::log(L[(size_t)i * d + i]);
  } else if (host_cholesky(d, prior->std, L.data(), &logdetL) != 0) {
    set_error(err, PMCG_ECHOL, __LINE__, "prior covariance is not positive definite");
    return;
  }
  // L^-1 by forward substitution of the identity columns; stored as packed rows
  std::vector<double> Wt((size_t)d * (d + 1) / 2), Winv((size_t)d * d, 0.0);
  for (int c = 0; c < d; c++) {
    for (int i = c; i < d; i++) {
      double t = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; k++) t -= L[(size_t)i * d + k] * Winv[(size_t)k * d + c];
      Winv[(size_t)i * d + c] = t / L[(size_t)i * d + i];
    }
  }
  for (int i = 0, o = 0; i < d; i++)
    for (int j = 0; j <= i; j++) Wt[o++] = Winv[(size_t)i * d + j];
  PriorDev pd;
  pd.d = d;
  pd.df = prior->df > 0 ? prior->df : -1;
  for (int i = 0; i < d; i++) pd.idx[i] = idx[i];
  if (pd.df > 0) {
    const double nu = pd.df;
    pd.lconst = std::lgamma(0.5 * (nu + d)) - std::lgamma(0.5 * nu) - 0.5 * d * std::log(nu * PMCG_PI) - logdetL;
  } else {
    pd.lconst = -0.5 * d * PMCG_LN2PI - logdetL;
  }
  const size_t nw = Wt.size();
  Carver cv;
  for (int pass = 0; pass < 2; pass++) {
    cv.off = 0;
    pd.mu = cv.take<double>(d); pd.Wt = cv.take<double>(nw);
    pd.mu32 = cv.take<float>(d); pd.Wt32 = cv.take<float>(nw);
    if (pass == 0) {
      if (!CK(cudaMalloc(&pd.arena, cv.off + 256), "prior buffers")) return;
      cv.base = (char *)pd.arena;
    }
  }
  std::vector<float> mu32(prior->mean, prior->mean + d), Wt32(Wt.begin(), Wt.end());
  const bool ok = CK(cudaMemcpy(pd.mu, prior->mean, 8 * (size_t)d, cudaMemcpyHostToDevice), "prior upload") &&
                  CK(cudaMemcpy(pd.Wt, Wt.data(), 8 * nw, cudaMemcpyHostToDevice), "prior upload") &&
                  CK(cudaMemcpy(pd.mu32, mu32.data(), 4 * (size_t)d, cudaMemcpyHostToDevice), "prior upload") &&
                  CK(cudaMemcpy(pd.Wt32, Wt32.data(), 4 * nw, cudaMemcpyHostToDevice), "prior upload");
  if (!ok) { cudaFree(pd.arena); return; }
  if (p->prior.arena) cudaFree(p->prior.arena);
  p->prior = pd;
  p->has_prior = true;
  restamp(p);
}

extern "C" void pmcg_posterior_add_snia(pmcg_posterior *p, const pmcg_sn_data *sd, error **err) {
  if (!p || !sd || sd->nsn < 1 || sd->quad_nodes < 1 || sd->quad_nodes > 16 || !(sd->h > 0.0)) {
    set_error(err, PMCG_EARG, __LINE__, "invalid SN data");
    return;
  }
  const int ips[6] = {sd->ip_Omegam, sd->ip_Omegade, sd->ip_w0, sd->ip_M, sd->ip_alpha, sd->ip_beta};
  for (int q = 0; q < 6; q++) {
    if (ips[q] < -1 || ips[q] >= p->npar) {
      set_error(err, PMCG_EARG, __LINE__, "SN parameter index %d outside [-1, %d)", ips[q], p->npar);
      return;
    }
  }
  const int n = sd->nsn, G = sd->quad_nodes;
  std::vector<int> ix(n);
  for (int i = 0; i < n; i++) ix[i] = i;
  std::stable_sort(ix.begin(), ix.end(), [&](int a, int b) { return sd->z[a] < sd->z[b]; });
  if (!(sd->z[ix[0]] > 0.0)) {
    set_error(err, PMCG_EARG, __LINE__, "SN redshifts must be positive");
    return;
  }
  // Gauss-Legendre nodes by Newton iteration on P_G.
  std::vector<double> xg(G), wg(G);
  for (int i = 0; i < G; i++) {
    double t = std::cos(M_PI * (i + 0.75) / (G + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= G; k++) { double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
      if (G == 1) { p1 = t; p0 = 1.0; }
      dp = G * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    double p0 = 1.0, p1 = t;
    for (int k = 2; k <= G; k++) { double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
    if (G == 1) { p1 = t; p0 = 1.0; }
    dp = G * (t * p1 - p0) / (t * t - 1.0);
    xg[i] = t;
    wg[i] = 2.0 / ((1.0 - t * t) * dp * dp);
  }
  const double ckms = 299792.458;
  std::vector<double> z(n), spv2(n), mB(n), x1(n), c(n), cov6(6 * (size_t)n), za2(n), za3(n), zla(n);
  std::vector<double> na2((size_t)n * G), na3((size_t)n * G), nla((size_t)n * G), nw((size_t)n * G);
  double zprev = 0.0;
  for (int t = 0; t < n; t++) {
    int i = ix[t];
    z[t] = sd->z[i]; mB[t] = sd->mB[i]; x1[t] = sd->x1[i]; c[t] = sd->c[i];
    for (int q = 0; q < 6; q++) cov6[6 * (size_t)t + q] = sd->cov6[6 * (size_t)i + q];
    double spv = (5.0 / std::log(10.0)) * sd->v_pec / (ckms * z[t]);
    spv2[t] = spv * spv;
    double a = 1.0 + z[t];
    za2[t] = a * a; za3[t] = a * a * a; zla[t] = std::log(a);
    double hw = 0.5 * (z[t] - zprev), cc = 0.5 * (z[t] + zprev);
    for (int g = 0; g < G; g++) {
      double ag = 1.0 + cc + hw * xg[g];
      size_t q = (size_t)t * G + g;
      na2[q] = ag * ag; na3[q] = ag * ag * ag; nla[q] = std::log(ag); nw[q] = hw * wg[g];
    }
    zprev = z[t];
  }
  Plugin pl;
  pl.type = kPluginSn;
  SnDev &s = pl.sn;
  s.nsn = n; s.G = G; s.chi2mode = sd->chi2mode; s.add_logdet = sd->add_logdet;
  s.ip_om = sd->ip_Omegam; s.ip_ode = sd->ip_Omegade; s.ip_w0 = sd->ip_w0; s.ip_M = sd->ip_M;
  s.ip_alpha = sd->ip_alpha; s.ip_beta = sd->ip_beta;
  s.neg_M = sd->neg_M ? 1 : 0; s.neg_beta = sd->neg_beta ? 1 : 0;
  s.def_om = sd->def_Omegam; s.def_w0 = sd->def_w0; s.def_M = sd->def_M; s.def_alpha = sd->def_alpha;
  s.def_beta = sd->def_beta;
  s.dh = ckms / (100.0 * sd->h);
  s.sig_int2 = sd->sig_int * sd->sig_int;
  s.fdef_om = (float)s.def_om; s.fdef_w0 = (float)s.def_w0; s.fdef_M = (float)s.def_M;
  s.fdef_alpha = (float)s.def_alpha; s.fdef_beta = (float)s.def_beta;
  Carver cv;
  for (int pass = 0; pass < 2; pass++) {
    cv.off = 0;
    s.z = cv.take<double>(n); s.spv2 = cv.take<double>(n); s.mB = cv.take<double>(n); s.x1 = cv.take<double>(n);
    s.c = cv.take<double>(n); s.cov6 = cv.take<double>(6 * (size_t)n);
    s.za2 = cv.take<double>(n); s.za3 = cv.take<double>(n); s.zla = cv.take<double>(n);
    s.na2 = cv.take<double>((size_t)n * G); s.na3 = cv.take<double>((size_t)n * G);
    s.nla = cv.take<double>((size_t)n * G); s.nw = cv.take<double>((size_t)n * G);
    s.fnode = cv.take<float4>((size_t)n * G); s.fsn = cv.take<float4>(3 * (size_t)n); s.fzl2 = cv.take<float>(n);
    if (pass == 0) {
      if (!CK(cudaMalloc(&s.arena, cv.off + 256), "SN buffers")) return;
      cv.base = (char *)s.arena;
    }
  }
  auto up = [&](void *dst, const void *src, size_t bytes) {
    return CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "SN upload");
  };
  // reference model of the single-precision path (flat LambdaCDM 0.3/0.7, the
  // same nodes): D_M,ref and the reference residual m_B - mu_ref - M_ref
  const double il2 = 1.0 / std::log(2.0);
  std::vector<float4> fnode((size_t)n * G), fsn(3 * (size_t)n);
  std::vector<float> fzl2(n);
  {
    double I = 0.0;
    for (int t = 0; t < n; t++) {
      for (int g = 0; g < G; g++) {
        const size_t q = (size_t)t * G + g;
        I += nw[q] / std::sqrt(0.3 * na3[q] + 0.7);
        fnode[(size_t)g * n + t] = make_float4((float)na3[q], (float)na2[q], (float)(nla[q] * il2), (float)nw[q]);
      }
      const double mu_ref = 5.0 * std::log10((1.0 + z[t]) * s.dh * I) + 25.0;
      const double *W = &cov6[6 * (size_t)t];
      fsn[t] = make_float4((float)(mB[t] - mu_ref - (double)s.mref), (float)x1[t], (float)c[t], (float)(1.0 / I));
      fsn[n + t] = make_float4((float)(W[0] + s.sig_int2 + spv2[t]), (float)W[1], (float)W[2], (float)(2.0 * W[3]));
      fsn[2 * (size_t)n + t] = make_float4((float)(-2.0 * W[4]), (float)(-2.0 * W[5]), (float)za3[t], (float)za2[t]);
      fzl2[t] = (float)(zla[t] * il2);
    }
  }
  bool ok = up(s.z, z.data(), 8 * n) && up(s.spv2, spv2.data(), 8 * n) && up(s.mB, mB.data(), 8 * n) &&
            up(s.x1, x1.data(), 8 * n) && up(s.c, c.data(), 8 * n) && up(s.cov6, cov6.data(), 48 * (size_t)n) &&
            up(s.za2, za2.data(), 8 * n) && up(s.za3, za3.data(), 8 * n) && up(s.zla, zla.data(), 8 * n) &&
            up(s.na2, na2.data(), 8 * na2.size()) && up(s.na3, na3.data(), 8 * na3.size()) &&
            up(s.nla, nla.data(), 8 * nla.size()) && up(s.nw, nw.data(), 8 * nw.size()) &&
            up(s.fnode, fnode.data(), sizeof(float4) * fnode.size()) &&
            up(s.fsn, fsn.data(), sizeof(float4) * fsn.size()) && up(s.fzl2, fzl2.data(), 4 * (size_t)n);
  if (!ok) { cudaFree(s.arena); return; }
  p->plugins.push_back(pl);
  restamp(p);
}

extern "C" void pmcg_posterior_add_template(pmcg_posterior *p, int ndata, const double *A, const double *C,
                                            const double *dobs, error **err) {
  if (!p || ndata < 1 || !A || !C || !dobs) {
    set_error(err, PMCG_EARG, __LINE__, "invalid template data");
    return;
  }
  const int M = ndata, D = p->npar, P = 1 + D + D * (D + 1) / 2;
  // C = L L^T (FP64), At = L^-1 A, dt = L^-1 dobs: set-up, once per posterior.
  std::vector<double> L((size_t)M * M), At((size_t)M * P), dt(M);
  if (host_cholesky(M, C, L.data(), nullptr) != 0) {
    set_error(err, PMCG_ECHOL, __LINE__, "template data covariance is not positive definite");
    return;
  }
  for (int i = 0; i < M; i++) {
    const double *Li = &L[(size_t)i * M];
    for (int q = 0; q < P; q++) {
      double t = A[(size_t)i * P + q];
      for (int j = 0; j < i; j++) t -= Li[j] * At[(size_t)j * P + q];
      At[(size_t)i * P + q] = t / Li[i];
    }
    double t = dobs[i];
    for (int j = 0; j < i; j++) t -= Li[j] * dt[j];
    dt[i] = t / Li[i];
  }
  Plugin pl;
  pl.type = kPluginTpl;
  TplDev &t = pl.tpl;
  t.M = M; t.P = P; t.Dpar = D;
  // Gram form of the single-precision path: G = At^T At, b = At^T dt, c0 = dt.dt (FP64)
  const bool gram = P <= kGramMaxP && D <= 16;
  const int Pp = (P + 3) & ~3;
  std::vector<float> G32, b32;
  if (gram) {
    std::vector<double> Gm((size_t)P * P, 0.0), bv(P, 0.0);
    double c0 = 0.0;
    for (int i = 0; i < M; i++) {
      const double *a = &At[(size_t)i * P];
      for (int p1 = 0; p1 < P; p1++) {
        const double ap = a[p1];
        bv[p1] += ap * dt[i];
        for (int p2 = 0; p2 <= p1; p2++) Gm[(size_t)p1 * P + p2] += ap * a[p2];
      }
      c0 += dt[i] * dt[i];
    }
    G32.assign((size_t)Pp * Pp, 0.f);
    b32.assign(Pp, 0.f);
    for (int p1 = 0; p1 < P; p1++) {
      b32[p1] = (float)bv[p1];
      for (int p2 = 0; p2 <= p1; p2++) {
        G32[(size_t)p1 * Pp + p2] = (float)Gm[(size_t)p1 * P + p2];
        G32[(size_t)p2 * Pp + p1] = (float)Gm[(size_t)p1 * P + p2];
      }
    }
    t.c0 = c0;
  }
  // Tensor-core form (D <= 12): chi2 = |U phi|^2, U^T U = At'^T At', At' = At
  // with column 0 replaced by At_0 - dt (phi_0 = 1); U in FP32 [96 x 96].
  const bool tc = D <= kTplUmmaMaxD;
  std::vector<float> U32;
  if (tc) {
    std::vector<double> Gp((size_t)P * P, 0.0), Lg((size_t)P * P);
    std::vector<double> a(P);
    for (int i = 0; i < M; i++) {
      for (int q = 0; q < P; q++) a[q] = At[(size_t)i * P + q];
      a[0] -= dt[i];
      for (int p1 = 0; p1 < P; p1++)
        for (int p2 = 0; p2 <= p1; p2++) Gp[(size_t)p1 * P + p2] += a[p1] * a[p2];
    }
    for (int p1 = 0; p1 < P; p1++)
      for (int p2 = 0; p2 < p1; p2++) Gp[(size_t)p2 * P + p1] = Gp[(size_t)p1 * P + p2];
    if (host_cholesky(P, Gp.data(), Lg.data(), nullptr) != 0) {
      set_error(err, PMCG_ECHOL, __LINE__, "template Gram matrix is not positive definite (fewer data than monomials?)");
      return;
    }
    U32.assign(96 * 96, 0.f);
    for (int i = 0; i < P; i++)
      for (int j = i; j < P; j++) U32[(size_t)i * 96 + j] = (float)Lg[(size_t)j * P + i];   // U = L^T
  }
  Carver cv;
  float *dU32 = nullptr;
  for (int pass = 0; pass < 2; pass++) {
    cv.off = 0;
    t.At = cv.take<double>((size_t)M * P); t.dt = cv.take<double>(M);
    t.At32 = cv.take<float>((size_t)M * P); t.dt32 = cv.take<float>(M);
    if (gram) { t.G32 = cv.take<float>((size_t)Pp * Pp); t.b32 = cv.take<float>(Pp); }
    if (tc) { t.uimg = cv.take<unsigned char>(tpl_uimage_bytes()); dU32 = cv.take<float>(96 * 96); }
    if (pass == 0) {
      if (!CK(cudaMalloc(&t.arena, cv.off + 256), "template buffers")) return;
      cv.base = (char *)t.arena;
    }
  }
  std::vector<float> At32(At.begin(), At.end()), dt32(dt.begin(), dt.end());
  bool ok = CK(cudaMemcpy(t.At, At.data(), 8 * At.size(), cudaMemcpyHostToDevice), "template upload") &&
            CK(cudaMemcpy(t.dt, dt.data(), 8 * dt.size(), cudaMemcpyHostToDevice), "template upload") &&
            CK(cudaMemcpy(t.At32, At32.data(), 4 * At32.size(), cudaMemcpyHostToDevice), "template upload") &&
            CK(cudaMemcpy(t.dt32, dt32.data(), 4 * dt32.size(), cudaMemcpyHostToDevice), "template upload");
  if (ok && gram)
    ok = CK(cudaMemcpy(t.G32, G32.data(), 4 * G32.size(), cudaMemcpyHostToDevice), "template upload") &&
         CK(cudaMemcpy(t.b32, b32.data(), 4 * b32.size(), cudaMemcpyHostToDevice), "template upload");
  if (ok && tc)
    ok = CK(cudaMemcpy(dU32, U32.data(), 4 * U32.size(), cudaMemcpyHostToDevice), "template upload") &&
         CK(launch_tpl_uimage(dU32, t.uimg, 0), "template operand image") &&
         CK(cudaDeviceSynchronize(), "template operand image");
  if (!ok) { cudaFree(t.arena); return; }
  p->plugins.push_back(pl);
  restamp(p);
}

// Batched log-posterior over N points (one Work scratch per call).
extern "C" void pmcg_posterior_log_pdf_batch(const pmcg_posterior *p, size_t N, const double *X, double *logpost,
                                             short *flg, int on_device, int precision, void *stream, error **err) {
  (void)stream;
  if (!p || N == 0) return;
  Work w;
  if (!work_alloc(w, 1, p->npar, -1, precision ? 1 : 0, N, err)) { work_free(w); return; }
  const int D = p->npar;
  const cudaMemcpyKind in = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind out = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  bool ok = CK(cudaMemcpyAsync(w.X64, X, sizeof(double) * N * D, in, w.s), "X upload");
  if (ok && precision) ok = CK(launch_x64_to_x32(N, D, w.ldx, w.X64, w.X32, w.s), "convert");
  std::vector<short> ones(N, 1);
  ok = ok && CK(cudaMemcpyAsync(w.flg, ones.data(), sizeof(short) * N, cudaMemcpyHostToDevice, w.s), "flg");
  ok = ok && stage_logpost(w, p, err);
  ok = ok && CK(cudaMemcpyAsync(logpost, w.logpost, sizeof(double) * N, out, w.s), "logpost");
  if (ok && flg) ok = CK(cudaMemcpyAsync(flg, w.flg, sizeof(short) * N, out, w.s), "flg");
  ok = ok && CK(cudaStreamSynchronize(w.s), "posterior");
  work_free(w);
}

extern "C" double pmcg_posterior_log_pdf_void(void *post, const double *x, error **err) {
  double lp = 0.0;
  short f = 1;
  pmcg_posterior_log_pdf_batch((const pmcg_posterior *)post, 1, x, &lp, &f, 0, PMCG_FP64, nullptr, err);
  if (!f) set_error(err, PMCG_EARG, __LINE__, "likelihood error at this point");
  return lp;
}

extern "C" void pmcg_mix_log_pdf_batch(const mix_mvdens *m, size_t N, const double *X, double *logq, double *lt,
                                       int precision, error **err) {
  if (!m || N == 0) return;
  Work w;
  if (!work_alloc(w, m->ncomp, m->ndim, m->comp[0]->df, precision ? 1 : 0, N, err)) { work_free(w); return; }
  const int D = m->ndim;
  bool ok = upload_mix(w.prop, m, w.s, err);
  ok = ok && CK(cudaMemcpyAsync(w.X64, X, sizeof(double) * N * D, cudaMemcpyHostToDevice, w.s), "X upload");
  if (ok && precision) ok = CK(launch_x64_to_x32(N, D, w.ldx, w.X64, w.X32, w.s), "convert");
  ok = ok && stage_logq(w, err);
  ok = ok && CK(cudaMemcpyAsync(logq, w.logq, sizeof(double) * N, cudaMemcpyDeviceToHost, w.s), "logq");
  if (ok && lt) {
    if (precision) {
      std::vector<float> t((size_t)m->ncomp * N);
      ok = CK(cudaMemcpyAsync(t.data(), w.lt32, 4 * t.size(), cudaMemcpyDeviceToHost, w.s), "lt") &&
           CK(cudaStreamSynchronize(w.s), "lt");
      for (size_t i = 0; ok && i < t.size(); i++) lt[i] = t[i];
    } else {
      ok = CK(cudaMemcpyAsync(lt, w.lt64, 8 * (size_t)m->ncomp * N, cudaMemcpyDeviceToHost, w.s), "lt");
    }
  }
  ok = ok && CK(cudaMemcpyAsync(w.hstats, w.dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, w.s), "status") &&
       CK(cudaStreamSynchronize(w.s), "mixture log-pdf");
  if (ok && w.hstats->tc_err != 0)
    set_error(err, PMCG_ETIMEOUT, __LINE__, "tensor-core log-density: a pipeline wait expired");
  work_free(w);
}

extern "C" double mix_mvdens_log_pdf(mix_mvdens *m, const double *x, error **err) {
  double r = 0.0;
  pmcg_mix_log_pdf_batch(m, 1, x, &r, nullptr, PMCG_FP64, err);
  return r;
}
extern "C" double mix_mvdens_log_pdf_void(void *m, const double *x, error **err) {
  return mix_mvdens_log_pdf((mix_mvdens *)m, x, err);
}
extern "C" double mvdens_log_pdf(mvdens *g, const double *x, error **err) {
  mix_mvdens mm;
  double one = 1.0;
  mvdens *cp[1] = {g};
  mm.ncomp = 1; mm.ndim = g->ndim; mm.wght = &one; mm.comp = cp;
  return mix_mvdens_log_pdf(&mm, x, err);
}
extern "C" double mvdens_log_pdf_void(void *g, const double *x, error **err) {
  return mvdens_log_pdf((mvdens *)g, x, err);
}

// ===================================================================== runs
extern "C" pmcg_run *pmcg_run_create(const mix_mvdens *proposal, const pmcg_posterior *post, const parabox *pb,
                                     size_t nsamples, int precision, uint64_t seed, error **err) {
  if (!proposal || !post || nsamples == 0) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_create: null argument or zero samples");
    return nullptr;
  }
  if (post->npar != proposal->ndim || (pb && pb->ndim != proposal->ndim)) {
    set_error(err, PMCG_EDIM, __LINE__, "dimensions of proposal/posterior/box differ");
    return nullptr;
  }
  pmcg_run *r = new pmcg_run();
  if (!work_alloc(r->w, proposal->ncomp, proposal->ndim, proposal->comp[0]->df, precision ? 1 : 0, nsamples,
                  err) ||
      !upload_mix(r->w.prop, proposal, r->w.s, err, precision != 0)) {
    work_free(r->w);
    delete r;
    return nullptr;
  }
  r->post = post;
  r->seed = seed;
  if (pb) {
    r->box = true;
    r->hmin.assign(pb->min, pb->min + pb->ndim);
    r->hmax.assign(pb->max, pb->max + pb->ndim);
    if (!upload_box(r->w, pb->min, pb->max, err)) { work_free(r->w); delete r; return nullptr; }
  }
  for (int i = 0; i <= PMCG_NSTAGE; i++) cudaEventCreate(&r->ev[i]);
  return r;
}

static void drop_run_graph(pmcg_run *r) {
  if (r->gexec) cudaGraphExecDestroy(r->gexec);
  r->gexec = nullptr;
}

// Capture one single-precision iteration (parameter upload, the five stages,
// statistics download) as a graph; false leaves the run on direct launches.
static bool capture_run_graph(pmcg_run *r) {
  Work &w = r->w;
  if (!r->dpar && (cudaMalloc(&r->dpar, sizeof(pmcg_iter_params)) != cudaSuccess ||
                   cudaMallocHost(&r->hpar, sizeof(pmcg_iter_params)) != cudaSuccess))
    return false;
  error *cerr = nullptr;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(w.s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return false;
  w.launches = 0;
  bool ok = cudaMemcpyAsync(r->dpar, r->hpar, sizeof(pmcg_iter_params), cudaMemcpyHostToDevice, w.s) == cudaSuccess;
  ok = ok && stage_draw(w, r->box, r->seed, 0u, &cerr, &r->dpar->call) && stage_logq(w, &cerr) &&
       stage_logpost(w, r->post, &cerr, false) && stage_weights(w, 1.0, true, &cerr, &r->dpar->beta) &&
       stage_em(w, &cerr);
  ok = ok && cudaMemcpyAsync(w.hstats, w.dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, w.s) == cudaSuccess;
  const bool ended = cudaStreamEndCapture(w.s, &g) == cudaSuccess;
  ok = ok && ended && g && cudaGraphInstantiate(&r->gexec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (cerr) purgeError(&cerr);
  if (!ok) {
    r->gexec = nullptr;
    cudaGetLastError();  // the failed capture is not an error of the run
    return false;
  }
  r->graph_tc = tc_on(w);
  r->graph_launches = w.launches;
  return true;
}

namespace pmcg {
// An iteration in two halves: the launch (a replayed graph is queued on the
// run's stream without waiting; otherwise the stages run and their statistics
// are fetched) and the completion (wait, check, timing, revival, statistics).
static bool run_launch(pmcg_run *r, double beta, error **err) {
  Work &w = r->w;
  w.launches = 0;
  if (r->img_stale) {
    if (w.prop.bimg && !CK(launch_umma_bimage(w.prop.view(), w.prop.bimg, w.s), "operand image")) return false;
    r->img_stale = false;
  }
  const bool stages = r->timing == 1;
  if (w.prec == PMCG_MIXED && !stages && !r->graph_off) {
    if (r->gexec && r->graph_tc != tc_on(w)) drop_run_graph(r);
    if (!r->gexec && !capture_run_graph(r)) r->graph_off = true;
  }
  r->pending_graph = false;
  if (r->gexec && !stages) {
    r->hpar->beta = beta;
    r->hpar->call = r->calls;
    if (r->timing) cudaEventRecord(r->ev[0], w.s);
    const bool ok = CK(cudaGraphLaunch(r->gexec, w.s), "iteration graph");
    if (r->timing) cudaEventRecord(r->ev[PMCG_NSTAGE], w.s);
    w.launches = r->graph_launches;
    r->calls++;
    r->last_launches = w.launches;
    r->pending_graph = ok;
    return ok;
  }
  auto mark = [&](int i) { if (r->timing) cudaEventRecord(r->ev[i], w.s); };
  mark(0);
  bool ok = stage_draw(w, r->box, r->seed, r->calls, err);
  mark(1);
  ok = ok && stage_logq(w, err);
  mark(2);
  ok = ok && stage_logpost(w, r->post, err, false);
  mark(3);
  ok = ok && stage_weights(w, beta, true, err);
  mark(4);
  ok = ok && stage_em(w, err);
  mark(5);
  r->calls++;
  r->last_launches = w.launches;
  return ok && fetch_stats(w, err);
}

static bool run_finish(pmcg_run *r, pmcg_iter_stats *stats, error **err) {
  Work &w = r->w;
  const bool stages = r->timing == 1;
  if (r->pending_graph) {
    r->pending_graph = false;
    if (!CK(cudaStreamSynchronize(w.s), "iteration") || !check_stats(w, err)) return false;
  }
  if (r->timing) {
    float ms = 0.f;
    if (stages) {
      for (int i = 0; i < PMCG_NSTAGE; i++) {
        cudaEventElapsedTime(&ms, r->ev[i], r->ev[i + 1]);
        r->stage_ms[i] += ms;
      }
    } else {
      cudaEventElapsedTime(&ms, r->ev[0], r->ev[PMCG_NSTAGE]);
      r->iter_ms += ms;
    }
    r->timed++;
  }
  if (!run_revive_dead(r, err)) return false;
  if (stats) {
    const DevStats &h = *w.hstats;
    stats->ln_evidence = h.ln_evidence;
    stats->perplexity = h.perplexity;
    stats->ess = h.ess;
    stats->enc = h.enc;
    stats->logSum = h.logSum;
    stats->maxW = h.maxW;
    stats->nok = (size_t)h.nok;
    stats->ndead = h.ndead;
  }
  return true;
}
}  // namespace pmcg

// A run with an asynchronous iteration in flight accepts only pmcg_run_iterate_wait
// (and pmcg_run_free, which waits for the stream).
static bool run_in_flight(const pmcg_run *r, error **err, const char *fn) {
  if (!r->launched) return false;
  set_error(err, PMCG_EARG, __LINE__, "%s: an iteration started by pmcg_run_iterate_async was not waited for", fn);
  return true;
}

extern "C" void pmcg_run_iterate(pmcg_run *r, double beta, pmcg_iter_stats *stats, error **err) {
  if (run_in_flight(r, err, "pmcg_run_iterate")) return;
  if (run_launch(r, beta, err)) run_finish(r, stats, err);
}

extern "C" void pmcg_run_iterate_async(pmcg_run *r, double beta, error **err) {
  if (r->launched) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_iterate_async: the previous iteration was not waited for");
    return;
  }
  r->launched = true;
  r->launch_ok = run_launch(r, beta, &r->launch_err);
  if (!r->launch_ok && !r->launch_err)
    set_error(&r->launch_err, PMCG_ECUDA, __LINE__, "iteration launch failed");
  (void)err;
}

extern "C" void pmcg_run_iterate_wait(pmcg_run *r, pmcg_iter_stats *stats, error **err) {
  if (!r->launched) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_iterate_wait: no iteration was started");
    return;
  }
  r->launched = false;
  if (!r->launch_ok) {
    r->pending_graph = false;
    if (err && !*err) *err = r->launch_err;   // the launch's error chain, as a synchronous call gives it
    else purgeError(&r->launch_err);
    r->launch_err = nullptr;
    return;
  }
  run_finish(r, stats, err);
}

extern "C" void pmcg_run_get_proposal(pmcg_run *r, mix_mvdens *out, error **err) {
  if (run_in_flight(r, err, "pmcg_run_get_proposal")) return;
  Work &w = r->w;
  if (out->ncomp != w.K || out->ndim != w.D) {
    set_error(err, PMCG_EDIM, __LINE__, "output proposal shape differs");
    return;
  }
  const int K = w.K, D = w.D;
  std::vector<double> wt(K), mu((size_t)K * D), L((size_t)K * D * D);
  bool ok = CK(cudaMemcpyAsync(wt.data(), w.prop.w, 8 * K, cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(mu.data(), w.prop.mu, 8 * mu.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(L.data(), w.prop.L, 8 * L.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaStreamSynchronize(w.s), "proposal");
  if (!ok) return;
  for (int k = 0; k < K; k++) {
    out->wght[k] = wt[k];
    mvdens *c = out->comp[k];
    c->df = w.df;
    memcpy(c->mean, &mu[(size_t)k * D], 8 * D);
    memcpy(c->std, &L[(size_t)k * D * D], 8 * (size_t)D * D);
    c->chol = 1;
    double ld = 0.0;
    for (int i = 0; i < D; i++) ld += std::log(c->std[i * D + i]);
    c->det = 2.0 * ld;
  }
}

extern "C" void pmcg_run_set_proposal(pmcg_run *r, const mix_mvdens *proposal, error **err) {
  if (run_in_flight(r, err, "pmcg_run_set_proposal")) return;
  Work &w = r->w;
  if (!proposal || proposal->ncomp != w.K || proposal->ndim != w.D || proposal->comp[0]->df != w.df) {
    set_error(err, PMCG_EDIM, __LINE__, "proposal shape differs from the run's");
    return;
  }
  upload_mix(w.prop, proposal, w.s, err, w.prec != 0);
}

extern "C" void pmcg_run_set_dead_comp(pmcg_run *r, int mode, double fshift, error **err) {
  if (!r || (mode != PMCG_DEAD_BURY && mode != PMCG_DEAD_REVIVE) || !(fshift > 0.0)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_set_dead_comp: invalid mode %d or fshift %g", mode, fshift);
    return;
  }
  if (run_in_flight(r, err, "pmcg_run_set_dead_comp")) return;
  if (mode == PMCG_DEAD_REVIVE && r->hmin.empty()) {
    set_error(err, PMCG_EARG, __LINE__, "reviving components needs the run's prior box");
    return;
  }
  r->dead_mode = mode;
  r->fshift = fshift;
  r->nrevive = 1;
}

namespace pmcg {
// update_and_deal_with_dead's revive branch (exec/cosmo_pmc.c:252-275) with
// revive_comp (:205-236) and comp_shift_mean (wrappers/src/param.c:471-489).
bool run_revive_dead(pmcg_run *r, error **err) {
  if (r->dead_mode != PMCG_DEAD_REVIVE) return true;
  r->nrevive *= 2;  // every update in revive mode (:259)
  Work &w = r->w;
  if (w.hstats->ndead == 0) return true;
  const int K = w.K, D = w.D;
  std::vector<double> wt(K), mu((size_t)K * D), L((size_t)K * D * D);
  bool ok = CK(cudaMemcpyAsync(wt.data(), w.prop.w, 8 * K, cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(mu.data(), w.prop.mu, 8 * mu.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(L.data(), w.prop.L, 8 * L.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaStreamSynchronize(w.s), "proposal");
  if (!ok) return false;
  const uint32_t call = r->calls - 1;   // the call of the iteration that made this update
  const double fs = r->fshift / (double)r->nrevive;
  bool changed = false;
  for (int i = 0; i < K; i++) {
    if (!(wt[i] < 1e-12)) continue;
    int imax = -1;
    double wmax = 0.0;
    for (int j = 0; j < K; j++)
      if (wt[j] > wmax) { wmax = wt[j]; imax = j; }
    if (imax < 0) {
      set_error(err, PMCG_ENEGWEIGHT, __LINE__, "Components weights are all zero");
      return false;
    }
    // copy of the largest component, mean shifted inside the box
    std::memcpy(&L[(size_t)i * D * D], &L[(size_t)imax * D * D], sizeof(double) * D * D);
    uint32_t k = 0;
    for (int d = 0; d < D; d++) {
      const double box = r->hmax[d] - r->hmin[d];
      double m;
      do {
        if (++k > 50) {
          set_error(err, PMCG_ESTEPS, __LINE__,
                    "Could not place proposal component in box. Make sure that fshift is not too large");
          return false;
        }
        P4 c;
        c.x = 0xFFFFFFF0u; c.y = (uint32_t)i; c.z = k - 1; c.w = call;
        const P4 o = philox4x32_10(c, (uint32_t)r->seed, (uint32_t)(r->seed >> 32));
        const double u = u53(o.x, o.y);
        m = mu[(size_t)imax * D + d] + (-fs * box + 2.0 * fs * box * u);
      } while (m < r->hmin[d] || m > r->hmax[d]);
      mu[(size_t)i * D + d] = m;
    }
    wt[imax] /= 2.0;
    wt[i] = wt[imax];
    changed = true;
  }
  if (!changed) return true;
  double sum = 0.0;
  for (int i = 0; i < K; i++) sum += wt[i];
  if (!(sum > 0.0) || !std::isfinite(sum)) {
    set_error(err, PMCG_ENEGWEIGHT, __LINE__, "Sum of weight is %g", sum);
    return false;
  }
  for (int i = 0; i < K; i++) wt[i] /= sum;
  if (w.prec != 0 && !f32_range_ok(wt, mu, L, K, D, err)) return false;
  return CK(devmix_upload(w.prop, wt.data(), mu.data(), L.data(), w.s), "proposal upload") &&
         CK(cudaStreamSynchronize(w.s), "proposal upload");
}
}  // namespace pmcg

extern "C" void pmcg_run_get_sample(pmcg_run *r, pmc_simu *psim, error **err) {
  if (run_in_flight(r, err, "pmcg_run_get_sample")) return;
  Work &w = r->w;
  if (psim->ndim != w.D) { set_error(err, PMCG_EDIM, __LINE__, "sample dimension differs"); return; }
  pmc_simu_realloc(psim, w.N, err);
  if (isError(err ? *err : nullptr)) return;
  bool ok = true;
  if (w.prec) ok = CK(launch_x32_to_x64(w.N, w.D, w.ldx, w.X32, w.X64, w.s), "convert");
  ok = ok && CK(cudaMemcpyAsync(psim->X, w.X64, 8 * w.N * w.D, cudaMemcpyDeviceToHost, w.s), "X") &&
       CK(cudaMemcpyAsync(psim->weights, w.logw, 8 * w.N, cudaMemcpyDeviceToHost, w.s), "weights") &&
       CK(cudaMemcpyAsync(psim->flg, w.flg, 2 * w.N, cudaMemcpyDeviceToHost, w.s), "flg") &&
       CK(cudaMemcpyAsync(psim->indices, w.idx, 4 * w.N, cudaMemcpyDeviceToHost, w.s), "indices") &&
       CK(cudaStreamSynchronize(w.s), "sample");
  if (!ok) return;
  psim->isLog = 1;
  psim->logSum = w.hstats->logSum;
  psim->maxW = w.hstats->maxW;
  psim->nok = (size_t)w.hstats->nok;
}

extern "C" void pmcg_run_free(pmcg_run **r) {
  if (!r || !*r) return;
  if ((*r)->w.s) cudaStreamSynchronize((*r)->w.s);   // an iteration may be in flight
  purgeError(&(*r)->launch_err);
  drop_run_graph(*r);
  if ((*r)->dpar) cudaFree((*r)->dpar);
  if ((*r)->hpar) cudaFreeHost((*r)->hpar);
  for (int i = 0; i <= PMCG_NSTAGE; i++)
    if ((*r)->ev[i]) cudaEventDestroy((*r)->ev[i]);
  work_free((*r)->w);
  delete *r;
  *r = nullptr;
}

extern "C" void pmcg_run_set_timing(pmcg_run *r, int on) {
  r->timing = (on == 1 || on == 2) ? on : 0;
  for (int i = 0; i < PMCG_NSTAGE; i++) r->stage_ms[i] = 0.0;
  r->iter_ms = 0.0;
  r->timed = 0;
}

extern "C" int pmcg_run_stage_ms(pmcg_run *r, double *ms, int nstage) {
  for (int i = 0; i < nstage && i < PMCG_NSTAGE; i++) ms[i] = r->timing == 1 ? r->stage_ms[i] : 0.0;
  return r->timing == 1 ? r->timed : 0;
}

extern "C" int pmcg_run_iteration_ms(pmcg_run *r, double *ms) {
  double t = r->iter_ms;
  if (r->timing == 1)
    for (int i = 0; i < PMCG_NSTAGE; i++) t += r->stage_ms[i];
  if (ms) *ms = t;
  return r->timing ? r->timed : 0;
}

extern "C" double pmcg_run_time_stage(pmcg_run *r, int stage, int reps, error **err) {
  if (run_in_flight(r, err, "pmcg_run_time_stage")) return -1.0;
  Work &w = r->w;
  if ((stage != 1 && stage != 2) || reps < 1 || r->calls == 0) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_time_stage: stage 1 or 2 of a run that has iterated, reps >= 1");
    return -1.0;
  }
  bool ok = true;
  if (!CK(cudaEventRecord(r->ev[0], w.s), "event")) return -1.0;
  for (int i = 0; i < reps && ok; i++) ok = (stage == 1) ? stage_logq(w, err) : stage_logpost(w, r->post, err, false);
  if (!ok || !CK(cudaEventRecord(r->ev[1], w.s), "event") ||
      !CK(cudaMemcpyAsync(w.hstats, w.dstats, sizeof(DevStats), cudaMemcpyDeviceToHost, w.s), "status") ||
      !CK(cudaStreamSynchronize(w.s), "stage timing"))
    return -1.0;
  if (w.hstats->tc_err != 0) {
    set_error(err, PMCG_ETIMEOUT, __LINE__, "tensor-core log-density: a pipeline wait expired");
    return -1.0;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
  return (double)ms / reps;
}

extern "C" int pmcg_run_last_launches(const pmcg_run *r) { return r->last_launches; }

extern "C" int pmcg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

extern "C" void pmcg_device_synchronize(error **err) { CK(cudaDeviceSynchronize(), "device synchronize"); }

// ===================================================================== drop-in
namespace pmcg {

static int g_dropin_precision = PMCG_FP64;

// Ranges of the drop-in draw copied to the host while the next range draws.
constexpr int kDrawChunks = 8;

struct SimMirror {
  Work w;
  void *pscratch = nullptr;  // post-processing scratch (allocated on first use)
  cudaStream_t cs = nullptr;             // device-to-host copies of the sample
  cudaEvent_t ev[kDrawChunks] = {};      // range drawn and converted
  cudaEvent_t drawn = nullptr;           // the draw done and its flags saved (before the look-ahead)
  short *flg0 = nullptr;                 // the draw's flags, copied to the host behind X
  int *dnok = nullptr, *hnok = nullptr;  // the draw's count of samples in the box (device, pinned host)
  bool x_valid = false;    // device X/flg/indices/counts match the host sample
  bool lt_valid = false;   // logq/lt/Q valid for (X, snapshot proposal)
  bool w_valid = false;    // logw and the device statistics valid
  // Look-ahead: the posterior of the last weight step (and its stamp); after a
  // draw its log-posterior is evaluated while X travels to the host, and
  // lp_valid says w.logpost holds it (w.flg then carries its likelihood flags).
  const pmcg_posterior *post = nullptr;
  uint64_t post_stamp = 0;
  bool lp_valid = false;
  std::vector<double> snap_w, snap_mu, snap_L;
  // the update's download buffers: swapped with the snapshot after each update,
  // so they are allocated (and their pages touched) once, not every iteration
  std::vector<double> upd_w, upd_mu, upd_L;
  double *mom = nullptr;   // scratch of the weighted moments (allocated on first use)
  // Speculation (single precision, sample copied in ranges): after the
  // look-ahead, while X still travels to the host, the weight step for the
  // beta of the last two weight steps (when they agree), the normalisation and
  // the EM update run ahead, the update into a second proposal (`spec_mix`, with
  // its own statistics `spec_st`). The calls that follow use these results when
  // their arguments match, else compute as usual; the same kernels on the same
  // inputs, so the same values. spec: 0 none, 1 ready after the draw, 2 after
  // a matching weight step, 3 after the normalisation; -1: started and not
  // finished (the flags may have changed).
  DevMix spec_mix;
  DevStats *spec_st = nullptr;
  short *flg1 = nullptr;   // the flags as the look-ahead left them (restored on a miss)
  int spec = 0;
  bool flg_dirty = false;  // the speculation changed w.flg; flg1 holds the flags before it
  double spec_beta = 0.0;
  double beta_last = NAN, beta_prev = NAN;
};

static void mirror_delete(SimMirror *m) {
  if (m->cs) cudaStreamSynchronize(m->cs);
  if (m->w.s) cudaStreamSynchronize(m->w.s);
  for (cudaEvent_t &e : m->ev)
    if (e) cudaEventDestroy(e);
  if (m->drawn) cudaEventDestroy(m->drawn);
  if (m->flg0) cudaFree(m->flg0);
  if (m->dnok) cudaFree(m->dnok);
  if (m->hnok) cudaFreeHost(m->hnok);
  if (m->flg1) cudaFree(m->flg1);
  if (m->spec_st) cudaFree(m->spec_st);
  devmix_free(m->spec_mix);
  if (m->cs) cudaStreamDestroy(m->cs);
  work_free(m->w);
  if (m->mom) cudaFree(m->mom);
  if (m->pscratch) cudaFree(m->pscratch);
  delete m;
}

static std::mutex g_mu;
static std::unordered_map<const pmc_simu *, SimMirror *> g_sims;
// Per-sample settings of the drop-in entry points (-1: the process default).
struct SimSettings {
  int prec = -1, tc = -1;
};
static std::unordered_map<const pmc_simu *, SimSettings> g_sim_set;

static SimMirror *mirror_for(const pmc_simu *psim, int K, int D, int df, error **err) {
  std::lock_guard<std::mutex> lk(g_mu);
  SimMirror *&m = g_sims[psim];
  const auto set = g_sim_set.find(psim);
  const SimSettings ss = set == g_sim_set.end() ? SimSettings() : set->second;
  const int prec = ss.prec >= 0 ? ss.prec : g_dropin_precision;
  if (m && (m->w.K != K || m->w.D != D || m->w.df != df || m->w.N != psim->nsamples || m->w.prec != prec)) {
    mirror_delete(m);
    m = nullptr;
  }
  if (!m) {
    m = new SimMirror();
    bool ok = work_alloc(m->w, K, D, df, prec, psim->nsamples, err) &&
              CK(cudaStreamCreateWithFlags(&m->cs, cudaStreamNonBlocking), "copy stream");
    for (cudaEvent_t &e : m->ev) ok = ok && CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    ok = ok && CK(cudaEventCreateWithFlags(&m->drawn, cudaEventDisableTiming), "event") &&
         CK(cudaMalloc(&m->flg0, sizeof(short) * psim->nsamples + 16), "flag copy") &&
         CK(cudaMalloc(&m->dnok, sizeof(int)), "count") && CK(cudaMallocHost(&m->hnok, sizeof(int)), "count");
    if (!ok) {
      mirror_delete(m);
      m = nullptr;
      g_sims.erase(psim);
      return nullptr;
    }
  }
  m->w.tc = ss.tc;
  return m;
}

static SimMirror *find_mirror(const pmc_simu *psim) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_sims.find(psim);
  return it == g_sims.end() ? nullptr : it->second;
}

// Mirror for the weight-only entry points: any existing mirror of this
// sample size is reused; otherwise a one-component mirror is made.
static SimMirror *mirror_any(const pmc_simu *psim, error **err) {
  SimMirror *m = find_mirror(psim);
  if (m && m->w.N == psim->nsamples) return m;
  return mirror_for(psim, 1, psim->ndim, -1, err);
}

void forget_simu(const pmc_simu *p) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_sim_set.erase(p);
  auto it = g_sims.find(p);
  if (it == g_sims.end()) return;
  mirror_delete(it->second);
  g_sims.erase(it);
}

void forget_mix(const mix_mvdens *) {}

void forget_posterior(const pmcg_posterior *p) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &kv : g_sims)
    if (kv.second->post == p) {
      kv.second->post = nullptr;
      kv.second->lp_valid = false;
    }
}

// The host proposal equals the mirror's snapshot (Cholesky-form components
// compared in place, without flattening): bitwise on the means and the lower
// triangles, by value on the weights.
static bool same_as_snapshot(const SimMirror *m, const mix_mvdens *p) {
  const int K = p->ncomp, D = p->ndim;
  if ((int)m->snap_w.size() != K || m->snap_mu.size() != (size_t)K * D || m->snap_L.size() != (size_t)K * D * D)
    return false;
  for (int k = 0; k < K; k++) {
    const mvdens *c = p->comp[k];
    if (c->ndim != D || !c->chol || p->wght[k] != m->snap_w[k]) return false;
    if (memcmp(c->mean, &m->snap_mu[(size_t)k * D], sizeof(double) * D) != 0) return false;
    const double *Ls = &m->snap_L[(size_t)k * D * D];
    for (int i = 0; i < D; i++)
      if (memcmp(c->std + (size_t)i * D, Ls + (size_t)i * D, sizeof(double) * (i + 1)) != 0) return false;
  }
  return true;
}

// Upload the proposal when it differs from the mirror's snapshot.
static bool sync_proposal(SimMirror *m, const mix_mvdens *prop, error **err) {
  if (same_as_snapshot(m, prop)) return true;
  std::vector<double> w, mu, L;
  if (!flatten_mix(prop, w, mu, L, err)) return false;
  if (w == m->snap_w && mu == m->snap_mu && L == m->snap_L) return true;
  m->spec = 0;
  if (!CK(devmix_upload(m->w.prop, w.data(), mu.data(), L.data(), m->w.s), "proposal upload")) return false;
  m->snap_w.swap(w);
  m->snap_mu.swap(mu);
  m->snap_L.swap(L);
  m->lt_valid = false;
  return true;
}

// Make the device sample match the host one (after a host-side rewrite).
static bool sync_sample(SimMirror *m, const pmc_simu *psim, error **err) {
  if (m->x_valid) return true;
  m->spec = 0;
  m->flg_dirty = false;   // the host flags are uploaded below
  Work &w = m->w;
  bool ok = CK(cudaMemcpyAsync(w.X64, psim->X, 8 * w.N * w.D, cudaMemcpyHostToDevice, w.s), "X upload") &&
            CK(cudaMemcpyAsync(w.flg, psim->flg, 2 * w.N, cudaMemcpyHostToDevice, w.s), "flg upload") &&
            CK(cudaMemcpyAsync(w.idx, psim->indices, 4 * w.N, cudaMemcpyHostToDevice, w.s), "indices upload") &&
            CK(launch_counts(w.N, w.K, w.idx, w.counts, w.s), "counts");
  if (ok && w.prec) ok = CK(launch_x64_to_x32(w.N, w.D, w.ldx, w.X64, w.X32, w.s), "convert");
  if (!ok) return false;
  m->x_valid = true;
  m->lt_valid = false;
  m->w_valid = false;
  m->lp_valid = false;
  return true;
}

// Make the device log-weights and statistics match the host weights.
static bool restore_flags(SimMirror *m, error **err);

static bool sync_weights(SimMirror *m, const pmc_simu *psim, error **err) {
  if (m->w_valid) return true;
  m->spec = 0;
  if (!restore_flags(m, err)) return false;
  Work &w = m->w;
  m->lp_valid = false;  // w.logpost is overwritten below
  bool ok = CK(cudaMemcpyAsync(w.logpost, psim->weights, 8 * w.N, cudaMemcpyHostToDevice, w.s), "weights upload");
  if (ok && !psim->isLog) ok = CK(launch_log_weights(w.N, w.logpost, w.flg, w.s), "log weights");
  ok = ok && stage_weights(w, 1.0, false, err) && fetch_stats(w, err);
  if (ok) m->w_valid = true;
  return ok;
}

}  // namespace pmcg

extern "C" void pmcg_set_dropin_precision(int precision) { g_dropin_precision = precision ? PMCG_MIXED : PMCG_FP64; }

extern "C" int pmcg_set_tensor_cores(int on) {
  const int prev = g_use_tensor_cores;
  g_use_tensor_cores = on ? 1 : 0;
  return prev;
}

extern "C" int pmcg_run_set_tensor_cores(pmcg_run *r, int on, error **err) {
  if (!r || on < -1 || on > 1) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_run_set_tensor_cores: on is 1, 0 or -1");
    return -2;
  }
  if (run_in_flight(r, err, "pmcg_run_set_tensor_cores")) return -2;
  const int prev = r->w.tc;
  r->w.tc = on;
  return prev;
}

extern "C" void pmcg_simu_set_precision(const pmc_simu *psim, int precision, error **err) {
  if (!psim || (precision != -1 && precision != PMCG_FP64 && precision != PMCG_MIXED)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_simu_set_precision: PMCG_FP64, PMCG_MIXED or -1");
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  g_sim_set[psim].prec = precision;   // a mirror of another precision is replaced at its next use
}

extern "C" void pmcg_simu_set_tensor_cores(const pmc_simu *psim, int on, error **err) {
  if (!psim || on < -1 || on > 1) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_simu_set_tensor_cores: on is 1, 0 or -1");
    return;
  }
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_sim_set[psim].tc = on;
  }
  // whatever was evaluated ahead with the other kernel is evaluated again
  pmcg_simu_host_modified(const_cast<pmc_simu *>(psim));
}

extern "C" void pmcg_simu_host_modified(pmc_simu *psim) {
  SimMirror *m = find_mirror(psim);
  if (m) {
    m->x_valid = m->lt_valid = m->w_valid = m->lp_valid = false;
    m->spec = 0;
  }
}

namespace pmcg {
// The speculative weight step, normalisation and EM update (see SimMirror).
static bool speculate(SimMirror *m, error **err) {
  Work &w = m->w;
  // buffers on first use (each once; a failed allocation is retried next time)
  if (!m->spec_mix.arena && !CK(devmix_alloc(m->spec_mix, w.K, w.D, w.df), "speculative proposal")) {
    devmix_free(m->spec_mix);
    return false;
  }
  if (!m->spec_st && !CK(cudaMalloc(&m->spec_st, sizeof(DevStats)), "speculative statistics")) {
    m->spec_st = nullptr;
    return false;
  }
  if (!m->flg1 && !CK(cudaMalloc(&m->flg1, sizeof(short) * w.N + 16), "flag copy")) {
    m->flg1 = nullptr;
    return false;
  }
  if (!CK(cudaMemcpyAsync(m->flg1, w.flg, 2 * w.N, cudaMemcpyDeviceToDevice, w.s), "flags")) return false;
  m->flg_dirty = true;  // the flags may change from here on: unless the results are used, they are restored
  m->spec = -1;
  m->spec_mix.cst = w.prop.cst;
  if (!stage_weights(w, m->beta_last, true, err) ||
      !CK(launch_normalise(w.N, w.logw, w.flg, w.dstats, w.wbar, w.s), "normalise") ||
      !CK(cudaMemcpyAsync(m->spec_st, w.dstats, sizeof(DevStats), cudaMemcpyDeviceToDevice, w.s), "statistics") ||
      !CK(cudaMemcpyAsync(m->spec_mix.arena, w.prop.arena, devmix_bytes(w.K, w.D), cudaMemcpyDeviceToDevice, w.s),
          "proposal") ||
      !stage_em_into(w, m->spec_mix, m->spec_st, err))
    return false;
  m->spec = 1;
  m->spec_beta = m->beta_last;
  return true;
}

// The flags as the look-ahead left them, when a speculation changed them and
// its results are not used.
static bool restore_flags(SimMirror *m, error **err) {
  if (!m->flg_dirty) return true;
  m->flg_dirty = false;
  return CK(cudaMemcpyAsync(m->w.flg, m->flg1, 2 * m->w.N, cudaMemcpyDeviceToDevice, m->w.s), "flags");
}
}  // namespace pmcg

extern "C" size_t simulate_mix_mvdens(pmc_simu *psim, mix_mvdens *proposal, void *rng, parabox *pb,
                                      error **err) {
  if (!psim || !proposal || !rng || proposal->ndim != psim->ndim || (pb && pb->ndim != psim->ndim)) {
    set_error(err, PMCG_EARG, __LINE__, "simulate_mix_mvdens: invalid arguments");
    return 0;
  }
  uint64_t rseed = 0;
  uint32_t *rcalls = nullptr;
  if (!rng_stream(rng, &rseed, &rcalls, err)) return 0;
  SimMirror *m = mirror_for(psim, proposal->ncomp, proposal->ndim, proposal->comp[0]->df, err);
  if (!m) return 0;
  Work &w = m->w;
  if (!sync_proposal(m, proposal, err)) return 0;
  if (pb && !upload_box(w, pb->min, pb->max, err)) return 0;
  // The host-bound FP64 sample is the largest transfer of the drop-in step: in
  // the single-precision path the draw runs in kDrawChunks sample ranges, each
  // converted and copied to the host (copy stream) while the next one draws.
  const int C = (w.prec && w.N >= (size_t)kDrawChunks * 4096) ? kDrawChunks : 1;
  const bool box = pb != nullptr;
  bool ok = true;
  if (w.prec == 1 && C > 1) {
    w.launches += 3 * C;
    ok = CK(cudaMemsetAsync(w.counts, 0, sizeof(int) * w.K, w.s), "counts");
    for (int c = 0; ok && c < C; c++) {
      const size_t n0 = w.N * c / C, n1 = w.N * (c + 1) / C;
      ok = CK(launch_draw_grouped_range(w.prop.view(), w.N, n0, n1, rseed, *rcalls, box ? w.bmin : nullptr,
                                        box ? w.bmax : nullptr, w.X32, w.idx, w.flg, w.counts, w.perm, w.cursor,
                                        w.s),
              "draw kernels") &&
           CK(launch_x32_to_x64(n1 - n0, w.D, w.ldx, w.X32 + n0 * w.ldx, w.X64 + n0 * w.D, w.s), "convert") &&
           CK(cudaEventRecord(m->ev[c], w.s), "event") && CK(cudaStreamWaitEvent(m->cs, m->ev[c], 0), "wait") &&
           CK(cudaMemcpyAsync(psim->X + n0 * w.D, w.X64 + n0 * w.D, 8 * (n1 - n0) * w.D, cudaMemcpyDeviceToHost,
                              m->cs),
              "X");
    }
  } else {
    ok = stage_draw(w, box, rseed, *rcalls, err);
    if (ok && w.prec) ok = CK(launch_x32_to_x64(w.N, w.D, w.ldx, w.X32, w.X64, w.s), "convert");
    ok = ok && CK(cudaEventRecord(m->ev[0], w.s), "event") && CK(cudaStreamWaitEvent(m->cs, m->ev[0], 0), "wait") &&
         CK(cudaMemcpyAsync(psim->X, w.X64, 8 * w.N * w.D, cudaMemcpyDeviceToHost, m->cs), "X");
  }
  // The draw's flags are saved on the device (the look-ahead below may flag
  // samples by likelihood); indices and flags follow X on the copy stream, so
  // the look-ahead does not queue behind the host copies.
  ok = ok && CK(cudaMemcpyAsync(m->flg0, w.flg, 2 * w.N, cudaMemcpyDeviceToDevice, w.s), "flags") &&
       CK(launch_count_flags(w.N, m->flg0, m->dnok, w.s), "count") &&
       CK(cudaEventRecord(m->drawn, w.s), "event") && CK(cudaStreamWaitEvent(m->cs, m->drawn, 0), "wait") &&
       CK(cudaMemcpyAsync(psim->indices, w.idx, 4 * w.N, cudaMemcpyDeviceToHost, m->cs), "indices") &&
       CK(cudaMemcpyAsync(psim->flg, m->flg0, 2 * w.N, cudaMemcpyDeviceToHost, m->cs), "flg") &&
       CK(cudaMemcpyAsync(m->hnok, m->dnok, sizeof(int), cudaMemcpyDeviceToHost, m->cs), "count");
  // Look-ahead while X travels to the host: the weight step that follows a draw
  // needs log q under this proposal and, most often, the log-posterior of the
  // posterior it used last time; both are pure functions of X, queued after
  // the draw's flags are saved and not waited for here. The weight step keeps
  // what matches its arguments and recomputes the rest.
  bool lt = false, lp = false;
  m->spec = 0;
  if (ok) {
    error *lerr = nullptr;
    lt = stage_logq(w, &lerr);
    if (lt && m->post && m->post->stamp == m->post_stamp) lp = stage_logpost(w, m->post, &lerr, false);
    // the rest of the iteration, for the beta of the last two weight steps
    if (lt && lp && C > 1 && m->beta_last == m->beta_prev && std::isfinite(m->beta_last)) speculate(m, &lerr);
    if (lerr) purgeError(&lerr);
  }
  const bool copied = CK(cudaStreamSynchronize(m->cs), "sample copy");  // even after a failure
  ok = ok && copied;
  const size_t nok = ok ? (size_t)*m->hnok : 0;
  (*rcalls)++;
  if (!ok) {
    cudaStreamSynchronize(w.s);
    return 0;
  }
  m->x_valid = true;
  m->lt_valid = lt;
  m->lp_valid = lp;
  m->w_valid = false;
  psim->isLog = 1;
  return nok;
}

extern "C" size_t generic_get_importance_weight_and_deduced_verb(pmc_simu *psim, mix_mvdens *proposal,
                                                                 logpdf_fn *q, logpdf_fn *post,
                                                                 retrieve_ded_fn *ded, void *extra, double beta,
                                                                 int quiet, error **err) {
  (void)ded;
  (void)quiet;
  // the caller's own posterior callback with a registered extra pointer (the
  // reference passes posterior_log_pdf_common_void and &config->base), or the
  // library's callback with the device posterior itself
  const pmcg_posterior *p = extra ? registered_posterior(extra) : nullptr;
  if (!p && post == pmcg_posterior_log_pdf_void) p = (const pmcg_posterior *)extra;
  if (q != mix_mvdens_log_pdf_void || !p) {
    set_error(err, PMCG_EUNSUPPORTED, __LINE__,
              "the device weight step needs q = mix_mvdens_log_pdf_void and either post = "
              "pmcg_posterior_log_pdf_void with extra = pmcg_posterior*, or an extra pointer registered with "
              "pmcg_register_posterior");
    return 0;
  }
  SimMirror *m = mirror_for(psim, proposal->ncomp, proposal->ndim, proposal->comp[0]->df, err);
  if (!m) return 0;
  Work &w = m->w;
  if (!sync_sample(m, psim, err) || !sync_proposal(m, proposal, err)) return 0;
  bool ok = m->lt_valid || stage_logq(w, err);
  const bool lp_hit = m->lp_valid && m->post == p && m->post_stamp == p->stamp;
  const bool spec_hit = ok && lp_hit && m->spec == 1 && beta == m->spec_beta;
  if (spec_hit) m->flg_dirty = false;   // the speculation's flags are this weight step's
  else ok = ok && restore_flags(m, err);
  m->spec = spec_hit ? 2 : 0;
  if (ok && !lp_hit) {
    // a look-ahead for another posterior flagged samples by its likelihood:
    // the draw's flags come back first
    if (m->lp_valid) ok = CK(cudaMemcpyAsync(w.flg, m->flg0, 2 * w.N, cudaMemcpyDeviceToDevice, w.s), "flags");
    ok = ok && stage_logpost(w, p, err, false);
  }
  m->lp_valid = false;
  m->beta_prev = m->beta_last;
  m->beta_last = beta;
  if (!spec_hit) ok = ok && stage_weights(w, beta, true, err);
  ok = ok && CK(cudaMemcpyAsync(psim->weights, w.logw, 8 * w.N, cudaMemcpyDeviceToHost, w.s), "weights") &&
       CK(cudaMemcpyAsync(psim->flg, w.flg, 2 * w.N, cudaMemcpyDeviceToHost, w.s), "flg");
  if (!ok) return 0;
  if (!fetch_stats(w, err)) return 0;
  m->lt_valid = true;
  m->w_valid = true;
  m->post = p;
  m->post_stamp = p->stamp;
  psim->isLog = 1;
  psim->logSum = w.hstats->logSum;
  psim->maxW = w.hstats->maxW;
  psim->nok = (size_t)w.hstats->nok;
  return psim->nok;
}

extern "C" double normalize_importance_weight(pmc_simu *psim, error **err) {
  SimMirror *m = mirror_any(psim, err);
  if (!m) return 0.0;
  Work &w = m->w;
  if (!m->x_valid) {
    m->spec = 0;
    m->flg_dirty = false;
    if (!CK(cudaMemcpyAsync(w.flg, psim->flg, 2 * w.N, cudaMemcpyHostToDevice, w.s), "flg upload")) return 0.0;
  }
  if (!sync_weights(m, psim, err)) return 0.0;
  const bool spec_hit = m->spec == 2;  // normalised ahead from the same weights
  m->spec = spec_hit ? 3 : 0;
  bool ok = (spec_hit || CK(launch_normalise(w.N, w.logw, w.flg, w.dstats, w.wbar, w.s), "normalise")) &&
            CK(cudaMemcpyAsync(psim->weights, w.wbar, 8 * w.N, cudaMemcpyDeviceToHost, w.s), "weights") &&
            CK(cudaStreamSynchronize(w.s), "normalise");
  if (!ok) return 0.0;
  psim->isLog = 0;
  psim->logSum = w.hstats->logSum;
  psim->maxW = w.hstats->maxW;
  return psim->logSum;
}

// clip_weights (exec/cosmo_pmc.c:395-399; the manual: the nclipw points with
// the largest weights are not considered in subsequent calculations of moments,
// perplexity, evidence, Manual/manual.tex:636-642, 2105-2106). pmclib's routine
// is absent, so the semantics are pinned here: the nclipw largest weights among
// counted samples (ties to the lower index) get flg = 0, chosen on the device
// by a stable sort; a normalised sample (isLog = 0) is renormalised over the
// samples kept (logSum, maxW updated), a log-weight sample keeps its weights.
extern "C" void clip_weights(pmc_simu *psim, int nclipw, FILE *out, error **err) {
  if (!psim || nclipw < 0) {
    set_error(err, PMCG_EARG, __LINE__, "clip_weights: invalid arguments");
    return;
  }
  if (nclipw == 0 || psim->nsamples == 0) return;
  SimMirror *m = mirror_any(psim, err);
  if (!m) return;
  Work &w = m->w;
  m->spec = 0;  // the weights change: an update made ahead no longer applies
  if (!m->x_valid) m->flg_dirty = false;
  if (!m->x_valid && !CK(cudaMemcpyAsync(w.flg, psim->flg, 2 * w.N, cudaMemcpyHostToDevice, w.s), "flg upload"))
    return;
  if (!sync_weights(m, psim, err)) return;
  if (!m->pscratch &&
      !CK(cudaMalloc(&m->pscratch, post_scratch_bytes(w.N) + sizeof(double) * (8 * (size_t)w.D + 64)),
          "post-processing scratch"))
    return;
  int *dcount = reinterpret_cast<int *>(reinterpret_cast<char *>(m->pscratch) + post_scratch_bytes(w.N));
  int nclip = 0;
  bool ok = CK(launch_clip_largest(w.N, w.logw, w.flg, nclipw, m->pscratch, dcount, w.s), "clip") &&
            CK(cudaMemcpyAsync(&nclip, dcount, sizeof(int), cudaMemcpyDeviceToHost, w.s), "clip count") &&
            stage_weights(w, 1.0, false, err) && fetch_stats(w, err) &&
            CK(cudaMemcpyAsync(psim->flg, w.flg, 2 * w.N, cudaMemcpyDeviceToHost, w.s), "flags");
  if (ok && !psim->isLog)
    ok = CK(launch_normalise(w.N, w.logw, w.flg, w.dstats, w.wbar, w.s), "normalise") &&
         CK(cudaMemcpyAsync(psim->weights, w.wbar, 8 * w.N, cudaMemcpyDeviceToHost, w.s), "weights");
  ok = ok && CK(cudaStreamSynchronize(w.s), "clip");
  if (!ok) return;
  if (!psim->isLog) psim->logSum = w.hstats->logSum;
  psim->maxW = w.hstats->maxW;
  if (out) fprintf(out, "clip_weights: %d of the largest weights discarded\n", nclip);
}

// Replaces every sample's weight by its log-posterior, as exec/importance_sample.c:26-91
// does point by point: flg = 1, or 0 outside the posterior's prior box or on a
// likelihood error; isLog = 1; maxW. Returns the number of counted samples.
extern "C" size_t importance_sample(pmc_simu *psim, const pmcg_posterior *post, int quiet, error **err) {
  (void)quiet;
  if (!psim || !post || psim->nsamples == 0) {
    set_error(err, PMCG_EARG, __LINE__, "importance_sample: null sample or posterior");
    return 0;
  }
  if (post->npar != psim->ndim) {
    set_error(err, PMCG_EDIM, __LINE__, "posterior has %d parameters, the sample %d", post->npar, psim->ndim);
    return 0;
  }
  const int D = psim->ndim;
  const bool box = !post->min.empty();
  for (size_t n = 0; n < psim->nsamples; n++) {
    short in = 1;
    if (box)
      for (int i = 0; i < D; i++) {
        const double x = psim->X[n * D + i];
        if (!(x >= post->min[i] && x <= post->max[i])) { in = 0; break; }
      }
    psim->flg[n] = in;
  }
  pmcg_simu_host_modified(psim);
  SimMirror *m = mirror_any(psim, err);
  if (!m) return 0;
  Work &w = m->w;
  m->spec = 0;
  bool ok = sync_sample(m, psim, err) && restore_flags(m, err) && stage_logpost(w, post, err) &&
            CK(cudaMemcpyAsync(psim->weights, w.logpost, 8 * w.N, cudaMemcpyDeviceToHost, w.s), "log posterior") &&
            CK(cudaMemcpyAsync(psim->flg, w.flg, 2 * w.N, cudaMemcpyDeviceToHost, w.s), "flg") &&
            CK(cudaStreamSynchronize(w.s), "importance sample");
  if (!ok) return 0;
  m->lt_valid = m->w_valid = m->lp_valid = false;
  size_t count = 0;
  double mw = -INFINITY;
  for (size_t n = 0; n < psim->nsamples; n++) {
    if (!psim->flg[n] || !std::isfinite(psim->weights[n])) { psim->flg[n] = 0; continue; }
    count++;
    if (psim->weights[n] > mw) mw = psim->weights[n];
  }
  psim->isLog = 1;
  psim->maxW = mw;
  psim->nok = count;
  m->x_valid = false;  // flags were rewritten on the host
  return count;
}

// Weighted mean [ndim] and covariance [ndim x ndim] of the sample with its
// (normalised) weights, on the device (the means and covariances of the
// reference's post-processing, exec/exec_helper.c:63-349).
extern "C" void pmcg_weighted_moments(pmc_simu *psim, double *mean, double *cov, error **err) {
  if (!psim || !mean || !cov) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_weighted_moments: null argument");
    return;
  }
  SimMirror *m = mirror_any(psim, err);
  if (!m) return;
  Work &w = m->w;
  const int D = w.D;
  if (!sync_sample(m, psim, err) || !sync_weights(m, psim, err)) return;
  if (!m->mom && !CK(cudaMalloc(&m->mom, sizeof(double) * (moments_scratch_doubles(D) + D + (size_t)D * D)),
                     "moments scratch"))
    return;
  double *dmean = m->mom + moments_scratch_doubles(D), *dcov = dmean + D;
  bool ok = CK(launch_normalise(w.N, w.logw, w.flg, w.dstats, w.wbar, w.s), "normalise") &&
            CK(launch_moments(w.N, D, w.X64, w.wbar, w.flg, m->mom, dmean, dcov, w.s), "moments") &&
            CK(cudaMemcpyAsync(mean, dmean, sizeof(double) * D, cudaMemcpyDeviceToHost, w.s), "mean") &&
            CK(cudaMemcpyAsync(cov, dcov, sizeof(double) * D * D, cudaMemcpyDeviceToHost, w.s), "covariance") &&
            CK(cudaStreamSynchronize(w.s), "moments");
  (void)ok;
}

// Normalised weights of the sample on the device (wbar), with the post-processing
// scratch; false on failure (err set).
static bool post_setup(SimMirror *m, pmc_simu *psim, error **err) {
  Work &w = m->w;
  if (!sync_sample(m, psim, err) || !sync_weights(m, psim, err)) return false;
  if (!m->pscratch &&
      !CK(cudaMalloc(&m->pscratch, post_scratch_bytes(w.N) + sizeof(double) * (8 * (size_t)w.D + 64)),
          "post-processing scratch"))
    return false;
  return CK(launch_normalise(w.N, w.logw, w.flg, w.dstats, w.wbar, w.s), "normalise");
}

extern "C" void pmcg_weighted_summary(pmc_simu *psim, int use_median, double *center, double *sigma, error **err) {
  if (!psim || !center || !sigma) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_weighted_summary: null argument");
    return;
  }
  SimMirror *m = mirror_any(psim, err);
  if (!m || !post_setup(m, psim, err)) return;
  Work &w = m->w;
  const int D = w.D;
  if (!m->mom && !CK(cudaMalloc(&m->mom, sizeof(double) * (moments_scratch_doubles(D) + D + (size_t)D * D)),
                     "moments scratch"))
    return;
  double *dmean = m->mom + moments_scratch_doubles(D), *dcov = dmean + D;
  // outputs after the sort scratch: centre [D], limits [6D], status [D] (ints)
  char *tail = reinterpret_cast<char *>(m->pscratch) + post_scratch_bytes(w.N);
  double *dc = reinterpret_cast<double *>(tail), *ds = dc + D;
  int *dst = reinterpret_cast<int *>(ds + 6 * D);
  std::vector<int> st(D);
  bool ok = CK(launch_moments(w.N, D, w.X64, w.wbar, w.flg, m->mom, dmean, dcov, w.s), "moments") &&
            CK(launch_post_summary(w.N, D, w.X64, w.wbar, w.flg, dmean, use_median, m->pscratch, dc, ds, dst, w.s),
               "summary") &&
            CK(cudaMemcpyAsync(center, dc, sizeof(double) * D, cudaMemcpyDeviceToHost, w.s), "centre") &&
            CK(cudaMemcpyAsync(sigma, ds, sizeof(double) * 6 * D, cudaMemcpyDeviceToHost, w.s), "limits") &&
            CK(cudaMemcpyAsync(st.data(), dst, sizeof(int) * D, cudaMemcpyDeviceToHost, w.s), "status") &&
            CK(cudaStreamSynchronize(w.s), "summary");
  if (!ok) return;
  for (int a = 0; a < D; a++)
    if (st[a] != 0) {
      set_error(err, PMCG_EARG, __LINE__,
                st[a] == 1 ? "parameter %d: no counted sample" : "parameter %d: the weights do not reach 1/2", a);
      return;
    }
}

extern "C" void pmcg_weighted_hist1d(pmc_simu *psim, int nbin, const double *min, const double *max, double *hist,
                                     error **err) {
  if (!psim || !min || !max || !hist || nbin < 1) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_weighted_hist1d: invalid arguments");
    return;
  }
  for (int a = 0; a < psim->ndim; a++)
    if (!(max[a] > min[a])) {
      set_error(err, PMCG_EARG, __LINE__, "histogram range of parameter %d is empty", a);
      return;
    }
  SimMirror *m = mirror_any(psim, err);
  if (!m || !post_setup(m, psim, err)) return;
  Work &w = m->w;
  double *dh = nullptr;
  if (!CK(cudaMallocAsync(&dh, sizeof(double) * (size_t)nbin * w.D, w.s), "histogram")) return;
  bool ok = CK(launch_post_hist1d(w.N, w.D, w.X64, w.wbar, w.flg, nbin, min, max, (double)w.N, m->pscratch, dh, w.s),
               "histograms") &&
            CK(cudaMemcpyAsync(hist, dh, sizeof(double) * (size_t)nbin * w.D, cudaMemcpyDeviceToHost, w.s),
               "histograms");
  cudaFreeAsync(dh, w.s);
  ok = CK(cudaStreamSynchronize(w.s), "histograms") && ok;
  (void)ok;
}

extern "C" void pmcg_weighted_hist2d(pmc_simu *psim, int nbin, int p, int q, const double *min, const double *max,
                                     double *hist, error **err) {
  if (!psim || !min || !max || !hist || nbin < 1 || p < 0 || q < 0 || p >= psim->ndim || q >= psim->ndim ||
      (long long)nbin * nbin >= (1ll << 31)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_weighted_hist2d: invalid arguments");
    return;
  }
  if (!(max[p] > min[p]) || !(max[q] > min[q])) {
    set_error(err, PMCG_EARG, __LINE__, "histogram range is empty");
    return;
  }
  SimMirror *m = mirror_any(psim, err);
  if (!m || !post_setup(m, psim, err)) return;
  Work &w = m->w;
  double *dh = nullptr;
  const size_t nb2 = (size_t)nbin * nbin;
  if (!CK(cudaMallocAsync(&dh, sizeof(double) * nb2, w.s), "histogram")) return;
  bool ok = CK(launch_post_hist2d(w.N, w.D, w.X64, w.wbar, w.flg, nbin, p, q, min, max, (double)w.N, m->pscratch, dh,
                                  w.s),
               "histogram") &&
            CK(cudaMemcpyAsync(hist, dh, sizeof(double) * nb2, cudaMemcpyDeviceToHost, w.s), "histogram");
  cudaFreeAsync(dh, w.s);
  ok = CK(cudaStreamSynchronize(w.s), "histogram") && ok;
  (void)ok;
}

extern "C" void update_prop_rb(mix_mvdens *proposal, pmc_simu *psim, error **err) {
  SimMirror *m = mirror_for(psim, proposal->ncomp, proposal->ndim, proposal->comp[0]->df, err);
  if (!m) return;
  Work &w = m->w;
  if (!sync_sample(m, psim, err) || !sync_proposal(m, proposal, err) || !sync_weights(m, psim, err)) return;
  // From here the device proposal is the updated one; until it is copied back,
  // the host proposal no longer matches the snapshot (a failed update leaves
  // the host proposal as it was, which the next call then uploads).
  m->snap_w.clear();
  if (m->spec >= 2) {
    // updated ahead from this sample, these weights and this proposal: the
    // second proposal becomes the device proposal, with its statistics
    m->spec = 0;
    std::swap(w.prop, m->spec_mix);
    if (!CK(cudaMemcpyAsync(w.dstats, m->spec_st, sizeof(DevStats), cudaMemcpyDeviceToDevice, w.s), "statistics"))
      return;
    m->lt_valid = true;
    if (!fetch_stats(w, err)) return;
  } else {
    m->spec = 0;
    if (!m->lt_valid && !stage_logq(w, err)) return;
    m->lt_valid = true;
    if (!stage_em(w, err) || !fetch_stats(w, err)) return;
  }
  const int K = w.K, D = w.D;
  std::vector<double> &wt = m->upd_w, &mu = m->upd_mu, &L = m->upd_L;
  wt.resize(K);
  mu.resize((size_t)K * D);
  L.resize((size_t)K * D * D);
  bool ok = CK(cudaMemcpyAsync(wt.data(), w.prop.w, 8 * K, cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(mu.data(), w.prop.mu, 8 * mu.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaMemcpyAsync(L.data(), w.prop.L, 8 * L.size(), cudaMemcpyDeviceToHost, w.s), "proposal") &&
            CK(cudaStreamSynchronize(w.s), "update");
  if (!ok) return;
  for (int k = 0; k < K; k++) {
    proposal->wght[k] = wt[k];
    mvdens *c = proposal->comp[k];
    if (wt[k] > 0.0) {
      memcpy(c->mean, &mu[(size_t)k * D], 8 * D);
      memcpy(c->std, &L[(size_t)k * D * D], 8 * (size_t)D * D);
      c->chol = 1;
      double ld = 0.0;
      for (int i = 0; i < D; i++) ld += std::log(c->std[i * D + i]);
      c->det = 2.0 * ld;
    }
  }
  // The device proposal now equals the host one: the downloaded arrays are the
  // snapshot (the update writes zeros above the diagonal; a buried component
  // keeps its parameters on the device and on the host).
  m->snap_w.swap(wt);
  m->snap_mu.swap(mu);
  m->snap_L.swap(L);
  m->lt_valid = false;
}

extern "C" double perplexity_and_ess(pmc_simu *psim, int mode, double *ess, error **err) {
  (void)mode;
  SimMirror *m = mirror_any(psim, err);
  if (!m) return 0.0;
  if (!m->x_valid &&
      !CK(cudaMemcpyAsync(m->w.flg, psim->flg, 2 * m->w.N, cudaMemcpyHostToDevice, m->w.s), "flg upload"))
    return 0.0;
  if (!sync_weights(m, psim, err)) return 0.0;
  if (ess) *ess = m->w.hstats->ess;
  return m->w.hstats->perplexity;
}

extern "C" double evidence(pmc_simu *psim, double *ln_evi, error **err) {
  SimMirror *m = mirror_any(psim, err);
  if (!m) return 0.0;
  if (!m->x_valid &&
      !CK(cudaMemcpyAsync(m->w.flg, psim->flg, 2 * m->w.N, cudaMemcpyHostToDevice, m->w.s), "flg upload"))
    return 0.0;
  if (!sync_weights(m, psim, err)) return 0.0;
  if (ln_evi) *ln_evi = m->w.hstats->ln_evidence;
  return std::exp(m->w.hstats->ln_evidence);
}
