// pmcg_host.cpp — host-side part of the pmclib-compatible C ABI: the error
// chain, density/sample containers, the prior box, the random stream handle,
// the tempering schedule and the mix_mvdens text format. None of these
// touches a per-sample computation; the hot path is in pmcg_engine.cu.
#include "../../include/pmcg.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "pmcg_internal.h"

// ------------------------------------------------------------------ errors
extern "C" error *addError(int code, const char *text, error *next, int line) {
  error *e = (error *)calloc(1, sizeof(error));
  if (!e) return next;
  e->errValue = code;
  e->line = line;
  snprintf(e->errText, sizeof(e->errText), "%s", text ? text : "");
  snprintf(e->errWhere, sizeof(e->errWhere), "libpmcg");
  e->next = next;
  return e;
}

extern "C" int isError(const error *err) { return err != nullptr && err->errValue != 0; }
extern "C" int getErrorValue(const error *err) { return err ? err->errValue : 0; }

extern "C" void purgeError(error **err) {
  if (!err) return;
  error *e = *err;
  while (e) {
    error *n = e->next;
    free(e);
    e = n;
  }
  *err = nullptr;
}

extern "C" void printError(FILE *f, const error *err) {
  for (const error *e = err; e; e = e->next)
    fprintf(f, "Error %d (%s:%d): %s\n", e->errValue, e->errWhere, e->line, e->errText);
}

namespace pmcg {
void set_error(error **err, int code, int line, const char *fmt, ...) {
  if (!err) return;
  char buf[384];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  *err = addError(code, buf, *err, line);
}

int host_cholesky(int D, const double *C, double *L, double *logdetL) {
  double ld = 0.0;
  for (int i = 0; i < D * D; i++) L[i] = 0.0;
  for (int j = 0; j < D; j++) {
    double s = C[j * D + j];
    for (int k = 0; k < j; k++) s -= L[j * D + k] * L[j * D + k];
    if (!(s > 0.0) || !std::isfinite(s)) return -1;
    double d = std::sqrt(s);
    L[j * D + j] = d;
    ld += std::log(d);
    for (int i = j + 1; i < D; i++) {
      double t = C[i * D + j];
      for (int k = 0; k < j; k++) t -= L[i * D + k] * L[j * D + k];
      L[i * D + j] = t / d;
    }
  }
  if (logdetL) *logdetL = ld;
  return 0;
}

// Flatten a host mixture into (w, mu, L) with Cholesky factors.
bool flatten_mix(const mix_mvdens *m, std::vector<double> &w, std::vector<double> &mu, std::vector<double> &L,
                 error **err) {
  const int K = m->ncomp, D = m->ndim;
  w.assign(m->wght, m->wght + K);
  mu.resize((size_t)K * D);
  L.resize((size_t)K * D * D);
  for (int k = 0; k < K; k++) {
    const mvdens *c = m->comp[k];
    if (c->ndim != D) {
      set_error(err, PMCG_EDIM, __LINE__, "component %d has dimension %d, mixture %d", k, c->ndim, D);
      return false;
    }
    memcpy(&mu[(size_t)k * D], c->mean, sizeof(double) * D);
    if (c->chol) {
      for (int i = 0; i < D; i++)
        for (int j = 0; j < D; j++) L[(size_t)k * D * D + i * D + j] = (j <= i) ? c->std[i * D + j] : 0.0;
    } else if (host_cholesky(D, c->std, &L[(size_t)k * D * D], nullptr) != 0) {
      set_error(err, PMCG_ECHOL, __LINE__, "covariance of component %d is not positive definite", k);
      return false;
    }
  }
  return true;
}
}  // namespace pmcg

using pmcg::set_error;

// ------------------------------------------------------------------ densities
extern "C" mvdens *mvdens_alloc(int ndim, error **err) {
  if (ndim < 1) { set_error(err, PMCG_EARG, __LINE__, "ndim %d", ndim); return nullptr; }
  mvdens *m = (mvdens *)calloc(1, sizeof(mvdens));
  if (!m) { set_error(err, PMCG_EALLOC, __LINE__, "mvdens"); return nullptr; }
  m->ndim = ndim;
  m->df = -1;
  m->band_limit = ndim;
  m->mean = (double *)calloc((size_t)ndim, sizeof(double));
  m->std = (double *)calloc((size_t)ndim * ndim, sizeof(double));
  if (!m->mean || !m->std) {
    free(m->mean); free(m->std); free(m);
    set_error(err, PMCG_EALLOC, __LINE__, "mvdens arrays");
    return nullptr;
  }
  for (int i = 0; i < ndim; i++) m->std[i * ndim + i] = 1.0;
  return m;
}

extern "C" void mvdens_free(mvdens **m) {
  if (!m || !*m) return;
  free((*m)->mean);
  free((*m)->std);
  free(*m);
  *m = nullptr;
}

extern "C" mix_mvdens *mix_mvdens_alloc(int ncomp, int ndim, error **err) {
  if (ncomp < 1) { set_error(err, PMCG_EARG, __LINE__, "ncomp %d", ncomp); return nullptr; }
  mix_mvdens *m = (mix_mvdens *)calloc(1, sizeof(mix_mvdens));
  if (!m) { set_error(err, PMCG_EALLOC, __LINE__, "mix_mvdens"); return nullptr; }
  m->ncomp = ncomp;
  m->ndim = ndim;
  m->wght = (double *)calloc((size_t)ncomp, sizeof(double));
  m->comp = (mvdens **)calloc((size_t)ncomp, sizeof(mvdens *));
  if (!m->wght || !m->comp) {
    free(m->wght); free(m->comp); free(m);
    set_error(err, PMCG_EALLOC, __LINE__, "mix_mvdens arrays");
    return nullptr;
  }
  for (int k = 0; k < ncomp; k++) {
    m->wght[k] = 1.0 / ncomp;
    m->comp[k] = mvdens_alloc(ndim, err);
    if (!m->comp[k]) { mix_mvdens_free(&m); return nullptr; }
  }
  return m;
}

extern "C" void mix_mvdens_free(mix_mvdens **m) {
  if (!m || !*m) return;
  pmcg::forget_mix(*m);
  if ((*m)->comp)
    for (int k = 0; k < (*m)->ncomp; k++) mvdens_free(&(*m)->comp[k]);
  free((*m)->comp);
  free((*m)->wght);
  free(*m);
  *m = nullptr;
}

extern "C" void mix_mvdens_copy(mix_mvdens *dst, const mix_mvdens *src, error **err) {
  if (!dst || !src || dst->ncomp != src->ncomp || dst->ndim != src->ndim) {
    set_error(err, PMCG_EDIM, __LINE__, "mix_mvdens_copy: shape mismatch");
    return;
  }
  const int D = src->ndim;
  memcpy(dst->wght, src->wght, sizeof(double) * src->ncomp);
  for (int k = 0; k < src->ncomp; k++) {
    mvdens *a = dst->comp[k];
    const mvdens *b = src->comp[k];
    a->df = b->df; a->band_limit = b->band_limit; a->chol = b->chol; a->det = b->det;
    memcpy(a->mean, b->mean, sizeof(double) * D);
    memcpy(a->std, b->std, sizeof(double) * D * D);
  }
}

extern "C" void mvdens_cholesky_decomp(mvdens *m, error **err) {
  if (!m || m->chol) return;
  const int D = m->ndim;
  std::vector<double> L((size_t)D * D);
  double ld;
  if (pmcg::host_cholesky(D, m->std, L.data(), &ld) != 0) {
    set_error(err, PMCG_ECHOL, __LINE__, "covariance is not positive definite");
    return;
  }
  memcpy(m->std, L.data(), sizeof(double) * D * D);
  m->chol = 1;
  m->det = 2.0 * ld;
}

extern "C" void mix_mvdens_cholesky_decomp(mix_mvdens *m, error **err) {
  for (int k = 0; k < m->ncomp; k++) {
    mvdens_cholesky_decomp(m->comp[k], err);
    if (isError(err ? *err : nullptr)) return;
  }
}

extern "C" void mvdens_from_meanvar(mvdens *m, const double *mean, const double *cov, double correct) {
  const int D = m->ndim;
  if (mean) memcpy(m->mean, mean, sizeof(double) * D);
  if (cov) {
    for (int i = 0; i < D * D; i++) m->std[i] = cov[i] * correct;
    m->chol = 0;
  }
}

extern "C" double effective_number_of_components(const mix_mvdens *m, error **err) {
  double s = 0.0;
  for (int k = 0; k < m->ncomp; k++) s += m->wght[k] * m->wght[k];
  if (!(s > 0.0)) {
    set_error(err, PMCG_ENEGWEIGHT, __LINE__, "all component weights are zero");
    return 0.0;
  }
  return 1.0 / s;
}

// Text format of Manual/manual.tex:3199-3260 (covariance written, chol flag 0).
static void dump_mvdens(FILE *f, const mvdens *c) {
  const int D = c->ndim;
  fprintf(f, "%d %d %d %d\n", D, c->df, c->band_limit, 0);
  for (int i = 0; i < D; i++) fprintf(f, "%.17g ", c->mean[i]);
  fprintf(f, "\n");
  for (int i = 0; i < D; i++) {
    for (int j = 0; j < D; j++) {
      double v;
      if (c->chol) {
        v = 0.0;
        for (int q = 0; q <= (i < j ? i : j); q++) v += c->std[i * D + q] * c->std[j * D + q];
      } else {
        v = c->std[i * D + j];
      }
      fprintf(f, "%.17g ", v);
    }
    fprintf(f, "\n");
  }
}

extern "C" void mix_mvdens_dump(FILE *f, const mix_mvdens *m) {
  fprintf(f, "%d %d\n", m->ncomp, m->ndim);
  for (int k = 0; k < m->ncomp; k++) {
    fprintf(f, "%.17g\n", m->wght[k]);
    dump_mvdens(f, m->comp[k]);
  }
}

extern "C" void mix_mvdens_print(FILE *f, const mix_mvdens *m) { mix_mvdens_dump(f, m); }

extern "C" mix_mvdens *mix_mvdens_dwnp(FILE *f, error **err) {
  int K, D;
  if (fscanf(f, "%d %d", &K, &D) != 2 || K < 1 || D < 1) {
    set_error(err, PMCG_EIO, __LINE__, "mix_mvdens header");
    return nullptr;
  }
  mix_mvdens *m = mix_mvdens_alloc(K, D, err);
  if (!m) return nullptr;
  for (int k = 0; k < K; k++) {
    mvdens *c = m->comp[k];
    int d, df, bl, ch;
    if (fscanf(f, "%lf", &m->wght[k]) != 1 || fscanf(f, "%d %d %d %d", &d, &df, &bl, &ch) != 4 || d != D) {
      set_error(err, PMCG_EIO, __LINE__, "component %d header", k);
      mix_mvdens_free(&m);
      return nullptr;
    }
    c->df = df; c->band_limit = bl; c->chol = ch;
    for (int i = 0; i < D; i++)
      if (fscanf(f, "%lf", &c->mean[i]) != 1) { set_error(err, PMCG_EIO, __LINE__, "mean"); mix_mvdens_free(&m); return nullptr; }
    for (int i = 0; i < D * D; i++)
      if (fscanf(f, "%lf", &c->std[i]) != 1) { set_error(err, PMCG_EIO, __LINE__, "matrix"); mix_mvdens_free(&m); return nullptr; }
    if (ch) {
      double ld = 0.0;
      for (int i = 0; i < D; i++) ld += std::log(c->std[i * D + i]);
      c->det = 2.0 * ld;
    }
  }
  return m;
}

// ------------------------------------------------------------------ prior box
extern "C" parabox *init_parabox(int ndim, error **err) {
  parabox *pb = (parabox *)calloc(1, sizeof(parabox));
  if (!pb) { set_error(err, PMCG_EALLOC, __LINE__, "parabox"); return nullptr; }
  pb->ndim = ndim;
  pb->min = (double *)malloc(sizeof(double) * ndim);
  pb->max = (double *)malloc(sizeof(double) * ndim);
  for (int i = 0; i < ndim; i++) { pb->min[i] = -INFINITY; pb->max[i] = INFINITY; }
  return pb;
}

extern "C" void add_slab(parabox *pb, int dim, double min, double max, error **err) {
  if (!pb || dim < 0 || dim >= pb->ndim || !(max > min)) {
    set_error(err, PMCG_EARG, __LINE__, "add_slab(%d, %g, %g)", dim, min, max);
    return;
  }
  pb->min[dim] = min;
  pb->max[dim] = max;
}

extern "C" void free_parabox(parabox **pb) {
  if (!pb || !*pb) return;
  free((*pb)->min);
  free((*pb)->max);
  free(*pb);
  *pb = nullptr;
}

extern "C" int isinBox(const parabox *pb, const double *x) {
  for (int i = 0; i < pb->ndim; i++)
    if (x[i] < pb->min[i] || x[i] > pb->max[i]) return 0;
  return 1;
}

// ------------------------------------------------------------------ samples
extern "C" pmc_simu *pmc_simu_init_plus_ded(size_t nsamples, int ndim, int n_ded, error **err) {
  pmc_simu *p = (pmc_simu *)calloc(1, sizeof(pmc_simu));
  if (!p) { set_error(err, PMCG_EALLOC, __LINE__, "pmc_simu"); return nullptr; }
  p->ndim = ndim;
  p->n_ded = n_ded;
  pmc_simu_realloc(p, nsamples, err);
  if (isError(err ? *err : nullptr)) { pmc_simu_free(&p); return nullptr; }
  return p;
}

extern "C" pmc_simu *pmc_simu_init_mpi(size_t nsamples, int ndim, int n_ded, error **err) {
  return pmc_simu_init_plus_ded(nsamples, ndim, n_ded, err);
}

// Sample arrays are page-locked when a CUDA device is present, so the
// drop-in entry points copy them at full host-link bandwidth; without a
// device they are ordinary heap memory (the device entry points then fail).
static void *host_alloc(size_t bytes, int pinned) {
  void *p = nullptr;
  if (pinned) return cudaMallocHost(&p, bytes) == cudaSuccess ? p : nullptr;
  return malloc(bytes);
}
static void host_free(void *p, int pinned) {
  if (!p) return;
  if (pinned) cudaFreeHost(p);
  else free(p);
}

extern "C" void pmc_simu_realloc(pmc_simu *p, size_t nsamples, error **err) {
  if (nsamples > p->maxsamples) {
    if (p->maxsamples == 0) {
      int n = 0;
      p->pinned = (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
    }
    const int pin = p->pinned;
    size_t D = (size_t)p->ndim, Dd = (size_t)(p->n_ded > 0 ? p->n_ded : 0), old = p->nsamples;
    double *X = (double *)host_alloc(sizeof(double) * nsamples * D, pin);
    double *Xd = Dd ? (double *)host_alloc(sizeof(double) * nsamples * Dd, pin) : nullptr;
    double *w = (double *)host_alloc(sizeof(double) * nsamples, pin);
    short *f = (short *)host_alloc(sizeof(short) * nsamples, pin);
    int *ix = (int *)host_alloc(sizeof(int) * nsamples, pin);
    if (!X || (Dd && !Xd) || !w || !f || !ix) {
      host_free(X, pin); host_free(Xd, pin); host_free(w, pin); host_free(f, pin); host_free(ix, pin);
      set_error(err, PMCG_EALLOC, __LINE__, "pmc_simu_realloc(%zu)", nsamples);
      return;
    }
    if (p->X) {
      memcpy(X, p->X, sizeof(double) * old * D);
      if (Dd && p->X_ded) memcpy(Xd, p->X_ded, sizeof(double) * old * Dd);
      memcpy(w, p->weights, sizeof(double) * old);
      memcpy(f, p->flg, sizeof(short) * old);
      memcpy(ix, p->indices, sizeof(int) * old);
    }
    host_free(p->X, pin); host_free(p->X_ded, pin); host_free(p->weights, pin);
    host_free(p->flg, pin); host_free(p->indices, pin);
    p->X = X; p->X_ded = Xd; p->weights = w; p->flg = f; p->indices = ix;
    p->maxsamples = nsamples;
  }
  p->nsamples = nsamples;
  pmcg_simu_host_modified(p);
}

// ------------------------------------------------------------------ sample files
// The CosmoPMC sample file (exec/exec_helper.c:351-427): a header ("# npar =
// .., n_ded = ..", column titles, parameter names) and one row per counted
// sample: the unnormalised log-weight, minus the component index, the
// parameters and the deduced parameters, each "%16.9g".
// The sample file of exec/exec_helper.c:351-427 (header, then one row per
// counted sample: unnormalised log-weight, -component, parameters, deduced
// parameters, %16.9g); name_of(i) gives parameter i's name for the header.
template <typename NameOf>
static void write_pmc_simu(const char *name, const pmc_simu *psim, NameOf name_of, error **err) {
  FILE *f = fopen(name, "w");
  if (!f) {
    set_error(err, PMCG_EIO, __LINE__, "cannot open %s for writing", name);
    return;
  }
  const int D = psim->ndim, Dd = psim->n_ded > 0 ? psim->n_ded : 0;
  fprintf(f, "# npar = %d, n_ded = %d\n", D, Dd);
  fprintf(f, "#         weight            chi2");
  for (int i = 0; i < D; i++) fprintf(f, "        param[%d]", i);
  for (int i = 0; i < Dd; i++) fprintf(f, "    param_ded[%d]", i);
  fprintf(f, "\n#                               ");
  for (int i = 0; i < D; i++) fprintf(f, "%16s", name_of(i));
  fprintf(f, "\n");
  const double lognorm = psim->logSum;
  for (size_t n = 0; n < psim->nsamples; n++) {
    if (psim->flg[n] == 0) continue;
    double logw = psim->weights[n];
    if (!psim->isLog) logw = std::log(logw);
    logw += lognorm;  // back to the unnormalised log-weight
    fprintf(f, "%16.9g%16.9g", logw, -(double)psim->indices[n]);
    for (int i = 0; i < D; i++) fprintf(f, "%16.9g", psim->X[n * D + i]);
    for (int i = 0; i < Dd; i++) fprintf(f, "%16.9g", psim->X_ded[n * Dd + i]);
    fprintf(f, "\n");
  }
  if (fclose(f) != 0) set_error(err, PMCG_EIO, __LINE__, "write error on %s", name);
}

// The par_t name table (the reference's spar_t strings), set by the caller.
static std::mutex g_names_mu;
static std::vector<std::string> g_par_names;

extern "C" void pmcg_set_par_names(int n, const char *const *names) {
  std::lock_guard<std::mutex> lk(g_names_mu);
  g_par_names.clear();
  for (int i = 0; i < n && names; i++) g_par_names.emplace_back(names[i] ? names[i] : "p");
}

extern "C" void out_pmc_simu_cosmo_pmc(const char *name, const pmc_simu *psim, const void *par, double norm,
                                       error **err) {
  (void)norm;
  std::lock_guard<std::mutex> lk(g_names_mu);
  const int *codes = (const int *)par;
  write_pmc_simu(name, psim, [&](int i) -> const char * {
    if (!codes || codes[i] < 0 || codes[i] >= (int)g_par_names.size()) return "p";
    return g_par_names[codes[i]].c_str();
  }, err);
}

extern "C" void pmcg_out_pmc_simu_names(const char *name, const pmc_simu *psim, const char *const *names,
                                        error **err) {
  write_pmc_simu(name, psim, [&](int i) -> const char * { return (names && names[i]) ? names[i] : "p"; }, err);
}

// Reads a sample file written as above (at most nsamples rows; comment lines
// start with '#'). The weights come back normalised (isLog = 0) with logSum
// and maxW of the file's unnormalised log-weights, every row counted (flg = 1)
// and the component index restored from the second column. proposal, when
// given, must match npar. nclipw > 0: then clip_weights(psim, nclipw) (the
// nclipw largest weights flagged out, the rest renormalised), as the resumed
// run of exec/cosmo_pmc.c:416-417 asks with the run's nclipw.
extern "C" pmc_simu *pmc_simu_from_file(FILE *f, size_t nsamples, int npar, int n_ded, const mix_mvdens *proposal,
                                        int nclipw, error **err) {
  if (!f || npar < 1 || nsamples == 0) {
    set_error(err, PMCG_EARG, __LINE__, "pmc_simu_from_file: invalid arguments");
    return nullptr;
  }
  if (nclipw < 0) {
    set_error(err, PMCG_EARG, __LINE__, "pmc_simu_from_file: nclipw = %d", nclipw);
    return nullptr;
  }
  if (proposal && proposal->ndim != npar) {
    set_error(err, PMCG_EDIM, __LINE__, "proposal has %d parameters, the sample %d", proposal->ndim, npar);
    return nullptr;
  }
  const int Dd = n_ded > 0 ? n_ded : 0, ncol = 2 + npar + Dd;
  pmc_simu *p = pmc_simu_init_plus_ded(nsamples, npar, Dd, err);
  if (!p) return nullptr;
  std::vector<double> row((size_t)ncol);
  size_t n = 0;
  char line[65536];
  while (n < nsamples && fgets(line, sizeof line, f)) {
    const char *c = line;
    while (*c == ' ' || *c == '\t') c++;
    if (*c == '#' || *c == '\n' || *c == '\0') continue;
    int got = 0;
    char *end = nullptr;
    for (; got < ncol; got++) {
      row[got] = strtod(c, &end);
      if (end == c) break;
      c = end;
    }
    if (got != ncol) {
      set_error(err, PMCG_EIO, __LINE__, "sample file row %zu: %d of %d columns", n + 1, got, ncol);
      pmc_simu_free(&p);
      return nullptr;
    }
    p->weights[n] = row[0];
    p->indices[n] = (int)std::lround(-row[1]);
    for (int i = 0; i < npar; i++) p->X[n * npar + i] = row[2 + i];
    for (int i = 0; i < Dd; i++) p->X_ded[n * Dd + i] = row[2 + npar + i];
    p->flg[n] = 1;
    n++;
  }
  if (n == 0) {
    set_error(err, PMCG_EIO, __LINE__, "sample file holds no sample");
    pmc_simu_free(&p);
    return nullptr;
  }
  p->nsamples = n;
  double mx = -INFINITY;
  for (size_t i = 0; i < n; i++) mx = std::max(mx, p->weights[i]);
  double s = 0.0;
  for (size_t i = 0; i < n; i++) s += std::exp(p->weights[i] - mx);
  const double ls = mx + std::log(s);
  for (size_t i = 0; i < n; i++) p->weights[i] = std::exp(p->weights[i] - ls);
  p->isLog = 0;
  p->logSum = ls;
  p->maxW = mx;
  p->nok = n;
  pmcg_simu_host_modified(p);
  if (nclipw > 0) {
    error *e = nullptr;
    clip_weights(p, nclipw, nullptr, &e);
    if (isError(e)) {
      if (err && !*err) *err = e;
      else purgeError(&e);
      pmc_simu_free(&p);
      return nullptr;
    }
    size_t nok = 0;
    for (size_t i = 0; i < n; i++) nok += p->flg[i] != 0;
    p->nok = nok;
  }
  return p;
}

extern "C" void pmc_simu_free(pmc_simu **p) {
  if (!p || !*p) return;
  pmcg::forget_simu(*p);
  const int pin = (*p)->pinned;
  host_free((*p)->X, pin);
  host_free((*p)->X_ded, pin);
  host_free((*p)->weights, pin);
  host_free((*p)->flg, pin);
  host_free((*p)->indices, pin);
  free(*p);
  *p = nullptr;
}

// ------------------------------------------------------------------ random streams
// The library's own generators, and the streams of foreign generators (the
// caller's gsl_rng*): key from the seed hook at first sight, call count kept
// here. One lock for both tables.
namespace {
struct ForeignStream {
  uint64_t seed;
  uint32_t calls;
};
std::mutex g_rng_mu;
std::unordered_set<const void *> g_own_rngs;
std::unordered_map<const void *, ForeignStream> g_foreign;
pmcg_rng_seed_fn *g_seed_hook = nullptr;
}  // namespace

extern "C" pmcg_rng *pmcg_rng_alloc(uint64_t seed) {
  pmcg_rng *r = (pmcg_rng *)calloc(1, sizeof(pmcg_rng));
  if (r) {
    r->seed = seed;
    std::lock_guard<std::mutex> lk(g_rng_mu);
    g_own_rngs.insert(r);
  }
  return r;
}

extern "C" void pmcg_rng_free(pmcg_rng **r) {
  if (!r || !*r) return;
  {
    std::lock_guard<std::mutex> lk(g_rng_mu);
    g_own_rngs.erase(*r);
  }
  free(*r);
  *r = nullptr;
}

extern "C" void pmcg_set_rng_seed_hook(pmcg_rng_seed_fn *fn) {
  std::lock_guard<std::mutex> lk(g_rng_mu);
  g_seed_hook = fn;
}

extern "C" void pmcg_rng_forget(void *rng) {
  std::lock_guard<std::mutex> lk(g_rng_mu);
  g_foreign.erase(rng);
}

namespace pmcg {
bool rng_stream(void *rng, uint64_t *seed, uint32_t **calls, error **err) {
  std::lock_guard<std::mutex> lk(g_rng_mu);
  if (g_own_rngs.count(rng)) {
    pmcg_rng *r = (pmcg_rng *)rng;
    *seed = r->seed;
    *calls = &r->calls;
    return true;
  }
  auto it = g_foreign.find(rng);
  if (it == g_foreign.end()) {
    if (!g_seed_hook) {
      set_error(err, PMCG_EARG, __LINE__,
                "simulate_mix_mvdens: the generator is not a pmcg_rng and no seed hook is set "
                "(pmcg_set_rng_seed_hook)");
      return false;
    }
    it = g_foreign.emplace(rng, ForeignStream{g_seed_hook(rng), 0u}).first;
  }
  *seed = it->second.seed;
  *calls = &it->second.calls;
  return true;
}
}  // namespace pmcg

// get_tempering_beta, exec/cosmo_pmc.c:464-495.
extern "C" double get_tempering_beta(int tempering, int iter, double t_min, int nmax, error **err) {
  switch (tempering) {
    case PMCG_TEMPERING_NONE:
      return 1.0;
    case PMCG_TEMPERING_LINEAR:
      if (iter == nmax - 1) return 1.0;
      return (double)iter / (nmax - 2.0) * (1.0 - t_min) + t_min;
    case PMCG_TEMPERING_LOG:
      if (iter == nmax - 1) return 1.0;
      if (t_min <= 0) {
        set_error(err, PMCG_EARG, __LINE__, "Minimal temperature needs to be positive, found %g", t_min);
        return 0.0;
      }
      return std::exp((double)iter / (nmax - 2.0) * (-std::log(t_min)) + std::log(t_min));
    default:
      set_error(err, PMCG_EARG, __LINE__, "Unknown tempering type %d", tempering);
      return 0.0;
  }
}

extern "C" const char *pmcg_version(void) { return "pmcg 0.1 (sm_103a)"; }
