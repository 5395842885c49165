// pmcg_serve.cu — a serving loop for PMC jobs with continuous batching.
//
// Clients submit jobs (proposal, posterior, sample size, iteration count,
// tempering schedule, seed) from any thread; one server thread owns the GPU.
// At every epoch boundary it admits queued jobs while free slots and the
// device-memory budget allow (each job's footprint is the exact size of the
// buffers its run allocates), binds the batch to the resident jobs when that
// set changed, and runs one iteration of every resident job: the smaller jobs
// in one persistent launch (k_batch.cu), jobs of at least alone_min_samples
// samples and jobs the batch does not take (D > 32, several likelihoods) with
// their own CUDA graphs on their own streams, concurrently. A job
// that arrives while others are on the
// GPU therefore joins the next epoch and overlaps with them. Each job's
// arithmetic depends only on its own inputs, so its result is the same alone
// and in any mix. Failed jobs (an iteration error) are retired with their
// error code; the others carry on. All waits are bounded.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "pmcg_engine.h"

using pmcg::set_error;

namespace pmcg {

struct Job {
  int64_t id = 0;
  mix_mvdens *prop = nullptr;          // private copy
  const pmcg_posterior *post = nullptr;
  parabox *pb = nullptr;               // private copy
  size_t N = 0;
  int niter = 0, tempering = 0;
  double tmin = 0.0;
  uint64_t seed = 0;
  size_t bytes = 0;
  bool alone = false;                  // iterates on its own stream, not in the batch
  // progress
  pmcg_run *run = nullptr;
  int iter = 0;
  int status = 1;  // 1 queued, 2 running, 0 done, < 0 error
  pmcg_iter_stats last = {};
  std::vector<double> final_w, final_mu, final_L;
  double t_submit = 0, t_start = 0, t_finish = 0;
};

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace pmcg

using namespace pmcg;

struct pmcg_server {
  pmcg_server_opts opts = {};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job *> queue;
  std::map<int64_t, Job *> jobs;
  std::vector<Job *> active;
  pmcg_batch *batch = nullptr;
  bool dirty = true, stop = false;   // dirty: a job was admitted or retired since the last binding
  int64_t next_id = 1;
  size_t bytes_in_use = 0, peak_bytes = 0;
  int peak_jobs = 0;
  long long epochs = 0;
  double t0 = 0;
  int device = 0;
  std::thread th;
};

namespace pmcg {

static void free_job(Job *j) {
  if (j->run) pmcg_run_free(&j->run);
  if (j->prop) mix_mvdens_free(&j->prop);
  if (j->pb) free_parabox(&j->pb);
  delete j;
}

static void retire(pmcg_server *s, Job *j, int status) {
  if (status == 0 && j->run) {
    const int K = j->prop->ncomp, D = j->prop->ndim;
    error *e = nullptr;
    mix_mvdens *out = mix_mvdens_alloc(K, D, &e);
    if (out) {
      pmcg_run_get_proposal(j->run, out, &e);
      if (!isError(e)) {
        j->final_w.assign(out->wght, out->wght + K);
        j->final_mu.resize((size_t)K * D);
        j->final_L.resize((size_t)K * D * D);
        for (int k = 0; k < K; k++) {
          memcpy(&j->final_mu[(size_t)k * D], out->comp[k]->mean, sizeof(double) * D);
          memcpy(&j->final_L[(size_t)k * D * D], out->comp[k]->std, sizeof(double) * D * D);
        }
      } else {
        status = getErrorValue(e);
      }
      mix_mvdens_free(&out);
    } else {
      // no host proposal to copy the result into: the job is not a success
      status = isError(e) ? getErrorValue(e) : PMCG_EALLOC;
    }
    purgeError(&e);
  }
  if (j->run) pmcg_run_free(&j->run);
  std::lock_guard<std::mutex> lk(s->mu);
  s->bytes_in_use -= j->bytes;
  j->status = status;
  j->t_finish = now_s() - s->t0;
  s->dirty = true;
  s->cv_done.notify_all();
}

static void server_loop(pmcg_server *s) {
  cudaSetDevice(s->device);
  std::vector<double> betas;
  std::vector<pmcg_iter_stats> st;
  for (;;) {
    std::vector<Job *> admitted;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->active.empty() && s->queue.empty() && !s->stop)
        s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
      if (s->stop) break;
      // admission: free slots and the device-memory budget, first come first served
      while (!s->queue.empty() && (int)(s->active.size() + admitted.size()) < s->opts.max_jobs &&
             s->bytes_in_use + s->queue.front()->bytes <= s->opts.hbm_budget_bytes) {
        Job *j = s->queue.front();
        s->queue.pop_front();
        s->bytes_in_use += j->bytes;
        admitted.push_back(j);
      }
      if (s->bytes_in_use > s->peak_bytes) s->peak_bytes = s->bytes_in_use;
    }
    for (Job *j : admitted) {
      error *e = nullptr;
      j->run = pmcg_run_create(j->prop, j->post, j->pb, j->N, PMCG_MIXED, j->seed, &e);
      // revival needs the job's prior box; jobs without one keep burying
      if (j->run && j->pb && s->opts.dead_comp == PMCG_DEAD_REVIVE)
        pmcg_run_set_dead_comp(j->run, PMCG_DEAD_REVIVE, s->opts.fshift, &e);
      if (!j->run || isError(e)) {
        int code = getErrorValue(e);
        purgeError(&e);
        retire(s, j, code ? code : PMCG_EALLOC);
        continue;
      }
      j->t_start = now_s() - s->t0;
      j->status = 2;
      s->active.push_back(j);
      s->dirty = true;
    }
    if (s->active.empty()) continue;
    if ((int)s->active.size() > s->peak_jobs) s->peak_jobs = (int)s->active.size();
    // Jobs of at least alone_min_samples samples fill the GPU by themselves:
    // they iterate on their own streams (their CUDA graphs, the tensor-core
    // kernels) beside the batch of the smaller ones; so do the jobs the batch
    // does not take (D > 32, or not exactly one likelihood).
    std::vector<Job *> small, large;
    for (Job *j : s->active) (j->alone ? large : small).push_back(j);
    if (s->dirty) {
      // a job came or went: bind the batched set to the batch (its arrays are
      // kept). Run pointers are not compared: a new run may reuse a freed one's
      // address.
      std::vector<pmcg_run *> runs;
      for (Job *j : small) runs.push_back(j->run);
      error *e = nullptr;
      if (runs.empty()) {
        if (s->batch) pmcg_batch_free(&s->batch);
      } else if (s->batch) {
        pmcg_batch_rebind(s->batch, (int)runs.size(), runs.data(), &e);
        if (isError(e)) pmcg_batch_free(&s->batch);
      } else {
        s->batch = pmcg_batch_create((int)runs.size(), runs.data(), &e);
      }
      if (s->batch && s->opts.autotune) pmcg_batch_autotune(s->batch, &e);
      if (!runs.empty() && !s->batch) {
        int code = getErrorValue(e);
        purgeError(&e);
        for (Job *j : small) retire(s, j, code ? code : PMCG_EUNSUPPORTED);
        s->active.swap(large);
        continue;
      }
      purgeError(&e);
      s->dirty = false;
    }
    auto beta_of = [](Job *j) {
      error *e = nullptr;
      double bt = get_tempering_beta(j->tempering, j->iter, j->tmin, j->niter, &e);
      if (isError(e)) bt = 1.0;
      purgeError(&e);
      return bt;
    };
    for (Job *j : large) {
      error *e = nullptr;
      pmcg_run_iterate_async(j->run, beta_of(j), &e);   // a launch error comes back from the wait
      purgeError(&e);
    }
    const size_t R = small.size();
    betas.resize(R);
    st.assign(R, pmcg_iter_stats{});
    for (size_t r = 0; r < R; r++) betas[r] = beta_of(small[r]);
    int batch_code = 0;
    if (R > 0) {
      error *e = nullptr;
      pmcg_batch_iterate(s->batch, betas.data(), st.data(), &e);
      if (isError(e)) {  // a launch failure: retire every batched job with the error
        batch_code = getErrorValue(e);
        purgeError(&e);
        pmcg_batch_free(&s->batch);
        s->dirty = true;
      }
    }
    std::vector<pmcg_iter_stats> lst(large.size());
    std::vector<int> lcode(large.size(), 0);
    for (size_t i = 0; i < large.size(); i++) {
      error *e = nullptr;
      pmcg_run_iterate_wait(large[i]->run, &lst[i], &e);
      if (isError(e)) lcode[i] = getErrorValue(e);
      purgeError(&e);
    }
    s->epochs++;
    std::vector<Job *> keep;
    auto settle = [&](Job *j, int code, const pmcg_iter_stats &js) {
      j->last = js;
      j->iter++;
      if (code != 0) retire(s, j, code);
      else if (j->iter >= j->niter) retire(s, j, 0);
      else keep.push_back(j);
    };
    for (size_t r = 0; r < R; r++) settle(small[r], batch_code ? batch_code : st[r].status, st[r]);
    for (size_t i = 0; i < large.size(); i++) settle(large[i], lcode[i], lst[i]);
    s->active.swap(keep);
  }
  if (s->batch) pmcg_batch_free(&s->batch);
  for (Job *j : s->active)
    if (j->run) pmcg_run_free(&j->run);
  s->active.clear();
}

}  // namespace pmcg

extern "C" pmcg_server *pmcg_server_create(const pmcg_server_opts *opts, error **err) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error(err, PMCG_ECUDA, __LINE__, "pmcg_server_create: no CUDA device");
    return nullptr;
  }
  pmcg_server *s = new pmcg_server();
  if (opts) s->opts = *opts;
  cudaGetDevice(&s->device);
  if (s->opts.max_jobs <= 0) s->opts.max_jobs = 512;
  if (!(s->opts.fshift > 0.0)) s->opts.fshift = 0.1;
  if (s->opts.alone_min_samples == 0) s->opts.alone_min_samples = (size_t)1 << 16;
  if (s->opts.dead_comp != PMCG_DEAD_REVIVE) s->opts.dead_comp = PMCG_DEAD_BURY;
  if (s->opts.hbm_budget_bytes == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    s->opts.hbm_budget_bytes = (size_t)(0.8 * (double)fr);
  }
  s->t0 = now_s();
  s->th = std::thread(server_loop, s);
  return s;
}

extern "C" int64_t pmcg_server_submit(pmcg_server *s, const mix_mvdens *proposal, const pmcg_posterior *post,
                                      const parabox *pb, size_t nsamples, int niter, int tempering, double t_min,
                                      uint64_t seed, error **err) {
  if (!s || !proposal || !post || nsamples == 0 || niter < 1 || proposal->ndim != post->npar ||
      (pb && pb->ndim != proposal->ndim)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_server_submit: invalid job");
    return 0;
  }
  if (proposal->ndim > kMaxD || post->plugins.empty()) {
    set_error(err, PMCG_EUNSUPPORTED, __LINE__, "served jobs need D <= %d and a likelihood", kMaxD);
    return 0;
  }
  Job *j = new Job();
  j->prop = mix_mvdens_alloc(proposal->ncomp, proposal->ndim, err);
  if (!j->prop) { delete j; return 0; }
  mix_mvdens_copy(j->prop, proposal, err);
  if (pb) {
    j->pb = init_parabox(pb->ndim, err);
    for (int i = 0; j->pb && i < pb->ndim; i++) { j->pb->min[i] = pb->min[i]; j->pb->max[i] = pb->max[i]; }
  }
  if (isError(err ? *err : nullptr)) { free_job(j); return 0; }
  j->post = post;
  j->N = nsamples;
  j->niter = niter;
  j->tempering = tempering;
  j->tmin = t_min;
  j->seed = seed;
  // the batch takes D <= 32 and one likelihood; larger jobs, and the others,
  // iterate alone beside it
  j->alone = nsamples >= s->opts.alone_min_samples || proposal->ndim > 32 || post->plugins.size() != 1;
  j->bytes = work_bytes(proposal->ncomp, proposal->ndim, proposal->comp[0]->df, PMCG_MIXED, nsamples);
  std::lock_guard<std::mutex> lk(s->mu);
  if (j->bytes > s->opts.hbm_budget_bytes) {
    set_error(err, PMCG_EALLOC, __LINE__, "job needs %zu device bytes, budget is %zu", j->bytes,
              s->opts.hbm_budget_bytes);
    free_job(j);
    return 0;
  }
  j->id = s->next_id++;
  j->t_submit = now_s() - s->t0;
  s->jobs[j->id] = j;
  s->queue.push_back(j);
  s->cv_work.notify_one();
  return j->id;
}

extern "C" int pmcg_server_wait(pmcg_server *s, int64_t job, double timeout_s, pmcg_job_result *res,
                                mix_mvdens *final_proposal, error **err) {
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job);
  if (it == s->jobs.end()) {
    set_error(err, PMCG_EARG, __LINE__, "unknown job %lld", (long long)job);
    return -1;
  }
  Job *j = it->second;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  while (j->status > 0) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && j->status > 0) {
      set_error(err, PMCG_ETIMEOUT, __LINE__, "job %lld not finished within %g s", (long long)job, timeout_s);
      return 0;
    }
  }
  if (res) {
    res->status = j->status;
    res->iterations = j->iter;
    res->ln_evidence = j->last.ln_evidence;
    res->perplexity = j->last.perplexity;
    res->ess = j->last.ess;
    res->enc = j->last.enc;
    res->submit_s = j->t_submit;
    res->start_s = j->t_start;
    res->finish_s = j->t_finish;
  }
  if (final_proposal && j->status == 0) {
    const int K = j->prop->ncomp, D = j->prop->ndim;
    if (final_proposal->ncomp != K || final_proposal->ndim != D) {
      set_error(err, PMCG_EDIM, __LINE__, "final proposal shape differs");
      return -1;
    }
    for (int k = 0; k < K; k++) {
      final_proposal->wght[k] = j->final_w[k];
      mvdens *c = final_proposal->comp[k];
      c->df = j->prop->comp[k]->df;
      memcpy(c->mean, &j->final_mu[(size_t)k * D], sizeof(double) * D);
      memcpy(c->std, &j->final_L[(size_t)k * D * D], sizeof(double) * D * D);
      c->chol = 1;
      double ld = 0.0;
      for (int i = 0; i < D; i++) ld += log(c->std[i * D + i]);
      c->det = 2.0 * ld;
    }
  }
  return 1;
}

extern "C" void pmcg_server_info(pmcg_server *s, pmcg_server_info_t *info) {
  std::lock_guard<std::mutex> lk(s->mu);
  info->queued = (int)s->queue.size();
  info->resident = (int)s->active.size();
  info->peak_resident = s->peak_jobs;
  info->bytes_in_use = s->bytes_in_use;
  info->peak_bytes = s->peak_bytes;
  info->budget_bytes = s->opts.hbm_budget_bytes;
  info->epochs = s->epochs;
}

extern "C" void pmcg_server_free(pmcg_server **ps) {
  if (!ps || !*ps) return;
  pmcg_server *s = *ps;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  for (auto &kv : s->jobs) free_job(kv.second);
  delete s;
  *ps = nullptr;
}
