// pmcg_internal.h — host-side helpers shared by pmcg_host.cpp and
// pmcg_engine.cu (internal; not part of the C ABI).
#pragma once
#include <vector>

#include "../../include/pmcg.h"

namespace pmcg {
void set_error(error **err, int code, int line, const char *fmt, ...);
int host_cholesky(int D, const double *C, double *L, double *logdetL);
bool flatten_mix(const mix_mvdens *m, std::vector<double> &w, std::vector<double> &mu, std::vector<double> &L,
                 error **err);
// Drop the device mirrors the library keeps for a host object.
void forget_mix(const mix_mvdens *m);
void forget_simu(const pmc_simu *p);
// Forget a posterior that is about to be freed (the drop-in mirrors keep the
// last one they weighed with).
void forget_posterior(const pmcg_posterior *p);
// The stream of a draw's generator argument: a pmcg_rng of this library, or a
// foreign generator keyed by the seed hook the first time it is seen. On
// success *seed and *calls (the call counter to use and advance) are set.
bool rng_stream(void *rng, uint64_t *seed, uint32_t **calls, error **err);
// The device posterior registered for a callback's extra pointer (or null).
const pmcg_posterior *registered_posterior(const void *extra);
}  // namespace pmcg
