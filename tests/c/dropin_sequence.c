/*
 * A C caller of libpmcg that runs the CosmoPMC driver's iteration sequence
 * through the pmclib-named entry points, as one process runs it:
 * run_pmc_iteration_MPI (exec/cosmo_pmc.c:293-402) with post_processing's
 * diagnostics (:441-455):
 *
 *   pmc_simu_realloc -> simulate_mix_mvdens (the caller's own generator)
 *   -> generic_get_importance_weight_and_deduced_verb (mix_mvdens_log_pdf_void,
 *      the caller's posterior_log_pdf_common_void, &config)
 *   -> normalize_importance_weight -> update_prop_rb -> out_pmc_simu_cosmo_pmc
 *      (the caller's par_t codes) -> perplexity_and_ess, evidence,
 *      effective_number_of_components
 *
 * The posterior is built from a CosmoPMC-style configuration by
 * pmcg_posterior_from_config and registered for &config; the generator is a
 * stand-in for the driver's gsl_rng whose stream key the library takes from
 * the seed hook. Compiled by the tests with gcc against include/pmcg.h and
 * linked to libpmcg.so.
 *
 * Input (stdin, whitespace separated):
 *   npar niter nsamples seed beta
 *   par_t codes [npar]; min [npar]; max [npar]
 *   nsn; per supernova: z m s c cov6[6]
 *   Theta2[3] sig_int v_pec h Omega_m w0_de chi2mode add_logdetCov quad_nodes special
 *   ncomp df; per component: weight mean[npar] covariance[npar*npar]
 *   output directory
 * Output (stdout), per iteration:
 *   iter <k> <nok> <ln evidence> <perplexity> <ess> <enc> <logSum>
 *   comp <k> <j> <chol> <weight> <mean[npar]> <std[npar*npar]>  (updated proposal;
 *   std is the lower Cholesky factor when chol is 1)
 *   and the sample file <outdir>/pmcsim_<k>.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "pmcg.h"

/* stand-in for the driver's gsl_rng */
typedef struct {
  unsigned long seed;
} caller_rng;

static uint64_t seed_from_caller_rng(void *r) { return (uint64_t)((caller_rng *)r)->seed; }

/* the caller's own posterior callback (the reference's posterior_log_pdf_common_void,
 * wrappers/src/param.c:948-954); the weight step evaluates the posterior registered
 * for its extra pointer on the device instead of calling it */
static double posterior_log_pdf_common_void(void *config, const double *x, error **err) {
  (void)config;
  (void)x;
  *err = addError(PMCG_EUNSUPPORTED, "host callback called", *err, __LINE__);
  return 0.0;
}

/* the part of config_base this caller keeps */
typedef struct {
  int npar;
  int *par;
  double *min, *max;
} caller_config;

#define READ1(fmt, p)                                   \
  do {                                                  \
    if (scanf(fmt, p) != 1) {                           \
      fprintf(stderr, "input error at %s\n", #p);       \
      return 2;                                         \
    }                                                   \
  } while (0)

#define CHECK(err)                                      \
  do {                                                  \
    if (isError(err)) {                                 \
      printError(stderr, err);                          \
      return 1;                                         \
    }                                                   \
  } while (0)

int main(void) {
  int npar, niter, nsamples;
  unsigned long seed;
  double beta;
  READ1("%d", &npar);
  READ1("%d", &niter);
  READ1("%d", &nsamples);
  READ1("%lu", &seed);
  READ1("%lf", &beta);
  caller_config config;
  config.npar = npar;
  config.par = malloc(sizeof(int) * npar);
  config.min = malloc(sizeof(double) * npar);
  config.max = malloc(sizeof(double) * npar);
  for (int i = 0; i < npar; i++) READ1("%d", &config.par[i]);
  for (int i = 0; i < npar; i++) READ1("%lf", &config.min[i]);
  for (int i = 0; i < npar; i++) READ1("%lf", &config.max[i]);

  pmcg_snia_config sn;
  READ1("%d", &sn.nsn);
  double *z = malloc(sizeof(double) * sn.nsn), *m = malloc(sizeof(double) * sn.nsn);
  double *s = malloc(sizeof(double) * sn.nsn), *c = malloc(sizeof(double) * sn.nsn);
  double *cov6 = malloc(sizeof(double) * 6 * sn.nsn);
  for (int i = 0; i < sn.nsn; i++) {
    READ1("%lf", &z[i]);
    READ1("%lf", &m[i]);
    READ1("%lf", &s[i]);
    READ1("%lf", &c[i]);
    for (int q = 0; q < 6; q++) READ1("%lf", &cov6[6 * i + q]);
  }
  sn.z = z;
  sn.m = m;
  sn.s = s;
  sn.c = c;
  sn.cov6 = cov6;
  for (int q = 0; q < 3; q++) READ1("%lf", &sn.Theta2[q]);
  READ1("%lf", &sn.sig_int);
  READ1("%lf", &sn.v_pec);
  READ1("%lf", &sn.h);
  READ1("%lf", &sn.Omega_m);
  READ1("%lf", &sn.w0_de);
  READ1("%d", &sn.chi2mode);
  READ1("%d", &sn.add_logdetCov);
  READ1("%d", &sn.quad_nodes);
  READ1("%d", &sn.special);

  error *err = NULL;
  int ncomp, df;
  READ1("%d", &ncomp);
  READ1("%d", &df);
  mix_mvdens *proposal = mix_mvdens_alloc(ncomp, npar, &err);
  CHECK(err);
  for (int k = 0; k < ncomp; k++) {
    READ1("%lf", &proposal->wght[k]);
    proposal->comp[k]->df = df;
    for (int i = 0; i < npar; i++) READ1("%lf", &proposal->comp[k]->mean[i]);
    for (int i = 0; i < npar * npar; i++) READ1("%lf", &proposal->comp[k]->std[i]);
  }
  char outdir[512];
  if (scanf("%511s", outdir) != 1) return 2;
  mix_mvdens_cholesky_decomp(proposal, &err);
  CHECK(err);

  /* the configuration's posterior on the device, standing in for the callback */
  const int data[1] = {PMCG_DATA_SNIA};
  const void *states[1] = {&sn};
  pmcg_posterior *post =
      pmcg_posterior_from_config(npar, config.par, config.min, config.max, 1, data, states, NULL, NULL, 0.0, &err);
  CHECK(err);
  pmcg_register_posterior(&config, post);

  /* the par_t name table (the reference's spar_t strings for the codes used here) */
  const char *names[40];
  for (int i = 0; i < 40; i++) names[i] = "p";
  names[PMCG_P_OMEGAM] = "Omega_m";
  names[PMCG_P_OMEGADE] = "Omega_de";
  names[PMCG_P_W0DE] = "w_0_de";
  names[PMCG_P_M] = "M";
  names[PMCG_P_ALPHA] = "alpha";
  names[PMCG_P_BETA] = "beta";
  pmcg_set_par_names(40, names);

  caller_rng rng = {seed};
  pmcg_set_rng_seed_hook(seed_from_caller_rng);
  parabox *pb = init_parabox(npar, &err);
  CHECK(err);
  for (int i = 0; i < npar; i++) {
    add_slab(pb, i, config.min[i], config.max[i], &err);
    CHECK(err);
  }

  pmc_simu *psim = pmc_simu_init_mpi(nsamples, npar, 0, &err);
  CHECK(err);
  for (int iter = 0; iter < niter; iter++) {
    pmc_simu_realloc(psim, nsamples, &err);
    CHECK(err);
    size_t nok = simulate_mix_mvdens(psim, proposal, &rng, pb, &err);
    CHECK(err);
    if (nok == 0) {
      fprintf(stderr, "No point simulated\n");
      return 1;
    }
    nok = generic_get_importance_weight_and_deduced_verb(psim, proposal, mix_mvdens_log_pdf_void,
                                                         posterior_log_pdf_common_void, NULL, (void *)&config, beta,
                                                         1, &err);
    CHECK(err);
    double norm = normalize_importance_weight(psim, &err);
    CHECK(err);
    update_prop_rb(proposal, psim, &err);
    CHECK(err);
    char name[600];
    snprintf(name, sizeof(name), "%s/pmcsim_%d", outdir, iter);
    out_pmc_simu_cosmo_pmc(name, psim, config.par, norm, &err);
    CHECK(err);
    double ess = 0.0, ln_evi = 0.0;
    double perp = perplexity_and_ess(psim, MC_UNORM, &ess, &err);
    CHECK(err);
    evidence(psim, &ln_evi, &err);
    CHECK(err);
    double enc = effective_number_of_components(proposal, &err);
    CHECK(err);
    printf("iter %d %zu %.17g %.17g %.17g %.17g %.17g\n", iter, psim->nok, ln_evi, perp, ess, enc, psim->logSum);
    for (int k = 0; k < ncomp; k++) {
      printf("comp %d %d %d %.17g", iter, k, proposal->comp[k]->chol, proposal->wght[k]);
      for (int i = 0; i < npar; i++) printf(" %.17g", proposal->comp[k]->mean[i]);
      for (int i = 0; i < npar * npar; i++) printf(" %.17g", proposal->comp[k]->std[i]);
      printf("\n");
    }
  }
  pmc_simu_free(&psim);
  free_parabox(&pb);
  pmcg_register_posterior(&config, NULL);
  pmcg_rng_forget(&rng);
  pmcg_posterior_free(&post);
  mix_mvdens_free(&proposal);
  free(config.par);
  free(config.min);
  free(config.max);
  free(z);
  free(m);
  free(s);
  free(c);
  free(cov6);
  return 0;
}
