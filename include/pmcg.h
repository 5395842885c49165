/*
 * pmcg.h — C ABI of libpmcg, a GB300 (sm_103a) Population Monte Carlo
 * iteration engine that stands in for pmclib underneath CosmoPMC.
 *
 * Part 1 re-declares the pmclib types and entry points that the CosmoPMC
 * driver binds (exec/cosmo_pmc.c); their names, argument meaning and
 * error behaviour follow the reference call sites cited beside each one.
 * pmclib itself is an external library that the reference only includes
 * (exec/cosmo_pmc.h:26-31), so the struct layouts below are this
 * library's own, carrying exactly the fields the reference reads.
 *
 * Part 2 is the GB300-native surface the reference has no counterpart for:
 * device-resident runs, batched likelihood evaluation, and the batch/serve
 * engines.
 *
 * No symbol here takes or returns a CUDA or torch type; streams are passed
 * as `void*` (a cudaStream_t, NULL = the library's own stream).
 */
#ifndef PMCG_H
#define PMCG_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ------------------------------------------------------------------ *
 * Error chain (pmctools errorlist semantics: negative codes, newest   *
 * first; exec/cosmo_pmc.c uses forwardError/quitOnError on it).       *
 * ------------------------------------------------------------------ */
typedef struct _err {
  char errWhere[128];
  char errText[384];
  int errValue;
  int line;
  struct _err *next;
} error;

#define PMCG_OK              0
#define pmcg_base        -9000
#define PMCG_ECUDA        (-1 + pmcg_base)  /* CUDA runtime error (text holds cudaGetErrorString) */
#define PMCG_EDIM         (-2 + pmcg_base)  /* dimension mismatch / unsupported size            */
#define PMCG_ECHOL        (-3 + pmcg_base)  /* covariance not positive definite (pmclib mv_cholesky) */
#define PMCG_ENOSAMPLE    (-4 + pmcg_base)  /* no point inside the prior box (pmc_nosamplep)      */
#define PMCG_ENEGWEIGHT   (-5 + pmcg_base)  /* all component weights zero (pmc_negWeight)        */
#define PMCG_EUNSUPPORTED (-6 + pmcg_base)  /* callback/feature not supported on the device path  */
#define PMCG_EALLOC       (-7 + pmcg_base)  /* host or device allocation failed                   */
#define PMCG_EARG         (-8 + pmcg_base)  /* invalid argument                                   */
#define PMCG_ETIMEOUT     (-9 + pmcg_base)  /* bounded wait ran out (serving loop)                */
#define PMCG_EIO          (-10 + pmcg_base) /* file read/write error                              */
#define PMCG_ENOWEIGHT    (-11 + pmcg_base) /* every sample has zero weight                       */
#define PMCG_ESTEPS       (-12 + pmcg_base) /* evaluation limit reached (pmclib math_tooManySteps) */
#define PMCG_EPRECISION   (-13 + pmcg_base) /* proposal given to a PMCG_MIXED run narrower than single
                                                precision resolves around its mean (use PMCG_FP64) */

error *addError(int code, const char *text, error *next, int line);
int isError(const error *err);
int getErrorValue(const error *err);
void purgeError(error **err);
void printError(FILE *f, const error *err);

/* ------------------------------------------------------------------ *
 * Densities: mvdens / mix_mvdens (Manual/manual.tex:3199-3260;       *
 * fields read at wrappers/src/param.c:543-549,1506-1528 and          *
 * exec/cosmo_pmc.c:211-234).                                          *
 * ------------------------------------------------------------------ */
typedef struct {
  int ndim;
  int df;          /* <= 0: Gaussian (pmclib writes -1); > 0: Student-t degrees of freedom */
  double *mean;    /* [ndim] */
  double *std;     /* [ndim*ndim] row-major covariance, or its lower Cholesky factor when chol==1 */
  int band_limit;  /* covariance entries with |i-j| >= band_limit are zero after an update */
  int chol;        /* 1 if std holds the Cholesky factor */
  double det;      /* log det of the covariance (valid when chol==1) */
} mvdens;

typedef struct {
  int ncomp;
  int ndim;
  double *wght;    /* [ncomp], sum 1; a buried component has weight 0 */
  mvdens **comp;   /* [ncomp] */
} mix_mvdens;

mvdens *mvdens_alloc(int ndim, error **err);
void mvdens_free(mvdens **m);
mix_mvdens *mix_mvdens_alloc(int ncomp, int ndim, error **err);
void mix_mvdens_free(mix_mvdens **m);
void mix_mvdens_copy(mix_mvdens *dst, const mix_mvdens *src, error **err);          /* cosmo_pmc.c:366 */
void mvdens_cholesky_decomp(mvdens *m, error **err);                                /* param.c:56,1476 */
void mix_mvdens_cholesky_decomp(mix_mvdens *m, error **err);                        /* param.c:700,1526 */
void mvdens_from_meanvar(mvdens *m, const double *mean, const double *cov, double correct); /* cosmo_pmc.c:230 */
double mvdens_log_pdf(mvdens *m, const double *x, error **err);                     /* param.c:1023 */
double mvdens_log_pdf_void(void *m, const double *x, error **err);                  /* param.c:1489 */
double mix_mvdens_log_pdf(mix_mvdens *m, const double *x, error **err);
double mix_mvdens_log_pdf_void(void *m, const double *x, error **err);              /* cosmo_pmc.c:343, param.c:1534 */
void mix_mvdens_dump(FILE *f, const mix_mvdens *m);                                 /* cosmo_pmc.c:37 */
mix_mvdens *mix_mvdens_dwnp(FILE *f, error **err);                                  /* cosmo_pmc.c:415 */
void mix_mvdens_print(FILE *f, const mix_mvdens *m);                                /* cosmo_pmc.c:29 */
double effective_number_of_components(const mix_mvdens *m, error **err);            /* cosmo_pmc.c:84 */

/* ------------------------------------------------------------------ *
 * Prior box (parabox; built at wrappers/src/param.c:915-926, passed  *
 * to the draw at exec/cosmo_pmc.c:320). Axis-aligned slabs.          *
 * ------------------------------------------------------------------ */
typedef struct {
  int ndim;
  double *min;     /* [ndim], -inf when the coordinate has no slab */
  double *max;     /* [ndim], +inf when the coordinate has no slab */
} parabox;

parabox *init_parabox(int ndim, error **err);
void add_slab(parabox *pb, int dim, double min, double max, error **err);
void free_parabox(parabox **pb);
int isinBox(const parabox *pb, const double *x);

/* ------------------------------------------------------------------ *
 * PMC sample (pmc_simu; fields used at exec/exec_helper.c:72-110,    *
 * 408-423 and exec/importance_sample.c:34-41,265-284).               *
 * ------------------------------------------------------------------ */
typedef struct {
  size_t nsamples;   /* samples drawn this iteration */
  size_t maxsamples; /* capacity */
  int ndim;
  int n_ded;
  double *X;         /* [nsamples*ndim] row-major */
  double *X_ded;     /* [nsamples*n_ded] deduced parameters: left as they are by the device path,
                        as the reference's retrieve_ded leaves them for the likelihoods that path
                        evaluates (SNIa, Mvdens and MixMvdens register no deduced function:
                        wrappers/src/sn.c:14, wrappers/src/param.c:1446-1447,1499-1500) */
  double *weights;   /* log-weights when isLog==1, normalised weights when isLog==0 */
  short *flg;        /* 1 = sample counts; 0 = outside the prior box or likelihood error */
  int *indices;      /* component each sample was drawn from */
  int isLog;
  double logSum;     /* log sum_{flg} exp(log-weight) */
  double maxW;       /* max log-weight over flg==1 */
  size_t nok;        /* samples with flg==1 after the weight step */
  int pinned;        /* 1 when the arrays are page-locked (set by the allocator) */
} pmc_simu;

pmc_simu *pmc_simu_init_mpi(size_t nsamples, int ndim, int n_ded, error **err);     /* cosmo_pmc.c:633 */
pmc_simu *pmc_simu_init_plus_ded(size_t nsamples, int ndim, int n_ded, error **err);/* cosmo_pmc.c:429 */
/* Sample files (exec/exec_helper.c:351-427): writes the counted samples as
 * "unnormalised log-weight, -component, parameters, deduced parameters"
 * (%16.9g) under the CosmoPMC header. par: the caller's par_t array (the
 * reference's parameter codes, tools/include/par.h:11-33, an enum read as
 * int; may be NULL); the header's name row prints names[par[i]] of the table
 * given to pmcg_set_par_names (the reference's spar_t strings), "p" without
 * one. norm is unused (kept for the reference's signature,
 * exec/exec_helper.h:61). */
void out_pmc_simu_cosmo_pmc(const char *name, const pmc_simu *psim, const void *par, double norm,
                            error **err);                                           /* cosmo_pmc.c:391 */
/* The name table for the par_t codes 0..n-1 (the reference builds it from its
 * spar_t macro); copied. No counterpart in the reference (its names are a
 * macro of the caller's build). */
void pmcg_set_par_names(int n, const char *const *names);
/* The same file with the parameter names given directly (names may be NULL). */
void pmcg_out_pmc_simu_names(const char *name, const pmc_simu *psim, const char *const *names, error **err);
/* Reads such a file (at most nsamples rows; exec/importance_sample.c:198,
 * exec/cosmo_pmc.c:416): weights normalised (isLog = 0, logSum, maxW of the
 * file's log-weights), flg = 1, indices from the second column. proposal
 * (optional) must match npar. nclipw > 0 then applies clip_weights(psim,
 * nclipw) (below): the resumed run's clipping (exec/cosmo_pmc.c:416-417). */
pmc_simu *pmc_simu_from_file(FILE *f, size_t nsamples, int npar, int n_ded, const mix_mvdens *proposal, int nclipw,
                             error **err);
void pmc_simu_realloc(pmc_simu *psim, size_t nsamples, error **err);                /* cosmo_pmc.c:313 */
void pmc_simu_free(pmc_simu **psim);                                                /* cosmo_pmc.c:738 */

/* Random streams. The draw samples from a counter-based generator on the
 * device, Philox4x32-10 (Salmon et al. 2011), keyed by a 64-bit seed; each
 * draw call consumes one counter block per sample and advances a call count.
 * The generator argument of the draw is the caller's own: a pmcg_rng of this
 * library, or any other generator pointer (the gsl_rng* that cosmo_pmc passes,
 * exec/cosmo_pmc.c:320), whose stream key the library takes once, the first
 * time it sees the pointer, from the seed hook (e.g. two gsl_rng_get calls);
 * the library then counts that generator's draw calls itself. */
typedef struct {
  uint64_t seed;
  uint32_t calls;
} pmcg_rng;

pmcg_rng *pmcg_rng_alloc(uint64_t seed);
void pmcg_rng_free(pmcg_rng **r);
/* The seed hook for foreign generators (NULL: none; a draw with a foreign
 * generator is then PMCG_EARG). No counterpart in the reference. */
typedef uint64_t pmcg_rng_seed_fn(void *rng);
void pmcg_set_rng_seed_hook(pmcg_rng_seed_fn *fn);
/* Forget a foreign generator's stream (before the caller frees it). */
void pmcg_rng_forget(void *rng);

/* Draw psim->nsamples points from the proposal into psim->X/indices/flg.
 * Points outside `pb` get flg=0 (weight 0, no redraw). Returns the number
 * inside the box. rng: a pmcg_rng*, or the caller's generator (see above).
 * Replaces pmclib simulate_mix_mvdens (exec/cosmo_pmc.c:320). */
size_t simulate_mix_mvdens(pmc_simu *psim, mix_mvdens *proposal, void *rng, parabox *pb, error **err);

/* Log-density callback type (wrappers/src/param.c:948). */
typedef double logpdf_fn(void *extra, const double *x, error **err);
typedef void retrieve_ded_fn(const void *extra, double *x_ded);

/* Importance log-weights: logw = beta*logpost(x) - log q(x); errors give
 * flg=0. q must be mix_mvdens_log_pdf_void; the posterior is either
 * post = pmcg_posterior_log_pdf_void with extra = pmcg_posterior*, or the
 * caller's own callback (posterior_log_pdf_common_void with &config->base,
 * exec/cosmo_pmc.c:343-345) for an extra pointer registered with
 * pmcg_register_posterior: the registered device posterior is evaluated in
 * its place. Both densities are evaluated on the GPU for the whole sample;
 * any other combination is rejected with PMCG_EUNSUPPORTED (there is no CPU
 * evaluation path). Returns the number of samples with flg==1.
 * Replaces pmclib (exec/cosmo_pmc.c:343-345). */
size_t generic_get_importance_weight_and_deduced_verb(pmc_simu *psim, mix_mvdens *proposal,
    logpdf_fn *q, logpdf_fn *post, retrieve_ded_fn *ded, void *extra, double beta, int quiet, error **err);

/* logSum = log sum exp(logw) over flg==1; weights become normalised
 * (isLog=0). Returns logSum (exec/cosmo_pmc.c:378). */
double normalize_importance_weight(pmc_simu *psim, error **err);
/* The nclipw largest weights among counted samples (ties to the lower index)
 * get flg = 0; a normalised sample is renormalised over the samples kept.
 * Replaces pmclib clip_weights (exec/cosmo_pmc.c:395-399); out (optional)
 * receives one line. */
void clip_weights(pmc_simu *psim, int nclipw, FILE *out, error **err);

/* Rao-Blackwellised EM update of the proposal from the last weighted
 * sample; dead components (fewer than 20 draws or weight < 1/N, or a
 * non-positive-definite update) are buried (weight 0) and the weights
 * renormalised (exec/cosmo_pmc.c:247; Manual/manual.tex:479-500). */
void update_prop_rb(mix_mvdens *proposal, pmc_simu *psim, error **err);

#define MC_UNORM 1
/* perplexity = exp(-sum wbar ln wbar)/N, *ess = 1/sum wbar^2
 * (exec/cosmo_pmc.c:46; Manual/manual.tex:556-575). */
double perplexity_and_ess(pmc_simu *psim, int mode, double *ess, error **err);
/* ln E = logSum - ln N; returns E (exec/cosmo_pmc.c:62). */
double evidence(pmc_simu *psim, double *ln_evi, error **err);

/* Tempering schedule (exec/cosmo_pmc.c:464-495). */
#define PMCG_TEMPERING_NONE   0
#define PMCG_TEMPERING_LINEAR 1
#define PMCG_TEMPERING_LOG    2
double get_tempering_beta(int tempering, int iter, double t_min, int nmax, error **err);

/* Tell the library that the caller rewrote psim->X, flg or weights on the
 * host: the device copy is re-uploaded before the next call, and whatever was
 * evaluated ahead from it (log q, the log posterior, the weight step,
 * normalisation and EM update of a repeated beta) is recomputed. */
void pmcg_simu_host_modified(pmc_simu *psim);

/* Importance sampling of an existing sample with another posterior
 * (exec/importance_sample.c:26-91): every sample's weight becomes its
 * log-posterior, evaluated on the device; flg = 0 outside the posterior's
 * prior box or on a likelihood error; isLog = 1, maxW set. Returns the number
 * of counted samples. The reference takes a config_base; here the posterior
 * is a pmcg_posterior. */
typedef struct pmcg_posterior pmcg_posterior;
size_t importance_sample(pmc_simu *psim, const pmcg_posterior *post, int quiet, error **err);
/* Weighted mean [ndim] and covariance [ndim x ndim] of the sample with its
 * weights (normalised on the device; log or linear, as psim->isLog says), as
 * the reference's post-processing computes them (exec/exec_helper.c:63-349). */
void pmcg_weighted_moments(pmc_simu *psim, double *mean, double *cov, error **err);
/* Marginal summary of every parameter on the device, as mean_sigma_from_psim
 * (exec/exec_helper.c:63-120) with median_from_psim and sigma_from_psim
 * (:160-271): center[i] = weighted mean (use_median = 0) or median, and
 * sigma[6i .. 6i+5] the one-sided 68.27 / 95.45 / 99.73 % limits to the right
 * then to the left of it (-1 where the sample ends first), from the normalised
 * weights of the samples with flg != 0. The reference copies the counted
 * samples by sample index (tmp[i]) but sorts the first n entries; here the
 * counted samples are compacted (its intent). A median whose first sample
 * already carries more than half the weight is that sample's value. */
void pmcg_weighted_summary(pmc_simu *psim, int use_median, double *center, double *sigma, error **err);
/* Weighted histograms of the sample, as create_1d_hist / create_2d_hist
 * (wrappers/src/param.c:1229-1357): the normalised weights times nsamples,
 * nbin bins per parameter over [min[p], max[p]] (bin j: e_j <= x < e_{j+1},
 * e_j = min + j (max - min) / nbin, the last bin closed at max; samples
 * outside or with flg == 0 not counted; the reference's accumulation lives in
 * pmclib, absent, so this binning is pinned here). hist1d: hist[p*nbin + b];
 * hist2d for parameters (p, q): hist[bp*nbin + bq]. */
void pmcg_weighted_hist1d(pmc_simu *psim, int nbin, const double *min, const double *max, double *hist,
                          error **err);
void pmcg_weighted_hist2d(pmc_simu *psim, int nbin, int p, int q, const double *min, const double *max,
                          double *hist, error **err);

/* Precision of the drop-in entry points above: PMCG_FP64 (default, the
 * plain FP64 path) or PMCG_MIXED. Process-wide default for every sample that
 * has no setting of its own (pmcg_simu_set_precision). */
void pmcg_set_dropin_precision(int precision);
/* Per sample (the drop-in's handle, as the reference's pmc_simu is its
 * iteration state): the precision of the drop-in calls on psim (PMCG_FP64,
 * PMCG_MIXED, or -1 for the process default) and its tensor-core setting
 * (1, 0, or -1 for the process default; changing it re-evaluates whatever was
 * computed ahead). Kept until pmc_simu_free. Two samples in one process can
 * run at different precisions. PMCG_EARG for other values. */
void pmcg_simu_set_precision(const pmc_simu *psim, int precision, error **err);
void pmcg_simu_set_tensor_cores(const pmc_simu *psim, int on, error **err);

/* Single-precision (PMCG_MIXED) mixture log-densities with D <= 32 on the
 * tensor cores: tcgen05 TF32 products in three-term split form, TMEM
 * accumulators (1 = on, the default; 0 = the CUDA-core kernel). Batched runs
 * (pmcg_batch_*, the serving loop) always use the CUDA-core kernel, so a run
 * alone reproduces its batched results bit for bit with 0. Returns the
 * previous setting. No counterpart in the reference (a GPU execution choice).
 * Process-wide default for every run without a setting of its own. */
int pmcg_set_tensor_cores(int on);

/* ------------------------------------------------------------------ *
 * Part 2 — device posterior plugins (the batched counterpart of the  *
 * per-point func_likeli_t of wrappers/include/init_wrappers.h:15-42). *
 * ------------------------------------------------------------------ */

/* Flat box prior: logpr_default = -sum log(max-min) added once per point
 * (wrappers/src/param.c:124-129, 988-1003). */
pmcg_posterior *pmcg_posterior_alloc(int npar, const double *min, const double *max, error **err);
void pmcg_posterior_free(pmcg_posterior **p);

/* Gaussian(-mixture) target likelihood (likeli_MixMvdens / likeli_Mvdens,
 * wrappers/src/param.c:1485-1537). The mixture is copied and
 * Cholesky-decomposed if needed. */
void pmcg_posterior_add_mixmvdens(pmcg_posterior *p, const mix_mvdens *target, error **err);

/* SN Ia likelihood (likeli_SNIa, wrappers/src/sn.c:138-281).
 * Per supernova: z, m_B, x1 (stretch), colour c and the 3x3 covariance of
 * (m_B, x1, c) as 6 numbers (mm, xx, cc, mx, mc, xc).
 * mu_obs = m_B - M + alpha*x1 - beta*c; D_L from a Gauss-Legendre quadrature
 * of 1/E(z) between consecutive sorted redshifts. */
#define PMCG_SN_CHI2_FULL 0   /* M is a sampled parameter */
#define PMCG_SN_CHI2_MARG 1   /* M analytically marginalised */
typedef struct {
  int nsn;
  const double *z, *mB, *x1, *c;
  const double *cov6;        /* [nsn*6] */
  double sig_int;            /* intrinsic dispersion (mag) */
  double v_pec;              /* peculiar velocity (km/s) */
  double h;                  /* Hubble parameter inside D_L (absorbed in M) */
  int chi2mode;              /* PMCG_SN_CHI2_FULL / _MARG */
  int add_logdet;            /* add -1/2 sum ln sigma_i^2 */
  int quad_nodes;            /* Gauss-Legendre nodes per redshift interval (1..16) */
  /* parameter indices in the sample vector, -1 when absent */
  int ip_Omegam, ip_Omegade, ip_w0, ip_M, ip_alpha, ip_beta;
  /* defaults for absent parameters */
  double def_Omegam, def_w0, def_M, def_alpha, def_beta;
  /* 1: the parameter at ip_M (ip_beta) holds -M (-beta), the reference's
   * storage (par_files/cosmo_SN.par:9); 0: +M (+beta) */
  int neg_M, neg_beta;
} pmcg_sn_data;
void pmcg_posterior_add_snia(pmcg_posterior *p, const pmcg_sn_data *sn, error **err);

/* Dense template likelihood: d(theta) = A phi(theta), phi = the monomials of
 * degree <= 2 in the npar parameters (1, theta_i, theta_i theta_j for i<=j);
 * logL = -1/2 (d_obs - d)^T C^-1 (d_obs - d). A is [ndata x nphi] row-major,
 * C [ndata x ndata]. C is Cholesky-factored in FP64 at set-up. */
void pmcg_posterior_add_template(pmcg_posterior *p, int ndata, const double *A, const double *C,
                                 const double *dobs, error **err);

/* Special prior, as prior_log_pdf_special (wrappers/src/param.c:1055-1101),
 * added once per point with the flat box prior (:994-999). It is a constant:
 * the log of the box volume of the affected parameters minus the log of the
 * special prior's volume.
 *  PMCG_SPECIAL_NONE: 0.
 *  PMCG_SPECIAL_UNITY: + sum log(max - min) (cancels the flat prior).
 *  PMCG_SPECIAL_DE_CONSERVATIVE: ind_w0 (< 0: no w0_de parameter, nothing
 *    added) alone: log(max_w0 - min_w0) - log(2/3); with ind_w1 >= 0:
 *    log(max_w0 - min_w0) + log(max_w1 - min_w1) - log(1/2 (2/3)^2 / (1 - a_acc))
 *    - log(1/2 (2/3)^2). a_acc is the scale factor constant that nicaea (the
 *    reference's cosmology library, absent here) supplies; the caller passes it.
 *    A w0_de range narrower than [-1, -1/3] is PMCG_EARG (the reference's
 *    mk_special_prior). The per-point dark-energy range test that the
 *    reference's likelihood plugins apply under this prior lives in nicaea and
 *    is not provided.
 * Calling again replaces the previous choice. */
#define PMCG_SPECIAL_NONE 0
#define PMCG_SPECIAL_UNITY 1
#define PMCG_SPECIAL_DE_CONSERVATIVE 2
void pmcg_posterior_set_special(pmcg_posterior *p, int special, int ind_w0, int ind_w1, double a_acc, error **err);

/* Gaussian or Student-t prior on a subset of the parameters (the config prior
 * with indprior, wrappers/src/param.c:1009-1026): mvdens_log_pdf(prior, x_sub)
 * is added to every point's log-posterior, x_sub = the parameters j with
 * indprior[j] == 1 in increasing order (indprior NULL: every parameter);
 * prior->ndim must equal their number. The prior is copied (covariance, or its
 * Cholesky factor when prior->chol == 1). A second call replaces the first. */
void pmcg_posterior_add_mvdens_prior(pmcg_posterior *p, const mvdens *prior, const int *indprior, error **err);

/* The device posterior that stands in for the caller's posterior callback
 * with this extra pointer (the reference passes &config->base) in the weight
 * step; post NULL removes the entry. The posterior must outlive the entry. */
void pmcg_register_posterior(const void *extra, const pmcg_posterior *post);

/* ------------------------------------------------------------------ *
 * The reference's configuration: data types of its data section      *
 * (wrappers/include/types.h:5-21) and the par_t codes                *
 * (tools/include/par.h:11-33) the device plugins read.               *
 * ------------------------------------------------------------------ */
#define PMCG_DATA_MVDENS     0
#define PMCG_DATA_MIXMVDENS  1
#define PMCG_DATA_SNIA       3
#define PMCG_P_OMEGAM   0   /* p_Omegam */
#define PMCG_P_OMEGADE  2   /* p_Omegade: given -> non-flat, Omega_K = 1 - Omega_m - Omega_de */
#define PMCG_P_H100     3   /* p_h100: absorbed in M for SNe (Manual/manual.tex:1321-1322) */
#define PMCG_P_W0DE    14   /* p_w0de */
#define PMCG_P_M       37   /* p_M: the parameter holds -M (par_files/cosmo_SN.par:9) */
#define PMCG_P_ALPHA   38   /* p_alpha */
#define PMCG_P_BETA    39   /* p_beta: the parameter holds -beta */

/* An SN Ia data set as the reference reads it (read_from_config_SNIa and
 * init_SNIa, wrappers/src/sn.c:20-130; the SN_SALT light-curve columns): peak
 * magnitude m, stretch s, colour c and the covariance of (m, s, c); the SN
 * parameter file's Theta2 = (-M, alpha, -beta) defaults; the cosmology file's
 * Omega_m and w0_de defaults. The distance modulus is m - M + alpha (s - 1)
 * - beta c (Manual/manual.tex:1290-1295). */
typedef struct {
  int nsn;
  const double *z, *m, *s, *c;
  const double *cov6;        /* [nsn*6]: mm, ss, cc, ms, mc, sc */
  double Theta2[3];          /* -M, alpha, -beta */
  double sig_int, v_pec, h;
  double Omega_m, w0_de;
  int chi2mode;              /* PMCG_SN_CHI2_FULL (chi2_simple) or PMCG_SN_CHI2_MARG */
  int add_logdetCov;
  int quad_nodes;            /* Gauss-Legendre nodes per redshift interval (1..16; 0: 4) */
  int special;               /* PMCG_SPECIAL_* (sspecial of the data section) */
} pmcg_snia_config;

/* The device posterior of a reference configuration (config_base,
 * posterior_log_pdf_common, wrappers/src/param.c:958-1041): npar parameters
 * with par_t codes par[] and the flat box [min, max]; ndata data sets of types
 * data[] with states data_state[]: PMCG_DATA_SNIA -> const pmcg_snia_config*,
 * PMCG_DATA_MIXMVDENS -> const mix_mvdens*, PMCG_DATA_MVDENS -> const mvdens*
 * (likeli_MixMvdens / likeli_Mvdens, :1485-1537). The special prior is the
 * first data set's (:998, a_acc as for pmcg_posterior_set_special); prior
 * (NULL: none) is the config prior over the parameters flagged by indprior
 * (:1009-1026). SN parameters follow likeli_SNIa (wrappers/src/sn.c:167-224)
 * and the flatness rules of set_base_parameters (wrappers/src/param.c:
 * 1544-1656): Omega_de absent -> flat. SN parameters the device plugin does not
 * model (Omega_K, the physical densities, w1_de, the polynomial dark energy,
 * log beta, beta_z, stretch/colour offsets, Theta1, beta_d), other data types
 * and an SN data set other than the first are PMCG_EUNSUPPORTED. */
pmcg_posterior *pmcg_posterior_from_config(int npar, const int *par, const double *min, const double *max,
                                           int ndata, const int *data, const void *const *data_state,
                                           const mvdens *prior, const int *indprior, double a_acc, error **err);

/* Single-point log-posterior (the per-point callback shape); evaluates one
 * point on the GPU. Passing this function to the weight step selects the
 * batched device evaluation. */
double pmcg_posterior_log_pdf_void(void *post, const double *x, error **err);

/* Batched log-posterior of N points. X and logpost/flg are host pointers
 * when on_device==0, device pointers otherwise. flg[n] is 0 on a
 * likelihood error. Precision: PMCG_FP64 or PMCG_MIXED. */
#define PMCG_FP64  0
#define PMCG_MIXED 1
void pmcg_posterior_log_pdf_batch(const pmcg_posterior *p, size_t N, const double *X, double *logpost,
                                  short *flg, int on_device, int precision, void *stream, error **err);

/* Fisher matrix F[a*npar + b] = -d^2 log P / d theta_a d theta_b of a posterior
 * at pos, by the reference's central differences (exec/go_fishing.c:37-86):
 * steps h = fh (max - min) with fh = 0.001 (exec/mkmax.h:33), four points per
 * element (the diagonal from f(+2h) - 2 f(0) + f(-2h)); every stencil point of
 * the matrix is evaluated in one batched FP64 device call. Every point must lie
 * in the prior box and pass the likelihood (else PMCG_EARG).
 * diag_only: the diagonal alone, off-diagonal elements 0 (the 'Fisher_diag'
 * initial type, exec/go_fishing.c:100,134). force_positive: afterwards |F_aa|
 * on the diagonal and 0 off it (go_fishing's -f, force_positive, :248-260).
 * Returns 1 when F is positive definite (a Cholesky decomposition succeeds, the
 * test at :433-446), 0 when it is not (F is still written), -1 on error. */
int pmcg_fisher_matrix(const pmcg_posterior *post, const double *pos, const double *min, const double *max,
                       int diag_only, int force_positive, double *F, error **err);
/* Maximum of the posterior by Nelder-Mead simplex searches (Nelder & Mead
 * 1965), the 'amoeba' method of exec/max_post.c:182-224 / exec/mkmax.c:409-520:
 * the objective is -log P, with MC_LOGBIG (1e30 here) outside [min, max] or
 * where the likelihood fails (post_cg, exec/mkmax.c:9-40); the start simplex
 * of a search is its start point and, for each parameter j, the start point
 * moved by (max_j - min_j) / 5 along j; a search stops when
 * 2 |f_hi - f_lo| / (|f_hi| + |f_lo| + 1e-10) < ftol, and more than max_evals
 * evaluations is PMCG_ESTEPS (the reference's NMAX = 5000). The nstart
 * searches (starts: [nstart x npar]) advance together: each round evaluates
 * every active search's trial points in one batched FP64 device call.
 * best: [nstart x npar], each search's best vertex; logp: [nstart] its log P.
 * Returns the index of the search with the highest log P (-1 on error). */
int pmcg_max_posterior(const pmcg_posterior *post, int nstart, const double *starts, const double *min,
                       const double *max, double ftol, int max_evals, double *best, double *logp, error **err);
/* Initial proposal from a Fisher matrix F at pos, as
 * read_initial_proposal_from_config (wrappers/src/param.c:511-625): equal
 * weights, covariances fvar F^-1 (stored in comp->std with chol = 0: decompose
 * with mix_mvdens_cholesky_decomp), means
 *  PMCG_FISHER_RSHIFT: pos shifted per parameter by a uniform draw in
 *    [-fshift (max-min), +fshift (max-min)], redrawn until inside [min, max]
 *    (comp_shift_mean, :472-489; the draws come from rng, one call);
 *  PMCG_FISHER_EIGEN: pos - r, pos + r with r = fshift (lambda_i / lambda_max) e_i
 *    along the eigenvectors of F^-1, largest eigenvalue first (at most 2 npar
 *    components). */
#define PMCG_FISHER_RSHIFT 0
#define PMCG_FISHER_EIGEN 1
void pmcg_fisher_proposal(mix_mvdens *proposal, const double *F, const double *pos, const double *min,
                          const double *max, int type, double fshift, double fvar, pmcg_rng *rng, error **err);

/* Batched mixture log-density of N points (host pointers); lt (optional,
 * [ncomp x N]) receives log(alpha_k) + log f_k(x_n). */
void pmcg_mix_log_pdf_batch(const mix_mvdens *m, size_t N, const double *X, double *logq, double *lt,
                            int precision, error **err);

/* ------------------------------------------------------------------ *
 * Part 2 — device-resident PMC runs                                   *
 * ------------------------------------------------------------------ */
typedef struct pmcg_run pmcg_run;

typedef struct {
  double ln_evidence;  /* logSum - ln N */
  double perplexity;
  double ess;
  double enc;          /* of the updated proposal */
  double logSum;
  double maxW;
  size_t nok;          /* samples with flg==1 */
  int ndead;           /* components with weight 0 after this update */
  int status;          /* 0, or the PMCG_E* code of a failed iteration (batch runs) */
} pmcg_iter_stats;

/* A run keeps its proposal, sample and scratch on the GPU. nsamples is
 * fixed at creation. pb may be NULL (no box). A PMCG_MIXED run refuses a
 * proposal (here and in pmcg_run_set_proposal) with a component narrower than
 * single precision resolves around its mean, max_i sum_j |(L^-1)_ij mu_j| >
 * 2^18 (PMCG_EPRECISION); its EM update buries such a component, as the dead
 * rule buries an update that is not positive definite. */
pmcg_run *pmcg_run_create(const mix_mvdens *proposal, const pmcg_posterior *post, const parabox *pb,
                          size_t nsamples, int precision, uint64_t seed, error **err);
/* One PMC iteration (draw, log q, log posterior, weights, evidence,
 * perplexity, EM update, dead-component burial). stats may be NULL. */
void pmcg_run_iterate(pmcg_run *r, double beta, pmcg_iter_stats *stats, error **err);
/* The same iteration in two halves: _async queues it on the run's stream (a
 * single-precision run replays its CUDA graph without waiting; otherwise the
 * stages run to completion here) and _wait completes it (waits, checks,
 * revives dead components in revive mode, fills stats; the launch's errors are
 * reported here). Iterations of several runs started before any is waited for
 * run concurrently on their streams. One iteration in flight per run: until
 * its _wait, every other call on the run (and a batch holding it) returns
 * PMCG_EARG; pmcg_run_free waits for the stream. */
void pmcg_run_iterate_async(pmcg_run *r, double beta, error **err);
void pmcg_run_iterate_wait(pmcg_run *r, pmcg_iter_stats *stats, error **err);
void pmcg_run_get_proposal(pmcg_run *r, mix_mvdens *out, error **err);
/* Replace the run's proposal (same ncomp/ndim/df), e.g. to restart or to
 * apply a host-side revive step between iterations. */
void pmcg_run_set_proposal(pmcg_run *r, const mix_mvdens *proposal, error **err);
/* Copy the last sample (X, log-weights, flg, indices) into psim. */
void pmcg_run_get_sample(pmcg_run *r, pmc_simu *psim, error **err);
/* Dead components after each update (sdead_comp, exec/cosmo_pmc.c:239-284):
 * PMCG_DEAD_BURY (default) keeps them buried; PMCG_DEAD_REVIVE revives each
 * component whose weight is below 1e-12 as revive_comp does (:205-236): the
 * counter Nrevive doubles at every update (from 1), and each dead component in
 * index order becomes a copy of the component of largest weight (mean and
 * covariance) whose mean is shifted, coordinate by coordinate, by a uniform
 * draw in [-f (max-min), f (max-min)], f = fshift / Nrevive, redrawn while it
 * leaves the box (more than 50 draws for one component: PMCG_ESTEPS); the two
 * share the larger one's weight equally. fshift: 0.1 for the reference's
 * non-Fisher starts (FSHIFT_DEFAULT), its fshift for the Fisher ones. The draws
 * come from the run's random stream (Philox counter {0xFFFFFFF0, component,
 * draw, call}), so a revival is reproducible. Needs the run's prior box. */
#define PMCG_DEAD_BURY   0
#define PMCG_DEAD_REVIVE 1
void pmcg_run_set_dead_comp(pmcg_run *r, int mode, double fshift, error **err);
/* The run's tensor-core setting (1, 0, or -1: the process default of
 * pmcg_set_tensor_cores); returns the previous one (-2 with PMCG_EARG for
 * another value or while an asynchronous iteration is in flight). Two runs in
 * one process can use different settings. */
int pmcg_run_set_tensor_cores(pmcg_run *r, int on, error **err);
void pmcg_run_free(pmcg_run **r);
/* Timing with CUDA events on the run's stream. on = 1: per stage (draw,
 * logq, logpost, weights, em; every kernel launched directly), read with
 * pmcg_run_stage_ms; on = 2: whole iterations as they run in production
 * (single-precision runs replay one captured CUDA graph per iteration), read
 * with pmcg_run_iteration_ms; 0 off. Each call clears the sums; both readers
 * return the number of iterations covered. */
#define PMCG_NSTAGE 5
void pmcg_run_set_timing(pmcg_run *r, int on);
int pmcg_run_stage_ms(pmcg_run *r, double *ms, int nstage);
int pmcg_run_iteration_ms(pmcg_run *r, double *ms);
/* Re-evaluates stage 1 (proposal log-density) or 2 (log-posterior) of the
 * run's current sample reps times on the run's stream and returns the mean
 * milliseconds per evaluation (CUDA events); the results are unchanged. The
 * run must have iterated once. No counterpart in the reference (profiling). */
double pmcg_run_time_stage(pmcg_run *r, int stage, int reps, error **err);
/* Number of kernel launches issued by the last pmcg_run_iterate call. */
int pmcg_run_last_launches(const pmcg_run *r);

/* ------------------------------------------------------------------ *
 * Part 2 — batched runs: one persistent launch per iteration          *
 * ------------------------------------------------------------------ */
/* A batch iterates many independent runs (uneven dimension, component count,
 * sample count and likelihood) with one cooperative kernel per iteration,
 * captured with its copies in a CUDA graph. Every run must be PMCG_MIXED with
 * D <= 32 and a posterior with exactly one likelihood (mixture, SN Ia or
 * template). The runs keep their state (pmcg_run_get_proposal/_sample work as
 * usual) and give the same results as when iterated alone with the
 * CUDA-core log-density (pmcg_set_tensor_cores(0)). The batch references the
 * runs; free it before them. */
typedef struct pmcg_batch pmcg_batch;
pmcg_batch *pmcg_batch_create(int nruns, pmcg_run *const *runs, error **err);
/* Bind another set of runs to an existing batch (its device and pinned arrays
 * are kept and grown when short; the CUDA graph is captured again at the second
 * iteration of the new set). Cheaper than free + create when the set changes
 * often (the serving loop). On failure the batch must be freed. */
void pmcg_batch_rebind(pmcg_batch *b, int nruns, pmcg_run *const *runs, error **err);
/* betas [nruns] (NULL: all 1); stats [nruns] (NULL allowed). A run whose
 * iteration fails reports stats[r].status != 0 without disturbing the others.
 * A failure before the update (no sample in the box: PMCG_ENOWEIGHT) keeps the
 * run's proposal; an update that buries every component (PMCG_ENEGWEIGHT, the
 * reference's pmc_negWeight) leaves the buried proposal, as when the run is
 * iterated alone: give the run a new proposal (pmcg_run_set_proposal) before
 * iterating it again, or its later iterations report PMCG_ENOWEIGHT. */
void pmcg_batch_iterate(pmcg_batch *b, const double *betas, pmcg_iter_stats *stats, error **err);
/* Time the non-mutating stages under each candidate (the grouped SN
 * kernel's threads per block: 64, 128, 256; samples per thread of the
 * log-density stages; resident blocks per SM), keep the fastest and cache it
 * for batches of the same shape. Results do not depend on the choice. */
void pmcg_batch_autotune(pmcg_batch *b, error **err);
void pmcg_batch_config(const pmcg_batch *b, int *samples_per_thread, int *blocks_per_sm, int *grid, int *graph);
/* Threads per block of the grouped SN kernel (the autotuner's third knob). */
int pmcg_batch_sn_block(const pmcg_batch *b);
double pmcg_batch_last_ms(const pmcg_batch *b);
/* Stage timing (profiling): while on, each iteration launches its stages one
 * by one (same stages, same results) with CUDA events between them;
 * pmcg_batch_stage_ms fills ms[PMCG_BATCH_STAGES] with the last iteration's
 * per-stage times (draw, log q, log posterior, subset prior, weight tiles,
 * weight merge, EM weight factor, EM statistics, EM finalise, mixture
 * preparation, renormalise, constants) and returns 0, or -1 when the last
 * iteration was not timed by stage. */
#define PMCG_BATCH_STAGES 12
void pmcg_batch_set_stage_timing(pmcg_batch *b, int on);
int pmcg_batch_stage_ms(const pmcg_batch *b, double *ms);
void pmcg_batch_free(pmcg_batch **b);

/* ------------------------------------------------------------------ *
 * Part 2 — serving: continuous batching of PMC jobs                   *
 * ------------------------------------------------------------------ */
/* A server thread owns the GPU. Jobs are admitted at epoch boundaries while
 * free slots and the device-memory budget allow (a job's footprint is the exact
 * size of its run's buffers); every epoch runs one iteration of all resident
 * jobs in one batch launch, so jobs that arrive while others run join the next
 * epoch and overlap with them. A job's result depends only on its own inputs
 * (same alone and in any mix). Served jobs: D <= 64; jobs with D > 32 or other
 * than one likelihood iterate alone beside the batch, as the large ones. */
typedef struct pmcg_server pmcg_server;
typedef struct {
  size_t hbm_budget_bytes;  /* 0: 80% of the free device memory at creation */
  int max_jobs;             /* resident jobs at most (0: 512) */
  int autotune;             /* tune each new batch shape (cached per shape) */
  int dead_comp;            /* PMCG_DEAD_BURY (0) or PMCG_DEAD_REVIVE for every job with a prior box */
  double fshift;            /* revival shift (0: 0.1) */
  size_t alone_min_samples; /* jobs of at least this many samples iterate with their own CUDA graph on
                               their own stream (tensor-core kernels), beside the batch of the others
                               (0: 2^16; SIZE_MAX: every job the batch takes is batched) */
} pmcg_server_opts;
typedef struct {
  int status;               /* 0 done, > 0 queued/running, < 0 PMCG_E* error */
  int iterations;           /* iterations completed */
  double ln_evidence, perplexity, ess, enc;  /* of the last iteration */
  double submit_s, start_s, finish_s;        /* server clock (s) */
} pmcg_job_result;
typedef struct {
  int queued, resident, peak_resident;
  size_t bytes_in_use, peak_bytes, budget_bytes;
  long long epochs;
} pmcg_server_info_t;
pmcg_server *pmcg_server_create(const pmcg_server_opts *opts, error **err);
/* Thread-safe. The proposal and box are copied; the posterior is referenced
 * and must outlive the job. Tempering as get_tempering_beta(tempering, iter,
 * t_min, niter). Returns the job id (> 0), or 0 with an error. */
int64_t pmcg_server_submit(pmcg_server *s, const mix_mvdens *proposal, const pmcg_posterior *post, const parabox *pb,
                           size_t nsamples, int niter, int tempering, double t_min, uint64_t seed, error **err);
/* Waits at most timeout_s: returns 1 when the job finished (res filled,
 * final_proposal filled if not NULL and the job succeeded), 0 on timeout
 * (PMCG_ETIMEOUT), -1 on an unknown job. */
int pmcg_server_wait(pmcg_server *s, int64_t job, double timeout_s, pmcg_job_result *res,
                     mix_mvdens *final_proposal, error **err);
void pmcg_server_info(pmcg_server *s, pmcg_server_info_t *info);
/* Stops the loop after the current epoch and frees every job. */
void pmcg_server_free(pmcg_server **s);

/* ------------------------------------------------------------------ *
 * Part 2 — importance weights without allocation                      *
 * ------------------------------------------------------------------ */
/* No counterpart in the reference. For callers that cannot let a library
 * allocate device memory (code inside another framework's memory pool,
 * serving loops where an allocation would synchronise the device, runtimes
 * that forbid driver allocations after start-up): the caller passes device
 * arrays logpost[N], logq[N], flg[N] (in/out) and logw[N] (out); the
 * log-weights (beta*logpost - logq, -inf and flg=0 where not finite) are
 * written on `stream` (NULL = default stream) and the scalars are returned in
 * *stats (host). The partial sums use a fixed device array inside the library
 * (one per GPU, held until exit), which limits N to 8,388,608 (larger N:
 * PMCG_EDIM). The first call on a device looks the array up; make it before
 * any stream capture. Each call is synchronous: it waits for `stream` before
 * it returns the scalars. Calls that overlap on the GPU share that array and
 * race. */
typedef struct {
  double logSum, maxW, ln_evidence, perplexity, ess;
  size_t nok;
} pmcg_weight_stats;
void pmcg_importance_weights_noalloc(size_t N, double beta, const double *logpost, const double *logq, short *flg,
                                     double *logw, pmcg_weight_stats *stats, void *stream, error **err);

/* Library / device information. */
const char *pmcg_version(void);
int pmcg_device_count(void);
void pmcg_device_synchronize(error **err);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* PMCG_H */
