/*
 * pmc_oracle.h — FP64 CPU restatement of one CosmoPMC PMC iteration.
 *
 * TEST INFRASTRUCTURE ONLY. The library never links, loads or calls this
 * code; only the tests, the smoke check and the benchmark's CPU-baseline leg
 * use it, to compare the CUDA path's results with.
 *
 * Parity with pmclib/nicaea is unpinned: both are external libraries that
 * the reference clones at install time (install_CosmoPMC.sh:241-266) and
 * that are absent here. This restatement follows the reference call sites
 * (exec/cosmo_pmc.c, wrappers/src/param.c, wrappers/src/sn.c), the formulas
 * of Manual/manual.tex, Cappe et al. 2008 (arXiv:0710.4242) for the
 * Rao-Blackwellised EM update and Wraith et al. 2009 (arXiv:0903.0837,
 * eq. 18) for the perplexity. It is pinned to scipy and analytic answers
 * by tests/golden.
 */
#ifndef PMC_ORACLE_H
#define PMC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 (Salmon et al. 2011) and the random layout of one draw. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_randoms(uint64_t seed, uint32_t call, size_t n0, size_t N, int D, int nu,
                 double *u, double *z, double *chi2);

/* Dense FP64 linear algebra on small D x D row-major matrices. */
int orc_cholesky(int D, const double *C, double *L, double *logdetL);
void orc_cumweights(int K, const double *w, double *cw);

/* (a) draw */
size_t orc_draw(int K, int D, int df, const double *cw, const double *w, const double *mu,
                const double *L, size_t N, const double *u, const double *z, const double *chi2,
                const double *bmin, const double *bmax, double *X, int *idx, short *flg);

/* (b) mixture log-pdf; lt [K x N] and Q [K x N] optional. */
void orc_mix_logpdf(int K, int D, int df, const double *w, const double *mu, const double *L,
                    const double *logdetL, size_t N, const double *X, const short *flg,
                    double *logq, double *lt, double *Q);

/* (c) SN Ia likelihood. Data sorted by redshift is not required. */
typedef struct {
  int nsn;
  const double *z, *mB, *x1, *c, *cov6;
  double sig_int, v_pec, h;
  int chi2mode, add_logdet, quad_nodes;
  int ip_om, ip_ode, ip_w0, ip_M, ip_alpha, ip_beta;
  double def_om, def_w0, def_M, def_alpha, def_beta;
  int neg_M, neg_beta;   /* 1: the parameter holds -M (-beta), par_files/cosmo_SN.par:9 */
} orc_sn;
void orc_gauss_legendre(int G, double *x, double *w);
double orc_sn_loglike_one(const orc_sn *sn, const double *p, int *status);
void orc_sn_loglike(const orc_sn *sn, size_t N, int D, const double *X, const short *flg,
                    double *logL, short *ok);
double orc_lum_dist(double om, double ode, double w0, double h, double z, int G, int nsub, int *status);

/* (c) dense template likelihood (whitened form). */
int orc_tpl_prepare(int M, int P, const double *A, const double *C, const double *dobs,
                    double *At, double *dt);
int orc_tpl_nphi(int D);
void orc_tpl_phi(int D, const double *theta, double *phi);
void orc_tpl_loglike(int M, int D, const double *At, const double *dt, size_t N,
                     const double *X, const short *flg, double *logL);

/* (d) weights, normalisation, evidence, perplexity/ESS, ENC */
void orc_logweights(size_t N, double beta, const double *logpost, const double *logq,
                    const short *flg, double *logw);
int orc_normalize(size_t N, const double *logw, const short *flg, double *wbar,
                  double *logSum, double *maxW);
double orc_perplexity(size_t N, const double *wbar, const short *flg, double *ess);
double orc_enc(int K, const double *w);
double orc_tempering_beta(int type, int iter, double tmin, int nmax);

/* (e) Rao-Blackwellised EM update; w/mu/L/logdetL updated in place.
 * dead[k] = 1 for buried components. Returns 0, or a negative code. */
int orc_update_rb(int K, int D, int df, double *w, double *mu, double *L, double *logdetL,
                  int band_limit, size_t N, const double *X, const double *wbar, const short *flg,
                  const double *lt, const double *logq, const double *Q, const int *idx, int *dead);

/* One whole iteration with a Gaussian-mixture target (the CPU baseline). */
typedef struct {
  double ln_evidence, perplexity, ess, enc, logSum, maxW;
  size_t nok;
  int ndead;
} orc_stats;
int orc_iterate_mix(int K, int D, int df, double *w, double *mu, double *L, double *logdetL,
                    int Kt, int Dt_df, const double *wt, const double *mut, const double *Lt,
                    const double *logdetLt, double logprior, const double *bmin, const double *bmax,
                    size_t N, uint64_t seed, uint32_t call, double beta, orc_stats *st,
                    double *X, double *logw_out, int *idx_out);

int orc_num_threads(void);

/* Special prior (prior_log_pdf_special, wrappers/src/param.c:1055-1101): the
 * constant added once per point to the flat prior. special 0 none, 1 unity,
 * 2 de_conservative (ind_w0/ind_w1 < 0: absent). Returns 0, or -1 when the w0
 * range is narrower than [-1, -1/3] (the reference's mk_special_prior). */
int orc_prior_special(int special, int npar, const double *min, const double *max, int ind_w0, int ind_w1,
                      double a_acc, double *out);

/* Revival of dead components (sdead_comp revive: update_and_deal_with_dead,
 * exec/cosmo_pmc.c:252-275; revive_comp :205-236; comp_shift_mean,
 * wrappers/src/param.c:471-489), the draws from the library's stream (Philox
 * counter {0xFFFFFFF0, component, draw, call} keyed by seed; the reference's
 * gsl_rng is absent). nrevive: the counter after its doubling for this update.
 * w/mu/L updated in place. Returns 0, -1 all weights zero, -2 more than 50
 * draws for one component, -3 invalid weight sum. */
int orc_revive(int K, int D, double *w, double *mu, double *L, const double *bmin, const double *bmax,
               double fshift, int nrevive, uint64_t seed, uint32_t call);

/* Post-processing: marginal centre (mean or median) and one-sided 68.27 /
 * 95.45 / 99.73 % limits per parameter (sigma[6a .. 6a+5]: right, then left),
 * and weighted histograms (exec/exec_helper.c:63-271,
 * wrappers/src/param.c:1229-1357). */
void orc_weighted_summary(size_t N, int D, const double *X, const double *wbar, const short *flg, int use_median,
                          double *center, double *sigma, int *status);
void orc_hist1d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin, const double *lo,
                const double *hi, double scale, double *hist);
void orc_hist2d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin, int p, int q,
                const double *lo, const double *hi, double scale, double *hist);

#ifdef __cplusplus
}
#endif

#endif
