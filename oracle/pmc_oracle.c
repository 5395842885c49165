/*
 * pmc_oracle.c — FP64 CPU restatement of one CosmoPMC PMC iteration.
 *
 * TEST INFRASTRUCTURE ONLY: the results libpmcg's CUDA path is compared with, and the
 * timed CPU baseline. Nothing in the library links or calls it.
 *
 * Parity with pmclib/nicaea is unpinned (both external and absent); the
 * formulas follow the reference call sites and manual cited per function,
 * and tests/golden pins them to scipy and analytic answers.
 */
#include "pmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846
#define ORC_LN2PI 1.83787706640934548356
#define ORC_C_KMS 299792.458
#define ORC_MINCOUNT 20
#define ORC_ECHOL (-9003)
#define ORC_ENEGWEIGHT (-9005)
#define ORC_ENOWEIGHT (-9011)
#define ORC_EALLOC (-9007)

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------- *
 * Philox4x32-10, Salmon, Moraes, Dror & Shaw, SC'11, "Parallel      *
 * random numbers: as easy as 1, 2, 3" (round function and constants *
 * as published there).                                              *
 * ---------------------------------------------------------------- */
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 53-bit dyadic uniform in [0,1) from two 32-bit words. */
static inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* Random layout of one draw call for sample n (counter {slot, n_lo, n_hi,
 * call}, key = seed): slot 0 words 0-1 = component uniform; slot 1+m gives
 * normals 2m, 2m+1 by Box-Muller. Normals 0..D-1 are the Gaussian vector,
 * D..D+nu-1 build the chi^2_nu variate of the Student-t draw. */
void orc_randoms(uint64_t seed, uint32_t call, size_t n0, size_t N, int D, int nu,
                 double *u, double *z, double *chi2) {
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  int nn = D + (nu > 0 ? nu : 0);
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)N; ii++) {
    size_t n = n0 + (size_t)ii;
    uint32_t ctr[4] = {0u, (uint32_t)n, (uint32_t)((uint64_t)n >> 32), call};
    uint32_t o[4];
    orc_philox(ctr, key, o);
    u[ii] = u53(o[0], o[1]);
    double c2 = 0.0;
    for (int m = 0; 2 * m < nn; m++) {
      ctr[0] = 1u + (uint32_t)m;
      orc_philox(ctr, key, o);
      double a = u53(o[0], o[1]), b = u53(o[2], o[3]);
      double r = sqrt(-2.0 * log1p(-a));
      double t = 2.0 * ORC_PI * b;
      double g[2] = {r * cos(t), r * sin(t)};
      for (int e = 0; e < 2; e++) {
        int j = 2 * m + e;
        if (j < D) z[(size_t)ii * D + j] = g[e];
        else if (j < nn) c2 += g[e] * g[e];
      }
    }
    if (chi2) chi2[ii] = (nu > 0) ? c2 : 1.0;
  }
}

/* ---------------------------------------------------------------- *
 * Cholesky (mvdens_cholesky_decomp, wrappers/src/param.c:56,1476)   *
 * ---------------------------------------------------------------- */
int orc_cholesky(int D, const double *C, double *L, double *logdetL) {
  double ld = 0.0;
  for (int i = 0; i < D * D; i++) L[i] = 0.0;
  for (int j = 0; j < D; j++) {
    double s = C[j * D + j];
    for (int k = 0; k < j; k++) s -= L[j * D + k] * L[j * D + k];
    if (!(s > 0.0) || !isfinite(s)) return ORC_ECHOL;
    double d = sqrt(s);
    L[j * D + j] = d;
    ld += log(d);
    for (int i = j + 1; i < D; i++) {
      double t = C[i * D + j];
      for (int k = 0; k < j; k++) t -= L[i * D + k] * L[j * D + k];
      L[i * D + j] = t / d;
    }
  }
  if (logdetL) *logdetL = ld;
  return 0;
}

/* Cumulative weights, summed in component order. */
void orc_cumweights(int K, const double *w, double *cw) {
  double s = 0.0;
  for (int k = 0; k < K; k++) { s += w[k]; cw[k] = s; }
}

/* ---------------------------------------------------------------- *
 * (a) Draw (simulate_mix_mvdens, exec/cosmo_pmc.c:320). Component   *
 * k = min{k : u < C_k}; x = mu_k + L_k z (* sqrt(nu/chi2) for t).   *
 * Points outside [bmin,bmax] get flg = 0 (no redraw).               *
 * ---------------------------------------------------------------- */
size_t orc_draw(int K, int D, int df, const double *cw, const double *w, const double *mu,
                const double *L, size_t N, const double *u, const double *z, const double *chi2,
                const double *bmin, const double *bmax, double *X, int *idx, short *flg) {
  int klast = -1;
  for (int k = 0; k < K; k++) if (w[k] > 0.0) klast = k;
  size_t nok = 0;
#pragma omp parallel for schedule(static) reduction(+ : nok)
  for (long long nn = 0; nn < (long long)N; nn++) {
    size_t n = (size_t)nn;
    int k = klast;
    for (int j = 0; j < K; j++) if (u[n] < cw[j]) { k = j; break; }
    double s = (df > 0) ? sqrt((double)df / chi2[n]) : 1.0;
    const double *Lk = L + (size_t)k * D * D;
    const double *zn = z + n * D;
    int in = 1;
    for (int i = 0; i < D; i++) {
      double acc = 0.0;
      for (int j = 0; j <= i; j++) acc += Lk[i * D + j] * zn[j];
      double xi = mu[(size_t)k * D + i] + s * acc;
      X[n * D + i] = xi;
      if (bmin && (xi < bmin[i] || xi > bmax[i])) in = 0;
    }
    idx[n] = k;
    flg[n] = (short)in;
    nok += (size_t)in;
  }
  return nok;
}

/* ---------------------------------------------------------------- *
 * (b) Mixture log-pdf (mix_mvdens_log_pdf, exec/cosmo_pmc.c:343).   *
 * Gaussian: -Q/2 - log|L| - D/2 log 2pi; Student-t: lgamma terms    *
 * - (nu+D)/2 log(1+Q/nu). lt = log alpha_k + log f_k, logq = LSE.   *
 * ---------------------------------------------------------------- */
void orc_mix_logpdf(int K, int D, int df, const double *w, const double *mu, const double *L,
                    const double *logdetL, size_t N, const double *X, const short *flg,
                    double *logq, double *lt, double *Q) {
  (void)flg;
  double cst;
  if (df > 0) {
    double nu = (double)df;
    cst = lgamma(0.5 * (nu + D)) - lgamma(0.5 * nu) - 0.5 * D * log(nu * ORC_PI);
  } else {
    cst = -0.5 * D * ORC_LN2PI;
  }
#pragma omp parallel
  {
    double *y = (double *)malloc(sizeof(double) * (size_t)D);
    double *l = (double *)malloc(sizeof(double) * (size_t)K);
#pragma omp for schedule(static)
    for (long long nn = 0; nn < (long long)N; nn++) {
      size_t n = (size_t)nn;
      const double *x = X + n * D;
      double m = -INFINITY;
      for (int k = 0; k < K; k++) {
        const double *Lk = L + (size_t)k * D * D;
        double q = 0.0;
        for (int i = 0; i < D; i++) {
          double t = x[i] - mu[(size_t)k * D + i];
          for (int j = 0; j < i; j++) t -= Lk[i * D + j] * y[j];
          y[i] = t / Lk[i * D + i];
          q += y[i] * y[i];
        }
        double lf;
        if (df > 0) lf = cst - logdetL[k] - 0.5 * (df + D) * log1p(q / df);
        else lf = cst - logdetL[k] - 0.5 * q;
        l[k] = (w[k] > 0.0) ? log(w[k]) + lf : -INFINITY;
        if (l[k] > m) m = l[k];
        if (lt) lt[(size_t)k * N + n] = l[k];
        if (Q) Q[(size_t)k * N + n] = q;
      }
      double s = 0.0;
      for (int k = 0; k < K; k++) s += exp(l[k] - m);
      logq[n] = m + log(s);
    }
    free(y);
    free(l);
  }
}

/* ---------------------------------------------------------------- *
 * (c) SN Ia likelihood (likeli_SNIa, wrappers/src/sn.c:138-281;     *
 * chi^2 of Manual/manual.tex:1290-1365, SALT2 x1 form; M optionally *
 * marginalised, Goliath et al. 2001).                               *
 * ---------------------------------------------------------------- */
void orc_gauss_legendre(int G, double *x, double *w) {
  /* Newton iteration on P_G from the Chebyshev guess. */
  for (int i = 0; i < G; i++) {
    double t = cos(ORC_PI * (i + 0.75) / (G + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= G; k++) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      if (G == 1) { p1 = t; p0 = 1.0; }
      dp = G * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / dp;
      t -= dt;
      if (fabs(dt) < 1e-16) break;
    }
    {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= G; k++) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      if (G == 1) { p1 = t; p0 = 1.0; }
      dp = G * (t * p1 - p0) / (t * t - 1.0);
    }
    x[i] = t;
    w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
  }
}

static inline double inv_E(double om, double ok, double ode, double w0, double z, int *bad) {
  double a = 1.0 + z;
  double e2 = om * a * a * a + ok * a * a + ode * exp(3.0 * (1.0 + w0) * log(a));
  if (!(e2 > 0.0)) { *bad = 1; return 0.0; }
  return 1.0 / sqrt(e2);
}

/* Transverse comoving distance in units of c/H0 from I = int dz/E. */
static inline double sk_of(double ok, double I, int *bad) {
  if (fabs(ok) < 1e-10) return I * (1.0 + ok * I * I / 6.0);
  if (ok > 0.0) { double s = sqrt(ok); return sinh(s * I) / s; }
  double s = sqrt(-ok);
  if (s * I >= ORC_PI) { *bad = 1; return 0.0; }
  return sin(s * I) / s;
}

double orc_lum_dist(double om, double ode, double w0, double h, double z, int G, int nsub, int *status) {
  double xg[16], wg[16];
  orc_gauss_legendre(G, xg, wg);
  double ok = 1.0 - om - ode, I = 0.0;
  int bad = 0;
  for (int s = 0; s < nsub; s++) {
    double a = z * s / nsub, b = z * (s + 1) / nsub, hw = 0.5 * (b - a), c = 0.5 * (a + b);
    for (int g = 0; g < G; g++) I += hw * wg[g] * inv_E(om, ok, ode, w0, c + hw * xg[g], &bad);
  }
  inv_E(om, ok, ode, w0, z, &bad);
  double dm = sk_of(ok, I, &bad);
  *status = !bad;
  return (1.0 + z) * (ORC_C_KMS / (100.0 * h)) * dm;
}

static int cmp_dbl_idx(const void *a, const void *b, void *ctx) {
  const double *z = (const double *)ctx;
  double za = z[*(const int *)a], zb = z[*(const int *)b];
  if (za < zb) return -1;
  if (za > zb) return 1;
  return (*(const int *)a) - (*(const int *)b);
}

/* Sorting with a context pointer, portable (insertion sort on indices; nsn
 * is at most a few thousand and this runs once per call in the oracle). */
static void sort_idx(int n, int *ix, const double *z) {
  for (int i = 0; i < n; i++) ix[i] = i;
  for (int i = 1; i < n; i++) {
    int v = ix[i], j = i - 1;
    while (j >= 0 && cmp_dbl_idx(&ix[j], &v, (void *)z) > 0) { ix[j + 1] = ix[j]; j--; }
    ix[j + 1] = v;
  }
}

static double sn_loglike_sorted(const orc_sn *sn, const int *ix, const double *xg, const double *wg,
                                const double *p, int *status) {
  double om = sn->ip_om >= 0 ? p[sn->ip_om] : sn->def_om;
  double ode, ok;
  if (sn->ip_ode >= 0) { ode = p[sn->ip_ode]; ok = 1.0 - om - ode; }
  else { ode = 1.0 - om; ok = 0.0; }
  double w0 = sn->ip_w0 >= 0 ? p[sn->ip_w0] : sn->def_w0;
  double M = sn->ip_M >= 0 ? (sn->neg_M ? -p[sn->ip_M] : p[sn->ip_M]) : sn->def_M;
  double al = sn->ip_alpha >= 0 ? p[sn->ip_alpha] : sn->def_alpha;
  double be = sn->ip_beta >= 0 ? (sn->neg_beta ? -p[sn->ip_beta] : p[sn->ip_beta]) : sn->def_beta;
  double dh = ORC_C_KMS / (100.0 * sn->h);
  int G = sn->quad_nodes, bad = 0;
  double I = 0.0, zprev = 0.0;
  double A = 0.0, B = 0.0, C = 0.0, chi2 = 0.0, sl = 0.0;
  for (int t = 0; t < sn->nsn; t++) {
    int i = ix[t];
    double zi = sn->z[i], hw = 0.5 * (zi - zprev), cc = 0.5 * (zi + zprev);
    for (int g = 0; g < G; g++) I += hw * wg[g] * inv_E(om, ok, ode, w0, cc + hw * xg[g], &bad);
    inv_E(om, ok, ode, w0, zi, &bad);
    zprev = zi;
    double dm = sk_of(ok, I, &bad);
    if (bad || !(dm > 0.0)) { *status = 0; return 0.0; }
    double mu_th = 5.0 * log10((1.0 + zi) * dh * dm) + 25.0;
    const double *W = sn->cov6 + (size_t)i * 6;
    double spv = (5.0 / log(10.0)) * sn->v_pec / (ORC_C_KMS * zi);
    double s2 = W[0] + al * al * W[1] + be * be * W[2] + 2.0 * al * W[3] - 2.0 * be * W[4] -
                2.0 * al * be * W[5] + sn->sig_int * sn->sig_int + spv * spv;
    if (!(s2 > 0.0)) { *status = 0; return 0.0; }
    double d = sn->mB[i] + al * sn->x1[i] - be * sn->c[i] - mu_th;
    if (sn->chi2mode == 0) { d -= M; chi2 += d * d / s2; }
    else { A += d * d / s2; B += d / s2; C += 1.0 / s2; }
    sl += log(s2);
  }
  if (sn->chi2mode != 0) chi2 = A - B * B / C + log(C / (2.0 * ORC_PI));
  double ll = -0.5 * chi2 - (sn->add_logdet ? 0.5 * sl : 0.0);
  *status = isfinite(ll) ? 1 : 0;
  return ll;
}

double orc_sn_loglike_one(const orc_sn *sn, const double *p, int *status) {
  double xg[16], wg[16];
  orc_gauss_legendre(sn->quad_nodes, xg, wg);
  int *ix = (int *)malloc(sizeof(int) * (size_t)sn->nsn);
  sort_idx(sn->nsn, ix, sn->z);
  double r = sn_loglike_sorted(sn, ix, xg, wg, p, status);
  free(ix);
  return r;
}

void orc_sn_loglike(const orc_sn *sn, size_t N, int D, const double *X, const short *flg,
                    double *logL, short *ok) {
  double xg[16], wg[16];
  orc_gauss_legendre(sn->quad_nodes, xg, wg);
  int *ix = (int *)malloc(sizeof(int) * (size_t)sn->nsn);
  sort_idx(sn->nsn, ix, sn->z);
#pragma omp parallel for schedule(dynamic, 16)
  for (long long nn = 0; nn < (long long)N; nn++) {
    size_t n = (size_t)nn;
    if (flg && !flg[n]) { logL[n] = 0.0; if (ok) ok[n] = 0; continue; }
    int st = 1;
    logL[n] = sn_loglike_sorted(sn, ix, xg, wg, X + n * D, &st);
    if (ok) ok[n] = (short)st;
  }
  free(ix);
}

/* ---------------------------------------------------------------- *
 * (c) Dense template likelihood. C = L L^T (FP64), At = L^-1 A,     *
 * dt = L^-1 dobs, logL = -1/2 |dt - At phi|^2. Structural analogue  *
 * of likeli_Mvdens (wrappers/src/param.c:1485-1493).                *
 * ---------------------------------------------------------------- */
int orc_tpl_nphi(int D) { return 1 + D + D * (D + 1) / 2; }

void orc_tpl_phi(int D, const double *th, double *phi) {
  int p = 0;
  phi[p++] = 1.0;
  for (int i = 0; i < D; i++) phi[p++] = th[i];
  for (int i = 0; i < D; i++)
    for (int j = i; j < D; j++) phi[p++] = th[i] * th[j];
}

int orc_tpl_prepare(int M, int P, const double *A, const double *C, const double *dobs,
                    double *At, double *dt) {
  double *L = (double *)malloc(sizeof(double) * (size_t)M * M);
  if (!L) return ORC_EALLOC;
  int rc = orc_cholesky(M, C, L, NULL);
  if (rc) { free(L); return rc; }
  /* forward substitution, column by column of [A | dobs] */
  for (int i = 0; i < M; i++) {
    const double *Li = L + (size_t)i * M;
    for (int p = 0; p < P; p++) {
      double t = A[(size_t)i * P + p];
      for (int j = 0; j < i; j++) t -= Li[j] * At[(size_t)j * P + p];
      At[(size_t)i * P + p] = t / Li[i];
    }
    double t = dobs[i];
    for (int j = 0; j < i; j++) t -= Li[j] * dt[j];
    dt[i] = t / Li[i];
  }
  free(L);
  return 0;
}

void orc_tpl_loglike(int M, int D, const double *At, const double *dt, size_t N,
                     const double *X, const short *flg, double *logL) {
  int P = orc_tpl_nphi(D);
#pragma omp parallel
  {
    double *phi = (double *)malloc(sizeof(double) * (size_t)P);
#pragma omp for schedule(static)
    for (long long nn = 0; nn < (long long)N; nn++) {
      size_t n = (size_t)nn;
      if (flg && !flg[n]) { logL[n] = 0.0; continue; }
      orc_tpl_phi(D, X + n * D, phi);
      double chi2 = 0.0;
      for (int m = 0; m < M; m++) {
        double r = dt[m];
        for (int p = 0; p < P; p++) r -= At[(size_t)m * P + p] * phi[p];
        chi2 += r * r;
      }
      logL[n] = -0.5 * chi2;
    }
    free(phi);
  }
}

/* ---------------------------------------------------------------- *
 * (d) Importance weights, normalisation, evidence, perplexity/ESS,   *
 * ENC (exec/cosmo_pmc.c:46-87,343-378; Manual/manual.tex:556-610).  *
 * ---------------------------------------------------------------- */
void orc_logweights(size_t N, double beta, const double *logpost, const double *logq,
                    const short *flg, double *logw) {
  for (size_t n = 0; n < N; n++) {
    double l = beta * logpost[n] - logq[n];
    logw[n] = (flg[n] && isfinite(l)) ? l : -INFINITY;
  }
}

int orc_normalize(size_t N, const double *logw, const short *flg, double *wbar,
                  double *logSum, double *maxW) {
  double m = -INFINITY;
  for (size_t n = 0; n < N; n++) if (flg[n] && logw[n] > m) m = logw[n];
  if (!isfinite(m)) return ORC_ENOWEIGHT;
  double s = 0.0;
  for (size_t n = 0; n < N; n++) if (flg[n]) s += exp(logw[n] - m);
  double ls = m + log(s);
  for (size_t n = 0; n < N; n++) wbar[n] = flg[n] ? exp(logw[n] - ls) : 0.0;
  *logSum = ls;
  *maxW = m;
  return 0;
}

double orc_perplexity(size_t N, const double *wbar, const short *flg, double *ess) {
  double H = 0.0, s2 = 0.0;
  for (size_t n = 0; n < N; n++) {
    if (!flg[n] || !(wbar[n] > 0.0)) continue;
    H -= wbar[n] * log(wbar[n]);
    s2 += wbar[n] * wbar[n];
  }
  if (ess) *ess = 1.0 / s2;
  return exp(H) / (double)N;
}

double orc_enc(int K, const double *w) {
  double s = 0.0;
  for (int k = 0; k < K; k++) s += w[k] * w[k];
  return 1.0 / s;
}

/* get_tempering_beta (exec/cosmo_pmc.c:464-495). */
double orc_tempering_beta(int type, int iter, double tmin, int nmax) {
  if (type == 0) return 1.0;
  if (iter == nmax - 1) return 1.0;
  if (type == 1) return (double)iter / (nmax - 2.0) * (1.0 - tmin) + tmin;
  return exp((double)iter / (nmax - 2.0) * (-log(tmin)) + log(tmin));
}

/* ---------------------------------------------------------------- *
 * (e) Rao-Blackwellised EM (update_prop_rb, exec/cosmo_pmc.c:247;   *
 * Cappe et al. 2008). rho = alpha_k f_k / q; Student-t tau =        *
 * (nu+D)/(nu+Q) in the mean and covariance numerators and the mean  *
 * normaliser. Dead rule: fewer than 20 draws or weight < 1/N        *
 * (Manual/manual.tex:479-490), or a non-positive-definite update.   *
 * ---------------------------------------------------------------- */
int orc_update_rb(int K, int D, int df, double *w, double *mu, double *L, double *logdetL,
                  int band_limit, size_t N, const double *X, const double *wbar, const short *flg,
                  const double *lt, const double *logq, const double *Q, const int *idx, int *dead) {
  double *nw = (double *)calloc((size_t)K, sizeof(double));
  size_t *cnt = (size_t *)calloc((size_t)K, sizeof(size_t));
  if (!nw || !cnt) { free(nw); free(cnt); return ORC_EALLOC; }
  for (size_t n = 0; n < N; n++) if (idx[n] >= 0 && idx[n] < K) cnt[idx[n]]++;
#pragma omp parallel
  {
    double *m1 = (double *)malloc(sizeof(double) * (size_t)D);
    double *S = (double *)malloc(sizeof(double) * (size_t)D * D);
    double *Lk = (double *)malloc(sizeof(double) * (size_t)D * D);
#pragma omp for schedule(dynamic, 1)
    for (int k = 0; k < K; k++) {
      dead[k] = 0;
      if (!(w[k] > 0.0)) { dead[k] = 1; nw[k] = 0.0; continue; }
      double s0 = 0.0, st = 0.0;
      for (int i = 0; i < D; i++) m1[i] = 0.0;
      for (size_t n = 0; n < N; n++) {
        if (!flg[n] || wbar[n] == 0.0) continue;
        double v = wbar[n] * exp(lt[(size_t)k * N + n] - logq[n]);
        double tau = (df > 0) ? (df + D) / (df + Q[(size_t)k * N + n]) : 1.0;
        s0 += v;
        st += v * tau;
        for (int i = 0; i < D; i++) m1[i] += v * tau * X[n * D + i];
      }
      if (!(st > 0.0) || cnt[k] < ORC_MINCOUNT || s0 < 1.0 / (double)N) {
        dead[k] = 1; nw[k] = 0.0; continue;
      }
      for (int i = 0; i < D; i++) m1[i] /= st;
      for (int i = 0; i < D * D; i++) S[i] = 0.0;
      for (size_t n = 0; n < N; n++) {
        if (!flg[n] || wbar[n] == 0.0) continue;
        double v = wbar[n] * exp(lt[(size_t)k * N + n] - logq[n]);
        double tau = (df > 0) ? (df + D) / (df + Q[(size_t)k * N + n]) : 1.0;
        const double *x = X + n * D;
        for (int i = 0; i < D; i++)
          for (int j = 0; j <= i; j++) S[i * D + j] += v * tau * (x[i] - m1[i]) * (x[j] - m1[j]);
      }
      for (int i = 0; i < D; i++)
        for (int j = 0; j <= i; j++) {
          double c = S[i * D + j] / s0;
          if (band_limit > 0 && i - j >= band_limit) c = 0.0;
          S[i * D + j] = c;
          S[j * D + i] = c;
        }
      double ld;
      if (orc_cholesky(D, S, Lk, &ld) != 0) { dead[k] = 1; nw[k] = 0.0; continue; }
      nw[k] = s0;
      memcpy(mu + (size_t)k * D, m1, sizeof(double) * (size_t)D);
      memcpy(L + (size_t)k * D * D, Lk, sizeof(double) * (size_t)D * D);
      logdetL[k] = ld;
    }
    free(m1);
    free(S);
    free(Lk);
  }
  double tot = 0.0;
  for (int k = 0; k < K; k++) tot += nw[k];
  int rc = 0;
  if (!(tot > 0.0)) rc = ORC_ENEGWEIGHT;
  else for (int k = 0; k < K; k++) w[k] = nw[k] / tot;
  free(nw);
  free(cnt);
  return rc;
}

/* ---------------------------------------------------------------- *
 * One whole iteration with a Gaussian-mixture target               *
 * (run_pmc_iteration_MPI + post_processing, exec/cosmo_pmc.c:293-   *
 * 461, single process).                                             *
 * ---------------------------------------------------------------- */
int orc_iterate_mix(int K, int D, int df, double *w, double *mu, double *L, double *logdetL,
                    int Kt, int t_df, const double *wt, const double *mut, const double *Lt,
                    const double *logdetLt, double logprior, const double *bmin, const double *bmax,
                    size_t N, uint64_t seed, uint32_t call, double beta, orc_stats *st,
                    double *X_out, double *logw_out, int *idx_out) {
  int rc = 0;
  double *u = malloc(sizeof(double) * N), *z = malloc(sizeof(double) * N * D);
  double *chi2 = malloc(sizeof(double) * N), *X = X_out ? X_out : malloc(sizeof(double) * N * D);
  int *idx = idx_out ? idx_out : malloc(sizeof(int) * N);
  short *flg = malloc(sizeof(short) * N);
  double *logq = malloc(sizeof(double) * N), *lp = malloc(sizeof(double) * N);
  double *lt = malloc(sizeof(double) * N * K), *Q = malloc(sizeof(double) * N * K);
  double *logw = logw_out ? logw_out : malloc(sizeof(double) * N), *wbar = malloc(sizeof(double) * N);
  double *cw = malloc(sizeof(double) * K);
  int *dead = malloc(sizeof(int) * K);
  if (!u || !z || !chi2 || !X || !idx || !flg || !logq || !lp || !lt || !Q || !logw || !wbar || !cw || !dead) {
    rc = ORC_EALLOC;
    goto out;
  }
  orc_randoms(seed, call, 0, N, D, df, u, z, chi2);
  orc_cumweights(K, w, cw);
  orc_draw(K, D, df, cw, w, mu, L, N, u, z, chi2, bmin, bmax, X, idx, flg);
  orc_mix_logpdf(K, D, df, w, mu, L, logdetL, N, X, NULL, logq, lt, Q);
  orc_mix_logpdf(Kt, D, t_df, wt, mut, Lt, logdetLt, N, X, NULL, lp, NULL, NULL);
  for (size_t n = 0; n < N; n++) lp[n] += logprior;
  orc_logweights(N, beta, lp, logq, flg, logw);
  size_t nok = 0;
  for (size_t n = 0; n < N; n++) { if (!isfinite(logw[n])) flg[n] = 0; nok += (size_t)(flg[n] != 0); }
  double ls, mw;
  rc = orc_normalize(N, logw, flg, wbar, &ls, &mw);
  if (rc) goto out;
  if (st) {
    st->logSum = ls;
    st->maxW = mw;
    st->ln_evidence = ls - log((double)N);
    st->perplexity = orc_perplexity(N, wbar, flg, &st->ess);
    st->nok = nok;
  }
  rc = orc_update_rb(K, D, df, w, mu, L, logdetL, D, N, X, wbar, flg, lt, logq, Q, idx, dead);
  if (st) {
    st->enc = orc_enc(K, w);
    st->ndead = 0;
    for (int k = 0; k < K; k++) st->ndead += dead[k];
  }
out:
  free(u); free(z); free(chi2);
  if (!X_out) free(X);
  if (!idx_out) free(idx);
  free(flg); free(logq); free(lp); free(lt); free(Q);
  if (!logw_out) free(logw);
  free(wbar); free(cw); free(dead);
  return rc;
}

/* ------------------------------------------------------------------ post-processing
 * Marginal summaries and histograms of a weighted sample, following
 * exec/exec_helper.c:63-271 (mean_sigma_from_psim, median_from_psim,
 * sigma_from_psim) with the counted samples compacted (the reference copies
 * them to tmp[i] by sample index but sorts the first n entries), the scan
 * for imean capped at the last sample, and a median whose first sample carries
 * more than half of the weight taken as that sample; and the weighted
 * histograms of wrappers/src/param.c:1229-1357 with the binning pinned in
 * include/pmcg.h (pmclib's accumulation is absent). Sequential sums in the
 * reference's order. */
typedef struct { double par, w; } orc_pw;
static int orc_pw_cmp(const void *a, const void *b) {
  const double x = ((const orc_pw *)a)->par, y = ((const orc_pw *)b)->par;
  return (x < y) ? -1 : (x > y);
}

/* status[a]: 0 ok, 1 no counted sample, 2 the weights do not reach 1/2 */
void orc_weighted_summary(size_t N, int D, const double *X, const double *wbar, const short *flg, int use_median,
                          double *center, double *sigma, int *status) {
  const double conf[3] = {0.682689492137085897 / 2.0, 0.954499736103641585 / 2.0, 0.997300203936739810 / 2.0};
  orc_pw *t = (orc_pw *)malloc(sizeof(orc_pw) * (N ? N : 1));
  for (int a = 0; a < D; a++) {
    size_t n = 0;
    double mean = 0.0;
    for (size_t i = 0; i < N; i++) {
      if (flg[i] == 0) continue;
      mean += wbar[i] * X[i * D + a];
      t[n].par = X[i * D + a];
      t[n].w = wbar[i];
      n++;
    }
    status[a] = 0;
    if (n == 0) { status[a] = 1; continue; }
    qsort(t, n, sizeof(orc_pw), orc_pw_cmp);
    double c = mean;
    if (use_median) {
      double m = 0.0;
      size_t i;
      for (i = 0; i < n; i++) {
        m += t[i].w;
        if (m == 0.5) { c = t[i].par; break; }
        if (m > 0.5) { c = (i == 0) ? t[0].par : 0.5 * (t[i].par + t[i - 1].par); break; }
      }
      if (i == n) { status[a] = 2; continue; }
    }
    size_t imean = 0;
    while (t[imean].par < c && imean < n - 1) imean++;
    for (int j = 0; j < 3; j++) {
      double sum = 0.0;
      size_t i = imean;
      while (sum <= conf[j] && i < n) { sum += t[i].w; i++; }
      sigma[6 * a + j] = (i == n) ? -1.0 : t[i].par - c;
    }
    for (int j = 0; j < 3; j++) {
      double sum = 0.0;
      long long i = (long long)imean - 1;
      while (sum <= conf[j] && i >= 0) { sum += t[i].w; i--; }
      sigma[6 * a + 3 + j] = (i == -1) ? -1.0 : c - t[i].par;
    }
    center[a] = c;
  }
  free(t);
}

static double orc_edge(double lo, double hi, int nbin, int j) {
  return (j == nbin) ? hi : lo + (hi - lo) * (double)j / (double)nbin;
}
static int orc_bin(double x, double lo, double hi, int nbin) {
  if (!(x >= lo && x <= hi)) return -1;
  int j = (int)floor((x - lo) / (hi - lo) * (double)nbin);
  j = j < 0 ? 0 : (j > nbin - 1 ? nbin - 1 : j);
  if (x < orc_edge(lo, hi, nbin, j)) j--;
  else if (j < nbin - 1 && x >= orc_edge(lo, hi, nbin, j + 1)) j++;
  return j;
}

void orc_hist1d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin, const double *lo,
                const double *hi, double scale, double *hist) {
  memset(hist, 0, sizeof(double) * (size_t)D * nbin);
  for (int a = 0; a < D; a++)
    for (size_t i = 0; i < N; i++) {
      if (!flg[i]) continue;
      const int b = orc_bin(X[i * D + a], lo[a], hi[a], nbin);
      if (b >= 0) hist[(size_t)a * nbin + b] += wbar[i] * scale;
    }
}

void orc_hist2d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin, int p, int q,
                const double *lo, const double *hi, double scale, double *hist) {
  memset(hist, 0, sizeof(double) * (size_t)nbin * nbin);
  for (size_t i = 0; i < N; i++) {
    if (!flg[i]) continue;
    const int bp = orc_bin(X[i * D + p], lo[p], hi[p], nbin), bq = orc_bin(X[i * D + q], lo[q], hi[q], nbin);
    if (bp >= 0 && bq >= 0) hist[(size_t)bp * nbin + bq] += wbar[i] * scale;
  }
}

/* ---------------------------------------------------------------- special prior
 * prior_log_pdf_special, wrappers/src/param.c:1055-1101: unity returns
 * sum log(max - min) (minus the default flat prior); de_conservative returns
 * the box volume of w0 (and w1) minus the special prior's volume, and fails
 * when the w0 range is narrower than [-1, -1/3] (:1082-1084). */
int orc_prior_special(int special, int npar, const double *min, const double *max, int ind_w0, int ind_w1,
                      double a_acc, double *out) {
  *out = 0.0;
  if (special == 1) {
    double s = 0.0;
    for (int i = 0; i < npar; i++) s += log(max[i] - min[i]);
    *out = s;
    return 0;
  }
  if (special != 2 || ind_w0 < 0) return 0;
  if (min[ind_w0] > -1.0 || max[ind_w0] < -1.0 / 3.0) return -1;
  if (ind_w1 < 0) {
    *out = log(max[ind_w0] - min[ind_w0]) - log(2.0 / 3.0);
  } else {
    *out = log(max[ind_w0] - min[ind_w0]) + log(max[ind_w1] - min[ind_w1]) -
           log(0.5 * 2.0 / 3.0 * 2.0 / 3.0 / (1.0 - a_acc)) - log(0.5 * 2.0 / 3.0 * 2.0 / 3.0);
  }
  return 0;
}

/* ---------------------------------------------------------------- revival
 * The revive branch of update_and_deal_with_dead (exec/cosmo_pmc.c:252-275):
 * each component of weight below 1e-12, in index order, becomes a copy of the
 * component of largest weight (revive_comp, :205-236) whose mean is shifted by
 * comp_shift_mean (wrappers/src/param.c:471-489): per coordinate a uniform
 * shift in [-f box, f box], f = fshift / nrevive, redrawn while outside the
 * box, at most 50 draws in all; the two then share the larger weight. */
int orc_revive(int K, int D, double *w, double *mu, double *L, const double *bmin, const double *bmax,
               double fshift, int nrevive, uint64_t seed, uint32_t call) {
  const double fs = fshift / (double)nrevive;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (int i = 0; i < K; i++) {
    if (!(w[i] < 1e-12)) continue;
    int imax = -1;
    double wmax = 0.0;
    for (int j = 0; j < K; j++)
      if (w[j] > wmax) { wmax = w[j]; imax = j; }
    if (imax < 0) return -1;
    memcpy(L + (size_t)i * D * D, L + (size_t)imax * D * D, sizeof(double) * D * D);
    uint32_t k = 0;
    for (int d = 0; d < D; d++) {
      const double box = bmax[d] - bmin[d];
      double m;
      do {
        if (++k > 50) return -2;
        uint32_t ctr[4] = {0xFFFFFFF0u, (uint32_t)i, k - 1, call}, o[4];
        orc_philox(ctr, key, o);
        m = mu[(size_t)imax * D + d] + (-fs * box + 2.0 * fs * box * u53(o[0], o[1]));
      } while (m < bmin[d] || m > bmax[d]);
      mu[(size_t)i * D + d] = m;
    }
    w[imax] /= 2.0;
    w[i] = w[imax];
  }
  double sum = 0.0;
  for (int i = 0; i < K; i++) sum += w[i];
  if (!(sum > 0.0) || !isfinite(sum)) return -3;
  for (int i = 0; i < K; i++) w[i] /= sum;
  return 0;
}
