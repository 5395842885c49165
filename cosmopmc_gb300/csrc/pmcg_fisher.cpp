// pmcg_fisher.cpp — the start of a PMC run: the maximum of the posterior by
// Nelder-Mead searches advanced together (exec/max_post.c:182-224), the Fisher
// matrix there by central differences (exec/go_fishing.c:37-86), and the
// initial PMC proposals built from it (wrappers/src/param.c:472-625). Every
// posterior evaluation is a batched FP64 device call: all stencil points of the
// matrix at once, all searches' trial points of a round at once.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pmcg.h"
#include "pmcg_engine.h"
#include "pmcg_internal.h"

namespace {

// Step factor of the central differences: h = fh (max - min) (exec/mkmax.h:33).
constexpr double kFh = 0.001;

// Philox4x32-10 on the host (the library's counter generator, 64-bit products).
void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32), lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Uniform in [0, 1) for (slot, index, attempt) of the rng's current call.
double uniform_host(const pmcg_rng *rng, uint32_t index, uint32_t attempt) {
  uint32_t c[4] = {0xF1500000u | (attempt & 0xFFFFFu), index, 0u, rng->calls};
  philox_host(c, (uint32_t)rng->seed, (uint32_t)(rng->seed >> 32));
  return ((double)(c[0] >> 5) * 67108864.0 + (double)(c[1] >> 6)) * (1.0 / 9007199254740992.0);
}

// Inverse of a symmetric positive-definite matrix (Gauss-Jordan, partial pivoting).
bool invert(int n, const double *A, double *Ainv) {
  std::vector<double> a(A, A + (size_t)n * n);
  for (int i = 0; i < n * n; i++) Ainv[i] = 0.0;
  for (int i = 0; i < n; i++) Ainv[i * n + i] = 1.0;
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(a[(size_t)r * n + c]) > std::fabs(a[(size_t)p * n + c])) p = r;
    if (!(std::fabs(a[(size_t)p * n + c]) > 0.0)) return false;
    if (p != c)
      for (int j = 0; j < n; j++) {
        std::swap(a[(size_t)p * n + j], a[(size_t)c * n + j]);
        std::swap(Ainv[(size_t)p * n + j], Ainv[(size_t)c * n + j]);
      }
    const double d = 1.0 / a[(size_t)c * n + c];
    for (int j = 0; j < n; j++) { a[(size_t)c * n + j] *= d; Ainv[(size_t)c * n + j] *= d; }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      const double f = a[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int j = 0; j < n; j++) {
        a[(size_t)r * n + j] -= f * a[(size_t)c * n + j];
        Ainv[(size_t)r * n + j] -= f * Ainv[(size_t)c * n + j];
      }
    }
  }
  return true;
}

// Eigenvalues and eigenvectors (columns of V) of a symmetric matrix: cyclic
// Jacobi rotations until the off-diagonal part vanishes to rounding.
void jacobi(int n, const double *A, double *lambda, double *V) {
  std::vector<double> a(A, A + (size_t)n * n);
  for (int i = 0; i < n * n; i++) V[i] = 0.0;
  for (int i = 0; i < n; i++) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        const double v = a[(size_t)i * n + j] * a[(size_t)i * n + j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double theta = (a[(size_t)q * n + q] - a[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {  // columns p, q
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {  // rows p, q
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; i++) lambda[i] = a[(size_t)i * n + i];
}

// Lower Cholesky factor in place succeeds: the positiveness test of a Fisher matrix.
bool positive_definite(int n, const double *A) {
  std::vector<double> l(A, A + (size_t)n * n);
  for (int j = 0; j < n; j++) {
    double d = l[(size_t)j * n + j];
    for (int k = 0; k < j; k++) d -= l[(size_t)j * n + k] * l[(size_t)j * n + k];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    l[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; i++) {
      double v = l[(size_t)i * n + j];
      for (int k = 0; k < j; k++) v -= l[(size_t)i * n + k] * l[(size_t)j * n + k];
      l[(size_t)i * n + j] = v / d;
    }
  }
  return true;
}

}  // namespace

using pmcg::set_error;

// Log-posterior of P points (FP64, one batched device call) into lp/flg. The
// evaluation reports into a chain of its own, so a failure is seen whether or
// not the caller passed an error pointer and an error already in the caller's
// chain does not stop the work; a failure is moved to the front of the
// caller's chain (or dropped when there is none) and false returned.
static bool eval_points(const pmcg_posterior *post, size_t P, const double *X, double *lp, short *flg,
                        error **err) {
  error *ev = nullptr;
  pmcg_posterior_log_pdf_batch(post, P, X, lp, flg, 0, PMCG_FP64, nullptr, &ev);
  if (!isError(ev)) {
    purgeError(&ev);
    return true;
  }
  if (err) {
    error *tail = ev;
    while (tail->next) tail = tail->next;
    tail->next = *err;
    *err = ev;
  } else {
    purgeError(&ev);
  }
  return false;
}

extern "C" int pmcg_fisher_matrix(const pmcg_posterior *post, const double *pos, const double *min,
                                  const double *max, int diag_only, int force_positive, double *F, error **err) {
  if (!post || !pos || !min || !max || !F) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_fisher_matrix: null argument");
    return -1;
  }
  const int D = post->npar;
  std::vector<double> h(D);
  for (int a = 0; a < D; a++) {
    h[a] = kFh * (max[a] - min[a]);
    if (!(h[a] > 1e-20)) {
      set_error(err, PMCG_EARG, __LINE__, "parameter %d: step fh (max - min) too small", a);
      return -1;
    }
  }
  // four points (+,+), (+,-), (-,+), (-,-) per element a >= b (a == b alone
  // with diag_only); the diagonal's (+,-) and (-,+) are both the centre
  const int sgn[4][2] = {{+1, +1}, {+1, -1}, {-1, +1}, {-1, -1}};
  std::vector<int> ea, eb;
  for (int a = 0; a < D; a++)
    for (int b = diag_only ? a : 0; b <= a; b++) {
      ea.push_back(a);
      eb.push_back(b);
    }
  const size_t nel = ea.size(), P = 4 * nel;
  std::vector<double> X(P * D);
  for (size_t e = 0; e < nel; e++)
    for (int j = 0; j < 4; j++) {
      double *x = &X[(4 * e + j) * D];
      std::memcpy(x, pos, sizeof(double) * D);
      x[ea[e]] += sgn[j][0] * h[ea[e]];
      x[eb[e]] += sgn[j][1] * h[eb[e]];
    }
  std::vector<double> lp(P);
  std::vector<short> flg(P);
  if (!eval_points(post, P, X.data(), lp.data(), flg.data(), err)) return -1;
  for (int i = 0; i < D * D; i++) F[i] = 0.0;
  for (size_t e = 0; e < nel; e++) {
    const int a = ea[e], b = eb[e];
    for (int j = 0; j < 4; j++)
      if (!flg[4 * e + j]) {
        set_error(err, PMCG_EARG, __LINE__,
                  "Fisher element (%d,%d): a stencil point leaves the prior box or fails the likelihood", a, b);
        return -1;
      }
    const double *f = &lp[4 * e];
    const double fab = -(f[0] - f[1] - f[2] + f[3]) / (4.0 * h[a] * h[b]);
    F[(size_t)a * D + b] = fab;
    F[(size_t)b * D + a] = fab;
  }
  if (force_positive)
    for (int a = 0; a < D; a++)
      for (int b = 0; b < D; b++) F[(size_t)a * D + b] = a == b ? std::fabs(F[(size_t)a * D + b]) : 0.0;
  return positive_definite(D, F) ? 1 : 0;
}

extern "C" void pmcg_fisher_proposal(mix_mvdens *proposal, const double *F, const double *pos, const double *min,
                                     const double *max, int type, double fshift, double fvar, pmcg_rng *rng,
                                     error **err) {
  if (!proposal || !F || !pos || !min || !max || (type == PMCG_FISHER_RSHIFT && !rng)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_fisher_proposal: null argument");
    return;
  }
  const int D = proposal->ndim, K = proposal->ncomp;
  if (type != PMCG_FISHER_RSHIFT && type != PMCG_FISHER_EIGEN) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_fisher_proposal: unknown type %d", type);
    return;
  }
  if (type == PMCG_FISHER_EIGEN && K > 2 * D) {
    set_error(err, PMCG_EARG, __LINE__,
              "Number of proposal components cannot be larger than twice the number of parameters (%d > %d)", K,
              2 * D);
    return;
  }
  std::vector<double> cov((size_t)D * D);
  if (!invert(D, F, cov.data())) {
    set_error(err, PMCG_EARG, __LINE__, "the Fisher matrix is singular");
    return;
  }
  for (int k = 0; k < K; k++) {
    mvdens *c = proposal->comp[k];
    for (int i = 0; i < D * D; i++) c->std[i] = fvar * cov[i];
    c->chol = 0;
    proposal->wght[k] = 1.0 / K;
  }
  if (type == PMCG_FISHER_RSHIFT) {
    // comp_shift_mean: per parameter a uniform shift in [-fshift box, fshift box],
    // redrawn until the mean lies in the box
    const int kTries = 1000;
    for (int k = 0; k < K; k++)
      for (int i = 0; i < D; i++) {
        const double box = max[i] - min[i];
        double m = 0.0;
        int t = 0;
        do {
          if (t >= kTries) {
            set_error(err, PMCG_EARG, __LINE__,
                      "Could not place proposal component in box: fshift too large or the Fisher matrix "
                      "inconsistent");
            return;
          }
          const double u = uniform_host(rng, (uint32_t)(k * D + i), (uint32_t)t);
          m = pos[i] + fshift * box * (2.0 * u - 1.0);
          t++;
        } while (m < min[i] || m > max[i]);
        proposal->comp[k]->mean[i] = m;
      }
    rng->calls++;
    return;
  }
  // eigen: directions of F^-1 by decreasing eigenvalue, components at -r then +r
  std::vector<double> lam(D), V((size_t)D * D);
  jacobi(D, cov.data(), lam.data(), V.data());
  std::vector<int> order(D);
  for (int i = 0; i < D; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return lam[x] > lam[y]; });
  const double lmax = lam[order[0]];
  for (int k = 0; k < K; k++) {
    const int d = order[k / 2];
    const double sign = (k % 2 == 0) ? -1.0 : 1.0;
    for (int j = 0; j < D; j++)
      proposal->comp[k]->mean[j] = pos[j] + sign * fshift * lam[d] / lmax * V[(size_t)j * D + d];
  }
}

// ------------------------------------------------------------------ maximum posterior
namespace {

constexpr double kLogBig = 1e30;  // objective outside the box or where log P fails
constexpr double kRtolTiny = 1e-10;

// One Nelder-Mead search (reflection 1, expansion 2, contraction 1/2, shrink
// 1/2) on f = -log P. `want` holds the points it needs evaluated next.
struct Simplex {
  int D = 0, lo = 0, hi = 0, nhi = 0, phase = 0, evals = 0;
  bool done = false;
  std::vector<double> x, f, c, xr, xt, want;
  double fr = 0.0;
  enum { kInit, kReflect, kExpand, kContract, kShrink };

  double *v(int i) { return &x[(size_t)i * D]; }

  void order() {
    lo = 0;
    hi = 0;
    for (int i = 1; i <= D; i++) {
      if (f[i] < f[lo]) lo = i;
      if (f[i] > f[hi]) hi = i;
    }
    nhi = (hi == 0) ? 1 : 0;
    for (int i = 0; i <= D; i++)
      if (i != hi && f[i] > f[nhi]) nhi = i;
  }
  // the point c + a (c - x_hi) (a = 1 reflects, 2 expands, -1/2 contracts)
  void along(double a, std::vector<double> &out) {
    out.resize(D);
    for (int j = 0; j < D; j++) out[j] = c[j] + a * (c[j] - v(hi)[j]);
  }
  void replace_hi(const std::vector<double> &p, double fp) {
    std::copy(p.begin(), p.end(), v(hi));
    f[hi] = fp;
  }
  // the next iteration: convergence test, centroid, reflected point
  void next(double ftol) {
    order();
    const double rtol = 2.0 * std::fabs(f[hi] - f[lo]) / (std::fabs(f[hi]) + std::fabs(f[lo]) + kRtolTiny);
    if (rtol < ftol) {
      done = true;
      want.clear();
      return;
    }
    c.assign(D, 0.0);
    for (int i = 0; i <= D; i++)
      if (i != hi)
        for (int j = 0; j < D; j++) c[j] += v(i)[j];
    for (int j = 0; j < D; j++) c[j] /= D;
    along(1.0, xr);
    want = xr;
    phase = kReflect;
  }
  // results of the points in `want`, in order
  void take(const double *fv, double ftol) {
    switch (phase) {
      case kInit:
        std::copy(fv, fv + D + 1, f.begin());
        next(ftol);
        break;
      case kReflect:
        fr = fv[0];
        if (fr < f[lo]) {
          along(2.0, xt);
          want = xt;
          phase = kExpand;
        } else if (fr < f[nhi]) {
          replace_hi(xr, fr);
          next(ftol);
        } else {
          if (fr < f[hi]) replace_hi(xr, fr);
          along(-0.5, xt);
          want = xt;
          phase = kContract;
        }
        break;
      case kExpand:
        if (fv[0] < fr) replace_hi(xt, fv[0]);
        else replace_hi(xr, fr);
        next(ftol);
        break;
      case kContract:
        if (fv[0] < f[hi]) {
          replace_hi(xt, fv[0]);
          next(ftol);
        } else {  // shrink every vertex halfway to the best one
          want.clear();
          for (int i = 0; i <= D; i++) {
            if (i == lo) continue;
            for (int j = 0; j < D; j++) {
              v(i)[j] = v(lo)[j] + 0.5 * (v(i)[j] - v(lo)[j]);
              want.push_back(v(i)[j]);
            }
          }
          phase = kShrink;
        }
        break;
      case kShrink: {
        int q = 0;
        for (int i = 0; i <= D; i++)
          if (i != lo) f[i] = fv[q++];
        next(ftol);
        break;
      }
    }
  }
};

}  // namespace

extern "C" int pmcg_max_posterior(const pmcg_posterior *post, int nstart, const double *starts, const double *min,
                                  const double *max, double ftol, int max_evals, double *best, double *logp,
                                  error **err) {
  if (!post || nstart < 1 || !starts || !min || !max || !best || !logp || !(ftol > 0.0)) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_max_posterior: invalid argument");
    return -1;
  }
  const int D = post->npar;
  if (max_evals < D + 1) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_max_posterior: max_evals below the %d start points", D + 1);
    return -1;
  }
  std::vector<Simplex> S(nstart);
  for (int s = 0; s < nstart; s++) {
    Simplex &m = S[s];
    m.D = D;
    m.x.resize((size_t)(D + 1) * D);
    m.f.assign(D + 1, kLogBig);
    for (int i = 0; i <= D; i++) {
      std::memcpy(m.v(i), starts + (size_t)s * D, sizeof(double) * D);
      if (i > 0) m.v(i)[i - 1] += (max[i - 1] - min[i - 1]) / 5.0;
    }
    m.want = m.x;
    m.phase = Simplex::kInit;
  }
  std::vector<double> X, lp, fv;
  std::vector<short> flg;
  std::vector<size_t> off(nstart + 1);
  for (;;) {
    X.clear();
    for (int s = 0; s < nstart; s++) {
      off[s] = X.size() / D;
      if (!S[s].done) {
        if (S[s].evals + (int)(S[s].want.size() / D) > max_evals) {
          set_error(err, PMCG_ESTEPS, __LINE__, "search %d: more than %d evaluations without converging", s,
                    max_evals);
          return -1;
        }
        X.insert(X.end(), S[s].want.begin(), S[s].want.end());
        S[s].evals += (int)(S[s].want.size() / D);
      }
    }
    off[nstart] = X.size() / D;
    const size_t P = off[nstart];
    if (P == 0) break;
    lp.resize(P);
    flg.resize(P);
    if (!eval_points(post, P, X.data(), lp.data(), flg.data(), err)) return -1;
    fv.resize(P);
    for (size_t q = 0; q < P; q++) {
      bool in = flg[q] != 0 && std::isfinite(lp[q]);
      for (int j = 0; j < D && in; j++) in = X[q * D + j] >= min[j] && X[q * D + j] <= max[j];
      fv[q] = in ? -lp[q] : kLogBig;
    }
    for (int s = 0; s < nstart; s++)
      if (!S[s].done) S[s].take(&fv[off[s]], ftol);
  }
  int ib = 0;
  for (int s = 0; s < nstart; s++) {
    Simplex &m = S[s];
    std::memcpy(best + (size_t)s * D, m.v(m.lo), sizeof(double) * D);
    logp[s] = (m.f[m.lo] >= kLogBig) ? -INFINITY : -m.f[m.lo];
    if (logp[s] > logp[ib]) ib = s;
  }
  return ib;
}
