// pmcg_kernels.h — host-side launchers of the libpmcg CUDA kernels (internal).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "pmcg_common.cuh"

// Allows `dyn` bytes of dynamic shared memory for kernel `fn` when the kernel's
// static shared memory plus `dyn` exceeds the 48 KB a launch gets by default.
template <typename KernelT>
inline cudaError_t allow_dyn_smem(KernelT fn, size_t dyn) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, (const void *)fn);
  if (e != cudaSuccess) return e;
  if (dyn + fa.sharedSizeBytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

namespace pmcg {

constexpr int kMaxD = 64;    // largest parameter dimension
constexpr int kMaxK = 256;   // largest component count
// Largest row sum max_i sum_j |(L^-1)_ij mu_j| of a component that single
// precision still resolves: the coordinates of a single-precision sample carry
// a relative rounding of 2^-24, which moves y = L^-1 (x - mu) by about 2^-24
// times this sum; above 2^18 that is more than 0.016 (the proposal is narrower
// than single precision resolves around its mean).
constexpr double kF32RangeMax = 262144.0;
// Tiles of the weight reduction (one partial record per 2048 samples).
size_t weight_tiles(size_t N);
// Sample chunks per component of the EM statistics.
int em_chunks(int K, size_t N);
// Components staged per barrier by the FP32 log-pdf.
int mix_chunk(int D, int ldx, int K);

// Per-iteration scalars computed on the device (one small D2H per iteration).
struct DevStats {
  double logSum, maxW, H, sumw2, nok;
  double ln_evidence, perplexity, ess, enc;
  double wsum;      // sum of updated weights before renormalisation
  int ndead;        // components with weight 0 after the update
  int status;       // 0 ok, else a PMCG_E* code
  int tc_err;       // set by the tensor-core log-density when one of its waits expired
  int f32_range;    // single-precision runs: components of this update buried because
                    // they are narrower than single precision resolves (counted in ndead)
};

// Device-resident mixture; one allocation, carved into the arrays below.
struct DevMix {
  int K = 0, D = 0, df = -1, ldx = 0;
  double *w = nullptr, *cw = nullptr, *mu = nullptr, *L = nullptr, *Wt = nullptr, *b = nullptr;
  double *logdetL = nullptr, *lconst = nullptr;
  float *W32 = nullptr, *b32 = nullptr, *lconst32 = nullptr, *L32 = nullptr, *mu32 = nullptr;
  unsigned char *bimg = nullptr;  // tensor-core operand image (D <= 32)
  double cst = 0.0;  // log normalising constant of a component, set on the host at allocation
  unsigned *em_done = nullptr;  // component blocks finished in the EM update (0 between launches)
  void *arena = nullptr;
  __host__ __device__ DevMixView view() const {
    DevMixView v;
    v.K = K; v.D = D; v.df = df; v.ldx = ldx;
    v.w = w; v.cw = cw; v.mu = mu; v.L = L; v.Wt = Wt; v.b = b; v.lconst = lconst;
    v.W32 = W32; v.b32 = b32; v.lconst32 = lconst32; v.L32 = L32; v.mu32 = mu32; v.bimg = bimg; v.cst = cst;
    return v;
  }
};

// Tensor-core (tcgen05) proposal log-density, D <= 32 (k_umma.cu).
size_t umma_bimage_bytes(int K);
cudaError_t launch_umma_bimage(const DevMixView &m, unsigned char *img, cudaStream_t s);
cudaError_t launch_umma_logq(const DevMixView &m, const unsigned char *bimg, size_t N, const float *X, double *out,
                             int accumulate, double add, float *lt, float *Qo, int *errflag, cudaStream_t s);
// Process-wide switch for the tensor-core log-density (set by pmcg_set_tensor_cores).
extern int g_use_tensor_cores;

cudaError_t devmix_alloc(DevMix &m, int K, int D, int df);
size_t devmix_bytes(int K, int D);
void devmix_free(DevMix &m);
// Upload w, mu, L (host, FP64) and derive L^-1, L^-1 mu, constants, cumulative weights.
cudaError_t devmix_upload(DevMix &m, const double *w, const double *mu, const double *L, cudaStream_t s);
// Recompute the derived arrays from w, mu, L already on the device.
cudaError_t devmix_prepare(DevMix &m, cudaStream_t s);

inline int round4(int d) { return (d + 3) & ~3; }

// (a) draw. X64 [N x D] (FP64 path) or X32 [N x ldx] (mixed path). pre_* optional.
// callp (optional): the call counter read from device memory instead of call.
cudaError_t launch_draw(int precision, const DevMixView &m, size_t N, uint64_t seed, uint32_t call,
                        const double *bmin, const double *bmax, const double *pre_u, const double *pre_z,
                        const double *pre_chi2, double *X64, float *X32, int *idx, short *flg, int *counts,
                        cudaStream_t s, const uint32_t *callp = nullptr);

// (a) single-precision draws in component order (three launches; counts must
// start at zero). perm: N ints, cursor: 2K ints of scratch. Same values as
// launch_draw(precision 1) without pre-drawn variates. callp (optional): the
// call counter read from device memory instead of call.
cudaError_t launch_draw_grouped(const DevMixView &m, size_t N, uint64_t seed, uint32_t call, const double *bmin,
                                const double *bmax, float *X32, int *idx, short *flg, int *counts, int *perm,
                                int *cursor, cudaStream_t s, const uint32_t *callp = nullptr);
// The samples [n0, n1) of an N-point draw alone (values depend only on the
// sample index, so ranges drawn in any order give the whole draw); counts
// accumulate over ranges.
cudaError_t launch_draw_grouped_range(const DevMixView &m, size_t N, size_t n0, size_t n1, uint64_t seed,
                                      uint32_t call, const double *bmin, const double *bmax, float *X32, int *idx,
                                      short *flg, int *counts, int *perm, int *cursor, cudaStream_t s,
                                      const uint32_t *callp = nullptr);

// (b) mixture log-pdf of N points. out[n] = LSE (accumulate=0) or out[n] += LSE + add (accumulate=1).
// lt/Q optional, [K x N].
cudaError_t launch_mixlogpdf(int precision, const DevMixView &m, size_t N, const double *X64, const float *X32,
                             double *out, int accumulate, double add, double *lt64, double *Q64, float *lt32,
                             float *Q32, cudaStream_t s);

// (d) weights + reduction; writes logw and the scalars of DevStats. fast: the
// per-sample factors e^{l-m} in single precision (single-precision runs).
// betap (optional): beta read from device memory. done (optional): a device
// counter that is zero between calls; the last tile block then merges the
// records (one launch), else a second kernel does.
cudaError_t launch_weights(size_t N, double beta, const double *logpost, const double *logq, short *flg,
                           double *logw, WRed *partials, DevStats *st, cudaStream_t s, int fast = 0,
                           const double *betap = nullptr, unsigned *done = nullptr);

// (e) EM statistics, finalisation (Cholesky on the device) and renormalisation.
size_t em_partials_size(int precision, int K, int D, int *S_out, size_t N);
// emmask (mixed path, optional): em_mask_words(K, N) words of scratch for the
// listing bits; null keeps the per-sample test inside the statistics kernel.
size_t em_mask_words(int K, size_t N);
cudaError_t launch_em(int precision, DevMix &m, size_t N, const double *X64, const float *X32,
                      const double *logw, const double *logq, const double *lt64, const double *Q64,
                      const float *lt32, const float *Q32, const int *counts, double *partials, int S,
                      DevStats *st, int band_limit, float *aw32, uint32_t *emmask, cudaStream_t s);

// (f) Weighted mean [D] and covariance [D x D] (device outputs) of X [N x D]
// with normalised weights wbar (flg == 0 excluded); scratch of
// moments_scratch_doubles(D) doubles.
size_t moments_scratch_doubles(int D);
cudaError_t launch_moments(size_t N, int D, const double *X, const double *wbar, const short *flg, double *scratch,
                           double *mean_out, double *cov_out, cudaStream_t s);

// Post-processing (k_post.cu): per parameter, sort (value, weight), FP64 scan,
// then the centre and limits, or the 1-D bin masses; 2-D histograms by joint
// bin index. scratch: post_scratch_bytes(N) bytes; status[a] 0 ok, 1 no
// counted sample, 2 weights below 1/2 (median).
size_t post_scratch_bytes(size_t N);
cudaError_t launch_post_summary(size_t N, int D, const double *X, const double *wbar, const short *flg,
                                const double *mean, int use_median, void *scratch, double *center, double *sigma,
                                int *status, cudaStream_t s);
cudaError_t launch_post_hist1d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin,
                               const double *lo, const double *hi, double scale, void *scratch, double *hist,
                               cudaStream_t s);
cudaError_t launch_post_hist2d(size_t N, int D, const double *X, const double *wbar, const short *flg, int nbin,
                               int p, int q, const double *lo, const double *hi, double scale, void *scratch,
                               double *hist, cudaStream_t s);

// Weight clipping (k_post.cu): flg = 0 for the k largest log-weights among
// counted samples (ties to the lower index); count: how many were clipped.
// scratch: post_scratch_bytes(N) bytes.
cudaError_t launch_clip_largest(size_t N, const double *logw, short *flg, int k, void *scratch, int *count,
                                cudaStream_t s);

// Convert the mixed-precision sample to FP64 row-major.
cudaError_t launch_x32_to_x64(size_t N, int D, int ldx, const float *X32, double *X64, cudaStream_t s);
// Normalised weights wbar = exp(logw - logSum) (0 where flg == 0).
cudaError_t launch_normalise(size_t N, const double *logw, const short *flg, const DevStats *st, double *wbar,
                             cudaStream_t s);

// (c) SN Ia likelihood. Constant data lives in SnDev.
struct SnDev {
  int nsn = 0, G = 0, chi2mode = 0, add_logdet = 0;
  int ip_om = -1, ip_ode = -1, ip_w0 = -1, ip_M = -1, ip_alpha = -1, ip_beta = -1;
  int neg_M = 0, neg_beta = 0;  // 1: the parameter holds -M (-beta)
  double def_om = 0.3, def_w0 = -1.0, def_M = -19.3, def_alpha = 0.0, def_beta = 0.0;
  double dh = 0.0, sig_int2 = 0.0;
  // sorted by redshift: z, 1/z-dependent peculiar-velocity variance, m_B, x1, c, cov6;
  // per node (nsn*G): a^2, a^3, ln a, weight * half-interval
  double *z = nullptr, *spv2 = nullptr, *mB = nullptr, *x1 = nullptr, *c = nullptr, *cov6 = nullptr;
  double *na2 = nullptr, *na3 = nullptr, *nla = nullptr, *nw = nullptr;
  double *za2 = nullptr, *za3 = nullptr, *zla = nullptr;  // at the SN redshifts
  // single-precision path: residuals relative to a reference model (flat
  // LambdaCDM 0.3/0.7, M = M_ref, alpha = beta = 0) so every per-supernova
  // quantity stays O(1). Nodes as float4 (a^3, a^2, log2 a, weight x
  // half-interval), node-major [G x nsn] so a warp reads 32 consecutive
  // supernovae; per supernova three float4 planes [3 x nsn]:
  //   0: dref = m_B - mu_ref - M_ref, x1, c, 1 / D_M,ref (same quadrature)
  //   1: cov_mm + sig_int^2 + sig_pv^2, cov_x1x1, cov_cc, 2 cov_mx1
  //   2: -2 cov_mc, -2 cov_x1c, (1+z)^3, (1+z)^2
  // and log2(1+z) [nsn]
  float4 *fnode = nullptr, *fsn = nullptr;
  float *fzl2 = nullptr;
  // reference magnitude (a float value, so the set-up in FP64 and the body in
  // FP32 subtract the same number) and float copies of the scalars
  float mref = -19.3f;
  float fdef_om = 0.3f, fdef_w0 = -1.0f, fdef_M = -19.3f, fdef_alpha = 0.0f, fdef_beta = 0.0f;
  void *arena = nullptr;
};
// assign != 0: logpost = add + logL for the samples it evaluates (the others
// keep what logpost held); otherwise logpost += logL.
cudaError_t launch_sn(int precision, const SnDev &sn, size_t N, int D, const double *X64, const float *X32,
                      int ldx, double *logpost, short *flg, cudaStream_t s, int assign = 0, double add = 0.0);

// (c) dense template likelihood (whitened): logpost += -1/2 |dt - At phi(x)|^2.
struct TplDev {
  int M = 0, P = 0, Dpar = 0;
  double *At = nullptr, *dt = nullptr;   // [M x P], [M]
  float *At32 = nullptr, *dt32 = nullptr;
  // Gram form of the single-precision path (P <= kGramMaxP): chi2 = c0 - 2 phi.b
  // + phi^T G phi with G = At^T At ([Pp x Pp], Pp = P rounded up to 4), b = At^T dt,
  // c0 = dt.dt (computed in FP64 at set-up)
  float *G32 = nullptr, *b32 = nullptr;
  double c0 = 0.0;
  unsigned char *uimg = nullptr;  // tensor-core operand image of U (D <= kTplUmmaMaxD), else null
  void *arena = nullptr;
};
constexpr int kGramMaxP = 96;
// Single precision on the tensor cores (k_tpl_umma.cu), D <= 12 (P <= 96):
// chi2 = |U phi|^2 with U the upper Cholesky factor of At'^T At' (At' = At with
// column 0 replaced by At_0 - dt). uimg: tpl_uimage_bytes() bytes, written from
// U32 ([96 x 96] row-major FP32, zero beyond P) by launch_tpl_uimage.
constexpr int kTplUmmaMaxD = 12;
size_t tpl_uimage_bytes();
cudaError_t launch_tpl_uimage(const float *U32, unsigned char *img, cudaStream_t s);
// assign != 0: logpost = add + log L where flg = 1; otherwise logpost += log L.
cudaError_t launch_tpl_umma(const unsigned char *uimg, int Dp, size_t N, const float *X, int ldx, double *logpost,
                            const short *flg, int *errflag, cudaStream_t s, int assign = 0, double add = 0.0);
cudaError_t launch_tpl(int precision, const TplDev &t, size_t N, const double *X64, const float *X32, int ldx,
                       double *logpost, const short *flg, cudaStream_t s);

// (c) Gaussian / Student-t prior on a subset of the parameters (the config
// prior with indprior of posterior_log_pdf_common, wrappers/src/param.c:1009-1026):
// logpost[n] += lconst - 1/2 Q (Gaussian) or lconst - (nu+d)/2 ln(1 + Q/nu),
// Q = |L^-1 (x_sub - mu)|^2, x_sub = the parameters idx[0..d).
struct PriorDev {
  int d = 0, df = -1;
  int idx[kMaxD] = {};
  double lconst = 0.0;   // log normalising constant, -log det L included
  double *mu = nullptr, *Wt = nullptr;       // [d], L^-1 packed by rows [d(d+1)/2]
  float *mu32 = nullptr, *Wt32 = nullptr;
  void *arena = nullptr;
};
cudaError_t launch_prior(int precision, const PriorDev &p, size_t N, int D, const double *X64, const float *X32,
                         int ldx, double *logpost, cudaStream_t s);

// Helpers.
cudaError_t launch_fill_f64(double *p, size_t n, double v, cudaStream_t s);
cudaError_t launch_x64_to_x32(size_t N, int D, int ldx, const double *X64, float *X32, cudaStream_t s);
cudaError_t launch_counts(size_t N, int K, const int *idx, int *counts, cudaStream_t s);
// *out = number of samples with flg != 0 (zeroes *out first).
cudaError_t launch_count_flags(size_t N, const short *flg, int *out, cudaStream_t s);
cudaError_t launch_log_weights(size_t N, double *w, const short *flg, cudaStream_t s);

}  // namespace pmcg
