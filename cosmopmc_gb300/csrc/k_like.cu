// k_like.cu — (c) per-sample log-likelihoods on the device.
//
// SN Ia: likeli_SNIa (wrappers/src/sn.c:138-281) with nicaea's SetDl/chi2_SN
// restated: luminosity distances from a Gauss-Legendre quadrature of 1/E(z)
// between consecutive sorted redshifts (one warp per sample; the cumulative
// integral is a warp prefix scan), distance modulus and the SALT2-form chi^2
// of Manual/manual.tex:1290-1365, optionally with M marginalised analytically.
//
// Template: logL = -1/2 |dt - At phi(theta)|^2 with At = L^-1 A, dt = L^-1 d_obs
// prepared once in FP64 (structural analogue of likeli_Mvdens,
// wrappers/src/param.c:1485-1493).
//
// Prior on a parameter subset: the config prior of posterior_log_pdf_common
// (wrappers/src/param.c:1009-1026), a Gaussian or Student-t density of the
// parameters flagged by indprior, added to every point's log-posterior.
//
// The bodies are shared with the batch kernel (pmcg_bodies.cuh).
#include "pmcg_bodies.cuh"

namespace pmcg {

template <bool F32, bool BATCH>
__global__ void __launch_bounds__(128) sn_kernel(SnDev sn, size_t N, int D, const double *__restrict__ X64,
                                                 const float *__restrict__ X32, int ldx, double *__restrict__ logpost,
                                                 short *__restrict__ flg, int assign, double add) {
  const size_t n = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  body_sn<F32, BATCH>(sn, N, D, X64, X32, ldx, logpost, flg, n, assign, add);
}

// Single precision below 2^16 samples (a few waves of warps): loads batched
// ahead of use (measured at N = 10^4: 60.5 -> 51.6 us; two warps per sample,
// half the supernovae each, measured no faster: the second warp waits resident
// for the first half's distance integral); above, the form with fewer
// registers (measured at N = 2^18: 0.85 -> 0.76 ms per iteration).
constexpr size_t kSnBatchBelow = (size_t)1 << 16;

cudaError_t launch_sn(int precision, const SnDev &sn, size_t N, int D, const double *X64, const float *X32,
                      int ldx, double *logpost, short *flg, cudaStream_t s, int assign, double add) {
  if (N == 0) return cudaSuccess;
  unsigned grid = (unsigned)((N + 3) / 4);
  if (precision == 0)
    sn_kernel<false, false><<<grid, 128, 0, s>>>(sn, N, D, X64, X32, ldx, logpost, flg, assign, add);
  else if (N < kSnBatchBelow)
    sn_kernel<true, true><<<grid, 128, 0, s>>>(sn, N, D, X64, X32, ldx, logpost, flg, assign, add);
  else sn_kernel<true, false><<<grid, 128, 0, s>>>(sn, N, D, X64, X32, ldx, logpost, flg, assign, add);
  return cudaGetLastError();
}

template <typename Real>
__global__ void __launch_bounds__(128) tpl_kernel(TplDev t, size_t N, const double *__restrict__ X64,
                                                  const float *__restrict__ X32, int ldx,
                                                  double *__restrict__ logpost, const short *__restrict__ flg) {
  extern __shared__ double tsm[];
  body_tpl<Real>(t, N, X64, X32, ldx, logpost, flg, blockIdx.x, reinterpret_cast<Real *>(tsm), 0, 0.0);
}

cudaError_t launch_tpl(int precision, const TplDev &t, size_t N, const double *X64, const float *X32, int ldx,
                       double *logpost, const short *flg, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  if (t.Dpar > 64) return cudaErrorInvalidValue;
  unsigned grid = (unsigned)((N + 127) / 128);
  cudaError_t e;
  if (precision == 0) {
    size_t smem = tpl_smem<double>(t.P, 128);
    if ((e = allow_dyn_smem(tpl_kernel<double>, smem)) != cudaSuccess) return e;
    tpl_kernel<double><<<grid, 128, smem, s>>>(t, N, X64, X32, ldx, logpost, flg);
  } else {
    size_t smem = tpl_smem<float>(t.P, 128);
    if ((e = allow_dyn_smem(tpl_kernel<float>, smem)) != cudaSuccess) return e;
    tpl_kernel<float><<<grid, 128, smem, s>>>(t, N, X64, X32, ldx, logpost, flg);
  }
  return cudaGetLastError();
}

template <typename Real>
__global__ void __launch_bounds__(128) prior_kernel(PriorDev p, size_t N, int D, const double *__restrict__ X64,
                                                    const float *__restrict__ X32, int ldx,
                                                    double *__restrict__ logpost) {
  body_prior_any<Real>(p, N, D, X64, X32, ldx, logpost, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}

cudaError_t launch_prior(int precision, const PriorDev &p, size_t N, int D, const double *X64, const float *X32,
                         int ldx, double *logpost, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  if (p.d < 1 || p.d > kMaxD) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((N + 127) / 128);
  if (precision == 0) prior_kernel<double><<<grid, 128, 0, s>>>(p, N, D, X64, X32, ldx, logpost);
  else prior_kernel<float><<<grid, 128, 0, s>>>(p, N, D, X64, X32, ldx, logpost);
  return cudaGetLastError();
}

}  // namespace pmcg
