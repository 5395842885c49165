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
#include "pmcg_kernels.h"

namespace pmcg {

__device__ __forceinline__ double sk_dev(double ok, double I, int &bad) {
  if (fabs(ok) < 1e-10) return I * (1.0 + ok * I * I / 6.0);
  if (ok > 0.0) { double s = sqrt(ok); return sinh(s * I) / s; }
  double s = sqrt(-ok);
  if (s * I >= PMCG_PI) { bad = 1; return 0.0; }
  return sin(s * I) / s;
}

template <bool F32>
__global__ void __launch_bounds__(128) sn_kernel(SnDev sn, size_t N, int D, const double *__restrict__ X64,
                                                 const float *__restrict__ X32, int ldx, double *__restrict__ logpost,
                                                 short *__restrict__ flg) {
  const int lane = threadIdx.x & 31;
  const size_t n = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (n >= N) return;
  if (!flg[n]) return;
  auto par = [&](int ip, double def) -> double {
    if (ip < 0) return def;
    return F32 ? (double)X32[n * ldx + ip] : X64[n * D + ip];
  };
  const double om = par(sn.ip_om, sn.def_om);
  double ode, ok;
  if (sn.ip_ode >= 0) { ode = par(sn.ip_ode, 0.0); ok = 1.0 - om - ode; }
  else { ode = 1.0 - om; ok = 0.0; }
  const double w0 = par(sn.ip_w0, sn.def_w0);
  const double M = par(sn.ip_M, sn.def_M);
  const double al = par(sn.ip_alpha, sn.def_alpha);
  const double be = par(sn.ip_beta, sn.def_beta);
  const double ex = 3.0 * (1.0 + w0);
  const float omf = (float)om, okf = (float)ok, odef = (float)ode, exf = (float)ex;
  const int G = sn.G, nsn = sn.nsn;
  int bad = 0;
  double carry = 0.0, chi2 = 0.0, A = 0.0, B = 0.0, C = 0.0, sl = 0.0;
  for (int base = 0; base < nsn; base += 32) {
    const int i = base + lane;
    double Ii = 0.0;
    if (i < nsn) {
      if (F32) {
        float acc = 0.f;
        for (int g = 0; g < G; g++) {
          const int q = i * G + g;
          float e2 = omf * sn.fna3[q] + okf * sn.fna2[q] + odef * expf(exf * sn.fnla[q]);
          if (!(e2 > 0.f)) bad = 1;
          else acc += sn.fnw[q] * rsqrtf(e2);
        }
        Ii = (double)acc;
      } else {
        for (int g = 0; g < G; g++) {
          const int q = i * G + g;
          double e2 = om * sn.na3[q] + ok * sn.na2[q] + ode * exp(ex * sn.nla[q]);
          if (!(e2 > 0.0)) bad = 1;
          else Ii += sn.nw[q] / sqrt(e2);
        }
      }
      double e2z = om * sn.za3[i] + ok * sn.za2[i] + ode * exp(ex * sn.zla[i]);
      if (!(e2z > 0.0)) bad = 1;
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      double t = __shfl_up_sync(0xffffffffu, Ii, o);
      if (lane >= o) Ii += t;
    }
    const double I = carry + Ii;
    carry = __shfl_sync(0xffffffffu, I, 31);
    if (i < nsn) {
      const double zi = sn.z[i];
      const double dm = sk_dev(ok, I, bad);
      if (!(dm > 0.0)) bad = 1;
      const double mu_th = 5.0 * log10((1.0 + zi) * sn.dh * fmax(dm, 1e-300)) + 25.0;
      const double *W = sn.cov6 + (size_t)i * 6;
      const double s2 = W[0] + al * al * W[1] + be * be * W[2] + 2.0 * al * W[3] - 2.0 * be * W[4] -
                        2.0 * al * be * W[5] + sn.sig_int2 + sn.spv2[i];
      if (!(s2 > 0.0)) bad = 1;
      double d = sn.mB[i] + al * sn.x1[i] - be * sn.c[i] - mu_th;
      const double is2 = 1.0 / s2;
      if (sn.chi2mode == 0) { d -= M; chi2 += d * d * is2; }
      else { A += d * d * is2; B += d * is2; C += is2; }
      sl += log(s2);
    }
  }
  bad = __any_sync(0xffffffffu, bad);
  chi2 = warp_sum(chi2); A = warp_sum(A); B = warp_sum(B); C = warp_sum(C); sl = warp_sum(sl);
  if (lane == 0) {
    if (bad) { flg[n] = 0; return; }
    if (sn.chi2mode != 0) chi2 = A - B * B / C + log(C / (2.0 * PMCG_PI));
    double ll = -0.5 * chi2 - (sn.add_logdet ? 0.5 * sl : 0.0);
    if (!isfinite(ll)) flg[n] = 0;
    else logpost[n] += ll;
  }
}

cudaError_t launch_sn(int precision, const SnDev &sn, size_t N, int D, const double *X64, const float *X32,
                      int ldx, double *logpost, short *flg, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  unsigned grid = (unsigned)((N + 3) / 4);
  if (precision == 0) sn_kernel<false><<<grid, 128, 0, s>>>(sn, N, D, X64, X32, ldx, logpost, flg);
  else sn_kernel<true><<<grid, 128, 0, s>>>(sn, N, D, X64, X32, ldx, logpost, flg);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ template
// Block = 128 samples; phi(theta) kept transposed in shared memory
// ([P][128], conflict-free); At staged in tiles of kMT rows, transposed so
// each thread reads 8 consecutive rows with two float4/double2 broadcasts.
constexpr int kMT = 32;

template <typename Real>
__global__ void __launch_bounds__(128) tpl_kernel(TplDev t, size_t N, const double *__restrict__ X64,
                                                  const float *__restrict__ X32, int ldx,
                                                  double *__restrict__ logpost, const short *__restrict__ flg) {
  extern __shared__ double tsm[];
  const int P = t.P, Dp = t.Dpar, M = t.M;
  Real *sphi = reinterpret_cast<Real *>(tsm);       // [P][128]
  Real *sA = sphi + (size_t)P * 128;                // [P][kMT]
  Real *sd = sA + (size_t)P * kMT;                  // [kMT]
  const size_t n = (size_t)blockIdx.x * 128 + threadIdx.x;
  const bool act = n < N && flg[n];
  {
    Real th[64];
    for (int i = 0; i < Dp; i++)
      th[i] = act ? (sizeof(Real) == 8 ? (Real)X64[n * Dp + i] : (Real)X32[n * ldx + i]) : (Real)0;
    int p = 0;
    sphi[(p++) * 128 + threadIdx.x] = (Real)1;
    for (int i = 0; i < Dp; i++) sphi[(p++) * 128 + threadIdx.x] = th[i];
    for (int i = 0; i < Dp; i++)
      for (int j = i; j < Dp; j++) sphi[(p++) * 128 + threadIdx.x] = th[i] * th[j];
  }
  Real chi2 = 0;
  double chi2d = 0.0;
  const Real *Asrc = (sizeof(Real) == 8) ? (const Real *)t.At : (const Real *)t.At32;
  const Real *dsrc = (sizeof(Real) == 8) ? (const Real *)t.dt : (const Real *)t.dt32;
  for (int m0 = 0; m0 < M; m0 += kMT) {
    const int mt = min(kMT, M - m0);
    __syncthreads();
    for (int e = threadIdx.x; e < P * kMT; e += 128) {
      int p = e / kMT, r = e - p * kMT;
      sA[e] = (r < mt) ? Asrc[(size_t)(m0 + r) * P + p] : (Real)0;
    }
    for (int r = threadIdx.x; r < kMT; r += 128) sd[r] = (r < mt) ? dsrc[m0 + r] : (Real)0;
    __syncthreads();
    for (int r0 = 0; r0 < kMT; r0 += 8) {
      Real acc[8];
#pragma unroll
      for (int q = 0; q < 8; q++) acc[q] = sd[r0 + q];
      for (int p = 0; p < P; p++) {
        const Real f = sphi[p * 128 + threadIdx.x];
        const Real *a = sA + p * kMT + r0;
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] -= a[q] * f;
      }
#pragma unroll
      for (int q = 0; q < 8; q++) chi2 += acc[q] * acc[q];
    }
    chi2d += (double)chi2;
    chi2 = 0;
  }
  if (act) logpost[n] += -0.5 * chi2d;
}

cudaError_t launch_tpl(int precision, const TplDev &t, size_t N, const double *X64, const float *X32, int ldx,
                       double *logpost, const short *flg, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  if (t.Dpar > 64) return cudaErrorInvalidValue;
  unsigned grid = (unsigned)((N + 127) / 128);
  size_t es = precision == 0 ? sizeof(double) : sizeof(float);
  size_t smem = ((size_t)t.P * 128 + (size_t)t.P * kMT + kMT) * es;
  cudaError_t e;
  if (precision == 0) {
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(tpl_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
      return e;
    tpl_kernel<double><<<grid, 128, smem, s>>>(t, N, X64, X32, ldx, logpost, flg);
  } else {
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(tpl_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
      return e;
    tpl_kernel<float><<<grid, 128, smem, s>>>(t, N, X64, X32, ldx, logpost, flg);
  }
  return cudaGetLastError();
}

}  // namespace pmcg
