// k_mix.cu — (b) Gaussian / Student-t mixture log-density of a whole sample,
// and the device-side preparation of a mixture (L^-1, L^-1 mu, constants,
// cumulative weights). Replaces pmclib mix_mvdens_log_pdf, which the
// reference evaluates point by point inside the weight loop
// (exec/cosmo_pmc.c:343) and for the MixMvdens target
// (wrappers/src/param.c:1531-1537).
#include "pmcg_kernels.h"

namespace pmcg {

// ------------------------------------------------------------------ allocation
cudaError_t devmix_alloc(DevMix &m, int K, int D, int df) {
  m.K = K; m.D = D; m.df = df; m.ldx = round4(D);
  const int T = D * (D + 1) / 2;
  size_t nd = (size_t)K * (1 + 1 + D + D * D + T + D + 1 + 1);
  size_t nf = (size_t)K * ((size_t)D * m.ldx + D + 1 + (size_t)D * D + D + 3);
  size_t bytes = nd * sizeof(double) + nf * sizeof(float) + 256;
  cudaError_t e = cudaMalloc(&m.arena, bytes);
  if (e != cudaSuccess) { m.arena = nullptr; return e; }
  double *p = (double *)m.arena;
  m.w = p; p += K;
  m.cw = p; p += K;
  m.mu = p; p += (size_t)K * D;
  m.L = p; p += (size_t)K * D * D;
  m.Wt = p; p += (size_t)K * T;
  m.b = p; p += (size_t)K * D;
  m.logdetL = p; p += K;
  m.lconst = p; p += K;
  float *f = (float *)p;
  m.W32 = f; f += (size_t)K * D * m.ldx;
  m.b32 = f; f += (size_t)K * D;
  m.lconst32 = f; f += K;
  m.L32 = f; f += (size_t)K * D * D;
  m.mu32 = f;
  return cudaSuccess;
}

void devmix_free(DevMix &m) {
  if (m.arena) cudaFree(m.arena);
  m.arena = nullptr;
}

// Per component: W = L^-1 by column substitution, b = W mu, log|L|.
__global__ void mix_prepare_comp_kernel(DevMixView m, double *logdetL, double *Wt, double *b, float *W32,
                                        float *b32, float *L32, float *mu32) {
  const int k = blockIdx.x, D = m.D, T = D * (D + 1) / 2, ldx = m.ldx;
  extern __shared__ double s[];
  double *sL = s;            // D*D
  double *sW = s + D * D;    // D*D
  const double *Lk = m.L + (size_t)k * D * D;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    sL[e] = Lk[e];
    sW[e] = 0.0;
    L32[(size_t)k * D * D + e] = (float)Lk[e];
  }
  for (int i = threadIdx.x; i < D; i += blockDim.x) mu32[(size_t)k * D + i] = (float)m.mu[(size_t)k * D + i];
  __syncthreads();
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    sW[j * D + j] = 1.0 / sL[j * D + j];
    for (int i = j + 1; i < D; i++) {
      double t = 0.0;
      for (int q = j; q < i; q++) t += sL[i * D + q] * sW[q * D + j];
      sW[i * D + j] = -t / sL[i * D + i];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    double t = 0.0;
    for (int j = 0; j <= i; j++) t += sW[i * D + j] * m.mu[(size_t)k * D + j];
    b[(size_t)k * D + i] = t;
    b32[(size_t)k * D + i] = (float)t;
  }
  for (int e = threadIdx.x; e < D * ldx; e += blockDim.x) {
    int i = e / ldx, j = e - i * ldx;
    W32[(size_t)k * D * ldx + e] = (j <= i && j < D) ? (float)sW[i * D + j] : 0.0f;
  }
  for (int e = threadIdx.x; e < T; e += blockDim.x) {
    int i = (int)((sqrt(8.0 * e + 1.0) - 1.0) * 0.5);
    while (tri_idx(i + 1, 0) <= e) i++;
    while (tri_idx(i, 0) > e) i--;
    int j = e - tri_idx(i, 0);
    Wt[(size_t)k * T + e] = sW[i * D + j];
  }
  if (threadIdx.x == 0) {
    double ld = 0.0;
    for (int i = 0; i < D; i++) ld += log(sL[i * D + i]);
    logdetL[k] = ld;
  }
}

// Cumulative weights (summed in component order, as the host and the
// oracle do) and the per-component log constants.
__global__ void mix_prepare_consts_kernel(DevMixView m, const double *logdetL, double *cw, double *lconst,
                                          float *lconst32) {
  const int K = m.K, D = m.D;
  double cst;
  if (m.df > 0) {
    double nu = (double)m.df;
    cst = lgamma(0.5 * (nu + D)) - lgamma(0.5 * nu) - 0.5 * D * log(nu * PMCG_PI);
  } else {
    cst = -0.5 * D * PMCG_LN2PI;
  }
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < K; k++) { s += m.w[k]; cw[k] = s; }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double l = (m.w[k] > 0.0) ? log(m.w[k]) + cst - logdetL[k] : -INFINITY;
    lconst[k] = l;
    lconst32[k] = (float)l;
  }
}

cudaError_t devmix_prepare(DevMix &m, cudaStream_t s) {
  DevMixView v = m.view();
  size_t smem = 2 * (size_t)m.D * m.D * sizeof(double);
  mix_prepare_comp_kernel<<<m.K, 64, smem, s>>>(v, m.logdetL, m.Wt, m.b, m.W32, m.b32, m.L32, m.mu32);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mix_prepare_consts_kernel<<<1, 256, 0, s>>>(v, m.logdetL, m.cw, m.lconst, m.lconst32);
  return cudaGetLastError();
}

cudaError_t devmix_upload(DevMix &m, const double *w, const double *mu, const double *L, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemcpyAsync(m.w, w, sizeof(double) * m.K, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(m.mu, mu, sizeof(double) * m.K * m.D, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(m.L, L, sizeof(double) * m.K * m.D * m.D, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  return devmix_prepare(m, s);
}

// ------------------------------------------------------------------ FP64 log-pdf
// One thread per sample; each component's packed L^-1 and L^-1 mu are staged in
// shared memory and read as broadcasts. y = L^-1 x - L^-1 mu, Q = |y|^2.
template <int MAXD>
__global__ void __launch_bounds__(128) mixlogpdf_f64_kernel(DevMixView m, size_t N, const double *__restrict__ X,
                                                            double *__restrict__ out, int accumulate, double add,
                                                            double *__restrict__ lt, double *__restrict__ Qo) {
  extern __shared__ double s_w[];
  __shared__ double s_lc;
  const int D = m.D, K = m.K, T = D * (D + 1) / 2;
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = n < N;
  double x[MAXD];
#pragma unroll
  for (int i = 0; i < MAXD; i++) x[i] = (act && i < D) ? X[n * D + i] : 0.0;
  double mx = -INFINITY, sm = 0.0;
  const double nu = (double)m.df, hnd = 0.5 * ((double)m.df + D);
  for (int k = 0; k < K; k++) {
    __syncthreads();
    for (int e = threadIdx.x; e < T + D; e += blockDim.x)
      s_w[e] = (e < T) ? m.Wt[(size_t)k * T + e] : m.b[(size_t)k * D + (e - T)];
    if (threadIdx.x == 0) s_lc = m.lconst[k];
    __syncthreads();
    const double lc = s_lc;
    if (lc == -INFINITY) {
      if (act && lt) lt[(size_t)k * N + n] = -INFINITY;
      if (act && Qo) Qo[(size_t)k * N + n] = 0.0;
      continue;
    }
    double q = 0.0;
#pragma unroll
    for (int i = 0; i < MAXD; i++) {
      if (i < D) {
        double acc = -s_w[T + i];
#pragma unroll
        for (int j = 0; j <= i; j++) acc = fma(s_w[i * (i + 1) / 2 + j], x[j], acc);
        q = fma(acc, acc, q);
      }
    }
    const double l = (m.df > 0) ? lc - hnd * log1p(q / nu) : lc - 0.5 * q;
    lse_add(mx, sm, l);
    if (act) {
      if (lt) lt[(size_t)k * N + n] = l;
      if (Qo) Qo[(size_t)k * N + n] = q;
    }
  }
  if (act) {
    double r = mx + log(sm);
    if (accumulate) out[n] += r + add;
    else out[n] = r;
  }
}

// ------------------------------------------------------------------ FP32 log-pdf
// SPT samples per thread share every broadcast float4 of L^-1 from shared
// memory; CH components are staged per barrier.
template <int MAXD, int SPT>
__global__ void __launch_bounds__(128) mixlogpdf_f32_kernel(DevMixView m, size_t N, const float *__restrict__ X,
                                                            double *__restrict__ out, int accumulate, double add,
                                                            float *__restrict__ lt, float *__restrict__ Qo, int CH) {
  extern __shared__ float4 s4[];
  float *sw = reinterpret_cast<float *>(s4);
  const int D = m.D, K = m.K, ldx = m.ldx;
  const int CS = D * ldx + ldx + 4;  // floats per staged component: W rows, b, lconst
  const size_t base = (size_t)blockIdx.x * blockDim.x * SPT + threadIdx.x;
  float x[SPT][MAXD];
#pragma unroll
  for (int s = 0; s < SPT; s++) {
    const size_t n = base + (size_t)s * blockDim.x;
#pragma unroll
    for (int j4 = 0; j4 < MAXD / 4; j4++) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (n < N && 4 * j4 < ldx) v = *reinterpret_cast<const float4 *>(X + n * ldx + 4 * j4);
      x[s][4 * j4] = v.x; x[s][4 * j4 + 1] = v.y; x[s][4 * j4 + 2] = v.z; x[s][4 * j4 + 3] = v.w;
    }
  }
  float mx[SPT], sm[SPT];
#pragma unroll
  for (int s = 0; s < SPT; s++) { mx[s] = -INFINITY; sm[s] = 0.f; }
  const float nu = (float)m.df, hnd = 0.5f * ((float)m.df + (float)D), rnu = 1.0f / (float)m.df;
  for (int kc = 0; kc < K; kc += CH) {
    const int nk = min(CH, K - kc);
    __syncthreads();
    for (int e = threadIdx.x; e < nk * D * ldx; e += blockDim.x) {
      int kk = e / (D * ldx), r = e - kk * D * ldx;
      sw[kk * CS + r] = m.W32[(size_t)(kc + kk) * D * ldx + r];
    }
    for (int e = threadIdx.x; e < nk * (ldx + 4); e += blockDim.x) {
      int kk = e / (ldx + 4), r = e - kk * (ldx + 4);
      float v = 0.f;
      if (r < D) v = m.b32[(size_t)(kc + kk) * D + r];
      else if (r == ldx) v = m.lconst32[kc + kk];
      sw[kk * CS + D * ldx + r] = v;
    }
    __syncthreads();
    for (int kk = 0; kk < nk; kk++) {
      const float *Wk = sw + kk * CS;
      const float *bk = Wk + D * ldx;
      const float lc = bk[ldx];
      const int k = kc + kk;
      if (lc == -INFINITY) {
#pragma unroll
        for (int s = 0; s < SPT; s++) {
          const size_t n = base + (size_t)s * blockDim.x;
          if (n < N) {
            if (lt) lt[(size_t)k * N + n] = -INFINITY;
            if (Qo) Qo[(size_t)k * N + n] = 0.f;
          }
        }
        continue;
      }
      float q[SPT];
#pragma unroll
      for (int s = 0; s < SPT; s++) q[s] = 0.f;
#pragma unroll
      for (int i = 0; i < MAXD; i++) {
        if (i < D) {
          float acc[SPT];
          const float bi = bk[i];
#pragma unroll
          for (int s = 0; s < SPT; s++) acc[s] = -bi;
#pragma unroll
          for (int j4 = 0; j4 <= i / 4; j4++) {
            const float4 w = *reinterpret_cast<const float4 *>(Wk + i * ldx + 4 * j4);
#pragma unroll
            for (int s = 0; s < SPT; s++) {
              acc[s] = fmaf(w.x, x[s][4 * j4], acc[s]);
              acc[s] = fmaf(w.y, x[s][4 * j4 + 1], acc[s]);
              acc[s] = fmaf(w.z, x[s][4 * j4 + 2], acc[s]);
              acc[s] = fmaf(w.w, x[s][4 * j4 + 3], acc[s]);
            }
          }
#pragma unroll
          for (int s = 0; s < SPT; s++) q[s] = fmaf(acc[s], acc[s], q[s]);
        }
      }
#pragma unroll
      for (int s = 0; s < SPT; s++) {
        const float l = (m.df > 0) ? lc - hnd * log1pf(q[s] * rnu) : lc - 0.5f * q[s];
        if (l > mx[s]) { sm[s] = sm[s] * expf(mx[s] - l) + 1.f; mx[s] = l; }
        else sm[s] += expf(l - mx[s]);
        const size_t n = base + (size_t)s * blockDim.x;
        if (n < N) {
          if (lt) lt[(size_t)k * N + n] = l;
          if (Qo) Qo[(size_t)k * N + n] = q[s];
        }
      }
    }
  }
  (void)nu;
#pragma unroll
  for (int s = 0; s < SPT; s++) {
    const size_t n = base + (size_t)s * blockDim.x;
    if (n < N) {
      double r = (double)mx[s] + (double)logf(sm[s]);
      if (accumulate) out[n] += r + add;
      else out[n] = r;
    }
  }
}

template <typename KernelT>
static cudaError_t set_smem(KernelT k, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

cudaError_t launch_mixlogpdf(int precision, const DevMixView &m, size_t N, const double *X64, const float *X32,
                             double *out, int accumulate, double add, double *lt64, double *Q64, float *lt32,
                             float *Q32, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  if (m.D < 1 || m.D > kMaxD || m.K < 1 || m.K > kMaxK) return cudaErrorInvalidValue;
  const int bs = 128;
  if (precision == 0) {
    const int T = m.D * (m.D + 1) / 2;
    size_t smem = (size_t)(T + m.D) * sizeof(double);
    unsigned grid = (unsigned)((N + bs - 1) / bs);
#define PMCG_MLP64(MD)                                                                       \
  {                                                                                          \
    cudaError_t e = set_smem(mixlogpdf_f64_kernel<MD>, smem);                                \
    if (e != cudaSuccess) return e;                                                          \
    mixlogpdf_f64_kernel<MD><<<grid, bs, smem, s>>>(m, N, X64, out, accumulate, add, lt64, Q64); \
    return cudaGetLastError();                                                               \
  }
    if (m.D <= 8) PMCG_MLP64(8);
    if (m.D <= 16) PMCG_MLP64(16);
    if (m.D <= 32) PMCG_MLP64(32);
    PMCG_MLP64(64);
#undef PMCG_MLP64
  }
  constexpr int SPT = 2;
  const int CS = m.D * m.ldx + m.ldx + 4;
  int CH = (int)((40 * 1024) / (CS * sizeof(float)));
  if (CH < 1) CH = 1;
  if (CH > m.K) CH = m.K;
  size_t smem = (size_t)CH * CS * sizeof(float);
  unsigned grid = (unsigned)((N + (size_t)bs * SPT - 1) / ((size_t)bs * SPT));
#define PMCG_MLP32(MD)                                                                                  \
  {                                                                                                     \
    cudaError_t e = set_smem(mixlogpdf_f32_kernel<MD, SPT>, smem);                                      \
    if (e != cudaSuccess) return e;                                                                     \
    mixlogpdf_f32_kernel<MD, SPT><<<grid, bs, smem, s>>>(m, N, X32, out, accumulate, add, lt32, Q32, CH); \
    return cudaGetLastError();                                                                          \
  }
  if (m.ldx <= 8) PMCG_MLP32(8);
  if (m.ldx <= 16) PMCG_MLP32(16);
  if (m.ldx <= 32) PMCG_MLP32(32);
  PMCG_MLP32(64);
#undef PMCG_MLP32
}

}  // namespace pmcg
