// k_mix.cu — (b) Gaussian / Student-t mixture log-density of a whole sample,
// and the device-side preparation of a mixture (L^-1, L^-1 mu, constants,
// cumulative weights). Replaces pmclib mix_mvdens_log_pdf, which the
// reference evaluates point by point inside the weight loop
// (exec/cosmo_pmc.c:343) and for the MixMvdens target
// (wrappers/src/param.c:1531-1537). The FP32 and preparation bodies are
// shared with the batch kernel (pmcg_bodies.cuh).
#include <cmath>
#include "pmcg_bodies.cuh"

namespace pmcg {

// ------------------------------------------------------------------ allocation
// Every array starts on a 256-byte boundary (the single-precision factors are
// read as float4, the tensor-core image by bulk copies). The tensor-core image
// of L^-1 (slot 13) exists for D <= 32 only.
static size_t devmix_layout(int K, int D, size_t off[15]) {
  const size_t T = (size_t)D * (D + 1) / 2, Kz = (size_t)K, ldx = (size_t)round4(D);
  const size_t nd[8] = {Kz, Kz, Kz * D, Kz * D * D, Kz * T, Kz * D, Kz, Kz};
  const size_t nf[5] = {Kz * D * ldx, Kz * D, Kz, Kz * D * ldx, Kz * D};
  size_t o = 0;
  for (int i = 0; i < 8; i++) { off[i] = o; o = (o + nd[i] * sizeof(double) + 255) & ~(size_t)255; }
  for (int i = 0; i < 5; i++) { off[8 + i] = o; o = (o + nf[i] * sizeof(float) + 255) & ~(size_t)255; }
  off[13] = o;
  if (D <= 32) o = (o + umma_bimage_bytes(K) + 255) & ~(size_t)255;
  off[14] = o;  // EM update counter
  return o + 256;
}

size_t devmix_bytes(int K, int D) {
  size_t off[15];
  return devmix_layout(K, D, off);
}

cudaError_t devmix_alloc(DevMix &m, int K, int D, int df) {
  m.K = K; m.D = D; m.df = df; m.ldx = round4(D);
  if (df > 0) {
    const double nu = (double)df;
    m.cst = std::lgamma(0.5 * (nu + D)) - std::lgamma(0.5 * nu) - 0.5 * D * std::log(nu * PMCG_PI);
  } else {
    m.cst = -0.5 * D * PMCG_LN2PI;
  }
  size_t off[15];
  const size_t o = devmix_layout(K, D, off);
  cudaError_t e = cudaMalloc(&m.arena, o);
  if (e != cudaSuccess) { m.arena = nullptr; return e; }
  char *a = (char *)m.arena;
  m.w = (double *)(a + off[0]);
  m.cw = (double *)(a + off[1]);
  m.mu = (double *)(a + off[2]);
  m.L = (double *)(a + off[3]);
  m.Wt = (double *)(a + off[4]);
  m.b = (double *)(a + off[5]);
  m.logdetL = (double *)(a + off[6]);
  m.lconst = (double *)(a + off[7]);
  m.W32 = (float *)(a + off[8]);
  m.b32 = (float *)(a + off[9]);
  m.lconst32 = (float *)(a + off[10]);
  m.L32 = (float *)(a + off[11]);
  m.mu32 = (float *)(a + off[12]);
  m.bimg = (D <= 32) ? (unsigned char *)(a + off[13]) : nullptr;
  m.em_done = (unsigned *)(a + off[14]);
  if ((e = cudaMemset(m.em_done, 0, sizeof(unsigned))) != cudaSuccess) return e;
  return cudaSuccess;
}

void devmix_free(DevMix &m) {
  if (m.arena) cudaFree(m.arena);
  m.arena = nullptr;
}

__global__ void mix_prepare_comp_kernel(DevMixView m, double *logdetL, double *Wt, double *b, float *W32,
                                        float *b32, float *L32, float *mu32) {
  extern __shared__ double s[];
  body_prepare_comp(m, logdetL, Wt, b, W32, b32, L32, mu32, blockIdx.x, s);
}

__global__ void mix_prepare_consts_kernel(DevMixView m, const double *logdetL, double *cw, double *lconst,
                                          float *lconst32) {
  body_prepare_consts(m, logdetL, cw, lconst, lconst32);
}

cudaError_t devmix_prepare(DevMix &m, cudaStream_t s) {
  DevMixView v = m.view();
  const size_t smem = prepare_smem(m.D);
  cudaError_t e;
  if ((e = allow_dyn_smem(mix_prepare_comp_kernel, smem)) != cudaSuccess) return e;
  mix_prepare_comp_kernel<<<m.K, 256, smem, s>>>(v, m.logdetL, m.Wt, m.b, m.W32, m.b32, m.L32, m.mu32);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mix_prepare_consts_kernel<<<1, 256, 0, s>>>(v, m.logdetL, m.cw, m.lconst, m.lconst32);
  e = cudaGetLastError();
  if (e != cudaSuccess || !m.bimg) return e;
  return launch_umma_bimage(v, m.bimg, s);
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
    else out[n] = r + add;
  }
}

// ------------------------------------------------------------------ FP32 log-pdf
template <int MAXD, int SPT>
__global__ void __launch_bounds__(128) mixlogpdf_f32_kernel(DevMixView m, size_t N, const float *__restrict__ X,
                                                            double *__restrict__ out, int accumulate, double add,
                                                            float *__restrict__ lt, float *__restrict__ Qo, int CH) {
  extern __shared__ float4 s4[];
  body_mixlogpdf_f32<MAXD, SPT>(m, N, X, out, accumulate, add, lt, Qo, CH, blockIdx.x,
                                reinterpret_cast<float *>(s4));
}

template <typename KernelT>
static cudaError_t set_smem(KernelT k, size_t smem) {
  return allow_dyn_smem(k, smem);
}

// Components staged per barrier for the FP32 log-pdf (about 40 KB of L^-1).
int mix_chunk(int D, int ldx, int K) {
  const int CS = mix_cs(D, ldx);
  int CH = (int)((40 * 1024) / (CS * sizeof(float)));
  if (CH < 1) CH = 1;
  if (CH > K) CH = K;
  return CH;
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
  const int CH = mix_chunk(m.D, m.ldx, m.K);
  size_t smem = (size_t)CH * mix_cs(m.D, m.ldx) * sizeof(float);
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
