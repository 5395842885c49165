// pmcg_bodies.cuh — the per-work-item bodies of the engine's kernels.
//
// Each body processes one work item (a tile of samples, one component, one run)
// with whatever block size it is launched with. The standalone kernels (one
// launch per stage and run) and the persistent batch kernel (all stages of all
// runs in one cooperative launch) call the same bodies, so a run gives
// bit-identical results alone and inside a batch.
//
// Conventions: `smem` is the block's dynamic shared memory; a body that uses
// __syncthreads() is entered by every thread of the block, and callers that
// loop over items put a __syncthreads() between items.
#pragma once
#include "pmcg_kernels.h"

namespace pmcg {

constexpr int kTileW = 2048;   // samples per weight / weight-factor tile
constexpr int kTile32 = 64;    // samples per EM staging tile (mixed)
constexpr int kFlushTiles = 16;
constexpr int kMinCount = 20;  // MINCOUNT, Manual/manual.tex:483

__host__ __device__ inline int em_E(int D) { return 2 + D + D * (D + 1) / 2; }
__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// ================================================================== (a) draw
// Box-Muller pair from one Philox block. FP64 path: two 53-bit uniforms (the
// oracle's mapping). FP32 path: the same 53-bit integers, 1-a and b, converted
// to float from two 32-bit halves (within one unit of the last place of the
// correctly rounded value; 32-bit conversions avoid the 64-bit conversion
// unit, slow on GB300), so its normals equal the FP64 ones to single
// precision, tails included.
template <typename Real>
__device__ __forceinline__ void box_muller(P4 o, Real &g0, Real &g1);

template <>
__device__ __forceinline__ void box_muller<double>(P4 o, double &g0, double &g1) {
  double a = u53(o.x, o.y), b = u53(o.z, o.w);
  double r = sqrt(-2.0 * log1p(-a));
  double sn, cs;
  sincospi(2.0 * b, &sn, &cs);
  g0 = r * cs;
  g1 = r * sn;
}
// An integer below 2^53 as float from its high (>= 2^26) and low 26-bit parts.
__device__ __forceinline__ float u53_to_float(unsigned long long A) {
  return fmaf(__uint2float_rn((unsigned)(A >> 26)), 67108864.0f, __uint2float_rn((unsigned)(A & 0x3FFFFFFull)));
}

template <>
__device__ __forceinline__ void box_muller<float>(P4 o, float &g0, float &g1) {
  const unsigned long long A = ((unsigned long long)(o.x >> 5) << 26) | (unsigned long long)(o.y >> 6);
  const float two53inv = 1.1102230246251565e-16f;  // 2^-53
  // -2 ln(1-a): from the exact small a below 1/2 (log1p), from the exact
  // complement c = 1-a <= 1/2 above, so r keeps single precision at both ends.
  // There |log2 c| >= 1, so the MUFU log2 (absolute error near 2^-22) is
  // within a few 1e-7 relative.
  float r2;
  if (A < (1ull << 52)) {
    r2 = -2.0f * log1pf(-(u53_to_float(A) * two53inv));
  } else {
    float l2;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l2) : "f"(u53_to_float((1ull << 53) - A) * two53inv));
    r2 = -1.3862943611198906f * l2;  // -2 ln 2
  }
  // b = B / 2^53 with B = (z >> 5) 2^26 + (w >> 6): z / 2^32 to single precision
  const float b = __uint2float_rn(o.z) * 2.3283064365386963e-10f;  // 2^-32
  float r = sqrtf(r2);
  float sn, cs;
  sincospif(2.0f * b, &sn, &cs);
  g0 = r * cs;
  g1 = r * sn;
}

// Staging rows use stride ldo+1 (odd) so the per-thread row stores do not
// collide in one bank.
template <typename Real>
__host__ __device__ inline size_t draw_smem(int K, int ldo, int threads) {
  return align16((size_t)K * 8 + (size_t)K * 4) + (size_t)threads * (ldo + 1) * sizeof(Real);
}

// Normals of sample n (counter {1+m, n, call}) into z[0..D), zero above; the
// sum of squares of the nu extra normals into c2 (Student-t), else c2 = 0.
template <int MAXD, typename Real>
__device__ __forceinline__ void draw_normals(int D, int nu, uint32_t nlo, uint32_t nhi, uint32_t call, uint32_t key0,
                                             uint32_t key1, Real (&z)[MAXD], Real &c2) {
  c2 = (Real)0;
#pragma unroll
  for (int mm = 0; mm < MAXD / 2; mm++) {
    if (2 * mm < D) {
      P4 c = {1u + (uint32_t)mm, nlo, nhi, call};
      P4 o = philox4x32_10(c, key0, key1);
      Real g0, g1;
      box_muller<Real>(o, g0, g1);
      z[2 * mm] = g0;
      if (2 * mm + 1 < D) {
        z[2 * mm + 1] = g1;
      } else {
        z[2 * mm + 1] = (Real)0;
        if (nu > 0) c2 += g1 * g1;
      }
    } else {
      z[2 * mm] = (Real)0;
      z[2 * mm + 1] = (Real)0;
    }
  }
  const int jstart = (D % 2 == 0) ? D : D + 1;
  for (int j = jstart; j < D + nu; j += 2) {
    P4 c = {1u + (uint32_t)(j / 2), nlo, nhi, call};
    P4 o = philox4x32_10(c, key0, key1);
    Real g0, g1;
    box_muller<Real>(o, g0, g1);
    c2 += g0 * g0;
    if (j + 1 < D + nu) c2 += g1 * g1;
  }
}

// Student-t scale sqrt(nu / chi2): FP64 in the FP64 path, single precision
// (correctly rounded division and square root) in the mixed path.
template <typename Real>
__device__ __forceinline__ Real student_scale(int df, Real c2) {
  if (sizeof(Real) == 8) return (Real)sqrt((double)df / (double)c2);
  return (Real)sqrtf((float)df / (float)c2);
}

// x = mu_k + sc L_k z in single precision from the rows of L_k (stride ldx,
// zero above the diagonal: float4 reads) and mu_k; SHARED: the rows are staged
// in shared memory (plain loads), otherwise read-only global loads. Returns 0
// when a coordinate leaves the box.
template <int MAXD, bool SHARED>
__device__ __forceinline__ int draw_transform_rows(int D, int ldx, const float *Lk, const float *mk,
                                                   const float (&z)[MAXD], float sc, const double *__restrict__ bmin,
                                                   const double *__restrict__ bmax, float *xo, int xstride) {
  int in = 1;
#pragma unroll
  for (int i = 0; i < MAXD; i++) {
    if (i < D) {
      float acc = 0.f;
#pragma unroll
      for (int j4 = 0; j4 <= i / 4; j4++) {
        const float4 *q = reinterpret_cast<const float4 *>(Lk + (size_t)i * ldx + 4 * j4);
        const float4 l4 = SHARED ? *q : __ldg(q);
        acc = fmaf(l4.x, z[4 * j4], acc);
        acc = fmaf(l4.y, z[4 * j4 + 1], acc);
        acc = fmaf(l4.z, z[4 * j4 + 2], acc);
        acc = fmaf(l4.w, z[4 * j4 + 3], acc);
      }
      const float xi = (SHARED ? mk[i] : __ldg(&mk[i])) + sc * acc;
      xo[i * xstride] = xi;
      if (bmin && ((double)xi < bmin[i] || (double)xi > bmax[i])) in = 0;
    }
  }
  return in;
}
// The same rows as draw_transform_rows, stored to the sample's row (ldx
// floats, zero padded) four at a time as each group of four is complete, so
// no finished row stays in registers (the draw kernel's occupancy is set by
// its registers).
template <int MAXD, bool SHARED>
__device__ __forceinline__ int draw_transform_store(int D, int ldx, const float *Lk, const float *mk,
                                                    const float (&z)[MAXD], float sc, const double *__restrict__ bmin,
                                                    const double *__restrict__ bmax, float *__restrict__ row) {
  int in = 1;
#pragma unroll
  for (int i4 = 0; i4 < MAXD / 4; i4++) {
    if (4 * i4 < ldx) {
      float xv[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const int i = 4 * i4 + r;
        xv[r] = 0.f;
        if (i < D) {
          float acc = 0.f;
#pragma unroll
          for (int j4 = 0; j4 <= i / 4; j4++) {
            const float4 *q = reinterpret_cast<const float4 *>(Lk + (size_t)i * ldx + 4 * j4);
            const float4 l4 = SHARED ? *q : __ldg(q);
            acc = fmaf(l4.x, z[4 * j4], acc);
            acc = fmaf(l4.y, z[4 * j4 + 1], acc);
            acc = fmaf(l4.z, z[4 * j4 + 2], acc);
            acc = fmaf(l4.w, z[4 * j4 + 3], acc);
          }
          const float xi = (SHARED ? mk[i] : __ldg(&mk[i])) + sc * acc;
          xv[r] = xi;
          if (bmin && ((double)xi < bmin[i] || (double)xi > bmax[i])) in = 0;
        }
      }
      *reinterpret_cast<float4 *>(row + 4 * i4) = make_float4(xv[0], xv[1], xv[2], xv[3]);
    }
  }
  return in;
}
template <int MAXD>
__device__ __forceinline__ int draw_transform_f32(const DevMixView &m, int k, const float (&z)[MAXD], float sc,
                                                  const double *__restrict__ bmin, const double *__restrict__ bmax,
                                                  float *xo, int xstride) {
  return draw_transform_rows<MAXD, false>(m.D, m.ldx, m.L32 + (size_t)k * m.D * m.ldx, m.mu32 + (size_t)k * m.D, z,
                                          sc, bmin, bmax, xo, xstride);
}

// Samples n0 .. n0+blockDim-1: one thread per sample, rows staged in shared
// memory and written with coalesced stores. Component k = min{k : u < C_k}.
template <int MAXD, typename Real>
__device__ __forceinline__ void body_draw(const DevMixView &m, size_t N, uint32_t key0, uint32_t key1, uint32_t call,
                                          const double *__restrict__ bmin, const double *__restrict__ bmax,
                                          const double *__restrict__ pre_u, const double *__restrict__ pre_z,
                                          const double *__restrict__ pre_chi2, double *__restrict__ X64,
                                          float *__restrict__ X32, int *__restrict__ idx, short *__restrict__ flg,
                                          int *__restrict__ counts, size_t n0, unsigned char *smem) {
  const int K = m.K, D = m.D, df = m.df;
  const int ldo = (sizeof(Real) == 8) ? D : m.ldx;
  double *s_cw = reinterpret_cast<double *>(smem);
  int *s_cnt = reinterpret_cast<int *>(smem + (size_t)K * 8);
  Real *s_x = reinterpret_cast<Real *>(smem + align16((size_t)K * 8 + (size_t)K * 4));
  for (int k = threadIdx.x; k < K; k += blockDim.x) { s_cw[k] = m.cw[k]; s_cnt[k] = 0; }
  __syncthreads();
  const size_t n = n0 + threadIdx.x;
  if (n < N) {
    const uint32_t nlo = (uint32_t)n, nhi = (uint32_t)(n >> 32);
    double u;
    if (pre_u) {
      u = pre_u[n];
    } else {
      P4 c = {0u, nlo, nhi, call};
      P4 o = philox4x32_10(c, key0, key1);
      u = u53(o.x, o.y);
    }
    int k = -1;
    for (int j = 0; j < K; j++)
      if (u < s_cw[j]) { k = j; break; }
    if (k < 0)
      for (int j = K - 1; j >= 0; j--)
        if (m.w[j] > 0.0) { k = j; break; }
    if (k < 0) k = 0;
    const int nu = df > 0 ? df : 0;
    Real z[MAXD];
    Real c2 = (Real)0;
    if (pre_z) {
#pragma unroll
      for (int i = 0; i < MAXD; i++) z[i] = (i < D) ? (Real)pre_z[n * D + i] : (Real)0;
      c2 = pre_chi2 ? (Real)pre_chi2[n] : (Real)1;
    } else {
      draw_normals<MAXD, Real>(D, nu, nlo, nhi, call, key0, key1, z, c2);
    }
    const Real sc = (df > 0) ? student_scale<Real>(df, c2) : (Real)1;
    const int lds = ldo + 1;
    int in = 1;
    if (sizeof(Real) == 8) {
      const double *Lk = m.L + (size_t)k * D * D;
      const double *mk = m.mu + (size_t)k * D;
#pragma unroll
      for (int i = 0; i < MAXD; i++) {
        if (i < D) {
          Real acc = (Real)0;
#pragma unroll
          for (int j = 0; j <= i; j++) acc += (Real)__ldg(&Lk[i * D + j]) * z[j];
          Real xi = (Real)__ldg(&mk[i]) + sc * acc;
          s_x[threadIdx.x * lds + i] = xi;
          if (bmin && ((double)xi < bmin[i] || (double)xi > bmax[i])) in = 0;
        }
      }
    } else {
      float zf[MAXD];
#pragma unroll
      for (int i = 0; i < MAXD; i++) zf[i] = (float)z[i];
      in = draw_transform_f32<MAXD>(m, k, zf, (float)sc, bmin, bmax, reinterpret_cast<float *>(s_x) + threadIdx.x * lds, 1);
    }
    for (int i = D; i < ldo; i++) s_x[threadIdx.x * lds + i] = (Real)0;
    idx[n] = k;
    flg[n] = (short)in;
    atomicAdd(&s_cnt[k], 1);
  }
  __syncthreads();
  // coalesced copy-out: each warp writes whole rows
  const int rows = (N > n0) ? (int)((N - n0 < (size_t)blockDim.x) ? (N - n0) : (size_t)blockDim.x) : 0;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int r = threadIdx.x >> 5; r < rows; r += nw) {
    for (int c = lane; c < ldo; c += 32) {
      const Real v = s_x[r * (ldo + 1) + c];
      if (sizeof(Real) == 8) X64[(n0 + r) * ldo + c] = (double)v;
      else X32[(n0 + r) * ldo + c] = (float)v;
    }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    if (s_cnt[k]) atomicAdd(&counts[k], s_cnt[k]);
}

// ================================================================== (b) FP32 log-pdf
__host__ __device__ inline int mix_cs(int D, int ldx) { return D * ldx + ldx + 4; }

// Samples item*blockDim*SPT + s*blockDim + tid (s < SPT); CH components staged per
// barrier; every broadcast float4 of L^-1 feeds SPT samples.
template <int MAXD, int SPT>
__device__ __forceinline__ void body_mixlogpdf_f32(const DevMixView &m, size_t N, const float *__restrict__ X,
                                                   double *__restrict__ out, int accumulate, double add,
                                                   float *__restrict__ lt, float *__restrict__ Qo, int CH,
                                                   size_t item, float *sw) {
  const int D = m.D, K = m.K, ldx = m.ldx;
  const int CS = mix_cs(D, ldx);
  const size_t base = item * blockDim.x * SPT + threadIdx.x;
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
  const float hnd = 0.5f * ((float)m.df + (float)D), rnu = 1.0f / (float)m.df;
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
#pragma unroll
  for (int s = 0; s < SPT; s++) {
    const size_t n = base + (size_t)s * blockDim.x;
    if (n < N) {
      double r = (double)mx[s] + (double)logf(sm[s]);
      if (accumulate) out[n] += r + add;
      else out[n] = r + add;
    }
  }
}

// ================================================================== (c) SN Ia
__device__ __forceinline__ double sk_dev(double ok, double I, int &bad) {
  if (fabs(ok) < 1e-10) return I * (1.0 + ok * I * I / 6.0);
  if (ok > 0.0) { double s = sqrt(ok); return sinh(s * I) / s; }
  double s = sqrt(-ok);
  if (s * I >= PMCG_PI) { bad = 1; return 0.0; }
  return sin(s * I) / s;
}

__device__ __forceinline__ float sk_f(float ok, float I, int &bad) {
  if (fabsf(ok) < 1e-7f) return I * (1.f + ok * I * I * (1.f / 6.f));
  if (ok > 0.f) { const float s = sqrtf(ok); return sinhf(s * I) / s; }
  const float s = sqrtf(-ok);
  if (s * I >= 3.14159265f) { bad = 1; return 0.f; }
  return sinf(s * I) / s;
}

// Error-free sum of two floats (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (hi, lo) += v for a float-float pair (about 44 significant bits).
__device__ __forceinline__ void ff_add(float &hi, float &lo, float vhi, float vlo) {
  float s, e;
  two_sum_f(hi, vhi, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, vlo));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}
// Warp tree sum of one float per lane, carried as float-float; lane 0 holds the
// result.
__device__ __forceinline__ void warp_sum_ff(float v, float &hi, float &lo) {
  hi = v; lo = 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_down_sync(0xffffffffu, hi, o), l2 = __shfl_down_sync(0xffffffffu, lo, o);
    ff_add(hi, lo, h2, l2);
  }
}

// PTX approximate transcendental and reciprocal instructions (MUFU): ex2,
// lg2 and rcp with relative error of order 2^-22, used where a few 1e-7 of
// relative error per supernova is far below the single-precision tolerance.
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Transverse comoving distance S_k(I) = sinh(sqrt(Ok) I)/sqrt(Ok) (Ok > 0),
// I (Ok = 0), sin(sqrt(-Ok) I)/sqrt(-Ok) (Ok < 0). All three are the one power
// series I * sum_j u^j / (2j+1)! in u = Ok I^2; for |u| <= 4 eight terms leave
// a truncation below 2e-10 relative (4^8/17!), evaluated by Horner's rule
// without branches. Larger |u| takes the closed forms; the sine branch
// reaches its first zero (a closed universe's antipode) at u = -pi^2.
__device__ __forceinline__ float sk_series_f(float ok, float I, int &bad) {
  const float u = ok * I * I;
  if (fabsf(u) <= 4.f) {
    float p = 1.f / 1307674368000.f;              // 1/15!
    p = fmaf(p, u, 1.f / 6227020800.f);           // 1/13!
    p = fmaf(p, u, 1.f / 39916800.f);             // 1/11!
    p = fmaf(p, u, 1.f / 362880.f);               // 1/9!
    p = fmaf(p, u, 1.f / 5040.f);                 // 1/7!
    p = fmaf(p, u, 1.f / 120.f);                  // 1/5!
    p = fmaf(p, u, 1.f / 6.f);                    // 1/3!
    p = fmaf(p, u, 1.f);
    return I * p;
  }
  return sk_f(ok, I, bad);
}

// Single-precision SN body (one warp per sample): the node sums, the distance,
// the residual and its weight in FP32, with every residual taken relative to
// the reference model (d = dref + alpha x1 - beta c - (M - M_ref)
// - 5 log10(D_M / D_M,ref)), so no O(20 mag) quantities are differenced in
// single precision. The cumulative distance integral is a warp scan in FP32
// inside each block of 32 supernovae plus a float-float carry across blocks
// (its rounding does not accumulate over the survey), and the sums over
// supernovae are per-lane FP32 partials reduced across the warp in
// float-float; only the final combination runs in FP64 (GB300 issues FP64 at
// a small fraction of the FP32 rate). Node and supernova data are float4
// planes indexed by supernova, so each warp load is 512 contiguous bytes.
// The marginalised mode uses residuals without M, shift-invariant in
// A - B^2/C.
// BATCH: each block's loads are issued before their first use (more registers:
// for small samples, where few warps per SM leave the load latency exposed);
// otherwise each node is loaded as it is used (fewer registers, more resident
// warps: for large samples). Both give the same values.
template <bool BATCH = false>
__device__ __forceinline__ void body_sn_f32(const SnDev &sn, size_t N, const float *__restrict__ X32, int ldx,
                                            double *__restrict__ logpost, short *__restrict__ flg, size_t n,
                                            int assign, double add) {
  const int lane = threadIdx.x & 31;
  if (n >= N) return;
  if (!flg[n]) return;
  auto par = [&](int ip, float def) -> float { return ip < 0 ? def : X32[n * ldx + ip]; };
  const float omf = par(sn.ip_om, sn.fdef_om);
  float odef, okf;
  if (sn.ip_ode >= 0) { odef = par(sn.ip_ode, 0.f); okf = (1.f - omf) - odef; }
  else { odef = 1.f - omf; okf = 0.f; }
  const float exf = 3.f * (1.f + par(sn.ip_w0, sn.fdef_w0));
  // a parameter may hold -M or -beta (the reference's storage)
  const float Mf = (sn.ip_M >= 0 && sn.neg_M) ? -par(sn.ip_M, 0.f) : par(sn.ip_M, sn.fdef_M);
  const float dMf = Mf - sn.mref;
  const float al = par(sn.ip_alpha, sn.fdef_alpha);
  const float be = (sn.ip_beta >= 0 && sn.neg_beta) ? -par(sn.ip_beta, 0.f) : par(sn.ip_beta, sn.fdef_beta);
  const float a2 = al * al, b2 = be * be, ab = al * be;
  const int G = sn.G, nsn = sn.nsn;
  const float4 *__restrict__ node = sn.fnode;
  const float4 *__restrict__ p0 = sn.fsn, *__restrict__ p1 = sn.fsn + nsn, *__restrict__ p2 = sn.fsn + 2 * nsn;
  const float k5 = 1.50514997831990598f;  // 5 log10(2): 5 log10(x) = k5 log2(x)
  int bad = 0;
  float chi = 0.f, clo = 0.f;  // carry of the distance integral (float-float)
  float chi2 = 0.f, A = 0.f, B = 0.f, Cs = 0.f, sl = 0.f;
  for (int base = 0; base < nsn; base += 32) {
    const int i = base + lane;
    float p = 0.f;
    float4 q0, q1, q2;
    if (i < nsn) {
      // BATCH: the supernova planes first, then the nodes four at a time
      // (in-order accumulation as in the single-node loop)
      float zl2 = 0.f;
      if (BATCH) { q0 = p0[i]; q1 = p1[i]; q2 = p2[i]; zl2 = sn.fzl2[i]; }
      int g = 0;
      if (BATCH)
      for (; g + 4 <= G; g += 4) {
        float4 nd[4];
#pragma unroll
        for (int u = 0; u < 4; u++) nd[u] = node[(size_t)(g + u) * nsn + i];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const float e2 = fmaf(omf, nd[u].x, fmaf(okf, nd[u].y, odef * ex2_approx(exf * nd[u].z)));
          bad |= !(e2 > 0.f);
          p = fmaf(nd[u].w, rsqrt_approx(e2), p);
        }
      }
      for (; g < G; g++) {
        const float4 nd = node[(size_t)g * nsn + i];
        const float e2 = fmaf(omf, nd.x, fmaf(okf, nd.y, odef * ex2_approx(exf * nd.z)));
        bad |= !(e2 > 0.f);
        p = fmaf(nd.w, rsqrt_approx(e2), p);
      }
      if (!BATCH) { q0 = p0[i]; q1 = p1[i]; q2 = p2[i]; zl2 = sn.fzl2[i]; }
      const float e2z = fmaf(omf, q2.z, fmaf(okf, q2.w, odef * ex2_approx(exf * zl2)));
      bad |= !(e2z > 0.f);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float t = __shfl_up_sync(0xffffffffu, p, o);
      if (lane >= o) p += t;
    }
    float Is, Ie;
    two_sum_f(chi, p, Is, Ie);
    const float I = Is + (Ie + clo);
    ff_add(chi, clo, __shfl_sync(0xffffffffu, p, 31), 0.f);
    if (i < nsn) {
      const float dm = sk_series_f(okf, I, bad);
      bad |= !(dm > 0.f);
      const float dmu = k5 * lg2_approx(fmaxf(dm, 1e-30f) * q0.w);
      const float s2 = fmaf(ab, q2.y, fmaf(be, q2.x, fmaf(al, q1.w, fmaf(b2, q1.z, fmaf(a2, q1.y, q1.x)))));
      bad |= !(s2 > 0.f);
      const float d = fmaf(al, q0.y, fmaf(-be, q0.z, q0.x)) - dmu;
      const float is2 = rcp_approx(s2);
      if (sn.chi2mode == 0) { const float dd = d - dMf; chi2 = fmaf(dd * dd, is2, chi2); }
      else { A = fmaf(d * d, is2, A); B = fmaf(d, is2, B); Cs += is2; }
      if (sn.add_logdet) sl += lg2_approx(s2);
    }
  }
  bad = __any_sync(0xffffffffu, bad);
  float h0, l0, h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f, h3 = 0.f, l3 = 0.f;
  if (sn.chi2mode == 0) warp_sum_ff(chi2, h0, l0);
  else { warp_sum_ff(A, h0, l0); warp_sum_ff(B, h1, l1); warp_sum_ff(Cs, h2, l2); }
  if (sn.add_logdet) warp_sum_ff(sl, h3, l3);
  if (lane == 0) {
    if (bad) { flg[n] = 0; return; }
    double c2 = (double)h0 + (double)l0;
    if (sn.chi2mode != 0) {
      const double Bd = (double)h1 + (double)l1, Cd = (double)h2 + (double)l2;
      c2 = c2 - Bd * Bd / Cd + log(Cd / (2.0 * PMCG_PI));
    }
    // sum of log2 s^2 over supernovae, times ln 2
    const double ll = -0.5 * c2 - (sn.add_logdet ? 0.5 * 0.69314718055994531 * ((double)h3 + (double)l3) : 0.0);
    if (!isfinite(ll)) flg[n] = 0;
    else if (assign) logpost[n] = add + ll;
    else logpost[n] += ll;
  }
}

// One warp per sample n; the cumulative distance integral over redshift-sorted
// supernovae is a warp prefix scan of per-interval Gauss-Legendre sums.
// assign != 0: logpost[n] = add + logL; otherwise logpost[n] += logL.
template <bool F32, bool BATCH = false>
__device__ __forceinline__ void body_sn(const SnDev &sn, size_t N, int D, const double *__restrict__ X64,
                                        const float *__restrict__ X32, int ldx, double *__restrict__ logpost,
                                        short *__restrict__ flg, size_t n, int assign, double add) {
  if (F32) {
    body_sn_f32<BATCH>(sn, N, X32, ldx, logpost, flg, n, assign, add);
    return;
  }
  const int lane = threadIdx.x & 31;
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
  // a parameter may hold -M or -beta (the reference's storage)
  const double M = (sn.ip_M >= 0 && sn.neg_M) ? -par(sn.ip_M, 0.0) : par(sn.ip_M, sn.def_M);
  const double al = par(sn.ip_alpha, sn.def_alpha);
  const double be = (sn.ip_beta >= 0 && sn.neg_beta) ? -par(sn.ip_beta, 0.0) : par(sn.ip_beta, sn.def_beta);
  const double ex = 3.0 * (1.0 + w0);
  const int G = sn.G, nsn = sn.nsn;
  int bad = 0;
  double carry = 0.0, chi2 = 0.0, A = 0.0, B = 0.0, C = 0.0, sl = 0.0;
  for (int base = 0; base < nsn; base += 32) {
    const int i = base + lane;
    double Ii = 0.0;
    if (i < nsn) {
      for (int g = 0; g < G; g++) {
        const int q = i * G + g;
        double e2 = om * sn.na3[q] + ok * sn.na2[q] + ode * exp(ex * sn.nla[q]);
        if (!(e2 > 0.0)) bad = 1;
        else Ii += sn.nw[q] / sqrt(e2);
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
    else if (assign) logpost[n] = add + ll;
    else logpost[n] += ll;
  }
}

// ================================================================== (c) subset prior
// Gaussian / Student-t prior on a parameter subset, added to logpost[n] (one
// thread per sample). The centred coordinates x_sub - mu are formed first (so
// the single-precision form differences O(1) numbers, not O(|mu|) ones), then
// y = L^-1 (x_sub - mu) row by row from the packed factor (broadcast loads:
// every thread reads the same entry) and Q = |y|^2; the variable term in the
// working precision, the constant added in FP64.
template <typename Real, int MAXD>
__device__ __forceinline__ void body_prior(const PriorDev &p, size_t N, int D, const double *__restrict__ X64,
                                           const float *__restrict__ X32, int ldx, double *__restrict__ logpost,
                                           size_t n) {
  if (n >= N) return;
  const int d = p.d;
  const Real *mu = (sizeof(Real) == 8) ? (const Real *)p.mu : (const Real *)p.mu32;
  const Real *W = (sizeof(Real) == 8) ? (const Real *)p.Wt : (const Real *)p.Wt32;
  Real c[MAXD];
#pragma unroll
  for (int i = 0; i < MAXD; i++) {
    if (i < d) {
      const int j = p.idx[i];
      const Real x = (sizeof(Real) == 8) ? (Real)X64[n * D + j] : (Real)X32[n * ldx + j];
      c[i] = x - __ldg(mu + i);
    }
  }
  Real q = 0;
  int off = 0;
#pragma unroll
  for (int i = 0; i < MAXD; i++) {
    if (i < d) {
      Real y = 0;
#pragma unroll
      for (int j = 0; j <= i; j++) y = fma(__ldg(W + off + j), c[j], y);
      q = fma(y, y, q);
      off += i + 1;
    }
  }
  Real v;
  if (p.df > 0) {
    const Real t = q / (Real)p.df;
    if constexpr (sizeof(Real) == 4) v = -0.5f * ((float)p.df + (float)d) * log1pf(t);
    else v = -0.5 * ((double)p.df + d) * log1p(t);
  } else {
    v = (Real)-0.5 * q;
  }
  logpost[n] += p.lconst + (double)v;
}

// The prior body with its register footprint chosen by the prior's dimension
// (the same choice in the standalone kernel and the batch kernel).
template <typename Real>
__device__ __forceinline__ void body_prior_any(const PriorDev &p, size_t N, int D, const double *X64,
                                               const float *X32, int ldx, double *logpost, size_t n) {
  if (p.d <= 8) body_prior<Real, 8>(p, N, D, X64, X32, ldx, logpost, n);
  else if (p.d <= 20) body_prior<Real, 20>(p, N, D, X64, X32, ldx, logpost, n);
  else body_prior<Real, kMaxD>(p, N, D, X64, X32, ldx, logpost, n);
}

// ================================================================== (c) template
constexpr int kMT = 32;
template <typename Real>
__host__ __device__ inline size_t tpl_smem(int P, int threads) {
  size_t s = ((size_t)P * threads + (size_t)P * kMT + kMT) * sizeof(Real);
  if (sizeof(Real) == 4 && P <= kGramMaxP) {  // Gram form: phi [P][threads], G [Pp][Pp], b [Pp]
    const size_t Pp = (size_t)((P + 3) & ~3);
    const size_t g = ((size_t)P * threads + Pp * Pp + Pp) * sizeof(float);
    if (g > s) s = g;
  }
  return s;
}

// Single-precision template likelihood in Gram form (P <= MAXP): per sample
// chi2 = c0 - 2 phi.b + phi^T G phi, G = At^T At precomputed (P(P+1)/2 distinct
// products instead of M P); G rows staged in shared memory (float4 broadcasts),
// phi in registers; the three terms combined in FP64. For the c2 shape (P = 91,
// M = 2048) that is 22x fewer multiply-adds than the residual form.
template <int MAXP>
__device__ __forceinline__ void body_tpl_gram(const TplDev &t, size_t N, const float *__restrict__ X32, int ldx,
                                              double *__restrict__ logpost, const short *__restrict__ flg,
                                              size_t item, float *sm, int assign, double add) {
  const int P = t.P, Dp = t.Dpar, B = blockDim.x, Pp = (P + 3) & ~3;
  float *sphi = sm;                        // [P][B]
  float *sG = sphi + (size_t)P * B;        // [Pp][Pp]
  float *sb = sG + (size_t)Pp * Pp;        // [Pp]
  for (int e = threadIdx.x; e < Pp * Pp; e += B) sG[e] = t.G32[e];
  for (int e = threadIdx.x; e < Pp; e += B) sb[e] = t.b32[e];
  const size_t n = item * B + threadIdx.x;
  const bool act = n < N && flg[n];
  {
    float th[16];
    for (int i = 0; i < Dp; i++) th[i] = act ? X32[n * ldx + i] : 0.f;
    int p = 0;
    sphi[(p++) * B + threadIdx.x] = 1.f;
    for (int i = 0; i < Dp; i++) sphi[(p++) * B + threadIdx.x] = th[i];
    for (int i = 0; i < Dp; i++)
      for (int j = i; j < Dp; j++) sphi[(p++) * B + threadIdx.x] = th[i] * th[j];
  }
  __syncthreads();
  float phi[MAXP];
#pragma unroll
  for (int p = 0; p < MAXP; p++) phi[p] = (p < P) ? sphi[p * B + threadIdx.x] : 0.f;
  float q = 0.f, pb = 0.f;
#pragma unroll
  for (int i = 0; i < MAXP; i++) {
    if (i < P) {
      // inner = 0.5 G_ii phi_i + sum_{j<i} G_ij phi_j  (q = 2 sum_i phi_i inner)
      const float4 *row = reinterpret_cast<const float4 *>(sG + (size_t)i * Pp);
      float inner = 0.f;
#pragma unroll
      for (int j4 = 0; j4 <= i / 4; j4++) {
        const float4 g = row[j4];
        const int j = 4 * j4;
        inner = fmaf(g.x, j < i ? phi[j] : (j == i ? 0.5f * phi[i] : 0.f), inner);
        inner = fmaf(g.y, j + 1 < i ? phi[j + 1] : (j + 1 == i ? 0.5f * phi[i] : 0.f), inner);
        inner = fmaf(g.z, j + 2 < i ? phi[j + 2] : (j + 2 == i ? 0.5f * phi[i] : 0.f), inner);
        inner = fmaf(g.w, j + 3 < i ? phi[j + 3] : (j + 3 == i ? 0.5f * phi[i] : 0.f), inner);
      }
      q = fmaf(phi[i], inner, q);
      pb = fmaf(phi[i], sb[i], pb);
    }
  }
  if (act) {
    const double chi2 = t.c0 - 2.0 * (double)pb + 2.0 * (double)q;
    if (assign) logpost[n] = add - 0.5 * chi2;
    else logpost[n] += -0.5 * chi2;
  }
}

// Samples item*blockDim .. +blockDim-1; phi(theta) transposed in shared memory
// ([P][blockDim], conflict-free), At staged kMT rows at a time and read as
// broadcasts. assign != 0: logpost = add + logL; otherwise logpost += logL.
template <typename Real>
__device__ __forceinline__ void body_tpl(const TplDev &t, size_t N, const double *__restrict__ X64,
                                         const float *__restrict__ X32, int ldx, double *__restrict__ logpost,
                                         const short *__restrict__ flg, size_t item, Real *sm, int assign,
                                         double add) {
  if (sizeof(Real) == 4 && t.G32 != nullptr) {
    const float *X32f = reinterpret_cast<const float *>(X32);
    float *smf = reinterpret_cast<float *>(sm);
    if (t.P <= 32) body_tpl_gram<32>(t, N, X32f, ldx, logpost, flg, item, smf, assign, add);
    else body_tpl_gram<kGramMaxP>(t, N, X32f, ldx, logpost, flg, item, smf, assign, add);
    return;
  }
  const int P = t.P, Dp = t.Dpar, M = t.M, B = blockDim.x;
  Real *sphi = sm;                        // [P][B]
  Real *sA = sphi + (size_t)P * B;        // [P][kMT]
  Real *sd = sA + (size_t)P * kMT;        // [kMT]
  const size_t n = item * B + threadIdx.x;
  const bool act = n < N && flg[n];
  {
    Real th[64];
    for (int i = 0; i < Dp; i++)
      th[i] = act ? (sizeof(Real) == 8 ? (Real)X64[n * Dp + i] : (Real)X32[n * ldx + i]) : (Real)0;
    int p = 0;
    sphi[(p++) * B + threadIdx.x] = (Real)1;
    for (int i = 0; i < Dp; i++) sphi[(p++) * B + threadIdx.x] = th[i];
    for (int i = 0; i < Dp; i++)
      for (int j = i; j < Dp; j++) sphi[(p++) * B + threadIdx.x] = th[i] * th[j];
  }
  Real chi2 = 0;
  double chi2d = 0.0;
  const Real *Asrc = (sizeof(Real) == 8) ? (const Real *)t.At : (const Real *)t.At32;
  const Real *dsrc = (sizeof(Real) == 8) ? (const Real *)t.dt : (const Real *)t.dt32;
  for (int m0 = 0; m0 < M; m0 += kMT) {
    const int mt = min(kMT, M - m0);
    __syncthreads();
    for (int e = threadIdx.x; e < P * kMT; e += B) {
      int p = e / kMT, r = e - p * kMT;
      sA[e] = (r < mt) ? Asrc[(size_t)(m0 + r) * P + p] : (Real)0;
    }
    for (int r = threadIdx.x; r < kMT; r += B) sd[r] = (r < mt) ? dsrc[m0 + r] : (Real)0;
    __syncthreads();
    for (int r0 = 0; r0 < kMT; r0 += 8) {
      Real acc[8];
#pragma unroll
      for (int q = 0; q < 8; q++) acc[q] = sd[r0 + q];
      for (int p = 0; p < P; p++) {
        const Real f = sphi[p * B + threadIdx.x];
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
  if (act) {
    if (assign) logpost[n] = add - 0.5 * chi2d;
    else logpost[n] += -0.5 * chi2d;
  }
}

// ================================================================== (d) weights
// FAST (single-precision runs): each factor e^{x}, x <= 0, is evaluated in
// single precision (relative error ~1e-7, below the FP32 log-densities it
// weighs); the sums stay FP64. Otherwise everything is FP64.
template <bool FAST>
__device__ __forceinline__ double wexp(double x) {
  return FAST ? (double)expf((float)x) : exp(x);
}
template <bool FAST = false>
__device__ __forceinline__ void wred_add(WRed &r, double l) {
  if (l > r.m) {
    double e = wexp<FAST>(r.m - l);  // r.m == -inf gives 0
    r.s = r.s * e + 1.0;
    r.t = r.t * e + l;
    r.q = r.q * e * e + 1.0;
    r.m = l;
  } else {
    double e = wexp<FAST>(l - r.m);
    r.s += e;
    r.t += e * l;
    r.q += e * e;
  }
  r.n += 1.0;
}

// Block reduction of a WRed in a fixed order; thread 0 receives the result.
template <bool FAST = false>
__device__ __forceinline__ WRed block_wred(WRed r, WRed *s_r) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) r = wred_merge<FAST>(r, wred_shfl(r, o));
  if ((threadIdx.x & 31) == 0) s_r[threadIdx.x >> 5] = r;
  __syncthreads();
  WRed a = s_r[0];
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) a = wred_merge<FAST>(a, s_r[w]);
  return a;
}

// Order-preserving 64-bit key of a double (larger key <=> larger value; every
// key of a non-NaN value is above 0).
__device__ __forceinline__ unsigned long long dkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// Samples tile*kTileW .. +kTileW-1: log-weights and the tile's partial record.
// logq == nullptr means log q = 0 (re-normalising given log-weights).
// FAST (single-precision runs, 256 threads, 8 samples per thread): the tile
// maximum m first (integer compare of order keys), then e = exp(l - m) in
// single precision with per-thread FP32 partials of s, q and sum e (l - m) over
// the thread's 8 samples, summed across threads in FP64 (GB300 issues FP64 at
// a small fraction of the FP32 rate: about 6 FP64 operations per sample
// instead of a rescaling merge per sample). Otherwise the FP64 online record.
template <bool FAST = false>
__device__ __forceinline__ void body_weights_tile(size_t N, double beta, const double *__restrict__ logpost,
                                                  const double *__restrict__ logq, short *__restrict__ flg,
                                                  double *__restrict__ logw, WRed *__restrict__ part, size_t tile,
                                                  WRed *s_r) {
  const size_t base = tile * kTileW;
  if constexpr (FAST) {
    constexpr int PER = kTileW / 256;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double l[PER], lq[PER];
    short fl[PER];
    unsigned long long mk = 0ull;
    // every load first (in bounds for n < N; values of unflagged samples are
    // not used), so a thread waits for one round of loads, not one per sample
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const size_t n = base + threadIdx.x + (size_t)j * 256;
      fl[j] = 0;
      l[j] = 0.0;
      lq[j] = 0.0;
      if (n < N) {
        fl[j] = flg[n];
        l[j] = logpost[n];
        if (logq) lq[j] = logq[n];
      }
    }
#pragma unroll
    for (int j = 0; j < PER; j++) {
      const size_t n = base + threadIdx.x + (size_t)j * 256;
      double v = -INFINITY;
      if (n < N) {
        if (fl[j]) {
          v = beta * l[j] - lq[j];
          if (!isfinite(v)) { v = -INFINITY; flg[n] = 0; }
        }
        logw[n] = v;
      }
      l[j] = v;
      if (v > -INFINITY) mk = (dkey(v) > mk) ? dkey(v) : mk;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, mk, o);
      mk = (t > mk) ? t : mk;
    }
    unsigned long long *s_key = reinterpret_cast<unsigned long long *>(s_r);   // [8]
    double *s_sum = reinterpret_cast<double *>(s_r) + 8;                      // [8][4]
    if (lane == 0) s_key[warp] = mk;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < 8; w++) mk = (s_key[w] > mk) ? s_key[w] : mk;
    const double m = mk ? dkey_value(mk) : -INFINITY;
    float fs = 0.f, ft = 0.f, fq = 0.f;
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
      if (l[j] > -INFINITY) {
        const float d = (float)(l[j] - m);
        const float e = expf(d);
        fs += e;
        ft = fmaf(e, d, ft);
        fq = fmaf(e, e, fq);
        cnt++;
      }
    }
    double ds = fs, dt = ft, dq = fq;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ds += __shfl_down_sync(0xffffffffu, ds, o);
      dt += __shfl_down_sync(0xffffffffu, dt, o);
      dq += __shfl_down_sync(0xffffffffu, dq, o);
      cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
      s_sum[4 * warp] = ds; s_sum[4 * warp + 1] = dt; s_sum[4 * warp + 2] = dq; s_sum[4 * warp + 3] = (double)cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      WRed r = wred_empty();
      double S = 0.0, T = 0.0, Q = 0.0, C = 0.0;
      for (int w = 0; w < 8; w++) { S += s_sum[4 * w]; T += s_sum[4 * w + 1]; Q += s_sum[4 * w + 2]; C += s_sum[4 * w + 3]; }
      if (mk) { r.m = m; r.s = S; r.t = T + m * S; r.q = Q; }
      r.n = C;
      part[tile] = r;
    }
    return;
  }
  WRed r = wred_empty();
  for (int q = threadIdx.x; q < kTileW; q += blockDim.x) {
    const size_t n = base + q;
    if (n >= N) break;
    double l = -INFINITY;
    if (flg[n]) {
      l = beta * logpost[n] - (logq ? logq[n] : 0.0);
      if (!isfinite(l)) { l = -INFINITY; flg[n] = 0; }
    }
    logw[n] = l;
    if (l > -INFINITY) wred_add<FAST>(r, l);
  }
  WRed a = block_wred<FAST>(r, s_r);
  if (threadIdx.x == 0) part[tile] = a;
}

// Merge the nb tile records of one sample and derive logSum, evidence,
// perplexity and ESS. The largest tile maximum M comes first (order keys,
// integer compares); every record is then rescaled once to M (s e, t e, q e^2
// with e = e^{m_b - M}) and s, t, q, n are plain sums, per thread strided,
// then in a fixed tree: one exponential per record instead of two per merge,
// and no exponential on the tree's dependent path. s_r: 8 records of shared
// scratch (blockDim.x <= 256).
template <bool FAST = false>
__device__ __forceinline__ void body_weights_final(int nb, const WRed *__restrict__ part, size_t N, DevStats *st,
                                                   WRed *s_r) {
  unsigned long long *skey = reinterpret_cast<unsigned long long *>(s_r);  // [8]
  double *ssum = reinterpret_cast<double *>(s_r) + 8;                      // [8][4]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned long long km = 0ull;  // below the key of every value, -inf included
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const unsigned long long kb = dkey(part[b].m);
    km = kb > km ? kb : km;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, km, o);
    km = v > km ? v : km;
  }
  if (lane == 0) skey[warp] = km;
  __syncthreads();
  km = 0ull;
  for (int w = 0; w < nw; w++) km = skey[w] > km ? skey[w] : km;
  const double M = dkey_value(km);
  double s = 0.0, t = 0.0, q = 0.0, n = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const WRed r = part[b];
    n += r.n;
    if (r.m == -INFINITY) continue;
    const double e = FAST ? (double)expf((float)(r.m - M)) : exp(r.m - M);
    s = fma(r.s, e, s);
    t = fma(r.t, e, t);
    q = fma(r.q * e, e, q);
  }
  s = warp_sum(s);
  t = warp_sum(t);
  q = warp_sum(q);
  n = warp_sum(n);
  if (lane == 0) {
    ssum[4 * warp] = s;
    ssum[4 * warp + 1] = t;
    ssum[4 * warp + 2] = q;
    ssum[4 * warp + 3] = n;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  st->f32_range = 0;  // set again by this iteration's update if needed
  WRed a;
  a.m = M;
  a.s = a.t = a.q = a.n = 0.0;
  for (int w = 0; w < nw; w++) {
    a.s += ssum[4 * w];
    a.t += ssum[4 * w + 1];
    a.q += ssum[4 * w + 2];
    a.n += ssum[4 * w + 3];
  }
  if (a.n == 0.0 || a.m == -INFINITY) {
    st->status = -9011;  // PMCG_ENOWEIGHT
    st->nok = 0.0;
    return;
  }
  st->status = 0;
  const double ls = a.m + log(a.s);
  st->logSum = ls;
  st->maxW = a.m;
  st->H = ls - a.t / a.s;
  st->sumw2 = a.q / (a.s * a.s);
  st->nok = a.n;
  st->ln_evidence = ls - log((double)N);
  st->perplexity = exp(st->H) / (double)N;
  st->ess = 1.0 / st->sumw2;
}

// ================================================================== (e) EM, mixed
// Per-sample single-precision weight factor aw = log w - logSum - log q
// (-inf where flg == 0): one FP64 subtraction per sample, not per component.
__device__ __forceinline__ void body_em_factor(size_t N, const double *__restrict__ logw,
                                               const double *__restrict__ logq, const DevStats *__restrict__ st,
                                               float *__restrict__ aw, size_t tile) {
  const double ls = st->logSum;
  const size_t base = tile * kTileW;
  for (int q = threadIdx.x; q < kTileW; q += blockDim.x) {
    const size_t n = base + q;
    if (n >= N) break;
    const double l = logw[n];
    aw[n] = (l > -INFINITY) ? (float)(l - ls - logq[n]) : -INFINITY;
  }
}

// Rows per staging tile of the EM statistics: 64 for D > 16, 256 for D <= 16
// (each tile costs three barriers, so small-D tiles carry more rows; measured
// at the template workload, D = 12 with every pair listed: 128 -> 256 rows took
// the EM stage from 0.322 to 0.289 ms; 128 rows for D > 16 gained nothing);
// the list buffer holds two tiles plus one pass of listing (at most 256
// entries).
__host__ __device__ inline int em_tile_rows(int Dp) { return Dp <= 16 ? 4 * kTile32 : kTile32; }
__host__ __device__ inline int em_list_buf(int Dp) { return 2 * em_tile_rows(Dp) + 256; }
// Row stride of the augmented whitened rows (Dp + 4 columns): a multiple of 4
// floats (float4 rows) whose quotient by 4 is odd, so the 16-byte stores of 8
// consecutive rows fall in 8 different 4-bank groups (conflict-free).
__host__ __device__ inline int em_row_stride(int Dp) { return (((Dp + 4) / 4) & 1) ? Dp + 4 : Dp + 8; }
// Row stride of the gathered sample rows (Dp columns), by the same rule.
__host__ __device__ inline int em_x_stride(int Dp) { return ((Dp / 4) & 1) ? Dp : Dp + 4; }
// A pair whose single-precision weight vt = exp(aw + lt) / itau underflows
// (aw + lt below log FLT_MIN = -87.3) adds exactly nothing in FP32 and less
// than 1e-38 relative in any precision: such pairs are skipped.
constexpr float kEmLogMin = -87.0f;

// Whitening schedule of one warp: a count, then up to 16 (slice, row block) tasks.
constexpr int kEmSchedStride = 17;

__host__ __device__ inline void em32_layout(int D, int ldx, int threads, size_t *tile_bytes, size_t *red_bytes) {
  const int Dp = ldx, Da = Dp + 4, nb = Da / 4, NB = nb * (nb + 1) / 2, G = threads / NB;
  const int T = em_tile_rows(Dp);
  *tile_bytes = (size_t)(Dp * Dp + Dp + T * em_row_stride(Dp) + 2 * T * em_x_stride(Dp) + 3 * em_list_buf(Dp) + 40 +
                         (threads / 32) * kEmSchedStride) *
                sizeof(float);
  *red_bytes = (size_t)G * NB * 16 * sizeof(float2);
}

// Statistics of component k over sample chunk s, accumulated in the component's
// whitened frame a = L_k^-1 (x - mu_k) (entries O(1)); a covariance of condition
// 1e6 cannot be represented to its small eigenvalues in FP32 in the raw frame.
//
// The chunk is scanned 256 samples at a time; the pairs whose weight does not
// underflow (aw + lt > kEmLogMin) are compacted, in sample order (warp ballots
// and a block prefix), into a staging list. Every full tile of T listed
// samples is then gathered (x rows in 16-byte copies, cp.async into one of two
// buffers, the next tile's rows while this tile is processed), whitened with
// L^-1 staged transposed (float4 broadcasts; the (slice, row block) tasks
// spread over the warps longest first; rows stored as float4 at a stride that
// keeps 8 consecutive rows in distinct banks), and accumulated: the augmented rows [a, 1, 1/tau, 0, 0]
// with weight vt give in the lower triangle of sum vt a a^T: S2 (whitened), S1
// (row Dp), St (Dp,Dp) and S0 (Dp+1,Dp). Each thread owns one 4x4 block for one
// sample group; FP32 sums are flushed into float-float pairs every kFlushTiles tiles. The
// order of every sum depends only on the run's own data (deterministic).
// mask (optional): bit j of word mask[k * W + w] set iff sample 32 w + j is
// listed for component k (em_mask_kernel). With a mask the block walks 32-sample
// words instead of testing every sample; the list and every sum are identical.
__device__ __forceinline__ void body_em_stats_f32(const DevMixView &m, size_t N, int S, const float *__restrict__ X,
                                                  const float *__restrict__ aw, const float *__restrict__ lt,
                                                  const float *__restrict__ Qv, double *__restrict__ part, int k,
                                                  int s, unsigned char *smem, const uint32_t *__restrict__ mask = nullptr) {
  const int D = m.D, E = em_E(D);
  if (m.w[k] <= 0.0) return;
  const int Dp = m.ldx, Da = Dp + 4, nb = Da / 4, NB = nb * (nb + 1) / 2, nib = Dp / 4;
  const int ldt = em_x_stride(Dp);
  const int G = blockDim.x / NB;
  float *sWT = reinterpret_cast<float *>(smem);   // [Dp][Dp]  (L^-1)^T
  float *sb = sWT + Dp * Dp;                      // [Dp]      L^-1 mu
  const int T = em_tile_rows(Dp), LB = em_list_buf(Dp);
  const int flush_tiles = kFlushTiles * kTile32 / T;  // the same rows per FP32 partial for every T
  const int lda = em_row_stride(Dp);
  float *sa = sb + Dp;                            // [T][lda] augmented whitened rows
  float *sx = sa + T * lda;                       // [2][T][ldt] gathered rows, two buffers
  float *lvt = sx + 2 * T * ldt;                  // [LB] listed vt
  float *ltau = lvt + LB;                         // [LB] listed 1/tau
  int *lidx = reinterpret_cast<int *>(ltau + LB);  // [LB] listed sample offsets
  int *wcnt = lidx + LB;                          // [32] per-warp counts
  int *sched = wcnt + 32;                         // [nwarp][kEmSchedStride] whitening tasks
  const size_t chunk = (N + S - 1) / S;
  const size_t n0 = (size_t)s * chunk, n1 = (n0 + chunk < N) ? n0 + chunk : N;
  const float nu = (float)m.df, rnd = 1.0f / ((float)m.df + (float)D);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  for (int e = tid; e < Dp * Dp; e += blockDim.x) {
    int i = e / Dp, j = e - i * Dp;
    sWT[j * Dp + i] = (i < D) ? m.W32[(size_t)k * D * Dp + (size_t)i * Dp + j] : 0.f;
  }
  for (int i = tid; i < Dp; i += blockDim.x) sb[i] = (i < D) ? m.b32[(size_t)k * D + i] : 0.f;
  // The whitening tasks (32-row slice, 4-row block ib; cost ib + 1) of a tile,
  // longest first, each to the least-loaded warp: every warp's share is within
  // one task of the mean (which warp computes an output does not change it).
  if (tid == 0) {
    int *load = wcnt;   // free until the listing
    for (int w = 0; w < nwarp; w++) { load[w] = 0; sched[w * kEmSchedStride] = 0; }
    for (int ib = nib - 1; ib >= 0; ib--) {
      for (int sl = 0; sl < T / 32; sl++) {
        int best = 0;
        for (int w = 1; w < nwarp; w++)
          if (load[w] < load[best]) best = w;
        int *sw = sched + best * kEmSchedStride;
        if (sw[0] < kEmSchedStride - 1) sw[1 + sw[0]++] = (sl << 4) | ib;
        load[best] += ib + 1;
      }
    }
  }
  __syncthreads();
  const int blk = tid % NB, grp = tid / NB;
  const bool active = grp < G;
  int bi = 0;
  while ((bi + 1) * (bi + 2) / 2 <= blk) bi++;
  const int bj = blk - bi * (bi + 1) / 2;
  // per-tile FP32 sums acc; every flush adds them exactly (TwoSum) into a
  // float-float pair (chi, clo): FP32 instructions only, where an FP64 add costs
  // a warp-wide pass of the narrow FP64 pipe
  float acc[16], chi[16], clo[16];
#pragma unroll
  for (int e = 0; e < 16; e++) { acc[e] = 0.f; chi[e] = 0.f; clo[e] = 0.f; }
  int tiles = 0;

  // Gather the rows of listed entries [at, at + nt) (nt <= T) into dst, 16
  // bytes per copy (cp.async, one commit group; rows past nt are zeroed).
  const int cpr = Dp / 4;   // 16-byte chunks per row
  auto gather = [&](int at, int nt, float *dst) {
    for (int c = tid; c < T * cpr; c += blockDim.x) {
      const int r = c / cpr, q = c - r * cpr;
      float *d = dst + r * ldt + 4 * q;
      if (r < nt) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(d)),
                     "l"(X + (n0 + (size_t)lidx[at + r]) * Dp + 4 * q)
                     : "memory");
      } else {
        *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // Accumulate listed entries [at, at + nt) (nt <= T) from their gathered rows
  // src; `next`: a later gather is in flight (wait for all groups but that one).
  auto process = [&](int at, int nt, const float *src, bool next) {
    for (int r = tid; r < T; r += blockDim.x)
      *reinterpret_cast<float4 *>(sa + r * lda + Dp) = make_float4(1.f, (r < nt) ? ltau[at + r] : 1.f, 0.f, 0.f);
    if (next) asm volatile("cp.async.wait_group 1;" ::: "memory");
    else asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    const int ntask = sched[warp * kEmSchedStride];
    for (int u = 0; u < ntask; u++) {
      const int code = sched[warp * kEmSchedStride + 1 + u];
      const int ib = code & 15;
      const int r = (code >> 4) * 32 + lane;
      float o0 = -sb[4 * ib], o1 = -sb[4 * ib + 1], o2 = -sb[4 * ib + 2], o3 = -sb[4 * ib + 3];
      const float *xr = src + r * ldt;
      const int jmax = 4 * ib + 4;
      for (int j = 0; j < jmax; j += 4) {
        const float4 x4 = *reinterpret_cast<const float4 *>(xr + j);
        const float xs[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
          const float4 w4 = *reinterpret_cast<const float4 *>(sWT + (j + jj) * Dp + 4 * ib);
          o0 = fmaf(w4.x, xs[jj], o0); o1 = fmaf(w4.y, xs[jj], o1);
          o2 = fmaf(w4.z, xs[jj], o2); o3 = fmaf(w4.w, xs[jj], o3);
        }
      }
      const bool live = r < nt;
      *reinterpret_cast<float4 *>(sa + r * lda + 4 * ib) =
          live ? make_float4(o0, o1, o2, o3) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    if (active) {
      for (int q = grp; q < nt; q += G) {
        const float w = lvt[at + q];
        float4 ai = *reinterpret_cast<const float4 *>(sa + q * lda + 4 * bi);
        const float4 aj = *reinterpret_cast<const float4 *>(sa + q * lda + 4 * bj);
        ai.x *= w; ai.y *= w; ai.z *= w; ai.w *= w;
        acc[0] = fmaf(ai.x, aj.x, acc[0]);   acc[1] = fmaf(ai.x, aj.y, acc[1]);
        acc[2] = fmaf(ai.x, aj.z, acc[2]);   acc[3] = fmaf(ai.x, aj.w, acc[3]);
        acc[4] = fmaf(ai.y, aj.x, acc[4]);   acc[5] = fmaf(ai.y, aj.y, acc[5]);
        acc[6] = fmaf(ai.y, aj.z, acc[6]);   acc[7] = fmaf(ai.y, aj.w, acc[7]);
        acc[8] = fmaf(ai.z, aj.x, acc[8]);   acc[9] = fmaf(ai.z, aj.y, acc[9]);
        acc[10] = fmaf(ai.z, aj.z, acc[10]); acc[11] = fmaf(ai.z, aj.w, acc[11]);
        acc[12] = fmaf(ai.w, aj.x, acc[12]); acc[13] = fmaf(ai.w, aj.y, acc[13]);
        acc[14] = fmaf(ai.w, aj.z, acc[14]); acc[15] = fmaf(ai.w, aj.w, acc[15]);
      }
    }
    if (++tiles == flush_tiles) {
      tiles = 0;
#pragma unroll
      for (int e = 0; e < 16; e++) { ff_add(chi[e], clo[e], acc[e], 0.f); acc[e] = 0.f; }
    }
    __syncthreads();
  };

  int fill = 0;  // listed entries (identical in every thread)
  int cur = 0;   // gather buffer of the next tile: sx + cur * T * ldt
  // Process every full tile where it lies, the next tile's rows gathered while
  // this one is processed, then move the remainder (fewer than T entries, so
  // at most one per thread) to the front.
  auto drain = [&]() {
    int at = 0;
    if (fill >= T) gather(0, T, sx + cur * T * ldt);
    while (fill - at >= T) {
      const bool next = fill - at >= 2 * T;
      if (next) gather(at + T, T, sx + (cur ^ 1) * T * ldt);
      process(at, T, sx + cur * T * ldt, next);
      at += T;
      cur ^= 1;
    }
    if (at > 0) {
      const int rem = fill - at;
      int ri = 0;
      float rv = 0.f, rt = 0.f;
      if (tid < rem) { ri = lidx[at + tid]; rv = lvt[at + tid]; rt = ltau[at + tid]; }
      __syncthreads();
      if (tid < rem) { lidx[tid] = ri; lvt[tid] = rv; ltau[tid] = rt; }
      __syncthreads();
      fill = rem;
    }
  };
  if (mask != nullptr) {
    const size_t W = (N + 31) / 32;
    const size_t wbeg = n0 / 32, wend = (n1 + 31) / 32;
    for (size_t wb = wbeg; wb < wend && n0 < n1; wb += blockDim.x) {
      const size_t wi = wb + tid;
      uint32_t bits = 0u;
      if (wi < wend) {
        bits = mask[(size_t)k * W + wi];
        const size_t base = wi * 32;
        if (base < n0) bits &= ~0u << (unsigned)(n0 - base);
        if (base + 32 > n1) bits &= (1u << (unsigned)(n1 - base)) - 1u;
      }
      const int c = __popc(bits);
      int incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) wcnt[warp] = incl;
      __syncthreads();
      int off = 0, tot = 0;
      for (int w = 0; w < nwarp; w++) {
        const int cw = wcnt[w];
        off += (w < warp) ? cw : 0;
        tot += cw;
      }
      const int pos = off + incl - c;   // position of this word's first entry in this pass
      // the warp's entry range in this pass: [wlo, whi)
      const int wlo = __shfl_sync(0xffffffffu, pos, 0), whi = __shfl_sync(0xffffffffu, pos + c, 31);
      const unsigned ltmask = (1u << lane) - 1u;
      // emit in rounds that fit the list buffer, processing full tiles in
      // between. Each warp expands its own 32 words, one word per step and one
      // bit per lane, so the entries of a word land in consecutive list slots
      // (conflict-free) and a warp whose entries all lie outside the round
      // skips it; then the new entries' weights are read one entry per thread.
      for (int done = 0; done < tot;) {
        const int take = min(LB - fill, tot - done);
        if (whi > done && wlo < done + take) {
          for (int j = 0; j < 32; j++) {
            const uint32_t bj = __shfl_sync(0xffffffffu, bits, j);
            const int pj = __shfl_sync(0xffffffffu, pos, j);
            if (pj + __popc(bj) <= done || pj >= done + take) continue;   // warp-uniform
            if ((bj >> lane) & 1u) {
              const int p = pj + __popc(bj & ltmask);
              if (p >= done && p < done + take)
                lidx[fill + p - done] = (int)((wb + (size_t)(warp * 32 + j)) * 32 + lane - n0);
            }
          }
        }
        __syncthreads();
        for (int q = fill + tid; q < fill + take; q += blockDim.x) {
          const size_t n = n0 + (size_t)lidx[q];
          const float e = aw[n] + lt[(size_t)k * N + n];
          const float v = expf(e);
          const float it = (m.df > 0) ? (nu + Qv[(size_t)k * N + n]) * rnd : 1.f;
          lvt[q] = (m.df > 0) ? v / it : v;
          ltau[q] = it;
        }
        fill += take;
        done += take;
        __syncthreads();
        drain();
      }
      __syncthreads();  // wcnt is rewritten by the next pass
    }
  } else
  for (size_t c0 = n0; c0 < n1; c0 += blockDim.x) {
    const size_t n = c0 + tid;
    bool act = false;
    float vt = 0.f, it = 1.f;
    if (n < n1) {
      const float e = aw[n] + lt[(size_t)k * N + n];
      if (e > kEmLogMin) {
        act = true;
        const float v = expf(e);
        if (m.df > 0) it = (nu + Qv[(size_t)k * N + n]) * rnd;
        vt = (m.df > 0) ? v / it : v;
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, act);
    if (lane == 0) wcnt[warp] = __popc(bal);
    __syncthreads();
    int off = 0, tot = 0;
    for (int w = 0; w < nwarp; w++) {
      const int c = wcnt[w];
      off += (w < warp) ? c : 0;
      tot += c;
    }
    if (act) {
      const int pos = fill + off + __popc(bal & ((1u << lane) - 1u));
      lidx[pos] = (int)(n - n0);
      lvt[pos] = vt;
      ltau[pos] = it;
    }
    fill += tot;
    __syncthreads();
    drain();
  }
  if (fill > 0) {
    gather(0, fill, sx + cur * T * ldt);
    process(0, fill, sx + cur * T * ldt, false);
  }
#pragma unroll
  for (int e = 0; e < 16; e++) ff_add(chi[e], clo[e], acc[e], 0.f);
  __syncthreads();
  // entry-major [16][G][NB] pairs: for each entry a warp writes consecutive
  // words (grp * NB + blk == tid)
  float2 *red = reinterpret_cast<float2 *>(smem);
  if (active) {
#pragma unroll
    for (int e = 0; e < 16; e++) red[((size_t)e * G + grp) * NB + blk] = make_float2(chi[e], clo[e]);
  }
  __syncthreads();
  double *out = part + ((size_t)k * S + s) * E;
  // one (block, entry) per thread: the float-float sum over the G groups in a
  // fixed order, then one exact conversion (hi + lo spans at most 48 bits)
  for (int be = tid; be < NB * 16; be += blockDim.x) {
    const int e = be / NB, b = be - e * NB;
    int rbi = 0;
    while ((rbi + 1) * (rbi + 2) / 2 <= b) rbi++;
    const int rbj = b - rbi * (rbi + 1) / 2;
    {
      float2 v = red[(size_t)e * G * NB + b];
      for (int g = 1; g < G; g++) {
        const float2 u = red[((size_t)e * G + g) * NB + b];
        ff_add(v.x, v.y, u.x, u.y);
      }
      const double t = (double)v.x + (double)v.y;
      const int r = 4 * rbi + e / 4, c = 4 * rbj + e % 4;
      if (r < D && c <= r) out[2 + D + tri_idx(r, c)] = t;
      else if (r == Dp && c < D) out[2 + c] = t;
      else if (r == Dp && c == Dp) out[1] = t;
      else if (r == Dp + 1 && c == Dp) out[0] = t;
    }
  }
}

// ================================================================== (e) EM finalise
__host__ __device__ inline size_t finalize_smem(int D, int whitened) {
  (void)whitened;
  return (size_t)(em_E(D) + 3 * D * D + 3 * D) * sizeof(double);  // C padded to D x (D + 1)
}

// Component k: fixed-order sum of the chunk partials, new mean and covariance
// (mapped back from the whitened frame with the old factor when whitened: mu' =
// mu + L d, Sigma' = L Sigma_w L^T), band limit, FP64 Cholesky; the dead rule
// buries the component (weight 0, parameters kept).
__device__ __forceinline__ void body_em_finalize(const DevMixView &m, double *w, double *mu, double *L, size_t N,
                                                 int S, const double *__restrict__ part,
                                                 const int *__restrict__ counts, int band_limit, int whitened, int k,
                                                 const DevStats *stats, double *sh, int *s_dead) {
  const int D = m.D, E = em_E(D);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double *st = sh;             // E
  const int ldc = D + 1;       // row stride of C: a column read by 32 lanes spans all banks
  double *C = st + E;          // D*ldc
  double *Lo = C + D * ldc;    // D*D old factor (whitened only)
  double *T = Lo + D * D;      // D*D scratch (whitened only); then D: mean shift
  double *rp = T + D * D + D;  // D reciprocal pivots
  if (stats->status != 0) return;  // the weight step failed: keep the proposal
  if (m.w[k] <= 0.0) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    // chunk order; loads issued eight at a time
    const double *pe = part + (size_t)k * S * E + e;
    double t = 0.0;
    int s = 0;
    for (; s + 8 <= S; s += 8) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = pe[(size_t)(s + u) * E];
#pragma unroll
      for (int u = 0; u < 8; u++) t += v[u];
    }
    for (; s < S; s++) t += pe[(size_t)s * E];
    st[e] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double S0 = st[0], St = st[1];
    *s_dead = (counts[k] < kMinCount) || !(S0 >= 1.0 / (double)N) || !(St > 0.0) || !isfinite(S0) || !isfinite(St);
  }
  __syncthreads();
  if (*s_dead) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  const double S0 = st[0], St = st[1];
  // the weighted mean shift d = S1 / St (D divisions in parallel) and 1 / S0
  double *dm = whitened ? T + D * D : C + D * ldc;
  for (int i = threadIdx.x; i < D; i += blockDim.x) dm[i] = st[2 + i] / St;
  __syncthreads();
  const double rS0 = 1.0 / S0;
  for (int i = warp; i < D; i += nw)
    for (int j = lane; j < D; j += 32) {
      const int a = i > j ? i : j, b = i > j ? j : i;
      C[i * ldc + j] = (st[2 + D + tri_idx(a, b)] - St * dm[i] * dm[j]) * rS0;
      if (whitened) Lo[i * D + j] = (j <= i) ? m.L[(size_t)k * D * D + i * D + j] : 0.0;
    }
  __syncthreads();
  // Whitened frame without a band limit: Sigma' = Lo C Lo^T and L' = Lo chol(C)
  // is its Cholesky factor (a product of lower-triangular factors with positive
  // diagonals), so the well-conditioned C is factorised and one triangular
  // product (D^3/6 multiply-adds) replaces the two dense ones (D^3).
  const bool banded = band_limit > 0 && band_limit < D;
  const bool via_lo = whitened && !banded;
  if (whitened && banded) {
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // T = Lo C
      int i = e / D, j = e - i * D;
      double t = 0.0;
      for (int q = 0; q <= i; q++) t += Lo[i * D + q] * C[q * ldc + j];
      T[e] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // C = T Lo^T
      int i = e / D, j = e - i * D;
      double t = 0.0;
      for (int q = 0; q <= j; q++) t += T[i * D + q] * Lo[j * D + q];
      C[i * ldc + j] = t;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {  // symmetrise exactly
      int i = e / D, j = e - i * D;
      if (j < i) T[e] = 0.5 * (C[i * ldc + j] + C[j * ldc + i]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      int i = e / D, j = e - i * D;
      if (j < i) { C[i * ldc + j] = T[e]; C[j * ldc + i] = T[e]; }
    }
    __syncthreads();
  }
  if (banded) {
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      int i = e / D, j = e - i * D;
      if ((i > j ? i - j : j - i) >= band_limit) C[i * ldc + j] = 0.0;
    }
    __syncthreads();
  }
  // Right-looking Cholesky of the lower triangle, one barrier per column: the
  // columns stay unscaled (the update uses 1/p_j^2 = rp_j^2) and the thread
  // that updates the next diagonal entry (thread 0: warp 0 takes the first row
  // and lane 0 its first column) derives the next pivot; columns are scaled by
  // rp_j at the end. Rows go to warps and columns to lanes.
  auto pivot = [&](int j) {
    double d = C[j * ldc + j];
    if (!(d > 0.0) || !isfinite(d)) { *s_dead = 1; d = 1.0; }
    // one reciprocal square root for both the pivot and its inverse: the FP64
    // pipe is narrow and this chain runs on one thread between barriers
    const double r = rsqrt(d);
    C[j * ldc + j] = d * r;
    rp[j] = r;
  };
  if (threadIdx.x == 0) pivot(0);
  __syncthreads();
  for (int j = 0; j < D; j++) {
    const double r2 = rp[j] * rp[j];
    for (int i = j + 1 + warp; i < D; i += nw) {
      const double cij = C[i * ldc + j] * r2;
      for (int c = j + 1 + lane; c <= i; c += 32) C[i * ldc + c] = fma(-cij, C[c * ldc + j], C[i * ldc + c]);
    }
    if (threadIdx.x == 0 && j + 1 < D) pivot(j + 1);
    __syncthreads();
  }
  for (int i = warp; i < D; i += nw)
    for (int j = lane; j < i; j += 32) C[i * ldc + j] *= rp[j];
  __syncthreads();
  if (*s_dead) {
    if (threadIdx.x == 0) w[k] = 0.0;
    return;
  }
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    double d;
    if (whitened) {
      d = 0.0;
      for (int q = 0; q <= i; q++) d += Lo[i * D + q] * dm[q];
    } else {
      d = dm[i];
    }
    mu[(size_t)k * D + i] = m.mu[(size_t)k * D + i] + d;
  }
  __syncthreads();
  for (int i = warp; i < D; i += nw)
    for (int j = lane; j < D; j += 32) {
      double v = 0.0;
      if (j <= i) {
        if (via_lo) {
          for (int q = j; q <= i; q++) v = fma(Lo[i * D + q], C[q * ldc + j], v);
        } else {
          v = C[i * ldc + j];
        }
      }
      L[(size_t)k * D * D + i * D + j] = v;
    }
  if (threadIdx.x == 0) w[k] = S0;
}

// Renormalise the surviving weights (fixed order), count the dead, ENC.
__device__ __forceinline__ void body_em_renorm(int K, double *w, DevStats *st) {
  // one warp: the total in component order by lane 0, the divisions in
  // parallel (FP64 division is long-latency), fixed-tree sums of squares
  if (threadIdx.x >= 32) return;
  if (st->status != 0) return;  // the weight step failed: keep the proposal
  __shared__ double s_tot, s_w[kMaxK];
  for (int k = threadIdx.x; k < K; k += 32) s_w[k] = w[k];  // staged by the warp
  __syncwarp();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int k = 0; k < K; k++) tot += s_w[k];
    s_tot = tot;
    st->wsum = tot;
  }
  __syncwarp();
  const double tot = s_tot;
  if (!(tot > 0.0) || !isfinite(tot)) {
    if (threadIdx.x == 0) {
      st->status = -9005;  // PMCG_ENEGWEIGHT
      st->ndead = K;
      st->enc = 0.0;
    }
    return;
  }
  double s2 = 0.0;
  int nd = 0;
  for (int k = threadIdx.x; k < K; k += 32) {
    const double v = w[k] / tot;
    w[k] = v;
    s2 += v * v;
    nd += (v == 0.0);
  }
  s2 = warp_sum(s2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nd += __shfl_down_sync(0xffffffffu, nd, o);
  if (threadIdx.x == 0) {
    st->ndead = nd;
    st->enc = 1.0 / s2;
  }
}

// ================================================================== mixture preparation
__host__ __device__ inline size_t prepare_smem(int D) { return (2 * (size_t)D * D + 2 * (size_t)D) * sizeof(double); }

// Component k: W = L^-1 by column substitution, b = W mu, log|L|, and the
// single-precision copies used by the mixed kernels.
// Component k's derived arrays: L^-1 (packed and single precision), L^-1 mu,
// the single-precision factor and mean, log det L. rmax (optional, shared):
// receives max_i sum_j |(L^-1)_ij mu_j| as the bits of a non-negative double
// (atomicMax), for the single-precision range check; zero it before the call.
__device__ __forceinline__ void body_prepare_comp(const DevMixView &m, double *logdetL, double *Wt, double *b,
                                                  float *W32, float *b32, float *L32, float *mu32, int k,
                                                  double *s, unsigned long long *rmax = nullptr) {
  const int D = m.D, T = D * (D + 1) / 2, ldx = m.ldx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double *sL = s;            // D*D
  double *sW = s + D * D;    // D*D
  double *sR = sW + D * D;   // D: 1 / L_ii
  double *sG = sR + D;       // D: log L_ii
  const double *Lk = m.L + (size_t)k * D * D;
  // rows to warps, columns to lanes (rows padded to ldx, zero above the diagonal)
  for (int i = warp; i < D; i += nw)
    for (int j = lane; j < ldx; j += 32) {
      const double v = (j < D) ? Lk[i * D + j] : 0.0;
      if (j < D) {
        sL[i * D + j] = v;
        sW[i * D + j] = (i == j) ? 1.0 : 0.0;
      }
      L32[(size_t)k * D * ldx + (size_t)i * ldx + j] = (j <= i) ? (float)v : 0.0f;
    }
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    mu32[(size_t)k * D + i] = (float)m.mu[(size_t)k * D + i];
    sR[i] = 1.0 / Lk[i * D + i];
    sG[i] = log(Lk[i * D + i]);
  }
  __syncthreads();
  // L W = I by right-looking forward substitution with one barrier per step:
  // the rows U of W stay unscaled (W_q = U_q / L_qq); step q subtracts
  // (L_iq / L_qq) U_q from every later row, in the order of q as a column
  // substitution would; rows are scaled at the end.
  for (int q = 0; q < D; q++) {
    const double rq = sR[q];
    for (int i = q + 1 + warp; i < D; i += nw) {
      const double f = sL[i * D + q] * rq;
      for (int j = lane; j <= q; j += 32) sW[i * D + j] = fma(-f, sW[q * D + j], sW[i * D + j]);
    }
    __syncthreads();
  }
  for (int i = warp; i < D; i += nw)
    for (int j = lane; j <= i; j += 32) sW[i * D + j] *= sR[i];
  __syncthreads();
  for (int i = warp; i < D; i += nw) {
    // b_i = sum_j W_ij mu_j (lanes over j, fixed-order warp tree)
    double t = 0.0, ta = 0.0;
    for (int j = lane; j <= i; j += 32) {
      const double wj = sW[i * D + j], mj = m.mu[(size_t)k * D + j];
      t = fma(wj, mj, t);
      ta = fma(fabs(wj), fabs(mj), ta);
    }
    t = warp_sum(t);
    if (rmax) ta = warp_sum(ta);
    if (lane == 0) {
      b[(size_t)k * D + i] = t;
      b32[(size_t)k * D + i] = (float)t;
      if (rmax) atomicMax(rmax, (unsigned long long)__double_as_longlong(isfinite(ta) ? ta : 1e300));
    }
    for (int j = lane; j < ldx; j += 32)
      W32[(size_t)k * D * ldx + (size_t)i * ldx + j] = (j <= i && j < D) ? (float)sW[i * D + j] : 0.0f;
    for (int j = lane; j <= i; j += 32) Wt[(size_t)k * T + tri_idx(i, j)] = sW[i * D + j];
  }
  if (threadIdx.x == 0) {
    double ld = 0.0;
    for (int i = 0; i < D; i++) ld += sG[i];
    logdetL[k] = ld;
  }
}

// Cumulative weights (summed in component order, as the host and the oracle
// do) and the per-component log constants.
__device__ __forceinline__ void body_prepare_consts(const DevMixView &m, const double *logdetL, double *cw,
                                                    double *lconst, float *lconst32) {
  const int K = m.K;
  const double cst = m.cst;  // log normalising constant, from the host
  __shared__ double s_cw[kMaxK];
  for (int k = threadIdx.x; k < K; k += blockDim.x) s_cw[k] = m.w[k];
  __syncthreads();
  if (threadIdx.x == 0) {  // in component order, from shared memory
    double s = 0.0;
    for (int k = 0; k < K; k++) { s += s_cw[k]; s_cw[k] = s; }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) cw[k] = s_cw[k];
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double l = (m.w[k] > 0.0) ? log(m.w[k]) + cst - logdetL[k] : -INFINITY;
    lconst[k] = l;
    lconst32[k] = (float)l;
  }
}

}  // namespace pmcg
