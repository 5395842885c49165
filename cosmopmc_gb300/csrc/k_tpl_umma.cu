// k_tpl_umma.cu — (c) dense template likelihood on the 5th-generation tensor
// cores (single precision).
//
// The template likelihood (analogue of likeli_Mvdens, wrappers/src/param.c:
// 1485-1493) is chi2(theta) = |dt - At phi(theta)|^2 with At = L^-1 A and
// dt = L^-1 d_obs whitened by the data covariance C = L L^T. The first
// monomial is phi_0 = 1, so with At' = At whose column 0 is At_0 - dt,
// chi2 = |At' phi|^2 = phi^T G' phi, G' = At'^T At' = U^T U (U upper
// triangular, the FP64 Cholesky factor taken at set-up). Per sample
// chi2 = |U phi|^2: a [N x P] x [P x P] product followed by a sum of squares.
// Unlike the Gram form c0 - 2 phi.b + phi^T G phi, no large terms of opposite
// sign are differenced.
//
//  * tcgen05.mma kind::tf32 with the three-term split (phi_hi U_hi + phi_hi
//    U_lo + phi_lo U_hi), FP32 accumulators in TMEM: single-precision accuracy.
//  * Shapes: P <= 96 (12 K-steps of 8). A = the tile's 128 samples' phi rows
//    (M = 128), B = the rows of U (N = output index). U is upper triangular, so
//    the rows with non-zeros in K-step s are rows 0 .. 8s+7: the K-steps are
//    issued from the last one down, N = 96 for the first (which initialises
//    every accumulator column) and N = 16 ceil((8s+8)/16) after it.
//  * CTA = 5 warps, persistent (one per SM). U's operand image (hi and lo,
//    72 KB) is copied into shared memory once (cp.async.bulk + mbarrier). Warps
//    0-3 own one sample each per tile (thread t = accumulator lane t): they
//    read the accumulator of the previous tile, stage phi of the next tile
//    (TF32 hi/lo, 128-byte swizzled, K-major) and write the log-likelihoods;
//    warp 4's first thread issues the 36 MMAs of each tile and commits them.
//    One operand buffer and one accumulator: a tile's staging waits for the
//    previous tile's MMAs (shared memory holds U, phi hi and lo: 168 KB).
//  * Every mbarrier wait is bounded (about one second): on expiry the CTA
//    raises an abort flag that every other wait observes, sets the error
//    flag, lets its copies and MMAs in flight land (bounded) and frees TMEM.
#include "pmcg_bodies.cuh"
#include "umma_image.cuh"
#include "umma_ptx.cuh"

namespace pmcg {

constexpr int kTuTile = 128;                   // samples per tile (accumulator lanes)
constexpr int kTuK = 96;                       // largest P (3 swizzle chunks of 32 floats)
constexpr int kTuChunkA = kTuTile * 128;       // bytes of one 32-float chunk of 128 rows (16 KB)
constexpr int kTuChunkB = kTuK * 128;          // bytes of one 32-float chunk of 96 rows (12 KB)
constexpr int kTuOpA = 3 * kTuChunkA;          // phi hi (or lo): 48 KB
constexpr int kTuOpB = 3 * kTuChunkB;          // U hi (or lo): 36 KB
constexpr int kTuImage = 2 * kTuOpB;           // U's operand image: hi then lo (72 KB)
constexpr int kTuEpi = 128;                    // 4 staging / epilogue warps
constexpr int kTuThreads = kTuEpi + 32;        // + 1 producer warp
constexpr int kTuSmem = 2 * kTuOpA + kTuImage + 1024 + 64;

size_t tpl_uimage_bytes() { return (size_t)kTuImage; }

// Byte offset of element (row, col < 96) in a 3-chunk, 128-byte-swizzled,
// K-major operand whose chunks are `chunk` bytes apart.
__host__ __device__ __forceinline__ uint32_t tu_off(int row, int col, int chunk) {
  return (uint32_t)((col >> 5) * chunk) + sw128_off(row, col & 31);
}

// U (FP32, [96 x 96] row-major, zero beyond P) into the operand image.
__global__ void tpl_uimage_kernel(const float *__restrict__ U32, unsigned char *img) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kTuK * kTuK; e += gridDim.x * blockDim.x) {
    const int n = e / kTuK, j = e - n * kTuK;
    const float u = U32[e];
    const float h = tf32_round(u);
    const float l = tf32_round(u - h);
    *reinterpret_cast<float *>(img + tu_off(n, j, kTuChunkB)) = h;
    *reinterpret_cast<float *>(img + kTuOpB + tu_off(n, j, kTuChunkB)) = l;
  }
}

cudaError_t launch_tpl_uimage(const float *U32, unsigned char *img, cudaStream_t s) {
  tpl_uimage_kernel<<<36, 256, 0, s>>>(U32, img);
  return cudaGetLastError();
}

// phi(theta) of one sample (1, theta_i, theta_i theta_j for i <= j; zero up to
// 96) split into TF32 (hi, lo) and written to row `row` of both operands. D is
// a compile-time constant, so every index of v is too (v stays in registers).
template <int D>
__device__ __forceinline__ void tu_stage_row(const float (&th)[D], unsigned char *sAh, unsigned char *sAl, int row) {
  float v[kTuK];
#pragma unroll
  for (int p = 0; p < kTuK; p++) v[p] = 0.f;
  v[0] = 1.f;
#pragma unroll
  for (int i = 0; i < D; i++) v[1 + i] = th[i];
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int j = i; j < D; j++) v[1 + D + i * D - i * (i - 1) / 2 + (j - i)] = th[i] * th[j];
#pragma unroll
  for (int c4 = 0; c4 < kTuK / 4; c4++) {
    float4 h, l;
    h.x = tf32_round(v[4 * c4 + 0]); l.x = tf32_round(v[4 * c4 + 0] - h.x);
    h.y = tf32_round(v[4 * c4 + 1]); l.y = tf32_round(v[4 * c4 + 1] - h.y);
    h.z = tf32_round(v[4 * c4 + 2]); l.z = tf32_round(v[4 * c4 + 2] - h.z);
    h.w = tf32_round(v[4 * c4 + 3]); l.w = tf32_round(v[4 * c4 + 3] - h.w);
    const uint32_t off = tu_off(row, 4 * c4, kTuChunkA);
    *reinterpret_cast<float4 *>(sAh + off) = h;
    *reinterpret_cast<float4 *>(sAl + off) = l;
  }
}

// Parameters of sample n, zero beyond N.
template <int D>
__device__ __forceinline__ void tu_fetch(const float *__restrict__ X, int ldx, size_t N, size_t n, float (&th)[D]) {
#pragma unroll
  for (int i = 0; i < D; i++) th[i] = (n < N) ? __ldg(X + n * ldx + i) : 0.f;
}

template <int D>
__global__ void __launch_bounds__(kTuThreads, 1)
    tpl_umma_kernel(const unsigned char *__restrict__ uimg, size_t N, const float *__restrict__ X,
                    int ldx, double *__restrict__ logpost, const short *__restrict__ flg,
                    int *__restrict__ errflag, int assign, double add) {
  extern __shared__ __align__(1024) unsigned char tu_raw[];
  unsigned char *base = tu_raw + ((1024 - (smem_u32(tu_raw) & 1023)) & 1023);
  unsigned char *sAh = base, *sAl = base + kTuOpA;   // phi of the tile: hi, lo
  unsigned char *sB = base + 2 * kTuOpA;             // U: hi, lo
  uint64_t *bars = reinterpret_cast<uint64_t *>(sB + kTuImage);
  uint32_t *tmem_hold = reinterpret_cast<uint32_t *>(bars + 3);
  __shared__ int s_abort;
  volatile int *abort = &s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t ntiles = (N + kTuTile - 1) / kTuTile;
  const int my_tiles = (int)((ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x);
  constexpr int P = 1 + D + D * (D + 1) / 2;
  constexpr int KS = (P + 7) >> 3;
  const uint32_t bload = smem_u32(&bars[0]), afull = smem_u32(&bars[1]), mfull = smem_u32(&bars[2]);
  const uint32_t sA_u = smem_u32(sAh), sB_u = smem_u32(sB);

  if (tid == 0) {
    s_abort = 0;
    mbar_init(bload, 1);
    mbar_init(afull, kTuEpi / 32);  // one arrival per staging warp
    mbar_init(mfull, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_hold)),
                 "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_hold;

  if (warp == kTuEpi / 32) {
    // ================================================================ producer
    if (lane == 0) {
      bulk_load(sB_u, uimg, kTuImage, bload);
      bool ok = mbar_wait(bload, 0, abort);
      int committed = -1;
      const uint64_t a_desc = sw128_desc(sA_u), b_desc = sw128_desc(sB_u);
      for (int i = 0; i < my_tiles && ok; i++) {
        if (!mbar_wait(afull, (uint32_t)(i & 1), abort)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (int s = KS - 1; s >= 0; s--) {
          const uint32_t ao = (uint32_t)((s >> 2) * kTuChunkA + (s & 3) * 32);
          const uint32_t bo = (uint32_t)((s >> 2) * kTuChunkB + (s & 3) * 32);
          const bool first = (s == KS - 1);
          const uint32_t n = first ? (uint32_t)kTuK : (uint32_t)(((8 * s + 8 + 15) >> 4) << 4);
          const uint32_t idesc = um_idesc(n);
          umma_tf32(tmem, desc_add(a_desc, ao), desc_add(b_desc, bo), idesc, first ? 0u : 1u);
          umma_tf32(tmem, desc_add(a_desc, ao), desc_add(b_desc, kTuOpB + bo), idesc, 1u);
          umma_tf32(tmem, desc_add(a_desc, kTuOpA + ao), desc_add(b_desc, bo), idesc, 1u);
        }
        umma_commit(mfull);
        committed = i;
      }
      if (!ok) {
        atomicExch(errflag, 1);
        // let the copy of U and the last MMAs land before shared memory and TMEM go
        mbar_drain(bload, 0);
        if (committed >= 0) mbar_drain(mfull, (uint32_t)(committed & 1));
      }
    }
  } else {
    // ================================================================ staging / epilogue
    float th[D];
    bool ok = true;
    tu_fetch<D>(X, ldx, N, (size_t)blockIdx.x * kTuTile + tid, th);
    size_t n_prev = 0;
    short f_prev = 0;
    double lp_prev = 0.0;
    for (int i = 0; i <= my_tiles && ok; i++) {
      float chi2 = 0.f;
      if (i > 0) {
        // the MMAs of tile i-1 are complete: its accumulator is final and the operands are free
        if (!mbar_wait_warp(mfull, (uint32_t)((i - 1) & 1), abort)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        unsigned long long acc = 0ull;
#pragma unroll
        for (int c = 0; c < kTuK / 32; c++) {
          float v[32];
          tmem_ld32_nowait(taddr + (uint32_t)(c * 32), v);
          tmem_ld_wait();
#pragma unroll
          for (int e = 0; e < 32; e += 2) sq2_acc(acc, v[e], v[e + 1]);
        }
        chi2 = sum2(acc);
        asm volatile("tcgen05.fence::before_thread_sync;");
      }
      if (i < my_tiles) {
        tu_stage_row<D>(th, sAh, sAl, tid);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_warp(afull);
      }
      if (i > 0 && f_prev) logpost[n_prev] = lp_prev - 0.5 * (double)chi2;
      if (i < my_tiles) {
        // this tile's flag and log-posterior, and the next tile's parameters: loads
        // in flight while the MMAs run
        n_prev = (blockIdx.x + (size_t)i * gridDim.x) * kTuTile + tid;
        f_prev = (n_prev < N) ? flg[n_prev] : (short)0;
        lp_prev = (n_prev < N) ? (assign ? add : logpost[n_prev]) : 0.0;
        if (i + 1 < my_tiles) tu_fetch<D>(X, ldx, N, (blockIdx.x + (size_t)(i + 1) * gridDim.x) * kTuTile + tid, th);
      }
    }
    if (!ok) atomicExch(errflag, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
  }
}

cudaError_t launch_tpl_umma(const unsigned char *uimg, int Dp, size_t N, const float *X, int ldx, double *logpost,
                            const short *flg, int *errflag, cudaStream_t s, int assign, double add) {
  if (N == 0) return cudaSuccess;
  if (!uimg || Dp < 1 || Dp > kTplUmmaMaxD) return cudaErrorInvalidValue;
  int dev = 0, sms = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (kTuSmem > maxsm) return cudaErrorInvalidValue;
  const size_t ntiles = (N + kTuTile - 1) / kTuTile;
  const unsigned grid = (unsigned)(ntiles < (size_t)sms ? ntiles : (size_t)sms);
  cudaError_t e = cudaSuccess;
#define PMCG_TU(DV)                                                                                           \
  case DV:                                                                                                    \
    if ((e = cudaFuncSetAttribute(tpl_umma_kernel<DV>, cudaFuncAttributeMaxDynamicSharedMemorySize,          \
                                  kTuSmem)) != cudaSuccess)                                                   \
      return e;                                                                                               \
    tpl_umma_kernel<DV><<<grid, kTuThreads, kTuSmem, s>>>(uimg, N, X, ldx, logpost, flg, errflag, assign,    \
                                                          add);                                               \
    break;
  switch (Dp) {
    PMCG_TU(1) PMCG_TU(2) PMCG_TU(3) PMCG_TU(4) PMCG_TU(5) PMCG_TU(6)
    PMCG_TU(7) PMCG_TU(8) PMCG_TU(9) PMCG_TU(10) PMCG_TU(11) PMCG_TU(12)
    default: return cudaErrorInvalidValue;
  }
#undef PMCG_TU
  return cudaGetLastError();
}

}  // namespace pmcg
