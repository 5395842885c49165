// k_umma.cu — (b) mixture log-density on the 5th-generation tensor cores.
//
// Y = X L^-1^T for every (sample, component): a [N x 32] x [32 x K*32] product,
// followed per (sample, component) by Q = |L^-1 (x - mu)|^2, the Gaussian or
// Student-t log-density and an online log-sum-exp over components. Same
// result contract as the CUDA-core kernel (body_mixlogpdf_f32).
//
//  * tcgen05.mma kind::tf32, accumulators in TMEM. Single-precision accuracy
//    from three TF32 products (three-term split): x = x_hi + x_lo,
//    W = W_hi + W_lo, xW ~ x_hi W_hi + x_hi W_lo + x_lo W_hi.
//  * Components in groups of 8: N = 256 operand rows per MMA (an MMA has a
//    fixed issue cost, so each should be as wide as the instruction allows).
//  * L^-1 is lower triangular: the operand rows are ordered by 8-row block
//    (n = block*64 + component*8 + row), so K-step s only multiplies the rows
//    of blocks >= s (N = 64 (KS - s), KS = ceil(D/8)): 10 of 16 block
//    products for D = 32.
//  * The shift -L^-1 mu is folded into the product: it is stored (hi, lo) in
//    the never-read upper-triangle blocks of the operand image and added by
//    one more K-step against a constant operand of ones, so the accumulators
//    hold y = L^-1 (x - mu) and the epilogue only forms |y|^2.
//  * CTA = 10 warps, persistent (one per SM); tiles of 256 samples = two
//    M=128 accumulators of 256 TMEM columns each, one per sample half. Warp 9
//    streams each group's operand image (cp.async.bulk into a 2-stage ring,
//    mbarrier complete_tx; a stage is refilled once both accumulators' MMAs
//    reading it are complete). Warp 8 issues the MMAs (one thread): each item
//    on accumulator 0, then on accumulator 1, so that accumulator 0 is read
//    while accumulator 1's MMAs run and the other way round. Warps 4t .. 4t+3
//    stage half t's samples (TF32 hi/lo, 128-byte swizzle; the next tile's rows
//    as soon as the last group's MMAs are complete), read accumulator t
//    (tcgen05.ld 32x32b; one sample and all eight components per thread) and
//    evaluate the densities.
//  * Every mbarrier wait is bounded (about one second): on expiry the CTA
//    raises an abort flag that every other wait observes, sets the error
//    flag, lets its copies and MMAs in flight land (bounded) and frees TMEM.
#include "pmcg_bodies.cuh"
#include "umma_image.cuh"
#include "umma_ptx.cuh"

namespace pmcg {

constexpr int kUmTile = 256;                  // samples per CTA tile
constexpr int kUmStages = 2;                  // operand ring
constexpr int kUmSmemA = 4 * kUmHalf;         // two accumulators x (hi, lo)
constexpr int kUmSmemOnes = kUmHalf;          // constant operand of the shift K-step
constexpr int kUmSmemB = kUmStages * kUmCopyBytes;
constexpr int kUmEpi = 256;                   // 8 epilogue warps
constexpr int kUmThreads = kUmEpi + 64;       // + the MMA warp and the copy warp

// Barriers: bfull[2], bempty[2], mfull[2], tfree[2], afull[2]
constexpr int kUmBars = 2 * kUmStages + 6;

size_t umma_bimage_bytes(int K) { return (size_t)((K + kUmGC - 1) / kUmGC) * kUmGroupStride; }

static size_t umma_smem_bytes(int K) {
  const int G = (K + kUmGC - 1) / kUmGC;
  return (size_t)kUmSmemA + kUmSmemOnes + kUmSmemB + 1024 + (size_t)G * kUmGC * sizeof(float) + kUmBars * 8 + 16;
}

// The whole image (every group and row, the log-constants): after an upload.
__global__ void umma_bimage_kernel(DevMixView m, unsigned char *img) {
  const int g = blockIdx.x;
  // block (g, y) writes operand rows 32 y .. 32 y + 31
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x)
    umma_image_entry(m, img, g, blockIdx.y * 32 + (e >> 5), e & 31);
  if (blockIdx.y == 0 && threadIdx.x < kUmGC) {
    const int k = g * kUmGC + threadIdx.x;
    reinterpret_cast<float *>(img + (size_t)g * kUmGroupStride + kUmCopyBytes)[threadIdx.x] =
        (k < m.K) ? m.lconst32[k] : -INFINITY;
  }
}

cudaError_t launch_umma_bimage(const DevMixView &m, unsigned char *img, cudaStream_t s) {
  const int G = (m.K + kUmGC - 1) / kUmGC;
  umma_bimage_kernel<<<dim3(G, 8), 256, 0, s>>>(m, img);
  return cudaGetLastError();
}

// The MMAs of one group for one accumulator (A at a0: hi, then lo 16 KB on;
// B at b0: hi operand, lo 32 KB on): K-steps of the triangular product (three
// split terms each), then the shift K-step.
template <int KS>
__device__ __forceinline__ void issue_group(uint32_t d, uint64_t a0, uint64_t b0, uint64_t ones) {
#pragma unroll
  for (int ks = 0; ks < KS; ks++) {
    const uint32_t idesc = um_idesc((uint32_t)(64 * (KS - ks)));
    const uint32_t bo = (uint32_t)(ks * 8192 + ks * 32), ao = (uint32_t)(ks * 32);
    const uint32_t dd = d + (uint32_t)(64 * ks);
    umma_tf32(dd, desc_add(a0, ao), desc_add(b0, bo), idesc, ks > 0);
    umma_tf32(dd, desc_add(a0, ao), desc_add(b0, kUmOpBytes + bo), idesc, 1);
    umma_tf32(dd, desc_add(a0, kUmHalf + ao), desc_add(b0, bo), idesc, 1);
  }
  // shift K-step: rows < 64 min(KS, 3) from the hi operand, rows 192..255 from the lo operand
  constexpr int nh = 64 * (KS < 3 ? KS : 3);
  umma_tf32(d, ones, desc_add(b0, 96), um_idesc((uint32_t)nh), 1);
  if (KS == 4) umma_tf32(d + 192, ones, desc_add(b0, kUmOpBytes + 96), um_idesc(64), 1);
}

// ------------------------------------------------------------------ kernel
template <bool STUDENT, int KS>
__global__ void __launch_bounds__(kUmThreads, 1)
    umma_logq_kernel(DevMixView m, const unsigned char *__restrict__ bimg, size_t N, const float *__restrict__ X,
                     double *__restrict__ out, int accumulate, double add, float *__restrict__ lt,
                     float *__restrict__ Qo, int *__restrict__ errflag) {
  extern __shared__ __align__(1024) unsigned char um_raw[];
  // 1024-byte aligned operand base (swizzle atoms)
  unsigned char *base = um_raw + ((1024 - (smem_u32(um_raw) & 1023)) & 1023);
  unsigned char *sA = base;                          // [acc 0 hi][acc 0 lo][acc 1 hi][acc 1 lo]
  unsigned char *sOnes = sA + kUmSmemA;              // rows of (col 24, col 25) = (1, 1)
  unsigned char *sB = sOnes + kUmSmemOnes;           // ring of kUmStages x (hi, lo)
  const int D = m.D, K = m.K, ldx = m.ldx;
  const int G = (K + kUmGC - 1) / kUmGC;
  // KS = ceil(D / 8): K-steps of 8 (and 8-row blocks)
  float *s_lc = reinterpret_cast<float *>(sB + kUmSmemB);        // [G][8]
  uint64_t *bars = reinterpret_cast<uint64_t *>(s_lc + (size_t)G * kUmGC);
  uint32_t *tmem_hold = reinterpret_cast<uint32_t *>(bars + kUmBars);
  __shared__ int s_abort;
  volatile int *abort = &s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t ntiles = (N + kUmTile - 1) / kUmTile;
  const int my_tiles = (int)((ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x);
  const int items = my_tiles * G;

  // barrier addresses: bfull(s) = bfull0 + 8 s, mfull(t) = mfull0 + 8 t, ...
  const uint32_t bfull0 = smem_u32(&bars[0]), bempty0 = smem_u32(&bars[kUmStages]);
  const uint32_t mfull0 = smem_u32(&bars[2 * kUmStages]), tfree0 = smem_u32(&bars[2 * kUmStages + 2]);
  const uint32_t afull0 = smem_u32(&bars[2 * kUmStages + 4]);
  const uint32_t sA_u = smem_u32(sA), sOnes_u = smem_u32(sOnes), sB_u = smem_u32(sB);

  if (tid == 0) {
    s_abort = 0;
    // a stage is empty when both accumulators' MMAs reading it are complete
#pragma unroll
    for (int s = 0; s < kUmStages; s++) { mbar_init(bfull0 + 8 * s, 1); mbar_init(bempty0 + 8 * s, 2); }
    mbar_init(mfull0, 1); mbar_init(mfull0 + 8, 1);
    // epilogue barriers count the four warps of one sample half (one arrival per warp)
    mbar_init(tfree0, kUmEpi / 64); mbar_init(tfree0 + 8, kUmEpi / 64);
    mbar_init(afull0, kUmEpi / 64); mbar_init(afull0 + 8, kUmEpi / 64);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // constant operand of the shift K-step and the log-constants of every group
  for (int e = tid; e < 128 * 32; e += blockDim.x) {
    const int r = e >> 5, j = e & 31;
    *reinterpret_cast<float *>(sOnes + sw128_off(r, j)) = (j == 24 || j == 25) ? 1.f : 0.f;
  }
  for (int e = tid; e < G * kUmGC; e += blockDim.x)
    s_lc[e] = *reinterpret_cast<const float *>(bimg + (size_t)(e / kUmGC) * kUmGroupStride + kUmCopyBytes +
                                               (e % kUmGC) * 4);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_hold)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_hold;

  if (warp >= kUmEpi / 32) {
    // ================================================================ producers
    // warp 9 streams the operand images: group q's image goes into stage q mod 2
    // as soon as both accumulators' MMAs of item q - 2 are complete, apart from
    // the MMA issue (a thread whose MMAs wait in the tensor pipe's queue would
    // hold the copies back and leave both accumulators waiting for the next
    // group's operands).
    // warp 8 issues every MMA: item q on accumulator 0, then on accumulator 1.
    // Accumulator 0's MMAs run ahead of accumulator 1's in the pipe, so each
    // accumulator is read while the other's MMAs run (issued by two threads,
    // the two accumulators' MMAs fell into lockstep and were read together with
    // the pipe idle). Measured at N = 2^20 (D = 32, K = 64): 0.466 -> 0.406 ms.
    if (lane == 0 && warp == kUmEpi / 32 + 1) {
      bool ok = true;
      int issued = 0;
      for (int q = 0; q < items; q++) {
        const int st = q % kUmStages;
        if (q >= kUmStages && !mbar_wait(bempty0 + 8 * st, (uint32_t)((q / kUmStages - 1) & 1), abort)) {
          ok = false;
          break;
        }
        bulk_load(sB_u + (uint32_t)st * kUmCopyBytes, bimg + (size_t)(q % G) * kUmGroupStride, kUmCopyBytes,
                  bfull0 + 8 * st);
        issued++;
      }
      if (!ok) atomicExch(errflag, 1);
      // the copies still in flight land before shared memory is released (the
      // last phase of each stage; on the normal path they are complete)
      for (int q = (issued > kUmStages ? issued - kUmStages : 0); q < issued; q++)
        mbar_drain(bfull0 + 8 * (q % kUmStages), (uint32_t)((q / kUmStages) & 1));
    } else if (lane == 0) {
      bool ok = true;
      int last0 = -1, last1 = -1;                                   // last item committed per accumulator
      const uint64_t ones_desc = sw128_desc(sOnes_u + 96);          // columns 24..31 of the ones operand
      const uint64_t b_desc = sw128_desc(sB_u);
      for (int q = 0; q < items && ok; q++) {
        const int g = q % G, st = q % kUmStages;
        if (!mbar_wait(bfull0 + 8 * st, (uint32_t)((q / kUmStages) & 1), abort)) { ok = false; break; }
#pragma unroll 1
        for (int t = 0; t < 2; t++) {
          if (g == 0 && !mbar_wait(afull0 + 8 * t, (uint32_t)((q / G) & 1), abort)) { ok = false; break; }
          // accumulator t was read for item q-1
          if (q >= 1 && !mbar_wait(tfree0 + 8 * t, (uint32_t)((q - 1) & 1), abort)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;");
          issue_group<KS>(tmem + (uint32_t)t * 256, desc_add(sw128_desc(sA_u), (uint32_t)(2 * t) * kUmHalf),
                          desc_add(b_desc, (uint32_t)st * kUmCopyBytes), ones_desc);
          umma_commit(mfull0 + 8 * t);
          umma_commit(bempty0 + 8 * st);
          if (t == 0) last0 = q;
          else last1 = q;
        }
      }
      if (!ok) atomicExch(errflag, 1);
      // this thread's MMAs still in flight land before shared memory and TMEM
      // are released (complete on the normal path; bounded after an abort)
      if (last0 >= 0) mbar_drain(mfull0, (uint32_t)(last0 & 1));
      if (last1 >= 0) mbar_drain(mfull0 + 8, (uint32_t)(last1 & 1));
    }
  } else {
    // ================================================================ epilogue
    // warp w: TMEM lane quarter w&3 of accumulator t = w>>2; one sample, all eight components
    const int quarter = warp & 3, ta = warp >> 2;
    const int srow = ta * 128 + quarter * 32 + lane;         // sample row within the tile
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    // l = lc - (nu+D)/2 ln(1 + Q/nu) = lc - hndl log2(1 + Q/nu); MUFU log2 and
    // exp2 (relative error near 2^-22): a few 1e-6 in l, below the TF32-split
    // products' error, and off the path that returns the accumulators
    const float hndl = 0.5f * ((float)m.df + (float)D) * 0.69314718055994531f, rnu = 1.0f / (float)m.df;
    const float kLog2e = 1.44269504088896341f;
    // the four warps of half ta stage its 128 sample rows (8 float4 per thread)
    const int ht = tid & 127;
    float4 xr[8];
    auto fetch = [&](size_t tile) {
      const size_t n0 = tile * kUmTile + (size_t)ta * 128;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int s = (ht >> 3) + 16 * j, c = ht & 7;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n0 + s < N && c * 4 < D) {
          v = __ldg(reinterpret_cast<const float4 *>(X + (n0 + s) * ldx + c * 4));
          if (c * 4 + 1 >= D) v.y = 0.f;
          if (c * 4 + 2 >= D) v.z = 0.f;
          if (c * 4 + 3 >= D) v.w = 0.f;
        }
        xr[j] = v;
      }
    };
    auto stage = [&]() {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int r = (ht >> 3) + 16 * j, c = ht & 7, t = ta;
        const uint32_t off = (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
        const float4 v = xr[j];
        float4 h, l;
        h.x = tf32_round(v.x); h.y = tf32_round(v.y); h.z = tf32_round(v.z); h.w = tf32_round(v.w);
        l.x = tf32_round(v.x - h.x); l.y = tf32_round(v.y - h.y);
        l.z = tf32_round(v.z - h.z); l.w = tf32_round(v.w - h.w);
        *reinterpret_cast<float4 *>(sA + (2 * t) * kUmHalf + off) = h;
        *reinterpret_cast<float4 *>(sA + (2 * t + 1) * kUmHalf + off) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive_warp(afull0 + 8 * ta);
    };

    bool ok = true;
    fetch(blockIdx.x);
    stage();
    for (int i = 0; i < my_tiles && ok; i++) {
      const size_t tile = blockIdx.x + (size_t)i * gridDim.x;
      const size_t n = tile * kUmTile + srow;
      const bool more = i + 1 < my_tiles;
      // The next tile's rows: an L2 prefetch now (no registers held), the
      // register fetch before the last group, and the staging right after the
      // last group's MMAs complete, before its accumulator is read: the fetched
      // rows are not live while the accumulators are read, and the producer
      // can start the next tile while the last group is still being read
      // (measured: log q 0.473 -> 0.460 ms, the 16-component target 0.160 ->
      // 0.144 ms at N = 2^20; two 32-column loads per wait spilled registers
      // and were slower).
      if (more) {
        const size_t nn = (tile + gridDim.x) * kUmTile + (size_t)ta * 128 + ht;
        if (nn < N) asm volatile("prefetch.global.L2 [%0];" ::"l"(X + nn * ldx));
      }
      float mx[2] = {-INFINITY, -INFINITY}, sm[2] = {0.f, 0.f};
      // one group of eight components; `last` is a constant at each call site,
      // so the fetched rows are live only between the fetch and the staging
      auto group = [&](int g, bool last) -> bool {
        const int q = i * G + g;
        if (!mbar_wait_warp(mfull0 + 8 * ta, (uint32_t)(q & 1), abort)) return false;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // every MMA reading this half's operand rows is complete (the last
        // group's commit has arrived): stage the next tile's half
        if (last && more) stage();
        // y of component c, row block rb: columns 64 rb + 8 c + r (32 columns = 4 components per load)
        const uint32_t tcol = tmem + lane_base + (uint32_t)(ta * 256);
        unsigned long long q2[8];
#pragma unroll
        for (int c = 0; c < 8; c++) q2[c] = 0ull;
#pragma unroll
        for (int rb = 0; rb < KS; rb++) {
#pragma unroll
          for (int hc = 0; hc < 2; hc++) {
            float v[32];
            tmem_ld32_nowait(tcol + (uint32_t)(rb * 64 + hc * 32), v);
            tmem_ld_wait();
#pragma unroll
            for (int c = 0; c < 4; c++) {
#pragma unroll
              for (int e = 0; e < 8; e += 2) sq2_acc(q2[hc * 4 + c], v[c * 8 + e], v[c * 8 + e + 1]);
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive_warp(tfree0 + 8 * ta);                  // accumulator free for the next group
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const int k = g * kUmGC + c;
          if (k >= K) break;
          const float qv = sum2(q2[c]);
          const float lc = s_lc[g * kUmGC + c];
          float l;
          if (lc == -INFINITY) l = -INFINITY;
          else l = STUDENT ? lc - hndl * lg2_approx(fmaf(qv, rnu, 1.f)) : lc - 0.5f * qv;
          // two running log-sum-exps (even and odd components), each updated
          // without a branch on the new maximum: half the dependent chain and
          // no divergence (measured at N = 2^20: log q 0.406 -> 0.401 ms, the
          // 16-component Gaussian target 0.142 -> 0.122 ms)
          float &cm = mx[c & 1], &cs = sm[c & 1];
          if (l > -INFINITY) {
            const float mn = fmaxf(cm, l);
            cs = fmaf(cs, ex2_approx((cm - mn) * kLog2e), ex2_approx((l - mn) * kLog2e));
            cm = mn;
          }
          if (n < N && lt) {
            lt[(size_t)k * N + n] = l;
            if (Qo) Qo[(size_t)k * N + n] = (lc == -INFINITY) ? 0.f : qv;
          }
        }
        return true;
      };
      for (int g = 0; g < G - 1 && ok; g++) ok = group(g, false);
      if (ok) {
        if (more) fetch(tile + gridDim.x);
        ok = group(G - 1, true);
      }
      if (!ok) break;
      if (n < N) {
        // merge the two chains (a chain that saw no finite density has mx = -inf, sm = 0)
        const float m = fmaxf(mx[0], mx[1]);
        float sum = 0.f;
        if (mx[0] > -INFINITY) sum = fmaf(sm[0], ex2_approx((mx[0] - m) * kLog2e), sum);
        if (mx[1] > -INFINITY) sum = fmaf(sm[1], ex2_approx((mx[1] - m) * kLog2e), sum);
        const double r = (double)m + (double)logf(sum);
        if (accumulate) out[n] += r + add;
        else out[n] = r + add;
      }
    }
    if (!ok) atomicExch(errflag, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// On by default: validated against the CUDA-core kernel and the FP64 oracle.
int g_use_tensor_cores = 1;

cudaError_t launch_umma_logq(const DevMixView &m, const unsigned char *bimg, size_t N, const float *X, double *out,
                             int accumulate, double add, float *lt, float *Qo, int *errflag, cudaStream_t s) {
  if (m.D > 32 || m.K < 1 || N == 0 || !bimg) return cudaErrorInvalidValue;
  const size_t smem = umma_smem_bytes(m.K);
  int dev = 0, sms = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)maxsm) return cudaErrorInvalidValue;
  const size_t ntiles = (N + kUmTile - 1) / kUmTile;
  const unsigned grid = (unsigned)(ntiles < (size_t)sms ? ntiles : (size_t)sms);
  const int KS = (m.D + 7) >> 3;
  cudaError_t e = cudaSuccess;
#define PMCG_UMMA(ST, KSV)                                                                                    \
  {                                                                                                           \
    cudaFuncAttributes fa;                                                                                    \
    if ((e = cudaFuncGetAttributes(&fa, (const void *)umma_logq_kernel<ST, KSV>)) != cudaSuccess) return e;   \
    if (fa.maxThreadsPerBlock < kUmThreads) return cudaErrorLaunchOutOfResources;                             \
    if ((e = cudaFuncSetAttribute(umma_logq_kernel<ST, KSV>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                  (int)smem)) != cudaSuccess)                                                 \
      return e;                                                                                               \
    umma_logq_kernel<ST, KSV><<<grid, kUmThreads, smem, s>>>(m, bimg, N, X, out, accumulate, add, lt, Qo,       \
                                                             errflag);                                        \
  }
  if (m.df > 0) {
    if (KS == 1) PMCG_UMMA(true, 1) else if (KS == 2) PMCG_UMMA(true, 2) else if (KS == 3) PMCG_UMMA(true, 3)
    else PMCG_UMMA(true, 4)
  } else {
    if (KS == 1) PMCG_UMMA(false, 1) else if (KS == 2) PMCG_UMMA(false, 2) else if (KS == 3) PMCG_UMMA(false, 3)
    else PMCG_UMMA(false, 4)
  }
#undef PMCG_UMMA
  return cudaGetLastError();
}

}  // namespace pmcg
