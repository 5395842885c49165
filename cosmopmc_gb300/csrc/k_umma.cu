// k_umma.cu — (b) proposal log-density on the 5th-generation tensor cores.
//
// Y = X L^-1^T for every (sample, component): a [N x 32] x [32 x K*32] product,
// followed per (sample, component) by y - L^-1 mu, Q = |y|^2, the Gaussian or
// Student-t log-density and an online log-sum-exp over components.
//
//  * tcgen05.mma kind::tf32, issued by one thread, accumulators in TMEM.
//    Single-precision accuracy with three TF32 products (3xTF32 split):
//    x = x_hi + x_lo, W = W_hi + W_lo, xW ~ x_hi W_hi + x_hi W_lo + x_lo W_hi.
//  * CTA = 256 threads, persistent (one per SM), tiles of 256 samples = two
//    M=128 accumulators; components in groups of 4 (N = 128 columns each).
//  * A (samples) is staged by the threads (split into hi/lo) into the 128-byte
//    swizzled K-major layout; B (L^-1 rows, hi/lo) is pre-swizzled once per
//    proposal into that layout in global memory and streamed per group with
//    cp.async.bulk into a double buffer (mbarrier complete_tx).
//  * TMEM: 512 columns = two buffers of (2 tiles x 128 columns); the MMAs of
//    group g+1 run while the 8 warps read group g (tcgen05.ld 32x32b) and
//    evaluate the densities.
//  * Every mbarrier wait is bounded: on expiry the kernel sets an error flag,
//    stops issuing work, drains and frees its TMEM and returns.
#include "pmcg_bodies.cuh"

namespace pmcg {

constexpr int kUmTile = 256;                 // samples per CTA tile
constexpr int kUmGC = 4;                     // components per group (N = 128)
constexpr int kUmHalf = 128 * 128;           // bytes of one 128-row x 32-float operand (16 KB)
constexpr int kUmGroupBytes = 2 * kUmHalf;   // B image of one group: hi + lo (32 KB)
constexpr int kUmSmemA = 4 * kUmHalf;        // two tiles x (hi, lo)
constexpr int kUmSmemB = 2 * kUmGroupBytes;  // double buffer
constexpr int kUmSmem = kUmSmemA + kUmSmemB + 1024 + 128;  // + 1024 alignment slack + barriers
constexpr long long kUmWaitLimit = 1ll << 26;   // iteration cap of one wait
constexpr uint64_t kUmWaitNs = 1000000000ull;   // wall-time bound of one wait (1 s)

size_t umma_bimage_bytes(int K) { return (size_t)((K + kUmGC - 1) / kUmGC) * kUmGroupBytes; }

// Byte offset of element (row, col) (col < 32 floats) in a 128-byte-swizzled,
// K-major operand: 8-row atoms of 1024 bytes, 16-byte chunk c of row r stored
// at chunk c ^ (r mod 8).
__host__ __device__ __forceinline__ uint32_t sw128_off(int row, int col) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((col >> 2) ^ (row & 7)) & 7) << 4) + (col & 3) * 4);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ------------------------------------------------------------------ B image
// Group g, component c (k = 4g + c), row i, column j: W_k[i][j] split into
// TF32 hi and lo, zero for padding rows / columns / components.
__global__ void umma_bimage_kernel(DevMixView m, unsigned char *img) {
  const int g = blockIdx.x, D = m.D, K = m.K, ldx = m.ldx;
  unsigned char *hi = img + (size_t)g * kUmGroupBytes, *lo = hi + kUmHalf;
  for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
    const int n = e >> 5, j = e & 31, c = n >> 5, i = n & 31, k = g * kUmGC + c;
    float w = 0.f;
    if (k < K && i < D && j < D) w = m.W32[(size_t)k * D * ldx + (size_t)i * ldx + j];
    const float h = tf32_round(w);
    const float l = tf32_round(w - h);
    *reinterpret_cast<float *>(hi + sw128_off(n, j)) = h;
    *reinterpret_cast<float *>(lo + sw128_off(n, j)) = l;
  }
}

cudaError_t launch_umma_bimage(const DevMixView &m, unsigned char *img, cudaStream_t s) {
  const int G = (m.K + kUmGC - 1) / kUmGC;
  umma_bimage_kernel<<<G, 256, 0, s>>>(m, img);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Parity wait on an mbarrier, bounded by about one second of wall time (and an
// iteration cap); false when the bound ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  uint64_t t0 = 0;
  for (long long it = 0; it < kUmWaitLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255) == 0) {
      const uint64_t t = global_ns();
      if (it == 0) t0 = t;
      else if (t - t0 > kUmWaitNs) return false;
    }
  }
  return false;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (tcgen05 descriptor version 1).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
  d |= (uint64_t)1 << 16;                         // leading byte offset (unused with this swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset
  d |= (uint64_t)1 << 46;                         // descriptor version
  d |= (uint64_t)2 << 61;                         // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D f32, A/B tf32, both K-major, M=128, N=128.
constexpr uint32_t kUmIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kUmIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ kernel
template <bool STUDENT>
__global__ void __launch_bounds__(256, 1) umma_logq_kernel(DevMixView m, const unsigned char *__restrict__ bimg,
                                                           size_t N, const float *__restrict__ X,
                                                           double *__restrict__ out, int accumulate, double add,
                                                           float *__restrict__ lt, float *__restrict__ Qo,
                                                           int *__restrict__ errflag) {
  extern __shared__ __align__(1024) unsigned char um_raw[];
  // 1024-byte aligned operand base (swizzle atoms)
  unsigned char *base = um_raw + ((1024 - (smem_u32(um_raw) & 1023)) & 1023);
  unsigned char *sA = base;                       // [tile 0 hi][tile 0 lo][tile 1 hi][tile 1 lo]
  unsigned char *sB = base + kUmSmemA;            // [buffer 0][buffer 1], each hi + lo
  uint64_t *bars = reinterpret_cast<uint64_t *>(sB + kUmSmemB);  // 0,1: B loaded; 2,3: MMA done
  uint32_t *tmem_hold = reinterpret_cast<uint32_t *>(bars + 4);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int D = m.D, K = m.K, ldx = m.ldx;
  const int G = (K + kUmGC - 1) / kUmGC;
  const size_t ntiles = (N + kUmTile - 1) / kUmTile;
  const uint32_t barB0 = smem_u32(&bars[0]), barB1 = smem_u32(&bars[1]);
  const uint32_t barM0 = smem_u32(&bars[2]), barM1 = smem_u32(&bars[3]);
  const uint32_t sA_u = smem_u32(sA), sB_u = smem_u32(sB);

  if (tid == 0) {
    mbar_init(barB0, 1); mbar_init(barB1, 1); mbar_init(barM0, 1); mbar_init(barM1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
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

  // Phase bookkeeping. Loads (B buffers) and MMA commits are issued by thread 0
  // only; at most one of each is outstanding per barrier, so a parity wait on
  // the count of completed phases is unambiguous.
  uint32_t issB[2] = {0, 0}, doneB[2] = {0, 0};   // thread 0
  uint32_t issM[2] = {0, 0}, doneM[2] = {0, 0};   // issM: thread 0; doneM: every thread
  const float hnd = 0.5f * ((float)m.df + (float)D), rnu = 1.0f / (float)m.df;
  const int mt = warp >> 2;                      // accumulator (sample half) this warp reads
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;

  auto load_group = [&](int g) {
    const int buf = g & 1;
    bulk_load(sB_u + (uint32_t)buf * kUmGroupBytes, bimg + (size_t)g * kUmGroupBytes, kUmGroupBytes,
              buf ? barB1 : barB0);
    issB[buf]++;
  };
  // Thread 0: wait for the B image of group g, then issue its 24 MMAs (two
  // tiles x three split products x four K steps of 8) and commit them.
  auto issue_group = [&](int g) -> bool {
    const int buf = g & 1;
    if (!mbar_wait(buf ? barB1 : barB0, doneB[buf] & 1)) return false;
    doneB[buf]++;
    const uint32_t bB = sB_u + (uint32_t)buf * kUmGroupBytes;
    asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const uint32_t d = tmem + (uint32_t)buf * 256 + t * 128;
      const uint32_t aH = sA_u + (2 * t) * kUmHalf, aL = sA_u + (2 * t + 1) * kUmHalf;
#pragma unroll
      for (int ks = 0; ks < 4; ks++) {
        const uint32_t ko = ks * 32;
        umma_tf32(d, sw128_desc(aH + ko), sw128_desc(bB + ko), ks > 0);
        umma_tf32(d, sw128_desc(aH + ko), sw128_desc(bB + kUmHalf + ko), 1);
        umma_tf32(d, sw128_desc(aL + ko), sw128_desc(bB + ko), 1);
      }
    }
    umma_commit(buf ? barM1 : barM0);
    issM[buf]++;
    return true;
  };

  bool aborted = false;  // uniform over the CTA
  bool pabort = false;   // thread 0: a B-image wait expired
  for (size_t tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
    const size_t n0 = tile * kUmTile;
    // ---- stage A: 256 rows x 8 chunks of 4 floats, split into TF32 hi / lo;
    // columns >= D (row padding) and rows >= N are zero
    for (int e = tid; e < kUmTile * 8; e += blockDim.x) {
      const int s = e >> 3, c = e & 7;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (n0 + s < N && c * 4 < D) {
        v = *reinterpret_cast<const float4 *>(X + (n0 + s) * ldx + c * 4);
        if (c * 4 + 1 >= D) v.y = 0.f;
        if (c * 4 + 2 >= D) v.z = 0.f;
        if (c * 4 + 3 >= D) v.w = 0.f;
      }
      const int t = s >> 7, r = s & 127;
      const uint32_t off = (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
      float4 h, l;
      h.x = tf32_round(v.x); h.y = tf32_round(v.y); h.z = tf32_round(v.z); h.w = tf32_round(v.w);
      l.x = tf32_round(v.x - h.x); l.y = tf32_round(v.y - h.y); l.z = tf32_round(v.z - h.z); l.w = tf32_round(v.w - h.w);
      *reinterpret_cast<float4 *>(sA + (2 * t) * kUmHalf + off) = h;
      *reinterpret_cast<float4 *>(sA + (2 * t + 1) * kUmHalf + off) = l;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      load_group(0);
      if (G > 1) load_group(1);
      if (!issue_group(0)) pabort = true;
    }
    float mx = -INFINITY, sm = 0.f;
    const size_t n = n0 + (size_t)mt * 128 + (warp & 3) * 32 + lane;
    for (int g = 0; g < G; g++) {
      const int buf = g & 1;
      // thread 0 issues group g+1 into the other TMEM buffer before the epilogue of g
      if (tid == 0 && g + 1 < G && !pabort && !issue_group(g + 1)) pabort = true;
      const bool ok = mbar_wait(buf ? barM1 : barM0, doneM[buf] & 1);
      if (ok) doneM[buf]++;
      if (__syncthreads_or(!ok || pabort)) {
        aborted = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      __syncwarp();  // tcgen05.ld is warp-collective
#pragma unroll
      for (int c = 0; c < kUmGC; c++) {
        const int k = g * kUmGC + c;
        float v[32];
        tmem_ld32(tmem + lane_base + (uint32_t)(buf * 256 + mt * 128 + c * 32), v);
        if (k >= K) continue;
        const float lc = m.lconst32[k];
        float q = 0.f;
        const float *bk = m.b32 + (size_t)k * D;
#pragma unroll
        for (int i = 0; i < 32; i++) {
          if (i < D) {
            const float y = v[i] - __ldg(&bk[i]);
            q = fmaf(y, y, q);
          }
        }
        float l;
        if (lc == -INFINITY) l = -INFINITY;
        else l = STUDENT ? lc - hnd * log1pf(q * rnu) : lc - 0.5f * q;
        if (l > mx) { sm = sm * expf(mx - l) + 1.f; mx = l; }
        else if (l > -INFINITY) sm += expf(l - mx);
        if (n < N && lt) {
          lt[(size_t)k * N + n] = l;
          if (Qo) Qo[(size_t)k * N + n] = (lc == -INFINITY) ? 0.f : q;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();  // TMEM buffer and B buffer of group g are free again
      if (tid == 0 && g + 2 < G) load_group(g + 2);
    }
    if (aborted) break;
    if (n < N) {
      const double r = (double)mx + (double)logf(sm);
      if (accumulate) out[n] += r + add;
      else out[n] = r;
    }
    __syncthreads();  // A is rewritten by the next tile
  }
  if (aborted && tid == 0) {
    atomicExch(errflag, 1);
    // let every copy and MMA still in flight land (bounded) before the
    // shared memory and TMEM are released
    for (int b = 0; b < 2; b++) {
      while (doneB[b] < issB[b] && mbar_wait(b ? barB1 : barB0, doneB[b] & 1)) doneB[b]++;
      while (doneM[b] < issM[b] && mbar_wait(b ? barM1 : barM0, doneM[b] & 1)) doneM[b]++;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

int g_use_tensor_cores = 0;

cudaError_t launch_umma_logq(const DevMixView &m, const unsigned char *bimg, size_t N, const float *X, double *out,
                             int accumulate, double add, float *lt, float *Qo, int *errflag, cudaStream_t s) {
  if (m.D > 32 || N == 0) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t ntiles = (N + kUmTile - 1) / kUmTile;
  const unsigned grid = (unsigned)(ntiles < (size_t)sms ? ntiles : (size_t)sms);
  cudaError_t e;
  if (m.df > 0) {
    if ((e = cudaFuncSetAttribute(umma_logq_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUmSmem)) !=
        cudaSuccess)
      return e;
    umma_logq_kernel<true><<<grid, 256, kUmSmem, s>>>(m, bimg, N, X, out, accumulate, add, lt, Qo, errflag);
  } else {
    if ((e = cudaFuncSetAttribute(umma_logq_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUmSmem)) !=
        cudaSuccess)
      return e;
    umma_logq_kernel<false><<<grid, 256, kUmSmem, s>>>(m, bimg, N, X, out, accumulate, add, lt, Qo, errflag);
  }
  return cudaGetLastError();
}

}  // namespace pmcg
