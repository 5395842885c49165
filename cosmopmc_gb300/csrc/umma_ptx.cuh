// umma_ptx.cuh — inline-PTX building blocks of the tcgen05 kernels (k_umma.cu:
// mixture log-density; k_tpl_umma.cu: template likelihood): shared-memory
// addresses, mbarrier waits bounded by wall time, bulk copies, shared-memory
// matrix and instruction descriptors, tcgen05.mma / commit / ld.
#pragma once
#include "pmcg_common.cuh"

namespace pmcg {

constexpr long long kUmWaitLimit = 1ll << 26;   // iteration cap of one wait
constexpr uint64_t kUmWaitNs = 1000000000ull;   // wall-time bound of one wait (1 s)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Parity wait bounded by about one second of wall time (and an iteration
// cap). Gives up early when another role of the CTA raised the abort flag;
// raises it on expiry. Returns false when the CTA is aborting. The clock and
// the flag are only consulted every 256 polls, off the fast path.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort) {
  uint64_t t0 = 0;
  for (long long it = 1; it <= kUmWaitLimit; it++) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (*abort) return false;
      const uint64_t t = global_ns();
      if (it == 256) t0 = t;
      else if (t - t0 > kUmWaitNs) break;
    }
  }
  *abort = 1;
  return false;
}

// Bounded wait that ignores the abort flag (draining after an abort).
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity) {
  uint64_t t0 = 0;
  for (long long it = 1; it <= kUmWaitLimit; it++) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255) == 0) {
      const uint64_t t = global_ns();
      if (it == 256) t0 = t;
      else if (t - t0 > kUmWaitNs) return false;
    }
  }
  return false;
}

// Warp-level forms: one lane polls (keeps the shared-memory traffic of
// waiting warps off the tensor cores' operand reads) and the warp proceeds
// together; one arrival per warp after __syncwarp.
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity, volatile int *abort) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, abort) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive_warp(uint32_t bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
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

// Instruction descriptor: D f32, A/B tf32, both K-major, M=128, N = n.
__device__ __forceinline__ uint32_t um_idesc(uint32_t n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Descriptor of base + off bytes from the descriptor of base (off < 256 KB -
// base, a multiple of 16): only the start-address field changes.
__device__ __forceinline__ uint64_t desc_add(uint64_t d, uint32_t off) { return d + (uint64_t)(off >> 4); }

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes (no wait).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, float *v) {
  uint32_t *r = reinterpret_cast<uint32_t *>(v);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

// acc += (a, b)^2 elementwise on a packed pair (one f32x2 FMA); volatile keeps
// it in program order with the TMEM loads and waits around it.
__device__ __forceinline__ void sq2_acc(unsigned long long &acc, float a, float b) {
  asm volatile("{\n\t.reg .b64 t;\n\tmov.b64 t, {%1, %2};\n\tfma.rn.f32x2 %0, t, t, %0;\n\t}"
      : "+l"(acc)
      : "f"(a), "f"(b));
}
__device__ __forceinline__ float sum2(unsigned long long acc) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(acc));
  return a + b;
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace pmcg
