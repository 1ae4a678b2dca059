// lg_tc.cuh -- tcgen05 / mbarrier helpers shared by the tensor-core Gram kernels.
//
// Operands are staged in shared memory in the canonical K-major no-swizzle
// layout (8 x 16-byte core matrices; LBO = 128 B between the two K halves of a
// 16-wide K chunk, SBO = 256 B between 8-row groups), one BF16 x BF16 -> FP32
// tcgen05.mma (M = 128, N = 80, K = 16) is issued by one thread, and completion
// is signalled through tcgen05.commit on an mbarrier.  Every wait is bounded.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace lg {

namespace tc {

constexpr int kThreads = 128;
constexpr int kStageEntries = 64;           // 4 MMAs of K = 16
constexpr int kChunkA = 128 * 16 * 2;       // 4096 B: M=128 x K=16 bf16
constexpr int kChunkB = 80 * 16 * 2;        // 2560 B: N=80 x K=16 bf16
constexpr int kStageBytes = 4 * (kChunkA + kChunkB);  // 26624 B
constexpr int kN = 80;
constexpr int kDS = kN + 1;  // row stride of the accumulator copy in shared memory (odd: no bank conflicts)
constexpr int kTmemCols = 128;
constexpr int kQueueCap = kStageEntries + kThreads;
constexpr long long kSpinLimit = 1ll << 24;  // ~1 s of polling

__device__ inline uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ inline uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: kind::f16, BF16 A/B, FP32 D, K-major A and B, M=128, N=80
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ inline bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait that may suspend the thread for up to hint_ns while the phase is
// incomplete (the waiting warp then takes no issue slots from its neighbours)
__device__ inline bool mbar_try_wait_hint(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

__device__ inline uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait; returns false on expiry
__device__ inline bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ inline void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
}

__device__ inline void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ inline void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ inline void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ inline void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline float schr2f(float ri) {
  if (ri > 2.0f) return 0.0f;
  if (ri > 1.0f) {
    float rj = ri / 12.0f - 0.5f;
    rj = rj * ri + 0.625f;
    rj = rj * ri + 1.666667f;
    return (rj * ri - 5.0f) * ri + 4.0f - 0.6666667f / ri;
  }
  if (ri > 0.0f) {
    float rk = ri * ri;
    float rj = (-0.25f * ri + 0.5f) * ri + 0.625f;
    return (rj * ri - 1.666667f) * rk + 1.0f;
  }
  return 1.0f;
}

__device__ inline uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// hi/lo split of two FP32 values into BF16 pairs: hi = the upper 16 bits (a
// truncation, |v - hi| < 2^-8 |v|), packed by one byte permute; lo = v - hi is
// exact in FP32 and rounded once to BF16, so hi + lo carries v to 2^-17.
__device__ inline void split_bf16x2(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  const uint32_t b0 = __float_as_uint(v0), b1 = __float_as_uint(v1);
  hi = __byte_perm(b0, b1, 0x7632);
  const float l0 = v0 - __uint_as_float(b0 & 0xffff0000u);
  const float l1 = v1 - __uint_as_float(b1 & 0xffff0000u);
  lo = pack_bf16(l0, l1);
}

// Pairs of FP32 values in one 64-bit register for the packed f32x2 arithmetic
// of sm_100 and later: one instruction does the work of two FP32 ones.  The
// low half holds the first value.
__device__ inline unsigned long long f2_pack(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ inline float2 f2_unpack(unsigned long long v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ inline unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ inline unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                            unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ inline unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// split_bf16x2 of a packed pair: the same hi and lo, with one packed
// subtraction for the two residuals
__device__ inline void split_bf16x2_packed(unsigned long long v, uint32_t& hi, uint32_t& lo) {
  hi = __byte_perm((uint32_t)v, (uint32_t)(v >> 32), 0x7632);
  const float2 l = f2_unpack(f2_sub(v, v & 0xffff0000ffff0000ull));
  lo = pack_bf16(l.x, l.y);
}

}  // namespace tc

}  // namespace lg
