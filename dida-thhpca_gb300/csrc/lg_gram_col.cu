// lg_gram_col.cu -- mixed-precision Gram matrices of a group of levels of one
// grid column, with every observation's ensemble row read once for the group.
//
// The solves of one column at different levels share the column's neighbour
// list; the vertical localisation only changes the weights (and which ln p
// window of the bucketed records contributes).  Reading each record's ensemble
// row once per level, as one CTA per solve does, re-reads the same rows about
// as often as a record lies in the windows of neighbouring levels (~8 times at
// 0.2 ln p and 32 levels).  Here one persistent CTA per SM takes work items
// (column, group of up to kG = 8 consecutive levels):
//
//   producer warp   streams the union of the group's record windows in stages
//                   of 64 records: the records (entry, ln p, rdiaginv*rloc, d)
//                   to a shared ring, and the 64-member FP32 ensemble rows of
//                   the entries with cp.async (16-byte chunks) into a Y ring of
//                   kRing stages; completion is tracked per stage by an
//                   mbarrier (cp.async.mbarrier.arrive.noinc).  The records of
//                   the next stage are loaded while this stage's rows are issued.
//   8 converter warps  each owns 16 records of a stage (two 8-record groups)
//                   for all 64 members: per level whose window meets the stage
//                   it computes its records' weights w = rdiaginv*rloc*GC_vertical,
//                   splits y~ = sqrt(w) y into BF16 hi + lo and writes its part of
//                   A = [hi; lo] (M = 128, K = 64, K-major no-swizzle) into one of
//                   kOps operand buffers, then signals the buffer's mbarrier.
//                   t = Y~^T d~ is accumulated in FP32 registers.
//   MMA warp        waits for all eight parts of a buffer and issues four
//                   tcgen05.mma (N = 64, B = the hi rows of A) into the level's
//                   own 64 TMEM columns, committing to the buffer's mbarrier.
// The converter warps never wait on each other inside an item; they meet on a
// named barrier only for the epilogue, which copies the accumulators out.
//
//   C = D[0:64,:] + D[64:128,:] + D[64:128,:]^T   (hi hi + lo hi + hi lo), in FP32,
//   then converted to FP64 -- the same quantities as lg_gram_tc.cu
//   (letkf_core.F90:58-75,146-195).
//
// Every mbarrier wait is bounded; on expiry the CTA records LG_ERR_TIMEOUT,
// raises a shared abort flag that ends every other wait at once, waits (bounded)
// for its own MMAs and copies, frees its tensor memory and returns.
#include <climits>

#include "lg_device.cuh"
#include "lg_internal.h"
#include "lg_tc.cuh"

namespace lg {
namespace colk {

constexpr int kConv = 256;                      // converter threads (warps 0-7)
constexpr int kProducer = kConv / 32;           // warp 8
constexpr int kMmaWarp = kProducer + 1;         // warp 9
constexpr int kThreads = kConv + 64;
constexpr int kG = 8;                           // levels per work item
constexpr int kN = 64;                          // accumulator columns per level
constexpr int kRows = 64;                       // records per stage (4 MMAs of K = 16)
constexpr int kChunkA = 128 * 16 * 2;           // 4096 B: M = 128 x K = 16 BF16
constexpr int kOpBytes = 4 * kChunkA;           // 16 KB
constexpr int kYBytes = kRows * 64 * 4;         // 16 KB: 64 rows of 64 FP32
constexpr int kDS = kN + 1;                     // accumulator copy row stride (odd)
// shared-memory layout for kRing Y/record stages and kOps operand buffers:
// Y ring | operand buffers | record ring | sqrt(w), sqrt(w) d of the converter warps
template <int kRing, int kOps>
struct Layout {
  static constexpr int kOffY = 0;
  static constexpr int kOffOps = kOffY + kRing * kYBytes;
  static constexpr int kOffRec = kOffOps + kOps * kOpBytes;
  static constexpr int kOffW = kOffRec + kRing * kRows * 16;
  static constexpr int kBytes = kOffW + 8 * 2 * kG * 16 * 4;
  static_assert(64 * kDS * 4 <= kOps * kOpBytes, "epilogue staging must fit the operand buffers");
};

// instruction descriptor: kind::f16, BF16 A/B, FP32 D, K-major A and B, M = 128, N = 64
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ inline void mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
}

__device__ inline void arrive(uint64_t* bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(
                   tc::smem_u32(bar))
               : "memory");
}

__device__ inline void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst)), "l"(src)
               : "memory");
}

__device__ inline void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(tc::smem_u32(bar))
               : "memory");
}

__device__ inline void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ inline void conv_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kConv) : "memory"); }

// the two converter warps of quarter q (named barriers 2..5, 64 threads)
__device__ inline void quarter_sync(int q) {
  asm volatile("bar.sync %0, 64;" ::"r"(2 + q) : "memory");
}

// Gaspari-Cohn weight in FP32 for the mixed path (the polynomial of the
// reference's schr2, letkf_yb.F90:262-286), with an approximate reciprocal:
// its rounding is far below the BF16 split the weights feed.
__device__ inline float gc_fast(float ri) {
  if (ri > 2.0f) return 0.0f;
  if (ri > 1.0f) {
    float rj = ri * (1.0f / 12.0f) - 0.5f;
    rj = rj * ri + 0.625f;
    rj = rj * ri + 1.666667f;
    return (rj * ri - 5.0f) * ri + 4.0f - __fdividef(0.6666667f, ri);
  }
  if (ri > 0.0f) {
    const float rk = ri * ri;
    const float rj = (-0.25f * ri + 0.5f) * ri + 0.625f;
    return (rj * ri - 1.666667f) * rk + 1.0f;
  }
  return 1.0f;
}

// Wait for a phase, suspending between polls; gives up after limit_ns of wall
// time (2 s unless the context sets another, raising the CTA's abort flag) or
// as soon as another thread has given up.
__device__ inline bool wait(uint64_t* bar, uint32_t parity, volatile int* abort,
                            unsigned long long limit_ns) {
  if (tc::mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = tc::global_ns();
  while (true) {
    if (tc::mbar_try_wait_hint(bar, parity, 1000u)) return true;
    if (*abort) return false;
    if (tc::global_ns() - t0 > limit_ns) {
      *abort = 1;
      return false;
    }
  }
}

// ln p of level kk (1-based) at column col and its window [w0, w1) of records.
// The producer, MMA and converter warps each compute an item's windows, and
// they must agree to the bit: a window one record stage wider in one role than
// in another leaves the roles waiting for each other.  The function is
// therefore compiled once (not inlined): inlined copies of its FP32
// expressions can be contracted into fused multiply-adds differently at each
// call site, and with 512 ln p buckets such a difference crossed a bucket
// boundary on the clustered 2e6-observation workload and the Gram's waits ran
// out.
__device__ __noinline__ void level_window(const Geometry& g, const ListDev& l,
                                          const RecDev& rec, const double* axb, int col, int kk,
                                          float& al, int& w0, int& w1) {
  w0 = 0;
  w1 = l.cnt[col];
  al = 0.0f;
  if (!(g.vert_dist > 0.0)) return;
  const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
  const size_t ci = (size_t)(glat - 1 + g.halo) +
                    (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
  // in FP32 (the weights it feeds are FP32), converted without the FP64 pipe
  const float aps = d2f_bits(axb[g.ps_row + (size_t)g.n * ci]);
  const float ptop = d2f_bits(g.ptop), p0 = d2f_bits(g.p0);
  auto lev = [&](int k1) {
    if (g.vcoord == LG_VCOORD_SIGMA) return d2f_bits(g.ca[k1 - 1]) * (aps - ptop) + ptop;
    return d2f_bits(g.ca[k1 - 1]) * (p0 - ptop) + d2f_bits(g.cb[k1 - 1]) * (aps - ptop) + ptop;
  };
  al = logf(0.5f * (lev(kk) + lev(kk + 1)));
  const float span = 2.0f * (float)g.vert_dist;
  int b_lo = (int)floorf((al - span - rec.lo) * rec.inv_dz) - 1;
  int b_hi = (int)floorf((al + span - rec.lo) * rec.inv_dz) + 1;
  b_lo = b_lo < 0 ? 0 : (b_lo > rec.nb - 1 ? rec.nb - 1 : b_lo);
  b_hi = b_hi < 0 ? 0 : (b_hi > rec.nb - 1 ? rec.nb - 1 : b_hi);
  const int* bo = rec.boff + (size_t)col * (rec.nb + 1);
  w0 = bo[b_lo];
  w1 = bo[b_hi + 1];
}

// work item -> column and its first level (1-based) and level count.  Items are
// numbered level-group-major, so that the round-robin assignment gives every
// CTA a mix of level groups (near-surface groups have the longest record
// windows; column-major numbering gave each CTA a single group whenever the
// grid size was a multiple of the group count).
__device__ inline void item_levels(const SolveBatch& b, int item, int& col, int& kk0, int& G) {
  col = b.first_col + item % b.ncols;
  kk0 = (item / b.ncols) * kG + 1;
  G = min(kG, b.levels - kk0 + 1);
}

}  // namespace colk

// kRing: stages of records and ensemble rows in flight; kOps: operand buffers
// between the converter warps and the MMA warp.  <6, 4> fills an SM's shared
// memory (one CTA per SM, 174 KB); <2, 2> (74 KB) leaves ~154 KB of it to kernels of the
// other solve streams (tridiagonalisation, QL) running beside it: the
// tridiagonalisation is latency-bound below about two warps per SM
// sub-partition, so every 17 KB it gets back is a matrix in flight.
// 128 registers a thread (40 K of the SM's 64 K, launched as 320 threads): the
// compiler would otherwise take ~164 for the unrolled epilogue and leave the
// FP64 kernels beside the Gram short of registers.
template <int kRing, int kOps>
__global__ void __maxnreg__(128)
    gram_col_kernel(Geometry g, HxDev hx, ListDev l, SolveBatch b, const double* axb,
                    double* Cout, double* tout, int* err, RecDev rec) {
  using namespace colk;
  using Lay = Layout<kRing, kOps>;
  constexpr int kOffY = Lay::kOffY, kOffOps = Lay::kOffOps, kOffRec = Lay::kOffRec,
                kOffW = Lay::kOffW;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t full[kRing], empty[kRing], ready[kOps], opdone[kOps], tmem_free;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float s_t[4][64];
  __shared__ volatile int s_abort;
  __shared__ int s_go;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int k = g.ens;
  const int ngrp = (b.levels + kG - 1) / kG;
  const int nitems = b.ncols * ngrp;
  const bool vertical = g.vert_dist > 0.0;
  float* Y = reinterpret_cast<float*>(smem + kOffY);
  unsigned char* ops = smem + kOffOps;
  float4* R = reinterpret_cast<float4*>(smem + kOffRec);

  if (tid == 0) {
    for (int i = 0; i < kRing; ++i) {
      tc::mbar_init(&full[i], 64);  // 32 record arrivals + 32 copy-completion arrivals
      tc::mbar_init(&empty[i], 8);  // one per converter warp
    }
    for (int i = 0; i < kOps; ++i) {
      tc::mbar_init(&ready[i], 8);  // one per converter warp
      tc::mbar_init(&opdone[i], 1);  // tcgen05.commit
    }
    tc::mbar_init(&tmem_free, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
  }
  // the Y ring starts at zero: members >= k are never copied and stay 0
  for (int i = tid; i < kRing * kYBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(smem + kOffY)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(&tmem_base_sh)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_base_sh;

  const unsigned long long wait_ns =
      g.tc_wait_ns > 0 ? (unsigned long long)g.tc_wait_ns : 2000000000ull;
  // lane 0 waits, the warp follows its outcome (keeps the warp converged)
  auto wait_warp = [&](uint64_t* bar, int parity) {
    int r = 0;
    if (lane == 0) r = wait(bar, (uint32_t)(parity & 1), &s_abort, wait_ns) ? 1 : 0;
    return __shfl_sync(0xffffffffu, r, 0) != 0;
  };
  // the item's levels: lane lv (< G) holds level lv's ln p and record window;
  // [u0, u1) is the union of the windows.  Every role computes its own copy.
  auto item_windows = [&](int item, int& col, int& kk0, int& G, float& al, int& w0, int& w1,
                          int& u0, int& u1) {
    item_levels(b, item, col, kk0, G);
    al = 0.0f;
    w0 = INT_MAX;
    w1 = 0;
    if (lane < G) level_window(g, l, rec, axb, col, kk0 + lane, al, w0, w1);
    u0 = w0;
    u1 = w1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      u0 = min(u0, __shfl_xor_sync(0xffffffffu, u0, o));
      u1 = max(u1, __shfl_xor_sync(0xffffffffu, u1, o));
    }
  };

  if (warp == kProducer) {
    // ------------------------------------------------------------ producer
    int pst = 0;
    const int half = lane >> 4, part = lane & 15;
    const int cpr = k >> 2;  // 16-byte chunks per ensemble row
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);  // weight 0: padding
    bool ok = true;
    for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
      int col, kk0, G, w0, w1, u0, u1;
      float al;
      item_windows(item, col, kk0, G, al, w0, w1, u0, u1);
      if (u1 <= u0) continue;
      const int64_t base = l.off[col];
      const int nst = (u1 - u0 + kRows - 1) / kRows;
      auto ldrec = [&](int st, float4& a, float4& c) {
        const int i0 = u0 + st * kRows + lane, i1 = i0 + 32;
        a = i0 < u1 ? rec.r[base + i0] : z4;
        c = i1 < u1 ? rec.r[base + i1] : z4;
      };
      float4 r0, r1;
      ldrec(0, r0, r1);
      for (int st = 0; st < nst; ++st, ++pst) {
        const int slot = pst % kRing;
        if (pst >= kRing && !wait_warp(&empty[slot], pst / kRing - 1)) {
          ok = false;
          break;
        }
        float4* Rs = R + slot * kRows;
        Rs[lane] = r0;
        Rs[lane + 32] = r1;
        arrive(&full[slot]);
        __syncwarp();
        if (st + 1 < nst) ldrec(st + 1, r0, r1);  // in flight while this stage's rows are issued
        float* Ys = Y + (size_t)slot * kRows * 64;
        for (int row = half; row < kRows; row += 2) {
          const float4 rr = Rs[row];
          if (part < cpr && rr.z > 0.0f)
            cp_async16(Ys + row * 64 + part * 4,
                       hx.yb32 + (size_t)__float_as_int(rr.x) * k + part * 4);
        }
        cp_async_arrive(&full[slot]);
      }
    }
    cp_async_wait_all();
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issuer
    int p = 0, mma_items = 0;  // items with at least one MMA so far
    bool ok = true;
    for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
      int col, kk0, G, w0, w1, u0, u1;
      float al;
      item_windows(item, col, kk0, G, al, w0, w1, u0, u1);
      const int nst = u1 > u0 ? (u1 - u0 + kRows - 1) / kRows : 0;
      unsigned started = 0u;
      for (int st = 0; st < nst && ok; ++st) {
        const int r0 = u0 + st * kRows;
        for (int lv = 0; lv < kG; ++lv) {
          const int lw0 = __shfl_sync(0xffffffffu, w0, lv), lw1 = __shfl_sync(0xffffffffu, w1, lv);
          if (!(r0 + kRows > lw0 && r0 < lw1)) continue;
          // before the item's first MMA: the previous MMA item's epilogue has
          // copied its accumulators out of tensor memory
          if (started == 0u && mma_items > 0 && !wait_warp(&tmem_free, mma_items - 1)) {
            ok = false;
            break;
          }
          const int buf = p % kOps;
          if (!wait_warp(&ready[buf], p / kOps)) {
            ok = false;
            break;
          }
          if (lane == 0) {
            tc::fence_after();
            const uint32_t a0 = tc::smem_u32(ops + buf * kOpBytes);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const uint64_t da = tc::make_desc(a0 + c * kChunkA, 128, 256);
              mma(tmem + (uint32_t)(lv * kN), da, da, (((started >> lv) & 1u) || c > 0) ? 1u : 0u);
            }
            tc::mma_commit(&opdone[buf]);
          }
          __syncwarp();
          started |= 1u << lv;
          ++p;
        }
      }
      if (started) ++mma_items;
    }
    // this warp's MMAs are complete before the tensor memory is freed
    if (p > 0 && lane == 0) {
      const int o = p - 1;
      for (long long it = 0; it < tc::kSpinLimit; ++it)
        if (tc::mbar_try_wait(&opdone[o % kOps], (uint32_t)((o / kOps) & 1))) break;
    }
  } else {
    // ------------------------------------------------------------ converters
    const int m = tid & 63, q = tid >> 6;  // member; quarter q owns record groups q, q + 4
    const float inv_vd = vertical ? (float)(1.0 / g.vert_dist) : 0.0f;
    // sqrt(w) and sqrt(w) d of a quarter's 16 records for the item's levels,
    // [stage parity][quarter][sqrt(w) | sqrt(w) d][kG][16]: the two warps of a
    // quarter compute alternate levels and meet on the quarter's named barrier
    float* Wbase = reinterpret_cast<float*>(smem + kOffW);
    int cst = 0, p = 0;
    unsigned long long nnz = 0;  // non-zero (record, level) weights, each counted once
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
      int col, kk0, G, w0, w1, u0, u1;
      float al;
      item_windows(item, col, kk0, G, al, w0, w1, u0, u1);
      const int nst = u1 > u0 ? (u1 - u0 + kRows - 1) / kRows : 0;
      unsigned started = 0u;
      // t of each level as two FP32 partial sums (even and odd records) in one
      // packed register, added at the end
      unsigned long long tacc[kG];
#pragma unroll
      for (int lv = 0; lv < kG; ++lv) tacc[lv] = 0ull;
      bool ok = true;
      // Every converter warp runs all nst stages and reaches every quarter
      // barrier, also after a failed wait (then it only skips the work), so the
      // two warps of a quarter never wait for each other in vain.
      for (int st = 0; st < nst; ++st, ++cst) {
        const int slot = cst % kRing;
        if (ok) ok = wait_warp(&full[slot], cst / kRing);
        const int r0 = u0 + st * kRows;
        const float4* Rs = R + slot * kRows;
        float* SW = Wbase + ((cst & 1) * 4 + q) * (2 * kG * 16);
        float* SD = SW + kG * 16;
        {
          // weights of the quarter's 16 records (lane & 15) for levels of this
          // warp's parity: lv = (warp & 1) + 2 (lane >> 4) + 4 j
          const int r = lane & 15;
          const int row = r < 8 ? q * 8 + r : (q + 4) * 8 + (r - 8);
          const float4 rc = Rs[row];
#pragma unroll
          for (int j = 0; j < kG / 4; ++j) {
            const int lv = (warp & 1) + 2 * (lane >> 4) + 4 * j;
            const float lal = __shfl_sync(0xffffffffu, al, lv);
            const int lw0 = __shfl_sync(0xffffffffu, w0, lv), lw1 = __shfl_sync(0xffffffffu, w1, lv);
            float wt = rc.z, sw = 0.0f, sd = 0.0f;
            if (wt > 0.0f && r0 + row >= lw0 && r0 + row < lw1) {
              if (vertical) {
                const float z = fabsf(lal - rc.y) * inv_vd;
                wt *= g.gc_filter_vertical ? gc_fast(z) : (z > 2.0f ? 0.0f : 1.0f);
              }
              if (wt > 0.0f) {
                sw = wt * rsqrtf(wt);
                sd = rc.w * sw;
              }
            }
            nnz += sw > 0.0f ? 1u : 0u;
            SW[lv * 16 + r] = sw;
            SD[lv * 16 + r] = sd;
          }
        }
        float y[16];
        const float* Ys = Y + (size_t)slot * kRows * 64;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) y[h * 8 + jj] = Ys[((q + 4 * h) * 8 + jj) * 64 + m];
        quarter_sync(q);  // both warps' weights of the quarter are written
        if (!ok) continue;
        if (lane == 0) arrive(&empty[slot]);  // this warp has read the stage
#pragma unroll
        for (int lv = 0; lv < kG; ++lv) {
          const int lw0 = __shfl_sync(0xffffffffu, w0, lv), lw1 = __shfl_sync(0xffffffffu, w1, lv);
          if (!(r0 + kRows > lw0 && r0 < lw1)) continue;
          const int buf = p % kOps;
          if (p >= kOps && !wait_warp(&opdone[buf], p / kOps - 1)) {
            ok = false;
            break;
          }
          unsigned char* A = ops + buf * kOpBytes;
          const float4* sw4 = reinterpret_cast<const float4*>(SW + lv * 16);
          const float4* sd4 = reinterpret_cast<const float4*>(SD + lv * 16);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int gi = q + 4 * h;
            // weights of the group's 8 records (0 for padding: the ring holds finite
            // values there, and zeros for members >= k)
            const float4 wa = sw4[2 * h], wb = sw4[2 * h + 1];
            const float4 da = sd4[2 * h], db = sd4[2 * h + 1];
            const float swv[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
            const float sdv[8] = {da.x, da.y, da.z, da.w, db.x, db.y, db.z, db.w};
            uint32_t hi[4], lo[4];
#pragma unroll
            for (int jj = 0; jj < 8; jj += 2) {
              // two records at a time in the packed f32x2 instructions
              const unsigned long long v = tc::f2_mul(tc::f2_pack(y[h * 8 + jj], y[h * 8 + jj + 1]),
                                                      tc::f2_pack(swv[jj], swv[jj + 1]));
              tacc[lv] = tc::f2_fma(v, tc::f2_pack(sdv[jj], sdv[jj + 1]), tacc[lv]);
              tc::split_bf16x2_packed(v, hi[jj / 2], lo[jj / 2]);
            }
            const int chunk = gi >> 1, kc = gi & 1;
            const int off_hi = (m >> 3) * 256 + kc * 128 + (m & 7) * 16;
            const int mlo = m + 64;
            const int off_lo = (mlo >> 3) * 256 + kc * 128 + (mlo & 7) * 16;
            *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_hi) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
            *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_lo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
          }
          tc::fence_proxy_async();
          __syncwarp();
          if (lane == 0) arrive(&ready[buf]);
          started |= 1u << lv;
          ++p;
        }
      }
      // item end: the eight converter warps meet here whatever happened above
      if (ok && p > 0) ok = wait_warp(&opdone[(p - 1) % kOps], (p - 1) / kOps);
      if (!ok) s_abort = 1;
      conv_sync();
      if (tid == 0) s_go = s_abort ? 0 : 1;
      conv_sync();
      if (!s_go) break;
      tc::fence_after();
      // Epilogue in one 64 x 64 FP32 staging copy S (row stride kDS) in the
      // operand buffers: C[i][j] = hi[i][j] + (lo[i][j] + lo[j][i]), where hi is
      // accumulator row i (TMEM lanes 0..63) and lo row 64 + i.  The lo rows go
      // to S first; then each hi-row thread folds its row's lower triangle into
      // S in place -- it reads S[i][j] (its own row) and S[j][i] for j < i (the
      // upper triangle of row j, which no thread writes) -- and C is written
      // from the lower triangle.  A warp reads TMEM lanes 32 (warp % 4) ..;
      // warps 0-3 take columns 0..31, warps 4-7 columns 32..63.
      float* S = reinterpret_cast<float*>(ops);
      const int wq = warp & 3, cb = (warp >> 2) * 32;
      const int levels = b.levels;
      for (int lv = 0; lv < G; ++lv) {
        const size_t s = (size_t)(col - b.first_col) * levels + (kk0 - 1 + lv);
        double* C = Cout + s * k * k;
        double* t = tout + s * k;
        if (!((started >> lv) & 1u)) {
          for (int i = tid; i < k * k; i += kConv) C[i] = 0.0;
          for (int i = tid; i < k; i += kConv) t[i] = 0.0;
          continue;
        }
        const uint32_t taddr = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)(lv * kN + cb);
        if (wq >= 2) {
          const int r = (wq - 2) * 32 + lane;
#pragma unroll
          for (int c0 = 0; c0 < 32; c0 += 16) {
            float v[16];
            tc::tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) S[r * kDS + cb + c0 + i] = v[i];
          }
        }
        float tv = 0.0f;
#pragma unroll
        for (int u = 0; u < kG; ++u)
          if (u == lv) {
            const float2 t2 = tc::f2_unpack(tacc[u]);
            tv = t2.x + t2.y;
          }
        s_t[q][m] = tv;
        conv_sync();
        if (wq < 2) {
          const int i = wq * 32 + lane;
#pragma unroll
          for (int c0 = 0; c0 < 32; c0 += 16) {
            float v[16];
            tc::tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
            for (int ii = 0; ii < 16; ++ii) {
              const int j = cb + c0 + ii;
              if (j <= i) S[i * kDS + j] = v[ii] + (S[i * kDS + j] + S[j * kDS + i]);
            }
          }
        }
        conv_sync();
        for (int idx = tid; idx < k * k; idx += kConv) {
          const int i = idx % k, j = idx / k;
          C[idx] = f2d_bits(i >= j ? S[i * kDS + j] : S[j * kDS + i]);
        }
        if (tid < k) t[tid] = f2d_bits((s_t[0][tid] + s_t[1][tid]) + (s_t[2][tid] + s_t[3][tid]));
        conv_sync();
      }
      tc::fence_before();
      conv_sync();
      if (tid == 0 && started) arrive(&tmem_free);  // only items that used tensor memory
    }
    if (b.work) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nnz += __shfl_xor_sync(0xffffffffu, nnz, o);
      if (lane == 0 && nnz) atomicAdd(b.work, nnz);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  if (tid == 0 && s_abort) atomicExch(err, LG_ERR_TIMEOUT);
}

bool gram_col_supported(int ens) { return ens <= 64 && ens % 4 == 0; }

void launch_gram_col(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                     const double* axb, double* C, double* t, int* err, const RecDev& rec,
                     bool lean, int ctas, cudaStream_t stream) {
  if (b.nsolves == 0) return;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const int ngrp = (b.levels + colk::kG - 1) / colk::kG;
  const int nitems = b.ncols * ngrp;
  const int grid = std::min(nitems, ctas > 0 ? ctas : sms);
  if (lean) {
    constexpr int bytes = colk::Layout<2, 2>::kBytes;
    cudaFuncSetAttribute(gram_col_kernel<2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    gram_col_kernel<2, 2><<<grid, colk::kThreads, bytes, stream>>>(g, hx, l, b, axb, C, t, err, rec);
  } else {
    constexpr int bytes = colk::Layout<6, 4>::kBytes;
    cudaFuncSetAttribute(gram_col_kernel<6, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    gram_col_kernel<6, 4><<<grid, colk::kThreads, bytes, stream>>>(g, hx, l, b, axb, C, t, err, rec);
  }
}

}  // namespace lg
