// lg_gram_tc128.cu -- mixed-precision Gram matrices for ensembles of 65..128
// members on the 5th-generation tensor cores (one CTA per solve).
//
// Same quantities as lg_gram_tc.cu (letkf_core.F90:58-75,146-195):
//
//   y~_e = y_e * s_e  (s_e = sqrt(rdiaginv * rloc_k), FP32), split y~ = hi + lo (BF16)
//   D0 = hi hi^T,  D1 = lo hi^T       two tcgen05.mma (M = 128, N = 128, K = 16) per
//                                     16 records, FP32 accumulators in tensor memory
//                                     (columns 0..127 and 128..255)
//   C  = D0 + D1 + D1^T               (hi hi + lo hi + hi lo; lo lo, 2^-16, dropped)
//   t  = sum_e y~_e (s_e d_e)         on the CUDA cores in FP32 (full-precision
//                                     products, no split)
//
// With up to 128 members an operand row of 64 records is one 128 x 64 BF16 tile:
// rows are members (members >= ens are zero rows), K-major without swizzle in
// 8 x 16-byte core matrices (LBO = 128 B between the two K halves of a 16-wide
// chunk, SBO = 256 B between 8-row groups).  The hi tile is both A of the first
// MMA and B of both.
//
// 256 threads: member m = tid % 128, record half h = tid / 128 (records
// 32 h .. 32 h + 31 of a stage).  The records of a solve are consumed in stages
// of 64 consecutive ones (zero weights add zero rows); the records of stage
// s + 2 and the ensemble values of stage s + 1 are loaded while stage s is
// scaled, split and issued, and two stage buffers let the conversion of a stage
// overlap the MMAs of the previous one.  Inputs are either an analysis chunk
// (mode 0: the column's ln p-bucketed records, the level's window) or an
// explicit core batch (mode 1: hxens, rdiaginv, dep, rloc of each solve).
// Every mbarrier wait is bounded; on expiry the kernel records LG_ERR_TIMEOUT,
// still waits (bounded) for its own MMAs, frees its tensor memory and returns.
#include "lg_device.cuh"
#include "lg_internal.h"
#include "lg_tc.cuh"

namespace lg {
namespace t128 {

constexpr int kThreads = 256;
constexpr int kRows = 64;                    // records per stage
constexpr int kChunk = 128 * 16 * 2;         // 4096 B: 128 rows x K = 16 BF16
constexpr int kOpBytes = 4 * kChunk;         // 16 KB: one 128 x 64 tile
constexpr int kStageBytes = 2 * kOpBytes;    // hi | lo
constexpr int kDS = 129;                     // row stride of the D1 copy (odd: no bank conflicts)
constexpr int kSmem = 128 * kDS * 4 > 2 * kStageBytes ? 128 * kDS * 4 : 2 * kStageBytes;
constexpr int kTmemCols = 256;
// instruction descriptor: kind::f16, BF16 A/B, FP32 D, K-major A and B, M = 128, N = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ inline void mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
}

}  // namespace t128

__global__ void __launch_bounds__(t128::kThreads) gram_tc128_kernel(Geometry g, HxDev hx,
                                                                  ListDev l, SolveBatch b,
                                                                  const double* axb,
                                                                  double* Cout, double* tout,
                                                                  int* err, RecDev rec) {
  using namespace t128;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int r_ent[3][kRows];
  __shared__ float r_s[3][kRows];  // sqrt(weight)
  __shared__ float r_d[3][kRows];  // sqrt(weight) * innovation
  __shared__ float s_t[2][128];
  __shared__ float s_al;
  __shared__ unsigned s_nnz;

  const int s = blockIdx.x;
  const int k = g.ens;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = tid & 127, half = tid >> 7;
  const bool batch = b.mode == 1;
  const bool vertical = !batch && g.vert_dist > 0.0;

  int64_t base = 0;
  int w1 = 0, col = 0, kk = 1;
  if (batch) {
    base = b.b_off[s];
    w1 = b.b_nobsl[s];
  } else {
    solve_col_level(b, s, col, kk);
    base = l.off[col];
    w1 = l.cnt[col];
  }
  if (tid == 0) {
    s_nnz = 0u;
    s_al = 0.0f;
    if (vertical) {
      const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
      const size_t ci = (size_t)(glat - 1 + g.halo) +
                        (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
      const double aps = axb[g.ps_row + (size_t)g.n * ci];
      auto lev = [&](int k1) {
        if (g.vcoord == LG_VCOORD_SIGMA) return g.ca[k1 - 1] * (aps - g.ptop) + g.ptop;
        return g.ca[k1 - 1] * (g.p0 - g.ptop) + g.cb[k1 - 1] * (aps - g.ptop) + g.ptop;
      };
      s_al = (float)log(0.5 * (lev(kk) + lev(kk + 1)));
    }
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(&tmem_base_sh)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem_d = tmem_base_sh;
  const float al = s_al;
  const float inv_vd = vertical ? (float)(1.0 / g.vert_dist) : 0.0f;
  // the level's record window (ln p buckets within 2 vert_dist, one bucket of slack)
  int w0 = 0;
  if (vertical) {
    const float span = 2.0f * (float)g.vert_dist;
    int b_lo = (int)floorf((al - span - rec.lo) * rec.inv_dz) - 1;
    int b_hi = (int)floorf((al + span - rec.lo) * rec.inv_dz) + 1;
    b_lo = b_lo < 0 ? 0 : (b_lo > rec.nb - 1 ? rec.nb - 1 : b_lo);
    b_hi = b_hi < 0 ? 0 : (b_hi > rec.nb - 1 ? rec.nb - 1 : b_hi);
    const int* bo = rec.boff + (size_t)col * (rec.nb + 1);
    w0 = bo[b_lo];
    w1 = bo[b_hi + 1];
  }
  const int nrec = w1 - w0;
  const int nst = nrec > 0 ? (nrec + kRows - 1) / kRows : 0;

  // records of stage st into buffer st % 3 (one warp, two records per lane)
  auto load_records = [&](int st) {
    const int buf = st % 3;
    for (int e = lane; e < kRows; e += 32) {
      const int i = w0 + st * kRows + e;
      int ent = 0;
      float sw = 0.0f, sd = 0.0f;
      if (i < w1) {
        float w, d;
        if (batch) {
          ent = i;
          w = b.b_rdiag[base + i] * (float)b.b_rloc[base + i];
          d = (float)b.b_dep[base + i];
        } else {
          const float4 rr = rec.r[base + i];
          ent = __float_as_int(rr.x);
          w = rr.z;
          if (vertical) {
            const float z = fabsf(al - rr.y) * inv_vd;
            w *= g.gc_filter_vertical ? tc::schr2f(z) : (z > 2.0f ? 0.0f : 1.0f);
          }
          d = rr.w;
        }
        if (w > 0.0f) {
          sw = sqrtf(w);
          sd = d * sw;
          atomicAdd(&s_nnz, 1u);
        }
      }
      r_ent[buf][e] = ent;
      r_s[buf][e] = sw;
      r_d[buf][e] = sd;
    }
  };
  // this thread's 32 raw ensemble values (member m, records 32 half ..) of stage st
  auto load_y = [&](int st, float* v) {
    const int buf = st % 3;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int e = half * 32 + j;
      float y = 0.0f;
      if (m < k && r_s[buf][e] > 0.0f) {
        const int ent = r_ent[buf][e];
        y = batch ? (float)b.b_hx[(size_t)(base + ent) * k + m] : hx.yb32[(size_t)ent * k + m];
      }
      v[j] = y;
    }
  };

  float cur[32], nxt[32];
  float tacc = 0.0f;
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  if (nst > 0) {
    if (warp == 0) load_records(0);
    if (warp == 1 && nst > 1) load_records(1);
    __syncthreads();
    load_y(0, cur);
  }
  for (int st = 0; st < nst; ++st) {
    if (st + 1 < nst) load_y(st + 1, nxt);
    if (st + 2 < nst && warp == (st & 7)) load_records(st + 2);
    const int buf = st & 1;
    if (st >= 2) {  // the MMAs that read this buffer two stages ago are complete
      if (!tc::mbar_wait(&mbar[buf], phase[buf])) ok = false;
      phase[buf] ^= 1u;
    }
    unsigned char* Ahi = smem_raw + buf * kStageBytes;
    unsigned char* Alo = Ahi + kOpBytes;
    const int rb = st % 3;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gi = half * 4 + j;  // 8-record group of the stage
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int jj = 0; jj < 8; jj += 2) {
        const float v0 = cur[j * 8 + jj] * r_s[rb][gi * 8 + jj];
        const float v1 = cur[j * 8 + jj + 1] * r_s[rb][gi * 8 + jj + 1];
        tacc = fmaf(v0, r_d[rb][gi * 8 + jj], tacc);
        tacc = fmaf(v1, r_d[rb][gi * 8 + jj + 1], tacc);
        tc::split_bf16x2(v0, v1, hi[jj / 2], lo[jj / 2]);
      }
      const int chunk = gi >> 1, kc = gi & 1;
      const int off = chunk * kChunk + (m >> 3) * 256 + kc * 128 + (m & 7) * 16;
      *reinterpret_cast<uint4*>(Ahi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(Alo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      const uint32_t a_hi = tc::smem_u32(Ahi), a_lo = tc::smem_u32(Alo);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint64_t dh = tc::make_desc(a_hi + c * kChunk, 128, 256);
        const uint64_t dl = tc::make_desc(a_lo + c * kChunk, 128, 256);
        const uint32_t acc = (st > 0 || c > 0) ? 1u : 0u;
        mma(tmem_d, dh, dh, acc);
        mma(tmem_d + 128, dl, dh, acc);
      }
      tc::mma_commit(&mbar[buf]);
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) cur[i] = nxt[i];
  }

  s_t[half][m] = tacc;
  double* C = Cout + (size_t)s * k * k;
  double* t = tout + (size_t)s * k;
  if (nst == 0) {
    __syncthreads();
    for (int i = tid; i < k * k; i += kThreads) C[i] = 0.0;
    for (int i = tid; i < k; i += kThreads) t[i] = 0.0;
  } else {
    // the last commit covers every earlier MMA of this CTA
    const int last = (nst - 1) & 1;
    if (!tc::mbar_wait(&mbar[last], phase[last])) ok = false;
    tc::fence_after();
    __syncthreads();  // every thread is past its last read of the stage buffers
    float* S = reinterpret_cast<float*>(smem_raw);  // D1, 128 x kDS
    // warp w reads tensor-memory lanes 32 (w % 4) ..; warps 0-3 take columns
    // 0..63 of each accumulator, warps 4-7 columns 64..127
    const int wq = warp & 3, cb = (warp >> 2) * 64;
    const int i = wq * 32 + lane;
    const uint32_t lane_addr = tmem_d + ((uint32_t)(wq * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(lane_addr + 128u + (uint32_t)(cb + c0), v);
#pragma unroll
      for (int ii = 0; ii < 16; ++ii) S[i * kDS + cb + c0 + ii] = v[ii];
    }
    __syncthreads();
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(lane_addr + (uint32_t)(cb + c0), v);
      if (i < k) {
#pragma unroll
        for (int ii = 0; ii < 16; ++ii) {
          const int j = cb + c0 + ii;
          if (j < k)
            C[(size_t)i + (size_t)j * k] =
                f2d_bits(v[ii] + (S[i * kDS + j] + S[j * kDS + i]));
        }
      }
    }
    if (tid < k) t[tid] = f2d_bits(s_t[0][tid] + s_t[1][tid]);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(kTmemCols));
  if (!ok) atomicExch(err, LG_ERR_TIMEOUT);
  if (b.work && tid == 0 && s_nnz) atomicAdd(b.work, (unsigned long long)s_nnz);
}

bool gram_tc128_supported(int ens) { return ens > 64 && ens <= 128; }

void launch_gram_tc128(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                       const double* axb, double* C, double* t, int* err, const RecDev& rec,
                       cudaStream_t stream) {
  if (b.nsolves == 0) return;
  constexpr int smem = t128::kSmem + 1024;
  cudaFuncSetAttribute(gram_tc128_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  gram_tc128_kernel<<<b.nsolves, t128::kThreads, smem, stream>>>(g, hx, l, b, axb, C, t, err,
                                                                 rec);
}

}  // namespace lg
