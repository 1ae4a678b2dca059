// lg_gram_tf32.cu -- FP32-accurate Gram matrices on the 5th-generation tensor
// cores (tcgen05.mma.kind::tf32), for ensembles of up to 64 members; one CTA
// per solve.  The FP32 variant of the mixed path (LG_PREC_MIXED_TF32), beside
// the BF16 one of lg_gram_tc.cu / lg_gram_col.cu.
//
// Same quantities (letkf_core.F90:58-75,146-195):
//
//   y~_e = y_e * s_e  (s_e = sqrt(rdiaginv * rloc_k), FP32), split y~ = hi + lo
//   with hi = y~ with its 13 low mantissa bits cleared (a TF32 number) and
//   lo = y~ - hi (exact in FP32, read by the tensor core as TF32): hi + lo
//   carries y~ to about 2^-21, against about 2^-16 for the BF16 hi/lo split.
//   D = [hi ; lo] hi^T               one tcgen05.mma (M = 128, N = 64, K = 8)
//                                    per 8 records, FP32 accumulator in tensor
//                                    memory (rows 0..63 hi hi^T, 64..127 lo hi^T)
//   C = D[0:64] + D[64:128] + D[64:128]^T     (hi hi + lo hi + hi lo)
//   t = sum_e y~_e (s_e d_e)         on the CUDA cores in FP32
// The FP32 accumulation (about sqrt(p) 2^-24 relative) then bounds the error
// rather than the operand split.
//
// Operand tile of a stage of 64 records: 128 rows (members, then the same
// members' lo parts; rows of members >= ens are zero) x 64 TF32, K-major
// without swizzle: 8 x 16-byte core matrices (4 TF32 along K), LBO = 128 B
// between the two K halves of an 8-wide chunk, SBO = 256 B between 8-row
// groups -- the BF16 layout in bytes.  B is the hi half of the same tile.
//
// 128 threads: member m = tid % 64, record half h = tid / 64.  Records of
// stage s + 2 and ensemble values of stage s + 1 are loaded while stage s is
// scaled, split and issued; two stage buffers let the conversion overlap the
// MMAs.  Inputs: an analysis chunk (mode 0: the column's ln p-bucketed
// records, the level's window) or an explicit core batch (mode 1).  Every
// mbarrier wait is bounded; on expiry the kernel records LG_ERR_TIMEOUT, still
// waits (bounded) for its own MMAs, frees its tensor memory and returns.
#include "lg_device.cuh"
#include "lg_internal.h"
#include "lg_tc.cuh"

namespace lg {
namespace tf32k {

constexpr int kThreads = 128;
constexpr int kRows = 64;                  // records per stage
constexpr int kChunk = 128 * 8 * 4;        // 4096 B: 128 rows x K = 8 TF32
constexpr int kStageBytes = 8 * kChunk;    // 32 KB: 128 x 64 TF32
constexpr int kDS = 65;                    // row stride of the accumulator copy
constexpr int kSmem = 2 * kStageBytes;     // two stages; the 128 x kDS copy (33 KB) reuses them
constexpr int kTmemCols = 64;
// instruction descriptor: kind::tf32 (A, B TF32 = 2), FP32 D, K-major A and B, M = 128, N = 64
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ inline void mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
}

// hi = v with the 13 low mantissa bits cleared; lo = v - hi (exact)
__device__ inline void split_tf32(float v, uint32_t& hi, uint32_t& lo) {
  const uint32_t b = __float_as_uint(v) & 0xffffe000u;
  hi = b;
  lo = __float_as_uint(v - __uint_as_float(b));
}

}  // namespace tf32k

__global__ void __launch_bounds__(tf32k::kThreads) gram_tf32_kernel(Geometry g, HxDev hx,
                                                                  ListDev l, SolveBatch b,
                                                                  const double* axb,
                                                                  double* Cout, double* tout,
                                                                  int* err, RecDev rec) {
  using namespace tf32k;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int r_ent[3][kRows];
  __shared__ float r_s[3][kRows];  // sqrt(weight)
  __shared__ float r_d[3][kRows];  // sqrt(weight) * innovation
  __shared__ float s_t[2][64];
  __shared__ float s_al;
  __shared__ unsigned s_nnz;

  const int s = blockIdx.x;
  const int k = g.ens;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = tid & 63, half = tid >> 6;
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
    if (st + 2 < nst && warp == (st & 3)) load_records(st + 2);
    const int buf = st & 1;
    if (st >= 2) {
      if (!tc::mbar_wait(&mbar[buf], phase[buf])) ok = false;
      phase[buf] ^= 1u;
    }
    unsigned char* A = smem_raw + buf * kStageBytes;
    const int rb = st % 3;
    // this thread's 32 records: 8 groups of 4 (one 16-byte piece each), for
    // row m (hi) and row 64 + m (lo)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int q = half * 8 + j;  // 4-record group of the stage (0..15)
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = q * 4 + u;
        const float v = cur[j * 4 + u] * r_s[rb][e];
        tacc = fmaf(v, r_d[rb][e], tacc);
        tf32k::split_tf32(v, hi[u], lo[u]);
      }
      const int chunk = q >> 1, kc = q & 1;
      const int mlo = m + 64;
      const int off_hi = chunk * kChunk + (m >> 3) * 256 + kc * 128 + (m & 7) * 16;
      const int off_lo = chunk * kChunk + (mlo >> 3) * 256 + kc * 128 + (mlo & 7) * 16;
      *reinterpret_cast<uint4*>(A + off_hi) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(A + off_lo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      const uint32_t a0 = tc::smem_u32(A);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const uint64_t da = tc::make_desc(a0 + c * kChunk, 128, 256);
        mma(tmem_d, da, da, (st > 0 || c > 0) ? 1u : 0u);
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
    const int last = (nst - 1) & 1;
    if (!tc::mbar_wait(&mbar[last], phase[last])) ok = false;
    tc::fence_after();
    __syncthreads();
    float* D = reinterpret_cast<float*>(smem_raw);  // 128 x kDS
    // warp w reads tensor-memory lanes 32 w .. 32 w + 31 (accumulator rows)
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(warp * 32 + lane) * kDS + c0 + i] = v[i];
    }
    __syncthreads();
    for (int idx = tid; idx < k * k; idx += kThreads) {
      const int i = idx % k, j = idx / k;
      C[idx] = f2d_bits(D[i * kDS + j] + (D[(64 + i) * kDS + j] + D[(64 + j) * kDS + i]));
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

bool gram_tf32_supported(int ens) { return ens <= 64; }

void launch_gram_tf32(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                      const double* axb, double* C, double* t, int* err, const RecDev& rec,
                      cudaStream_t stream) {
  if (b.nsolves == 0) return;
  constexpr int smem = tf32k::kSmem + 1024;
  cudaFuncSetAttribute(gram_tf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  gram_tf32_kernel<<<b.nsolves, tf32k::kThreads, smem, stream>>>(g, hx, l, b, axb, C, t, err,
                                                                 rec);
}

}  // namespace lg
