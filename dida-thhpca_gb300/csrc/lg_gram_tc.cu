// lg_gram_tc.cu -- mixed-precision Gram matrix on the 5th-generation tensor cores.
//
// Same quantities as lg_gram.cu (letkf_core.F90:58-75,146-195), computed as one
// BF16 x BF16 -> FP32 tcgen05.mma per 16 local entries:
//
//   y~_e = y_e * s_e  (s_e = sqrt(rdiaginv * rloc_k), FP32), split y~ = hi + lo (BF16)
//   d~_e = s_e * d_e, split d~ = dhi + dlo
//   A (M = 128 x K) = [ hi^T ; lo^T ]            rows 0..63 hi, 64..127 lo (members)
//   B (K x N = 80)   = [ hi | dhi | dlo | 0 ]    columns 0..63 members, 64/65 innovation
//   D = A B  (FP32 accumulator in tensor memory)
//   C = D[0:64,0:64] + D[64:128,0:64] + D[64:128,0:64]^T     (hi hi + lo hi + hi lo)
//   t = D[0:64,64] + D[0:64,65] + D[64:128,64]
// The lo x lo and lo x dlo terms (relative 2^-16) are dropped.  The three
// accumulator terms are summed in FP32 before the conversion to FP64: the two
// small ones are 2^-8 of the first, so the sum's rounding (2^-24) stays below
// the accumulation error of the tensor-core sums themselves.
//
// One CTA (4 warps) per solve.  Nonzero-weight entries are compacted into a
// shared queue, 64 at a time they are scaled, split and written to one of two
// shared-memory stages in the canonical K-major no-swizzle UMMA layout (8x16-byte
// core matrices: LBO = 128 B between the two K halves of a 16-wide chunk,
// SBO = 256 B between 8-row groups); thread 0 issues four MMAs per stage and
// commits them to the stage's mbarrier, so the next stage's preparation
// overlaps the tensor-core work.  Every mbarrier wait is bounded; on expiry the
// kernel records LG_ERR_TIMEOUT, still waits (bounded) for its own MMAs, frees
// its tensor memory and returns.
#include <cuda_bf16.h>

#include "lg_device.cuh"
#include "lg_internal.h"
#include "lg_tc.cuh"

namespace lg {



__global__ void __launch_bounds__(tc::kThreads) gram_tc_kernel(Geometry g, HxDev hx, ListDev l,
                                                              SolveBatch b, const double* axb,
                                                              double* Cout, double* tout,
                                                              int* err, RecDev rec) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* stage_base = smem_raw;  // 2 stages
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int q_ent[kQueueCap];
  __shared__ float q_s[kQueueCap];
  __shared__ int q_n;
  __shared__ float s_al;
  __shared__ int s_fail;

  const int s = blockIdx.x;
  const int k = g.ens;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  int64_t base = 0;
  int p = 0;
  int col = 0;
  bool vertical = false;
  const bool use_rec = (b.mode == 0) && rec.r != nullptr;
  if (b.mode == 0) {
    int kk;
    solve_col_level(b, s, col, kk);
    base = l.off[col];
    p = l.cnt[col];
    vertical = g.vert_dist > 0.0;
    if (vertical && tid == 0) {
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
  } else {
    base = b.b_off[s];
    p = b.b_nobsl[s];
  }
  // zero both stages once (the padding rows of B stay zero), init barriers
  for (int i = tid; i < 2 * kStageBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(stage_base)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    q_n = 0;
    s_fail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_d = tmem_base_sh;
  const float al = s_al;
  const float inv_vd = vertical ? (float)(1.0 / g.vert_dist) : 0.0f;

  int scan = 0;
  if (use_rec && vertical) {
    // only the ln p buckets within 2 vert_dist of this level (one bucket of slack)
    const float span = 2.0f * (float)g.vert_dist;
    int b_lo = (int)floorf((al - span - rec.lo) * rec.inv_dz) - 1;
    int b_hi = (int)floorf((al + span - rec.lo) * rec.inv_dz) + 1;
    b_lo = b_lo < 0 ? 0 : (b_lo > rec.nb - 1 ? rec.nb - 1 : b_lo);
    b_hi = b_hi < 0 ? 0 : (b_hi > rec.nb - 1 ? rec.nb - 1 : b_hi);
    const int* bo = rec.boff + (size_t)col * (rec.nb + 1);
    scan = bo[b_lo];
    p = bo[b_hi + 1];
  }
  int nproc = 0;
  int stage = 0;      // stages issued
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  while (true) {
    // compact nonzero-weight entries into the queue
    while (true) {
      __syncthreads();
      const int qn0 = q_n;
      __syncthreads();  // everyone has read q_n before the next atomics
      if (qn0 >= kStageEntries || scan >= p) break;
      const int i = scan + tid;
      if (i < p) {
        int ent;
        float w;
        if (use_rec) {
          const float4 rr = rec.r[base + i];
          ent = __float_as_int(rr.x);
          w = rr.z;
          if (vertical) {
            const float z = fabsf(al - rr.y) * inv_vd;
            w *= g.gc_filter_vertical ? schr2f(z) : (z > 2.0f ? 0.0f : 1.0f);
          }
        } else if (b.mode == 0) {
          ent = l.ent[base + i];
          float rl = (float)l.rloc[base + i];
          if (vertical) {
            const float z = fabsf(al - (float)hx.lnp[ent]) * inv_vd;
            rl *= g.gc_filter_vertical ? schr2f(z) : (z > 2.0f ? 0.0f : 1.0f);
          }
          w = hx.rdiag[ent] * rl;
        } else {
          ent = i;
          w = b.b_rdiag[base + i] * (float)b.b_rloc[base + i];
        }
        if (w > 0.0f) {
          const int slot = atomicAdd(&q_n, 1);
          q_ent[slot] = ent;
          q_s[slot] = sqrtf(w);
        }
      }
      scan += kThreads;
    }
    const int qn = q_n;
    if (qn == 0) break;
    const int nt = qn < kStageEntries ? qn : kStageEntries;
    nproc += nt;
    const int buf = stage & 1;
    if (stage >= 2) {  // the MMAs that read this buffer two stages ago must be done
      if (!mbar_wait(&mbar[buf], phase[buf])) ok = false;
      phase[buf] ^= 1u;
    }
    unsigned char* A = stage_base + buf * kStageBytes;
    unsigned char* B = A + 4 * kChunkA;
    // scale, split and store: thread -> member m, entry groups of 8
    {
      const int m = tid & 63, g0 = tid >> 6;
      for (int gi = g0; gi < 8; gi += 2) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int jj = 0; jj < 8; jj += 2) {
          float v[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int e = gi * 8 + jj + u;
            float x = 0.0f;
            if (e < nt && m < k) {
              const int ent = q_ent[e];
              const float* y = (b.mode == 0) ? hx.yb32 + (size_t)ent * k : nullptr;
              const float yv = (b.mode == 0) ? y[m] : (float)b.b_hx[(size_t)(base + ent) * k + m];
              x = yv * q_s[e];
            }
            v[u] = x;
          }
          __nv_bfloat162 h2 = __floats2bfloat162_rn(v[0], v[1]);
          const float2 hf = __bfloat1622float2(h2);
          hi[jj / 2] = *reinterpret_cast<uint32_t*>(&h2);
          lo[jj / 2] = pack_bf16(v[0] - hf.x, v[1] - hf.y);
        }
        const int chunk = gi >> 1, kc = gi & 1;
        const int off_row = (m >> 3) * 256 + kc * 128 + (m & 7) * 16;
        *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_row) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        const int mlo = m + 64;
        const int off_lo = (mlo >> 3) * 256 + kc * 128 + (mlo & 7) * 16;
        *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_lo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        *reinterpret_cast<uint4*>(B + chunk * kChunkB + off_row) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      }
      // innovation rows 64 (hi) and 65 (lo) of B
      if (tid < 8) {
        const int gi = tid;
        float dv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int e = gi * 8 + j;
          float x = 0.0f;
          if (e < nt) {
            const int ent = q_ent[e];
            const double d = (b.mode == 0) ? hx.dis[ent] : b.b_dep[base + ent];
            x = (float)d * q_s[e];
          }
          dv[j] = x;
        }
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          __nv_bfloat162 h2 = __floats2bfloat162_rn(dv[j], dv[j + 1]);
          const float2 hf = __bfloat1622float2(h2);
          hi[j / 2] = *reinterpret_cast<uint32_t*>(&h2);
          lo[j / 2] = pack_bf16(dv[j] - hf.x, dv[j + 1] - hf.y);
        }
        const int chunk = gi >> 1, kc = gi & 1;
        const int r64 = 8 * 256 + kc * 128 + 0 * 16, r65 = 8 * 256 + kc * 128 + 1 * 16;
        *reinterpret_cast<uint4*>(B + chunk * kChunkB + r64) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(B + chunk * kChunkB + r65) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint64_t da = make_desc(a0 + c * kChunkA, 128, 256);
        const uint64_t db = make_desc(b0 + c * kChunkB, 128, 256);
        mma_bf16(tmem_d, da, db, (stage > 0 || c > 0) ? 1u : 0u);
      }
      mma_commit(&mbar[buf]);
    }
    ++stage;
    // drop the consumed entries from the queue
    const int rem = qn - nt;
    int te = 0;
    float ts = 0.0f;
    if (tid < rem) {
      te = q_ent[nt + tid];
      ts = q_s[nt + tid];
    }
    __syncthreads();
    if (tid < rem) {
      q_ent[tid] = te;
      q_s[tid] = ts;
    }
    if (tid == 0) q_n = rem;
  }

  double* C = Cout + (size_t)s * k * k;
  double* t = tout + (size_t)s * k;
  if (stage == 0) {
    for (int i = tid; i < k * k; i += kThreads) C[i] = 0.0;
    for (int i = tid; i < k; i += kThreads) t[i] = 0.0;
  } else {
    // wait for the last commit (it covers every earlier MMA of this thread)
    const int last = (stage - 1) & 1;
    if (!mbar_wait(&mbar[last], phase[last])) ok = false;
    fence_after();
    float* D = reinterpret_cast<float*>(stage_base);  // 128 x kDS, reuses the stages
    for (int c0 = 0; c0 < kN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(warp * 32 + lane) * kDS + c0 + i] = v[i];
    }
    __syncthreads();
    for (int idx = tid; idx < k * k; idx += kThreads) {
      const int i = idx % k, j = idx / k;
      C[idx] = (double)(D[i * kDS + j] + (D[(64 + i) * kDS + j] + D[(64 + j) * kDS + i]));
    }
    for (int i = tid; i < k; i += kThreads)
      t[i] = (double)(D[i * kDS + 64] + (D[i * kDS + 65] + D[(64 + i) * kDS + 64]));
  }
  if (!ok && tid == 0) s_fail = 1;
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(kTmemCols));
  if (s_fail && tid == 0) atomicExch(err, LG_ERR_TIMEOUT);
  if (b.work && tid == 0) atomicAdd(b.work, (unsigned long long)nproc);
}

// a tensor-core Gram exists for every ensemble size the library accepts
bool gram_tc_supported(int ens) { return ens <= 128; }

void launch_gram_tc(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                    const double* axb, double* C, double* t, int* err, cudaStream_t stream,
                    const RecDev* rec) {
  if (b.nsolves == 0) return;
  const size_t smem = 2 * tc::kStageBytes + 1024;
  RecDev r{};
  if (rec) r = *rec;
  if (gram_tc128_supported(g.ens)) {
    launch_gram_tc128(g, hx, l, b, axb, C, t, err, r, stream);
    return;
  }
  cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  gram_tc_kernel<<<b.nsolves, tc::kThreads, smem, stream>>>(g, hx, l, b, axb, C, t, err, r);
}

}  // namespace lg

namespace lg {

// Streaming variant for the analysis path: the solve's records (ln p-bucketed,
// see records_kernel) are consumed in fixed stages of 64 consecutive records,
// zero-weight ones included (they add zero rows), so no compaction is needed
// and the loads can run ahead: the records of stage s+2 and the Y rows of
// stage s+1 are in flight while stage s is scaled, split and issued.
__global__ void __launch_bounds__(tc::kThreads) gram_tc_stream_kernel(Geometry g, HxDev hx,
                                                                     ListDev l, SolveBatch b,
                                                                     const double* axb,
                                                                     double* Cout, double* tout,
                                                                     int* err, RecDev rec) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* stage_base = smem_raw;
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int r_ent[3][kStageEntries];
  __shared__ float r_s[3][kStageEntries];   // sqrt(weight)
  __shared__ float r_d[3][kStageEntries];   // sqrt(weight) * innovation
  __shared__ float s_al;
  __shared__ int s_fail;
  __shared__ unsigned s_nnz;

  const int s = blockIdx.x;
  const int k = g.ens;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int col, kk;
  solve_col_level(b, s, col, kk);
  const int64_t base = l.off[col];
  const bool vertical = g.vert_dist > 0.0;
  if (tid == 0) {
    s_fail = 0;
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
  }
  for (int i = tid; i < 2 * kStageBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(stage_base)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_d = tmem_base_sh;
  const float al = s_al;
  const float inv_vd = vertical ? (float)(1.0 / g.vert_dist) : 0.0f;
  // record window of this level
  int w0 = 0, w1 = l.cnt[col];
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
  const int nst = (nrec + kStageEntries - 1) / kStageEntries;
  const int m = tid & 63, g0 = tid >> 6;

  // records of stage st into buffer st % 3 by warp wq (two records per lane)
  auto load_records = [&](int st) {
    const int buf = st % 3;
    for (int e = lane; e < kStageEntries; e += 32) {
      const int i = w0 + st * kStageEntries + e;
      int ent = 0;
      float sw = 0.0f, sd = 0.0f;
      if (i < w1) {
        const float4 rr = rec.r[base + i];
        ent = __float_as_int(rr.x);
        float w = rr.z;
        if (vertical) {
          const float z = fabsf(al - rr.y) * inv_vd;
          w *= g.gc_filter_vertical ? schr2f(z) : (z > 2.0f ? 0.0f : 1.0f);
        }
        if (w > 0.0f) {
          sw = sqrtf(w);
          sd = rr.w * sw;
          atomicAdd(&s_nnz, 1u);
        }
      }
      r_ent[buf][e] = ent;
      r_s[buf][e] = sw;
      r_d[buf][e] = sd;
    }
  };
  // this thread's 32 raw Y values (member m) of stage st
  auto load_y = [&](int st, float* v) {
    const int buf = st % 3;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const int e = (g0 + 2 * j) * 8 + jj;
        v[j * 8 + jj] = (m < k && r_s[buf][e] > 0.0f)
                            ? hx.yb32[(size_t)r_ent[buf][e] * k + m] : 0.0f;
      }
  };

  float cur[32], nxt[32];
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
      if (!mbar_wait(&mbar[buf], phase[buf])) ok = false;
      phase[buf] ^= 1u;
    }
    unsigned char* A = stage_base + buf * kStageBytes;
    unsigned char* B = A + 4 * kChunkA;
    const int rb = st % 3;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gi = g0 + 2 * j;
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int jj = 0; jj < 8; jj += 2) {
        const float v0 = cur[j * 8 + jj] * r_s[rb][gi * 8 + jj];
        const float v1 = cur[j * 8 + jj + 1] * r_s[rb][gi * 8 + jj + 1];
        split_bf16x2(v0, v1, hi[jj / 2], lo[jj / 2]);
      }
      const int chunk = gi >> 1, kc = gi & 1;
      const int off_row = (m >> 3) * 256 + kc * 128 + (m & 7) * 16;
      const int mlo = m + 64;
      const int off_lo = (mlo >> 3) * 256 + kc * 128 + (mlo & 7) * 16;
      *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_row) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(A + chunk * kChunkA + off_lo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      *reinterpret_cast<uint4*>(B + chunk * kChunkB + off_row) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    }
    if (tid < 8) {
      const int gi = tid;
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const float d0 = r_d[rb][gi * 8 + j], d1 = r_d[rb][gi * 8 + j + 1];
        __nv_bfloat162 h2 = __floats2bfloat162_rn(d0, d1);
        const float2 hf = __bfloat1622float2(h2);
        hi[j / 2] = *reinterpret_cast<uint32_t*>(&h2);
        lo[j / 2] = pack_bf16(d0 - hf.x, d1 - hf.y);
      }
      const int chunk = gi >> 1, kc = gi & 1;
      const int r64 = 8 * 256 + kc * 128, r65 = 8 * 256 + kc * 128 + 16;
      *reinterpret_cast<uint4*>(B + chunk * kChunkB + r64) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(B + chunk * kChunkB + r65) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint64_t da = make_desc(a0 + c * kChunkA, 128, 256);
        const uint64_t db = make_desc(b0 + c * kChunkB, 128, 256);
        mma_bf16(tmem_d, da, db, (st > 0 || c > 0) ? 1u : 0u);
      }
      mma_commit(&mbar[buf]);
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) cur[i] = nxt[i];
  }

  double* C = Cout + (size_t)s * k * k;
  double* t = tout + (size_t)s * k;
  if (nst == 0) {
    for (int i = tid; i < k * k; i += kThreads) C[i] = 0.0;
    for (int i = tid; i < k; i += kThreads) t[i] = 0.0;
  } else {
    const int last = (nst - 1) & 1;
    if (!mbar_wait(&mbar[last], phase[last])) ok = false;
    fence_after();
    float* D = reinterpret_cast<float*>(stage_base);
    for (int c0 = 0; c0 < kN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(warp * 32 + lane) * kDS + c0 + i] = v[i];
    }
    __syncthreads();
    for (int idx = tid; idx < k * k; idx += kThreads) {
      const int i = idx % k, j = idx / k;
      C[idx] = (double)(D[i * kDS + j] + (D[(64 + i) * kDS + j] + D[(64 + j) * kDS + i]));
    }
    for (int i = tid; i < k; i += kThreads)
      t[i] = (double)(D[i * kDS + 64] + (D[i * kDS + 65] + D[(64 + i) * kDS + 64]));
  }
  if (!ok && tid == 0) s_fail = 1;
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(kTmemCols));
  if (s_fail && tid == 0) atomicExch(err, LG_ERR_TIMEOUT);
  if (b.work && tid == 0 && s_nnz) atomicAdd(b.work, (unsigned long long)s_nnz);
}

void launch_gram_tc_stream(const Geometry& g, const HxDev& hx, const ListDev& l,
                           const SolveBatch& b, const double* axb, double* C, double* t, int* err,
                           const RecDev& rec, cudaStream_t stream) {
  if (b.nsolves == 0) return;
  if (gram_tc128_supported(g.ens)) {
    launch_gram_tc128(g, hx, l, b, axb, C, t, err, rec, stream);
    return;
  }
  const size_t smem = 2 * tc::kStageBytes + 1024;
  cudaFuncSetAttribute(gram_tc_stream_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  gram_tc_stream_kernel<<<b.nsolves, tc::kThreads, smem, stream>>>(g, hx, l, b, axb, C, t, err,
                                                                   rec);
}

}  // namespace lg
