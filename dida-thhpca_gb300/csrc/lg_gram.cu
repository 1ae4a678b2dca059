// lg_gram.cu -- FP64 weighted Gram matrix and innovation projection per solve.
//
// For one LETKF solve with local entries e (letkf_core.F90:58-75,146-195):
//   rloc_k(e) = rloc(e) * schr2(|ln p_k - ln p_e| / vert_dist)   (vertical path,
//               vertical_localization, letkf_yb.F90:240-260)
//   rr(e)     = sqrt(rdiaginv(e) * rloc_k(e))
//   C         = sum_e (y_e rr_e)(y_e rr_e)^T        (dgemm 'n','t', k x k x p)
//   t         = sum_e (y_e rr_e) rr_e d_e           (Pa * t = overline_w)
// Entries with zero weight contribute nothing and are compacted out before the
// tile products.  One CTA per solve; 4x4 register blocks of the lower triangle.
#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

constexpr int kTE = 32;        // entries per tile
constexpr int kGramThreads = 256;

__device__ inline double alnp_level(const Geometry& g, int kk, double aps) {
  // ps2alnp (obs_make.F90:418-437), with ph_lev(nz+1) evaluated
  auto lev = [&](int k1) {
    if (g.vcoord == LG_VCOORD_SIGMA)
      return __dadd_rn(__dmul_rn(g.ca[k1 - 1], __dsub_rn(aps, g.ptop)), g.ptop);
    const double t1 = __dmul_rn(g.ca[k1 - 1], __dsub_rn(g.p0, g.ptop));
    const double t2 = __dmul_rn(g.cb[k1 - 1], __dsub_rn(aps, g.ptop));
    return __dadd_rn(__dadd_rn(t1, t2), g.ptop);
  };
  return log(__dmul_rn(0.5, __dadd_rn(lev(kk), lev(kk + 1))));
}

// Thread roles.  The lower triangle of C is cut into 4 x 4 register blocks
// (NB = nb (nb + 1) / 2 of them, nb = ceil(k / 4)).  With NB <= 256 the
// threads form G = floor(256 / NB) groups, each owning every block, and group
// g takes the entries g, g + G, ... of each tile, so that nearly all threads
// multiply (55 blocks at 40 members: four groups, 220 threads); the groups'
// partial sums are added in group order at the end.  Above 256 blocks each
// thread owns kMaxBlk blocks.  The queue of non-zero-weight entries is filled
// 256 candidates at a time by all threads (weights in parallel, compacted by
// warp ballots in list order), so the result does not depend on timing.
template <int kMaxBlk>
__global__ void __launch_bounds__(kGramThreads, kMaxBlk == 1 ? 3 : 1)
    gram64_kernel(Geometry g, HxDev hx, ListDev l, SolveBatch b, const double* axb,
                  double* Cout, double* tout) {
  constexpr int kQueueCap = kTE + kGramThreads;
  const int s = blockIdx.x;
  const int k = g.ens;
  const int kp = (k + 3) & ~3;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  extern __shared__ double smem[];
  double* ytile = smem;                     // kTE x kp
  double* rd = ytile + kTE * kp;            // kTE: rr * dep
  double* red = smem;                       // at the end: groups' partial sums
  __shared__ int q_ent[kQueueCap];
  __shared__ double q_rr[kQueueCap];
  __shared__ int s_wcnt[kGramThreads / 32];
  __shared__ int q_n;
  __shared__ double s_al;

  int64_t base = 0;
  int p = 0;
  int col = 0, kk = 1;
  bool vertical = false;
  if (b.mode == 0) {
    solve_col_level(b, s, col, kk);
    base = l.off[col];
    p = l.cnt[col];
    vertical = g.vert_dist > 0.0;
    if (vertical && tid == 0) {
      const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
      const size_t ci = (size_t)(glat - 1 + g.halo) +
                        (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
      s_al = alnp_level(g, kk, axb[g.ps_row + (size_t)g.n * ci]);
    }
  } else {
    base = b.b_off[s];
    p = b.b_nobsl[s];
  }
  if (tid == 0) q_n = 0;
  __syncthreads();
  const double al = s_al;

  const int nb = kp / 4;
  const int NB = nb * (nb + 1) / 2;
  const int G = kMaxBlk == 1 ? max(1, kGramThreads / NB) : 1;
  const int grp = kMaxBlk == 1 ? tid / NB : 0;
  int bi[kMaxBlk], bj[kMaxBlk];
  double acc[kMaxBlk][16];
#pragma unroll
  for (int q = 0; q < kMaxBlk; ++q) {
    const int id = kMaxBlk == 1 ? (grp < G ? tid - grp * NB : NB) : tid + q * kGramThreads;
    bi[q] = -1;
    bj[q] = 0;
    if (id < NB) {
      int r = 0;  // row of the block: r (r + 1) / 2 <= id < (r + 1) (r + 2) / 2
      while ((r + 1) * (r + 2) / 2 <= id) ++r;
      bi[q] = r;
      bj[q] = id - r * (r + 1) / 2;
    }
#pragma unroll
    for (int z = 0; z < 16; ++z) acc[q][z] = 0.0;
  }
  double tacc = 0.0;  // t_i for i = tid (tid < k)

  int scan = 0;
  int nproc = 0;
  while (true) {
    // refill: every thread weighs one candidate of the next 256; the non-zero
    // ones join the queue in list order
    while (true) {
      const int qn0 = q_n;
      if (qn0 >= kTE || scan >= p) break;
      const int i = scan + tid;
      double rr = 0.0;
      int ent = 0;
      if (i < p) {
        double rl, rdg;
        if (b.mode == 0) {
          ent = l.ent[base + i];
          rl = l.rloc[base + i];
          rdg = (double)hx.rdiag[ent];
          if (vertical) {
            const double z = fabs(al - hx.lnp[ent]) / g.vert_dist;
            rl = rl * (g.gc_filter_vertical ? schr2(z) : schr(z));
          }
        } else {
          ent = i;
          rl = b.b_rloc[base + i];
          rdg = (double)b.b_rdiag[base + i];
        }
        rr = sqrt(rdg * rl);
      }
      const bool nz = rr != 0.0;
      const unsigned m = __ballot_sync(0xffffffffu, nz);
      if (lane == 0) s_wcnt[warp] = __popc(m);
      __syncthreads();
      int off = qn0, tot = 0;
#pragma unroll
      for (int w = 0; w < kGramThreads / 32; ++w) {
        const int c = s_wcnt[w];
        off += w < warp ? c : 0;
        tot += c;
      }
      if (nz) {
        const int pos = off + __popc(m & ((1u << lane) - 1u));
        q_ent[pos] = ent;
        q_rr[pos] = rr;
      }
      __syncthreads();  // every thread has read s_wcnt and q_n
      if (tid == 0) q_n = qn0 + tot;
      scan += kGramThreads;
      __syncthreads();
    }
    const int qn = q_n;
    if (qn == 0) break;
    const int nt = qn < kTE ? qn : kTE;
    nproc += nt;
    // stage the tile: ytile[e][i] = y_e[i] * rr_e, rd[e] = rr_e * d_e
    for (int idx = tid; idx < kTE * kp; idx += kGramThreads) {
      const int e = idx / kp, i = idx - e * kp;
      double v = 0.0;
      if (e < nt && i < k) {
        const int ent = q_ent[e];
        const double* y = (b.mode == 0) ? hx.yb + (size_t)ent * k
                                        : b.b_hx + (size_t)(base + ent) * k;
        v = y[i] * q_rr[e];
      }
      ytile[idx] = v;
    }
    if (tid < kTE) {
      double v = 0.0;
      if (tid < nt) {
        const int ent = q_ent[tid];
        const double d = (b.mode == 0) ? hx.dis[ent] : b.b_dep[base + ent];
        v = q_rr[tid] * d;
      }
      rd[tid] = v;
    }
    // the queue's remainder moves to its front
    const int rem = qn - nt;
    int tmp_e = 0;
    double tmp_r = 0.0;
    if (tid < rem) {
      tmp_e = q_ent[nt + tid];
      tmp_r = q_rr[nt + tid];
    }
    __syncthreads();  // tile staged; remainder read
    if (tid < rem) {
      q_ent[tid] = tmp_e;
      q_rr[tid] = tmp_r;
    }
    if (tid == 0) q_n = rem;
    // products: this thread's blocks over its group's entries of the tile
#pragma unroll
    for (int q = 0; q < kMaxBlk; ++q) {
      if (bi[q] < 0) continue;
      const double* ya = ytile + 4 * bi[q];
      const double* yc = ytile + 4 * bj[q];
#pragma unroll 2
      for (int e = grp; e < nt; e += G) {
        const double a0 = ya[e * kp], a1 = ya[e * kp + 1], a2 = ya[e * kp + 2], a3 = ya[e * kp + 3];
        const double c0 = yc[e * kp], c1 = yc[e * kp + 1], c2 = yc[e * kp + 2], c3 = yc[e * kp + 3];
        acc[q][0] += a0 * c0; acc[q][1] += a0 * c1; acc[q][2] += a0 * c2; acc[q][3] += a0 * c3;
        acc[q][4] += a1 * c0; acc[q][5] += a1 * c1; acc[q][6] += a1 * c2; acc[q][7] += a1 * c3;
        acc[q][8] += a2 * c0; acc[q][9] += a2 * c1; acc[q][10] += a2 * c2; acc[q][11] += a2 * c3;
        acc[q][12] += a3 * c0; acc[q][13] += a3 * c1; acc[q][14] += a3 * c2; acc[q][15] += a3 * c3;
      }
    }
    if (tid < k) {
      for (int e = 0; e < nt; ++e) tacc += ytile[e * kp + tid] * rd[e];
    }
    __syncthreads();
  }
  // the groups' partial sums, added in group order
  if (kMaxBlk == 1 && G > 1) {
    const int blk = tid - grp * NB;
    if (grp > 0 && grp < G && bi[0] >= 0)
      for (int z = 0; z < 16; ++z) red[((size_t)(grp - 1) * NB + blk) * 16 + z] = acc[0][z];
    __syncthreads();
    if (grp == 0)
      for (int g2 = 1; g2 < G; ++g2)
        for (int z = 0; z < 16; ++z) acc[0][z] += red[((size_t)(g2 - 1) * NB + blk) * 16 + z];
  }
  double* C = Cout + (size_t)s * k * k;
  if (grp == 0) {
#pragma unroll
    for (int q = 0; q < kMaxBlk; ++q) {
      if (bi[q] < 0) continue;
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c) {
          const int i = 4 * bi[q] + a, j = 4 * bj[q] + c;
          if (i < k && j < k) {
            C[i + (size_t)k * j] = acc[q][4 * a + c];
            C[j + (size_t)k * i] = acc[q][4 * a + c];
          }
        }
    }
  }
  if (tid < k) tout[(size_t)s * k + tid] = tacc;
  if (b.work && tid == 0) atomicAdd(b.work, (unsigned long long)nproc);
}

void launch_gram64(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                   const double* axb, double* C, double* t, cudaStream_t stream) {
  if (b.nsolves == 0) return;
  const int kp = (g.ens + 3) & ~3;
  const int nb = kp / 4;
  const int NB = nb * (nb + 1) / 2;
  const size_t tile = sizeof(double) * (kTE * kp + kTE);
  if (NB <= kGramThreads) {
    const int G = std::max(1, kGramThreads / NB);
    const size_t red = sizeof(double) * (size_t)(G - 1) * NB * 16;
    const size_t smem = std::max(tile, red);
    cudaFuncSetAttribute(gram64_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    gram64_kernel<1><<<b.nsolves, kGramThreads, smem, stream>>>(g, hx, l, b, axb, C, t);
  } else {
    gram64_kernel<3><<<b.nsolves, kGramThreads, tile, stream>>>(g, hx, l, b, axb, C, t);
  }
}

}  // namespace lg
