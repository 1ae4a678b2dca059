// lg_search.cu -- per-column local observation selection.
//
// Restates gen_yb_dis / gen_yb_dis_vertical's selection
// (x86/DA/LETKF/src/letkf_yb.F90:75-146,176-234): for the column centre
// (grid_lat(j), grid_lon(i)), visit the neighbour blocks of the column's block
// in comm_info_init order, then observation types, then the block's
// observations in index order; keep an observation when its Gaspari-Cohn (or
// box) weight of ri = dist/local_dist is positive, i.e. ri <= 2, and append all
// of its (level, variable) entries; stop at MAX_OBS entries.
//
// One warp per column, 32 candidates per step.  The decision is made in FP32
// on the cosine of the angular distance when it is farther than 1e-5 from the
// threshold cos(2L/a), and otherwise by the exact FP64 formula of
// latlon_dist_r8 (pro_info.F90:149-161) evaluated without contraction, so the
// kept set and its order equal the reference's.  Two passes: count, then fill
// at the prefix-summed offsets.
#include <cuda/std/functional>
#include <cub/device/device_scan.cuh>

#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

struct SearchArgs {
  float vlo, vhi;  // FP32 cosine band around the threshold
};

__global__ void __launch_bounds__(256) search_kernel(Geometry g, ObsDev ob, ListDev l, int fill,
                                                     SearchArgs sa, unsigned long long* band) {
  const int idx = blockIdx.x * (blockDim.x / 32) + (threadIdx.x / 32);
  const int ncol = g.num_lat * g.num_lon;
  if (idx >= (l.col_list ? l.n_list : ncol)) return;
  const int col = l.col_list ? l.col_list[idx] : idx;
  const unsigned lane = threadIdx.x & 31u;
  const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
  const int b = g.lon_block[glon - 1] * g.global_nx + g.lat_block[glat - 1];
  // column centre (letkf_yb.F90:23-24), REAL(4) grid promoted to REAL(8)
  const double clat = (double)g.glat[glat - 1], clon = (double)g.glon[glon - 1];
  const double ccx = cos(deg2rad_r8(clat)), csx = sin(deg2rad_r8(clat));
  const double cyr = deg2rad_r8(clon);
  const float pf = 3.14159274101257324f;
  const float fcx = cosf((float)clat / 180.0f * pf), fsx = sinf((float)clat / 180.0f * pf);
  const float fyr = (float)clon / 180.0f * pf;
  const int T = g.n_types;
  const int cap = g.max_obs > 0 ? g.max_obs : 0x7fffffff;
  int64_t written = 0;  // entries appended so far (uncapped count)
  const int64_t out0 = fill ? l.off[col] : 0;
  unsigned long long nband = 0;
  bool done = false;
  for (int q = g.nb_off[b]; q < g.nb_off[b + 1] && !done; ++q) {
    const int nbk = g.nb_blk[q];
    for (int t = 0; t < T && !done; ++t) {
      const int j0 = ob.bt_off[nbk * T + t], j1 = ob.bt_off[nbk * T + t + 1];
      for (int jb = j0; jb < j1 && !done; jb += 32) {
        const int j = jb + (int)lane;
        bool keep = false;
        double ri = 0.0;
        int nent = 0;
        if (j < j1) {
          const int o = ob.copy_obs[j];
          if (fabs(ob.olat[o]) <= g.obs_polar) {
            const float v32 = ob.fcx[o] * fcx * cosf(ob.fyr[o] - fyr) + ob.fsx[o] * fsx;
            const bool in_band = v32 <= sa.vhi && v32 >= sa.vlo;
            // the keep decision is identical in both passes; the fill pass also
            // evaluates ri exactly for every kept copy to obtain its weight
            if (in_band || (fill && v32 > sa.vhi)) {
              double dist = latlon_dist_pre(ob.dcx[o], ob.dsx[o], ob.dyr[o], ccx, csx, cyr);
              ri = __ddiv_rn(__dmul_rn(dist, 1.0), g.local_dist);
            }
            if (in_band) {
              keep = loc_fn(ri, g.gc_filter) > 0.0;
              if (!fill && fabs(ri - 2.0) < 1e-12) nband++;
            } else {
              keep = v32 > sa.vhi;
            }
            if (keep) nent = ob.copy_eoff[j + 1] - ob.copy_eoff[j];
          }
        }
        // inclusive warp prefix of entry counts
        int incl = nent;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
          int v = __shfl_up_sync(0xffffffffu, incl, s);
          if ((int)lane >= s) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (fill && keep) {
          const double gc = (ri <= 2.0) ? loc_fn(ri, g.gc_filter) : 0.0;
          const int64_t pos0 = written + incl - nent;
          const int e0 = ob.copy_eoff[j];
          for (int m = 0; m < nent; ++m) {
            const int64_t pos = pos0 + m;
            if (pos < cap) {
              l.ent[out0 + pos] = e0 + m;
              l.rloc[out0 + pos] = gc;
            }
          }
        }
        written += total;
        if (written >= cap) done = true;
      }
    }
  }
  if (!fill && lane == 0) {
    l.cnt[col] = (int)(written < cap ? written : cap);
    if (l.capped) l.capped[col] = written >= cap;
    if (l.col_stats) {
      atomicMax(&l.col_stats[0], (int)(written < cap ? written : cap));
      if (written >= cap) atomicAdd(&l.col_stats[1], 1);
    }
  }
  if (!fill && band) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) nband += __shfl_down_sync(0xffffffffu, nband, s);
    if (lane == 0 && nband) atomicAdd(band, nband);
  }
}

void launch_search(const Geometry& g, const ObsDev& o, ListDev l, int fill,
                   unsigned long long* band, cudaStream_t stream) {
  const int ncol = g.num_lat * g.num_lon;
  // cos(2L/a): ri <= 2  <=>  acos(v) <= 2L/a
  const double th = 2.0 * g.local_dist / earth_r4();
  SearchArgs sa;
  if (th >= 3.14159) {
    sa.vlo = -3.0f;
    sa.vhi = -2.0f;  // everything within reach: every candidate is exact-checked (fill) or kept
  } else {
    const double v = cos(th);
    sa.vlo = (float)(v - 1e-5);
    sa.vhi = (float)(v + 1e-5);
  }
  const int warps = 8;
  const int nc = l.col_list ? l.n_list : ncol;
  if (nc == 0) return;
  search_kernel<<<(nc + warps - 1) / warps, 32 * warps, 0, stream>>>(g, o, l, fill, sa, band);
}

// The scan accumulates in 64 bits: ExclusiveSum would add the int counts in
// int (its accumulator is the input's value type), and a list of more than
// 2^31 entries (a large globe, or a window of one) would wrap.  An int64_t
// initial value makes the accumulator int64_t.
size_t scan_tmp_bytes(int n) {
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveScan(nullptr, bytes, (const int*)nullptr, (int64_t*)nullptr,
                                 ::cuda::std::plus<int64_t>{}, (int64_t)0, n + 1);
  return bytes;
}

// off[i] = sum_{c<i} cnt[c] for i = 0..n (cnt[n] is read as the scan's
// extra element, so the caller keeps cnt sized n+1 with cnt[n] = 0)
void launch_scan_counts(const int* cnt, int64_t* off, int n, void* tmp, size_t tmp_bytes,
                        cudaStream_t stream) {
  cub::DeviceScan::ExclusiveScan(tmp, tmp_bytes, cnt, off, ::cuda::std::plus<int64_t>{},
                                 (int64_t)0, n + 1, stream);
}

}  // namespace lg

namespace lg {

// Per-column entry records for the mixed-precision Gram, grouped by ln p bucket.
//
// For every column the list entries are copied, in a stable counting sort by
// bucket(ln p) = floor((ln p - lo) / dz), into (entry, ln p, rdiaginv * rloc)
// records; boff[col * (nb + 1) + b] is the first record of bucket b.  A level's
// non-zero vertical weights (|ln p_k - ln p| <= 2 vert_dist) then lie in a
// contiguous bucket range, so each solve scans only its window instead of the
// whole list.  One warp per column; the ranking inside a bucket uses the lane
// order, so the layout is deterministic.
__global__ void __launch_bounds__(128) records_kernel(int col0, int ncol, ListDev l, HxDev hx,
                                                      float lo, float inv_dz, int nb, int* boff,
                                                      float4* rec) {
  const int warps = blockDim.x / 32;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int idx = blockIdx.x * warps + w;
  extern __shared__ int cur_all[];
  int* cur = cur_all + w * (nb + 1);
  if (idx >= ncol) return;
  const int col = col0 + idx;
  for (int b = lane; b <= nb; b += 32) cur[b] = 0;
  __syncwarp();
  const int64_t base = l.off[col];
  const int p = l.cnt[col];
  // FP64 -> FP32 by integer operations (d2f_bits: round to nearest even, as the
  // conversion instruction, which issues on the FP64 pipe; magnitudes below
  // 2^-126 become zero): four conversions per list entry
  auto bucket = [&](int ent) {
    int b = (int)floorf((d2f_bits(hx.lnp[ent]) - lo) * inv_dz);
    return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
  };
  // histogram
  for (int i0 = 0; i0 < p; i0 += 32) {
    const int i = i0 + lane;
    if (i < p) atomicAdd(&cur[bucket(l.ent[base + i]) + 1], 1);
  }
  __syncwarp();
  // cur[b] <- first record of bucket b (the scan of the shifted counts): each
  // lane scans a run of consecutive buckets from the total of the runs before
  // it, which a shuffle scan over the warp provides
  {
    const int run = (nb + 32) / 32;  // ceil((nb + 1) / 32)
    const int b0 = min(nb + 1, lane * run), b1 = min(nb + 1, b0 + run);
    int sum = 0;
    for (int b = b0; b < b1; ++b) sum += cur[b];
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    int acc = incl - sum;
    for (int b = b0; b < b1; ++b) {
      acc += cur[b];
      cur[b] = acc;
    }
  }
  __syncwarp();
  for (int b = lane; b <= nb; b += 32) boff[(size_t)col * (nb + 1) + b] = cur[b];
  __syncwarp();
  // stable scatter
  const unsigned lt = (1u << lane) - 1u;
  for (int i0 = 0; i0 < p; i0 += 32) {
    const int i = i0 + lane;
    const bool ok = i < p;
    int ent = 0, b = nb;  // nb: out-of-range marker for inactive lanes
    if (ok) {
      ent = l.ent[base + i];
      b = bucket(ent);
    }
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(same & lt);
    const int start = cur[b];
    __syncwarp();
    if (ok) {
      const int64_t pos = base + start + rank;
      rec[pos] = make_float4(__int_as_float(ent), d2f_bits(hx.lnp[ent]),
                             hx.rdiag[ent] * d2f_bits(l.rloc[base + i]), d2f_bits(hx.dis[ent]));
    }
    if (ok && rank == 0) cur[b] = start + __popc(same);
    __syncwarp();
  }
}

void launch_records(int col0, int ncol, const ListDev& l, const HxDev& hx, float lo,
                    float inv_dz, int nb, int* boff, float4* rec, cudaStream_t stream) {
  if (ncol <= 0) return;
  const int warps = 4;
  const size_t smem = sizeof(int) * warps * (nb + 1);
  records_kernel<<<(ncol + warps - 1) / warps, 32 * warps, smem, stream>>>(
      col0, ncol, l, hx, lo, inv_dz, nb, boff, rec);
}

}  // namespace lg

namespace lg {

// Cell-indexed selection.  Same decisions and output order as search_kernel;
// candidates come from the cells of each (block, type) segment that overlap
// the column's spherical cap of radius 2L (plus a margin), instead of from the
// whole segment.  The fill pass marks kept copies in a bitmap over the
// segment's positions (observation-index order) and then emits them in that
// order.
__device__ inline bool keep_copy(const Geometry& g, const ObsDev& ob, int j, float fcx, float fsx,
                                 float fyr, double ccx, double csx, double cyr,
                                 const SearchArgs& sa, bool want_ri, double* ri_out,
                                 unsigned long long* nband) {
  const int o = ob.copy_obs[j];
  if (!(fabs(ob.olat[o]) <= g.obs_polar)) return false;
  const float v32 = ob.fcx[o] * fcx * cosf(ob.fyr[o] - fyr) + ob.fsx[o] * fsx;
  const bool in_band = v32 <= sa.vhi && v32 >= sa.vlo;
  double ri = 0.0;
  if (in_band || (want_ri && v32 > sa.vhi)) {
    const double dist = latlon_dist_pre(ob.dcx[o], ob.dsx[o], ob.dyr[o], ccx, csx, cyr);
    ri = __ddiv_rn(__dmul_rn(dist, 1.0), g.local_dist);
  }
  bool keep;
  if (in_band) {
    keep = loc_fn(ri, g.gc_filter) > 0.0;
    if (nband && fabs(ri - 2.0) < 1e-12) (*nband)++;
  } else {
    keep = v32 > sa.vhi;
  }
  if (ri_out) *ri_out = ri;
  return keep;
}

// position of the n-th (0-based) set bit of w, by halving the window
__device__ inline int nth_set_bit(unsigned w, int n) {
  int pos = 0;
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) {
    const unsigned low = w & ((1u << sh) - 1u);
    const int c = __popc(low);
    if (n >= c) {
      n -= c;
      w >>= sh;
      pos += sh;
    } else {
      w = low;
    }
  }
  return pos;
}

// Gaspari-Cohn in FP32 for the mixed path's weights (the polynomial of schr2)
__device__ inline float schr2_f32(float ri) {
  if (ri > 2.0f) return 0.0f;
  if (ri > 1.0f) {
    float rj = ri * (1.0f / 12.0f) - 0.5f;
    rj = rj * ri + 0.625f;
    rj = rj * ri + 1.666667f;
    return (rj * ri - 5.0f) * ri + 4.0f - 0.6666667f / ri;
  }
  if (ri > 0.0f) {
    const float rk = ri * ri;
    const float rj = (-0.25f * ri + 0.5f) * ri + 0.625f;
    return (rj * ri - 1.666667f) * rk + 1.0f;
  }
  return 1.0f;
}

// cos of a longitude difference x in (-3 pi, 3 pi) radians for the FP32
// prefilter: x reduced to [-pi, pi] by the nearest multiple of the FP32 2 pi
// (error below 3e-7 for these x), then the hardware approximation __cosf
// (absolute error 2^-21.41 on [-pi, pi], CUDA Programming Guide, intrinsic
// functions).  The prefilter decides only candidates whose FP32 cosine of the
// angular distance is more than 1e-5 from the threshold's (the band between
// SearchArgs::vlo and vhi goes to the exact FP64 test), and this cosine and
// the FP32 products around it are off by less than 1e-6, so every decision is
// the exact test's.
__device__ inline float cos_prefilter(float x) {
  const float k2pi = 6.28318530717958648f;
  const float r = x - k2pi * rintf(x * (1.0f / k2pi));
  return __cosf(r);
}

__global__ void __launch_bounds__(128) search_cells_kernel(Geometry g, ObsDev ob, CellIndex ci,
                                                           ListDev l, int fill, SearchArgs sa,
                                                           unsigned long long* band,
                                                           const int* skip) {
  if (skip && *skip) return;
  const int warps = blockDim.x / 32;
  const int w = threadIdx.x >> 5;
  const int idx = blockIdx.x * warps + w;
  const int ncol = g.num_lat * g.num_lon;
  extern __shared__ unsigned int bitmap_all[];
  unsigned int* bitmap = bitmap_all + (size_t)w * ci.bitmap_words;
  if (idx >= (l.col_list ? l.n_list : ncol)) return;
  const int col = l.col_list ? l.col_list[idx] : idx;
  const unsigned lane = threadIdx.x & 31u;
  const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
  const int b = g.lon_block[glon - 1] * g.global_nx + g.lat_block[glat - 1];
  const double clat = (double)g.glat[glat - 1], clon = (double)g.glon[glon - 1];
  const double ccx = cos(deg2rad_r8(clat)), csx = sin(deg2rad_r8(clat));
  const double cyr = deg2rad_r8(clon);
  const float pf = 3.14159274101257324f;
  const float fcx = cosf((float)clat / 180.0f * pf), fsx = sinf((float)clat / 180.0f * pf);
  const float fyr = (float)clon / 180.0f * pf;
  // cap of angular radius theta (degrees) around the centre, in cell units
  const float theta = ci.cap_deg;
  const int r_lo = max(0, (int)floorf(((float)clat - theta + 90.0f) * ci.inv_cell));
  const int r_hi = min(ci.nrows - 1, (int)floorf(((float)clat + theta + 90.0f) * ci.inv_cell));
  float dlon = 180.0f;
  if (fabsf((float)clat) + theta < 89.0f) {
    const float sr = sinf(theta * (pf / 180.0f)) / cosf((float)clat * (pf / 180.0f));
    if (sr < 1.0f) dlon = asinf(sr) * (180.0f / pf) * 1.001f + ci.cell_deg;
  }
  // longitude window [clon - dlon, clon + dlon] in degrees, split at 0/360 into
  // at most two pieces of cell columns
  const float w0 = (float)clon - dlon, w1 = (float)clon + dlon;
  auto cidx = [&](float lon) {
    const int c = (int)floorf(lon * ci.inv_cell);
    return c < 0 ? 0 : (c > ci.ncols - 1 ? ci.ncols - 1 : c);
  };
  int pa0, pa1, pb0 = 1, pb1 = 0;
  if (dlon >= 180.0f || w1 - w0 >= 360.0f) {
    pa0 = 0;
    pa1 = ci.ncols - 1;
  } else if (w0 < 0.0f) {
    pa0 = cidx(w0 + 360.0f); pa1 = ci.ncols - 1; pb0 = 0; pb1 = cidx(w1);
  } else if (w1 >= 360.0f) {
    pa0 = cidx(w0); pa1 = ci.ncols - 1; pb0 = 0; pb1 = cidx(w1 - 360.0f);
  } else {
    pa0 = cidx(w0); pa1 = cidx(w1);
  }
  const int T = g.n_types;
  const int cap = g.max_obs > 0 ? g.max_obs : 0x7fffffff;
  const bool exact_rloc = ci.exact_rloc;
  int64_t written = 0;
  const int64_t out0 = fill ? l.off[col] : 0;
  unsigned long long nband = 0;
  bool done = false;
  for (int q = g.nb_off[b]; q < g.nb_off[b + 1] && !done; ++q) {
    const int nbk = g.nb_blk[q];
    for (int t = 0; t < T && !done; ++t) {
      const int seg = nbk * T + t;
      const int j0 = ob.bt_off[seg], len = ob.bt_off[seg + 1] - j0;
      if (len == 0) continue;
      const int nent = ob.copy_eoff[j0 + 1] - ob.copy_eoff[j0];  // same type in a segment
      const int4 box = ci.box[seg];                                // row0, nrows, col0, ncols
      const int* cs = ci.cell_start + ci.cell_off[seg];
      const int* perm = ci.perm + j0;
      const float4* cand = ci.cand + j0;
      if (fill)
        for (int wd = lane; wd < (len + 31) / 32; wd += 32) bitmap[wd] = 0u;
      __syncwarp();
      int64_t seg_count = 0;
      const int rr0 = max(r_lo, box.x), rr1 = min(r_hi, box.x + box.y - 1);
      for (int r = rr0; r <= rr1; ++r) {
        for (int piece = 0; piece < 2; ++piece) {
          const int p0 = piece == 0 ? pa0 : pb0, p1 = piece == 0 ? pa1 : pb1;
          const int cc0 = max(p0, box.z), cc1 = min(p1, box.z + box.w - 1);
          if (cc0 > cc1) continue;
          const int rowb = (r - box.x) * box.w;
          const int i0 = cs[rowb + (cc0 - box.z)], i1 = cs[rowb + (cc1 - box.z) + 1];
          for (int ib = i0; ib < i1; ib += 32) {
            const int i = ib + (int)lane;
            bool keep = false;
            int pos = 0;
            if (i < i1) {
              pos = perm[i];
              const float4 cd = cand[i];
              if (cd.w != 0.0f) {  // within obs_polar
                const float v32 = cd.x * fcx * cos_prefilter(cd.z - fyr) + cd.y * fsx;
                if (v32 > sa.vhi) {
                  keep = true;
                } else if (v32 >= sa.vlo) {  // in the band: the exact FP64 test
                  keep = keep_copy(g, ob, j0 + pos, fcx, fsx, fyr, ccx, csx, cyr, sa, false,
                                   nullptr, fill ? nullptr : &nband);
                }
              }
            }
            if (fill) {
              if (keep) atomicOr(&bitmap[pos >> 5], 1u << (pos & 31));
            } else {
              seg_count += __popc(__ballot_sync(0xffffffffu, keep));
            }
          }
        }
      }
      if (!fill) {
        written += seg_count * nent;
        if (written >= cap) done = true;
        continue;
      }
      __syncwarp();
      // Emit the kept copies of this segment in position (observation-index)
      // order, 32 bitmap words at a time.  The kept copies of the block are
      // dealt one per lane (copy t of the block to lane t mod 32) rather than
      // word by word, so that every lane evaluates a weight: the weights are
      // FP64 work and the words hold very different numbers of kept copies.
      const int words = (len + 31) / 32;
      for (int wb = 0; wb < words && !done; wb += 32) {
        const int wd = wb + (int)lane;
        const unsigned int bits = wd < words ? bitmap[wd] : 0u;
        int incl = __popc(bits);  // kept copies up to and including this lane's word
#pragma unroll
        for (int sft = 1; sft < 32; sft <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, sft);
          if ((int)lane >= sft) incl += v;
        }
        const int kept = __shfl_sync(0xffffffffu, incl, 31);
        for (int t0 = 0; t0 < kept; t0 += 32) {
          const int t = t0 + (int)lane;
          // word holding kept copy t: the first lane whose inclusive count exceeds t
          int wl = 0;
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const int v = __shfl_sync(0xffffffffu, incl, wl + step - 1);
            if (v <= t) wl += step;
          }
          const unsigned int wbits = __shfl_sync(0xffffffffu, bits, wl & 31);
          const int before = __shfl_sync(0xffffffffu, incl, wl & 31) - __popc(wbits);
          if (t >= kept) continue;
          const int bit = nth_set_bit(wbits, t - before);
          const int j = j0 + (wb + wl) * 32 + bit;
          const int o = ob.copy_obs[j];
          double gc;
          if (exact_rloc) {
            const double dist = latlon_dist_pre(ob.dcx[o], ob.dsx[o], ob.dyr[o], ccx, csx, cyr);
            const double ri = __ddiv_rn(__dmul_rn(dist, 1.0), g.local_dist);
            // a copy kept by the exact test has ri <= 2; clamp rounding beyond it
            gc = loc_fn(fmin(ri, 2.0), g.gc_filter);
          } else {  // mixed path: the weight only needs FP32 accuracy
            const float v32 = fminf(ob.fcx[o] * fcx * cosf(ob.fyr[o] - fyr) + ob.fsx[o] * fsx, 1.0f);
            const float ri = fminf(6371.393f * acosf(v32) / (float)g.local_dist, 2.0f);
            gc = f2d_bits(g.gc_filter ? schr2_f32(ri) : 1.0f);  // off the FP64 pipe
          }
          const int e0 = ob.copy_eoff[j];
          int64_t posw = written + (int64_t)t * nent;
          for (int m = 0; m < nent; ++m, ++posw) {
            if (posw < cap) {
              l.ent[out0 + posw] = e0 + m;
              l.rloc[out0 + posw] = gc;
            }
          }
        }
        written += (int64_t)kept * nent;
        if (written >= cap) done = true;
      }
      __syncwarp();
    }
  }
  if (!fill && lane == 0) {
    l.cnt[col] = (int)(written < cap ? written : cap);
    if (l.capped) l.capped[col] = written >= cap;
    if (l.col_stats) {
      atomicMax(&l.col_stats[0], (int)(written < cap ? written : cap));
      if (written >= cap) atomicAdd(&l.col_stats[1], 1);
    }
  }
  if (!fill && band) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) nband += __shfl_down_sync(0xffffffffu, nband, s);
    if (lane == 0 && nband) atomicAdd(band, nband);
  }
}

void launch_search_cells(const Geometry& g, const ObsDev& o, const CellIndex& ci, ListDev l,
                         int fill, unsigned long long* band, cudaStream_t stream,
                         const int* skip) {
  const int ncol = g.num_lat * g.num_lon;
  const double th = 2.0 * g.local_dist / earth_r4();
  SearchArgs sa;
  if (th >= 3.14159) {
    sa.vlo = -3.0f;
    sa.vhi = -2.0f;
  } else {
    const double v = cos(th);
    sa.vlo = (float)(v - 1e-5);
    sa.vhi = (float)(v + 1e-5);
  }
  const int warps = 4;
  const size_t smem = sizeof(unsigned int) * (size_t)warps * ci.bitmap_words;
  cudaFuncSetAttribute(search_cells_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  const int nc = l.col_list ? l.n_list : ncol;
  if (nc == 0) return;
  search_cells_kernel<<<(nc + warps - 1) / warps, 32 * warps, smem, stream>>>(g, o, ci, l, fill,
                                                                                 sa, band, skip);
}

__global__ void clear_selection_kernel(const int* fresh, int* cnt, int n, int* col_stats,
                                       unsigned long long* band) {
  if (*fresh) return;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) cnt[i] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    col_stats[0] = 0;
    col_stats[1] = 0;
    *band = 0ull;
  }
}

void launch_clear_selection(const int* fresh, int* cnt, int n, int* col_stats,
                            unsigned long long* band, cudaStream_t stream) {
  const int blocks = std::max(1, std::min((n + 255) / 256, 152 * 4));
  clear_selection_kernel<<<blocks, 256, 0, stream>>>(fresh, cnt, n, col_stats, band);
}

}  // namespace lg
