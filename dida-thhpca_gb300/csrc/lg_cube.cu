// lg_cube.cu -- application of cube solves to the columns they cover.
//
// With da_block_interval cube_n > 1 (and da_vertical_interval cube_nz on the
// vertical path) the reference solves letkf_core once per cube of
// cube_n x cube_n columns of a block (and level group), from the list of the
// cube's centre grid point, and applies that trans to every column (and level)
// of the cube: letkf_compute_nooverlap (letkf_compute.F90:12-154, xb_2_xa
// :259-329), letkf_compute_nooverlap_vertical (:386-554).  With
// da_block_overlap > 0 the cubes step by cube_n - overlap and each column's
// analysis is the average over the cubes covering it (letkf_compute :156-256,
// xb_add2_xa :332-382).  The solves' trans (k x k, column-major: trans(i, e))
// are computed beforehand; this kernel forms, per column and row,
//   dist(e) = axb + sum_i xb(i) trans(i, e),   mean over e,   xa = dist - mean,
// accumulated over the covering cubes and divided by their number.
#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

namespace {

// block (0-based) of a global grid point: pro_info_get_indx inverted (the first
// res blocks hold sec + 1 points, the others sec)
__device__ inline int block_of(int p, int npts, int nblk) {
  const int sec = npts / nblk, res = npts % nblk;
  const int big = res * (sec + 1);
  return p <= big ? (p - 1) / (sec + 1) : res + (p - 1 - big) / sec;
}

// first cube (0-based) along one axis whose span [1 + m st, m st + cn] holds p
__device__ inline int first_cube(int p, int cn, int st) { return p > cn ? (p - cn + st - 1) / st : 0; }

template <int NT>
__global__ void __launch_bounds__(NT) cube_apply_kernel(Geometry g, CubeDev cd, const double* trans,
                                                        const double* xb, const double* axb,
                                                        double* xa, double* axa) {
  const int col = blockIdx.x;
  const int k = g.ens, n = g.n, LDT = k + 1;  // odd stride: conflict-free staging and reads
  const int tid = threadIdx.x;
  extern __shared__ double sm[];
  double* Tt = sm;            // Tt[e + LDT i] = trans(i, e)
  double* xs = Tt + k * LDT;  // k
  double* red = xs + k;       // NT / 32
  const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
  const int bx = block_of(glat, g.num_lat, g.global_nx), by = block_of(glon, g.num_lon, g.global_ny);
  const int b = by * g.global_nx + bx;
  const int4 bk = g.blk[b];  // s_lat, e_lat, s_lon, e_lon (1-based)
  const int nxl = bk.y - bk.x + 1;
  const int j = glat - bk.x + 1, i = glon - bk.z + 1;
  const int st = cd.stride, cn = cd.cube_n;
  const int ncj = (nxl - 1) / st + 1;
  const int mj0 = first_cube(j, cn, st), mj1 = (j - 1) / st;
  const int mi0 = first_cube(i, cn, st), mi1 = (i - 1) / st;
  const int count = (mj1 - mj0 + 1) * (mi1 - mi0 + 1);
  const size_t ci = (size_t)(glat - 1 + g.halo) +
                    (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
  auto block_sum = [&](double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    return s;
  };
  auto apply_row = [&](int r, bool first) {
    const double* xr = xb + (size_t)k * (r + (size_t)n * ci);
    __syncthreads();
    if (tid < k) xs[tid] = xr[tid];
    __syncthreads();
    double val = 0.0;
    if (tid < k) {
      double sum = 0.0;
      for (int q = 0; q < k; ++q) sum += xs[q] * Tt[tid + LDT * q];
      val = axb[r + (size_t)n * ci] + sum;
    }
    const double mean = block_sum(val) / (double)k;
    double* xo = xa + (size_t)k * (r + (size_t)n * ci);
    if (tid < k) xo[tid] = first ? val - mean : xo[tid] + (val - mean);
    if (tid == 0) axa[r + (size_t)n * ci] = first ? mean : axa[r + (size_t)n * ci] + mean;
  };
  bool first = true;
  for (int mi = mi0; mi <= mi1; ++mi)
    for (int mj = mj0; mj <= mj1; ++mj) {
      const int cube = cd.cube_off[b] + mi * ncj + mj;
      for (int gi = 0; gi < cd.ngroups; ++gi) {
        const double* T = trans + ((size_t)cube * cd.ngroups + gi) * k * k;
        __syncthreads();
        for (int idx = tid; idx < k * k; idx += NT) Tt[idx / k + LDT * (idx % k)] = T[idx];
        __syncthreads();
        if (!cd.grouped) {
          for (int r = 0; r < n; ++r) apply_row(r, first);
          continue;
        }
        // rows of levels sk..ek of the 3-D variables; the 2-D ones with the last group
        const int sk = gi * cd.cube_nz + 1, ek = min(sk + cd.cube_nz - 1, g.nz);
        for (int v = 0; v < g.n_var; ++v) {
          if (g.var_lev[v] == 1) {
            if (ek == g.nz) apply_row(g.var_start[v], first);
          } else {
            for (int kk = sk; kk <= ek; ++kk) apply_row(g.var_start[v] + kk - 1, first);
          }
        }
      }
      first = false;
    }
  if (count > 1) {
    __syncthreads();
    for (int r = 0; r < n; ++r) {
      double* xo = xa + (size_t)k * (r + (size_t)n * ci);
      if (tid < k) xo[tid] = xo[tid] / (double)count;
      if (tid == 0) axa[r + (size_t)n * ci] = axa[r + (size_t)n * ci] / (double)count;
    }
  }
}

}  // namespace

void launch_cube_apply(const Geometry& g, const CubeDev& cd, const double* trans,
                       const double* xb, const double* axb, double* xa, double* axa,
                       cudaStream_t stream) {
  const int ncol = g.num_lat * g.num_lon;
  const int k = g.ens;
  const size_t smem = sizeof(double) * ((size_t)k * (k + 1) + k + 4);
  if (k <= 64) {
    cudaFuncSetAttribute(cube_apply_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cube_apply_kernel<64><<<ncol, 64, smem, stream>>>(g, cd, trans, xb, axb, xa, axa);
  } else {
    cudaFuncSetAttribute(cube_apply_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cube_apply_kernel<128><<<ncol, 128, smem, stream>>>(g, cd, trans, xb, axb, xa, axa);
  }
}

}  // namespace lg
