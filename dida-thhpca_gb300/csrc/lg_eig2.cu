// lg_eig2.cu -- FP64 eigensolve + transform for the analysis path, organised
// around the FP64 pipe of GB300.
//
// The FP64 pipe of this GPU retires about one warp instruction per 17 cycles per
// SM whatever the number of active lanes, so scalar FP64 code costs as much as
// full-warp code.  The solve (letkf_core.F90:98-225 + the update of
// letkf_compute.F90:501-552) is therefore split so that every FP64 instruction
// carries 32 useful lanes:
//
//   tridiag_kernel  one warp per matrix: Householder reduction C = Q T Q^T
//                   (tred2's reduction half, FP64), writes diag, off-diagonal and
//                   the reflectors (u_i, h_i).
//   ql_kernel       one LANE per matrix: implicit QL iteration with Wilkinson
//                   shifts on (d, e) -> eigenvalues; each Givens rotation
//                   (c, s, i) is appended to a per-matrix log instead of being
//                   accumulated into an eigenvector matrix.
//   vec_kernel      one LANE per (matrix, vector), FP64 (FP64 path) or FP32 (mixed
//                   path: the Xb.W contraction; eigenvalues, rotations and
//                   reflectors are still FP64 results): for t and every state row x the
//                   solve owns, y = Q^T x, then the logged rotations forward
//                   (y <- Z^T y); for t: overline_w-coefficients t_j / lambda_j;
//                   for rows: dot = sum_j y_j t_j / lambda_j  (= overline_w . x),
//                   y <- f(lambda) y, the rotations backward (Z y), then Q y
//                   = W x.  xa = axb + W x + dot, recentred, is written directly.
//
// W and V are never formed; the cost per matrix is the reduction (2k^3/3 FMA)
// plus O(k^2) per vector.  A matrix whose QL needs more rotations than the log
// holds, or (mixed path) whose reduction has an h beyond the FP32 reflector
// range, is flagged and redone in FP64 by eig_apply_kernel (lg_eig.cu).
#include <float.h>
#include <stdlib.h>

#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

namespace e2 {
__device__ inline size_t tri_stride(int n) { return (size_t)n * (n + 3); }  // D,E,H + U
__device__ inline size_t uoff(int i) { return (size_t)i * (i - 1) / 2; }   // row i of U (i >= 1)
}  // namespace e2

// ---------------------------------------------------------------- tridiag
// scratch layout per solve: D[n] | E[n] | H[n] | U[n(n-1)/2]
//
// The matrix is held as its packed lower triangle, row j at j(j+1)/2 (16.6 KB for
// 64 members, so 13 warps fit an SM).  The shared-memory access patterns below
// are free of bank conflicts within a half-warp -- consecutive elements of a
// row, the same column of consecutive rows j (offsets j(j+1)/2 + c, and
// j(j+1)/2 is a permutation modulo 16 over any 16 consecutive j), or a
// broadcast -- except the column runs of the split rows in the matrix-vector
// product, where a few conflicts cost less than idle FP64 lanes.  The kernel
// is bound by the FP64 pipe, so the instruction count is what is minimised: the
// reflector needs no pre-scaling unless the row's squared norm leaves
// [2^-900, 2^900], the matrix-vector product runs every lane over the same
// number of terms (no divergent split at the diagonal), and the rank-2 update
// is two fused multiply-adds per element.
__device__ inline int tri_idx(int j) { return j * (j + 1) / 2; }

// 1/x by the Newton-Raphson iteration r <- r + r (1 - x r) from the hardware
// approximation (PTX rcp.approx.ftz.f64); two steps reach full double
// precision for the reflector norms here (normal numbers, checked before).
__device__ inline double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// biased exponent of a double (0 for zero and subnormals, 2047 for inf/NaN)
__device__ inline int dexp(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }

// Scalar tests and exact scalings on the bit pattern, off the FP64 pipe:
// x == 0.0 (either sign); x >= 0.0 for a non-NaN x (-0 included); -x; x / 2
// for a normal x with biased exponent >= 2.
__device__ inline bool is_zero_bits(double x) {
  return ((__double2hiint(x) & 0x7fffffff) | __double2loint(x)) == 0;
}
__device__ inline bool nonneg_bits(double x) { return __double2hiint(x) >= 0 || is_zero_bits(x); }
__device__ inline double neg_bits(double x) {
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
__device__ inline double half_bits(double x) {
  return __hiloint2double(__double2hiint(x) - (1 << 20), __double2loint(x));
}
// 2 x for every double x, exactly as the FP64 pipe rounds it: a subnormal's
// magnitude bits shift left by one (carrying into the exponent where the
// result is normal), a normal's exponent goes up by one, the largest binade
// overflows to infinity, and zero, infinity and NaN stay as they are.
__device__ inline double twice_bits(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long sign = u & 0x8000000000000000ull;
  unsigned long long mag = u ^ sign;
  const unsigned e = (unsigned)(mag >> 52);
  if (e == 0u)
    mag <<= 1;
  else if (e < 2046u)
    mag += 1ull << 52;
  else if (e == 2046u)
    mag = 0x7ff0000000000000ull;
  return __longlong_as_double((long long)(sign | mag));
}

// Sum of one finite double per lane over the warp, on the integer pipe: each
// value is aligned at the warp's largest exponent into a signed 128-bit fixed
// point number (parts below 2^-64 of that exponent's unit truncated), the 32
// numbers are added exactly through a shuffle tree, and the total is rounded
// once to nearest-even.  The result is the correctly rounded sum when the
// exponents span at most 64 binades; otherwise its error is below 32 units of
// 2^-116 of the largest term's binade plus the final rounding -- far inside a
// tree of FP64 additions' bound (about 5 * 2^-53 of the largest term) -- and
// the FP64 pipe issues nothing.  Subnormal inputs count as zero.
//
// kWarp: the sum over the warp; otherwise over aligned groups of f lanes (f a
// power of two, the same in every lane), each group getting its own sum.  All
// 32 lanes run the same shuffles either way (no early return in the grouped
// form, where the groups' exponents differ).
template <bool kWarp>
__device__ inline double sum_exact(double v, int f) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  int emax;
  if constexpr (kWarp) {
    emax = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
    if (emax == 0) return 0.0;
  } else {
    emax = e;
    for (int o = f >> 1; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  unsigned long long hi = 0, lo = 0;
  if (e != 0) {
    const unsigned long long m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = emax - e;
    if (sh == 0) {
      hi = m;
    } else if (sh < 64) {
      hi = m >> sh;
      lo = m << (64 - sh);
    } else if (sh == 64) {
      lo = m;
    } else if (sh < 128) {
      lo = m >> (sh - 64);
    }
    if (b >> 63) {  // two's complement
      lo = ~lo + 1;
      hi = ~hi + (lo == 0 ? 1 : 0);
    }
  }
  auto add = [&](int o) {
    const unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    const unsigned long long ls = lo + l2;
    hi = hi + h2 + (ls < lo ? 1 : 0);
    lo = ls;
  };
  if constexpr (kWarp) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) add(o);
  } else {
    for (int o = f >> 1; o > 0; o >>= 1) add(o);
  }
  const bool neg = (long long)hi < 0;
  if (neg) {
    lo = ~lo + 1;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  int p;  // leading one
  if (hi) {
    p = 127 - __clzll((long long)hi);
  } else if (lo) {
    p = 63 - __clzll((long long)lo);
  } else {
    return 0.0;
  }
  unsigned long long mant, half = 0, sticky = 0;
  const int drop = p - 52;
  if (drop <= 0) {
    mant = lo << (-drop);
  } else {
    mant = drop >= 64 ? hi >> (drop - 64) : (hi << (64 - drop)) | (lo >> drop);
    const int rb = drop - 1;  // highest dropped bit
    if (rb >= 64) {
      half = (hi >> (rb - 64)) & 1;
      sticky = lo != 0 || (hi & ((1ull << (rb - 64)) - 1)) != 0;
    } else {
      half = (lo >> rb) & 1;
      sticky = rb > 0 && (lo & ((1ull << rb) - 1)) != 0;
    }
  }
  mant += (half && (sticky || (mant & 1))) ? 1 : 0;  // may carry into the exponent
  // 2^p in units of 2^(emax - 1139): biased exponent p + emax - 116
  const unsigned long long bits = ((unsigned long long)(p + emax - 116 - 1) << 52) + mant;
  const double r = __longlong_as_double((long long)bits);
  return neg ? neg_bits(r) : r;
}
__device__ inline double warp_sum_exact(double v) { return sum_exact<true>(v, 32); }
// the sum over this lane's aligned group of f lanes (f = 1, 2, 4, .., 32)
__device__ inline double group_sum_exact(double v, int f) { return sum_exact<false>(v, f); }

// u32 = 1 (mixed path): the reflectors are written in FP32 for the FP32 vector
// kernel, normalised as v = u / sqrt(h) (P = I - v v^T, |v|^2 = 2 whatever the
// size of h, so a rounding-level row of a low-rank matrix neither overflows nor
// underflows in FP32), at the start of the U region, followed by one float per
// step: 1 where the step has a reflector, 0 where it has none.  A matrix with
// an h outside [2^-200, 2^200] is marked by H[0] = 1 (the QL kernel passes it
// to the FP64 fallback solver); the double H is kept for reference.
__device__ inline float rsqrt_f32_of(double h) {
  // 1/sqrt(h) for a normal h in [2^-200, 2^200]: h = m 2^e2 with e2 even and m
  // in [1, 4) (exponent bits only), then rsqrtf(m) 2^(-e2/2)
  const int hb = __double2hiint(h);
  const int e2 = (((hb >> 20) & 0x7ff) - 1023) & ~1;
  const double m = __hiloint2double(hb - (e2 << 20), __double2loint(h));
  return rsqrtf(d2f_bits(m)) * __int_as_float((127 - e2 / 2) << 23);
}

__global__ void __launch_bounds__(32) tridiag_kernel(int n, int nsolves, const double* Cin,
                                                     double* tri, int u32) {
  const int s = blockIdx.x;
  if (s >= nsolves) return;
  const int lane = threadIdx.x;
  extern __shared__ double sm[];
  const int np = n * (n + 1) / 2;
  double* P = sm;      // packed lower triangle
  double* q = P + np;  // n
  const double* C = Cin + (size_t)s * n * n;
  {
    // element t of the packed triangle is (j, c) with t = j(j+1)/2 + c, c <= j
    int j = 0, c = lane;
    while (c > j) {
      c -= j + 1;
      ++j;
    }
    for (int t = lane; t < np; t += 32) {
      P[t] = C[(size_t)j * n + c];
      c += 32;
      while (c > j) {
        c -= j + 1;
        ++j;
      }
    }
  }
  double* out = tri + (size_t)s * e2::tri_stride(n);
  double* D = out;
  double* E = out + n;
  double* H = out + 2 * n;
  double* U = out + 3 * n;
  __syncwarp();
  auto wsum = [](double v) { return warp_sum_exact(v); };
  float* U32 = reinterpret_cast<float*>(U);
  float* Act32 = U32 + (size_t)n * (n - 1) / 2;
  bool extreme = false;  // some h outside the FP32 reflector range
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    double* row = P + tri_idx(i);  // u: row i, columns 0..l
    double h = 0.0, ei;
    if (l > 0) {
      double ss = 0.0;
      for (int c = lane; c <= l; c += 32) ss = fma(row[c], row[c], ss);
      double h0 = wsum(ss);
      double sc = 1.0;
      bool scaled = false;
      // outside [2^-900, 2^900] (checked on the exponent bits), and not zero
      const int eh = dexp(h0);
      if ((eh < 1023 - 900 || eh > 1023 + 900) && !is_zero_bits(h0)) {
        // extreme magnitudes: scale the row by its 1-norm first (as tred2 does)
        double a1 = 0.0;
        for (int c = lane; c <= l; c += 32) a1 += fabs(row[c]);
        sc = wsum(a1);
        scaled = true;
        const double inv = 1.0 / sc;
        ss = 0.0;
        for (int c = lane; c <= l; c += 32) {
          const double v = row[c] * inv;
          row[c] = v;
          ss = fma(v, v, ss);
        }
        h0 = wsum(ss);
        __syncwarp();
      }
      if (is_zero_bits(h0)) {
        ei = row[l];
      } else {
        const double f = row[l];
        const double sq = sqrt(h0);
        const double gg = nonneg_bits(f) ? neg_bits(sq) : sq;  // -sign(sqrt(h0), f)
        ei = scaled ? sc * gg : gg;
        h = h0 - f * gg;
        __syncwarp();
        if (lane == 0) row[l] = f - gg;
        __syncwarp();
        // p = A u / h over the R = l + 1 rows; element (j, c) is read from row j
        // for c <= j and from row c (column j) for c > j.  With R > 32, lanes
        // first take whole rows, one each, in rounds of 32 (rows 0 .. nfull - 1,
        // nfull the largest multiple of 32 below R).  The remaining r rows
        // (1..32) are split over groups of f lanes (f the largest power of two
        // with r f <= 32), each lane summing a run of ceil(R / f) columns, and
        // the group sums meet in exact fixed-point sums on the integer pipe:
        // the FP64 pipe then issues about R + ceil(R / f) instructions instead
        // of R per 32 rows.
        const double inv_h = rcp_nr(h);
        double fs = 0.0;
        const int R = l + 1;
        const int nfull = R > 32 ? ((R - 1) / 32) * 32 : 0;
        for (int j0 = 0; j0 < nfull; j0 += 32) {
          const int j = j0 + lane;
          const int tj = tri_idx(j);
          double gj = 0.0;
          int tc = 0;  // c(c+1)/2
          for (int c = 0; c < R; ++c) {
            const int off = (c <= j) ? tj + c : tc + j;
            gj = fma(P[off], row[c], gj);
            tc += c + 1;
          }
          const double pj = gj * inv_h;
          q[j] = pj;
          fs = fma(pj, row[j], fs);
        }
        {
          const int r = R - nfull;                     // 1..32
          const int lf = 31 - __clz(32 / r);           // f = 2^lf, r f <= 32
          const int f = 1 << lf;
          const int cl = (R + f - 1) >> lf;            // columns per lane
          const int ri = lane >> lf, pi = lane & (f - 1);
          const bool act = ri < r;
          const int j = nfull + (act ? ri : 0);
          const int c0 = act ? min(R, pi * cl) : 0;
          const int c1 = act ? min(R, c0 + cl) : 0;
          const int tj = tri_idx(j);
          double gj = 0.0;
          int tc = tri_idx(c0);
          for (int c = c0; c < c1; ++c) {
            const int off = (c <= j) ? tj + c : tc + j;
            gj = fma(P[off], row[c], gj);
            tc += c + 1;
          }
          if (f > 1) gj = group_sum_exact(gj, f);  // f is the same in every lane
          const double pj = gj * inv_h;
          if (act && pi == 0) {
            q[j] = pj;
            fs = fma(pj, row[j], fs);
          }
        }
        __syncwarp();  // q[j] of a split row was written by its group's first lane
        // h lies in [2^-901, 2^902] (h0 is range-checked or rescaled above and
        // h0 <= h <= 2 h0), so 1/h is normal and halving it is exact
        const double kq = wsum(fs) * half_bits(inv_h);
        for (int j = lane; j <= l; j += 32) q[j] = fma(-kq, row[j], q[j]);
        __syncwarp();
        // A -= u q^T + q u^T over the packed rows 0..l, lane t, t+32, ...
        {
          const int tot = tri_idx(l + 1);
          int j = 0, c = lane;
          while (c > j) {
            c -= j + 1;
            ++j;
          }
          for (int t = lane; t < tot; t += 32) {
            P[t] = fma(-row[j], q[c], fma(-q[j], row[c], P[t]));
            c += 32;
            while (c > j) {
              c -= j + 1;
              ++j;
            }
          }
        }
        __syncwarp();
      }
    } else {
      ei = row[l];
    }
    // reflector of step i: u = row i (scaled), h
    if (u32) {
      const int eh = dexp(h);
      const bool in_range = eh >= 1023 - 200 && eh <= 1023 + 200;
      extreme |= !is_zero_bits(h) && !in_range;
      const float sv = in_range ? rsqrt_f32_of(h) : 0.0f;
      for (int c = lane; c < i; c += 32) U32[e2::uoff(i) + c] = d2f_bits(row[c]) * sv;
      if (lane == 0) Act32[i] = in_range ? 1.0f : 0.0f;
    } else {
      for (int c = lane; c < i; c += 32) U[e2::uoff(i) + c] = row[c];
    }
    if (lane == 0) {
      H[i] = h;
      E[i] = ei;
    }
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) D[i] = P[tri_idx(i) + i];
  if (lane == 0) {
    H[0] = extreme ? 1.0 : 0.0;
    E[0] = 0.0;
    if (u32) Act32[0] = 0.0f;
  }
}

// Four warps per matrix, for 65..128 members.  With one warp per matrix the
// packed triangle (up to 66 KB) leaves room for three CTAs, i.e. three warps,
// per SM, and the FP64 pipe stays about a third busy (latency-bound); four
// warps per matrix give twelve.  Same outputs as tridiag_kernel.  Each step's
// scalars (square root, reflector norm, reciprocal) are computed once by
// thread 0 and broadcast through shared memory, since an FP64 instruction
// costs a full warp slot however few lanes it has; block sums are exact warp
// sums combined by thread 0; the matrix-vector product splits the step's R
// rows over groups of G lanes (G the largest power of two with R G <= 128,
// at most 32), so it issues about R^2 / 32 FP64 instructions.
constexpr int kTriWarps = 4;
__global__ void __launch_bounds__(32 * kTriWarps) tridiag_mw_kernel(int n, int nsolves,
                                                                   const double* Cin,
                                                                   double* tri, int u32) {
  constexpr int NT = 32 * kTriWarps;
  const int s = blockIdx.x;
  if (s >= nsolves) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  extern __shared__ double sm[];
  __shared__ double s_part[kTriWarps];
  __shared__ double s_res;
  __shared__ double s_sc[3];  // inv_h, h, e_i of the step
  const int np = n * (n + 1) / 2;
  double* P = sm;      // packed lower triangle
  double* q = P + np;  // n
  const double* C = Cin + (size_t)s * n * n;
  {
    int j = 0, c = tid;
    while (c > j) {
      c -= j + 1;
      ++j;
    }
    for (int t = tid; t < np; t += NT) {
      P[t] = C[(size_t)j * n + c];
      c += NT;
      while (c > j) {
        c -= j + 1;
        ++j;
      }
    }
  }
  __syncthreads();
  double* out = tri + (size_t)s * e2::tri_stride(n);
  double* D = out;
  double* E = out + n;
  double* H = out + 2 * n;
  double* U = out + 3 * n;
  float* U32 = reinterpret_cast<float*>(U);
  float* Act32 = U32 + (size_t)n * (n - 1) / 2;
  // sum of one value per thread over the block: exact per warp, the four warp
  // sums added by thread 0 in a fixed order; every thread gets the result
  auto block_sum = [&](double v) -> double {
    const double w = warp_sum_exact(v);
    if (lane == 0) s_part[warp] = w;
    __syncthreads();
    if (tid == 0) s_res = (s_part[0] + s_part[1]) + (s_part[2] + s_part[3]);
    __syncthreads();
    return s_res;
  };
  bool extreme = false;
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    double* row = P + tri_idx(i);
    double h = 0.0, ei;
    if (l > 0) {
      double ss = 0.0;
      for (int c = tid; c <= l; c += NT) ss = fma(row[c], row[c], ss);
      double h0 = block_sum(ss);
      double sc = 1.0;
      bool scaled = false;
      const int eh = dexp(h0);
      if ((eh < 1023 - 900 || eh > 1023 + 900) && !is_zero_bits(h0)) {
        double a1 = 0.0;
        for (int c = tid; c <= l; c += NT) a1 += fabs(row[c]);
        sc = block_sum(a1);
        scaled = true;
        const double inv = 1.0 / sc;
        ss = 0.0;
        for (int c = tid; c <= l; c += NT) {
          const double v = row[c] * inv;
          row[c] = v;
          ss = fma(v, v, ss);
        }
        h0 = block_sum(ss);
      }
      if (is_zero_bits(h0)) {
        ei = row[l];
      } else {
        if (tid == 0) {
          const double f = row[l];
          const double sq = sqrt(h0);
          const double gg = nonneg_bits(f) ? neg_bits(sq) : sq;  // -sign(sqrt(h0), f)
          s_sc[2] = scaled ? sc * gg : gg;
          const double hh = h0 - f * gg;
          s_sc[1] = hh;
          s_sc[0] = rcp_nr(hh);
          row[l] = f - gg;
        }
        __syncthreads();
        const double inv_h = s_sc[0];
        h = s_sc[1];
        ei = s_sc[2];
        // p = A u / h over the R = l + 1 rows, G lanes per row
        const int R = l + 1;
        int lf = 31 - __clz(NT / R);
        lf = lf > 5 ? 5 : lf;
        const int G = 1 << lf;
        const int cl = (R + G - 1) >> lf;  // columns per lane
        const int ri = tid >> lf, pi = tid & (G - 1);
        const bool act = ri < R;
        const int j = act ? ri : 0;
        const int c0 = act ? min(R, pi * cl) : 0;
        const int c1 = act ? min(R, c0 + cl) : 0;
        const int tj = tri_idx(j);
        double gj = 0.0;
        int tcc = tri_idx(c0);
        for (int c = c0; c < c1; ++c) {
          const int off = (c <= j) ? tj + c : tcc + j;
          gj = fma(P[off], row[c], gj);
          tcc += c + 1;
        }
        if (G > 1) gj = group_sum_exact(gj, G);  // G is the same in every lane
        double fs = 0.0;
        if (act && pi == 0) {
          const double pj = gj * inv_h;
          q[j] = pj;
          fs = pj * row[j];
        }
        // h lies in [2^-901, 2^902], so 1/h is normal and halving it is exact
        const double kq = block_sum(fs) * half_bits(inv_h);
        for (int jj = tid; jj <= l; jj += NT) q[jj] = fma(-kq, row[jj], q[jj]);
        __syncthreads();
        // A -= u q^T + q u^T over the packed rows 0..l
        {
          const int tot = tri_idx(l + 1);
          int jr = 0, c = tid;
          while (c > jr) {
            c -= jr + 1;
            ++jr;
          }
          for (int t = tid; t < tot; t += NT) {
            P[t] = fma(-row[jr], q[c], fma(-q[jr], row[c], P[t]));
            c += NT;
            while (c > jr) {
              c -= jr + 1;
              ++jr;
            }
          }
        }
        __syncthreads();
      }
    } else {
      ei = row[l];
    }
    // reflector of step i: u = row i (scaled), h
    if (u32) {
      const int eh = dexp(h);
      const bool in_range = eh >= 1023 - 200 && eh <= 1023 + 200;
      extreme |= !is_zero_bits(h) && !in_range;
      const float sv = in_range ? rsqrt_f32_of(h) : 0.0f;
      for (int c = tid; c < i; c += NT) U32[e2::uoff(i) + c] = d2f_bits(row[c]) * sv;
      if (tid == 0) Act32[i] = in_range ? 1.0f : 0.0f;
    } else {
      for (int c = tid; c < i; c += NT) U[e2::uoff(i) + c] = row[c];
    }
    if (tid == 0) {
      H[i] = h;
      E[i] = ei;
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += NT) D[i] = P[tri_idx(i) + i];
  if (tid == 0) {
    H[0] = extreme ? 1.0 : 0.0;
    E[0] = 0.0;
    if (u32) Act32[0] = 0.0f;
  }
}

// ---------------------------------------------------------------- QL
// lane-private arrays in shared memory are interleaved [index][lane]
template <typename LT>
__device__ inline LT make_rot(double c, double s);
template <>
__device__ inline double2 make_rot<double2>(double c, double s) { return make_double2(c, s); }
template <>
__device__ inline float2 make_rot<float2>(double c, double s) {
  return make_float2(d2f_bits(c), d2f_bits(s));  // not on the FP64 pipe
}

// LT: element type of the rotation log (double2 for the FP64 path, float2 when the
// rotations are only replayed in FP32 by the mixed-precision vector kernel)
template <typename LT>
__global__ void __launch_bounds__(256) ql_kernel(int n, int nsolves, double shift, double srho,
                                                 const double* tri, double* lam, LT* rot_cs,
                                                 unsigned char* rot_i, int* rot_n, int rot_cap,
                                                 int* overflow_list, int* overflow_n,
                                                 int* eig_fail, int max_iter) {
  const int warps = blockDim.x / 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int s = (blockIdx.x * warps + w) * 32 + lane;
  extern __shared__ double sm[];
  double* d = sm + (size_t)w * 64 * n;  // n x 32
  double* e = d + (size_t)32 * n;       // n x 32
#define DD(i) d[(i) * 32 + lane]
#define EE(i) e[(i) * 32 + lane]
  const bool live = s < nsolves;
  bool marked = false;  // an h outside the FP32 reflector range (mixed path): FP64 fallback
  if (live) {
    const double* T = tri + (size_t)s * e2::tri_stride(n);
    marked = T[2 * n] != 0.0;
    for (int i = 0; i < n; ++i) {
      DD(i) = T[i];
      EE(i) = (i + 1 < n) ? T[n + i + 1] : 0.0;  // e[i] = T(i, i+1)
    }
  }
  LT* cs_log = rot_cs + (size_t)(live ? s : 0) * rot_cap;
  unsigned char* i_log = rot_i + (size_t)(live ? s : 0) * rot_cap;
  // tql2's test |e_j| <= eps (|d_j| + |d_j+1|), with an integer pre-test on the
  // biased exponents: a normal e_j with exponent >= max(exp d_j, exp d_j+1) - 49
  // exceeds eps (|d_j| + |d_j+1|) < 2^-51 max(|d_j|, |d_j+1|), so the common
  // "not negligible" answer costs no FP64 instruction.
  auto bexp = [](double x) { return (__double2hiint(x) >> 20) & 0x7ff; };
  auto negligible = [&](int j) {
    const double ej = EE(j), a = DD(j), b = DD(j + 1);
    const int ee = bexp(ej);
    if (ee > 0 && ee + 49 >= max(bexp(a), bexp(b))) return false;
    return fabs(ej) <= DBL_EPSILON * (fabs(a) + fabs(b));
  };
  // The lanes of a warp run their QL sweeps in step: one sweep per pass of the
  // loop below, from the lane's first split m below l up to l, as in tql2.
  int l = 0, iter = 0, nrot = 0;
  bool fail = false, over = marked, done = !live || marked;
  while (true) {
    int m = n - 1;
    if (!done) {
      while (l < n - 1 && negligible(l)) {
        ++l;
        iter = 0;
      }
      if (l >= n - 1) {
        done = true;
      } else if (++iter > max_iter) {
        fail = true;
        done = true;
      } else {
        for (m = l + 1; m < n - 1; ++m)
          if (negligible(m)) break;
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (!done) {
      double g = (DD(l + 1) - DD(l)) / twice_bits(EE(l));
      double r = sqrt(g * g + 1.0);
      g = DD(m) - DD(l) + EE(l) / (g + (g >= 0.0 ? r : -r));
      double sn = 1.0, cn = 1.0, p = 0.0;
      bool early = false;
      // d[i + 1] of the next rotation is the d[i] this one reads (a rotation
      // writes only d[i + 1] and e[i + 1]): carried in a register, not reloaded
      double d_hi = DD(m);
      for (int i = m - 1; i >= l; --i) {
        const double ei = EE(i);
        const double d_lo = DD(i);
        const double f = sn * ei, b = cn * ei;
        const double q2 = f * f + g * g;
        // q2 == 0 on the bit pattern (off the FP64 pipe): a sum of squares is
        // never -0, and a NaN is not zero either way
        if ((__double2hiint(q2) | __double2loint(q2)) == 0) {
          EE(i + 1) = 0.0;
          DD(i + 1) = d_hi - p;
          EE(m) = 0.0;
          early = true;
          break;
        }
        // one reciprocal square root gives both r and 1/r
        const double rinv = rsqrt(q2);
        r = q2 * rinv;
        EE(i + 1) = r;
        sn = f * rinv;
        cn = g * rinv;
        g = d_hi - p;
        r = (d_lo - g) * sn + twice_bits(cn) * b;  // 2 cn off the FP64 pipe
        p = sn * r;
        DD(i + 1) = g + p;
        d_hi = d_lo;
        g = cn * r - b;
        if (nrot < rot_cap) {
          cs_log[nrot] = make_rot<LT>(cn, sn);
          i_log[nrot] = (unsigned char)i;
        } else {
          over = true;
        }
        ++nrot;
      }
      if (!early) {
        DD(l) -= p;
        EE(l) = g;
        EE(m) = 0.0;
      }
    }
  }
  if (!live) return;
  if constexpr (sizeof(LT) == sizeof(float2)) {
    // mixed path: the FP32 vector kernel's per-eigenvalue factors, computed once
    // here in FP64: 1/lambda_j and sqrt((k-1)/lambda_j) - sqrt(rho)
    float2* fl = reinterpret_cast<float2*>(lam + (size_t)s * n);
    const double km1 = (double)(n - 1);
    for (int i = 0; i < n; ++i) {
      const double li = DD(i) * 1.0 + shift;
      fl[i] = make_float2(d2f_bits(1.0 / li), d2f_bits(sqrt(km1 / li) - srho));
    }
  } else {
    for (int i = 0; i < n; ++i) lam[(size_t)s * n + i] = DD(i) * 1.0 + shift;
  }
  rot_n[s] = over ? -1 : nrot;
  if (fail) atomicAdd(eig_fail, 1);
  if (over) overflow_list[atomicAdd(overflow_n, 1)] = s;
#undef DD
#undef EE
}

// ---------------------------------------------------------------- vectors + update
// Streaming reads of the rotation log and the reflectors.  Both were written by
// an earlier launch and, at the full sizes, are no longer in L2 when the vector
// kernel reads them (a chunk's logs are about a gigabyte).  A lane replays its
// rotations one after another, each depending on the previous through the
// vector, so one load per rotation would leave the chain waiting on DRAM at
// every step.  The log is therefore read kRotBatch entries at a time, one batch
// ahead of the rotations that use it (the loads of a batch are independent and
// in flight together); every load asks L2 for the whole 256-byte segment
// around it, and a bulk prefetch every kAheadBatches batches brings the next
// window of entries into L2 (prefetch_log).  The reflector block of a solve is
// prefetched into L2 before each Householder pass and its step flags read once
// (load_step_mask).  The data are read-only for the kernel (non-coherent
// loads).
constexpr int kRotBatch = 8;

template <typename LT>
__device__ inline LT ld_stream(const LT* p);
template <>
__device__ inline float2 ld_stream<float2>(const float2* p) {
  float2 v;
  asm("ld.global.nc.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}
template <>
__device__ inline double2 ld_stream<double2>(const double2* p) {
  double2 v;
  asm("ld.global.nc.L2::256B.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}
template <>
__device__ inline float ld_stream<float>(const float* p) {
  float v;
  asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
template <>
__device__ inline double ld_stream<double>(const double* p) {
  double v;
  asm("ld.global.nc.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// One bulk prefetch into L2 of the 16-byte-aligned interior of [p, p + bytes)
// (a solve's reflector block, or a window of its rotation log).
__device__ inline void prefetch_l2(const void* p, size_t bytes) {
  const size_t a0 = __cvta_generic_to_global(p);
  const size_t a = (a0 + 15) & ~(size_t)15, e = (a0 + bytes) & ~(size_t)15;
  if (e > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a))
                 : "memory");
}

// Steps of the reduction that have a reflector (FP32 flags of the mixed path),
// read once as a bit mask for up to 128 members; the flag loads are
// independent, so they wait on memory once instead of once per step.
struct StepMask {
  unsigned long long lo = 0, hi = 0;
  __device__ bool has(int i) const { return ((i < 64 ? lo >> i : hi >> (i - 64)) & 1ull) != 0; }
};
__device__ inline StepMask load_step_mask(const float* act, int n) {
  StepMask m;
  for (int i = 1; i < n; ++i) {
    if (ld_stream(act + i) != 0.0f) {
      if (i < 64)
        m.lo |= 1ull << i;
      else
        m.hi |= 1ull << (i - 64);
    }
  }
  return m;
}

// Eight consecutive log entries 8b .. 8b + 7 (the log of a solve starts on a
// 64-byte boundary and its capacity is a multiple of 8, so these loads are
// aligned vector loads inside the solve's log; entries past the solve's count
// are read but never used).
template <typename LT>
struct RotBatch {
  LT cs[kRotBatch];
  uint2 ix;  // eight one-byte indices
  __device__ int idx(int j) const { return (int)(((j < 4 ? ix.x : ix.y) >> (8 * (j & 3))) & 0xffu); }
};

// The log entries of kAheadBatches batches, starting at batch b0 (clipped to
// the solve's nb batches), into L2 with one bulk prefetch each for the
// rotations and their indices: issued every kAheadBatches batches, a window
// ahead of the batch loads, so that those find the entries in L2.
constexpr int kAheadBatches = 32;  // 256 entries: 2 KB (FP32 log), 4 KB (FP64)
template <typename LT>
__device__ inline void prefetch_log(const LT* cs, const unsigned char* ix, int b0, int nb) {
  const int a = max(b0, 0), e = min(b0 + kAheadBatches, nb);
  if (e <= a) return;
  prefetch_l2(cs + (size_t)a * kRotBatch, sizeof(LT) * (size_t)(e - a) * kRotBatch);
  prefetch_l2(ix + (size_t)a * kRotBatch, (size_t)(e - a) * kRotBatch);
}

template <typename LT>
__device__ inline void load_rot_batch(RotBatch<LT>& rb, const LT* cs, const unsigned char* ix,
                                      int b) {
  const size_t r0 = (size_t)b * kRotBatch;
  if constexpr (sizeof(LT) == sizeof(float2)) {
    const float4* p = reinterpret_cast<const float4*>(cs + r0);
#pragma unroll
    for (int j = 0; j < kRotBatch / 2; ++j) {
      float4 v;
      asm("ld.global.nc.L2::256B.v4.f32 {%0, %1, %2, %3}, [%4];"
          : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
          : "l"(p + j));
      rb.cs[2 * j] = LT{v.x, v.y};
      rb.cs[2 * j + 1] = LT{v.z, v.w};
    }
  } else {
#pragma unroll
    for (int j = 0; j < kRotBatch; ++j) rb.cs[j] = ld_stream(cs + r0 + j);
  }
  asm("ld.global.nc.L2::256B.v2.u32 {%0, %1}, [%2];" : "=r"(rb.ix.x), "=r"(rb.ix.y) : "l"(ix + r0));
}

// lanes: solve-slot q = lane / per, vector v = lane % per (v = 0: t, v >= 1: row v-1)
// VT: arithmetic of the vector transforms (double: FP64 path; float: the mixed
// path's Xb.W contraction, with eigenvalues, rotations and reflectors from FP64)
template <typename VT, typename LT>
__global__ void __launch_bounds__(256) __maxnreg__(sizeof(VT) == sizeof(float) ? 72 : 128) vec_kernel(Geometry g, SolveBatch b, const double* tin,
                                                  const double* tri, const double* lam,
                                                  const LT* rot_cs,
                                                  const unsigned char* rot_i, const int* rot_n,
                                                  int rot_cap, const double* xb,
                                                  const double* axb, double* xa, double* axa) {
  constexpr bool kF32 = sizeof(VT) == sizeof(float);  // mixed path: FP32 reflectors and factors
  // FP32 <-> FP64 conversions of the mixed path by bit operations (off the FP64 pipe)
  auto to_vt = [](double x) -> VT {
    if constexpr (kF32) return d2f_bits(x); else return x;
  };
  auto to_d = [](VT x) -> double {
    if constexpr (kF32) return f2d_bits(x); else return x;
  };
  const int n = g.ens;
  const bool vertical = g.vert_dist > 0.0;
  const int nvec_max = 1 + (vertical ? g.n_var : g.n);
  const int per = nvec_max;
  const int slots = 32 / per;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int warps = blockDim.x / 32;
  const int q = lane / per, v = lane % per;
  const int s = (blockIdx.x * warps + w) * slots + q;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  VT* sm = reinterpret_cast<VT*>(sm_raw);
  VT* y = sm + (size_t)w * 32 * n;  // this warp's lane vectors, n x 32 interleaved
  // per-slot t_j / lambda_j, shared by the row lanes of the slot
  VT* tslot = sm + (size_t)warps * 32 * n + (size_t)w * slots * n;
#define YY(i) y[(i) * 32 + lane]
  // y <- y - u (u . y) / h over the first i entries (the FP32 reflectors are
  // normalised: no division)
  auto reflect = [&](const auto* u, int i, bool div, double h) {
    VT dot = 0;
    for (int kk = 0; kk < i; ++kk) dot += (VT)u[kk] * YY(kk);
    if (div) dot /= (VT)h;
    for (int kk = 0; kk < i; ++kk) YY(kk) -= (VT)u[kk] * dot;
  };
  const bool active = (lane < slots * per) && (s < b.nsolves);
  int r_state = -1;  // state row of this lane
  size_t ci = 0;
  int nrot = 0;
  const double* T = nullptr;
  const double* L = nullptr;
  if (active) {
    const int col = b.first_col + s / b.levels;
    const int kk = s % b.levels + 1;
    const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
    ci = (size_t)(glat - 1 + g.halo) + (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
    if (v >= 1) {
      if (vertical) {
        const int var = v - 1;
        if (g.var_lev[var] == 1) {
          if (kk == g.nz) r_state = g.var_start[var];
        } else {
          r_state = g.var_start[var] + kk - 1;
        }
      } else {
        r_state = v - 1;
      }
    }
    nrot = rot_n[s];
    T = tri + (size_t)s * e2::tri_stride(n);
    L = lam + (size_t)s * n;
  }
  const bool work = active && nrot >= 0 && (v == 0 || r_state >= 0);
  if (work) {
    // load x
    if (v == 0) {
      for (int i = 0; i < n; ++i) YY(i) = to_vt(tin[(size_t)s * n + i]);
    } else {
      const double* xr = xb + (size_t)n * (r_state + (size_t)g.n * ci);
      for (int i = 0; i < n; ++i) YY(i) = to_vt(xr[i]);
    }
    // y = Q^T x = P_1 ... P_{n-1} x  (P_{n-1} first)
    if constexpr (kF32) {
      const float* U32 = reinterpret_cast<const float*>(T + 3 * n);
      const float* Act32 = U32 + (size_t)n * (n - 1) / 2;
      prefetch_l2(U32, sizeof(float) * ((size_t)n * (n - 1) / 2 + n));
      const StepMask act = load_step_mask(Act32, n);
      for (int i = n - 1; i >= 1; --i) {
        if (!act.has(i)) continue;
        reflect(U32 + e2::uoff(i), i, false, 1.0);  // v = u / sqrt(h): P = I - v v^T
      }
    } else {
      const double* H = T + 2 * n;
      const double* U = T + 3 * n;
      prefetch_l2(H, sizeof(double) * ((size_t)n + (size_t)n * (n - 1) / 2));
      for (int i = n - 1; i >= 1; --i) {
        const double h = H[i];
        if (h == 0.0) continue;
        reflect(U + e2::uoff(i), i, true, h);
      }
    }
    // y = Z^T y: rotations in generation order
    const LT* cs = rot_cs + (size_t)s * rot_cap;
    const unsigned char* ix = rot_i + (size_t)s * rot_cap;
    const int nb = (nrot + kRotBatch - 1) / kRotBatch;
    RotBatch<LT> cur, nxt;
    if (nb > 0) load_rot_batch(cur, cs, ix, 0);
    for (int bb = 0; bb < nb; ++bb) {
      if ((bb & (kAheadBatches - 1)) == 0) prefetch_log(cs, ix, bb + kAheadBatches, nb);
      if (bb + 1 < nb) load_rot_batch(nxt, cs, ix, bb + 1);
#pragma unroll
      for (int j = 0; j < kRotBatch; ++j) {
        if (bb * kRotBatch + j < nrot) {
          const LT c = cur.cs[j];
          const int i = cur.idx(j);
          const VT a0 = YY(i), a1 = YY(i + 1);
          YY(i) = (VT)c.x * a0 - (VT)c.y * a1;
          YY(i + 1) = (VT)c.y * a0 + (VT)c.x * a1;
        }
      }
      cur = nxt;
    }
    if (v == 0) {
      VT* ts = tslot + (size_t)q * n;
      if constexpr (kF32) {
        const float2* fl = reinterpret_cast<const float2*>(L);
        for (int j = 0; j < n; ++j) ts[j] = YY(j) * fl[j].x;
      } else {
        for (int j = 0; j < n; ++j) ts[j] = (VT)((double)YY(j) / L[j]);
      }
    }
  }
  __syncwarp();
  VT dotw = 0;
  // W = sqrt(rho) I + V (f - sqrt(rho)) V^T with f_j = sqrt((k-1)/lambda_j): only
  // the deviation, whose size is that of the analysis increment, goes through
  // the VT-precision transforms; sqrt(rho) x is added in FP64 below.
  const double srho = sqrt(g.inflation);
  if (work && v >= 1) {
    const VT* ts = tslot + (size_t)q * n;
    if constexpr (kF32) {
      const float2* fl = reinterpret_cast<const float2*>(L);
      for (int j = 0; j < n; ++j) {
        dotw += YY(j) * ts[j];
        YY(j) *= fl[j].y;
      }
    } else {
      const double km1 = (double)(n - 1);
      for (int j = 0; j < n; ++j) {
        dotw += YY(j) * ts[j];
        YY(j) *= (VT)(sqrt(km1 / L[j]) - srho);
      }
    }
    // y = Z y: rotations in reverse order
    const LT* cs = rot_cs + (size_t)s * rot_cap;
    const unsigned char* ix = rot_i + (size_t)s * rot_cap;
    const int nb = (nrot + kRotBatch - 1) / kRotBatch;
    RotBatch<LT> cur, nxt;
    if (nb > 0) load_rot_batch(cur, cs, ix, nb - 1);
    for (int bb = nb - 1; bb >= 0; --bb) {
      if (((nb - 1 - bb) & (kAheadBatches - 1)) == 0)
        prefetch_log(cs, ix, bb - 2 * kAheadBatches + 1, nb);
      if (bb > 0) load_rot_batch(nxt, cs, ix, bb - 1);
#pragma unroll
      for (int j = kRotBatch - 1; j >= 0; --j) {
        if (bb * kRotBatch + j < nrot) {
          const LT c = cur.cs[j];
          const int i = cur.idx(j);
          const VT a0 = YY(i), a1 = YY(i + 1);
          YY(i) = (VT)c.x * a0 + (VT)c.y * a1;
          YY(i + 1) = -(VT)c.y * a0 + (VT)c.x * a1;
        }
      }
      cur = nxt;
    }
    // y = Q y = P_{n-1} ... P_1 y  (P_1 first)
    if constexpr (kF32) {
      const float* U32 = reinterpret_cast<const float*>(T + 3 * n);
      const float* Act32 = U32 + (size_t)n * (n - 1) / 2;
      prefetch_l2(U32, sizeof(float) * ((size_t)n * (n - 1) / 2 + n));
      const StepMask act = load_step_mask(Act32, n);
      for (int i = 1; i < n; ++i) {
        if (!act.has(i)) continue;
        reflect(U32 + e2::uoff(i), i, false, 1.0);
      }
    } else {
      const double* H = T + 2 * n;
      const double* U = T + 3 * n;
      prefetch_l2(H, sizeof(double) * ((size_t)n + (size_t)n * (n - 1) / 2));
      for (int i = 1; i < n; ++i) {
        const double h = H[i];
        if (h == 0.0) continue;
        reflect(U + e2::uoff(i), i, true, h);
      }
    }
    // xa = axb + sqrt(rho) x + (W - sqrt(rho) I) x + overline_w . x, recentred
    const double ab = axb[r_state + (size_t)g.n * ci];
    const double* xr = xb + (size_t)n * (r_state + (size_t)g.n * ci);
    double mean = 0.0;
    const double dotw_d = to_d(dotw);
    for (int ee = 0; ee < n; ++ee)
      mean += ab + (srho * xr[ee] + (to_d(YY(ee)) + dotw_d));
    mean /= (double)n;
    double* xo = xa + (size_t)n * (r_state + (size_t)g.n * ci);
    for (int ee = 0; ee < n; ++ee)
      xo[ee] = (ab + (srho * xr[ee] + (to_d(YY(ee)) + dotw_d))) - mean;
    axa[r_state + (size_t)g.n * ci] = mean;
  }
#undef YY
}

// ---------------------------------------------------------------- explicit trans
// Mixed path, cube solves: trans(i, j) = sqrt(rho) [i == j] + D(i, j) + wbar(i)
// (column-major, as letkf_core returns it) with the deviation
// D = V diag(f - sqrt(rho)) V^T and wbar = V diag(1/lambda) V^T t, formed by
// the vector pipeline of vec_kernel in FP32 -- FP32 reflectors, the rotation
// log, the eigenvalue factors -- on t (thread 0) and the unit vectors e_j
// (thread j + 1), one block per solve.  A solve whose rotation log overflowed
// or whose reflectors left the FP32 range (rot_n < 0) is skipped: the FP64
// fallback forms its trans.
__global__ void __launch_bounds__(128) trans_kernel(int n, SolveBatch b, const double* tin,
                                                    const double* tri, const double* lam,
                                                    const float2* rot_cs,
                                                    const unsigned char* rot_i, const int* rot_n,
                                                    int rot_cap, double srho, double* trans_out) {
  const int s = blockIdx.x;
  const int nt = blockDim.x, v = threadIdx.x;
  const int nrot = rot_n[s];
  if (nrot < 0) return;  // the whole block: the FP64 fallback forms this trans
  extern __shared__ float yt[];  // n x nt, [i][thread]
#define YV(i) yt[(i) * nt + v]
  const double* T = tri + (size_t)s * e2::tri_stride(n);
  const float2* fl = reinterpret_cast<const float2*>(lam + (size_t)s * n);
  if (v <= n) {
    if (v == 0) {
      for (int i = 0; i < n; ++i) YV(i) = d2f_bits(tin[(size_t)s * n + i]);
    } else {
      for (int i = 0; i < n; ++i) YV(i) = (i == v - 1) ? 1.0f : 0.0f;
    }
    const float* U32 = reinterpret_cast<const float*>(T + 3 * n);
    const float* Act32 = U32 + (size_t)n * (n - 1) / 2;
    // y = Q^T x (P_{n-1} first)
    for (int i = n - 1; i >= 1; --i) {
      if (Act32[i] == 0.0f) continue;
      const float* u = U32 + e2::uoff(i);
      float dot = 0.0f;
      for (int kk = 0; kk < i; ++kk) dot += u[kk] * YV(kk);
      for (int kk = 0; kk < i; ++kk) YV(kk) -= u[kk] * dot;
    }
    // y = Z^T y: rotations in generation order
    const float2* cs = rot_cs + (size_t)s * rot_cap;
    const unsigned char* ix = rot_i + (size_t)s * rot_cap;
    for (int r = 0; r < nrot; ++r) {
      const float2 c = cs[r];
      const int i = ix[r];
      const float a0 = YV(i), a1 = YV(i + 1);
      YV(i) = c.x * a0 - c.y * a1;
      YV(i + 1) = c.y * a0 + c.x * a1;
    }
    // 1/lambda for t, f - sqrt(rho) for the unit vectors
    for (int j = 0; j < n; ++j) YV(j) *= (v == 0) ? fl[j].x : fl[j].y;
    // y = Z y: rotations in reverse order
    for (int r = nrot - 1; r >= 0; --r) {
      const float2 c = cs[r];
      const int i = ix[r];
      const float a0 = YV(i), a1 = YV(i + 1);
      YV(i) = c.x * a0 + c.y * a1;
      YV(i + 1) = -c.y * a0 + c.x * a1;
    }
    // y = Q y (P_1 first)
    for (int i = 1; i < n; ++i) {
      if (Act32[i] == 0.0f) continue;
      const float* u = U32 + e2::uoff(i);
      float dot = 0.0f;
      for (int kk = 0; kk < i; ++kk) dot += u[kk] * YV(kk);
      for (int kk = 0; kk < i; ++kk) YV(kk) -= u[kk] * dot;
    }
  }
#undef YV
  __syncthreads();
  double* To = trans_out + ((size_t)b.first_solve + s) * n * n;
  for (int idx = v; idx < n * n; idx += nt) {
    const int i = idx % n, j = idx / n;
    double val = f2d_bits(yt[i * nt + j + 1]) + f2d_bits(yt[i * nt]);
    if (i == j) val += srho;
    To[idx] = val;
  }
}

void launch_trans(const Geometry& g, const SolveBatch& b, const double* t, const double* tri,
                  const double* lam, const void* rot_cs, const unsigned char* rot_i,
                  const int* rot_n, int rot_cap, double* trans, cudaStream_t stream) {
  const int n = g.ens;
  if (b.nsolves == 0) return;
  const int nt = ((n + 1 + 31) / 32) * 32;
  const size_t smem = sizeof(float) * (size_t)n * nt;
  cudaFuncSetAttribute(trans_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  trans_kernel<<<b.nsolves, nt, smem, stream>>>(n, b, t, tri, lam,
                                                static_cast<const float2*>(rot_cs), rot_i, rot_n,
                                                rot_cap, sqrt(g.inflation), trans);
}

// ------------------------------------------------------------ host launchers
size_t eig2_tri_doubles(int n) { return (size_t)n * (n + 3); }

bool eig2_supported(const Geometry& g) {
  const bool vertical = g.vert_dist > 0.0;
  const int per = 1 + (vertical ? g.n_var : g.n);
  return g.ens <= 128 && per <= 16;
}

template <typename VT, typename LT>
void launch_eig2_t(const Geometry& g, const SolveBatch& b, const double* C, const double* t,
                   const double* xb, const double* axb, double* xa, double* axa, double* tri,
                   double* lam, LT* rot_cs, unsigned char* rot_i, int* rot_n, int rot_cap,
                   int* overflow_list, int* overflow_n, int* eig_fail, int ql_warps,
                   int vec_warps, int phases, cudaStream_t stream, cudaEvent_t ev_tri,
                   cudaEvent_t ev_ql) {
  const int n = g.ens;
  constexpr size_t kSmemMax = 227 * 1024;
  const int ns = b.nsolves;
  if (ns == 0) return;
  // 1. tridiagonalisation
  if (phases & kEigTridiag) {
    const size_t smem_t = sizeof(double) * ((size_t)n * (n + 1) / 2 + n);
    const int u32 = sizeof(VT) == sizeof(float) ? 1 : 0;
    // four warps per matrix above 64 members (up to 66 KB of triangle per
    // CTA); LETKF_GB300_TRI_MW=1 takes them for every size (a diagnostic)
    static const bool mw_all = getenv("LETKF_GB300_TRI_MW") != nullptr;
    if (n > 64 || mw_all) {
      cudaFuncSetAttribute(tridiag_mw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_t);
      tridiag_mw_kernel<<<ns, 32 * kTriWarps, smem_t, stream>>>(n, ns, C, tri, u32);
    } else {
      cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_t);
      tridiag_kernel<<<ns, 32, smem_t, stream>>>(n, ns, C, tri, u32);
    }
    if (ev_tri) record_event(ev_tri, stream);
  }
  if (phases & kEigQL) {
    // 2. QL, one solve per lane; a block takes at most a third of the SM's
    // shared memory (at 128 members one warp's d and e are 64 KB), so that
    // three QL blocks, or QL blocks and those of the other streams, share an SM
    ql_warps = std::max(1, std::min(ql_warps, (int)(kSmemMax / (3 * sizeof(double) * 64 * n))));
    const size_t smem_q = sizeof(double) * (size_t)ql_warps * 64 * n;
    cudaFuncSetAttribute(ql_kernel<LT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_q);
    const int ql_blocks = (ns + 32 * ql_warps - 1) / (32 * ql_warps);
    ql_kernel<LT><<<ql_blocks, 32 * ql_warps, smem_q, stream>>>(
        n, ns, (double)(n - 1) / g.inflation, sqrt(g.inflation), tri, lam, rot_cs, rot_i, rot_n,
        rot_cap, overflow_list, overflow_n, eig_fail, g.ql_max_iter > 0 ? g.ql_max_iter : 60);
    if (ev_ql) record_event(ev_ql, stream);
  }
  if (phases & kEigVectors) {
    // 3. vectors and update
    const bool vertical = g.vert_dist > 0.0;
    const int per = 1 + (vertical ? g.n_var : g.n);
    const int slots = 32 / per;
    const size_t vper = sizeof(VT) * ((size_t)32 * n + (size_t)slots * n);
    const int vwarps = std::max(1, std::min(vec_warps, (int)(kSmemMax / vper)));
    const size_t smem_v = sizeof(VT) * ((size_t)vwarps * 32 * n + (size_t)vwarps * slots * n);
    cudaFuncSetAttribute(vec_kernel<VT, LT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_v);
    const int vblocks = (ns + slots * vwarps - 1) / (slots * vwarps);
    vec_kernel<VT, LT><<<vblocks, 32 * vwarps, smem_v, stream>>>(g, b, t, tri, lam, rot_cs, rot_i,
                                                                 rot_n, rot_cap, xb, axb, xa, axa);
  }
}

void launch_eig2(const Geometry& g, const SolveBatch& b, const double* C, const double* t,
                 const double* xb, const double* axb, double* xa, double* axa, double* tri,
                 double* lam, void* rot_cs, unsigned char* rot_i, int* rot_n, int rot_cap,
                 int* overflow_list, int* overflow_n, int* eig_fail, bool fp32_vectors,
                 int ql_warps, int vec_warps, int phases, cudaStream_t stream,
                 cudaEvent_t ev_tri, cudaEvent_t ev_ql) {
  if (fp32_vectors)
    launch_eig2_t<float, float2>(g, b, C, t, xb, axb, xa, axa, tri, lam,
                                 static_cast<float2*>(rot_cs), rot_i, rot_n, rot_cap,
                                 overflow_list, overflow_n, eig_fail, ql_warps, vec_warps, phases,
                                 stream, ev_tri, ev_ql);
  else
    launch_eig2_t<double, double2>(g, b, C, t, xb, axb, xa, axa, tri, lam,
                                   static_cast<double2*>(rot_cs), rot_i, rot_n, rot_cap,
                                   overflow_list, overflow_n, eig_fail, ql_warps, vec_warps,
                                   phases, stream, ev_tri, ev_ql);
}

}  // namespace lg
