// lg_eig.cu -- FP64 symmetric eigensolve of C + the LETKF transform and update.
//
// Per solve (letkf_core.F90:98-225, letkf_compute.F90:259-329,501-552):
//   (V, lambda) = eig(C)                       dsyevd in the reference
//   lambda     += (k-1)/rho
//   overline_w  = V diag(1/lambda) V^T t        (= Pa * sum_e Yb R^-1 d)
//   W           = V diag(sqrt((k-1)/lambda)) V^T
//   xa(:, r)    = axb(r) + W xb(:, r) + (overline_w . xb(:, r)) 1   for the rows
//                 this solve owns, then recentred (axa = mean, xa -= axa)
// The eigensolver is Householder tridiagonalisation with accumulated
// transformations followed by the implicit QL iteration with shifts (the
// Martin-Reinsch-Wilkinson tred2/tql2 pair), in FP64, one CTA per matrix with
// the matrix in shared memory (row stride k+1 to avoid bank conflicts).
// W is never formed for the update: each row is transformed as
// V (f .* (V^T x)), which costs 4k^2 per row instead of k^3.
#include <float.h>

#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

template <int NT>
struct Blk {
  __device__ static inline void sync() {
    if (NT == 32) __syncwarp(); else __syncthreads();
  }
  // sum over the CTA; every thread gets the result
  __device__ static inline double sum(double v, double* red) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
    if (NT == 32) return v;
    const int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) t += red[i];
    return t;
  }
};

template <int NT>
__global__ void __launch_bounds__(NT) eig_apply_kernel(Geometry g, SolveBatch b, const double* Cin,
                                                       const double* tin, const double* xb,
                                                       const double* axb, double* xa,
                                                       double* axa, double* trans_out,
                                                       double* wbar_out, int* eig_fail) {
  using B = Blk<NT>;
  for (int ii = blockIdx.x;; ii += gridDim.x) {
  int s;
  if (b.solve_list) {
    if (ii >= *b.solve_count) return;
    s = b.solve_list[ii];
  } else {
    if (ii >= b.nsolves) return;
    s = ii;
  }
  const int n = g.ens;
  const int LD = n | 1;  // odd row stride
  const int tid = threadIdx.x;
  extern __shared__ double sm[];
  double* a = sm;                  // n x LD
  double* d = a + n * LD;          // n
  double* e = d + n;               // n
  double* tv = e + n;              // n
  double* u = tv + n;              // n
  double* wb = u + n;              // n
  double* x = wb + n;              // n
  double* red = x + n;             // 8
  __shared__ int s_fail;

  const double* C = Cin + (size_t)s * n * n;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;  // C column-major
    a[i * LD + j] = C[idx];
  }
  for (int i = tid; i < n; i += NT) tv[i] = tin[(size_t)s * n + i];
  if (tid == 0) s_fail = 0;
  __syncthreads();

  // ---- Householder reduction to tridiagonal form (a -> Q, d, e) ----
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    double h = 0.0;
    if (l > 0) {
      double sc = 0.0;
      for (int kk = tid; kk <= l; kk += NT) sc += fabs(a[i * LD + kk]);
      const double scale = B::sum(sc, red);
      if (scale == 0.0) {
        if (tid == 0) e[i] = a[i * LD + l];
        B::sync();
      } else {
        double hh = 0.0;
        for (int kk = tid; kk <= l; kk += NT) {
          const double v = a[i * LD + kk] / scale;
          a[i * LD + kk] = v;
          hh += v * v;
        }
        h = B::sum(hh, red);
        const double f = a[i * LD + l];
        const double gg = (f >= 0.0) ? -sqrt(h) : sqrt(h);
        h -= f * gg;
        B::sync();
        if (tid == 0) {
          e[i] = scale * gg;
          a[i * LD + l] = f - gg;
        }
        B::sync();
        // p = A u / h  (stored in e[0..l]); a[j][i] = u_j / h
        double fs = 0.0;
        for (int j = tid; j <= l; j += NT) {
          a[j * LD + i] = a[i * LD + j] / h;
          double gj = 0.0;
          for (int kk = 0; kk <= j; ++kk) gj += a[j * LD + kk] * a[i * LD + kk];
          for (int kk = j + 1; kk <= l; ++kk) gj += a[kk * LD + j] * a[i * LD + kk];
          e[j] = gj / h;
          fs += e[j] * a[i * LD + j];
        }
        const double ff = B::sum(fs, red);
        const double hh2 = ff / (h + h);
        for (int j = tid; j <= l; j += NT) e[j] = e[j] - hh2 * a[i * LD + j];
        B::sync();
        // A -= u q^T + q u^T on the lower triangle
        for (int j = 0; j <= l; ++j) {
          const double fj = a[i * LD + j], gj = e[j];
          for (int kk = tid; kk <= j; kk += NT) a[j * LD + kk] -= (fj * e[kk] + gj * a[i * LD + kk]);
        }
        B::sync();
      }
    } else {
      if (tid == 0) e[i] = a[i * LD + l];
      B::sync();
    }
    if (tid == 0) d[i] = h;
    B::sync();
  }
  if (tid == 0) {
    d[0] = 0.0;
    e[0] = 0.0;
  }
  B::sync();
  // accumulate the transformations into Q
  for (int i = 0; i < n; ++i) {
    const int l = i - 1;
    if (d[i] != 0.0) {
      for (int j = tid; j <= l; j += NT) {
        double gj = 0.0;
        for (int kk = 0; kk <= l; ++kk) gj += a[i * LD + kk] * a[kk * LD + j];
        for (int kk = 0; kk <= l; ++kk) a[kk * LD + j] -= gj * a[kk * LD + i];
      }
    }
    B::sync();
    if (tid == 0) {
      d[i] = a[i * LD + i];
      a[i * LD + i] = 1.0;
    }
    for (int j = tid; j <= l; j += NT) {
      a[j * LD + i] = 0.0;
      a[i * LD + j] = 0.0;
    }
    B::sync();
  }

  // ---- implicit QL iteration on (d, e); rotations accumulate into a ----
  if (tid == 0) {
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = 0.0;
  }
  B::sync();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      // thread 0 finds the split point; everyone reads it
      __shared__ int s_m;
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= DBL_EPSILON * dd) break;
        }
        s_m = m;
      }
      B::sync();
      const int m = s_m;
      if (m == l) break;
      if (++iter > (g.ql_max_iter > 0 ? g.ql_max_iter : 60)) {
        if (tid == 0) s_fail = 1;
        break;
      }
      double gsh = 0.0;
      if (tid == 0) {
        double gg = (d[l + 1] - d[l]) / (2.0 * e[l]);
        const double r = hypot(gg, 1.0);
        gsh = d[m] - d[l] + e[l] / (gg + (gg >= 0.0 ? fabs(r) : -fabs(r)));
      }
      double sn = 1.0, cs = 1.0, pp = 0.0, gv = gsh;
      bool early = false;
      for (int i = m - 1; i >= l; --i) {
        double sv = 0.0, cv = 0.0;
        int brk = 0;
        if (tid == 0) {
          const double f = sn * e[i], bb = cs * e[i];
          const double r = sqrt(f * f + gv * gv);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= pp;
            e[m] = 0.0;
            brk = 1;
          } else {
            const double rinv = 1.0 / r;
            sn = f * rinv;
            cs = gv * rinv;
            gv = d[i + 1] - pp;
            const double rr = (d[i] - gv) * sn + 2.0 * cs * bb;
            pp = sn * rr;
            d[i + 1] = gv + pp;
            gv = cs * rr - bb;
            sv = sn;
            cv = cs;
          }
        }
        // broadcast the rotation
        if (NT == 32) {
          brk = __shfl_sync(0xffffffffu, brk, 0);
          sv = __shfl_sync(0xffffffffu, sv, 0);
          cv = __shfl_sync(0xffffffffu, cv, 0);
        } else {
          __shared__ double s_rot[2];
          __shared__ int s_brk;
          if (tid == 0) {
            s_rot[0] = sv;
            s_rot[1] = cv;
            s_brk = brk;
          }
          __syncthreads();
          sv = s_rot[0];
          cv = s_rot[1];
          brk = s_brk;
          __syncthreads();
        }
        if (brk) {
          early = true;
          break;
        }
        for (int r = tid; r < n; r += NT) {
          const double f = a[r * LD + i + 1];
          const double z = a[r * LD + i];
          a[r * LD + i + 1] = sv * z + cv * f;
          a[r * LD + i] = cv * z - sv * f;
        }
      }
      if (tid == 0 && !early) {
        d[l] -= pp;
        e[l] = gv;
        e[m] = 0.0;
      }
      B::sync();
    }
  }
  __syncthreads();

  // ---- transform: lambda, overline_w, W applied to the rows ----
  const double km1 = (double)(n - 1);
  for (int i = tid; i < n; i += NT) {
    const double lam = d[i] * 1.0 + km1 / g.inflation;
    d[i] = lam;
    double ui = 0.0;
    for (int r = 0; r < n; ++r) ui += a[r * LD + i] * tv[r];
    u[i] = ui / lam;
    e[i] = sqrt(km1 / lam);  // f_i
  }
  __syncthreads();
  for (int r = tid; r < n; r += NT) {
    double w = 0.0;
    for (int i = 0; i < n; ++i) w += a[r * LD + i] * u[i];
    wb[r] = w;
  }
  __syncthreads();
  if (s_fail && tid == 0) atomicAdd(eig_fail, 1);
  __syncthreads();
  if (tid == 0) s_fail = 0;

  if (b.mode == 1 || b.s_col) {
    // explicit trans(i, j) = W(i, j) + overline_w(i), column-major (cube
    // solves: at the solve's index in the analysis; applied by the cube kernel)
    const size_t so = b.s_col ? (size_t)b.first_solve + s : (size_t)s;
    double* T = trans_out + so * n * n;
    for (int i = tid; i < n; i += NT) {
      for (int j = 0; j < n; ++j) {
        double w = 0.0;
        for (int m = 0; m < n; ++m) w += a[i * LD + m] * e[m] * a[j * LD + m];
        T[i + (size_t)n * j] = w + wb[i];
      }
      if (wbar_out) wbar_out[so * n + i] = wb[i];
    }
    __syncthreads();
    continue;
  }

  // rows owned by this solve
  const int col = b.first_col + s / b.levels;
  const int kk = s % b.levels + 1;
  const int glat = col % g.num_lat + 1, glon = col / g.num_lat + 1;
  const size_t ci = (size_t)(glat - 1 + g.halo) +
                    (size_t)(g.num_lat + 2 * g.halo) * (size_t)(glon - 1 + g.halo);
  const bool vertical = g.vert_dist > 0.0;
  const int nrows_total = vertical ? g.n_var : g.n;
  for (int q = 0; q < nrows_total; ++q) {
    int r;
    if (vertical) {
      const int v = q;
      if (g.var_lev[v] == 1) {
        if (kk != g.nz) continue;
        r = g.var_start[v];
      } else {
        r = g.var_start[v] + kk - 1;
      }
    } else {
      r = q;
    }
    const double* xr = xb + (size_t)n * (r + (size_t)g.n * ci);
    for (int i = tid; i < n; i += NT) x[i] = xr[i];
    __syncthreads();
    double dotw = 0.0;
    for (int i = tid; i < n; i += NT) {
      double v = 0.0;
      for (int rr = 0; rr < n; ++rr) v += a[rr * LD + i] * x[rr];
      u[i] = v * e[i];
      dotw += wb[i] * x[i];
    }
    const double wdotx = B::sum(dotw, red);
    __syncthreads();
    const double ab = axb[r + (size_t)g.n * ci];
    double val[4];
    double ssum = 0.0;
    int qq = 0;
    for (int ee = tid; ee < n; ee += NT, ++qq) {
      double v = 0.0;
      for (int i = 0; i < n; ++i) v += a[ee * LD + i] * u[i];
      val[qq] = ab + (v + wdotx);
      ssum += val[qq];
    }
    const double mean = B::sum(ssum, red) / (double)n;
    double* xo = xa + (size_t)n * (r + (size_t)g.n * ci);
    qq = 0;
    for (int ee = tid; ee < n; ee += NT, ++qq) xo[ee] = val[qq] - mean;
    if (tid == 0) axa[r + (size_t)g.n * ci] = mean;
    __syncthreads();
  }
  __syncthreads();
  }  // solves of this CTA
}

void launch_eig_apply(const Geometry& g, const SolveBatch& b, const double* C, const double* t,
                      const double* xb, const double* axb, double* xa, double* axa,
                      double* trans, double* wbar, int* eig_fail, cudaStream_t stream) {
  if (b.nsolves == 0) return;
  const int n = g.ens;
  const int LD = n | 1;
  const size_t smem = sizeof(double) * ((size_t)n * LD + 6 * n + 8);
  const int grid = b.solve_list ? std::min(b.nsolves, 152 * 6) : b.nsolves;
  if (n <= 64) {
    // one warp per matrix: the QL rotations are broadcast by shuffles, no block barriers
    cudaFuncSetAttribute(eig_apply_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    eig_apply_kernel<32><<<grid, 32, smem, stream>>>(g, b, C, t, xb, axb, xa, axa, trans,
                                                          wbar, eig_fail);
  } else {
    cudaFuncSetAttribute(eig_apply_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    eig_apply_kernel<128><<<grid, 128, smem, stream>>>(g, b, C, t, xb, axb, xa, axa,
                                                            trans, wbar, eig_fail);
  }
}

}  // namespace lg
