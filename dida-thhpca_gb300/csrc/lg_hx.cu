// lg_hx.cu -- observation operator H(x) for every member (FP64).
//
// One warp per block-observation copy.  Restates, per copy:
//   find_obs_grid           x86/DA/LETKF/src/letkf_obs.F90:192-248
//   ps2ph_3d_interp         x86/DA/LETKF/src/obs_make.F90:345-381
//   obs_interpolation_3d_2  x86/DA/LETKF/src/obs_make.F90:233-342
//   member-mean removal     x86/DA/LETKF/src/letkf_obs.F90:156-183
// with the reference's operation order and no contraction (this file is built
// with -fmad=false).  Lanes own members e = lane, lane+32, ...; the member mean
// is summed sequentially in member order, as the Fortran loop does.
#include <algorithm>

#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

__constant__ TypeTable c_types;

void set_type_table(const TypeTable& t, cudaStream_t stream) {
  cudaMemcpyToSymbolAsync(c_types, &t, sizeof(TypeTable), 0, cudaMemcpyHostToDevice, stream);
}

__global__ void obs_trig_kernel(int n, const double* lat, const double* lon, double* dcx,
                                double* dsx, double* dyr, float* fcx, float* fsx, float* fyr) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  double xr = deg2rad_r8(lat[o]);
  dcx[o] = cos(xr);
  dsx[o] = sin(xr);
  dyr[o] = deg2rad_r8(lon[o]);
  const float pf = 3.14159274101257324f;
  float xf = (float)lat[o] / 180.0f * pf;
  fcx[o] = cosf(xf);
  fsx[o] = sinf(xf);
  fyr[o] = (float)lon[o] / 180.0f * pf;
}

// the selection's per-slot candidate data, gathered once per observation set so
// that the candidate loop reads one contiguous float4 instead of chasing
// copy -> observation -> trigonometry
__global__ void cell_cands_kernel(ObsDev o, double obs_polar, const int* slot_obs, int nslots,
                                  float4* cand) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const int ob = slot_obs[s];
  cand[s] = make_float4(o.fcx[ob], o.fsx[ob], o.fyr[ob],
                        fabs(o.olat[ob]) <= obs_polar ? 1.0f : 0.0f);
}

void launch_cell_cands(const ObsDev& o, double obs_polar, const int* slot_obs, int nslots,
                       float4* cand, cudaStream_t stream) {
  if (nslots == 0) return;
  cell_cands_kernel<<<(nslots + 255) / 256, 256, 0, stream>>>(o, obs_polar, slot_obs, nslots,
                                                              cand);
}

void launch_obs_trig(const ObsDev& o, double* dcx, double* dsx, double* dyr, float* fcx,
                     float* fsx, float* fyr, cudaStream_t stream) {
  if (o.n_obs == 0) return;
  obs_trig_kernel<<<(o.n_obs + 255) / 256, 256, 0, stream>>>(o.n_obs, o.olat, o.olon, dcx, dsx,
                                                               dyr, fcx, fsx, fyr);
}

// bilinear value (r1*t2 + r2*(1-t2)) of row r at the 2x2 stencil for member e
__device__ inline double bilin(const double* xb, const double* axb, int k, int n, int e, int r,
                               size_t c11, size_t c21, size_t c12, size_t c22, double t1,
                               double t2) {
  const double u1 = __dsub_rn(1.0, t1), u2 = __dsub_rn(1.0, t2);
  double a11 = __dadd_rn(xb[e + (size_t)k * (r + (size_t)n * c11)], axb[r + (size_t)n * c11]);
  double a21 = __dadd_rn(xb[e + (size_t)k * (r + (size_t)n * c21)], axb[r + (size_t)n * c21]);
  double a12 = __dadd_rn(xb[e + (size_t)k * (r + (size_t)n * c12)], axb[r + (size_t)n * c12]);
  double a22 = __dadd_rn(xb[e + (size_t)k * (r + (size_t)n * c22)], axb[r + (size_t)n * c22]);
  double r1 = __dadd_rn(__dmul_rn(a11, t1), __dmul_rn(a21, u1));
  double r2 = __dadd_rn(__dmul_rn(a12, t1), __dmul_rn(a22, u1));
  return __dadd_rn(__dmul_rn(r1, t2), __dmul_rn(r2, u2));
}

constexpr int kMaxMemberSlots = 4;  // ens <= 128

__global__ void __launch_bounds__(128) hx_kernel(Geometry g, ObsDev ob, const double* xb,
                                                 const double* axb, HxDev hx, int* err,
                                                 int64_t j0, int64_t j1) {
  const int64_t j = j0 + (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x / 32);
  if (j >= j1) return;
  const unsigned lane = threadIdx.x & 31u;
  const int k = g.ens, n = g.n;
  const int o = ob.copy_obs[j];
  const int4 bk = g.blk[ob.copy_block[j]];
  const int s_lat = bk.x, e_lat = bk.y, s_lon = bk.z, e_lon = bk.w;
  const int nxl = e_lat - s_lat + 1, nyl = e_lon - s_lon + 1;
  const double lat = ob.olat[o], lon = ob.olon[o];
  // find_obs_grid: first local index with grid >= obs coordinate
  int tx = 0, ty = 0;
  for (int base = 1; base <= nxl + 1 && tx == 0; base += 32) {
    int i = base + (int)lane;
    bool hit = (i <= nxl + 1) && ((double)g.glat[s_lat + i - 2] >= lat);
    unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m) tx = base + __ffs(m) - 1;
  }
  for (int base = 1; base <= nyl + 1 && ty == 0; base += 32) {
    int i = base + (int)lane;
    bool hit = (i <= nyl + 1) && ((double)g.glon[s_lon + i - 2] >= lon);
    unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m) ty = base + __ffs(m) - 1;
  }
  const int ti = c_types.nz[0] >= 0 ? ob.otype[o] : 0;
  const int onz = c_types.nz[ti], onv = c_types.nvar[ti];
  const int64_t ebase = ob.copy_eoff[j];
  if (tx == 0 || ty == 0) {
    if (lane == 0) atomicExch(err, LG_ERR_OBS_OUTSIDE);
    return;
  }
  double ax = 0.0, ay = 0.0;
  if (tx > 1) {
    float gt = g.glat[s_lat + tx - 2], gp = g.glat[s_lat + tx - 3];
    double dlat = (double)__fsub_rn(gt, gp);  // REAL(4) subtraction
    ax = __ddiv_rn(__dadd_rn(__dsub_rn(dlat, lat), (double)gp), dlat);
  }
  if (ty > 1) {
    float gt = g.glon[s_lon + ty - 2], gp = g.glon[s_lon + ty - 3];
    double dlon = (double)__fsub_rn(gt, gp);
    ay = __ddiv_rn(__dadd_rn(__dsub_rn(dlon, lon), (double)gp), dlon);
  }
  const int nlat_e = g.num_lat + 2 * g.halo;
  auto colidx = [&](int glat, int glon) -> size_t {
    return (size_t)(glat - 1 + g.halo) + (size_t)nlat_e * (size_t)(glon - 1 + g.halo);
  };
  const int la0 = s_lat + tx - 2, la1 = s_lat + tx - 1;
  const int lo0 = s_lon + ty - 2, lo1 = s_lon + ty - 1;
  const size_t c11 = colidx(la0, lo0), c21 = colidx(la1, lo0);
  const size_t c12 = colidx(la0, lo1), c22 = colidx(la1, lo1);
  const double t1 = ax, t2 = ay;
  const double* oph = ob.oph + ob.ph_off[o];
  const double* yo = ob.oyo + ob.val_off[o];
  const double* ri = ob.orinv + ob.val_off[o];

  double ps[kMaxMemberSlots];
#pragma unroll
  for (int q = 0; q < kMaxMemberSlots; ++q) {
    const int e = (int)lane + 32 * q;
    ps[q] = (e < k) ? bilin(xb, axb, k, n, e, g.ps_row, c11, c21, c12, c22, t1, t2) : 0.0;
  }
  // ph_pos for each obs level; the search index persists across levels
  // (obs_make.F90:252-272).  Levels are processed in order; at most 64 per type.
  //
  // The search walks up the member's half levels half_ph(j) = (ph_lev(j) +
  // ph_lev(j + 1)) / 2 for j = 1..nz (half_ph(nz + 1) = half_ph(nz)).  Each
  // step needs one new full level: the state of member slot q is its index jj,
  // b = ph_lev(jj + 1) (jj <= nz), hp = half_ph(jj) and hpm = half_ph(jj - 1)
  // (jj >= 2), every value formed by the reference's operations in its order,
  // so the search and the weights below are bit for bit those of evaluating
  // half_ph afresh at every step.
  // ph_lev: da_hybrid_coord_calc_ph_lev / da_sigma_coord_calc_ph_lev
  // (x86/DA/utils/vert_coord_mod.F90:547-563), level kk 1-based
  const double p0pt = __dsub_rn(g.p0, g.ptop);
  auto ph_lev = [&](int kk, double psd) -> double {
    if (g.vcoord == LG_VCOORD_SIGMA) return __dadd_rn(__dmul_rn(g.ca[kk - 1], psd), g.ptop);
    return __dadd_rn(__dadd_rn(__dmul_rn(g.ca[kk - 1], p0pt), __dmul_rn(g.cb[kk - 1], psd)),
                     g.ptop);
  };
  int jj[kMaxMemberSlots];
  double psd[kMaxMemberSlots], lev_b[kMaxMemberSlots], hp[kMaxMemberSlots],
      hpm[kMaxMemberSlots];
#pragma unroll
  for (int q = 0; q < kMaxMemberSlots; ++q) {
    jj[q] = 1;
    psd[q] = __dsub_rn(ps[q], g.ptop);
    const double a = ph_lev(1, psd[q]);
    lev_b[q] = ph_lev(2, psd[q]);
    hp[q] = __dmul_rn(0.5, __dadd_rn(a, lev_b[q]));
    hpm[q] = 0.0;
  }
  bool has3d = false;  // the log-p weights are needed only for 3-D variables
  for (int kv = 0; kv < onv; ++kv) has3d |= g.var_lev[c_types.var[ti][kv]] > 1;
  for (int l = 0; l < onz; ++l) {
    const double po = oph[l];
    const double lnpo = log(po);
    int pp[kMaxMemberSlots];
#pragma unroll
    for (int q = 0; q < kMaxMemberSlots; ++q) {
      const int e = (int)lane + 32 * q;
      if (e < k) {
        // while (jj <= nz && po > half_ph(jj)) jj++; half_ph(nz + 1) is
        // half_ph(nz), so hp needs no update when jj reaches nz + 1
        while (jj[q] <= g.nz && po > hp[q]) {
          hpm[q] = hp[q];
          ++jj[q];
          if (jj[q] <= g.nz) {
            const double a = lev_b[q];
            lev_b[q] = ph_lev(jj[q] + 1, psd[q]);
            hp[q] = __dmul_rn(0.5, __dadd_rn(a, lev_b[q]));
          }
        }
      }
      pp[q] = jj[q] - 1;
    }
    // vertical interpolation weight in log p of each member for this level,
    // shared by the level's variables: with p = jj - 1 in [1, nz), half_ph(p + 1)
    // is hp and half_ph(p) is hpm
    double t3[kMaxMemberSlots];
#pragma unroll
    for (int q = 0; q < kMaxMemberSlots; ++q) {
      const int e = (int)lane + 32 * q;
      const int p = pp[q];
      t3[q] = 0.0;
      if (has3d && e < k && p >= 1 && p < g.nz) {
        const double lp1 = log(hp[q]);
        t3[q] = __ddiv_rn(__dsub_rn(lp1, lnpo), __dsub_rn(lp1, log(hpm[q])));
      }
    }
    for (int kv = 0; kv < onv; ++kv) {
      const int vid = c_types.var[ti][kv];
      const int vs = g.var_start[vid];
      const int64_t ent = ebase + (int64_t)l * onv + kv;
      double y[kMaxMemberSlots];
#pragma unroll
      for (int q = 0; q < kMaxMemberSlots; ++q) {
        const int e = (int)lane + 32 * q;
        y[q] = 0.0;
        if (e >= k) continue;
        if (g.var_lev[vid] > 1) {
          const int p = pp[q];
          if (p >= 1 && p < g.nz) {
            const int tl = vs + p - 1;
            const double r1 = bilin(xb, axb, k, n, e, tl, c11, c21, c12, c22, t1, t2);
            const double r3 = bilin(xb, axb, k, n, e, tl + 1, c11, c21, c12, c22, t1, t2);
            y[q] = __dadd_rn(__dmul_rn(r1, t3[q]), __dmul_rn(r3, __dsub_rn(1.0, t3[q])));
          } else {
            const int tl = (p == 0) ? vs : vs + g.nz - 1;
            y[q] = bilin(xb, axb, k, n, e, tl, c11, c21, c12, c22, t1, t2);
          }
        } else {
          y[q] = bilin(xb, axb, k, n, e, vs, c11, c21, c12, c22, t1, t2);
        }
      }
      // member mean (letkf_obs.F90:160-164): per-lane partial sums over the
      // member slots, then a shuffle tree (the reference sums in member order;
      // the two agree to rounding, far inside the 1e-12 parity bound)
      double sum_y = 0.0;
#pragma unroll
      for (int q = 0; q < kMaxMemberSlots; ++q)
        if ((int)lane + 32 * q < k) sum_y = __dadd_rn(sum_y, y[q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum_y = __dadd_rn(sum_y, __shfl_xor_sync(0xffffffffu, sum_y, o));
      sum_y = __ddiv_rn(sum_y, (double)k);
#pragma unroll
      for (int q = 0; q < kMaxMemberSlots; ++q) {
        const int e = (int)lane + 32 * q;
        if (e < k) {
          const double d = __dsub_rn(y[q], sum_y);
          hx.yb[(size_t)ent * k + e] = d;
          if (hx.yb32) hx.yb32[(size_t)ent * k + e] = (float)d;
        }
      }
      if (lane == 0) {
        hx.dis[ent] = __dsub_rn(yo[l * onv + kv], sum_y);
        hx.lnp[ent] = lnpo;  // letkf_yb.F90:211, with the observation's own ph
        hx.rdiag[ent] = (float)ri[l * onv + kv];
      }
    }
  }
}

void launch_hx(const Geometry& g, const ObsDev& o, const double* xb, const double* axb,
               HxDev hx, int* err, cudaStream_t stream, int64_t j0, int64_t j1) {
  if (j1 < 0 || j1 > o.n_copies) j1 = o.n_copies;
  if (j0 < 0) j0 = 0;
  if (j1 <= j0) return;
  const int warps = 4;
  const int64_t blocks = (j1 - j0 + warps - 1) / warps;
  hx_kernel<<<(unsigned)blocks, 32 * warps, 0, stream>>>(g, o, xb, axb, hx, err, j0, j1);
}

// Packed H(x) rows, ens + 3 doubles per entry (yb[0 .. ens), dis, ln p,
// rdiaginv): the unit of the observation exchange between column shards (the
// role of comm_obs_data, x86/DA/LETKF/src/letkf_obs.F90:251-466).  One thread
// per row element; consecutive threads take consecutive elements.
__global__ void hx_export_kernel(int k, int64_t e0, int64_t nrows, HxDev hx, double* rows) {
  const int64_t w = k + 3, total = nrows * w;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / w;
    const int c = (int)(i - r * w);
    const int64_t e = e0 + r;
    double v;
    if (c < k) v = hx.yb[(size_t)e * k + c];
    else if (c == k) v = hx.dis[e];
    else if (c == k + 1) v = hx.lnp[e];
    else v = (double)hx.rdiag[e];  // exact
    rows[i] = v;
  }
}

__global__ void hx_import_kernel(int k, int64_t e0, int64_t nrows, HxDev hx, const double* rows) {
  const int64_t w = k + 3, total = nrows * w;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / w;
    const int c = (int)(i - r * w);
    const int64_t e = e0 + r;
    const double v = rows[i];
    if (c < k) {
      hx.yb[(size_t)e * k + c] = v;
      if (hx.yb32) hx.yb32[(size_t)e * k + c] = (float)v;  // as hx_kernel rounds it
    } else if (c == k) {
      hx.dis[e] = v;
    } else if (c == k + 1) {
      hx.lnp[e] = v;
    } else {
      hx.rdiag[e] = (float)v;  // a float value: exact
    }
  }
}

void launch_hx_export(int ens, int64_t e0, int64_t e1, const HxDev& hx, double* rows,
                      cudaStream_t stream) {
  if (e1 <= e0) return;
  const int64_t total = (e1 - e0) * (ens + 3);
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  hx_export_kernel<<<blocks, 256, 0, stream>>>(ens, e0, e1 - e0, hx, rows);
}

void launch_hx_import(int ens, int64_t e0, int64_t e1, HxDev hx, const double* rows,
                      cudaStream_t stream) {
  if (e1 <= e0) return;
  const int64_t total = (e1 - e0) * (ens + 3);
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
  hx_import_kernel<<<blocks, 256, 0, stream>>>(ens, e0, e1 - e0, hx, rows);
}

__global__ void nan_check_kernel(const double* x, size_t n, int* err) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (; i < n; i += stride) bad |= (x[i] != x[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(err, LG_ERR_NAN);
}

void launch_nan_check(const double* x, size_t n, int* err, cudaStream_t stream) {
  if (n == 0) return;
  nan_check_kernel<<<152 * 8, 256, 0, stream>>>(x, n, err);
}

}  // namespace lg
