// lg_coupler.cu -- GMCORE state to the DA background layout.
//
// The step before the analysis in the coupled cycle: GMCORE's u and v live on
// the C grid (u at half longitudes, v at half latitudes), pt and ps at cell
// centres; gmcore2da_send_coupling (gmcore_coupler.F90:153-284) moves u and v
// to the centres,
//   u(i, j) = (u_f(i, j) + u_f(i-1, j)) / 2,
//   v(i, j) = 2 (v_f(i, j-1) area_subcell(1, j) + v_f(i, j) area_subcell(2, j)) / area_cell(j),
// and the coupler delivers the four fields as the DA's xb(ens, n, lat, lon)
// with n = ps, u levels, v levels, pt levels and the longitude halo filled
// periodically (module_da_coupler.F90:91-147, 350-414).  One GPU holds the
// whole globe, so the MCT transfer is one HBM-bound kernel, members fastest on
// both sides (coalesced reads and writes).
#include "lg_internal.h"

namespace lg {

namespace {

// one block per (longitude with halo, latitude) column, a thread per member,
// the rows in a loop: no integer division, reads and writes contiguous in the
// members.  The v weights 2 area_subcell(., j) / area_cell(j) are formed once
// per latitude (two FP64 operations per v value instead of a division; the
// result differs from the reference's expression by rounding only).
__global__ void gmcore_to_da_kernel(int ens, int num_lat, int num_lon, int nz, int halo,
                                    const double* ps, const double* u_half, const double* v_half,
                                    const double* pt, const double* area_subcell,
                                    const double* area_cell, double* xb) {
  const int le = blockIdx.x;  // 0-based longitude with halo
  const int jj = blockIdx.y;  // 0-based latitude
  const int m = threadIdx.x;
  if (m >= ens) return;
  const int n = 1 + 3 * nz;
  const int nlat_e = num_lat + 2 * halo;
  int ii = le - halo;  // 0-based longitude, periodic
  ii = ii < 0 ? ii + num_lon : (ii >= num_lon ? ii - num_lon : ii);
  const int iw = ii == 0 ? num_lon - 1 : ii - 1;
  const double w_s = 2.0 * area_subcell[2 * jj] / area_cell[jj];
  const double w_n = 2.0 * area_subcell[2 * jj + 1] / area_cell[jj];
  const size_t plane = (size_t)num_lat * num_lon * ens;
  const size_t vplane = (size_t)(num_lat + 1) * num_lon * ens;
  const size_t cell = ((size_t)jj * num_lon + ii) * ens + m;
  const size_t west = ((size_t)jj * num_lon + iw) * ens + m;
  const size_t vs0 = ((size_t)jj * num_lon + ii) * ens + m, vn0 = vs0 + (size_t)num_lon * ens;
  double* out = xb + ((size_t)le * nlat_e + (jj + halo)) * n * ens + m;
  out[0] = ps[cell];
  for (int k = 0; k < nz; ++k) {
    out[(size_t)(1 + k) * ens] = (u_half[k * plane + cell] + u_half[k * plane + west]) * 0.5;
    out[(size_t)(1 + nz + k) * ens] = fma(v_half[k * vplane + vn0], w_n, v_half[k * vplane + vs0] * w_s);
    out[(size_t)(1 + 2 * nz + k) * ens] = pt[k * plane + cell];
  }
}

}  // namespace

cudaError_t launch_gmcore_to_da(int ens, int num_lat, int num_lon, int nz, int halo,
                                const double* ps, const double* u_half, const double* v_half,
                                const double* pt, const double* area_subcell,
                                const double* area_cell, double* xb, cudaStream_t stream) {
  const dim3 grid(num_lon + 2 * halo, num_lat);
  const int threads = ((ens + 31) / 32) * 32;
  gmcore_to_da_kernel<<<grid, threads, 0, stream>>>(ens, num_lat, num_lon, nz, halo, ps, u_half,
                                                    v_half, pt, area_subcell, area_cell, xb);
  return cudaGetLastError();
}

}  // namespace lg
