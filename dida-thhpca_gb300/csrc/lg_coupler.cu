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
// whole globe, so the MCT transfer is one kernel: every output element is one
// thread, members fastest on both sides (coalesced reads and writes).
#include "lg_internal.h"

namespace lg {

namespace {

__global__ void gmcore_to_da_kernel(int ens, int num_lat, int num_lon, int nz, int halo,
                                    const double* ps, const double* u_half, const double* v_half,
                                    const double* pt, const double* area_subcell,
                                    const double* area_cell, double* xb) {
  const int n = 1 + 3 * nz;
  const int nlon_e = num_lon + 2 * halo, nlat_e = num_lat + 2 * halo;
  const size_t total = (size_t)nlon_e * num_lat * n * ens;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t % ens);
    size_t q = t / ens;
    const int row = (int)(q % n);
    q /= n;
    const int jj = (int)(q % num_lat);   // 0-based latitude
    const int le = (int)(q / num_lat);   // 0-based longitude with halo
    int ii = le - halo;                  // 0-based longitude, periodic
    ii = ii < 0 ? ii + num_lon : (ii >= num_lon ? ii - num_lon : ii);
    const size_t cell = ((size_t)jj * num_lon + ii) * ens + m;  // [lat][lon][ens]
    const size_t plane = (size_t)num_lat * num_lon * ens;
    double val;
    if (row == 0) {
      val = ps[cell];
    } else if (row <= nz) {
      const int k = row - 1;
      const int iw = ii == 0 ? num_lon - 1 : ii - 1;
      val = (u_half[k * plane + cell] + u_half[k * plane + ((size_t)jj * num_lon + iw) * ens + m]) / 2;
    } else if (row <= 2 * nz) {
      const int k = row - 1 - nz;
      // v_f at half latitudes 0..num_lat: j - 1 and j around full latitude j (1-based)
      const size_t vplane = (size_t)(num_lat + 1) * num_lon * ens;
      const double vs = v_half[k * vplane + ((size_t)jj * num_lon + ii) * ens + m];
      const double vn = v_half[k * vplane + ((size_t)(jj + 1) * num_lon + ii) * ens + m];
      val = 2 * (vs * area_subcell[2 * jj] + vn * area_subcell[2 * jj + 1]) / area_cell[jj];
    } else {
      const int k = row - 1 - 2 * nz;
      val = pt[k * plane + cell];
    }
    xb[(((size_t)le * nlat_e + (jj + halo)) * n + row) * ens + m] = val;
  }
}

}  // namespace

cudaError_t launch_gmcore_to_da(int ens, int num_lat, int num_lon, int nz, int halo,
                                const double* ps, const double* u_half, const double* v_half,
                                const double* pt, const double* area_subcell,
                                const double* area_cell, double* xb, cudaStream_t stream) {
  gmcore_to_da_kernel<<<152 * 16, 256, 0, stream>>>(ens, num_lat, num_lon, nz, halo, ps, u_half,
                                                     v_half, pt, area_subcell, area_cell, xb);
  return cudaGetLastError();
}

}  // namespace lg
