// lg_device.cuh -- device helpers shared by the LETKF kernels.
//
// The precision-sensitive helpers (Gaspari-Cohn, great-circle distance) mirror
// the reference's evaluation order: REAL(4) literals promoted to REAL(8), no
// fused multiply-add.  Every multiply/add below uses the explicit
// round-to-nearest intrinsics (__dmul_rn/__dadd_rn/__dsub_rn/__ddiv_rn) so that
// no contraction can happen whatever the compile flags.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lg {

constexpr int kWarp = 32;

// pi = atan(1.0) * 4 in REAL(4) (x86/DA/utils/pro_info.F90:156)
__host__ __device__ inline double pi_r4() { return (double)3.14159274101257324f; }
// a = 6371.393 REAL(4) literal (pro_info.F90:148)
__host__ __device__ inline double earth_r4() { return (double)6371.393f; }

// schr2: Gaspari-Cohn (x86/DA/LETKF/src/letkf_yb.F90:262-286)
__device__ inline double schr2(double ri) {
  const double c1666 = (double)1.666667f;
  const double c0666 = (double)0.6666667f;
  if (ri > 2.0) return 0.0;
  if (ri > 1.0) {
    double rj = __dsub_rn(__ddiv_rn(ri, 12.0), 0.5);
    rj = __dadd_rn(__dmul_rn(rj, ri), 0.625);
    rj = __dadd_rn(__dmul_rn(rj, ri), c1666);
    double t = __dmul_rn(__dsub_rn(__dmul_rn(rj, ri), 5.0), ri);
    return __dsub_rn(__dadd_rn(t, 4.0), __ddiv_rn(c0666, ri));
  }
  if (ri > 0.0) {
    double rk = __dmul_rn(ri, ri);
    double rj = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(-0.25, ri), 0.5), ri), 0.625);
    return __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(rj, ri), c1666), rk), 1.0);
  }
  return 1.0;
}

// schr: box (letkf_yb.F90:287-302)
__device__ inline double schr(double ri) { return ri > 2.0 ? 0.0 : 1.0; }

__device__ inline double loc_fn(double ri, int gc) { return gc ? schr2(ri) : schr(ri); }

// x/180*pi with the reference's two roundings
__device__ inline double deg2rad_r8(double x) { return __dmul_rn(__ddiv_rn(x, 180.0), pi_r4()); }

// latlon_dist_r8 (pro_info.F90:149-161) from precomputed per-point terms:
// cx = cos(x/180*pi), sx = sin(x/180*pi), yr = y/180*pi, point 1 = observation.
__device__ inline double latlon_dist_pre(double cx1, double sx1, double yr1, double cx2,
                                         double sx2, double yr2) {
  double c3 = cos(__dsub_rn(yr1, yr2));
  double v = __dadd_rn(__dmul_rn(__dmul_rn(cx1, cx2), c3), __dmul_rn(sx1, sx2));
  if (!(v < 1.0)) v = (v != v) ? v : 1.0;
  return __dmul_rn(earth_r4(), acos(v));
}

__device__ inline unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace lg
