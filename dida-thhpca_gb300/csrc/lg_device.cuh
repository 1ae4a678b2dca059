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

// Conversions between double and float by integer operations on the bit
// fields, so that they do not issue on the FP64 pipe (a warp instruction per
// ~16 cycles per SM on GB300, which the FP64 kernels beside them need).
// Finite inputs only; values below the float normal range become (signed) zero.

// double -> float, rounded to nearest, ties to even
__device__ inline float d2f_bits(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 of 52 mantissa bits
  const unsigned rest = lo & 0x1fffffffu;                  // the 29 dropped bits
  unsigned bits = ((unsigned)e << 23) | m;
  bits += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // may carry into e
  return __uint_as_float(sign | bits);
}

// float -> double (exact)
__device__ inline double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned ef = (u >> 23) & 0xffu;
  if (ef == 0u) return __hiloint2double((int)sign, 0);
  const unsigned hi = sign | ((ef + (1023u - 127u)) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)((u & 7u) << 29));
}

}  // namespace lg
