// lg_prepost.cu -- the DA caller's work around letkf_run, on the device.
//
// run_da_parallel (x86/DA/EnDNN/src/module_da_parallel.F90:165-263) splits the
// full members into mean and perturbations before the analysis and, after it,
// blends background and analysis (RTPP with gamma1/gamma2), keeps the
// background poleward of da_polar_letkf_lat, zeroes the halo, and reports the
// background and analysis spreads.  Both passes are single streaming sweeps
// over the ensemble (HBM-bound): one warp per (row, column) point, members
// across lanes.
#include "lg_device.cuh"
#include "lg_internal.h"

namespace lg {

// member mean (sum / real(ens), REAL(4) ens) and perturbations; NaN -> error
__global__ void split_mean_kernel(int ens, int64_t npts_rows, const double* xb_in, double* xb,
                                  double* axb, int* err) {
  const int64_t pr = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (pr >= npts_rows) return;
  const int lane = threadIdx.x & 31;
  const double* x = xb_in + (size_t)pr * ens;
  double s = 0.0;
  bool bad = false;
  for (int e = lane; e < ens; e += 32) {
    const double v = x[e];
    bad |= (v != v);
    s += v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicExch(err, LG_ERR_NAN);
    return;
  }
  const double m = s / (double)(float)ens;
  if (lane == 0) axb[pr] = m;
  for (int e = lane; e < ens; e += 32) xb[(size_t)pr * ens + e] = x[e] - m;
}

struct PostArgs {
  int ens, n, num_lat, num_lon, halo;
  double gamma1, gamma2, polar;
  const float* glat;
};

// xa_out, spreads (module_da_parallel.F90:219-257); spread arrays are interior-only
// (n, num_lat, num_lon), n fastest
__global__ void post_kernel(PostArgs a, const double* xb, const double* axb, const double* xa,
                            const double* axa, double* xa_out, double* spread_b,
                            double* spread_a) {
  const int nlat_e = a.num_lat + 2 * a.halo, nlon_e = a.num_lon + 2 * a.halo;
  const int64_t total = (int64_t)nlat_e * nlon_e * a.n;
  const int64_t pr = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (pr >= total) return;
  const int lane = threadIdx.x & 31;
  const int r = (int)(pr % a.n);
  const int64_t cidx = pr / a.n;
  const int li = (int)(cidx % nlat_e), lo = (int)(cidx / nlat_e);  // 0-based with halo
  const int j = li - a.halo + 1, i = lo - a.halo + 1;              // 1-based interior index
  double* out = xa_out + (size_t)pr * a.ens;
  if (i < 1 || i > a.num_lon || j < 1 || j > a.num_lat) {
    for (int e = lane; e < a.ens; e += 32) out[e] = 0.0;
    return;
  }
  const double* b = xb + (size_t)pr * a.ens;
  const double ab = axb[pr];
  double sb = 0.0, sa = 0.0;
  if (fabs((double)a.glat[j - 1]) <= a.polar) {
    const double* x = xa + (size_t)pr * a.ens;
    const double aa = axa[pr];
    for (int e = lane; e < a.ens; e += 32) {
      const double v = a.gamma1 * (ab + b[e]) + a.gamma2 * (aa + x[e]);
      out[e] = v;
      sb += b[e] * b[e];
      sa += (v - aa) * (v - aa);
    }
  } else {
    for (int e = lane; e < a.ens; e += 32) {
      out[e] = b[e] + ab;
      sb += b[e] * b[e];
    }
    sa = sb;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
    sa += __shfl_xor_sync(0xffffffffu, sa, o);
  }
  if (lane == 0) {
    const size_t s = (size_t)r + (size_t)a.n * ((size_t)(j - 1) + (size_t)a.num_lat * (i - 1));
    const double fe = (double)(float)a.ens;
    spread_b[s] = sqrt(sb / fe);
    spread_a[s] = sqrt(sa / fe);
  }
}

void launch_split_mean(int ens, int64_t npts_rows, const double* xb_in, double* xb, double* axb,
                       int* err, cudaStream_t stream) {
  if (npts_rows == 0) return;
  const int warps = 8;
  split_mean_kernel<<<(unsigned)((npts_rows + warps - 1) / warps), 32 * warps, 0, stream>>>(
      ens, npts_rows, xb_in, xb, axb, err);
}

void launch_post(int ens, int n, int num_lat, int num_lon, int halo, double gamma1, double gamma2,
                 double polar, const float* glat, const double* xb, const double* axb,
                 const double* xa, const double* axa, double* xa_out, double* spread_b,
                 double* spread_a, cudaStream_t stream) {
  PostArgs a{ens, n, num_lat, num_lon, halo, gamma1, gamma2, polar, glat};
  const int64_t total = (int64_t)(num_lat + 2 * halo) * (num_lon + 2 * halo) * n;
  const int warps = 8;
  post_kernel<<<(unsigned)((total + warps - 1) / warps), 32 * warps, 0, stream>>>(
      a, xb, axb, xa, axa, xa_out, spread_b, spread_a);
}

// Copy from page-locked host memory that the device can address (a mapped
// host allocation: on a Grace-based GB300 node these loads travel over the
// NVLink chip-to-chip link) into device memory, 16 bytes per load with four
// loads in flight per thread: the copy of lg_run's background when its host
// arrays allow it, instead of one copy-engine transfer.
__global__ void __launch_bounds__(256) copy_mapped_kernel(const uint4* __restrict__ src,
                                                          uint4* __restrict__ dst, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n; i += stride) dst[i] = src[i];
}

cudaError_t launch_copy_mapped(const void* src, void* dst, size_t bytes, cudaStream_t stream) {
  if (bytes == 0) return cudaSuccess;
  const size_t n = bytes / 16;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  copy_mapped_kernel<<<sms * 4, 256, 0, stream>>>(static_cast<const uint4*>(src),
                                                  static_cast<uint4*>(dst), n);
  return cudaGetLastError();
}

}  // namespace lg
