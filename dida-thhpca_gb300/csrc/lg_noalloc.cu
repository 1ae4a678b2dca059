// lg_noalloc.cu -- lg_core_batch_noalloc: the batched letkf_core without any
// device allocation.
//
// Some callers cannot allocate device memory at the moment they run the core:
// a host framework (a model coupler, an ML runtime) that owns the whole device
// heap through its own pool allocator and forbids any other allocator on the
// device, or a tight assimilation loop in which a cudaMalloc/cudaFree pair per
// call would synchronise the device and serialise the work around it.  For
// them this entry point keeps its working memory -- the per-solve Gram
// matrices, projected innovations and the eigensolver status word -- in one
// file-scope `static __device__` array of fixed size, loaded with the library
// and held by every GPU that loads it until the process exits.
//
// Limits and rules:
//   * capacity: kScratchDoubles doubles (8 MiB); a call needs
//     nbatch * (ens*ens + ens) + 8 of them and is rejected with LG_ERR_SHAPE
//     beyond that (e.g. at most 252 solves of 64 members per call);
//   * the device address of the array is looked up once per device, with that
//     device current, on the first call made on it (cudaGetSymbolAddress), so
//     that first call does set-up work; make it before any stream capture;
//   * every call shares the one array and its contents persist between calls;
//     the status word is cleared at the start of each call, everything else is
//     fully rewritten; calls that overlap on the GPU (different streams, or
//     different host threads) race on the array and must be serialised by the
//     caller;
//   * the inputs and outputs are the caller's device arrays, exactly as for
//     lg_core_batch; nothing here calls cudaMalloc, cudaFree or any allocating
//     library routine.
#include <cuda_runtime.h>

#include <mutex>

#include "lg_internal.h"

namespace {

constexpr size_t kScratchDoubles = (size_t)1 << 20;  // 8 MiB
static __device__ __align__(256) double g_core_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// device address of g_core_scratch on the current device, looked up once
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LG_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_core_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return LG_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return LG_OK;
}

}  // namespace

extern "C" int lg_core_batch_noalloc(int ens, int nbatch, const int* d_nobsl,
                                     const int64_t* d_off, const double* d_hxens,
                                     const float* d_rdiaginv, const double* d_dep,
                                     const double* d_rloc, double inflation, int precision,
                                     double* d_trans, double* d_wbar, void* stream_v) {
  if (ens < 2 || ens > 128 || nbatch < 0 || inflation <= 0.0) return LG_ERR_ARG;
  if (precision != LG_PREC_FP64 && precision != LG_PREC_MIXED) return LG_ERR_ARG;
  if (nbatch == 0) return LG_OK;
  if (!d_nobsl || !d_off || !d_trans || !d_wbar) return LG_ERR_ARG;
  const size_t need = (size_t)nbatch * ((size_t)ens * ens + ens) + 8;
  if (need > kScratchDoubles) return LG_ERR_SHAPE;
  double* scratch = nullptr;
  const int r = scratch_address(&scratch);
  if (r != LG_OK) return r;
  double* C = scratch;
  double* t = C + (size_t)nbatch * ens * ens;
  int* fail = reinterpret_cast<int*>(t + (size_t)nbatch * ens);
  cudaStream_t st = (cudaStream_t)stream_v;

  lg::Geometry geo{};
  geo.ens = ens;
  geo.inflation = inflation;
  geo.vert_dist = -1.0;
  lg::SolveBatch b{};
  b.mode = 1;
  b.nsolves = nbatch;
  b.levels = 1;
  b.b_nobsl = d_nobsl;
  b.b_off = d_off;
  b.b_hx = d_hxens;
  b.b_rdiag = d_rdiaginv;
  b.b_dep = d_dep;
  b.b_rloc = d_rloc;
  lg::HxDev hx{};
  lg::ListDev l{};
  if (cudaMemsetAsync(fail, 0, sizeof(int), st) != cudaSuccess) return LG_ERR_CUDA;
  if (precision == LG_PREC_MIXED && lg::gram_tc_supported(ens))
    lg::launch_gram_tc(geo, hx, l, b, nullptr, C, t, fail, st);
  else
    lg::launch_gram64(geo, hx, l, b, nullptr, C, t, st);
  lg::launch_eig_apply(geo, b, C, t, nullptr, nullptr, nullptr, nullptr, d_trans, d_wbar, fail,
                       st);
  int h_fail = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&h_fail, fail, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return LG_ERR_CUDA;
  if (h_fail < 0) return h_fail;  // a bounded tensor-core wait expired (LG_ERR_TIMEOUT)
  return h_fail ? LG_ERR_EIG : LG_OK;
}
