// lg_api.cu -- C ABI of the LETKF analysis step (include/letkf_gpu.h).
//
// Host-side responsibilities:
//   * the virtual block decomposition of the reference's DA ranks
//     (pro_info_get_indx, x86/DA/utils/pro_info.F90:96-125) and each block's
//     neighbour-block table (comm_info_init / nearest_dist,
//     x86/DA/LETKF/src/letkf_init.F90:100-164, 288-341), computed once per grid;
//   * the block observation lists that the Redis box query returns
//     (redis_wrapper.c:4158-4296: inclusive %.5f-formatted lon/lat bounds,
//     observations in index order), computed once per observation set;
//   * the analysis pipeline on the device: H(x) -> selection (count, scan,
//     fill) -> per-chunk Gram -> eigensolve + update, all on one stream.
// Host code is compiled with -ffp-contract=off: the neighbour-block distances
// are REAL(4) expressions whose rounding must not change by fusion.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <initializer_list>

#include <algorithm>
#include <thread>
#include <vector>

#include "lg_internal.h"

using lg::Geometry;

struct lg_ctx {
  lg_config cfg;
  int dev = 0;
  cudaStream_t own_stream = nullptr;
  Geometry geo{};
  int x_sec = 0, x_res = 0, y_sec = 0, y_res = 0;
  std::vector<int4> blk;
  std::vector<int> lat_block, lon_block, nb_off, nb_blk;
  std::vector<float> glat, glon;
  std::vector<int> var_start;
  bool have_grid = false, have_obs = false;
  // device geometry
  float *d_glat = nullptr, *d_glon = nullptr;
  double *d_ca = nullptr, *d_cb = nullptr;
  int4* d_blk = nullptr;
  int *d_lat_block = nullptr, *d_lon_block = nullptr, *d_nb_off = nullptr, *d_nb_blk = nullptr;
  // observations
  lg::TypeTable types{};
  lg::ObsDev obs{};
  // device buffers of the observation set, one slot per upload in the fixed
  // order lg_set_obs makes them; a slot is reallocated only when a set outgrows it
  struct ObsSlot {
    void* p = nullptr;
    size_t bytes = 0;
  };
  std::vector<ObsSlot> obs_slots;
  size_t obs_slot_next = 0;
  std::vector<int> h_copy_obs, h_copy_block, h_copy_eoff;
  lg::CellIndex cells{};
  bool have_cells = false;
  // H(x)
  lg::HxDev hx{};
  size_t hx_entries_cap = 0;
  // lists
  lg::ListDev lists{};
  size_t list_cap = 0;
  void* d_scan_tmp = nullptr;
  size_t scan_tmp_bytes = 0;
  int64_t list_total = 0;
  // solve workspace
  // per solve stream: Gram matrices and projected innovations of a chunk, and
  // the lane-parallel eigensolver's scratch (tridiagonal form, eigenvalues,
  // rotation log, overflow list and count)
  struct SolveLane {
    double *C = nullptr, *t = nullptr, *tri = nullptr, *lam = nullptr;
    double2* rot_cs = nullptr;
    unsigned char* rot_i = nullptr;
    int *rot_n = nullptr, *ovf_list = nullptr, *ovf_n = nullptr;
    size_t cap = 0;        // solves
    size_t rot_n_cap = 0;  // rotation-log entries per solve it was sized for
  };
  SolveLane lane[4];
  int rot_cap = 0;
  // extra solve streams (tune.solve_streams 2..4) and their ordering events
  cudaStream_t side_stream = nullptr, third_stream = nullptr, fourth_stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // lg_run: host copies beside the analysis
  cudaEvent_t ev_copy_in = nullptr, ev_copy_join = nullptr;
  // lg_run: the background comes in by longitude pieces, one event after each
  // (H(x) of a group of longitude blocks waits only for the pieces it reads)
  static constexpr int kCopyPieces = 4;
  cudaEvent_t ev_piece[kCopyPieces] = {};
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join3 = nullptr, ev_join4 = nullptr;
  // [Gram, tridiagonalisation (or eigensolve), QL, vectors done][buffer set]
  cudaEvent_t ev_phase[4][4] = {};
  // ln p bucketed records for the mixed-precision Gram
  float4* d_rec = nullptr;
  int* d_boff = nullptr;
  size_t rec_cap = 0;
  float lnp_lo = 0.0f;
  double lnp_span = 1.0;
  int boff_nb = 0;  // bucket count d_boff was sized for
  // launch shapes and bucket boundaries (lg_set_tuning / lg_autotune)
  lg_tuning tune{1024, LG_GRAM_AUTO, 512, 2, 4, 4, 0, 0.0};
  // status words: [0] err, [1] eig_fail, [2] nobsl_max, [3] n_capped
  int* d_status = nullptr;
  unsigned long long* d_band = nullptr;
  // staging for host-array runs
  double *d_xb = nullptr, *d_axb = nullptr, *d_xa = nullptr, *d_axa = nullptr;
  size_t state_elems = 0;
  double *d_xin = nullptr, *d_spb = nullptr, *d_spa = nullptr;  // run_da_parallel staging
  size_t da_elems = 0;
  lg_stats stats{};
  // analysis timing: [0] start, [1] H(x) end, [2] solves start, [3] end,
  // [4] selection start, [5] selection end
  cudaEvent_t ev[6] = {};
  cudaEvent_t ev_hx = nullptr;  // H(x) done (orders the records and Grams after it)
  cudaEvent_t ev_io[4] = {};    // lg_run: around the copy in, around the copy out
  std::vector<cudaEvent_t> kev;  // per-launch events of the solve phase
  unsigned long long* d_work = nullptr;
  // non-zero while the list counts and selection statistics on the device are
  // those prepare_capacity's count pass just computed for the coming analysis
  int* d_fresh = nullptr;
  // sizes fixed for the current observation set, and the captured analysis
  bool capacity_ready = false;
  int chunk = 1;
  // cube solves (cube_n > 1, cube_nz > 1 on the vertical path, or overlap > 0)
  bool cubes = false;
  bool cube_plan = false;
  int cube_ns = 0, cube_cs = 1, cube_ngroups = 1;  // solves, solves per chunk, level groups
  int* d_cube_off = nullptr;
  int *d_s_col = nullptr, *d_s_kk = nullptr, *d_centres = nullptr;
  double* d_trans = nullptr;
  size_t trans_cap = 0;
  bool use_eig2 = false;
  // mixed precision: the vector transform (Xb.W, w-bar) in FP64 from FP64
  // reflectors and rotations instead of FP32 (LETKF_GB300_VEC64=1 at
  // lg_create; a diagnostic that isolates the FP32 transform's share of the
  // mixed path's error)
  bool vec64 = false;
  // analysed columns [col0, col1) (lg_set_columns / lg_set_shard; col1 < 0: all)
  // and the shard's own longitude blocks [shard_by0, shard_by1) (H(x) of
  // lg_hx_device: the copies of those blocks; shard_by1 < 0: every block)
  int col0 = 0, col1 = -1;
  int shard_by0 = 0, shard_by1 = -1;
  int* d_window = nullptr;  // the window's columns, the selection's column list
  size_t window_cap = 0;
  // captured graphs, one per kind of call: [1] H(x) only (lg_hx_device),
  // [2] the analysis after H(x) (lg_analyse_device), [3] both (lg_run*)
  cudaGraphExec_t graph_exec[4] = {};
  const void* graph_key[4][12] = {};
  int64_t graph_launches[4] = {};
  bool graph_failed = false;
};

namespace {

#define CK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      fprintf(stderr, "letkf_gb300: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
      return LG_ERR_CUDA;                                                            \
    }                                                                                \
  } while (0)

// Test hook: LETKF_GB300_ALLOC_LIMIT_MB=m makes every device allocation above
// m MiB fail as an out-of-memory cudaMalloc would, so that the LG_ERR_NOMEM
// paths can be exercised on the host side without exhausting a GPU.
size_t alloc_limit_bytes() {
  const char* e = getenv("LETKF_GB300_ALLOC_LIMIT_MB");
  return e ? (size_t)std::max(0, atoi(e)) << 20 : (size_t)-1;
}

// test hook: LETKF_GB300_QL_ITERS=n caps the QL sweeps per eigenvalue (default 60)
int ql_iter_limit() {
  const char* e = getenv("LETKF_GB300_QL_ITERS");
  return e ? std::max(1, atoi(e)) : 60;
}

template <typename T>
int dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  if (sizeof(T) * n > alloc_limit_bytes()) return LG_ERR_NOMEM;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
  if (e != cudaSuccess) {
    fprintf(stderr, "letkf_gb300: device allocation of %zu bytes failed: %s\n", sizeof(T) * n,
            cudaGetErrorString(e));
    cudaGetLastError();
    return LG_ERR_NOMEM;
  }
  return LG_OK;
}

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

// pro_info_get_indx: x = latitude blocks, y = longitude blocks, 1-based
void get_indx(const lg_ctx* c, int bx, int by, int* tx_s, int* tx_e, int* ty_s, int* ty_e) {
  if (bx - 1 < c->x_res) {
    *tx_s = (bx - 1) * (c->x_sec + 1) + 1;
    *tx_e = *tx_s + c->x_sec;
  } else {
    *tx_s = (bx - 1) * c->x_sec + c->x_res + 1;
    *tx_e = *tx_s + c->x_sec - 1;
  }
  if (by - 1 < c->y_res) {
    *ty_s = (by - 1) * (c->y_sec + 1) + 1;
    *ty_e = *ty_s + c->y_sec;
  } else {
    *ty_s = (by - 1) * c->y_sec + c->y_res + 1;
    *ty_e = *ty_s + c->y_sec - 1;
  }
}

// latlon_dist_r8 on the host (pro_info.F90:149-161)
double host_dist_r8(double x1, double y1, double x2, double y2) {
  const double pi = (double)(atanf(1.0f) * 4.0f);
  const double a = (double)6371.393f;
  double v = cos(x1 / 180.0 * pi) * cos(x2 / 180.0 * pi) * cos(y1 / 180.0 * pi - y2 / 180.0 * pi) +
             sin(x1 / 180.0 * pi) * sin(x2 / 180.0 * pi);
  if (!(v < 1.0)) v = (v != v) ? v : 1.0;
  return a * acos(v);
}

// latlon_dist_r4 (pro_info.F90:163-175)
float host_dist_r4(float x1, float y1, float x2, float y2) {
  const float pi = atanf(1.0f) * 4.0f;
  float v = cosf(x1 / 180.0f * pi) * cosf(x2 / 180.0f * pi) * cosf(y1 / 180.0f * pi - y2 / 180.0f * pi) +
            sinf(x1 / 180.0f * pi) * sinf(x2 / 180.0f * pi);
  if (!(v < 1.0f)) v = (v != v) ? v : 1.0f;
  return 6371.393f * acosf(v);
}

float GL(const lg_ctx* c, int i) { return c->glat[i - 1]; }
float GN(const lg_ctx* c, int i) { return c->glon[i - 1]; }

// nearest_dist (letkf_init.F90:288-341)
double nearest_dist(const lg_ctx* c, int bx1, int by1, int bx2, int by2) {
  int xs1, xe1, ys1, ye1, xs2, xe2, ys2, ye2, tx1, tx2;
  get_indx(c, bx1, by1, &xs1, &xe1, &ys1, &ye1);
  get_indx(c, bx2, by2, &xs2, &xe2, &ys2, &ye2);
  if (bx1 > bx2) {
    tx1 = xs1; tx2 = xe2 + 1;
  } else if (bx1 < bx2) {
    tx1 = xe1 + 1; tx2 = xs2;
  } else if (bx1 > c->cfg.global_nx / 2) {
    tx1 = xe1 + 1; tx2 = xe2 + 1;
  } else {
    tx1 = xs1; tx2 = xs2;
  }
  float lat1 = GL(c, tx1), lat2 = GL(c, tx2);
  const double polar = c->cfg.obs_polar;
  if (fabs((double)lat1) > polar) lat1 = (float)(lat1 >= 0.0f ? fabs(polar) : -fabs(polar));
  if (fabs((double)lat2) > polar) lat2 = (float)(lat2 >= 0.0f ? fabs(polar) : -fabs(polar));
  const int gy = c->cfg.num_lon;
  if (by1 == by2) return (double)host_dist_r4(lat1, GN(c, ys1), lat2, GN(c, ys2));
  float d1 = host_dist_r4(lat1, GN(c, ys1), lat2, GN(c, (ye2 % gy) + 1));
  float d2 = host_dist_r4(lat1, GN(c, (ye1 % gy) + 1), lat2, GN(c, ys2));
  return (double)(d1 < d2 ? d1 : d2);
}

// comm_info_init (letkf_init.F90:100-164): neighbour blocks in traversal order
void neighbour_blocks(const lg_ctx* c, int bx, int by, std::vector<int>& out) {
  const int gnx = c->cfg.global_nx, gny = c->cfg.global_ny;
  const double L = c->cfg.local_dist;
  int s_lat, e_lat, s_lon, e_lon, tx_s, tx_e, ty_s, ty_e;
  get_indx(c, bx, by, &s_lat, &e_lat, &s_lon, &e_lon);
  int north_n = 0, south_n = 0;
  const double y1 = GN(c, s_lon), y2 = y1;
  double x1 = GL(c, s_lat);
  for (int tb = bx - 1; tb > 0; --tb) {
    get_indx(c, tb, by, &tx_s, &tx_e, &ty_s, &ty_e);
    if (host_dist_r8(x1, y1, (double)GL(c, tx_e + 1), y2) > L) break;
    north_n++;
  }
  x1 = GL(c, e_lat + 1);
  for (int tb = bx + 1; tb <= gnx; ++tb) {
    get_indx(c, tb, by, &tx_s, &tx_e, &ty_s, &ty_e);
    if (host_dist_r8(x1, y1, (double)GL(c, tx_s), y2) > L) break;
    south_n++;
  }
  for (int i = -north_n; i <= south_n; ++i) {
    const int tbx = bx + i;
    int west_n = 0, east_n = 0, tby = by;
    while (west_n <= (gny - 1) / 2) {
      tby = ((tby + gny - 2) % gny) + 1;
      if (nearest_dist(c, bx, by, tbx, tby) > L) break;
      west_n++;
    }
    tby = by;
    while (east_n <= (gny - 1) / 2) {
      tby = (tby % gny) + 1;
      if (nearest_dist(c, bx, by, tbx, tby) > L) break;
      east_n++;
    }
    if (west_n + east_n > gny - 1) east_n--;
    for (int j = -west_n; j <= east_n; ++j) {
      const int nby = ((by + j - 1 + gny) % gny) + 1;
      out.push_back((nby - 1) * gnx + (tbx - 1));
    }
  }
}

// Host threads for the observation ingest: one per core, at most 16, and
// none beyond one per min_per items.  LETKF_GB300_HOST_THREADS sets the count
// (at most one per item), which the tests use to compare thread counts.
int host_threads(int64_t n, int64_t min_per) {
  int hw = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  if (const char* env = getenv("LETKF_GB300_HOST_THREADS")) {
    hw = std::max(1, std::min(64, atoi(env)));
    min_per = 1;
  }
  return (int)std::max<int64_t>(1, std::min<int64_t>(hw, n / std::max<int64_t>(1, min_per)));
}

// fn(t, begin, end) over [0, n) in nt contiguous ascending ranges (range t on
// thread t); the same (nt, n) always gives the same ranges.  A range whose
// thread cannot be started runs on the calling thread.
template <typename F>
void run_ranges(int nt, int64_t n, F&& fn) {
  if (nt <= 1) {
    fn(0, (int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  int t = 1;
  try {
    th.reserve(nt - 1);
    for (; t < nt; ++t) th.emplace_back([&fn, t, nt, n] { fn(t, n * t / nt, n * (t + 1) / nt); });
  } catch (...) {
  }
  for (int u = t; u < nt; ++u) fn(u, n * u / nt, n * (u + 1) / nt);
  fn(0, (int64_t)0, n / nt);
  for (auto& x : th) x.join();
}

// %.5f-formatted box bound as the Redis server parses it
double box_bound(float v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.5f", (double)v);
  return strtod(buf, nullptr);
}

void release_streams(lg_ctx* c) {
  for (cudaStream_t* sp : {&c->own_stream, &c->side_stream, &c->third_stream, &c->fourth_stream,
                           &c->copy_stream})
    if (*sp) {
      cudaStreamDestroy(*sp);
      *sp = nullptr;
    }
  for (cudaEvent_t* ep : {&c->ev_fork, &c->ev_join, &c->ev_join3, &c->ev_join4, &c->ev_io[0],
                          &c->ev_io[1], &c->ev_io[2], &c->ev_io[3], &c->ev_copy_in,
                          &c->ev_copy_join})
    if (*ep) {
      cudaEventDestroy(*ep);
      *ep = nullptr;
    }
  for (auto& e : c->ev_piece)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
  for (auto& row : c->ev_phase)
    for (auto& e : row)
      if (e) {
        cudaEventDestroy(e);
        e = nullptr;
      }
}

void drop_graph(lg_ctx* c) {
  for (int i = 0; i < 4; ++i) {
    if (c->graph_exec[i]) cudaGraphExecDestroy(c->graph_exec[i]);
    c->graph_exec[i] = nullptr;
    for (auto& p : c->graph_key[i]) p = nullptr;
  }
}

// forget the observation set (its buffers stay allocated for the next one)
void free_obs(lg_ctx* c) {
  c->obs_slot_next = 0;
  c->obs = lg::ObsDev{};
  c->have_obs = false;
}

void release_obs_memory(lg_ctx* c) {
  for (auto& sl : c->obs_slots)
    if (sl.p) cudaFree(sl.p);
  c->obs_slots.clear();
  free_obs(c);
}

// the next observation buffer of n elements
template <typename T>
int scratch(lg_ctx* c, size_t n, T** out) {
  const size_t bytes = sizeof(T) * std::max<size_t>(n, 1);
  if (c->obs_slot_next == c->obs_slots.size()) c->obs_slots.push_back({});
  lg_ctx::ObsSlot& sl = c->obs_slots[c->obs_slot_next++];
  if (sl.bytes < bytes) {
    if (sl.p) cudaFree(sl.p);
    sl.p = nullptr;
    sl.bytes = 0;
    const size_t want = bytes + bytes / 4;  // headroom for a somewhat larger next set
    if (want > alloc_limit_bytes()) return LG_ERR_NOMEM;
    if (cudaMalloc(&sl.p, want) != cudaSuccess) {
      cudaGetLastError();
      return LG_ERR_NOMEM;
    }
    sl.bytes = want;
  }
  *out = static_cast<T*>(sl.p);
  return LG_OK;
}

template <typename T>
int upload(lg_ctx* c, const T* h, size_t n, const T** out) {
  T* d = nullptr;
  if (scratch(c, n, &d) != LG_OK) return LG_ERR_NOMEM;
  if (n) CK(cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice));
  *out = d;
  return LG_OK;
}

int ensure_hx(lg_ctx* c, size_t entries) {
  if (entries <= c->hx_entries_cap && c->hx.yb) return LG_OK;
  dfree(c->hx.yb); dfree(c->hx.yb32); dfree(c->hx.dis); dfree(c->hx.lnp); dfree(c->hx.rdiag);
  c->hx_entries_cap = 0;  // until every buffer of the new size exists
  const size_t cap = entries + 1;
  const size_t k = (size_t)c->cfg.ens;
  int r = LG_OK;
  r |= dalloc(&c->hx.yb, cap * k);
  if (lg::mixed_precision(c->cfg.precision)) r |= dalloc(&c->hx.yb32, cap * k);
  r |= dalloc(&c->hx.dis, cap);
  r |= dalloc(&c->hx.lnp, cap);
  r |= dalloc(&c->hx.rdiag, cap);
  if (r != LG_OK) return LG_ERR_NOMEM;
  c->hx_entries_cap = cap;
  return LG_OK;
}

// the analysed column range
int col_begin(const lg_ctx* c) { return c->col0; }
int col_end(const lg_ctx* c) {
  return c->col1 < 0 ? c->cfg.num_lat * c->cfg.num_lon : c->col1;
}
bool windowed(const lg_ctx* c) {
  return col_begin(c) != 0 || col_end(c) != c->cfg.num_lat * c->cfg.num_lon;
}

// copies [j0, j1) and entries [e0, e1) of the shard's own blocks: blocks
// b = by * global_nx + bx with by in [shard_by0, shard_by1), contiguous in the
// copy order (block, then type, then observation index)
void shard_copies(const lg_ctx* c, int64_t* j0, int64_t* j1, int64_t* e0, int64_t* e1) {
  const int gnx = c->cfg.global_nx;
  const int by1 = c->shard_by1 < 0 ? c->cfg.global_ny : c->shard_by1;
  const int b0 = c->shard_by0 * gnx, b1 = by1 * gnx;
  const std::vector<int>& cb = c->h_copy_block;
  *j0 = std::lower_bound(cb.begin(), cb.end(), b0) - cb.begin();
  *j1 = std::lower_bound(cb.begin(), cb.end(), b1) - cb.begin();
  *e0 = c->h_copy_eoff.empty() ? 0 : c->h_copy_eoff[*j0];
  *e1 = c->h_copy_eoff.empty() ? 0 : c->h_copy_eoff[*j1];
}

}  // namespace

extern "C" {

const char* lg_status_string(int s) {
  switch (s) {
    case LG_OK: return "LG_OK";
    case LG_ERR_ARG: return "LG_ERR_ARG";
    case LG_ERR_SHAPE: return "LG_ERR_SHAPE";
    case LG_ERR_UNSUPPORTED: return "LG_ERR_UNSUPPORTED";
    case LG_ERR_NAN: return "LG_ERR_NAN";
    case LG_ERR_OBS_OUTSIDE: return "LG_ERR_OBS_OUTSIDE";
    case LG_ERR_VARNAME: return "LG_ERR_VARNAME";
    case LG_ERR_EIG: return "LG_ERR_EIG";
    case LG_ERR_CUDA: return "LG_ERR_CUDA";
    case LG_ERR_NOMEM: return "LG_ERR_NOMEM";
    case LG_ERR_STATE: return "LG_ERR_STATE";
    case LG_ERR_TIMEOUT: return "LG_ERR_TIMEOUT";
    default: return "LG_ERR_UNKNOWN";
  }
}

int lg_create(lg_ctx** out, const lg_config* cfg) {
  if (!out || !cfg) return LG_ERR_ARG;
  *out = nullptr;
  const lg_config& g = *cfg;
  if (g.ens < 2 || g.ens > 128 || g.num_lat < 1 || g.num_lon < 1 || g.nz < 1 || g.halo < 1 ||
      g.n_var < 1 || g.n_var > LG_MAX_VARS || g.global_nx < 1 || g.global_ny < 1 ||
      g.global_nx > g.num_lat || g.global_ny > g.num_lon || g.local_dist <= 0.0 ||
      g.inflation <= 0.0 || g.ps_index < 1)
    return LG_ERR_ARG;
  // cubes (letkf_compute.F90): the loops step by cube_n - overlap
  if (g.cube_n < 1 || g.cube_nz < 1 || g.overlap < 0 || g.overlap >= g.cube_n) return LG_ERR_ARG;
  if (g.precision != LG_PREC_FP64 && !lg::mixed_precision(g.precision)) return LG_ERR_ARG;
  // the TF32 Gram holds [hi; lo] of every member in one M = 128 operand
  if (g.precision == LG_PREC_MIXED_TF32 && !lg::gram_tf32_supported(g.ens))
    return LG_ERR_UNSUPPORTED;
  int rows = 0;
  for (int v = 0; v < g.n_var; ++v) {
    if (g.var_lev[v] != 1 && g.var_lev[v] != g.nz) return LG_ERR_SHAPE;
    rows += g.var_lev[v];
  }
  if (g.ps_index > rows) return LG_ERR_ARG;
  lg_ctx* c = new lg_ctx();
  c->cfg = g;
  // overlapping cubes: letkf_run takes letkf_compute, which has no vertical
  // localisation, whatever da_vert_distance is (letkf.F90:227-235)
  if (g.overlap > 0) c->cfg.vert_dist = 0.0;
  c->cubes = g.cube_n > 1 || g.overlap > 0 || (g.cube_nz > 1 && c->cfg.vert_dist > 0.0);
  c->vec64 = getenv("LETKF_GB300_VEC64") != nullptr;
  cudaGetDevice(&c->dev);
  // Scheduling priorities of the solve streams (Gram, vector update, QL): a
  // level 0 (lowest, the default stream's), 1 or 2 (highest) each.  Pending
  // blocks of a higher-priority stream are dispatched first when SM resources
  // free up; the captured graph keeps them (per-node priorities).  Default:
  // the short vector updates (which free a buffer set for the next Gram) and
  // the latency-bound QL first, the Grams and tridiagonalisations (on the
  // caller's stream) filling the rest; LETKF_GB300_PRIO="g,v,q" overrides.
  int plev[3] = {0, 2, 2};
  if (const char* e = getenv("LETKF_GB300_PRIO"))
    sscanf(e, "%d,%d,%d", &plev[0], &plev[1], &plev[2]);
  int p_least = 0, p_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&p_least, &p_greatest);
  auto prio = [&](int lv) {
    lv = std::max(0, std::min(2, lv));
    return lv == 0 ? p_least : lv == 2 ? p_greatest : (p_least + p_greatest) / 2;
  };
  bool made = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithPriority(&c->side_stream, cudaStreamNonBlocking, prio(plev[0])) ==
                  cudaSuccess &&
              cudaStreamCreateWithPriority(&c->third_stream, cudaStreamNonBlocking, prio(plev[1])) ==
                  cudaSuccess &&
              cudaStreamCreateWithPriority(&c->fourth_stream, cudaStreamNonBlocking, prio(plev[2])) ==
                  cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_join3, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_join4, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreate(&c->ev_io[0]) == cudaSuccess && cudaEventCreate(&c->ev_io[1]) == cudaSuccess &&
              cudaEventCreate(&c->ev_io[2]) == cudaSuccess && cudaEventCreate(&c->ev_io[3]) == cudaSuccess &&
              cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_copy_in, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->ev_copy_join, cudaEventDisableTiming) == cudaSuccess;
  for (auto& row : c->ev_phase)
    for (auto& e : row)
      made = made && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  for (auto& e : c->ev_piece)
    made = made && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!made) {
    cudaGetLastError();
    release_streams(c);
    delete c;
    return LG_ERR_CUDA;
  }
  for (auto& e : c->ev) cudaEventCreate(&e);
  cudaEventCreateWithFlags(&c->ev_hx, cudaEventDisableTiming);
  Geometry& geo = c->geo;
  geo.ens = g.ens;
  geo.num_lat = g.num_lat;
  geo.num_lon = g.num_lon;
  geo.nz = g.nz;
  geo.halo = g.halo;
  geo.n_var = g.n_var;
  int cur = 0;
  for (int v = 0; v < g.n_var; ++v) {
    geo.var_start[v] = cur;
    geo.var_lev[v] = g.var_lev[v];
    cur += g.var_lev[v];
  }
  geo.n = cur;
  geo.ps_row = g.ps_index - 1;
  geo.vcoord = g.vcoord;
  geo.local_dist = g.local_dist;
  geo.vert_dist = c->cfg.vert_dist;  // 0 with overlapping cubes (see above)
  geo.inflation = g.inflation;
  geo.obs_polar = g.obs_polar;
  geo.gc_filter = g.gc_filter;
  geo.gc_filter_vertical = g.gc_filter_vertical;
  geo.max_obs = g.max_obs;
  geo.global_nx = g.global_nx;
  geo.global_ny = g.global_ny;
  geo.nblocks = g.global_nx * g.global_ny;
  geo.ql_max_iter = ql_iter_limit();
  // decomposition (module_da_parallel.F90:84-87 with pro_info_init's argument roles)
  c->x_sec = g.num_lat / g.global_nx;
  c->x_res = g.num_lat % g.global_nx;
  c->y_sec = g.num_lon / g.global_ny;
  c->y_res = g.num_lon % g.global_ny;
  if (dalloc(&c->d_status, 4) != LG_OK || dalloc(&c->d_band, 1) != LG_OK ||
      dalloc(&c->d_work, 1) != LG_OK || dalloc(&c->d_fresh, 1) != LG_OK ||
      cudaMemset(c->d_fresh, 0, sizeof(int)) != cudaSuccess) {
    lg_destroy(c);
    return LG_ERR_NOMEM;
  }
  *out = c;
  return LG_OK;
}

int lg_set_grid(lg_ctx* c, const float* grid_lat, const float* grid_lon, const double* coef_a,
                const double* coef_b, double p0, double ptop) {
  if (!c || !grid_lat || !grid_lon || !coef_a) return LG_ERR_ARG;
  if (c->cfg.vcoord == LG_VCOORD_HYBRID && !coef_b) return LG_ERR_ARG;
  const lg_config& g = c->cfg;
  c->glat.assign(grid_lat, grid_lat + g.num_lat + 1);
  c->glon.assign(grid_lon, grid_lon + g.num_lon + 1);
  c->glat[g.num_lat] = 90.0f;   // pro_info.F90:82-83
  c->glon[g.num_lon] = 360.0f;
  for (int i = 1; i < g.num_lat; ++i)
    if (!(c->glat[i] > c->glat[i - 1])) return LG_ERR_ARG;
  for (int i = 1; i < g.num_lon; ++i)
    if (!(c->glon[i] > c->glon[i - 1])) return LG_ERR_ARG;
  // blocks, column->block maps, neighbour tables
  const int nb = g.global_nx * g.global_ny;
  c->blk.assign(nb, int4{0, 0, 0, 0});
  c->lat_block.assign(g.num_lat, 0);
  c->lon_block.assign(g.num_lon, 0);
  c->nb_off.assign(nb + 1, 0);
  c->nb_blk.clear();
  for (int by = 1; by <= g.global_ny; ++by)
    for (int bx = 1; bx <= g.global_nx; ++bx) {
      const int b = (by - 1) * g.global_nx + (bx - 1);
      int s0, e0, s1, e1;
      get_indx(c, bx, by, &s0, &e0, &s1, &e1);
      c->blk[b] = int4{s0, e0, s1, e1};
      for (int i = s0; i <= e0; ++i) c->lat_block[i - 1] = bx - 1;
      for (int i = s1; i <= e1; ++i) c->lon_block[i - 1] = by - 1;
      neighbour_blocks(c, bx, by, c->nb_blk);
      c->nb_off[b + 1] = (int)c->nb_blk.size();
    }
  dfree(c->d_glat); dfree(c->d_glon); dfree(c->d_ca); dfree(c->d_cb); dfree(c->d_blk);
  dfree(c->d_lat_block); dfree(c->d_lon_block); dfree(c->d_nb_off); dfree(c->d_nb_blk);
  int r = LG_OK;
  r |= dalloc(&c->d_glat, g.num_lat + 1);
  r |= dalloc(&c->d_glon, g.num_lon + 1);
  r |= dalloc(&c->d_ca, g.nz + 1);
  r |= dalloc(&c->d_cb, g.nz + 1);
  r |= dalloc(&c->d_blk, nb);
  r |= dalloc(&c->d_lat_block, g.num_lat);
  r |= dalloc(&c->d_lon_block, g.num_lon);
  r |= dalloc(&c->d_nb_off, nb + 1);
  r |= dalloc(&c->d_nb_blk, c->nb_blk.size());
  if (r != LG_OK) return LG_ERR_NOMEM;
  std::vector<double> cb(g.nz + 1, 0.0);
  if (coef_b) cb.assign(coef_b, coef_b + g.nz + 1);
  CK(cudaMemcpy(c->d_glat, c->glat.data(), sizeof(float) * (g.num_lat + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_glon, c->glon.data(), sizeof(float) * (g.num_lon + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_ca, coef_a, sizeof(double) * (g.nz + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_cb, cb.data(), sizeof(double) * (g.nz + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_blk, c->blk.data(), sizeof(int4) * nb, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_lat_block, c->lat_block.data(), sizeof(int) * g.num_lat, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_lon_block, c->lon_block.data(), sizeof(int) * g.num_lon, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_nb_off, c->nb_off.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
  if (!c->nb_blk.empty())
    CK(cudaMemcpy(c->d_nb_blk, c->nb_blk.data(), sizeof(int) * c->nb_blk.size(), cudaMemcpyHostToDevice));
  Geometry& geo = c->geo;
  geo.p0 = p0;
  geo.ptop = ptop;
  geo.glat = c->d_glat;
  geo.glon = c->d_glon;
  geo.ca = c->d_ca;
  geo.cb = c->d_cb;
  geo.blk = c->d_blk;
  geo.lat_block = c->d_lat_block;
  geo.lon_block = c->d_lon_block;
  geo.nb_off = c->d_nb_off;
  geo.nb_blk = c->d_nb_blk;
  c->have_grid = true;
  return LG_OK;
}

int lg_set_obs(lg_ctx* c, const lg_obs_soa* o) {
  if (!c || !o) return LG_ERR_ARG;
  if (!c->have_grid) return LG_ERR_STATE;
  if (o->n_types < 1 || o->n_types > LG_MAX_OBS_TYPES || o->n_obs < 0) return LG_ERR_ARG;
  if (o->n_obs > 0 && (!o->type || !o->lat || !o->lon || !o->ph || !o->yo || !o->rinv))
    return LG_ERR_ARG;
  const lg_config& g = c->cfg;
  lg::TypeTable tt{};
  tt.n_types = o->n_types;
  for (int t = 0; t < o->n_types; ++t) {
    const lg_obs_type& ty = o->types[t];
    if (ty.nz < 1 || ty.nz > 64 || ty.nvar < 1 || ty.nvar > LG_MAX_OBS_VARS) return LG_ERR_ARG;
    tt.nz[t] = ty.nz;
    tt.nvar[t] = ty.nvar;
    for (int v = 0; v < ty.nvar; ++v) {
      if (ty.var[v] < 0 || ty.var[v] >= g.n_var) return LG_ERR_VARNAME;
      tt.var[t][v] = ty.var[v];
    }
  }
  // no analysis of the previous set may still read its buffers
  CK(cudaDeviceSynchronize());
  free_obs(c);
  c->capacity_ready = false;
  drop_graph(c);
  const int n = o->n_obs, T = o->n_types;
  std::vector<int64_t> ph_off(n + 1, 0), val_off(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    const int t = o->type[i];
    if (t < 0 || t >= T) return LG_ERR_ARG;
    ph_off[i + 1] = ph_off[i] + tt.nz[t];
    val_off[i + 1] = val_off[i] + (int64_t)tt.nz[t] * tt.nvar[t];
  }
  // block box queries: an observation belongs to every block whose inclusive
  // %.5f bounds contain it (1, 2 or 4 blocks)
  const int nb = g.global_nx * g.global_ny;
  std::vector<double> lo_lat(g.global_nx), hi_lat(g.global_nx), lo_lon(g.global_ny), hi_lon(g.global_ny);
  for (int bx = 1; bx <= g.global_nx; ++bx) {
    const int4 b = c->blk[bx - 1];
    lo_lat[bx - 1] = box_bound(GL(c, b.x));
    hi_lat[bx - 1] = box_bound(GL(c, b.y + 1));
  }
  for (int by = 1; by <= g.global_ny; ++by) {
    const int4 b = c->blk[(by - 1) * g.global_nx];
    lo_lon[by - 1] = box_bound(GN(c, b.z));
    hi_lon[by - 1] = box_bound(GN(c, b.w + 1));
  }
  // Counting pass on host threads over contiguous observation ranges, each
  // with its own (block, type) counts; the fill pass gives thread t the slots
  // after those of threads < t in every (block, type) segment, so that the
  // copies of a segment ascend by observation as in a serial pass.
  const size_t nbt = (size_t)nb * T;
  const int nth = host_threads(n, 1 << 15);
  std::vector<std::vector<int>> cnt_t(nth, std::vector<int>(nbt, 0));
  std::vector<int> rows_of(n * 2), cols_of(n * 2);
  std::vector<unsigned char> nrow(n), ncolb(n);
  run_ranges(nth, n, [&](int t, int64_t i0, int64_t i1) {
    int* cnt = cnt_t[t].data();
    for (int i = (int)i0; i < (int)i1; ++i) {
      const double la = o->lat[i], lo = o->lon[i];
      int nr = 0, nc = 0;
      // blocks are contiguous in latitude: binary search for the first
      int a = (int)(std::lower_bound(hi_lat.begin(), hi_lat.end(), la) - hi_lat.begin());
      for (int bx = a; bx < g.global_nx && nr < 2; ++bx) {
        if (la < lo_lat[bx]) break;
        if (la <= hi_lat[bx]) rows_of[2 * i + nr++] = bx;
      }
      int bcol = (int)(std::lower_bound(hi_lon.begin(), hi_lon.end(), lo) - hi_lon.begin());
      for (int by = bcol; by < g.global_ny && nc < 2; ++by) {
        if (lo < lo_lon[by]) break;
        if (lo <= hi_lon[by]) cols_of[2 * i + nc++] = by;
      }
      nrow[i] = (unsigned char)nr;
      ncolb[i] = (unsigned char)nc;
      for (int r = 0; r < nr; ++r)
        for (int q = 0; q < nc; ++q)
          cnt[((size_t)cols_of[2 * i + q] * g.global_nx + rows_of[2 * i + r]) * T + o->type[i]]++;
    }
  });
  std::vector<int> bt_off(nbt + 1, 0);
  for (size_t s = 0; s < nbt; ++s) {
    int run = bt_off[s];
    for (int t = 0; t < nth; ++t) {  // counts -> this thread's first slot
      const int k = cnt_t[t][s];
      cnt_t[t][s] = run;
      run += k;
    }
    bt_off[s + 1] = run;
  }
  const int64_t ncopies = bt_off[nbt];
  c->h_copy_obs.assign(ncopies, 0);
  c->h_copy_block.assign(ncopies, 0);
  run_ranges(nth, n, [&](int t, int64_t i0, int64_t i1) {
    int* fill = cnt_t[t].data();
    for (int i = (int)i0; i < (int)i1; ++i)
      for (int r = 0; r < nrow[i]; ++r)
        for (int q = 0; q < ncolb[i]; ++q) {
          const int b = cols_of[2 * i + q] * g.global_nx + rows_of[2 * i + r];
          const int j = fill[(size_t)b * T + o->type[i]]++;
          c->h_copy_obs[j] = i;
          c->h_copy_block[j] = b;
        }
  });
  c->h_copy_eoff.assign(ncopies + 1, 0);
  int64_t ent = 0;
  for (int64_t j = 0; j < ncopies; ++j) {
    c->h_copy_eoff[j] = (int)ent;
    const int t = o->type[c->h_copy_obs[j]];
    ent += (int64_t)tt.nz[t] * tt.nvar[t];
    if (ent > 0x7fffffff) return LG_ERR_SHAPE;
  }
  c->h_copy_eoff[ncopies] = (int)ent;
  // upload
  lg::ObsDev& d = c->obs;
  d.n_obs = n;
  d.n_copies = ncopies;
  d.n_entries = ent;
  int r = LG_OK;
  r |= upload(c, o->type, n, &d.otype);
  r |= upload(c, o->lat, n, &d.olat);
  r |= upload(c, o->lon, n, &d.olon);
  r |= upload(c, ph_off.data(), n + 1, &d.ph_off);
  r |= upload(c, val_off.data(), n + 1, &d.val_off);
  r |= upload(c, o->ph, (size_t)ph_off[n], &d.oph);
  r |= upload(c, o->yo, (size_t)val_off[n], &d.oyo);
  r |= upload(c, o->rinv, (size_t)val_off[n], &d.orinv);
  r |= upload(c, c->h_copy_obs.data(), ncopies, &d.copy_obs);
  r |= upload(c, c->h_copy_block.data(), ncopies, &d.copy_block);
  r |= upload(c, c->h_copy_eoff.data(), ncopies + 1, &d.copy_eoff);
  r |= upload(c, bt_off.data(), (size_t)nb * T + 1, &d.bt_off);
  double *dcx, *dsx, *dyr;
  float *fcx, *fsx, *fyr;
  r |= scratch(c, n, &dcx);
  r |= scratch(c, n, &dsx);
  r |= scratch(c, n, &dyr);
  r |= scratch(c, n, &fcx);
  r |= scratch(c, n, &fsx);
  r |= scratch(c, n, &fyr);
  if (r != LG_OK) {
    free_obs(c);
    return r < 0 ? r : LG_ERR_NOMEM;
  }
  d.dcx = dcx; d.dsx = dsx; d.dyr = dyr; d.fcx = fcx; d.fsx = fsx; d.fyr = fyr;
  lg::launch_obs_trig(d, dcx, dsx, dyr, fcx, fsx, fyr, c->own_stream);
  {
    // ln p range of the observations (log is monotonic: the logs of the
    // smallest and largest positive pressures)
    double pmin = 1e300, pmax = -1.0;
    for (int64_t i = 0; i < ph_off[n]; ++i) {
      const double v = o->ph[i];
      if (v > 0.0) {
        pmin = std::min(pmin, v);
        pmax = std::max(pmax, v);
      }
    }
    double lo = 0.0, hi = 0.0;
    if (pmax > 0.0) {
      lo = log(pmin);
      hi = log(pmax);
    }
    const double span = std::max(hi - lo, 1e-3) * (1.0 + 1e-6);
    c->lnp_lo = (float)(lo - 1e-6 * span);
    c->lnp_span = span;
  }
  c->types = tt;
  c->geo.n_types = T;
  lg::set_type_table(tt, c->own_stream);
  // cell index of every (block, type) segment for the selection
  {
    const double pi = 3.14159265358979323846;
    const double th = 2.0 * g.local_dist / (double)6371.393f;  // radians
    double cap_deg;
    if (th >= pi) {
      cap_deg = 180.0;
    } else {
      const double v = std::max(-1.0, cos(th) - 2e-5);       // prefilter band included
      cap_deg = acos(v) * 180.0 / pi + 0.01;
    }
    const double cell_deg = std::min(5.0, std::max(0.25, (cap_deg) / 4.0));
    lg::CellIndex& ci = c->cells;
    ci.cell_deg = (float)cell_deg;
    ci.inv_cell = (float)(1.0 / cell_deg);
    ci.cap_deg = (float)cap_deg;
    ci.nrows = (int)ceil(180.0 / cell_deg) + 1;
    ci.ncols = (int)ceil(360.0 / cell_deg) + 1;
    ci.exact_rloc = g.precision == LG_PREC_FP64;
    const int nseg = nb * T;
    std::vector<int4> box(nseg);
    std::vector<int> cell_off(nseg + 1, 0), cell_start, perm(ncopies);
    std::vector<int> rowc(ncopies), colc(ncopies);
    int max_len = 0;
    for (int sg = 0; sg < nseg; ++sg) max_len = std::max(max_len, bt_off[sg + 1] - bt_off[sg]);
    // segments are independent: cells and boxes, then (after the layout of
    // cell_start) the per-segment counting sort, each on host threads
    const int nts = host_threads(nseg, 1);
    run_ranges(nts, nseg, [&](int, int64_t s0, int64_t s1) {
      for (int sg = (int)s0; sg < (int)s1; ++sg) {
        const int j0 = bt_off[sg], j1 = bt_off[sg + 1];
        int r0 = ci.nrows, r1 = -1, c0 = ci.ncols, c1 = -1;
        for (int j = j0; j < j1; ++j) {
          const int oo = c->h_copy_obs[j];
          int r = (int)floorf(((float)o->lat[oo] + 90.0f) * ci.inv_cell);
          int cc = (int)floorf((float)o->lon[oo] * ci.inv_cell);
          r = std::min(std::max(r, 0), ci.nrows - 1);
          cc = std::min(std::max(cc, 0), ci.ncols - 1);
          rowc[j] = r;
          colc[j] = cc;
          r0 = std::min(r0, r); r1 = std::max(r1, r);
          c0 = std::min(c0, cc); c1 = std::max(c1, cc);
        }
        if (j1 == j0) { r0 = 0; r1 = 0; c0 = 0; c1 = 0; }
        box[sg] = int4{r0, r1 - r0 + 1, c0, c1 - c0 + 1};
      }
    });
    {
      size_t base = 0;
      for (int sg = 0; sg < nseg; ++sg) {
        cell_off[sg] = (int)base;
        base += (size_t)box[sg].y * box[sg].w + 1;
      }
      cell_off[nseg] = (int)base;
      cell_start.assign(base, 0);
    }
    run_ranges(nts, nseg, [&](int, int64_t s0, int64_t s1) {
      std::vector<int> fillp;
      for (int sg = (int)s0; sg < (int)s1; ++sg) {
        const int j0 = bt_off[sg], j1 = bt_off[sg + 1];
        const int r0 = box[sg].x, c0 = box[sg].z, ncl = box[sg].w;
        const int ncell = box[sg].y * ncl;
        int* cs = cell_start.data() + cell_off[sg];
        for (int j = j0; j < j1; ++j) cs[(rowc[j] - r0) * ncl + (colc[j] - c0) + 1]++;
        for (int q = 0; q < ncell; ++q) cs[q + 1] += cs[q];
        fillp.assign(cs, cs + ncell);
        for (int j = j0; j < j1; ++j) {  // stable: positions ascend within a cell
          const int cell = (rowc[j] - r0) * ncl + (colc[j] - c0);
          perm[j0 + fillp[cell]++] = j - j0;
        }
      }
    });
    ci.bitmap_words = std::max(1, (max_len + 31) / 32);
    const int4* d_box = nullptr;
    const int *d_cell_off = nullptr, *d_cell_start = nullptr, *d_perm = nullptr;
    int rr = LG_OK;
    rr |= upload(c, box.data(), box.size(), &d_box);
    rr |= upload(c, cell_off.data(), cell_off.size(), &d_cell_off);
    rr |= upload(c, cell_start.data(), cell_start.size(), &d_cell_start);
    rr |= upload(c, perm.data(), perm.size(), &d_perm);
    // per slot: its observation, then the candidate data gathered on the device
    std::vector<int> slot_obs(ncopies);
    run_ranges(nts, nseg, [&](int, int64_t s0, int64_t s1) {
      for (int sg = (int)s0; sg < (int)s1; ++sg)
        for (int j = bt_off[sg]; j < bt_off[sg + 1]; ++j)
          slot_obs[j] = c->h_copy_obs[bt_off[sg] + perm[j]];
    });
    const int* d_slot_obs = nullptr;
    float4* d_cand = nullptr;
    rr |= upload(c, slot_obs.data(), slot_obs.size(), &d_slot_obs);
    rr |= scratch(c, (size_t)ncopies, &d_cand);
    if (rr == LG_OK)
      lg::launch_cell_cands(c->obs, g.obs_polar, d_slot_obs, (int)ncopies, d_cand, c->own_stream);
    ci.cand = d_cand;
    if (rr != LG_OK) {
      free_obs(c);
      return LG_ERR_NOMEM;
    }
    ci.box = d_box;
    ci.cell_off = d_cell_off;
    ci.cell_start = d_cell_start;
    ci.perm = d_perm;
    // one warp's bitmap must fit in shared memory
    c->have_cells = (size_t)ci.bitmap_words * 4 * 4 <= (size_t)200 * 1024;
  }
  CK(cudaStreamSynchronize(c->own_stream));
  if (ensure_hx(c, (size_t)ent) != LG_OK) {
    free_obs(c);
    return LG_ERR_NOMEM;
  }
  c->have_obs = true;
  return LG_OK;
}

namespace {

enum class GramKind { kColumn, kColumnLean, kStream, kQueue };

// Timing events of an analysis go through lg::record_event (lg_internal.h), which
// keeps them valid inside a CUDA-graph capture.
cudaError_t record_event(cudaEvent_t e, cudaStream_t st) { return lg::record_event(e, st); }

// Milliseconds between two completed events; a failed query clears the error
// it raised (it must not surface in a later, unrelated call) and reads as 0.
float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.f;
  }
  return ms;
}

// Sizes every device buffer of the analysis for the current observation set:
// the neighbour lists depend only on the grid and the observation positions,
// so their total is known before any background arrives.  After this, an
// analysis enqueues work only (no host synchronisation, no allocation), which
// lets lg_run_device capture it into a CUDA graph.
// Cubes of each block (cube_n x cube_n columns stepping by cube_n - overlap,
// clipped at the block edge, letkf_compute.F90:52-66, 176-192) and their level
// groups (cube_nz levels on the vertical path, :431-436): the centre column
// ((sj + ej) / 2, (si + ei) / 2) and centre level ((sk + ek) / 2) of every solve.
// Fixed by the grid and configuration, so built once per context.
// mixed precision cube solves form their trans in FP32 from the tridiagonal
// form and the QL rotation log (trans_kernel); FP64 ones with eig_apply
bool cube_trans_fp32(const lg_ctx* c) {
  return lg::mixed_precision(c->cfg.precision) && c->cfg.ens <= 64;
}

int build_cube_plan(lg_ctx* c) {
  if (c->cube_plan) return LG_OK;
  const lg_config& g = c->cfg;
  const int nb = g.global_nx * g.global_ny;
  const int cn = g.cube_n, st = g.cube_n - g.overlap;
  const bool grouped = g.vert_dist > 0.0 && g.overlap == 0;
  const int ng = grouped ? (g.nz + g.cube_nz - 1) / g.cube_nz : 1;
  std::vector<int> off(nb + 1, 0), s_col, s_kk;
  for (int b = 0; b < nb; ++b) {
    const int4 bk = c->blk[b];
    const int nxl = bk.y - bk.x + 1, nyl = bk.w - bk.z + 1;
    const int ncj = (nxl - 1) / st + 1, nci = (nyl - 1) / st + 1;
    off[b + 1] = off[b] + ncj * nci;
    for (int mi = 0; mi < nci; ++mi) {
      const int si = 1 + mi * st, ei = std::min(si + cn - 1, nyl);
      for (int mj = 0; mj < ncj; ++mj) {
        const int sj = 1 + mj * st, ej = std::min(sj + cn - 1, nxl);
        const int glat = bk.x - 1 + (sj + ej) / 2, glon = bk.z - 1 + (si + ei) / 2;
        const int col = (glon - 1) * g.num_lat + (glat - 1);
        for (int gi = 0; gi < ng; ++gi) {
          const int sk = gi * g.cube_nz + 1, ek = std::min(sk + g.cube_nz - 1, g.nz);
          s_col.push_back(col);
          s_kk.push_back(grouped ? (sk + ek) / 2 : 1);
        }
      }
    }
  }
  // the distinct centre columns: the selection builds only their lists
  std::vector<int> centres(s_col);
  std::sort(centres.begin(), centres.end());
  centres.erase(std::unique(centres.begin(), centres.end()), centres.end());
  int r = LG_OK;
  r |= dalloc(&c->d_cube_off, off.size());
  r |= dalloc(&c->d_s_col, s_col.size());
  r |= dalloc(&c->d_s_kk, s_kk.size());
  r |= dalloc(&c->d_centres, centres.size());
  if (r != LG_OK) return LG_ERR_NOMEM;
  CK(cudaMemcpy(c->d_centres, centres.data(), sizeof(int) * centres.size(), cudaMemcpyHostToDevice));
  c->lists.col_list = c->d_centres;
  c->lists.n_list = (int)centres.size();
  CK(cudaMemcpy(c->d_cube_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_s_col, s_col.data(), sizeof(int) * s_col.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_s_kk, s_kk.data(), sizeof(int) * s_kk.size(), cudaMemcpyHostToDevice));
  c->cube_ns = (int)s_col.size();
  c->cube_ngroups = ng;
  c->cube_plan = true;
  return LG_OK;
}

int prepare_capacity(lg_ctx* c) {
  if (c->capacity_ready) return LG_OK;
  const lg_config& g = c->cfg;
  const Geometry& geo = c->geo;
  const int ncol = g.num_lat * g.num_lon;
  const int k = g.ens;
  cudaStream_t st = c->own_stream;
  if (!c->lists.cnt) {
    int r = LG_OK;
    r |= dalloc(&c->lists.cnt, ncol + 1);
    r |= dalloc(&c->lists.off, ncol + 1);
    r |= dalloc(&c->lists.capped, ncol);
    c->scan_tmp_bytes = lg::scan_tmp_bytes(ncol);
    r |= dalloc((char**)&c->d_scan_tmp, c->scan_tmp_bytes);
    if (r != LG_OK) return LG_ERR_NOMEM;
  }
  if (c->cubes) {
    // the cube plan first: only the cube centres' lists are built
    const int r = build_cube_plan(c);
    if (r != LG_OK) return r;
  } else if (windowed(c)) {
    // a column window: the selection builds the window's lists only
    const int n = col_end(c) - col_begin(c);
    if ((size_t)n > c->window_cap) {
      dfree(c->d_window);
      c->window_cap = 0;
      if (dalloc(&c->d_window, (size_t)n) != LG_OK) return LG_ERR_NOMEM;
      c->window_cap = (size_t)n;
    }
    std::vector<int> cols(n);
    for (int i = 0; i < n; ++i) cols[i] = col_begin(c) + i;
    CK(cudaMemcpy(c->d_window, cols.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    c->lists.col_list = c->d_window;
    c->lists.n_list = n;
  } else {
    c->lists.col_list = nullptr;
    c->lists.n_list = 0;
  }
  // The count pass, with the selection statistics, as the analysis runs it: on
  // the cell-indexed path the analysis that follows takes these counts and
  // statistics instead of counting again (d_fresh, cleared by that analysis).
  const bool cells = c->have_cells && !getenv("LETKF_GB300_LINEAR_SEARCH");
  CK(cudaMemsetAsync(c->d_fresh, 0, sizeof(int), st));
  CK(cudaMemsetAsync(c->lists.cnt, 0, sizeof(int) * (ncol + 1), st));
  CK(cudaMemsetAsync(c->d_status + 2, 0, sizeof(int) * 2, st));
  CK(cudaMemsetAsync(c->d_band, 0, sizeof(unsigned long long), st));
  lg::ListDev lcount = c->lists;
  lcount.col_stats = c->d_status + 2;  // nobsl_max, n_capped
  if (cells)
    lg::launch_search_cells(geo, c->obs, c->cells, lcount, 0, c->d_band, st);
  else
    lg::launch_search(geo, c->obs, lcount, 0, c->d_band, st);
  lg::launch_scan_counts(c->lists.cnt, c->lists.off, ncol, c->d_scan_tmp, c->scan_tmp_bytes, st);
  if (cells) CK(cudaMemsetAsync(c->d_fresh, 1, sizeof(int), st));  // done by the sync below
  CK(cudaGetLastError());
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, c->lists.off + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if ((size_t)total > c->list_cap || !c->lists.ent) {
    dfree(c->lists.ent);
    dfree(c->lists.rloc);
    const size_t cap = (size_t)total + 1024;
    if (dalloc(&c->lists.ent, cap) != LG_OK || dalloc(&c->lists.rloc, cap) != LG_OK) {
      c->list_cap = 0;
      return LG_ERR_NOMEM;
    }
    c->list_cap = cap;
  }
  c->list_total = total;
  const bool mixed_tc = lg::mixed_precision(g.precision) && lg::gram_tc_supported(k);
  if (mixed_tc && (c->rec_cap < c->list_cap || !c->d_boff || c->boff_nb != c->tune.lnp_buckets)) {
    dfree(c->d_rec); dfree(c->d_boff);
    int r = LG_OK;
    r |= dalloc(&c->d_rec, c->list_cap);
    r |= dalloc(&c->d_boff, (size_t)ncol * (c->tune.lnp_buckets + 1));
    if (r != LG_OK) { c->rec_cap = 0; c->boff_nb = 0; return LG_ERR_NOMEM; }
    c->rec_cap = c->list_cap;
    c->boff_nb = c->tune.lnp_buckets;
  }
  // solve chunks bounded by the Gram workspace (tune.chunk_mb; LETKF_GB300_CHUNK_MB
  // overrides it, e.g. to keep a profiler capture's device footprint small)
  const int levels = g.vert_dist > 0.0 ? g.nz : 1;
  const size_t per_col = (size_t)levels * k * k * sizeof(double);
  size_t budget = (size_t)c->tune.chunk_mb << 20;
  if (const char* env = getenv("LETKF_GB300_CHUNK_MB")) budget = (size_t)std::max(1, atoi(env)) << 20;
  const int nsel = col_end(c) - col_begin(c);
  c->chunk = (int)std::min<size_t>((size_t)nsel, std::max<size_t>(1, budget / per_col));
  c->use_eig2 = lg::eig2_supported(geo);
  c->rot_cap = 3 * k * k;
  // test hook: a small log forces the overflow fallback path
  if (const char* env = getenv("LETKF_GB300_ROT_CAP")) c->rot_cap = std::max(1, atoi(env));
  // a multiple of 8 entries: the vector kernel reads each solve's log in
  // aligned groups of eight
  c->rot_cap = (c->rot_cap + 7) & ~7;
  if (c->cubes) {
    // cube solves: one buffer set of Gram matrices for a chunk of solves, and
    // every solve's trans (the columns of a cube may take it from several)
    int r = build_cube_plan(c);
    if (r != LG_OK) return r;
    c->cube_cs = (int)std::min<size_t>((size_t)c->cube_ns,
                                       std::max<size_t>(1, budget / ((size_t)k * k * sizeof(double))));
    // mixed precision: tridiagonal form and rotation log for the FP32 trans
    const bool eig2 = cube_trans_fp32(c);
    // two buffer sets: chunks alternate between two streams
    for (int li = 0; li < 2; ++li) {
    lg_ctx::SolveLane& L = c->lane[li];
    if (L.cap < (size_t)c->cube_cs || L.rot_n_cap != (eig2 ? (size_t)c->rot_cap : 0)) {
      dfree(L.C); dfree(L.t); dfree(L.tri); dfree(L.lam); dfree(L.rot_cs); dfree(L.rot_i);
      dfree(L.rot_n); dfree(L.ovf_list); dfree(L.ovf_n);
      L.cap = 0;
      L.rot_n_cap = 0;
      const size_t cap = (size_t)c->cube_cs;
      r |= dalloc(&L.C, cap * k * k);
      r |= dalloc(&L.t, cap * k);
      r |= dalloc(&L.ovf_n, 1);
      if (eig2) {
        r |= dalloc(&L.tri, cap * lg::eig2_tri_doubles(k));
        r |= dalloc(&L.lam, cap * k);
        r |= dalloc(&L.rot_cs, (cap * (size_t)c->rot_cap + 1) / 2);  // float2 entries
        r |= dalloc(&L.rot_i, cap * (size_t)c->rot_cap);
        r |= dalloc(&L.rot_n, cap);
        r |= dalloc(&L.ovf_list, cap);
      }
      if (r != LG_OK) return LG_ERR_NOMEM;
      L.cap = cap;
      L.rot_n_cap = eig2 ? (size_t)c->rot_cap : 0;
    }
    }
    if (c->trans_cap < (size_t)c->cube_ns) {
      dfree(c->d_trans);
      c->trans_cap = 0;
      if (dalloc(&c->d_trans, (size_t)c->cube_ns * k * k) != LG_OK) return LG_ERR_NOMEM;
      c->trans_cap = (size_t)c->cube_ns;
    }
    const int nq = (c->cube_ns + c->cube_cs - 1) / c->cube_cs;
    while ((int)c->kev.size() < 7 * nq) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      c->kev.push_back(e);
    }
    c->capacity_ready = true;
    return LG_OK;
  }
  const int nl = c->tune.solve_streams;
  // rotation log entries: (cos, sin) as two doubles, or two floats where only
  // the FP32 vector kernel replays them (mixed precision)
  const size_t rot_pairs_per_slot = lg::mixed_precision(g.precision) && !c->vec64 ? 2 : 1;
  for (int li = 0; li < 4; ++li) {
    lg_ctx::SolveLane& L = c->lane[li];
    const size_t cap = li < nl ? (size_t)c->chunk * levels : 0;
    if (L.cap >= cap && (cap > 0 || L.cap == 0) && L.rot_n_cap == (size_t)c->rot_cap) continue;
    dfree(L.C); dfree(L.t); dfree(L.tri); dfree(L.lam); dfree(L.rot_cs); dfree(L.rot_i);
    dfree(L.rot_n); dfree(L.ovf_list); dfree(L.ovf_n);
    L.cap = 0;
    L.rot_n_cap = 0;
    if (cap == 0) continue;
    int r = LG_OK;
    r |= dalloc(&L.C, cap * k * k);
    r |= dalloc(&L.t, cap * k);
    r |= dalloc(&L.ovf_n, 1);
    if (c->use_eig2) {
      r |= dalloc(&L.tri, cap * lg::eig2_tri_doubles(k));
      r |= dalloc(&L.lam, cap * k);
      r |= dalloc(&L.rot_cs, (cap * (size_t)c->rot_cap + rot_pairs_per_slot - 1) /
                                 rot_pairs_per_slot);
      r |= dalloc(&L.rot_i, cap * (size_t)c->rot_cap);
      r |= dalloc(&L.rot_n, cap);
      r |= dalloc(&L.ovf_list, cap);
    }
    if (r != LG_OK) return LG_ERR_NOMEM;
    L.cap = cap;
    L.rot_n_cap = (size_t)c->rot_cap;
  }
  const int nchunks = (nsel + c->chunk - 1) / c->chunk;
  while ((int)c->kev.size() < 7 * nchunks) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->kev.push_back(e);
  }
  c->capacity_ready = true;
  return LG_OK;
}

// Host arrays of lg_run whose copies are part of the captured analysis (all
// four pinned): the background goes in on the copy stream beside the
// selection, and each chunk's analysed columns come out as soon as its vector
// update is done, beside the later chunks.
struct HostIO {
  const double *xb, *axb;
  double *xa, *axa;
  // device addresses of xb and axb where the device can read them directly
  // (mapped page-locked memory, 16-byte aligned sizes and addresses): the
  // background then comes in by a copy kernel instead of the copy engine
  const double *xb_map = nullptr, *axb_map = nullptr;
};

// Interior columns [c0, c1) of a [lon + 2 halo][lat + 2 halo][epc] array, device
// to host: a partial first longitude row, the full rows as one 2-D copy, a
// partial last row.
cudaError_t copy_cols_d2h(const lg_config& g, double* dst, const double* src, size_t epc, int c0,
                          int c1, cudaStream_t s) {
  const int nl = g.num_lat, h = g.halo;
  const size_t nlat_e = (size_t)nl + 2 * h, pitch = nlat_e * epc * sizeof(double);
  auto off = [&](int lat, int lon) { return ((size_t)(h + lat) + nlat_e * (size_t)(h + lon)) * epc; };
  int c = c0;
  while (c < c1) {
    const int lon = c / nl, lat = c % nl;
    if (lat == 0 && c + nl <= c1) {  // full rows
      const int rows = (c1 - c) / nl;
      cudaError_t e = cudaMemcpy2DAsync(dst + off(0, lon), pitch, src + off(0, lon), pitch,
                                        (size_t)nl * epc * sizeof(double), rows,
                                        cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) return e;
      c += rows * nl;
    } else {
      const int lat1 = std::min(nl, lat + (c1 - c));
      cudaError_t e = cudaMemcpyAsync(dst + off(lat, lon), src + off(lat, lon),
                                      (size_t)(lat1 - lat) * epc * sizeof(double),
                                      cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) return e;
      c += lat1 - lat;
    }
  }
  return cudaSuccess;
}

// Parts of an analysis: H(x) (of every block copy, or of the shard's own
// copies), and everything after it (selection and solves of the analysed
// columns, with the H(x) in the context's buffers).
enum : int { kPhaseHx = 1, kPhaseAnalysis = 2, kPhaseAll = 3 };

// Every kernel of one analysis, on stream st; no host synchronisation.
int enqueue_analysis(lg_ctx* c, const double* xb, const double* axb, double* xa, double* axa,
                     cudaStream_t st, int64_t* launches_out, const HostIO* io = nullptr,
                     int phases = kPhaseAll, bool own_copies = false) {
  const lg_config& g = c->cfg;
  const Geometry& geo = c->geo;
  const int ncol = g.num_lat * g.num_lon;
  const int k = g.ens;
  int64_t launches = 0;
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(int) * 2, st));  // error, eigensolver failures
  if (phases & kPhaseAnalysis) {
    CK(cudaMemsetAsync(c->d_work, 0, sizeof(unsigned long long), st));
    // the counts and selection statistics (d_status[2..3], d_band), unless
    // prepare_capacity has just computed them for this analysis
    lg::launch_clear_selection(c->d_fresh, c->lists.cnt, ncol + 1, c->d_status + 2, c->d_band,
                               st);
    ++launches;
  }
  CK(record_event(c->ev[0], st));
  // H(x) on the side stream, beside the selection on st (the selection needs
  // only observation positions; the records and Grams wait for H(x))
  CK(cudaEventRecord(c->ev_fork, st));
  CK(cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
  // Copy pieces of the background (lg_run with host arrays, the whole globe's
  // H(x)): up to kCopyPieces groups of longitude blocks; piece p holds the
  // longitudes up to group p's last one + 1, in whole rows of the
  // [lon + 2 halo] arrays, and each row's bytes are a multiple of 16 (the copy
  // kernel's unit).  One piece otherwise.
  const int lon_e = g.num_lon + 2 * g.halo;
  int npiece = 1;
  size_t piece_row[lg_ctx::kCopyPieces + 1] = {0, (size_t)lon_e};
  int piece_by[lg_ctx::kCopyPieces + 1] = {0, g.global_ny};
  if (io && (phases & kPhaseHx) && !own_copies) {
    const size_t row_x = sizeof(double) * (size_t)(g.num_lat + 2 * g.halo) * c->geo.n * k;
    const size_t row_a = sizeof(double) * (size_t)(g.num_lat + 2 * g.halo) * c->geo.n;
    const int np = std::min(lg_ctx::kCopyPieces, g.global_ny);
    if (np > 1 && row_x % 16 == 0 && row_a % 16 == 0) {
      npiece = np;
      for (int p = 0; p <= np; ++p) piece_by[p] = (int)((int64_t)g.global_ny * p / np);
      piece_row[0] = 0;
      for (int p = 1; p < np; ++p) {
        // last longitude (1-based) of the group's last block, then + 1 and the halo
        const int e_lon = c->blk[(size_t)(piece_by[p] - 1) * g.global_nx].w;
        piece_row[p] = std::min<size_t>((size_t)lon_e, (size_t)e_lon + 1 + g.halo);
      }
      piece_row[np] = (size_t)lon_e;
    }
  }
  if (io) {
    // the background in, on the copy stream; H(x) (and everything after it) waits
    const size_t cols = (size_t)(g.num_lat + 2 * g.halo) * (g.num_lon + 2 * g.halo);
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_fork, 0));
    CK(record_event(c->ev_io[0], c->copy_stream));
    const size_t bx = sizeof(double) * cols * c->geo.n * k, ba = sizeof(double) * cols * c->geo.n;
    // rows (longitudes with the halo) of the xb and axb arrays per copy piece
    const size_t rx = bx / lon_e, ra = ba / lon_e;
    for (int p = 0; p < npiece; ++p) {
      const size_t r0 = piece_row[p], r1 = piece_row[p + 1];
      if (io->xb_map && io->axb_map) {
        CK(lg::launch_copy_mapped(io->xb_map + r0 * rx / 8, (double*)xb + r0 * rx / 8,
                                  (r1 - r0) * rx, c->copy_stream));
        CK(lg::launch_copy_mapped(io->axb_map + r0 * ra / 8, (double*)axb + r0 * ra / 8,
                                  (r1 - r0) * ra, c->copy_stream));
        launches += 2;
      } else {
        CK(cudaMemcpyAsync((double*)xb + r0 * rx / 8, io->xb + r0 * rx / 8, (r1 - r0) * rx,
                           cudaMemcpyHostToDevice, c->copy_stream));
        CK(cudaMemcpyAsync((double*)axb + r0 * ra / 8, io->axb + r0 * ra / 8, (r1 - r0) * ra,
                           cudaMemcpyHostToDevice, c->copy_stream));
      }
      if (npiece > 1) CK(cudaEventRecord(c->ev_piece[p], c->copy_stream));
    }
    CK(record_event(c->ev_io[1], c->copy_stream));
    CK(cudaEventRecord(c->ev_copy_in, c->copy_stream));
    if (npiece == 1) CK(cudaStreamWaitEvent(c->side_stream, c->ev_copy_in, 0));
  }
  if (phases & kPhaseHx) {
    int64_t j0 = 0, j1 = c->obs.n_copies, e0 = 0, e1 = 0;
    if (own_copies) shard_copies(c, &j0, &j1, &e0, &e1);
    if (io && npiece > 1) {
      // H(x) of longitude-block group p after copy piece p, which ends at the
      // group's last longitude + 1 (the stencil's eastern column); the pieces
      // before it are in by then
      for (int p = 0; p < npiece; ++p) {
        CK(cudaStreamWaitEvent(c->side_stream, c->ev_piece[p], 0));
        const std::vector<int>& cb = c->h_copy_block;
        const int64_t a = std::lower_bound(cb.begin(), cb.end(), piece_by[p] * g.global_nx) -
                          cb.begin();
        const int64_t b = std::lower_bound(cb.begin(), cb.end(), piece_by[p + 1] * g.global_nx) -
                          cb.begin();
        lg::launch_hx(geo, c->obs, xb, axb, c->hx, c->d_status, c->side_stream, a, b);
        launches += b > a;
      }
      // everything after H(x) (records, Grams, updates) reads the whole background
      CK(cudaStreamWaitEvent(c->side_stream, c->ev_copy_in, 0));
    } else {
      lg::launch_hx(geo, c->obs, xb, axb, c->hx, c->d_status, c->side_stream, j0, j1);
      launches += j1 > j0;
    }
  }
  CK(record_event(c->ev[1], c->side_stream));
  CK(cudaEventRecord(c->ev_hx, c->side_stream));
  if (!(phases & kPhaseAnalysis)) {
    // H(x) only: the selection and solve events are empty intervals
    CK(cudaStreamWaitEvent(st, c->ev_hx, 0));
    for (int e : {4, 5, 2, 3}) CK(record_event(c->ev[e], st));
    CK(cudaGetLastError());
    *launches_out = launches;
    return LG_OK;
  }
  CK(record_event(c->ev[4], st));
  // selection: count, scan, fill (the lists' capacity was sized by prepare_capacity)
  const bool cells = c->have_cells && !getenv("LETKF_GB300_LINEAR_SEARCH");
  lg::ListDev lcount = c->lists;
  lcount.col_stats = c->d_status + 2;  // nobsl_max, n_capped
  if (cells)
    lg::launch_search_cells(geo, c->obs, c->cells, lcount, 0, c->d_band, st, c->d_fresh);
  else
    lg::launch_search(geo, c->obs, lcount, 0, c->d_band, st);
  CK(cudaMemsetAsync(c->d_fresh, 0, sizeof(int), st));  // later analyses count again
  lg::launch_scan_counts(c->lists.cnt, c->lists.off, ncol, c->d_scan_tmp, c->scan_tmp_bytes, st);
  launches += 3;  // count pass + the scan's init and scan kernels
  if (cells)
    lg::launch_search_cells(geo, c->obs, c->cells, c->lists, 1, nullptr, st);
  else
    lg::launch_search(geo, c->obs, c->lists, 1, nullptr, st);
  launches += 1;
  CK(record_event(c->ev[5], st));
  CK(cudaStreamWaitEvent(st, c->ev_hx, 0));
  const bool mixed_tc = lg::mixed_precision(g.precision) && lg::gram_tc_supported(k);
  lg::RecDev rec{};
  if (mixed_tc) {
    const int nb = c->tune.lnp_buckets;
    const float inv_dz = (float)(nb / c->lnp_span);
    lg::launch_records(col_begin(c), col_end(c) - col_begin(c), c->lists, c->hx, c->lnp_lo,
                       inv_dz, nb, c->d_boff, c->d_rec, st);
    launches += 1;
    rec.r = c->d_rec;
    rec.boff = c->d_boff;
    rec.nb = nb;
    rec.lo = c->lnp_lo;
    rec.inv_dz = inv_dz;
  }
  CK(record_event(c->ev[2], st));
  auto finish = [&]() -> int {
    CK(record_event(c->ev[3], st));
    if (io) {
      // the copies not hidden behind the analysis
      CK(record_event(c->ev_io[2], st));
      CK(cudaEventRecord(c->ev_copy_join, c->copy_stream));
      CK(cudaStreamWaitEvent(st, c->ev_copy_join, 0));
      CK(record_event(c->ev_io[3], st));
    }
    CK(cudaGetLastError());
    *launches_out = launches;
    return LG_OK;
  };
  if (c->cubes) {
    // Cube solves, on st: per chunk of solves the Gram at each solve's centre
    // column and level (per-solve kernels) and the solve's explicit trans
    // (FP64 eigensolver); then every column from the cubes that cover it.
    // chunks alternate between st and the side stream, each with its own
    // buffer set, so the Gram of one runs beside the eigensolve of the other
    const int cs = c->cube_cs, ns = c->cube_ns;
    CK(cudaEventRecord(c->ev_fork, st));
    CK(cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
    const cudaStream_t st0 = st;
    for (int q = 0; q * cs < ns; ++q) {
      lg_ctx::SolveLane& L = c->lane[q & 1];
      const cudaStream_t st = (q & 1) ? c->side_stream : st0;  // this chunk's stream
      cudaEvent_t* kv = &c->kev[7 * q];
      lg::SolveBatch b{};
      b.mode = 0;
      b.levels = 1;
      b.s_col = c->d_s_col;
      b.s_kk = c->d_s_kk;
      b.first_solve = q * cs;
      b.nsolves = std::min(cs, ns - q * cs);
      b.work = c->d_work;
      CK(record_event(kv[0], st));
      if (g.precision == LG_PREC_MIXED_TF32)
        lg::launch_gram_tf32(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, rec, st);
      else if (mixed_tc)
        lg::launch_gram_tc_stream(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, rec, st);
      else
        lg::launch_gram64(geo, c->hx, c->lists, b, axb, L.C, L.t, st);
      CK(record_event(kv[1], st));
      CK(record_event(kv[2], st));
      if (cube_trans_fp32(c)) {
        CK(cudaMemsetAsync(L.ovf_n, 0, sizeof(int), st));
        lg::launch_eig2(geo, b, L.C, L.t, xb, axb, xa, axa, L.tri, L.lam, L.rot_cs, L.rot_i,
                        L.rot_n, c->rot_cap, L.ovf_list, L.ovf_n, c->d_status + 1, true,
                        c->tune.ql_warps, c->tune.vec_warps, lg::kEigTridiag | lg::kEigQL, st,
                        kv[3], kv[4]);
        CK(record_event(kv[5], st));
        lg::launch_trans(geo, b, L.t, L.tri, L.lam, L.rot_cs, L.rot_i, L.rot_n, c->rot_cap,
                         c->d_trans, st);
        // solves the QL left to the FP64 solver (log overflow, FP32 reflector range)
        lg::SolveBatch fb = b;
        fb.solve_list = L.ovf_list;
        fb.solve_count = L.ovf_n;
        lg::launch_eig_apply(geo, fb, L.C, L.t, xb, axb, xa, axa, c->d_trans, nullptr,
                             c->d_status + 1, st);
        CK(record_event(kv[6], st));
        launches += 5;
      } else {
        lg::launch_eig_apply(geo, b, L.C, L.t, xb, axb, xa, axa, c->d_trans, nullptr,
                             c->d_status + 1, st);
        for (int e = 3; e < 7; ++e) CK(record_event(kv[e], st));
        launches += 2;
      }
    }
    CK(cudaEventRecord(c->ev_join, c->side_stream));
    CK(cudaStreamWaitEvent(st, c->ev_join, 0));
    const lg::CubeDev cd{g.cube_n, g.cube_nz, g.cube_n - g.overlap, c->cube_ngroups,
                         (g.vert_dist > 0.0 && g.overlap == 0) ? 1 : 0, c->d_cube_off};
    lg::launch_cube_apply(geo, cd, c->d_trans, xb, axb, xa, axa, st);
    launches += 1;
    if (io) {
      CK(cudaEventRecord(c->ev_phase[3][0], st));
      CK(cudaStreamWaitEvent(c->copy_stream, c->ev_phase[3][0], 0));
      CK(copy_cols_d2h(g, io->xa, xa, (size_t)c->geo.n * k, 0, ncol, c->copy_stream));
      CK(copy_cols_d2h(g, io->axa, axa, (size_t)c->geo.n, 0, ncol, c->copy_stream));
    }
    return finish();
  }
  const int levels = g.vert_dist > 0.0 ? g.nz : 1;
  const int chunk = c->chunk;
  const int c0w = col_begin(c), c1w = col_end(c);  // the analysed columns
  const int nchunks = (c1w - c0w + chunk - 1) / chunk;
  // tensor-core Gram variant.  Auto: the lean column Gram beside the phase
  // pipeline's other streams, the full-size one otherwise; per-solve streaming
  // where the column kernel does not apply.
  GramKind gram_kind = !lg::gram_col_supported(k)       ? GramKind::kStream
                       : c->tune.solve_streams >= 3 ? GramKind::kColumnLean
                                                    : GramKind::kColumn;
  if (c->tune.gram_kernel == LG_GRAM_COLUMN && lg::gram_col_supported(k))
    gram_kind = GramKind::kColumn;
  if (c->tune.gram_kernel == LG_GRAM_COLUMN_LEAN && lg::gram_col_supported(k))
    gram_kind = GramKind::kColumnLean;
  if (c->tune.gram_kernel == LG_GRAM_STREAM) gram_kind = GramKind::kStream;
  if (c->tune.gram_kernel == LG_GRAM_QUEUE) gram_kind = GramKind::kQueue;
  if (const char* e = getenv("LETKF_GB300_GRAM")) {
    if (!strcmp(e, "col") && lg::gram_col_supported(k)) gram_kind = GramKind::kColumn;
    if (!strcmp(e, "lean") && lg::gram_col_supported(k)) gram_kind = GramKind::kColumnLean;
    if (!strcmp(e, "stream")) gram_kind = GramKind::kStream;
    if (!strcmp(e, "queue")) gram_kind = GramKind::kQueue;
  }
  // Solve schedule over chunks of columns (tune.solve_streams):
  //   1: every chunk on st;
  //   2: chunks alternate between st and a second stream, each with its own
  //      scratch, so the Gram of one chunk runs beside the eigensolve of another;
  //   3: a phase pipeline over three buffer sets -- Grams on one stream,
  //      tridiagonalisation + QL on st, vectors/update on a third, ordered by
  //      events -- so the FP64 eigensolve of chunk q runs beside the Gram of
  //      chunk q+1 and the vector update of chunk q-1;
  //   4: the same with QL on a stream of its own and four buffer sets, so the
  //      QL of chunk q (latency-bound: one lane per matrix, few warps per SM)
  //      runs beside the tridiagonalisation of chunk q+1 (FP64-pipe-bound).
  // A buffer set is reused by chunk q only after the vector update of chunk
  // q - nl (the last reader of its Gram matrices and eigensolver scratch).
  // Per-chunk timing events (7 per chunk, each on its phase's stream): [0] Gram
  // start, [1] Gram end, [2] eigensolve start, [3] after tridiag, [4] after QL,
  // [5] vectors start, [6] vectors end.
  const int nl = c->tune.solve_streams;
  if (nl >= 2) {
    CK(cudaEventRecord(c->ev_fork, st));
    CK(cudaStreamWaitEvent(c->side_stream, c->ev_fork, 0));
    if (nl >= 3) CK(cudaStreamWaitEvent(c->third_stream, c->ev_fork, 0));
    if (nl == 4) CK(cudaStreamWaitEvent(c->fourth_stream, c->ev_fork, 0));
  }
  const bool fp32_vec = lg::mixed_precision(g.precision) && !c->vec64;
  for (int q = 0; q < nchunks; ++q) {
    const int set = q % nl;
    lg_ctx::SolveLane& L = c->lane[set];
    cudaStream_t s = (nl == 2 && (q & 1)) ? c->side_stream : st;
    cudaStream_t s_g = nl >= 3 ? c->side_stream : s, s_e = s;
    cudaStream_t s_v = nl >= 3 ? c->third_stream : s;
    cudaStream_t s_q = nl == 4 ? c->fourth_stream : s_e;
    cudaEvent_t* kv = &c->kev[7 * q];
    lg::SolveBatch b{};
    b.mode = 0;
    b.first_col = c0w + q * chunk;
    b.ncols = std::min(chunk, c1w - b.first_col);
    b.levels = levels;
    b.nsolves = b.ncols * levels;
    b.work = c->d_work;
    // Gram (phase pipeline: after the buffer set's previous vector update)
    if (nl >= 3 && q >= nl) CK(cudaStreamWaitEvent(s_g, c->ev_phase[3][set], 0));
    CK(record_event(kv[0], s_g));
    if (g.precision == LG_PREC_MIXED_TF32)
      lg::launch_gram_tf32(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, rec, s_g);
    else if (mixed_tc && (gram_kind == GramKind::kColumn || gram_kind == GramKind::kColumnLean))
      lg::launch_gram_col(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, rec,
                          gram_kind == GramKind::kColumnLean, c->tune.gram_ctas, s_g);
    else if (mixed_tc && gram_kind == GramKind::kStream)
      lg::launch_gram_tc_stream(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, rec, s_g);
    else if (mixed_tc)
      lg::launch_gram_tc(geo, c->hx, c->lists, b, axb, L.C, L.t, c->d_status, s_g, &rec);
    else
      lg::launch_gram64(geo, c->hx, c->lists, b, axb, L.C, L.t, s_g);
    CK(cudaMemsetAsync(L.ovf_n, 0, sizeof(int), s_g));
    CK(record_event(kv[1], s_g));
    if (nl >= 3) {
      CK(cudaEventRecord(c->ev_phase[0][set], s_g));
      CK(cudaStreamWaitEvent(s_e, c->ev_phase[0][set], 0));
    }
    CK(record_event(kv[2], s_e));
    if (c->use_eig2) {
      if (s_q == s_e) {
        lg::launch_eig2(geo, b, L.C, L.t, xb, axb, xa, axa, L.tri, L.lam, L.rot_cs, L.rot_i,
                        L.rot_n, c->rot_cap, L.ovf_list, L.ovf_n, c->d_status + 1, fp32_vec,
                        c->tune.ql_warps, c->tune.vec_warps, lg::kEigTridiag | lg::kEigQL, s_e,
                        kv[3], kv[4]);
      } else {
        lg::launch_eig2(geo, b, L.C, L.t, xb, axb, xa, axa, L.tri, L.lam, L.rot_cs, L.rot_i,
                        L.rot_n, c->rot_cap, L.ovf_list, L.ovf_n, c->d_status + 1, fp32_vec,
                        c->tune.ql_warps, c->tune.vec_warps, lg::kEigTridiag, s_e, kv[3],
                        nullptr);
        CK(cudaEventRecord(c->ev_phase[1][set], s_e));
        CK(cudaStreamWaitEvent(s_q, c->ev_phase[1][set], 0));
        lg::launch_eig2(geo, b, L.C, L.t, xb, axb, xa, axa, L.tri, L.lam, L.rot_cs, L.rot_i,
                        L.rot_n, c->rot_cap, L.ovf_list, L.ovf_n, c->d_status + 1, fp32_vec,
                        c->tune.ql_warps, c->tune.vec_warps, lg::kEigQL, s_q, nullptr, kv[4]);
      }
      if (nl >= 3) {
        CK(cudaEventRecord(c->ev_phase[2][set], s_q));
        CK(cudaStreamWaitEvent(s_v, c->ev_phase[2][set], 0));
      }
      CK(record_event(kv[5], s_v));
      lg::launch_eig2(geo, b, L.C, L.t, xb, axb, xa, axa, L.tri, L.lam, L.rot_cs, L.rot_i,
                      L.rot_n, c->rot_cap, L.ovf_list, L.ovf_n, c->d_status + 1, fp32_vec,
                      c->tune.ql_warps, c->tune.vec_warps, lg::kEigVectors, s_v);
      // matrices whose rotation log overflowed: accumulate-eigenvector solver
      lg::SolveBatch fb = b;
      fb.solve_list = L.ovf_list;
      fb.solve_count = L.ovf_n;
      lg::launch_eig_apply(geo, fb, L.C, L.t, xb, axb, xa, axa, nullptr, nullptr,
                           c->d_status + 1, s_v);
      launches += 4;
    } else {
      lg::launch_eig_apply(geo, b, L.C, L.t, xb, axb, xa, axa, nullptr, nullptr,
                           c->d_status + 1, s_e);
      CK(record_event(kv[3], s_e));
      CK(record_event(kv[4], s_e));
      if (nl >= 3) {
        CK(cudaEventRecord(c->ev_phase[2][set], s_e));
        CK(cudaStreamWaitEvent(s_v, c->ev_phase[2][set], 0));
      }
      CK(record_event(kv[5], s_v));
      launches += 1;
    }
    CK(record_event(kv[6], s_v));
    if (nl >= 3 || io) CK(cudaEventRecord(c->ev_phase[3][set], s_v));
    if (io) {
      // this chunk's columns are final: out beside the later chunks
      CK(cudaStreamWaitEvent(c->copy_stream, c->ev_phase[3][set], 0));
      const int c0 = b.first_col, c1 = b.first_col + b.ncols;
      CK(copy_cols_d2h(g, io->xa, xa, (size_t)c->geo.n * k, c0, c1, c->copy_stream));
      CK(copy_cols_d2h(g, io->axa, axa, (size_t)c->geo.n, c0, c1, c->copy_stream));
    }
    launches += 1;
  }
  if (nl >= 2) {
    CK(cudaEventRecord(c->ev_join, c->side_stream));
    CK(cudaStreamWaitEvent(st, c->ev_join, 0));
    if (nl >= 3) {
      CK(cudaEventRecord(c->ev_join3, c->third_stream));
      CK(cudaStreamWaitEvent(st, c->ev_join3, 0));
    }
    if (nl == 4) {
      CK(cudaEventRecord(c->ev_join4, c->fourth_stream));
      CK(cudaStreamWaitEvent(st, c->ev_join4, 0));
    }
  }
  return finish();
}

}  // namespace

namespace {
// One analysis on device arrays; with io, the host copies of lg_run run inside
// it (see HostIO).
int run_analysis(lg_ctx* c, const double* xb, const double* axb, double* xa, double* axa,
                 cudaStream_t st, const HostIO* io, int phases = kPhaseAll,
                 bool own_copies = false) {
  const lg_config& g = c->cfg;
  const int nsel = col_end(c) - col_begin(c);
  lg_stats& S = c->stats;
  memset(&S, 0, sizeof S);
  int r = prepare_capacity(c);
  if (r != LG_OK) return r;
  int64_t launches = 0;
  // The whole analysis is captured once into a CUDA graph per (arrays, stream)
  // and replayed afterwards; LETKF_GB300_NO_GRAPH=1 runs it eagerly.
  const bool graphs = !getenv("LETKF_GB300_NO_GRAPH") && !c->graph_failed;
  const void* key[12] = {xb, axb, xa, axa, st, io ? io->xb : nullptr, io ? io->axb : nullptr,
                         io ? io->xa : nullptr, io ? io->axa : nullptr,
                         (const void*)(intptr_t)c->col0, (const void*)(intptr_t)c->col1,
                         (const void*)(intptr_t)(phases | (own_copies ? 4 : 0) |
                                                 (c->shard_by0 << 3) | ((c->shard_by1 + 1) << 16) |
                                                 ((io && io->xb_map) ? (1 << 30) : 0))};
  bool ran = false;
  if (graphs) {
    cudaGraphExec_t& gx = c->graph_exec[phases];
    if (gx && memcmp(key, c->graph_key[phases], sizeof key) != 0) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
    if (!gx) {
      cudaGraph_t graph = nullptr;
      bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess;
      int er = LG_OK;
      if (ok) er = enqueue_analysis(c, xb, axb, xa, axa, st, &launches, io, phases, own_copies);
      const cudaError_t ee = ok ? cudaStreamEndCapture(st, &graph) : cudaErrorUnknown;
      ok = ok && er == LG_OK && ee == cudaSuccess && graph != nullptr;
      if (ok)
        ok = cudaGraphInstantiateWithFlags(&gx, graph,
                                           cudaGraphInstantiateFlagUseNodePriority) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
      if (!ok) {
        cudaGetLastError();
        gx = nullptr;
        c->graph_failed = true;  // keep running eagerly from now on
      } else {
        memcpy(c->graph_key[phases], key, sizeof key);
        c->graph_launches[phases] = launches;
      }
    }
    if (gx) {
      CK(cudaGraphLaunch(gx, st));
      launches = c->graph_launches[phases];
      ran = true;
    }
  }
  if (!ran) {
    r = enqueue_analysis(c, xb, axb, xa, axa, st, &launches, io, phases, own_copies);
    if (r != LG_OK) return r;
  }
  int status[4];
  unsigned long long band = 0, work = 0;
  CK(cudaMemcpyAsync(status, c->d_status, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&band, c->d_band, sizeof(band), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&work, c->d_work, sizeof(work), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const int nchunks = !(phases & kPhaseAnalysis) ? 0
                      : c->cubes ? (c->cube_ns + c->cube_cs - 1) / c->cube_cs
                                 : (nsel + c->chunk - 1) / c->chunk;
  for (int q = 0; q < nchunks; ++q) {
    const cudaEvent_t* kv = &c->kev[7 * q];
    const float a = elapsed_ms(kv[0], kv[1]);
    const float t1 = elapsed_ms(kv[2], kv[3]);
    const float t2 = elapsed_ms(kv[3], kv[4]);
    const float t3 = elapsed_ms(kv[5], kv[6]);
    S.ms_gram += a;
    S.ms_tridiag += t1;
    S.ms_ql += t2;
    S.ms_vec += t3;
    S.ms_eig += t1 + t2 + t3;
  }
  S.n_chunks = nchunks;
  S.ms_hx = elapsed_ms(c->ev[0], c->ev[1]);
  S.ms_search = elapsed_ms(c->ev[4], c->ev[5]);
  S.ms_solve = elapsed_ms(c->ev[2], c->ev[3]);
  S.ms_total = elapsed_ms(c->ev[0], c->ev[3]);
  S.n_launches = launches;
  S.n_gram_entries = (int64_t)work;
  const bool analysed = (phases & kPhaseAnalysis) != 0;
  S.n_columns = analysed ? nsel : 0;
  S.n_solves = !analysed ? 0
               : c->cubes ? (int64_t)c->cube_ns
                          : (int64_t)nsel * (g.vert_dist > 0.0 ? g.nz : 1);
  S.n_copies = c->obs.n_copies;
  S.n_entries = c->obs.n_entries;
  S.nobsl_total = analysed ? c->list_total : 0;
  S.n_band = analysed ? (int64_t)band : 0;
  S.n_eig_fail = status[1];
  S.nobsl_max = analysed ? status[2] : 0;
  S.n_capped = analysed ? status[3] : 0;
  if (io) {
    S.ms_h2d = elapsed_ms(c->ev_io[0], c->ev_io[1]);
    S.ms_d2h = elapsed_ms(c->ev_io[2], c->ev_io[3]);
  }
  if (status[0] != 0) return status[0];
  // some eigensolve hit the sweep limit: the analysis is written (the
  // reference prints dsyevd's ierr and goes on), the caller is told
  if (status[1] != 0) return LG_ERR_EIG;
  return LG_OK;
}

bool pinned(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// the device address of page-locked host memory p of `bytes` bytes, when the
// device can read it directly and address and size are 16-byte multiples;
// nullptr otherwise (LETKF_GB300_COPY_ENGINE=1 always gives nullptr)
const double* mapped(const void* p, size_t bytes) {
  if (getenv("LETKF_GB300_COPY_ENGINE")) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
  if (((uintptr_t)a.devicePointer | bytes) % 16 != 0) return nullptr;
  return static_cast<const double*>(a.devicePointer);
}
}  // namespace

int lg_run_device(lg_ctx* c, int ntimes, const double* xb, const double* axb, double* xa,
                  double* axa, void* stream_v) {
  (void)ntimes;
  if (!c || !xb || !axb || !xa || !axa) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  return run_analysis(c, xb, axb, xa, axa, st, nullptr);
}

int lg_set_wait_limit(lg_ctx* c, int64_t ns) {
  if (!c || ns < 0) return LG_ERR_ARG;
  c->geo.tc_wait_ns = ns;
  drop_graph(c);  // the limit is a kernel argument of the captured analysis
  return LG_OK;
}

int lg_list_counts(lg_ctx* c, int* counts, int64_t* total) {
  if (!c || !counts) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  if (c->cubes) return LG_ERR_UNSUPPORTED;
  const int ncol = c->cfg.num_lat * c->cfg.num_lon;
  if (!c->lists.cnt) {
    int r = LG_OK;
    r |= dalloc(&c->lists.cnt, ncol + 1);
    r |= dalloc(&c->lists.off, ncol + 1);
    r |= dalloc(&c->lists.capped, ncol);
    c->scan_tmp_bytes = lg::scan_tmp_bytes(ncol);
    r |= dalloc((char**)&c->d_scan_tmp, c->scan_tmp_bytes);
    if (r != LG_OK) return LG_ERR_NOMEM;
  }
  cudaStream_t st = c->own_stream;
  lg::ListDev l = c->lists;
  l.col_list = nullptr;  // every column
  l.n_list = 0;
  CK(cudaMemsetAsync(c->d_fresh, 0, sizeof(int), st));  // the counts are overwritten
  CK(cudaMemsetAsync(l.cnt, 0, sizeof(int) * (ncol + 1), st));
  if (c->have_cells && !getenv("LETKF_GB300_LINEAR_SEARCH"))
    lg::launch_search_cells(c->geo, c->obs, c->cells, l, 0, nullptr, st);
  else
    lg::launch_search(c->geo, c->obs, l, 0, nullptr, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(counts, l.cnt, sizeof(int) * ncol, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (total) {
    int64_t t = 0;
    for (int i = 0; i < ncol; ++i) t += counts[i];
    *total = t;
  }
  c->capacity_ready = false;  // the next analysis recounts its own columns
  drop_graph(c);              // and recaptures against whatever it sizes
  return LG_OK;
}

int lg_set_columns(lg_ctx* c, int col_begin, int col_end) {
  if (!c) return LG_ERR_ARG;
  const int ncol = c->cfg.num_lat * c->cfg.num_lon;
  if (col_begin < 0 || col_end > ncol || col_begin >= col_end) return LG_ERR_ARG;
  if (c->cubes && (col_begin != 0 || col_end != ncol)) return LG_ERR_UNSUPPORTED;
  c->col0 = col_begin;
  c->col1 = col_end;
  c->shard_by0 = 0;
  c->shard_by1 = -1;
  c->capacity_ready = false;
  drop_graph(c);
  return LG_OK;
}

int lg_set_shard(lg_ctx* c, int lon_block_begin, int lon_block_end) {
  if (!c) return LG_ERR_ARG;
  if (!c->have_grid) return LG_ERR_STATE;
  const lg_config& g = c->cfg;
  if (lon_block_begin < 0 || lon_block_end > g.global_ny || lon_block_begin >= lon_block_end)
    return LG_ERR_ARG;
  // the blocks' longitudes, all latitudes (pro_info_get_indx with bx = 1)
  int s0, e0, lon_s, lon_e, s1, e1, lon_s2, lon_e2;
  get_indx(c, 1, lon_block_begin + 1, &s0, &e0, &lon_s, &lon_e);
  get_indx(c, 1, lon_block_end, &s1, &e1, &lon_s2, &lon_e2);
  const int r = lg_set_columns(c, (lon_s - 1) * g.num_lat, lon_e2 * g.num_lat);
  if (r != LG_OK) return r;
  c->shard_by0 = lon_block_begin;
  c->shard_by1 = lon_block_end;
  return LG_OK;
}

int lg_shard_entries(const lg_ctx* c, int64_t* entry_begin, int64_t* entry_end,
                     int64_t* n_entries) {
  if (!c || !entry_begin || !entry_end) return LG_ERR_ARG;
  if (!c->have_obs) return LG_ERR_STATE;
  int64_t j0, j1;
  shard_copies(c, &j0, &j1, entry_begin, entry_end);
  if (n_entries) *n_entries = c->obs.n_entries;
  return LG_OK;
}

int lg_hx_device(lg_ctx* c, const double* xb, const double* axb, void* stream_v) {
  if (!c || !xb || !axb) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  return run_analysis(c, xb, axb, nullptr, nullptr, st, nullptr, kPhaseHx, true);
}

int lg_analyse_device(lg_ctx* c, const double* xb, const double* axb, double* xa, double* axa,
                      void* stream_v) {
  if (!c || !xb || !axb || !xa || !axa) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  return run_analysis(c, xb, axb, xa, axa, st, nullptr, kPhaseAnalysis, false);
}

int lg_hx_export(const lg_ctx* c, double* d_rows, void* stream_v) {
  if (!c || !d_rows) return LG_ERR_ARG;
  if (!c->have_obs) return LG_ERR_STATE;
  int64_t j0, j1, e0, e1;
  shard_copies(c, &j0, &j1, &e0, &e1);
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  lg::launch_hx_export(c->cfg.ens, e0, e1, c->hx, d_rows, st);
  CK(cudaGetLastError());
  return LG_OK;
}

int lg_hx_import(lg_ctx* c, const double* d_rows, int64_t entry_begin, int64_t entry_end,
                 void* stream_v) {
  if (!c || (!d_rows && entry_end > entry_begin)) return LG_ERR_ARG;
  if (!c->have_obs) return LG_ERR_STATE;
  if (entry_begin < 0 || entry_end < entry_begin || entry_end > c->obs.n_entries)
    return LG_ERR_SHAPE;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  lg::launch_hx_import(c->cfg.ens, entry_begin, entry_end, c->hx, d_rows, st);
  CK(cudaGetLastError());
  return LG_OK;
}

int lg_run(lg_ctx* c, int ntimes, const double* xb, const double* axb, double* xa, double* axa) {
  if (!c || !xb || !axb || !xa || !axa) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  const lg_config& g = c->cfg;
  const size_t nlat_e = g.num_lat + 2 * g.halo, nlon_e = g.num_lon + 2 * g.halo;
  const size_t cols = nlat_e * nlon_e;
  const size_t n = c->geo.n, k = g.ens;
  if (c->state_elems < cols * n * k) {
    dfree(c->d_xb); dfree(c->d_axb); dfree(c->d_xa); dfree(c->d_axa);
    int r = LG_OK;
    r |= dalloc(&c->d_xb, cols * n * k);
    r |= dalloc(&c->d_xa, cols * n * k);
    r |= dalloc(&c->d_axb, cols * n);
    r |= dalloc(&c->d_axa, cols * n);
    if (r != LG_OK) { c->state_elems = 0; return LG_ERR_NOMEM; }
    c->state_elems = cols * n * k;
  }
  cudaStream_t st = c->own_stream;
  if (pinned(xb) && pinned(axb) && pinned(xa) && pinned(axa)) {
    // page-locked host arrays: the copies run inside the analysis, overlapped
    HostIO io{xb, axb, xa, axa};
    io.xb_map = mapped(xb, sizeof(double) * cols * n * k);
    io.axb_map = mapped(axb, sizeof(double) * cols * n);
    return run_analysis(c, c->d_xb, c->d_axb, c->d_xa, c->d_axa, st, &io);
  }
  CK(cudaEventRecord(c->ev_io[0], st));
  CK(cudaMemcpyAsync(c->d_xb, xb, sizeof(double) * cols * n * k, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_axb, axb, sizeof(double) * cols * n, cudaMemcpyHostToDevice, st));
  CK(cudaEventRecord(c->ev_io[1], st));
  int r = lg_run_device(c, ntimes, c->d_xb, c->d_axb, c->d_xa, c->d_axa, st);
  if (r != LG_OK) return r;
  // the analysed interior columns only (every interior column unless a window
  // is set): for each longitude the interior latitudes are contiguous
  CK(cudaEventRecord(c->ev_io[2], st));
  CK(copy_cols_d2h(g, xa, c->d_xa, n * k, col_begin(c), col_end(c), st));
  CK(copy_cols_d2h(g, axa, c->d_axa, n, col_begin(c), col_end(c), st));
  CK(cudaEventRecord(c->ev_io[3], st));
  CK(cudaStreamSynchronize(st));
  c->stats.ms_h2d = elapsed_ms(c->ev_io[0], c->ev_io[1]);
  c->stats.ms_d2h = elapsed_ms(c->ev_io[2], c->ev_io[3]);
  return LG_OK;
}

int lg_split_mean_device(lg_ctx* c, const double* d_xb_in, double* d_xb, double* d_axb,
                         void* stream_v) {
  if (!c || !d_xb_in || !d_xb || !d_axb) return LG_ERR_ARG;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  const lg_config& g = c->cfg;
  const int64_t rows =
      (int64_t)(g.num_lat + 2 * g.halo) * (g.num_lon + 2 * g.halo) * (int64_t)c->geo.n;
  int h_err = 0;
  CK(cudaMemsetAsync(c->d_status + 3, 0, sizeof(int), st));
  lg::launch_split_mean(g.ens, rows, d_xb_in, d_xb, d_axb, c->d_status + 3, st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&h_err, c->d_status + 3, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return h_err;
}

int lg_post_device(lg_ctx* c, double gamma1, double gamma2, double polar_lat, const double* d_xb,
                   const double* d_axb, const double* d_xa, const double* d_axa,
                   double* d_xa_out, double* d_spread_b, double* d_spread_a, void* stream_v) {
  if (!c || !d_xb || !d_axb || !d_xa || !d_axa || !d_xa_out || !d_spread_b || !d_spread_a)
    return LG_ERR_ARG;
  if (!c->have_grid) return LG_ERR_STATE;
  cudaStream_t st = stream_v ? (cudaStream_t)stream_v : c->own_stream;
  const lg_config& g = c->cfg;
  lg::launch_post(g.ens, c->geo.n, g.num_lat, g.num_lon, g.halo, gamma1, gamma2, polar_lat,
                  c->d_glat, d_xb, d_axb, d_xa, d_axa, d_xa_out, d_spread_b, d_spread_a, st);
  CK(cudaGetLastError());
  return LG_OK;
}

int lg_run_da_parallel(lg_ctx* c, int ntimes, double gamma1, double gamma2, double polar_lat,
                       const double* xb_in, double* xa_out, double* spread_b, double* spread_a) {
  if (!c || !xb_in || !xa_out || !spread_b || !spread_a) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  // the blend and spreads cover the whole globe: not with a column window or shard
  if (windowed(c)) return LG_ERR_UNSUPPORTED;
  const lg_config& g = c->cfg;
  const size_t cols = (size_t)(g.num_lat + 2 * g.halo) * (g.num_lon + 2 * g.halo);
  const size_t n = c->geo.n, k = g.ens;
  const size_t inner = (size_t)g.num_lat * g.num_lon * n;
  if (c->state_elems < cols * n * k) {
    dfree(c->d_xb); dfree(c->d_axb); dfree(c->d_xa); dfree(c->d_axa);
    int r = LG_OK;
    r |= dalloc(&c->d_xb, cols * n * k);
    r |= dalloc(&c->d_xa, cols * n * k);
    r |= dalloc(&c->d_axb, cols * n);
    r |= dalloc(&c->d_axa, cols * n);
    if (r != LG_OK) { c->state_elems = 0; return LG_ERR_NOMEM; }
    c->state_elems = cols * n * k;
  }
  if (c->da_elems < cols * n * k) {
    dfree(c->d_xin); dfree(c->d_spb); dfree(c->d_spa);
    int r = LG_OK;
    r |= dalloc(&c->d_xin, cols * n * k);
    r |= dalloc(&c->d_spb, inner);
    r |= dalloc(&c->d_spa, inner);
    if (r != LG_OK) { c->da_elems = 0; return LG_ERR_NOMEM; }
    c->da_elems = cols * n * k;
  }
  cudaStream_t st = c->own_stream;
  CK(cudaMemcpyAsync(c->d_xin, xb_in, sizeof(double) * cols * n * k, cudaMemcpyHostToDevice, st));
  int r = lg_split_mean_device(c, c->d_xin, c->d_xb, c->d_axb, st);
  if (r != LG_OK) return r;
  r = lg_run_device(c, ntimes, c->d_xb, c->d_axb, c->d_xa, c->d_axa, st);
  if (r != LG_OK) return r;
  r = lg_post_device(c, gamma1, gamma2, polar_lat, c->d_xb, c->d_axb, c->d_xa, c->d_axa,
                     c->d_xin, c->d_spb, c->d_spa, st);
  if (r != LG_OK) return r;
  CK(cudaMemcpyAsync(xa_out, c->d_xin, sizeof(double) * cols * n * k, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(spread_b, c->d_spb, sizeof(double) * inner, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(spread_a, c->d_spa, sizeof(double) * inner, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return LG_OK;
}

int lg_get_tuning(const lg_ctx* c, lg_tuning* out) {
  if (!c || !out) return LG_ERR_ARG;
  *out = c->tune;
  return LG_OK;
}

int lg_set_tuning(lg_ctx* c, const lg_tuning* t) {
  if (!c || !t) return LG_ERR_ARG;
  if (t->chunk_mb < 16 || t->chunk_mb > 65536 || t->gram_kernel < LG_GRAM_AUTO ||
      t->gram_kernel > LG_GRAM_COLUMN_LEAN || t->lnp_buckets < 8 || t->lnp_buckets > 1024 ||
      t->ql_warps < 1 || t->ql_warps > 6 || t->vec_warps < 1 || t->vec_warps > 8 ||
      t->solve_streams < 1 || t->solve_streams > 4 || t->gram_ctas < 0 || t->gram_ctas > 4096)
    return LG_ERR_ARG;
  c->tune = *t;
  c->capacity_ready = false;  // chunk size and bucket count size buffers
  drop_graph(c);
  return LG_OK;
}

int lg_autotune(lg_ctx* c, const double* xb, const double* axb, double* xa, double* axa,
                void* stream, lg_tuning* best) {
  if (!c || !xb || !axb || !xa || !axa || !best) return LG_ERR_ARG;
  if (!c->have_grid || !c->have_obs) return LG_ERR_STATE;
  const lg_config& g = c->cfg;
  const bool mixed = g.precision == LG_PREC_MIXED;  // the BF16 Gram variants to tune
  const bool vertical = g.vert_dist > 0.0;
  lg_tuning cur = c->tune;
  if (cur.gram_kernel == LG_GRAM_AUTO)
    cur.gram_kernel = !lg::gram_col_supported(g.ens) ? LG_GRAM_STREAM
                      : cur.solve_streams >= 3          ? LG_GRAM_COLUMN_LEAN
                                                        : LG_GRAM_COLUMN;
  // one untimed analysis (buffer sizing, graph capture), then the faster of two
  auto measure = [&](const lg_tuning& t, double* ms) -> int {
    int r = lg_set_tuning(c, &t);
    if (r != LG_OK) return r;
    if ((r = lg_run_device(c, 0, xb, axb, xa, axa, stream)) != LG_OK) return r;
    double m = 1e300;
    for (int rep = 0; rep < 2; ++rep) {
      if ((r = lg_run_device(c, 0, xb, axb, xa, axa, stream)) != LG_OK) return r;
      m = std::min(m, c->stats.ms_total);
    }
    *ms = m;
    return LG_OK;
  };
  double best_ms = 0.0;
  int r = measure(cur, &best_ms);
  if (r != LG_OK) return r;
  auto try_param = [&](int lg_tuning::*field, std::initializer_list<int> cands) -> int {
    for (int v : cands) {
      if (cur.*field == v) continue;
      lg_tuning t = cur;
      t.*field = v;
      double ms = 0.0;
      const int rr = measure(t, &ms);
      if (rr == LG_ERR_NOMEM) {  // the candidate does not fit next to the resident data
        cudaGetLastError();
        continue;
      }
      if (rr != LG_OK) return rr;
      if (ms < best_ms) {
        best_ms = ms;
        cur = t;
      }
    }
    return LG_OK;
  };
  if ((r = try_param(&lg_tuning::solve_streams, {1, 2, 3, 4})) != LG_OK) return r;
  if ((r = try_param(&lg_tuning::chunk_mb, {256, 512, 1024, 2048, 4096})) != LG_OK) return r;
  if (mixed) {
    if (lg::gram_col_supported(g.ens)) {
      if ((r = try_param(&lg_tuning::gram_kernel, {LG_GRAM_COLUMN, LG_GRAM_COLUMN_LEAN,
                                                   LG_GRAM_STREAM, LG_GRAM_QUEUE})) != LG_OK)
        return r;
    } else if ((r = try_param(&lg_tuning::gram_kernel, {LG_GRAM_STREAM, LG_GRAM_QUEUE})) != LG_OK) {
      return r;
    }
    if (vertical && (r = try_param(&lg_tuning::lnp_buckets, {32, 64, 128, 256, 512})) != LG_OK)
      return r;
    if ((cur.gram_kernel == LG_GRAM_COLUMN || cur.gram_kernel == LG_GRAM_COLUMN_LEAN) &&
        (r = try_param(&lg_tuning::gram_ctas, {0, 76, 114})) != LG_OK)
      return r;
  }
  if ((r = try_param(&lg_tuning::ql_warps, {1, 2, 4})) != LG_OK) return r;
  if ((r = try_param(&lg_tuning::vec_warps, {2, 4, 8})) != LG_OK) return r;

  cur.ms = best_ms;
  if ((r = lg_set_tuning(c, &cur)) != LG_OK) return r;
  // leave the context sized and captured for the chosen settings
  if ((r = lg_run_device(c, 0, xb, axb, xa, axa, stream)) != LG_OK) return r;
  *best = cur;
  return LG_OK;
}

int lg_get_stats(const lg_ctx* c, lg_stats* st) {
  if (!c || !st) return LG_ERR_ARG;
  *st = c->stats;
  return LG_OK;
}

int lg_gmcore_to_da_device(int ens, int num_lat, int num_lon, int nz, int halo,
                           const double* d_ps, const double* d_u_half, const double* d_v_half,
                           const double* d_pt, const double* d_area_subcell,
                           const double* d_area_cell, double* d_xb, void* stream) {
  if (ens < 1 || ens > 1024 || num_lat < 1 || num_lat > 65535 || num_lon < 1 || nz < 1 ||
      halo < 0 || halo > num_lon)
    return LG_ERR_ARG;
  if (!d_ps || !d_u_half || !d_v_half || !d_pt || !d_area_subcell || !d_area_cell || !d_xb)
    return LG_ERR_ARG;
  CK(lg::launch_gmcore_to_da(ens, num_lat, num_lon, nz, halo, d_ps, d_u_half, d_v_half, d_pt,
                             d_area_subcell, d_area_cell, d_xb, (cudaStream_t)stream));
  return LG_OK;
}

int lg_obs_from_records(int nz, int nvar, int n_records, const float* lon, const float* lat,
                        const float* lev, const float* val, const float* noise, int max_obs,
                        int* n_obs, double* lat_out, double* lon_out, double* ph_out,
                        double* yo_out, double* rinv_out) {
  if (nz < 1 || nz > 64 || nvar < 1 || nvar > LG_MAX_OBS_VARS || n_records < 0 || max_obs < 0 ||
      !n_obs)
    return LG_ERR_ARG;
  if (n_records > 0 && (!lon || !lat || !lev || !val)) return LG_ERR_ARG;
  if (max_obs > 0 && (!lat_out || !lon_out || !ph_out || !yo_out || !rinv_out)) return LG_ERR_ARG;
  const int nval = 2 * nvar + 1;
  int idx = -1;           // current observation
  int next_level = 1;     // profiles: the level the next record must fill
  for (int r = 0; r < n_records; ++r) {
    const float lv = lev[r];
    const int l = (int)lv;
    if ((float)l != lv || l < 1 || l > nz) return LG_ERR_SHAPE;
    if (l == 1) {
      if (idx >= 0 && next_level != nz + 1) return LG_ERR_SHAPE;  // previous profile incomplete
      ++idx;
      if (idx >= max_obs) return LG_ERR_SHAPE;
      lat_out[idx] = (double)lat[r];
      lon_out[idx] = (double)lon[r];
      next_level = 1;
    }
    if (idx < 0 || l != next_level) return LG_ERR_SHAPE;  // levels in order 1..nz
    ++next_level;
    const float* v = val + (size_t)r * nval;
    ph_out[(size_t)idx * nz + (l - 1)] = (double)v[2 * nvar];
    for (int n = 0; n < nvar; ++n) {
      const float sd = v[2 * n + 1];
      // REAL(4): val_buf(2n-1) + randn * val_buf(2n);  1.0 / val_buf(2n)**2
      const float pert = noise ? noise[(size_t)n * n_records + r] * sd : 0.0f;
      const float yo = v[2 * n] + pert;
      const float ri = 1.0f / (sd * sd);
      const size_t e = ((size_t)idx * nz + (l - 1)) * nvar + n;
      yo_out[e] = (double)yo;
      rinv_out[e] = (double)ri;
    }
  }
  if (idx >= 0 && next_level != nz + 1) return LG_ERR_SHAPE;
  *n_obs = idx + 1;
  return LG_OK;
}

int lg_get_timeline(const lg_ctx* c, float* ms, int cap, int* nchunks) {
  if (!c || !nchunks || cap < 0) return LG_ERR_ARG;
  const int nq = (int)c->stats.n_chunks;
  *nchunks = nq;
  if (!ms) return LG_OK;
  if (nq <= 0 || (int)c->kev.size() < 7 * nq) return LG_ERR_STATE;
  const int n = std::min(cap, 7 * nq);
  for (int i = 0; i < n; ++i) ms[i] = elapsed_ms(c->ev[0], c->kev[i]);
  return LG_OK;
}

int lg_get_lists(const lg_ctx* c, int* counts, int* entries, double* rloc, int64_t* total) {
  if (!c || !total) return LG_ERR_ARG;
  if (!c->lists.off) return LG_ERR_STATE;
  *total = c->list_total;
  const int ncol = c->cfg.num_lat * c->cfg.num_lon;
  if (counts) CK(cudaMemcpy(counts, c->lists.cnt, sizeof(int) * ncol, cudaMemcpyDeviceToHost));
  if (entries && c->list_total)
    CK(cudaMemcpy(entries, c->lists.ent, sizeof(int) * c->list_total, cudaMemcpyDeviceToHost));
  if (rloc && c->list_total)
    CK(cudaMemcpy(rloc, c->lists.rloc, sizeof(double) * c->list_total, cudaMemcpyDeviceToHost));
  return LG_OK;
}

int lg_get_column_list(const lg_ctx* c, int col, int cap, int* entries, double* rloc,
                       int* count) {
  if (!c || !count || col < 0 || cap < 0) return LG_ERR_ARG;
  if (!c->lists.off) return LG_ERR_STATE;
  const int ncol = c->cfg.num_lat * c->cfg.num_lon;
  if (col >= ncol) return LG_ERR_ARG;
  int n = 0;
  int64_t off = 0;
  CK(cudaMemcpy(&n, c->lists.cnt + col, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&off, c->lists.off + col, sizeof(int64_t), cudaMemcpyDeviceToHost));
  *count = n;
  const int m = std::min(n, cap);
  if (entries && m) CK(cudaMemcpy(entries, c->lists.ent + off, sizeof(int) * m, cudaMemcpyDeviceToHost));
  if (rloc && m) CK(cudaMemcpy(rloc, c->lists.rloc + off, sizeof(double) * m, cudaMemcpyDeviceToHost));
  return LG_OK;
}

int lg_copy_layout(const lg_ctx* c, int* copy_obs, int* copy_block, int64_t* copy_entry_off,
                   int64_t* n_copies) {
  if (!c || !n_copies) return LG_ERR_ARG;
  if (!c->have_obs) return LG_ERR_STATE;
  const int64_t n = (int64_t)c->h_copy_obs.size();
  *n_copies = n;
  if (copy_obs) memcpy(copy_obs, c->h_copy_obs.data(), sizeof(int) * n);
  if (copy_block) memcpy(copy_block, c->h_copy_block.data(), sizeof(int) * n);
  if (copy_entry_off)
    for (int64_t j = 0; j <= n; ++j) copy_entry_off[j] = c->h_copy_eoff[j];
  return LG_OK;
}

int lg_get_hx(const lg_ctx* c, double* yb, double* dis) {
  if (!c) return LG_ERR_ARG;
  if (!c->have_obs) return LG_ERR_STATE;
  const size_t ne = (size_t)c->obs.n_entries;
  if (yb) CK(cudaMemcpy(yb, c->hx.yb, sizeof(double) * ne * c->cfg.ens, cudaMemcpyDeviceToHost));
  if (dis) CK(cudaMemcpy(dis, c->hx.dis, sizeof(double) * ne, cudaMemcpyDeviceToHost));
  return LG_OK;
}

void lg_destroy(lg_ctx* c) {
  if (!c) return;
  drop_graph(c);
  release_obs_memory(c);
  dfree(c->d_glat); dfree(c->d_glon); dfree(c->d_ca); dfree(c->d_cb); dfree(c->d_blk);
  dfree(c->d_lat_block); dfree(c->d_lon_block); dfree(c->d_nb_off); dfree(c->d_nb_blk);
  dfree(c->hx.yb); dfree(c->hx.yb32); dfree(c->hx.dis); dfree(c->hx.lnp); dfree(c->hx.rdiag);
  dfree(c->lists.cnt); dfree(c->lists.off); dfree(c->lists.ent); dfree(c->lists.rloc);
  dfree(c->lists.capped);
  if (c->d_scan_tmp) cudaFree(c->d_scan_tmp);
  for (auto& L : c->lane) {
    dfree(L.C); dfree(L.t); dfree(L.tri); dfree(L.lam); dfree(L.rot_cs); dfree(L.rot_i);
    dfree(L.rot_n); dfree(L.ovf_list); dfree(L.ovf_n);
  }
  dfree(c->d_status); dfree(c->d_band);
  dfree(c->d_rec); dfree(c->d_boff);
  dfree(c->d_cube_off); dfree(c->d_s_col); dfree(c->d_s_kk); dfree(c->d_trans); dfree(c->d_centres);
  dfree(c->d_xb); dfree(c->d_axb); dfree(c->d_xa); dfree(c->d_axa);
  dfree(c->d_xin); dfree(c->d_spb); dfree(c->d_spa);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->ev_hx) cudaEventDestroy(c->ev_hx);
  for (auto& e : c->kev) cudaEventDestroy(e);
  dfree(c->d_work);
  dfree(c->d_fresh);
  dfree(c->d_window);
  release_streams(c);
  delete c;
}

int lg_core_batch(int ens, int nbatch, const int* d_nobsl, const int64_t* d_off,
                  const double* d_hxens, const float* d_rdiaginv, const double* d_dep,
                  const double* d_rloc, double inflation, int precision, double* d_trans,
                  double* d_wbar, void* stream_v) {
  if (ens < 2 || ens > 128 || nbatch < 0 || inflation <= 0.0) return LG_ERR_ARG;
  if (precision != LG_PREC_FP64 && !lg::mixed_precision(precision)) return LG_ERR_ARG;
  if (precision == LG_PREC_MIXED_TF32 && !lg::gram_tf32_supported(ens)) return LG_ERR_UNSUPPORTED;
  if (nbatch == 0) return LG_OK;
  if (!d_nobsl || !d_off || !d_trans || !d_wbar) return LG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream_v;
  Geometry geo{};
  geo.ens = ens;
  geo.inflation = inflation;
  geo.vert_dist = -1.0;
  geo.ql_max_iter = ql_iter_limit();
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
  double *C = nullptr, *t = nullptr;
  int* fail = nullptr;
  if (dalloc(&C, (size_t)nbatch * ens * ens) != LG_OK || dalloc(&t, (size_t)nbatch * ens) != LG_OK ||
      dalloc(&fail, 1) != LG_OK) {
    dfree(C); dfree(t); dfree(fail);
    return LG_ERR_NOMEM;
  }
  int result = LG_OK;
  cudaMemsetAsync(fail, 0, sizeof(int), st);
  lg::HxDev hx{};
  lg::ListDev l{};
  if (precision == LG_PREC_MIXED_TF32)
    lg::launch_gram_tf32(geo, hx, l, b, nullptr, C, t, fail, lg::RecDev{}, st);
  else if (precision == LG_PREC_MIXED && lg::gram_tc_supported(ens))
    lg::launch_gram_tc(geo, hx, l, b, nullptr, C, t, fail, st);
  else
    lg::launch_gram64(geo, hx, l, b, nullptr, C, t, st);
  lg::launch_eig_apply(geo, b, C, t, nullptr, nullptr, nullptr, nullptr, d_trans, d_wbar, fail, st);
  int h_fail = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&h_fail, fail, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    result = LG_ERR_CUDA;
  else if (h_fail < 0)
    result = LG_ERR_TIMEOUT;  // a bounded tensor-core wait expired
  else if (h_fail)
    result = LG_ERR_EIG;
  dfree(C); dfree(t); dfree(fail);
  return result;
}

int lg_letkf_core(int nanals, int nobsl, const double* hxens, const float* rdiaginv,
                  const double* dep, const double* rloc, double* trans, double* overline_w,
                  double inflation_factor) {
  if (nanals < 2 || nanals > 128 || nobsl < 0 || !trans || !overline_w) return LG_ERR_ARG;
  if (nobsl > 0 && (!hxens || !rdiaginv || !dep || !rloc)) return LG_ERR_ARG;
  double *dh = nullptr, *dd = nullptr, *dr = nullptr, *dt = nullptr, *dw = nullptr;
  float* df = nullptr;
  int* dn = nullptr;
  int64_t* doff = nullptr;
  const size_t p = (size_t)nobsl, k = (size_t)nanals;
  int r = LG_OK;
  r |= dalloc(&dh, p * k);
  r |= dalloc(&df, p);
  r |= dalloc(&dd, p);
  r |= dalloc(&dr, p);
  r |= dalloc(&dt, k * k);
  r |= dalloc(&dw, k);
  r |= dalloc(&dn, 1);
  r |= dalloc(&doff, 1);
  if (r == LG_OK) {
    const int64_t zero = 0;
    bool ok = true;
    if (p) {
      ok = ok && cudaMemcpy(dh, hxens, sizeof(double) * p * k, cudaMemcpyHostToDevice) == cudaSuccess;
      ok = ok && cudaMemcpy(df, rdiaginv, sizeof(float) * p, cudaMemcpyHostToDevice) == cudaSuccess;
      ok = ok && cudaMemcpy(dd, dep, sizeof(double) * p, cudaMemcpyHostToDevice) == cudaSuccess;
      ok = ok && cudaMemcpy(dr, rloc, sizeof(double) * p, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    ok = ok && cudaMemcpy(dn, &nobsl, sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemcpy(doff, &zero, sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
      r = lg_core_batch(nanals, 1, dn, doff, dh, df, dd, dr, inflation_factor, LG_PREC_FP64, dt,
                        dw, nullptr);
    } else {
      cudaGetLastError();
      r = LG_ERR_CUDA;
    }
    if (r == LG_OK || r == LG_ERR_EIG) {
      if (cudaMemcpy(trans, dt, sizeof(double) * k * k, cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(overline_w, dw, sizeof(double) * k, cudaMemcpyDeviceToHost) != cudaSuccess)
        r = LG_ERR_CUDA;
    }
  } else {
    r = LG_ERR_NOMEM;
  }
  dfree(dh); dfree(df); dfree(dd); dfree(dr); dfree(dt); dfree(dw); dfree(dn); dfree(doff);
  return r;
}

void letkf_core_(const int* nanals, const int* nobsl, const double* hxens, const float* rdiaginv,
                 const double* dep, const double* rloc, double* trans, double* overline_w,
                 const double* inflation_factor, const int* pflag) {
  (void)pflag;
  const int r = lg_letkf_core(*nanals, *nobsl, hxens, rdiaginv, dep, rloc, trans, overline_w,
                              *inflation_factor);
  if (r != LG_OK && r != LG_ERR_EIG) fprintf(stderr, "letkf_core_: %s\n", lg_status_string(r));
}

}  // extern "C"
