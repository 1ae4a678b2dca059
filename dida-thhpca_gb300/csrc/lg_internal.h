// lg_internal.h -- context layout and kernel entry points of the LETKF library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/letkf_gpu.h"

namespace lg {

// Observation-type tables, per analysis (constant memory, set by lg_set_obs).
struct TypeTable {
  int n_types;
  int nz[LG_MAX_OBS_TYPES];
  int nvar[LG_MAX_OBS_TYPES];
  int var[LG_MAX_OBS_TYPES][LG_MAX_OBS_VARS];
};

// Geometry and model constants visible to all kernels.
struct Geometry {
  int ens, num_lat, num_lon, nz, halo, n, n_var, ps_row;  // ps_row 0-based
  int var_start[LG_MAX_VARS];                             // 0-based first row
  int var_lev[LG_MAX_VARS];
  int vcoord;
  double p0, ptop;
  double local_dist, vert_dist, inflation, obs_polar;
  int gc_filter, gc_filter_vertical, max_obs;
  int global_nx, global_ny, nblocks, n_types;
  // QL sweep limit per eigenvalue (tql2 and dsyevd stop at 30-60 sweeps); 0 = 60.
  // A small value forces non-convergence (a host-side test of LG_ERR_EIG).
  int ql_max_iter;
  // wall-clock limit of the column Gram's pipeline waits [ns]; 0 = 2 s.  A
  // tiny value makes them run out (a host-side test of LG_ERR_TIMEOUT); the
  // waits of a CTA's clean-up for its own MMAs and copies keep their full bound.
  long long tc_wait_ns;
  // device arrays
  const float* glat;     // num_lat+1
  const float* glon;     // num_lon+1
  const double* ca;      // nz+1
  const double* cb;      // nz+1
  const int4* blk;       // (s_lat, e_lat, s_lon, e_lon), 1-based, per block
  const int* lat_block;  // num_lat: 0-based block row of each latitude
  const int* lon_block;  // num_lon: 0-based block column of each longitude
  const int* nb_off;     // nblocks+1
  const int* nb_blk;     // neighbour blocks in traversal order
};

// Observations and their block copies on the device.
struct ObsDev {
  int n_obs;
  int64_t n_copies, n_entries;
  const int* otype;
  const double* olat;
  const double* olon;
  const int64_t* ph_off;
  const int64_t* val_off;
  const double* oph;
  const double* oyo;
  const double* orinv;
  // per observation trig terms for the distance test
  const double* dcx;  // cos(lat/180*pi)
  const double* dsx;  // sin(lat/180*pi)
  const double* dyr;  // lon/180*pi
  const float* fcx;
  const float* fsx;
  const float* fyr;
  // copies
  const int* copy_obs;
  const int* copy_block;
  const int* copy_eoff;  // n_copies+1 entry offsets
  const int* bt_off;     // nblocks*n_types+1: copies of (block, type)
};

// Cell index of each (block, type) segment of copies, for the selection.
struct CellIndex {
  int nrows, ncols;        // global cell grid
  float cell_deg, inv_cell;
  float cap_deg;           // search radius in degrees (2L/a with the prefilter margin)
  int bitmap_words;        // max over segments of ceil(len/32)
  int exact_rloc;          // 1: FP64 weights (FP64 path); 0: FP32 weights (mixed path)
  const int4* box;         // per segment: row0, nrows, col0, ncols
  const int* cell_off;     // per segment: offset of its cell_start block
  const int* cell_start;   // per segment: nrows*ncols+1 offsets into perm
  const int* perm;         // per copy slot: segment positions sorted by cell
  const float4* cand;      // per copy slot, in perm order: the observation's FP32 cos(lat),
                           // sin(lat), lon [rad] and 1 if |lat| <= obs_polar, else 0
};

// H(x) results per copy entry.
struct HxDev {
  double* yb;     // n_entries * ens
  float* yb32;    // n_entries * ens (mixed path operand)
  double* dis;    // n_entries
  double* lnp;    // n_entries, log(ph)
  float* rdiag;   // n_entries, REAL(4) R^-1
};

// Per-column neighbour lists.
struct ListDev {
  int* cnt;          // columns
  int64_t* off;      // columns+1
  int* ent;          // total entries
  double* rloc;      // total entries
  int* capped;       // columns (1 if truncated at max_obs)
  // selection only: build the lists of these columns alone (cube centres);
  // the counts of the others stay as they are (zero)
  const int* col_list = nullptr;
  int n_list = 0;
  // count pass only, optional: [0] = max over columns of the count, [1] += 1
  // per column truncated at max_obs (lg_stats.nobsl_max, n_capped)
  int* col_stats = nullptr;
};

// Per-column entry records grouped by ln p bucket (mixed-precision Gram input).
struct RecDev {
  const float4* r;    // list-sized: (entry index bits, ln p, rdiaginv * rloc, innovation), FP32
  const int* boff;    // columns x (nb+1)
  int nb;
  float lo, inv_dz;
};

// A batch of LETKF solves: which list entries feed it and where results go.
struct SolveBatch {
  int mode;          // 0 = analysis columns, 1 = explicit core batch
  int first_col;     // mode 0: first column of the chunk
  int ncols;         // mode 0: columns in the chunk
  int levels;        // solves per column (nz for the vertical path, else 1)
  int nsolves;
  // mode 1 inputs
  const int* b_nobsl;
  const int64_t* b_off;
  const double* b_hx;
  const float* b_rdiag;
  const double* b_dep;
  const double* b_rloc;
  unsigned long long* work;  // optional: += nonzero-weight entries processed
  // optional: process only the solves listed in solve_list[0 .. *solve_count)
  const int* solve_list;
  const int* solve_count;
  // mode 0 with cubes: solve s of the batch is solve first_solve + s of the
  // analysis, at centre column s_col[.] and centre level s_kk[.] (1-based);
  // its trans goes to eig_apply's trans output
  const int* s_col;
  const int* s_kk;
  int first_solve;
};

// column and level (1-based) of solve s of a mode-0 batch
__host__ __device__ inline void solve_col_level(const SolveBatch& b, int s, int& col, int& kk) {
  if (b.s_col) {
    col = b.s_col[b.first_solve + s];
    kk = b.s_kk[b.first_solve + s];
  } else {
    col = b.first_col + s / b.levels;
    kk = s % b.levels + 1;
  }
}

// the mixed-precision analysis path (tensor-core Gram, FP32 vector transform):
// BF16 hi/lo (LG_PREC_MIXED) or TF32 hi/lo (LG_PREC_MIXED_TF32) contractions
inline bool mixed_precision(int p) { return p == LG_PREC_MIXED || p == LG_PREC_MIXED_TF32; }

// kernels (host launchers), all asynchronous on `stream`
// cand[slot] of every copy slot (slot_obs[slot] = observation of the slot)
void launch_cell_cands(const ObsDev& o, double obs_polar, const int* slot_obs, int nslots,
                       float4* cand, cudaStream_t stream);
void launch_obs_trig(const ObsDev& o, double* dcx, double* dsx, double* dyr, float* fcx,
                     float* fsx, float* fyr, cudaStream_t stream);
void set_type_table(const TypeTable& t, cudaStream_t stream);
// H(x) of the block copies [j0, j1) (j1 < 0: through the last copy)
void launch_hx(const Geometry& g, const ObsDev& o, const double* xb, const double* axb,
               HxDev hx, int* err, cudaStream_t stream, int64_t j0 = 0, int64_t j1 = -1);
// H(x) rows of entries [e0, e1) packed as ens + 3 doubles each -- yb[ens], dis,
// ln p, rdiaginv -- out of (export) or into (import; also the FP32 operand copy
// of yb on the mixed path) the context's H(x) buffers
void launch_hx_export(int ens, int64_t e0, int64_t e1, const HxDev& hx, double* rows,
                      cudaStream_t stream);
void launch_hx_import(int ens, int64_t e0, int64_t e1, HxDev hx, const double* rows,
                      cudaStream_t stream);
void launch_search(const Geometry& g, const ObsDev& o, ListDev l, int fill,
                   unsigned long long* band, cudaStream_t stream);
// skip (count pass only, may be null): when *skip is non-zero the launch does
// nothing -- the counts and statistics are already those of this selection
void launch_search_cells(const Geometry& g, const ObsDev& o, const CellIndex& ci, ListDev l,
                         int fill, unsigned long long* band, cudaStream_t stream,
                         const int* skip = nullptr);
// zero the selection's counts (n ints), its two statistics and the band
// counter, unless *fresh is non-zero (the count pass that sized the lists has
// just computed them for the same columns and observations)
void launch_clear_selection(const int* fresh, int* cnt, int n, int* col_stats,
                            unsigned long long* band, cudaStream_t stream);
void launch_scan_counts(const int* cnt, int64_t* off, int n, void* tmp, size_t tmp_bytes,
                        cudaStream_t stream);
size_t scan_tmp_bytes(int n);
void launch_gram64(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                   const double* axb, double* C, double* t, cudaStream_t stream);
bool gram_tc_supported(int ens);
void launch_gram_tc(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                    const double* axb, double* C, double* t, int* err, cudaStream_t stream,
                    const RecDev* rec = nullptr);
// Records a timing event on st.  Inside a stream capture a plain cudaEventRecord
// only orders the capture and is never recorded when the graph runs, so there
// the event becomes an external event-record node of the graph; outside a
// capture the external flag is not allowed and a plain record is made.
inline cudaError_t record_event(cudaEvent_t e, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaError_t q = cudaStreamIsCapturing(st, &cs);
  if (q != cudaSuccess) return q;
  return cs == cudaStreamCaptureStatusActive
             ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal)
             : cudaEventRecord(e, st);
}
bool gram_col_supported(int ens);
// TF32 hi/lo per-solve tcgen05 Gram (LG_PREC_MIXED_TF32), ens <= 64; analysis
// records (mode 0) or a core batch (mode 1)
bool gram_tf32_supported(int ens);
void launch_gram_tf32(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                      const double* axb, double* C, double* t, int* err, const RecDev& rec,
                      cudaStream_t stream);
// 65..128 members: per-solve tcgen05 Gram (analysis records or a core batch);
// launch_gram_tc and launch_gram_tc_stream route these sizes to it
bool gram_tc128_supported(int ens);
void launch_gram_tc128(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                       const double* axb, double* C, double* t, int* err, const RecDev& rec,
                       cudaStream_t stream);
void launch_gram_col(const Geometry& g, const HxDev& hx, const ListDev& l, const SolveBatch& b,
                     const double* axb, double* C, double* t, int* err, const RecDev& rec,
                     bool lean, int ctas, cudaStream_t stream);
void launch_gram_tc_stream(const Geometry& g, const HxDev& hx, const ListDev& l,
                           const SolveBatch& b, const double* axb, double* C, double* t, int* err,
                           const RecDev& rec, cudaStream_t stream);
// records of the columns col0 .. col0 + ncol - 1
void launch_records(int col0, int ncol, const ListDev& l, const HxDev& hx, float lo, float inv_dz,
                    int nb, int* boff, float4* rec, cudaStream_t stream);
// Cube solves (da_block_interval cube_n, da_vertical_interval cube_nz,
// da_block_overlap): cubes of cube_n x cube_n columns of a block, stepping by
// stride = cube_n - overlap from each block's first column, numbered block by
// block (longitude outer, latitude inner as the reference loops); solve
// (cube, level group) = cube * ngroups + group.
struct CubeDev {
  int cube_n, cube_nz, stride, ngroups;
  int grouped;          // vertical path without overlap: level groups of cube_nz levels
  const int* cube_off;  // nblocks + 1: first cube of each block
};
void launch_cube_apply(const Geometry& g, const CubeDev& cd, const double* trans,
                       const double* xb, const double* axb, double* xa, double* axa,
                       cudaStream_t stream);

cudaError_t launch_gmcore_to_da(int ens, int num_lat, int num_lon, int nz, int halo,
                                const double* ps, const double* u_half, const double* v_half,
                                const double* pt, const double* area_subcell,
                                const double* area_cell, double* xb, cudaStream_t stream);

void launch_eig_apply(const Geometry& g, const SolveBatch& b, const double* C, const double* t,
                      const double* xb, const double* axb, double* xa, double* axa,
                      double* trans, double* wbar, int* eig_fail, cudaStream_t stream);
size_t eig2_tri_doubles(int n);
bool eig2_supported(const Geometry& g);
// mixed path, cube solves: explicit trans of each solve from the tridiagonal
// form and rotation log (solves with rot_n < 0 are left to eig_apply)
void launch_trans(const Geometry& g, const SolveBatch& b, const double* t, const double* tri,
                  const double* lam, const void* rot_cs, const unsigned char* rot_i,
                  const int* rot_n, int rot_cap, double* trans, cudaStream_t stream);
// phases of launch_eig2 (a bit mask)
constexpr int kEigTridiag = 1, kEigQL = 2, kEigVectors = 4, kEigAll = 7;
void launch_eig2(const Geometry& g, const SolveBatch& b, const double* C, const double* t,
                 const double* xb, const double* axb, double* xa, double* axa, double* tri,
                 double* lam, void* rot_cs, unsigned char* rot_i, int* rot_n, int rot_cap,
                 int* overflow_list, int* overflow_n, int* eig_fail, bool fp32_vectors,
                 int ql_warps, int vec_warps, int phases, cudaStream_t stream,
                 cudaEvent_t ev_after_tri = nullptr, cudaEvent_t ev_after_ql = nullptr);
void launch_split_mean(int ens, int64_t npts_rows, const double* xb_in, double* xb, double* axb,
                       int* err, cudaStream_t stream);
void launch_post(int ens, int n, int num_lat, int num_lon, int halo, double gamma1, double gamma2,
                 double polar, const float* glat, const double* xb, const double* axb,
                 const double* xa, const double* axa, double* xa_out, double* spread_b,
                 double* spread_a, cudaStream_t stream);
void launch_nan_check(const double* x, size_t n, int* err, cudaStream_t stream);
// bytes (a multiple of 16) from device-addressable page-locked host memory src
// (16-byte aligned) to device memory dst (16-byte aligned), by a copy kernel
cudaError_t launch_copy_mapped(const void* src, void* dst, size_t bytes, cudaStream_t stream);

}  // namespace lg
