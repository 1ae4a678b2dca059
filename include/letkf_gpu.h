/*
 * letkf_gpu.h -- C ABI of the GB300 LETKF analysis step.
 *
 * Drop-in boundary for the LETKF analysis call of DIDA-THHPCA's DA component
 * (x86/DA/LETKF).  Plain C, no C++ or CUDA types in any signature; every
 * pointer is caller-owned; every entry point returns LG_OK (0) or a negative
 * LG_ERR_* status and never aborts the process.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   lg_create / lg_set_grid   <- letkf_init            x86/DA/LETKF/src/letkf_init.F90:2-98
 *                                pro_info_init         x86/DA/utils/pro_info.F90:26-93
 *                                da_vert_coord_init    x86/DA/utils/vert_coord_mod.F90:33-545
 *   lg_set_obs                <- gen_obs_struct's Redis reads + comm_obs_data
 *                                                     x86/DA/LETKF/src/letkf_obs.F90:16-98, 251-466
 *                                                     x86/DA/LETKF/src/read_obs_mod.F90:73-449
 *   lg_run / lg_run_device    <- letkf_run(ntimes, xb, axb, xa, axa)
 *                                                     x86/DA/LETKF/src/letkf.F90:157-257
 *   lg_core_batch             <- letkf_core (column-batched)
 *                                                     x86/DA/LETKF/src/letkf_core.F90:14-233
 *   letkf_core_               <- letkf_core, Fortran implicit-interface symbol
 *                                (same ABI as sw/DA/LETKF/src/letkf_half/letkf_core_half_master.c:24-26)
 *   lg_destroy                <- letkf_final           x86/DA/LETKF/src/letkf_final.F90:2-13
 *
 * Array conventions follow the reference exactly (Fortran column-major):
 *   xb, xa  : double [ens][n][num_lat + 2*halo][num_lon + 2*halo] with ens fastest,
 *             i.e. Fortran xb(ens, n, 1-halo:num_lat+halo, 1-halo:num_lon+halo)
 *   axb, axa: double [n][num_lat + 2*halo][num_lon + 2*halo], n fastest
 * Only interior points of xa/axa are written; halo points are left untouched.
 * "lat" is the reference's x direction (nx), "lon" its y direction (ny).
 *
 * Threading: one context per host thread; calls on one context are serialised
 * by the caller.  The context owns all device buffers.
 */
#ifndef LETKF_GPU_H_
#define LETKF_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LG_MAX_VARS 16       /* DA variables (ps,u,v,pt,...) */
#define LG_MAX_OBS_TYPES 16  /* observation types (AIRCAR, SATWND, ...) */
#define LG_MAX_OBS_VARS 8    /* variables per observation type */

/* status codes */
#define LG_OK 0
#define LG_ERR_ARG -1           /* null pointer / bad argument */
#define LG_ERR_SHAPE -2         /* inconsistent sizes */
#define LG_ERR_UNSUPPORTED -3   /* option combination not implemented */
#define LG_ERR_NAN -4           /* NaN found in the background (module_da_parallel.F90:190-193) */
#define LG_ERR_OBS_OUTSIDE -5   /* obs outside its block's grid (letkf_obs.F90:211-231) */
#define LG_ERR_VARNAME -6       /* obs variable not among DA variables (letkf_obs.F90:113-117) */
#define LG_ERR_EIG -7           /* eigensolver did not converge (letkf_core.F90:119-122) */
#define LG_ERR_CUDA -8          /* CUDA runtime error */
#define LG_ERR_NOMEM -9         /* device or host allocation failed */
#define LG_ERR_STATE -10        /* call order violated (grid/obs not set) */
#define LG_ERR_TIMEOUT -11      /* a bounded device wait ran out */

/* precision of the analysis */
#define LG_PREC_FP64 0   /* plain FP64 everywhere (parity path) */
#define LG_PREC_MIXED 1  /* BF16 hi/lo tensor-core contractions, FP64 eigensolve */
#define LG_PREC_MIXED_TF32 2 /* as LG_PREC_MIXED with the Gram contractions as TF32 hi/lo
                                tensor-core products (about 2^-21 per operand instead of
                                2^-16: the FP32 variant); ens <= 64 */

/* vertical coordinate (da_vert_coord_init scheme) */
#define LG_VCOORD_HYBRID 0  /* ph = a*(p0-ptop) + b*(ps-ptop) + ptop */
#define LG_VCOORD_SIGMA 1   /* ph = a*(ps-ptop) + ptop  (ptop = pt) */

/* Mirrors the namelist_da / namelist_total fields letkf_init reads
 * (letkf_init.F90:27-81, da_namelist_mod.F90:79-89). */
typedef struct lg_config {
  int ens;             /* ensemble size k (svr_ensemble) */
  int num_lat;         /* global latitudes (reference nx direction) */
  int num_lon;         /* global longitudes (reference ny direction) */
  int nz;              /* model levels (num_lev) */
  int halo;            /* da_halo, >= 1 */
  int n_var;           /* DA variables, 2-D ones first (var_info ordering) */
  int var_lev[LG_MAX_VARS]; /* 1 for a 2-D variable, nz for a 3-D one */
  int ps_index;        /* 1-based row of surface pressure in n (ps_pos) */
  double local_dist;   /* da_loc_distance [km] */
  double vert_dist;    /* da_vert_distance [ln p]; <= 0 selects the 2-D path */
  double inflation;    /* da_inflation_factor (rho) */
  double obs_polar;    /* obs with |lat| > obs_polar are dropped (91 = keep all) */
  int gc_filter;       /* da_gc_enable: Gaspari-Cohn (1) or box (0) horizontally */
  int gc_filter_vertical; /* da_gc_enable_vertical */
  int max_obs;         /* MAX_OBS cap on local entries per column; 0 = no cap */
  int global_nx;       /* virtual decomposition: blocks in latitude */
  int global_ny;       /* virtual decomposition: blocks in longitude */
  int cube_n;          /* da_block_interval: one solve per cube of cube_n x cube_n columns of
                          a block, from the list of its centre column (>= 1) */
  int cube_nz;         /* da_vertical_interval: one solve per cube_nz levels at their centre
                          level (vertical localisation without overlap; >= 1) */
  int overlap;         /* da_block_overlap, 0 <= overlap < cube_n: cubes step by
                          cube_n - overlap and each column is the average over the cubes
                          covering it; as in the reference this path has no vertical
                          localisation (vert_dist is ignored) */
  int precision;       /* LG_PREC_FP64, LG_PREC_MIXED or LG_PREC_MIXED_TF32 */
  int vcoord;          /* LG_VCOORD_HYBRID or LG_VCOORD_SIGMA */
} lg_config;

/* One observation type: a fixed (levels x variables) record shape
 * (read_obs_mod.F90:15-27, 99-146). */
typedef struct lg_obs_type {
  int nz;                      /* obs_nz: levels per observation */
  int nvar;                    /* obs_nvar: variables per level */
  int var[LG_MAX_OBS_VARS];    /* 0-based DA variable index of each obs variable */
} lg_obs_type;

/* Structure-of-arrays observation set for the whole globe.  It replaces the
 * Redis observation store plus comm_obs_data: the library builds every virtual
 * block's observation list from it with the Redis box-query semantics
 * (redis_wrapper.c:4158-4296: inclusive lon/lat bounds printed with %.5f,
 * result ordered by observation index).  Observation o has type type[o]; its
 * nz levels occupy ph[ph_off(o) .. +nz) and its nz*nvar values occupy
 * yo/rinv[val_off(o) .. +nz*nvar) in (var fastest, level slowest) order, where
 * the offsets are the running sums over o' < o. */
typedef struct lg_obs_soa {
  int n_types;
  const lg_obs_type* types; /* n_types */
  int n_obs;
  const int* type;          /* n_obs */
  const double* lat;        /* n_obs, degrees (float-valued in the reference) */
  const double* lon;        /* n_obs, degrees in [0, 360) */
  const double* ph;         /* sum of nz over obs: observation pressure [Pa] */
  const double* yo;         /* sum of nz*nvar over obs: observed (perturbed) values */
  const double* rinv;       /* sum of nz*nvar over obs: 1/sigma^2 */
} lg_obs_soa;

typedef struct lg_stats {
  int64_t n_columns;        /* analysed grid columns */
  int64_t n_solves;         /* letkf_core solves */
  int64_t n_copies;         /* block-observation copies (obs counted once per block box) */
  int64_t n_entries;        /* (copy, level, var) entries with H(x) */
  int64_t nobsl_total;      /* sum over columns of local entries */
  int64_t nobsl_max;        /* max local entries of one column */
  int64_t n_capped;         /* columns truncated at max_obs */
  int64_t n_band;           /* candidate pairs with |ri-2| < 1e-12 (decision sensitive to libm ulps) */
  int64_t n_eig_fail;       /* eigensolves that hit the sweep limit */
  double ms_hx, ms_search, ms_solve, ms_total; /* last lg_run phase times (device events) */
  double ms_gram;           /* sum of Gram-kernel launch durations of the last lg_run */
  double ms_eig;            /* sum of eigensolve+update launch durations */
  int64_t n_launches;       /* kernels this library launched in the last lg_run */
  int64_t n_gram_entries;   /* sum over solves of nonzero-weight entries (Gram work) */
  double ms_tridiag;        /* eigensolve split: Householder reduction kernels */
  double ms_ql;             /* implicit QL kernels */
  double ms_vec;            /* vector transform + update kernels (incl. overflow fallback) */
  int64_t n_chunks;         /* solve chunks (launches of each solve-phase kernel) */
  double ms_h2d, ms_d2h;    /* lg_run only: background copy in before the analysis and
                               analysis copy out after it (device events); 0 otherwise */
} lg_stats;

typedef struct lg_ctx lg_ctx;

/* Create a context on the current CUDA device.  Validates the configuration. */
int lg_create(lg_ctx** ctx, const lg_config* cfg);

/* Model grid and vertical coordinate.
 * grid_lat: num_lat+1 floats (REAL(4) as in pro_info.F90:11-12); entry num_lat is forced to 90.
 * grid_lon: num_lon+1 floats; entry num_lon is forced to 360 (pro_info.F90:77-83).
 * coef_a, coef_b: nz+1 doubles: hybrid hyai/hybi, or sigma sigi (coef_b unused).
 * p0, ptop: hybrid reference and top pressure [Pa]; sigma uses ptop as pt. */
int lg_set_grid(lg_ctx* ctx, const float* grid_lat, const float* grid_lon,
                const double* coef_a, const double* coef_b, double p0, double ptop);

/* Observations for the next analysis (host arrays, copied). */
int lg_set_obs(lg_ctx* ctx, const lg_obs_soa* obs);

/* One complete analysis, host arrays (letkf_run).  ntimes is the DA cycle index;
 * it selected the Redis time slot in the reference and is recorded only. */
int lg_run(lg_ctx* ctx, int ntimes, const double* xb, const double* axb, double* xa, double* axa);

/* Same with device pointers on the context's stream (cudaStream_t passed as void*,
 * NULL = legacy default stream). */
int lg_run_device(lg_ctx* ctx, int ntimes, const double* d_xb, const double* d_axb,
                  double* d_xa, double* d_axa, void* stream);

/* Column windows and column shards.  The reference spreads the globe over a
 * 2-D grid of MPI ranks, each analysing its own block of columns after one
 * exchange of observations with its neighbour blocks (comm_obs_data,
 * x86/DA/LETKF/src/letkf_obs.F90:251-466; decomposition
 * x86/DA/EnDNN/src/module_da_parallel.F90:75-109).  Here one context holds
 * the whole globe's geometry and observations, and an analysis can be
 * restricted to a range of columns:
 *
 * lg_set_columns: analyse only grid columns [col_begin, col_end) (column
 *   c = (lon-1)*num_lat + (lat-1)); neighbour lists, solves and xa/axa values
 *   are produced for those columns alone (lg_run copies out only them) and
 *   the lists' device memory scales with the range, so a large globe can be
 *   analysed window by window.  H(x) of lg_run* still covers every
 *   observation copy.  LG_ERR_UNSUPPORTED with cubes.
 * lg_set_shard: the shard of a column-sharded analysis: longitude blocks
 *   [lon_block_begin, lon_block_end) of the virtual decomposition (0-based),
 *   i.e. their columns at every latitude, plus the block copies of those
 *   blocks as the shard's own observations (lg_shard_entries gives their
 *   entry range).  One shard per process and GPU; the shards of a run
 *   partition the longitude blocks.
 * A sharded analysis step, per process:
 *   lg_hx_device(own background)   H(x) of the shard's own copies; the
 *                                  background must be valid on the shard's
 *                                  columns and their halo
 *   lg_hx_export(rows)             the own entries' H(x) rows, ens + 3 doubles
 *                                  each (yb[ens], innovation, ln p, rdiaginv)
 *   (caller: all-gather of the rows of every shard, e.g. over NCCL)
 *   lg_hx_import(rows of shard r, its entry range)  for every other shard
 *   lg_analyse_device(...)         selection and solves of the shard's columns
 *                                  with the H(x) now in the context
 * lg_run_device with a shard set recomputes H(x) of every copy from the
 * background it is given and analyses the shard's columns.  All of these
 * enqueue on the stream (NULL: the context's own) and, except the export and
 * import, synchronise with it before returning. */
int lg_set_columns(lg_ctx* ctx, int col_begin, int col_end);
/* Local entries of every column's neighbour list for the current observation
 * set (the selection's count pass alone; nothing is stored): counts has
 * num_lat*num_lon ints, *total (optional) their sum.  For planning windows
 * whose lists fit a memory budget (each entry costs 12 bytes, 28 in mixed
 * precision).  LG_ERR_UNSUPPORTED with cubes. */
int lg_list_counts(lg_ctx* ctx, int* counts, int64_t* total);
int lg_set_shard(lg_ctx* ctx, int lon_block_begin, int lon_block_end);
int lg_shard_entries(const lg_ctx* ctx, int64_t* entry_begin, int64_t* entry_end,
                     int64_t* n_entries);
int lg_hx_device(lg_ctx* ctx, const double* d_xb, const double* d_axb, void* stream);
int lg_hx_export(const lg_ctx* ctx, double* d_rows, void* stream);
int lg_hx_import(lg_ctx* ctx, const double* d_rows, int64_t entry_begin, int64_t entry_end,
                 void* stream);
int lg_analyse_device(lg_ctx* ctx, const double* d_xb, const double* d_axb, double* d_xa,
                      double* d_axa, void* stream);

/* The DA caller's pre-processing around letkf_run (run_da_parallel,
 * x86/DA/EnDNN/src/module_da_parallel.F90:186-211), device arrays over the whole
 * globe with halo: axb = sum(xb_in)/real(ens), xb = xb_in - axb.  Returns
 * LG_ERR_NAN if any member value is NaN (the reference stops there). */
int lg_split_mean_device(lg_ctx* ctx, const double* d_xb_in, double* d_xb, double* d_axb,
                         void* stream);

/* Its post-processing (module_da_parallel.F90:219-257): xa_out =
 * gamma1*(axb+xb) + gamma2*(axa+xa) where |grid_lat| <= polar_lat, the
 * background elsewhere, 0 in the halo; spread_b/spread_a (n, num_lat, num_lon),
 * interior only, sqrt(sum of squares / ens). */
int lg_post_device(lg_ctx* ctx, double gamma1, double gamma2, double polar_lat,
                   const double* d_xb, const double* d_axb, const double* d_xa,
                   const double* d_axa, double* d_xa_out, double* d_spread_b,
                   double* d_spread_a, void* stream);

/* run_da_parallel as a whole on host arrays (module_da_parallel.F90:165-263):
 * split, letkf_run, blend and spreads.  xb_in/xa_out have the xb layout.
 * Whole globe only: LG_ERR_UNSUPPORTED while a column window or shard is set. */
int lg_run_da_parallel(lg_ctx* ctx, int ntimes, double gamma1, double gamma2, double polar_lat,
                       const double* xb_in, double* xa_out, double* spread_b,
                       double* spread_a);

/* Observation records of one type as the reference's Redis observation store
 * returns them (RedisGetobserveF), reshaped as read_obs does
 * (x86/DA/LETKF/src/read_obs_mod.F90:338-449) into this library's observation
 * arrays.  Record r has lon[r], lat[r], lev[r] (1-based level) and 2*nvar+1
 * floats at val[r*(2*nvar+1)]: value and error sd of each variable in turn,
 * then the pressure [Pa].  nz == 1: one observation per record.  nz > 1
 * (profiles such as ADPUPA, GPSRO): a record with lev == 1 starts an
 * observation and gives its position, and each record fills level lev; every
 * level of every profile must be present (LG_ERR_SHAPE otherwise, as a missing
 * level would leave a zero pressure).  The observed value is perturbed as
 * read_obs does, value + noise * sd in REAL(4), with caller-supplied standard
 * normal noise[v * n_records + r] for variable v of record r (NULL: no
 * perturbation); rinv = 1 / sd^2 in REAL(4).  Outputs, caller-allocated for
 * max_obs observations: lat, lon (n_obs), ph (n_obs*nz), yo and rinv
 * (n_obs*nz*nvar, variable fastest, then level) -- the lg_obs_soa layout of one
 * type; *n_obs receives the count.  Host only; needs no device. */
int lg_obs_from_records(int nz, int nvar, int n_records, const float* lon, const float* lat,
                        const float* lev, const float* val, const float* noise, int max_obs,
                        int* n_obs, double* lat_out, double* lon_out, double* ph_out,
                        double* yo_out, double* rinv_out);

/* GMCORE state of all members to the DA background layout, on the device (the
 * coupler step before run_da_parallel: gmcore2da_send_coupling,
 * x86/ATM/gmcore_mct/gmcore_coupler.F90:153-284, and the receive into
 * xb(ens, n, lat, lon), x86/DA/EnDNN/src/module_da_coupler.F90:91-147,350-414).
 * Inputs, members fastest (GMCORE's (member, lon, lat, lev) arrays):
 *   ps           [lat][lon][ens]
 *   u_half       [nz][lat][lon][ens]    u_f: u east of each full longitude (C grid)
 *   v_half       [nz][lat + 1][lon][ens] v_f at half latitudes 0..num_lat (C grid)
 *   pt           [nz][lat][lon][ens]
 *   area_subcell [lat][2], area_cell [lat]  (GMCORE mesh; device arrays)
 * Output xb [lon + 2 halo][lat + 2 halo][1 + 3 nz][ens] (the lg_run layout with
 * rows ps, u, v, pt): u = (u_f(i) + u_f(i-1)) / 2 (periodic),
 * v = 2 (v_f(j-1) area_subcell(1,j) + v_f(j) area_subcell(2,j)) / area_cell(j)
 * (evaluated with the per-latitude weights 2 area_subcell / area_cell: equal
 * up to rounding); ens <= 1024;
 * the longitude halo is filled periodically, latitude halo rows are not
 * written.  Enqueued on stream (NULL: the default stream); no synchronisation. */
int lg_gmcore_to_da_device(int ens, int num_lat, int num_lon, int nz, int halo,
                           const double* d_ps, const double* d_u_half, const double* d_v_half,
                           const double* d_pt, const double* d_area_subcell,
                           const double* d_area_cell, double* d_xb, void* stream);

/* Wall-clock limit [ns] of the tensor-core Gram's pipeline waits (the column
 * Gram's mbarrier waits between its producer, converter and MMA warps);
 * 0 restores the default of 2 s.  On expiry a CTA raises LG_ERR_TIMEOUT,
 * waits (with the full bound) for its own MMAs and copies, frees its tensor
 * memory and returns, and the analysis returns LG_ERR_TIMEOUT.  For tests of
 * that path and for diagnosing a stalled device; no reference counterpart. */
int lg_set_wait_limit(lg_ctx* ctx, int64_t ns);

/* Statistics of the last lg_run. */
int lg_get_stats(const lg_ctx* ctx, lg_stats* st);

/* Timeline of the last lg_run's solve phase: for each chunk of columns, seven
 * instants in ms after the analysis started -- Gram start, Gram end,
 * eigensolve start, tridiagonalisation end, QL end, vector update start,
 * vector update end -- at ms[7*q .. 7*q+6].  Writes min(cap, 7*chunks) values;
 * *nchunks receives the chunk count (ms may be NULL to query it).  Diagnostic
 * only; no reference counterpart. */
int lg_get_timeline(const lg_ctx* ctx, float* ms, int cap, int* nchunks);

/* Launch shapes and bucket boundaries of the analysis.  None of them changes
 * an FP64 result; in mixed precision the Gram variant and the ln p buckets only
 * change the FP32 summation order.  No reference counterpart: the reference
 * has no GPU path to tune. */
#define LG_GRAM_AUTO 0   /* column groups where supported (the lean variant with three
                            or four solve streams), else per-solve streaming */
#define LG_GRAM_COLUMN 1 /* one CTA per SM over (column, 8 levels) items, rows read once per group */
#define LG_GRAM_STREAM 2 /* one CTA per solve streaming its ln p window of records */
#define LG_GRAM_QUEUE 3  /* one CTA per solve compacting non-zero weights through a queue */
#define LG_GRAM_COLUMN_LEAN 4 /* as LG_GRAM_COLUMN with a 2-stage ring (74 KB of shared
                                 memory), leaving room on each SM for other streams' kernels */

typedef struct lg_tuning {
  int chunk_mb;    /* Gram workspace per solve chunk [MiB] (sets solves per launch), 16..65536 */
  int gram_kernel; /* LG_GRAM_* (mixed precision) */
  int lnp_buckets; /* ln p buckets of the Gram records (mixed, vertical localisation), 8..1024:
                      the bucket boundaries that bound each level's record window */
  int ql_warps;    /* warps per block of the QL kernel, 1..6; a block takes at most a third
                      of an SM's shared memory (at most 2 warps at 64 members, 1 above) */
  int vec_warps;   /* warps per block of the vector/update kernel, 1..8 */
  int solve_streams; /* 1; 2: chunks alternate between two streams with their own scratch;
                        3: phase pipeline (Grams, eigensolves, vector updates on three
                        streams, three buffer sets); 4: as 3 with tridiagonalisation
                        and QL on separate streams, four buffer sets */
  int gram_ctas;   /* persistent CTAs of the column Gram, 0 = one per SM; fewer leave
                      whole SMs to the eigensolve beside it */
  double ms;       /* device time of one analysis with these settings (lg_autotune) */
} lg_tuning;

/* Current settings; defaults are the autotuned values of the 360x180x32, N=64,
 * 10^6-observation workload. */
int lg_get_tuning(const lg_ctx* ctx, lg_tuning* out);

/* Apply settings (validated; LG_ERR_ARG if out of range).  Buffers are resized
 * and the captured analysis graph is rebuilt at the next run. */
int lg_set_tuning(lg_ctx* ctx, const lg_tuning* t);

/* Autotuner: times complete analyses of the given device arrays (as
 * lg_run_device) over candidate settings -- solve streams, chunk size, Gram
 * variant, ln p bucket count, QL and vector block shapes -- one parameter at a time,
 * applies the fastest and returns it in *best (best->ms = its analysis time).
 * xa/axa are overwritten by the analyses. */
int lg_autotune(lg_ctx* ctx, const double* d_xb, const double* d_axb, double* d_xa,
                double* d_axa, void* stream, lg_tuning* best);

/* Neighbour lists of the last analysis (device-built), for parity checks.
 * counts: num_lat*num_lon ints, column c = (lon-1)*num_lat + (lat-1);
 * entries/rloc: total local entries in column order; entries hold the global
 * copy-entry index (see lg_copy_layout).  Pass NULL arrays to query the total
 * through *total only.  With cubes only the cube centres' lists are built (the
 * other columns count 0), and lg_stats.nobsl_total sums over those. */
int lg_get_lists(const lg_ctx* ctx, int* counts, int* entries, double* rloc, int64_t* total);

/* The neighbour list of one column of the last analysis (as lg_get_lists,
 * without copying every column's list): *count receives its length and the
 * first min(count, cap) entries / weights are written (NULL arrays: count
 * only).  Diagnostic for sampled parity checks; no reference counterpart. */
int lg_get_column_list(const lg_ctx* ctx, int col, int cap, int* entries, double* rloc,
                       int* count);

/* Layout of block-observation copies built by lg_set_obs: for each copy j
 * (ordered by block b = (by-1)*global_nx + (bx-1), then type, then observation
 * index), copy_obs[j] = observation index, copy_block[j] = b, and
 * copy_entry_off[j] = first copy-entry index (n_copies+1 values). */
int lg_copy_layout(const lg_ctx* ctx, int* copy_obs, int* copy_block,
                   int64_t* copy_entry_off, int64_t* n_copies);

/* H(x) of the last analysis: yb[n_entries][ens] (member fastest) and
 * dis[n_entries] per copy entry, after mean removal (letkf_obs.F90:156-183). */
int lg_get_hx(const lg_ctx* ctx, double* yb, double* dis);

void lg_destroy(lg_ctx* ctx);

/* Column-batched letkf_core on device arrays (letkf_core.F90:14-233):
 * for batch b with p_b = nobsl[b] entries starting at offset off[b]:
 *   hxens[(off[b]+j)*ens + i], rdiaginv[off[b]+j] (float), dep[off[b]+j], rloc[off[b]+j]
 *   -> trans[b*ens*ens + i + ens*j] (column-major ens x ens), wbar[b*ens + i].
 * precision: LG_PREC_FP64, LG_PREC_MIXED or LG_PREC_MIXED_TF32 (ens <= 64).
 * stream: cudaStream_t or NULL. */
int lg_core_batch(int ens, int nbatch, const int* d_nobsl, const int64_t* d_off,
                  const double* d_hxens, const float* d_rdiaginv, const double* d_dep,
                  const double* d_rloc, double inflation, int precision,
                  double* d_trans, double* d_wbar, void* stream);

/* lg_core_batch for callers that cannot allocate device memory: no counterpart
 * in the reference.  A host framework that owns the whole device heap through
 * its own pool allocator, or a tight loop in which cudaMalloc/cudaFree per call
 * would synchronise the device, cannot let the library allocate its working
 * memory; this entry point keeps it (Gram matrices, projected innovations,
 * status word) in one fixed static device array of 8 MiB instead, so it needs
 * nbatch * (ens*ens + ens) + 8 <= 1048576 doubles (e.g. at most 252 solves of
 * 64 members per call) and returns LG_ERR_SHAPE beyond that.  Same arguments
 * and results as lg_core_batch.  The array's device address is looked up on
 * the first call made on each device (set-up work), so make that first call
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller. */
int lg_core_batch_noalloc(int ens, int nbatch, const int* d_nobsl, const int64_t* d_off,
                          const double* d_hxens, const float* d_rdiaginv, const double* d_dep,
                          const double* d_rloc, double inflation, int precision,
                          double* d_trans, double* d_wbar, void* stream);

/* Fortran drop-in for the external letkf_core (all arguments by reference, host
 * arrays), so a build of the reference links this instead of its own letkf_core.
 * pflag is accepted and ignored.  Errors are reported through *ierr when the
 * caller passes the optional 11th argument through the lg_letkf_core variant. */
void letkf_core_(const int* nanals, const int* nobsl, const double* hxens,
                 const float* rdiaginv, const double* dep, const double* rloc,
                 double* trans, double* overline_w, const double* inflation_factor,
                 const int* pflag);

/* letkf_core_ with a status result. */
int lg_letkf_core(int nanals, int nobsl, const double* hxens, const float* rdiaginv,
                  const double* dep, const double* rloc, double* trans,
                  double* overline_w, double inflation_factor);

/* Human-readable name of a status code. */
const char* lg_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* LETKF_GPU_H_ */
