/*
 * letkf_oracle.c -- CPU ORACLE for the LETKF analysis step (TEST INFRASTRUCTURE).
 *
 * This file is the checker, never the product: only tests/, the smoke check and
 * bench.py's cpu_baseline / reference arm load it.  It is a plain-C restatement
 * of the reference's x86 LETKF hot path (DIDA-THHPCA, Fortran), following each
 * routine step by step, including its precision quirks (REAL(4) grid, REAL(4)
 * literals promoted to REAL(8), REAL(4) rdiaginv).  It must be compiled with
 * -ffp-contract=off so that no multiply-add is fused, as gfortran -O2 on
 * x86-64 does not fuse either.
 *
 * Parity pinning: the reference ships no golden vectors or known-answer tests
 * for this path (no test of letkf_run/letkf_core runs; x86/DA/LETKF/unit/main.f90
 * is stale).  The oracle is pinned by closed-form known-answer tests written for
 * this project (single observation scalar Kalman update, p = 0 inflation-only
 * case, recentring and symmetry invariants) under tests/.
 *
 * Vendor BLAS/LAPACK: the reference calls dgemm/dsyevd (MKL or lapack64,
 * x86/CMakeLists.txt:211-235).  The oracle dlopen()s the OpenBLAS copy that
 * scipy bundles (symbols scipy_dgemm_/scipy_dsyevd_) when a path is given,
 * and otherwise uses its own loops and a cyclic Jacobi eigensolver.
 *
 * Two reference defects are fixed, not emulated (their reference behaviour
 * reads uninitialised memory):
 *   1. ps2alnp leaves ph_lev(nz+1) unset (x86/DA/LETKF/src/obs_make.F90:429-434);
 *      the oracle computes it like the other levels.
 *   2. comm_obs_data never sends ph (x86/DA/LETKF/src/letkf_obs.F90:376-441), so
 *      neighbour-block observations reach gen_yb_dis_vertical with unset ph
 *      (letkf_yb.F90:211); the oracle uses the observation's own ph.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/letkf_gpu.h"

/* ------------------------------------------------------------------ BLAS */
typedef void (*dgemm_fn)(const char*, const char*, const int*, const int*, const int*,
                         const double*, const double*, const int*, const double*, const int*,
                         const double*, double*, const int*, size_t, size_t);
typedef void (*dsyevd_fn)(const char*, const char*, const int*, double*, const int*, double*,
                          double*, const int*, int*, const int*, int*, size_t, size_t);
typedef void (*setthreads_fn)(int);
static dgemm_fn p_dgemm = NULL;
static dsyevd_fn p_dsyevd = NULL;

int or_set_lapack(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 0;
  dgemm_fn g = (dgemm_fn)dlsym(h, "scipy_dgemm_");
  dsyevd_fn e = (dsyevd_fn)dlsym(h, "scipy_dsyevd_");
  if (!g) g = (dgemm_fn)dlsym(h, "dgemm_");
  if (!e) e = (dsyevd_fn)dlsym(h, "dsyevd_");
  setthreads_fn st = (setthreads_fn)dlsym(h, "scipy_openblas_set_num_threads");
  if (!st) st = (setthreads_fn)dlsym(h, "openblas_set_num_threads");
  if (!g || !e) return 0;
  if (st) st(1);  /* one BLAS thread per column thread */
  p_dgemm = g;
  p_dsyevd = e;
  return 1;
}
int or_lapack_loaded(void) { return p_dgemm != NULL && p_dsyevd != NULL; }

/* C = alpha*op(A)*op(B) + beta*C, column-major, fallback loops */
static void gemm(char ta, char tb, int m, int n, int k, const double* a, int lda,
                 const double* b, int ldb, double* c, int ldc) {
  if (p_dgemm) {
    const double one = 1.0, zero = 0.0;
    p_dgemm(&ta, &tb, &m, &n, &k, &one, a, &lda, b, &ldb, &zero, c, &ldc, 1, 1);
    return;
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int l = 0; l < k; ++l) {
        double av = (ta == 'n') ? a[i + (size_t)lda * l] : a[l + (size_t)lda * i];
        double bv = (tb == 'n') ? b[l + (size_t)ldb * j] : b[j + (size_t)ldb * l];
        s += av * bv;
      }
      c[i + (size_t)ldc * j] = s;
    }
}

/* symmetric eigen-decomposition, ascending eigenvalues, vectors overwrite a
 * (column-major n x n); returns 0 on success */
static int jacobi_eig(int n, double* a, double* w, double* v) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) v[i + n * j] = (i == j) ? 1.0 : 0.0;
  int sweep;
  for (sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double x = a[i + n * j] * a[i + n * j];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a[p + n * q];
        if (apq == 0.0) continue;
        double app = a[p + n * p], aqq = a[q + n * q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = a[k + n * p], akq = a[k + n * q];
          a[k + n * p] = c * akp - s * akq;
          a[k + n * q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = a[p + n * k], aqk = a[q + n * k];
          a[p + n * k] = c * apk - s * aqk;
          a[q + n * k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = v[k + n * p], vkq = v[k + n * q];
          v[k + n * p] = c * vkp - s * vkq;
          v[k + n * q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = a[i + n * i];
  /* sort ascending (selection), permuting vectors */
  for (int i = 0; i < n; ++i) {
    int m = i;
    for (int j = i + 1; j < n; ++j)
      if (w[j] < w[m]) m = j;
    if (m != i) {
      double t = w[i]; w[i] = w[m]; w[m] = t;
      for (int k = 0; k < n; ++k) {
        double x = v[k + n * i]; v[k + n * i] = v[k + n * m]; v[k + n * m] = x;
      }
    }
  }
  memcpy(a, v, sizeof(double) * n * n);
  return sweep >= 100 ? 1 : 0;
}

/* dsyevd('V','L', ...) equivalent; a: n x n column-major in, eigenvectors out */
static int syevd(int n, double* a, double* w, double* work, int* iwork, double* scratch) {
  if (n == 0) return 0;
  if (p_dsyevd) {
    int lwork = 2 * n * n + 6 * n + 1, liwork = 5 * n + 3, info = 0;
    p_dsyevd("V", "L", &n, a, &n, w, work, &lwork, iwork, &liwork, &info, 1, 1);
    return info;
  }
  /* Jacobi works on the full matrix: mirror the lower triangle */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < j; ++i) a[i + n * j] = a[j + n * i];
  return jacobi_eig(n, a, w, scratch);
}

/* ------------------------------------------------- precision-exact helpers */

/* pi = atan(1.0) * 4 evaluated in REAL(4) (pro_info.F90:156,170) */
static double pi_r4(void) { return (double)(atanf(1.0f) * 4.0f); }

/* latlon_dist_r8 (pro_info.F90:148-161): REAL(8) arithmetic with the REAL(4)
 * constants a = 6371.393 and pi = atan(1.0)*4 */
double or_latlon_dist_r8(double x1, double y1, double x2, double y2) {
  const double pi = pi_r4();
  const double a = (double)6371.393f;
  double c1 = cos(x1 / 180.0 * pi), c2 = cos(x2 / 180.0 * pi);
  double c3 = cos(y1 / 180.0 * pi - y2 / 180.0 * pi);
  double s1 = sin(x1 / 180.0 * pi), s2 = sin(x2 / 180.0 * pi);
  double v = c1 * c2 * c3 + s1 * s2;
  if (!(v < 1.0)) v = (v != v) ? v : 1.0; /* min(v, 1.0) */
  return a * acos(v);
}

/* latlon_dist_r4 (pro_info.F90:163-175): all REAL(4) */
float or_latlon_dist_r4(float x1, float y1, float x2, float y2) {
  const float pi = atanf(1.0f) * 4.0f;
  float c1 = cosf(x1 / 180.0f * pi), c2 = cosf(x2 / 180.0f * pi);
  float c3 = cosf(y1 / 180.0f * pi - y2 / 180.0f * pi);
  float s1 = sinf(x1 / 180.0f * pi), s2 = sinf(x2 / 180.0f * pi);
  float v = c1 * c2 * c3 + s1 * s2;
  if (!(v < 1.0f)) v = (v != v) ? v : 1.0f;
  return 6371.393f * acosf(v);
}

/* schr2: Gaspari-Cohn with REAL(4) literals promoted to REAL(8) (letkf_yb.F90:262-286) */
double or_schr2(double ri) {
  double rci, rj, rk;
  if (ri > 2.0) {
    rci = 0.0;
  } else if (ri > 1.0) {
    rj = ri / 12.0 - 0.5;
    rj = rj * ri + 0.625;
    rj = rj * ri + (double)1.666667f;
    rci = (rj * ri - 5.0) * ri + 4.0 - (double)0.6666667f / ri;
  } else if (ri > 0.0) {
    rk = ri * ri;
    rj = (-0.25 * ri + 0.5) * ri + 0.625;
    rci = (rj * ri - (double)1.666667f) * rk + 1.0;
  } else {
    rci = 1.0;
  }
  return rci;
}

/* schr: box function (letkf_yb.F90:287-302) */
double or_schr(double ri) { return ri > 2.0 ? 0.0 : 1.0; }

/* ------------------------------------------------------------ the context */
typedef struct or_ctx {
  lg_config cfg;
  int var_start[LG_MAX_VARS]; /* 1-based start row of each DA variable */
  int n;                      /* rows per column */
  int x_sec, x_res, y_sec, y_res;
  float* gl;                  /* grid_lat_global(1..num_lat+1) stored 0-based */
  float* gn;                  /* grid_lon_global(1..num_lon+1) */
  double* ca;                 /* vertical coefficient a (nz+1) */
  double* cb;                 /* vertical coefficient b (nz+1) */
  double p0, ptop;
  /* blocks */
  int nblocks;
  int* bs_lat; int* be_lat; int* bs_lon; int* be_lon; /* 1-based */
  int* nb_off; int* nb_blk;                           /* neighbour blocks in traversal order */
  /* observations */
  int n_types;
  lg_obs_type types[LG_MAX_OBS_TYPES];
  int n_obs;
  int* otype; double* olat; double* olon;
  int64_t* ph_off; int64_t* val_off;
  double* oph; double* oyo; double* orinv;
  /* copies: block-major, then type, then obs index */
  int64_t n_copies;
  int* copy_obs; int* copy_block;
  int64_t* copy_entry_off;       /* n_copies + 1 */
  int64_t* blk_copy_off;         /* nblocks * n_types + 1 */
  int64_t n_entries;
  /* H(x) results per copy entry */
  double* yb;                    /* n_entries * ens */
  double* dis;
  double* lnp;                   /* log(ph) per entry */
  int hx_done;
} or_ctx;

/* pro_info_get_indx (pro_info.F90:96-125); x = latitude, y = longitude */
static void get_indx(const or_ctx* c, int bx, int by, int* tx_s, int* tx_e, int* ty_s, int* ty_e) {
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

#define GLAT(c, i) ((c)->gl[(i)-1])  /* grid_lat_global(i), 1-based */
#define GLON(c, i) ((c)->gn[(i)-1])

/* nearest_dist (letkf_init.F90:288-341), REAL(4) latitudes and distance */
static double nearest_dist(const or_ctx* c, int bx1, int by1, int bx2, int by2) {
  int xs1, xe1, ys1, ye1, xs2, xe2, ys2, ye2, tx1, tx2, ty1, ty2;
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
  float lat1 = GLAT(c, tx1), lat2 = GLAT(c, tx2);
  const double polar = c->cfg.obs_polar;
  if (fabs((double)lat1) > polar) lat1 = (float)(lat1 >= 0.0f ? fabs(polar) : -fabs(polar));
  if (fabs((double)lat2) > polar) lat2 = (float)(lat2 >= 0.0f ? fabs(polar) : -fabs(polar));
  const int gy = c->cfg.num_lon;
  if (by1 == by2) {
    return (double)or_latlon_dist_r4(lat1, GLON(c, ys1), lat2, GLON(c, ys2));
  }
  ty1 = ys1; ty2 = (ye2 % gy) + 1;
  float d1 = or_latlon_dist_r4(lat1, GLON(c, ty1), lat2, GLON(c, ty2));
  ty1 = (ye1 % gy) + 1; ty2 = ys2;
  float d2 = or_latlon_dist_r4(lat1, GLON(c, ty1), lat2, GLON(c, ty2));
  return (double)(d1 < d2 ? d1 : d2);
}

/* comm_info_init (letkf_init.F90:100-164): neighbour blocks of block (bx,by)
 * in gen_yb_dis traversal order (lat offset i outer, lon offset j inner). */
static int neighbour_blocks(const or_ctx* c, int bx, int by, int* out) {
  const int gnx = c->cfg.global_nx, gny = c->cfg.global_ny;
  const double L = c->cfg.local_dist;
  int s_lat, e_lat, s_lon, e_lon, tx_s, tx_e, ty_s, ty_e;
  get_indx(c, bx, by, &s_lat, &e_lat, &s_lon, &e_lon);
  int north_n = 0, south_n = 0;
  double x1 = GLAT(c, s_lat), y1 = GLON(c, s_lon), y2 = y1, x2;
  int tmp_bx = bx - 1;
  while (tmp_bx > 0) {
    get_indx(c, tmp_bx, by, &tx_s, &tx_e, &ty_s, &ty_e);
    x2 = GLAT(c, tx_e + 1);
    if (or_latlon_dist_r8(x1, y1, x2, y2) > L) break;
    north_n++;
    tmp_bx--;
  }
  tmp_bx = bx + 1;
  x1 = GLAT(c, e_lat + 1);
  while (tmp_bx <= gnx) {
    get_indx(c, tmp_bx, by, &tx_s, &tx_e, &ty_s, &ty_e);
    x2 = GLAT(c, tx_s);
    if (or_latlon_dist_r8(x1, y1, x2, y2) > L) break;
    south_n++;
    tmp_bx++;
  }
  int cnt = 0;
  for (int i = -north_n; i <= south_n; ++i) {
    int tbx = bx + i, west_n = 0, east_n = 0, tby = by;
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
      int nby = ((by + j - 1 + gny) % gny) + 1;
      if (out) out[cnt] = (nby - 1) * gnx + (tbx - 1);
      cnt++;
    }
  }
  return cnt;
}

/* %.5f-rounded box bound as Redis parses it (redis_wrapper.c:4165,4183) */
static double box_bound(float v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.5f", (double)v);
  return strtod(buf, NULL);
}

void or_destroy(or_ctx* c);

or_ctx* or_create(const lg_config* cfg, const float* grid_lat, const float* grid_lon,
                  const double* coef_a, const double* coef_b, double p0, double ptop,
                  const lg_obs_soa* obs, int* status) {
  *status = LG_ERR_ARG;
  if (!cfg || !grid_lat || !grid_lon || !coef_a || !obs) return NULL;
  or_ctx* c = (or_ctx*)calloc(1, sizeof(or_ctx));
  c->cfg = *cfg;
  const lg_config* g = &c->cfg;
  /* letkf_init.F90:63-73 */
  int cur = 1;
  for (int v = 0; v < g->n_var; ++v) {
    c->var_start[v] = cur;
    cur += g->var_lev[v];
  }
  c->n = cur - 1;
  /* init_da_parallel (module_da_parallel.F90:84-87) with the lat/lon roles of
   * pro_info_init's arguments (module_da_parallel.F90:134) */
  c->x_sec = g->num_lat / g->global_nx;
  c->x_res = g->num_lat % g->global_nx;
  c->y_sec = g->num_lon / g->global_ny;
  c->y_res = g->num_lon % g->global_ny;
  c->gl = (float*)malloc(sizeof(float) * (g->num_lat + 1));
  c->gn = (float*)malloc(sizeof(float) * (g->num_lon + 1));
  memcpy(c->gl, grid_lat, sizeof(float) * (g->num_lat + 1));
  memcpy(c->gn, grid_lon, sizeof(float) * (g->num_lon + 1));
  c->gl[g->num_lat] = 90.0f;   /* pro_info.F90:82-83 */
  c->gn[g->num_lon] = 360.0f;
  c->ca = (double*)malloc(sizeof(double) * (g->nz + 1));
  c->cb = (double*)calloc(g->nz + 1, sizeof(double));
  memcpy(c->ca, coef_a, sizeof(double) * (g->nz + 1));
  if (coef_b) memcpy(c->cb, coef_b, sizeof(double) * (g->nz + 1));
  c->p0 = p0;
  c->ptop = ptop;
  /* blocks and neighbour tables */
  c->nblocks = g->global_nx * g->global_ny;
  c->bs_lat = (int*)malloc(sizeof(int) * c->nblocks);
  c->be_lat = (int*)malloc(sizeof(int) * c->nblocks);
  c->bs_lon = (int*)malloc(sizeof(int) * c->nblocks);
  c->be_lon = (int*)malloc(sizeof(int) * c->nblocks);
  c->nb_off = (int*)malloc(sizeof(int) * (c->nblocks + 1));
  c->nb_off[0] = 0;
  for (int by = 1; by <= g->global_ny; ++by)
    for (int bx = 1; bx <= g->global_nx; ++bx) {
      int b = (by - 1) * g->global_nx + (bx - 1);
      get_indx(c, bx, by, &c->bs_lat[b], &c->be_lat[b], &c->bs_lon[b], &c->be_lon[b]);
      c->nb_off[b + 1] = c->nb_off[b] + neighbour_blocks(c, bx, by, NULL);
    }
  c->nb_blk = (int*)malloc(sizeof(int) * (c->nb_off[c->nblocks] + 1));
  for (int by = 1; by <= g->global_ny; ++by)
    for (int bx = 1; bx <= g->global_nx; ++bx) {
      int b = (by - 1) * g->global_nx + (bx - 1);
      neighbour_blocks(c, bx, by, c->nb_blk + c->nb_off[b]);
    }
  /* observations */
  c->n_types = obs->n_types;
  memcpy(c->types, obs->types, sizeof(lg_obs_type) * obs->n_types);
  c->n_obs = obs->n_obs;
  c->otype = (int*)malloc(sizeof(int) * (obs->n_obs + 1));
  c->olat = (double*)malloc(sizeof(double) * (obs->n_obs + 1));
  c->olon = (double*)malloc(sizeof(double) * (obs->n_obs + 1));
  c->ph_off = (int64_t*)malloc(sizeof(int64_t) * (obs->n_obs + 1));
  c->val_off = (int64_t*)malloc(sizeof(int64_t) * (obs->n_obs + 1));
  c->ph_off[0] = 0;
  c->val_off[0] = 0;
  for (int o = 0; o < obs->n_obs; ++o) {
    int t = obs->type[o];
    if (t < 0 || t >= obs->n_types) { or_destroy(c); *status = LG_ERR_ARG; return NULL; }
    c->otype[o] = t;
    c->olat[o] = obs->lat[o];
    c->olon[o] = obs->lon[o];
    c->ph_off[o + 1] = c->ph_off[o] + obs->types[t].nz;
    c->val_off[o + 1] = c->val_off[o] + (int64_t)obs->types[t].nz * obs->types[t].nvar;
  }
  for (int t = 0; t < obs->n_types; ++t)
    for (int v = 0; v < obs->types[t].nvar; ++v)
      if (obs->types[t].var[v] < 0 || obs->types[t].var[v] >= g->n_var) {
        or_destroy(c); *status = LG_ERR_VARNAME; return NULL;
      }
  size_t nph = (size_t)c->ph_off[obs->n_obs], nval = (size_t)c->val_off[obs->n_obs];
  c->oph = (double*)malloc(sizeof(double) * (nph + 1));
  c->oyo = (double*)malloc(sizeof(double) * (nval + 1));
  c->orinv = (double*)malloc(sizeof(double) * (nval + 1));
  memcpy(c->oph, obs->ph, sizeof(double) * nph);
  memcpy(c->oyo, obs->yo, sizeof(double) * nval);
  memcpy(c->orinv, obs->rinv, sizeof(double) * nval);
  /* block box queries (read_obs_mod.F90:147-148, redis_wrapper.c:4158-4296) */
  const int T = c->n_types;
  c->blk_copy_off = (int64_t*)calloc((size_t)c->nblocks * T + 1, sizeof(int64_t));
  double* lo_lat = (double*)malloc(sizeof(double) * c->nblocks);
  double* hi_lat = (double*)malloc(sizeof(double) * c->nblocks);
  double* lo_lon = (double*)malloc(sizeof(double) * c->nblocks);
  double* hi_lon = (double*)malloc(sizeof(double) * c->nblocks);
  for (int b = 0; b < c->nblocks; ++b) {
    lo_lat[b] = box_bound(GLAT(c, c->bs_lat[b]));
    hi_lat[b] = box_bound(GLAT(c, c->be_lat[b] + 1));
    lo_lon[b] = box_bound(GLON(c, c->bs_lon[b]));
    hi_lon[b] = box_bound(GLON(c, c->be_lon[b] + 1));
  }
  /* count pass then fill pass */
  for (int pass = 0; pass < 2; ++pass) {
    int64_t* fill = NULL;
    if (pass == 1) {
      for (size_t i = 0; i < (size_t)c->nblocks * T; ++i) c->blk_copy_off[i + 1] += c->blk_copy_off[i];
      c->n_copies = c->blk_copy_off[(size_t)c->nblocks * T];
      c->copy_obs = (int*)malloc(sizeof(int) * (c->n_copies + 1));
      c->copy_block = (int*)malloc(sizeof(int) * (c->n_copies + 1));
      fill = (int64_t*)malloc(sizeof(int64_t) * ((size_t)c->nblocks * T + 1));
      memcpy(fill, c->blk_copy_off, sizeof(int64_t) * ((size_t)c->nblocks * T));
    }
    for (int b = 0; b < c->nblocks; ++b)
      for (int o = 0; o < c->n_obs; ++o) {
        double la = c->olat[o], lo = c->olon[o];
        if (lo >= lo_lon[b] && lo <= hi_lon[b] && la >= lo_lat[b] && la <= hi_lat[b]) {
          size_t slot = (size_t)b * T + c->otype[o];
          if (pass == 0) {
            c->blk_copy_off[slot + 1]++;
          } else {
            int64_t j = fill[slot]++;
            c->copy_obs[j] = o;
            c->copy_block[j] = b;
          }
        }
      }
    free(fill);
  }
  free(lo_lat); free(hi_lat); free(lo_lon); free(hi_lon);
  c->copy_entry_off = (int64_t*)malloc(sizeof(int64_t) * (c->n_copies + 1));
  c->copy_entry_off[0] = 0;
  for (int64_t j = 0; j < c->n_copies; ++j) {
    const lg_obs_type* ty = &c->types[c->otype[c->copy_obs[j]]];
    c->copy_entry_off[j + 1] = c->copy_entry_off[j] + (int64_t)ty->nz * ty->nvar;
  }
  c->n_entries = c->copy_entry_off[c->n_copies];
  c->yb = (double*)malloc(sizeof(double) * ((size_t)c->n_entries * g->ens + 1));
  c->dis = (double*)malloc(sizeof(double) * (c->n_entries + 1));
  c->lnp = (double*)malloc(sizeof(double) * (c->n_entries + 1));
  *status = LG_OK;
  return c;
}

void or_destroy(or_ctx* c) {
  if (!c) return;
  free(c->gl); free(c->gn); free(c->ca); free(c->cb);
  free(c->bs_lat); free(c->be_lat); free(c->bs_lon); free(c->be_lon);
  free(c->nb_off); free(c->nb_blk);
  free(c->otype); free(c->olat); free(c->olon); free(c->ph_off); free(c->val_off);
  free(c->oph); free(c->oyo); free(c->orinv);
  free(c->copy_obs); free(c->copy_block); free(c->copy_entry_off); free(c->blk_copy_off);
  free(c->yb); free(c->dis); free(c->lnp);
  free(c);
}

int64_t or_n_copies(const or_ctx* c) { return c->n_copies; }
int64_t or_n_entries(const or_ctx* c) { return c->n_entries; }
int or_n_rows(const or_ctx* c) { return c->n; }

int or_copy_layout(const or_ctx* c, int* copy_obs, int* copy_block, int64_t* copy_entry_off) {
  if (copy_obs) memcpy(copy_obs, c->copy_obs, sizeof(int) * c->n_copies);
  if (copy_block) memcpy(copy_block, c->copy_block, sizeof(int) * c->n_copies);
  if (copy_entry_off) memcpy(copy_entry_off, c->copy_entry_off, sizeof(int64_t) * (c->n_copies + 1));
  return LG_OK;
}

int or_neighbour_table(const or_ctx* c, int* off, int* blk) {
  if (off) memcpy(off, c->nb_off, sizeof(int) * (c->nblocks + 1));
  if (blk) memcpy(blk, c->nb_blk, sizeof(int) * c->nb_off[c->nblocks]);
  return c->nb_off[c->nblocks];
}

/* index helpers for the Fortran arrays xb(ens, n, 1-h:nlat+h, 1-h:nlon+h) */
static inline size_t col_index(const lg_config* g, int glat, int glon) {
  /* glat, glon 1-based global, may be in the halo */
  size_t la = (size_t)(glat - 1 + g->halo), lo = (size_t)(glon - 1 + g->halo);
  return la + (size_t)(g->num_lat + 2 * g->halo) * lo;
}

/* da_vert_coord_calc_ph_lev (vert_coord_mod.F90:547-563), k 1-based */
static inline double calc_ph_lev(const or_ctx* c, int k, double phs) {
  if (c->cfg.vcoord == LG_VCOORD_SIGMA) return c->ca[k - 1] * (phs - c->ptop) + c->ptop;
  return c->ca[k - 1] * (c->p0 - c->ptop) + c->cb[k - 1] * (phs - c->ptop) + c->ptop;
}

/* gen_obs_struct for one copy: find_obs_grid (letkf_obs.F90:192-248),
 * ps2ph_3d_interp (obs_make.F90:345-381), obs_interpolation_3d_2
 * (obs_make.F90:233-342) and the member-mean removal (letkf_obs.F90:156-183). */
static int hx_copy(or_ctx* c, int64_t j, const double* xb, const double* axb,
                   double* xb_ph /* ens*(nz+1) */, int* ph_pos /* ens*obs_nz */) {
  const lg_config* g = &c->cfg;
  const int ens = g->ens, nz = g->nz, n = c->n;
  const int o = c->copy_obs[j], b = c->copy_block[j];
  const lg_obs_type* oty = &c->types[c->otype[o]];
  const int s_lat = c->bs_lat[b], e_lat = c->be_lat[b], s_lon = c->bs_lon[b], e_lon = c->be_lon[b];
  const int nxl = e_lat - s_lat + 1, nyl = e_lon - s_lon + 1;
  const double lat = c->olat[o], lon = c->olon[o];
  /* find_obs_grid on the block-local grid grid_lat(1:nx+1) */
  int tx = 0, ty = 0;
  for (int i = 1; i <= nxl + 1; ++i)
    if ((double)GLAT(c, s_lat + i - 1) >= lat) { tx = i; break; }
  for (int i = 1; i <= nyl + 1; ++i)
    if ((double)GLON(c, s_lon + i - 1) >= lon) { ty = i; break; }
  if (tx == 0 || ty == 0) return LG_ERR_OBS_OUTSIDE;
  double ax = 0.0, ay = 0.0;
  if (tx > 1) {
    float gt = GLAT(c, s_lat + tx - 1), gp = GLAT(c, s_lat + tx - 2);
    double dlat = (double)(gt - gp);       /* REAL(4) subtraction */
    ax = (dlat - lat + (double)gp) / dlat;
  }
  if (ty > 1) {
    float gt = GLON(c, s_lon + ty - 1), gp = GLON(c, s_lon + ty - 2);
    double dlon = (double)(gt - gp);
    ay = (dlon - lon + (double)gp) / dlon;
  }
  /* global indices of the 2x2 stencil: (tx-1, ty-1) (tx, ty-1) (tx-1, ty) (tx, ty) */
  const int la0 = s_lat + tx - 2, la1 = s_lat + tx - 1;
  const int lo0 = s_lon + ty - 2, lo1 = s_lon + ty - 1;
  const size_t c11 = col_index(g, la0, lo0), c21 = col_index(g, la1, lo0);
  const size_t c12 = col_index(g, la0, lo1), c22 = col_index(g, la1, lo1);
  const double t1 = ax, t2 = ay;
  const int ps = g->ps_index - 1;
  /* ps2ph_3d_interp */
  for (int e = 0; e < ens; ++e) {
    double r1 = (xb[e + (size_t)ens * (ps + (size_t)n * c11)] + axb[ps + (size_t)n * c11]) * t1 +
                (xb[e + (size_t)ens * (ps + (size_t)n * c21)] + axb[ps + (size_t)n * c21]) * (1.0 - t1);
    double r2 = (xb[e + (size_t)ens * (ps + (size_t)n * c12)] + axb[ps + (size_t)n * c12]) * t1 +
                (xb[e + (size_t)ens * (ps + (size_t)n * c22)] + axb[ps + (size_t)n * c22]) * (1.0 - t1);
    double ps_tmp = r1 * t2 + r2 * (1.0 - t2);
    double lev_prev = calc_ph_lev(c, 1, ps_tmp);
    for (int i = 1; i <= nz; ++i) {
      double lev_next = calc_ph_lev(c, i + 1, ps_tmp);
      xb_ph[e + ens * (i - 1)] = 0.5 * (lev_prev + lev_next);
      lev_prev = lev_next;
    }
    xb_ph[e + ens * nz] = xb_ph[e + ens * (nz - 1)];
  }
  /* obs_interpolation_3d_2 */
  const double* oph = c->oph + c->ph_off[o];
  const int onz = oty->nz, onv = oty->nvar;
  for (int e = 0; e < ens; ++e) {
    int jj = 1;
    for (int i = 1; i <= onz; ++i) {
      while (jj <= nz && oph[i - 1] > xb_ph[e + ens * (jj - 1)]) jj++;
      ph_pos[e + ens * (i - 1)] = jj - 1;
    }
  }
  const int64_t ebase = c->copy_entry_off[j];
#define XB(e, r, cc) (xb[(e) + (size_t)ens * ((r) + (size_t)n * (cc))])
#define AXB(r, cc) (axb[(r) + (size_t)n * (cc)])
  for (int l = 1; l <= onz; ++l)
    for (int k = 1; k <= onv; ++k) {
      const int vid = oty->var[k - 1];
      double* ybo = c->yb + (size_t)(ebase + (l - 1) * onv + (k - 1)) * ens;
      if (g->var_lev[vid] > 1) {
        for (int e = 0; e < ens; ++e) {
          const int pp = ph_pos[e + ens * (l - 1)];
          if (pp >= 1 && pp < nz) {
            const int tl = c->var_start[vid] + pp - 1 - 1; /* 0-based row */
            const double php1 = xb_ph[e + ens * pp], php = xb_ph[e + ens * (pp - 1)];
            double t3 = (log(php1) - log(oph[l - 1])) / (log(php1) - log(php));
            double r1 = (XB(e, tl, c11) + AXB(tl, c11)) * t1 + (XB(e, tl, c21) + AXB(tl, c21)) * (1.0 - t1);
            double r2 = (XB(e, tl, c12) + AXB(tl, c12)) * t1 + (XB(e, tl, c22) + AXB(tl, c22)) * (1.0 - t1);
            double r3 = (XB(e, tl + 1, c11) + AXB(tl + 1, c11)) * t1 +
                        (XB(e, tl + 1, c21) + AXB(tl + 1, c21)) * (1.0 - t1);
            double r4 = (XB(e, tl + 1, c12) + AXB(tl + 1, c12)) * t1 +
                        (XB(e, tl + 1, c22) + AXB(tl + 1, c22)) * (1.0 - t1);
            r1 = r1 * t2 + r2 * (1.0 - t2);
            r3 = r3 * t2 + r4 * (1.0 - t2);
            ybo[e] = r1 * t3 + r3 * (1.0 - t3);
          } else {
            const int tl = (pp == 0 ? c->var_start[vid] : c->var_start[vid] + nz - 1) - 1;
            double r1 = (XB(e, tl, c11) + AXB(tl, c11)) * t1 + (XB(e, tl, c21) + AXB(tl, c21)) * (1.0 - t1);
            double r2 = (XB(e, tl, c12) + AXB(tl, c12)) * t1 + (XB(e, tl, c22) + AXB(tl, c22)) * (1.0 - t1);
            ybo[e] = r1 * t2 + r2 * (1.0 - t2);
          }
        }
      } else {
        const int tl = c->var_start[vid] - 1;
        for (int e = 0; e < ens; ++e) {
          double r1 = (XB(e, tl, c11) + AXB(tl, c11)) * t1 + (XB(e, tl, c21) + AXB(tl, c21)) * (1.0 - t1);
          double r2 = (XB(e, tl, c12) + AXB(tl, c12)) * t1 + (XB(e, tl, c22) + AXB(tl, c22)) * (1.0 - t1);
          ybo[e] = r1 * t2 + r2 * (1.0 - t2);
        }
      }
    }
#undef XB
#undef AXB
  /* mean removal (letkf_obs.F90:156-183) */
  const double* yo = c->oyo + c->val_off[o];
  for (int l = 0; l < onz; ++l)
    for (int k = 0; k < onv; ++k) {
      const int64_t ent = ebase + l * onv + k;
      double* ybo = c->yb + (size_t)ent * ens;
      double sum_y = 0.0;
      for (int e = 0; e < ens; ++e) sum_y = sum_y + ybo[e];
      sum_y = sum_y / (double)ens;
      c->dis[ent] = yo[l * onv + k] - sum_y;
      for (int e = 0; e < ens; ++e) ybo[e] = ybo[e] - sum_y;
      c->lnp[ent] = log(oph[l]);  /* letkf_yb.F90:211 (with the observation's own ph) */
    }
  return LG_OK;
}

int or_hx(or_ctx* c, const double* xb, const double* axb, int nthreads) {
  const int ens = c->cfg.ens, nz = c->cfg.nz;
  int maxonz = 1;
  for (int t = 0; t < c->n_types; ++t)
    if (c->types[t].nz > maxonz) maxonz = c->types[t].nz;
  int status = LG_OK;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    double* xb_ph = (double*)malloc(sizeof(double) * ens * (nz + 1));
    int* ph_pos = (int*)malloc(sizeof(int) * ens * maxonz);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
    for (int64_t j = 0; j < c->n_copies; ++j) {
      int s = hx_copy(c, j, xb, axb, xb_ph, ph_pos);
      if (s != LG_OK) status = s;
    }
    free(xb_ph);
    free(ph_pos);
  }
  c->hx_done = (status == LG_OK);
  return status;
}

/* H(x) of the block copies [j0, j1) only (one shard's own copies); the other
 * entries keep what they hold (set them with or_set_hx_rows) */
int or_hx_range(or_ctx* c, const double* xb, const double* axb, int64_t j0, int64_t j1,
                int nthreads) {
  const int ens = c->cfg.ens, nz = c->cfg.nz;
  if (j0 < 0 || j1 > c->n_copies || j0 > j1) return LG_ERR_ARG;
  int maxonz = 1;
  for (int t = 0; t < c->n_types; ++t)
    if (c->types[t].nz > maxonz) maxonz = c->types[t].nz;
  int status = LG_OK;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    double* xb_ph = (double*)malloc(sizeof(double) * ens * (nz + 1));
    int* ph_pos = (int*)malloc(sizeof(int) * ens * maxonz);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
    for (int64_t j = j0; j < j1; ++j) {
      int s = hx_copy(c, j, xb, axb, xb_ph, ph_pos);
      if (s != LG_OK) status = s;
    }
    free(xb_ph);
    free(ph_pos);
  }
  c->hx_done = (status == LG_OK);
  return status;
}

/* H(x) rows of entries [e0, e1), ens + 2 doubles each: yb[ens], dis, ln p */
int or_get_hx_rows(const or_ctx* c, double* rows, int64_t e0, int64_t e1) {
  const int ens = c->cfg.ens;
  if (e0 < 0 || e1 > c->n_entries || e0 > e1) return LG_ERR_ARG;
  for (int64_t e = e0; e < e1; ++e) {
    double* r = rows + (size_t)(e - e0) * (ens + 2);
    memcpy(r, c->yb + (size_t)e * ens, sizeof(double) * ens);
    r[ens] = c->dis[e];
    r[ens + 1] = c->lnp[e];
  }
  return LG_OK;
}

int or_set_hx_rows(or_ctx* c, const double* rows, int64_t e0, int64_t e1) {
  const int ens = c->cfg.ens;
  if (e0 < 0 || e1 > c->n_entries || e0 > e1) return LG_ERR_ARG;
  for (int64_t e = e0; e < e1; ++e) {
    const double* r = rows + (size_t)(e - e0) * (ens + 2);
    memcpy(c->yb + (size_t)e * ens, r, sizeof(double) * ens);
    c->dis[e] = r[ens];
    c->lnp[e] = r[ens + 1];
  }
  c->hx_done = 1;
  return LG_OK;
}

int or_get_hx(const or_ctx* c, double* yb, double* dis, double* lnp) {
  if (!c->hx_done) return LG_ERR_STATE;
  if (yb) memcpy(yb, c->yb, sizeof(double) * c->n_entries * c->cfg.ens);
  if (dis) memcpy(dis, c->dis, sizeof(double) * c->n_entries);
  if (lnp) memcpy(lnp, c->lnp, sizeof(double) * c->n_entries);
  return LG_OK;
}

/* block of a global column (1-based lat/lon) */
static int column_block(const or_ctx* c, int glat, int glon) {
  int bx = 1, by = 1, s, e, s2, e2;
  for (bx = 1; bx <= c->cfg.global_nx; ++bx) {
    get_indx(c, bx, 1, &s, &e, &s2, &e2);
    if (glat >= s && glat <= e) break;
  }
  for (by = 1; by <= c->cfg.global_ny; ++by) {
    get_indx(c, 1, by, &s, &e, &s2, &e2);
    if (glon >= s2 && glon <= e2) break;
  }
  return (by - 1) * c->cfg.global_nx + (bx - 1);
}

/* gen_yb_dis / gen_yb_dis_vertical selection (letkf_yb.F90:3-150,154-238) for
 * column c = (glon-1)*num_lat + (glat-1).  Writes copy-entry indices and the
 * horizontal localisation; returns nobsl, or -1 if the capacity is exceeded.
 * *band counts candidates whose ri lies within 1e-12 of 2. */
int or_column_list(const or_ctx* c, int col, int* entries, double* rloc, int cap, int* capped,
                   int64_t* band) {
  const lg_config* g = &c->cfg;
  const int glat = col % g->num_lat + 1, glon = col / g->num_lat + 1;
  const int b = column_block(c, glat, glon);
  const double center_lat = (double)GLAT(c, glat), center_lon = (double)GLON(c, glon);
  const int T = c->n_types;
  int nobsl = 0;
  if (capped) *capped = 0;
  for (int q = c->nb_off[b]; q < c->nb_off[b + 1]; ++q) {
    const int nbk = c->nb_blk[q];
    for (int t = 0; t < T; ++t) {
      const int64_t j0 = c->blk_copy_off[(size_t)nbk * T + t], j1 = c->blk_copy_off[(size_t)nbk * T + t + 1];
      for (int64_t j = j0; j < j1; ++j) {
        const int o = c->copy_obs[j];
        if (!(fabs(c->olat[o]) <= g->obs_polar)) continue;
        double dist = or_latlon_dist_r8(c->olat[o], c->olon[o], center_lat, center_lon);
        double ri = dist * 1.0 / g->local_dist;
        if (band && fabs(ri - 2.0) < 1e-12) (*band)++;
        double gc = g->gc_filter ? or_schr2(ri) : or_schr(ri);
        if (!(gc > 0.0)) continue;
        const int64_t nent = c->copy_entry_off[j + 1] - c->copy_entry_off[j];
        for (int64_t m = 0; m < nent; ++m) {
          if (entries) {
            if (nobsl >= cap) return -1;
            entries[nobsl] = (int)(c->copy_entry_off[j] + m);
            rloc[nobsl] = gc;
          }
          nobsl++;
          if (g->max_obs > 0 && nobsl >= g->max_obs) {
            if (capped) *capped = 1;
            return nobsl;
          }
        }
      }
    }
  }
  return nobsl;
}

/* letkf_core (letkf_core.F90:14-233), step for step.
 * ws must hold 4*k*k + 2*k*p + 2*p + 2*k*k+6*k+1 + k doubles; iws 5*k+3 ints. */
static int core_ws(int k, int p, const double* hxens_in, const float* rdiaginv, const double* dep,
                   const double* rloc, double infl, double* trans, double* wbar, double* ws,
                   int* iws) {
  double* work1 = ws;
  double* eivec = work1 + k * k;
  double* pa = eivec + k * k;
  double* scratch = pa + k * k;
  double* eival = scratch + k * k;
  double* hx = eival + k;
  double* work2 = hx + (size_t)k * p;
  double* rrloc = work2 + (size_t)k * p;
  double* lwork = rrloc + p;
  for (int nob = 0; nob < p; ++nob) {
    rrloc[nob] = (double)rdiaginv[nob] * rloc[nob];
    rrloc[nob] = sqrt(rrloc[nob]);
    for (int i = 0; i < k; ++i) hx[i + (size_t)k * nob] = hxens_in[i + (size_t)k * nob] * rrloc[nob];
  }
  gemm('n', 't', k, k, p, hx, k, hx, k, work1, k);
  int ierr = syevd(k, work1, eival, lwork, iws, scratch);
  const double rho = 1.0;
  for (int i = 0; i < k; ++i) eival[i] = eival[i] * rho + (double)(k - 1) / infl;
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) {
      eivec[i + k * j] = work1[i + k * j];
      work1[i + k * j] = work1[i + k * j] / eival[j];
    }
  gemm('n', 't', k, k, k, work1, k, eivec, k, pa, k);
  for (int nob = 0; nob < p; ++nob)
    for (int i = 0; i < k; ++i) hx[i + (size_t)k * nob] = hx[i + (size_t)k * nob] * rrloc[nob];
  gemm('n', 'n', k, p, k, pa, k, hx, k, work2, k);
  for (int i = 0; i < k; ++i) wbar[i] = 0.0;
  for (int nob = 0; nob < p; ++nob)
    for (int i = 0; i < k; ++i) wbar[i] = wbar[i] + work2[i + (size_t)k * nob] * dep[nob];
  for (int j = 0; j < k; ++j) {
    double r = sqrt((double)(k - 1) / eival[j]);
    for (int i = 0; i < k; ++i) work1[i + k * j] = eivec[i + k * j] * r;
  }
  gemm('n', 't', k, k, k, work1, k, eivec, k, trans, k);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) trans[i + k * j] = trans[i + k * j] + wbar[i];
  return ierr;
}

static size_t core_ws_doubles(int k, int p) {
  return (size_t)5 * k * k + 2 * (size_t)k * p + 2 * (size_t)p + 2 * (size_t)k * k + 6 * k + 1 + k + 64;
}

int or_core(int k, int p, const double* hxens, const float* rdiaginv, const double* dep,
            const double* rloc, double infl, double* trans, double* wbar) {
  double* ws = (double*)malloc(sizeof(double) * core_ws_doubles(k, p));
  int* iws = (int*)malloc(sizeof(int) * (5 * k + 3));
  int r = core_ws(k, p, hxens, rdiaginv, dep, rloc, infl, trans, wbar, ws, iws);
  free(ws);
  free(iws);
  return r;
}

/* one column: selection, core(s), update (letkf_compute.F90:12-154 and 386-554) */
typedef struct col_ws {
  int cap;
  int* ent; double* rloc_h; double* rloc; float* rdiag; double* dep; double* yb; double* lnp;
  double* ws; size_t ws_n; int* iws;
  double* trans; double* wbar; double* alnp; double* xcol;
} col_ws;

static void ws_ensure(col_ws* w, int k, int nz, int need) {
  if (need <= w->cap) return;
  int cap = need + need / 2 + 64;
  w->ent = (int*)realloc(w->ent, sizeof(int) * cap);
  w->rloc_h = (double*)realloc(w->rloc_h, sizeof(double) * cap);
  w->rloc = (double*)realloc(w->rloc, sizeof(double) * cap);
  w->rdiag = (float*)realloc(w->rdiag, sizeof(float) * cap);
  w->dep = (double*)realloc(w->dep, sizeof(double) * cap);
  w->lnp = (double*)realloc(w->lnp, sizeof(double) * cap);
  w->yb = (double*)realloc(w->yb, sizeof(double) * (size_t)cap * k);
  w->ws_n = core_ws_doubles(k, cap);
  w->ws = (double*)realloc(w->ws, sizeof(double) * w->ws_n);
  w->cap = cap;
  (void)nz;
}

/* gen_yb_dis[_vertical] for column col into w: yb, dep, rdiaginv, horizontal
 * rloc and obs ln p of the list; returns nobsl (< 0 on a capacity error) */
static int gather_list(const or_ctx* c, int col, col_ws* w, int* capped, int64_t* band) {
  const lg_config* g = &c->cfg;
  const int k = g->ens, nz = g->nz;
  int nobsl = or_column_list(c, col, NULL, NULL, 0, NULL, NULL);
  ws_ensure(w, k, nz, nobsl + 1);
  nobsl = or_column_list(c, col, w->ent, w->rloc_h, w->cap, capped, band);
  if (nobsl < 0) return nobsl;
  for (int i = 0; i < nobsl; ++i) {
    const int64_t ent = w->ent[i];
    memcpy(w->yb + (size_t)i * k, c->yb + (size_t)ent * k, sizeof(double) * k);
    w->dep[i] = c->dis[ent];
    /* rdiaginv is REAL(4) (letkf_compute.F90:30): entry -> its observation value */
    int64_t lo = 0, hi = c->n_copies;  /* copy of this entry by binary search */
    while (hi - lo > 1) {
      int64_t mid = (lo + hi) / 2;
      if (c->copy_entry_off[mid] <= ent) lo = mid; else hi = mid;
    }
    const int o = c->copy_obs[lo];
    const int64_t m = ent - c->copy_entry_off[lo];
    w->rdiag[i] = (float)c->orinv[c->val_off[o] + m];
    w->lnp[i] = c->lnp[ent];
  }
  return nobsl;
}

static int analyse_column(const or_ctx* c, int col, const double* xb, const double* axb,
                          double* xa, double* axa, col_ws* w, lg_stats* st) {
  const lg_config* g = &c->cfg;
  const int k = g->ens, nz = g->nz, n = c->n;
  const int glat = col % g->num_lat + 1, glon = col / g->num_lat + 1;
  int capped = 0;
  int64_t band = 0;
  const int nobsl = gather_list(c, col, w, &capped, &band);
  if (nobsl < 0) return LG_ERR_SHAPE;
  const size_t cc = col_index(g, glat, glon);
  double* xcol = xa + (size_t)k * n * cc;
  double* acol = axa + (size_t)n * cc;
  const double* xbc = xb + (size_t)k * n * cc;
  const double* abc = axb + (size_t)n * cc;
  int ierr = 0;
  if (g->vert_dist <= 0.0) {
    ierr |= core_ws(k, nobsl, w->yb, w->rdiag, w->dep, w->rloc_h, g->inflation, w->trans, w->wbar,
                    w->ws, w->iws);
    /* xb_2_xa (letkf_compute.F90:259-329) */
    gemm('t', 'n', k, n, k, w->trans, k, xbc, k, xcol, k);
    for (int r = 0; r < n; ++r)
      for (int e = 0; e < k; ++e) xcol[e + (size_t)k * r] = xcol[e + (size_t)k * r] + abc[r];
    if (st) st->n_solves++;
  } else {
    /* ps2alnp (obs_make.F90:418-437), ph_lev(nz+1) computed */
    const double aps = abc[g->ps_index - 1];
    for (int i = 1; i <= nz; ++i) {
      double v = 0.5 * (calc_ph_lev(c, i, aps) + calc_ph_lev(c, i + 1, aps));
      w->alnp[i - 1] = log(v);
    }
    for (int kk = 1; kk <= nz; ++kk) {  /* cube_nz = 1: sk = ek = center_k = kk */
      const double al = w->alnp[kk - 1];
      for (int i = 0; i < nobsl; ++i) {  /* vertical_localization (letkf_yb.F90:240-260) */
        double z = fabs(al - w->lnp[i]) / g->vert_dist;
        w->rloc[i] = w->rloc_h[i] * (g->gc_filter_vertical ? or_schr2(z) : or_schr(z));
      }
      ierr |= core_ws(k, nobsl, w->yb, w->rdiag, w->dep, w->rloc, g->inflation, w->trans, w->wbar,
                      w->ws, w->iws);
      if (st) st->n_solves++;
      for (int v = 0; v < g->n_var; ++v) {
        if (g->var_lev[v] == 1) {
          if (kk != nz) continue;
          const int r = c->var_start[v] - 1;
          for (int e = 0; e < k; ++e) {
            double s = 0.0;
            for (int i = 0; i < k; ++i) s += xbc[i + (size_t)k * r] * w->trans[i + k * e];
            xcol[e + (size_t)k * r] = abc[r] + s;
          }
        } else {
          const int r = c->var_start[v] + kk - 1 - 1;
          for (int e = 0; e < k; ++e) {
            double s = 0.0;
            for (int i = 0; i < k; ++i) s += xbc[i + (size_t)k * r] * w->trans[i + k * e];
            xcol[e + (size_t)k * r] = abc[r] + s;
          }
        }
      }
    }
  }
  /* recentre (letkf_compute.F90:314-327, 539-552) */
  for (int r = 0; r < n; ++r) {
    double s = 0.0;
    for (int e = 0; e < k; ++e) s = s + xcol[e + (size_t)k * r];
    s = s / (double)k;
    acol[r] = s;
    for (int e = 0; e < k; ++e) xcol[e + (size_t)k * r] = xcol[e + (size_t)k * r] - s;
  }
  if (st) {
    st->n_columns++;
    st->nobsl_total += nobsl;
    if (nobsl > st->nobsl_max) st->nobsl_max = nobsl;
    st->n_capped += capped;
    st->n_band += band;
    st->n_eig_fail += ierr != 0;
  }
  return LG_OK;
}

/* One cube of letkf_compute_nooverlap[_vertical] (letkf_compute.F90:12-154,
 * 386-554) or of letkf_compute with overlapping cubes (:156-256): block b,
 * block-local latitudes sj..ej and longitudes si..ei (1-based).  The list is
 * the one of the cube's centre grid point (gen_yb_dis at grid((sj+ej)/2),
 * grid((si+ei)/2), letkf_yb.F90:23-24,165-166).
 *   accumulate = 0: xb_2_xa / the vertical update into xa, then recentred;
 *   accumulate = 1: xb_add2_xa (:332-382): each column's recentred analysis
 *                   and mean are added to xa, axa (averaged by the caller). */
static int analyse_cube(const or_ctx* c, int b, int sj, int ej, int si, int ei, const double* xb,
                        const double* axb, double* xa, double* axa, col_ws* w, lg_stats* st,
                        int accumulate) {
  const lg_config* g = &c->cfg;
  const int k = g->ens, nz = g->nz, n = c->n;
  const int glat0 = c->bs_lat[b] - 1, glon0 = c->bs_lon[b] - 1;  /* local 1 -> global */
  const int cglat = glat0 + (sj + ej) / 2, cglon = glon0 + (si + ei) / 2;
  const int ccol = (cglon - 1) * g->num_lat + (cglat - 1);
  int capped = 0;
  int64_t band = 0;
  const int nobsl = gather_list(c, ccol, w, &capped, &band);
  if (nobsl < 0) return LG_ERR_SHAPE;
  int ierr = 0;
  if (accumulate || g->vert_dist <= 0.0) {
    ierr |= core_ws(k, nobsl, w->yb, w->rdiag, w->dep, w->rloc_h, g->inflation, w->trans, w->wbar,
                    w->ws, w->iws);
    if (st) st->n_solves++;
    for (int ii = si; ii <= ei; ++ii)
      for (int jj = sj; jj <= ej; ++jj) {
        const size_t cc = col_index(g, glat0 + jj, glon0 + ii);
        double* xcol = xa + (size_t)k * n * cc;
        double* acol = axa + (size_t)n * cc;
        const double* xbc = xb + (size_t)k * n * cc;
        const double* abc = axb + (size_t)n * cc;
        for (int r = 0; r < n; ++r) {
          double* dist = w->xcol;  /* k */
          double mean = 0.0;
          for (int e = 0; e < k; ++e) {
            double sum = 0.0;
            for (int i = 0; i < k; ++i) sum += xbc[i + (size_t)k * r] * w->trans[i + k * e];
            dist[e] = abc[r] + sum;
            mean = mean + dist[e];
          }
          mean = mean / (double)k;
          if (accumulate) {
            acol[r] += mean;
            for (int e = 0; e < k; ++e) xcol[e + (size_t)k * r] += dist[e] - mean;
          } else {
            acol[r] = mean;
            for (int e = 0; e < k; ++e) xcol[e + (size_t)k * r] = dist[e] - mean;
          }
        }
      }
  } else {
    /* ps2alnp at the centre column, one solve per level group */
    const double aps = axb[(size_t)n * col_index(g, cglat, cglon) + g->ps_index - 1];
    for (int i = 1; i <= nz; ++i) {
      double v = 0.5 * (calc_ph_lev(c, i, aps) + calc_ph_lev(c, i + 1, aps));
      w->alnp[i - 1] = log(v);
    }
    for (int kk = 1; kk <= nz; kk += g->cube_nz) {
      const int sk = kk, ek = kk + g->cube_nz - 1 > nz ? nz : kk + g->cube_nz - 1;
      const double al = w->alnp[(sk + ek) / 2 - 1];
      for (int i = 0; i < nobsl; ++i) {  /* vertical_localization (letkf_yb.F90:240-260) */
        double z = fabs(al - w->lnp[i]) / g->vert_dist;
        w->rloc[i] = w->rloc_h[i] * (g->gc_filter_vertical ? or_schr2(z) : or_schr(z));
      }
      ierr |= core_ws(k, nobsl, w->yb, w->rdiag, w->dep, w->rloc, g->inflation, w->trans, w->wbar,
                      w->ws, w->iws);
      if (st) st->n_solves++;
      for (int ii = si; ii <= ei; ++ii)
        for (int jj = sj; jj <= ej; ++jj) {
          const size_t cc = col_index(g, glat0 + jj, glon0 + ii);
          double* xcol = xa + (size_t)k * n * cc;
          const double* xbc = xb + (size_t)k * n * cc;
          const double* abc = axb + (size_t)n * cc;
          for (int v = 0; v < g->n_var; ++v) {
            int r0, r1;  /* 0-based rows updated by this group */
            if (g->var_lev[v] == 1) {
              if (ek != nz) continue;
              r0 = r1 = c->var_start[v] - 1;
            } else {
              r0 = c->var_start[v] + sk - 2;
              r1 = c->var_start[v] + ek - 2;
            }
            for (int r = r0; r <= r1; ++r)
              for (int e = 0; e < k; ++e) {
                double sum = 0.0;
                for (int i = 0; i < k; ++i) sum += xbc[i + (size_t)k * r] * w->trans[i + k * e];
                xcol[e + (size_t)k * r] = abc[r] + sum;
              }
          }
        }
    }
    /* recentre the cube's columns (letkf_compute.F90:539-552) */
    for (int ii = si; ii <= ei; ++ii)
      for (int jj = sj; jj <= ej; ++jj) {
        const size_t cc = col_index(g, glat0 + jj, glon0 + ii);
        double* xcol = xa + (size_t)k * n * cc;
        double* acol = axa + (size_t)n * cc;
        for (int r = 0; r < n; ++r) {
          double sum = 0.0;
          for (int e = 0; e < k; ++e) sum = sum + xcol[e + (size_t)k * r];
          sum = sum / (double)k;
          acol[r] = sum;
          for (int e = 0; e < k; ++e) xcol[e + (size_t)k * r] = xcol[e + (size_t)k * r] - sum;
        }
      }
  }
  if (st) {
    st->n_columns += (int64_t)(ei - si + 1) * (ej - sj + 1);
    st->nobsl_total += nobsl;
    if (nobsl > st->nobsl_max) st->nobsl_max = nobsl;
    st->n_capped += capped;
    st->n_band += band;
    st->n_eig_fail += ierr != 0;
  }
  return LG_OK;
}

/* cube analysis of block b: the cube loops of letkf_compute_nooverlap[_vertical]
 * (overlap 0: stride cube_n) or letkf_compute (stride cube_n - overlap, each
 * column averaged over the cubes that cover it) */
static int analyse_block_cubes(const or_ctx* c, int b, const double* xb, const double* axb,
                               double* xa, double* axa, col_ws* w, lg_stats* st) {
  const lg_config* g = &c->cfg;
  const int k = g->ens, n = c->n;
  const int nxl = c->be_lat[b] - c->bs_lat[b] + 1, nyl = c->be_lon[b] - c->bs_lon[b] + 1;
  const int ov = g->overlap, stride = g->cube_n - ov;
  int status = LG_OK;
  double* cnt = NULL;
  if (ov > 0) {
    cnt = (double*)calloc((size_t)nxl * nyl, sizeof(double));
    for (int ii = 1; ii <= nyl; ++ii)
      for (int jj = 1; jj <= nxl; ++jj) {
        const size_t cc = col_index(g, c->bs_lat[b] - 1 + jj, c->bs_lon[b] - 1 + ii);
        memset(xa + (size_t)k * n * cc, 0, sizeof(double) * k * n);
        memset(axa + (size_t)n * cc, 0, sizeof(double) * n);
      }
  }
  for (int i = 1; i <= nyl; i += stride) {
    const int si = i, ei = i + g->cube_n - 1 > nyl ? nyl : i + g->cube_n - 1;
    for (int j = 1; j <= nxl; j += stride) {
      const int sj = j, ej = j + g->cube_n - 1 > nxl ? nxl : j + g->cube_n - 1;
      const int r = analyse_cube(c, b, sj, ej, si, ei, xb, axb, xa, axa, w, st, ov > 0);
      if (r != LG_OK) status = r;
      if (cnt)
        for (int ii = si; ii <= ei; ++ii)
          for (int jj = sj; jj <= ej; ++jj) cnt[(size_t)(ii - 1) * nxl + (jj - 1)] += 1.0;
    }
  }
  if (cnt) {
    for (int ii = 1; ii <= nyl; ++ii)
      for (int jj = 1; jj <= nxl; ++jj) {
        const double q = cnt[(size_t)(ii - 1) * nxl + (jj - 1)];
        const size_t cc = col_index(g, c->bs_lat[b] - 1 + jj, c->bs_lon[b] - 1 + ii);
        for (size_t e = 0; e < (size_t)k * n; ++e) xa[(size_t)k * n * cc + e] /= q;
        for (int r = 0; r < n; ++r) axa[(size_t)n * cc + r] /= q;
      }
    free(cnt);
  }
  return status;
}

/* letkf_core on column col's horizontal list (gen_yb_dis + letkf_core):
 * trans(k x k, column-major), for tests of the cube paths */
int or_column_trans(const or_ctx* c, int col, double* trans) {
  if (!c->hx_done) return LG_ERR_STATE;
  const int k = c->cfg.ens;
  col_ws w;
  memset(&w, 0, sizeof w);
  w.iws = (int*)malloc(sizeof(int) * (5 * k + 3));
  w.wbar = (double*)malloc(sizeof(double) * k);
  int capped = 0;
  int64_t band = 0;
  const int nobsl = gather_list(c, col, &w, &capped, &band);
  int r = nobsl < 0 ? LG_ERR_SHAPE : LG_OK;
  if (r == LG_OK && core_ws(k, nobsl, w.yb, w.rdiag, w.dep, w.rloc_h, c->cfg.inflation, trans,
                            w.wbar, w.ws, w.iws) != 0)
    r = LG_ERR_EIG;
  free(w.ent); free(w.rloc_h); free(w.rloc); free(w.rdiag); free(w.dep); free(w.yb); free(w.lnp);
  free(w.ws); free(w.iws); free(w.wbar);
  return r;
}

/* analysis of global columns [c0, c1) after or_hx; with cubes, the whole globe */
int or_analysis(const or_ctx* c, const double* xb, const double* axb, double* xa, double* axa,
                int c0, int c1, int nthreads, lg_stats* st_out) {
  if (!c->hx_done) return LG_ERR_STATE;
  const lg_config* g = &c->cfg;
  const int k = g->ens;
  /* cube_n > 1, cube_nz > 1 or overlap > 0: whole blocks of cubes (the whole
   * globe only; overlapping cubes are averaged across each block) */
  const int cubes = g->cube_n > 1 || g->overlap > 0 || (g->cube_nz > 1 && g->vert_dist > 0.0);
  if (g->cube_n < 1 || g->cube_nz < 1 || g->overlap < 0 || g->overlap >= g->cube_n)
    return LG_ERR_ARG;  /* the reference's cube loops would not advance */
  if (cubes && (c0 != 0 || c1 != g->num_lat * g->num_lon)) return LG_ERR_ARG;
  int status = LG_OK;
  lg_stats tot;
  memset(&tot, 0, sizeof tot);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    col_ws w;
    memset(&w, 0, sizeof w);
    w.iws = (int*)malloc(sizeof(int) * (5 * k + 3));
    w.trans = (double*)malloc(sizeof(double) * k * k);
    w.wbar = (double*)malloc(sizeof(double) * k);
    w.alnp = (double*)malloc(sizeof(double) * (g->nz + 1));
    w.xcol = (double*)malloc(sizeof(double) * k);
    lg_stats st;
    memset(&st, 0, sizeof st);
    if (cubes) {
      /* cubes never cross blocks: blocks in parallel, each block's cubes in order */
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int b = 0; b < c->nblocks; ++b) {
        int s = analyse_block_cubes(c, b, xb, axb, xa, axa, &w, &st);
        if (s != LG_OK) status = s;
      }
    } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int col = c0; col < c1; ++col) {
        int s = analyse_column(c, col, xb, axb, xa, axa, &w, &st);
        if (s != LG_OK) status = s;
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      tot.n_columns += st.n_columns;
      tot.n_solves += st.n_solves;
      tot.nobsl_total += st.nobsl_total;
      if (st.nobsl_max > tot.nobsl_max) tot.nobsl_max = st.nobsl_max;
      tot.n_capped += st.n_capped;
      tot.n_band += st.n_band;
      tot.n_eig_fail += st.n_eig_fail;
    }
    free(w.ent); free(w.rloc_h); free(w.rloc); free(w.rdiag); free(w.dep); free(w.yb); free(w.lnp);
    free(w.ws); free(w.iws); free(w.trans); free(w.wbar); free(w.alnp); free(w.xcol);
  }
  tot.n_copies = c->n_copies;
  tot.n_entries = c->n_entries;
  if (st_out) *st_out = tot;
  return status;
}

/* analysis of the listed global columns (any order, each once) after or_hx:
 * the per-column path of or_analysis over a sample spread across the globe,
 * for bounded CPU timings and sampled parity checks (no cubes) */
int or_analysis_cols(const or_ctx* c, const double* xb, const double* axb, double* xa,
                     double* axa, const int* cols, int ncols, int nthreads, lg_stats* st_out) {
  if (!c->hx_done) return LG_ERR_STATE;
  const lg_config* g = &c->cfg;
  const int k = g->ens;
  const int ncol_all = g->num_lat * g->num_lon;
  if (g->cube_n > 1 || g->overlap > 0 || (g->cube_nz > 1 && g->vert_dist > 0.0))
    return LG_ERR_UNSUPPORTED;
  for (int i = 0; i < ncols; ++i)
    if (cols[i] < 0 || cols[i] >= ncol_all) return LG_ERR_ARG;
  int status = LG_OK;
  lg_stats tot;
  memset(&tot, 0, sizeof tot);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    col_ws w;
    memset(&w, 0, sizeof w);
    w.iws = (int*)malloc(sizeof(int) * (5 * k + 3));
    w.trans = (double*)malloc(sizeof(double) * k * k);
    w.wbar = (double*)malloc(sizeof(double) * k);
    w.alnp = (double*)malloc(sizeof(double) * (g->nz + 1));
    w.xcol = (double*)malloc(sizeof(double) * k);
    lg_stats st;
    memset(&st, 0, sizeof st);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int i = 0; i < ncols; ++i) {
      int s = analyse_column(c, cols[i], xb, axb, xa, axa, &w, &st);
      if (s != LG_OK) status = s;
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    {
      tot.n_columns += st.n_columns;
      tot.n_solves += st.n_solves;
      tot.nobsl_total += st.nobsl_total;
      if (st.nobsl_max > tot.nobsl_max) tot.nobsl_max = st.nobsl_max;
      tot.n_capped += st.n_capped;
      tot.n_band += st.n_band;
      tot.n_eig_fail += st.n_eig_fail;
    }
    free(w.ent); free(w.rloc_h); free(w.rloc); free(w.rdiag); free(w.dep); free(w.yb); free(w.lnp);
    free(w.ws); free(w.iws); free(w.trans); free(w.wbar); free(w.alnp); free(w.xcol);
  }
  tot.n_copies = c->n_copies;
  tot.n_entries = c->n_entries;
  if (st_out) *st_out = tot;
  return status;
}

/* run_da_parallel pre-processing (module_da_parallel.F90:186-211): member mean
 * and perturbations of full members xb_in(ens, n, lat, lon) over npts columns;
 * returns LG_ERR_NAN if a NaN is found. */
int or_split_mean(int ens, int n, int64_t npts, const double* xb_in, double* xb, double* axb) {
  for (int64_t p = 0; p < npts; ++p)
    for (int r = 0; r < n; ++r) {
      const double* x = xb_in + (size_t)ens * (r + (size_t)n * p);
      double s = 0.0;
      for (int e = 0; e < ens; ++e) {
        if (x[e] != x[e]) return LG_ERR_NAN;
        s += x[e];
      }
      const double m = s / (double)(float)ens;
      axb[r + (size_t)n * p] = m;
      for (int e = 0; e < ens; ++e) xb[e + (size_t)ens * (r + (size_t)n * p)] = x[e] - m;
    }
  return LG_OK;
}

/* run_da_parallel post-processing (module_da_parallel.F90:219-257) on whole-globe
 * arrays with halo: RTPP blend gamma1*(axb+xb) + gamma2*(axa+xa) where
 * |grid_lat(j)| <= polar, background elsewhere, zero in the halo; spreads
 * (n, num_lat, num_lon) interior only. */
int or_post(int ens, int n, int num_lat, int num_lon, int halo, const float* grid_lat,
            double gamma1, double gamma2, double polar, const double* xb, const double* axb,
            const double* xa, const double* axa, double* xa_out, double* spread_b,
            double* spread_a) {
  const int nlat_e = num_lat + 2 * halo, nlon_e = num_lon + 2 * halo;
  for (int lo = 0; lo < nlon_e; ++lo)
    for (int li = 0; li < nlat_e; ++li)
      for (int k = 0; k < n; ++k) {
        const size_t pr = (size_t)k + (size_t)n * ((size_t)li + (size_t)nlat_e * lo);
        const int j = li - halo + 1, i = lo - halo + 1;
        double* out = xa_out + pr * ens;
        if (i < 1 || i > num_lon || j < 1 || j > num_lat) {
          for (int e = 0; e < ens; ++e) out[e] = 0.0;
          continue;
        }
        const double* b = xb + pr * ens;
        const size_t s = (size_t)k + (size_t)n * ((size_t)(j - 1) + (size_t)num_lat * (i - 1));
        double sb = 0.0, sa = 0.0;
        if (fabs((double)grid_lat[j - 1]) <= polar) {
          const double* x = xa + pr * ens;
          for (int e = 0; e < ens; ++e)
            out[e] = gamma1 * (axb[pr] + b[e]) + gamma2 * (axa[pr] + x[e]);
          for (int e = 0; e < ens; ++e) {
            sb = sb + b[e] * b[e];
            sa = sa + (out[e] - axa[pr]) * (out[e] - axa[pr]);
          }
        } else {
          for (int e = 0; e < ens; ++e) out[e] = b[e] + axb[pr];
          for (int e = 0; e < ens; ++e) {
            sb = sb + b[e] * b[e];
            sa = sa + b[e] * b[e];
          }
        }
        spread_b[s] = sqrt(sb / (double)(float)ens);
        spread_a[s] = sqrt(sa / (double)(float)ens);
      }
  return LG_OK;
}
