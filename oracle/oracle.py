"""ctypes wrapper of the C oracle (TEST INFRASTRUCTURE, never the product).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm use this module, as the checker of the GPU path.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "dida-thhpca_gb300"))
from letkf_gb300 import LgConfig, LgObsSoa, LgStats, model_grid, vertical_coord  # noqa: E402

from .build import build as _build  # noqa: E402

_lib = None


def _openblas_path():
    """Path of the OpenBLAS copy bundled with scipy, if any."""
    try:
        import scipy
    except ImportError:
        return None
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
    cands = [c for c in cands if "64_" not in os.path.basename(c)] or cands
    return cands[0] if cands else None


def lib(use_lapack: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    L = C.CDLL(_build())
    P = C.POINTER
    L.or_set_lapack.argtypes = [C.c_char_p]
    L.or_create.restype = C.c_void_p
    L.or_create.argtypes = [P(LgConfig), P(C.c_float), P(C.c_float), P(C.c_double),
                            P(C.c_double), C.c_double, C.c_double, P(LgObsSoa), P(C.c_int)]
    L.or_destroy.argtypes = [C.c_void_p]
    L.or_destroy.restype = None
    L.or_hx.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), C.c_int]
    L.or_get_hx.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(C.c_double)]
    L.or_hx_range.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), C.c_int64, C.c_int64,
                              C.c_int]
    L.or_get_hx_rows.argtypes = [C.c_void_p, P(C.c_double), C.c_int64, C.c_int64]
    L.or_set_hx_rows.argtypes = [C.c_void_p, P(C.c_double), C.c_int64, C.c_int64]
    L.or_n_copies.restype = C.c_int64
    L.or_n_copies.argtypes = [C.c_void_p]
    L.or_n_entries.restype = C.c_int64
    L.or_n_entries.argtypes = [C.c_void_p]
    L.or_copy_layout.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int64)]
    L.or_neighbour_table.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int)]
    L.or_column_list.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_double), C.c_int,
                                 P(C.c_int), P(C.c_int64)]
    L.or_analysis.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(C.c_double),
                              P(C.c_double), C.c_int, C.c_int, C.c_int, P(LgStats)]
    L.or_analysis_cols.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(C.c_double),
                                   P(C.c_double), P(C.c_int), C.c_int, C.c_int, P(LgStats)]
    L.or_column_trans.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
    L.or_core.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_float), P(C.c_double),
                          P(C.c_double), C.c_double, P(C.c_double), P(C.c_double)]
    L.or_latlon_dist_r8.restype = C.c_double
    L.or_latlon_dist_r8.argtypes = [C.c_double] * 4
    L.or_latlon_dist_r4.restype = C.c_float
    L.or_latlon_dist_r4.argtypes = [C.c_float] * 4
    L.or_schr2.restype = C.c_double
    L.or_schr2.argtypes = [C.c_double]
    L.or_schr.restype = C.c_double
    L.or_schr.argtypes = [C.c_double]
    L.or_split_mean.argtypes = [C.c_int, C.c_int, C.c_int64, P(C.c_double), P(C.c_double),
                                P(C.c_double)]
    L.or_post.argtypes = [C.c_int] * 5 + [P(C.c_float), C.c_double, C.c_double, C.c_double] + [
        P(C.c_double)] * 7
    if use_lapack:
        p = _openblas_path()
        if p:
            L.or_set_lapack(p.encode())
    _lib = L
    return L


def lapack_loaded() -> bool:
    return bool(lib().or_lapack_loaded())


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """Reference restatement for one configuration and observation set."""

    def __init__(self, cfg, obs):
        L = lib()
        self.cfg = cfg
        self._c = cfg.to_c()
        lat, lon = model_grid(cfg)
        a, b, p0, ptop = vertical_coord(cfg)
        self._keep = (lat, lon, a, b)
        soa = obs.to_c()
        self._obs = obs
        st = C.c_int()
        self.h = L.or_create(C.byref(self._c), _p(lat, C.c_float), _p(lon, C.c_float),
                             _p(a, C.c_double), _p(b, C.c_double), p0, ptop, C.byref(soa),
                             C.byref(st))
        if not self.h:
            raise RuntimeError(f"or_create failed: {st.value}")
        self.n_copies = int(L.or_n_copies(self.h))
        self.n_entries = int(L.or_n_entries(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    def hx(self, xb: np.ndarray, axb: np.ndarray, nthreads: int = 0):
        st = lib().or_hx(self.h, _p(xb, C.c_double), _p(axb, C.c_double), nthreads)
        if st != 0:
            raise RuntimeError(f"or_hx: {st}")
        yb = np.zeros((self.n_entries, self.cfg.ens))
        dis = np.zeros(self.n_entries)
        lnp = np.zeros(self.n_entries)
        lib().or_get_hx(self.h, _p(yb, C.c_double), _p(dis, C.c_double), _p(lnp, C.c_double))
        return yb, dis, lnp

    def hx_range(self, xb, axb, j0: int, j1: int, nthreads: int = 0):
        """H(x) of the block copies [j0, j1) only."""
        st = lib().or_hx_range(self.h, _p(xb, C.c_double), _p(axb, C.c_double), j0, j1, nthreads)
        if st != 0:
            raise RuntimeError(f"or_hx_range: {st}")

    def hx_rows(self, e0: int, e1: int):
        """H(x) rows of entries [e0, e1): (e1 - e0) x (ens + 2) -- yb, dis, ln p."""
        rows = np.zeros((max(0, e1 - e0), self.cfg.ens + 2))
        if lib().or_get_hx_rows(self.h, _p(rows, C.c_double), e0, e1) != 0:
            raise RuntimeError("or_get_hx_rows")
        return rows

    def set_hx_rows(self, rows, e0: int, e1: int):
        rows = np.ascontiguousarray(rows, np.float64)
        if lib().or_set_hx_rows(self.h, _p(rows, C.c_double), e0, e1) != 0:
            raise RuntimeError("or_set_hx_rows")

    def copy_layout(self):
        co = np.zeros(max(1, self.n_copies), np.int32)
        cb = np.zeros(max(1, self.n_copies), np.int32)
        ce = np.zeros(self.n_copies + 1, np.int64)
        lib().or_copy_layout(self.h, _p(co, C.c_int), _p(cb, C.c_int), _p(ce, C.c_int64))
        return co[:self.n_copies], cb[:self.n_copies], ce

    def neighbour_table(self):
        n = lib().or_neighbour_table(self.h, None, None)
        nb = self.cfg.global_nx * self.cfg.global_ny
        off = np.zeros(nb + 1, np.int32)
        blk = np.zeros(max(1, n), np.int32)
        lib().or_neighbour_table(self.h, _p(off, C.c_int), _p(blk, C.c_int))
        return off, blk[:n]

    def column_list(self, col: int):
        n = lib().or_column_list(self.h, col, None, None, 0, None, None)
        ent = np.zeros(max(1, n), np.int32)
        rl = np.zeros(max(1, n))
        capped = C.c_int()
        band = C.c_int64()
        n2 = lib().or_column_list(self.h, col, _p(ent, C.c_int), _p(rl, C.c_double), n,
                                  C.byref(capped), C.byref(band))
        assert n2 == n
        return ent[:n], rl[:n]

    def column_trans(self, col: int):
        """letkf_core on column col's horizontal list: trans[j, i] = Fortran
        trans(i, j) (the k x k array, column-major in memory)."""
        k = self.cfg.ens
        t = np.zeros((k, k))
        r = lib().or_column_trans(self.h, col, _p(t, C.c_double))
        if r != 0:
            raise RuntimeError(f"or_column_trans: {r}")
        return t

    def analysis(self, xb, axb, xa, axa, c0=0, c1=None, nthreads: int = 0):
        if c1 is None:
            c1 = self.cfg.num_lat * self.cfg.num_lon
        st = LgStats()
        r = lib().or_analysis(self.h, _p(xb, C.c_double), _p(axb, C.c_double),
                              _p(xa, C.c_double), _p(axa, C.c_double), c0, c1, nthreads,
                              C.byref(st))
        if r != 0:
            raise RuntimeError(f"or_analysis: {r}")
        return st.as_dict()


    def analysis_cols(self, xb, axb, xa, axa, cols, nthreads: int = 0):
        """Analysis of the listed columns only (the others of xa/axa untouched)."""
        cols = np.ascontiguousarray(cols, np.int32)
        st = LgStats()
        r = lib().or_analysis_cols(self.h, _p(xb, C.c_double), _p(axb, C.c_double),
                                   _p(xa, C.c_double), _p(axa, C.c_double), _p(cols, C.c_int),
                                   int(cols.size), nthreads, C.byref(st))
        if r != 0:
            raise RuntimeError(f"or_analysis_cols: {r}")
        return st.as_dict()


def sample_columns(cfg, n_lat_bands: int, n_lons: int, seed: int = 0):
    """A column sample spread over the globe: for each of n_lons longitudes
    (evenly spaced, with a seeded offset) one column in each of n_lat_bands
    equal latitude bands (a seeded latitude inside the band), plus the two polar
    rows.  Column index c = (lon - 1) * num_lat + (lat - 1)."""
    rng = np.random.default_rng(seed)
    nl, nn = cfg.num_lat, cfg.num_lon
    lons = (np.arange(n_lons) * nn // n_lons + rng.integers(0, max(1, nn // n_lons))) % nn
    edges = np.linspace(0, nl, n_lat_bands + 1).astype(int)
    cols = []
    for lo in lons:
        for b in range(n_lat_bands):
            a, z = edges[b], max(edges[b] + 1, edges[b + 1])
            cols.append(lo * nl + int(rng.integers(a, z)))
        cols.append(lo * nl)            # southernmost row
        cols.append(lo * nl + nl - 1)   # northernmost row
    return np.unique(np.asarray(cols, np.int32))


def core(hxens, rdiaginv, dep, rloc, inflation):
    """letkf_core restated: hxens (p, k) member fastest -> trans (k,k) with
    trans[j, i] = Fortran trans(i, j), overline_w (k)."""
    p, k = hxens.shape
    hx = np.ascontiguousarray(hxens, np.float64)
    rd = np.ascontiguousarray(rdiaginv, np.float32)
    dp = np.ascontiguousarray(dep, np.float64)
    rl = np.ascontiguousarray(rloc, np.float64)
    trans = np.zeros((k, k))
    wbar = np.zeros(k)
    lib().or_core(k, p, _p(hx, C.c_double), _p(rd, C.c_float), _p(dp, C.c_double),
                  _p(rl, C.c_double), inflation, _p(trans, C.c_double), _p(wbar, C.c_double))
    return trans, wbar


def split_mean(ens, xb_in):
    """run_da_parallel pre-processing: (xb, axb) from full members (..., n, ens)."""
    shp = xb_in.shape
    n = shp[-2]
    npts = int(np.prod(shp[:-2]))
    xb = np.zeros_like(xb_in)
    axb = np.zeros(shp[:-1])
    r = lib().or_split_mean(ens, n, npts, _p(np.ascontiguousarray(xb_in), C.c_double),
                            _p(xb, C.c_double), _p(axb, C.c_double))
    return r, xb, axb


def post(cfg, gamma1, gamma2, polar, xb, axb, xa, axa):
    """run_da_parallel post-processing: xa_out and the two spreads."""
    from letkf_gb300 import model_grid
    lat, _ = model_grid(cfg)
    xa_out = np.zeros_like(xb)
    sb = np.zeros((cfg.num_lon, cfg.num_lat, xb.shape[-2]))
    sa = np.zeros_like(sb)
    lib().or_post(cfg.ens, xb.shape[-2], cfg.num_lat, cfg.num_lon, cfg.halo, _p(lat, C.c_float),
                  gamma1, gamma2, polar, _p(xb, C.c_double), _p(axb, C.c_double),
                  _p(xa, C.c_double), _p(axa, C.c_double), _p(xa_out, C.c_double),
                  _p(sb, C.c_double), _p(sa, C.c_double))
    return xa_out, sb, sa
