"""Host-side mirror of the reference LETKF interface over the GB300 C ABI.

The reference drives its analysis with three Fortran calls
(x86/DA/LETKF/src/letkf_init.F90:2, letkf.F90:157, letkf_final.F90:2); this
module exposes the same sequence -- ``letkf_init`` / ``letkf_run`` /
``letkf_final`` -- on a :class:`Letkf` context backed by
``_build/libletkf_gb300.so`` (CUDA kernels for sm_103a behind ``include/letkf_gpu.h``).

There is no CPU fallback: constructing a context without the compiled library
raises :class:`RuntimeError`.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libletkf_gb300.so")

LG_MAX_VARS = 16
LG_MAX_OBS_TYPES = 16
LG_MAX_OBS_VARS = 8

LG_OK = 0
LG_PREC_FP64 = 0
LG_PREC_MIXED = 1
LG_PREC_MIXED_TF32 = 2
LG_VCOORD_HYBRID = 0
LG_VCOORD_SIGMA = 1

STATUS = {
    0: "LG_OK", -1: "LG_ERR_ARG", -2: "LG_ERR_SHAPE", -3: "LG_ERR_UNSUPPORTED",
    -4: "LG_ERR_NAN", -5: "LG_ERR_OBS_OUTSIDE", -6: "LG_ERR_VARNAME", -7: "LG_ERR_EIG",
    -8: "LG_ERR_CUDA", -9: "LG_ERR_NOMEM", -10: "LG_ERR_STATE", -11: "LG_ERR_TIMEOUT",
}


class LgConfig(C.Structure):
    _fields_ = [
        ("ens", C.c_int), ("num_lat", C.c_int), ("num_lon", C.c_int), ("nz", C.c_int),
        ("halo", C.c_int), ("n_var", C.c_int), ("var_lev", C.c_int * LG_MAX_VARS),
        ("ps_index", C.c_int), ("local_dist", C.c_double), ("vert_dist", C.c_double),
        ("inflation", C.c_double), ("obs_polar", C.c_double), ("gc_filter", C.c_int),
        ("gc_filter_vertical", C.c_int), ("max_obs", C.c_int), ("global_nx", C.c_int),
        ("global_ny", C.c_int), ("cube_n", C.c_int), ("cube_nz", C.c_int),
        ("overlap", C.c_int), ("precision", C.c_int), ("vcoord", C.c_int),
    ]


class LgObsType(C.Structure):
    _fields_ = [("nz", C.c_int), ("nvar", C.c_int), ("var", C.c_int * LG_MAX_OBS_VARS)]


class LgObsSoa(C.Structure):
    _fields_ = [
        ("n_types", C.c_int), ("types", C.POINTER(LgObsType)), ("n_obs", C.c_int),
        ("type", C.POINTER(C.c_int)), ("lat", C.POINTER(C.c_double)),
        ("lon", C.POINTER(C.c_double)), ("ph", C.POINTER(C.c_double)),
        ("yo", C.POINTER(C.c_double)), ("rinv", C.POINTER(C.c_double)),
    ]


class LgStats(C.Structure):
    _fields_ = [
        ("n_columns", C.c_int64), ("n_solves", C.c_int64), ("n_copies", C.c_int64),
        ("n_entries", C.c_int64), ("nobsl_total", C.c_int64), ("nobsl_max", C.c_int64),
        ("n_capped", C.c_int64), ("n_band", C.c_int64), ("n_eig_fail", C.c_int64),
        ("ms_hx", C.c_double), ("ms_search", C.c_double), ("ms_solve", C.c_double),
        ("ms_total", C.c_double), ("ms_gram", C.c_double), ("ms_eig", C.c_double),
        ("n_launches", C.c_int64), ("n_gram_entries", C.c_int64),
        ("ms_tridiag", C.c_double), ("ms_ql", C.c_double), ("ms_vec", C.c_double),
        ("n_chunks", C.c_int64), ("ms_h2d", C.c_double), ("ms_d2h", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# ----------------------------------------------------------------- configs
LG_GRAM_AUTO, LG_GRAM_COLUMN, LG_GRAM_STREAM, LG_GRAM_QUEUE, LG_GRAM_COLUMN_LEAN = 0, 1, 2, 3, 4


class LgTuning(C.Structure):
    """lg_tuning: launch shapes and bucket boundaries (lg_set_tuning / lg_autotune)."""
    _fields_ = [("chunk_mb", C.c_int), ("gram_kernel", C.c_int), ("lnp_buckets", C.c_int),
                ("ql_warps", C.c_int), ("vec_warps", C.c_int), ("solve_streams", C.c_int),
                ("gram_ctas", C.c_int), ("ms", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


@dataclasses.dataclass
class Config:
    """Python view of lg_config plus the synthetic-workload description."""
    name: str
    ens: int
    num_lat: int
    num_lon: int
    nz: int
    var_names: Sequence[str]          # 2-D variables first
    local_dist: float
    vert_dist: float
    inflation: float
    n_obs: int
    global_nx: int
    global_ny: int
    halo: int = 1
    obs_polar: float = 91.0
    gc_filter: int = 1
    gc_filter_vertical: int = 1
    max_obs: int = 10000
    precision: int = LG_PREC_FP64
    vcoord: int = LG_VCOORD_HYBRID
    obs_sigma: Optional[dict] = None   # per variable obs error sd
    sh_degree: int = 30
    ar1: float = 0.8
    clustered_frac: float = 0.0        # fraction of obs in Gaussian clusters
    n_clusters: int = 8
    cluster_sigma_deg: float = 5.0
    seed: int = 0
    cube_n: int = 1      # da_block_interval: one solve per cube_n x cube_n columns
    cube_nz: int = 1     # da_vertical_interval: one solve per cube_nz levels (vertical)
    overlap: int = 0     # da_block_overlap: cubes step by cube_n - overlap, averaged

    @property
    def var_lev(self):
        return [1 if v == "ps" or self.nz == 1 else self.nz for v in self.var_names]

    @property
    def n_rows(self):
        return int(sum(self.var_lev))

    def to_c(self) -> LgConfig:
        c = LgConfig()
        c.ens = self.ens
        c.num_lat = self.num_lat
        c.num_lon = self.num_lon
        c.nz = self.nz
        c.halo = self.halo
        c.n_var = len(self.var_names)
        for i, lv in enumerate(self.var_lev):
            c.var_lev[i] = lv
        c.ps_index = 1
        c.local_dist = self.local_dist
        c.vert_dist = self.vert_dist
        c.inflation = self.inflation
        c.obs_polar = self.obs_polar
        c.gc_filter = self.gc_filter
        c.gc_filter_vertical = self.gc_filter_vertical
        c.max_obs = self.max_obs
        c.global_nx = self.global_nx
        c.global_ny = self.global_ny
        c.cube_n = self.cube_n
        c.cube_nz = self.cube_nz
        c.overlap = self.overlap
        c.precision = self.precision
        c.vcoord = self.vcoord
        return c

    def replace(self, **kw) -> "Config":
        return dataclasses.replace(self, **kw)


def preset(name: str) -> Config:
    """The five workloads of the benchmark description plus reduced test cases.

    cfg1: 72x36 (5 deg), 1 level, 1 variable, N=16, 2000 obs, GC 1000 km, rho 1.1.
    cfg2: 360x180x32, ps,u,v,pt, N=40, 1e5 obs, GC 800 km + 0.2 ln p, rho 1.05.
    cfg3: as cfg2 with N=64 and 1e6 obs, MAX_OBS lifted (mixed precision).
    cfg4: as cfg3 with 2e6 obs, 70 % in 8 Gaussian clusters (sigma 5 deg).
    cfg5: 720x360x32, N=128, 4e6 obs (mixed), GC 500 km, rho 1.03.
    """
    sig = {"ps": 100.0, "u": 1.0, "v": 1.0, "pt": 0.5}
    four = ("ps", "u", "v", "pt")
    if name == "cfg1":
        return Config("cfg1", 16, 36, 72, 1, ("x",), 1000.0, -1.0, 1.1, 2000, 4, 4,
                      obs_sigma={"x": 0.5}, sh_degree=10, vcoord=LG_VCOORD_SIGMA)
    if name == "cfg2":
        return Config("cfg2", 40, 180, 360, 32, four, 800.0, 0.2, 1.05, 100_000, 8, 8,
                      obs_sigma=sig)
    if name == "cfg3":
        return Config("cfg3", 64, 180, 360, 32, four, 800.0, 0.2, 1.05, 1_000_000, 8, 8,
                      obs_sigma=sig, max_obs=0, precision=LG_PREC_MIXED)
    if name == "cfg4":
        return Config("cfg4", 64, 180, 360, 32, four, 800.0, 0.2, 1.05, 2_000_000, 8, 8,
                      obs_sigma=sig, max_obs=0, precision=LG_PREC_MIXED, clustered_frac=0.7)
    if name == "cfg5":
        return Config("cfg5", 128, 360, 720, 32, four, 500.0, 0.2, 1.03, 4_000_000, 16, 16,
                      obs_sigma=sig, max_obs=0, precision=LG_PREC_MIXED, clustered_frac=0.5)
    # profiling case: cfg3's kernels at a quarter of the columns and observations
    # (inputs above L2, a few GB on the device) for ncu captures
    if name == "prof":
        return Config("prof", 64, 90, 180, 32, four, 800.0, 0.2, 1.05, 250_000, 8, 8,
                      obs_sigma=sig, max_obs=0, precision=LG_PREC_MIXED, sh_degree=20)
    # reduced cases for tests (seconds on the CPU oracle)
    if name == "tiny2d":
        return Config("tiny2d", 8, 18, 36, 1, ("x",), 1500.0, -1.0, 1.1, 300, 2, 3,
                      obs_sigma={"x": 0.5}, sh_degree=6, vcoord=LG_VCOORD_SIGMA)
    if name == "tiny3d":
        return Config("tiny3d", 16, 18, 36, 8, four, 1500.0, 0.3, 1.05, 600, 2, 3,
                      obs_sigma=sig, sh_degree=6)
    if name == "small3d":
        return Config("small3d", 40, 36, 72, 32, four, 1000.0, 0.2, 1.05, 4000, 4, 4,
                      obs_sigma=sig, sh_degree=10)
    raise KeyError(name)


# wrf_l32 hybrid coefficients (x86/DA/utils/vert_coord_mod.F90:330-402).  The
# reference writes them as default-REAL literals, so their values are the
# nearest REAL(4) numbers; the float32 round trip reproduces that.
_WRF_L32_A = [
    0.0, 0.0027008056640625, 0.0076868347823620, 0.0158526937798342, 0.0276367470939261,
    0.0414515552099706, 0.0562277844155789, 0.0724737972365225, 0.0893795253309864,
    0.1063548465048298, 0.1254725257849640, 0.1479642011314251, 0.1744233770857367,
    0.2054476619883455, 0.2362396334209435, 0.2617261684535087, 0.2783057827853432,
    0.2816243248017372, 0.2683280168286641, 0.2429473354807992, 0.2108099294331058,
    0.1759998110016148, 0.1415334037742616, 0.1095123294032484, 0.0812761592574764,
    0.0575423961814687, 0.0385285881906738, 0.0240694984015316, 0.0137226170696702,
    0.0068720184783044, 0.0027973066609278, 0.0007580797514921, 0.0,
]
_WRF_L32_B = [
    0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
    0.0001056069805219, 0.0059397906834944, 0.0235374270991938, 0.0576439176162314,
    0.1139578493851603, 0.1932313936022966, 0.2808764820852269, 0.3715629284436812,
    0.4612091687348547, 0.5467954414732804, 0.6262219272258057, 0.6981497395977654,
    0.7618575996945027, 0.8171268253424389, 0.8641240158900223, 0.9032994538662682,
    0.9352560448161740, 0.9607227915792738, 0.9804356127137464, 1.0,
]
PTOP = 219.4  # GMCORE namelist default ptop = 2.194e2_r8 (x86/ATM/utils/namelist_mod.F90:68)
P0 = 1.0e5


def vertical_coord(cfg: Config):
    """(coef_a, coef_b, p0, ptop) for the configuration's levels."""
    if cfg.vcoord == LG_VCOORD_HYBRID:
        if cfg.nz == 32:
            a = np.asarray(_WRF_L32_A, np.float32).astype(np.float64)
            b = np.asarray(_WRF_L32_B, np.float32).astype(np.float64)
        else:  # a smooth hybrid profile with nz levels for reduced test cases
            s = np.linspace(0.0, 1.0, cfg.nz + 1)
            b = np.clip((s - 0.3) / 0.7, 0.0, 1.0) ** 1.5
            a = (s - b) * 0.9
            a = a.astype(np.float32).astype(np.float64)
            b = b.astype(np.float32).astype(np.float64)
        return a, b, P0, PTOP
    s = np.linspace(0.0, 1.0, cfg.nz + 1).astype(np.float32).astype(np.float64)
    return s, np.zeros_like(s), P0, float(np.float32(219.406699761748))


def model_grid(cfg: Config):
    """Cell-centred lat/lon grid as REAL(4), with the reference's closing
    entries 90 and 360 (pro_info.F90:77-83)."""
    dlat = 180.0 / cfg.num_lat
    dlon = 360.0 / cfg.num_lon
    lat = np.empty(cfg.num_lat + 1, np.float32)
    lat[:-1] = (-90.0 + dlat * (np.arange(cfg.num_lat) + 0.5)).astype(np.float32)
    lat[-1] = 90.0
    lon = np.empty(cfg.num_lon + 1, np.float32)
    lon[:-1] = (dlon * np.arange(cfg.num_lon)).astype(np.float32)
    lon[-1] = 360.0
    return lat, lon


# ----------------------------------------------------------------- library
_lib = None


def gmcore_to_da(ps, u_half, v_half, pt, area_subcell, area_cell, halo: int, stream=None):
    """lg_gmcore_to_da_device on torch CUDA float64 tensors (members last):
    ps [lat, lon, ens], u_half [nz, lat, lon, ens], v_half [nz, lat + 1, lon, ens],
    pt [nz, lat, lon, ens], area_subcell [lat, 2], area_cell [lat] -> the DA
    background xb [lon + 2 halo, lat + 2 halo, 1 + 3 nz, ens] (latitude halo
    rows zero)."""
    import torch
    lib = load_library()
    nz, num_lat, num_lon, ens = u_half.shape
    xb = torch.zeros((num_lon + 2 * halo, num_lat + 2 * halo, 1 + 3 * nz, ens),
                     dtype=torch.float64, device=ps.device)
    args = [t.contiguous() for t in (ps, u_half, v_half, pt, area_subcell, area_cell)]
    check(lib.lg_gmcore_to_da_device(ens, num_lat, num_lon, nz, halo,
                                     *[C.c_void_p(t.data_ptr()) for t in args],
                                     C.c_void_p(xb.data_ptr()),
                                     C.c_void_p(stream) if stream is not None else None),
          "lg_gmcore_to_da_device")
    return xb


def obs_from_records(nz: int, nvar: int, lon, lat, lev, val, noise=None):
    """lg_obs_from_records: one type's observation records in the Redis store's
    layout (val: records x (2*nvar+1) float32 -- value and error sd per
    variable, then pressure) -> (lat, lon, ph, yo, rinv) arrays in the
    lg_obs_soa layout of that type.  noise: (nvar, records) standard normals
    for the perturbation, or None."""
    lib = load_library()
    f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    lon, lat, lev, val = f32(lon), f32(lat), f32(lev), f32(val)
    nrec = lon.size
    max_obs = nrec
    out = [np.zeros(max(1, max_obs * m)) for m in (1, 1, nz, nz * nvar, nz * nvar)]
    n = C.c_int()
    nz_ = None if noise is None else f32(noise)
    check(lib.lg_obs_from_records(nz, nvar, nrec, _ptr(lon, C.c_float), _ptr(lat, C.c_float),
                                  _ptr(lev, C.c_float), _ptr(val, C.c_float),
                                  None if nz_ is None else _ptr(nz_, C.c_float), max_obs,
                                  C.byref(n), *[_ptr(a, C.c_double) for a in out]),
          "lg_obs_from_records")
    m = n.value
    lat_o, lon_o, ph, yo, rinv = out
    return (lat_o[:m], lon_o[:m], ph[:m * nz].reshape(m, nz), yo[:m * nz * nvar].reshape(m, nz, nvar),
            rinv[:m * nz * nvar].reshape(m, nz, nvar))


def load_library(path: str = LIB_PATH):
    """Load the compiled C ABI; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    P = C.POINTER
    lib.lg_create.argtypes = [P(C.c_void_p), P(LgConfig)]
    lib.lg_set_grid.argtypes = [C.c_void_p, P(C.c_float), P(C.c_float), P(C.c_double),
                                P(C.c_double), C.c_double, C.c_double]
    lib.lg_set_obs.argtypes = [C.c_void_p, P(LgObsSoa)]
    lib.lg_run.argtypes = [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double),
                           P(C.c_double), P(C.c_double)]
    lib.lg_run_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]
    lib.lg_get_stats.argtypes = [C.c_void_p, P(LgStats)]
    lib.lg_get_timeline.argtypes = [C.c_void_p, P(C.c_float), C.c_int, P(C.c_int)]
    lib.lg_gmcore_to_da_device.argtypes = [C.c_int] * 5 + [C.c_void_p] * 8
    lib.lg_obs_from_records.argtypes = [C.c_int, C.c_int, C.c_int] + [P(C.c_float)] * 5 + [
        C.c_int, P(C.c_int)] + [P(C.c_double)] * 5
    lib.lg_get_tuning.argtypes = [C.c_void_p, P(LgTuning)]
    lib.lg_set_tuning.argtypes = [C.c_void_p, P(LgTuning)]
    lib.lg_autotune.argtypes = [C.c_void_p] + [C.c_void_p] * 5 + [P(LgTuning)]
    lib.lg_get_lists.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_double),
                                 P(C.c_int64)]
    lib.lg_get_column_list.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_int), P(C.c_double),
                                       P(C.c_int)]
    lib.lg_copy_layout.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int64),
                                   P(C.c_int64)]
    lib.lg_get_hx.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
    lib.lg_destroy.argtypes = [C.c_void_p]
    lib.lg_destroy.restype = None
    lib.lg_core_batch.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lg_letkf_core.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_float),
                                  P(C.c_double), P(C.c_double), P(C.c_double),
                                  P(C.c_double), C.c_double]
    lib.lg_split_mean_device.argtypes = [C.c_void_p] * 4 + [C.c_void_p]
    lib.lg_post_device.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double] + [C.c_void_p] * 8
    lib.lg_run_da_parallel.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double,
                                       P(C.c_double), P(C.c_double), P(C.c_double),
                                       P(C.c_double)]
    lib.lg_core_batch_noalloc.argtypes = lib.lg_core_batch.argtypes
    lib.lg_set_columns.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.lg_list_counts.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int64)]
    lib.lg_set_wait_limit.argtypes = [C.c_void_p, C.c_int64]
    lib.lg_set_shard.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.lg_shard_entries.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_int64)]
    lib.lg_hx_device.argtypes = [C.c_void_p] * 4
    lib.lg_hx_export.argtypes = [C.c_void_p] * 3
    lib.lg_hx_import.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
    lib.lg_analyse_device.argtypes = [C.c_void_p] * 6
    lib.lg_status_string.restype = C.c_char_p
    lib.lg_status_string.argtypes = [C.c_int]
    _lib = lib
    return lib


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def check(status: int, what: str = ""):
    if status != LG_OK:
        raise RuntimeError(f"{what}: {STATUS.get(status, status)}")


class ObsSet:
    """Observation SoA in the layout of lg_obs_soa (read_obs_mod.F90:15-27)."""

    def __init__(self, types, type_idx, lat, lon, ph, yo, rinv):
        self.types = list(types)              # list of (nz, nvar, [var ids])
        self.type = np.ascontiguousarray(type_idx, np.int32)
        self.lat = np.ascontiguousarray(lat, np.float64)
        self.lon = np.ascontiguousarray(lon, np.float64)
        self.ph = np.ascontiguousarray(ph, np.float64)
        self.yo = np.ascontiguousarray(yo, np.float64)
        self.rinv = np.ascontiguousarray(rinv, np.float64)
        self._keep = None

    @property
    def n_obs(self):
        return int(self.type.shape[0])

    def to_c(self) -> LgObsSoa:
        arr = (LgObsType * max(1, len(self.types)))()
        for i, (nz, nvar, vids) in enumerate(self.types):
            arr[i].nz = nz
            arr[i].nvar = nvar
            for j, v in enumerate(vids):
                arr[i].var[j] = v
        s = LgObsSoa()
        s.n_types = len(self.types)
        s.types = C.cast(arr, C.POINTER(LgObsType))
        s.n_obs = self.n_obs
        s.type = _ptr(self.type, C.c_int)
        s.lat = _ptr(self.lat, C.c_double)
        s.lon = _ptr(self.lon, C.c_double)
        s.ph = _ptr(self.ph, C.c_double)
        s.yo = _ptr(self.yo, C.c_double)
        s.rinv = _ptr(self.rinv, C.c_double)
        self._keep = arr
        return s


class Letkf:
    """One LETKF context on the current CUDA device (letkf_init .. letkf_final)."""

    def __init__(self, cfg: Config):
        self.lib = load_library()
        self.cfg = cfg
        self._c = cfg.to_c()
        h = C.c_void_p()
        check(self.lib.lg_create(C.byref(h), C.byref(self._c)), "lg_create")
        self.h = h
        lat, lon = model_grid(cfg)
        a, b, p0, ptop = vertical_coord(cfg)
        self.grid_lat, self.grid_lon = lat, lon
        check(self.lib.lg_set_grid(self.h, _ptr(lat, C.c_float), _ptr(lon, C.c_float),
                                   _ptr(a, C.c_double), _ptr(b, C.c_double), p0, ptop),
              "lg_set_grid")

    # letkf_init happens in the constructor; set_obs replaces the Redis reads
    def set_obs(self, obs: ObsSet):
        soa = obs.to_c()
        check(self.lib.lg_set_obs(self.h, C.byref(soa)), "lg_set_obs")

    def letkf_run(self, ntimes: int, xb: np.ndarray, axb: np.ndarray, xa: np.ndarray,
                  axa: np.ndarray):
        """Host arrays, Fortran layout flattened C-contiguous (see letkf_gpu.h)."""
        for a in (xb, axb, xa, axa):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        check(self.lib.lg_run(self.h, ntimes, _ptr(xb, C.c_double), _ptr(axb, C.c_double),
                              _ptr(xa, C.c_double), _ptr(axa, C.c_double)), "lg_run")

    def letkf_run_device(self, ntimes: int, xb, axb, xa, axa, stream=None):
        """torch CUDA tensors (float64, contiguous)."""
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_run_device(self.h, ntimes, C.c_void_p(xb.data_ptr()),
                                     C.c_void_p(axb.data_ptr()), C.c_void_p(xa.data_ptr()),
                                     C.c_void_p(axa.data_ptr()), s), "lg_run_device")

    # ------------------------------------------------ windows and shards
    def set_columns(self, col_begin: int, col_end: int):
        """Analyse only columns [col_begin, col_end) (c = lon * num_lat + lat, 0-based)."""
        check(self.lib.lg_set_columns(self.h, col_begin, col_end), "lg_set_columns")

    def set_wait_limit(self, ns: int):
        """lg_set_wait_limit: the tensor-core Gram's wait limit in ns (0: 2 s)."""
        check(self.lib.lg_set_wait_limit(self.h, ns), "lg_set_wait_limit")

    def list_counts(self) -> np.ndarray:
        """Local entries of every column's list (the count pass only)."""
        counts = np.zeros(self.cfg.num_lat * self.cfg.num_lon, np.int32)
        total = C.c_int64()
        check(self.lib.lg_list_counts(self.h, _ptr(counts, C.c_int), C.byref(total)),
              "lg_list_counts")
        return counts

    def windows(self, max_entries: int):
        """Column windows [(c0, c1), ...] covering the globe in order, each of
        whole longitudes and at most max_entries list entries (a longitude
        above the budget is a window of its own)."""
        cnt = self.list_counts().reshape(self.cfg.num_lon, self.cfg.num_lat).sum(axis=1)
        out, start, acc = [], 0, 0
        for lon, c in enumerate(cnt):
            if acc and acc + c > max_entries:
                out.append((start * self.cfg.num_lat, lon * self.cfg.num_lat))
                start, acc = lon, 0
            acc += int(c)
        out.append((start * self.cfg.num_lat, self.cfg.num_lon * self.cfg.num_lat))
        return out

    def set_shard(self, lon_block_begin: int, lon_block_end: int):
        """This context's shard: longitude blocks [begin, end) of the virtual decomposition."""
        check(self.lib.lg_set_shard(self.h, lon_block_begin, lon_block_end), "lg_set_shard")

    def shard_entries(self):
        """(entry_begin, entry_end, n_entries): the shard's own H(x) entries."""
        a, b, n = C.c_int64(), C.c_int64(), C.c_int64()
        check(self.lib.lg_shard_entries(self.h, C.byref(a), C.byref(b), C.byref(n)),
              "lg_shard_entries")
        return a.value, b.value, n.value

    def hx_device(self, xb, axb, stream=None):
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_hx_device(self.h, C.c_void_p(xb.data_ptr()), C.c_void_p(axb.data_ptr()),
                                    s), "lg_hx_device")

    def hx_export(self, rows, stream=None):
        """rows: CUDA float64 tensor of (entry_end - entry_begin) x (ens + 3)."""
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_hx_export(self.h, C.c_void_p(rows.data_ptr()), s), "lg_hx_export")

    def hx_import(self, rows, entry_begin: int, entry_end: int, stream=None):
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_hx_import(self.h, C.c_void_p(rows.data_ptr()), entry_begin, entry_end,
                                    s), "lg_hx_import")

    def analyse_device(self, xb, axb, xa, axa, stream=None):
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_analyse_device(self.h, *[C.c_void_p(t.data_ptr()) for t in
                                                   (xb, axb, xa, axa)], s), "lg_analyse_device")

    def run_da_parallel(self, ntimes: int, gamma1: float, gamma2: float, polar_lat: float,
                        xb_in: np.ndarray, xa_out: np.ndarray, spread_b: np.ndarray,
                        spread_a: np.ndarray):
        """run_da_parallel (module_da_parallel.F90:165-263) on host arrays: full
        members in, blended members and spreads out."""
        check(self.lib.lg_run_da_parallel(self.h, ntimes, gamma1, gamma2, polar_lat,
                                          _ptr(xb_in, C.c_double), _ptr(xa_out, C.c_double),
                                          _ptr(spread_b, C.c_double), _ptr(spread_a, C.c_double)),
              "lg_run_da_parallel")

    def tuning(self) -> dict:
        t = LgTuning()
        check(self.lib.lg_get_tuning(self.h, C.byref(t)), "lg_get_tuning")
        return t.as_dict()

    def set_tuning(self, **kw):
        t = LgTuning()
        check(self.lib.lg_get_tuning(self.h, C.byref(t)), "lg_get_tuning")
        for key, v in kw.items():
            setattr(t, key, v)
        check(self.lib.lg_set_tuning(self.h, C.byref(t)), "lg_set_tuning")

    def autotune(self, xb, axb, xa, axa, stream=None) -> dict:
        """lg_autotune on torch CUDA tensors; returns the chosen settings."""
        t = LgTuning()
        s = C.c_void_p(stream) if stream is not None else None
        check(self.lib.lg_autotune(self.h, C.c_void_p(xb.data_ptr()), C.c_void_p(axb.data_ptr()),
                                   C.c_void_p(xa.data_ptr()), C.c_void_p(axa.data_ptr()), s,
                                   C.byref(t)), "lg_autotune")
        return t.as_dict()

    def stats(self) -> dict:
        st = LgStats()
        check(self.lib.lg_get_stats(self.h, C.byref(st)), "lg_get_stats")
        return st.as_dict()

    def timeline(self) -> np.ndarray:
        """lg_get_timeline: [chunks, 7] ms after the analysis start (Gram
        start/end, eigensolve start, tridiag end, QL end, vectors start/end)."""
        nq = C.c_int()
        check(self.lib.lg_get_timeline(self.h, None, 0, C.byref(nq)), "lg_get_timeline")
        ms = np.zeros(max(1, 7 * nq.value), np.float32)
        if nq.value:
            check(self.lib.lg_get_timeline(self.h, _ptr(ms, C.c_float), 7 * nq.value,
                                           C.byref(nq)), "lg_get_timeline")
        return ms[:7 * nq.value].reshape(nq.value, 7)

    def lists(self):
        total = C.c_int64()
        check(self.lib.lg_get_lists(self.h, None, None, None, C.byref(total)), "lg_get_lists")
        ncol = self.cfg.num_lat * self.cfg.num_lon
        counts = np.zeros(ncol, np.int32)
        ent = np.zeros(max(1, total.value), np.int32)
        rloc = np.zeros(max(1, total.value), np.float64)
        check(self.lib.lg_get_lists(self.h, _ptr(counts, C.c_int), _ptr(ent, C.c_int),
                                    _ptr(rloc, C.c_double), C.byref(total)), "lg_get_lists")
        return counts, ent[:total.value], rloc[:total.value]

    def column_list(self, col: int):
        """Neighbour list (entries, weights) of one column of the last analysis."""
        n = C.c_int()
        check(self.lib.lg_get_column_list(self.h, col, 0, None, None, C.byref(n)),
              "lg_get_column_list")
        ent = np.zeros(max(1, n.value), np.int32)
        rloc = np.zeros(max(1, n.value), np.float64)
        check(self.lib.lg_get_column_list(self.h, col, n.value, _ptr(ent, C.c_int),
                                          _ptr(rloc, C.c_double), C.byref(n)),
              "lg_get_column_list")
        return ent[:n.value], rloc[:n.value]

    def copy_layout(self):
        n = C.c_int64()
        check(self.lib.lg_copy_layout(self.h, None, None, None, C.byref(n)), "lg_copy_layout")
        co = np.zeros(max(1, n.value), np.int32)
        cb = np.zeros(max(1, n.value), np.int32)
        ce = np.zeros(n.value + 1, np.int64)
        check(self.lib.lg_copy_layout(self.h, _ptr(co, C.c_int), _ptr(cb, C.c_int),
                                      _ptr(ce, C.c_int64), C.byref(n)), "lg_copy_layout")
        return co[:n.value], cb[:n.value], ce

    def hx(self, n_entries: int):
        yb = np.zeros((n_entries, self.cfg.ens), np.float64)
        dis = np.zeros(n_entries, np.float64)
        check(self.lib.lg_get_hx(self.h, _ptr(yb, C.c_double), _ptr(dis, C.c_double)),
              "lg_get_hx")
        return yb, dis

    def letkf_final(self):
        if getattr(self, "h", None):
            self.lib.lg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.letkf_final()
        except Exception:
            pass


def letkf_core(hxens: np.ndarray, rdiaginv: np.ndarray, dep: np.ndarray, rloc: np.ndarray,
               inflation: float):
    """Single-column letkf_core through the C ABI (host arrays).
    hxens: (nobsl, k) member fastest.  Returns trans (k, k) column-major as
    trans[j, i] = trans(i, j) of the Fortran array, and overline_w (k)."""
    lib = load_library()
    p, k = hxens.shape
    hx = np.ascontiguousarray(hxens, np.float64)
    rd = np.ascontiguousarray(rdiaginv, np.float32)
    dp = np.ascontiguousarray(dep, np.float64)
    rl = np.ascontiguousarray(rloc, np.float64)
    trans = np.zeros((k, k), np.float64)
    wbar = np.zeros(k, np.float64)
    check(lib.lg_letkf_core(k, p, _ptr(hx, C.c_double), _ptr(rd, C.c_float),
                            _ptr(dp, C.c_double), _ptr(rl, C.c_double), _ptr(trans, C.c_double),
                            _ptr(wbar, C.c_double), inflation), "lg_letkf_core")
    return trans, wbar
