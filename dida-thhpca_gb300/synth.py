"""Seeded synthetic LETKF workloads (background ensemble + observations).

No public dataset or observation archive exists for the reference's analysis
step (its observations live in a Redis cluster, its backgrounds come from a
running GMCORE ensemble), so the benchmark inputs are generated here with the
shapes and value ranges of each workload:

* fields are random spherical-harmonic fields of degree <= L with N(0,1)
  coefficients (4-pi normalised, scaled to unit expected RMS), combined per
  level with a vertical AR(1) correlation;
* members = per-variable base + scale*truth + pert_scale*independent field;
* observations are uniform on the sphere (optionally 8 Gaussian clusters),
  with REAL(4) positions/values as the reference's Redis store holds them,
  yo = H(truth) + N(0, sigma^2), rinv = 1/sigma^2 evaluated in REAL(4)
  (read_obs_mod.F90:438).

All randomness comes from numpy's PCG64 with the configuration seed.  The
field synthesis runs either in numpy (tests) or in torch on a CUDA device
(full-size benchmark inputs); both follow the same recipe.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from letkf_gb300 import Config, ObsSet, model_grid, vertical_coord, LG_VCOORD_SIGMA

# (base, truth scale, perturbation scale) per variable
_SCALES = {"ps": (1.0e5, 1000.0, 200.0), "u": (0.0, 10.0, 2.0), "v": (0.0, 10.0, 2.0),
           "pt": (300.0, 5.0, 1.0), "x": (0.0, 1.0, 1.0)}


def _legendre(lmax: int, x: np.ndarray) -> np.ndarray:
    """4-pi normalised associated Legendre functions P[l, m, i] at x = sin(lat)."""
    x = np.asarray(x, np.float64)
    u = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = np.zeros((lmax + 1, lmax + 1, x.size))
    P[0, 0] = 1.0
    for m in range(1, lmax + 1):
        f = math.sqrt(3.0) if m == 1 else math.sqrt((2.0 * m + 1.0) / (2.0 * m))
        P[m, m] = f * u * P[m - 1, m - 1]
    for m in range(0, lmax):
        P[m + 1, m] = math.sqrt(2.0 * m + 3.0) * x * P[m, m]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt((2.0 * l + 1.0) * (l - m - 1.0) * (l + m - 1.0) /
                          ((2.0 * l - 3.0) * (l * l - m * m)))
            P[l, m] = a * x * P[l - 1, m] - b * P[l - 2, m]
    return P


def _extended_axes(cfg: Config):
    lat, lon = model_grid(cfg)
    h = cfg.halo
    dlat = 180.0 / cfg.num_lat
    dlon = 360.0 / cfg.num_lon
    lat_e = -90.0 + dlat * (np.arange(-h, cfg.num_lat + h) + 0.5)
    lon_e = dlon * np.arange(-h, cfg.num_lon + h)
    return lat, lon, lat_e, lon_e


class FieldSynth:
    """Random SH fields on the halo-extended model grid."""

    def __init__(self, cfg: Config, backend: str = "numpy", device=None):
        self.cfg = cfg
        self.L = cfg.sh_degree
        _, _, lat_e, lon_e = _extended_axes(cfg)
        self.P = _legendre(self.L, np.sin(np.radians(lat_e)))          # (L+1, L+1, nlat_e)
        m = np.arange(self.L + 1)[:, None]
        lam = np.radians(lon_e)[None, :]
        self.cosm = np.cos(m * lam)                                     # (M, nlon_e)
        self.sinm = np.sin(m * lam)
        self.backend = backend
        self.device = device
        self.norm = 1.0 / (self.L + 1)
        if backend == "torch":
            import torch
            self.torch = torch
            self.tP = torch.as_tensor(self.P, device=device)
            self.tcos = torch.as_tensor(self.cosm, device=device)
            self.tsin = torch.as_tensor(self.sinm, device=device)

    def coeffs(self, rng: np.random.Generator, nf: int):
        L = self.L
        c = rng.standard_normal((nf, L + 1, L + 1))
        s = rng.standard_normal((nf, L + 1, L + 1))
        lm = np.arange(L + 1)
        mask = (lm[None, :] <= lm[:, None]).astype(np.float64)  # m <= l
        c *= mask
        s *= mask
        s[:, :, 0] = 0.0
        return c, s

    def synth(self, c: np.ndarray, s: np.ndarray):
        """fields (nf, nlat_e, nlon_e) from coefficients (nf, l, m)."""
        if self.backend == "torch":
            t = self.torch
            tc = t.as_tensor(c, device=self.device)
            ts = t.as_tensor(s, device=self.device)
            A = t.einsum("flm,lmi->fim", tc, self.tP)
            B = t.einsum("flm,lmi->fim", ts, self.tP)
            return (A @ self.tcos + B @ self.tsin) * self.norm
        A = np.einsum("flm,lmi->fim", c, self.P, optimize=True)
        B = np.einsum("flm,lmi->fim", s, self.P, optimize=True)
        return (A @ self.cosm + B @ self.sinm) * self.norm


@dataclass
class Workload:
    cfg: Config
    xb: object       # perturbations, Fortran xb(ens, n, lat_e, lon_e) as C array (lon_e, lat_e, n, ens)
    axb: object      # mean, C array (lon_e, lat_e, n)
    truth: np.ndarray  # (lon_e, lat_e, n) numpy
    obs: ObsSet


def _fields_3d(fs: FieldSynth, rng, nf_groups: int, nz: int, ar1: float, out_fn):
    """Generate nf_groups vertically-AR(1)-correlated stacks of nz levels; calls
    out_fn(level, fields(nf_groups, nlat_e, nlon_e)) for each level."""
    prev = None
    q = math.sqrt(max(0.0, 1.0 - ar1 * ar1))
    for lev in range(nz):
        c, s = fs.coeffs(rng, nf_groups)
        g = fs.synth(c, s)
        cur = g if prev is None else ar1 * prev + q * g
        out_fn(lev, cur)
        prev = cur


def make_workload(cfg: Config, backend: str = "numpy", device=None) -> Workload:
    """Background ensemble (mean/perturbation split as run_da_parallel does,
    module_da_parallel.F90:186-211) and observations for cfg."""
    rng = np.random.default_rng(cfg.seed)
    fs = FieldSynth(cfg, backend, device)
    lat, lon, lat_e, lon_e = _extended_axes(cfg)
    k, n, nz = cfg.ens, cfg.n_rows, cfg.nz
    nlat_e, nlon_e = lat_e.size, lon_e.size
    if backend == "torch":
        import torch
        xb_in = torch.empty((nlon_e, nlat_e, n, k), dtype=torch.float64, device=device)
        truth_t = torch.empty((nlon_e, nlat_e, n), dtype=torch.float64, device=device)
    else:
        xb_in = np.empty((nlon_e, nlat_e, n, k), np.float64)
        truth_t = np.empty((nlon_e, nlat_e, n), np.float64)
    row = 0
    for v, lv in zip(cfg.var_names, cfg.var_lev):
        base, tsc, psc = _SCALES.get(v, (0.0, 1.0, 1.0))
        nlev = lv

        def put(lev, F, row0=row, base=base, tsc=tsc, psc=psc):
            # F: (k+1, nlat_e, nlon_e): index 0 = truth, 1..k = perturbations
            tr = base + tsc * F[0]
            truth_t[:, :, row0 + lev] = tr.T
            mem = tr[None] + psc * F[1:]
            if backend == "torch":
                xb_in[:, :, row0 + lev, :] = mem.permute(2, 1, 0)
            else:
                xb_in[:, :, row0 + lev, :] = np.transpose(mem, (2, 1, 0))

        _fields_3d(fs, rng, k + 1, nlev, cfg.ar1, put)
        row += nlev
    # mean / perturbation split (run_da_parallel pre-processing)
    if backend == "torch":
        axb = xb_in.sum(dim=3) / float(np.float32(k))
        xb = xb_in - axb[..., None]
        truth = truth_t.cpu().numpy()
        del xb_in
    else:
        axb = xb_in.sum(axis=3) / float(np.float32(k))
        xb = xb_in - axb[..., None]
        truth = truth_t
    obs = make_obs(cfg, truth, rng)
    return Workload(cfg, xb, axb, truth, obs)


def _bilinear(cfg: Config, field2d: np.ndarray, la: np.ndarray, lo: np.ndarray):
    """Bilinear interpolation of a (lon_e, lat_e) field at obs points."""
    lat, lon, lat_e, lon_e = _extended_axes(cfg)
    dlat = 180.0 / cfg.num_lat
    dlon = 360.0 / cfg.num_lon
    fi = (la - lat_e[0]) / dlat
    fj = (lo - lon_e[0]) / dlon
    i0 = np.clip(np.floor(fi).astype(np.int64), 0, lat_e.size - 2)
    j0 = np.clip(np.floor(fj).astype(np.int64), 0, lon_e.size - 2)
    wi = fi - i0
    wj = fj - j0
    f = field2d
    return ((1 - wi) * (1 - wj) * f[j0, i0] + wi * (1 - wj) * f[j0, i0 + 1] +
            (1 - wi) * wj * f[j0 + 1, i0] + wi * wj * f[j0 + 1, i0 + 1])


def obs_locations(cfg: Config, rng: np.random.Generator, n: int):
    n_cl = int(round(cfg.clustered_frac * n))
    n_un = n - n_cl
    lat = np.degrees(np.arcsin(rng.uniform(-1.0, 1.0, n_un)))
    lon = rng.uniform(0.0, 360.0, n_un)
    if n_cl:
        clat = np.degrees(np.arcsin(rng.uniform(-0.9, 0.9, cfg.n_clusters)))
        clon = rng.uniform(0.0, 360.0, cfg.n_clusters)
        which = rng.integers(0, cfg.n_clusters, n_cl)
        dla = rng.normal(0.0, cfg.cluster_sigma_deg, n_cl)
        dlo = rng.normal(0.0, cfg.cluster_sigma_deg, n_cl)
        cla = np.clip(clat[which] + dla, -89.9, 89.9)
        clo = np.mod(clon[which] + dlo / np.cos(np.radians(cla)), 360.0)
        lat = np.concatenate([lat, cla])
        lon = np.concatenate([lon, clo])
        perm = rng.permutation(n)
        lat, lon = lat[perm], lon[perm]
    lat32 = lat.astype(np.float32)
    lon32 = lon.astype(np.float32)
    lon32[lon32 >= np.float32(360.0)] = np.float32(0.0)
    return lat32.astype(np.float64), lon32.astype(np.float64)


def make_obs(cfg: Config, truth: np.ndarray, rng: np.random.Generator) -> ObsSet:
    """Observation set: one type per DA variable (each observation is one
    (level, variable) entry, obs_nz = obs_nvar = 1)."""
    n = cfg.n_obs
    lat, lon = obs_locations(cfg, rng, n)
    nv = len(cfg.var_names)
    types = [(1, 1, [v]) for v in range(nv)]
    tidx = rng.integers(0, nv, n).astype(np.int32) if nv > 1 else np.zeros(n, np.int32)
    lev = rng.integers(0, cfg.nz, n)
    a, b, p0, ptop = vertical_coord(cfg)
    var_start = np.concatenate([[0], np.cumsum(cfg.var_lev)[:-1]])
    ps_truth = _bilinear(cfg, truth[:, :, 0], lat, lon)
    ph = np.empty(n)
    yo = np.empty(n)
    rinv = np.empty(n)
    sig = cfg.obs_sigma or {}
    noise = rng.standard_normal(n)
    for t in range(nv):
        sel = np.nonzero(tidx == t)[0]
        if sel.size == 0:
            continue
        vname = cfg.var_names[t]
        lv = cfg.var_lev[t]
        r = var_start[t] + (lev[sel] if lv > 1 else 0)
        val = np.empty(sel.size)
        for rr in np.unique(r):
            m = r == rr
            val[m] = _bilinear(cfg, truth[:, :, rr], lat[sel][m], lon[sel][m])
        s32 = np.float32(sig.get(vname, 1.0))
        rinv[sel] = float(np.float32(1.0) / (s32 * s32))
        yo[sel] = (val.astype(np.float32) + (noise[sel] * s32).astype(np.float32)).astype(
            np.float32)
        if lv > 1:
            ps = ps_truth[sel]
            if cfg.vcoord == LG_VCOORD_SIGMA:
                lev_p = lambda kk: a[kk] * (ps - ptop) + ptop
            else:
                lev_p = lambda kk: a[kk] * (p0 - ptop) + b[kk] * (ps - ptop) + ptop
            L = lev[sel]
            ph[sel] = (0.5 * (lev_p(L) + lev_p(L + 1))).astype(np.float32)
        else:
            ph[sel] = yo[sel] if vname == "ps" else np.float32(1.0e5)
    return ObsSet(types, tidx, lat, lon, ph.astype(np.float64), yo.astype(np.float64),
                  rinv.astype(np.float64))
