"""CPU tests of the oracle (no GPU): closed-form known-answer tests that pin
letkf_core, the precision helpers and the selection rules.

The reference ships no golden vectors for this path, so these are the pins:
  * p = 0: trans = sqrt(rho) I, overline_w = 0 (inflation only);
  * one observation: the scalar Kalman update in ensemble space;
  * W symmetric, W 1 = sqrt(rho) 1 for zero-mean Yb, W^2 (C + (k-1)/rho I) = (k-1) I;
  * schr2 = Gaspari-Cohn with REAL(4) constants, positive on (0, 2], zero beyond;
  * latlon_dist with REAL(4) pi and radius;
  * the single-longitude-block duplication of comm_info_init.
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle
    return oracle


def gc_exact(r):
    r = abs(r)
    if r <= 1.0:
        return (((-0.25 * r + 0.5) * r + 0.625) * r - 5.0 / 3.0) * r * r + 1.0
    if r <= 2.0:
        return ((((r / 12.0 - 0.5) * r + 0.625) * r + 5.0 / 3.0) * r - 5.0) * r + 4.0 - 2.0 / (3.0 * r)
    return 0.0


def test_schr2_matches_gaspari_cohn_and_is_positive(orc):
    L = orc.lib()
    for r in np.linspace(0.0, 2.5, 2001):
        v = L.or_schr2(float(r))
        assert abs(v - gc_exact(r)) < 2e-6
        if r <= 2.0:
            assert v > 0.0
        else:
            assert v == 0.0
    assert L.or_schr2(0.0) == 1.0
    # REAL(4) literal 1.666667 leaves a positive residue at ri = 2
    assert 1e-6 < L.or_schr2(2.0) < 2e-6
    assert L.or_schr(2.0) == 1.0 and L.or_schr(2.0000001) == 0.0


def test_latlon_dist_uses_real4_constants(orc):
    L = orc.lib()
    a = float(np.float32(6371.393))
    pi_f = float(np.float32(math.pi))
    d = L.or_latlon_dist_r8(0.0, 0.0, 0.0, 90.0)
    # cos(90/180*pi_f) is not exactly 0: the distance is a*acos(cos(pi_f/2))
    assert abs(d - a * math.acos(math.cos(90.0 / 180.0 * pi_f))) < 1e-9
    # cos^2 + sin^2 rounds below 1, so a point's distance to itself is ~1e-4 km, not 0
    assert 0.0 <= L.or_latlon_dist_r8(10.0, 20.0, 10.0, 20.0) < 1e-3
    d4 = L.or_latlon_dist_r4(0.0, 0.0, 0.0, 90.0)
    assert abs(d4 - a * math.pi / 2) < 1.0


def test_core_no_observations_is_pure_inflation(orc):
    for k in (2, 16, 40):
        trans, wbar = orc.core(np.zeros((0, k)), np.zeros(0, np.float32), np.zeros(0),
                               np.zeros(0), 1.1)
        assert np.allclose(trans, math.sqrt(1.1) * np.eye(k), atol=1e-13)
        assert np.allclose(wbar, 0.0)


def test_core_single_observation_closed_form(orc):
    rng = np.random.default_rng(1)
    k, rho = 16, 1.05
    y = rng.standard_normal(k)
    y -= y.mean()
    rinv = np.float32(4.0)
    rloc = 0.6
    dep = 0.7
    trans, wbar = orc.core(y[None, :], np.array([rinv]), np.array([dep]), np.array([rloc]), rho)
    trans = trans.T  # trans[i, j] = Fortran trans(i, j)
    w = float(rinv) * rloc
    alpha = (k - 1) / rho
    lam = w * y @ y
    v = y / np.linalg.norm(y)
    wbar_ref = w * dep * y / (lam + alpha)
    W_ref = math.sqrt(rho) * (np.eye(k) - np.outer(v, v)) + \
        math.sqrt((k - 1) / (lam + alpha)) * np.outer(v, v)
    assert np.allclose(wbar, wbar_ref, rtol=1e-12, atol=1e-14)
    assert np.allclose(trans, W_ref + wbar_ref[:, None], rtol=1e-12, atol=1e-13)


def test_core_invariants(orc):
    rng = np.random.default_rng(2)
    k, p, rho = 24, 60, 1.1
    hx = rng.standard_normal((p, k))
    hx -= hx.mean(axis=1, keepdims=True)
    rd = (rng.uniform(0.5, 3.0, p)).astype(np.float32)
    dep = rng.standard_normal(p)
    rloc = rng.uniform(0.0, 1.0, p)
    trans, wbar = orc.core(hx, rd, dep, rloc, rho)
    T = trans.T
    W = T - wbar[:, None]
    assert np.allclose(W, W.T, atol=1e-12)
    assert np.allclose(W @ np.ones(k), math.sqrt(rho) * np.ones(k), atol=1e-10)
    s = np.sqrt(rd.astype(np.float64) * rloc)
    Yt = (hx * s[:, None]).T
    Cm = Yt @ Yt.T
    alpha = (k - 1) / rho
    assert np.allclose(W @ W @ (Cm + alpha * np.eye(k)), (k - 1) * np.eye(k), atol=1e-8)
    Pa = np.linalg.inv(Cm + alpha * np.eye(k))
    assert np.allclose(wbar, Pa @ (Yt @ (s * dep)), atol=1e-12)


def _run_oracle(name, **over):
    import letkf_gb300 as lg
    import synth
    from oracle import oracle

    cfg = lg.preset(name).replace(**over)
    w = synth.make_workload(cfg)
    o = oracle.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    st = o.analysis(w.xb, w.axb, xa, axa)
    return cfg, w, o, xa, axa, st


def test_analysis_recentres_and_improves_2d():
    cfg, w, o, xa, axa, st = _run_oracle("cfg1")
    h = cfg.halo
    assert np.abs(xa[h:-h, h:-h].mean(axis=-1)).max() < 1e-12
    err_b = np.sqrt(np.mean((w.axb - w.truth)[h:-h, h:-h] ** 2))
    err_a = np.sqrt(np.mean((axa - w.truth)[h:-h, h:-h] ** 2))
    assert err_a < err_b
    assert st["n_eig_fail"] == 0 and st["n_columns"] == cfg.num_lat * cfg.num_lon


def test_single_lon_block_lists_every_observation_twice():
    cfg, w, o, xa, axa, st = _run_oracle("tiny2d", global_ny=1, global_nx=2)
    off, blk = o.neighbour_table()
    for b in range(cfg.global_nx):
        nb = blk[off[b]:off[b + 1]]
        vals, cnt = np.unique(nb, return_counts=True)
        assert (cnt == 2).all()


def test_neighbour_table_contains_own_block():
    cfg, w, o, xa, axa, st = _run_oracle("tiny3d")
    off, blk = o.neighbour_table()
    for b in range(cfg.global_nx * cfg.global_ny):
        assert b in set(blk[off[b]:off[b + 1]].tolist())


def test_boundary_observation_is_copied_into_both_blocks():
    import letkf_gb300 as lg
    import synth
    from oracle import oracle

    cfg = lg.preset("tiny2d")
    w = synth.make_workload(cfg)
    lat, lon = lg.model_grid(cfg)
    # block boundary latitude between the two latitude blocks
    xs = cfg.num_lat // cfg.global_nx
    obs = w.obs
    obs.lat[0] = float(lat[xs])  # first latitude of block 2 = upper bound of block 1
    o = oracle.Oracle(cfg, obs)
    co, cb, ce = o.copy_layout()
    assert (co == 0).sum() == 2


def test_post_processing_kat():
    """gamma1 = 0, gamma2 = 1 returns the analysis; poleward rows keep the
    background; spreads are the RMS over members."""
    import letkf_gb300 as lg
    from oracle import oracle

    cfg = lg.preset("tiny2d")
    rng = np.random.default_rng(5)
    shp = (cfg.num_lon + 2, cfg.num_lat + 2, 1, cfg.ens)
    xb = rng.standard_normal(shp)
    xa = rng.standard_normal(shp)
    axb = rng.standard_normal(shp[:-1])
    axa = rng.standard_normal(shp[:-1])
    xo, sb, sa = oracle.post(cfg, 0.0, 1.0, 80.0, xb, axb, xa, axa)
    lat, _ = lg.model_grid(cfg)
    for j in range(cfg.num_lat):
        if abs(lat[j]) <= 80.0:
            assert np.allclose(xo[1:-1, j + 1], (axa[..., None] + xa)[1:-1, j + 1])
        else:
            assert np.allclose(xo[1:-1, j + 1], (axb[..., None] + xb)[1:-1, j + 1])
    assert np.allclose(sb[:, :, 0], np.sqrt((xb[1:-1, 1:-1, 0] ** 2).mean(-1)))
    assert (xo[0] == 0).all()


def _block_bounds(n, nb):
    """pro_info_get_indx (pro_info.F90:96-125): 1-based (start, end) per block."""
    sec, res = n // nb, n % nb
    out = []
    for b in range(1, nb + 1):
        if b - 1 < res:
            s = (b - 1) * (sec + 1) + 1
            out.append((s, s + sec))
        else:
            s = (b - 1) * sec + res + 1
            out.append((s, s + sec - 1))
    return out


def _cube_expected(cfg, w, o):
    """The cube loops of letkf_compute_nooverlap (overlap 0) and letkf_compute
    (overlap > 0, letkf_compute.F90:12-154, 156-256) restated in numpy for a
    horizontal-only configuration, each cube's trans from its centre column."""
    h, k = cfg.halo, cfg.ens
    xb, axb = w.xb, w.axb
    xa = np.zeros_like(xb)
    axa = np.zeros_like(axb)
    cnt = np.zeros(axb.shape[:2])
    ncubes = 0
    stride = cfg.cube_n - cfg.overlap
    for (la0, la1) in _block_bounds(cfg.num_lat, cfg.global_nx):
        for (lo0, lo1) in _block_bounds(cfg.num_lon, cfg.global_ny):
            nxl, nyl = la1 - la0 + 1, lo1 - lo0 + 1
            for i in range(1, nyl + 1, stride):
                si, ei = i, min(i + cfg.cube_n - 1, nyl)
                for j in range(1, nxl + 1, stride):
                    sj, ej = j, min(j + cfg.cube_n - 1, nxl)
                    cglat, cglon = la0 - 1 + (sj + ej) // 2, lo0 - 1 + (si + ei) // 2
                    t = o.column_trans((cglon - 1) * cfg.num_lat + (cglat - 1))
                    ncubes += 1
                    for ii in range(si, ei + 1):
                        for jj in range(sj, ej + 1):
                            x, y = h + lo0 - 1 + ii - 1, h + la0 - 1 + jj - 1
                            dist = axb[x, y][:, None] + xb[x, y] @ t.T
                            mean = dist.mean(axis=1)
                            xa[x, y] += dist - mean[:, None]
                            axa[x, y] += mean
                            cnt[x, y] += 1
    inner = (slice(h, -h), slice(h, -h))
    assert np.all(cnt[inner] >= 1)
    xa[inner] /= cnt[inner][..., None, None]
    axa[inner] /= cnt[inner][..., None]
    return xa, axa, ncubes


@pytest.mark.parametrize("cube_n,overlap", [(3, 0), (3, 1), (2, 1)])
def test_cube_analysis_matches_numpy_restatement(cube_n, overlap):
    """Horizontal cubes (one solve per cube from its centre column's list),
    with and without overlap (averaged over the covering cubes)."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc
    cfg = lg.preset("tiny2d").replace(cube_n=cube_n, overlap=overlap)
    w = synth.make_workload(cfg)
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    st = o.analysis(w.xb, w.axb, xa, axa)
    xe, ae, ncubes = _cube_expected(cfg, w, o)
    h = cfg.halo
    full = (xa + axa[..., None])[h:-h, h:-h]
    full_e = (xe + ae[..., None])[h:-h, h:-h]
    scale = np.abs(full_e).max()
    assert np.abs(full - full_e).max() <= 1e-12 * scale
    assert st["n_solves"] == ncubes and st["n_columns"] >= cfg.num_lat * cfg.num_lon


def test_cube_centre_columns_and_levels_match_per_column_analysis():
    """Vertical path: with cube_n = 2 the centre column of every cube has the
    per-column analysis; with cube_nz = 3 the 3-D rows at each level group's
    centre level have it (the group's solve is the centre level's)."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc
    base = lg.preset("tiny3d")
    w = synth.make_workload(base)

    def run(cfg):
        o = orc.Oracle(cfg, w.obs)
        o.hx(w.xb, w.axb)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        o.analysis(w.xb, w.axb, xa, axa)
        return xa, axa

    ref = run(base)
    h = base.halo
    cub = run(base.replace(cube_n=2))
    for (la0, la1) in _block_bounds(base.num_lat, base.global_nx):
        for (lo0, lo1) in _block_bounds(base.num_lon, base.global_ny):
            nxl, nyl = la1 - la0 + 1, lo1 - lo0 + 1
            for i in range(1, nyl + 1, 2):
                ci = (i + min(i + 1, nyl)) // 2
                for j in range(1, nxl + 1, 2):
                    cj = (j + min(j + 1, nxl)) // 2
                    x, y = h + lo0 - 1 + ci - 1, h + la0 - 1 + cj - 1
                    assert np.array_equal(cub[0][x, y], ref[0][x, y])
                    assert np.array_equal(cub[1][x, y], ref[1][x, y])
    vz = run(base.replace(cube_nz=3))
    rows = []
    r0 = 0
    for name, lv in zip(base.var_names, base.var_lev):
        if lv > 1:
            for sk in range(1, base.nz + 1, 3):
                ek = min(sk + 2, base.nz)
                rows.append(r0 + (sk + ek) // 2 - 1)
        r0 += lv
    inner = (slice(h, -h), slice(h, -h))
    assert np.array_equal(vz[0][inner][:, :, rows], ref[0][inner][:, :, rows])
    other = [r for r in range(base.n_rows) if r not in rows]
    assert not np.array_equal(vz[0][inner][:, :, other], ref[0][inner][:, :, other])
