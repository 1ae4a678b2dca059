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
