"""GPU parity at the full benchmark grids (360 x 180 x 32, ps/u/v/pt), plain
FP64 path, through the C ABI, against the CPU oracle on a column sample.

The whole-globe oracle analysis takes minutes to hours on the host at these
sizes, so the oracle analyses a deterministic sample of columns spread over
the globe (every latitude band and many longitudes, both polar rows, and the
rows and columns on the virtual block boundaries, where observations appear in
two blocks' lists) and the GPU analysis of the whole globe is compared there.

Bars (the plain FP64 path's contract):
  * neighbour lists (entry indices, order, count) bit-exact, weights within 1e-13;
  * analysis (xa + axa) within 1e-10 relative to the oracle's increment scale
    over the sampled columns.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_ANALYSIS = 1e-10


def _block_boundary_columns(cfg, lat_step, lon_step):
    """Columns on the first/last latitude row and longitude column of every
    virtual block, thinned by lat_step / lon_step along the boundary."""
    nl, nn = cfg.num_lat, cfg.num_lon
    lat_rows, lon_cols = set(), set()
    x_sec, x_res = divmod(nl, cfg.global_nx)
    y_sec, y_res = divmod(nn, cfg.global_ny)
    s = 0
    for bx in range(cfg.global_nx):
        e = s + x_sec + (1 if bx < x_res else 0)
        lat_rows.update((s, e - 1))
        s = e
    s = 0
    for by in range(cfg.global_ny):
        e = s + y_sec + (1 if by < y_res else 0)
        lon_cols.update((s, e - 1))
        s = e
    cols = set()
    for la in lat_rows:
        for lo in range(0, nn, lon_step):
            cols.add(lo * nl + la)
    for lo in lon_cols:
        for la in range(0, nl, lat_step):
            cols.add(lo * nl + la)
    return cols


def _compare_sampled(cfg, cols):
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    st = ctx.stats()
    assert st["n_eig_fail"] == 0
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    st_o = o.analysis_cols(w.xb, w.axb, xa_o, axa_o, cols)
    # lists: bit-exact entries and order, weights to 1e-13
    nmax = 0
    for col in cols:
        e_g, r_g = ctx.column_list(int(col))
        e_o, r_o = o.column_list(int(col))
        assert e_g.size == e_o.size, f"count mismatch at column {col}: {e_g.size} vs {e_o.size}"
        assert np.array_equal(e_g, e_o), f"order mismatch at column {col}"
        np.testing.assert_allclose(r_g, r_o, rtol=0, atol=1e-13)
        nmax = max(nmax, e_o.size)
    assert st["nobsl_max"] >= nmax
    assert st_o["nobsl_max"] == nmax
    # analysis at the sampled columns
    h = cfg.halo
    lon = cols // cfg.num_lat + h
    lat = cols % cfg.num_lat + h
    full_g = xa[lon, lat] + axa[lon, lat][..., None]
    full_o = xa_o[lon, lat] + axa_o[lon, lat][..., None]
    bg = w.xb[lon, lat] + w.axb[lon, lat][..., None]
    assert np.all(np.isfinite(full_g))
    scale = np.abs(full_o - bg).max()
    err = np.abs(full_g - full_o).max() / scale
    assert err < RTOL_ANALYSIS, f"{cfg.name}: analysis rel err {err:.3e} on {cols.size} columns"
    ctx.letkf_final()
    return st, err


def test_cfg2_fp64_drop_in_matches_oracle_on_sampled_columns():
    """cfg2: 360x180x32, N=40, 1e5 observations, 800 km + 0.2 ln p, the plain
    FP64 drop-in configuration.  Sample: every 53rd column, the block-boundary
    rows and columns, every 5th column of both polar rows."""
    import letkf_gb300 as lg

    cfg = lg.preset("cfg2")
    sel = set(range(0, cfg.num_lat * cfg.num_lon, 53))
    sel |= _block_boundary_columns(cfg, lat_step=11, lon_step=13)
    for lo in range(0, cfg.num_lon, 5):
        sel.update((lo * cfg.num_lat, lo * cfg.num_lat + cfg.num_lat - 1))
    cols = np.asarray(sorted(sel), np.int32)
    assert cols.size > 1500
    _compare_sampled(cfg, cols)


def test_cfg3_fp64_matches_oracle_on_sampled_columns():
    """cfg3's workload (N=64, 1e6 observations, MAX_OBS lifted: ~15 700 local
    entries per column) through the plain FP64 path: 16 latitude bands x 16
    longitudes plus both polar rows."""
    import letkf_gb300 as lg
    from oracle import oracle as orc

    cfg = lg.preset("cfg3").replace(precision=lg.LG_PREC_FP64)
    cols = orc.sample_columns(cfg, 16, 16)
    assert cols.size >= 256
    assert np.unique(cols // cfg.num_lat).size >= 16
    st, _ = _compare_sampled(cfg, cols)
    assert st["nobsl_max"] > 10000  # the regime above the reference's MAX_OBS
