"""run_da_parallel around the analysis (module_da_parallel.F90:165-263) on the
GPU: mean/perturbation split, letkf_run, RTPP blend with polar bypass and the
background/analysis spreads, against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_run_da_parallel_matches_oracle():
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset("tiny3d")
    w = synth.make_workload(cfg)
    xb_in = np.ascontiguousarray(w.xb + w.axb[..., None])
    g1, g2, polar = 0.6, 0.4, 75.0
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa_out = np.zeros_like(xb_in)
    sb = np.zeros((cfg.num_lon, cfg.num_lat, cfg.n_rows))
    sa = np.zeros_like(sb)
    ctx.run_da_parallel(0, g1, g2, polar, xb_in, xa_out, sb, sa)
    # oracle: split, analysis, post
    r, xb, axb = orc.split_mean(cfg.ens, xb_in)
    assert r == 0
    o = orc.Oracle(cfg, w.obs)
    o.hx(xb, axb)
    xa = np.zeros_like(xb)
    axa = np.zeros_like(axb)
    o.analysis(xb, axb, xa, axa)
    xo, sbo, sao = orc.post(cfg, g1, g2, polar, xb, axb, xa, axa)
    h = cfg.halo
    inc = np.abs(xo[h:-h, h:-h] - xb_in[h:-h, h:-h]).max()
    assert np.abs(xa_out - xo).max() <= 1e-10 * max(inc, 1e-300)
    np.testing.assert_allclose(sb, sbo, rtol=1e-12)
    np.testing.assert_allclose(sa, sao, rtol=1e-9)
    # halo zero, polar rows keep the background
    assert (xa_out[:h] == 0).all() and (xa_out[:, :h] == 0).all()
    lat, _ = lg.model_grid(cfg)
    polar_rows = np.nonzero(np.abs(lat[:-1]) > polar)[0]
    assert polar_rows.size > 0
    for j in polar_rows:
        np.testing.assert_allclose(xa_out[h:-h, j + h], xb_in[h:-h, j + h], rtol=1e-14, atol=1e-12)
    ctx.letkf_final()


def test_nan_in_background_is_reported():
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset("tiny2d")
    w = synth.make_workload(cfg)
    xb_in = np.ascontiguousarray(w.xb + w.axb[..., None])
    xb_in[3, 4, 0, 2] = np.nan
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa_out = np.zeros_like(xb_in)
    sb = np.zeros((cfg.num_lon, cfg.num_lat, cfg.n_rows))
    sa = np.zeros_like(sb)
    with pytest.raises(RuntimeError, match="LG_ERR_NAN"):
        ctx.run_da_parallel(0, 0.0, 1.0, 90.0, xb_in, xa_out, sb, sa)
    ctx.letkf_final()
