"""GPU parity of the cube analyses (da_block_interval cube_n, da_vertical_interval
cube_nz, da_block_overlap): one solve per cube (and level group) from the
list of its centre column, applied to every column (and level) of the cube,
overlapping cubes averaged -- against the oracle's restatement of
letkf_compute_nooverlap[_vertical] and letkf_compute."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("tiny2d", dict(cube_n=3)),
    ("tiny2d", dict(cube_n=3, overlap=1)),
    ("tiny2d", dict(cube_n=2, overlap=1)),
    ("tiny3d", dict(cube_n=2)),
    ("tiny3d", dict(cube_nz=3)),
    ("tiny3d", dict(cube_n=2, cube_nz=2)),
    ("tiny3d", dict(cube_n=3, overlap=1)),  # overlap: horizontal localisation only
]


def _oracle(cfg, w):
    from oracle import oracle as orc
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    st = o.analysis(w.xb, w.axb, xa, axa)
    return xa, axa, st


def _rel_err(cfg, w, got, ref):
    h = cfg.halo
    full_g = (got[0] + got[1][..., None])[h:-h, h:-h]
    full_o = (ref[0] + ref[1][..., None])[h:-h, h:-h]
    inc_o = full_o - (w.xb + w.axb[..., None])[h:-h, h:-h]
    assert np.all(np.isfinite(full_g))
    return np.abs(full_g - full_o).max() / np.abs(inc_o).max()


@pytest.mark.parametrize("name,over", CASES)
def test_cube_analysis_fp64_matches_oracle(name, over, monkeypatch):
    import letkf_gb300 as lg
    import synth
    monkeypatch.setenv("LETKF_GB300_CHUNK_MB", "1")  # several chunks of solves
    cfg = lg.preset(name).replace(**over)
    w = synth.make_workload(cfg)
    xa_o, axa_o, st_o = _oracle(cfg, w)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    st = ctx.stats()
    assert st["n_solves"] == st_o["n_solves"] and st["n_eig_fail"] == 0
    assert _rel_err(cfg, w, (xa, axa), (xa_o, axa_o)) < 1e-10, (name, over)
    # a second analysis (graph replay) gives the same result
    xa2 = np.zeros_like(w.xb)
    axa2 = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa2, axa2)
    assert np.array_equal(xa2, xa) and np.array_equal(axa2, axa)
    ctx.letkf_final()


@pytest.mark.parametrize("name,over", [("tiny3d", dict(cube_n=2, cube_nz=2)),
                                       ("tiny2d", dict(cube_n=3, overlap=1))])
def test_cube_analysis_mixed_within_tolerance(name, over):
    import letkf_gb300 as lg
    import synth
    from test_gpu_mixed import TOL_INCREMENT, increment_rel_rms
    base = lg.preset(name).replace(**over)
    cfg = base.replace(precision=lg.LG_PREC_MIXED)
    w = synth.make_workload(cfg)
    xa_o, axa_o, _ = _oracle(base, w)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    errs = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
    assert max(errs.values()) <= TOL_INCREMENT, errs
    ctx.letkf_final()


def test_cube_mixed_fallback_for_overflowed_rotation_logs(monkeypatch):
    """Mixed cube solves whose QL rotation log overflows get their trans from
    the FP64 solver instead of the FP32 pipeline: a 50-entry log sends almost
    every solve there, and the analysis stays within the tolerance."""
    import letkf_gb300 as lg
    import synth
    from test_gpu_mixed import TOL_INCREMENT, increment_rel_rms
    monkeypatch.setenv("LETKF_GB300_ROT_CAP", "50")
    base = lg.preset("tiny3d").replace(cube_n=2)
    cfg = base.replace(precision=lg.LG_PREC_MIXED)
    w = synth.make_workload(cfg)
    xa_o, axa_o, _ = _oracle(base, w)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    errs = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
    assert max(errs.values()) <= TOL_INCREMENT, errs
    ctx.letkf_final()


def test_cube_lists_only_at_centres():
    """With cubes the selection builds only the cube centres' lists; each one
    equals the oracle's list of that column."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc
    cfg = lg.preset("tiny3d").replace(cube_n=3)
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    counts, ent, _ = ctx.lists()
    o = orc.Oracle(cfg, w.obs)
    off = np.concatenate([[0], np.cumsum(counts)])
    nz_cols = np.nonzero(counts)[0]
    assert 0 < nz_cols.size < cfg.num_lat * cfg.num_lon // 4
    for col in nz_cols[:: max(1, nz_cols.size // 12)]:
        e_o, _ = o.column_list(int(col))
        assert np.array_equal(ent[off[col]:off[col + 1]], e_o)
    ctx.letkf_final()


@pytest.mark.parametrize("over", [dict(cube_n=3, overlap=1), dict(cube_n=2, cube_nz=3)])
def test_cube_host_run_pinned_matches_pageable(over):
    """lg_run with page-locked host arrays on the cube path (copies inside the
    captured analysis) equals the pageable-array path bit for bit."""
    import torch

    import letkf_gb300 as lg
    import synth
    cfg = lg.preset("tiny3d").replace(**over)
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.full_like(w.xb, 3.0)
    axa = np.full_like(w.axb, 3.0)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    pin = [torch.from_numpy(a).pin_memory() for a in (w.xb, w.axb)]
    out = [torch.full(a.shape, 3.0, dtype=torch.float64).pin_memory() for a in (w.xb, w.axb)]
    pxb, paxb, pxa, paxa = (t.numpy() for t in pin + out)
    ctx.letkf_run(0, pxb, paxb, pxa, paxa)
    assert np.array_equal(pxa, xa) and np.array_equal(paxa, axa)
    ctx.letkf_final()
