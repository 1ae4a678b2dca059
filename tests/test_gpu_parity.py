"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bars (the reference's own tolerance for the plain FP64 path):
  * neighbour lists (entry indices, order, count) bit-exact, weights within 1e-13;
  * H(x) and innovations within 1e-12 relative (libm vs CUDA log ulps);
  * analysis (xa + axa) within 1e-10 relative to the oracle's increment scale.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_ANALYSIS = 1e-10


def _run_both(name, **over):
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset(name).replace(**over)
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    o = orc.Oracle(cfg, w.obs)
    yb_o, dis_o, _ = o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    st_o = o.analysis(w.xb, w.axb, xa_o, axa_o)
    return cfg, w, ctx, o, (xa, axa), (xa_o, axa_o, yb_o, dis_o, st_o)


def _rel_err(cfg, w, got, ref):
    h = cfg.halo
    xa, axa = got
    xa_o, axa_o = ref
    full_g = (xa + axa[..., None])[h:-h, h:-h]
    full_o = (xa_o + axa_o[..., None])[h:-h, h:-h]
    bg = (w.xb + w.axb[..., None])[h:-h, h:-h]
    scale = np.abs(full_o - bg).max()
    return np.abs(full_g - full_o).max() / scale


@pytest.mark.parametrize("name", ["tiny2d", "tiny3d", "cfg1", "small3d"])
def test_analysis_matches_oracle(name):
    cfg, w, ctx, o, got, ref = _run_both(name)
    xa_o, axa_o, yb_o, dis_o, st_o = ref
    # copy layout identical
    co, cb, ce = ctx.copy_layout()
    co_o, cb_o, ce_o = o.copy_layout()
    assert np.array_equal(co, co_o) and np.array_equal(cb, cb_o) and np.array_equal(ce, ce_o)
    # H(x)
    yb, dis = ctx.hx(o.n_entries)
    assert np.allclose(yb, yb_o, rtol=1e-12, atol=1e-12 * np.abs(yb_o).max())
    assert np.allclose(dis, dis_o, rtol=1e-12, atol=1e-12 * np.abs(dis_o).max())
    # neighbour lists bit-exact, every column
    counts, ent, rloc = ctx.lists()
    off = np.concatenate([[0], np.cumsum(counts)])
    ncol = cfg.num_lat * cfg.num_lon
    for col in range(ncol):
        e_o, r_o = o.column_list(col)
        assert counts[col] == e_o.size, f"count mismatch at column {col}"
        assert np.array_equal(ent[off[col]:off[col + 1]], e_o), f"order mismatch at column {col}"
        # rloc in [0, 1]; near ri = 2 the Gaspari-Cohn polynomial cancels to ~1e-6,
        # so a 1-ulp libm difference in ri shows as ~1e-15 absolute
        np.testing.assert_allclose(rloc[off[col]:off[col + 1]], r_o, rtol=0, atol=1e-13)
    st = ctx.stats()
    assert st["nobsl_total"] == st_o["nobsl_total"]
    assert st["n_eig_fail"] == 0
    err = _rel_err(cfg, w, got, ref[:2])
    assert err < RTOL_ANALYSIS, f"{name}: analysis rel err {err:.3e}"
    ctx.letkf_final()


@pytest.mark.parametrize("ens", [96, 128])
def test_analysis_matches_oracle_above_64_members(ens):
    """The analysis path's eigensolve (warp-per-matrix tridiagonalisation whose
    matrix-vector product takes whole rows in rounds of 32 lanes, lane-per-matrix
    QL) at ensemble sizes above 64, FP64, against the oracle."""
    cfg, w, ctx, o, got, ref = _run_both("tiny3d", ens=ens)
    counts, ent, _ = ctx.lists()
    off = np.concatenate([[0], np.cumsum(counts)])
    for col in range(0, cfg.num_lat * cfg.num_lon, 5):
        e_o, _ = o.column_list(col)
        assert np.array_equal(ent[off[col]:off[col + 1]], e_o)
    assert ctx.stats()["n_eig_fail"] == 0
    err = _rel_err(cfg, w, got, ref[:2])
    assert err < RTOL_ANALYSIS, f"ens={ens}: analysis rel err {err:.3e}"
    ctx.letkf_final()


def test_max_obs_cap_truncates_like_reference():
    cfg, w, ctx, o, got, ref = _run_both("small3d", max_obs=40)
    counts, ent, _ = ctx.lists()
    assert counts.max() == 40
    off = np.concatenate([[0], np.cumsum(counts)])
    for col in range(0, cfg.num_lat * cfg.num_lon, 97):
        e_o, _ = o.column_list(col)
        assert np.array_equal(ent[off[col]:off[col + 1]], e_o)
    assert _rel_err(cfg, w, got, ref[:2]) < RTOL_ANALYSIS


def test_single_lon_block_duplicates_every_observation():
    """global_ny = 1: comm_info_init yields west_n=1, east_n=0, so the own block
    is visited twice and every local observation appears twice."""
    cfg, w, ctx, o, got, ref = _run_both("tiny2d", global_ny=1, global_nx=2)
    counts, ent, _ = ctx.lists()
    off = np.concatenate([[0], np.cumsum(counts)])
    col = cfg.num_lat // 2
    lst = ent[off[col]:off[col + 1]]
    vals, cnt = np.unique(lst, return_counts=True)
    assert (cnt % 2 == 0).all() and lst.size > 0
    assert _rel_err(cfg, w, got, ref[:2]) < RTOL_ANALYSIS


def test_box_localisation_and_polar_discard():
    cfg, w, ctx, o, got, ref = _run_both("tiny3d", gc_filter=0, gc_filter_vertical=0,
                                         obs_polar=60.0)
    counts, ent, rloc = ctx.lists()
    assert set(np.unique(rloc)) <= {1.0}
    co, cb, ce = ctx.copy_layout()
    obs_of_entry = np.repeat(co, np.diff(ce))
    assert (np.abs(w.obs.lat[obs_of_entry[ent]]) <= 60.0).all()
    assert _rel_err(cfg, w, got, ref[:2]) < RTOL_ANALYSIS


def test_core_batch_matches_oracle_core():
    import letkf_gb300 as lg
    from oracle import oracle as orc

    rng = np.random.default_rng(3)
    for k, p in [(16, 0), (16, 1), (40, 37), (64, 500), (128, 300)]:
        hx = rng.standard_normal((p, k))
        hx -= hx.mean(axis=1, keepdims=True)
        rd = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
        dep = rng.standard_normal(p)
        rloc = rng.uniform(0.0, 1.0, p)
        trans, wbar = lg.letkf_core(hx, rd, dep, rloc, 1.05)
        trans_o, wbar_o = orc.core(hx, rd, dep, rloc, 1.05)
        assert np.allclose(trans, trans_o, rtol=1e-11, atol=1e-11), (k, p)
        assert np.allclose(wbar, wbar_o, rtol=1e-11, atol=1e-11), (k, p)


def test_rotation_log_overflow_falls_back_to_accumulating_solver(monkeypatch):
    """With a 5-rotation log every QL overflows; those solves are redone by the
    eigenvector-accumulating solver and the analysis must still match."""
    monkeypatch.setenv("LETKF_GB300_ROT_CAP", "5")
    cfg, w, ctx, o, got, ref = _run_both("tiny3d")
    assert _rel_err(cfg, w, got, ref[:2]) < RTOL_ANALYSIS
    ctx.letkf_final()


def test_linear_and_cell_indexed_selection_agree(monkeypatch):
    """The cell-indexed selection and the plain scan of every neighbour-block
    copy must produce identical lists."""
    import letkf_gb300 as lg
    import synth
    cfg = lg.preset("small3d")
    w = synth.make_workload(cfg)
    out = []
    for linear in (False, True):
        if linear:
            monkeypatch.setenv("LETKF_GB300_LINEAR_SEARCH", "1")
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        out.append(ctx.lists())
        ctx.letkf_final()
    (c0, e0, r0), (c1, e1, r1) = out
    assert np.array_equal(c0, c1) and np.array_equal(e0, e1) and np.array_equal(r0, r1)


def test_repeated_runs_replay_the_captured_graph():
    """The first lg_run captures the analysis into a CUDA graph and later runs
    replay it; a second background through the same context must still match
    the oracle, and an eager run (LETKF_GB300_NO_GRAPH) must agree bit for bit."""
    import os
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset("tiny3d")
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    o = orc.Oracle(cfg, w.obs)
    results = []
    for scale in (1.0, 1.3):
        xb = np.ascontiguousarray(w.xb * scale)
        xa = np.zeros_like(xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, xb, w.axb, xa, axa)
        o.hx(xb, w.axb)
        xa_o = np.zeros_like(xb)
        axa_o = np.zeros_like(w.axb)
        o.analysis(xb, w.axb, xa_o, axa_o)
        w2 = synth.Workload(cfg, xb, w.axb, w.truth, w.obs)
        assert _rel_err(cfg, w2, (xa, axa), (xa_o, axa_o)) < RTOL_ANALYSIS
        results.append((xa.copy(), axa.copy()))
    ctx.letkf_final()
    os.environ["LETKF_GB300_NO_GRAPH"] = "1"
    try:
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xb = np.ascontiguousarray(w.xb * 1.3)
        xa = np.zeros_like(xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, xb, w.axb, xa, axa)
        assert np.array_equal(xa, results[1][0]) and np.array_equal(axa, results[1][1])
        ctx.letkf_final()
    finally:
        del os.environ["LETKF_GB300_NO_GRAPH"]


def test_first_analysis_takes_the_sizing_counts():
    """After lg_set_obs the first analysis takes the neighbour-list counts and
    selection statistics of the count pass that sized the lists; later analyses
    count again.  Lists, statistics and analyses must agree bit for bit, for a
    second observation set and back, in both precisions."""
    import letkf_gb300 as lg
    import synth

    keys = ("nobsl_total", "nobsl_max", "n_capped", "n_band")
    for prec in (lg.LG_PREC_FP64, lg.LG_PREC_MIXED):
        cfg = lg.preset("small3d").replace(max_obs=40, precision=prec)
        w = synth.make_workload(cfg)
        o = w.obs
        m = o.n_obs // 2
        half = lg.ObsSet(o.types, o.type[:m], o.lat[:m], o.lon[:m], o.ph[:m], o.yo[:m],
                         o.rinv[:m])

        def run(ctx):
            xa = np.zeros_like(w.xb)
            axa = np.zeros_like(w.axb)
            ctx.letkf_run(0, w.xb, w.axb, xa, axa)
            st = ctx.stats()
            return xa, axa, ctx.lists(), {k: st[k] for k in keys}

        def same(a, b):
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            for x, y in zip(a[2], b[2]):
                assert np.array_equal(x, y)
            assert a[3] == b[3], (a[3], b[3])

        ctx = lg.Letkf(cfg)
        ctx.set_obs(o)
        first = run(ctx)
        same(first, run(ctx))
        assert first[3]["n_capped"] > 0 and first[3]["nobsl_max"] == 40
        ctx.set_obs(half)
        h1 = run(ctx)
        same(h1, run(ctx))
        assert h1[3]["nobsl_total"] < first[3]["nobsl_total"]
        ctx.set_obs(o)
        same(run(ctx), first)
        ctx.letkf_final()
