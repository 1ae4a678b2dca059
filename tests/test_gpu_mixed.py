"""GPU tests of the mixed-precision path (BF16 hi/lo tensor-core contractions,
FP64 eigensolve) against the FP64 oracle.

Bar: relative RMS of the analysis increment (xa_full - xb_full) <= 1e-4 per
variable, the tolerance the mixed path is specified to.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_INCREMENT = 1e-4


def increment_rel_rms(cfg, w, got, ref):
    """Per-variable relative RMS of the increment difference.  A non-finite
    analysis value anywhere in the interior makes every entry inf, so that a
    comparison against a tolerance fails (a NaN would compare false and slip
    through max())."""
    h = cfg.halo
    xa, axa = got
    xa_o, axa_o = ref
    if not (np.all(np.isfinite(xa[h:-h, h:-h])) and np.all(np.isfinite(axa[h:-h, h:-h]))):
        return {v: float("inf") for v in cfg.var_names}
    bg = (w.xb + w.axb[..., None])[h:-h, h:-h]
    inc_g = (xa + axa[..., None])[h:-h, h:-h] - bg
    inc_o = (xa_o + axa_o[..., None])[h:-h, h:-h] - bg
    out = {}
    r0 = 0
    for v, lv in zip(cfg.var_names, cfg.var_lev):
        sl = slice(r0, r0 + lv)
        d = inc_g[:, :, sl] - inc_o[:, :, sl]
        val = float(np.sqrt(np.mean(d ** 2)) / np.sqrt(np.mean(inc_o[:, :, sl] ** 2)))
        out[v] = val if np.isfinite(val) else float("inf")
        r0 += lv
    return out


def test_core_batch_mixed_close_to_fp64():
    import letkf_gb300 as lg
    from oracle import oracle as orc
    import ctypes as C
    import torch

    rng = np.random.default_rng(7)
    for k, p in [(16, 0), (16, 5), (40, 300), (64, 2000), (100, 700), (128, 0), (128, 3000)]:
        hx = rng.standard_normal((p, k))
        hx -= hx.mean(axis=1, keepdims=True)
        rd = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
        dep = rng.standard_normal(p)
        rloc = rng.uniform(0.0, 1.0, p)
        trans_o, wbar_o = orc.core(hx, rd, dep, rloc, 1.05)
        dev = torch.device("cuda")
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
        d_hx, d_rd, d_dep, d_rl = t(hx), t(rd), t(dep), t(rloc)
        d_n = torch.tensor([p], dtype=torch.int32, device=dev)
        d_off = torch.tensor([0], dtype=torch.int64, device=dev)
        d_tr = torch.zeros((k, k), dtype=torch.float64, device=dev)
        d_wb = torch.zeros(k, dtype=torch.float64, device=dev)
        L = lg.load_library()
        ptr = lambda x: C.c_void_p(x.data_ptr())
        st = L.lg_core_batch(k, 1, ptr(d_n), ptr(d_off), ptr(d_hx), ptr(d_rd), ptr(d_dep),
                             ptr(d_rl), 1.05, lg.LG_PREC_MIXED, ptr(d_tr), ptr(d_wb), None)
        assert st == 0
        torch.cuda.synchronize()
        tr, wb = d_tr.cpu().numpy(), d_wb.cpu().numpy()
        # BF16 hi/lo products with FP32 accumulation: ~1e-5 relative on trans
        rel = np.linalg.norm(tr - trans_o) / np.linalg.norm(trans_o)
        assert rel < 5e-5, (k, p, rel)
        if p:
            relw = np.linalg.norm(wb - wbar_o) / np.linalg.norm(wbar_o)
            assert relw < 1e-4, (k, p, relw)


@pytest.mark.parametrize("name,over", [("small3d", {}), ("tiny3d", {"ens": 64})])
def test_mixed_analysis_increment_within_1e4(name, over):
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset(name).replace(precision=lg.LG_PREC_MIXED, **over)
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa_o, axa_o)
    errs = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
    assert max(errs.values()) <= TOL_INCREMENT, errs
    # lists are computed exactly in both precisions
    counts, ent, _ = ctx.lists()
    e_o, _ = o.column_list(5)
    off = np.concatenate([[0], np.cumsum(counts)])
    assert np.array_equal(ent[off[5]:off[6]], e_o)
    ctx.letkf_final()


def _increment_rel_rms_cols(cfg, w, got, ref, cols):
    """increment_rel_rms restricted to the listed columns."""
    h = cfg.halo
    lon = cols // cfg.num_lat + h
    lat = cols % cfg.num_lat + h
    xa, axa = got
    xa_o, axa_o = ref
    g = xa[lon, lat] + axa[lon, lat][..., None]
    o = xa_o[lon, lat] + axa_o[lon, lat][..., None]
    bg = w.xb[lon, lat] + w.axb[lon, lat][..., None]
    if not np.all(np.isfinite(g)):
        return {v: float("inf") for v in cfg.var_names}
    out, r0 = {}, 0
    for v, lv in zip(cfg.var_names, cfg.var_lev):
        sl = slice(r0, r0 + lv)
        d = (g - bg)[:, sl] - (o - bg)[:, sl]
        out[v] = float(np.sqrt(np.mean(d ** 2)) / np.sqrt(np.mean((o - bg)[:, sl] ** 2)))
        r0 += lv
    return out


@pytest.mark.parametrize("name", ["tiny3d", "small3d"])
def test_mixed_128_members_on_tensor_cores_within_1e4(name):
    """N = 128 (the large-cycle ensemble size) in mixed precision: the Gram runs
    on the tcgen05 kernel for 65..128 members (Gram work counted, no FP64
    Gram), and the increment meets the 1e-4 bar against the FP64 oracle --
    tiny3d over the whole globe, small3d over every 7th column."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset(name).replace(precision=lg.LG_PREC_MIXED, ens=128)
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    st = ctx.stats()
    assert st["n_gram_entries"] > 0 and st["n_eig_fail"] == 0
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    if name == "tiny3d":
        o.analysis(w.xb, w.axb, xa_o, axa_o)
        errs = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
    else:
        cols = np.arange(0, cfg.num_lat * cfg.num_lon, 7, dtype=np.int32)
        o.analysis_cols(w.xb, w.axb, xa_o, axa_o, cols)
        errs = _increment_rel_rms_cols(cfg, w, (xa, axa), (xa_o, axa_o), cols)
    assert max(errs.values()) <= TOL_INCREMENT, errs
    ctx.letkf_final()


def test_core_batch_tf32_against_fp64_and_bf16():
    """The TF32 hi/lo Gram (LG_PREC_MIXED_TF32, the FP32 variant) keeps about
    2^-21 of each operand against the BF16 split's 2^-16.  Both accumulate in
    FP32, whose rounding (about sqrt(p) 2^-24 of the sums) bounds both once p
    reaches thousands; so the TF32 results meet the BF16 bounds everywhere and
    are clearly closer to FP64 where the operand split dominates (p ~ 300)."""
    import ctypes as C
    import torch
    import letkf_gb300 as lg
    from oracle import oracle as orc

    rng = np.random.default_rng(23)
    L = lg.load_library()
    ptr = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    dev = torch.device("cuda")
    for k, p in [(16, 5), (40, 300), (64, 2000), (64, 0)]:
        hx = rng.standard_normal((p, k))
        hx -= hx.mean(axis=1, keepdims=True)
        rd = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
        dep = rng.standard_normal(p)
        rloc = rng.uniform(0.0, 1.0, p)
        trans_o, wbar_o = orc.core(hx, rd, dep, rloc, 1.05)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
        d = [t(hx), t(rd), t(dep), t(rloc)]
        d_n = torch.tensor([p], dtype=torch.int32, device=dev)
        d_off = torch.tensor([0], dtype=torch.int64, device=dev)
        rel = {}
        for prec in (lg.LG_PREC_MIXED, lg.LG_PREC_MIXED_TF32):
            d_tr = torch.zeros((k, k), dtype=torch.float64, device=dev)
            d_wb = torch.zeros(k, dtype=torch.float64, device=dev)
            st = L.lg_core_batch(k, 1, ptr(d_n), ptr(d_off), *[ptr(x) for x in d], 1.05, prec,
                                 ptr(d_tr), ptr(d_wb), None)
            assert st == 0
            torch.cuda.synchronize()
            tr, wb = d_tr.cpu().numpy(), d_wb.cpu().numpy()
            rel[prec] = (np.linalg.norm(tr - trans_o) / np.linalg.norm(trans_o),
                         np.linalg.norm(wb - wbar_o) / max(np.linalg.norm(wbar_o), 1e-300))
        r16, r32 = rel[lg.LG_PREC_MIXED], rel[lg.LG_PREC_MIXED_TF32]
        assert r32[0] < 5e-5 and (p == 0 or r32[1] < 1e-4), (k, p, r32)
        if 0 < p <= 300:
            assert r32[0] < r16[0] / 2, (k, p, r16, r32)
    # the TF32 Gram holds every member's hi and lo parts in one 128-row operand
    d0 = torch.zeros(1, dtype=torch.int32, device=dev)
    assert L.lg_core_batch(128, 1, ptr(d0), ptr(d0), None, None, None, None, 1.05,
                           lg.LG_PREC_MIXED_TF32, ptr(d0), ptr(d0), None) == -3


def test_tf32_analysis_within_1e4():
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    base = lg.preset("small3d")
    w = synth.make_workload(base)
    o = orc.Oracle(base, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa_o, axa_o)
    errs = {}
    for prec in (lg.LG_PREC_MIXED, lg.LG_PREC_MIXED_TF32):
        cfg = base.replace(precision=prec)
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        assert ctx.stats()["n_gram_entries"] > 0
        ctx.letkf_final()
        errs[prec] = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
    e16, e32 = errs[lg.LG_PREC_MIXED], errs[lg.LG_PREC_MIXED_TF32]
    assert max(e32.values()) <= TOL_INCREMENT, e32
    assert max(e32.values()) <= 1.5 * max(e16.values()), (e16, e32)
    with pytest.raises(RuntimeError, match="LG_ERR_UNSUPPORTED"):
        lg.Letkf(base.replace(precision=lg.LG_PREC_MIXED_TF32, ens=128))


def test_mixed_gram_with_fp64_transform(monkeypatch):
    """The BF16 Gram with the vector transform in FP64 (LETKF_GB300_VEC64, the
    diagnostic that isolates the FP32 transform's share of the error): within
    the bar, and no farther from the oracle than the default FP32 transform
    plus a margin."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset("small3d").replace(precision=lg.LG_PREC_MIXED)
    w = synth.make_workload(cfg)
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa_o, axa_o)
    errs = {}
    for vec64 in (False, True):
        if vec64:
            monkeypatch.setenv("LETKF_GB300_VEC64", "1")
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        ctx.letkf_final()
        errs[vec64] = max(increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o)).values())
    assert errs[True] <= TOL_INCREMENT and errs[True] <= 1.5 * errs[False], errs


@pytest.mark.parametrize("name", ["small3d", "tiny2d"])
def test_tensor_core_gram_variants_agree(name, monkeypatch):
    """The column-group Gram (default), the per-solve streaming Gram and the
    per-solve compaction-queue Gram all meet the increment tolerance and agree
    with one another far inside it (tiny2d has no vertical localisation: one
    level per column)."""
    import letkf_gb300 as lg
    import synth
    from oracle import oracle as orc

    cfg = lg.preset(name).replace(precision=lg.LG_PREC_MIXED)
    w = synth.make_workload(cfg)
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa_o, axa_o)
    got = {}
    for kind in ("col", "lean", "stream", "queue"):
        monkeypatch.setenv("LETKF_GB300_GRAM", kind)
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        ctx.letkf_final()
        errs = increment_rel_rms(cfg, w, (xa, axa), (xa_o, axa_o))
        assert max(errs.values()) <= TOL_INCREMENT, (kind, errs)
        got[kind] = (xa, axa)
    for kind in ("lean", "stream", "queue"):
        errs = increment_rel_rms(cfg, w, got[kind], got["col"])
        assert max(errs.values()) <= 1e-5, (kind, errs)


def test_mixed_schedules_agree_bit_for_bit(monkeypatch):
    """With the Gram variant fixed, the solve schedule (one stream, alternating
    streams, three- and four-stage phase pipelines) does not change a
    mixed-precision analysis; 1 MiB chunks make every schedule reuse its
    buffer sets many times."""
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset("small3d").replace(precision=lg.LG_PREC_MIXED)
    w = synth.make_workload(cfg)
    monkeypatch.setenv("LETKF_GB300_GRAM", "lean")
    monkeypatch.setenv("LETKF_GB300_CHUNK_MB", "1")
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    ref = None
    for nl in (1, 2, 3, 4):
        ctx.set_tuning(solve_streams=nl)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        assert ctx.stats()["n_chunks"] > 4 * nl
        h = cfg.halo
        assert np.all(np.isfinite(xa[h:-h, h:-h])) and np.all(np.isfinite(axa[h:-h, h:-h])), nl
        if ref is None:
            ref = (xa, axa)
        else:
            assert np.array_equal(xa, ref[0]) and np.array_equal(axa, ref[1]), nl
    ctx.letkf_final()
