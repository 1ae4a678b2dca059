"""GPU tests of the launch-shape settings and the autotuner (lg_set_tuning,
lg_autotune): settings are validated, no setting changes an FP64 analysis by a
single bit, and the autotuned mixed-precision analysis stays within the
increment tolerance of the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _workload(name, **over):
    import letkf_gb300 as lg
    import synth
    cfg = lg.preset(name).replace(**over)
    return cfg, synth.make_workload(cfg)


def _device_run(ctx, w):
    import torch
    dev = torch.device("cuda")
    xb = torch.as_tensor(w.xb, device=dev)
    axb = torch.as_tensor(w.axb, device=dev)
    xa = torch.zeros_like(xb)
    axa = torch.zeros_like(axb)
    return xb, axb, xa, axa


def test_set_tuning_validates_and_round_trips():
    import letkf_gb300 as lg
    cfg, w = _workload("tiny3d")
    ctx = lg.Letkf(cfg)
    t = ctx.tuning()
    assert t["chunk_mb"] >= 16 and t["ql_warps"] >= 1 and t["vec_warps"] >= 1
    ctx.set_tuning(chunk_mb=64, ql_warps=2, vec_warps=8, lnp_buckets=32)
    t2 = ctx.tuning()
    assert (t2["chunk_mb"], t2["ql_warps"], t2["vec_warps"], t2["lnp_buckets"]) == (64, 2, 8, 32)
    for bad in ({"chunk_mb": 1}, {"ql_warps": 0}, {"ql_warps": 7}, {"vec_warps": 9},
                {"lnp_buckets": 4}, {"gram_kernel": 9}, {"solve_streams": 5}, {"gram_ctas": -1}):
        with pytest.raises(RuntimeError, match="LG_ERR_ARG"):
            ctx.set_tuning(**bad)
    ctx.letkf_final()


def test_fp64_analysis_is_bit_identical_under_every_setting(monkeypatch):
    import letkf_gb300 as lg
    cfg, w = _workload("tiny3d")
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    ref = None
    # "mb1": 1 MiB chunks (LETKF_GB300_CHUNK_MB), 11 chunks of 64 columns, so
    # every schedule reuses its buffer sets
    for kw in ({}, {"chunk_mb": 16}, {"ql_warps": 4, "vec_warps": 2}, {"vec_warps": 8},
               {"solve_streams": 2, "chunk_mb": 16}, {"solve_streams": 3, "chunk_mb": 16},
               {"solve_streams": 4, "chunk_mb": 16}, {"solve_streams": 2, "mb1": 1},
               {"solve_streams": 3, "mb1": 1}, {"solve_streams": 4, "mb1": 1},
               {"solve_streams": 1}):
        kw = dict(kw)
        if kw.pop("mb1", 0):
            monkeypatch.setenv("LETKF_GB300_CHUNK_MB", "1")
        else:
            monkeypatch.delenv("LETKF_GB300_CHUNK_MB", raising=False)
        ctx.set_tuning(**kw)
        xa = np.zeros_like(w.xb)
        axa = np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        st = ctx.stats()
        assert st["ms_h2d"] > 0.0 and st["ms_d2h"] > 0.0  # host-array run: copies timed
        tl = ctx.timeline()
        assert tl.shape == (st["n_chunks"], 7) and tl.shape[0] >= 1
        eps = 1e-3  # event timestamps are ms floats
        for a, b in ((0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (5, 6)):
            assert np.all(tl[:, b] >= tl[:, a] - eps), (kw, a, b, tl)
        if ref is None:
            ref = (xa, axa)
        else:
            assert np.array_equal(xa, ref[0]) and np.array_equal(axa, ref[1]), kw
    ctx.letkf_final()


def test_autotune_mixed_keeps_the_increment_within_tolerance():
    import letkf_gb300 as lg
    from oracle import oracle as orc
    from test_gpu_mixed import TOL_INCREMENT, increment_rel_rms
    cfg, w = _workload("small3d", precision=lg.LG_PREC_MIXED)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xb, axb, xa, axa = _device_run(ctx, w)
    best = ctx.autotune(xb, axb, xa, axa)
    assert best["ms"] > 0.0
    assert best["gram_kernel"] in (lg.LG_GRAM_COLUMN, lg.LG_GRAM_COLUMN_LEAN, lg.LG_GRAM_STREAM,
                                   lg.LG_GRAM_QUEUE)
    assert ctx.tuning()["chunk_mb"] == best["chunk_mb"]
    ctx.letkf_run_device(0, xb, axb, xa, axa)
    import torch
    torch.cuda.synchronize()
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa_o = np.zeros_like(w.xb)
    axa_o = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa_o, axa_o)
    errs = increment_rel_rms(cfg, w, (xa.cpu().numpy(), axa.cpu().numpy()), (xa_o, axa_o))
    assert max(errs.values()) <= TOL_INCREMENT, (best, errs)
    ctx.letkf_final()


@pytest.mark.parametrize("mb1,engine", [(False, False), (True, False), (False, True)])
def test_host_run_pinned_overlapped_copies_match_pageable(mb1, engine, monkeypatch):
    """lg_run with page-locked host arrays copies the background in beside the
    selection (by a copy kernel reading the mapped host memory, or with
    LETKF_GB300_COPY_ENGINE by the copy engine) and each chunk's columns out
    beside the later chunks; the result is bit-identical to the pageable-array
    path (copies before and after), and the halo of the host arrays is left
    untouched.  1 MiB chunks split longitude rows, exercising the partial-row
    copies."""
    import torch

    import letkf_gb300 as lg
    if mb1:
        monkeypatch.setenv("LETKF_GB300_CHUNK_MB", "1")
    if engine:
        monkeypatch.setenv("LETKF_GB300_COPY_ENGINE", "1")
    for prec in (lg.LG_PREC_FP64, lg.LG_PREC_MIXED):
        cfg, w = _workload("tiny3d", precision=prec)
        ctx = lg.Letkf(cfg)
        ctx.set_obs(w.obs)
        xa = np.full_like(w.xb, 7.0)
        axa = np.full_like(w.axb, 7.0)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        assert ctx.stats()["n_chunks"] > (5 if mb1 else 0)
        pin = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True) for a in (w.xb, w.axb)]
        pin[0].copy_(torch.from_numpy(w.xb))
        pin[1].copy_(torch.from_numpy(w.axb))
        out = [torch.full(a.shape, 7.0, dtype=torch.float64).pin_memory() for a in (w.xb, w.axb)]
        pxb, paxb, pxa, paxa = (t.numpy() for t in pin + out)
        for _ in range(2):  # capture, then graph replay
            ctx.letkf_run(0, pxb, paxb, pxa, paxa)
            st = ctx.stats()
            assert st["ms_h2d"] > 0.0 and st["ms_d2h"] > 0.0
            assert np.array_equal(pxa, xa) and np.array_equal(paxa, axa), prec
        h = cfg.halo
        assert np.all(pxa[:h] == 7.0) and np.all(paxa[:, :h] == 7.0)
        ctx.letkf_final()


def test_pinned_arrays_off_16_byte_alignment_use_the_copy_engine():
    """Page-locked host arrays whose address is not a multiple of 16 bytes
    cannot be read by the 16-byte loads of the copy kernel: lg_run copies them
    with the copy engine instead, with the same result."""
    import torch

    import letkf_gb300 as lg
    cfg, w = _workload("tiny3d", precision=lg.LG_PREC_MIXED)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)

    def pinned_off8(a):
        buf = torch.empty(a.size + 1, dtype=torch.float64, pin_memory=True)
        v = buf.numpy()[1:].reshape(a.shape)  # 8 bytes past a 16-byte boundary
        assert v.ctypes.data % 16 == 8
        v[...] = a
        return v

    pxb, paxb = pinned_off8(w.xb), pinned_off8(w.axb)
    pxa, paxa = pinned_off8(np.zeros_like(w.xb)), pinned_off8(np.zeros_like(w.axb))
    ctx.letkf_run(0, pxb, paxb, pxa, paxa)
    h = cfg.halo
    assert np.array_equal(pxa[h:-h, h:-h], xa[h:-h, h:-h])
    assert np.array_equal(paxa[h:-h, h:-h], axa[h:-h, h:-h])
    ctx.letkf_final()


def test_observation_sets_of_changing_size_reuse_buffers():
    """One context through a small, a larger and the small observation set
    again (buffers kept across sets, grown when outgrown) gives the same
    analyses as fresh contexts."""
    import letkf_gb300 as lg
    import synth
    small = lg.preset("tiny3d")
    big = small.replace(n_obs=3 * small.n_obs, seed=5)
    ws, wb = synth.make_workload(small), synth.make_workload(big)

    def fresh(cfg, w):
        c = lg.Letkf(cfg)
        c.set_obs(w.obs)
        xa, axa = np.zeros_like(w.xb), np.zeros_like(w.axb)
        c.letkf_run(0, w.xb, w.axb, xa, axa)
        c.letkf_final()
        return xa, axa

    ref_s, ref_b = fresh(small, ws), fresh(big, wb)
    ctx = lg.Letkf(small)
    for w, ref in ((ws, ref_s), (wb, ref_b), (ws, ref_s)):
        ctx.set_obs(w.obs)
        xa, axa = np.zeros_like(w.xb), np.zeros_like(w.axb)
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
        assert np.array_equal(xa, ref[0]) and np.array_equal(axa, ref[1])
    ctx.letkf_final()


def test_observation_ingest_is_independent_of_host_threads(monkeypatch):
    """lg_set_obs's host passes (block assignment of the observations, cell
    index of every block segment) on 1 and on 5 host threads give the same
    copy layout, selection lists and analysis, bit for bit."""
    import letkf_gb300 as lg
    import synth
    cfg = lg.preset("tiny3d").replace(n_obs=2000, seed=11)
    w = synth.make_workload(cfg)
    out = []
    for nt in ("1", "5"):
        monkeypatch.setenv("LETKF_GB300_HOST_THREADS", nt)
        c = lg.Letkf(cfg)
        c.set_obs(w.obs)
        xa, axa = np.zeros_like(w.xb), np.zeros_like(w.axb)
        c.letkf_run(0, w.xb, w.axb, xa, axa)
        out.append((c.copy_layout(), c.lists(), xa, axa))
        c.letkf_final()
    (lay1, lst1, xa1, axa1), (lay5, lst5, xa5, axa5) = out
    assert all(np.array_equal(a, b) for a, b in zip(lay1, lay5))
    assert all(np.array_equal(a, b) for a, b in zip(lst1, lst5))
    assert np.array_equal(xa1, xa5) and np.array_equal(axa1, axa5)
