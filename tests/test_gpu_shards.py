"""Column windows and column shards through the C ABI on one GPU.

Shards: every shard's context computes H(x) of its own block copies from a
background that holds only its own longitudes (plus a one-longitude halo),
exports its H(x) rows, imports the other shards' rows and analyses its own
columns.  The shards' steps run one after another on the one GPU (no kernel
waits on another shard's kernels); the rows are handed over through device
tensors, as the all-gather of bench.py would.  Windows: lg_set_columns
analyses the globe in pieces.  Both must reproduce the whole-globe analysis
bit for bit, in both precisions, and leave the columns outside untouched.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(name, precision):
    import torch
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset(name).replace(precision=precision)
    dev = torch.device("cuda")
    w = synth.make_workload(cfg)
    xb = torch.as_tensor(np.ascontiguousarray(w.xb), device=dev)
    axb = torch.as_tensor(np.ascontiguousarray(w.axb), device=dev)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = torch.zeros_like(xb)
    axa = torch.zeros_like(axb)
    ctx.letkf_run_device(0, xb, axb, xa, axa)
    torch.cuda.synchronize()
    st = ctx.stats()
    ctx.letkf_final()
    return cfg, w, xb, axb, xa, axa, st


@pytest.mark.parametrize("name,world", [("small3d", 2), ("small3d", 4), ("tiny3d", 3)])
@pytest.mark.parametrize("precision", [0, 1])
def test_shards_reproduce_the_whole_globe(name, world, precision):
    import torch
    import letkf_gb300 as lg
    import shard

    cfg, w, xb, axb, xa_full, axa_full, st_full = _setup(name, precision)
    h = cfg.halo
    ranges = shard.lon_block_ranges(cfg.global_ny, world)
    ctxs, slabs, rows, ents = [], [], [], []
    for by0, by1 in ranges:
        c = lg.Letkf(cfg)
        c.set_obs(w.obs)
        c.set_shard(by0, by1)
        c0, c1 = shard.shard_columns(cfg, (by0, by1))
        lon0, lon1 = c0 // cfg.num_lat, c1 // cfg.num_lat
        xs = torch.zeros_like(xb)
        axs = torch.zeros_like(axb)
        xs[lon0:lon1 + 2 * h] = xb[lon0:lon1 + 2 * h]
        axs[lon0:lon1 + 2 * h] = axb[lon0:lon1 + 2 * h]
        c.hx_device(xs, axs)
        e0, e1, n = c.shard_entries()
        r = torch.empty((e1 - e0, cfg.ens + 3), dtype=torch.float64, device=xb.device)
        c.hx_export(r)
        torch.cuda.synchronize()
        ctxs.append(c)
        slabs.append((xs, axs, lon0, lon1))
        rows.append(r)
        ents.append((e0, e1))
    assert ents[0][0] == 0 and ents[-1][1] == n
    xa = torch.full_like(xb, 7.0)
    axa = torch.full_like(axb, 7.0)
    n_solves = 0
    for i, c in enumerate(ctxs):
        for j, (e0, e1) in enumerate(ents):
            if j != i and e1 > e0:
                c.hx_import(rows[j], e0, e1)
        xs, axs, lon0, lon1 = slabs[i]
        xa_s = torch.full_like(xb, 7.0)
        axa_s = torch.full_like(axb, 7.0)
        c.analyse_device(xs, axs, xa_s, axa_s)
        torch.cuda.synchronize()
        n_solves += c.stats()["n_solves"]
        own = slice(lon0 + h, lon1 + h)
        # nothing outside the shard's columns is written
        assert bool((xa_s[:lon0 + h] == 7.0).all()) and bool((xa_s[lon1 + h:] == 7.0).all())
        xa[own, h:-h] = xa_s[own, h:-h]
        axa[own, h:-h] = axa_s[own, h:-h]
        c.letkf_final()
    assert n_solves == st_full["n_solves"]
    assert torch.equal(xa[h:-h, h:-h], xa_full[h:-h, h:-h])
    assert torch.equal(axa[h:-h, h:-h], axa_full[h:-h, h:-h])


@pytest.mark.parametrize("precision", [0, 1])
def test_column_windows_reproduce_the_whole_globe(precision):
    import torch
    import letkf_gb300 as lg

    cfg, w, xb, axb, xa_full, axa_full, st_full = _setup("small3d", precision)
    ncol = cfg.num_lat * cfg.num_lon
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = torch.zeros_like(xb)
    axa = torch.zeros_like(axb)
    # uneven windows, one not aligned to whole longitudes
    edges = [0, 700, 701, 1500, ncol]
    total = 0
    for a, b in zip(edges[:-1], edges[1:]):
        ctx.set_columns(a, b)
        ctx.letkf_run_device(0, xb, axb, xa, axa)
        torch.cuda.synchronize()
        st = ctx.stats()
        assert st["n_columns"] == b - a
        total += st["nobsl_total"]
    assert total == st_full["nobsl_total"]
    h = cfg.halo
    assert torch.equal(xa[h:-h, h:-h], xa_full[h:-h, h:-h])
    assert torch.equal(axa[h:-h, h:-h], axa_full[h:-h, h:-h])
    # host arrays through lg_run: only the window's columns are written
    ctx.set_columns(100, 400)
    hxa = np.full(w.xb.shape, 3.0)
    haxa = np.full(w.axb.shape, 3.0)
    ctx.letkf_run(0, np.ascontiguousarray(w.xb), np.ascontiguousarray(w.axb), hxa, haxa)
    full = xa_full.cpu().numpy()
    for col in (99, 100, 399, 400):
        lon, lat = col // cfg.num_lat + h, col % cfg.num_lat + h
        if 100 <= col < 400:
            assert np.array_equal(hxa[lon, lat], full[lon, lat])
        else:
            assert (hxa[lon, lat] == 3.0).all()
    ctx.letkf_final()


def test_list_counts_and_windows_cover_the_globe():
    import torch
    import letkf_gb300 as lg

    cfg, w, xb, axb, xa_full, axa_full, st_full = _setup("small3d", 0)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    counts = ctx.list_counts()
    assert int(counts.sum()) == st_full["nobsl_total"]
    assert int(counts.max()) == st_full["nobsl_max"]
    budget = int(counts.sum()) // 5
    wins = ctx.windows(budget)
    assert len(wins) >= 5 and wins[0][0] == 0 and wins[-1][1] == cfg.num_lat * cfg.num_lon
    xa = torch.zeros_like(xb)
    axa = torch.zeros_like(axb)
    for a, b in wins:
        assert counts[a:b].sum() <= budget or b - a == cfg.num_lat
        ctx.set_columns(a, b)
        ctx.letkf_run_device(0, xb, axb, xa, axa)
    torch.cuda.synchronize()
    h = cfg.halo
    assert torch.equal(xa[h:-h, h:-h], xa_full[h:-h, h:-h])
    ctx.letkf_final()


def test_window_arguments_validated():
    import letkf_gb300 as lg
    cfg = lg.preset("tiny3d")
    ctx = lg.Letkf(cfg)
    ncol = cfg.num_lat * cfg.num_lon
    for a, b in ((-1, 5), (5, 5), (0, ncol + 1)):
        with pytest.raises(RuntimeError, match="LG_ERR_ARG"):
            ctx.set_columns(a, b)
    with pytest.raises(RuntimeError, match="LG_ERR_ARG"):
        ctx.set_shard(0, cfg.global_ny + 1)
    # run_da_parallel post-processes the whole globe: refused with a window set
    import synth
    w = synth.make_workload(cfg)
    ctx.set_obs(w.obs)
    ctx.set_columns(0, cfg.num_lat)
    full = np.ascontiguousarray(w.xb + w.axb[..., None])
    out = np.zeros_like(full)
    sp = np.zeros((cfg.num_lon, cfg.num_lat, cfg.n_rows))
    with pytest.raises(RuntimeError, match="LG_ERR_UNSUPPORTED"):
        ctx.run_da_parallel(0, 0.0, 1.0, 90.0, full, out, sp, sp.copy())
    ctx.letkf_final()
