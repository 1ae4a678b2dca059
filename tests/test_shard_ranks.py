"""Column shards over two processes on the CPU (gloo): the exchange step of a
sharded analysis (the role of comm_obs_data, x86/DA/LETKF/src/letkf_obs.F90:
251-466), with the oracle standing in for each process's GPU.

Each rank keeps only its own longitude slab of the background (its shard's
longitudes plus a one-longitude halo), computes H(x) of its own block copies,
all-gathers the packed H(x) rows with shard.gather_rows (the collective that
bench.py runs over NCCL) and imports the other ranks' rows.  The result must
be the one-rank H(x) of every entry, bit for bit, and the analysis of the
rank's own columns must equal the one-rank analysis of those columns.
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def own_slab(cfg, xb, axb, lon0, lon1):
    """The background a shard holds: longitudes [lon0, lon1) of the interior
    plus `halo` longitudes on each side (halo-extended indices lon0 ..
    lon1 + 2 halo - 1), every latitude; zero elsewhere."""
    h = cfg.halo
    xs, axs = np.zeros_like(xb), np.zeros_like(axb)
    xs[lon0:lon1 + 2 * h] = xb[lon0:lon1 + 2 * h]
    axs[lon0:lon1 + 2 * h] = axb[lon0:lon1 + 2 * h]
    return xs, axs


def _rank(rank, world, port, name, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as tdist

    import letkf_gb300 as lg
    import shard
    import synth
    from oracle import oracle as orc

    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg = lg.preset(name)
        w = synth.make_workload(cfg)
        # the one-rank analysis
        ref = orc.Oracle(cfg, w.obs)
        ref.hx(w.xb, w.axb, 1)
        rows_ref = ref.hx_rows(0, ref.n_entries)
        xa_r, axa_r = np.zeros_like(w.xb), np.zeros_like(w.axb)
        ref.analysis(w.xb, w.axb, xa_r, axa_r, 0, None, 1)
        # this rank's shard
        by0, by1 = shard.lon_block_ranges(cfg.global_ny, world)[rank]
        c0, c1 = shard.shard_columns(cfg, (by0, by1))
        lon0, lon1 = c0 // cfg.num_lat, c1 // cfg.num_lat
        o = orc.Oracle(cfg, w.obs)
        _, cb, ce = o.copy_layout()
        j0 = int(np.searchsorted(cb, by0 * cfg.global_nx))
        j1 = int(np.searchsorted(cb, by1 * cfg.global_nx))
        e0, e1 = int(ce[j0]), int(ce[j1])
        xb_s, axb_s = own_slab(cfg, w.xb, w.axb, lon0, lon1)
        o.hx_range(xb_s, axb_s, j0, j1, 1)
        mine = torch.from_numpy(o.hx_rows(e0, e1))
        parts = shard.gather_rows(mine, e0, e1)
        covered = np.zeros(o.n_entries, bool)
        for r, (a, b, part) in enumerate(parts):
            covered[a:b] = True
            if r != rank:
                o.set_hx_rows(part.numpy(), a, b)
        hx_same = bool(covered.all()) and np.array_equal(o.hx_rows(0, o.n_entries), rows_ref)
        lists_same = all(np.array_equal(o.column_list(col)[0], ref.column_list(col)[0])
                         for col in range(c0, c1, 7))
        xa, axa = np.zeros_like(w.xb), np.zeros_like(w.axb)
        o.analysis(xb_s, axb_s, xa, axa, c0, c1, 1)
        h = cfg.halo
        own = slice(lon0 + h, lon1 + h)
        xa_same = (np.array_equal(xa[own, h:-h], xa_r[own, h:-h])
                   and np.array_equal(axa[own, h:-h], axa_r[own, h:-h]))
        tdist.barrier()
        out.put((rank, (c0, c1), (e0, e1), hx_same, lists_same, xa_same))
    finally:
        tdist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("tiny3d", 2), ("tiny3d", 3), ("small3d", 2)])
def test_sharded_exchange_reproduces_one_rank_analysis(name, world):
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, name, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import letkf_gb300 as lg
    cfg = lg.preset(name)
    # the shards partition the columns and the entries
    cols = [r[1] for r in res]
    ents = [r[2] for r in res]
    assert cols[0][0] == 0 and cols[-1][1] == cfg.num_lat * cfg.num_lon
    assert all(cols[i][1] == cols[i + 1][0] for i in range(world - 1))
    assert all(ents[i][1] == ents[i + 1][0] for i in range(world - 1))
    for rank, _, _, hx_same, lists_same, xa_same in res:
        assert hx_same, f"rank {rank}: gathered H(x) differs from the one-rank H(x)"
        assert lists_same, f"rank {rank}: neighbour lists differ"
        assert xa_same, f"rank {rank}: analysis of its columns differs"


def test_lon_block_ranges_partition():
    import shard
    for ny in (1, 3, 8, 16):
        for world in range(1, ny + 1):
            rr = shard.lon_block_ranges(ny, world)
            assert rr[0][0] == 0 and rr[-1][1] == ny
            assert all(a < b for a, b in rr)
            assert all(rr[i][1] == rr[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in rr]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.lon_block_ranges(4, 5)
