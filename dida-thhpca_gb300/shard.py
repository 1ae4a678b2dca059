"""Column-sharded LETKF analysis: one process and one GPU per shard.

The reference analyses the globe on a 2-D grid of MPI ranks
(x86/DA/EnDNN/src/module_da_parallel.F90:75-109).  Each rank computes H(x) of
the observations in its own block, sends them to the neighbour blocks that
need them once per analysis (comm_obs_data, x86/DA/LETKF/src/letkf_obs.F90:
251-466), and then analyses its own columns with no further communication.

Here a shard is a range of longitude blocks of the same virtual decomposition
(so every shard owns whole latitude circles of columns, and its own
observation copies are one contiguous range of the copy order).  One step:

  1. lg_hx_device      H(x) of the shard's own block copies, from its own
                       columns of the background (and their halo);
  2. lg_hx_export      the own entries' rows, ens + 3 doubles each;
  3. all-gather        every shard's rows to every shard (one collective:
                       the exchange step; padded to the longest shard);
  4. lg_hx_import      the other shards' rows into the context;
  5. lg_analyse_device selection and solves of the shard's columns.

The collective goes through torch.distributed: NCCL between GPUs, gloo on
the CPU in tests.  Nothing else is exchanged; each shard writes only its own
columns of the analysis.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple


def lon_block_ranges(global_ny: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous, as-even-as-possible ranges of the global_ny longitude
    blocks, one per shard (the first global_ny % world shards get one more)."""
    if world < 1 or world > global_ny:
        raise ValueError(f"cannot split {global_ny} longitude blocks over {world} shards")
    base, rem = divmod(global_ny, world)
    out, s = [], 0
    for r in range(world):
        n = base + (1 if r < rem else 0)
        out.append((s, s + n))
        s += n
    return out


def gather_rows(rows, entry_begin: int, entry_end: int, group=None):
    """All-gather every shard's packed H(x) rows.  rows: (entry_end -
    entry_begin) x width tensor of this shard's entries.  Returns, for every
    shard r, (entry_begin_r, entry_end_r, rows_r)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    width = rows.shape[1]
    meta = torch.tensor([entry_begin, entry_end], dtype=torch.int64, device=rows.device)
    metas = [torch.zeros_like(meta) for _ in range(world)]
    dist.all_gather(metas, meta, group=group)
    ranges = [(int(m[0]), int(m[1])) for m in metas]
    nmax = max(1, max(e1 - e0 for e0, e1 in ranges))
    buf = torch.zeros((nmax, width), dtype=rows.dtype, device=rows.device)
    buf[:rows.shape[0]] = rows
    bufs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    return [(e0, e1, b[:e1 - e0]) for (e0, e1), b in zip(ranges, bufs)]


def exchange_hx(ctx, stream=None, group=None):
    """Steps 2-4: export this shard's H(x) rows, all-gather, import the
    others'.  ctx: a letkf_gb300.Letkf with its shard set and lg_hx_device
    done on the current CUDA stream (stream = its handle)."""
    import torch
    import torch.distributed as dist

    e0, e1, _ = ctx.shard_entries()
    dev = torch.device("cuda", torch.cuda.current_device())
    rows = torch.empty((max(0, e1 - e0), ctx.cfg.ens + 3), dtype=torch.float64, device=dev)
    if e1 > e0:
        ctx.hx_export(rows, stream)
    me = dist.get_rank(group)
    for r, (a, b, part) in enumerate(gather_rows(rows, e0, e1, group)):
        if r != me and b > a:
            ctx.hx_import(part.contiguous(), a, b, stream)


def sharded_step(ctx, xb, axb, xa, axa, stream=None, group=None):
    """One sharded analysis step (steps 1-5) on this process's shard."""
    ctx.hx_device(xb, axb, stream)
    exchange_hx(ctx, stream, group)
    ctx.analyse_device(xb, axb, xa, axa, stream)


def shard_columns(cfg, by_range: Sequence[int]) -> Tuple[int, int]:
    """Grid columns [c0, c1) of longitude blocks [by0, by1) (pro_info_get_indx
    with the reference's remainder rule: the first num_lon % global_ny blocks
    get one more longitude)."""
    y_sec, y_res = divmod(cfg.num_lon, cfg.global_ny)

    def lon_start(by):  # 0-based first longitude of block by
        return by * (y_sec + 1) if by < y_res else by * y_sec + y_res

    by0, by1 = by_range
    return lon_start(by0) * cfg.num_lat, lon_start(by1) * cfg.num_lat
