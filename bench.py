#!/usr/bin/env python
"""LETKF analysis benchmark on GB300: grid columns per second.

One "step" is one complete LETKF analysis (H(x) of every member, per-column
local observation search, one solve per column and level, Xa update) of the
synthetic workload named by --config (default cfg3: 360x180x32, ps/u/v/pt,
N=64, 1e6 observations, Gaspari-Cohn 800 km + 0.2 ln p, rho 1.05).

value : columns / (device time of one analysis) with the background already
        resident in HBM (lg_run_device), CUDA events on the launching stream.
e2e   : the same metric through the host-array call a DA driver makes
        (lg_set_obs + lg_run with pinned host buffers: observation ingest and the
        background H2D copy, analysis D2H copy inside the timed region).
e2e is the median over its steps.
contraction_variants : (mixed runs, N <= 64) the same workload with the Gram
        contractions as TF32 hi/lo tensor-core products (LG_PREC_MIXED_TF32, the
        FP32 variant) beside the timed BF16 hi/lo ones, each with its time and
        its increment error against plain FP64.
fp64  : (mixed runs) after the timed mixed analyses, the plain-FP64 GPU path on
        the same inputs: its time per analysis, the speed-up of the mixed path
        over it, and the mixed analysis' per-variable increment error against it
        (relative RMS over every interior point; the bar is 1e-4).
cpu_baseline / --impl reference : the CPU oracle (C restatement of the
        reference's Fortran hot path; the Fortran itself cannot be built here)
        on the host cores, over a bounded sample of columns spread over every
        latitude band and longitude sector, extrapolated.

Inputs (3.4 GB background for cfg3) exceed the 129 MB L2, so no flush is done
between steps.  For --gpus N > 1 (torchrun) the globe is column-sharded: rank
r analyses the columns of its range of longitude blocks (shard.py), each step
one all-gather of the shards' H(x) rows over NCCL (the observation exchange);
value is the globe's columns / the slowest rank's step time (strong scaling:
the total work is fixed).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "dida-thhpca_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "LETKF grid columns/s, mixed vs plain FP64 on one GB300 at <=1e-4 rel RMS"
UNIT = "columns/s"
# DRAM bytes (read + write) per solve of the solve-phase kernels, from a
# one-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the
# 180x90x32 / N=64 / 2.5e5-observation workload in 256 MiB chunks (8192
# solves per launch); the traffic grows in proportion to the solves.
PROFILED_DRAM_BYTES_PER_SOLVE = {
    "tridiag": 25.7e3,
    "gram": 29.3e3,
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg3")
    ap.add_argument("--ens", type=int, default=0, help="override the ensemble size")
    ap.add_argument("--precision", default=None, choices=[None, "fp64", "mixed", "tf32"])
    ap.add_argument("--no-tf32", action="store_true",
                    help="skip the TF32 (FP32-variant) Gram beside the BF16 one")
    ap.add_argument("--variant-steps", type=int, default=3,
                    help="timed analyses of the TF32 variant (after one untimed one)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the bounded oracle sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the plain-FP64 analysis of the same workload (mixed runs only)")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="timed plain-FP64 analyses after one untimed one")
    ap.add_argument("--list-gb", type=float, default=64.0,
                    help="device memory for neighbour lists; above it the globe is analysed "
                         "in column windows")
    ap.add_argument("--fresh-background", action="store_true",
                    help="a fresh seeded perturbation ensemble before every step (default "
                         "for cfg5, the ten-analysis cycle)")
    ap.add_argument("--tune", default="",
                    help="launch settings before timing, e.g. chunk_mb=2048,solve_streams=2")
    ap.add_argument("--autotune", action="store_true",
                    help="run lg_autotune on the workload (untimed) before the warm-up")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def job_rate(ms_local, ncol_total, world, device=None):
    """Whole-job columns/s: the columns all ranks analysed together over the
    slowest rank's step time (max over ranks when a process group is up)."""
    import torch
    ms = ms_local
    if world > 1:
        import torch.distributed as tdist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, ncol_total / (ms * 1e-3)


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def fp64_peak_tflops(torch, dev):
    """cuBLAS DGEMM throughput, the FP64 denominator for the FP64-bound kernels."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(3):
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def workload_config(cfg):
    """The `config` object of both arms' lines: the workload, by its shape."""
    return {"workload": f"{cfg.name}: {cfg.num_lon}x{cfg.num_lat}x{cfg.nz}, "
                        f"{'/'.join(cfg.var_names)}, N={cfg.ens}, {cfg.n_obs} obs"
                        + (f" ({int(100 * cfg.clustered_frac)}% clustered)"
                           if cfg.clustered_frac else "")
                        + f", L={cfg.local_dist:g} km, vert {cfg.vert_dist:g} ln p, "
                          f"rho={cfg.inflation}",
            "columns": cfg.num_lat * cfg.num_lon,
            "l2": "inputs larger than L2; no flush between steps"}


def spread_order(cfg, seed=0, n_bands=12, n_sectors=16):
    """All grid columns in an order whose every prefix is spread over the
    globe: rounds of one seeded random column from each of n_bands latitude
    bands x n_sectors longitude sectors, the cells of a round in random order.
    Column index c = lon * num_lat + lat (0-based)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    nl, nn = cfg.num_lat, cfg.num_lon
    lat_b = np.minimum(np.arange(nl) * n_bands // nl, n_bands - 1)
    lon_s = np.minimum(np.arange(nn) * n_sectors // nn, n_sectors - 1)
    cells = [[] for _ in range(n_bands * n_sectors)]
    for lo in range(nn):
        for la in range(nl):
            cells[lat_b[la] * n_sectors + lon_s[lo]].append(lo * nl + la)
    for c in cells:
        rng.shuffle(c)
    order = []
    rnd = 0
    while True:
        layer = [c[rnd] for c in cells if rnd < len(c)]
        if not layer:
            break
        rng.shuffle(layer)
        order.extend(layer)
        rnd += 1
    return np.asarray(order, np.int32)


def cpu_sample(cfg, obs, xb, axb, seconds, nthreads, seed=0):
    """Oracle timing on a bounded sample: H(x) of every observation, then
    columns in a globe-spread order (every latitude band and longitude sector)
    until ~seconds elapse; returns columns/s for a full analysis (H(x) + all
    columns at the sampled rate) and the sample's description."""
    import numpy as np
    from oracle import oracle as orc

    o = orc.Oracle(cfg, obs)
    t0 = time.perf_counter()
    o.hx(xb, axb, nthreads)
    t_hx = time.perf_counter() - t0
    ncol = cfg.num_lat * cfg.num_lon
    order = spread_order(cfg, seed)
    xa = np.zeros_like(xb)
    axa = np.zeros_like(axb)
    done, t_cols, chunk = 0, 0.0, max(2 * nthreads, 64)
    while (t_cols < seconds or done < 64) and done < ncol:
        cols = order[done:done + chunk]
        t0 = time.perf_counter()
        o.analysis_cols(xb, axb, xa, axa, cols, nthreads)
        t_cols += time.perf_counter() - t0
        done += cols.size
        rate = done / max(t_cols, 1e-6)
        chunk = int(min(4 * chunk, max(2 * nthreads, rate * (seconds - t_cols))))
        chunk = max(chunk, 2 * nthreads)
    t_full = t_hx + t_cols * ncol / done
    used = order[:done]
    lats = used % cfg.num_lat
    lons = used // cfg.num_lat
    info = {
        "sample": f"H(x) of all {obs.n_obs} obs ({t_hx:.2f} s) + {done} of {ncol} columns "
                  f"({t_cols:.2f} s; {np.unique(lons).size} longitudes, latitude rows "
                  f"{int(lats.min()) + 1}..{int(lats.max()) + 1} of {cfg.num_lat}), "
                  f"extrapolated to the full analysis",
        "sample_columns": int(done), "sample_seconds": round(t_cols, 3),
        "hx_seconds": round(t_hx, 3),
        "lapack": "OpenBLAS dgemm/dsyevd" if orc.lapack_loaded() else "built-in loops + Jacobi"}
    return ncol / t_full, info


def increment_rel_rms(cfg, xb, axb, got, ref, lons=None):
    """Per-variable relative RMS of the analysis-increment difference between
    two analyses (torch tensors in the lg_run layout, interior points, or the
    interior longitudes [lons[0], lons[1]) only): rms(inc_got - inc_ref) /
    rms(inc_ref), inc = xa + axa - (xb + axb).  A non-finite value anywhere
    makes the variable's entry inf."""
    import torch
    h = cfg.halo
    lon0, lon1 = lons if lons else (0, xb.shape[0] - 2 * h)
    out = {}
    r0 = 0
    for v, lv in zip(cfg.var_names, cfg.var_lev):
        sl = slice(r0, r0 + lv)
        num = torch.zeros((), dtype=torch.float64, device=xb.device)
        den = torch.zeros((), dtype=torch.float64, device=xb.device)
        finite = True
        for i0 in range(h + lon0, h + lon1, 64):
            j = slice(i0, min(i0 + 64, h + lon1))
            bg = xb[j, h:-h, sl] + axb[j, h:-h, sl, None]
            ig = got[0][j, h:-h, sl] + got[1][j, h:-h, sl, None] - bg
            io = ref[0][j, h:-h, sl] + ref[1][j, h:-h, sl, None] - bg
            finite = finite and bool(torch.isfinite(ig).all()) and bool(torch.isfinite(io).all())
            num += ((ig - io) ** 2).sum()
            den += (io ** 2).sum()
        val = float(torch.sqrt(num / den)) if finite and float(den) > 0 else float("inf")
        out[v] = val
        r0 += lv
    return out


def reference_arm(args):
    """--impl reference: the CPU oracle port on all host cores, same workload."""
    import numpy as np
    import letkf_gb300 as lg
    import synth

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = lg.preset(args.config)
    w = synth.make_workload(cfg)
    nthreads = os.cpu_count() or 1
    per_step = max(2.0, 120.0 / max(1, args.steps + args.warmup))
    vals = []
    info = {}
    xb_h, axb_h = np.ascontiguousarray(w.xb), np.ascontiguousarray(w.axb)
    step_s = []
    for i in range(args.warmup + args.steps):
        # each step its own globe-spread sample (seed = step index)
        t0 = time.perf_counter()
        v, info = cpu_sample(cfg, w.obs, xb_h, axb_h, per_step, nthreads, seed=i)
        if i >= args.warmup:
            vals.append(v)
            step_s.append(time.perf_counter() - t0)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        # a step is one bounded sample (its wall time); the full analysis at
        # the sampled rate is extrapolated separately
        "ms_per_step": 1e3 * statistics.median(step_s),
        "ms_per_full_analysis_extrapolated": 1e3 * cfg.num_lat * cfg.num_lon / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded spherical-harmonic ensemble, uniform observations)",
        "config": workload_config(cfg),
        "run": {"precision": "fp64 (the reference's own arithmetic)", "threads": nthreads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": info["sample"], "sample_columns": info["sample_columns"],
                         "sample_seconds": info["sample_seconds"],
                         "hx_seconds": info["hx_seconds"],
                         "extrapolated": "columns/s of a full analysis = columns / (H(x) time "
                                         "+ sample time x columns / sample columns)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C restatement of the reference's Fortran letkf_run (no Fortran compiler, MPI or "
                "Redis on this image); " + info["lapack"],
    }
    print(json.dumps(line), flush=True)


def rotate_perturbations(xb, seed):
    """A fresh perturbation ensemble from the current one: X <- X Q with Q a
    seeded random orthogonal matrix acting on the space orthogonal to the
    member-mean vector (Q 1 = 1).  The members stay zero-mean and their sample
    covariance is unchanged; every member becomes a new combination of the
    old ones.  In place, in slabs of longitudes (xb: lon, lat, rows, k)."""
    import numpy as np
    import torch
    k = xb.shape[-1]
    rng = np.random.default_rng(seed)
    g, _ = np.linalg.qr(rng.standard_normal((k - 1, k - 1)))
    # orthonormal basis of the complement of the ones vector (Helmert rows)
    basis = np.zeros((k, k - 1))
    for j in range(1, k):
        basis[:j, j - 1] = 1.0 / np.sqrt(j * (j + 1))
        basis[j, j - 1] = -j / np.sqrt(j * (j + 1))
    q = basis @ g @ basis.T + np.full((k, k), 1.0 / k)
    qt = torch.as_tensor(q, dtype=xb.dtype, device=xb.device)
    for i0 in range(0, xb.shape[0], 32):
        sl = xb[i0:i0 + 32]
        sl.copy_(torch.matmul(sl, qt))


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    import numpy as np
    import torch

    import letkf_gb300 as lg
    import synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import lg_build
    lg_build.build()

    cfg = lg.preset(args.config)
    if args.ens:
        cfg = cfg.replace(ens=args.ens)
    if args.precision:
        cfg = cfg.replace(precision={"mixed": lg.LG_PREC_MIXED, "tf32": lg.LG_PREC_MIXED_TF32,
                                     "fp64": lg.LG_PREC_FP64}[args.precision])
    w = synth.make_workload(cfg, backend="torch", device=dev)
    ncol = cfg.num_lat * cfg.num_lon
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xb, axb = w.xb.contiguous(), w.axb.contiguous()
    xa = torch.zeros_like(xb)
    axa = torch.zeros_like(axb)
    stream = torch.cuda.current_stream(dev)
    if args.tune:
        ctx.set_tuning(**{kv.split("=")[0]: int(kv.split("=")[1]) for kv in args.tune.split(",")})
    if args.autotune:
        ctx.autotune(xb, axb, xa, axa, stream.cuda_stream)
    tuning = ctx.tuning()
    if dist:
        import shard
        by_range = shard.lon_block_ranges(cfg.global_ny, world)[rank]
        ctx.set_shard(*by_range)
        shard_cols = shard.shard_columns(cfg, by_range)
    # column windows when the whole globe's neighbour lists (12 bytes an entry,
    # 28 with the mixed path's Gram records) exceed the list budget
    mixed = cfg.precision in (lg.LG_PREC_MIXED, lg.LG_PREC_MIXED_TF32)
    bytes_per_entry = 28 if mixed else 12
    windows = [(0, ncol)]
    if not dist:
        counts = ctx.list_counts()
        if int(counts.sum()) * bytes_per_entry > args.list_gb * 2 ** 30:
            windows = ctx.windows(int(args.list_gb * 2 ** 30 / bytes_per_entry))
    fresh = args.fresh_background or args.config == "cfg5"
    win_ms = [0.0] * len(windows)

    def step():
        """One analysis of the globe; returns the summed stats of its calls."""
        if dist:
            shard.sharded_step(ctx, xb, axb, xa, axa, stream.cuda_stream)
            return ctx.stats()
        if len(windows) == 1:
            ctx.letkf_run_device(0, xb, axb, xa, axa, stream.cuda_stream)
            return ctx.stats()
        tot = None
        for wi, (a, b) in enumerate(windows):
            ctx.set_columns(a, b)
            ctx.letkf_run_device(0, xb, axb, xa, axa, stream.cuda_stream)
            st_w = ctx.stats()
            win_ms[wi] = st_w["ms_total"]
            if tot is None:
                tot = dict(st_w)
            else:
                for key, v in st_w.items():
                    if key == "nobsl_max":
                        tot[key] = max(tot[key], v)
                    elif key not in ("n_copies", "n_entries"):
                        tot[key] += v
        return tot

    for _ in range(args.warmup):
        step()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    acc = {"ms_gram": 0.0, "ms_eig": 0.0, "ms_hx": 0.0, "ms_search": 0.0, "ms_tridiag": 0.0,
           "ms_ql": 0.0, "ms_vec": 0.0, "n_launches": 0, "n_gram_entries": 0, "n_chunks": 0}
    step_ms = []
    if fresh:
        # each step on a fresh seeded perturbation ensemble, drawn (untimed)
        # before the step's own events
        for i in range(args.steps):
            rotate_perturbations(xb, 1000 + i)
            torch.cuda.synchronize()
            e0.record(stream)
            st = step()
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            for key in acc:
                acc[key] += st[key]
        ms = sum(step_ms) / args.steps
    else:
        e0.record(stream)
        for _ in range(args.steps):
            st = step()
            for key in acc:
                acc[key] += st[key]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
    clocks = sampler.stop()
    ms, value = job_rate(ms, ncol, world, dev)
    # the analysis front of the last timed step: H(x), selection and Gram
    # records before the first chunk's Gram starts (the library's own events)
    front_ms = None
    if len(windows) == 1 and not dist:
        tl = ctx.timeline()
        if tl.size:
            front_ms = round(float(tl.reshape(-1, 7)[0, 0]), 2)
    # the timed configuration's analysis, kept for the comparison with plain FP64
    fp64_arm = mixed and not args.no_fp64 and world == 1
    if fp64_arm:
        xa_mixed, axa_mixed = xa.clone(), axa.clone()
    # the other tensor-core contraction on the same workload (BF16 hi/lo and
    # TF32 hi/lo, the FP32 variant, side by side), timed outside the main region
    variants = {}
    if (cfg.precision == lg.LG_PREC_MIXED and not args.no_tf32 and world == 1
            and len(windows) == 1 and cfg.ens <= 64):
        ctx_v = lg.Letkf(cfg.replace(precision=lg.LG_PREC_MIXED_TF32))
        ctx_v.set_obs(w.obs)
        xa_v, axa_v = torch.zeros_like(xa), torch.zeros_like(axa)
        ctx_v.letkf_run_device(0, xb, axb, xa_v, axa_v, stream.cuda_stream)
        torch.cuda.synchronize()
        v0 = torch.cuda.Event(enable_timing=True)
        v1 = torch.cuda.Event(enable_timing=True)
        v0.record(stream)
        for _ in range(args.variant_steps):
            ctx_v.letkf_run_device(0, xb, axb, xa_v, axa_v, stream.cuda_stream)
        v1.record(stream)
        torch.cuda.synchronize()
        ms_v = v0.elapsed_time(v1) / args.variant_steps
        st_v = ctx_v.stats()
        ctx_v.letkf_final()
        variants["tf32"] = {"ms_per_step": ms_v, "value": ncol / (ms_v * 1e-3),
                            "ms_gram_last": st_v["ms_gram"], "xa": (xa_v, axa_v)}
        # the BF16 Gram with the vector transform in FP64 (reflectors, rotation
        # log and Xb.W from the FP64 eigensolve): the FP32 transform's share of
        # the error and its time
        os.environ["LETKF_GB300_VEC64"] = "1"
        try:
            ctx_w = lg.Letkf(cfg)
        finally:
            del os.environ["LETKF_GB300_VEC64"]
        ctx_w.set_obs(w.obs)
        xa_w, axa_w = torch.zeros_like(xa), torch.zeros_like(axa)
        ctx_w.letkf_run_device(0, xb, axb, xa_w, axa_w, stream.cuda_stream)
        torch.cuda.synchronize()
        v0.record(stream)
        for _ in range(args.variant_steps):
            ctx_w.letkf_run_device(0, xb, axb, xa_w, axa_w, stream.cuda_stream)
        v1.record(stream)
        torch.cuda.synchronize()
        ms_w = v0.elapsed_time(v1) / args.variant_steps
        ctx_w.letkf_final()
        variants["bf16_fp64_transform"] = {"ms_per_step": ms_w, "value": ncol / (ms_w * 1e-3),
                                           "xa": (xa_w, axa_w)}
        variants["bf16"] = {"ms_per_step": ms, "value": value,
                            "xa": (xa_mixed, axa_mixed) if fp64_arm else None}

    # Per-kernel durations without overlap: one more analysis on a single solve
    # stream (outside the timed region) gives every kernel its own event time;
    # in the timed two-stream configuration the Gram of one chunk runs beside the
    # eigensolve of another, so per-phase stream times overlap.
    if len(windows) == 1:
        if tuning["solve_streams"] != 1:
            ctx.set_tuning(solve_streams=1)
            step()
        iso = step()
        torch.cuda.synchronize()
        if tuning["solve_streams"] != 1:
            ctx.set_tuning(solve_streams=tuning["solve_streams"])
    else:
        iso = dict(st)  # the last timed step's per-kernel sums (streams overlapping)
    if dist:
        iso["ms_hx"] = 0.0  # H(x) ran in its own call (lg_hx_device) before the exchange
    # the analysis is finite everywhere it writes (interior points)
    h = cfg.halo
    if not (bool(torch.isfinite(xa[h:-h, h:-h]).all()) and bool(torch.isfinite(axa[h:-h, h:-h]).all())):
        raise RuntimeError("non-finite analysis values")

    # roofline of the dominant kernel: algorithmic FLOPs of its launches in one
    # analysis over the sum of their event-timed durations
    peaks = measured_peaks()
    k = cfg.ens
    solves = iso["n_solves"]
    fp64_peak = fp64_peak_tflops(torch, dev)
    kernels = {
        # symmetric Gram p k (k+1) + Yb^T R^-1 d 2 p k, over the non-zero-weight
        # (entry, level) pairs: the flops the product needs, counting each
        # off-diagonal pair once (the FP64 kernel computes one triangle)
        "gram": {"ms": iso["ms_gram"], "bound": "tensor" if mixed else "fp64",
                 "flops": 1.0 * iso["n_gram_entries"] * k * (k + 1) + 2.0 * iso["n_gram_entries"] * k},
        # Householder tridiagonalisation of a symmetric k x k matrix: 4k^3/3
        "tridiag": {"ms": iso["ms_tridiag"], "bound": "fp64", "flops": solves * 4.0 * k ** 3 / 3.0},
        "ql": {"ms": iso["ms_ql"], "bound": "fp64", "flops": None},
        "vec_update": {"ms": iso["ms_vec"], "bound": "fp32" if mixed else "fp64", "flops": None},
        "search": {"ms": iso["ms_search"], "bound": "fp32/l2", "flops": None},
        "hx": {"ms": iso["ms_hx"], "bound": "hbm", "flops": None},
    }
    for name, kk in kernels.items():
        if kk["flops"] and kk["ms"] > 0:
            kk["achieved_tflops"] = kk["flops"] / (kk["ms"] * 1e-3) / 1e12
    dom_name = max((n for n in kernels if kernels[n]["flops"]), key=lambda n: kernels[n]["ms"])
    dom = kernels[dom_name]
    if dom["bound"] == "tensor":
        peak, peak_src = peaks.get("bf16_tflops", 1900.0), "bf16 burst, MEASURED_PEAKS.json"
    else:
        peak, peak_src = fp64_peak, "cuBLAS DGEMM measured in this run (FP64 is not in MEASURED_PEAKS.json)"
    achieved = dom.get("achieved_tflops", 0.0)
    launches_dom = max(1, iso["n_chunks"])
    traffic = None
    # the profiled figures are of the mixed path's kernels (column Gram, tridiag)
    if dom_name in PROFILED_DRAM_BYTES_PER_SOLVE and (mixed or dom_name != "gram"):
        traffic = PROFILED_DRAM_BYTES_PER_SOLVE[dom_name] * solves / launches_dom
    roofline = {"bound": dom["bound"], "kernel": dom_name, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak if peak else None, "traffic": traffic,
                "traffic_note": "DRAM bytes per launch: ncu per-solve figure (profiles/) x solves per launch",
                "peak_source": peak_src, "launches": launches_dom,
                "ms_per_launch": dom["ms"] / launches_dom,
                "share_of_single_stream_step": dom["ms"] / iso["ms_total"] if iso["ms_total"] else None}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak",
        "vs_baseline": None,
        "dtype": {lg.LG_PREC_MIXED: "bf16/f32 contractions, f64 eig",
                  lg.LG_PREC_MIXED_TF32: "tf32/f32 contractions, f64 eig",
                  lg.LG_PREC_FP64: "f64"}[cfg.precision],
        "data": "synthetic (seeded spherical-harmonic ensemble, %s observations)" % (
            "uniform" if not cfg.clustered_frac else
            f"{int(100 * cfg.clustered_frac)}% clustered + uniform"),
        "config": workload_config(cfg),
        "run": {"precision": {lg.LG_PREC_MIXED: "mixed", lg.LG_PREC_MIXED_TF32: "mixed-tf32",
                              lg.LG_PREC_FP64: "fp64"}[cfg.precision],
                   "solves_per_step": st["n_solves"],
                   "list_entries_per_step": st["nobsl_total"],
                   "gram_entries_per_step": iso["n_gram_entries"],
                   "l2": "inputs (background %.1f GB) larger than L2; no flush" % (
                       xb.numel() * 8 / 1e9),
                   "column_windows": len(windows),
                   "fresh_background": ("a fresh seeded perturbation ensemble before every "
                                        "step (random orthogonal rotation of the members' "
                                        "perturbations), untimed") if fresh else None,
                   "parallelism": (f"column shards over {world} GPUs (longitude blocks, one "
                                   f"H(x) all-gather per step)") if world > 1 else "single GPU",
                   "tuning": {kk: v for kk, v in tuning.items() if kk != "ms"}},
        "clocks": clocks,
        "gpu_launches": acc["n_launches"],
        "selection": {key: st[key] for key in ("nobsl_total", "nobsl_max", "n_capped", "n_band",
                                                "n_eig_fail", "n_copies", "n_entries")},
        "selection_note": "n_band: candidate pairs with |ri - 2| < 1e-12, where a 1-ulp libm "
                          "difference could flip a list decision; n_eig_fail: eigensolves "
                          "that hit the QL sweep limit",
        "front_ms": front_ms,
        "front_note": "ms from the analysis start to the first Gram (H(x) beside the "
                      "selection, then the Gram records), last timed step",
        "phases_ms": {n: round(v["ms"], 3) for n, v in kernels.items()},
        "phases_note": ("kernel event times of one single-stream analysis (no overlap)"
                        if len(windows) == 1 else
                        "kernel event times summed over the windows of the last timed step "
                        "(solve streams overlapping)"),
        "kernels": {n: {kk: v[kk] for kk in ("bound", "achieved_tflops") if kk in v}
                    for n, v in kernels.items()},
        "roofline": roofline,
        "fp64_peak_tflops": fp64_peak,
    }

    # end to end, sharded: each rank copies in its own background slab (its
    # longitudes and their halo) from page-locked host memory, runs the sharded
    # step and copies its columns of the analysis out
    if not args.no_e2e and dist:
        h = cfg.halo
        lon0, lon1 = shard_cols[0] // cfg.num_lat, shard_cols[1] // cfg.num_lat
        sl = slice(lon0, lon1 + 2 * h)
        own = slice(lon0 + h, lon1 + h)
        hxb = torch.empty(xb[sl].shape, dtype=torch.float64, pin_memory=True)
        haxb = torch.empty(axb[sl].shape, dtype=torch.float64, pin_memory=True)
        hxa = torch.empty(xa[own].shape, dtype=torch.float64, pin_memory=True)
        haxa = torch.empty(axa[own].shape, dtype=torch.float64, pin_memory=True)
        hxb.copy_(xb[sl])
        haxb.copy_(axb[sl])
        ts = []
        for _ in range(args.e2e_steps):
            tdist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            xb[sl].copy_(hxb, non_blocking=True)
            axb[sl].copy_(haxb, non_blocking=True)
            step()
            hxa.copy_(xa[own], non_blocking=True)
            haxa.copy_(axa[own], non_blocking=True)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        ms_e, val_e = job_rate(1e3 * statistics.median(ts), ncol, world, dev)
        line["e2e"] = {"value": val_e, "unit": UNIT,
                       "h2d_bytes_per_step": int(hxb.nbytes + haxb.nbytes),
                       "d2h_bytes_per_step": int(hxa.nbytes + haxa.nbytes),
                       "steps": len(ts), "statistic": "median over the e2e steps, max over ranks",
                       "per_rank": "bytes of rank 0's slab and columns"}

    # end to end through the host-array C ABI call
    if not args.no_e2e and rank == 0 and not dist:
        hxb = torch.empty(xb.shape, dtype=torch.float64, pin_memory=True)
        haxb = torch.empty(axb.shape, dtype=torch.float64, pin_memory=True)
        hxa = torch.zeros(xb.shape, dtype=torch.float64, pin_memory=True)
        haxa = torch.zeros(axb.shape, dtype=torch.float64, pin_memory=True)
        hxb.copy_(xb)
        haxb.copy_(axb)
        nxb, naxb, nxa, naxa = (t.numpy() for t in (hxb, haxb, hxa, haxa))
        ctx.set_obs(w.obs)
        ctx.letkf_run(0, nxb, naxb, nxa, naxa)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xb.copy_(hxb, non_blocking=True)
        torch.cuda.synchronize()
        print("e2e host buffers: pinned H2D %.1f GB/s" % (hxb.numel() * 8 / (time.perf_counter() - t0) / 1e9),
              file=sys.stderr)
        ts = []
        for _ in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.set_obs(w.obs)
            t1 = time.perf_counter()
            ctx.letkf_run(0, nxb, naxb, nxa, naxa)
            ts.append(time.perf_counter() - t0)
            st_e = ctx.stats()
            print("e2e step: lg_set_obs %.1f ms, lg_run %.1f ms (copy in %.1f ms, device analysis "
                  "%.1f ms, copy out %.1f ms)" % (1e3 * (t1 - t0), 1e3 * (ts[-1] - (t1 - t0)),
                                                 st_e["ms_h2d"], st_e["ms_total"], st_e["ms_d2h"]),
                  file=sys.stderr)
        o = w.obs
        h2d = nxb.nbytes + naxb.nbytes + sum(a.nbytes for a in (o.type, o.lat, o.lon, o.ph, o.yo, o.rinv))
        h = cfg.halo
        d2h = (nxa[h:-h, h:-h].nbytes + naxa[h:-h, h:-h].nbytes)
        line["e2e"] = {"value": ncol / statistics.median(ts), "unit": UNIT,
                       "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                       "steps": len(ts), "ms_per_step": [round(1e3 * t, 1) for t in ts],
                       "statistic": "median over the e2e steps"}

    if fp64_arm and rank == 0:
        # The same workload through the plain-FP64 path (FP64 Gram, FP64
        # eigensolve and transform): its time per analysis, and the mixed
        # analysis' per-variable increment error against it over every
        # interior point.  Outside the mixed timed region.
        ctx.letkf_final()
        ctx64 = lg.Letkf(cfg.replace(precision=lg.LG_PREC_FP64))
        ctx64.set_obs(w.obs)
        # with column windows: the middle window only (whole longitudes), and
        # the mixed path's time of that window in the last timed step
        wa, wb = windows[len(windows) // 2]
        lons = (wa // cfg.num_lat, wb // cfg.num_lat)
        if len(windows) > 1:
            ctx64.set_columns(wa, wb)
        ctx64.letkf_run_device(0, xb, axb, xa, axa, stream.cuda_stream)  # untimed
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.fp64_steps):
            ctx64.letkf_run_device(0, xb, axb, xa, axa, stream.cuda_stream)
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1) / args.fp64_steps
        st64 = ctx64.stats()
        ms_mixed = ms if len(windows) == 1 else win_ms[len(windows) // 2]
        errs = increment_rel_rms(cfg, xb, axb, (xa_mixed, axa_mixed), (xa, axa),
                                 None if len(windows) == 1 else lons)
        for vd in variants.values():
            if vd.get("xa") is not None:
                ev = increment_rel_rms(cfg, xb, axb, vd["xa"], (xa, axa))
                vd["increment_rel_rms"] = ev
                vd["increment_rel_rms_max"] = max(ev.values())
                vd["speedup_vs_fp64"] = ms64 / vd["ms_per_step"]
        line["fp64"] = {
            "ms_per_step": ms64, "steps": args.fp64_steps, "value": (wb - wa) / (ms64 * 1e-3),
            "columns": wb - wa, "mixed_ms_same_columns": ms_mixed,
            "speedup_vs_fp64": ms64 / ms_mixed,
            "increment_rel_rms": errs,
            "increment_rel_rms_max": max(errs.values()),
            "tolerance": 1e-4,
            "within_tolerance": max(errs.values()) <= 1e-4,
            "ms_gram": st64["ms_gram"], "ms_total_last": st64["ms_total"],
            "selection": {key: st64[key] for key in ("nobsl_total", "nobsl_max", "n_band",
                                                      "n_eig_fail")},
            "note": ("plain FP64 GPU path on the same inputs; increment = xa + axa - (xb + axb), "
                     "rel RMS of (mixed - FP64) per variable over all interior points"
                     + ("" if len(windows) == 1 else
                        f" of the window of columns [{wa}, {wb}) (longitudes {lons[0]}.."
                        f"{lons[1] - 1}); speed-up against the mixed time of that window")),
        }
        ctx64.letkf_final()
        ctx = None

    if not args.no_cpu_baseline and rank == 0 and not dist:
        xb_h = xb.cpu().numpy()
        axb_h = axb.cpu().numpy()
        nthreads = os.cpu_count() or 1
        v, info = cpu_sample(cfg, w.obs, xb_h, axb_h, args.cpu_seconds, nthreads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                                "sample": info["sample"] + "; " + info["lapack"]}
    if variants:
        line["contraction_variants"] = {
            name: {kk: v for kk, v in vd.items() if kk != "xa"} for name, vd in variants.items()}
        line["contraction_variants_note"] = (
            "the Gram contractions as BF16 hi/lo (the timed value) and as TF32 hi/lo tensor-core "
            "products (the FP32 variant), and the BF16 Gram with the vector transform (Xb.W, "
            "w-bar) in FP64 instead of FP32; same workload; errors against the plain-FP64 "
            "analysis")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ctx is not None:
        ctx.letkf_final()
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
