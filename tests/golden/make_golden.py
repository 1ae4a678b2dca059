"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

The reference itself cannot be run here (Fortran, MPI and a Redis cluster are
absent), so these vectors pin the oracle's own outputs on the seeded synthetic
workloads: they guard the oracle against regressions (tests/test_golden.py) and
give the GPU tests a committed target besides the live oracle.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "dida-thhpca_gb300"))

import letkf_gb300 as lg  # noqa: E402
import synth  # noqa: E402
from oracle import oracle as orc  # noqa: E402

CASES = ("tiny2d", "tiny3d")
XA_COLUMNS = (0, 7, 300, 647)


def input_digest(w):
    return np.array([w.xb.sum(), (w.xb ** 2).sum(), w.axb.sum(), w.obs.yo.sum(),
                     w.obs.lat.sum(), w.obs.lon.sum()])


def run_case(name):
    cfg = lg.preset(name)
    w = synth.make_workload(cfg)
    o = orc.Oracle(cfg, w.obs)
    o.hx(w.xb, w.axb)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    o.analysis(w.xb, w.axb, xa, axa)
    ncol = cfg.num_lat * cfg.num_lon
    counts = np.zeros(ncol, np.int32)
    ents, rlocs = [], []
    for c in range(ncol):
        e, r = o.column_list(c)
        counts[c] = e.size
        ents.append(e)
        rlocs.append(r)
    h = cfg.halo
    cols = []
    for c in XA_COLUMNS:
        glat, glon = c % cfg.num_lat, c // cfg.num_lat
        cols.append(xa[glon + h, glat + h])
    return dict(digest=input_digest(w), counts=counts, entries=np.concatenate(ents),
                rloc=np.concatenate(rlocs), axa=axa[h:-h, h:-h].copy(),
                xa_columns=np.stack(cols), xa_column_ids=np.array(XA_COLUMNS))


def main():
    for name in CASES:
        out = run_case(name)
        path = os.path.join(HERE, f"{name}_oracle.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
