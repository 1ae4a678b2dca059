"""lg_core_batch_noalloc: the batched letkf_core for callers that cannot
allocate device memory (a host framework that owns the device heap through its
own pool, or a loop in which cudaMalloc's synchronisation is not acceptable).
It keeps its scratch in a fixed static device array, so two calls in a row
must give the same results as lg_core_batch, which allocates its own scratch,
and a batch larger than the array must be refused.

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LG_ERR_SHAPE = -2


def _lib():
    import letkf_gb300 as lg
    L = lg.load_library()
    L.lg_core_batch_noalloc.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 6 + [
        C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return lg, L


def _batch(rng, k, sizes):
    hx, rd, dep, rl = [], [], [], []
    for p in sizes:
        y = rng.standard_normal((p, k))
        hx.append(y - y.mean(axis=1, keepdims=True))
        rd.append((1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32))
        dep.append(rng.standard_normal(p))
        rl.append(rng.uniform(0.0, 1.0, p))
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    return (np.concatenate(hx), np.concatenate(rd), np.concatenate(dep), np.concatenate(rl),
            np.asarray(sizes, np.int32), off)


def _run(L, fn, k, arrays, precision, torch):
    hx, rd, dep, rl, n, off = arrays
    dev = torch.device("cuda")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    d = [t(hx), t(rd), t(dep), t(rl), t(n), t(off)]
    nb = len(n)
    tr = torch.zeros((nb, k, k), dtype=torch.float64, device=dev)
    wb = torch.zeros((nb, k), dtype=torch.float64, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())
    st = getattr(L, fn)(k, nb, P(d[4]), P(d[5]), P(d[0]), P(d[1]), P(d[2]), P(d[3]), 1.05,
                        precision, P(tr), P(wb), None)
    torch.cuda.synchronize()
    return st, tr.cpu().numpy(), wb.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_allocating_core_twice(precision):
    import torch
    lg, L = _lib()
    rng = np.random.default_rng(11)
    k = 64
    tol = 1e-12 if precision == 0 else 1e-6
    for sizes in ([300, 0, 7, 1200, 64], [50, 2000, 3, 400]):  # two calls in a row
        arrays = _batch(rng, k, sizes)
        st_a, tr_a, wb_a = _run(L, "lg_core_batch", k, arrays, precision, torch)
        st_b, tr_b, wb_b = _run(L, "lg_core_batch_noalloc", k, arrays, precision, torch)
        assert st_a == 0 and st_b == 0
        assert np.allclose(tr_b, tr_a, rtol=tol, atol=tol)
        assert np.allclose(wb_b, wb_a, rtol=tol, atol=tol)


def test_noalloc_rejects_batches_beyond_its_scratch():
    import torch
    lg, L = _lib()
    k = 64
    nb = 4096  # 4096 * (64*64 + 64) doubles > the 8 MiB array
    dev = torch.device("cuda")
    n = torch.zeros(nb, dtype=torch.int32, device=dev)
    off = torch.zeros(nb, dtype=torch.int64, device=dev)
    tr = torch.zeros((nb, k, k), dtype=torch.float64, device=dev)
    wb = torch.zeros((nb, k), dtype=torch.float64, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())
    st = L.lg_core_batch_noalloc(k, nb, P(n), P(off), None, None, None, None, 1.05, 0, P(tr),
                                 P(wb), None)
    assert st == LG_ERR_SHAPE
