"""Failure reporting of the GPU path, with every failure made on the host side
(no fault, trap or hang of the GPU is involved):

  * eigensolver non-convergence -- a QL sweep limit of one sweep per
    eigenvalue (LETKF_GB300_QL_ITERS) makes the tql2-style iteration stop
    unconverged; the batched core returns LG_ERR_EIG, an analysis is still
    written (the reference prints dsyevd's ierr and goes on) and lg_run
    returns LG_ERR_EIG with lg_stats.n_eig_fail counting the solves;
  * device allocation failure -- LETKF_GB300_ALLOC_LIMIT_MB makes every
    allocation above the limit fail as an out-of-memory cudaMalloc would;
    the call returns LG_ERR_NOMEM and the same context works once memory is
    available again;
  * the Fortran drop-in symbol letkf_core_ (all arguments by reference) gives
    the oracle's letkf_core results.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LG_ERR_EIG = -7
LG_ERR_NOMEM = -9


def _random_core_case(rng, k, p):
    hx = rng.standard_normal((p, k))
    hx -= hx.mean(axis=1, keepdims=True)
    rd = (1.0 / rng.uniform(0.5, 2.0, p) ** 2).astype(np.float32)
    dep = rng.standard_normal(p)
    rloc = rng.uniform(0.0, 1.0, p)
    return hx, rd, dep, rloc


def test_ql_sweep_limit_reports_eig_and_context_recovers(monkeypatch):
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset("tiny3d")
    w = synth.make_workload(cfg)
    # reference analysis with the normal sweep limit
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa_ref = np.zeros_like(w.xb)
    axa_ref = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa_ref, axa_ref)
    assert ctx.stats()["n_eig_fail"] == 0
    ctx.letkf_final()

    monkeypatch.setenv("LETKF_GB300_QL_ITERS", "1")
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    with pytest.raises(RuntimeError, match="LG_ERR_EIG"):
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    st = ctx.stats()
    assert 0 < st["n_eig_fail"] <= st["n_solves"]
    ctx.letkf_final()
    # the batched core reports it as its status
    rng = np.random.default_rng(5)
    hx, rd, dep, rloc = _random_core_case(rng, 40, 300)
    with pytest.raises(RuntimeError, match="LG_ERR_EIG"):
        lg.letkf_core(hx, rd, dep, rloc, 1.05)

    monkeypatch.delenv("LETKF_GB300_QL_ITERS")
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    assert ctx.stats()["n_eig_fail"] == 0
    assert np.array_equal(xa, xa_ref) and np.array_equal(axa, axa_ref)
    ctx.letkf_final()


def test_allocation_failure_reports_nomem_and_context_recovers(monkeypatch):
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset("small3d")
    w = synth.make_workload(cfg)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa_ref = np.zeros_like(w.xb)
    axa_ref = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa_ref, axa_ref)
    ctx.letkf_final()

    # the solve workspace of small3d (about 1 GiB of Gram matrices) cannot be had
    monkeypatch.setenv("LETKF_GB300_ALLOC_LIMIT_MB", "64")
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    with pytest.raises(RuntimeError, match="LG_ERR_NOMEM"):
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    monkeypatch.delenv("LETKF_GB300_ALLOC_LIMIT_MB")
    # same context, memory available again: a normal, identical analysis
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    assert np.array_equal(xa, xa_ref) and np.array_equal(axa, axa_ref)
    ctx.letkf_final()


def test_tensor_core_wait_limit_reports_timeout_and_context_recovers():
    """A wait limit of 1 ns makes the column Gram's first pipeline wait run
    out: its CTAs raise LG_ERR_TIMEOUT, wait (fully bounded) for their own MMAs
    and copies, free their tensor memory and return, and the analysis returns
    LG_ERR_TIMEOUT.  With the default limit back, the same context's next
    analysis equals a fresh context's bit for bit."""
    import letkf_gb300 as lg
    import synth

    cfg = lg.preset("small3d").replace(precision=lg.LG_PREC_MIXED, ens=64)
    w = synth.make_workload(cfg)
    ref = lg.Letkf(cfg)
    ref.set_obs(w.obs)
    xa_ref = np.zeros_like(w.xb)
    axa_ref = np.zeros_like(w.axb)
    ref.letkf_run(0, w.xb, w.axb, xa_ref, axa_ref)
    ref.letkf_final()

    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    ctx.set_tuning(gram_kernel=lg.LG_GRAM_COLUMN_LEAN)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.set_wait_limit(1)
    with pytest.raises(RuntimeError, match="LG_ERR_TIMEOUT"):
        ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    ctx.set_wait_limit(0)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    assert np.array_equal(xa, xa_ref) and np.array_equal(axa, axa_ref)
    ctx.letkf_final()


def test_alloc_limit_in_the_batched_core(monkeypatch):
    import torch
    import letkf_gb300 as lg

    L = lg.load_library()
    k, nb = 64, 512
    dev = torch.device("cuda")
    n = torch.zeros(nb, dtype=torch.int32, device=dev)
    off = torch.zeros(nb, dtype=torch.int64, device=dev)
    tr = torch.zeros((nb, k, k), dtype=torch.float64, device=dev)
    wb = torch.zeros((nb, k), dtype=torch.float64, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    monkeypatch.setenv("LETKF_GB300_ALLOC_LIMIT_MB", "1")  # the 16 MiB of Gram matrices fail
    st = L.lg_core_batch(k, nb, P(n), P(off), None, None, None, None, 1.05, 0, P(tr), P(wb), None)
    assert st == LG_ERR_NOMEM
    monkeypatch.delenv("LETKF_GB300_ALLOC_LIMIT_MB")
    st = L.lg_core_batch(k, nb, P(n), P(off), None, None, None, None, 1.05, 0, P(tr), P(wb), None)
    assert st == 0
    torch.cuda.synchronize()
    # p = 0 everywhere: trans = sqrt(rho) I, overline_w = 0
    eye = np.sqrt(1.05) * np.eye(k)
    assert np.allclose(tr.cpu().numpy(), eye[None], rtol=1e-14, atol=1e-14)
    assert not wb.cpu().numpy().any()


@pytest.mark.parametrize("k,p", [(16, 0), (40, 37), (64, 900)])
def test_fortran_symbol_by_reference_matches_oracle(k, p):
    """letkf_core_(nanals, nobsl, hxens, rdiaginv, dep, rloc, trans, overline_w,
    inflation_factor, pflag), every argument a pointer as an implicit-interface
    Fortran call passes it (letkf_compute.F90:105-111)."""
    import letkf_gb300 as lg
    from oracle import oracle as orc

    L = lg.load_library()
    P = C.POINTER
    L.letkf_core_.argtypes = [P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_float),
                              P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                              P(C.c_double), P(C.c_int)]
    L.letkf_core_.restype = None
    rng = np.random.default_rng(17 + k + p)
    hx, rd, dep, rloc = _random_core_case(rng, k, p)
    hx = np.ascontiguousarray(hx)
    trans = np.zeros((k, k))
    wbar = np.full(k, np.nan)
    nanals, nobsl, pflag = C.c_int(k), C.c_int(p), C.c_int(0)
    infl = C.c_double(1.05)
    ptr = lambda a, t: a.ctypes.data_as(P(t))  # noqa: E731
    L.letkf_core_(C.byref(nanals), C.byref(nobsl), ptr(hx, C.c_double), ptr(rd, C.c_float),
                  ptr(dep, C.c_double), ptr(rloc, C.c_double), ptr(trans, C.c_double),
                  ptr(wbar, C.c_double), C.byref(infl), C.byref(pflag))
    trans_o, wbar_o = orc.core(hx, rd, dep, rloc, 1.05)
    assert np.allclose(trans, trans_o, rtol=1e-11, atol=1e-11)
    assert np.allclose(wbar, wbar_o, rtol=1e-11, atol=1e-11)
