"""Golden fixtures (tests/golden/*_oracle.npz, made by tests/golden/make_golden.py):
the oracle must reproduce them on CPU, and the GPU path must match them on GPU."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("tiny2d", "tiny3d")


def _load(name):
    return dict(np.load(os.path.join(HERE, "golden", f"{name}_oracle.npz")))


def _workload(name):
    import letkf_gb300 as lg
    import synth
    cfg = lg.preset(name)
    return cfg, synth.make_workload(cfg)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    from golden.make_golden import run_case
    gold = _load(name)
    got = run_case(name)
    np.testing.assert_allclose(got["digest"], gold["digest"], rtol=1e-12)
    assert np.array_equal(got["counts"], gold["counts"])
    assert np.array_equal(got["entries"], gold["entries"])
    np.testing.assert_allclose(got["rloc"], gold["rloc"], rtol=0, atol=1e-13)
    scale = np.abs(gold["axa"]).max()
    np.testing.assert_allclose(got["axa"], gold["axa"], rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(got["xa_columns"], gold["xa_columns"], rtol=0,
                               atol=1e-11 * np.abs(gold["xa_columns"]).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(name):
    import letkf_gb300 as lg
    gold = _load(name)
    cfg, w = _workload(name)
    ctx = lg.Letkf(cfg)
    ctx.set_obs(w.obs)
    xa = np.zeros_like(w.xb)
    axa = np.zeros_like(w.axb)
    ctx.letkf_run(0, w.xb, w.axb, xa, axa)
    counts, ent, rloc = ctx.lists()
    assert np.array_equal(counts, gold["counts"])
    assert np.array_equal(ent, gold["entries"])
    np.testing.assert_allclose(rloc, gold["rloc"], rtol=0, atol=1e-13)
    h = cfg.halo
    inc = np.abs(gold["axa"] - w.axb[h:-h, h:-h]).max()
    assert np.abs(axa[h:-h, h:-h] - gold["axa"]).max() <= 1e-10 * inc
    for c, col in zip(gold["xa_column_ids"], gold["xa_columns"]):
        glat, glon = c % cfg.num_lat, c // cfg.num_lat
        assert np.abs(xa[glon + h, glat + h] - col).max() <= 1e-10 * max(inc, np.abs(col).max())
    ctx.letkf_final()
