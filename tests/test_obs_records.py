"""Observation ingest from the Redis store's record layout (lg_obs_from_records,
host only): records reshaped as read_obs does (read_obs_mod.F90:338-449),
checked against a float32 numpy restatement of that routine."""
import numpy as np
import pytest


def _read_obs(nz, nvar, lon, lat, lev, val, noise):
    """read_obs's reshaping in REAL(4): profiles start at lev == 1."""
    f = np.float32
    lat_o, lon_o, ph, yo, rinv = [], [], [], [], []
    for r in range(lon.size):
        if lev[r] == 1:
            lat_o.append(float(lat[r]))
            lon_o.append(float(lon[r]))
            ph.append(np.zeros(nz))
            yo.append(np.zeros((nz, nvar)))
            rinv.append(np.zeros((nz, nvar)))
        l = int(lev[r]) - 1
        ph[-1][l] = float(val[r, 2 * nvar])
        for n in range(nvar):
            sd = f(val[r, 2 * n + 1])
            pert = f(noise[n, r]) * sd if noise is not None else f(0.0)
            yo[-1][l, n] = float(f(f(val[r, 2 * n]) + f(pert)))
            rinv[-1][l, n] = float(f(f(1.0) / f(sd * sd)))
    return (np.array(lat_o), np.array(lon_o), np.array(ph), np.array(yo), np.array(rinv))


def _records(rng, nobs, nz, nvar):
    n = nobs * nz
    lon = np.repeat(rng.uniform(0, 360, nobs), nz).astype(np.float32)
    lat = np.repeat(rng.uniform(-90, 90, nobs), nz).astype(np.float32)
    lev = np.tile(np.arange(1, nz + 1), nobs).astype(np.float32)
    val = np.zeros((n, 2 * nvar + 1), np.float32)
    for k in range(nvar):
        val[:, 2 * k] = rng.normal(280.0, 10.0, n)
        val[:, 2 * k + 1] = rng.uniform(0.5, 3.0, n)
    val[:, 2 * nvar] = rng.uniform(1e4, 1e5, n)
    noise = rng.standard_normal((nvar, n)).astype(np.float32)
    return lon, lat, lev, val, noise


@pytest.mark.parametrize("nz,nvar", [(1, 1), (1, 2), (4, 2), (7, 1)])
def test_records_match_read_obs(built_lib, nz, nvar):
    import letkf_gb300 as lg
    rng = np.random.default_rng(nz * 10 + nvar)
    lon, lat, lev, val, noise = _records(rng, 50, nz, nvar)
    for nse in (noise, None):
        got = lg.obs_from_records(nz, nvar, lon, lat, lev, val, nse)
        ref = _read_obs(nz, nvar, lon, lat, lev, val, nse)
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)


def test_records_reject_broken_profiles(built_lib):
    import letkf_gb300 as lg
    rng = np.random.default_rng(3)
    lon, lat, lev, val, noise = _records(rng, 5, 3, 1)
    bad_cases = []
    lev2 = lev.copy(); lev2[4] = 3.0; bad_cases.append(lev2)      # level skipped
    lev3 = lev.copy(); lev3[0] = 2.0; bad_cases.append(lev3)      # profile not starting at 1
    lev4 = lev.copy(); lev4[7] = 4.0; bad_cases.append(lev4)      # level beyond nz
    lev5 = lev.copy(); lev5[2] = 1.5; bad_cases.append(lev5)      # not an integer level
    for lv in bad_cases:
        with pytest.raises(RuntimeError, match="LG_ERR_SHAPE"):
            lg.obs_from_records(3, 1, lon, lat, lv, val, noise)
    # the last profile cut short
    with pytest.raises(RuntimeError, match="LG_ERR_SHAPE"):
        lg.obs_from_records(3, 1, lon[:-1], lat[:-1], lev[:-1], val[:-1], noise[:, :-1])
    out = lg.obs_from_records(3, 1, lon[:0], lat[:0], lev[:0], val[:0], None)
    assert out[0].size == 0
