"""GMCORE state to the DA background layout (lg_gmcore_to_da_device): C-grid u
and v moved to the cell centres as gmcore2da_send_coupling does
(gmcore_coupler.F90:153-284), the four fields laid out as xb(ens, n, lat, lon)
with a periodic longitude halo -- against a numpy restatement (exact, v to
rounding)."""
import numpy as np
import pytest


def _restated(ps, uh, vh, pt, asub, acell, halo):
    nz, nlat, nlon, ens = uh.shape
    u = (uh + np.roll(uh, 1, axis=2)) / 2                       # u_f(i) + u_f(i-1), periodic
    v = 2 * (vh[:, :-1] * asub[None, :, 0, None, None] + vh[:, 1:] * asub[None, :, 1, None, None]) \
        / acell[None, :, None, None]
    rows = np.concatenate([ps[None], u, v, pt], axis=0)         # [n][lat][lon][ens]
    xb = np.zeros((nlon + 2 * halo, nlat + 2 * halo, 1 + 3 * nz, ens))
    inner = np.transpose(rows, (2, 1, 0, 3))                    # [lon][lat][n][ens]
    idx = (np.arange(-halo, nlon + halo)) % nlon
    xb[:, halo:halo + nlat] = inner[idx]
    return xb


def test_gmcore_to_da_rejects_bad_arguments(built_lib):
    import letkf_gb300 as lg
    L = lg.load_library()
    assert L.lg_gmcore_to_da_device(0, 4, 4, 1, 1, *([None] * 8)) == -1
    assert L.lg_gmcore_to_da_device(4, 4, 4, 1, 1, *([None] * 8)) == -1


@pytest.mark.gpu
@pytest.mark.parametrize("ens,nlat,nlon,nz,halo", [(8, 9, 16, 3, 1), (64, 18, 36, 8, 2)])
def test_gmcore_to_da_matches_restatement(ens, nlat, nlon, nz, halo):
    import torch

    import letkf_gb300 as lg
    rng = np.random.default_rng(ens + nz)
    ps = rng.normal(1e5, 500, (nlat, nlon, ens))
    uh = rng.normal(0, 10, (nz, nlat, nlon, ens))
    vh = rng.normal(0, 10, (nz, nlat + 1, nlon, ens))
    pt = rng.normal(300, 5, (nz, nlat, nlon, ens))
    asub = rng.uniform(0.5, 1.5, (nlat, 2))
    acell = asub.sum(axis=1) * rng.uniform(0.9, 1.1, nlat)
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev) for a in (ps, uh, vh, pt, asub, acell)]
    got = lg.gmcore_to_da(*t, halo=halo).cpu().numpy()
    ref = _restated(ps, uh, vh, pt, asub, acell, halo)
    # ps, pt copies and the u average exact; v to rounding (per-latitude weights)
    assert np.array_equal(got[:, :, : 1 + nz], ref[:, :, : 1 + nz])
    assert np.array_equal(got[:, :, 1 + 2 * nz:], ref[:, :, 1 + 2 * nz:])
    v_g, v_r = got[:, :, 1 + nz: 1 + 2 * nz], ref[:, :, 1 + nz: 1 + 2 * nz]
    assert np.abs(v_g - v_r).max() <= 1e-14 * np.abs(v_r).max()
