"""Bit-exact parity of the CUDA local-observation search with the oracle:
same selected observations in the same order, per grid point."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, dt, dev):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def scale_setup(seed=1, nlon=24, nlat=20, nlev=5, nobs=6000, sigma_obs=12.0e3):
    case = S.regional_case(seed, nlon=nlon, nlat=nlat, nlev=nlev, ne=8, nobs=nobs, sigma_obs=sigma_obs,
                           with_grid_ensemble=False)
    perm, grd = O.scale_sort_obs(nlon, nlat, case["ri"], case["rj"])
    srt = {k: case[k][perm] for k in ("ri", "rj", "lev", "dat", "err", "cls")}
    return case, perm, grd, srt


@pytest.mark.parametrize("sigma_obs,var_local", [(12.0e3, None), (5.0e3, [1.0, 0.0, 0.5])])
def test_scale_search_bit_exact(cuda, sigma_obs, var_local):
    import torch

    from letkf_gb300.core import search_scale

    case, perm, grd, srt = scale_setup(sigma_obs=sigma_obs)
    prm = S.scale_params(case)
    nobs = perm.size
    varloc = (np.arange(nobs) % 3).astype(np.int32)
    so = O.ScaleObs(case["nlon"], case["nlat"], grd, srt["ri"], srt["rj"], srt["lev"], srt["dat"], srt["err"],
                    srt["cls"], np.zeros(nobs), np.zeros(nobs), varloc, 1, 1, prm["dx"], prm["dy"],
                    prm["dlon_zero"], prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"], var_local)
    obs = {k: _t(srt[k], torch.float64, cuda) for k in ("ri", "rj", "lev", "dat", "err")}
    obs["cls"] = _t(srt["cls"], torch.int32, cuda)
    obs["varloc"] = _t(varloc, torch.int32, cuda)
    pts = {k: _t(case[p], torch.float64, cuda) for k, p in (("ri", "pri"), ("rj", "prj"), ("rlev", "prlev"))}
    offs, idx, rloc, rdiag = search_scale(case["nlon"], case["nlat"], _t(grd, torch.int32, cuda), obs, pts, prm,
                                          var_local)
    offs, idx, rloc, rdiag = (x.cpu().numpy() for x in (offs, idx, rloc, rdiag))
    npts = case["pri"].size
    total = 0
    for p in range(npts):
        ri, rl, rd = so.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p])
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(idx[s], ri, err_msg=f"point {p}")
        np.testing.assert_allclose(rloc[s], rl, rtol=1e-14, atol=0)
        np.testing.assert_allclose(rdiag[s], rd, rtol=1e-14, atol=0)
        total += ri.size
    assert total > 1000


def test_scale_search_empty_and_edges(cuda):
    """No observations at all, and points on the domain corners."""
    import torch

    from letkf_gb300.core import search_scale

    case, perm, grd, srt = scale_setup(nobs=500)
    prm = S.scale_params(case)
    empty = np.zeros_like(grd)
    obs = {k: _t(srt[k], torch.float64, cuda) for k in ("ri", "rj", "lev", "dat", "err")}
    obs["cls"] = _t(srt["cls"], torch.int32, cuda)
    obs["varloc"] = _t(np.zeros(perm.size), torch.int32, cuda)
    pts = {"ri": _t([1.0, case["nlon"], 1.0], torch.float64, cuda), "rj": _t([1.0, case["nlat"], 3.5], torch.float64, cuda),
           "rlev": _t([9.0e4, 5.0e4, 1.0e4], torch.float64, cuda)}
    offs, idx, _, _ = search_scale(case["nlon"], case["nlat"], _t(empty, torch.int32, cuda), obs, pts, prm)
    assert offs.cpu().numpy().tolist() == [0, 0, 0, 0]
    so = O.ScaleObs(case["nlon"], case["nlat"], grd, srt["ri"], srt["rj"], srt["lev"], srt["dat"], srt["err"],
                    srt["cls"], np.zeros(perm.size), np.zeros(perm.size), np.zeros(perm.size), 1, 1, prm["dx"],
                    prm["dy"], prm["dlon_zero"], prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"])
    offs, idx, _, _ = search_scale(case["nlon"], case["nlat"], _t(grd, torch.int32, cuda), obs, pts, prm)
    offs, idx = offs.cpu().numpy(), idx.cpu().numpy()
    for p, (a, b, c) in enumerate(zip([1.0, case["nlon"], 1.0], [1.0, case["nlat"], 3.5], [9.0e4, 5.0e4, 1.0e4])):
        ri, _, _ = so.obs_local(a, b, c)
        np.testing.assert_array_equal(idx[offs[p]:offs[p + 1]], ri)


def speedy_setup(seed=2, nstations=250):
    c = S.speedy_case(seed, nstations=nstations)
    perm, grd = O.speedy_sort_obs(c["lon"], c["lat"], c["olon"], c["olat"])
    srt = {k: c[k][perm] for k in ("elm", "olon", "olat", "olev", "odat", "oerr")}
    return c, perm, grd, srt


@pytest.mark.parametrize("sigma_obs", [500.0e3, 2000.0e3])
def test_speedy_search_bit_exact(cuda, sigma_obs):
    import math

    import torch

    from letkf_gb300.core import search_speedy

    c, perm, grd, srt = speedy_setup()
    dist_zero = sigma_obs * math.sqrt(10.0 / 3.0) * 2.0
    dlat_zero = dist_zero / 3.1415926535 / 6371.3e3 * 180.0
    dlon_zero = dlat_zero / np.cos(3.1415926535 * c["glat"] / 180.0)
    so = O.SpeedyObs(c["lon"], c["lat"], grd, srt["elm"], srt["olon"], srt["olat"], srt["olev"], srt["odat"],
                     srt["oerr"], dist_zero, c["dist_zerov"], dlat_zero, sigma_obs, c["sigma_obsv"], c["var_local"])
    # points: every 7th horizontal point at levels 1, 4, 7
    hp = np.arange(0, c["glon"].size, 7)
    ilev = np.repeat([1, 4, 7], hp.size).astype(np.int32)
    hp3 = np.tile(hp, 3)
    logp = c["logpfm"][ilev - 1, hp3]
    grid = {"lon": _t(c["lon"], torch.float64, cuda), "lat": _t(c["lat"], torch.float64, cuda),
            "nobsgrd": _t(grd, torch.int32, cuda)}
    obs = {"elm": srt["elm"], "lon": srt["olon"], "lat": srt["olat"], "lev": srt["olev"], "dat": srt["odat"],
           "err": srt["oerr"]}
    obs = {k: _t(v, torch.float64, cuda) for k, v in obs.items()}
    pts = {"lon": _t(c["glon"][hp3], torch.float64, cuda), "lat": _t(c["glat"][hp3], torch.float64, cuda),
           "dlon_zero": _t(dlon_zero[hp3], torch.float64, cuda), "ilev": _t(ilev, torch.int32, cuda),
           "logpfm": _t(logp, torch.float64, cuda)}
    offs, idx, rloc, rdiag = search_speedy(grid, obs, pts, (dist_zero, c["dist_zerov"], dlat_zero, sigma_obs,
                                                             c["sigma_obsv"]), c["var_local"])
    offs, idx, rloc, rdiag = (x.cpu().numpy() for x in (offs, idx, rloc, rdiag))
    total = 0
    for p in range(hp3.size):
        ri, rl, rd = so.obs_local(c["glon"][hp3[p]], c["glat"][hp3[p]], dlon_zero[hp3[p]], int(ilev[p]), logp[p])
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(idx[s], ri, err_msg=f"point {p}")
        np.testing.assert_allclose(rloc[s], rl, rtol=1e-13, atol=1e-300)
        np.testing.assert_array_equal(rdiag[s], rd)
        total += ri.size
    assert total > 1000


# ------------------------------------------------------------------------- GFS
@pytest.mark.parametrize("var_local", [None, [1.0, 0.5, 0.0, 1.0, 0.8, 1.0]])
def test_gfs_search_matches_oracle(cuda, var_local):
    """GFS obs_local (gfs/letkf/letkf_tools.f90:686-925) on the SPEEDY bucket
    layout: lists and order bit-exact, rloc/rdiag to 1e-13, including tv, rain
    (own cut-offs), TC track obs (no vertical distance), ps and points near
    the poles and the date line; with and without variable localisation."""
    import math

    import torch

    from letkf_gb300.core import search_gfs
    from letkf_gb300.drivers import speedy_sort_obs

    c = S.speedy_case(9, nstations=400)
    rng = np.random.default_rng(9)
    elm = c["elm"].copy()
    n = elm.size
    pick = rng.choice(n, n // 5, replace=False)
    elm[pick[: n // 20]] = 3074                 # Tv
    elm[pick[n // 20: n // 10]] = 19999         # rain
    elm[pick[n // 10: n // 10 + 30]] = 99991    # TC track
    lev = c["olev"].copy()
    perm, grd = speedy_sort_obs(c["lon"], c["lat"], c["olon"], c["olat"])
    srt = {"elm": elm[perm], "olon": c["olon"][perm], "olat": c["olat"][perm], "olev": lev[perm],
           "odat": c["odat"][perm], "oerr": c["oerr"][perm]}
    so = O.SpeedyObs(c["lon"], c["lat"], grd, srt["elm"], srt["olon"], srt["olat"], srt["olev"], srt["odat"],
                     srt["oerr"], c["dist_zero"], c["dist_zerov"], c["dlat_zero"], c["sigma_obs"], c["sigma_obsv"],
                     np.ones(7))
    f = math.sqrt(10.0 / 3.0) * 2.0
    prm = {"dist_zero": 500e3 * f, "dist_zerov": 0.4 * f, "dist_zero_rain": 350e3 * f, "dist_zerov_rain": 0.4 * f,
           "sigma_obs": 500e3, "sigma_obsv": 0.4, "sigma_obs_rain": 350e3, "base_obsv_rain": 85000.0}
    plon = np.concatenate([rng.uniform(0, 360, 300), [0.0, 359.9, 180.0, 3.75]])
    plat = np.concatenate([rng.uniform(-88, 88, 300), [87.0, -87.0, 0.0, 89.5]])
    prlev = np.exp(rng.uniform(np.log(2e4), np.log(1.0e5), plon.size))
    dv = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    grid = {"lon": dv(c["lon"]), "lat": dv(c["lat"]), "nobsgrd": dv(grd, torch.int32)}
    obs = {"elm": dv(srt["elm"]), "lon": dv(srt["olon"]), "lat": dv(srt["olat"]), "lev": dv(srt["olev"]),
           "dat": dv(srt["odat"]), "err": dv(srt["oerr"])}
    offs, idx, rloc, rdiag = search_gfs(grid, obs, {"lon": dv(plon), "lat": dv(plat), "rlev": dv(prlev)}, prm,
                                        var_local)
    offs, idx, rloc, rdiag = (x.cpu().numpy() for x in (offs, idx, rloc, rdiag))
    params = [prm[k] for k in ("dist_zero", "dist_zerov", "dist_zero_rain", "dist_zerov_rain", "sigma_obs",
                               "sigma_obsv", "sigma_obs_rain", "base_obsv_rain")]
    total = 0
    kinds = set()
    for p in range(plon.size):
        ri, rl, rd = O.gfs_obs_local(so, params, plon[p], plat[p], prlev[p], var_local)
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(idx[s], ri, err_msg=f"point {p}")
        np.testing.assert_allclose(rloc[s], rl, rtol=1e-13, atol=0)
        np.testing.assert_array_equal(rdiag[s], rd)
        total += ri.size
        kinds.update(int(round(e)) for e in srt["elm"][ri])
    assert total > 1000
    assert {3074, 19999, 14593}.issubset(kinds)
