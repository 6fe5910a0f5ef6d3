"""Committed golden fixtures (tests/golden/, made by make_golden.py from the
oracle): the oracle must still reproduce them (CPU), and the CUDA path must
match them (GPU): FP64 core within 1e-10 relative, local observation lists
bit-exact in content and order."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL = 1e-10


def _load(name):
    return np.load(os.path.join(GOLD, name))


def _close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(np.asarray(a) - b).max() / scale
    assert err <= rtol, f"relative error {err:.3e} > {rtol:.1e}"


def _core_case(g, c):
    p = f"c{c}_"
    ne, L, wloc, minfl, infl = g[p + "meta"]
    return (int(ne), int(L), bool(wloc), None if minfl < 0 else float(minfl), float(infl), g[p + "hdxb"],
            g[p + "rdiag"], g[p + "rloc"], g[p + "dep"], g[p + "trans"], g[p + "transm"], g[p + "pao"],
            float(g[p + "infl"]))


# ------------------------------------------------------------------ oracle (CPU)
def test_oracle_reproduces_core_fixture():
    g = _load("core_cases.npz")
    for c in range(int(g["ncase"])):
        ne, L, wloc, minfl, infl, Y, rd, rl, d, tr, tm, pa, infl_out = _core_case(g, c)
        r = O.letkf_core(Y, rd, rl, d, infl, nobsl=L, want_transm=True, want_pao=True, rdiag_wloc=wloc,
                         minfl=minfl)
        assert r["status"] == 0
        _close(r["trans"], tr, 1e-12)
        _close(r["pao"], pa, 1e-12)
        if L:
            _close(r["transm"], tm, 1e-12)
        assert abs(r["parm_infl"] - infl_out) <= 1e-12 * abs(infl_out)


def test_oracle_reproduces_scale_search_fixture():
    g = _load("scale_search.npz")
    perm, grd = O.scale_sort_obs(int(g["nlon"]), int(g["nlat"]), *_unsorted_scale_positions(g))
    np.testing.assert_array_equal(grd, g["nobsgrd"])
    nobs = g["obs_ri"].size
    so = O.ScaleObs(int(g["nlon"]), int(g["nlat"]), g["nobsgrd"], g["obs_ri"], g["obs_rj"], g["obs_lev"],
                    g["obs_dat"], g["obs_err"], g["obs_cls"], np.zeros(nobs), np.zeros(nobs), g["varloc"], 1, 1,
                    float(g["prm_dx"]), float(g["prm_dy"]), float(g["prm_dlon_zero"]), float(g["prm_dlat_zero"]),
                    float(g["prm_sigma_obs"]), float(g["prm_sigma_obsv"]), list(g["var_local"]))
    offs = g["offs"]
    for p in range(offs.size - 1):
        i, rl, rd = so.obs_local(g["pri"][p], g["prj"][p], g["prlev"][p])
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(i, g["idx"][s])
        np.testing.assert_allclose(rl, g["rloc"][s], rtol=1e-13, atol=0)
        np.testing.assert_allclose(rd, g["rdiag"][s], rtol=1e-13, atol=0)


def _unsorted_scale_positions(g):
    """Undo the stored sort so the oracle's sort is exercised again."""
    inv = np.empty_like(g["perm"])
    inv[g["perm"]] = np.arange(g["perm"].size)
    return g["obs_ri"][inv], g["obs_rj"][inv]


def test_oracle_reproduces_speedy_search_fixture():
    g = _load("speedy_search.npz")
    P = g["params"]
    so = O.SpeedyObs(g["lon"], g["lat"], g["nobsgrd"], g["obs_elm"], g["obs_olon"], g["obs_olat"], g["obs_olev"],
                     g["obs_odat"], g["obs_oerr"], P[0], P[1], P[2], P[3], P[4], g["var_local"])
    offs = g["offs"]
    for p in range(offs.size - 1):
        i, rl, rd = so.obs_local(g["plon"][p], g["plat"][p], g["pdlon_zero"][p], int(g["pilev"][p]),
                                 g["plogpfm"][p])
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(i, g["idx"][s])
        np.testing.assert_allclose(rl, g["rloc"][s], rtol=1e-13, atol=1e-300)
        np.testing.assert_array_equal(rd, g["rdiag"][s])


def test_oracle_reproduces_l96_fixture():
    g = _load("l96_analysis.npz")
    nx, ne = g["xf"].shape
    offs = g["offs"]
    for ix in range(1, nx + 1):
        idx, rl = O.l96_select(g["h"], ix, 3.0)
        s = slice(offs[ix - 1], offs[ix])
        np.testing.assert_array_equal(idx, g["idx"][s])
        np.testing.assert_allclose(rl, g["rloc"][s], rtol=1e-14)
        r = O.letkf_core(g["hdxf"][idx], np.full(idx.size, float(g["obserr"]) ** 2), rl, g["dep"][idx], 1.05)
        _close(r["trans"], g["trans"][ix - 1], 1e-12)


# ---------------------------------------------------------------- CUDA path (GPU)
def _t(a, dt, dev):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.mark.gpu
def test_gpu_core_matches_core_fixture(cuda):
    from letkf_gb300.core import letkf_core

    g = _load("core_cases.npz")
    for c in range(int(g["ncase"])):
        ne, L, wloc, minfl, infl, Y, rd, rl, d, tr, tm, pa, infl_out = _core_case(g, c)
        trans, transm, pao, infl_g = letkf_core(ne, Y.shape[0], L, Y, rd, rl, d, infl, transm=True, pao=True,
                                                rdiag_wloc=wloc, minfl=minfl)
        _close(trans, tr, RTOL)
        _close(pao, pa, RTOL)
        if L:
            _close(transm, tm, RTOL)
        assert abs(infl_g - infl_out) <= RTOL * abs(infl_out)


@pytest.mark.gpu
def test_gpu_scale_search_matches_fixture(cuda):
    import torch

    from letkf_gb300.core import SCALE_PARAM_ORDER, search_scale

    g = _load("scale_search.npz")
    prm = {k: float(g["prm_" + k]) for k in SCALE_PARAM_ORDER}
    obs = {k: _t(g["obs_" + k], torch.float64, cuda) for k in ("ri", "rj", "lev", "dat", "err")}
    obs["cls"] = _t(g["obs_cls"], torch.int32, cuda)
    obs["varloc"] = _t(g["varloc"], torch.int32, cuda)
    pts = {k: _t(g[p], torch.float64, cuda) for k, p in (("ri", "pri"), ("rj", "prj"), ("rlev", "prlev"))}
    offs, idx, rloc, rdiag = search_scale(int(g["nlon"]), int(g["nlat"]), _t(g["nobsgrd"], torch.int32, cuda), obs,
                                          pts, prm, list(g["var_local"]))
    np.testing.assert_array_equal(offs.cpu().numpy(), g["offs"])
    np.testing.assert_array_equal(idx.cpu().numpy(), g["idx"])
    np.testing.assert_allclose(rloc.cpu().numpy(), g["rloc"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(rdiag.cpu().numpy(), g["rdiag"], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_gpu_speedy_search_matches_fixture(cuda):
    import torch

    from letkf_gb300.core import search_speedy

    g = _load("speedy_search.npz")
    grid = {"lon": _t(g["lon"], torch.float64, cuda), "lat": _t(g["lat"], torch.float64, cuda),
            "nobsgrd": _t(g["nobsgrd"], torch.int32, cuda)}
    obs = {k: _t(g["obs_" + s], torch.float64, cuda)
           for k, s in (("elm", "elm"), ("lon", "olon"), ("lat", "olat"), ("lev", "olev"), ("dat", "odat"),
                        ("err", "oerr"))}
    pts = {"lon": _t(g["plon"], torch.float64, cuda), "lat": _t(g["plat"], torch.float64, cuda),
           "dlon_zero": _t(g["pdlon_zero"], torch.float64, cuda), "ilev": _t(g["pilev"], torch.int32, cuda),
           "logpfm": _t(g["plogpfm"], torch.float64, cuda)}
    offs, idx, rloc, rdiag = search_speedy(grid, obs, pts, tuple(g["params"]), g["var_local"])
    np.testing.assert_array_equal(offs.cpu().numpy(), g["offs"])
    np.testing.assert_array_equal(idx.cpu().numpy(), g["idx"])
    np.testing.assert_allclose(rloc.cpu().numpy(), g["rloc"], rtol=1e-13, atol=1e-300)
    np.testing.assert_array_equal(rdiag.cpu().numpy(), g["rdiag"])


def test_oracle_reproduces_scale_obsope_fixture():
    g = _load("scale_obsope.npz")
    hx, qc, qcm = O.scale_obsope(g["v3d"], g["v2d"], int(g["khalo"]), g["elem"], g["ri"], g["rj"], g["rlev"],
                                 g["rotc"])
    np.testing.assert_array_equal(qcm, g["qc_member"])
    np.testing.assert_array_equal(qc, g["qc"])
    np.testing.assert_allclose(hx, g["hx"], rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_gpu_scale_obsope_matches_fixture(cuda):
    """Values within 1e-12 of each observation's largest magnitude over the
    members (log and pow differ by an ulp from the host), qc equal."""
    import torch

    from letkf_gb300.core import scale_obsope

    g = _load("scale_obsope.npz")
    t = lambda a, dt=torch.float64: _t(a, dt, cuda)
    hx, qc, qcm = scale_obsope(t(g["v3d"]), t(g["v2d"]), int(g["khalo"]), t(g["elem"], torch.int32), t(g["ri"]),
                               t(g["rj"]), t(g["rlev"]), t(g["rotc"]), want_member_qc=True)
    np.testing.assert_array_equal(qcm.cpu().numpy(), g["qc_member"])
    np.testing.assert_array_equal(qc.cpu().numpy(), g["qc"])
    scale = np.abs(g["hx"]).max(axis=1, keepdims=True)
    assert (np.abs(hx.cpu().numpy() - g["hx"]) <= 1e-12 * scale).all()
