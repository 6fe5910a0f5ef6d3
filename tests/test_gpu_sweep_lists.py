"""Selected observation lists of the fused sweep kernels, the MAX_NOBS_PER_GRID
selection and the bounded-wait failure path.

The mixed-form sweeps (tensor-core and SIMT) search each point's local
observations themselves: an FP32 filter plus an FP64 re-test of the band
around the cut-off.  The selection probe records what that search accepted,
in the order it enters the Gram, and these tests require the index lists and
their order to equal the oracle's obs_local (scale/letkf/letkf_tools.f90:
853-1178) exactly, including observations placed on the cut-off
13.33333333 (scale/letkf/letkf_obs.f90:30).  rloc is FP32 in the mixed form,
from FP32 coordinate differences (a grid coordinate of 256 carries 1.5e-5 of
absolute rounding into a distance of about one cell): relative tolerance 2e-4.  The MAX_NOBS_PER_GRID lists (letkf_tools.f90:
1041-1156) are integer work: equal to the oracle's, entry for entry."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(seed=3, nlon=24, nlat=20, nlev=6, ne=40, nobs=2500, sigma_obs=10.0e3):
    case = S.regional_case(seed, nlon=nlon, nlat=nlat, nlev=nlev, ne=ne, nobs=nobs, sigma_obs=sigma_obs,
                           dtype=np.float32)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(nlon, nlat, case["ri"], case["rj"])
    case["hdxf"] = case["hdxf"].astype(np.float32)
    return case, prm, perm, grd


def _oracle(case, prm, perm, grd, varloc=None, var_local=None, uid=None, typ=None, nid=1, ntyp=1, max_nobs=0):
    n = perm.size
    vl = np.zeros(n, np.int32) if varloc is None else varloc[perm]
    u = np.ones(n) if uid is None else uid[perm]
    t = np.ones(n) if typ is None else typ[perm]
    # ScaleObs takes 0-based uid / type
    return O.ScaleObs(case["nlon"], case["nlat"], grd, case["ri"][perm], case["rj"][perm], case["lev"][perm],
                      case["dat"][perm], case["err"][perm], case["cls"][perm], u - 1, t - 1, vl, nid, ntyp,
                      prm["dx"], prm["dy"], prm["dlon_zero"], prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"],
                      var_local, max_nobs_per_grid=max_nobs)


def _sweep(case, prm, ne, tc=1, varloc=None, var_local=None, rz=None):
    from letkf_gb300.sweep import OPT_TENSOR_CORES, PREC_MIXED, Sweep

    npts = case["pri"].size
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    sw.set_points(case["pri"], case["prj"], case["prlev"], rz)
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], case["dep"], case["cls"],
               case["hdxf"], varloc=varloc, var_local_row=var_local)
    sw.set_option(OPT_TENSOR_CORES, tc)
    sw.set_background(case["xb"])
    sw.set_inflation(np.full(npts, 1.05))
    return sw


def _check_lists(sw, so, perm, case, points, cap, rz=None):
    cnt, obs, rl = sw.probe()
    for k, p in enumerate(points):
        z = 0.0 if rz is None else rz[p]
        idx, rloc, _ = so.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p], z)
        assert cnt[k] == idx.size, (p, cnt[k], idx.size)
        assert idx.size <= cap
        np.testing.assert_array_equal(obs[k, :idx.size], perm[idx], err_msg=f"point {p}")
        np.testing.assert_allclose(rl[k, :idx.size], rloc, rtol=2e-4, atol=0, err_msg=f"point {p}")


@pytest.mark.parametrize("ne,tc,with_varloc", [(40, 1, False), (64, 1, True), (20, 1, False), (64, 0, False),
                                              (100, 1, True)])
def test_fused_search_lists_equal_oracle(cuda, ne, tc, with_varloc):
    """Every point's accepted list and order in the tensor-core (ne <= 64) and
    SIMT (tc = 0, ne = 100) sweeps equal the oracle's obs_local."""
    case, prm, perm, grd = _case(ne=ne)
    varloc = (case["var"] % 3).astype(np.int32) if with_varloc else None
    var_local = [1.0, 0.5, 0.0] if with_varloc else None
    so = _oracle(case, prm, perm, grd, varloc, var_local)
    npts = case["pri"].size
    cap = 4096
    sw = _sweep(case, prm, ne, tc, varloc, var_local)
    points = np.arange(npts, dtype=np.int32)
    sw.set_probe(points, cap)
    sw.run()
    dg = sw.diagnostics()
    _check_lists(sw, so, perm, case, points, cap)
    cnt, obs, rl = sw.probe()
    np.testing.assert_array_equal(cnt, dg["nobsl"])
    assert dg["nobsl"].max() > 100
    if tc == 1 and ne <= 128:
        # the tensor-core sweeps keep each column's horizontal candidates for
        # its next levels: without that cache, the same bits throughout
        from letkf_gb300.sweep import OPT_COLUMN_UNIT

        xa = sw.analysis()
        sw.set_option(OPT_COLUMN_UNIT, 0)
        sw.set_inflation(np.full(npts, 1.05))
        sw.run()
        cnt0, obs0, rl0 = sw.probe()
        np.testing.assert_array_equal(cnt0, cnt)
        np.testing.assert_array_equal(obs0, obs)
        np.testing.assert_array_equal(rl0, rl)
        np.testing.assert_array_equal(sw.analysis(), xa)
    sw.close()


def test_probe_leaves_the_analysis_unchanged(cuda):
    case, prm, perm, grd = _case(ne=40)
    npts = case["pri"].size
    sw = _sweep(case, prm, 40)
    sw.run()
    xa0 = sw.analysis()
    sw.set_inflation(np.full(npts, 1.05))
    sw.set_probe(np.arange(0, npts, 7, dtype=np.int32), 1024)
    sw.run()
    xa1 = sw.analysis()
    sw.close()
    np.testing.assert_array_equal(xa0, xa1)


def _cutoff_case(ne=40):
    """Observations on and around the cut-off ndist = 13.33333333 of a few grid
    points: at the point's level along x, y and diagonals at relative offsets
    from -2e-3 to 2e-3 (the FP32 filter's band and beyond) and within a few
    ulps of the cut-off; radar observations (height vertical coordinate) above
    and below the point at the same relative offsets."""
    nlon = nlat = 48
    dx = 3000.0
    sigma = 10.0e3
    dz2 = float(np.float32(13.33333333))
    reach = sigma * np.sqrt(dz2) / dx  # cut-off distance in grid units
    eps = np.concatenate([np.linspace(-2e-3, 2e-3, 21), np.arange(-12, 13) * 1e-16, [-1e-9, 1e-9, -1e-12, 1e-12]])
    dirs = [(1.0, 0.0), (-1.0, 0.0), (0.0, 1.0), (0.0, -1.0), (0.6, 0.8), (-0.8, 0.6)]
    pts = [(24.0, 24.0, 50000.0, 1500.0), (23.37, 25.61, 70000.0, 800.0)]
    ri, rj, lev, cls = [], [], [], []
    for (pi, pj, pl, pz) in pts:
        for (ux, uy) in dirs:
            for e in eps:
                d = reach * (1.0 + e)
                ri.append(pi + ux * d)
                rj.append(pj + uy * d)
                lev.append(pl)
                cls.append(0)
        # radar (class 4, radial velocity): nd_v = |lev - rz| / sigma_obsz_radar
        zreach = 1000.0 * np.sqrt(dz2)
        for sgn in (1.0, -1.0):
            for e in eps:
                ri.append(pi)
                rj.append(pj)
                lev.append(pz + sgn * zreach * (1.0 + e))
                cls.append(4)
    ri, rj, lev, cls = map(np.array, (ri, rj, lev, cls))
    cls = cls.astype(np.int32)
    nobs = ri.size
    rng = np.random.default_rng(5)
    hdxf = rng.standard_normal((nobs, ne)).astype(np.float32)
    hdxf -= hdxf.mean(1, keepdims=True)
    case = dict(nlon=nlon, nlat=nlat, nvar=2, dx=dx, dy=dx, ri=ri, rj=rj, lev=lev, dat=np.zeros(nobs),
                err=np.ones(nobs), cls=cls, hdxf=hdxf, dep=rng.standard_normal(nobs), sigma_obs=sigma,
                sigma_obsv=0.4)
    case["pri"] = np.array([p[0] for p in pts])
    case["prj"] = np.array([p[1] for p in pts])
    case["prlev"] = np.array([p[2] for p in pts])
    rz = np.array([p[3] for p in pts])
    xb = rng.standard_normal((2, len(pts), ne)).astype(np.float32)
    case["xb"] = xb
    return case, rz


@pytest.mark.parametrize("tc,ne", [(1, 40), (0, 40)])
def test_fused_search_on_the_cutoff(cuda, tc, ne):
    case, rz = _cutoff_case(ne)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(case["nlon"], case["nlat"], case["ri"], case["rj"])
    so = _oracle(case, prm, perm, grd)
    sw = _sweep(case, prm, ne, tc, rz=rz)
    points = np.arange(case["pri"].size, dtype=np.int32)
    sw.set_probe(points, 2048)
    sw.run()
    _check_lists(sw, so, perm, case, points, 2048, rz=rz)
    cnt, _, _ = sw.probe()
    # both sides of the cut-off are present: some on-the-line candidates are
    # accepted and some rejected
    n_line = case["ri"].size // 2
    assert 0 < cnt[0] < n_line
    sw.close()


@pytest.mark.parametrize("unit", [3, 2, 16])
def test_column_cache_on_the_cutoff(cuda, unit):
    """The cut-off case with each point in a column of three levels, the
    on-the-line level second or third, so that its list comes from the column
    cache (the horizontal survivors kept by the column's first level): lists
    equal the oracle's, and equal, bit for bit with rloc, those of the run
    without the cache.  unit 2 splits a column over two runs of positions."""
    from letkf_gb300.sweep import OPT_COLUMN_UNIT

    case, rz = _cutoff_case(40)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(case["nlon"], case["nlat"], case["ri"], case["rj"])
    so = _oracle(case, prm, perm, grd)
    pi, pj, pl = case["pri"], case["prj"], case["prlev"]
    # per column: another level first, then the cut-off level (point 0) or
    # two others then the cut-off level (point 1)
    levs = [(pl[0] * 0.8, pl[0], pl[0] * 1.1), (pl[1] * 1.05, pl[1] * 0.9, pl[1])]
    zs = [(rz[0] + 500.0, rz[0], rz[0] - 300.0), (rz[1] - 200.0, rz[1] + 100.0, rz[1])]
    case["pri"] = np.repeat(pi, 3)
    case["prj"] = np.repeat(pj, 3)
    case["prlev"] = np.array([v for c in levs for v in c])
    rzc = np.array([v for c in zs for v in c])
    case["xb"] = np.repeat(case["xb"], 3, axis=1)
    sw = _sweep(case, prm, 40, 1, rz=rzc)
    sw.set_option(OPT_COLUMN_UNIT, unit)
    points = np.arange(case["pri"].size, dtype=np.int32)
    sw.set_probe(points, 2048)
    sw.run()
    _check_lists(sw, so, perm, case, points, 2048, rz=rzc)
    cnt, obs, rl = sw.probe()
    n_line = case["ri"].size // 2
    assert 0 < cnt[1] < n_line and cnt[5] > 0
    xa = sw.analysis()
    sw.set_option(OPT_COLUMN_UNIT, 0)
    sw.set_inflation(np.full(points.size, 1.05))
    sw.run()
    cnt0, obs0, rl0 = sw.probe()
    xa0 = sw.analysis()
    sw.close()
    np.testing.assert_array_equal(cnt0, cnt)
    np.testing.assert_array_equal(obs0, obs)
    np.testing.assert_array_equal(rl0, rl)
    np.testing.assert_array_equal(xa0, xa)


def test_fused_search_matches_golden_fixture(cuda):
    """The fused search on the committed SCALE search fixture's observations
    and points: lists and order equal the fixture's."""
    import os

    from letkf_gb300.core import SCALE_PARAM_ORDER
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "scale_search.npz"))
    prm = {k: float(g["prm_" + k]) for k in SCALE_PARAM_ORDER}
    inv = np.empty_like(g["perm"])
    inv[g["perm"]] = np.arange(g["perm"].size)
    un = lambda a: np.asarray(a)[inv]  # back to the input order
    nobs = g["obs_ri"].size
    ne = 32
    rng = np.random.default_rng(2)
    hdxf = rng.standard_normal((nobs, ne)).astype(np.float32)
    npts = g["pri"].size
    sw = Sweep(ne, 1, int(g["nlon"]), int(g["nlat"]), npts, prm, precision=PREC_MIXED)
    sw.set_points(g["pri"], g["prj"], g["prlev"])
    sw.set_obs(un(g["obs_ri"]), un(g["obs_rj"]), un(g["obs_lev"]), un(g["obs_dat"]), un(g["obs_err"]),
               rng.standard_normal(nobs), un(g["obs_cls"]), hdxf, varloc=un(g["varloc"]),
               var_local_row=list(g["var_local"]))
    np.testing.assert_array_equal(sw.nobsgrd(), g["nobsgrd"])
    sw.set_background(rng.standard_normal((1, npts, ne)).astype(np.float32))
    sw.set_inflation(np.ones(npts))
    cap = int(np.diff(g["offs"]).max()) + 1
    sw.set_probe(np.arange(npts, dtype=np.int32), cap)
    sw.run()
    cnt, obs, rl = sw.probe()
    sw.close()
    offs = g["offs"]
    np.testing.assert_array_equal(cnt, np.diff(offs))
    for p in range(npts):
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(obs[p, :cnt[p]], g["perm"][g["idx"][s]])
        np.testing.assert_allclose(rl[p, :cnt[p]], g["rloc"][s], rtol=2e-4, atol=0)


# ---------------------------------------------------------------- MAX_NOBS_PER_GRID
def _groups(n, seed=9, nid=3, ntyp=2):
    rng = np.random.default_rng(seed)
    return rng.integers(1, nid + 1, n).astype(np.int32), rng.integers(1, ntyp + 1, n).astype(np.int32), nid, ntyp


@pytest.mark.parametrize("max_nobs", [1, 8, 64])
def test_limited_search_equals_oracle(cuda, max_nobs):
    import torch

    from letkf_gb300.core import search_scale_limited

    case, prm, perm, grd = _case(nobs=4000)
    uid, typ, nid, ntyp = _groups(perm.size)
    varloc = (case["var"] % 3).astype(np.int32)
    var_local = [1.0, 0.7, 0.0]
    so = _oracle(case, prm, perm, grd, varloc, var_local, uid, typ, nid, ntyp, max_nobs)
    so_all = _oracle(case, prm, perm, grd, varloc, var_local, uid, typ, nid, ntyp, 0)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    obs = {k: t(case[k][perm]) for k in ("ri", "rj", "lev", "dat", "err")}
    obs["cls"] = t(case["cls"][perm], torch.int32)
    obs["varloc"] = t(varloc[perm], torch.int32)
    obs["uid"] = t(uid[perm], torch.int32)
    obs["typ"] = t(typ[perm], torch.int32)
    pts = {"ri": t(case["pri"]), "rj": t(case["prj"]), "rlev": t(case["prlev"])}
    offs, idx, rloc, rdiag = search_scale_limited(case["nlon"], case["nlat"], t(grd, torch.int32), obs, pts, prm,
                                                  max_nobs, nid, var_local)
    offs, idx, rloc, rdiag = (x.cpu().numpy() for x in (offs, idx, rloc, rdiag))
    limited = 0
    for p in range(case["pri"].size):
        i, rl, rd = so.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p])
        s = slice(offs[p], offs[p + 1])
        np.testing.assert_array_equal(idx[s], i, err_msg=f"point {p}")
        np.testing.assert_allclose(rloc[s], rl, rtol=1e-13, atol=0)
        np.testing.assert_allclose(rdiag[s], rd, rtol=1e-13, atol=0)
        limited += i.size < so_all.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p])[0].size
    assert np.diff(offs).max() <= nid * ntyp * max_nobs
    if max_nobs < 64:
        assert limited > 0  # the limit acted on some points


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_sweep_with_max_nobs_per_grid_against_oracle(cuda, prec):
    """The sweep with LETKF_OPT_MAX_NOBS_PER_GRID against the oracle's SCALE grid
    loop with the same limit: FP64 within 1e-10 of spread, mixed form within
    1e-4; local counts exact."""
    from letkf_gb300.sweep import OPT_MAX_NOBS_PER_GRID, PREC_F64, PREC_MIXED, Sweep

    ne, M = 32, 6
    case, prm, perm, grd = _case(ne=ne, nobs=3000)
    uid, typ, nid, ntyp = _groups(perm.size, seed=4)
    so = _oracle(case, prm, perm, grd, uid=uid, typ=typ, nid=nid, ntyp=ntyp, max_nobs=M)
    hd = case["hdxf"].astype(np.float64)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    xa_ref, infl_ref, nl_ref = so.sweep(hd[perm], case["dep"][perm], xb, case["pri"], case["prj"], case["prlev"],
                                        infl0)
    f64 = prec == "f64"
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_F64 if f64 else PREC_MIXED)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], case["dep"], case["cls"],
               hd if f64 else case["hdxf"])
    sw.set_obs_groups(uid, typ, nid, ntyp)
    sw.set_option(OPT_MAX_NOBS_PER_GRID, M)
    sw.set_background(xb if f64 else case["xb"])
    sw.set_inflation(infl0)
    sw.run()
    xa = sw.analysis().astype(np.float64)
    dg = sw.diagnostics()
    sw.close()
    np.testing.assert_array_equal(dg["nobsl"], nl_ref)
    assert nl_ref.max() <= nid * ntyp * M and nl_ref.max() > 0
    spread = np.sqrt(((xb - xb.mean(-1, keepdims=True)) ** 2).sum(-1) / (ne - 1)).mean()
    if f64:
        assert np.abs(xa - xa_ref).max() / spread < 1e-10
        np.testing.assert_allclose(dg["infl"], infl_ref, rtol=1e-12)
    else:
        em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
        pert = lambda x: x - x.mean(-1, keepdims=True)
        ep = np.sqrt(np.mean((pert(xa) - pert(xa_ref)) ** 2)) / spread
        assert em < 1e-4 and ep < 1e-4, (em, ep)


def test_sweep_max_nobs_needs_groups(cuda):
    from letkf_gb300.lib import LETKF_ERR_ARG, LetkfError
    from letkf_gb300.sweep import OPT_MAX_NOBS_PER_GRID

    case, prm, perm, grd = _case(ne=20, nobs=500)
    sw = _sweep(case, prm, 20)
    sw.set_option(OPT_MAX_NOBS_PER_GRID, 4)
    with pytest.raises(LetkfError) as e:
        sw.run()
    assert e.value.status == LETKF_ERR_ARG
    sw.close()


# ---------------------------------------------------------------- bounded waits
@pytest.mark.parametrize("ne", [40, 128])
def test_bounded_wait_gives_up_then_the_handle_recovers(cuda, ne):
    """A wait that runs out (injected: a barrier nothing arrives at) ends the
    tensor-core sweep with LETKF_ERR_TIMEOUT instead of hanging; the context
    stays usable and the next normal run on the same handle gives the same
    analysis as before.  The reference stops the program instead
    (common/common_mtx.f90:61-64,75-78)."""
    from letkf_gb300.lib import LETKF_ERR_TIMEOUT, LetkfError
    from letkf_gb300.sweep import OPT_FAULT_WAIT

    case, prm, perm, grd = _case(ne=ne)
    npts = case["pri"].size
    sw = _sweep(case, prm, ne)
    sw.run()
    xa0 = sw.analysis()
    for polls in (1, 64):
        sw.set_inflation(np.full(npts, 1.05))
        sw.set_option(OPT_FAULT_WAIT, polls)
        sw.run()
        with pytest.raises(LetkfError) as e:
            sw.analysis()
        assert e.value.status == LETKF_ERR_TIMEOUT
    sw.set_option(OPT_FAULT_WAIT, 0)
    sw.set_inflation(np.full(npts, 1.05))
    sw.run()
    np.testing.assert_array_equal(sw.analysis(), xa0)
    sw.close()
