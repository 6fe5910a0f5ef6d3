"""The device-resident analysis sweep (search + core + update of every point)
against the oracle's SCALE grid loop.

FP64 plain form: analysis within 1e-10 of the oracle (relative to the
background spread).  Mixed form: analysis-mean and spread RMS error below
1e-4 of the background spread.  Both: local obs counts bit-exact."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _setup(seed=3, nlon=24, nlat=20, nlev=6, ne=40, nobs=2500, sigma_obs=10.0e3, f32=False, var_local=None,
           err_scale=1.0):
    case = S.regional_case(seed, nlon=nlon, nlat=nlat, nlev=nlev, ne=ne, nobs=nobs, sigma_obs=sigma_obs,
                           dtype=np.float32 if f32 else np.float64)
    case["err"] = case["err"] * err_scale
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(nlon, nlat, case["ri"], case["rj"])
    nob = perm.size
    varloc = (case["var"] % 3).astype(np.int32)
    hdxf = case["hdxf"].astype(np.float32).astype(np.float64) if f32 else case["hdxf"]
    dep = case["dep"]
    so = O.ScaleObs(nlon, nlat, grd, case["ri"][perm], case["rj"][perm], case["lev"][perm], case["dat"][perm],
                    case["err"][perm], case["cls"][perm], np.zeros(nob), np.zeros(nob), varloc[perm], 1, 1,
                    prm["dx"], prm["dy"], prm["dlon_zero"], prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"],
                    var_local)
    return case, prm, perm, grd, so, varloc, hdxf, dep


def _spread(xb):
    return np.sqrt(((xb - xb.mean(-1, keepdims=True)) ** 2).sum(-1) / (xb.shape[-1] - 1)).mean()


@pytest.mark.parametrize("ne", [20, 40, 64])
def test_tc_polish_against_oracle(cuda, ne):
    """The anchored polish step on the tensor cores (LETKF_OPT_TC_POLISH)
    meets the mixed-form bar against the oracle."""
    from letkf_gb300.sweep import OPT_TC_POLISH, OPT_TENSOR_CORES, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=ne, f32=True)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    xa_ref, infl_ref, nl_ref = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0)
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
               hdxf.astype(np.float32))
    sw.set_option(OPT_TENSOR_CORES, 1)
    sw.set_option(OPT_TC_POLISH, 1)
    sw.set_background(case["xb"])
    sw.set_inflation(infl0)
    sw.run()
    xa = sw.analysis().astype(np.float64)
    dg = sw.diagnostics()
    sw.close()
    assert (dg["status"] == 0).all()
    spread = _spread(xb)
    em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
    ep = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True)) - (xa_ref - xa_ref.mean(-1, keepdims=True))) ** 2))
    ep /= spread
    assert em < 1e-4 and ep < 1e-4, (em, ep)
    np.testing.assert_allclose(dg["infl"], infl_ref, rtol=1e-4)


@pytest.mark.parametrize("ne,var_local,eig,tc,scaled", [(40, None, 0, 1, 1), (64, [1.0, 0.5, 0.0], 0, 1, 1),
                                                      (20, None, 0, 1, 1), (50, None, 0, 1, 1), (64, None, 0, 1, 0),
                                                      (64, None, 0, 0, 1),
                                                      (100, None, 0, 1, 1), (64, None, 1, 1, 1),
                                                      (128, None, 0, 1, 1), (128, [1.0, 0.5, 0.0], 0, 1, 0),
                                                      (72, None, 0, 1, 1), (128, None, 0, 0, 1)])
def test_mixed_sweep_against_oracle(cuda, ne, var_local, eig, tc, scaled):
    """tc=1 and eig=0 run the tcgen05 sweeps (ne <= 64: sweep_tc; 64 < ne <=
    128: sweep_tc128; spectrum-scaled or plain Newton-Schulz steps; background
    rows by TMA bulk copy when ne is a multiple of 4, by plain loads for
    ne = 50); otherwise the SIMT sweep."""
    from letkf_gb300.sweep import OPT_EIGENSOLVER, OPT_TC_NS_SCALING, OPT_TENSOR_CORES, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=ne, f32=True, var_local=var_local)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    xa_ref, infl_ref, nl_ref = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0,
                                        minfl=1.0)
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED, minfl=1.0)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
               hdxf.astype(np.float32), varloc=varloc if var_local is not None else None, var_local_row=var_local)
    np.testing.assert_array_equal(sw.nobsgrd(), grd)
    sw.set_option(OPT_EIGENSOLVER, eig)
    sw.set_option(OPT_TENSOR_CORES, tc)
    sw.set_option(OPT_TC_NS_SCALING, scaled)
    sw.set_background(case["xb"])
    sw.set_inflation(infl0)
    sw.run()
    xa = sw.analysis().astype(np.float64)
    dg = sw.diagnostics()
    sw.close()
    np.testing.assert_array_equal(dg["nobsl"], nl_ref)
    assert (dg["status"] == 0).all()
    assert nl_ref.max() > 100 and (nl_ref == 0).sum() >= 0
    spread = _spread(xb)
    em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
    ep = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True)) - (xa_ref - xa_ref.mean(-1, keepdims=True))) ** 2))
    ep /= spread
    assert em < 1e-4, f"analysis-mean error {em:.2e} of spread"
    assert ep < 1e-4, f"analysis-perturbation error {ep:.2e} of spread"
    np.testing.assert_allclose(dg["infl"], infl_ref, rtol=1e-4)


def test_f64_sweep_against_oracle(cuda):
    from letkf_gb300.sweep import PREC_F64, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=32, nobs=5000)
    xb = case["xb"]
    npts = case["pri"].size
    infl0 = np.linspace(0.9, 1.2, npts)
    xa_ref, infl_ref, nl_ref = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0,
                                        minfl=1.0)
    sw = Sweep(32, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_F64, minfl=1.0)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"], hdxf)
    sw.set_background(xb)
    sw.set_inflation(infl0)
    sw.run()
    xa = sw.analysis()
    dg = sw.diagnostics()
    sw.close()
    np.testing.assert_array_equal(dg["nobsl"], nl_ref)
    spread = _spread(xb)
    err = np.abs(xa - xa_ref).max() / spread
    assert err < 1e-10, f"FP64 sweep error {err:.2e} of spread"
    np.testing.assert_allclose(dg["infl"], infl_ref, rtol=1e-12)


def test_mixed_sweep_no_obs(cuda):
    """Every point without local obs: xa = mean + sqrt(infl) xb' and infl unchanged (common_letkf.f90:82-96)."""
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=20, nobs=10, f32=True)
    npts = case["pri"].size
    sw = Sweep(20, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"][:0], case["rj"][:0], case["lev"][:0], case["dat"][:0], case["err"][:0], dep[:0],
               case["cls"][:0], np.zeros((0, 20), np.float32))
    sw.set_background(case["xb"])
    sw.set_inflation(np.full(npts, 1.21))
    sw.run()
    xa = sw.analysis().astype(np.float64)
    dg = sw.diagnostics()
    sw.close()
    xb = case["xb"].astype(np.float64)
    m = xb.mean(-1, keepdims=True)
    np.testing.assert_allclose(xa, m + 1.1 * (xb - m), rtol=0, atol=2e-6 * np.abs(xb).max())
    assert (dg["nobsl"] == 0).all()
    np.testing.assert_array_equal(dg["infl"], 1.21)


def test_tc_sweep_defers_points_to_the_jacobi_pass(cuda):
    """Points with a non-positive inflation term c = (k-1)/rho cannot use
    Newton-Schulz; the tensor-core sweep hands them to the Jacobi pass, whose
    results must equal those of the all-Jacobi sweep exactly."""
    from letkf_gb300.sweep import EIG_JACOBI, OPT_EIGENSOLVER, OPT_TENSOR_CORES, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=64, f32=True)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    infl0[::7] = -0.5
    out = []
    for tc, eig in ((1, 0), (0, EIG_JACOBI)):
        sw = Sweep(64, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
        sw.set_points(case["pri"], case["prj"], case["prlev"])
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
                   hdxf.astype(np.float32))
        sw.set_option(OPT_TENSOR_CORES, tc)
        sw.set_option(OPT_EIGENSOLVER, eig)
        sw.set_background(case["xb"])
        sw.set_inflation(infl0)
        sw.run()
        out.append((sw.analysis(), sw.diagnostics()))
        sw.close()
    (xa_tc, dg_tc), (xa_j, dg_j) = out
    neg = np.zeros(npts, bool)
    neg[::7] = True
    np.testing.assert_array_equal(dg_tc["status"][neg], dg_j["status"][neg])
    np.testing.assert_array_equal(xa_tc[:, neg], xa_j[:, neg])
    np.testing.assert_array_equal(dg_tc["infl"][neg], dg_j["infl"][neg])
    spread = _spread(case["xb"].astype(np.float64))
    ok = ~neg
    assert np.abs(xa_tc[:, ok].astype(np.float64) - xa_j[:, ok]).max() < 1e-3 * spread


@pytest.mark.parametrize("tc", [1, 0])
def test_graph_replay_equals_eager_runs(cuda, tc):
    """The mixed-form run as a CUDA graph: replays give the eager run's bits;
    new background data is read by the replay; a new stream or a changed
    option captures again."""
    import torch

    from letkf_gb300 import lib as L
    from letkf_gb300.sweep import OPT_GRAPH, OPT_TENSOR_CORES, OPT_TC_NS_SCALING, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=64, f32=True)
    npts = case["pri"].size
    xb2 = (case["xb"] * 1.01 + 0.1).astype(np.float32)

    def make(graph):
        sw = Sweep(64, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
        sw.set_points(case["pri"], case["prj"], case["prlev"])
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
                   hdxf.astype(np.float32))
        sw.set_option(OPT_TENSOR_CORES, tc)
        sw.set_option(OPT_GRAPH, graph)
        return sw

    def run(sw, xb, stream=None):
        sw.set_background(xb)
        sw.set_inflation(np.full(npts, 1.05))
        sw.run(stream)
        torch.cuda.synchronize()
        return sw.analysis().copy(), sw.diagnostics()["infl"].copy()

    ref = make(0)
    e1, i1 = run(ref, case["xb"])
    e2, i2 = run(ref, xb2)
    ref.close()
    sw = make(1)
    st = torch.cuda.Stream()
    n0 = L.launch_count()
    for xb, (e, i) in ((case["xb"], (e1, i1)), (case["xb"], (e1, i1)), (xb2, (e2, i2))):
        g, gi = run(sw, xb, st.cuda_stream)
        np.testing.assert_array_equal(g, e)
        np.testing.assert_array_equal(gi, i)
    assert L.launch_count() - n0 == 3 * 2   # replays count their kernels: sweep + deferred-point pass
    g, _ = run(sw, case["xb"])                                 # the handle's own stream: a new capture
    np.testing.assert_array_equal(g, e1)
    sw.set_option(OPT_TC_NS_SCALING, 0)                        # new kernel arguments: a new capture
    g, _ = run(sw, case["xb"], st.cuda_stream)
    assert np.abs(g.astype(np.float64) - e1).max() < 1e-3 * _spread(case["xb"].astype(np.float64))
    sw.set_option(OPT_TC_NS_SCALING, 1)
    # fewer observations reuse the resident buffers; same bits as a fresh handle
    sub = slice(0, len(case["ri"]) // 2)
    obs_sub = (case["ri"][sub], case["rj"][sub], case["lev"][sub], case["dat"][sub], case["err"][sub], dep[sub],
               case["cls"][sub], hdxf[sub].astype(np.float32))
    sw.set_obs(*obs_sub)
    g, gi = run(sw, case["xb"], st.cuda_stream)
    fresh = make(0)
    fresh.set_obs(*obs_sub)
    f, fi = run(fresh, case["xb"])
    fresh.close()
    np.testing.assert_array_equal(g, f)
    np.testing.assert_array_equal(gi, fi)
    sw.close()


@pytest.mark.parametrize("ne", [40, 100])
def test_autotune_keeps_inflation_and_picks_a_valid_variant(cuda, ne):
    """letkf_sweep_autotune times the variants on a sample of points, keeps
    the fastest and restores the inflation field; the tuned run still meets
    the mixed-form bar against the oracle."""
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=ne, f32=True)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.linspace(1.0, 1.2, npts)
    xa_ref, infl_ref, nl_ref = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0)
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    sw.set_points(case["pri"], case["prj"], case["prlev"])
    sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
               hdxf.astype(np.float32))
    sw.set_background(case["xb"])
    sw.set_inflation(infl0)
    choice = sw.autotune(sample_points=npts // 2)
    assert choice["us_per_1000_points"] > 0
    if ne > 128:
        assert not choice["tensor_cores"]
    np.testing.assert_array_equal(sw.diagnostics()["infl"], infl0)
    sw.run()
    xa = sw.analysis().astype(np.float64)
    dg = sw.diagnostics()
    sw.close()
    np.testing.assert_array_equal(dg["nobsl"], nl_ref)
    spread = _spread(xb)
    em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
    assert em < 1e-4, f"analysis-mean error {em:.2e} of spread after autotune ({choice})"


@pytest.mark.parametrize("precision", [0, 1])
def test_tile_handles_reproduce_the_single_domain_sweep(cuda, precision):
    """The multi-GPU decomposition on one device: one handle per tile (its
    points, the observations of its halo in global order) run one after the
    other must reproduce the single-domain sweep exactly."""
    from letkf_gb300 import shard
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(nlon=36, nlat=16, nlev=3, ne=32, nobs=3000,
                                                         sigma_obs=5.0e3, f32=True)
    npts = case["pri"].size
    nlon, nlat, nlev = case["nlon"], case["nlat"], case["nlev"]
    dt = np.float32 if precision == PREC_MIXED else np.float64

    def run(pts, sel):
        sw = Sweep(32, case["nvar"], nlon, nlat, pts.size, prm, precision=precision)
        sw.set_points(case["pri"][pts], case["prj"][pts], case["prlev"][pts])
        sw.set_obs(case["ri"][sel], case["rj"][sel], case["lev"][sel], case["dat"][sel], case["err"][sel],
                   dep[sel], case["cls"][sel], hdxf[sel].astype(dt))
        sw.set_background(case["xb"][:, pts, :].astype(dt))
        sw.set_inflation(np.full(pts.size, 1.03))
        sw.run()
        out = sw.analysis(), sw.diagnostics()
        sw.close()
        return out

    xa_all, dg_all = run(np.arange(npts), np.arange(case["ri"].size))
    for world in (2, 3):
        xa = np.zeros_like(xa_all)
        infl = np.zeros(npts)
        nobsl = np.zeros(npts, dtype=np.int64)
        for r in range(world):
            tile = shard.tile_of(r, world, nlon, nlat)
            pts = shard.tile_points(tile, nlon, nlat, nlev)
            sel = np.nonzero(shard.halo_mask(case["ri"], case["rj"], tile, nlon, nlat, prm["dlon_zero"],
                                             prm["dlat_zero"]))[0]
            assert sel.size < case["ri"].size
            x, dg = run(pts, sel)
            xa[:, pts] = x
            infl[pts] = dg["infl"]
            nobsl[pts] = dg["nobsl"]
        np.testing.assert_array_equal(nobsl, dg_all["nobsl"])
        np.testing.assert_array_equal(infl, dg_all["infl"])
        np.testing.assert_array_equal(xa, xa_all)


@pytest.mark.parametrize("tile,shuffle,ne,prec", [(4, False, 40, 1), (0, True, 64, 1), (8, False, 100, 1),
                                                  (4, False, 50, 1), (4, True, 20, 0)])
def test_run_host_overlapped_equals_run(cuda, tile, shuffle, ne, prec):
    """letkf_sweep_run_host (background in, analysis and copies out in pieces
    overlapped with the sweep) equals set_background + run + get_analysis bit
    for bit: banded and scattered processing orders, several piece counts,
    page-locked and pageable host buffers; the plain form runs the three calls."""
    import torch

    from letkf_gb300.sweep import PREC_F64, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=ne, f32=True)
    npts = case["pri"].size
    order = np.random.default_rng(5).permutation(npts) if shuffle else np.arange(npts)
    pri, prj, prlev = (np.ascontiguousarray(case[k][order]) for k in ("pri", "prj", "prlev"))
    dt = np.float32 if prec == 1 else np.float64
    xbh = np.ascontiguousarray(case["xb"][:, order].astype(dt))
    infl0 = np.full(npts, 1.05)
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED if prec else PREC_F64)
    try:
        sw.set_points(pri, prj, prlev, tile=tile)
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
                   hdxf.astype(np.float32) if prec else hdxf)
        sw.set_background(xbh)
        sw.set_inflation(infl0)
        sw.run()
        ref = sw.analysis()
        infl_ref = sw.diagnostics()["infl"]
        pin_b = torch.from_numpy(xbh).pin_memory()
        for nchunks in (1, 3, 7, 16):
            pin_a = torch.zeros(xbh.shape, dtype=pin_b.dtype).pin_memory()
            sw.set_background(np.zeros_like(xbh))      # the run must bring the background in itself
            sw.set_inflation(infl0)
            sw.run_host(pin_b.data_ptr(), pin_a.data_ptr(), nchunks)
            np.testing.assert_array_equal(pin_a.numpy(), ref, err_msg=f"nchunks {nchunks}")
            np.testing.assert_array_equal(sw.diagnostics()["infl"], infl_ref)
        sw.set_background(np.zeros_like(xbh))
        sw.set_inflation(infl0)
        np.testing.assert_array_equal(sw.run_host(xbh, nchunks=5), ref)   # pageable buffers
    finally:
        sw.close()


@pytest.mark.parametrize("err_scale", [1.0, 0.1])
def test_polish_probe_keeps_the_mixed_form_accurate(cuda, err_scale):
    """The default polish probe (LETKF_OPT_POLISH_PROBE 9) skips the FP32 polish
    only where the anchored residual shows the tensor-core transform already
    accurate: on a well- and an ill-conditioned case (observation errors x0.1)
    the analysis meets the mixed-form bar and stays within 3x (or 1e-5 of
    spread) of the always-polished sweep, and a probe that never asks for the
    polish (10^-1) is no more accurate."""
    from letkf_gb300.sweep import OPT_POLISH_PROBE, PREC_MIXED, Sweep

    ne = 64
    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=ne, f32=True, err_scale=err_scale)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    xa_ref, _, _ = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0)
    spread = _spread(xb)
    err = {}
    sw = Sweep(ne, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    try:
        sw.set_points(case["pri"], case["prj"], case["prlev"])
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
                   hdxf.astype(np.float32))
        sw.set_background(case["xb"])
        for probe in (9, 0, 1):
            sw.set_option(OPT_POLISH_PROBE, probe)
            sw.set_inflation(infl0)
            sw.run()
            xa = sw.analysis().astype(np.float64)
            assert (sw.diagnostics()["status"] == 0).all()
            em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
            ep = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True))
                                  - (xa_ref - xa_ref.mean(-1, keepdims=True))) ** 2)) / spread
            err[probe] = (em, ep)
    finally:
        sw.close()
    (em9, ep9), (em0, ep0), (em1, ep1) = err[9], err[0], err[1]
    assert em9 < 1e-4 and ep9 < 1e-4, err
    assert em9 <= max(3 * em0, 1e-5) and ep9 <= max(3 * ep0, 1e-5), err
    assert ep1 >= 0.9 * ep9, err


@pytest.mark.parametrize("tc", [1, 0])
def test_ill_conditioned_points_go_to_the_jacobi_pass(cuda, tc):
    """Observation errors x0.1 give most points a spectrum bound s / c beyond
    the Newton-Schulz range: the sweep hands them (and any point whose
    transform does not certify) to the Jacobi pass, so the analysis stays
    finite and within the mixed-form bar of the oracle, with the local counts
    bit-exact; LETKF_OPT_NS_COND 0 (no bound) relies on the certificate alone."""
    from letkf_gb300.sweep import OPT_NS_COND, OPT_TENSOR_CORES, PREC_MIXED, Sweep

    case, prm, perm, grd, so, varloc, hdxf, dep = _setup(ne=64, f32=True, err_scale=0.1)
    xb = case["xb"].astype(np.float64)
    npts = case["pri"].size
    infl0 = np.full(npts, 1.05)
    xa_ref, infl_ref, nl_ref = so.sweep(hdxf[perm], dep[perm], xb, case["pri"], case["prj"], case["prlev"], infl0)
    spread = _spread(xb)
    sw = Sweep(64, case["nvar"], case["nlon"], case["nlat"], npts, prm, precision=PREC_MIXED)
    try:
        sw.set_points(case["pri"], case["prj"], case["prlev"])
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], dep, case["cls"],
                   hdxf.astype(np.float32))
        sw.set_background(case["xb"])
        sw.set_option(OPT_TENSOR_CORES, tc)
        for cond in (5, 0):
            sw.set_option(OPT_NS_COND, cond)
            sw.set_inflation(infl0)
            sw.run()
            xa = sw.analysis().astype(np.float64)
            dg = sw.diagnostics()
            assert np.isfinite(xa).all()
            assert (dg["status"] == 0).all()
            np.testing.assert_array_equal(dg["nobsl"], nl_ref)
            assert sw.deferred() > npts // 2
            em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
            ep = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True))
                                  - (xa_ref - xa_ref.mean(-1, keepdims=True))) ** 2)) / spread
            assert em < 1e-4 and ep < 1e-4, (cond, em, ep)
            np.testing.assert_allclose(dg["infl"], infl_ref, rtol=1e-4)
    finally:
        sw.close()
