"""Domain decomposition on the GPU: a regional domain split into 2-D tiles
(the SCALE process tiles, scale/letkf/letkf_obs.f90:886-985), each tile
analysed by its own sweep handle from the observations of its halo.  Every
point's local list, its order and so its analysis are those of the
single-domain sweep, so the reassembled analysis equals it bit for bit."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ntiles,ne", [(4, 40), (6, 64), (2, 100)])
def test_tiles_equal_the_single_domain(cuda, ntiles, ne):
    from letkf_gb300.shard import halo_mask, tile_of, tile_sweep
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    nlon, nlat, nlev = 36, 30, 5
    case = S.regional_case(4, nlon=nlon, nlat=nlat, nlev=nlev, ne=ne, nobs=4000, nvar=2, sigma_obs=9.0e3,
                           dtype=np.float32)
    prm = S.scale_params(case)
    npts = case["pri"].size
    obs = {k: case[k] for k in ("ri", "rj", "lev", "dat", "err", "dep", "cls")}
    obs["hdxf"] = case["hdxf"].astype(np.float32)
    pts = (case["pri"], case["prj"], case["prlev"])
    xb = case["xb"].astype(np.float32)

    one = Sweep(ne, 2, nlon, nlat, npts, prm, precision=PREC_MIXED)
    one.set_points(*pts)
    one.set_obs(*(obs[k] for k in ("ri", "rj", "lev", "dat", "err", "dep", "cls")), obs["hdxf"])
    one.set_background(xb)
    one.set_inflation(np.full(npts, 1.05))
    one.run()
    xa1 = one.analysis()
    one.close()

    xa = np.full_like(xa1, np.nan)
    covered = np.zeros(npts, dtype=int)
    for k in range(ntiles):
        tile = tile_of(k, ntiles, nlon, nlat)
        points, sw, nkept = tile_sweep(tile, nlon, nlat, nlev, pts, obs, prm, ne, 2, PREC_MIXED)
        # the halo is a strict subset of the observations for an inner split
        assert 0 < nkept <= obs["ri"].size
        assert nkept == int(halo_mask(obs["ri"], obs["rj"], tile, nlon, nlat, prm["dlon_zero"],
                                      prm["dlat_zero"]).sum())
        sw.set_background(np.ascontiguousarray(xb[:, points]))
        sw.set_inflation(np.full(points.size, 1.05))
        sw.run()
        xa[:, points] = sw.analysis()
        sw.close()
        covered[points] += 1
    assert (covered == 1).all()
    np.testing.assert_array_equal(xa, xa1)


def test_device_background_written_on_the_default_stream(cuda):
    """set_background with a device pointer whose data the default stream is
    still computing: the copy waits for it (the handle's own streams do not
    synchronise with the default stream), so the analysis equals the one from
    a host copy of the same background."""
    import torch

    from letkf_gb300.sweep import PREC_MIXED, Sweep

    case = S.regional_case(7, nlon=24, nlat=20, nlev=4, ne=32, nobs=2500, nvar=2, dtype=np.float32)
    prm = S.scale_params(case)
    npts = case["pri"].size
    xb = case["xb"].astype(np.float32)

    def handle():
        sw = Sweep(32, 2, 24, 20, npts, prm, precision=PREC_MIXED)
        sw.set_points(case["pri"], case["prj"], case["prlev"])
        sw.set_obs(case["ri"], case["rj"], case["lev"], case["dat"], case["err"], case["dep"], case["cls"],
                   case["hdxf"].astype(np.float32))
        sw.set_inflation(np.full(npts, 1.05))
        return sw

    ref = handle()
    ref.set_background(xb)
    ref.run()
    xa_ref = ref.analysis()
    ref.close()

    sw = handle()
    torch.cuda.synchronize()
    # a long chain on the default stream, then the background as its result
    big = torch.randn(4096, 4096, device=cuda)
    for _ in range(30):
        big = torch.tanh(big @ big)
    xb_dev = torch.as_tensor(xb, device=cuda) + 0.0 * big[0, 0]
    sw.set_background_device(xb_dev.data_ptr())
    sw.run()
    xa = sw.analysis()
    sw.close()
    np.testing.assert_array_equal(xa, xa_ref)
