"""SPEEDY observation operator on the device (letkf_speedy_obsope) against the
oracle: phys2ijk + Trans_XtoY + the obsope.f90 range rules for every member.
qc (per member and combined) must agree exactly; hx within 1e-12 relative
(the kernel rounds every product and sum like the oracle; only log/exp may
differ by an ulp)."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, dev, dt=None):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt or torch.float64, device=dev)


def _case(seed, ne, nobs, nlon=96, nlat=48):
    rng = np.random.default_rng(seed)
    lon, lat = S.speedy_grid(nlon, nlat)
    v3d, v2d = S.speedy_members(rng, ne, nlon, nlat)
    obs = S.speedy_obs_records(rng, nobs, lon, lat, nlon)
    return lat, v3d, v2d, obs


def _check(hx, qc, qcm, ref):
    rhx, rqc, rqcm = ref
    np.testing.assert_array_equal(qcm, rqcm)
    np.testing.assert_array_equal(qc, rqc)
    scale = np.maximum(np.abs(rhx), 1e-30)
    bad = np.abs(hx - rhx) > 1e-12 * scale
    assert not bad.any(), (np.argwhere(bad)[:5], hx[bad][:5], rhx[bad][:5])


@pytest.mark.parametrize("ne,nobs", [(1, 300), (20, 2000), (40, 3000), (67, 1500)])
def test_obsope_matches_oracle(cuda, ne, nobs):
    import torch

    from letkf_gb300.core import speedy_obsope

    lat, v3d, v2d, (el, lo, la, lv, od) = _case(ne, ne, nobs)
    ref = O.speedy_obsope(lat, S.SPEEDY_SIG, v3d, v2d, el, lo, la, lv, od)
    hx, qc, qcm = speedy_obsope(_t(lat, cuda), _t(S.SPEEDY_SIG, cuda), _t(v3d, cuda), _t(v2d, cuda),
                                _t(el, cuda, torch.int32), _t(lo, cuda), _t(la, cuda), _t(lv, cuda), _t(od, cuda),
                                want_member_qc=True)
    _check(hx.cpu().numpy(), qc.cpu().numpy(), qcm.cpu().numpy(), ref)
    assert 0.3 < ref[1].mean() < 0.95


def test_obsope_analysis_layout_matches_grd_layout(cuda):
    """The das_letkf layout [4, nlev, ne, nlat*nlon] (member stride nlat*nlon)
    gives the same bits as the grd-file layout [ne, 4, nlev, nlat, nlon]."""
    import torch

    from letkf_gb300.core import speedy_obsope

    ne = 12
    lat, v3d, v2d, (el, lo, la, lv, od) = _case(5, ne, 2500)
    args = (_t(el, cuda, torch.int32), _t(lo, cuda), _t(la, cuda), _t(lv, cuda), _t(od, cuda))
    g3 = _t(v3d, cuda)
    g2 = _t(v2d, cuda)
    hx0, qc0 = speedy_obsope(_t(lat, cuda), _t(S.SPEEDY_SIG, cuda), g3, g2, *args)
    gues3d = g3.permute(1, 2, 0, 3, 4).contiguous()                   # [4, nlev, ne, nlat, nlon]
    gues2d = g2.permute(1, 0, 2, 3).contiguous()                      # [2, ne, nlat, nlon]
    hx1, qc1 = speedy_obsope(_t(lat, cuda), _t(S.SPEEDY_SIG, cuda), gues3d.permute(2, 0, 1, 3, 4),
                             gues2d.permute(1, 0, 2, 3), *args)
    assert torch.equal(hx0, hx1) and torch.equal(qc0, qc1)
    ref = O.speedy_obsope(lat, S.SPEEDY_SIG, v3d, v2d, el, lo, la, lv, od)
    _check(hx0.cpu().numpy(), qc0.cpu().numpy(), ref[2], ref)


def test_obsope_feeds_departures(cuda):
    """H(x) -> member mean, perturbations, departures and the gross-error
    check (speedy/letkf/letkf_obs.f90:155-174) on the device against the
    oracle's H(x) followed by the same arithmetic in numpy."""
    import torch

    from letkf_gb300.core import obs_departure, speedy_obsope

    ne = 32
    lat, v3d, v2d, (el, lo, la, lv, od) = _case(11, ne, 1500)
    rhx, rqc, _ = O.speedy_obsope(lat, S.SPEEDY_SIG, v3d, v2d, el, lo, la, lv, od)
    planted = np.arange(el.size) % 50 == 0
    y = rhx.mean(1) + np.where(planted, 50.0, 0.1)
    err = np.ones(el.size)
    hx, qc = speedy_obsope(_t(lat, cuda), _t(S.SPEEDY_SIG, cuda), _t(v3d, cuda), _t(v2d, cuda),
                           _t(el, cuda, torch.int32), _t(lo, cuda), _t(la, cuda), _t(lv, cuda), _t(od, cuda))
    hdxf, dep, qc2 = obs_departure(hx, _t(y, cuda), _t(err, cuda), 10.0, qc)
    mean = rhx.sum(1) / ne
    ok = rqc == 1
    want_qc = (ok & ~(np.abs(y - mean) > 10.0 * err)).astype(np.int32)
    np.testing.assert_array_equal(qc2.cpu().numpy(), want_qc)
    assert want_qc.sum() < ok.sum()                 # some gross errors were planted
    d = dep.cpu().numpy()[ok]
    np.testing.assert_allclose(d, (y - mean)[ok], rtol=1e-11, atol=1e-9)
    np.testing.assert_allclose(hdxf.cpu().numpy()[ok], (rhx - mean[:, None])[ok], rtol=1e-9, atol=1e-9)
