"""Known answers of the oracle's SPEEDY observation operator (phys2ijk,
Trans_XtoY, calc_rh, itpl_2d/3d of speedy/common/common_obs_speedy.f90 and the
range rules of speedy/letkf/obsope.f90:53-104) on fields whose interpolants
are known in closed form."""
import math

import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

NLON, NLAT, NLEV = 96, 48, 7
LON, LAT = S.speedy_grid(NLON, NLAT)
SIG = S.SPEEDY_SIG
U, V, T, Q, RH, PS, RAIN = S.ID_U, S.ID_V, S.ID_T, S.ID_Q, S.ID_RH, S.ID_PS, S.ID_RAIN


def _linear_state(ne=2, a=0.5, b=-0.25, c=3.0, ps=1.0e5):
    """u = a i + b j + c k (1-based), every member alike; t, q constant."""
    i = np.arange(1, NLON + 1)[None, None, :]
    j = np.arange(1, NLAT + 1)[None, :, None]
    k = np.arange(1, NLEV + 1)[:, None, None]
    u = a * i + b * j + c * k + 0.0 * (i + j + k)
    v3d = np.zeros((ne, 4, NLEV, NLAT, NLON))
    v3d[:, 0] = u
    v3d[:, 1] = -u
    v3d[:, 2] = 260.0
    v3d[:, 3] = 2.0e-3
    v2d = np.zeros((ne, 2, NLAT, NLON))
    v2d[:, 0] = ps
    v2d[:, 1] = a * i[0] + b * j[0]
    return v3d, v2d


def _rj(rlat):
    j = int(np.searchsorted(LAT, rlat, side="right"))
    return j + (rlat - LAT[j - 1]) / (LAT[j] - LAT[j - 1])


def _calc_rh(t, q, p):
    e = q * p * 0.01 / (0.378 * q + 0.622)
    tc = t - 273.15
    esw = 6.11 * math.exp(17.3 * tc / (237.3 + tc))
    esi = 6.1121 * math.exp(22.587 * tc / (273.86 + tc))
    if tc >= 0.0:
        es = esw
    elif tc <= -15.0:
        es = esi
    else:
        es = esw * (15.0 + tc) / 15.0 + esi * (-tc) / 15.0
    return e / es


def _run(v3d, v2d, elem, rlon, rlat, rlev, odat=None):
    n = len(elem)
    odat = np.zeros(n) if odat is None else np.asarray(odat, float)
    return O.speedy_obsope(LAT, SIG, v3d, v2d, np.asarray(elem), np.asarray(rlon, float), np.asarray(rlat, float),
                           np.asarray(rlev, float), odat)


def test_linear_field_is_reproduced_at_full_levels():
    v3d, v2d = _linear_state()
    rng = np.random.default_rng(1)
    n = 40
    rlon = rng.uniform(5.0, 350.0, n)
    rlat = rng.uniform(-80.0, 80.0, n)
    kk = rng.integers(2, NLEV + 1, n)
    rlev = 1.0e5 * SIG[kk - 1]
    hx, qc, _ = _run(v3d, v2d, [U] * n, rlon, rlat, rlev)
    assert qc.all()
    ri = rlon / 360.0 * NLON + 1.0
    rj = np.array([_rj(x) for x in rlat])
    want = 0.5 * ri - 0.25 * rj + 3.0 * kk
    np.testing.assert_allclose(hx[:, 0], want, rtol=1e-12, atol=1e-9)
    np.testing.assert_array_equal(hx[:, 0], hx[:, 1])
    hv, _, _ = _run(v3d, v2d, [V] * n, rlon, rlat, rlev)
    np.testing.assert_allclose(hv[:, 0], -want, rtol=1e-12, atol=1e-9)


def test_log_pressure_interpolation_between_levels():
    """With ps uniform, plev(k) = ln(ps sig(k)) and rk is linear in ln p."""
    v3d, v2d = _linear_state(c=1.0, a=0.0, b=0.0)
    k0 = 3
    frac = 0.3
    lnp = (1 - frac) * math.log(1.0e5 * SIG[k0 - 1]) + frac * math.log(1.0e5 * SIG[k0])
    hx, qc, _ = _run(v3d, v2d, [T, U], [100.0, 100.0], [10.0, 10.0], [math.exp(lnp)] * 2)
    assert qc.tolist() == [1, 1]
    assert hx[0, 0] == 260.0 or abs(hx[0, 0] - 260.0) < 1e-10
    assert abs(hx[1, 0] - (k0 + frac)) < 1e-12


def test_longitude_wrap_and_exact_zero_and_360():
    v3d, v2d = _linear_state(a=1.0, b=0.0, c=0.0)
    lo = 360.0 - 0.4 * 360.0 / NLON
    hx, qc, _ = _run(v3d, v2d, [U, U, U, RAIN], [lo, 0.0, 360.0, lo], [20.0] * 4, [5.0e4] * 4)
    assert qc.all()
    ai = lo / 360.0 * NLON + 1.0 - NLON
    assert abs(hx[0, 0] - ((1 - ai) * NLON + ai * 1.0)) < 1e-9
    # lon 0 and 360 map to ri = nlon + 1: the wrapped column 1 with weight 1
    assert hx[1, 0] == pytest.approx(1.0, abs=1e-12)
    assert hx[2, 0] == pytest.approx(1.0, abs=1e-12)
    assert abs(hx[3, 0] - ((1 - ai) * NLON + ai * 1.0)) < 1e-9


def test_relative_humidity_at_full_levels_every_branch():
    ps = 1.0e5
    for tval in (290.0, 265.0, 250.0):       # tc >= 0, -15 < tc < 0, tc <= -15
        v3d, v2d = _linear_state(ps=ps)
        v3d[:, 2] = tval
        k0 = 4
        hx, qc, _ = _run(v3d, v2d, [RH], [45.0], [30.0], [ps * SIG[k0 - 1]])
        assert qc[0] == 1
        assert hx[0, 0] == pytest.approx(_calc_rh(tval, 2.0e-3, ps * SIG[k0 - 1]), rel=1e-12)
        assert O.speedy_calc_rh(tval, 2.0e-3, ps * SIG[k0 - 1]) == pytest.approx(
            _calc_rh(tval, 2.0e-3, ps * SIG[k0 - 1]), rel=1e-14)


def test_vertical_range_rules():
    v3d, v2d = _linear_state(a=0.0, b=0.0, c=1.0)
    below, above = 1.1e5, 5.0e3
    elem = [U, V, T, Q, RH, RAIN, U, T]
    rlev = [below] * 6 + [above, above]
    hx, qc, _ = _run(v3d, v2d, elem, [50.0] * 8, [0.0] * 8, rlev)
    # u/v below the lowest full level are clamped to rk = 1.00001; the rest are rejected
    assert qc.tolist() == [1, 1, 0, 0, 0, 0, 0, 0]
    assert hx[0, 0] == pytest.approx(1.0 + 1e-5, abs=1e-12)
    assert hx[1, 0] == pytest.approx(-(1.0 + 1e-5), abs=1e-12)
    assert (hx[2:] == 0.0).all()


def test_surface_pressure_and_missing_value():
    v3d, v2d = _linear_state()
    hx, qc, _ = _run(v3d, v2d, [PS, PS], [120.0, 120.0], [-30.0, -30.0], [0.0, 0.0], odat=[1.0e5, -999.0])
    assert qc.tolist() == [1, 0]
    assert hx[0, 0] == pytest.approx(1.0e5, rel=1e-14)
    assert hx[1, 0] == 0.0


def test_latitude_edges_and_nonpositive_level_and_unknown_code():
    v3d, v2d = _linear_state()
    elem = [U, U, U, U, 1234, T]
    rlat = [LAT[0], LAT[-1], -89.0, 89.0, 10.0, 10.0]
    rlev = [5.0e4] * 5 + [0.0]
    hx, qc, _ = _run(v3d, v2d, elem, [77.0] * 6, rlat, rlev)
    # rj = 1 exactly at lat(1): CEILING < 2, rejected; lat(nlat): rj = nlat, kept;
    # south of lat(1) / north of lat(nlat) (except on it) fall outside
    assert qc.tolist() == [0, 1, 0, 0, 1, 0]
    assert hx[4, 0] == 0.0


def test_member_qc_combines_by_minimum():
    """A level between two members' lowest full levels: kept for one member,
    rejected for the other; qc is the minimum."""
    v3d, v2d = _linear_state(ne=2)
    v2d[0, 0] = 1.00e5
    v2d[1, 0] = 0.95e5
    p = 0.5 * (1.00e5 + 0.95e5) * SIG[0]       # below member 1's lowest level, above member 0's
    hx, qc, qcm = _run(v3d, v2d, [T], [30.0], [30.0], [p])
    assert qcm[0].tolist() == [1, 0]
    assert qc[0] == 0
    assert hx[0, 1] == 0.0 and hx[0, 0] == pytest.approx(260.0, rel=1e-12)
