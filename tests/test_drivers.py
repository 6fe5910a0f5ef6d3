"""Model drivers on the device path: Lorenz-96 (lorenz96/letkf/letkf.f90:180-265)
and SPEEDY (speedy/letkf/letkf_tools.f90:44-203), against the golden L96
analysis and the oracle.  FP64 plain form: 1e-10 relative; local lists bit-exact."""
import os

import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from letkf_gb300.drivers import speedy_sort_obs, var_local_n2n
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(np.asarray(a) - b).max() / scale
    assert err <= rtol, f"relative error {err:.3e} > {rtol:.1e}"


# ------------------------------------------------------ bucket sort (device)
@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_speedy_sort_matches_oracle(cuda, seed):
    """The device bucket sort (letkf_sort_obs_latlon) equals the oracle's
    restatement of speedy/letkf/letkf_obs.f90:243-313: order and nobsgrd."""
    c = S.speedy_case(seed, nstations=150)
    # observations exactly on grid lines, next to 360, and outside the last band
    olon = np.concatenate([c["olon"], c["lon"][:6], [359.999999, 0.0, 360.0 - 1e-12]])
    olat = np.concatenate([c["olat"], c["lat"][:6], [c["lat"][-1], c["lat"][0], 89.9]])
    p1, g1 = speedy_sort_obs(c["lon"], c["lat"], olon, olat)
    p2, g2 = O.speedy_sort_obs(c["lon"], c["lat"], olon, olat)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(g1, g2)


@pytest.mark.gpu
def test_speedy_sort_empty(cuda):
    lon, lat = S.speedy_grid()
    p, g = speedy_sort_obs(lon, lat, np.zeros(0), np.zeros(0))
    assert p.size == 0 and not g.any()


@pytest.mark.gpu
def test_speedy_sort_selects_qc_on_the_device(cuda):
    """With qc the device sort keeps only qc == 1 (set_letkf_obs's selection
    before the sort): equal to the oracle sort of the selected subset."""
    import torch

    from letkf_gb300.core import sort_obs_latlon

    c = S.speedy_case(7, nstations=400)
    rng = np.random.default_rng(3)
    qc = (rng.uniform(size=c["olon"].size) < 0.8).astype(np.int32)
    f = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=cuda)
    perm, grd = sort_obs_latlon(f(c["lon"]), f(c["lat"]), f(c["olon"]), f(c["olat"]),
                                torch.as_tensor(qc, device=cuda))
    keep = np.nonzero(qc == 1)[0]
    p2, g2 = O.speedy_sort_obs(c["lon"], c["lat"], c["olon"][keep], c["olat"][keep])
    np.testing.assert_array_equal(perm.cpu().numpy(), keep[p2])
    np.testing.assert_array_equal(grd.cpu().numpy(), g2)


def test_var_local_n2n():
    vl = np.ones((6, 7))
    assert var_local_n2n(vl).tolist() == [0, 0, 0, 0, 0, 0]
    vl[2, 3] = 0.5
    vl[4] = vl[2]
    vl[5, 0] = 0.0
    assert var_local_n2n(vl).tolist() == [0, 0, 2, 0, 2, 5]


# ------------------------------------------------------------------- Lorenz-96
def _t(a, dt, dev):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,rtol", [("f64", 1e-10), ("mixed", 2e-5)])
def test_l96_analysis_matches_golden(cuda, precision, rtol):
    import torch

    from letkf_gb300.core import l96_obs_cell
    from letkf_gb300.drivers import l96_letkf

    g = np.load(os.path.join(GOLD, "l96_analysis.npz"))
    xf = _t(g["xf"], torch.float64, cuda)
    h = _t(g["h"], torch.float64, cuda)
    hxf = h @ xf
    y = _t(g["y"], torch.float64, cuda)
    cell = l96_obs_cell(h)
    assert cell.cpu().numpy().tolist() == list(range(1, 41))
    xa, infl = l96_letkf(xf, hxf, y, cell, obserr=float(g["obserr"]), precision=precision)
    _close(xa.cpu().numpy(), g["xa"], rtol)
    assert np.all(infl.cpu().numpy() == 1.05)


@pytest.mark.gpu
def test_l96_search_matches_oracle_with_shared_cells(cuda):
    """Observations scattered over the cells (several per cell, empty cells,
    a dense H with ties) on a 300-variable ring; lists in observation order."""
    import torch

    from letkf_gb300.core import l96_obs_cell, search_l96

    rng = np.random.default_rng(5)
    nx, ny = 300, 420
    cells = rng.integers(1, nx + 1, ny)
    h = np.zeros((ny, nx))
    h[np.arange(ny), cells - 1] = 1.0
    ties = rng.choice(ny, 30, replace=False)
    h[ties, (cells[ties] + 7) % nx] = 1.0      # a tie: the first maximum wins
    cell = l96_obs_cell(_t(h, torch.float64, cuda))
    ref_cell = np.array([np.nonzero(h[i] == h[i].max())[0][0] + 1 for i in range(ny)])
    np.testing.assert_array_equal(cell.cpu().numpy(), ref_cell)
    for xlocal in (3.0, 0.7, 40.0):
        pix = torch.arange(1, nx + 1, dtype=torch.int32, device=cuda)
        offs, idx, rloc, rdiag = search_l96(nx, cell, pix, xlocal, obserr=0.5)
        offs, idx, rloc = offs.cpu().numpy(), idx.cpu().numpy(), rloc.cpu().numpy()
        assert np.all(rdiag.cpu().numpy() == 0.25)
        for ix in range(1, nx + 1):
            ri, rl = O.l96_select(h, ix, xlocal)
            s = slice(offs[ix - 1], offs[ix])
            np.testing.assert_array_equal(idx[s], ri, err_msg=f"ix {ix} xlocal {xlocal}")
            np.testing.assert_allclose(rloc[s], rl, rtol=1e-14)


@pytest.mark.gpu
def test_l96_search_small_ring_and_no_obs(cuda):
    """A ring shorter than the cut-off window visits every cell once; no
    observations gives empty lists."""
    import torch

    from letkf_gb300.core import search_l96

    nx = 12
    h = np.eye(nx)
    cell = torch.arange(1, nx + 1, dtype=torch.int32, device=cuda)
    pix = torch.arange(1, nx + 1, dtype=torch.int32, device=cuda)
    offs, idx, rloc, _ = search_l96(nx, cell, pix, 3.0)
    offs, idx = offs.cpu().numpy(), idx.cpu().numpy()
    for ix in range(1, nx + 1):
        ri, _ = O.l96_select(h, ix, 3.0)
        np.testing.assert_array_equal(idx[offs[ix - 1]:offs[ix]], ri)
    offs, idx, _, _ = search_l96(nx, torch.zeros(0, dtype=torch.int32, device=cuda), pix, 3.0)
    assert offs.cpu().numpy().tolist() == [0] * (nx + 1)


@pytest.mark.gpu
def test_obs_departure_matches_sequential_mean(cuda):
    import torch

    from letkf_gb300.core import obs_departure

    rng = np.random.default_rng(3)
    for ne in (20, 64, 130):
        nobs = 1000 + ne
        hx = rng.standard_normal((nobs, ne)) * 3 + 10
        y = rng.standard_normal(nobs) * 2 + 10
        err = rng.uniform(0.1, 1.0, nobs)
        qc_in = (rng.uniform(size=nobs) > 0.1).astype(np.int32)
        hdxf, dep, qc = obs_departure(_t(hx, torch.float64, cuda), _t(y, torch.float64, cuda),
                                      _t(err, torch.float64, cuda), 3.0, _t(qc_in, torch.int32, cuda))
        hdxf, dep, qc = hdxf.cpu().numpy(), dep.cpu().numpy(), qc.cpu().numpy()
        for n in range(nobs):
            if qc_in[n] != 1:
                assert qc[n] == 0 and dep[n] == 0.0
                np.testing.assert_array_equal(hdxf[n], hx[n])
                continue
            s = hx[n, 0]
            for m in range(1, ne):
                s = s + hx[n, m]
            s = s / ne
            assert dep[n] == y[n] - s
            np.testing.assert_array_equal(hdxf[n], hx[n] - s)
            assert qc[n] == (0 if abs(y[n] - s) > 3.0 * err[n] else 1)


# ---------------------------------------------------------------------- SPEEDY
@pytest.mark.gpu
def test_speedy_das_letkf_matches_oracle(cuda):
    """Full 96x48x7 SPEEDY-grid analysis of u, v, t, q (k = 40) on the device;
    a subset of points checked against the oracle's obs_local + letkf_core +
    update, including the no-analysis of upper-level q."""
    import torch

    from letkf_gb300.drivers import speedy_letkf

    c = S.speedy_case(4, nstations=300)
    perm, grd = speedy_sort_obs(c["lon"], c["lat"], c["olon"], c["olat"])
    srt = {k: c[k][perm] for k in ("elm", "olon", "olat", "olev", "odat", "oerr")}
    hdxf, dep = c["hdxf"][perm], c["dep"][perm]
    f = lambda a: _t(a, torch.float64, cuda)
    grid = {"lon": f(c["lon"]), "lat": f(c["lat"]), "nobsgrd": _t(grd, torch.int32, cuda)}
    obs = {"elm": f(srt["elm"]), "lon": f(srt["olon"]), "lat": f(srt["olat"]), "lev": f(srt["olev"]),
           "dat": f(srt["odat"]), "err": f(srt["oerr"])}
    params = (c["dist_zero"], c["dist_zerov"], c["dlat_zero"], c["sigma_obs"], c["sigma_obsv"])
    nv3d, nlev, ne, nij = c["gues3d"].shape
    var_local = np.ones((nv3d, 7))
    infl = torch.full((nv3d, nlev, nij), 1.1, dtype=torch.float64, device=cuda)
    anal3d, _ = speedy_letkf(grid, obs, f(hdxf), f(dep), f(c["gues3d"]), f(c["logpfm"]), f(c["dlon_zero"]), params,
                             var_local, infl)
    anal3d = anal3d.cpu().numpy()
    infl = infl.cpu().numpy()
    so = O.SpeedyObs(c["lon"], c["lat"], grd, srt["elm"], srt["olon"], srt["olat"], srt["olev"], srt["odat"],
                     srt["oerr"], c["dist_zero"], c["dist_zerov"], c["dlat_zero"], c["sigma_obs"], c["sigma_obsv"],
                     var_local[0])
    checked = 0
    for p in range(0, nlev * nij, 53):
        ilev, ij = divmod(p, nij)
        ri, rl, rd = so.obs_local(c["glon"][ij], c["glat"][ij], c["dlon_zero"][ij], ilev + 1, c["logpfm"][ilev, ij])
        r = O.letkf_core(hdxf[ri] if ri.size else np.zeros((1, ne)), rd if ri.size else np.ones(1),
                         rl if ri.size else np.ones(1), dep[ri] if ri.size else np.zeros(1), 1.1, nobsl=ri.size)
        assert abs(infl[0, ilev, ij] - r["parm_infl"]) <= 1e-10 * abs(r["parm_infl"])
        for n in range(nv3d):
            xb = c["gues3d"][n, ilev, :, ij]
            m = xb[0]
            for k in range(1, ne):
                m = m + xb[k]
            m = m / ne
            xp = xb - m
            ref = m + xp @ (np.eye(ne) if (n == 3 and ilev + 1 >= 5) else r["trans"])
            _close(anal3d[n, ilev, :, ij], ref, 1e-10)
        checked += 1
    assert checked > 40


# ---------------------------------------------------------------- 4D Lorenz-96
@pytest.mark.gpu
@pytest.mark.parametrize("tlocal", [2.0, -1.0, 0.7])
def test_l96_search_4d_matches_oracle(cuda, tlocal):
    """4D selection (lorenz96/letkf/letkf.f90:217-254): three slots with their
    own H (scattered cells, ties), every analysis slot, lists in slot and
    observation order with tdif = |nn - n|."""
    import torch

    from letkf_gb300.core import l96_obs_cell, search_l96_4d

    rng = np.random.default_rng(17)
    nslot, nx, ny = 3, 120, 150
    h4d = np.zeros((nslot, ny, nx))
    for n in range(nslot):
        cells = rng.integers(1, nx + 1, ny)
        h4d[n, np.arange(ny), cells - 1] = 1.0
        ties = rng.choice(ny, 10, replace=False)
        h4d[n, ties, (cells[ties] + 5) % nx] = 1.0
    cell = torch.stack([l96_obs_cell(_t(h4d[n], torch.float64, cuda)) for n in range(nslot)])
    pix = torch.arange(1, nx + 1, dtype=torch.int32, device=cuda)
    for slot in range(nslot):
        offs, idx, rloc, rdiag = search_l96_4d(nx, cell, pix, slot, 3.0, 0.5, tlocal)
        offs, idx, rloc = offs.cpu().numpy(), idx.cpu().numpy(), rloc.cpu().numpy()
        assert np.all(rdiag.cpu().numpy() == 0.25)
        for ix in range(1, nx + 1):
            ri, rl = O.l96_select_4d(h4d, slot + 1, ix, 3.0, tlocal)
            s = slice(offs[ix - 1], offs[ix])
            np.testing.assert_array_equal(idx[s], ri, err_msg=f"slot {slot} ix {ix}")
            np.testing.assert_allclose(rloc[s], rl, rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_l96_letkf_4d_matches_oracle(cuda):
    """Two-slot 4D-LETKF analysis (nwindow = 2, fixed localisation and
    inflation) on the Lorenz-96 ring against the oracle's selection + core +
    update of each analysis slot."""
    import torch

    from letkf_gb300.core import l96_obs_cell
    from letkf_gb300.drivers import l96_letkf_4d

    rng = np.random.default_rng(23)
    nslot, nx, ne = 2, 40, 20
    xf = 8.0 + 2.0 * rng.standard_normal((nslot, nx, ne))
    h = np.eye(nx)
    hxf = np.stack([h @ xf[n] for n in range(nslot)])
    y = 8.0 + rng.standard_normal((nslot, nx))
    h4d = np.stack([h, h])
    cell = torch.stack([l96_obs_cell(_t(h, torch.float64, cuda))] * nslot)
    xa, infl = l96_letkf_4d(_t(xf, torch.float64, cuda), _t(hxf, torch.float64, cuda), _t(y, torch.float64, cuda),
                            cell, obserr=1.0, xlocal=3.0, tlocal=2.0)
    xa = xa.cpu().numpy()
    assert np.all(infl.cpu().numpy() == 1.05)
    # oracle: per-slot departures, then every analysis slot over both slots' observations
    hdxf, dep = [], []
    for n in range(nslot):
        m = hxf[n][:, 0].copy()
        for k in range(1, ne):
            m = m + hxf[n][:, k]
        m = m / ne
        hdxf.append(hxf[n] - m[:, None])
        dep.append(y[n] - m)
    hdxf, dep = np.concatenate(hdxf), np.concatenate(dep)
    for nn in range(nslot):
        xm = xf[nn][:, 0].copy()
        for k in range(1, ne):
            xm = xm + xf[nn][:, k]
        xm = xm / ne
        for ix in range(1, nx + 1):
            ri, rl = O.l96_select_4d(h4d, nn + 1, ix, 3.0, 2.0)
            r = O.letkf_core(hdxf[ri], np.ones(ri.size), rl, dep[ri], 1.05)
            ref = xm[ix - 1] + (xf[nn][ix - 1] - xm[ix - 1]) @ r["trans"]
            _close(xa[nn, ix - 1], ref, 1e-10)


def test_oracle_l96_select_4d_reduces_to_one_slot_and_weights_time():
    """One slot equals the single-slot selection; further slots repeat the
    spatial weights times exp(-0.5 (tdif/tlocal)^2) in slot order."""
    nx = 40
    h = np.eye(nx)
    i1, r1 = O.l96_select(h, 7, 3.0, 2.0)
    i4, r4 = O.l96_select_4d(h[None], 1, 7, 3.0, 2.0)
    np.testing.assert_array_equal(i1, i4)
    np.testing.assert_array_equal(r1, r4)
    i3, r3 = O.l96_select_4d(np.stack([h, h, h]), 2, 7, 3.0, 2.0)
    n = i1.size
    assert i3.size == 3 * n
    np.testing.assert_array_equal(i3[:n], i1)
    np.testing.assert_array_equal(i3[n:2 * n], i1 + nx)
    np.testing.assert_allclose(r3[n:2 * n], r1, rtol=1e-15)                       # tdif = 0
    np.testing.assert_allclose(r3[:n], r1 * np.exp(-0.5 * 0.25), rtol=1e-15)       # tdif = 1
    _, rneg = O.l96_select_4d(np.stack([h, h, h]), 2, 7, 3.0, -1.0)
    np.testing.assert_allclose(rneg[:n], r1, rtol=1e-15)                          # no time localisation


# -------------------------------------------------- adaptive localisation (L96)
def _np_correl(a, b):
    return np.corrcoef(a, b)[0, 1]


def _l96_adapt_case(seed, nslot=1, nx=40, ny=40, ne=20):
    """Random H with one cell per observation, correlated members: returns
    (h4d, hdxf [nslot*ny, ne], xf [nslot, nx, ne])."""
    rng = np.random.default_rng(seed)
    h4d = np.zeros((nslot, ny, nx))
    for n in range(nslot):
        cells = rng.integers(1, nx + 1, ny)
        h4d[n, np.arange(ny), cells - 1] = 1.0
    xf = 8.0 + 2.0 * rng.standard_normal((nslot, nx, ne))
    hd = []
    for n in range(nslot):
        hx = h4d[n] @ xf[n] + 0.3 * rng.standard_normal((ny, ne))
        m = hx[:, 0].copy()
        for k in range(1, ne):
            m = m + hx[:, k]
        hd.append(hx - (m / ne)[:, None])
    return h4d, np.concatenate(hd), xf


def _dxf(xrow):
    m = xrow[0]
    for v in xrow[1:]:
        m = m + v
    return xrow - m / xrow.size


def test_oracle_l96_adaptive_mode0_is_the_fixed_selection():
    h4d, hdxf, xf = _l96_adapt_case(3, nslot=3)
    for ix in (1, 17, 40):
        for slot in (1, 2, 3):
            i0, r0 = O.l96_select_4d(h4d, slot, ix, 3.0, 2.0)
            i1, r1 = O.l96_select_adaptive(h4d, hdxf, _dxf(xf[slot - 1, ix - 1]), slot, ix, 0)
            np.testing.assert_array_equal(i0, i1)
            np.testing.assert_array_equal(r0, r1)


@pytest.mark.parametrize("mode,sa,sb", [(1, 1.0, 1.0), (2, 1.0, 1.0), (1, 0.5, 2.0), (2, 2.0, 0.5)])
def test_oracle_l96_adaptive_weights_are_the_correlations(mode, sa, sb):
    """msw_local 1/2 (lorenz96/letkf/letkf.f90:237-249) against numpy's
    correlation coefficients: every observation within xmaxloc is a candidate,
    weighted wa**sa * wb**sb (times the fixed weights in mode 2), kept from 1e-4."""
    nslot, ne = 2, 21          # odd k: ceil(k/2) = 11 members in the first half
    h4d, hdxf, xf = _l96_adapt_case(5, nslot=nslot, ne=ne)
    nx, ny = h4d.shape[2], h4d.shape[1]
    xmaxloc = 3.0 * 2.0 * np.sqrt(10.0 / 3.0)
    for slot in (1, 2):
        for ix in (1, 9, 33):
            d = _dxf(xf[slot - 1, ix - 1])
            idx, rloc = O.l96_select_adaptive(h4d, hdxf, d, slot, ix, mode, sa, sb)
            exp_i, exp_r = [], []
            for n in range(nslot):
                for i in range(ny):
                    j = int(np.argmax(h4d[n, i])) + 1
                    dist = min(abs(j - ix), nx - abs(j - ix))
                    if dist >= xmaxloc:
                        continue
                    row = hdxf[n * ny + i]
                    c1 = _np_correl(row[:11], d[:11])
                    c2 = _np_correl(row[11:], d[11:])
                    c3 = _np_correl(row, d)
                    r = (1.0 - 0.5 * abs(c1 - c2)) ** sa * abs(c3) ** sb
                    if mode == 2:
                        r *= np.exp(-0.5 * (dist / 3.0) ** 2) * np.exp(-0.5 * (abs(slot - 1 - n) / 2.0) ** 2)
                    if r >= 1e-4:
                        exp_i.append(n * ny + i)
                        exp_r.append(r)
            np.testing.assert_array_equal(idx, exp_i)
            np.testing.assert_allclose(rloc, exp_r, rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("nslot,mode,sa,sb", [(1, 1, 1.0, 1.0), (1, 2, 1.0, 1.0), (3, 1, 1.0, 1.0),
                                               (3, 2, 0.5, 2.0), (3, 0, 1.0, 1.0), (1, 1, 2.0, 0.5)])
def test_l96_search_adaptive_matches_oracle(cuda, nslot, mode, sa, sb):
    """Device selection with msw_local against the oracle for every point and
    analysis slot: lists bit-exact; weights bit-exact with sa = sb = 1 (the
    same rounded operations), within 1e-14 otherwise (pow)."""
    import torch

    from letkf_gb300.core import l96_obs_cell, search_l96_adaptive

    ne = 21
    h4d, hdxf, xf = _l96_adapt_case(11 + nslot + mode, nslot=nslot, nx=60, ny=70, ne=ne)
    nx = h4d.shape[2]
    cell = torch.stack([l96_obs_cell(_t(h4d[n], torch.float64, cuda)) for n in range(nslot)])
    pix = torch.arange(1, nx + 1, dtype=torch.int32, device=cuda)
    hd = _t(hdxf, torch.float64, cuda)
    for slot in range(nslot):
        offs, idx, rloc, rdiag = search_l96_adaptive(nx, cell, pix, slot, hd, _t(xf[slot], torch.float64, cuda),
                                                     mode, sa, sb, 3.0, 0.5, 2.0)
        offs, idx, rloc = offs.cpu().numpy(), idx.cpu().numpy(), rloc.cpu().numpy()
        assert np.all(rdiag.cpu().numpy() == 0.25)
        for ix in range(1, nx + 1):
            ri, rl = O.l96_select_adaptive(h4d, hdxf, _dxf(xf[slot, ix - 1]), slot + 1, ix, mode, sa, sb)
            s = slice(offs[ix - 1], offs[ix])
            np.testing.assert_array_equal(idx[s], ri, err_msg=f"slot {slot} ix {ix}")
            if mode == 1 and sa == 1.0 and sb == 1.0:
                np.testing.assert_array_equal(rloc[s], rl)
            else:
                np.testing.assert_allclose(rloc[s], rl, rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_l96_search_adaptive_rejects_unknown_mode(cuda):
    import torch

    from letkf_gb300.core import search_l96_adaptive
    from letkf_gb300.lib import LETKF_ERR_ARG, LetkfError

    cell = torch.ones(4, dtype=torch.int32, device=cuda)
    pix = torch.arange(1, 9, dtype=torch.int32, device=cuda)
    with pytest.raises(LetkfError) as e:
        search_l96_adaptive(8, cell, pix, 0, torch.zeros(4, 6, dtype=torch.float64, device=cuda),
                            torch.zeros(8, 6, dtype=torch.float64, device=cuda), 3)
    assert e.value.status == LETKF_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_l96_letkf_adaptive_matches_oracle(cuda, mode):
    """Lorenz-96 analysis with adaptive localisation (msw_local 1, 2) against
    the oracle's selection + core + update at every point (FP64, 1e-10)."""
    import torch

    from letkf_gb300.core import l96_obs_cell
    from letkf_gb300.drivers import l96_letkf

    rng = np.random.default_rng(29 + mode)
    nx, ne = 40, 20
    xf = 8.0 + 2.0 * rng.standard_normal((nx, ne))
    h = np.eye(nx)[::2]                               # every other variable observed
    hxf = h @ xf
    y = 8.0 + rng.standard_normal(h.shape[0])
    cell = l96_obs_cell(_t(h, torch.float64, cuda))
    xa, infl = l96_letkf(_t(xf, torch.float64, cuda), _t(hxf, torch.float64, cuda), _t(y, torch.float64, cuda),
                         cell, obserr=1.0, xlocal=3.0, msw_local=mode)
    xa = xa.cpu().numpy()
    assert np.all(infl.cpu().numpy() == 1.05)
    m = hxf[:, 0].copy()
    for k in range(1, ne):
        m = m + hxf[:, k]
    m = m / ne
    hdxf, dep = hxf - m[:, None], y - m
    for ix in range(1, nx + 1):
        d = _dxf(xf[ix - 1])
        ri, rl = O.l96_select_adaptive(h, hdxf, d, 1, ix, mode)
        r = O.letkf_core(hdxf[ri], np.ones(ri.size), rl, dep[ri], 1.05)
        ref = (xf[ix - 1] - d) + d @ r["trans"]
        _close(xa[ix - 1], ref, 1e-10)


@pytest.mark.gpu
def test_l96_letkf_4d_adaptive_matches_oracle(cuda):
    """Two-slot 4D-LETKF with msw_local = 2 against the oracle chain."""
    import torch

    from letkf_gb300.core import l96_obs_cell
    from letkf_gb300.drivers import l96_letkf_4d

    rng = np.random.default_rng(31)
    nslot, nx, ne = 2, 40, 20
    xf = 8.0 + 2.0 * rng.standard_normal((nslot, nx, ne))
    h = np.eye(nx)
    hxf = np.stack([h @ xf[n] for n in range(nslot)])
    y = 8.0 + rng.standard_normal((nslot, nx))
    cell = torch.stack([l96_obs_cell(_t(h, torch.float64, cuda))] * nslot)
    xa, _ = l96_letkf_4d(_t(xf, torch.float64, cuda), _t(hxf, torch.float64, cuda), _t(y, torch.float64, cuda),
                         cell, obserr=1.0, xlocal=3.0, tlocal=2.0, msw_local=2)
    xa = xa.cpu().numpy()
    hdxf, dep = [], []
    for n in range(nslot):
        m = hxf[n][:, 0].copy()
        for k in range(1, ne):
            m = m + hxf[n][:, k]
        m = m / ne
        hdxf.append(hxf[n] - m[:, None])
        dep.append(y[n] - m)
    hdxf, dep = np.concatenate(hdxf), np.concatenate(dep)
    h4d = np.stack([h, h])
    for nn in range(nslot):
        for ix in range(1, nx + 1):
            d = _dxf(xf[nn, ix - 1])
            ri, rl = O.l96_select_adaptive(h4d, hdxf, d, nn + 1, ix, 2, 1.0, 1.0, 3.0, 2.0)
            r = O.letkf_core(hdxf[ri], np.ones(ri.size), rl, dep[ri], 1.05)
            ref = (xf[nn, ix - 1] - d) + d @ r["trans"]
            _close(xa[nn, ix - 1], ref, 1e-10)
