"""The SPEEDY letkf program on the device (drivers.speedy_cycle): member grd
files + an observation file -> H(x) -> departures and QC -> bucket sort ->
das_letkf -> analysis files, inflation file, mean/spread files.  Checked
against the oracle chain (obsope H(x), set_letkf_obs arithmetic, bucket
sort, obs_local + letkf_core + update) on the same REAL(4) file values."""
import os

import numpy as np
import pytest

from letkf_gb300 import speedy_io as IO
from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ERR = {S.ID_U: 1.0, S.ID_V: 1.0, S.ID_T: 1.0, S.ID_Q: 1.0e-3, S.ID_RH: 0.1, S.ID_PS: 100.0, S.ID_RAIN: 1.0e-4}


def test_speedy_cycle_files_match_oracle(cuda, tmp_path):
    from letkf_gb300.drivers import GROSS_ERROR, speedy_cycle, speedy_localization

    rng = np.random.default_rng(21)
    ne, nlon, nlat, nlev = 16, 96, 48, 7
    lon, lat = S.speedy_grid(nlon, nlat)
    sig = S.SPEEDY_SIG
    v3d, v2d = S.speedy_members(rng, ne, nlon, nlat, nlev)
    gues = []
    for m in range(ne):
        p = str(tmp_path / f"gs01{m + 1:03d}.grd")
        IO.write_grd4(p, v3d[m], v2d[m])
        gues.append(p)
    f3 = v3d.astype(np.float32).astype(np.float64)
    f2 = v2d.astype(np.float32).astype(np.float64)
    el, lo, la, lv, _ = S.speedy_obs_records(rng, 1200, lon, lat, nlon, with_edges=False)
    hx0, qc0, _ = O.speedy_obsope(lat, sig, f3, f2, el, lo, la, lv, np.zeros(el.size))
    err = np.array([ERR[int(e)] for e in el])
    y = hx0.mean(1) + err * rng.standard_normal(el.size)
    y[::97] += 40.0 * err[::97]                        # gross errors
    op = str(tmp_path / "obs01.dat")
    IO.write_obs(op, el, lo, la, lv, y, err)
    anal = [str(tmp_path / f"anal{m + 1:03d}.grd") for m in range(ne)]
    infl_path = str(tmp_path / "infl_mul.grd")
    out = speedy_cycle(gues, op, anal, lon, lat, sig, infl_path=infl_path, cov_infl_mul=-1.01, sigma_obs=1000.0e3,
                       sigma_obsv=0.1, mean_spread_prefix=str(tmp_path) + os.sep, device=cuda)

    # ---- oracle chain on the values the files hold
    obs = IO.read_obs(op)
    e_i = np.rint(obs["elem"]).astype(np.int32)
    rhx, rqc, _ = O.speedy_obsope(lat, sig, f3, f2, e_i, obs["lon"], obs["lat"], obs["lev"], obs["dat"])
    mean = rhx[:, 0].copy()
    for m in range(1, ne):
        mean = mean + rhx[:, m]
    mean = mean / ne
    dep = obs["dat"] - mean
    qc = (rqc == 1) & ~(np.abs(dep) > GROSS_ERROR * obs["err"])
    assert qc.sum() < (rqc == 1).sum()
    keep = np.nonzero(qc)[0]
    perm, grd = O.speedy_sort_obs(lon, lat, obs["lon"][keep], obs["lat"][keep])
    order = keep[perm]
    assert out["nobs_assimilated"] == order.size
    hdxf = rhx[order] - mean[order, None]
    params, dlon_zero = speedy_localization(lat, 1000.0e3, 0.1, nlon)
    so = O.SpeedyObs(lon, lat, grd, obs["elem"][order], obs["lon"][order], obs["lat"][order], obs["lev"][order],
                     obs["dat"][order], obs["err"][order], *params, np.ones(7))
    nij = nlon * nlat
    gues3d = f3.reshape(ne, 4, nlev, nij).transpose(1, 2, 0, 3)          # [4, nlev, ne, nij]
    ps = f2[:, 0].reshape(ne, nij)
    mps = ps[0].copy()
    for m in range(1, ne):
        mps = mps + ps[m]
    mps = mps / ne
    logpfm = np.log(mps[None, :] * sig[:, None])
    a3 = out["anal3d"].cpu().numpy()
    infl = out["infl3d"].cpu().numpy()
    checked = 0
    for p in range(0, nlev * nij, 61):
        ilev, ij = divmod(p, nij)
        glon, glat = lon[ij % nlon], lat[ij // nlon]
        ri, rl, rd = so.obs_local(glon, glat, dlon_zero[ij], ilev + 1, logpfm[ilev, ij])
        r = O.letkf_core(hdxf[ri] if ri.size else np.zeros((1, ne)), rd if ri.size else np.ones(1),
                         rl if ri.size else np.ones(1), dep[order][ri] if ri.size else np.zeros(1), 1.01,
                         nobsl=ri.size)
        assert abs(infl[0, ilev, ij] - r["parm_infl"]) <= 1e-9 * abs(r["parm_infl"])
        for n in range(4):
            xb = gues3d[n, ilev, :, ij]
            mb = xb[0]
            for k in range(1, ne):
                mb = mb + xb[k]
            mb = mb / ne
            w = np.eye(ne) if (n == 3 and ilev + 1 >= 5) else r["trans"]
            ref = mb + (xb - mb) @ w
            np.testing.assert_allclose(a3[n, ilev, :, ij], ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
        checked += 1
    assert checked > 100

    # ---- files: analyses are the device result rounded to REAL(4); inflation written back
    for m in (0, ne - 1):
        w3, _ = IO.read_grd4(anal[m], nlon, nlat, nlev)
        assert np.array_equal(w3.reshape(4, nlev, nij), a3[:, :, m, :].astype(np.float32))
    i3, _ = IO.read_grd4(infl_path, nlon, nlat, nlev)
    assert np.array_equal(i3.reshape(4, nlev, nij), infl.astype(np.float32))
    for tag in ("gues_me", "gues_sp", "anal_me", "anal_sp"):
        assert os.path.getsize(str(tmp_path / f"{tag}.grd")) == IO.grd_nbytes(nlon, nlat, nlev)
    # a second cycle reads the inflation field back
    out2 = speedy_cycle(anal, op, [a + ".2" for a in anal], lon, lat, sig, infl_path=infl_path, cov_infl_mul=-1.01,
                        device=cuda)
    assert out2["nobs_assimilated"] > 0
