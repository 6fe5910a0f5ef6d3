"""Host-side drivers that replace the reference's das_letkf grid loops with
the device path of this library (search -> gather -> batched core -> update).

* ``l96_letkf``   -- lorenz96/letkf/letkf.f90:180-265 (one time slot)
* ``l96_letkf_4d`` -- the same with nwindow > 1 time slots (4D-LETKF)
* ``speedy_letkf`` -- speedy/letkf/letkf_tools.f90:44-203 (das_letkf)
* ``speedy_sort_obs`` -- speedy/letkf/letkf_obs.f90:243-313 (bucket sort)
* ``speedy_obs_setup`` -- set_letkf_obs (speedy/letkf/letkf_obs.f90:48-313) with
  H(x) of every member computed on the device (obsope.f90)
* ``speedy_cycle`` -- the letkf program (speedy/letkf/letkf.f90) from member grd
  files and an observation file to analysis files

* ``scale_obs_setup`` -- set_letkf_obs of the SCALE driver for conventional
  observations with H(x) of every member computed on the device (obsope_cal)

The regional SCALE-style driver is the resident ``sweep.Sweep`` handle.  All
compute runs in libletkf_gpu.so; torch only holds device memory and does
layout transposes.
"""
from __future__ import annotations

import os

import numpy as np

from . import core as K


# ----------------------------------------------------------------------- SPEEDY
def speedy_sort_obs(lon, lat, olon, olat, device=None):
    """Stable bucket sort of observations by (latitude band, longitude cell)
    (speedy/letkf/letkf_obs.f90:243-313), on the device (letkf_sort_obs_latlon).
    Band j (1-based, 1..nlat-1) holds lat(j) <= y < lat(j+1); cell i holds
    lon(i) <= x < lon(i+1), the last cell up to 360.  Host arrays in, host
    arrays out: (perm, nobsgrd[nlat, nlon]) with nobsgrd[j-1, i-1] the
    cumulative count through cell (i, j); observations outside every band are
    dropped, and row nlat of nobsgrd is never written by the reference (0).
    Longitudes must lie in [0, 360): the reference counts an observation at
    360 in its band but places it in no cell, leaving an unfilled slot that
    the next band's first cell range covers; here it is dropped."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    perm, grd = K.sort_obs_latlon(t(lon), t(lat), t(olon), t(olat))
    return perm.cpu().numpy(), grd.cpu().numpy()


def var_local_n2n(var_local):
    """speedy/letkf/letkf_tools.f90:50-57: variable n reuses the transform of
    the first variable i <= n with an identical localisation row (0-based)."""
    vl = np.asarray(var_local, dtype=np.float64)
    tiny = np.finfo(np.float64).tiny
    n2n = np.zeros(vl.shape[0], dtype=np.int64)
    for n in range(1, vl.shape[0]):
        for i in range(n + 1):
            n2n[n] = i
            if np.max(np.abs(vl[i] - vl[n])) < tiny:
                break
    return n2n


def speedy_letkf(grid, obs, hdxf, dep, gues3d, logpfm, dlon_zero, params, var_local, infl3d, gues2d=None,
                 infl2d=None, iv3d_q=3, q_top_lev=5, stream=None):
    """das_letkf of speedy/letkf/letkf_tools.f90:44-203 on the device.

    grid: dict lon, lat (float64 device), nobsgrd (int32 [nlat, nlon] device).
    obs: dict elm, lon, lat, lev, dat, err (float64 device, bucket-sorted).
    hdxf: float64 [nobs, ne]; dep: float64 [nobs] (sorted like obs).
    gues3d: float64 [nv3d, nlev, ne, nij] full members; gues2d [nv2d, ne, nij].
    logpfm: float64 [nlev, nij]; dlon_zero: float64 [nij].
    params: (dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv).
    var_local: [nv3d + nv2d, 7] localisation rows (u, v, t, q, rh, ps, rain).
    infl3d: float64 [nv3d, nlev, nij] (in/out, the reference's work3d);
    infl2d: float64 [nv2d, nij].
    Returns (anal3d, anal2d) shaped like the inputs.  Per (point, variable
    group) the status of the core is checked; a failed eigensolve raises."""
    import torch

    nv3d, nlev, ne, nij = gues3d.shape
    nv2d = 0 if gues2d is None else gues2d.shape[0]
    dev = gues3d.device
    n2n = var_local_n2n(var_local)
    npts = nlev * nij
    ilev = torch.arange(1, nlev + 1, dtype=torch.int32, device=dev).repeat_interleave(nij)
    ijx = torch.arange(nij, device=dev).repeat(nlev)          # point p = (ilev - 1) * nij + ij
    nlon = grid["lon"].numel()
    jj, ii = torch.div(ijx, nlon, rounding_mode="floor"), ijx % nlon
    pts3 = {"lon": grid["lon"][ii].contiguous(), "lat": grid["lat"][jj].contiguous(),
            "dlon_zero": dlon_zero[ijx].contiguous(), "ilev": ilev.contiguous(),
            "logpfm": logpfm.reshape(-1).contiguous()}
    # members with the member index fastest: [nv][npts][ne]
    xb3 = gues3d.permute(0, 1, 3, 2).reshape(nv3d, npts, ne).contiguous()
    xa3 = torch.empty_like(xb3)
    trans_of = {}

    def analyse(group, pts, infl):
        offs, idx, rloc, rdiag = K.search_speedy(grid, obs, pts, params, var_local[group], stream)
        rows, dl = K.gather_rows(idx, hdxf, dep, stream)
        out = K.core_batch_f64(ne, offs, rows, rdiag, rloc, dl, infl, stream=stream)
        if bool((out["status"] != K.LETKF_OK).any()):
            raise K.LetkfError(int(out["status"].max()), "speedy_letkf: eigensolver")
        return out["trans"]

    for n in range(nv3d):
        g = int(n2n[n])
        if g < n:
            infl3d[n] = infl3d[g]
        else:
            pinf = infl3d[n].reshape(-1).contiguous()
            trans_of[n] = analyse(n, pts3, pinf)
            infl3d[n] = pinf.reshape(nlev, nij)
        tr = trans_of[g]
        if n == iv3d_q and nlev >= q_top_lev:
            # no analysis of upper-level q (letkf_tools.f90:173-178): identity transform
            eye = torch.eye(ne, dtype=torch.float64, device=dev)
            lo = (q_top_lev - 1) * nij
            tr = tr.clone()
            tr[lo:] = eye
        xa3[n] = K.update_f64(xb3[n:n + 1], tr, None, stream)[0]
    anal3d = xa3.reshape(nv3d, nlev, nij, ne).permute(0, 1, 3, 2).contiguous()
    anal2d = None
    if nv2d:
        pts2 = {k: v[:nij].contiguous() for k, v in pts3.items()}
        xb2 = gues2d.permute(0, 2, 1).contiguous()
        xa2 = torch.empty_like(xb2)
        for n in range(nv2d):
            g = int(n2n[nv3d + n])
            if g < nv3d + n:
                if g < nv3d:
                    tr = trans_of[g][:nij]
                    infl2d[n] = infl3d[g][0]
                else:
                    tr = trans_of[g]
                    infl2d[n] = infl2d[g - nv3d]
            else:
                pinf = infl2d[n].contiguous()
                tr = trans_of[nv3d + n] = analyse(nv3d + n, pts2, pinf)
                infl2d[n] = pinf
            xa2[n] = K.update_f64(xb2[n:n + 1], tr.contiguous(), None, stream)[0]
        anal2d = xa2.permute(0, 2, 1).contiguous()
    return anal3d, anal2d


PI = 3.1415926535      # common/common.f90:28
RE = 6371.3e3          # common/common.f90:35
GROSS_ERROR = 10.0     # speedy/letkf/letkf_obs.f90:50


def speedy_localization(lat, sigma_obs=1000.0e3, sigma_obsv=0.1, nlon=96):
    """dist_zero, dist_zerov, dlat_zero and dlon_zero per grid point
    (speedy/letkf/letkf_obs.f90:82-88); grid points are lon fastest."""
    dist_zero = sigma_obs * np.sqrt(10.0 / 3.0) * 2.0
    dist_zerov = sigma_obsv * np.sqrt(10.0 / 3.0) * 2.0
    dlat_zero = dist_zero / PI / RE * 180.0
    glat = np.repeat(np.asarray(lat, dtype=np.float64), nlon)
    dlon_zero = dlat_zero / np.cos(PI * glat / 180.0)
    return (dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv), dlon_zero


def speedy_obs_setup(lon, lat, sig, g3, g2, obs, gross_error=GROSS_ERROR, stream=None):
    """set_letkf_obs (speedy/letkf/letkf_obs.f90:48-313) for one time slot with
    H(x) computed on the device for every member (obsope.f90) instead of read
    from per-member obs2 files: qc = min over members, member mean, hdxf = Hx
    - mean, dep = y - mean, the gross-error check |dep| > 10 err, selection of
    qc = 1 and the bucket sort.  obs: host dict elem, lon, lat, lev, dat, err
    (SI units, as read_obs gives).  Returns (grid, obs_dev, hdxf, dep) ready
    for ``speedy_letkf`` (all on the device) and the host qc before
    selection."""
    import torch

    dev = g3.device
    nv3d, nlev, ne, nij = g3.shape
    nlon, nlat = len(lon), len(lat)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    elem_i = (np.sign(obs["elem"]) * np.floor(np.abs(obs["elem"]) + 0.5)).astype(np.int32)
    v3 = g3.reshape(nv3d, nlev, ne, nlat, nlon).permute(2, 0, 1, 3, 4)
    v2 = g2.reshape(g2.shape[0], ne, nlat, nlon).permute(1, 0, 2, 3)
    hx, qc = K.speedy_obsope(t(lat), t(sig), v3, v2, t(elem_i, torch.int32), t(obs["lon"]), t(obs["lat"]),
                             t(obs["lev"]), t(obs["dat"]), stream=stream)
    hdxf, dep, qc2 = K.obs_departure(hx, t(obs["dat"]), t(obs["err"]), gross_error, qc, stream)
    # selection of qc = 1 and the bucket sort on the device, then the records,
    # perturbations and departures gathered into the sorted order
    glon, glat = t(lon), t(lat)
    olon, olat = t(obs["lon"]), t(obs["lat"])
    perm, grd = K.sort_obs_latlon(glon, glat, olon, olat, qc2, stream)
    one = lambda a: K.gather_rows(perm, a.reshape(-1, 1), None, stream)[0].reshape(-1)
    obs_dev = {"elm": one(t(obs["elem"])), "lon": one(olon), "lat": one(olat), "lev": one(t(obs["lev"])),
               "dat": one(t(obs["dat"])), "err": one(t(obs["err"]))}
    hd_s, dep_s = K.gather_rows(perm, hdxf, dep, stream)
    grid = {"lon": glon, "lat": glat, "nobsgrd": grd}
    return grid, obs_dev, hd_s, dep_s, qc2.cpu().numpy()


def speedy_cycle(gues_paths, obs_path, anal_paths, lon, lat, sig, infl_path=None, cov_infl_mul=-1.01,
                 sigma_obs=1000.0e3, sigma_obsv=0.1, var_local=None, gross_error=GROSS_ERROR, mean_spread_prefix=None,
                 byteorder=">", device=None, stream=None):
    """The SPEEDY letkf program (speedy/letkf/letkf.f90) on the device:
    read_ens_mpi of the background members, set_letkf_obs with H(x) from the
    device, write_ensmspr_mpi('gues'), das_letkf (speedy/letkf/letkf_tools.f90:
    44-212, the inflation field from infl_mul.grd when cov_infl_mul < 0 and it
    exists, else |cov_infl_mul|; written back when cov_infl_mul < 0),
    write_ens_mpi('anal') and write_ensmspr_mpi('anal').  mean_spread_prefix
    is a directory/name prefix for the gues/anal _me/_sp files (None: not
    written).  Returns a summary dict."""
    import torch

    from . import speedy_io as IO

    device = device or torch.device("cuda")
    nlon, nlat, nlev = len(lon), len(lat), len(sig)
    nij = nlon * nlat
    g3, g2 = IO.load_ensemble(gues_paths, nlon, nlat, nlev, byteorder=byteorder, device=device, stream=stream)
    nv3d, _, ne, _ = g3.shape
    nv2d = g2.shape[0]
    obs = IO.read_obs(obs_path, byteorder)
    if mean_spread_prefix is not None:
        IO.write_mean_spread(mean_spread_prefix + "gues", g3, g2, nlon, nlat, byteorder, stream)
    if var_local is None:
        var_local = np.ones((nv3d + nv2d, 7))
    params, dlon_zero = speedy_localization(lat, sigma_obs, sigma_obsv, nlon)
    nobs_used = 0
    if obs["elem"].size:
        grid, obs_dev, hdxf, dep, qc = speedy_obs_setup(lon, lat, sig, g3, g2, obs, gross_error, stream)
        nobs_used = int(obs_dev["elm"].numel())
    # multiplicative inflation (speedy/letkf/letkf_tools.f90:114-140)
    if cov_infl_mul > 0.0:
        infl3d = torch.full((nv3d, nlev, nij), cov_infl_mul, dtype=torch.float64, device=device)
        infl3d[:, nlev - 1, :] = 1.01
        infl2d = torch.full((nv2d, nij), cov_infl_mul, dtype=torch.float64, device=device)
    elif infl_path is not None and os.path.exists(infl_path):
        w3, w2 = IO.read_grd4(infl_path, nlon, nlat, nlev, nv3d, nv2d, byteorder)
        infl3d = torch.as_tensor(w3.reshape(nv3d, nlev, nij).astype(np.float64), device=device)
        infl2d = torch.as_tensor(w2.reshape(nv2d, nij).astype(np.float64), device=device)
    else:
        infl3d = torch.full((nv3d, nlev, nij), -cov_infl_mul, dtype=torch.float64, device=device)
        infl2d = torch.full((nv2d, nij), -cov_infl_mul, dtype=torch.float64, device=device)
    if nobs_used == 0:
        a3, a2 = g3, g2                                    # no observation assimilated (:73-78)
    else:
        mean_ps = IO.mean_spread(g3, g2, stream)[1][0]      # ensemble-mean ps
        sigt = torch.as_tensor(np.asarray(sig, dtype=np.float64), device=device)
        logpfm = torch.log(mean_ps[None, :] * sigt[:, None]).contiguous()   # calc_pfull + DLOG (:143-145)
        a3, a2 = speedy_letkf(grid, obs_dev, hdxf, dep, g3, logpfm, torch.as_tensor(dlon_zero, device=device),
                              params, var_local, infl3d, g2, infl2d, stream=stream)
    IO.store_ensemble(anal_paths, a3, a2, byteorder, stream)
    if mean_spread_prefix is not None:
        IO.write_mean_spread(mean_spread_prefix + "anal", a3, a2, nlon, nlat, byteorder, stream)
    if cov_infl_mul < 0.0 and infl_path is not None:
        IO.write_grd4(infl_path, infl3d.cpu().numpy().reshape(nv3d, nlev, nlat, nlon),
                      infl2d.cpu().numpy().reshape(nv2d, nlat, nlon), byteorder)
    return {"ne": ne, "nobs_input": int(obs["elem"].size), "nobs_assimilated": nobs_used,
            "infl3d": infl3d, "infl2d": infl2d, "anal3d": a3, "anal2d": a2}


# -------------------------------------------------------------------- Lorenz-96
def l96_letkf(xf, hxf, y, obs_cell, obserr=1.0, xlocal=3.0, parm_infl=None, msw_infl=1.05, precision="f64",
              stream=None, msw_local=0, sa=1.0, sb=1.0):
    """One LETKF analysis of the Lorenz-96 driver (lorenz96/letkf/letkf.f90:
    180-265, one time slot).  msw_local 0 is the fixed localisation, 1 the
    adaptive one (correlation weights wa**sa * wb**sb, :237-243), 2 both.

    xf: float64 [nx, ne] background members; hxf: float64 [ny, ne] = H xf;
    y: float64 [ny]; obs_cell: int32 [ny] 1-based grid index of each
    observation (core.l96_obs_cell of H).  parm_infl: float64 [nx] (in/out;
    default msw_infl everywhere); with msw_infl > 0 it is reset to msw_infl
    after every core (the reference's fixed inflation).  precision "f64" (the
    plain form) or "mixed".  Returns (xa [nx, ne], parm_infl)."""
    import torch

    nx, ne = xf.shape
    dev = xf.device
    if parm_infl is None:
        parm_infl = torch.full((nx,), float(msw_infl), dtype=torch.float64, device=dev)
    hdxf, dep, _ = K.obs_departure(hxf, y, stream=stream)
    pix = torch.arange(1, nx + 1, dtype=torch.int32, device=dev)
    if msw_local == 0:
        offs, idx, rloc, rdiag = K.search_l96(nx, obs_cell, pix, xlocal, obserr, stream=stream)
    else:
        offs, idx, rloc, rdiag = K.search_l96_adaptive(nx, obs_cell, pix, 0, hdxf, xf, msw_local, sa, sb, xlocal,
                                                       obserr, stream=stream)
    rows, dl = K.gather_rows(idx, hdxf, dep, stream)
    if precision == "f64":
        out = K.core_batch_f64(ne, offs, rows, rdiag, rloc, dl, parm_infl, stream=stream)
        trans = out["trans"]
    elif precision == "mixed":
        f = lambda t: t.to(torch.float32).contiguous()
        out = K.core_batch_mixed(ne, offs, f(rows), f(rdiag), f(rloc), f(dl), parm_infl, stream=stream)
        trans = out["trans"].to(torch.float64)
    else:
        raise ValueError(f"precision {precision!r}")
    if bool((out["status"] != K.LETKF_OK).any()):
        raise K.LetkfError(int(out["status"].max()), "l96_letkf: eigensolver")
    if msw_infl > 0.0:
        parm_infl.fill_(float(msw_infl))
    xa = K.update_f64(xf.reshape(1, nx, ne).contiguous(), trans.contiguous(), None, stream)[0]
    return xa, parm_infl


def l96_letkf_4d(xf, hxf, y, obs_cell, obserr=1.0, xlocal=3.0, tlocal=2.0, parm_infl=None, msw_infl=1.05,
                 precision="f64", stream=None, msw_local=0, sa=1.0, sb=1.0):
    """4D-LETKF of the Lorenz-96 driver (lorenz96/letkf/letkf.f90:183-288,
    nwindow > 1; msw_local as in l96_letkf): xf float64 [nslot, nx, ne] first guesses
    of the slots; hxf [nslot, ny, ne] = H_n xf_n; y [nslot, ny]; obs_cell int32
    [nslot, ny] (l96_obs_cell of each slot's H).  Departures and perturbations
    per slot (:197-213), then for every analysis slot nn and point the
    observations of all slots with tdif = |nn - n| (:217-254), the core, the
    fixed-inflation reset and the update of slot nn.  parm_infl float64
    [nslot, nx] (in/out).  Returns (xa [nslot, nx, ne], parm_infl)."""
    import torch

    nslot, nx, ne = xf.shape
    ny = hxf.shape[1]
    dev = xf.device
    if parm_infl is None:
        parm_infl = torch.full((nslot, nx), float(abs(msw_infl)), dtype=torch.float64, device=dev)
    hd, dp = [], []
    for n in range(nslot):
        h_n, d_n, _ = K.obs_departure(hxf[n].contiguous(), y[n].contiguous(), stream=stream)
        hd.append(h_n)
        dp.append(d_n)
    hdxf = torch.cat(hd).contiguous()          # rows n*ny + i
    dep = torch.cat(dp).contiguous()
    pix = torch.arange(1, nx + 1, dtype=torch.int32, device=dev)
    xa = torch.empty_like(xf)
    for nn in range(nslot):
        if msw_local == 0:
            offs, idx, rloc, rdiag = K.search_l96_4d(nx, obs_cell, pix, nn, xlocal, obserr, tlocal, stream)
        else:
            offs, idx, rloc, rdiag = K.search_l96_adaptive(nx, obs_cell, pix, nn, hdxf, xf[nn], msw_local, sa, sb,
                                                           xlocal, obserr, tlocal, stream)
        rows, dl = K.gather_rows(idx, hdxf, dep, stream)
        pinf = parm_infl[nn].contiguous()
        if precision == "f64":
            out = K.core_batch_f64(ne, offs, rows, rdiag, rloc, dl, pinf, stream=stream)
            trans = out["trans"]
        elif precision == "mixed":
            f = lambda t: t.to(torch.float32).contiguous()
            out = K.core_batch_mixed(ne, offs, f(rows), f(rdiag), f(rloc), f(dl), pinf, stream=stream)
            trans = out["trans"].to(torch.float64)
        else:
            raise ValueError(f"precision {precision!r}")
        if bool((out["status"] != K.LETKF_OK).any()):
            raise K.LetkfError(int(out["status"].max()), "l96_letkf_4d: eigensolver")
        if msw_infl > 0.0:
            pinf.fill_(float(msw_infl))
        parm_infl[nn] = pinf
        xa[nn] = K.update_f64(xf[nn].reshape(1, nx, ne).contiguous(), trans.contiguous(), None, stream)[0]
    return xa, parm_infl


__all__ = ["speedy_sort_obs", "var_local_n2n", "speedy_letkf", "l96_letkf", "l96_letkf_4d", "speedy_obs_setup",
           "speedy_cycle"]


# ------------------------------------------------------------------------ SCALE
SCALE_GROSS_ERROR = 5.0  # scale/common/common_nml.f90:83
SCALE_IQC_GROSS_ERR = 5  # scale/common/common_obs_scale.f90:142
SCALE_PS = 14593


def scale_obs_setup(v3d, v2d, khalo, obs, rotc=None, stggrd=0, ps_adjust_thres=100.0, gross_error=SCALE_GROSS_ERROR,
                    stream=None):
    """set_letkf_obs of the SCALE driver for conventional observations
    (scale/letkf/letkf_obs.f90:260-600) with H(x) of every member from the
    device (letkf_scale_obsope, obsope_cal's conventional path) instead of
    per-member obsda files: qc the maximum over members (:272), the member
    mean (sequential sum, :562-566), Hdx and y - Hx (:574-577), the gross-error
    check |y - Hx| > GROSS_ERROR err (qc 5, :586-630) and the selection of
    qc 0.  v3d / v2d as core.scale_obsope takes them (device); obs: dict of
    arrays elem, ri, rj, lev, dat, err (the halo-domain ri / rj obsope uses).
    Returns (records, qc): records is a dict of host arrays for the selected
    observations, ri, rj, lev, dat, err, dep, cls (1 for ps, whose vertical
    coordinate in the search is the observed pressure; 0 otherwise) and hdxf
    [n, ne] float32, ready for Sweep.set_obs; qc holds every observation's
    SCALE code."""
    import torch

    dev = v3d.device
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    elem = t(obs["elem"], torch.int32)
    rc = None if rotc is None else t(rotc)
    hx, qc = K.scale_obsope(v3d, v2d, khalo, elem, t(obs["ri"]), t(obs["rj"]), t(obs["lev"]), rc, stggrd,
                            ps_adjust_thres, stream=stream)
    good = (qc == 0).to(torch.int32)  # the departure kernel takes 1 for a usable observation
    hdxf, dep, ok = K.obs_departure(hx, t(obs["dat"]), t(obs["err"]), gross_error, good, stream)
    qc_all = torch.where((good == 1) & (ok == 0), torch.full_like(qc, SCALE_IQC_GROSS_ERR), qc)
    sel = torch.nonzero(ok == 1).flatten()
    host = lambda a: a[sel].cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)[sel.cpu().numpy()]
    el = host(elem)
    rec = {"ri": host(obs["ri"]), "rj": host(obs["rj"]), "lev": host(obs["lev"]), "dat": host(obs["dat"]),
           "err": host(obs["err"]), "dep": host(dep), "cls": (el == SCALE_PS).astype(np.int32),
           "hdxf": hdxf[sel].to(torch.float32).cpu().numpy()}
    return rec, qc_all.cpu().numpy()

