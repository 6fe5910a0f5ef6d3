"""ctypes front end of the CPU oracle (test infrastructure only).

This module is the test oracle: tests/, __graft_entry__.smoke() and bench.py's
CPU legs import it; the package ``letkf_gb300`` never does.  All arrays are
float64 / int32 numpy arrays; column-major arrays are passed in Fortran order.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_libs = {}


def lib(timed=False):
    """The parity build (every operation rounded on its own, -O2), or with
    timed=True the build the CPU baseline is timed with (-O3, FMA contraction
    allowed); both export the same functions."""
    _lib = _libs.get(bool(timed))
    if _lib is None:
        path = _build.build(timed=bool(timed))
        _lib = C.CDLL(path)
        _libs[bool(timed)] = _lib
        d = C.c_double
        pd = C.POINTER(C.c_double)
        pi = C.POINTER(C.c_int)
        _lib.oracle_letkf_core.restype = C.c_int
        _lib.oracle_letkf_core.argtypes = [C.c_int, C.c_int, C.c_int, pd, pd, pd, pd, pd, pd, pd, pd,
                                           C.c_int, pd]
        _lib.oracle_letkf_core_batch.restype = C.c_int
        _lib.oracle_letkf_core_batch.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int64), pd, pd, pd, pd,
                                                 pd, pd, pd, pd, C.c_int, d, C.c_int, pi]
        _lib.oracle_mtx_eigen.restype = C.c_int
        _lib.oracle_mtx_eigen.argtypes = [C.c_int, C.c_int, pd, pd, pd, pi]
        _lib.oracle_pythag.restype = d
        _lib.oracle_pythag.argtypes = [d, d]
        _lib.oracle_com_distll_1.argtypes = [d, d, d, d, pd]
        _lib.oracle_speedy_sort_obs.restype = C.c_int
        _lib.oracle_speedy_sort_obs.argtypes = [C.c_int, C.c_int, pd, pd, C.c_int, pd, pd, pi, pi]
        _lib.oracle_gfs_obs_local.restype = C.c_int
        _lib.oracle_gfs_obs_local.argtypes = [C.c_void_p, C.c_void_p, d, d, d, pi, pd, pd]
        _lib.oracle_speedy_obs_local.restype = C.c_int
        _lib.oracle_speedy_obs_local.argtypes = [C.c_void_p, d, d, d, C.c_int, d, pi, pd, pd]
        _lib.oracle_scale_sort_obs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, pd, pd, pi, pi]
        _lib.oracle_scale_obs_local.restype = C.c_int
        _lib.oracle_scale_obs_local.argtypes = [C.c_void_p, d, d, d, d, pi, pd, pd]
        _lib.oracle_scale_dist_zero_fac.restype = d
        _lib.oracle_scale_dist_zero_fac_square.restype = d
        _lib.oracle_l96_select_4d.restype = C.c_int
        _lib.oracle_l96_select_4d.argtypes = [C.c_int, C.c_int, C.c_int, pd, C.c_int, C.c_int, d, d, pi, pd]
        _lib.oracle_l96_select.restype = C.c_int
        _lib.oracle_com_correl.restype = d
        _lib.oracle_com_correl.argtypes = [C.c_int, pd, pd]
        _lib.oracle_l96_select_adaptive.restype = C.c_int
        _lib.oracle_l96_select_adaptive.argtypes = [C.c_int, C.c_int, C.c_int, pd, pd, pd, C.c_int, C.c_int, C.c_int,
                                                    d, d, C.c_int, d, d, pi, pd]
        _lib.oracle_l96_select.argtypes = [C.c_int, C.c_int, pd, C.c_int, d, d, pi, pd]
        _lib.oracle_ensmean.argtypes = [C.c_int, C.c_int, pd, pd, pd]
        _lib.oracle_scale_sweep.restype = C.c_int
        _lib.oracle_scale_sweep.argtypes = [C.c_void_p, pd, pd, C.c_int, C.c_int, C.c_int, pi, C.c_int, pd, pd, pd,
                                            pd, pd, pd, pd, pi, d, C.c_int]
        _lib.oracle_scale_obs_local_batch.argtypes = [C.c_void_p, C.c_int, pd, pd, pd, pd, C.c_int, pi, pi, pd,
                                                      C.c_int]
        _lib.oracle_weight_rtpp.argtypes = [C.c_int, pd, d, pd]
        _lib.oracle_weight_rtps.argtypes = [C.c_int, pd, pd, pd, d, pd, pd]
        _lib.oracle_obs_analysis.restype = d
        _lib.oracle_obs_analysis.argtypes = [C.c_int, pd, d, pd, C.c_int, d, pd]
        _lib.oracle_efso.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64), pi, pd, pd, pd, pd,
                                     pd, pi, C.c_int, pd, pd, pd]
        i64 = C.c_int64
        _lib.oracle_speedy_calc_rh.restype = d
        _lib.oracle_speedy_calc_rh.argtypes = [d, d, d]
        _lib.oracle_scale_obsope.restype = C.c_int
        _lib.oracle_scale_obsope.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, pd, i64, i64, pd, i64,
                                             i64, C.c_int, pi, pd, pd, pd, pd, C.c_int, d, pd, pi, pi]
        _lib.oracle_speedy_obsope.restype = C.c_int
        _lib.oracle_speedy_obsope.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, pd, pd, pd, i64, i64, pd, i64, i64,
                                              C.c_int, pi, pd, pd, pd, pd, pd, pi, pi]
    return _lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _pi(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def _f64(a, order="C"):
    return np.ascontiguousarray(a, dtype=np.float64) if order == "C" else np.asfortranarray(a, dtype=np.float64)


def letkf_core(hdxb, rdiag, rloc, dep, parm_infl, nobsl=None, want_transm=False, want_pao=False,
               rdiag_wloc=False, minfl=None):
    """common/common_letkf.f90:50 letkf_core.  hdxb is (nobs, ne); rows
    0..nobsl-1 are used.  Returns dict(trans, transm, pao, parm_infl, status)."""
    hdxb = _f64(hdxb, "F")
    nobs, ne = hdxb.shape
    if nobsl is None:
        nobsl = nobs
    rdiag = _f64(rdiag)
    rloc = _f64(rloc)
    dep = _f64(dep)
    infl = np.array([parm_infl], dtype=np.float64)
    trans = np.zeros((ne, ne), dtype=np.float64, order="F")
    transm = np.zeros(ne) if want_transm else None
    pao = np.zeros((ne, ne), order="F") if want_pao else None
    mf = np.array([minfl], dtype=np.float64) if minfl is not None else None
    st = lib().oracle_letkf_core(ne, max(nobs, 1), nobsl, _pd(hdxb), _pd(rdiag), _pd(rloc), _pd(dep),
                                 _pd(infl), _pd(trans), _pd(transm), _pd(pao), int(bool(rdiag_wloc)),
                                 _pd(mf))
    return dict(trans=trans, transm=transm, pao=pao, parm_infl=float(infl[0]), status=int(st))


def letkf_core_batch(ne, offs, rows, rdiag, rloc, dep, infl, rdiag_wloc=False, minfl=0.0,
                     want_transm=False, want_pao=False, nthreads=0):
    """Per-point oracle over a packed ragged batch (rows[offs[p]:offs[p+1]] are
    point p's local obs, row-major [row][ne]).  Returns dict of arrays:
    trans (npts, ne, ne) with trans[p][m][k] = trans(k,m) of point p, i.e. the
    Fortran column-major matrix viewed row-major per point."""
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    npts = offs.size - 1
    rows = _f64(rows)
    infl = np.array(infl, dtype=np.float64).copy()
    trans = np.zeros((npts, ne, ne))
    transm = np.zeros((npts, ne)) if want_transm else None
    pao = np.zeros((npts, ne, ne)) if want_pao else None
    status = np.zeros(npts, dtype=np.int32)
    lib().oracle_letkf_core_batch(ne, npts, offs.ctypes.data_as(C.POINTER(C.c_int64)), _pd(rows),
                                  _pd(_f64(rdiag)), _pd(_f64(rloc)), _pd(_f64(dep)), _pd(infl), _pd(trans),
                                  _pd(transm), _pd(pao), int(bool(rdiag_wloc)), float(minfl), int(nthreads),
                                  _pi(status))
    return dict(trans=trans, transm=transm, pao=pao, parm_infl=infl, status=status)


def mtx_eigen(a):
    a = _f64(a, "F")
    n = a.shape[0]
    eival = np.zeros(n)
    eivec = np.zeros((n, n), order="F")
    nr = np.zeros(1, dtype=np.int32)
    st = lib().oracle_mtx_eigen(1, n, _pd(a), _pd(eival), _pd(eivec), _pi(nr))
    return eival, eivec, int(nr[0]), int(st)


def pythag(a, b):
    return lib().oracle_pythag(float(a), float(b))


def com_distll_1(alon, alat, blon, blat):
    out = np.zeros(1)
    lib().oracle_com_distll_1(float(alon), float(alat), float(blon), float(blat), _pd(out))
    return float(out[0])


def speedy_sort_obs(lon, lat, obslon, obslat):
    lon = _f64(lon)
    lat = _f64(lat)
    obslon = _f64(obslon)
    obslat = _f64(obslat)
    n = obslon.size
    perm = np.full(max(n, 1), -1, dtype=np.int32)
    grd = np.zeros(lon.size * lat.size, dtype=np.int32)
    placed = lib().oracle_speedy_sort_obs(lon.size, lat.size, _pd(lon), _pd(lat), n, _pd(obslon),
                                          _pd(obslat), _pi(perm), _pi(grd))
    return perm[:placed].copy(), grd.reshape(lat.size, lon.size)  # grd[j][i] = nobsgrd(i+1,j+1)


class _SpeedyObs(C.Structure):
    _fields_ = [("nlon", C.c_int), ("nlat", C.c_int), ("lon", C.c_void_p), ("lat", C.c_void_p),
                ("nobsgrd", C.c_void_p), ("nobs", C.c_int), ("obselm", C.c_void_p), ("obslon", C.c_void_p),
                ("obslat", C.c_void_p), ("obslev", C.c_void_p), ("obsdat", C.c_void_p), ("obserr", C.c_void_p),
                ("dist_zero", C.c_double), ("dist_zerov", C.c_double), ("dlat_zero", C.c_double),
                ("sigma_obs", C.c_double), ("sigma_obsv", C.c_double), ("var_local", C.c_void_p)]


class SpeedyObs:
    """Sorted SPEEDY obs set + search parameters for oracle obs_local calls."""

    def __init__(self, lon, lat, nobsgrd, elm, olon, olat, olev, odat, oerr, dist_zero, dist_zerov,
                 dlat_zero, sigma_obs, sigma_obsv, var_local_row):
        self._keep = [_f64(lon), _f64(lat), np.ascontiguousarray(nobsgrd, dtype=np.int32).ravel(),
                      _f64(elm), _f64(olon), _f64(olat), _f64(olev), _f64(odat), _f64(oerr),
                      _f64(var_local_row)]
        k = self._keep
        self.s = _SpeedyObs(k[0].size, k[1].size, k[0].ctypes.data, k[1].ctypes.data, k[2].ctypes.data,
                            k[3].size, k[3].ctypes.data, k[4].ctypes.data, k[5].ctypes.data, k[6].ctypes.data,
                            k[7].ctypes.data, k[8].ctypes.data, dist_zero, dist_zerov, dlat_zero, sigma_obs,
                            sigma_obsv, k[9].ctypes.data)

    def obs_local(self, lon1, lat1, dlon_zero, ilev, logpfm):
        n = max(self.s.nobs, 1)
        idx = np.zeros(n, dtype=np.int32)
        rloc = np.zeros(n)
        rdiag = np.zeros(n)
        nl = lib().oracle_speedy_obs_local(C.byref(self.s), lon1, lat1, dlon_zero, ilev, logpfm, _pi(idx),
                                           _pd(rloc), _pd(rdiag))
        if nl < 0:
            raise ValueError("unknown observation element id")
        return idx[:nl].copy(), rloc[:nl].copy(), rdiag[:nl].copy()


class _GfsParams(C.Structure):
    _fields_ = [("dist_zero", C.c_double), ("dist_zerov", C.c_double), ("dist_zero_rain", C.c_double),
                ("dist_zerov_rain", C.c_double), ("sigma_obs", C.c_double), ("sigma_obsv", C.c_double),
                ("sigma_obs_rain", C.c_double), ("base_obsv_rain", C.c_double), ("var_local", C.c_void_p)]


def gfs_obs_local(so, params, rlon, rlat, rlev, var_local=None):
    """obs_local of the GFS driver (gfs/letkf/letkf_tools.f90:686-925) on the
    sorted observations of a SpeedyObs `so`.  params: dist_zero, dist_zerov,
    dist_zero_rain, dist_zerov_rain, sigma_obs, sigma_obsv, sigma_obs_rain,
    base_obsv_rain; var_local: 6 weights or None.  Returns (idx, rloc, rdiag)."""
    vl = None if var_local is None else _f64(var_local)
    g = _GfsParams(*[float(x) for x in params], None if vl is None else vl.ctypes.data)
    n = max(so.s.nobs, 1)
    idx = np.zeros(n, dtype=np.int32)
    rloc = np.zeros(n)
    rdiag = np.zeros(n)
    nl = lib().oracle_gfs_obs_local(C.byref(so.s), C.byref(g), float(rlon), float(rlat), float(rlev), _pi(idx),
                                    _pd(rloc), _pd(rdiag))
    return idx[:nl].copy(), rloc[:nl].copy(), rdiag[:nl].copy()


def scale_sort_obs(nlon, nlat, obs_ri, obs_rj, ihalo=0, jhalo=0):
    obs_ri = _f64(obs_ri)
    obs_rj = _f64(obs_rj)
    n = obs_ri.size
    perm = np.zeros(max(n, 1), dtype=np.int32)
    grd = np.zeros((nlon + 1) * nlat, dtype=np.int32)
    lib().oracle_scale_sort_obs(nlon, nlat, ihalo, jhalo, n, _pd(obs_ri), _pd(obs_rj), _pi(perm), _pi(grd))
    return perm[:n].copy(), grd.reshape(nlat, nlon + 1)  # grd[j-1][i] = nobsgrd(i, j), i = 0..nlon


class _ScaleObs(C.Structure):
    _fields_ = [("nlon", C.c_int), ("nlat", C.c_int), ("nobsgrd", C.c_void_p), ("nobs", C.c_int),
                ("ri", C.c_void_p), ("rj", C.c_void_p), ("lev", C.c_void_p), ("dat", C.c_void_p),
                ("err", C.c_void_p), ("cls", C.c_void_p), ("uid", C.c_void_p), ("typ", C.c_void_p),
                ("varloc_idx", C.c_void_p), ("nid", C.c_int), ("ntyp", C.c_int), ("dx", C.c_double),
                ("dy", C.c_double), ("dlon_zero", C.c_double), ("dlat_zero", C.c_double),
                ("sigma_obs", C.c_double), ("sigma_obsv", C.c_double), ("sigma_obs_rain", C.c_double),
                ("sigma_obsv_rain", C.c_double), ("base_obsv_rain", C.c_double),
                ("sigma_obs_radar", C.c_double), ("sigma_obs_radar_noref", C.c_double),
                ("sigma_obsz_radar", C.c_double), ("radar_ref_thres_dbz", C.c_double),
                ("sigma_obs_tc", C.c_double), ("sigma_obsv_tc", C.c_double), ("var_local", C.c_void_p),
                ("max_nobs_per_grid", C.c_int)]


SCALE_PARAM_DEFAULTS = dict(sigma_obs_rain=350.0e3, sigma_obsv_rain=0.4, base_obsv_rain=85000.0,
                            sigma_obs_radar=2000.0, sigma_obs_radar_noref=2000.0, sigma_obsz_radar=1000.0,
                            radar_ref_thres_dbz=15.0, sigma_obs_tc=50.0e3, sigma_obsv_tc=0.4)


class ScaleObs:
    """Sorted SCALE obs set + search parameters for oracle obs_local calls."""

    def __init__(self, nlon, nlat, nobsgrd, ri, rj, lev, dat, err, cls, uid, typ, varloc_idx, nid, ntyp, dx,
                 dy, dlon_zero, dlat_zero, sigma_obs, sigma_obsv, var_local_row=None, max_nobs_per_grid=0,
                 **kw):
        p = dict(SCALE_PARAM_DEFAULTS)
        p.update(kw)
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32).ravel()
        self._keep = [i32(nobsgrd), _f64(ri), _f64(rj), _f64(lev), _f64(dat), _f64(err), i32(cls), i32(uid),
                      i32(typ), i32(varloc_idx), None if var_local_row is None else _f64(var_local_row)]
        k = self._keep
        self.s = _ScaleObs(nlon, nlat, k[0].ctypes.data, k[1].size, k[1].ctypes.data, k[2].ctypes.data,
                           k[3].ctypes.data, k[4].ctypes.data, k[5].ctypes.data, k[6].ctypes.data,
                           k[7].ctypes.data, k[8].ctypes.data, k[9].ctypes.data, nid, ntyp, dx, dy, dlon_zero,
                           dlat_zero, sigma_obs, sigma_obsv, p["sigma_obs_rain"], p["sigma_obsv_rain"],
                           p["base_obsv_rain"], p["sigma_obs_radar"], p["sigma_obs_radar_noref"],
                           p["sigma_obsz_radar"], p["radar_ref_thres_dbz"], p["sigma_obs_tc"],
                           p["sigma_obsv_tc"], None if k[10] is None else k[10].ctypes.data,
                           int(max_nobs_per_grid))

    def sweep(self, hdxf, dep, xb, pri, prj, prlev, infl, prz=None, subset=None, minfl=0.0, nthreads=0, timed=False):
        """SCALE grid loop (oracle_scale_sweep).  hdxf (nobs, ne) and dep in
        sorted order; xb (nv, npts, ne).  Returns (xa, infl, nobsl); with a
        subset only those points' entries are meaningful.  timed=True runs the
        -O3 build the CPU baseline is timed with (results equal to rounding)."""
        hdxf = _f64(hdxf)
        xb = _f64(xb)
        nv, npts, ne = xb.shape
        xa = np.zeros_like(xb)
        infl = np.array(infl, dtype=np.float64).copy()
        nobsl = np.zeros(npts, dtype=np.int32)
        sub = None if subset is None else np.ascontiguousarray(subset, dtype=np.int32)
        bad = lib(timed).oracle_scale_sweep(C.byref(self.s), _pd(hdxf), _pd(_f64(dep)), ne, nv, npts, _pi(sub),
                                       0 if sub is None else sub.size, _pd(_f64(pri)), _pd(_f64(prj)),
                                       _pd(_f64(prlev)), None if prz is None else _pd(_f64(prz)), _pd(xb), _pd(xa),
                                       _pd(infl), _pi(nobsl), float(minfl), int(nthreads))
        if bad:
            raise RuntimeError(f"oracle sweep: {bad} points failed")
        return xa, infl, nobsl

    def obs_local_batch(self, ri, rj, rlev, rz=None, cap=4096, nthreads=0):
        """obs_local of many points (OpenMP): (count [n], idx [n, cap] sorted
        indices, -1 past the count; rloc [n, cap])."""
        ri, rj, rlev = _f64(ri), _f64(rj), _f64(rlev)
        n = ri.size
        cnt = np.zeros(n, dtype=np.int32)
        idx = np.full((n, cap), -1, dtype=np.int32)
        rloc = np.zeros((n, cap))
        lib().oracle_scale_obs_local_batch(C.byref(self.s), n, _pd(ri), _pd(rj), _pd(rlev),
                                           None if rz is None else _pd(_f64(rz)), int(cap), _pi(cnt), _pi(idx),
                                           _pd(rloc), int(nthreads))
        return cnt, idx, rloc

    def obs_local(self, ri, rj, rlev, rz=0.0):
        n = max(self.s.nobs, 1)
        idx = np.zeros(n, dtype=np.int32)
        rloc = np.zeros(n)
        rdiag = np.zeros(n)
        nl = lib().oracle_scale_obs_local(C.byref(self.s), ri, rj, rlev, rz, _pi(idx), _pd(rloc), _pd(rdiag))
        return idx[:nl].copy(), rloc[:nl].copy(), rdiag[:nl].copy()


def scale_dist_zero_fac():
    return lib().oracle_scale_dist_zero_fac()


def scale_dist_zero_fac_square():
    return lib().oracle_scale_dist_zero_fac_square()


def l96_select(h, ix, xlocal=3.0, tlocal=2.0):
    """h is (ny, nx); ix is 1-based as in the reference."""
    h = _f64(h, "F")
    ny, nx = h.shape
    idx = np.zeros(ny, dtype=np.int32)
    rloc = np.zeros(ny)
    n = lib().oracle_l96_select(nx, ny, _pd(h), ix, xlocal, tlocal, _pi(idx), _pd(rloc))
    return idx[:n].copy(), rloc[:n].copy()


def l96_select_4d(h4d, slot, ix, xlocal=3.0, tlocal=2.0):
    """h4d is (nslot, ny, nx); slot and ix are 1-based as in the reference.
    Indices are rows n*ny + i of the slot-stacked observations."""
    h4d = np.asarray(h4d, dtype=np.float64)
    nslot, ny, nx = h4d.shape
    hf = np.ascontiguousarray(np.stack([np.asfortranarray(h4d[n]).ravel(order="F") for n in range(nslot)]))
    idx = np.zeros(max(nslot * ny, 1), dtype=np.int32)
    rloc = np.zeros(max(nslot * ny, 1))
    n = lib().oracle_l96_select_4d(nx, ny, nslot, _pd(hf), int(slot), int(ix), float(xlocal), float(tlocal),
                                   _pi(idx), _pd(rloc))
    return idx[:n].copy(), rloc[:n].copy()


def com_correl(v1, v2):
    """common/common.f90:111-128 (sequential sums)."""
    v1, v2 = _f64(v1), _f64(v2)
    return float(lib().oracle_com_correl(v1.size, _pd(v1), _pd(v2)))


def l96_select_adaptive(h4d, hdxf, dxf, slot, ix, msw_local, sa=1.0, sb=1.0, xlocal=3.0, tlocal=2.0):
    """Lorenz-96 selection with msw_local (0 fixed, 1 adaptive, 2 both).
    h4d (nslot, ny, nx); hdxf (nslot*ny, ne) slot-stacked obs-space
    perturbations; dxf (ne,) first-guess perturbations of point ix at the
    analysis slot; slot and ix 1-based."""
    h4d = np.asarray(h4d, dtype=np.float64)
    if h4d.ndim == 2:
        h4d = h4d[None]
    nslot, ny, nx = h4d.shape
    hf = np.ascontiguousarray(np.stack([np.asfortranarray(h4d[n]).ravel(order="F") for n in range(nslot)]))
    hd = _f64(hdxf)
    dx = _f64(dxf)
    idx = np.zeros(max(nslot * ny, 1), dtype=np.int32)
    rloc = np.zeros(max(nslot * ny, 1))
    n = lib().oracle_l96_select_adaptive(nx, ny, nslot, _pd(hf), _pd(hd), _pd(dx), dx.size, int(slot), int(ix),
                                         float(xlocal), float(tlocal), int(msw_local), float(sa), float(sb),
                                         _pi(idx), _pd(rloc))
    return idx[:n].copy(), rloc[:n].copy()


def ensmean(x):
    """x is (npts, ne); returns (mean, pert) with the sequential member sum."""
    x = _f64(x)
    npts, ne = x.shape
    mean = np.zeros(npts)
    pert = np.zeros_like(x)
    lib().oracle_ensmean(npts, ne, _pd(x), _pd(mean), _pd(pert))
    return mean, pert


def weight_rtpp(w, alpha):
    w = _f64(w, "F")
    out = np.zeros_like(w, order="F")
    lib().oracle_weight_rtpp(w.shape[0], _pd(w), float(alpha), _pd(out))
    return out


def weight_rtps(w, pa, xb, alpha):
    w = _f64(w, "F")
    pa = _f64(pa, "F")
    out = np.zeros_like(w, order="F")
    infl = np.zeros(1)
    lib().oracle_weight_rtps(w.shape[0], _pd(w), _pd(pa), _pd(_f64(xb)), float(alpha), _pd(out), _pd(infl))
    return out, float(infl[0])


def obs_analysis(trans, ybar, hdxf, mode=0, q_sprd_max=0.0):
    """gfs/letkf/letkf_tools.f90:466-497 at one observation location.  trans is
    (ne, ne) with trans[k, m] = trans(k+1, m+1).  Returns (anal[ne], mean)."""
    t = _f64(trans, "F")
    ne = t.shape[0]
    anal = np.zeros(ne)
    mean = lib().oracle_obs_analysis(ne, _pd(t), float(ybar), _pd(_f64(hdxf)), int(mode), float(q_sprd_max),
                                     _pd(anal))
    return anal, mean


def efso(ne, offs, idx, rdiag, rloc, hdxa, fcst, fcer, term, obsdep):
    """gfs/letkf/letkf_tools.f90:547-679.  fcst (nv, npts, ne), fcer (nv, npts),
    hdxa (nobs, ne).  Returns (djdy, obsense), each (nobs, nterm)."""
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    fcst = _f64(fcst)
    nv, npts, _ = fcst.shape
    term = np.ascontiguousarray(term, dtype=np.int32)
    nterm = int(term.max()) + 1
    hdxa = _f64(hdxa)
    nobs = hdxa.shape[0]
    djdy = np.zeros((nobs, nterm))
    obsense = np.zeros((nobs, nterm))
    lib().oracle_efso(ne, npts, nv, nterm, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                      _pi(np.ascontiguousarray(idx, dtype=np.int32)), _pd(_f64(rdiag)), _pd(_f64(rloc)), _pd(hdxa),
                      _pd(fcst), _pd(_f64(fcer)), _pi(term), nobs, _pd(_f64(obsdep)), _pd(djdy), _pd(obsense))
    return djdy, obsense


def scale_obsope(v3d, v2d, khalo, elem, ri, rj, rlev, rotc=None, stggrd=0, ps_adjust_thres=100.0):
    """SCALE conventional H(x) for every member (scale/obs/obsope_tools.f90:
    340-380).  v3d [ne, 6, nlath, nlonh, nlevh] (u, v, t, q, rh, p; C order,
    levels fastest), v2d [ne, 4, nlath, nlonh] (ps, t2m, q2m, topo).  Returns
    (hx [nobs, ne], qc [nobs], qc_member [nobs, ne])."""
    v3d = _f64(v3d)
    v2d = _f64(v2d)
    ne, _, nlath, nlonh, nlevh = v3d.shape
    elem = np.ascontiguousarray(elem, dtype=np.int32)
    nobs = elem.size
    hx = np.zeros((nobs, ne))
    qcm = np.zeros((nobs, ne), dtype=np.int32)
    qc = np.zeros(nobs, dtype=np.int32)
    rc = None if rotc is None else _f64(rotc)
    st = lib().oracle_scale_obsope(nlonh, nlath, nlevh - 2 * khalo, khalo, ne, _pd(v3d), 6 * nlath * nlonh * nlevh,
                                   nlath * nlonh * nlevh, _pd(v2d), 4 * nlath * nlonh, nlath * nlonh, nobs, _pi(elem),
                                   _pd(_f64(ri)), _pd(_f64(rj)), _pd(_f64(rlev)), _pd(rc), int(stggrd),
                                   float(ps_adjust_thres), _pd(hx), _pi(qcm), _pi(qc))
    if st:
        raise ValueError("oracle_scale_obsope: khalo >= 2 and nlev >= 2 expected")
    return hx, qc, qcm


def speedy_calc_rh(t, q, p):
    """speedy/common/common_obs_speedy.f90:84-109."""
    return lib().oracle_speedy_calc_rh(float(t), float(q), float(p))


def speedy_obsope(lat, sig, v3d, v2d, elem, rlon, rlat, rlev, odat):
    """SPEEDY H(x) for every member (speedy/letkf/obsope.f90:53-104).
    v3d [ne, 4, nlev, nlat, nlon], v2d [ne, 2, nlat, nlon] (C order).
    Returns (hx [nobs, ne], qc [nobs], qc_member [nobs, ne])."""
    v3d = _f64(v3d)
    v2d = _f64(v2d)
    ne, _, nlev, nlat, nlon = v3d.shape
    elem = np.ascontiguousarray(elem, dtype=np.int32)
    nobs = elem.size
    hx = np.zeros((nobs, ne))
    qcm = np.zeros((nobs, ne), dtype=np.int32)
    qc = np.zeros(nobs, dtype=np.int32)
    nij = nlat * nlon
    lib().oracle_speedy_obsope(nlon, nlat, nlev, ne, _pd(_f64(lat)), _pd(_f64(sig)), _pd(v3d), 4 * nlev * nij, nij,
                               _pd(v2d), 2 * nij, nij, nobs, _pi(elem), _pd(_f64(rlon)), _pd(_f64(rlat)),
                               _pd(_f64(rlev)), _pd(_f64(odat)), _pd(hx), _pi(qcm), _pi(qc))
    return hx, qc, qcm
