"""Host-side mirror of the SCALE-style das_letkf driver on one GPU.

``Sweep`` owns a letkf_sweep handle (include/letkf_gpu.h): grid points, the
bucket-sorted observations and the background / analysis ensembles stay in
device memory between calls; ``run`` analyses every point (local search,
letkf_core with transm / rdiag_wloc / minfl, update of every variable) the way
scale/letkf/letkf_tools.f90:38-476 does with relax_beta = 1.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .core import SCALE_PARAM_ORDER
from .lib import check, lib

PREC_F64 = 0
PREC_MIXED = 1
OPT_GRID_CAP = 1
OPT_MAX_SWEEPS = 2
OPT_EIGENSOLVER = 3
EIG_NEWTON_SCHULZ = 0
EIG_JACOBI = 1
OPT_TENSOR_CORES = 4
OPT_TC_NS_ITERS = 5
OPT_TC_NS_SCALING = 6
OPT_TC_NS_TOL = 7
OPT_POLISH_TOL = 8
OPT_GRAPH = 9
OPT_TC_POLISH = 10
OPT_TC_SCALE_BOUND = 11
OPT_POLISH_PROBE = 12
OPT_NS_COND = 13
OPT_MAX_NOBS_PER_GRID = 14
OPT_FAULT_WAIT = 15
OPT_GRID_SHARE = 16
OPT_COLUMN_UNIT = 17


class SweepDesc(C.Structure):
    _fields_ = [("ne", C.c_int), ("nv", C.c_int), ("nlon", C.c_int), ("nlat", C.c_int), ("npts", C.c_int),
                ("precision", C.c_int), ("params", C.c_double * 16), ("minfl", C.c_double)]


_SIGS = {
    "letkf_sweep_create": [C.c_void_p, C.c_void_p],
    "letkf_sweep_destroy": [C.c_void_p],
    "letkf_sweep_set_points": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "letkf_sweep_set_obs": [C.c_void_p, C.c_int] + [C.c_void_p] * 9 + [C.c_int, C.c_void_p, C.c_int],
    "letkf_sweep_set_background": [C.c_void_p, C.c_void_p, C.c_int],
    "letkf_sweep_set_inflation": [C.c_void_p, C.c_void_p, C.c_int],
    "letkf_sweep_set_option": [C.c_void_p, C.c_int, C.c_int],
    "letkf_sweep_run": [C.c_void_p, C.c_void_p],
    "letkf_sweep_run_host": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p],
    "letkf_sweep_autotune": [C.c_void_p, C.c_int, C.c_void_p],
    "letkf_sweep_get_analysis": [C.c_void_p, C.c_void_p, C.c_int],
    "letkf_sweep_get_diagnostics": [C.c_void_p] * 5,
    "letkf_sweep_deferred": [C.c_void_p, C.c_void_p],
    "letkf_sweep_sorted_obs": [C.c_void_p, C.c_void_p],
    "letkf_sweep_device_buffers": [C.c_void_p] * 5,
    "letkf_sweep_set_obs_groups": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int],
    "letkf_sweep_set_probe": [C.c_void_p, C.c_int, C.c_void_p, C.c_int],
    "letkf_sweep_get_probe": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
}


def _L():
    L = lib()
    if not getattr(L, "_sweep_sigs", False):
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = args
        L._sweep_sigs = True
    return L


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Sweep:
    """One analysis domain resident on the GPU."""

    def __init__(self, ne, nv, nlon, nlat, npts, params, precision=PREC_MIXED, minfl=0.0):
        d = SweepDesc()
        d.ne, d.nv, d.nlon, d.nlat, d.npts, d.precision = ne, nv, nlon, nlat, npts, precision
        for i, k in enumerate(SCALE_PARAM_ORDER):
            d.params[i] = float(params[k])
        d.minfl = float(minfl)
        self.desc = d
        self.h = C.c_void_p()
        check(_L().letkf_sweep_create(C.byref(self.h), C.byref(d)), "letkf_sweep_create")
        self.dtype = np.float64 if precision == PREC_F64 else np.float32

    def close(self):
        if self.h:
            _L().letkf_sweep_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_points(self, ri, rj, rlev, rz=None, tile=4):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ri, rj, rlev)]
        z = None if rz is None else np.ascontiguousarray(rz, dtype=np.float64)
        check(_L().letkf_sweep_set_points(self.h, *[_p(x) for x in a], _p(z), int(tile)), "set_points")

    def set_obs(self, ri, rj, lev, dat, err, dep, cls, hdxf, varloc=None, var_local_row=None):
        f = lambda x: np.ascontiguousarray(x, dtype=np.float64)
        i = lambda x: None if x is None else np.ascontiguousarray(x, dtype=np.int32)
        hd = np.ascontiguousarray(hdxf)
        f32 = hd.dtype == np.float32
        if not f32:
            hd = np.ascontiguousarray(hd, dtype=np.float64)
        vl = None if var_local_row is None else f(var_local_row)
        args = [f(ri), f(rj), f(lev), f(dat), f(err), f(dep), i(cls), i(varloc)]
        self._keep = args
        check(_L().letkf_sweep_set_obs(self.h, int(len(args[0])), *[_p(x) for x in args], _p(vl),
                                       0 if vl is None else vl.size, _p(hd), int(f32)), "set_obs")

    def set_obs_groups(self, uid, typ, nid, ntyp):
        """Element uid (1..nid) and type (1..ntyp) of each observation of the
        last set_obs, in its input order: the groups of MAX_NOBS_PER_GRID."""
        u = np.ascontiguousarray(uid, dtype=np.int32)
        t = np.ascontiguousarray(typ, dtype=np.int32)
        check(_L().letkf_sweep_set_obs_groups(self.h, _p(u), _p(t), int(nid), int(ntyp)), "set_obs_groups")

    def set_probe(self, points, cap):
        """Record, in the next runs, what the fused search accepts for these
        grid points (up to cap entries each); empty points switch it off."""
        pts = np.ascontiguousarray(points, dtype=np.int32)
        self._probe = (pts.size, int(cap))
        check(_L().letkf_sweep_set_probe(self.h, int(pts.size), _p(pts) if pts.size else None, int(cap)),
              "set_probe")

    def probe(self):
        """(count [n], obs [n, cap] input-order indices (-1 past the count),
        rloc [n, cap] float32) of the probed points after a run."""
        n, cap = self._probe
        cnt = np.empty(n, dtype=np.int32)
        obs = np.empty((n, cap), dtype=np.int32)
        rl = np.empty((n, cap), dtype=np.float32)
        check(_L().letkf_sweep_get_probe(self.h, _p(cnt), _p(obs), _p(rl)), "get_probe")
        return cnt, obs, rl

    def set_background(self, xb):
        xb = np.ascontiguousarray(xb, dtype=self.dtype)
        check(_L().letkf_sweep_set_background(self.h, _p(xb), 0), "set_background")

    def set_background_device(self, ptr):
        check(_L().letkf_sweep_set_background(self.h, C.c_void_p(ptr), 1), "set_background")

    def set_inflation(self, infl):
        infl = np.ascontiguousarray(infl, dtype=np.float64)
        check(_L().letkf_sweep_set_inflation(self.h, _p(infl), 0), "set_inflation")

    def set_option(self, opt, value):
        check(_L().letkf_sweep_set_option(self.h, int(opt), int(value)), "set_option")

    def run(self, stream=None):
        s = None if stream is None else C.c_void_p(stream)
        check(_L().letkf_sweep_run(self.h, s), "letkf_sweep_run")

    def run_host(self, xb, xa=None, nchunks=16, stream=None):
        """One analysis from host memory with the copies overlapped
        (letkf_sweep_run_host): xb is an array [nv, npts, ne] or a host
        address; xa likewise (a new array when None).  Page-locked buffers
        (torch pin_memory) let the copies run beside the analysis.  Returns xa."""
        d = self.desc
        if isinstance(xb, int):
            pb = C.c_void_p(xb)
        else:
            xb = np.ascontiguousarray(xb, dtype=self.dtype)
            if xb.size != d.nv * d.npts * d.ne:
                raise ValueError("run_host: xb must hold nv * npts * ne values")
            pb = _p(xb)
        if xa is None:
            xa = np.empty((d.nv, d.npts, d.ne), dtype=self.dtype)
        if not isinstance(xa, int) and (xa.dtype != self.dtype or not xa.flags.c_contiguous
                                        or xa.size != d.nv * d.npts * d.ne):
            raise ValueError("run_host: xa must be a contiguous [nv, npts, ne] array of the handle's type")
        pa = C.c_void_p(xa) if isinstance(xa, int) else _p(xa)
        s = None if stream is None else C.c_void_p(stream)
        check(_L().letkf_sweep_run_host(self.h, pb, pa, int(nchunks), s), "letkf_sweep_run_host")
        return xa

    def autotune(self, sample_points=32768):
        """Time the kernel / eigensolver variants on the first sample_points
        points (letkf_sweep_autotune) and keep the fastest; returns the
        choice as a dict.  Points, observations and background must be set;
        the inflation field is restored."""
        ch = np.zeros(4, dtype=np.int32)
        check(_L().letkf_sweep_autotune(self.h, int(sample_points), _p(ch)), "letkf_sweep_autotune")
        return {"tensor_cores": bool(ch[0]), "eigensolver": "newton-schulz" if ch[1] else "jacobi",
                "scaled_steps": bool(ch[2]), "us_per_1000_points": int(ch[3])}

    def analysis(self):
        d = self.desc
        xa = np.empty((d.nv, d.npts, d.ne), dtype=self.dtype)
        check(_L().letkf_sweep_get_analysis(self.h, _p(xa), 0), "get_analysis")
        return xa

    def analysis_into(self, host_ptr):
        check(_L().letkf_sweep_get_analysis(self.h, C.c_void_p(host_ptr), 0), "get_analysis")

    def deferred(self):
        """Points the last mixed-form run handed to the Jacobi pass."""
        n = C.c_int(0)
        check(_L().letkf_sweep_deferred(self.h, C.byref(n)), "letkf_sweep_deferred")
        return n.value

    def diagnostics(self):
        n = self.desc.npts
        infl = np.empty(n)
        nobsl = np.empty(n, dtype=np.int32)
        status = np.empty(n, dtype=np.int32)
        sweeps = np.empty(n, dtype=np.int32)
        check(_L().letkf_sweep_get_diagnostics(self.h, _p(infl), _p(nobsl), _p(status), _p(sweeps)), "diag")
        return dict(infl=infl, nobsl=nobsl, status=status, sweeps=sweeps)

    def nobsgrd(self):
        d = self.desc
        g = np.empty((d.nlat, d.nlon + 1), dtype=np.int32)
        check(_L().letkf_sweep_sorted_obs(self.h, _p(g)), "sorted_obs")
        return g

    def device_buffers(self):
        xb, xa, infl, nl = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(_L().letkf_sweep_device_buffers(self.h, C.byref(xb), C.byref(xa), C.byref(infl), C.byref(nl)),
              "device_buffers")
        return xb.value, xa.value, infl.value, nl.value
