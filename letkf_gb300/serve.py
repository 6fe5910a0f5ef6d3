"""Analysis server: ctypes binding of letkf_server_* (include/letkf_gpu.h).

    srv = Server(nslots=3)
    job = srv.submit_sweep(...)     # or submit_l96(...); returns at once
    res = srv.wait(job)             # job.xa holds the analysis
    srv.stats()                     # p50 / p99 latency, points/s, peak bytes

The scheduling (queue, admission by device footprint, slots, resident
domains) is native code in libletkf_gpu.so; this module only packs host
arrays into job descriptors and keeps them alive until the job finishes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .core import SCALE_PARAM_ORDER
from .lib import LETKF_OK, LetkfError, check, lib

LETKF_PENDING = 7
JOB_SCALE_SWEEP = 0
JOB_L96 = 1
PREC_F64 = 0
PREC_MIXED = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class ServerDesc(C.Structure):
    _fields_ = [("device", C.c_int), ("nslots", C.c_int), ("hbm_budget", C.c_size_t)]


class JobDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("domain", C.c_int64), ("precision", C.c_int), ("ne", C.c_int), ("nv", C.c_int),
                ("nlon", C.c_int), ("nlat", C.c_int), ("npts", C.c_int), ("pri", _dp), ("prj", _dp), ("prlev", _dp),
                ("params", C.c_double * 16), ("minfl", C.c_double), ("nobs", C.c_int), ("ori", _dp), ("orj", _dp),
                ("olev", _dp), ("odat", _dp), ("oerr", _dp), ("ocls", _ip), ("obs_cell", _ip),
                ("xlocal", C.c_double), ("obserr", C.c_double), ("msw_infl", C.c_double), ("dep", _dp),
                ("hdxf", C.c_void_p), ("xb", C.c_void_p), ("xa", C.c_void_p), ("infl", _dp)]


class JobResult(C.Structure):
    _fields_ = [("status", C.c_int), ("t_submit", C.c_double), ("t_start", C.c_double), ("t_done", C.c_double),
                ("device_bytes", C.c_size_t)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double), ("points_per_s", C.c_double),
                ("peak_bytes", C.c_size_t), ("resident_domains", C.c_int)]


_SIGS = {
    "letkf_server_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(ServerDesc)]),
    "letkf_server_submit": (C.c_int, [C.c_void_p, C.POINTER(JobDesc), C.POINTER(C.c_int64)]),
    "letkf_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(JobResult)]),
    "letkf_server_stats_get": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "letkf_server_destroy": (C.c_int, [C.c_void_p]),
}


def _L():
    L = lib()
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        if fn.argtypes != args:
            fn.restype = res
            fn.argtypes = args
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _out_like(x, out):
    if out is None:
        return np.empty_like(x)
    if out.shape != x.shape or out.dtype != x.dtype or not out.flags.c_contiguous:
        raise ValueError("xa must be a contiguous array of the input's shape and type")
    return out


class Job:
    """A submitted job: its id, descriptor and the arrays it references."""

    def __init__(self, desc, keep, xa, infl, npts):
        self.desc, self.keep, self.xa, self.infl, self.npts = desc, keep, xa, infl, npts
        self.id = -1
        self.result = None


class Server:
    def __init__(self, nslots=2, hbm_budget=0, device=0):
        self.h = C.c_void_p()
        d = ServerDesc(int(device), int(nslots), int(hbm_budget))
        check(_L().letkf_server_create(C.byref(self.h), C.byref(d)), "letkf_server_create")
        self.jobs = {}

    # ---------------------------------------------------------------- submit
    def _submit(self, job):
        jid = C.c_int64(-1)
        check(_L().letkf_server_submit(self.h, C.byref(job.desc), C.byref(jid)), "letkf_server_submit")
        job.id = int(jid.value)
        self.jobs[job.id] = job
        return job

    def submit_sweep(self, pri, prj, prlev, params, nlon, nlat, obs, hdxf, dep, xb, infl=None, precision=PREC_MIXED,
                     domain=-1, minfl=0.0, xa=None):
        """A regional sweep job (letkf_sweep_* semantics).  obs: dict ri, rj,
        lev, dat, err (float64) and cls (int32), unsorted; hdxf [nobs, ne];
        xb [nv, npts, ne] (float32 for PREC_MIXED, else float64); params: dict
        with the SCALE search parameters.  xa: the output array (like xb; a
        new array when None), for instance page-locked memory."""
        dt = np.float32 if precision == PREC_MIXED else np.float64
        xb = np.ascontiguousarray(xb, dtype=dt)
        nv, npts, ne = xb.shape
        hd = np.ascontiguousarray(hdxf, dtype=dt)
        keep = {"pri": _f64(pri), "prj": _f64(prj), "prlev": _f64(prlev), "xb": xb, "hdxf": hd, "dep": _f64(dep),
                "cls": np.ascontiguousarray(obs["cls"], dtype=np.int32)}
        for k in ("ri", "rj", "lev", "dat", "err"):
            keep["o" + k] = _f64(obs[k])
        xa = _out_like(xb, xa)
        inf = None if infl is None else _f64(infl).copy()
        d = JobDesc()
        d.kind, d.domain, d.precision, d.ne, d.nv = JOB_SCALE_SWEEP, int(domain), int(precision), ne, nv
        d.nlon, d.nlat, d.npts = int(nlon), int(nlat), npts
        d.pri, d.prj, d.prlev = (keep[k].ctypes.data_as(_dp) for k in ("pri", "prj", "prlev"))
        for i, k in enumerate(SCALE_PARAM_ORDER):
            d.params[i] = float(params[k])
        d.minfl = float(minfl)
        d.nobs = keep["ori"].size
        d.ori, d.orj, d.olev, d.odat, d.oerr = (keep[k].ctypes.data_as(_dp) for k in ("ori", "orj", "olev", "odat",
                                                                                       "oerr"))
        d.ocls = keep["cls"].ctypes.data_as(_ip)
        d.dep = keep["dep"].ctypes.data_as(_dp)
        d.hdxf, d.xb, d.xa = hd.ctypes.data, xb.ctypes.data, xa.ctypes.data
        d.infl = None if inf is None else inf.ctypes.data_as(_dp)
        return self._submit(Job(d, keep, xa, inf, npts))

    def submit_l96(self, xf, hdxf, dep, obs_cell, obserr=1.0, xlocal=3.0, msw_infl=1.05, infl=None,
                   precision=PREC_F64, domain=-1, xa=None):
        """A Lorenz-96 analysis job (lorenz96/letkf/letkf.f90:180-265): xf
        [nx, ne] float64 members, hdxf [ny, ne] and dep [ny] from
        core.obs_departure semantics, obs_cell [ny] 1-based grid indices."""
        xf = _f64(xf)
        nx, ne = xf.shape
        keep = {"xb": xf, "hdxf": _f64(hdxf), "dep": _f64(dep),
                "cell": np.ascontiguousarray(obs_cell, dtype=np.int32)}
        xa = _out_like(xf, xa)
        inf = None if infl is None else _f64(infl).copy()
        d = JobDesc()
        d.kind, d.domain, d.precision, d.ne, d.nv = JOB_L96, int(domain), int(precision), ne, 1
        d.nlon, d.nlat, d.npts = nx, 1, nx
        d.nobs = keep["cell"].size
        d.obs_cell = keep["cell"].ctypes.data_as(_ip)
        d.xlocal, d.obserr, d.msw_infl = float(xlocal), float(obserr), float(msw_infl)
        d.dep = keep["dep"].ctypes.data_as(_dp)
        d.hdxf, d.xb, d.xa = keep["hdxf"].ctypes.data, xf.ctypes.data, xa.ctypes.data
        d.infl = None if inf is None else inf.ctypes.data_as(_dp)
        return self._submit(Job(d, keep, xa, inf, nx))

    # ------------------------------------------------------------------ wait
    def wait(self, job, timeout=None, raise_on_error=True):
        if job.result is not None and job.result["status"] != LETKF_PENDING:
            # the server released the record when it handed the result out
            if raise_on_error and job.result["status"] != LETKF_OK:
                raise LetkfError(job.result["status"], f"server job {job.id}")
            return job.result
        r = JobResult()
        st = _L().letkf_server_wait(self.h, job.id, -1.0 if timeout is None else float(timeout), C.byref(r))
        job.result = {"status": int(r.status), "t_submit": r.t_submit, "t_start": r.t_start, "t_done": r.t_done,
                      "latency_s": r.t_done - r.t_submit, "device_bytes": int(r.device_bytes)}
        if raise_on_error and st not in (LETKF_OK, LETKF_PENDING):
            raise LetkfError(st, f"server job {job.id}")
        return job.result

    def stats(self):
        s = ServerStats()
        check(_L().letkf_server_stats_get(self.h, C.byref(s)), "letkf_server_stats_get")
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            _L().letkf_server_destroy(self.h)
            self.h = C.c_void_p()
            self.jobs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Server", "Job", "JOB_SCALE_SWEEP", "JOB_L96", "PREC_F64", "PREC_MIXED", "LETKF_PENDING"]
