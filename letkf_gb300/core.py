"""Host-side mirror of the reference's letkf_core interface and the batched
device entry points.

``letkf_core`` keeps the argument list, meaning and error behaviour of
SUBROUTINE letkf_core (common/common_letkf.f90:50): hdxb is (nobs, ne) with
only the first nobsl rows used, parm_infl is updated, transm / pao are the
optional outputs, rdiag_wloc and minfl the optional inputs.  Where the
reference STOPs (common/common_mtx.f90:61-64,75-78) this raises LetkfError.

The batched wrappers take torch CUDA tensors (device memory and streams are
torch's; the arithmetic is the library's) and call the C ABI with raw device
pointers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import LETKF_ERR_ARG, LETKF_OK, LetkfError, check, lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def letkf_core(ne, nobs, nobsl, hdxb, rdiag, rloc, dep, parm_infl, transm=False, pao=False, rdiag_wloc=False,
               minfl=None):
    """One LETKF analysis on the GPU (FP64 plain form).

    Returns ``(trans, transm, pao, parm_infl)``; ``transm`` / ``pao`` are None
    unless requested.  ``trans[k, m]`` is the weight of background member k
    in analysis member m (Fortran trans(k+1, m+1))."""
    hdxb = np.asfortranarray(hdxb, dtype=np.float64)
    if hdxb.shape != (nobs, ne):
        raise LetkfError(LETKF_ERR_ARG, f"hdxb shape {hdxb.shape} != (nobs, ne) = ({nobs}, {ne})")
    rdiag = np.ascontiguousarray(rdiag, dtype=np.float64)
    rloc = np.ascontiguousarray(rloc, dtype=np.float64)
    dep = np.ascontiguousarray(dep, dtype=np.float64)
    infl = np.array([parm_infl], dtype=np.float64)
    trans = np.zeros((ne, ne), dtype=np.float64, order="F")
    tm = np.zeros(ne) if transm else None
    pa = np.zeros((ne, ne), order="F") if pao else None
    mf = float(minfl) if minfl is not None else 0.0
    st = lib().letkf_core_c(ne, nobs, nobsl, _ptr(hdxb), _ptr(rdiag), _ptr(rloc), _ptr(dep), _ptr(infl),
                            _ptr(trans), _ptr(tm), _ptr(pa), int(bool(rdiag_wloc)), mf)
    check(st, "letkf_core")
    return trans, tm, pa, float(infl[0])


# ---------------------------------------------------------------- device side
def _dptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _viewptr(t):
    """Pointer to the first element of a strided CUDA view (the callee takes
    the strides separately)."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _stream(stream):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def core_batch_f64(ne, offs, rows, rdiag, rloc, dep, parm_infl, want_transm=False, want_pao=False,
                   rdiag_wloc=False, minfl=0.0, stream=None):
    """Batched FP64 plain form.  offs int64 [npts+1]; rows float64 [nrows, ne];
    parm_infl float64 [npts] is updated in place.  Returns dict of tensors
    (trans [npts, ne, ne] with trans[p, m, k] = trans_p(k, m), transm, pao,
    status)."""
    import torch

    npts = offs.numel() - 1
    dev = rows.device
    trans = torch.empty((npts, ne, ne), dtype=torch.float64, device=dev)
    tm = torch.empty((npts, ne), dtype=torch.float64, device=dev) if want_transm else None
    pa = torch.empty((npts, ne, ne), dtype=torch.float64, device=dev) if want_pao else None
    status = torch.empty(npts, dtype=torch.int32, device=dev)
    st = lib().letkf_core_batch_f64(ne, npts, _dptr(offs), _dptr(rows), _dptr(rdiag), _dptr(rloc), _dptr(dep),
                                    _dptr(parm_infl), _dptr(trans), _dptr(tm), _dptr(pa), int(bool(rdiag_wloc)),
                                    float(minfl), _dptr(status), _stream(stream))
    check(st, "letkf_core_batch_f64")
    return dict(trans=trans, transm=tm, pao=pa, status=status, parm_infl=parm_infl)


def core_batch_mixed(ne, offs, rows, rdiag, rloc, dep, parm_infl, want_transm=False, rdiag_wloc=False, minfl=0.0,
                     stream=None):
    """Batched mixed-precision core: float32 rows / rdiag / rloc / dep, float64
    parm_infl (in place).  Returns dict of tensors (float32 trans, transm)."""
    import torch

    npts = offs.numel() - 1
    dev = rows.device
    trans = torch.empty((npts, ne, ne), dtype=torch.float32, device=dev)
    tm = torch.empty((npts, ne), dtype=torch.float32, device=dev) if want_transm else None
    status = torch.empty(npts, dtype=torch.int32, device=dev)
    st = lib().letkf_core_batch_mixed(ne, npts, _dptr(offs), _dptr(rows), _dptr(rdiag), _dptr(rloc), _dptr(dep),
                                      _dptr(parm_infl), _dptr(trans), _dptr(tm), int(bool(rdiag_wloc)), float(minfl),
                                      _dptr(status), _stream(stream))
    check(st, "letkf_core_batch_mixed")
    return dict(trans=trans, transm=tm, status=status, parm_infl=parm_infl)


def core_batch_largek(ne, offs, rows, rdiag, rloc, dep, parm_infl, want_transm=False, rdiag_wloc=False, minfl=0.0,
                      stream=None):
    """Large-ensemble batched core (ne up to 1024; tensor-core Gram and
    Newton-Schulz): float32 rows / rdiag / rloc / dep, float64 parm_infl (in
    place).  Returns dict of tensors (float32 trans, transm, int32 status)."""
    import torch

    npts = offs.numel() - 1
    dev = rows.device
    trans = torch.empty((npts, ne, ne), dtype=torch.float32, device=dev)
    tm = torch.empty((npts, ne), dtype=torch.float32, device=dev) if want_transm else None
    status = torch.empty(npts, dtype=torch.int32, device=dev)
    st = lib().letkf_core_batch_largek(ne, npts, _dptr(offs), _dptr(rows), _dptr(rdiag), _dptr(rloc), _dptr(dep),
                                       _dptr(parm_infl), _dptr(trans), _dptr(tm), int(bool(rdiag_wloc)),
                                       float(minfl), _dptr(status), _stream(stream))
    check(st, "letkf_core_batch_largek")
    return dict(trans=trans, transm=tm, status=status, parm_infl=parm_infl)


def core_batch_largek_indexed(ne, offs, idx, ens_obs, dep_obs, rdiag, rloc, parm_infl, want_transm=False,
                              rdiag_wloc=False, minfl=0.0, stream=None):
    """Large-ensemble core over a search's index lists (letkf_core_batch_largek_indexed):
    offs int64 [npts+1], idx int32 [nrows] (observation of each entry),
    ens_obs [nobs, ne] float32 or bfloat16, dep_obs float32 [nobs], rdiag and
    rloc float32 [nrows], parm_infl float64 (in place)."""
    import torch

    npts = offs.numel() - 1
    dev = ens_obs.device
    trans = torch.empty((npts, ne, ne), dtype=torch.float32, device=dev)
    tm = torch.empty((npts, ne), dtype=torch.float32, device=dev) if want_transm else None
    status = torch.empty(npts, dtype=torch.int32, device=dev)
    bf = ens_obs.dtype == torch.bfloat16
    st = lib().letkf_core_batch_largek_indexed(ne, npts, _dptr(offs), _dptr(idx), _dptr(ens_obs), int(bf),
                                               _dptr(dep_obs), _dptr(rdiag), _dptr(rloc), _dptr(parm_infl),
                                               _dptr(trans), _dptr(tm), int(bool(rdiag_wloc)), float(minfl),
                                               _dptr(status), _stream(stream))
    check(st, "letkf_core_batch_largek_indexed")
    return dict(trans=trans, transm=tm, status=status, parm_infl=parm_infl)


def update_bf16(xmean, xpert, trans, transm=None, stream=None):
    """Update with BF16 storage (letkf_update_bf16): xmean float32 [nv, npts],
    xpert bfloat16 [nv, npts, ne]; returns (amean float32, apert bfloat16)."""
    import torch

    nv, npts, ne = xpert.shape
    amean = torch.empty_like(xmean)
    apert = torch.empty_like(xpert)
    check(lib().letkf_update_bf16(ne, npts, nv, _dptr(xmean), _dptr(xpert), _dptr(trans), _dptr(transm),
                                  _dptr(amean), _dptr(apert), _stream(stream)), "letkf_update_bf16")
    return amean, apert


def update_mixed(xb, trans, transm=None, stream=None):
    """FP32 update for any ne <= 512: xb float32 [nv, npts, ne], trans float32
    [npts, ne, ne] column-major per point; returns xa like xb."""
    import torch

    nv, npts, ne = xb.shape
    xa = torch.empty_like(xb)
    check(lib().letkf_update_mixed(ne, npts, nv, _dptr(xb), _dptr(trans), _dptr(transm), _dptr(xa),
                                   _stream(stream)), "letkf_update_mixed")
    return xa


def update_f64(xb, trans, transm=None, stream=None):
    """xb float64 [nv, npts, ne] full members; trans [npts, ne, ne] (column-
    major per point); returns xa like xb."""
    import torch

    nv, npts, ne = xb.shape
    xa = torch.empty_like(xb)
    st = lib().letkf_update_f64(ne, npts, nv, _dptr(xb), _dptr(trans), _dptr(transm), _dptr(xa), _stream(stream))
    check(st, "letkf_update_f64")
    return xa


class RelaxDesc(C.Structure):
    _fields_ = [("mode", C.c_int), ("alpha", C.c_double), ("beta", C.c_void_p), ("q_var", C.c_int),
                ("q_sprd_max", C.c_double)]


RELAX_NONE, RELAX_RTPP, RELAX_RTPS = 0, 1, 2


def update_relax_f64(xb, trans, transm=None, pao=None, mode=RELAX_NONE, alpha=0.0, beta=None, q_var=-1,
                     q_sprd_max=0.0, stream=None):
    """Relaxed update (scale/letkf/letkf_tools.f90:215-268): RTPP / RTPS,
    relax_beta weights and the q spread clip.  xb float64 [nv, npts, ne];
    trans / pao [npts, ne, ne] column-major per point; beta [nv, npts] or
    None.  Returns (xa, rtps_infl [nv, npts] or None)."""
    import torch

    nv, npts, ne = xb.shape
    xa = torch.empty_like(xb)
    infl = torch.empty((nv, npts), dtype=torch.float64, device=xb.device) if mode == RELAX_RTPS else None
    rd = RelaxDesc(int(mode), float(alpha), None if beta is None else beta.data_ptr(), int(q_var), float(q_sprd_max))
    st = lib().letkf_update_relax_f64(ne, npts, nv, _dptr(xb), _dptr(trans), _dptr(transm), _dptr(pao),
                                      C.byref(rd), _dptr(xa), _dptr(infl), _stream(stream))
    check(st, "letkf_update_relax_f64")
    return xa, infl


def relax_beta(ri, rj, rlev, nv, q_lo=-1, q_hi=-2, q_update_top=0.0, boundary_buffer_width=0.0, dx=1.0, dy=1.0,
               nlong=1, nlatg=1, ihalo=0, jhalo=0, stream=None):
    """relax_beta (scale/letkf/letkf_tools.f90:1182-1220) for every point and
    variable (0-based variable indices q_lo..q_hi); returns beta [nv, npts]."""
    import torch

    npts = ri.numel()
    beta = torch.empty((nv, npts), dtype=torch.float64, device=ri.device)
    check(lib().letkf_relax_beta(npts, nv, _dptr(ri), _dptr(rj), _dptr(rlev), int(q_lo), int(q_hi),
                                 float(q_update_top), float(boundary_buffer_width), float(dx), float(dy), int(nlong),
                                 int(nlatg), int(ihalo), int(jhalo), _dptr(beta), _stream(stream)), "relax_beta")
    return beta


def obs_analysis(trans, ybar, hdxf, relax_alpha=0.0, mode=None, q_sprd_max=0.0, stream=None):
    """Analysis ensemble at observation locations (gfs/letkf/letkf_tools.f90:
    466-497).  trans float64 [n, ne, ne] (merged T + wbar, column-major per
    point), ybar [n], hdxf [n, ne]; mode int32 [n] or None.  Returns (anal
    [n, ne], mean [n])."""
    import torch

    n, ne = hdxf.shape
    anal = torch.empty_like(hdxf)
    mean = torch.empty(n, dtype=torch.float64, device=hdxf.device)
    check(lib().letkf_obs_analysis(ne, n, _dptr(trans), _dptr(ybar), _dptr(hdxf), float(relax_alpha), _dptr(mode),
                                   float(q_sprd_max), _dptr(anal), _dptr(mean), _stream(stream)), "letkf_obs_analysis")
    return anal, mean


def efso(ne, offs, idx, rdiag, rloc, hdxa, fcst, fcer, term, obsdep, stream=None):
    """Observation sensitivity (gfs/letkf/letkf_tools.f90:547-679) on device
    tensors: local lists offs/idx/rdiag/rloc, hdxa [nobs, ne], fcst [nv, npts,
    ne], fcer [nv, npts], term (host list, one entry per variable), obsdep
    [nobs].  Returns (djdy, obsense), each [nobs, nterm]."""
    import torch

    nv, npts, _ = fcst.shape
    term = np.ascontiguousarray(term, dtype=np.int32)
    nterm = int(term.max()) + 1
    nobs = hdxa.shape[0]
    djdy = torch.empty((nobs, nterm), dtype=torch.float64, device=hdxa.device)
    obsense = torch.empty_like(djdy)
    check(lib().letkf_efso(ne, npts, nv, nterm, term.ctypes.data_as(C.c_void_p), _dptr(offs), _dptr(idx),
                           _dptr(rdiag), _dptr(rloc), nobs, _dptr(hdxa), _dptr(fcst), _dptr(fcer), _dptr(obsdep),
                           _dptr(djdy), _dptr(obsense), _stream(stream)), "letkf_efso")
    return djdy, obsense


SPEEDY_ELEM = {"u": 2819, "v": 2820, "t": 3073, "q": 3330, "rh": 3331, "ps": 14593, "rain": 9999}
SCALE_ELEM = {"u": 2819, "v": 2820, "t": 3073, "tv": 3074, "q": 3330, "rh": 3331, "ps": 14593}


def scale_obsope(v3d, v2d, khalo, elem, ri, rj, rlev, rotc=None, stggrd=0, ps_adjust_thres=100.0,
                 want_member_qc=False, stream=None):
    """SCALE observation operator for conventional observations, all members
    (scale/obs/obsope_tools.f90:340-380: phys2ijk and Trans_XtoY of
    scale/common/common_obs_scale.f90).  v3d: float64 [ne, 6, nlath, nlonh,
    nlevh] (u, v, t, q, rh, full pressure; levels fastest as the reference's
    v3dg; nlevh = nlev + 2 khalo), v2d: float64 [ne, 4, nlath, nlonh] (ps,
    t2m, q2m, topo), each contiguous per variable; observations elem (int32) /
    ri / rj (halo-domain grid coordinates) / rlev [nobs], rotc [nobs, 2] or
    None, all on the device.  Returns (hx [nobs, ne], qc [nobs] int32, the
    maximum over members) and, with want_member_qc, qc per member."""
    import torch

    ne, nv3, nlath, nlonh, nlevh = v3d.shape
    nlev = nlevh - 2 * khalo
    if nv3 != 6 or tuple(v2d.shape) != (ne, 4, nlath, nlonh):
        raise ValueError("scale_obsope: v3d [ne, 6, nlath, nlonh, nlevh] and v2d [ne, 4, nlath, nlonh] expected")
    for t in (v3d, v2d):
        if t.dtype != torch.float64 or not t[0, 0].is_contiguous():
            raise ValueError("scale_obsope: float64 fields, each variable contiguous, expected")
    nobs = elem.numel()
    hx = torch.empty((nobs, ne), dtype=torch.float64, device=v3d.device)
    qc = torch.empty(nobs, dtype=torch.int32, device=v3d.device)
    qcm = torch.empty((nobs, ne), dtype=torch.int32, device=v3d.device) if want_member_qc else None
    check(lib().letkf_scale_obsope(nlonh, nlath, nlev, int(khalo), ne, _viewptr(v3d), v3d.stride(0), v3d.stride(1),
                                   _viewptr(v2d), v2d.stride(0), v2d.stride(1), nobs, _dptr(elem), _dptr(ri),
                                   _dptr(rj), _dptr(rlev), _dptr(rotc), int(stggrd), float(ps_adjust_thres),
                                   _dptr(hx), _dptr(qcm), _dptr(qc), _stream(stream)), "letkf_scale_obsope")
    return (hx, qc, qcm) if want_member_qc else (hx, qc)


def speedy_obsope(lat, sig, v3d, v2d, elem, rlon, rlat, rlev, odat, want_member_qc=False, stream=None):
    """SPEEDY observation operator for all members (speedy/letkf/obsope.f90:
    53-104 with phys2ijk / Trans_XtoY of speedy/common/common_obs_speedy.f90).
    v3d: float64 view shaped [ne, 4, nlev, nlat, nlon] (u, v, t, q) whose two
    last dims are contiguous and whose variable stride is nlev times the level
    stride (a stack of grd files, or the analysis layout [4, nlev, ne, nij]
    permuted); v2d: [ne, 2, nlat, nlon] (ps, rain) likewise.  lat [nlat], sig
    [nlev], observations elem (int32 codes) / rlon / rlat / rlev / odat [nobs],
    all on the device.  Returns (hx [nobs, ne], qc [nobs] int32) and, with
    want_member_qc, qc per member [nobs, ne]."""
    import torch

    ne, nv3, nlev, nlat, nlon = v3d.shape
    if nv3 != 4 or v2d.shape[0] != ne or v2d.shape[1] < 2 or tuple(v2d.shape[2:]) != (nlat, nlon):
        raise ValueError("speedy_obsope: v3d [ne, 4, nlev, nlat, nlon] and v2d [ne, 2, nlat, nlon] expected")
    for t, rs in ((v3d, v3d.stride(2)), (v2d, v2d.stride(1))):
        if t.dtype != torch.float64 or t.stride(-1) != 1 or t.stride(-2) != nlon:
            raise ValueError("speedy_obsope: float64 fields with contiguous (lat, lon) planes expected")
    if v3d.stride(1) != nlev * v3d.stride(2):
        raise ValueError("speedy_obsope: v3d variable stride must be nlev times its level stride")
    nobs = elem.numel()
    hx = torch.empty((nobs, ne), dtype=torch.float64, device=v3d.device)
    qc = torch.empty(nobs, dtype=torch.int32, device=v3d.device)
    qcm = torch.empty((nobs, ne), dtype=torch.int32, device=v3d.device) if want_member_qc else None
    check(lib().letkf_speedy_obsope(nlon, nlat, nlev, ne, _dptr(lat), _dptr(sig), _viewptr(v3d), v3d.stride(0),
                                    v3d.stride(2), _viewptr(v2d), v2d.stride(0), v2d.stride(1), nobs, _dptr(elem),
                                    _dptr(rlon), _dptr(rlat), _dptr(rlev), _dptr(odat), _dptr(hx), _dptr(qcm),
                                    _dptr(qc), _stream(stream)), "letkf_speedy_obsope")
    return (hx, qc, qcm) if want_member_qc else (hx, qc)


def exclusive_scan(counts, stream=None):
    import torch

    offs = torch.empty(counts.numel() + 1, dtype=torch.int64, device=counts.device)
    check(lib().letkf_exclusive_scan(counts.numel(), _dptr(counts), _dptr(offs), _stream(stream)), "scan")
    return offs


def exclusive_scan_static(counts, offs, stream=None):
    """Allocation-free scan into the caller's offs (int64 [n+1]); returns the
    status code instead of raising, for callers that check it themselves."""
    return int(lib().letkf_exclusive_scan_static(counts.numel(), _dptr(counts), _dptr(offs), _stream(stream)))


def gather_rows(idx, ens, dep, stream=None):
    """rows[r] = ens[idx[r]], dep_out[r] = dep[idx[r]] (same dtype as ens)."""
    import torch

    nrows = idx.numel()
    ne = ens.shape[1]
    rows = torch.empty((nrows, ne), dtype=ens.dtype, device=ens.device)
    dout = torch.empty(nrows, dtype=ens.dtype, device=ens.device)
    check(lib().letkf_gather_rows(ne, nrows, _dptr(idx), _dptr(ens), _dptr(dep), ens.element_size(), _dptr(rows),
                                  _dptr(dout), _stream(stream)), "gather_rows")
    return rows, dout


SCALE_PARAM_ORDER = ("dx", "dy", "dlon_zero", "dlat_zero", "sigma_obs", "sigma_obsv", "sigma_obs_rain",
                     "sigma_obsv_rain", "base_obsv_rain", "sigma_obs_radar", "sigma_obs_radar_noref",
                     "sigma_obsz_radar", "radar_ref_thres_dbz", "sigma_obs_tc", "sigma_obsv_tc")


def search_scale(nlon, nlat, nobsgrd, obs, pts, params, var_local_row=None, stream=None):
    """SCALE Cartesian local search on device tensors.
    obs: dict of tensors ri, rj, lev, dat, err (float64), cls, varloc (int32), sorted.
    pts: dict ri, rj, rlev (float64) [, rz].  params: dict with SCALE_PARAM_ORDER keys.
    Returns (offs int64 [npts+1], idx int32, rloc, rdiag float64)."""
    import torch

    dev = obs["ri"].device
    npts = pts["ri"].numel()
    nobs = obs["ri"].numel()
    P = torch.tensor([float(params[k]) for k in SCALE_PARAM_ORDER] + [0.0], dtype=torch.float64)
    vl = None if var_local_row is None else torch.as_tensor(var_local_row, dtype=torch.float64, device=dev)
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    args = (nlon, nlat, _dptr(nobsgrd), nobs, _dptr(obs["ri"]), _dptr(obs["rj"]), _dptr(obs["lev"]),
            _dptr(obs["dat"]), _dptr(obs["err"]), _dptr(obs["cls"]), _dptr(obs["varloc"]), npts, _dptr(pts["ri"]),
            _dptr(pts["rj"]), _dptr(pts["rlev"]), _dptr(pts.get("rz")), _dptr(vl), C.c_void_p(P.data_ptr()))
    check(lib().letkf_search_scale(*args, None, _dptr(nobsl), None, None, None, _stream(stream)), "search_scale")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_scale(*args, _dptr(offs), _dptr(nobsl), _dptr(idx), _dptr(rloc), _dptr(rdiag),
                                   _stream(stream)), "search_scale")
    return offs, idx[:total], rloc[:total], rdiag[:total]


def search_scale_limited(nlon, nlat, nobsgrd, obs, pts, params, max_nobs_per_grid, nid, var_local_row=None,
                         stream=None):
    """SCALE search with the MAX_NOBS_PER_GRID limit (letkf_search_scale_limited).
    obs as for search_scale plus uid, typ (int32, 1-based element uid and obs
    type of each sorted observation); nid is the number of element uids.
    Returns (offs, idx, rloc, rdiag) as search_scale."""
    import torch

    dev = obs["ri"].device
    npts = pts["ri"].numel()
    nobs = obs["ri"].numel()
    P = torch.tensor([float(params[k]) for k in SCALE_PARAM_ORDER] + [0.0], dtype=torch.float64)
    vl = None if var_local_row is None else torch.as_tensor(var_local_row, dtype=torch.float64, device=dev)
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    args = (nlon, nlat, _dptr(nobsgrd), nobs, _dptr(obs["ri"]), _dptr(obs["rj"]), _dptr(obs["lev"]),
            _dptr(obs["dat"]), _dptr(obs["err"]), _dptr(obs["cls"]), _dptr(obs["varloc"]), _dptr(obs["uid"]),
            _dptr(obs["typ"]), int(nid), int(max_nobs_per_grid), npts, _dptr(pts["ri"]), _dptr(pts["rj"]),
            _dptr(pts["rlev"]), _dptr(pts.get("rz")), _dptr(vl), C.c_void_p(P.data_ptr()))
    check(lib().letkf_search_scale_limited(*args, None, _dptr(nobsl), None, None, None, _stream(stream)),
          "search_scale_limited")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_scale_limited(*args, _dptr(offs), _dptr(nobsl), _dptr(idx), _dptr(rloc),
                                           _dptr(rdiag), _stream(stream)), "search_scale_limited")
    return offs, idx[:total], rloc[:total], rdiag[:total]


def sort_obs_latlon(lon, lat, olon, olat, qc=None, stream=None):
    """SPEEDY / GFS bucket sort on the device (letkf_sort_obs_latlon): lon
    [nlon], lat [nlat], olon, olat [nobs] float64 tensors, qc optional int32
    (only qc == 1 kept).  Returns (perm int32 [nsorted]: input index of each
    kept observation in sorted order, nobsgrd int32 [nlat, nlon])."""
    import torch

    dev = olon.device
    nlon, nlat, nobs = lon.numel(), lat.numel(), olon.numel()
    perm = torch.empty(max(nobs, 1), dtype=torch.int32, device=dev)
    grd = torch.empty((nlat, nlon), dtype=torch.int32, device=dev)
    ns = C.c_int(0)
    check(lib().letkf_sort_obs_latlon(nlon, nlat, _dptr(lon), _dptr(lat), nobs, _dptr(olon), _dptr(olat),
                                      _dptr(qc), _dptr(perm), C.byref(ns), _dptr(grd), _stream(stream)),
          "sort_obs_latlon")
    return perm[:ns.value], grd


def search_speedy(grid, obs, pts, params, var_local_row, stream=None):
    """SPEEDY lat/lon local search on device tensors.
    grid: dict lon, lat (float64), nobsgrd (int32 [nlat, nlon]).
    obs: dict elm, lon, lat, lev, dat, err (float64), sorted.
    pts: dict lon, lat, dlon_zero, logpfm (float64), ilev (int32, 1-based).
    params: (dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv)."""
    import torch

    dev = obs["lon"].device
    npts = pts["lon"].numel()
    P = torch.tensor([float(x) for x in params], dtype=torch.float64)
    vl = torch.as_tensor(var_local_row, dtype=torch.float64, device=dev).contiguous()
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    nlat, nlon = grid["nobsgrd"].shape
    args = (nlon, nlat, _dptr(grid["lon"]), _dptr(grid["lat"]), _dptr(grid["nobsgrd"]), obs["lon"].numel(),
            _dptr(obs["elm"]), _dptr(obs["lon"]), _dptr(obs["lat"]), _dptr(obs["lev"]), _dptr(obs["dat"]),
            _dptr(obs["err"]), npts, _dptr(pts["lon"]), _dptr(pts["lat"]), _dptr(pts["dlon_zero"]),
            _dptr(pts["ilev"]), _dptr(pts["logpfm"]), _dptr(vl), C.c_void_p(P.data_ptr()))
    check(lib().letkf_search_speedy(*args, None, _dptr(nobsl), None, None, None, _stream(stream)), "search_speedy")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_speedy(*args, _dptr(offs), _dptr(nobsl), _dptr(idx), _dptr(rloc), _dptr(rdiag),
                                    _stream(stream)), "search_speedy")
    return offs, idx[:total], rloc[:total], rdiag[:total]


GFS_PARAM_ORDER = ("dist_zero", "dist_zerov", "dist_zero_rain", "dist_zerov_rain", "sigma_obs", "sigma_obsv",
                   "sigma_obs_rain", "base_obsv_rain")


def search_gfs(grid, obs, pts, params, var_local_row=None, stream=None):
    """GFS lat/lon search (gfs/letkf/letkf_tools.f90:686-955) on device tensors.
    grid: dict lon, lat (float64), nobsgrd (int32 [nlat, nlon]); obs: dict elm,
    lon, lat, lev, dat, err (float64, bucket-sorted); pts: dict lon, lat, rlev
    (float64, rlev = the point's pressure); params: dict with GFS_PARAM_ORDER
    keys; var_local_row: 6 weights or None (nvar = 0).  Returns (offs, idx,
    rloc, rdiag)."""
    import torch

    dev = obs["lon"].device
    npts = pts["lon"].numel()
    nlat, nlon = grid["nobsgrd"].shape
    nobs = obs["lon"].numel()
    P = torch.tensor([float(params[k]) for k in GFS_PARAM_ORDER], dtype=torch.float64)
    vl = None if var_local_row is None else torch.as_tensor(var_local_row, dtype=torch.float64, device=dev)
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    args = (nlon, nlat, _dptr(grid["lon"]), _dptr(grid["lat"]), _dptr(grid["nobsgrd"]), nobs, _dptr(obs["elm"]),
            _dptr(obs["lon"]), _dptr(obs["lat"]), _dptr(obs["lev"]), _dptr(obs["dat"]), _dptr(obs["err"]), npts,
            _dptr(pts["lon"]), _dptr(pts["lat"]), _dptr(pts["rlev"]), _dptr(vl),
            C.c_void_p(P.data_ptr()))
    check(lib().letkf_search_gfs(*args, None, _dptr(nobsl), None, None, None, _stream(stream)), "search_gfs")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_gfs(*args, _dptr(offs), None, _dptr(idx), _dptr(rloc), _dptr(rdiag), _stream(stream)),
          "search_gfs")
    return offs, idx[:total], rloc[:total], rdiag[:total]


def l96_obs_cell(h, stream=None):
    """Grid index (1-based) of each Lorenz-96 observation: the first maximum of
    its row of h (ny, nx) (lorenz96/letkf/letkf.f90:226-228).  h: device tensor."""
    import torch

    ny, nx = h.shape
    hf = h.to(torch.float64).t().contiguous()  # column-major (ny x nx)
    cell = torch.empty(ny, dtype=torch.int32, device=h.device)
    check(lib().letkf_l96_obs_cell(nx, ny, _dptr(hf), _dptr(cell), _stream(stream)), "l96_obs_cell")
    return cell


def obs_departure(hx, y, err=None, gross_error=0.0, qc=None, stream=None):
    """Observation-space perturbations and departures (speedy/letkf/
    letkf_obs.f90:157-174): hx float64 [nobs, ne] -> (hdxf, dep, qc_out)."""
    import torch

    nobs, ne = hx.shape
    hx = hx.contiguous()
    y = y.contiguous()
    hdxf = torch.empty_like(hx)
    dep = torch.empty(nobs, dtype=torch.float64, device=hx.device)
    qc_out = torch.empty(nobs, dtype=torch.int32, device=hx.device)
    check(lib().letkf_obs_departure(ne, nobs, _dptr(hx), _dptr(y), _dptr(err), float(gross_error), _dptr(qc),
                                    _dptr(hdxf), _dptr(dep), _dptr(qc_out), _stream(stream)), "obs_departure")
    return hdxf, dep, qc_out


def search_l96(nx, obs_cell, pix, xlocal=3.0, obserr=1.0, tdif=0.0, tlocal=-1.0, stream=None):
    """Lorenz-96 selection (lorenz96/letkf/letkf.f90:220-254) on device tensors.
    obs_cell int32 [ny] (1-based grid index per observation), pix int32 [npts]
    (1-based).  Returns (offs int64 [npts+1], idx int32, rloc, rdiag float64)."""
    import torch

    dev = obs_cell.device
    npts, ny = pix.numel(), obs_cell.numel()
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    args = (nx, ny, _dptr(obs_cell), npts, _dptr(pix), float(xlocal), float(tdif), float(tlocal), float(obserr))
    check(lib().letkf_search_l96(*args, None, _dptr(nobsl), None, None, None, _stream(stream)), "search_l96")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_l96(*args, _dptr(offs), None, _dptr(idx), _dptr(rloc), _dptr(rdiag), _stream(stream)),
          "search_l96")
    return offs, idx[:total], rloc[:total], rdiag[:total]


def search_l96_4d(nx, obs_cell, pix, slot, xlocal=3.0, obserr=1.0, tlocal=2.0, stream=None):
    """4D-LETKF selection of the Lorenz-96 driver (lorenz96/letkf/letkf.f90:
    217-254) for analysis slot `slot` (0-based): obs_cell int32 [nslot, ny]
    (1-based grid index per observation and slot), pix int32 [npts].  Returns
    (offs, idx, rloc, rdiag) with idx the row n*ny + i of the slot-stacked
    observations."""
    import torch

    dev = obs_cell.device
    nslot, ny = obs_cell.shape
    npts = pix.numel()
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    cell = obs_cell.contiguous()
    args = (nx, nslot, ny, _dptr(cell), npts, _dptr(pix), int(slot), float(xlocal), float(tlocal), float(obserr))
    check(lib().letkf_search_l96_4d(*args, None, _dptr(nobsl), None, None, None, _stream(stream)), "search_l96_4d")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_l96_4d(*args, _dptr(offs), None, _dptr(idx), _dptr(rloc), _dptr(rdiag),
                                    _stream(stream)), "search_l96_4d")
    return offs, idx[:total], rloc[:total], rdiag[:total]


def search_l96_adaptive(nx, obs_cell, pix, slot, hdxf, xf, msw_local=1, sa=1.0, sb=1.0, xlocal=3.0, obserr=1.0,
                        tlocal=2.0, stream=None):
    """Lorenz-96 selection with the localisation mode switch msw_local
    (lorenz96/letkf/letkf.f90:18-27,217-254): 0 fixed, 1 adaptive (ensemble
    correlation weights wa**sa * wb**sb), 2 both.  obs_cell int32 [nslot, ny]
    (or [ny] for one slot), pix int32 [npts] (1-based), slot 0-based analysis
    slot; hdxf float64 [nslot*ny, ne] slot-stacked obs-space perturbations, xf
    float64 [nx, ne] the analysis slot's first guess.  Returns (offs, idx, rloc,
    rdiag) with idx the row n*ny + i."""
    import torch

    dev = obs_cell.device
    cell = obs_cell.reshape(-1, obs_cell.shape[-1]).contiguous()
    nslot, ny = cell.shape
    npts = pix.numel()
    ne = xf.shape[1]
    if hdxf.shape != (nslot * ny, ne) or xf.shape[0] != nx:
        raise ValueError("search_l96_adaptive: hdxf must be [nslot*ny, ne] and xf [nx, ne]")
    hd = hdxf.to(torch.float64).contiguous()
    xr = xf.to(torch.float64).contiguous()
    nobsl = torch.empty(npts, dtype=torch.int32, device=dev)
    args = (nx, nslot, ny, _dptr(cell), npts, _dptr(pix), int(slot), float(xlocal), float(tlocal), float(obserr),
            int(msw_local), float(sa), float(sb), ne, _dptr(hd), _dptr(xr))
    check(lib().letkf_search_l96_adaptive(*args, None, _dptr(nobsl), None, None, None, _stream(stream)),
          "search_l96_adaptive")
    offs = exclusive_scan(nobsl, stream)
    total = int(offs[-1].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    rloc = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    rdiag = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    check(lib().letkf_search_l96_adaptive(*args, _dptr(offs), None, _dptr(idx), _dptr(rloc), _dptr(rdiag),
                                          _stream(stream)), "search_l96_adaptive")
    return offs, idx[:total], rloc[:total], rdiag[:total]


__all__ = ["letkf_core", "core_batch_f64", "core_batch_mixed", "update_f64", "exclusive_scan", "gather_rows",
           "search_scale", "search_speedy", "search_l96", "search_l96_4d", "search_l96_adaptive", "l96_obs_cell", "obs_departure", "update_relax_f64", "relax_beta", "core_batch_largek", "update_mixed", "obs_analysis", "efso", "RELAX_NONE", "RELAX_RTPP",
           "RELAX_RTPS", "LETKF_OK"]
