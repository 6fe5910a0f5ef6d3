"""SPEEDY driver files: ensemble grd files and observation records.

Grid files (speedy/common/common_speedy.f90:163-287) are direct-access, one
record of nlon*nlat REAL(4) per 2-D field (lon fastest): u at levels
1..nlev, then v, t, q, then ps and rain.  Observation files
(speedy/common/common_obs_speedy.f90:413-602) are Fortran sequential
unformatted: every record is a 4-byte length marker, REAL(4) values and the
marker again; obs records hold 6 values (elem, lon, lat, lev, dat, err) and
obs2 records 8 (the same plus hx and qc).  The reference builds with
-byteswapio (speedy/letkf/make_letkf.sh:6), so both kinds are big-endian by
default here; ``byteorder="<"`` reads little-endian files.

Ensembles go to the device as file bytes: the members' files are read back
to back into one pinned buffer, copied once, and ``letkf_grd_decode`` swaps,
widens and scatters them into the analysis layout [nv3d, nlev, ne, nlat*nlon]
(``speedy_letkf``'s gues3d) and [nv2d, ne, nlat*nlon]; writing is the
reverse through ``letkf_grd_encode``.  Observation files are small and are
parsed on the host with the reference's REAL(4) unit conversions.
"""
from __future__ import annotations

import os

import numpy as np

from .core import _dptr, _stream
from .lib import check, lib

ID_U, ID_V, ID_T, ID_Q, ID_RH, ID_PS, ID_RAIN = 2819, 2820, 3073, 3330, 3331, 14593, 9999
NV3D, NV2D = 4, 2


def grd_nrec(nlev, nv3d=NV3D, nv2d=NV2D):
    return nv3d * nlev + nv2d


def grd_nbytes(nlon, nlat, nlev, nv3d=NV3D, nv2d=NV2D):
    return 4 * nlon * nlat * grd_nrec(nlev, nv3d, nv2d)


def _swap(byteorder):
    """The device is little-endian: big-endian file bytes are swapped."""
    if byteorder not in (">", "<"):
        raise ValueError("byteorder must be '>' (big-endian) or '<' (little-endian)")
    return int(byteorder == ">")


# ------------------------------------------------------------------ host grd
def read_grd4(path, nlon, nlat, nlev, nv3d=NV3D, nv2d=NV2D, byteorder=">"):
    """read_grd4 (speedy/common/common_speedy.f90:196-224): returns float32
    (v3d [nv3d, nlev, nlat, nlon], v2d [nv2d, nlat, nlon])."""
    nrec = grd_nrec(nlev, nv3d, nv2d)
    need = grd_nbytes(nlon, nlat, nlev, nv3d, nv2d)
    size = os.path.getsize(path)
    if size < need:
        raise ValueError(f"{path}: {size} bytes, a grd file of {nrec} records of {nlon}x{nlat} needs {need}")
    a = np.fromfile(path, dtype=byteorder + "f4", count=need // 4).astype(np.float32)
    a = a.reshape(nrec, nlat, nlon)
    return a[:nv3d * nlev].reshape(nv3d, nlev, nlat, nlon), a[nv3d * nlev:]


def write_grd4(path, v3d, v2d, byteorder=">"):
    """write_grd4 (speedy/common/common_speedy.f90:259-287): v3d [nv3d, nlev,
    nlat, nlon], v2d [nv2d, nlat, nlon]; values are rounded to REAL(4)."""
    v3d = np.asarray(v3d)
    v2d = np.asarray(v2d)
    nlat, nlon = v3d.shape[-2:]
    out = np.concatenate([v3d.reshape(-1, nlat, nlon), v2d.reshape(-1, nlat, nlon)]).astype(byteorder + "f4")
    with open(path, "wb") as f:
        f.write(out.tobytes())


# --------------------------------------------------------------- device grd
def _read_members(paths, nbytes):
    import torch

    raw = torch.empty(len(paths) * nbytes, dtype=torch.uint8, pin_memory=True)
    view = raw.numpy()
    for m, p in enumerate(paths):
        size = os.path.getsize(p)
        if size < nbytes:
            raise ValueError(f"{p}: {size} bytes, expected at least {nbytes}")
        with open(p, "rb") as f:
            got = f.readinto(memoryview(view[m * nbytes:(m + 1) * nbytes]))
        if got != nbytes:
            raise OSError(f"{p}: short read ({got} of {nbytes} bytes)")
    return raw


def decode_members(raw, ne, nlon, nlat, nlev, nv3d=NV3D, nv2d=NV2D, byteorder=">", dtype=None, stream=None):
    """Device file bytes of ne members -> (gues3d [nv3d, nlev, ne, nij],
    gues2d [nv2d, ne, nij]) in float64 (or float32)."""
    import torch

    dtype = dtype or torch.float64
    nij = nlon * nlat
    nrec = grd_nrec(nlev, nv3d, nv2d)
    dev = raw.device
    g3 = torch.empty((nv3d, nlev, ne, nij), dtype=dtype, device=dev)
    g2 = torch.empty((nv2d, ne, nij), dtype=dtype, device=dev)
    f64 = int(dtype == torch.float64)
    sw = _swap(byteorder)
    # record r = n*nlev + k of member m -> g3[n, k, m, :]: rec stride ne*nij, member stride nij
    check(lib().letkf_grd_decode(nij, nrec, ne, _dptr(raw), sw, 0, nv3d * nlev, f64, _dptr(g3), nij, ne * nij,
                                 _stream(stream)), "letkf_grd_decode")
    check(lib().letkf_grd_decode(nij, nrec, ne, _dptr(raw), sw, nv3d * nlev, nv2d, f64, _dptr(g2), nij, ne * nij,
                                 _stream(stream)), "letkf_grd_decode")
    return g3, g2


def encode_members(g3, g2, byteorder=">", stream=None):
    """(gues3d [nv3d, nlev, ne, nij], gues2d [nv2d, ne, nij]) on the device ->
    device file bytes of the ne members, back to back."""
    import torch

    nv3d, nlev, ne, nij = g3.shape
    nv2d = g2.shape[0]
    nrec = grd_nrec(nlev, nv3d, nv2d)
    raw = torch.empty(ne * nrec * nij * 4, dtype=torch.uint8, device=g3.device)
    sw = _swap(byteorder)
    for t, r0, nr in ((g3, 0, nv3d * nlev), (g2, nv3d * nlev, nv2d)):
        if t.dtype not in (torch.float64, torch.float32):
            raise ValueError("encode_members: float64 or float32 fields expected")
        f64 = int(t.dtype == torch.float64)
        check(lib().letkf_grd_encode(nij, nrec, ne, _dptr(t), f64, nij, ne * nij, r0, nr, sw, _dptr(raw),
                                     _stream(stream)), "letkf_grd_encode")
    return raw


def load_ensemble(paths, nlon, nlat, nlev, nv3d=NV3D, nv2d=NV2D, byteorder=">", device=None, dtype=None,
                  stream=None):
    """read_ens_mpi (speedy/common/common_mpi_speedy.f90:354-382): the members'
    grd files (member m = paths[m]) -> device (gues3d [nv3d, nlev, ne, nij],
    gues2d [nv2d, ne, nij]), one H2D copy of the file bytes."""
    import torch

    device = device or torch.device("cuda")
    nbytes = grd_nbytes(nlon, nlat, nlev, nv3d, nv2d)
    raw = _read_members(list(paths), nbytes)
    s = stream if stream is not None else torch.cuda.current_stream(device)
    with torch.cuda.stream(s):
        draw = raw.to(device, non_blocking=True)
        out = decode_members(draw, len(paths), nlon, nlat, nlev, nv3d, nv2d, byteorder, dtype, s)
    s.synchronize()
    return out


def store_ensemble(paths, g3, g2, byteorder=">", stream=None):
    """write_ens_mpi (speedy/common/common_mpi_speedy.f90:386-414): device
    (anal3d, anal2d) in the analysis layout -> one grd file per member."""
    import torch

    nv3d, nlev, ne, nij = g3.shape
    if len(paths) != ne:
        raise ValueError(f"store_ensemble: {len(paths)} paths for {ne} members")
    s = stream if stream is not None else torch.cuda.current_stream(g3.device)
    with torch.cuda.stream(s):
        raw = encode_members(g3, g2, byteorder, s)
        host = torch.empty(raw.numel(), dtype=torch.uint8, pin_memory=True)
        host.copy_(raw, non_blocking=True)
    s.synchronize()
    per = raw.numel() // ne
    view = host.numpy()
    for m, p in enumerate(paths):
        with open(p, "wb") as f:
            f.write(memoryview(view[m * per:(m + 1) * per]))


def mean_spread(g3, g2, stream=None):
    """Ensemble mean and spread on the device (ensmean_grd and the spread of
    write_ensmspr_mpi): returns (mean3d [nv3d, nlev, nij], mean2d [nv2d, nij],
    sprd3d, sprd2d), float64."""
    import torch

    nv3d, nlev, ne, nij = g3.shape
    nv2d = g2.shape[0]
    m3 = torch.empty((nv3d, nlev, nij), dtype=torch.float64, device=g3.device)
    s3 = torch.empty_like(m3)
    m2 = torch.empty((nv2d, nij), dtype=torch.float64, device=g3.device)
    s2 = torch.empty_like(m2)
    for x, m, s, nrec in ((g3, m3, s3, nv3d * nlev), (g2, m2, s2, nv2d)):
        if x.dtype != torch.float64:
            raise ValueError("mean_spread: float64 fields expected")
        check(lib().letkf_ens_mean_spread(nij, nrec, ne, _dptr(x), nij, ne * nij, _dptr(m), _dptr(s),
                                          _stream(stream)), "letkf_ens_mean_spread")
    return m3, m2, s3, s2


def write_mean_spread(prefix, g3, g2, nlon, nlat, byteorder=">", stream=None):
    """write_ensmspr_mpi (speedy/common/common_mpi_speedy.f90:461-515):
    '<prefix>_me.grd' and '<prefix>_sp.grd'.  Returns the two paths."""
    m3, m2, s3, s2 = mean_spread(g3, g2, stream)
    nv3d, nlev = m3.shape[:2]
    paths = []
    for tag, a3, a2 in (("_me", m3, m2), ("_sp", s3, s2)):
        p = f"{prefix}{tag}.grd"
        write_grd4(p, a3.cpu().numpy().reshape(nv3d, nlev, nlat, nlon), a2.cpu().numpy().reshape(-1, nlat, nlon),
                   byteorder)
        paths.append(p)
    return paths


# ---------------------------------------------------------------- obs records
def _nint(x):
    """Fortran NINT: nearest integer, halves away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)


def read_records(path, nval, byteorder=">"):
    """Fortran sequential unformatted records, the first nval REAL(4) values of
    each (a longer record is read in part, as READ(iunit) wk does; a shorter
    one ends the file, like the IOSTAT loop of get_nobs)."""
    buf = np.fromfile(path, dtype=np.uint8) if os.path.getsize(path) else np.zeros(0, np.uint8)
    i4 = np.dtype(byteorder + "i4")
    f4 = np.dtype(byteorder + "f4")
    n = buf.size
    if n == 0:
        return np.zeros((0, nval), dtype=np.float32)
    first = int(np.frombuffer(buf[:4].tobytes(), dtype=i4)[0])
    rec = first + 8
    if first >= 4 * nval and n % rec == 0:
        m = buf.reshape(-1, rec)
        head = m[:, :4].copy().view(i4).ravel()
        tail = m[:, rec - 4:].copy().view(i4).ravel()
        if (head == first).all() and (tail == first).all():
            return m[:, 4:4 + 4 * nval].copy().view(f4).astype(np.float32)
    out, p = [], 0
    while p + 4 <= n:
        ln = int(np.frombuffer(buf[p:p + 4].tobytes(), dtype=i4)[0])
        if ln < 4 * nval or p + 8 + ln > n:
            break
        out.append(np.frombuffer(buf[p + 4:p + 4 + 4 * nval].tobytes(), dtype=f4))
        p += 8 + ln
    return np.array(out, dtype=np.float32).reshape(-1, nval)


def write_records(path, values, byteorder=">"):
    v = np.ascontiguousarray(values, dtype=byteorder + "f4")
    n, nval = v.shape
    marker = np.full((n, 1), 4 * nval, dtype=byteorder + "i4").view(np.uint8)
    body = v.view(np.uint8).reshape(n, 4 * nval)
    with open(path, "wb") as f:
        f.write(np.concatenate([marker, body, marker], axis=1).tobytes())


def get_nobs(path, nrec=6, byteorder=">"):
    """get_nobs (speedy/common/common_obs_speedy.f90:413-456): number of
    records and the count per element (u, v, t, q, rh, ps).  A missing file
    counts 0."""
    if not os.path.exists(path):
        return 0, {}
    w = read_records(path, nrec, byteorder)
    e = _nint(w[:, 0]) if len(w) else np.zeros(0, np.int64)
    names = {"u": ID_U, "v": ID_V, "t": ID_T, "q": ID_Q, "rh": ID_RH, "ps": ID_PS}
    return len(w), {k: int((e == c).sum()) for k, c in names.items()}


def _to_si(wk):
    """The REAL(4) unit conversions of read_obs / read_obs2: levels hPa -> Pa,
    ps values hPa -> Pa, RH values percent -> fraction."""
    wk = wk.copy()
    e = _nint(wk[:, 0])
    lev3 = np.isin(e, (ID_U, ID_V, ID_T, ID_Q, ID_RH))
    wk[lev3, 3] = wk[lev3, 3] * np.float32(100.0)
    ps = e == ID_PS
    wk[ps, 4] = wk[ps, 4] * np.float32(100.0)
    wk[ps, 5] = wk[ps, 5] * np.float32(100.0)
    rh = e == ID_RH
    wk[rh, 4] = wk[rh, 4] * np.float32(0.01)
    wk[rh, 5] = wk[rh, 5] * np.float32(0.01)
    return wk


def read_obs(path, byteorder=">"):
    """read_obs (speedy/common/common_obs_speedy.f90:458-501): dict of float64
    elem, lon, lat, lev, dat, err in SI units."""
    wk = _to_si(read_records(path, 6, byteorder))
    keys = ("elem", "lon", "lat", "lev", "dat", "err")
    return {k: wk[:, i].astype(np.float64) for i, k in enumerate(keys)}


def read_obs2(path, byteorder=">"):
    """read_obs2 (speedy/common/common_obs_speedy.f90:503-551): read_obs plus
    hx (float64) and qc (NINT, int32)."""
    wk = _to_si(read_records(path, 8, byteorder))
    keys = ("elem", "lon", "lat", "lev", "dat", "err", "hx")
    out = {k: wk[:, i].astype(np.float64) for i, k in enumerate(keys)}
    out["qc"] = _nint(wk[:, 7]).astype(np.int32)
    return out


def write_obs2(path, elem, lon, lat, lev, dat, err, hx, qc, byteorder=">"):
    """write_obs2 (speedy/common/common_obs_speedy.f90:553-600): values are
    rounded to REAL(4), then converted back to hPa / percent in REAL(4)."""
    wk = np.stack([np.asarray(a, dtype=np.float64).astype(np.float32)
                   for a in (elem, lon, lat, lev, dat, err, hx, np.asarray(qc, dtype=np.float64))], axis=1)
    e = _nint(wk[:, 0])
    lev3 = np.isin(e, (ID_U, ID_V, ID_T, ID_Q, ID_RH))
    wk[lev3, 3] = wk[lev3, 3] * np.float32(0.01)
    ps = e == ID_PS
    wk[ps, 4] = wk[ps, 4] * np.float32(0.01)
    wk[ps, 5] = wk[ps, 5] * np.float32(0.01)
    rh = e == ID_RH
    wk[rh, 4] = wk[rh, 4] * np.float32(100.0)
    wk[rh, 5] = wk[rh, 5] * np.float32(100.0)
    write_records(path, wk, byteorder)


def write_obs(path, elem, lon, lat, lev, dat, err, byteorder=">"):
    """The 6-value records read_obs reads (hPa levels, hPa ps, percent RH), as
    the reference's obsmake writes them."""
    wk = np.stack([np.asarray(a, dtype=np.float64).astype(np.float32) for a in (elem, lon, lat, lev, dat, err)],
                  axis=1)
    e = _nint(wk[:, 0])
    lev3 = np.isin(e, (ID_U, ID_V, ID_T, ID_Q, ID_RH))
    wk[lev3, 3] = wk[lev3, 3] * np.float32(0.01)
    ps = e == ID_PS
    wk[ps, 4] = wk[ps, 4] * np.float32(0.01)
    wk[ps, 5] = wk[ps, 5] * np.float32(0.01)
    rh = e == ID_RH
    wk[rh, 4] = wk[rh, 4] * np.float32(100.0)
    wk[rh, 5] = wk[rh, 5] * np.float32(100.0)
    write_records(path, wk, byteorder)


def load_obs2_members(paths, byteorder=">"):
    """set_letkf_obs's reading of one slot (speedy/letkf/letkf_obs.f90:118-133):
    every member's obs2 file (member m = paths[m], identical records) ->
    records of the first plus hx [nobs, ne] and qc_member [nobs, ne]."""
    first = None
    hx, qc = [], []
    for p in paths:
        r = read_obs2(p, byteorder)
        if first is None:
            first = r
        elif r["elem"].size != first["elem"].size:
            raise ValueError(f"{p}: {r['elem'].size} records, expected {first['elem'].size}")
        hx.append(r["hx"])
        qc.append(r["qc"])
    out = {k: v for k, v in first.items() if k not in ("hx", "qc")}
    out["hx"] = np.stack(hx, axis=1)
    out["qc_member"] = np.stack(qc, axis=1).astype(np.int32)
    return out
