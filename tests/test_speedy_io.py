"""SPEEDY file formats on the host: observation records (Fortran sequential
unformatted, speedy/common/common_obs_speedy.f90:413-602) and grd files
(direct access, speedy/common/common_speedy.f90:163-287).  Expected bytes are
built independently with ``struct`` from the Fortran record layout."""
import struct

import numpy as np
import pytest

from letkf_gb300 import speedy_io as IO

U, V, T, Q, RH, PS, RAIN = IO.ID_U, IO.ID_V, IO.ID_T, IO.ID_Q, IO.ID_RH, IO.ID_PS, IO.ID_RAIN


def _f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


def _records_bytes(rows, bo=">"):
    out = b""
    for r in rows:
        body = struct.pack(bo + "%df" % len(r), *r)
        out += struct.pack(bo + "i", len(body)) + body + struct.pack(bo + "i", len(body))
    return out


ROWS = [
    (U, 10.5, 35.25, 850.0, 3.5, 1.2),
    (T, 200.0, -45.0, 500.0, 250.25, 1.0),
    (PS, 359.0, 0.0, 0.0, 1003.5, 1.0),
    (RH, 120.0, 12.0, 700.0, 85.0, 10.0),
    (Q, 0.5, 80.0, 300.0, 1.0e-3, 1.0e-4),
    (RAIN, 33.0, 3.0, 1000.0, 2.0, 0.5),
]


@pytest.mark.parametrize("bo", [">", "<"])
def test_read_obs_units_and_byteorder(tmp_path, bo):
    p = tmp_path / "obs.dat"
    p.write_bytes(_records_bytes(ROWS, bo))
    o = IO.read_obs(str(p), byteorder=bo)
    assert o["elem"].tolist() == [float(r[0]) for r in ROWS]
    # REAL(4) conversions: hPa -> Pa levels (u/v/t/q/rh), ps value and error, RH percent -> fraction
    assert o["lev"][0] == _f32(_f32(850.0) * _f32(100.0))
    assert o["lev"][1] == _f32(_f32(500.0) * _f32(100.0))
    assert o["lev"][2] == 0.0
    assert o["dat"][2] == np.float32(np.float32(1003.5) * np.float32(100.0))
    assert o["err"][2] == np.float32(np.float32(1.0) * np.float32(100.0))
    assert o["dat"][3] == np.float32(np.float32(85.0) * np.float32(0.01))
    assert o["err"][3] == np.float32(np.float32(10.0) * np.float32(0.01))
    assert o["lev"][3] == np.float32(np.float32(700.0) * np.float32(100.0))
    assert o["lev"][5] == 1000.0                      # rain: no conversion
    assert o["dat"][4] == float(np.float32(1.0e-3))
    assert o["lon"].dtype == np.float64


def test_get_nobs_counts_and_missing_file(tmp_path):
    p = tmp_path / "obs.dat"
    p.write_bytes(_records_bytes(ROWS))
    n, per = IO.get_nobs(str(p), 6)
    assert n == 6
    assert per == {"u": 1, "v": 0, "t": 1, "q": 1, "rh": 1, "ps": 1}
    assert IO.get_nobs(str(tmp_path / "none.dat"))[0] == 0


def test_longer_records_read_in_part_and_truncated_tail_ends(tmp_path):
    rows8 = [r + (7.0, 1.0) for r in ROWS]
    data = _records_bytes(rows8) + struct.pack(">i", 32) + b"\0" * 10   # a cut-off last record
    p = tmp_path / "obs2.dat"
    p.write_bytes(data)
    w = IO.read_records(str(p), 6)
    assert w.shape == (6, 6)
    np.testing.assert_array_equal(w[:, 0], [r[0] for r in ROWS])
    # records of mixed lengths walk the markers
    mixed = _records_bytes(ROWS[:2]) + _records_bytes(rows8[2:4]) + _records_bytes([(U, 1.0)])
    p.write_bytes(mixed)
    w = IO.read_records(str(p), 6)
    assert w.shape == (4, 6)                          # the 2-value record is too short: READ fails, loop ends


def test_write_obs2_bytes_and_round_trip(tmp_path):
    elem = np.array([U, PS, RH], float)
    lon = np.array([10.1, 20.2, 30.3])
    lat = np.array([-5.5, 6.6, 7.7])
    lev = np.array([85000.0, 0.0, 50000.0])
    dat = np.array([1.5, 100350.0, 0.85])
    err = np.array([1.0, 100.0, 0.1])
    hx = np.array([1.25, 100300.0, 0.8])
    qc = np.array([1, 0, 1])
    p = tmp_path / "obs2.dat"
    IO.write_obs2(str(p), elem, lon, lat, lev, dat, err, hx, qc)
    want = []
    for i in range(3):
        wk = [_f32(x) for x in (elem[i], lon[i], lat[i], lev[i], dat[i], err[i], hx[i], float(qc[i]))]
        e = int(round(wk[0]))
        if e in (U, V, T, Q, RH):
            wk[3] = _f32(wk[3] * _f32(0.01))
        if e == PS:
            wk[4] = _f32(wk[4] * _f32(0.01))
            wk[5] = _f32(wk[5] * _f32(0.01))
        if e == RH:
            wk[4] = _f32(wk[4] * _f32(100.0))
            wk[5] = _f32(wk[5] * _f32(100.0))
        want.append(tuple(wk))
    assert p.read_bytes() == _records_bytes(want)
    r = IO.read_obs2(str(p))
    assert r["qc"].tolist() == [1, 0, 1]
    np.testing.assert_allclose(r["lev"], lev, rtol=1e-6)
    np.testing.assert_allclose(r["dat"], dat, rtol=1e-6)
    np.testing.assert_allclose(r["hx"], hx, rtol=1e-6)


def test_grd4_bytes_and_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    nlon, nlat, nlev = 8, 4, 3
    v3d = rng.standard_normal((4, nlev, nlat, nlon)).astype(np.float32)
    v2d = rng.standard_normal((2, nlat, nlon)).astype(np.float32)
    p = tmp_path / "x.grd"
    IO.write_grd4(str(p), v3d, v2d)
    data = p.read_bytes()
    assert len(data) == IO.grd_nbytes(nlon, nlat, nlev)
    # record 1 is u at level 1, lon fastest; record nv3d*nlev + 1 is ps
    assert data[:4] == struct.pack(">f", v3d[0, 0, 0, 0])
    assert data[4:8] == struct.pack(">f", v3d[0, 0, 0, 1])
    off = 4 * nlon * nlat * (4 * nlev)
    assert data[off:off + 4] == struct.pack(">f", v2d[0, 0, 0])
    a3, a2 = IO.read_grd4(str(p), nlon, nlat, nlev)
    np.testing.assert_array_equal(a3, v3d)
    np.testing.assert_array_equal(a2, v2d)
    with pytest.raises(ValueError):
        IO.read_grd4(str(p), nlon, nlat, nlev + 1)
