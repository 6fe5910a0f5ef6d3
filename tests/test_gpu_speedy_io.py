"""SPEEDY grd records on the device: letkf_grd_decode / letkf_grd_encode
(bit-exact against numpy's byte-order and REAL(4) conversions) and
letkf_ens_mean_spread (bit-exact against the member-order sums of ensmean_grd
and write_ensmspr_mpi), then files -> device ensemble -> H(x)."""
import numpy as np
import pytest

from letkf_gb300 import speedy_io as IO
from letkf_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _members(rng, ne, nlon, nlat, nlev):
    return rng.standard_normal((ne, IO.grd_nrec(nlev), nlat, nlon)).astype(np.float32) * 100.0


@pytest.mark.parametrize("bo,nlon,nlat", [(">", 96, 48), ("<", 96, 48), (">", 15, 7)])
def test_decode_into_analysis_layout(cuda, bo, nlon, nlat):
    """96 x 48 takes the 16-byte path, 15 x 7 (odd rows) the 4-byte one."""
    import torch

    rng = np.random.default_rng(1)
    ne, nlev = 5, 7
    x = _members(rng, ne, nlon, nlat, nlev)
    raw = torch.as_tensor(np.frombuffer(x.astype(bo + "f4").tobytes(), dtype=np.uint8).copy(), device=cuda)
    g3, g2 = IO.decode_members(raw, ne, nlon, nlat, nlev, byteorder=bo)
    nij = nlon * nlat
    want3 = x[:, :4 * nlev].reshape(ne, 4, nlev, nij).transpose(1, 2, 0, 3).astype(np.float64)
    want2 = x[:, 4 * nlev:].reshape(ne, 2, nij).transpose(1, 0, 2).astype(np.float64)
    assert np.array_equal(g3.cpu().numpy(), want3)
    assert np.array_equal(g2.cpu().numpy(), want2)
    f3, f2 = IO.decode_members(raw, ne, nlon, nlat, nlev, byteorder=bo, dtype=torch.float32)
    assert np.array_equal(f3.cpu().numpy(), want3.astype(np.float32))
    assert np.array_equal(f2.cpu().numpy(), want2.astype(np.float32))


@pytest.mark.parametrize("bo,nlon,nlat", [(">", 16, 8), ("<", 16, 8), (">", 15, 7)])
def test_encode_rounds_to_real4(cuda, bo, nlon, nlat):
    import torch

    rng = np.random.default_rng(2)
    ne, nlev = 3, 7
    nij = nlon * nlat
    g3 = rng.standard_normal((4, nlev, ne, nij)) * 1e3
    g2 = rng.standard_normal((2, ne, nij)) * 1e5
    raw = IO.encode_members(torch.as_tensor(g3, device=cuda), torch.as_tensor(g2, device=cuda), byteorder=bo)
    file_vals = np.concatenate([g3.transpose(2, 0, 1, 3).reshape(ne, 4 * nlev, nij),
                                g2.transpose(1, 0, 2)], axis=1)       # [ne, nrec, nij]
    want = np.frombuffer(file_vals.astype(bo + "f4").tobytes(), dtype=np.uint8)
    assert np.array_equal(raw.cpu().numpy(), want)


def test_files_round_trip_and_mean_spread(cuda, tmp_path):
    import torch

    rng = np.random.default_rng(3)
    ne, nlon, nlat, nlev = 6, 96, 48, 7
    x = _members(rng, ne, nlon, nlat, nlev)
    paths = []
    for m in range(ne):
        p = tmp_path / f"gs01{m + 1:03d}.grd"
        p.write_bytes(x[m].astype(">f4").tobytes())
        paths.append(str(p))
    g3, g2 = IO.load_ensemble(paths, nlon, nlat, nlev, device=cuda)
    out = [str(tmp_path / f"anal{m + 1:03d}.grd") for m in range(ne)]
    IO.store_ensemble(out, g3, g2)
    for a, b in zip(paths, out):
        assert open(a, "rb").read() == open(b, "rb").read()
    m3, m2, s3, s2 = IO.mean_spread(g3, g2)
    xd = x.astype(np.float64).reshape(ne, IO.grd_nrec(nlev), nlat * nlon)
    s = xd[0].copy()
    for m in range(1, ne):
        s = s + xd[m]
    mean = s / ne
    v = (xd[0] - mean) ** 2
    for m in range(1, ne):
        v = v + (xd[m] - mean) ** 2
    sprd = np.sqrt(v / (ne - 1))
    assert np.array_equal(m3.cpu().numpy().reshape(-1, nlat * nlon), mean[:4 * nlev])
    assert np.array_equal(m2.cpu().numpy(), mean[4 * nlev:])
    assert np.array_equal(s3.cpu().numpy().reshape(-1, nlat * nlon), sprd[:4 * nlev])
    assert np.array_equal(s2.cpu().numpy(), sprd[4 * nlev:])
    me, sp = IO.write_mean_spread(str(tmp_path / "gues"), g3, g2, nlon, nlat)
    a3, a2 = IO.read_grd4(me, nlon, nlat, nlev)
    assert np.array_equal(a3.reshape(-1, nlat * nlon), mean[:4 * nlev].astype(np.float32))
    b3, b2 = IO.read_grd4(sp, nlon, nlat, nlev)
    assert np.array_equal(b2.reshape(-1, nlat * nlon), sprd[4 * nlev:].astype(np.float32))


def test_files_to_obs_operator(cuda, tmp_path):
    """Member grd files and an obs file -> device ensemble -> H(x) on the
    device, against the oracle on the same REAL(4) values."""
    import torch

    from letkf_gb300.core import speedy_obsope
    from oracle import oracle as O

    rng = np.random.default_rng(4)
    ne, nlon, nlat, nlev = 8, 96, 48, 7
    lon, lat = S.speedy_grid(nlon, nlat)
    v3d, v2d = S.speedy_members(rng, ne, nlon, nlat, nlev)
    paths = []
    for m in range(ne):
        p = tmp_path / f"gs01{m + 1:03d}.grd"
        IO.write_grd4(str(p), v3d[m], v2d[m])
        paths.append(str(p))
    el, lo, la, lv, od = S.speedy_obs_records(rng, 800, lon, lat, nlon, with_edges=False)
    op = tmp_path / "obs01.dat"
    IO.write_obs(str(op), el, lo, la, lv, od, np.ones(el.size))
    obs = IO.read_obs(str(op))
    g3, g2 = IO.load_ensemble(paths, nlon, nlat, nlev, device=cuda)
    v3 = g3.reshape(4, nlev, ne, nlat, nlon).permute(2, 0, 1, 3, 4)
    v2 = g2.reshape(2, ne, nlat, nlon).permute(1, 0, 2, 3)
    elem = torch.as_tensor(np.rint(obs["elem"]).astype(np.int32), device=cuda)
    t = {k: torch.as_tensor(obs[k], device=cuda) for k in ("lon", "lat", "lev", "dat")}
    hx, qc = speedy_obsope(torch.as_tensor(lat, device=cuda), torch.as_tensor(S.SPEEDY_SIG, device=cuda), v3, v2,
                           elem, t["lon"], t["lat"], t["lev"], t["dat"])
    f3 = v3d.astype(np.float32).astype(np.float64)
    f2 = v2d.astype(np.float32).astype(np.float64)
    rhx, rqc, _ = O.speedy_obsope(lat, S.SPEEDY_SIG, f3, f2, np.rint(obs["elem"]).astype(np.int32), obs["lon"],
                                  obs["lat"], obs["lev"], obs["dat"])
    np.testing.assert_array_equal(qc.cpu().numpy(), rqc)
    np.testing.assert_allclose(hx.cpu().numpy(), rhx, rtol=1e-12, atol=0.0)
    assert rqc.sum() > 300
