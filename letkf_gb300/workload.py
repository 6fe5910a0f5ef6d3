"""The regional benchmark workload: 256 x 256 x 40 grid at 3 km, 6 variables,
k = 64 members, 1e6 clustered observations (0-2000 local obs per point).

Positions, field parameters and noise come from a numpy generator seeded once;
field values are evaluated either with numpy (host) or on the device (torch,
FP64 evaluation, FP32 storage), so both arms of the benchmark see the same
workload.  Background members and obs-space perturbations are smooth random
fields (synthetic.SmoothFields); hdxf = H(x_m) - mean, dep = y - mean
(speedy/letkf/letkf_obs.f90:157-174).
"""
from __future__ import annotations

import math

import numpy as np

from . import synthetic as S


class RegionalWorkload:
    def __init__(self, seed=0, nlon=256, nlat=256, nlev=40, ne=64, nobs=1_000_000, nvar=6, dx=3000.0,
                 sigma_obs=S.REGIONAL_SIGMA_OBS, sigma_obsv=S.REGIONAL_SIGMA_OBSV, corr_len=60.0e3):
        rng = np.random.default_rng(seed)
        self.nlon, self.nlat, self.nlev, self.ne, self.nobs, self.nvar, self.dx = nlon, nlat, nlev, ne, nobs, nvar, dx
        self.sigma_obs, self.sigma_obsv, self.corr_len = sigma_obs, sigma_obsv, corr_len
        self.ri, self.rj, self.lev, self.cls = S.regional_obs(rng, nobs, nlon, nlat)
        self.var = rng.integers(0, nvar, nobs).astype(np.int32)
        self.err = np.where(self.cls == 1, 100.0, 1.0)
        self.ps = 1.0e5 * (1 + 0.01 * rng.standard_normal(nobs))
        self.noise = rng.standard_normal(nobs)
        self.fields = S.SmoothFields(rng, ne + 1, nvar, 6, wavenum_scale=1.0, dims=3)
        self.plev = S.regional_levels(nlev)
        self.npts = nlon * nlat * nlev
        self.params = S.scale_params(dict(dx=dx, dy=dx, sigma_obs=sigma_obs, sigma_obsv=sigma_obsv))

    # ---- grid points: index p = lev * nlon * nlat + (j - 1) * nlon + (i - 1)
    def points(self, subset=None):
        p = np.arange(self.npts) if subset is None else np.asarray(subset)
        nij = self.nlon * self.nlat
        lev = p // nij
        ij = p - lev * nij
        j = ij // self.nlon + 1
        i = ij - (j - 1) * self.nlon + 1
        return i.astype(np.float64), j.astype(np.float64), self.plev[lev]

    def _obs_xyz(self):
        lnp = np.where(self.cls == 1, math.log(S.REGIONAL_P_BOT), np.log(self.lev))
        return np.stack([self.ri * self.dx / self.corr_len, self.rj * self.dx / self.corr_len, lnp / 0.8], -1)

    def _finish_obs(self, hx):
        """hx (ne+1, nobs) float64 -> hdxf (nobs, ne) float32, dep, dat (float64)."""
        ne = self.ne
        truth = hx[ne]
        hx32 = hx[:ne].astype(np.float32).astype(np.float64)
        hxm = hx32.sum(0) / ne
        hdxf = (hx32 - hxm).T.astype(np.float32)
        y = truth + self.err * self.noise
        dep = y - hxm
        dat = np.where(self.cls == 1, self.ps, y)
        return np.ascontiguousarray(hdxf), dep, dat

    def obs_numpy(self, chunk=200_000):
        xyz = self._obs_xyz()
        hx = np.empty((self.ne + 1, self.nobs))
        for c in range(0, self.nobs, chunk):
            s = slice(c, c + chunk)
            hx[:, s] = self.fields.eval(xyz[s], self.var[s])
        return self._finish_obs(hx)

    def obs_torch(self, device, chunk=200_000):
        import torch

        xyz = torch.as_tensor(self._obs_xyz(), device=device)
        var = torch.as_tensor(self.var, device=device, dtype=torch.int64)
        k = torch.as_tensor(self.fields.k, device=device)
        a = torch.as_tensor(self.fields.a, device=device)
        ph = torch.as_tensor(self.fields.phi, device=device)
        hx = torch.empty((self.ne + 1, self.nobs), dtype=torch.float64, device=device)
        for c in range(0, self.nobs, chunk):
            s = slice(c, c + chunk)
            arg = torch.einsum("nqd,nd->nq", k[var[s]], xyz[s])
            hx[:, s] = (a[:, var[s], :] * torch.cos(arg[None] + ph[:, var[s], :])).sum(-1)
        return self._finish_obs(hx.cpu().numpy())

    def _grid_xyz(self, subset=None):
        i, j, p = self.points(subset)
        return np.stack([i * self.dx / self.corr_len, j * self.dx / self.corr_len, np.log(p) / 0.8], -1)

    def background_numpy(self, subset=None):
        """xb [nv][n][ne] float32 for the points (all or subset)."""
        xyz = self._grid_xyz(subset)
        out = np.empty((self.nvar, xyz.shape[0], self.ne), dtype=np.float32)
        for v in range(self.nvar):
            out[v] = self.fields.eval(xyz, v)[: self.ne].T
        return out

    def background_torch(self, device, out=None, chunk=1 << 20):
        """xb [nv][npts][ne] float32 on the device (FP64 evaluation)."""
        import torch

        npts = self.npts
        if out is None:
            out = torch.empty((self.nvar, npts, self.ne), dtype=torch.float32, device=device)
        k = torch.as_tensor(self.fields.k, device=device)
        a = torch.as_tensor(self.fields.a[: self.ne], device=device)
        ph = torch.as_tensor(self.fields.phi[: self.ne], device=device)
        for c in range(0, npts, chunk):
            idx = np.arange(c, min(npts, c + chunk))
            xyz = torch.as_tensor(self._grid_xyz(idx), device=device)
            for v in range(self.nvar):
                arg = xyz @ k[v].T                                  # (n, nmode)
                val = (a[:, v, None, :] * torch.cos(arg[None] + ph[:, v, None, :])).sum(-1)  # (ne, n)
                out[v, c:c + idx.size] = val.T.to(torch.float32)
        return out

    def local_count_hint(self):
        return "0-2000 local obs per point (clustered density, sigma_h = %.0f m)" % self.sigma_obs


class GlobalWorkload:
    """The large-ensemble configuration: a 360 x 181 x 32 global lat/lon grid
    (1 degree, poles included, pressure levels uniform in ln p from 1000 to
    10 hPa), 6 variables, k = 512 members, 3e6 observations (u, v, t, q at
    positions uniform on the sphere and pressures uniform in ln p) searched
    with the SPEEDY lat/lon rule (speedy/letkf/letkf_tools.f90:272-603).
    Members and truth are smooth random fields on the sphere x ln p evaluated
    on the device; the obs are bucket-sorted (speedy/letkf/letkf_obs.f90:
    243-313).  Point p = lev * nlon * nlat + j * nlon + i."""

    def __init__(self, seed=0, nlon=360, nlat=181, nlev=32, ne=512, nobs=3_000_000, nvar=6, sigma_obs=60.0e3,
                 sigma_obsv=0.4):
        from .drivers import speedy_sort_obs

        rng = np.random.default_rng(seed)
        self.nlon, self.nlat, self.nlev, self.ne, self.nvar = nlon, nlat, nlev, ne, nvar
        self.lon = 360.0 / nlon * np.arange(nlon)
        self.lat = np.linspace(-90.0, 90.0, nlat)
        self.plev = np.exp(np.linspace(math.log(1.0e5), math.log(1.0e3), nlev))
        olon = rng.uniform(0.0, 360.0, nobs)
        olat = np.degrees(np.arcsin(rng.uniform(-1.0, 1.0, nobs)))
        olev = np.exp(rng.uniform(math.log(1.0e3), math.log(1.0e5), nobs))
        ovar = rng.integers(0, 4, nobs)
        elm = np.array([S.ID_U, S.ID_V, S.ID_T, S.ID_Q], dtype=np.float64)[ovar]
        err = np.array([1.0, 1.0, 1.0, 1.0e-3])[ovar]
        noise = rng.standard_normal(nobs)
        perm, self.nobsgrd = speedy_sort_obs(self.lon, self.lat, olon, olat)
        self.olon, self.olat, self.olev, self.elm, self.err = olon[perm], olat[perm], olev[perm], elm[perm], err[perm]
        self.ovar, self.noise = ovar[perm], noise[perm]
        self.nobs = perm.size
        amp = np.array([5.0, 5.0, 2.0, 1.0e-3, 3.0, 3.0])[:nvar] if nvar <= 6 else None
        self.fields = S.SmoothFields(rng, ne + 1, nvar, 6, wavenum_scale=6371.3e3 / 2.0e6, dims=4, amp=amp)
        self.sigma_obs, self.sigma_obsv = sigma_obs, sigma_obsv
        dist_zero = sigma_obs * math.sqrt(10.0 / 3.0) * 2.0
        dist_zerov = sigma_obsv * math.sqrt(10.0 / 3.0) * 2.0
        dlat_zero = dist_zero / 3.1415926535 / 6371.3e3 * 180.0   # speedy/letkf/letkf_obs.f90:82-88
        self.params = (dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv)
        self.npts = nlon * nlat * nlev

    @staticmethod
    def _xyz(lon, lat, lnp):
        lo, la = np.radians(lon), np.radians(lat)
        return np.stack([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la), (lnp - math.log(1.0e5)) / 2.0],
                        -1)

    def obs_torch(self, device, chunk=20_000):
        """hdxf float32 [nobs, ne], dep float64 [nobs], dat float64 (sorted order), on the device."""
        import torch

        ne = self.ne
        xyz = torch.as_tensor(self._xyz(self.olon, self.olat, np.log(self.olev)), device=device)
        var = torch.as_tensor(self.ovar, device=device)
        k = torch.as_tensor(self.fields.k, device=device)
        a = torch.as_tensor(self.fields.a, device=device)
        ph = torch.as_tensor(self.fields.phi, device=device)
        hdxf = torch.empty((self.nobs, ne), dtype=torch.float32, device=device)
        dep = torch.empty(self.nobs, dtype=torch.float64, device=device)
        dat = torch.empty(self.nobs, dtype=torch.float64, device=device)
        err = torch.as_tensor(self.err, device=device)
        noise = torch.as_tensor(self.noise, device=device)
        for c in range(0, self.nobs, chunk):
            s = slice(c, min(self.nobs, c + chunk))
            arg = torch.einsum("nqd,nd->nq", k[var[s]], xyz[s])
            hx = (a[:, var[s], :] * torch.cos(arg[None] + ph[:, var[s], :])).sum(-1)  # (ne+1, n)
            hx32 = hx[:ne].to(torch.float32).to(torch.float64)
            m = hx32.sum(0) / ne
            hdxf[s] = (hx32 - m).T.to(torch.float32)
            y = hx[ne] + err[s] * noise[s]
            dep[s] = y - m
            dat[s] = y
        return hdxf, dep, dat

    def search_params(self, sigma_obs):
        """(dist_zero, dist_zerov, dlat_zero, sigma_obs, sigma_obsv) for another
        horizontal localisation scale on the same observations."""
        dist_zero = sigma_obs * math.sqrt(10.0 / 3.0) * 2.0
        dist_zerov = self.sigma_obsv * math.sqrt(10.0 / 3.0) * 2.0
        dlat_zero = dist_zero / 3.1415926535 / 6371.3e3 * 180.0   # speedy/letkf/letkf_obs.f90:82-88
        return (dist_zero, dist_zerov, dlat_zero, sigma_obs, self.sigma_obsv)

    def points(self, idx, params=None):
        """lon, lat, dlon_zero, ilev (1-based), log p of the points idx."""
        params = self.params if params is None else params
        idx = np.asarray(idx)
        nij = self.nlon * self.nlat
        lev, ij = idx // nij, idx % nij
        j, i = ij // self.nlon, ij % self.nlon
        lat = self.lat[j]
        dlon = params[2] / np.maximum(np.cos(3.1415926535 * lat / 180.0), 1e-12)
        return self.lon[i], lat, dlon, (lev + 1).astype(np.int32), np.log(self.plev[lev])

    def background_torch(self, device, idx):
        """xb float32 [nv, len(idx), ne] at the points idx."""
        import torch

        lon, lat, _, ilev, lnp = self.points(idx)
        xyz = torch.as_tensor(self._xyz(lon, lat, lnp), device=device)
        k = torch.as_tensor(self.fields.k, device=device)
        a = torch.as_tensor(self.fields.a[: self.ne], device=device)
        ph = torch.as_tensor(self.fields.phi[: self.ne], device=device)
        out = torch.empty((self.nvar, len(idx), self.ne), dtype=torch.float32, device=device)
        for v in range(self.nvar):
            arg = xyz @ k[v].T
            out[v] = (a[:, v, None, :] * torch.cos(arg[None] + ph[:, v, None, :])).sum(-1).T.to(torch.float32)
        return out
