"""Seeded synthetic workloads with the shapes of the reference's configurations.

The reference ships no data sets; every case here is generated from a seed.
Background members are smooth random fields (a few random Fourier modes per
member and variable) so that obs-space perturbations correlate with the grid
perturbations as they would through an observation operator.  Observation
perturbations are the members' fields evaluated at the observation locations
minus their ensemble mean, departures are truth + noise minus the mean
(speedy/letkf/letkf_obs.f90:157-174).

  l96_case       Lorenz-96, N=40, F=8, RK4 (lorenz96/model/lorenz96.f90:93-128,
                 292-309), k=20 members = truth + N(0,1), 40 identity obs
  speedy_case    SPEEDY T30 grid 96x48x7, k=40, radiosonde-like profiles
  regional_case  Cartesian 3 km grid, nlon x nlat x nlev, k members, clustered obs
"""
from __future__ import annotations

import math

import numpy as np

# SPEEDY observation element ids (speedy/common/common_obs_speedy.f90:18-24)
ID_U, ID_V, ID_T, ID_Q, ID_RH, ID_PS, ID_RAIN = 2819, 2820, 3073, 3330, 3331, 14593, 9999


# --------------------------------------------------------------------------- L96
def l96_tendency(x, force, dt):
    """lorenz96/model/lorenz96.f90:292-309 (the tendency is multiplied by dt)."""
    return dt * ((np.roll(x, -1, -1) - np.roll(x, 2, -1)) * np.roll(x, 1, -1) - x + force)


def l96_rk4(x, kt, force=8.0, dt=0.005):
    """lorenz96/model/lorenz96.f90:93-128."""
    x = np.array(x, dtype=np.float64)
    for _ in range(kt):
        q1 = l96_tendency(x, force, dt)
        q2 = l96_tendency(x + 0.5 * q1, force, dt)
        q3 = l96_tendency(x + 0.5 * q2, force, dt)
        q4 = l96_tendency(x + q3, force, dt)
        x = x + (q1 + 2.0 * q2 + 2.0 * q3 + q4) / 6.0
    return x


def l96_case(seed=0, nx=40, ne=20, spinup_steps=2000, obserr=1.0):
    """One analysis time of the Lorenz-96 OSSE: truth, background members,
    identity observations (one per variable), departures and perturbations."""
    rng = np.random.default_rng(seed)
    truth = l96_rk4(8.0 + 0.01 * rng.standard_normal(nx), spinup_steps)
    xf = truth[None, :] + rng.standard_normal((ne, nx))
    h = np.eye(nx)  # ny = nx identity operator
    y = truth + obserr * rng.standard_normal(nx)
    hxf = xf @ h.T                      # (ne, ny)
    hxfm = hxf.sum(0) / ne
    hdxf = (hxf - hxfm).T               # (ny, ne)
    d = y - hxfm
    return dict(truth=truth, xf=xf, h=h, y=y, hdxf=hdxf, dep=d, obserr=obserr, xlocal=3.0, infl=1.05, ne=ne, nx=nx)


# ----------------------------------------------------------------- smooth fields
class SmoothFields:
    """Random Fourier-mode fields f_{m,v}(xyz) = sum_q a cos(k_q . xyz + phi)."""

    def __init__(self, rng, nmem, nvar, nmode, wavenum_scale, dims=3, amp=None):
        self.k = rng.standard_normal((nvar, nmode, dims)) * wavenum_scale
        self.a = rng.standard_normal((nmem, nvar, nmode)) / math.sqrt(nmode)
        if amp is not None:
            self.a *= np.asarray(amp, dtype=np.float64)[None, :, None]
        self.phi = rng.uniform(0, 2 * math.pi, (nmem, nvar, nmode))

    def eval(self, xyz, var, members=None):
        """xyz (n, dims); var scalar or (n,) int; returns (nmem, n)."""
        xyz = np.asarray(xyz, dtype=np.float64)
        var = np.broadcast_to(np.asarray(var), (xyz.shape[0],))
        mem = slice(None) if members is None else members
        k = self.k[var]                                      # (n, nmode, dims)
        arg = np.einsum("nqd,nd->nq", k, xyz)                # (n, nmode)
        a = self.a[mem][:, var, :]                           # (nm, n, nmode)
        ph = self.phi[mem][:, var, :]
        return np.sum(a * np.cos(arg[None] + ph), axis=-1)


# ----------------------------------------------------------------------- SPEEDY
def speedy_grid(nlon=96, nlat=48):
    """Longitudes 360/nlon*(i-1) (speedy/common/common_speedy.f90:65) and
    Gaussian latitudes from the Gauss-Legendre nodes, rounded to 3 decimals."""
    lon = 360.0 / nlon * np.arange(nlon)
    x, _ = np.polynomial.legendre.leggauss(nlat)
    lat = np.round(np.degrees(np.arcsin(x)), 3)
    return lon, np.sort(lat)


SPEEDY_SIG = np.array([0.95, 0.835, 0.685, 0.51, 0.34, 0.2, 0.08])


def speedy_case(seed=0, ne=40, nstations=600, nlon=96, nlat=48, nlev=7, sigma_obs=500.0e3, sigma_obsv=0.1):
    """SPEEDY-grid analysis: 3-D variables u, v, t, q on 96x48x7 plus ps.
    Radiosonde-like profiles at stations with uneven density; each profile
    reports u, v, t, q at the 7 sigma levels and ps (about 29 obs/station)."""
    rng = np.random.default_rng(seed)
    lon, lat = speedy_grid(nlon, nlat)
    R = 6371.3e3
    # stations: denser over a few "continents"
    centers = np.array([[260.0, 40.0], [10.0, 50.0], [110.0, 35.0], [300.0, -20.0]])
    ncl = int(0.7 * nstations)
    c = centers[rng.integers(0, len(centers), ncl)]
    slon = np.mod(c[:, 0] + 15 * rng.standard_normal(ncl), 360.0)
    slat = np.clip(c[:, 1] + 10 * rng.standard_normal(ncl), -85.0, 85.0)
    nu = nstations - ncl
    slon = np.concatenate([slon, rng.uniform(0, 360, nu)])
    slat = np.concatenate([slat, np.degrees(np.arcsin(rng.uniform(-0.99, 0.99, nu)))])
    ps_st = 1.0e5 * (1 + 0.02 * rng.standard_normal(nstations))
    # observation records
    elm, olon, olat, olev, odat, oerr, ovar = [], [], [], [], [], [], []
    errs = {ID_U: 1.0, ID_V: 1.0, ID_T: 1.0, ID_Q: 1.0e-3, ID_PS: 100.0}
    for s in range(nstations):
        for k in range(nlev):
            for e, v in ((ID_U, 0), (ID_V, 1), (ID_T, 2), (ID_Q, 3)):
                if rng.uniform() < 0.1:
                    continue  # missing report
                elm.append(e); olon.append(slon[s]); olat.append(slat[s])
                olev.append(ps_st[s] * SPEEDY_SIG[k]); oerr.append(errs[e]); ovar.append(v)
        elm.append(ID_PS); olon.append(slon[s]); olat.append(slat[s]); olev.append(ps_st[s])
        oerr.append(errs[ID_PS]); ovar.append(4)
    elm = np.array(elm, float); olon = np.array(olon); olat = np.array(olat); olev = np.array(olev)
    oerr = np.array(oerr); ovar = np.array(ovar)
    # smooth member fields on the sphere x ln(sigma)
    amp = np.array([5.0, 5.0, 2.0, 1.0e-3, 200.0])
    fields = SmoothFields(rng, ne + 1, 5, 6, wavenum_scale=R / 2.0e6, dims=4, amp=amp)

    def xyz(lo, la, lnsig):
        lo = np.radians(lo); la = np.radians(la)
        return np.stack([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la), lnsig / 2.0], -1)

    ps_mean = 1.0e5
    lnsig_obs = np.where(elm == ID_PS, 0.0, np.log(olev / ps_mean))
    hx = fields.eval(xyz(olon, olat, lnsig_obs), ovar)       # (ne+1, nobs); member ne is the truth
    truth_o = hx[ne]
    hx = hx[:ne]
    hxm = hx.sum(0) / ne
    y = truth_o + oerr * rng.standard_normal(olev.size)
    dep = y - hxm
    # surface-pressure reports carry the observed pressure (used by the vertical test)
    odat = np.where(elm == ID_PS, olev + y, y)
    hdxf = (hx - hxm).T                                        # (nobs, ne)
    # grid points (ij, ilev)
    glon, glat = np.meshgrid(lon, lat)                         # (nlat, nlon)
    glon = glon.ravel(); glat = glat.ravel()
    ps_grid = 1.0e5 * np.ones(glon.size)
    logpfm = np.log(ps_grid[None, :] * SPEEDY_SIG[:, None])   # (nlev, nij)
    gfield = np.stack([fields.eval(xyz(glon, glat, np.full(glon.size, math.log(SPEEDY_SIG[k]))), v)[:ne]
                       for v in range(4) for k in range(nlev)])  # (4*nlev, ne, nij)
    gues3d = gfield.reshape(4, nlev, ne, glon.size)
    dist_zero = sigma_obs * math.sqrt(10.0 / 3.0) * 2.0
    dist_zerov = sigma_obsv * math.sqrt(10.0 / 3.0) * 2.0
    dlat_zero = dist_zero / 3.1415926535 / R * 180.0     # speedy/letkf/letkf_obs.f90:82-88 (pi of common.f90)
    dlon_zero = dlat_zero / np.cos(3.1415926535 * glat / 180.0)
    return dict(lon=lon, lat=lat, elm=elm, olon=olon, olat=olat, olev=olev, odat=odat, oerr=oerr, hdxf=hdxf,
                dep=dep, glon=glon, glat=glat, logpfm=logpfm, dlon_zero=dlon_zero, dist_zero=dist_zero,
                dist_zerov=dist_zerov, dlat_zero=dlat_zero, sigma_obs=sigma_obs, sigma_obsv=sigma_obsv,
                gues3d=gues3d, ne=ne, nlev=nlev, var_local=np.ones(7))


def speedy_members(rng, ne, nlon=96, nlat=48, nlev=7):
    """Member states on the SPEEDY grid in grd-file order: v3d [ne, 4, nlev,
    nlat, nlon] (u, v m/s; t K, a troposphere-like profile crossing 0 C and
    -15 C so every calc_rh branch is met; q kg/kg, positive) and v2d [ne, 2,
    nlat, nlon] (ps Pa around 1e5, rain >= 0)."""
    shape3 = (ne, nlev, nlat, nlon)
    u = 10.0 * rng.standard_normal(shape3)
    v = 10.0 * rng.standard_normal(shape3)
    tprof = np.linspace(295.0, 215.0, nlev)[None, :, None, None]
    t = tprof + 8.0 * rng.standard_normal(shape3)
    qprof = np.geomspace(1.5e-2, 2.0e-5, nlev)[None, :, None, None]
    q = qprof * rng.uniform(0.2, 1.2, shape3)
    ps = 1.0e5 + 1.5e3 * rng.standard_normal((ne, nlat, nlon))
    rain = np.maximum(rng.standard_normal((ne, nlat, nlon)), 0.0) * 1.0e-4
    v3d = np.stack([u, v, t, q], axis=1)
    v2d = np.stack([ps, rain], axis=1)
    return np.ascontiguousarray(v3d), np.ascontiguousarray(v2d)


def speedy_obs_records(rng, nobs, lon, lat, nlon=96, with_edges=True):
    """Observation records (elem, rlon, rlat, rlev, odat) over the SPEEDY grid
    for the observation operator: all seven element codes, levels from above
    the model top to below the surface, and with_edges adds the corner cases
    (longitude 0 / 360 / grid-aligned / negative, latitudes on the table, past
    the outermost rows and at the poles, missing ps, non-positive levels and
    an unknown element code)."""
    codes = np.array([ID_U, ID_V, ID_T, ID_Q, ID_RH, ID_PS, ID_RAIN])
    elem = codes[rng.integers(0, codes.size, nobs)]
    rlon = rng.uniform(0.0, 360.0, nobs)
    rlat = np.degrees(np.arcsin(rng.uniform(-1.0, 1.0, nobs)))
    rlev = np.exp(rng.uniform(np.log(3.0e3), np.log(1.08e5), nobs))
    odat = rng.standard_normal(nobs)
    if with_edges:
        m = min(nobs, 64)
        pick = rng.choice(nobs, m, replace=False)
        kinds = np.arange(m) % 12
        for p, kd in zip(pick, kinds):
            if kd == 0:
                rlon[p] = 0.0
            elif kd == 1:
                rlon[p] = 360.0
            elif kd == 2:
                rlon[p] = 360.0 / nlon * rng.integers(0, nlon)
            elif kd == 3:
                rlon[p] = -rng.uniform(0.1, 10.0)
            elif kd == 4:
                rlat[p] = lat[rng.integers(0, lat.size)]
            elif kd == 5:
                rlat[p] = rng.choice([-90.0, 90.0, lat[0] - 0.5, lat[-1] + 0.5, lat[-1]])
            elif kd == 6:
                elem[p] = ID_PS
                odat[p] = -999.0
            elif kd == 7:
                rlev[p] = rng.choice([0.0, -5.0])
            elif kd == 8:
                elem[p] = 1234
            elif kd == 9:
                elem[p] = rng.choice([ID_U, ID_V])
                rlev[p] = 1.1e5
            elif kd == 10:
                elem[p] = rng.choice([ID_T, ID_Q, ID_RH])
                rlev[p] = 1.1e5
            else:
                rlev[p] = 5.0e2
    return elem.astype(np.int32), rlon, rlat, rlev, odat


# --------------------------------------------------------------------- regional
REGIONAL_P_TOP = 1.0e4
REGIONAL_P_BOT = 1.0e5


def regional_levels(nlev):
    """Full-level pressures, uniform in ln p from 1000 hPa to 100 hPa."""
    return np.exp(np.linspace(math.log(REGIONAL_P_BOT), math.log(REGIONAL_P_TOP), nlev))


def regional_obs(rng, nobs, nlon, nlat, void_frac=0.2, nmode=8, wavelength_cells=(40.0, 120.0), frac_ps=0.02):
    """Observation positions in grid coordinates (1-based ri, rj) drawn from a
    clustered density: a smooth random field G (nmode random plane waves of
    wavelength_cells) cut at the quantile void_frac, rho = max(G - t, 0), so
    that about void_frac of the domain has no observations and the rest is
    uneven.  A share frac_ps are surface-pressure reports (class 1).  Levels
    are uniform in ln p between 1000 and 100 hPa."""
    ang = rng.uniform(0, 2 * math.pi, nmode)
    wl = rng.uniform(*wavelength_cells, nmode)
    kx, ky = 2 * math.pi / wl * np.cos(ang), 2 * math.pi / wl * np.sin(ang)
    ph = rng.uniform(0, 2 * math.pi, nmode)

    def G(x, y):
        return np.cos(np.outer(x, kx) + np.outer(y, ky) + ph).sum(1)

    gx, gy = np.meshgrid(np.linspace(0.5, nlon + 0.5, 128), np.linspace(0.5, nlat + 0.5, 128))
    gs = G(gx.ravel(), gy.ravel())
    t = np.quantile(gs, void_frac)
    gmax = gs.max() - t
    ri = np.empty(0)
    rj = np.empty(0)
    while ri.size < nobs:
        m = 2 * (nobs - ri.size) + 1024
        x = rng.uniform(0.5, nlon + 0.5, m)
        y = rng.uniform(0.5, nlat + 0.5, m)
        keep = rng.uniform(0, gmax, m) < (G(x, y) - t)
        ri = np.concatenate([ri, x[keep]])
        rj = np.concatenate([rj, y[keep]])
    ri, rj = ri[:nobs], rj[:nobs]
    lnp = rng.uniform(math.log(REGIONAL_P_TOP), math.log(REGIONAL_P_BOT), nobs)
    cls = (rng.uniform(size=nobs) < frac_ps).astype(np.int32)
    return ri, rj, np.exp(lnp), cls


REGIONAL_SIGMA_OBS = 3.0e3   # horizontal localisation (m): 1e6 obs on 768 km x 768 km give 0-2035 local obs
REGIONAL_SIGMA_OBSV = 0.4    # vertical localisation (ln p)


def regional_case(seed=0, nlon=32, nlat=32, nlev=8, ne=64, nobs=20000, nvar=6, dx=3000.0,
                  sigma_obs=REGIONAL_SIGMA_OBS, sigma_obsv=REGIONAL_SIGMA_OBSV, dtype=np.float64,
                  with_grid_ensemble=True):
    """Cartesian regional case (SCALE-style search).  Small by default for
    tests; bench.py builds the full-size case on the device."""
    rng = np.random.default_rng(seed)
    ri, rj, lev, cls = regional_obs(rng, nobs, nlon, nlat)
    var = rng.integers(0, nvar, nobs)
    err = np.where(cls == 1, 100.0, 1.0)
    dat_ps = 1.0e5 * (1 + 0.01 * rng.standard_normal(nobs))
    Lc = 60.0e3
    fields = SmoothFields(rng, ne + 1, nvar, 6, wavenum_scale=1.0, dims=3)

    def xyz(x, y, lnp):
        return np.stack([x * dx / Lc, y * dx / Lc, lnp / 0.8], -1)

    lnp_o = np.where(cls == 1, math.log(REGIONAL_P_BOT), np.log(lev))
    hx = fields.eval(xyz(ri, rj, lnp_o), var)
    truth = hx[ne]
    hx = hx[:ne].astype(dtype).astype(np.float64)
    hxm = hx.sum(0) / ne
    hdxf = (hx - hxm).T
    y = truth + err * rng.standard_normal(nobs)
    dep = y - hxm
    plev = regional_levels(nlev)
    gi, gj = np.meshgrid(np.arange(1, nlon + 1, dtype=np.float64), np.arange(1, nlat + 1, dtype=np.float64))
    gi, gj = gi.ravel(), gj.ravel()
    nij = gi.size
    pri = np.tile(gi, nlev)
    prj = np.tile(gj, nlev)
    prlev = np.repeat(plev, nij)
    case = dict(nlon=nlon, nlat=nlat, nlev=nlev, ne=ne, nvar=nvar, dx=dx, dy=dx, ri=ri, rj=rj, lev=lev,
                dat=np.where(cls == 1, dat_ps, y), err=err, cls=cls, var=var, hdxf=hdxf, dep=dep, pri=pri, prj=prj,
                prlev=prlev, sigma_obs=sigma_obs, sigma_obsv=sigma_obsv)
    if with_grid_ensemble:
        xg = np.stack([fields.eval(xyz(pri, prj, np.log(prlev)), v)[:ne] for v in range(nvar)])  # (nvar, ne, npts)
        case["xb"] = np.ascontiguousarray(np.transpose(xg, (0, 2, 1)).astype(dtype))  # (nvar, npts, ne)
    return case


def scale_params(case):
    """SCALE search parameters for a regional case (scale/letkf/letkf_obs.f90:122-128)."""
    dzf = float(np.float32(3.651483717))
    so = case["sigma_obs"]
    return dict(dx=case["dx"], dy=case["dy"], dlon_zero=so * dzf / case["dx"], dlat_zero=so * dzf / case["dy"],
                sigma_obs=so, sigma_obsv=case["sigma_obsv"], sigma_obs_rain=350.0e3, sigma_obsv_rain=0.4,
                base_obsv_rain=85000.0, sigma_obs_radar=2000.0, sigma_obs_radar_noref=2000.0,
                sigma_obsz_radar=1000.0, radar_ref_thres_dbz=15.0, sigma_obs_tc=50.0e3, sigma_obsv_tc=0.4)
