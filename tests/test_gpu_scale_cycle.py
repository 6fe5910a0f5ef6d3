"""A SCALE cycle on the device: H(x) of every member by the conventional
observation operator (scale/obs/obsope_tools.f90:340-380), set_letkf_obs's
departures, gross-error check and selection (scale/letkf/letkf_obs.f90:
260-600), then the analysis sweep over the selected observations
(scale/letkf/letkf_tools.f90:38-476) -- against the same chain on the oracle:
qc equal, departures within 1e-9, analysis within 1e-4 of the background
spread."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KH = 2
ELEMS = np.array([2819, 2820, 3073, 3074, 3330, 3331, 14593], np.int32)
ERR = {2819: 2.0, 2820: 2.0, 3073: 1.0, 3074: 1.0, 3330: 1.0e-3, 3331: 0.1, 14593: 100.0}


def scale_domain(seed, ne=32, nlonh=28, nlath=24, nlev=8):
    rng = np.random.default_rng(seed)
    nlevh = nlev + 2 * KH
    J, I, K = np.meshgrid(np.arange(1, nlath + 1), np.arange(1, nlonh + 1), np.arange(1, nlevh + 1), indexing="ij")
    sig = np.exp(-0.35 * (np.arange(nlevh) - KH))
    v3d = np.empty((ne, 6, nlath, nlonh, nlevh))
    v2d = np.empty((ne, 4, nlath, nlonh))
    smooth = lambda ph: np.sin(I / 4.0 + ph[0]) * np.cos(J / 5.0 + ph[1]) + 0.3 * np.sin(K / 2.0 + ph[2])
    base = [smooth(rng.uniform(0, 6, 3)) for _ in range(5)]
    for m in range(ne):
        ps = 1.0e5 * (1 + 0.01 * np.sin(I[:, :, 0] / 6.0) + 0.002 * rng.standard_normal((nlath, nlonh)))
        v3d[m, 5] = ps[:, :, None] * sig[None, None, :]
        for n, (scale, off) in enumerate([(8, 2), (8, -1), (5, 270), (0.002, 0.006), (0.2, 0.6)]):
            v3d[m, n] = off + scale * (base[n] + 0.4 * smooth(rng.uniform(0, 6, 3)))
        v2d[m, 0] = ps
        v2d[m, 1] = 285 + rng.standard_normal((nlath, nlonh))
        v2d[m, 2] = 0.008 + 0.0005 * rng.standard_normal((nlath, nlonh))
        v2d[m, 3] = 20.0
    return v3d, v2d, sig


def observations(rng, v3d, v2d, sig, nobs=1500):
    ne, _, nlath, nlonh, nlevh = v3d.shape
    elem = rng.choice(ELEMS, nobs).astype(np.int32)
    ri = rng.uniform(3, nlonh - 2, nobs)
    rj = rng.uniform(3, nlath - 2, nobs)
    plo, phi = 1.0e5 * sig[KH + 1], 1.0e5 * sig[nlevh - KH - 2]
    rlev = np.exp(rng.uniform(np.log(phi), np.log(plo), nobs))
    sfc = elem == 14593
    rlev[sfc] = rng.uniform(0.0, 150.0, sfc.sum())  # heights; |z - topo| > 100 m is qc 10
    err = np.array([ERR[e] for e in elem])
    hx, qc, _ = O.scale_obsope(v3d, v2d, KH, elem, ri, rj, rlev)
    dat = hx.mean(1) + err * rng.standard_normal(nobs)
    bad = rng.random(nobs) < 0.05
    dat[bad] += 20 * err[bad]  # gross errors
    return {"elem": elem, "ri": ri, "rj": rj, "lev": rlev, "dat": dat, "err": err}


def oracle_setup(v3d, v2d, obs, gross=5.0):
    hx, qc, _ = O.scale_obsope(v3d, v2d, KH, obs["elem"], obs["ri"], obs["rj"], obs["lev"])
    ne = hx.shape[1]
    mean = hx[:, 0].copy()
    for m in range(1, ne):  # sequential member sum (scale/letkf/letkf_obs.f90:562-566)
        mean = mean + hx[:, m]
    mean = mean / ne
    dep = obs["dat"] - mean
    qc = qc.copy()
    qc[(qc == 0) & (np.abs(dep) > gross * obs["err"])] = 5
    sel = qc == 0
    return qc, sel, hx - mean[:, None], dep


def test_scale_cycle_on_the_device(cuda):
    import torch

    from letkf_gb300.drivers import scale_obs_setup
    from letkf_gb300.sweep import PREC_MIXED, Sweep

    rng = np.random.default_rng(21)
    v3d, v2d, sig = scale_domain(4)
    obs = observations(rng, v3d, v2d, sig)
    qc_ref, sel, hdxf_ref, dep_ref = oracle_setup(v3d, v2d, obs)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    rec, qc = scale_obs_setup(t(v3d), t(v2d), KH, obs)
    np.testing.assert_array_equal(qc, qc_ref)
    assert {0, 5, 10} <= set(np.unique(qc).tolist())
    np.testing.assert_allclose(rec["dep"], dep_ref[sel], rtol=0, atol=1e-9 * np.abs(obs["dat"]).max())
    np.testing.assert_array_equal(rec["ri"], obs["ri"][sel])

    # the analysis of t and q at the interior grid points of every model level
    ne, _, nlath, nlonh, nlevh = v3d.shape
    ii, jj, kk = np.meshgrid(np.arange(3, nlonh - 1), np.arange(3, nlath - 1), np.arange(KH + 1, nlevh - KH + 1),
                             indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    pri, prj = ii.astype(np.float64), jj.astype(np.float64)
    prlev = v3d[:, 5, jj - 1, ii - 1, kk - 1].mean(0)
    xb = np.stack([v3d[:, n, jj - 1, ii - 1, kk - 1].T for n in (2, 3)]).astype(np.float32)  # [2][npts][ne]
    npts = pri.size
    prm = S.scale_params({"dx": 3000.0, "dy": 3000.0, "sigma_obs": 12.0e3, "sigma_obsv": 0.4})
    sw = Sweep(ne, 2, nlonh, nlath, npts, prm, precision=PREC_MIXED)
    sw.set_points(pri, prj, prlev)
    sw.set_obs(rec["ri"], rec["rj"], rec["lev"], rec["dat"], rec["err"], rec["dep"], rec["cls"], rec["hdxf"])
    sw.set_background(xb)
    sw.set_inflation(np.full(npts, 1.05))
    sw.run()
    xa = sw.analysis().astype(np.float64)
    sw.close()

    # the oracle's grid loop over the oracle's selection (its sorted order)
    cls = (obs["elem"][sel] == 14593).astype(np.int32)
    perm, grd = O.scale_sort_obs(nlonh, nlath, obs["ri"][sel], obs["rj"][sel])
    nob = perm.size
    g = lambda a: np.asarray(a)[sel][perm]
    so = O.ScaleObs(nlonh, nlath, grd, g(obs["ri"]), g(obs["rj"]), g(obs["lev"]), g(obs["dat"]), g(obs["err"]),
                    cls[perm], np.zeros(nob), np.zeros(nob), np.zeros(nob, np.int32), 1, 1, prm["dx"], prm["dy"],
                    prm["dlon_zero"], prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"], None)
    hd = hdxf_ref[sel].astype(np.float32).astype(np.float64)[perm]
    xa_ref, _, nl_ref = so.sweep(hd, dep_ref[sel][perm], xb.astype(np.float64), pri, prj, prlev, np.full(npts, 1.05))
    assert nl_ref.max() > 20
    x64 = xb.astype(np.float64)
    spread = np.sqrt(((x64 - x64.mean(-1, keepdims=True)) ** 2).sum(-1) / (ne - 1)).mean()
    em = np.sqrt(np.mean((xa.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread
    ep = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True)) - (xa_ref - xa_ref.mean(-1, keepdims=True))) ** 2))
    assert em < 1e-4 and ep / spread < 1e-4, (em, ep / spread)
