"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference ships no tests, golden vectors or fixtures, and its Fortran does
not build here (no Fortran compiler), so the fixtures are oracle outputs on
seeded inputs.  They pin the oracle against regressions (CPU tests) and give
the CUDA path committed vectors to match (GPU tests).  Each case stores its
inputs and outputs so the tests need no generator.

    python tests/golden/make_golden.py [name.npz ...]   # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from letkf_gb300 import synthetic as S  # noqa: E402
from letkf_gb300.core import SCALE_PARAM_ORDER  # noqa: E402
from oracle import oracle as O  # noqa: E402

# (ne, L, rdiag_wloc, minfl, parm_infl): the branches of letkf_core
# (common/common_letkf.f90:50-243): plain, nobsl = 0, rdiag_wloc, minfl clamp,
# rank-deficient Gram with a tiny diagonal (mtx_eigen truncation) and k = 2.
CORE_CASES = [
    (8, 12, False, None, 1.05),
    (20, 21, False, None, 1.05),
    (40, 0, False, 1.5, 1.2),
    (16, 40, True, None, 0.95),
    (32, 60, False, 1.1, 1.02),
    (16, 3, False, None, 1.0e12),
    (2, 1, False, None, 1.0),
    (64, 150, False, None, 1.3),
]


def core_fixture(rng):
    out = {"ncase": np.int64(len(CORE_CASES))}
    for c, (ne, L, wloc, minfl, infl) in enumerate(CORE_CASES):
        n = max(L, 1)
        Y = rng.standard_normal((n, ne))
        Y -= Y.mean(1, keepdims=True)
        rd = rng.uniform(0.3, 3.0, n)
        rl = rng.uniform(0.01, 1.0, n)
        d = rng.standard_normal(n)
        r = O.letkf_core(Y, rd, rl, d, infl, nobsl=L, want_transm=True, want_pao=True, rdiag_wloc=wloc,
                         minfl=minfl)
        assert r["status"] == 0
        p = f"c{c}_"
        out.update({p + "hdxb": Y, p + "rdiag": rd, p + "rloc": rl, p + "dep": d,
                    p + "meta": np.array([ne, L, int(wloc), -1.0 if minfl is None else minfl, infl]),
                    p + "trans": r["trans"], p + "transm": r["transm"], p + "pao": r["pao"],
                    p + "infl": np.float64(r["parm_infl"])})
    return out


def scale_fixture():
    nlon, nlat, nlev = 16, 12, 4
    case = S.regional_case(5, nlon=nlon, nlat=nlat, nlev=nlev, ne=8, nobs=1000, sigma_obs=6.0e3,
                           with_grid_ensemble=False)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(nlon, nlat, case["ri"], case["rj"])
    srt = {k: case[k][perm] for k in ("ri", "rj", "lev", "dat", "err", "cls")}
    nobs = perm.size
    varloc = (np.arange(nobs) % 3).astype(np.int32)
    var_local = [1.0, 0.0, 0.5]
    so = O.ScaleObs(nlon, nlat, grd, srt["ri"], srt["rj"], srt["lev"], srt["dat"], srt["err"], srt["cls"],
                    np.zeros(nobs), np.zeros(nobs), varloc, 1, 1, prm["dx"], prm["dy"], prm["dlon_zero"],
                    prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"], var_local)
    pts = np.arange(0, case["pri"].size, 17)
    offs, idx, rloc, rdiag = [0], [], [], []
    for p in pts:
        i, rl, rd = so.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p])
        idx.append(i)
        rloc.append(rl)
        rdiag.append(rd)
        offs.append(offs[-1] + i.size)
    out = {"nlon": np.int64(nlon), "nlat": np.int64(nlat), "perm": perm, "nobsgrd": grd, "varloc": varloc,
           "var_local": np.array(var_local), "pri": case["pri"][pts], "prj": case["prj"][pts],
           "prlev": case["prlev"][pts], "offs": np.array(offs, dtype=np.int64),
           "idx": np.concatenate(idx).astype(np.int32), "rloc": np.concatenate(rloc),
           "rdiag": np.concatenate(rdiag)}
    for k in ("ri", "rj", "lev", "dat", "err", "cls"):
        out["obs_" + k] = srt[k]
    for k in SCALE_PARAM_ORDER:
        out["prm_" + k] = np.float64(prm[k])
    assert out["idx"].size > 300
    return out


def speedy_fixture():
    c = S.speedy_case(3, nstations=120)
    perm, grd = O.speedy_sort_obs(c["lon"], c["lat"], c["olon"], c["olat"])
    srt = {k: c[k][perm] for k in ("elm", "olon", "olat", "olev", "odat", "oerr")}
    sigma_obs = 500.0e3
    dist_zero = sigma_obs * math.sqrt(10.0 / 3.0) * 2.0
    dlat_zero = dist_zero / 3.1415926535 / 6371.3e3 * 180.0
    dlon_zero = dlat_zero / np.cos(3.1415926535 * c["glat"] / 180.0)
    so = O.SpeedyObs(c["lon"], c["lat"], grd, srt["elm"], srt["olon"], srt["olat"], srt["olev"], srt["odat"],
                     srt["oerr"], dist_zero, c["dist_zerov"], dlat_zero, sigma_obs, c["sigma_obsv"], c["var_local"])
    hp = np.arange(0, c["glon"].size, 11)
    ilev = np.repeat([1, 3, 7], hp.size).astype(np.int32)
    hp3 = np.tile(hp, 3)
    logp = c["logpfm"][ilev - 1, hp3]
    offs, idx, rloc, rdiag = [0], [], [], []
    for p in range(hp3.size):
        i, rl, rd = so.obs_local(c["glon"][hp3[p]], c["glat"][hp3[p]], dlon_zero[hp3[p]], int(ilev[p]), logp[p])
        idx.append(i)
        rloc.append(rl)
        rdiag.append(rd)
        offs.append(offs[-1] + i.size)
    out = {"lon": c["lon"], "lat": c["lat"], "perm": perm, "nobsgrd": grd,
           "params": np.array([dist_zero, c["dist_zerov"], dlat_zero, sigma_obs, c["sigma_obsv"]]),
           "var_local": np.asarray(c["var_local"], dtype=np.float64), "plon": c["glon"][hp3],
           "plat": c["glat"][hp3], "pdlon_zero": dlon_zero[hp3], "pilev": ilev, "plogpfm": logp,
           "offs": np.array(offs, dtype=np.int64), "idx": np.concatenate(idx).astype(np.int32),
           "rloc": np.concatenate(rloc), "rdiag": np.concatenate(rdiag)}
    for k in ("elm", "olon", "olat", "olev", "odat", "oerr"):
        out["obs_" + k] = srt[k]
    assert out["idx"].size > 200
    return out


def l96_fixture():
    """One LETKF analysis of Lorenz-96 (N = 40, k = 20, 40 identity obs, xlocal = 3,
    fixed inflation 1.05; lorenz96/letkf/letkf.f90:217-265) from a seeded state."""
    c = S.l96_case(11)
    xf = c["xf"].T.copy()                  # (nx, ne)
    nx, ne = xf.shape
    h = c["h"]
    xm = xf.sum(1) / ne
    dxf = xf - xm[:, None]
    hdxf, dep = c["hdxf"], c["dep"]
    trans_all, xa = [], np.zeros_like(xf)
    idx_all, rloc_all, offs = [], [], [0]
    for ix in range(1, nx + 1):
        idx, rl = O.l96_select(h, ix, 3.0)
        r = O.letkf_core(hdxf[idx], np.full(idx.size, c["obserr"] ** 2), rl, dep[idx], 1.05)
        xa[ix - 1] = xm[ix - 1] + dxf[ix - 1] @ r["trans"]
        idx_all.append(idx)
        rloc_all.append(rl)
        offs.append(offs[-1] + idx.size)
        trans_all.append(r["trans"])
    return {"xf": xf, "h": h, "y": c["y"], "hdxf": hdxf, "dep": dep, "obserr": np.float64(c["obserr"]), "xa": xa,
            "trans": np.array(trans_all), "offs": np.array(offs, dtype=np.int64),
            "idx": np.concatenate(idx_all).astype(np.int32), "rloc": np.concatenate(rloc_all)}


def scale_obsope_fixture():
    """The SCALE conventional observation operator (scale/obs/obsope_tools.f90:
    340-380) on 4 members of a 10 x 9 x (6 + 2 KHALO) domain with terrain
    (levels below ground in some columns): 240 observations of every element
    inside, outside, above and below the domain, rotated winds."""
    rng = np.random.default_rng(31)
    ne, nlonh, nlath, nlev, kh = 4, 10, 9, 6, 2
    nlevh = nlev + 2 * kh
    sig = np.exp(-0.45 * (np.arange(nlevh) - kh))
    J, I = np.meshgrid(np.arange(1, nlath + 1), np.arange(1, nlonh + 1), indexing="ij")
    zs = 300.0 * (1 + np.sin(I / 2.0) * np.cos(J / 3.0))
    v3d = np.empty((ne, 6, nlath, nlonh, nlevh))
    v2d = np.empty((ne, 4, nlath, nlonh))
    for m in range(ne):
        ps = 1.0e5 * np.exp(-zs / 8000.0) * (1 + 0.01 * rng.standard_normal((nlath, nlonh)))
        p = ps[:, :, None] * sig[None, None, :]
        v3d[m, 5] = np.where((zs > 450.0)[:, :, None] & (np.arange(nlevh) < kh + 2), -1.0, p)
        for n, (sc, off) in enumerate([(5, 3), (5, -2), (8, 260), (0.002, 0.005), (0.1, 0.6)]):
            v3d[m, n] = off + sc * rng.standard_normal((nlath, nlonh, nlevh))
        v2d[m] = np.stack([ps, 285 + rng.standard_normal((nlath, nlonh)),
                           0.008 + 0.001 * rng.standard_normal((nlath, nlonh)), zs])
    nobs = 240
    elem = rng.choice(np.array([2819, 2820, 3073, 3074, 3330, 3331, 14593, 4321], np.int32), nobs).astype(np.int32)
    ri = rng.uniform(0.5, nlonh + 0.3, nobs)
    rj = rng.uniform(0.5, nlath + 0.3, nobs)
    rlev = np.exp(rng.uniform(np.log(3e3), np.log(1.2e5), nobs))
    sfc = elem == 14593
    rlev[sfc] = rng.uniform(0.0, 900.0, sfc.sum())
    ang = rng.uniform(-0.6, 0.6, nobs)
    rotc = np.stack([np.cos(ang), np.sin(ang)], -1)
    hx, qc, qcm = O.scale_obsope(v3d, v2d, kh, elem, ri, rj, rlev, rotc)
    assert {0, 10, 20, 21, 22, 90} <= set(np.unique(qcm).tolist())
    return {"v3d": v3d, "v2d": v2d, "khalo": np.int32(kh), "elem": elem, "ri": ri, "rj": rj, "rlev": rlev,
            "rotc": rotc, "hx": hx, "qc": qc, "qc_member": qcm}


FIXTURES = {"core_cases.npz": lambda rng: core_fixture(rng), "scale_search.npz": lambda rng: scale_fixture(),
            "speedy_search.npz": lambda rng: speedy_fixture(), "l96_analysis.npz": lambda rng: l96_fixture(),
            "scale_obsope.npz": lambda rng: scale_obsope_fixture()}


def main(names=None):
    """Rewrite the named fixtures (all of them by default); the core cases
    draw from one seeded generator, so they are made first in this order."""
    rng = np.random.default_rng(20240601)
    files = {}
    for name, make in FIXTURES.items():
        d = make(rng)
        if not names or name in names:
            files[name] = d
    for name, d in files.items():
        path = os.path.join(HERE, name)
        np.savez_compressed(path, **d)
        print(f"{name}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
