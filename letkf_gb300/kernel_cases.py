"""Run every kernel of libletkf_gpu.so once on a profiling-size case.

    python -m letkf_gb300.kernel_cases [--only NAME ...]

Cases (seeded synthetic data, a few hundred MB on the device, larger than L2
where the kernel streams the ensemble):
  sweep_tc      tensor-core sweep of a 96x96x16 regional domain (147,456
                points, k = 64, 6 variables, 140,625 clustered obs) and its
                deferred-point pass
  sweep_tc40    tensor-core sweep of a 64x64x40 regional domain (163,840
                points in columns of 40 levels as the benchmark's, k = 64, 6
                variables, 62,500 clustered obs: the benchmark's density)
  sweep_simt    the same sweep on the SIMT kernel
  sweep_tc128   the tensor-core sweep of the same domain with k = 128
  search_700km  SPEEDY lat/lon search (count and fill) of 64 points of the
                360x181x32 global grid with 3e6 observations at 700 km
  largek_700km  the large-k step of 16 of those points (k = 512, BF16
                observation ensemble): search, the mixed-precision core and
                its FP64 pass (every point at 700 km), BF16-storage update
  scale_obsope  SCALE observation operator, 40 members of a 128x128x30
                domain (KHALO 2, 1.07 GB of FP64 fields), 100,000
                conventional observations of every element
  f64           FP64 plain form of 8,192 of those points: search (count,
                fill), gather, core_f64, update_f64
  l96           Lorenz-96 ring of 100,000 variables, k = 32: departures,
                selection, mixed core, update
  relax         RTPS update with relax_beta weights of 50,000 points, k = 64
  largek        large-ensemble core of 512 points, k = 512, 100-900 local obs
                each, and the FP32 update of 6 variables
  speedy_io     80 SPEEDY T63 member files (192x96, 7 levels, 30 records;
                177 MB of file bytes) decoded to FP64, ensemble mean and
                spread, encoded back
  obsope        SPEEDY observation operator on those 80 members (354 MB in
                FP64) for 300,000 observations of all seven elements
  obs_space     obs-space analysis of 20,000 observation locations (k = 64,
                655 MB of transforms) and EFSO over 50,000 points with 50
                local observations each
Used for the ncu summaries under profiles/; prints one line per case.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def _regional(ne=64, shape=(96, 96, 16), nobs=140_625):
    from .workload import RegionalWorkload

    return RegionalWorkload(5, *shape, ne, nobs, 6)


def case_sweep(dev, tc, ne=64, shape=(96, 96, 16), nobs=140_625):
    import torch

    from .sweep import OPT_TENSOR_CORES, PREC_MIXED, Sweep

    wl = _regional(ne, shape, nobs)
    hdxf, dep, dat = wl.obs_torch(dev)
    xb = wl.background_torch(dev)
    ri, rj, plev = wl.points()
    sw = Sweep(ne, wl.nvar, wl.nlon, wl.nlat, wl.npts, wl.params, precision=PREC_MIXED)
    sw.set_points(ri, rj, plev, tile=4)
    sw.set_obs(wl.ri, wl.rj, wl.lev, dat, wl.err, dep, wl.cls, hdxf)
    sw.set_option(OPT_TENSOR_CORES, int(tc))
    sw.set_background_device(xb.data_ptr())
    sw.set_inflation(np.ones(wl.npts))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sw.run()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sw.close()
    return f"{wl.npts} points, {wl.nobs} obs, {dt * 1e3:.1f} ms"


def case_f64(dev):
    import torch

    from .sweep import PREC_F64, Sweep

    wl = _regional()
    sub = np.arange(0, wl.npts, wl.npts // 8192)[:8192]
    hdxf, dep, dat = wl.obs_torch(dev)
    ri, rj, plev = wl.points(sub)
    sw = Sweep(64, wl.nvar, wl.nlon, wl.nlat, sub.size, wl.params, precision=PREC_F64)
    sw.set_points(ri, rj, plev, tile=0)
    sw.set_obs(wl.ri, wl.rj, wl.lev, dat, wl.err, dep, wl.cls, hdxf.astype(np.float64))
    sw.set_background(wl.background_numpy(sub).astype(np.float64))
    sw.set_inflation(np.ones(sub.size))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sw.run()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sw.close()
    return f"{sub.size} points, {dt * 1e3:.1f} ms"


def case_l96(dev):
    import torch

    from .drivers import l96_letkf

    rng = np.random.default_rng(3)
    nx, ne = 100_000, 32
    xf = torch.as_tensor(8.0 + rng.standard_normal((nx, ne)), device=dev)
    cell = torch.arange(1, nx + 1, dtype=torch.int32, device=dev)
    y = torch.as_tensor(8.0 + rng.standard_normal(nx), device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xa, _ = l96_letkf(xf, xf.clone(), y, cell, precision="mixed")
    torch.cuda.synchronize()
    return f"{nx} variables, {(time.perf_counter() - t0) * 1e3:.1f} ms"


def case_relax(dev):
    import torch

    from .core import RELAX_RTPS, relax_beta, update_relax_f64

    rng = np.random.default_rng(4)
    npts, ne, nv = 50_000, 64, 2
    q, _ = np.linalg.qr(rng.standard_normal((ne, ne)))
    w = torch.as_tensor(np.broadcast_to(q, (npts, ne, ne)).copy(), device=dev)
    pa = torch.as_tensor(np.broadcast_to(np.eye(ne) / (ne - 1), (npts, ne, ne)).copy(), device=dev)
    xb = torch.as_tensor(rng.standard_normal((nv, npts, ne)), device=dev)
    ri = torch.as_tensor(rng.uniform(1, 200, npts), device=dev)
    rj = torch.as_tensor(rng.uniform(1, 250, npts), device=dev)
    rl = torch.as_tensor(rng.uniform(1e4, 1e5, npts), device=dev)
    beta = relax_beta(ri, rj, rl, nv, 1, 1, 3e4, 30e3, 3e3, 3e3, 200, 250, 2, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    update_relax_f64(xb, w, None, pa, mode=RELAX_RTPS, alpha=0.8, beta=beta)
    torch.cuda.synchronize()
    return f"{npts} points, {(time.perf_counter() - t0) * 1e3:.1f} ms"


def case_largek(dev):
    import torch

    from .core import core_batch_largek, update_mixed

    rng = np.random.default_rng(6)
    ne, npts = 512, 512
    Ls = rng.integers(100, 900, npts)
    offs = torch.as_tensor(np.concatenate([[0], np.cumsum(Ls)]), dtype=torch.int64, device=dev)
    n = int(Ls.sum())
    rows = torch.randn((n, ne), device=dev)
    rows -= rows.mean(1, keepdim=True)
    rd = torch.rand(n, device=dev) * 2.7 + 0.3
    rl = torch.rand(n, device=dev) * 0.99 + 0.01
    dep = torch.randn(n, device=dev)
    infl = torch.full((npts,), 1.1, dtype=torch.float64, device=dev)
    xb = torch.randn((6, npts, ne), device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = core_batch_largek(ne, offs, rows, rd, rl, dep, infl, want_transm=True)
    update_mixed(xb, out["trans"], out["transm"])
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    ok = int((out["status"] == 0).sum())
    return f"{npts} points (k = {ne}, mean L = {Ls.mean():.0f}), {dt * 1e3:.1f} ms, {npts / dt:.0f} points/s, {ok} ok"


def case_search_700km(dev):
    import torch

    from .core import search_speedy
    from .workload import GlobalWorkload

    wl = GlobalWorkload(21)
    params = wl.search_params(700.0e3)
    idx = np.sort(np.random.default_rng(5).choice(wl.npts, 64, replace=False))
    lon, lat, dlon, ilev, lnp = wl.points(idx, params)
    f = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    grid = {"lon": f(wl.lon), "lat": f(wl.lat), "nobsgrd": torch.as_tensor(wl.nobsgrd, dtype=torch.int32, device=dev)}
    obs = {"elm": f(wl.elm), "lon": f(wl.olon), "lat": f(wl.olat), "lev": f(wl.olev), "dat": f(wl.olev),
           "err": f(wl.err)}
    pts = {"lon": f(lon), "lat": f(lat), "dlon_zero": f(dlon), "ilev": torch.as_tensor(ilev, device=dev),
           "logpfm": f(lnp)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    offs, oi, rl, rd = search_speedy(grid, obs, pts, params, np.ones(7))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return f"64 points of the 360x181x32 grid, 3e6 obs, 700 km: {int(offs[-1])} local obs, {dt * 1e3:.1f} ms"


def case_largek_700km(dev):
    import torch

    from .core import core_batch_largek_indexed, search_speedy, update_bf16
    from .workload import GlobalWorkload

    wl = GlobalWorkload(21)
    hdxf, dep, dat = wl.obs_torch(dev)
    hdxf16 = hdxf.to(torch.bfloat16)
    del hdxf
    dep32 = dep.to(torch.float32)
    params = wl.search_params(700.0e3)
    idx = np.sort(np.random.default_rng(5).choice(wl.npts, 16, replace=False))
    lon, lat, dlon, ilev, lnp = wl.points(idx, params)
    f = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    grid = {"lon": f(wl.lon), "lat": f(wl.lat), "nobsgrd": torch.as_tensor(wl.nobsgrd, dtype=torch.int32, device=dev)}
    obs = {"elm": f(wl.elm), "lon": f(wl.olon), "lat": f(wl.olat), "lev": f(wl.olev), "dat": dat, "err": f(wl.err)}
    pts = {"lon": f(lon), "lat": f(lat), "dlon_zero": f(dlon), "ilev": torch.as_tensor(ilev, device=dev),
           "logpfm": f(lnp)}
    xb = wl.background_torch(dev, idx)
    xmean = xb.double().mean(-1).to(torch.float32)
    xpert16 = (xb - xmean[..., None]).to(torch.bfloat16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    offs, oi, rl, rd = search_speedy(grid, obs, pts, params, np.ones(7))
    infl = torch.full((idx.size,), 1.05, dtype=torch.float64, device=dev)
    core = core_batch_largek_indexed(wl.ne, offs, oi, hdxf16, dep32, rd.to(torch.float32), rl.to(torch.float32),
                                     infl, want_transm=True)
    update_bf16(xmean, xpert16, core["trans"], core["transm"])
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    ok = int((core["status"] == 0).sum())
    return f"16 points, k = {wl.ne}, 700 km: {int(offs[-1])} local obs, {ok} LETKF_OK, {dt * 1e3:.1f} ms"


def case_scale_obsope(dev):
    import torch

    from .core import SCALE_ELEM, scale_obsope

    ne, nlonh, nlath, nlev, kh, nobs = 40, 128, 128, 30, 2, 100_000
    g = torch.Generator(device=dev).manual_seed(6)
    nlevh = nlev + 2 * kh
    sig = torch.exp(-torch.linspace(-0.2, 4.2, nlevh, dtype=torch.float64, device=dev))
    ps = 1.0e5 * (1 + 0.02 * torch.randn((ne, 1, nlath, nlonh, 1), generator=g, device=dev, dtype=torch.float64))
    v3d = torch.randn((ne, 6, nlath, nlonh, nlevh), generator=g, device=dev, dtype=torch.float64)
    v3d[:, 2] = 260 + 10 * v3d[:, 2]
    v3d[:, 3] = 0.005 + 0.002 * v3d[:, 3]
    v3d[:, 5] = (ps * sig)[:, 0]
    v2d = torch.randn((ne, 4, nlath, nlonh), generator=g, device=dev, dtype=torch.float64)
    v2d[:, 0] = ps[:, 0, :, :, 0]
    v2d[:, 1] = 285 + v2d[:, 1]
    v2d[:, 2] = 0.008 + 0.001 * v2d[:, 2]
    v2d[:, 3] = 200 + 100 * v2d[:, 3]
    codes = torch.tensor(list(SCALE_ELEM.values()), dtype=torch.int32, device=dev)
    elem = codes[torch.randint(0, codes.numel(), (nobs,), generator=g, device=dev)]
    ri = 1 + (nlonh - 1) * torch.rand(nobs, generator=g, device=dev, dtype=torch.float64)
    rj = 1 + (nlath - 1) * torch.rand(nobs, generator=g, device=dev, dtype=torch.float64)
    rlev = torch.exp(np.log(3e3) + (np.log(1e5) - np.log(3e3)) *
                     torch.rand(nobs, generator=g, device=dev, dtype=torch.float64))
    rlev = torch.where(elem == SCALE_ELEM["ps"],
                       300.0 * torch.rand(nobs, generator=g, device=dev, dtype=torch.float64), rlev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hx, qc = scale_obsope(v3d, v2d, kh, elem, ri, rj, rlev)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return f"{nobs} obs x {ne} members, {int((qc == 0).sum())} good, {dt * 1e3:.2f} ms"


def _speedy_members(dev, ne=80, nlon=192, nlat=96, nlev=7):
    import torch

    from . import synthetic as S

    rng = np.random.default_rng(8)
    lon, lat = S.speedy_grid(nlon, nlat)
    v3d, v2d = S.speedy_members(rng, ne, nlon, nlat, nlev)
    return rng, lon, lat, torch.as_tensor(v3d, device=dev), torch.as_tensor(v2d, device=dev)


def case_speedy_io(dev):
    import torch

    from . import speedy_io as IO

    ne, nlon, nlat, nlev = 80, 192, 96, 7
    rng = np.random.default_rng(9)
    raw = torch.as_tensor(rng.standard_normal(ne * IO.grd_nrec(nlev) * nlat * nlon).astype(">f4").view(np.uint8),
                          device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g3, g2 = IO.decode_members(raw, ne, nlon, nlat, nlev)
    IO.mean_spread(g3, g2)
    back = IO.encode_members(g3, g2)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert torch.equal(back, raw)
    return f"{ne} members x {raw.numel() // ne} bytes, {dt * 1e3:.1f} ms"


def case_obsope(dev):
    import torch

    from . import synthetic as S
    from .core import speedy_obsope

    rng, lon, lat, v3d, v2d = _speedy_members(dev)
    el, lo, la, lv, od = S.speedy_obs_records(rng, 300_000, lon, lat, 192, with_edges=False)
    t = lambda a, dt=torch.float64: torch.as_tensor(a, dtype=dt, device=dev)
    args = (t(lat), t(S.SPEEDY_SIG), v3d, v2d, t(el, torch.int32), t(lo), t(la), t(lv), t(od))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hx, qc = speedy_obsope(*args)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return f"{el.size} obs x {v3d.shape[0]} members, {dt * 1e3:.1f} ms, qc {float(qc.float().mean()):.2f}"


def case_obs_space(dev):
    import torch

    from .core import efso, obs_analysis

    rng = np.random.default_rng(10)
    ne, n = 64, 20_000
    trans = torch.randn((n, ne, ne), dtype=torch.float64, device=dev) * 0.1
    hdxf = torch.randn((n, ne), dtype=torch.float64, device=dev)
    ybar = torch.randn(n, dtype=torch.float64, device=dev)
    mode = torch.as_tensor(rng.integers(0, 3, n), dtype=torch.int32, device=dev)
    npts, nobs, nv = 50_000, 100_000, 6
    offs = torch.arange(0, 50 * (npts + 1), 50, dtype=torch.int64, device=dev)
    idx = torch.as_tensor(rng.integers(0, nobs, 50 * npts), dtype=torch.int32, device=dev)
    rd = torch.rand(50 * npts, dtype=torch.float64, device=dev) + 0.5
    rl = torch.rand(50 * npts, dtype=torch.float64, device=dev)
    hdxa = torch.randn((nobs, ne), dtype=torch.float64, device=dev)
    fcst = torch.randn((nv, npts, ne), dtype=torch.float64, device=dev)
    fcer = torch.randn((nv, npts), dtype=torch.float64, device=dev)
    obsdep = torch.randn(nobs, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    obs_analysis(trans, ybar, hdxf, 0.5, mode, 0.05)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    efso(ne, offs, idx, rd, rl, hdxa, fcst, fcer, [0, 0, 1, 2, -1, -1], obsdep)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return f"obs_analysis {n} obs {1e3 * (t1 - t0):.1f} ms; efso {npts} points {1e3 * (t2 - t1):.1f} ms"


CASES = {"sweep_tc": lambda d: case_sweep(d, True), "sweep_simt": lambda d: case_sweep(d, False),
         "sweep_tc40": lambda d: case_sweep(d, True, shape=(64, 64, 40), nobs=62_500),
         "sweep_tc128": lambda dev: case_sweep(dev, True, ne=128), "search_700km": case_search_700km,
         "f64": case_f64, "l96": case_l96, "relax": case_relax, "largek": case_largek,
         "speedy_io": case_speedy_io, "obsope": case_obsope, "obs_space": case_obs_space,
         "largek_700km": case_largek_700km, "scale_obsope": case_scale_obsope}


def main():
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", choices=list(CASES), default=list(CASES))
    args = ap.parse_args()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    for name in args.only:
        print(f"{name}: {CASES[name](dev)}", flush=True)


if __name__ == "__main__":
    main()
