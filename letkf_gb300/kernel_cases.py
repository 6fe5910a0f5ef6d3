"""Run every kernel of libletkf_gpu.so once on a profiling-size case.

    python -m letkf_gb300.kernel_cases [--only NAME ...]

Cases (seeded synthetic data, a few hundred MB on the device, larger than L2
where the kernel streams the ensemble):
  sweep_tc      tensor-core sweep of a 96x96x16 regional domain (147,456
                points, k = 64, 6 variables, 140,625 clustered obs) and its
                deferred-point pass
  sweep_simt    the same sweep on the SIMT kernel
  f64           FP64 plain form of 8,192 of those points: search (count,
                fill), gather, core_f64, update_f64
  l96           Lorenz-96 ring of 100,000 variables, k = 32: departures,
                selection, mixed core, update
  relax         RTPS update with relax_beta weights of 50,000 points, k = 64
  largek        large-ensemble core of 512 points, k = 512, 100-900 local obs
                each, and the FP32 update of 6 variables
Used for the ncu summaries under profiles/; prints one line per case.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def _regional():
    from .workload import RegionalWorkload

    return RegionalWorkload(5, 96, 96, 16, 64, 140_625, 6)


def case_sweep(dev, tc):
    import torch

    from .sweep import OPT_TENSOR_CORES, PREC_MIXED, Sweep

    wl = _regional()
    hdxf, dep, dat = wl.obs_torch(dev)
    xb = wl.background_torch(dev)
    ri, rj, plev = wl.points()
    sw = Sweep(64, wl.nvar, wl.nlon, wl.nlat, wl.npts, wl.params, precision=PREC_MIXED)
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


CASES = {"sweep_tc": lambda d: case_sweep(d, True), "sweep_simt": lambda d: case_sweep(d, False),
         "f64": case_f64, "l96": case_l96, "relax": case_relax, "largek": case_largek}


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
