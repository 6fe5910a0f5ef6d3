#!/usr/bin/env python
"""Benchmark: LETKF grid-point analyses per second on one GB300 (per rank).

Workload (per rank): the regional configuration -- 256 x 256 x 40 grid at
3 km, 6 variables updated per point, k = 64 members stored FP32, 1e6
clustered observations (0-2000 local obs per point).  One step = one full
analysis sweep: local search, letkf_core and the update of every grid point
(scale/letkf/letkf_tools.f90:38-476 with relax_beta = 1), mixed precision,
one persistent CUDA launch (and the Jacobi pass over any deferred points).

  value     device-resident throughput (points/s), CUDA events on the launch
            stream, inputs (4 GB background ensemble) larger than L2
  e2e       the same sweep through the public C ABI with pinned host buffers:
            per step H2D of the observations (sorted on the device), then
            letkf_sweep_run_host: H2D of the background, the sweep and D2H of
            the analysis in pieces whose copies overlap the analysis
  fp64      the FP64 plain form on a strided subset of the same points
  cpu_baseline  the CPU oracle (restatement of the reference path) on a
            bounded sample of points with all host threads
  error     analysis mean / spread RMS error of the mixed form against the
            FP64 oracle on that sample, relative to the background spread

``--impl reference`` times the CPU oracle alone (the reference arm).
``--decompose`` runs one regional domain as 2-D process tiles with their
halo observations (one exchange_obs all-gather per rank before the timed
region; ``--tiles K`` runs K tiles in turn on one GPU and compares the
reassembled analysis with the single-domain sweep bit for bit).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-point analyses/s"
UNIT = "points/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nlon", type=int, default=256)
    ap.add_argument("--nlat", type=int, default=256)
    ap.add_argument("--nlev", type=int, default=40)
    ap.add_argument("--ne", type=int, default=64)
    ap.add_argument("--nobs", type=int, default=1_000_000)
    ap.add_argument("--nv", type=int, default=6)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--fp64-stride", type=int, default=64, help="FP64 plain form on every n-th point")
    ap.add_argument("--no-extras", action="store_true", help="skip e2e, fp64, cpu baseline (profiling runs)")
    ap.add_argument("--e2e-chunks", type=int, default=16,
                    help="pieces of the e2e run whose copies overlap the analysis (1: copy in, run, copy out)")
    ap.add_argument("--eig", default="newton-schulz", choices=["newton-schulz", "jacobi"],
                    help="transform of the mixed form")
    ap.add_argument("--tc", type=int, default=1, choices=[0, 1],
                    help="1: Gram and Newton-Schulz on the tcgen05 tensor cores (ne <= 64)")
    ap.add_argument("--tc-ns", type=int, default=None, help="tensor-core Newton-Schulz iterations before the FP32 ones")
    ap.add_argument("--tc-scaling", type=int, default=1, choices=[0, 1],
                    help="1: spectrum-scaled tensor-core Newton-Schulz steps; 0: plain steps")
    ap.add_argument("--tc-tol", type=int, default=None, help="tensor-core phase exit at ||ZY-I||^2 < 10^-v")
    ap.add_argument("--polish-tol", type=int, default=None, help="FP32 polish last step at ||ZAZ/s-I||^2 < 10^-v")
    ap.add_argument("--polish-probe", type=int, default=None,
                    help="skip the FP32 polish where the anchored probe residual is below 10^-v (0: always polish)")
    ap.add_argument("--ns-cond", type=int, default=None,
                    help="Newton-Schulz only where the spectrum bound s/c < 10^v (0: no bound)")
    ap.add_argument("--decompose", action="store_true",
                    help="one regional domain split into 2-D tiles (one per rank, or --tiles on one GPU in turn), "
                         "each tile's halo observations exchanged once before the timed region")
    ap.add_argument("--tiles", type=int, default=None, help="tiles of --decompose on one GPU (default: the ranks)")
    ap.add_argument("--col-unit", type=int, default=None,
                    help="order positions a tensor-core CTA takes at a time with the column cache (0: off)")
    ap.add_argument("--tune-points", type=int, default=32768,
                    help="run the autotuner on this many points before timing (0: the options given)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-largek", action="store_true", help="skip the large-ensemble measurement")
    ap.add_argument("--no-configs", action="store_true", help="skip the Lorenz-96 and SPEEDY-grid parity lines")
    ap.add_argument("--largek-points", type=int, default=4096,
                    help="sampled points of the large-ensemble sweep at 60 km")
    ap.add_argument("--largek-700-points", type=int, default=64,
                    help="sampled points of the large-ensemble sweep at the stated 700 km")
    ap.add_argument("--serve-requests", type=int, default=500, help="requests of the serving measurement")
    ap.add_argument("--serve-slots", type=int, default=3, help="jobs on the device at once")
    ap.add_argument("--serve-load", type=float, default=0.7,
                    help="offered load: arrival rate x mean single-job service time")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def algorithmic_flops(nobsl, ne, nv):
    """Per sweep: sum over points of 2 L k^2 + 2 L k + 9 k^3 + 2 k^3 + 4 k^2
    (letkf_core; L > 0) + 2 V k^2 (update)."""
    L = nobsl.astype(np.float64)
    k = float(ne)
    core = np.where(L > 0, 2 * L * k * k + 2 * L * k + 11 * k ** 3 + 4 * k * k, 0.0)
    return float(core.sum() + nobsl.size * 2 * nv * k * k)


def algorithmic_bytes(npts, nv, ne, nobs):
    """Per sweep: ensemble read + write (FP32), obs ensemble + records once, FP64 mean."""
    return float(npts * nv * ne * 8 + nobs * ne * 4 + nobs * 48 + npts * nv * 8)


def load_traffic(kernel):
    p = os.path.join(ROOT, "profiles", f"{kernel.split('<')[0]}_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except OSError:
        return None


# --------------------------------------------------------------- CPU oracle
def cpu_oracle_setup(wl, obs):
    from oracle import oracle as O

    hdxf, dep, dat = obs
    perm, grd = O.scale_sort_obs(wl.nlon, wl.nlat, wl.ri, wl.rj)
    n = perm.size
    prm = wl.params
    so = O.ScaleObs(wl.nlon, wl.nlat, grd, wl.ri[perm], wl.rj[perm], wl.lev[perm], dat[perm], wl.err[perm],
                    wl.cls[perm], np.zeros(n), np.zeros(n), np.zeros(n), 1, 1, prm["dx"], prm["dy"], prm["dlon_zero"],
                    prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"])
    return so, np.ascontiguousarray(hdxf[perm], dtype=np.float64), np.ascontiguousarray(dep[perm])


def cpu_oracle_run(wl, so, hd, dp, idx, nthreads, infl=1.0, timed=False):
    """The oracle's SCALE grid loop on the points idx.  timed=True runs the
    -O3 build the CPU baseline is timed with; the parity build otherwise."""
    i, j, p = wl.points(idx)
    xb = wl.background_numpy(idx).astype(np.float64)
    t = time.perf_counter()
    xa, inf, nl = so.sweep(hd, dp, xb, i, j, p, np.full(idx.size, infl), nthreads=nthreads, timed=timed)
    return time.perf_counter() - t, xb, xa, inf, nl


def sample_points(wl, n, seed=1):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(wl.npts, size=min(n, wl.npts), replace=False))


def run_reference(args, rank, world):
    """Reference arm: the CPU oracle of the path on the host cores."""
    if rank != 0:
        return None
    from letkf_gb300.workload import RegionalWorkload

    wl = RegionalWorkload(args.seed, args.nlon, args.nlat, args.nlev, args.ne, args.nobs, args.nv)
    obs = wl.obs_numpy()
    so, hd, dp = cpu_oracle_setup(wl, obs)
    nthreads = os.cpu_count() or 1
    # size each step's sample from a probe so that a step takes about 1 s
    probe = sample_points(wl, 64, seed=99)
    dt, *_ = cpu_oracle_run(wl, so, hd, dp, probe, nthreads, timed=True)
    per_step = int(max(64, min(wl.npts, 64 * 1.0 / max(dt, 1e-6))))
    times, npts_done = [], 0
    for s in range(args.warmup + args.steps):
        idx = sample_points(wl, per_step, seed=1000 + s)
        dt, *_ = cpu_oracle_run(wl, so, hd, dp, idx, nthreads, timed=True)
        if s >= args.warmup:
            times.append(dt)
            npts_done += idx.size
    tot = sum(times)
    val = npts_done / tot
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_block(args, wl, form=REF_FORM),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": nthreads, "kind": "port", "build": CPU_BUILD,
                             "sample": f"{per_step} random grid points per step of the {wl.npts}-point sweep"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


GPU_FORM = ("mixed (FP32 ensemble, Gram and transform; FP64 member sums and mean-increment accumulation, "
            "analysis mean carried as an FP32 hi + lo pair)")
REF_FORM = ("FP64 plain form: the oracle's restatement of letkf_core, EISPACK rs and the SCALE obs_local, "
            "OpenMP over points (scale/letkf/letkf_tools.f90:175)")
CPU_BUILD = "gcc -O3 -ffp-contract=fast -fopenmp (oracle/_build/liboracle_timed.so; no -march=native)"


def config_block(args, wl, form=GPU_FORM):
    return {"workload": f"regional {args.nlon}x{args.nlat}x{args.nlev} (3 km), {args.nv} vars, k={args.ne}, "
                        f"{args.nobs} clustered obs, sigma_h={wl.sigma_obs:.0f} m, sigma_v={wl.sigma_obsv} ln p",
            "points_per_sweep": wl.npts, "ensemble": args.ne, "variables": args.nv, "observations": args.nobs,
            "local_obs": "0-2000 per point", "form": form,
            "l2": "inputs larger than L2 (background ensemble %.1f GB)" % (wl.npts * args.nv * args.ne * 4 / 1e9),
            "parallelism": f"dp{args.gpus} (independent domains per GPU)"}


# ------------------------------------------------------------------ serving
def run_serving(args, dev):
    """Poisson stream of analysis requests over resident domains of mixed sizes
    and ensemble sizes through the continuous-batching server: four regional
    128x128x20 grids (2 variables, 250k clustered obs, k = 20, 32, 64, 128,
    mixed precision) and three Lorenz-96 rings (N = 40, 1e4, 1e5; k = 20, 32,
    64; mixed core with the FP64 update).  The arrival rate is the offered load over the mean service
    time of a request alone.  Latency = submit -> analysis on the host."""
    import torch

    from letkf_gb300.serve import LETKF_PENDING, PREC_MIXED, Server
    from letkf_gb300.workload import RegionalWorkload

    # every host buffer a job reads or writes is page-locked
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    specs = []
    for i, ne in enumerate((20, 32, 64, 128)):
        wl = RegionalWorkload(100 + i, 128, 128, 20, ne, 250_000, 2)
        hdxf, dep, dat = wl.obs_torch(dev)  # host arrays (device evaluation)
        xb = wl.background_torch(dev)
        ri, rj, plev = wl.points()
        specs.append(dict(kind="sweep", name=f"regional 128x128x20 k={ne}", domain=i, pts=(ri, rj, plev),
                          params=wl.params, obs=dict(ri=pin(wl.ri), rj=pin(wl.rj), lev=pin(wl.lev), dat=pin(dat),
                                                     err=pin(wl.err), cls=pin(wl.cls.astype(np.int32))),
                          hdxf=pin(hdxf), dep=pin(dep), xb=pin(xb.cpu().numpy()), npts=wl.npts, wl=wl,
                          obs_np=(hdxf, dep, dat)))
        del xb
    for j, (nx, ne) in enumerate(((40, 20), (10_000, 32), (100_000, 64))):
        rng = np.random.default_rng(200 + j)
        xf = 8.0 + rng.standard_normal((nx, ne))
        m = xf.sum(1) / ne
        y = m + rng.standard_normal(nx)
        specs.append(dict(kind="l96", name=f"lorenz96 N={nx} k={ne}", domain=10 + j, xf=pin(xf),
                          hdxf=pin(xf - m[:, None]), dep=pin(y - m), cell=pin(np.arange(1, nx + 1, dtype=np.int32)),
                          npts=nx))

    pools = {}  # page-locked output buffers per domain, reused once a job's result has been collected

    def out_buf(sp):
        free = pools.setdefault(sp["name"], [])
        if free:
            return free.pop()
        like = sp["xf"] if sp["kind"] == "l96" else sp["xb"]
        return torch.empty(like.shape, dtype=torch.from_numpy(like[:0]).dtype, pin_memory=True).numpy()

    def submit(srv, sp, precision=PREC_MIXED, domain=None, xa=None):
        dom = sp["domain"] if domain is None else domain
        if sp["kind"] == "l96":
            return srv.submit_l96(sp["xf"], sp["hdxf"], sp["dep"], sp["cell"], precision=precision, domain=dom,
                                  xa=xa)
        ri, rj, plev = sp["pts"]
        return srv.submit_sweep(ri, rj, plev, sp["params"], 128, 128, sp["obs"], sp["hdxf"], sp["dep"], sp["xb"],
                                precision=PREC_MIXED, domain=dom, xa=xa)

    with Server(nslots=args.serve_slots) as srv:
        alone, first = [], []
        for sp in specs:  # each domain once, alone: service time, and the domain becomes resident
            t0 = time.perf_counter()
            j = submit(srv, sp, xa=out_buf(sp))
            srv.wait(j)
            alone.append(time.perf_counter() - t0)
            first.append(j.xa)
        mean_service = statistics.mean(alone)
        rate = args.serve_load / mean_service
        rng = np.random.default_rng(7)
        gaps = rng.exponential(1.0 / rate, args.serve_requests)
        picks = rng.integers(0, len(specs), args.serve_requests)
        jobs, pending = [], []

        def collect(block):
            # results collected (the latency is the server's submit -> done);
            # their output buffers return to the domain's pool
            keep = []
            for k, j in pending:
                r = srv.wait(j, timeout=None if block else 0.0)
                if r["status"] == LETKF_PENDING:
                    keep.append((k, j))
                else:
                    pools[specs[k]["name"]].append(j.xa)
                    j.xa = None
            pending[:] = keep

        t0 = time.perf_counter()
        t_next = 0.0
        for g, k in zip(gaps, picks):
            t_next += g
            collect(False)
            dt = t0 + t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            j = submit(srv, specs[k], xa=out_buf(specs[k]))
            jobs.append((k, j))
            pending.append((k, j))
        collect(True)
        st = srv.stats()
    lat = np.array([j.result["latency_s"] for _, j in jobs])
    span = max(j.result["t_done"] for _, j in jobs) - min(j.result["t_submit"] for _, j in jobs)
    points = sum(specs[k]["npts"] for k, _ in jobs)
    errors = serving_errors(specs, first, submit)
    per = {}
    for k, j in jobs:
        per.setdefault(specs[k]["name"], []).append(j.result["latency_s"])
    per_domain = {n: {"requests": len(v), "p50_ms": round(float(np.percentile(v, 50)) * 1e3, 1),
                      "p99_ms": round(float(np.percentile(v, 99)) * 1e3, 1)} for n, v in per.items()}
    return {"requests": int(args.serve_requests), "slots": int(args.serve_slots), "offered_load": args.serve_load,
            "arrival_rate_hz": rate, "p50_latency_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_latency_ms": float(np.percentile(lat, 99) * 1e3), "points_per_s": points / span,
            "jobs_per_s": len(jobs) / span,
            "service_alone_ms": {sp["name"]: round(a * 1e3, 2) for sp, a in zip(specs, alone)},
            "resident_domains": int(st["resident_domains"]), "peak_device_bytes": int(st["peak_bytes"]),
            "per_domain": per_domain, "error_vs_fp64_oracle": errors,
            "host_buffers": "page-locked (copied in the timed latency)"}


def serving_errors(specs, first, submit):
    """Analysis-mean and perturbation RMS error, over the background spread,
    of each domain's first served analysis: regional domains against the
    oracle's SCALE grid loop on 512 sampled points; Lorenz-96 rings against
    the same job in the FP64 plain form (within 1e-10 of the oracle by the
    tests)."""
    from letkf_gb300.serve import PREC_F64, Server

    out = {}
    nthreads = os.cpu_count() or 1
    for sp, xa in zip(specs, first):
        if sp["kind"] == "sweep":
            wl = sp["wl"]
            so, hd, dp = cpu_oracle_setup(wl, sp["obs_np"])
            idx = sample_points(wl, 512, seed=3)
            _, xb_s, xa_ref, _, _ = cpu_oracle_run(wl, so, hd, dp, idx, nthreads)
            got = xa[:, idx, :].astype(np.float64)
            xp = xb_s - xb_s.mean(-1, keepdims=True)
            points = int(idx.size)
            ref_name = "oracle"
        else:
            with Server(nslots=1) as s64:
                j = submit(s64, sp, precision=PREC_F64, domain=-1)
                s64.wait(j)
                xa_ref = j.xa[None]
            got = xa.astype(np.float64)[None]
            xb = np.asarray(sp["xf"], dtype=np.float64)[None]
            xp = xb - xb.mean(-1, keepdims=True)
            points = int(sp["npts"])
            ref_name = "FP64 plain form"
        spread = np.sqrt((xp ** 2).sum(-1) / (xp.shape[-1] - 1)).mean()
        pert = lambda x: x - x.mean(-1, keepdims=True)
        em = float(np.sqrt(np.mean((got.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread)
        ep = float(np.sqrt(np.mean((pert(got) - pert(xa_ref)) ** 2)) / spread)
        out[sp["name"]] = {"analysis_mean_rms_over_spread": em, "perturbation_rms_over_spread": ep,
                           "points": points, "reference": ref_name}
    return out


# --------------------------------------------------------------- large k
def run_configs(args, dev):
    """The two small configurations beside the headline: Lorenz-96 (N = 40, k = 20,
    40 identity obs, xlocal = 3, inflation 1.05) in the FP64 plain and mixed forms,
    and the SPEEDY grid (96x48x7, k = 40, radiosonde-like obs) in the FP64 plain
    form, each against the oracle (L96: every point; SPEEDY: every 61st point of
    u, v, t, q) with throughput from CUDA events."""
    import torch

    from letkf_gb300 import synthetic as S
    from letkf_gb300.core import l96_obs_cell
    from letkf_gb300.drivers import l96_letkf, speedy_letkf, speedy_sort_obs
    from oracle import oracle as O

    out = {}
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    ev = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    # ---- Lorenz-96 ----
    c = S.l96_case(11)
    xf = c["xf"].T.copy()
    nx, ne = xf.shape
    xm = xf.sum(1) / ne
    ref = np.zeros_like(xf)
    for ix in range(1, nx + 1):
        idx, rl = O.l96_select(c["h"], ix, 3.0)
        r = O.letkf_core(c["hdxf"][idx], np.full(idx.size, c["obserr"] ** 2), rl, c["dep"][idx], 1.05)
        ref[ix - 1] = xm[ix - 1] + (xf[ix - 1] - xm[ix - 1]) @ r["trans"]
    spread = np.sqrt(((xf - xm[:, None]) ** 2).sum(1) / (ne - 1)).mean()
    h = t(c["h"])
    cell = l96_obs_cell(h)
    l96 = {"workload": "Lorenz-96 N=40, k=20, 40 obs, xlocal=3, inflation 1.05"}
    for prec in ("f64", "mixed"):
        xft = t(xf)
        hxf = h @ xft
        y = t(c["y"])
        l96_letkf(xft, hxf, y, cell, obserr=float(c["obserr"]), precision=prec)
        torch.cuda.synchronize()
        e0, e1 = ev()
        e0.record()
        reps = 20
        for _ in range(reps):
            xa, _ = l96_letkf(xft, hxf, y, cell, obserr=float(c["obserr"]), precision=prec)
        e1.record()
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3 / reps
        err = float(np.abs(xa.cpu().numpy() - ref).max() / spread)
        l96[prec] = {"max_abs_error_over_spread": err, "ms_per_analysis": 1e3 * dt, "points_per_s": nx / dt}
    out["lorenz96"] = l96
    # ---- SPEEDY grid, FP64 plain form ----
    c = S.speedy_case(4)
    perm, grd = speedy_sort_obs(c["lon"], c["lat"], c["olon"], c["olat"])
    srt = {k: c[k][perm] for k in ("elm", "olon", "olat", "olev", "odat", "oerr")}
    hdxf, dep = c["hdxf"][perm], c["dep"][perm]
    grid = {"lon": t(c["lon"]), "lat": t(c["lat"]), "nobsgrd": t(grd, torch.int32)}
    obs = {"elm": t(srt["elm"]), "lon": t(srt["olon"]), "lat": t(srt["olat"]), "lev": t(srt["olev"]),
           "dat": t(srt["odat"]), "err": t(srt["oerr"])}
    params = (c["dist_zero"], c["dist_zerov"], c["dlat_zero"], c["sigma_obs"], c["sigma_obsv"])
    nv3d, nlev, ne, nij = c["gues3d"].shape
    var_local = np.ones((nv3d, 7))
    args_ = (grid, obs, t(hdxf), t(dep), t(c["gues3d"]), t(c["logpfm"]), t(c["dlon_zero"]), params, var_local)
    infl = torch.full((nv3d, nlev, nij), 1.1, dtype=torch.float64, device=dev)
    speedy_letkf(*args_, infl.clone())
    torch.cuda.synchronize()
    e0, e1 = ev()
    e0.record()
    anal3d, _ = speedy_letkf(*args_, infl)
    e1.record()
    torch.cuda.synchronize()
    dt = e0.elapsed_time(e1) / 1e3
    anal3d = anal3d.cpu().numpy()
    so = O.SpeedyObs(c["lon"], c["lat"], grd, srt["elm"], srt["olon"], srt["olat"], srt["olev"], srt["odat"],
                     srt["oerr"], c["dist_zero"], c["dist_zerov"], c["dlat_zero"], c["sigma_obs"], c["sigma_obsv"],
                     var_local[0])
    g3 = c["gues3d"]
    worst, npts = 0.0, 0
    sp = np.sqrt(((g3 - g3.mean(2, keepdims=True)) ** 2).sum(2) / (ne - 1)).mean()
    for p in range(0, nlev * nij, 61):
        ilev, ij = divmod(p, nij)
        ri, rl, rd = so.obs_local(c["glon"][ij], c["glat"][ij], c["dlon_zero"][ij], ilev + 1, c["logpfm"][ilev, ij])
        r = O.letkf_core(hdxf[ri] if ri.size else np.zeros((1, ne)), rd if ri.size else np.ones(1),
                         rl if ri.size else np.ones(1), dep[ri] if ri.size else np.zeros(1), 1.1, nobsl=ri.size)
        for n in range(nv3d):
            xb = g3[n, ilev, :, ij]
            m = xb[0]
            for k in range(1, ne):
                m = m + xb[k]
            m = m / ne
            w = np.eye(ne) if (n == 3 and ilev + 1 >= 5) else r["trans"]
            worst = max(worst, float(np.abs(anal3d[n, ilev, :, ij] - (m + (xb - m) @ w)).max() / sp))
        npts += 1
    out["speedy"] = {"workload": f"SPEEDY grid 96x48x7, k=40, {srt['elm'].size} radiosonde-like obs, u/v/t/q, FP64 plain form",
                     "points_per_s": nlev * nij / dt, "ms_per_analysis": 1e3 * dt,
                     "max_abs_error_over_spread": worst, "checked_points": npts, "target": 1e-10}
    return out


def run_largek(args, dev):
    """Large-ensemble configuration on samples of its points: 360x181x32
    global grid, 6 variables, k = 512 members stored BF16 (FP32 mean + BF16
    perturbations for the background and the analysis; BF16 obs-space
    perturbations), 3e6 observations, SPEEDY lat/lon search.  One step =
    search (count + fill), the large-k core over the search's index lists
    (no packed copies of the rows) and the BF16-storage update of the 6
    variables.  Two localisations: the stated 700 km (about 7e4 local
    observations per point) and 60 km (O(1e2-1e3), the range the hot-path
    scope names), each with its error against the FP64 oracle on a subset of
    the sampled points (same stored inputs)."""
    import torch

    from letkf_gb300.core import (core_batch_largek_indexed, search_speedy, update_bf16, update_mixed)
    from letkf_gb300.workload import GlobalWorkload
    from oracle import oracle as O

    wl = GlobalWorkload(21)
    hdxf, dep, dat = wl.obs_torch(dev)
    hdxf16 = hdxf.to(torch.bfloat16)
    del hdxf
    dep32 = dep.to(torch.float32)
    f = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    grid = {"lon": f(wl.lon), "lat": f(wl.lat), "nobsgrd": torch.as_tensor(wl.nobsgrd, dtype=torch.int32, device=dev)}
    obs = {"elm": f(wl.elm), "lon": f(wl.olon), "lat": f(wl.olat), "lev": f(wl.olev), "dat": dat, "err": f(wl.err)}
    vl = np.ones(7)
    out = {"storage": "background and analysis: FP32 mean + BF16 perturbations; obs-space perturbations BF16",
           "workload": f"global {wl.nlon}x{wl.nlat}x{wl.nlev}, {wl.nvar} vars, k={wl.ne}, {wl.nobs} obs, "
                       f"sigma_v={wl.sigma_obsv} ln p (SPEEDY lat/lon search)"}
    for sigma, npts_s, nerr in ((700.0e3, args.largek_700_points, 8), (60.0e3, args.largek_points, 256)):
        # (at 700 km the mixed-precision transform does not certify and the core's FP64 pass answers)
        params = wl.search_params(sigma)
        rng = np.random.default_rng(5)
        idx = np.sort(rng.choice(wl.npts, npts_s, replace=False))
        lon, lat, dlon, ilev, lnp = wl.points(idx, params)
        pts = {"lon": f(lon), "lat": f(lat), "dlon_zero": f(dlon), "ilev": torch.as_tensor(ilev, device=dev),
               "logpfm": f(lnp)}
        xb = wl.background_torch(dev, idx)
        xmean = xb.double().mean(-1).to(torch.float32)
        xpert16 = (xb - xmean[..., None]).to(torch.bfloat16)
        del xb
        infl0 = torch.full((idx.size,), 1.05, dtype=torch.float64, device=dev)

        def step():
            offs, oi, rloc, rdiag = search_speedy(grid, obs, pts, params, vl)
            infl = infl0.clone()
            core = core_batch_largek_indexed(wl.ne, offs, oi, hdxf16, dep32, rdiag.to(torch.float32),
                                             rloc.to(torch.float32), infl, want_transm=True)
            am, ap = update_bf16(xmean, xpert16, core["trans"], core["transm"])
            return offs, oi, rloc, rdiag, core, am, ap

        step()
        torch.cuda.synchronize()
        # three timed steps, the median reported (one step is a short, single sample)
        times = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            offs, oi, rloc, rdiag, core, am, ap = step()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        t = statistics.median(times)
        nl = np.diff(offs.cpu().numpy())
        status = core["status"].cpu().numpy()
        # FP64 oracle (the same stored BF16 rows, FP32 weights) on a subset
        sub = np.arange(0, idx.size, max(1, idx.size // nerr))[:nerr]
        o = offs.cpu().numpy()
        sel = np.concatenate([np.arange(o[p], o[p + 1]) for p in sub]) if nl[sub].sum() else np.zeros(0, np.int64)
        obs_rows = oi.cpu().numpy()[sel]
        R = hdxf16[torch.as_tensor(obs_rows, device=dev, dtype=torch.int64)].double().cpu().numpy() if sel.size \
            else np.zeros((1, wl.ne))
        rd_ = rdiag.to(torch.float32).double().cpu().numpy()[sel] if sel.size else np.ones(1)
        rl_ = rloc.to(torch.float32).double().cpu().numpy()[sel] if sel.size else np.ones(1)
        d_ = dep32.double().cpu().numpy()[obs_rows] if sel.size else np.zeros(1)
        so = np.concatenate([[0], np.cumsum(nl[sub])]).astype(np.int64)
        tc0 = time.perf_counter()
        ref = O.letkf_core_batch(wl.ne, so, R, rd_, rl_, d_, np.full(sub.size, 1.05), want_transm=True)
        t_oracle = time.perf_counter() - tc0
        xs = torch.as_tensor(sub, device=dev)
        x64 = (xmean[:, xs, None].double() + xpert16[:, xs, :].double()).cpu().numpy()
        xp = x64 - x64.mean(-1, keepdims=True)
        want = x64.mean(-1, keepdims=True) + np.einsum("vpk,pmk->vpm", xp, ref["trans"] + ref["transm"][:, None, :])
        spread = np.sqrt((xp ** 2).sum(-1) / (wl.ne - 1)).mean()
        pert = lambda x: x - x.mean(-1, keepdims=True)
        got_mean = am[:, xs].double().cpu().numpy()
        em = float(np.sqrt(np.mean((got_mean - want.mean(-1)) ** 2)) / spread)
        got_p16 = ap[:, xs, :].double().cpu().numpy()
        ep16 = float(np.sqrt(np.mean((got_p16 - pert(want)) ** 2)) / spread)
        # the same transforms through the FP32 update: the computation's own error
        xa32 = update_mixed((xmean[:, xs, None] + xpert16[:, xs, :].float()).contiguous(), core["trans"][xs],
                            core["transm"][xs]).double().cpu().numpy()
        ep32 = float(np.sqrt(np.mean((pert(xa32) - pert(want)) ** 2)) / spread)
        key = f"sigma_{sigma / 1e3:.0f}km"
        out[key] = {"sigma_h_m": sigma, "sample_points": int(idx.size), "value": idx.size / t, "unit": UNIT,
                    "ms_per_sample": t * 1e3, "ms_per_sample_runs": [round(x * 1e3, 1) for x in times],
                    "step": "search + large-k core over the index lists (tensor-core Gram and Newton-Schulz; FP64 "
                            "pass for points that do not certify) + BF16-storage update, CUDA events",
                    "local_obs": {"min": int(nl.min()), "mean": float(nl.mean()), "p50": float(np.median(nl)),
                                  "max": int(nl.max())},
                    "status_ok": int((status == 0).sum()),
                    "status_counts": {str(int(k)): int(v) for k, v in zip(*np.unique(status, return_counts=True))},
                    "error_vs_fp64_oracle": {"analysis_mean_rms_over_spread": em,
                                             "perturbation_rms_over_spread_bf16_stored": ep16,
                                             "perturbation_rms_over_spread_fp32_update": ep32,
                                             "points": int(sub.size), "oracle_seconds": round(t_oracle, 1),
                                             "target": 1e-4}}
        del offs, oi, rloc, rdiag, core, am, ap, xpert16, xmean
        torch.cuda.empty_cache()
    return out


def check_lists(sw, so, wl, idx, cap, stream, nthreads, chunk=16384):
    """The fused sweep's accepted observation lists (selection probe) against
    the oracle's obs_local on the sample points idx: every index in order
    must be equal; the largest relative rloc difference (FP32 on the device)
    is reported."""
    perm = so_perm(wl)
    entries, worst, equal = 0, 0.0, True
    for c0 in range(0, idx.size, chunk):
        pts = idx[c0:c0 + chunk].astype(np.int32)
        sw.set_probe(pts, cap)
        sw.run(stream.cuda_stream)
        cnt, obs, rl = sw.probe()
        i, j, p = wl.points(pts)
        ocnt, oidx, orl = so.obs_local_batch(i, j, p, cap=cap, nthreads=nthreads)
        equal &= bool((cnt == ocnt).all())
        ok = np.arange(cap)[None, :] < np.minimum(ocnt, cap)[:, None]
        mapped = np.where(ok, perm[np.maximum(oidx, 0)], -1)
        equal &= bool((np.where(ok, obs, -1) == mapped).all())
        if ok.any():
            worst = max(worst, float(np.max(np.abs(rl[ok] - orl[ok]) / orl[ok])))
        entries += int(ok.sum())
    sw.set_probe(np.zeros(0, np.int32), 1)
    return {"equal": equal, "points": int(idx.size), "entries": entries, "rloc_max_rel": worst}


def so_perm(wl):
    from oracle import oracle as O

    perm, _ = O.scale_sort_obs(wl.nlon, wl.nlat, wl.ri, wl.rj)
    return perm


# ----------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, dist):
    import torch

    from letkf_gb300 import lib as L
    from letkf_gb300.sweep import (OPT_COLUMN_UNIT, OPT_EIGENSOLVER, OPT_NS_COND, OPT_POLISH_PROBE, OPT_POLISH_TOL,
                                   OPT_TC_NS_ITERS, OPT_TC_NS_SCALING, OPT_TC_NS_TOL, OPT_TENSOR_CORES, PREC_F64,
                                   PREC_MIXED, Sweep)
    from letkf_gb300.workload import RegionalWorkload

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    wl = RegionalWorkload(args.seed + rank, args.nlon, args.nlat, args.nlev, args.ne, args.nobs, args.nv)
    hdxf, dep, dat = wl.obs_torch(dev)
    xb = wl.background_torch(dev)
    ri, rj, plev = wl.points()
    sw = Sweep(args.ne, args.nv, args.nlon, args.nlat, wl.npts, wl.params, precision=PREC_MIXED)
    sw.set_points(ri, rj, plev, tile=4)
    sw.set_obs(wl.ri, wl.rj, wl.lev, dat, wl.err, dep, wl.cls, hdxf)
    sw.set_option(OPT_EIGENSOLVER, 0 if args.eig == "newton-schulz" else 1)
    sw.set_option(OPT_TENSOR_CORES, args.tc)
    if args.tc_ns is not None:
        sw.set_option(OPT_TC_NS_ITERS, args.tc_ns)
    sw.set_option(OPT_TC_NS_SCALING, args.tc_scaling)
    if args.tc_tol is not None:
        sw.set_option(OPT_TC_NS_TOL, args.tc_tol)
    if args.polish_tol is not None:
        sw.set_option(OPT_POLISH_TOL, args.polish_tol)
    if args.polish_probe is not None:
        sw.set_option(OPT_POLISH_PROBE, args.polish_probe)
    if args.ns_cond is not None:
        sw.set_option(OPT_NS_COND, args.ns_cond)
    if args.col_unit is not None:
        sw.set_option(OPT_COLUMN_UNIT, args.col_unit)
    sw.set_background_device(xb.data_ptr())
    infl0 = np.ones(wl.npts)
    sw.set_inflation(infl0)
    tuned = sw.autotune(args.tune_points) if args.tune_points > 0 else None
    stream = torch.cuda.Stream(device=dev)
    for _ in range(args.warmup):
        sw.run(stream.cuda_stream)
    torch.cuda.synchronize()
    dg = sw.diagnostics()
    nobsl = dg["nobsl"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = L.launch_count()
    with ClockSampler(dev.index) as clk:
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for _ in range(args.steps):
                sw.run(stream.cuda_stream)
            ev1.record(stream)
        torch.cuda.synchronize()
    launches = L.launch_count() - n0
    t = ev0.elapsed_time(ev1) / 1e3
    if dist:
        tt = torch.tensor([t], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    value = world * wl.npts * args.steps / t
    ms = 1e3 * t / args.steps
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded smooth random fields, clustered obs)",
           "config": config_block(args, wl), "gpu_launches": int(launches), "clocks": clk.summary()}
    # roofline of the dominant kernel (the deferred-point pass is < 0.01 % of the step)
    tc_on = bool(args.tc and args.ne <= 64 and args.eig == "newton-schulz")
    if tuned is not None:
        tc_on = tuned["tensor_cores"]
    if tc_on:
        kernel = "sweep_tc_kernel" if args.ne <= 64 else "sweep_tc128_kernel"
    else:
        kernel = f"sweep_mixed_kernel<{32 if args.ne <= 32 else 64 if args.ne <= 64 else 128}>"
    peaks, src = measured_peaks()
    flops = algorithmic_flops(nobsl, args.ne, args.nv)
    ach = flops / (t / args.steps) / 1e12
    pk = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    trf = load_traffic(kernel)
    traffic = None
    if trf and trf.get("per_point_bytes"):
        traffic = trf["per_point_bytes"] * wl.npts
    out["roofline"] = {"bound": "tensor", "kernel": kernel, "achieved": ach, "peak": pk,
                       "unit": "TFLOP/s", "frac": ach / pk, "traffic": traffic,
                       "peak_source": f"bf16 dense sustained ({src})",
                       "algorithmic_flops_per_launch": flops,
                       "algorithmic_bytes_per_launch": algorithmic_bytes(wl.npts, args.nv, args.ne, args.nobs)}
    clkmhz = out["clocks"]["sm_mhz"] or 1900.0
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = nsm * 128 * 2 * clkmhz * 1e6 / 1e12
    out["roofline_fp32_simt"] = {"achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                                 "peak_source": f"{nsm} SMs x 128 FP32 lanes x 2 x median SM clock under load"}
    nl = nobsl.astype(np.float64)
    out["local_obs"] = {"min": int(nl.min()), "mean": float(nl.mean()), "p50": float(np.median(nl)),
                        "p99": float(np.percentile(nl, 99)), "max": int(nl.max()), "zero_frac": float((nl == 0).mean())}
    out["transform"] = {"method": args.eig, "tensor_cores": tc_on,
                        "scaled_steps": bool(args.tc_scaling), "autotune": tuned,
                        "deferred_to_jacobi": sw.deferred(),
                        "iterations_mean": float(dg["sweeps"][nobsl > 0].mean()) if (nobsl > 0).any() else 0.0,
                        "iterations_max": int(dg["sweeps"].max())}
    if args.no_extras:
        return out, sw
    # ---- e2e: host buffers through the C ABI ----
    xb_host = torch.empty(xb.shape, dtype=torch.float32, pin_memory=True)
    xb_host.copy_(xb)
    xa_host = torch.empty_like(xb_host, pin_memory=True)
    obs_bytes = args.nobs * (6 * 8 + 4 + args.ne * 4)
    # the step's observation records in pinned host memory, as the background
    pin = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).pin_memory().numpy()
    obs_host = [pin(x, np.float64) for x in (wl.ri, wl.rj, wl.lev, dat, wl.err, dep)]
    obs_host += [pin(wl.cls, np.int32), pin(hdxf, np.float32)]
    e2e_steps = max(2, min(args.steps, 5))
    # one untimed step: the piece plan of the host-buffer run is built once per handle
    sw.set_obs(*obs_host)
    sw.run_host(xb_host.data_ptr(), xa_host.data_ptr(), args.e2e_chunks, stream.cuda_stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    step_ms = []
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        sw.set_obs(*obs_host)
        sw.run_host(xb_host.data_ptr(), xa_host.data_ptr(), args.e2e_chunks, stream.cuda_stream)
        step_ms.append(round(1e3 * (time.perf_counter() - ts), 1))
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    if dist:
        tt = torch.tensor([te], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        te = float(tt.item())
    out["e2e"] = {"value": world * wl.npts * e2e_steps / te, "unit": UNIT, "steps": e2e_steps, "step_ms": step_ms,
                  "chunks": args.e2e_chunks,
                  "h2d_bytes_per_step": int(xb.numel() * 4 + obs_bytes), "d2h_bytes_per_step": int(xb.numel() * 4)}
    if rank != 0:
        return out, sw
    # ---- error vs the FP64 oracle on a sample, from a fresh inflation field ----
    sw.set_background_device(xb.data_ptr())
    sw.set_inflation(infl0)
    sw.run(stream.cuda_stream)
    torch.cuda.synchronize()
    xa = sw.analysis()
    so, hd, dp = cpu_oracle_setup(wl, (hdxf, dep, dat))
    nthreads = os.cpu_count() or 1
    probe = sample_points(wl, 64, seed=99)
    dtp, *_ = cpu_oracle_run(wl, so, hd, dp, probe, nthreads)
    nsample = int(max(256, min(131072, 64 * args.cpu_seconds / max(dtp, 1e-6))))
    idx = sample_points(wl, nsample, seed=7)
    # the reference answer from the parity build, the CPU figure from the -O3 build
    dtc_parity, xb_s, xa_ref, inf_ref, nl_ref = cpu_oracle_run(wl, so, hd, dp, idx, nthreads)
    dtc, *_ = cpu_oracle_run(wl, so, hd, dp, idx, nthreads, timed=True)
    out["cpu_baseline"] = {"value": idx.size / dtc, "unit": UNIT, "cores": nthreads, "kind": "port",
                           "build": CPU_BUILD, "parity_build_value": idx.size / dtc_parity,
                           "sample": f"{idx.size} random grid points of the {wl.npts}-point sweep "
                                     f"({dtc:.1f} s, OpenMP dynamic over points)"}
    xg = xa[:, idx, :].astype(np.float64)
    spread = np.sqrt(((xb_s - xb_s.mean(-1, keepdims=True)) ** 2).sum(-1) / (args.ne - 1)).mean()
    em = float(np.sqrt(np.mean((xg.mean(-1) - xa_ref.mean(-1)) ** 2)) / spread)
    pert = lambda x: x - x.mean(-1, keepdims=True)
    ep = float(np.sqrt(np.mean((pert(xg) - pert(xa_ref)) ** 2)) / spread)
    sa = lambda x: np.sqrt((pert(x) ** 2).sum(-1) / (args.ne - 1))
    es = float(np.sqrt(np.mean((sa(xg) - sa(xa_ref)) ** 2)) / spread)
    dgi = sw.diagnostics()
    lists = check_lists(sw, so, wl, idx, int(nl_ref.max()) + 1, stream, nthreads)
    out["error_vs_fp64_oracle"] = {"analysis_mean_rms_over_spread": em, "perturbation_rms_over_spread": ep,
                                   "analysis_spread_rms_over_spread": es,
                                   "nobsl_bit_exact": bool((dgi["nobsl"][idx] == nl_ref).all()),
                                   "lists_bit_exact": lists["equal"], "lists_checked": lists,
                                   "infl_max_rel": float(np.max(np.abs(dgi["infl"][idx] - inf_ref) / inf_ref)),
                                   "sample_points": int(idx.size), "target": 1e-4}
    # ---- FP64 plain form on a strided subset ----
    sub = np.arange(0, wl.npts, args.fp64_stride)
    si, sj, sp = wl.points(sub)
    s64 = Sweep(args.ne, args.nv, args.nlon, args.nlat, sub.size, wl.params, precision=PREC_F64)
    s64.set_points(si, sj, sp, tile=0)
    s64.set_obs(wl.ri, wl.rj, wl.lev, dat, wl.err, dep, wl.cls, hdxf.astype(np.float64))
    s64.set_background(xb[:, torch.as_tensor(sub, device=dev), :].double().cpu().numpy())
    s64.set_inflation(np.ones(sub.size))
    s64.run()
    torch.cuda.synchronize()
    s64.set_inflation(np.ones(sub.size))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    s64.run(torch.cuda.current_stream().cuda_stream)
    e1.record()
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3
    v64 = sub.size / t64
    out["fp64_plain"] = {"value": v64, "unit": UNIT, "sample": f"every {args.fp64_stride}th point ({sub.size} points)",
                         "mixed_over_fp64": (value / world) / v64}
    s64.close()
    if not args.no_serving:
        out["serving"] = run_serving(args, dev)
    if not args.no_largek:
        out["large_k"] = run_largek(args, dev)
    if not args.no_configs:
        out["configs"] = run_configs(args, dev)
    return out, sw


# ------------------------------------------------------- domain decomposition
def run_decompose(args, rank, world, dist):
    """One regional domain split into 2-D process tiles (shard.tile_of), as
    the reference's SCALE decomposition (scale/letkf/letkf_obs.f90:886-985).
    With N ranks each rank owns every N-th observation, one exchange_obs
    all-gather before the timed region gives each tile its halo, and each
    rank times its tile's sweep (max over ranks).  On one GPU, --tiles K runs
    the K tiles in turn as one step and compares the reassembled analysis
    with the single-domain sweep's, bit for bit.  value = the domain's points
    per step / step time."""
    import torch

    from letkf_gb300 import lib as L
    from letkf_gb300.shard import exchange_obs, rank_grid, tile_of, tile_sweep
    from letkf_gb300.sweep import PREC_MIXED, Sweep
    from letkf_gb300.workload import RegionalWorkload

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    wl = RegionalWorkload(args.seed, args.nlon, args.nlat, args.nlev, args.ne, args.nobs, args.nv)
    hdxf, dep, dat = wl.obs_torch(dev)
    xb = wl.background_torch(dev)
    pts = wl.points()
    obs = {"ri": wl.ri, "rj": wl.rj, "lev": wl.lev, "dat": dat, "err": wl.err, "dep": dep, "cls": wl.cls,
           "hdxf": hdxf}
    ntiles = world if world > 1 else (args.tiles or 1)
    px, py = rank_grid(ntiles)
    mine = [rank] if world > 1 else list(range(ntiles))
    t0 = time.perf_counter()
    parts = []
    for k in mine:
        tile = tile_of(k, ntiles, args.nlon, args.nlat)
        if world > 1:
            own = np.arange(wl.nobs) % world == rank
            local = {key: np.asarray(v)[own] for key, v in obs.items()}
            local["uid"] = np.nonzero(own)[0]
            halo = exchange_obs(local, tile, args.nlon, args.nlat, wl.params["dlon_zero"], wl.params["dlat_zero"])
            points, sw, nobs_t = tile_sweep(tile, args.nlon, args.nlat, args.nlev, pts, halo, wl.params, args.ne,
                                            args.nv, PREC_MIXED, halo=False)
        else:
            points, sw, nobs_t = tile_sweep(tile, args.nlon, args.nlat, args.nlev, pts, obs, wl.params, args.ne,
                                            args.nv, PREC_MIXED)
        xbt = xb[:, torch.as_tensor(points, device=dev), :].contiguous()
        torch.cuda.current_stream().synchronize()
        sw.set_background_device(xbt.data_ptr())
        sw.set_inflation(np.ones(points.size))
        parts.append({"tile": tile, "points": points, "sw": sw, "xb": xbt, "obs": nobs_t})
    t_setup = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    for _ in range(args.warmup):
        for pt in parts:
            pt["sw"].run(stream.cuda_stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = L.launch_count()
    with ClockSampler(dev.index) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            for pt in parts:
                pt["sw"].run(stream.cuda_stream)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = L.launch_count() - n0
    t = ev0.elapsed_time(ev1) / 1e3
    if dist:
        tt = torch.tensor([t], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    cfg = config_block(args, wl)
    cfg["parallelism"] = (f"{ntiles} tiles ({px} x {py}) over {world} rank(s), halo exchange before the timed "
                          f"region" + ("" if world > 1 else ", tiles in turn on one GPU"))
    out = {"metric": METRIC, "value": wl.npts * args.steps / t, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
           "scaling": "strong", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded smooth random fields, clustered obs)", "config": cfg,
           "gpu_launches": int(launches), "clocks": clk.summary(),
           "decompose": {"tiles": ntiles, "grid": [px, py], "setup_s": round(t_setup, 1),
                         "tiles_here": [{"tile": list(map(int, pt["tile"])), "points": int(pt["points"].size),
                                         "halo_obs": pt["obs"]} for pt in parts]}}
    if world == 1:
        # the reassembled analysis against the single-domain sweep's
        xa = np.zeros((args.nv, wl.npts, args.ne), np.float32)
        for pt in parts:
            pt["sw"].set_inflation(np.ones(pt["points"].size))
            pt["sw"].run(stream.cuda_stream)
            xa[:, pt["points"]] = pt["sw"].analysis()
        one = Sweep(args.ne, args.nv, args.nlon, args.nlat, wl.npts, wl.params, precision=PREC_MIXED)
        one.set_points(*pts, tile=4)
        one.set_obs(wl.ri, wl.rj, wl.lev, dat, wl.err, dep, wl.cls, hdxf)
        one.set_background_device(xb.data_ptr())
        one.set_inflation(np.ones(wl.npts))
        one.run(stream.cuda_stream)
        xa1 = one.analysis()
        one.close()
        out["decompose"]["equal_to_single_domain"] = bool(np.array_equal(xa, xa1))
        out["decompose"]["max_abs_diff"] = float(np.abs(xa - xa1).max())
        out["decompose"]["nonfinite"] = [int((~np.isfinite(xa)).sum()), int((~np.isfinite(xa1)).sum())]
        bad = np.nonzero(~np.isfinite(xa1).all(axis=(0, 2)))[0]
        out["decompose"]["nonfinite_points_single"] = bad[:20].tolist()
        bad = np.nonzero(~np.isfinite(xa).all(axis=(0, 2)))[0]
        out["decompose"]["nonfinite_points_tiles"] = bad[:20].tolist()
    for pt in parts:
        pt["sw"].close()
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist

        backend = "gloo" if args.impl == "reference" else "nccl"
        if args.impl != "reference":
            import torch

            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        tdist.init_process_group(backend)
        dist = tdist
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.decompose:
        line = run_decompose(args, rank, world, dist)
    else:
        line, sw = run_gpu(args, rank, world, dist)
        sw.close()
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
