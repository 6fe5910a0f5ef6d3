"""Multi-rank decomposition of the sweep (letkf_gb300.shard) on CPU ranks over
gloo.  Every rank owns an interleaved share of the observations, exchanges
them once, keeps its tile's halo and analyses its tile's points; the oracle
sweep stands in for the per-rank GPU sweep.  The reassembled analysis,
inflation and local counts must equal the single-domain sweep bit for bit
(same local lists in the same order)."""
import os
import socket
import tempfile

import numpy as np
import pytest

from letkf_gb300 import shard
from letkf_gb300 import synthetic as S


def test_tiles_cover_the_grid_once():
    for world in (1, 2, 3, 4, 6, 8):
        px, py = shard.rank_grid(world)
        assert px * py == world and px >= py
        seen = np.zeros((20, 24), dtype=int)
        for r in range(world):
            i0, i1, j0, j1 = shard.tile_of(r, world, 24, 20)
            seen[j0 - 1:j1, i0 - 1:i1] += 1
        assert (seen == 1).all()
        pts = np.concatenate([shard.tile_points(shard.tile_of(r, world, 24, 20), 24, 20, 3) for r in range(world)])
        assert np.array_equal(np.sort(pts), np.arange(24 * 20 * 3))


def test_halo_contains_every_selected_observation():
    from oracle import oracle as O

    case = S.regional_case(3, nlon=24, nlat=20, nlev=3, ne=8, nobs=3000, sigma_obs=9.0e3,
                           with_grid_ensemble=False)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(24, 20, case["ri"], case["rj"])
    srt = {k: case[k][perm] for k in ("ri", "rj", "lev", "dat", "err", "cls")}
    n = perm.size
    so = O.ScaleObs(24, 20, grd, srt["ri"], srt["rj"], srt["lev"], srt["dat"], srt["err"], srt["cls"], np.zeros(n),
                    np.zeros(n), np.zeros(n), 1, 1, prm["dx"], prm["dy"], prm["dlon_zero"], prm["dlat_zero"],
                    prm["sigma_obs"], prm["sigma_obsv"])
    for world in (2, 4):
        for r in range(world):
            tile = shard.tile_of(r, world, 24, 20)
            keep = shard.halo_mask(srt["ri"], srt["rj"], tile, 24, 20, prm["dlon_zero"], prm["dlat_zero"])
            for p in shard.tile_points(tile, 24, 20, 3)[::7]:
                idx, _, _ = so.obs_local(case["pri"][p], case["prj"][p], case["prlev"][p])
                assert keep[idx].all()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    return S.regional_case(7, nlon=36, nlat=16, nlev=3, ne=8, nobs=3000, nvar=2, sigma_obs=4.0e3)


def _sweep(case, obs, pts):
    """Oracle SCALE sweep of the points `pts` with the observations `obs`."""
    from oracle import oracle as O

    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(case["nlon"], case["nlat"], obs["ri"], obs["rj"])
    s = {k: v[perm] for k, v in obs.items()}
    n = perm.size
    so = O.ScaleObs(case["nlon"], case["nlat"], grd, s["ri"], s["rj"], s["lev"], s["dat"], s["err"], s["cls"],
                    np.zeros(n), np.zeros(n), np.zeros(n), 1, 1, prm["dx"], prm["dy"], prm["dlon_zero"],
                    prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"])
    xb = case["xb"][:, pts, :]
    infl = np.full(pts.size, 1.02)
    return so.sweep(s["hdxf"], s["dep"], xb, case["pri"][pts], case["prj"][pts], case["prlev"][pts], infl,
                    nthreads=1)


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        case = _case()
        prm = S.scale_params(case)
        nobs = case["ri"].size
        uid = np.arange(nobs)
        mine = uid % world == rank
        local = {"uid": uid[mine], "ri": case["ri"][mine], "rj": case["rj"][mine], "lev": case["lev"][mine],
                 "dat": case["dat"][mine], "err": case["err"][mine], "cls": case["cls"][mine],
                 "hdxf": case["hdxf"][mine], "dep": case["dep"][mine]}
        tile = shard.tile_of(rank, world, case["nlon"], case["nlat"])
        halo = shard.exchange_obs(local, tile, case["nlon"], case["nlat"], prm["dlon_zero"], prm["dlat_zero"])
        assert np.all(np.diff(halo["uid"]) > 0)
        pts = shard.tile_points(tile, case["nlon"], case["nlat"], case["nlev"])
        obs = {k: v for k, v in halo.items() if k != "uid"}
        xa, infl, nobsl = _sweep(case, obs, pts)
        npts = case["pri"].size
        xa_all = shard.gather_points(xa, pts, npts)
        infl_all = shard.gather_points(infl, pts, npts)
        nobsl_all = shard.gather_points(nobsl, pts, npts)
        if rank == 0:
            np.savez(os.path.join(out_dir, f"w{world}.npz"), xa=xa_all, infl=infl_all, nobsl=nobsl_all,
                     nhalo=halo["uid"].size)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_sweep_equals_single_domain(world):
    import torch.multiprocessing as mp

    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_rank_main, args=(world, _free_port(), d), nprocs=world, join=True)
        got = np.load(os.path.join(d, f"w{world}.npz"))
        case = _case()
        obs = {k: case[k] for k in ("ri", "rj", "lev", "dat", "err", "cls", "hdxf", "dep")}
        xa, infl, nobsl = _sweep(case, obs, np.arange(case["pri"].size))
        assert int(got["nhalo"]) < case["ri"].size          # the halo is a strict subset
        assert (nobsl > 0).mean() > 0.5
        np.testing.assert_array_equal(got["nobsl"], nobsl)
        np.testing.assert_array_equal(got["infl"], infl)
        np.testing.assert_array_equal(got["xa"], xa)


# ------------------------------------------------------------ failure detection
def _guard_main(rank, world, port, sport, out_dir, mode):
    """Cycle 0 runs on every rank; then rank world-1 leaves (mode "leave":
    announces it; mode "vanish": just exits) between cycles, with no device
    work or collective in flight.  The others must learn of it in their
    guard before cycle 1's work and exit cleanly instead of hanging."""
    import datetime
    import json

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    store = dist.TCPStore("127.0.0.1", sport, world, is_master=(rank == 0),
                          timeout=datetime.timedelta(seconds=20))
    guard = shard.CycleGuard(store, rank, world, timeout=1.5)
    result = {"rank": rank}
    try:
        case = _case()
        prm = S.scale_params(case)
        tile = shard.tile_of(rank, world, case["nlon"], case["nlat"])
        guard.enter(0)
        nobs = case["ri"].size
        uid = np.arange(nobs)
        mine = uid % world == rank
        local = {"uid": uid[mine], "ri": case["ri"][mine], "rj": case["rj"][mine]}
        halo = shard.exchange_obs(local, tile, case["nlon"], case["nlat"], prm["dlon_zero"], prm["dlat_zero"])
        result["cycle0_halo"] = int(halo["uid"].size)
        if rank == world - 1:
            if mode == "leave":
                guard.leave()
            result["left"] = True
        else:
            try:
                guard.enter(1)
                result["cycle1"] = "entered"
            except shard.RankLost as e:
                result["cycle1"] = "rank lost"
                result["missing"] = e.missing
                result["announced"] = e.left
        store.set(f"done/r{rank}", "1")
        if rank == 0:  # the store's host stays until the others are done with it
            store.wait([f"done/r{r}" for r in range(world - 1)], datetime.timedelta(seconds=20))
    finally:
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump(result, f)
        dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["leave", "vanish"])
def test_ranks_learn_that_a_rank_left_between_cycles(mode):
    import json
    import time

    import torch.multiprocessing as mp

    world = 3
    with tempfile.TemporaryDirectory() as d:
        t0 = time.time()
        mp.spawn(_guard_main, args=(world, _free_port(), _free_port(), d, mode), nprocs=world, join=True)
        took = time.time() - t0
        res = [json.load(open(os.path.join(d, f"r{r}.json"))) for r in range(world)]
    assert res[world - 1].get("left")
    for r in range(world - 1):
        assert res[r]["cycle1"] == "rank lost", res[r]
        assert res[r]["missing"] == [world - 1]
        assert res[r]["announced"] == ([world - 1] if mode == "leave" else [])
        assert res[r]["cycle0_halo"] > 0
    assert took < 60
