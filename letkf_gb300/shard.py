"""Domain decomposition of the SCALE-style sweep over ranks (one GPU each).

The reference splits the grid into 2-D process tiles and gives every process
the observations of its tile plus a halo of the localisation cut-off
(scale/letkf/letkf_obs.f90:886-985; scale/common/common_mpi_scale.f90).  Here
the same split feeds independent ``Sweep`` handles:

* ``rank_grid`` / ``tile_of``: near-square process grid, balanced i/j ranges;
* ``tile_points``: the rank's grid points (every level) in global numbering;
* ``halo_mask``: observations whose bucket cell (CEILING(r - 0.5) clamped to
  the domain, scale/letkf/letkf_obs.f90:751-763) lies within the cells any
  point of the tile can reach, [floor(i0 - dlon_zero), ceil(i1 + dlon_zero)];
* ``exchange_obs``: the one exchange step per cycle, an all-gather of every
  rank's observation records and obs-space ensemble rows, filtered to the halo
  and put back in global observation order.

Each rank keeps the global grid coordinates, so its bucket sort sees the
global observation order restricted to its halo: every point's local list
(content and order) is the one the single-domain sweep builds.  There is no
communication inside the analysis; ``gather_points`` reassembles a field.
"""
from __future__ import annotations

import math

import numpy as np


def rank_grid(world):
    """(px, py) with px * py == world, px >= py, as square as possible."""
    py = int(math.isqrt(world))
    while world % py:
        py -= 1
    return world // py, py


def _split(n, parts, k):
    base, rem = divmod(n, parts)
    lo = k * base + min(k, rem)
    return lo + 1, lo + base + (1 if k < rem else 0)  # 1-based inclusive


def tile_of(rank, world, nlon, nlat):
    """(i0, i1, j0, j1): 1-based inclusive grid ranges of `rank`'s tile."""
    px, py = rank_grid(world)
    if px > nlon or py > nlat:
        raise ValueError(f"{world} ranks do not tile a {nlon} x {nlat} grid")
    ri, rj = rank % px, rank // px
    i0, i1 = _split(nlon, px, ri)
    j0, j1 = _split(nlat, py, rj)
    return i0, i1, j0, j1


def tile_points(tile, nlon, nlat, nlev):
    """Global point ids p = lev * nlon * nlat + (j - 1) * nlon + (i - 1) of the
    tile, ordered by (lev, j, i)."""
    i0, i1, j0, j1 = tile
    i = np.arange(i0, i1 + 1)
    j = np.arange(j0, j1 + 1)
    lev = np.arange(nlev)
    p = lev[:, None, None] * (nlon * nlat) + (j[None, :, None] - 1) * nlon + (i[None, None, :] - 1)
    return p.ravel().astype(np.int64)


def obs_cells(ri, rj, nlon, nlat):
    """Bucket cell of each observation (scale/letkf/letkf_obs.f90:751-763)."""
    ci = np.clip(np.ceil(np.asarray(ri, dtype=np.float64) - 0.5).astype(np.int64), 1, nlon)
    cj = np.clip(np.ceil(np.asarray(rj, dtype=np.float64) - 0.5).astype(np.int64), 1, nlat)
    return ci, cj


def halo_mask(ri, rj, tile, nlon, nlat, dlon_zero, dlat_zero):
    """Observations a point of the tile can select (a superset by at most the
    cut-off's fractional cell)."""
    i0, i1, j0, j1 = tile
    ci, cj = obs_cells(ri, rj, nlon, nlat)
    ilo = max(int(math.floor(i0 - dlon_zero)), 1)
    ihi = min(int(math.ceil(i1 + dlon_zero)), nlon)
    jlo = max(int(math.floor(j0 - dlat_zero)), 1)
    jhi = min(int(math.ceil(j1 + dlat_zero)), nlat)
    return (ci >= ilo) & (ci <= ihi) & (cj >= jlo) & (cj <= jhi)


def exchange_obs(local, tile, nlon, nlat, dlon_zero, dlat_zero, group=None):
    """All-gather every rank's observations and keep this tile's halo.

    local: dict of numpy arrays with one entry per local observation; it must
    hold "uid" (global observation number, defines the order), "ri" and "rj";
    2-D arrays (e.g. the obs-space ensemble rows) are gathered row-wise.
    Returns the same keys for the halo observations, in uid order."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    allobs = {k: np.concatenate([p[k] for p in parts]) for k in local}
    order = np.argsort(allobs["uid"], kind="stable")
    allobs = {k: v[order] for k, v in allobs.items()}
    keep = halo_mask(allobs["ri"], allobs["rj"], tile, nlon, nlat, dlon_zero, dlat_zero)
    return {k: v[keep] for k, v in allobs.items()}


def gather_points(values, points, npts_total, group=None):
    """Reassemble a per-point field on every rank: values [..., n_local, ...]
    with the point axis second to last when 3-D ([nv, n, ne]) or first when
    1-D ([n]); points: this rank's global point ids."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(points), np.asarray(values)), group=group)
    v0 = parts[0][1]
    if v0.ndim == 1:
        out = np.zeros(npts_total, dtype=v0.dtype)
        for pts, v in parts:
            out[pts] = v
    else:
        out = np.zeros((v0.shape[0], npts_total) + v0.shape[2:], dtype=v0.dtype)
        for pts, v in parts:
            out[:, pts] = v
    return out


OBS_KEYS = ("ri", "rj", "lev", "dat", "err", "dep", "cls")


def tile_sweep(tile, nlon, nlat, nlev, pts, obs, params, ne, nv, precision, halo=True):
    """The analysis handle of one tile: its grid points (every level, global
    coordinates) and the observations of its halo.

    pts: (ri, rj, rlev) of all nlon * nlat * nlev points in global numbering;
    obs: dict with OBS_KEYS and "hdxf" [nobs, ne] in global observation order
    (halo=True keeps the tile's halo; False: obs is that halo already, e.g. from
    exchange_obs).  Returns (points, handle, observations kept)."""
    from .sweep import Sweep

    points = tile_points(tile, nlon, nlat, nlev)
    keep = (halo_mask(obs["ri"], obs["rj"], tile, nlon, nlat, params["dlon_zero"], params["dlat_zero"]) if halo
            else np.ones(len(obs["ri"]), dtype=bool))
    sw = Sweep(ne, nv, nlon, nlat, points.size, params, precision=precision)
    sw.set_points(pts[0][points], pts[1][points], pts[2][points], tile=4)
    sw.set_obs(*(np.asarray(obs[k])[keep] for k in OBS_KEYS), np.asarray(obs["hdxf"])[keep])
    return points, sw, int(keep.sum())


class RankLost(RuntimeError):
    """A rank of the decomposition left or did not arrive for a cycle."""

    def __init__(self, step, missing, left):
        self.step, self.missing, self.left = step, sorted(missing), sorted(left)
        super().__init__(f"cycle {step}: ranks {self.missing} did not arrive (left: {self.left})")


class CycleGuard:
    """Host-side liveness check between the cycles of a decomposed analysis.

    The reference has no failure detection: an error anywhere stops the MPI
    job (STOP 2 in common/common_mtx.f90:61-64,75-78, STOP 99 in
    scale/letkf/letkf_tools.f90:1159-1163).  Here every rank calls
    ``enter(step)`` before it launches the step's work: it marks itself as
    present in a key-value store (a ``torch.distributed`` TCPStore, hosted by a
    rank that stays, normally rank 0) and waits, at most ``timeout`` seconds,
    for the other ranks' marks.  A rank that leaves between cycles calls
    ``leave()``; the others then learn of it at once, and of a rank that simply
    stops arriving after the timeout.  Either way ``enter`` raises
    ``RankLost`` before any device work or collective of that step is issued,
    so no rank waits in a collective for a peer that is gone."""

    def __init__(self, store, rank, world, timeout=2.0, prefix="letkf/guard"):
        self.store, self.rank, self.world = store, int(rank), int(world)
        self.timeout, self.prefix = float(timeout), prefix

    def _key(self, what, r):
        return f"{self.prefix}/{what}/r{r}"

    def _left(self):
        return [r for r in range(self.world) if r != self.rank and self.store.check([self._key("left", r)])]

    def enter(self, step):
        import datetime

        self.store.set(self._key(f"step{step}", self.rank), "1")
        left = self._left()
        if left:
            raise RankLost(step, left, left)
        keys = [self._key(f"step{step}", r) for r in range(self.world)]
        try:
            self.store.wait(keys, datetime.timedelta(seconds=self.timeout))
        except RuntimeError:  # the store's timeout error
            missing = [r for r in range(self.world) if not self.store.check([keys[r]])]
            raise RankLost(step, missing, self._left()) from None

    def leave(self):
        self.store.set(self._key("left", self.rank), "1")


__all__ = ["rank_grid", "tile_of", "tile_points", "obs_cells", "halo_mask", "exchange_obs", "gather_points",
           "CycleGuard", "RankLost"]
