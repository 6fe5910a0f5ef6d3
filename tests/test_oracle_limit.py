"""The oracle's MAX_NOBS_PER_GRID selection against a second, independent
restatement written here in plain Python.

scale/letkf/letkf_tools.f90:1063-1128 keeps, per (element uid, obs type)
group, M slots ordered by rdiag through an insertion sort (a new observation
goes after every kept one with rdiag <= its own; when the group is full the
last one leaves and its slot number is reused) and :1141-1156 emits the
groups type-major, each in slot order.  The Python version below replays
that on the oracle's own unlimited list, so it checks the C restatement's
bookkeeping (slot numbers, eviction, emission order) without sharing code
with it."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O


def _limit_by_insertion(idx, rloc, rdiag, grp, M):
    state = {}
    for ob, rl, rd in zip(idx, rloc, rdiag):
        g = int(grp[ob])
        st = state.setdefault(g, {"n": 0, "order": [], "slot": {}})
        order = st["order"]  # slot numbers sorted by rdiag (insertion order among equals)
        if st["n"] >= M and rd >= st["slot"][order[-1]][2]:
            continue
        pos = len(order)
        for s, sl in enumerate(order):
            if rd < st["slot"][sl][2]:
                pos = s
                break
        if st["n"] < M:
            st["n"] += 1
            sl = st["n"]
        else:
            sl = order.pop()  # the last-priority observation leaves; its slot is reused
            if pos > len(order):
                pos = len(order)
        order.insert(pos, sl)
        st["slot"][sl] = (ob, rl, rd)
    out = []
    for g in sorted(state):
        st = state[g]
        for sl in range(1, st["n"] + 1):
            out.append(st["slot"][sl])
    if not out:
        return np.zeros(0, np.int32), np.zeros(0), np.zeros(0)
    o = np.array([x[0] for x in out], np.int32)
    return o, np.array([x[1] for x in out]), np.array([x[2] for x in out])


@pytest.mark.parametrize("M", [1, 2, 5, 16])
def test_oracle_limit_equals_insertion_replay(M):
    case = S.regional_case(11, nlon=16, nlat=14, nlev=3, ne=8, nobs=1500, with_grid_ensemble=False)
    prm = S.scale_params(case)
    perm, grd = O.scale_sort_obs(16, 14, case["ri"], case["rj"])
    n = perm.size
    rng = np.random.default_rng(M)
    nid, ntyp = 3, 4
    uid = rng.integers(0, nid, n)
    typ = rng.integers(0, ntyp, n)
    # many equal errors and some equal rdiag values make ties common
    err = case["err"][perm]
    args = (16, 14, grd, case["ri"][perm], case["rj"][perm], case["lev"][perm], case["dat"][perm], err,
            case["cls"][perm], uid, typ, np.zeros(n), nid, ntyp, prm["dx"], prm["dy"], prm["dlon_zero"],
            prm["dlat_zero"], prm["sigma_obs"], prm["sigma_obsv"])
    full = O.ScaleObs(*args)
    lim = O.ScaleObs(*args, max_nobs_per_grid=M)
    grp = typ * nid + uid
    acted = 0
    for p in range(0, case["pri"].size, 5):
        pt = (case["pri"][p], case["prj"][p], case["prlev"][p])
        i0, rl0, rd0 = full.obs_local(*pt)
        i1, rl1, rd1 = lim.obs_local(*pt)
        ie, rle, rde = _limit_by_insertion(i0, rl0, rd0, grp, M)
        np.testing.assert_array_equal(i1, ie)
        np.testing.assert_array_equal(rd1, rde)
        np.testing.assert_array_equal(rl1, rle)
        acted += i1.size < i0.size
    assert acted > 0


def test_oracle_limit_keeps_the_earlier_of_equal_rdiag():
    """Equal rdiag: the observation met first stays (letkf_tools.f90:1063-1066
    skips a new one whose rdiag is >= the largest kept)."""
    idx = np.arange(5, dtype=np.int32)
    rd = np.array([2.0, 1.0, 2.0, 2.0, 0.5])
    ie, _, rde = _limit_by_insertion(idx, rd * 0 + 1, rd, np.zeros(5, np.int64), 2)
    # after 0 (2.0), 1 (1.0): full; 2 and 3 (2.0) skipped; 4 (0.5) evicts 0 and takes slot 1
    np.testing.assert_array_equal(ie, [4, 1])
    np.testing.assert_array_equal(rde, [0.5, 1.0])
