"""Obs-space clients of the core (GFS driver) on the device against the oracle:
the analysis ensemble at observation locations (gfs/letkf/letkf_tools.f90:
466-497, with weight_RTPP :959-970) and the observation sensitivity EFSO
(gfs/letkf/letkf_tools.f90:547-679).  Tolerance 1e-12 relative (EFSO sums
over points with atomics: rounding-level order differences)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, dev, dt=None):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt or torch.float64, device=dev)


@pytest.mark.parametrize("ne,alpha", [(20, 0.0), (40, 0.3), (64, 0.5)])
def test_obs_analysis_matches_oracle(cuda, ne, alpha):
    import torch

    from letkf_gb300.core import obs_analysis

    rng = np.random.default_rng(ne)
    n = 60
    Ls = rng.integers(0, 40, n)
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    rows = rng.standard_normal((max(int(offs[-1]), 1), ne))
    rows -= rows.mean(1, keepdims=True)
    rd = rng.uniform(0.3, 3.0, rows.shape[0])
    rl = rng.uniform(0.05, 1.0, rows.shape[0])
    d = rng.standard_normal(rows.shape[0])
    ref = O.letkf_core_batch(ne, offs, rows, rd, rl, d, np.full(n, 1.05))   # trans with wbar merged
    hdxf = rng.standard_normal((n, ne)) * 1e-3
    hdxf -= hdxf.mean(1, keepdims=True)
    ybar = rng.uniform(4e-3, 6e-3, n)
    mode = rng.integers(0, 3, n).astype(np.int32)
    q_max = 0.05
    anal, mean = obs_analysis(_t(ref["trans"], cuda), _t(ybar, cuda), _t(hdxf, cuda), alpha,
                              _t(mode, cuda, torch.int32), q_max)
    anal, mean = anal.cpu().numpy(), mean.cpu().numpy()
    clipped = 0
    for p in range(n):
        w = ref["trans"][p].T                       # w[k, m] = trans(k, m)
        if alpha != 0.0:
            w = O.weight_rtpp(w, alpha)
        a, m = O.obs_analysis(w, ybar[p], hdxf[p], int(mode[p]), q_max)
        np.testing.assert_allclose(anal[p], a, rtol=1e-12, atol=1e-18)
        assert abs(mean[p] - m) <= 1e-12 * abs(m)
        if mode[p] == 2:
            raw, rm = O.obs_analysis(w, ybar[p], hdxf[p], 0)
            clipped += int(np.std(raw, ddof=1) / rm > q_max)
    assert clipped > 0


def test_efso_matches_oracle(cuda):
    from letkf_gb300.core import efso

    rng = np.random.default_rng(7)
    ne, npts, nobs, nv = 32, 300, 500, 5
    Ls = rng.integers(0, 50, npts)
    Ls[3] = 0
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    idx = rng.integers(0, nobs, int(offs[-1])).astype(np.int32)     # obs shared by many points
    rdiag = rng.uniform(0.5, 2.0, idx.size)
    rloc = rng.uniform(0.0, 1.0, idx.size)
    hdxa = rng.standard_normal((nobs, ne))
    fcst = rng.standard_normal((nv, npts, ne))
    fcer = rng.standard_normal((nv, npts))
    term = [0, 0, 1, 2, -1]                     # u, v -> 1; t -> 2; q -> 3; one variable without a term
    obsdep = rng.standard_normal(nobs)
    dj_ref, os_ref = O.efso(ne, offs, idx, rdiag, rloc, hdxa, fcst, fcer, term, obsdep)
    import torch

    dj, os_ = efso(ne, _t(offs, cuda, torch.int64), _t(idx, cuda, torch.int32), _t(rdiag, cuda), _t(rloc, cuda),
                   _t(hdxa, cuda), _t(fcst, cuda), _t(fcer, cuda), term, _t(obsdep, cuda))
    scale = np.abs(dj_ref).max()
    assert np.abs(dj.cpu().numpy() - dj_ref).max() <= 1e-12 * scale
    assert np.abs(os_.cpu().numpy() - os_ref).max() <= 1e-12 * np.abs(os_ref).max()
    assert (np.abs(dj_ref) > 0).sum() > nobs // 2
