"""RTPP / RTPS relaxation, relax_beta and the q spread clip of the SCALE driver
(scale/letkf/letkf_tools.f90:215-268,1182-1268) on the device, against the
reference formulas (oracle weight_rtpp / weight_rtps plus the driver's
composition written out in its operation order).  Tolerance 1e-12 relative."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _batch(rng, ne, npts):
    Ls = rng.integers(0, 60, npts)
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    n = max(int(offs[-1]), 1)
    rows = rng.standard_normal((n, ne))
    rows -= rows.mean(1, keepdims=True)
    rd = rng.uniform(0.3, 3.0, n)
    rl = rng.uniform(0.01, 1.0, n)
    d = rng.standard_normal(n)
    infl = rng.uniform(0.95, 1.2, npts)
    return O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True, want_pao=True, rdiag_wloc=True)


def _reference(xb, tr, tm, pa, mode, alpha, beta, q_var, q_max):
    """scale/letkf/letkf_tools.f90:215-268 for one point: xb [nv, ne] members,
    tr / pa [ne, ne] with tr[m][k] = trans(k, m) (column-major per point)."""
    nv, ne = xb.shape
    out = np.zeros_like(xb)
    infl_out = np.ones(nv)
    for v in range(nv):
        s = xb[v, 0]
        for m in range(1, ne):
            s = s + xb[v, m]
        mean = s / ne
        xp = xb[v] - mean
        b = beta[v]
        if b == 0.0:
            out[v] = mean + xp
            continue
        w = tr.T                          # w[k, m] = trans(k, m)
        if mode == 1:
            wr = O.weight_rtpp(w, alpha)
        elif mode == 2:
            wr, infl_out[v] = O.weight_rtps(w, pa.T, xp, alpha)
        else:
            wr = w
        for m in range(ne):
            a = mean
            for k in range(ne):
                t = (wr[k, m] + tm[k]) * b
                if k == m:
                    t = t + (1.0 - b)
                a = a + xp[k] * t
            out[v, m] = a
    if q_max > 0 and 0 <= q_var < nv:
        q = out[q_var]
        qm = q[0]
        for m in range(1, ne):
            qm = qm + q[m]
        qm = qm / ne
        sp = 0.0
        for m in range(ne):
            sp = sp + (q[m] - qm) * (q[m] - qm)
        sp = math.sqrt(sp / (ne - 1)) / qm
        if sp > q_max:
            out[q_var] = qm + (q - qm) * q_max / sp
    return out, infl_out


@pytest.mark.parametrize("ne,mode,alpha", [(20, 1, 0.5), (40, 2, 0.8), (24, 0, 0.0), (64, 2, 0.95)])
def test_relaxed_update_matches_reference(cuda, ne, mode, alpha):
    import torch

    from letkf_gb300.core import update_relax_f64

    rng = np.random.default_rng(ne + 7 * mode)
    npts, nv = 50, 3
    ref = _batch(rng, ne, npts)
    xb = rng.standard_normal((nv, npts, ne)) * 0.3 + 2.0
    xb[2] = np.abs(xb[2]) * 1e-3 + 5e-3          # a positive "q" whose spread the clip limits
    beta = rng.uniform(0, 1, (nv, npts))
    beta[:, ::5] = 1.0
    beta[:, 1::7] = 0.0
    q_max = 0.02
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    xa, infl = update_relax_f64(t(xb), t(ref["trans"]), t(ref["transm"]), t(ref["pao"]), mode=mode, alpha=alpha,
                                beta=t(beta), q_var=2, q_sprd_max=q_max)
    xa = xa.cpu().numpy()
    clipped = 0
    for p in range(npts):
        want, inf = _reference(xb[:, p], ref["trans"][p], ref["transm"][p], ref["pao"][p], mode, alpha, beta[:, p], 2,
                               q_max)
        scale = np.abs(want).max()
        assert np.abs(xa[:, p] - want).max() <= 1e-12 * scale, p
        if mode == 2:
            np.testing.assert_allclose(infl.cpu().numpy()[:, p], inf, rtol=1e-12)
        raw, _ = _reference(xb[:, p], ref["trans"][p], ref["transm"][p], ref["pao"][p], mode, alpha, beta[:, p], 2, 0.0)
        clipped += int(np.std(raw[2], ddof=1) / np.mean(raw[2]) > q_max)
    assert clipped > 5          # the clip was exercised


def test_relaxed_update_without_relaxation_equals_plain_update(cuda):
    import torch

    from letkf_gb300.core import update_f64, update_relax_f64

    rng = np.random.default_rng(3)
    ref = _batch(rng, 32, 40)
    xb = torch.as_tensor(rng.standard_normal((2, 40, 32)), device=cuda)
    tr = torch.as_tensor(ref["trans"], device=cuda)
    tm = torch.as_tensor(ref["transm"], device=cuda)
    a = update_f64(xb, tr, tm)
    b, _ = update_relax_f64(xb, tr, tm)
    assert torch.equal(a, b)


def test_relax_beta(cuda):
    import torch

    from letkf_gb300.core import relax_beta

    rng = np.random.default_rng(4)
    n = 500
    ri = rng.uniform(1, 60, n)
    rj = rng.uniform(1, 40, n)
    rlev = rng.uniform(5e3, 1e5, n)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=cuda)
    nv, q_lo, q_hi, top, bbw, dx, dy, nlong, nlatg, ih, jh = 6, 3, 4, 3.0e4, 20.0e3, 3.0e3, 3.0e3, 56, 36, 2, 2
    beta = relax_beta(t(ri), t(rj), t(rlev), nv, q_lo, q_hi, top, bbw, dx, dy, nlong, nlatg, ih, jh).cpu().numpy()
    for v in range(nv):
        for p in range(n):
            b = 1.0
            if rlev[p] < top and q_lo <= v <= q_hi:
                b = 0.0
            else:
                d = min(min(ri[p] - ih, nlong + ih + 1 - ri[p]) * dx, min(rj[p] - jh, nlatg + jh + 1 - rj[p]) * dy) / bbw
                if d < 1.0:
                    b = max(d, 0.0)
            assert beta[v, p] == b
    assert (beta == 0).any() and ((beta > 0) & (beta < 1)).any() and (beta == 1).any()
