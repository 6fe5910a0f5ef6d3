"""Large-ensemble core (ne > 128: HBM-resident matrices, tensor-core Gram and
Newton-Schulz) against the FP64 oracle.  Bars: transform and mean weights
within 1e-4 of the largest transform entry, inflation within 1e-5 relative,
and the analysis (update_mixed) within 1e-4 of the background spread."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _batch(rng, ne, Ls):
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    n = max(int(offs[-1]), 1)
    rows = rng.standard_normal((n, ne)).astype(np.float32).astype(np.float64)
    rows -= rows.mean(1, keepdims=True)
    rows = rows.astype(np.float32).astype(np.float64)
    rd = rng.uniform(0.3, 3.0, n).astype(np.float32).astype(np.float64)
    rl = rng.uniform(0.01, 1.0, n).astype(np.float32).astype(np.float64)
    d = rng.standard_normal(n).astype(np.float32).astype(np.float64)
    infl = rng.uniform(0.95, 1.3, len(Ls))
    return offs, rows, rd, rl, d, infl


@pytest.mark.parametrize("ne,wloc", [(160, False), (256, True), (512, False)])
def test_largek_core_matches_oracle(cuda, ne, wloc):
    import torch

    from letkf_gb300.core import core_batch_largek, update_mixed

    rng = np.random.default_rng(ne)
    Ls = [0, 1, 7, 64, 300, 700, 150, 2, 512, 90, 1000, 33]
    offs, rows, rd, rl, d, infl = _batch(rng, ne, Ls)
    ref = O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True, rdiag_wloc=wloc, minfl=1.0)
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_largek(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(d), pinf, want_transm=True,
                            rdiag_wloc=wloc, minfl=1.0)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    tr = out["trans"].cpu().numpy().astype(np.float64)
    tm = out["transm"].cpu().numpy().astype(np.float64)
    for p in range(len(Ls)):
        scale = np.abs(ref["trans"][p]).max()
        assert np.abs(tr[p] - ref["trans"][p]).max() <= 1e-4 * scale, (p, Ls[p])
        if Ls[p]:
            assert np.abs(tm[p] - ref["transm"][p]).max() <= 1e-4 * scale, (p, Ls[p])
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-5)
    # analysis through the FP32 update, 4 variables
    nv = 4
    xb = (rng.standard_normal((nv, len(Ls), ne)) * 0.5 + 3.0).astype(np.float32)
    xa = update_mixed(t(xb), out["trans"], out["transm"]).cpu().numpy().astype(np.float64)
    x64 = xb.astype(np.float64)
    xp = x64 - x64.mean(-1, keepdims=True)
    want = x64.mean(-1, keepdims=True) + np.einsum("vpk,pmk->vpm", xp, ref["trans"] + ref["transm"][:, None, :])
    spread = np.sqrt((xp ** 2).sum(-1) / (ne - 1)).mean()
    err = np.sqrt(np.mean((xa.mean(-1) - want.mean(-1)) ** 2)) / spread
    errp = np.sqrt(np.mean(((xa - xa.mean(-1, keepdims=True)) - (want - want.mean(-1, keepdims=True))) ** 2)) / spread
    assert err < 1e-4 and errp < 1e-4, (err, errp)


def test_largek_special_points(cuda):
    """No observations: sqrt(infl) I and infl unchanged; negative inflation
    (no minfl clamp): LETKF_ERR_CAPACITY with the identity."""
    import torch

    from letkf_gb300.core import core_batch_largek
    from letkf_gb300.lib import LETKF_ERR_CAPACITY

    rng = np.random.default_rng(1)
    ne = 200
    offs, rows, rd, rl, d, infl = _batch(rng, ne, [0, 40, 40])
    infl[:] = [0.5, -1.0, 1.1]
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_largek(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(d), pinf, want_transm=True)
    st = out["status"].cpu().numpy()
    tr = out["trans"].cpu().numpy()
    assert st[0] == 0 and st[1] == LETKF_ERR_CAPACITY and st[2] == 0
    np.testing.assert_allclose(tr[0], np.sqrt(0.5) * np.eye(ne), rtol=1e-6)
    np.testing.assert_array_equal(tr[1], np.eye(ne))
    assert pinf.cpu().numpy()[0] == 0.5
    ref = O.letkf_core_batch(ne, offs[2:] - offs[2], rows[offs[2]:], rd[offs[2]:], rl[offs[2]:], d[offs[2]:],
                             infl[2:], want_transm=True)
    assert np.abs(tr[2] - ref["trans"][0]).max() <= 1e-4 * np.abs(ref["trans"][0]).max()


@pytest.mark.parametrize("rd_scale", [1e-2, 1e-4])
def test_largek_ill_conditioned_points_are_certified_or_flagged(cuda, rd_scale):
    """Small observation-error variances stretch the spectrum of A: every point
    either returns a certified transform (finite, within 1e-3 of the oracle's
    largest entry) or is flagged (LETKF_ERR_EIG for no convergence,
    LETKF_ERR_CAPACITY where mtx_eigen's truncation could act); none returns a
    wrong transform with status OK."""
    import torch

    from letkf_gb300.core import core_batch_largek
    from letkf_gb300.lib import LETKF_ERR_CAPACITY, LETKF_ERR_EIG, LETKF_OK

    ne = 256
    rng = np.random.default_rng(int(1 / rd_scale))
    Ls = [300, 700, 150, 512, 90, 1000, 33, 400]
    offs, rows, rd, rl, d, infl = _batch(rng, ne, Ls)
    rd = (rd * rd_scale).astype(np.float32).astype(np.float64)
    ref = O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True)
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    out = core_batch_largek(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(d), t(infl, torch.float64),
                            want_transm=True)
    torch.cuda.synchronize()
    st = out["status"].cpu().numpy()
    assert set(np.unique(st)) <= {LETKF_OK, LETKF_ERR_EIG, LETKF_ERR_CAPACITY}
    tr = out["trans"].cpu().numpy().astype(np.float64)
    for p in np.where(st == LETKF_OK)[0]:
        assert np.isfinite(tr[p]).all(), p
        scale = np.abs(ref["trans"][p]).max()
        assert np.abs(tr[p] - ref["trans"][p]).max() <= 1e-3 * scale, (p, Ls[p])
