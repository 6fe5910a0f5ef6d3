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


@pytest.mark.parametrize("ne", [256, 512])
def test_indexed_bf16_lists_equal_the_packed_rows(cuda, ne):
    """The core over index lists into a BF16 observation ensemble (no packed
    copies) gives the same transforms, bit for bit, as the packed FP32 rows of
    the same values (BF16 values are exact in FP32); and it meets the oracle
    bar.  Lists repeat observations and run long (L up to 3000)."""
    import torch

    from letkf_gb300.core import core_batch_largek, core_batch_largek_indexed

    rng = np.random.default_rng(ne + 1)
    nobs = 5000
    ens = rng.standard_normal((nobs, ne))
    ens -= ens.mean(1, keepdims=True)
    ens16 = torch.as_tensor(ens, dtype=torch.bfloat16, device=cuda)
    ens64 = ens16.double().cpu().numpy()
    dep_obs = rng.standard_normal(nobs).astype(np.float32)
    Ls = [0, 3, 3000, 700, 128, 1]
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    idx = rng.integers(0, nobs, int(offs[-1])).astype(np.int32)
    rd = rng.uniform(0.3, 3.0, idx.size).astype(np.float32)
    rl = rng.uniform(0.01, 1.0, idx.size).astype(np.float32)
    infl = rng.uniform(0.95, 1.3, len(Ls))
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pa, pb = t(infl, torch.float64), t(infl, torch.float64)
    a = core_batch_largek_indexed(ne, t(offs, torch.int64), t(idx, torch.int32), ens16, t(dep_obs), t(rd), t(rl), pa,
                                  want_transm=True)
    rows = ens64[idx]
    b = core_batch_largek(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(dep_obs[idx]), pb, want_transm=True)
    torch.cuda.synchronize()
    for k in ("trans", "transm", "status"):
        assert torch.equal(a[k], b[k]), k
    assert torch.equal(pa, pb)
    ref = O.letkf_core_batch(ne, offs, rows, rd.astype(np.float64), rl.astype(np.float64),
                             dep_obs[idx].astype(np.float64), infl, want_transm=True)
    tr = a["trans"].cpu().numpy().astype(np.float64)
    for p in range(len(Ls)):
        scale = np.abs(ref["trans"][p]).max()
        assert np.abs(tr[p] - ref["trans"][p]).max() <= 1e-4 * scale, (p, Ls[p])


def test_update_bf16_storage(cuda):
    """letkf_update_bf16: FP32 mean + BF16 perturbations in and out.  The
    analysis mean within 1e-6 relative of the FP64 result on the same stored
    inputs; the perturbations within BF16 rounding (2^-8 relative)."""
    import torch

    from letkf_gb300.core import update_bf16

    rng = np.random.default_rng(7)
    nv, npts, ne = 3, 17, 320
    xmean = (rng.standard_normal((nv, npts)) * 10 + 280).astype(np.float32)
    xp = torch.as_tensor(rng.standard_normal((nv, npts, ne)), dtype=torch.bfloat16, device=cuda)
    a = rng.standard_normal((npts, ne, ne)) * 0.05
    tr = (np.eye(ne)[None] + (a + a.transpose(0, 2, 1))).astype(np.float32)  # column-major == symmetric
    tm = (rng.standard_normal((npts, ne)) * 0.01).astype(np.float32)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), device=cuda)
    am, ap = update_bf16(t(xmean), xp, t(tr), t(tm))
    x64 = xp.double().cpu().numpy()
    m = x64.mean(-1, keepdims=True)
    xd = x64 - m
    want_mean = xmean.astype(np.float64) + m[..., 0] + np.einsum("vpk,pk->vp", xd, tm.astype(np.float64))
    want_pert = np.einsum("vpk,pmk->vpm", xd, tr.astype(np.float64))
    assert np.abs(am.cpu().numpy() - want_mean).max() <= 1e-6 * np.abs(want_mean).max()
    got = ap.double().cpu().numpy()
    assert np.abs(got - want_pert).max() <= 2.0 ** -8 * np.abs(want_pert).max()
    assert np.sqrt(np.mean((got - want_pert) ** 2)) <= 2.0 ** -8 * np.sqrt(np.mean(want_pert ** 2))


def test_largek_long_lists_against_oracle(cuda):
    """k = 512 with local lists of 12,000 observations (the Gram over K = L in
    400 stages) through the indexed BF16 path, against the FP64 oracle."""
    import torch

    from letkf_gb300.core import core_batch_largek_indexed

    ne = 512
    rng = np.random.default_rng(12)
    nobs = 20000
    ens = rng.standard_normal((nobs, ne))
    ens -= ens.mean(1, keepdims=True)
    ens16 = torch.as_tensor(ens, dtype=torch.bfloat16, device=cuda)
    ens64 = ens16.double().cpu().numpy()
    dep_obs = rng.standard_normal(nobs).astype(np.float32)
    Ls = [12000, 10000]
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    idx = np.concatenate([rng.choice(nobs, L, replace=False) for L in Ls]).astype(np.int32)
    # error variances large enough that A stays well conditioned with this many observations
    rd = rng.uniform(50.0, 200.0, idx.size).astype(np.float32)
    rl = rng.uniform(0.01, 1.0, idx.size).astype(np.float32)
    infl = np.array([1.05, 1.2])
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_largek_indexed(ne, t(offs, torch.int64), t(idx, torch.int32), ens16, t(dep_obs), t(rd), t(rl),
                                    pinf, want_transm=True)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    ref = O.letkf_core_batch(ne, offs, ens64[idx], rd.astype(np.float64), rl.astype(np.float64),
                             dep_obs[idx].astype(np.float64), infl, want_transm=True, nthreads=2)
    tr = out["trans"].cpu().numpy().astype(np.float64)
    tm = out["transm"].cpu().numpy().astype(np.float64)
    for p in range(len(Ls)):
        scale = np.abs(ref["trans"][p]).max()
        assert np.abs(tr[p] - ref["trans"][p]).max() <= 1e-4 * scale, p
        assert np.abs(tm[p] - ref["transm"][p]).max() <= 1e-4 * scale, p
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-5)


def test_fp64_pass_answers_ill_conditioned_points(cuda):
    """Points the mixed-precision transform cannot certify (observation-error
    variances x1e-4: lambda_max / c up to ~1e5, tr(G) above the core's 1e6 c
    truncation guard) are redone in FP64 (Gram and Newton-Schulz): every point
    comes back LETKF_OK with its transform within 1e-5 of the oracle's largest
    entry and the inflation within 1e-8."""
    import torch

    from letkf_gb300.core import core_batch_largek
    from letkf_gb300.lib import LETKF_OK

    ne = 256
    rng = np.random.default_rng(10_000)
    Ls = [300, 700, 150, 512, 90, 1000, 33, 400]
    offs, rows, rd, rl, d, infl = _batch(rng, ne, Ls)
    rd = (rd * 1e-4).astype(np.float32).astype(np.float64)
    ref = O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True)
    t = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_largek(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(d), pinf, want_transm=True)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == LETKF_OK).all()
    tr = out["trans"].cpu().numpy().astype(np.float64)
    tm = out["transm"].cpu().numpy().astype(np.float64)
    for p in range(len(Ls)):
        scale = np.abs(ref["trans"][p]).max()
        assert np.abs(tr[p] - ref["trans"][p]).max() <= 1e-5 * scale, (p, Ls[p])
        assert np.abs(tm[p] - ref["transm"][p]).max() <= 1e-5 * scale, (p, Ls[p])
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-8)
