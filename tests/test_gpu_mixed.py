"""Mixed-precision batched core against the FP64 oracle.  Inputs are FP32
values (upcast exactly for the oracle); the bar is the analysis error
relative to the background spread, 1e-4."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ne", [20, 32, 40, 64, 100, 128])
def test_mixed_batch_against_oracle(cuda, ne):
    import torch

    from letkf_gb300.core import core_batch_mixed

    rng = np.random.default_rng(ne)
    Ls = list(rng.integers(0, 800, 30)) + [0, 1, 2000]
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    n = int(offs[-1])
    rows = rng.standard_normal((n, ne)).astype(np.float32)
    rows -= rows.mean(1, keepdims=True)
    rd = rng.uniform(0.3, 3.0, n).astype(np.float32)
    rl = rng.uniform(0.01, 1.0, n).astype(np.float32)
    d = rng.standard_normal(n).astype(np.float32)
    infl = rng.uniform(0.9, 1.3, len(Ls))
    ref = O.letkf_core_batch(ne, offs, rows.astype(np.float64), rd.astype(np.float64), rl.astype(np.float64),
                             d.astype(np.float64), infl, want_transm=True)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_mixed(ne, t(offs, torch.int64), t(rows, torch.float32), t(rd, torch.float32),
                           t(rl, torch.float32), t(d, torch.float32), pinf, want_transm=True)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    W = out["trans"].cpu().numpy().astype(np.float64)
    wb = out["transm"].cpu().numpy().astype(np.float64)
    # analysis perturbations / mean increments for unit-spread background members
    for p in range(len(Ls)):
        Xb = rng.standard_normal((4, ne))
        Xb -= Xb.mean(1, keepdims=True)
        spread = np.sqrt((Xb ** 2).sum(1) / (ne - 1)).mean()
        xa_ref = Xb @ ref["trans"][p].T
        xa = Xb @ W[p].T
        dm_ref = Xb @ ref["transm"][p]
        dm = Xb @ wb[p]
        assert np.sqrt(np.mean((xa - xa_ref) ** 2)) < 1e-4 * spread, p
        assert np.sqrt(np.mean((dm - dm_ref) ** 2)) < 1e-4 * spread, p
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-4)


@pytest.mark.parametrize("ne,rd_scale,bar", [(40, 1e-2, 1e-4), (64, 1e-2, 1e-4), (64, 1e-3, 5e-4)])
def test_mixed_batch_ill_conditioned_falls_back_to_jacobi(cuda, ne, rd_scale, bar):
    """Small observation-error variances (x1e-2, x1e-3) stretch the spectrum of
    A beyond what the FP32 Newton-Schulz iteration converges for on many
    points; those points are done again with the Jacobi eigensolver (their Gram
    recomputed), so every transform stays finite and close to the oracle: the
    mixed-form bar at x1e-2; at x1e-3 (condition numbers near 1e6, past FP32's
    reach at 1e-4) within 5e-4 of spread, where the plain FP64 form is the one
    to use."""
    import torch

    from letkf_gb300.core import core_batch_mixed

    rng = np.random.default_rng(100 + ne)
    Ls = list(rng.integers(50, 900, 24)) + [0, 1, 2000]
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    n = int(offs[-1])
    rows = rng.standard_normal((n, ne)).astype(np.float32)
    rows -= rows.mean(1, keepdims=True)
    rd = (rd_scale * rng.uniform(0.3, 3.0, n)).astype(np.float32)
    rl = rng.uniform(0.01, 1.0, n).astype(np.float32)
    d = rng.standard_normal(n).astype(np.float32)
    infl = rng.uniform(0.9, 1.3, len(Ls))
    ref = O.letkf_core_batch(ne, offs, rows.astype(np.float64), rd.astype(np.float64), rl.astype(np.float64),
                             d.astype(np.float64), infl, want_transm=True)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl, torch.float64)
    out = core_batch_mixed(ne, t(offs, torch.int64), t(rows, torch.float32), t(rd, torch.float32),
                           t(rl, torch.float32), t(d, torch.float32), pinf, want_transm=True)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    W = out["trans"].cpu().numpy().astype(np.float64)
    wb = out["transm"].cpu().numpy().astype(np.float64)
    assert np.isfinite(W).all() and np.isfinite(wb).all()
    for p in range(len(Ls)):
        Xb = rng.standard_normal((4, ne))
        Xb -= Xb.mean(1, keepdims=True)
        spread = np.sqrt((Xb ** 2).sum(1) / (ne - 1)).mean()
        assert np.sqrt(np.mean((Xb @ W[p].T - Xb @ ref["trans"][p].T) ** 2)) < bar * spread, p
        assert np.sqrt(np.mean((Xb @ wb[p] - Xb @ ref["transm"][p]) ** 2)) < bar * spread, p
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-4)
