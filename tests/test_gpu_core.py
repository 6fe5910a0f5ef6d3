"""GPU parity of the FP64 plain form (per-point C ABI and batched) against the
CPU oracle.  Tolerance: 1e-10 relative (the FP64 plain-form bar)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _case(rng, ne, L):
    Y = rng.standard_normal((max(L, 1), ne))
    Y -= Y.mean(1, keepdims=True)
    rd = rng.uniform(0.3, 3.0, max(L, 1))
    rl = rng.uniform(0.01, 1.0, max(L, 1))
    d = rng.standard_normal(max(L, 1))
    return Y, rd, rl, d


def _close(a, b, rtol=RTOL):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max() / scale
    assert err <= rtol, f"relative error {err:.3e} > {rtol:.1e}"


@pytest.mark.parametrize("ne,L,wloc,minfl,transm,pao", [
    (2, 1, False, None, False, False),
    (3, 5, False, None, True, True),
    (20, 21, False, None, False, False),
    (20, 0, False, 1.5, True, True),
    (40, 120, True, 1.02, True, False),
    (64, 700, False, None, True, True),
    (64, 17, True, None, False, True),
    (97, 300, False, 0.5, True, True),
    (128, 400, False, None, True, True),
])
def test_core_c_matches_oracle(cuda, ne, L, wloc, minfl, transm, pao):
    from letkf_gb300.core import letkf_core

    rng = np.random.default_rng(ne * 7919 + L)
    Y, rd, rl, d = _case(rng, ne, L)
    nobs = max(L, 1) + 3                     # leading dimension larger than nobsl
    H = np.zeros((nobs, ne))
    H[: Y.shape[0]] = Y
    R = np.ones(nobs)
    R[: rd.size] = rd
    RL = np.ones(nobs)
    RL[: rl.size] = rl
    D = np.zeros(nobs)
    D[: d.size] = d
    infl = 0.9
    ref = O.letkf_core(H, R, RL, D, infl, nobsl=L, want_transm=transm, want_pao=pao, rdiag_wloc=wloc, minfl=minfl)
    assert ref["status"] == 0
    T, tm, pa, pinf = letkf_core(ne, nobs, L, H, R, RL, D, infl, transm=transm, pao=pao, rdiag_wloc=wloc,
                                 minfl=minfl)
    _close(T, ref["trans"])
    if transm:
        _close(tm, ref["transm"]) if L else np.testing.assert_array_equal(tm, 0.0)
    if pao:
        _close(pa, ref["pao"])
    assert abs(pinf - ref["parm_infl"]) <= 1e-12 * abs(ref["parm_infl"])


def test_core_c_argument_errors(cuda):
    from letkf_gb300.core import letkf_core
    from letkf_gb300.lib import LETKF_ERR_ARG, LETKF_ERR_CAPACITY, LetkfError

    with pytest.raises(LetkfError) as e:
        letkf_core(4, 2, 3, np.zeros((2, 4)), np.ones(2), np.ones(2), np.zeros(2), 1.0)  # nobsl > nobs
    assert e.value.status == LETKF_ERR_ARG
    with pytest.raises(LetkfError) as e:
        letkf_core(200, 2, 2, np.zeros((2, 200)), np.ones(2), np.ones(2), np.zeros(2), 1.0)
    assert e.value.status == LETKF_ERR_CAPACITY


def test_core_c_eigen_failure_status(cuda):
    # a negative inflation makes every eigenvalue of (Gram + (k-1)/infl I) negative -> STOP 2 in the reference
    from letkf_gb300.core import letkf_core
    from letkf_gb300.lib import LETKF_ERR_EIG, LetkfError

    ne = 6
    H = np.zeros((2, ne))
    H[0, 0], H[0, 1] = 1e-3, -1e-3
    ref = O.letkf_core(H, [1.0, 1.0], [1.0, 1.0], [0.0, 0.0], -1.0, nobsl=2)
    assert ref["status"] == 2
    with pytest.raises(LetkfError) as e:
        letkf_core(ne, 2, 2, H, np.ones(2), np.ones(2), np.zeros(2), -1.0)
    assert e.value.status == LETKF_ERR_EIG


def _batch(rng, ne, Ls):
    offs = np.concatenate([[0], np.cumsum(Ls)]).astype(np.int64)
    n = int(offs[-1])
    rows = rng.standard_normal((max(n, 1), ne))
    rows -= rows.mean(1, keepdims=True)
    rd = rng.uniform(0.3, 3.0, max(n, 1))
    rl = rng.uniform(0.01, 1.0, max(n, 1))
    d = rng.standard_normal(max(n, 1))
    infl = rng.uniform(0.9, 1.3, len(Ls))
    return offs, rows, rd, rl, d, infl


@pytest.mark.parametrize("ne", [20, 40, 64])
def test_batch_f64_matches_oracle(cuda, ne):
    import torch

    from letkf_gb300.core import core_batch_f64

    rng = np.random.default_rng(100 + ne)
    Ls = list(rng.integers(0, 300, 37)) + [0, 1, 2, 1000]
    offs, rows, rd, rl, d, infl = _batch(rng, ne, Ls)
    ref = O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True, want_pao=True, rdiag_wloc=True,
                             minfl=1.0)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    pinf = t(infl)
    out = core_batch_f64(ne, t(offs, torch.int64), t(rows), t(rd), t(rl), t(d), pinf, want_transm=True,
                         want_pao=True, rdiag_wloc=True, minfl=1.0)
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    for p in range(len(Ls)):
        _close(out["trans"][p].cpu().numpy(), ref["trans"][p])
        _close(out["pao"][p].cpu().numpy(), ref["pao"][p])
        if Ls[p]:
            _close(out["transm"][p].cpu().numpy(), ref["transm"][p])
    np.testing.assert_allclose(pinf.cpu().numpy(), ref["parm_infl"], rtol=1e-12)


def test_update_f64_matches_reference_loop(cuda):
    import torch

    from letkf_gb300.core import update_f64

    rng = np.random.default_rng(5)
    nv, npts, ne = 3, 50, 20
    xb = rng.standard_normal((nv, npts, ne)) + 5.0
    W = rng.standard_normal((npts, ne, ne)) * 0.1        # [p][m][k] = trans_p(k, m)
    tm = rng.standard_normal((npts, ne)) * 0.1
    xa = update_f64(torch.as_tensor(xb, device=cuda), torch.as_tensor(W, device=cuda),
                    torch.as_tensor(tm, device=cuda)).cpu().numpy()
    for v in range(nv):
        mean, pert = O.ensmean(xb[v])
        for p in range(npts):
            ref = mean[p] + pert[p] @ (W[p].T + tm[p][:, None])
            np.testing.assert_allclose(xa[v, p], ref, rtol=1e-13, atol=1e-13)
