"""Known-answer tests that pin the CPU oracle (the reference ships no tests or
golden data, and its Fortran cannot be compiled here).  Each case follows
from the mathematics of common/common_letkf.f90:50-243."""
import math

import numpy as np
import pytest

from oracle import oracle as O


def _case(rng, ne, L, spread=1.0, err=1.0):
    Y = spread * rng.standard_normal((L, ne))
    Y -= Y.mean(1, keepdims=True)          # Yb 1 = 0 as for true perturbations
    rd = err ** 2 * rng.uniform(0.5, 2.0, L)
    rl = rng.uniform(0.05, 1.0, L)
    d = rng.standard_normal(L)
    return Y, rd, rl, d


def _dense(Y, rd, rl, d, infl, wloc=False):
    ne = Y.shape[1]
    w = (1.0 / rd) if wloc else (rl / rd)
    A = (Y * w[:, None]).T @ Y + (ne - 1) / infl * np.eye(ne)
    lam, V = np.linalg.eigh(A)
    Pa = V @ np.diag(1 / lam) @ V.T
    T = V @ np.diag(np.sqrt((ne - 1) / lam)) @ V.T
    wb = Pa @ ((Y * w[:, None]).T @ d)
    return T, Pa, wb


def test_nobsl_zero_branch():
    # common_letkf.f90:82-96: trans = sqrt(infl) I, transm = 0, pao = infl/(k-1) I, infl unchanged (no minfl)
    ne = 7
    r = O.letkf_core(np.zeros((3, ne)), np.ones(3), np.ones(3), np.zeros(3), 0.81, nobsl=0, want_transm=True,
                     want_pao=True, minfl=2.0)
    assert r["status"] == 0
    np.testing.assert_array_equal(r["trans"], 0.9 * np.eye(ne))
    np.testing.assert_array_equal(r["transm"], np.zeros(ne))
    np.testing.assert_array_equal(r["pao"], 0.81 / 6 * np.eye(ne))
    assert r["parm_infl"] == 0.81


@pytest.mark.parametrize("ne,L", [(20, 21), (40, 150), (64, 30), (8, 500)])
def test_against_dense_eigh(ne, L):
    rng = np.random.default_rng(ne * 1000 + L)
    Y, rd, rl, d = _case(rng, ne, L)
    r = O.letkf_core(Y, rd, rl, d, 1.1, want_transm=True, want_pao=True)
    T, Pa, wb = _dense(Y, rd, rl, d, 1.1)
    np.testing.assert_allclose(r["trans"], T, rtol=0, atol=1e-12 * np.abs(T).max())
    np.testing.assert_allclose(r["pao"], Pa, rtol=0, atol=1e-12 * np.abs(Pa).max())
    np.testing.assert_allclose(r["transm"], wb, rtol=0, atol=1e-11 * max(1.0, np.abs(wb).max()))


def test_column_sums_and_mean_weight_sum():
    # Yb 1 = 0 makes 1 an eigenvector with eigenvalue (k-1)/infl: W 1 = sqrt(infl) 1 and 1^T wbar = 0
    rng = np.random.default_rng(3)
    ne, L, infl = 20, 40, 1.3
    Y, rd, rl, d = _case(rng, ne, L)
    r = O.letkf_core(Y, rd, rl, d, infl, want_transm=True)
    np.testing.assert_allclose(r["trans"].sum(0), math.sqrt(infl), rtol=1e-12)
    assert abs(r["transm"].sum()) < 1e-12 * np.abs(r["transm"]).sum()


def test_transm_absent_adds_mean_weights():
    rng = np.random.default_rng(4)
    Y, rd, rl, d = _case(rng, 12, 30)
    a = O.letkf_core(Y, rd, rl, d, 1.0, want_transm=True)
    b = O.letkf_core(Y, rd, rl, d, 1.0)
    np.testing.assert_allclose(b["trans"], a["trans"] + a["transm"][:, None], rtol=0, atol=1e-14)
    assert a["parm_infl"] == b["parm_infl"]


def test_single_observation_closed_form():
    # one obs: A = c I + w y y^T, eigenvalues c (mult k-1) and c + w |y|^2
    rng = np.random.default_rng(5)
    ne, infl = 10, 1.2
    y = rng.standard_normal(ne)
    y -= y.mean()
    rd, rl, dep = 0.7, 0.4, 1.3
    r = O.letkf_core(y[None, :], [rd], [rl], [dep], infl, want_transm=True, want_pao=True)
    c = (ne - 1) / infl
    w = rl / rd
    s2 = y @ y
    u = y / math.sqrt(s2)
    P = np.outer(u, u)
    Pa = (np.eye(ne) - P) / c + P / (c + w * s2)
    T = math.sqrt(ne - 1) * ((np.eye(ne) - P) / math.sqrt(c) + P / math.sqrt(c + w * s2))
    wb = Pa @ (w * dep * y)
    np.testing.assert_allclose(r["pao"], Pa, atol=1e-14)
    np.testing.assert_allclose(r["trans"], T, atol=1e-13)
    np.testing.assert_allclose(r["transm"], wb, atol=1e-14)
    # inflation: p1 = dep^2 w, p2 = w |y|^2/(k-1), p3 = rloc
    p1, p2, p3 = dep * dep / rd * rl, w * s2 / (ne - 1), rl
    p4 = (p1 - p3) / p2 - infl
    so = 2.0 / p3 * ((infl * p2 + p3) / p2) ** 2
    gain = 0.04 ** 2 / (so + 0.04 ** 2)
    assert r["parm_infl"] == pytest.approx(infl + gain * p4, rel=1e-14)


def test_kalman_gain_posterior():
    # ensemble-space Pa equals the Kalman posterior in the span of the perturbations:
    # Xb Pa Xb^T (k-1) / infl-scaled == Pb - Pb H^T (H Pb H^T + R)^-1 H Pb with Pb = infl Xb Xb^T/(k-1)
    rng = np.random.default_rng(6)
    n, ne, L, infl = 15, 12, 9, 1.1
    Xb = rng.standard_normal((n, ne))
    Xb -= Xb.mean(1, keepdims=True)
    H = rng.standard_normal((L, n))
    Y = H @ Xb
    rd = rng.uniform(0.5, 2.0, L)
    r = O.letkf_core(Y, rd, np.ones(L), np.zeros(L), infl, want_pao=True)
    Pb = infl * Xb @ Xb.T / (ne - 1)
    R = np.diag(rd)
    Pa_kf = Pb - Pb @ H.T @ np.linalg.solve(H @ Pb @ H.T + R, H @ Pb)
    Pa_ens = infl * Xb @ (r["pao"] * (ne - 1) / infl) @ Xb.T / (ne - 1) * infl / infl
    np.testing.assert_allclose(Xb @ r["pao"] @ Xb.T, Pa_kf, atol=1e-10)
    assert Pa_ens.shape == (n, n)


def test_rdiag_wloc_equivalence():
    # SCALE passes rdiag = err^2 / rloc with rdiag_wloc: same weights as (err^2, rloc)
    rng = np.random.default_rng(7)
    Y, rd, rl, d = _case(rng, 16, 50)
    a = O.letkf_core(Y, rd, rl, d, 1.05, want_transm=True)
    b = O.letkf_core(Y, rd / rl, rl, d, 1.05, want_transm=True, rdiag_wloc=True)
    np.testing.assert_allclose(a["trans"], b["trans"], atol=1e-13)
    np.testing.assert_allclose(a["transm"], b["transm"], atol=1e-13)
    assert a["parm_infl"] == pytest.approx(b["parm_infl"], rel=1e-13)


def test_minfl_clamp():
    rng = np.random.default_rng(8)
    Y, rd, rl, d = _case(rng, 10, 20)
    a = O.letkf_core(Y, rd, rl, d, 0.5, minfl=1.2, want_pao=True)
    b = O.letkf_core(Y, rd, rl, d, 1.2, want_pao=True)
    np.testing.assert_array_equal(a["pao"], b["pao"])
    assert a["parm_infl"] == b["parm_infl"]
    c = O.letkf_core(Y, rd, rl, d, 1.5, minfl=1.2, want_pao=True)   # above the floor: untouched
    e = O.letkf_core(Y, rd, rl, d, 1.5, want_pao=True)
    np.testing.assert_array_equal(c["pao"], e["pao"])


def test_mtx_eigen_descending_and_pythag():
    rng = np.random.default_rng(9)
    B = rng.standard_normal((9, 9))
    A = B @ B.T + np.eye(9)
    lam, V, nr, st = O.mtx_eigen(A)
    assert st == 0 and nr == 9
    assert np.all(np.diff(lam) <= 0)
    np.testing.assert_allclose(lam, np.sort(np.linalg.eigvalsh(A))[::-1], rtol=1e-13)
    np.testing.assert_allclose(A @ V, V * lam, atol=1e-12)
    assert O.pythag(3.0, 4.0) == pytest.approx(5.0, rel=1e-15)
    assert O.pythag(0.0, 0.0) == 0.0


def test_mtx_eigen_errors():
    # all eigenvalues <= 0 -> STOP 2 (common_mtx.f90:75-78)
    lam, V, nr, st = O.mtx_eigen(-np.eye(4))
    assert st == 2
    # truncation: lambda < lambda_max sqrt(eps) zeroed (common_mtx.f90:66-73)
    A = np.diag([1.0, 1e-10, 2.0])
    lam, V, nr, st = O.mtx_eigen(A)
    assert st == 0 and nr == 2 and lam[-1] == 0.0 and np.all(V[:, -1] == 0)


def test_weight_rtpp_rtps():
    rng = np.random.default_rng(10)
    ne = 8
    W = rng.standard_normal((ne, ne))
    out = O.weight_rtpp(W, 0.3)
    np.testing.assert_allclose(out, 0.7 * W + 0.3 * np.eye(ne), atol=1e-15)
    Pa = np.eye(ne) * 0.1
    xb = rng.standard_normal(ne)
    w2, infl = O.weight_rtps(W, Pa, xb, 0.5)
    vg, va = xb @ xb, xb @ Pa @ xb
    assert infl == pytest.approx(0.5 * math.sqrt(vg / (va * (ne - 1))) - 0.5 + 1.0, rel=1e-14)
    np.testing.assert_allclose(w2, W * infl, atol=1e-14)


def test_batch_matches_single():
    rng = np.random.default_rng(11)
    ne = 10
    Ls = [0, 3, 17]
    offs = np.concatenate([[0], np.cumsum(Ls)])
    rows = rng.standard_normal((offs[-1], ne))
    rd = rng.uniform(0.5, 2, offs[-1])
    rl = rng.uniform(0.1, 1, offs[-1])
    d = rng.standard_normal(offs[-1])
    infl = np.array([1.0, 1.1, 1.2])
    b = O.letkf_core_batch(ne, offs, rows, rd, rl, d, infl, want_transm=True)
    for p in range(3):
        s = slice(offs[p], offs[p + 1])
        r = O.letkf_core(rows[s] if Ls[p] else np.zeros((1, ne)), rd[s] if Ls[p] else [1.0],
                         rl[s] if Ls[p] else [1.0], d[s] if Ls[p] else [0.0], infl[p], nobsl=Ls[p],
                         want_transm=True)
        np.testing.assert_array_equal(b["trans"][p], r["trans"].T)
        np.testing.assert_array_equal(b["transm"][p], r["transm"])
        assert b["parm_infl"][p] == r["parm_infl"]
