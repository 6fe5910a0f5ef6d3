"""The SCALE observation operator on the device (letkf_scale_obsope) against
the oracle restatement (oracle/obs_operator_scale.c) on random fields:
terrain-following pressure with some levels below ground, every element
(u, v, t, tv, q, rh, ps, an unknown code), observations inside, outside,
above and below the domain, the staggered grid and the rotation of the map
projection.  The kernel follows the reference's expression order with no
contracted multiply-add, so only log and pow differ by an ulp from the host:
values within 1e-12 of the observation's largest magnitude over the members
(a rotated wind can cancel to near zero), qc equal."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KH = 2
ELEMS = np.array([2819, 2820, 3073, 3074, 3330, 3331, 14593, 4321], np.int32)


def random_case(seed, ne=40, nlonh=36, nlath=30, nlev=20, nobs=4000):
    rng = np.random.default_rng(seed)
    nlevh = nlev + 2 * KH
    i = np.arange(1, nlonh + 1)
    j = np.arange(1, nlath + 1)
    J, I = np.meshgrid(j, i, indexing="ij")
    zs = 400.0 * (1 + np.sin(I / 5.0) * np.cos(J / 7.0))  # terrain height [m]
    sig = np.exp(-np.linspace(-0.2, 4.2, nlevh))          # halo levels below and above
    v3d = np.empty((ne, 6, nlath, nlonh, nlevh))
    v2d = np.empty((ne, 4, nlath, nlonh))
    for m in range(ne):
        ps = 1.0e5 * np.exp(-zs / 8000.0) * (1 + 0.01 * rng.standard_normal((nlath, nlonh)))
        p = ps[:, :, None] * sig[None, None, :]
        # below ground where the column is high: the lowest levels invalid
        low = (zs > 500.0)[:, :, None] & (np.arange(nlevh)[None, None, :] < KH + 2)
        p = np.where(low, -1.0, p)
        v3d[m, 5] = p
        for n in range(5):
            v3d[m, n] = rng.standard_normal((nlath, nlonh, nlevh)) * [5, 5, 10, 0.002, 0.1][n] + \
                        [3, -2, 260, 0.005, 0.6][n]
        v2d[m, 0] = ps
        v2d[m, 1] = 285 + rng.standard_normal((nlath, nlonh))
        v2d[m, 2] = 0.008 + 0.001 * rng.standard_normal((nlath, nlonh))
        v2d[m, 3] = zs
    elem = rng.choice(ELEMS, nobs).astype(np.int32)
    ri = rng.uniform(0.5, nlonh + 0.3, nobs)
    rj = rng.uniform(0.5, nlath + 0.3, nobs)
    rlev = np.exp(rng.uniform(np.log(5e2), np.log(1.2e5), nobs))
    sfc = elem == 14593
    rlev[sfc] = rng.uniform(0.0, 1200.0, sfc.sum())  # observation heights [m]
    ang = rng.uniform(-0.6, 0.6, nobs)
    rotc = np.stack([np.cos(ang), np.sin(ang)], -1)
    return v3d, v2d, elem, ri, rj, rlev, rotc


def _close(hx, hx0):
    scale = np.abs(hx0).max(axis=1, keepdims=True)
    assert (np.abs(hx - hx0) <= 1e-12 * scale).all(), float((np.abs(hx - hx0) / np.maximum(scale, 1e-300)).max())


@pytest.mark.parametrize("stggrd,seed", [(0, 1), (1, 2)])
def test_scale_obsope_matches_oracle(cuda, stggrd, seed):
    import torch

    from letkf_gb300.core import scale_obsope

    v3d, v2d, elem, ri, rj, rlev, rotc = random_case(seed)
    hx0, qc0, qcm0 = O.scale_obsope(v3d, v2d, KH, elem, ri, rj, rlev, rotc, stggrd=stggrd)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    hx, qc, qcm = scale_obsope(t(v3d), t(v2d), KH, t(elem, torch.int32), t(ri), t(rj), t(rlev), t(rotc),
                               stggrd=stggrd, want_member_qc=True)
    torch.cuda.synchronize()
    hx, qc, qcm = hx.cpu().numpy(), qc.cpu().numpy(), qcm.cpu().numpy()
    np.testing.assert_array_equal(qcm, qcm0)
    np.testing.assert_array_equal(qc, qc0)
    _close(hx, hx0)
    # every outcome occurs
    assert {0, 10, 20, 21, 22, 90} <= set(np.unique(qcm0).tolist())
    assert (qc0 == 0).sum() > len(qc0) // 4


def test_scale_obsope_no_rotation_and_shared_fields(cuda):
    """rotc NULL means (1, 0)."""
    import torch

    from letkf_gb300.core import scale_obsope

    v3d, v2d, elem, ri, rj, rlev, _ = random_case(3, ne=4, nobs=500)
    hx0, qc0, _ = O.scale_obsope(v3d, v2d, KH, elem, ri, rj, rlev)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=cuda)
    hx, qc = scale_obsope(t(v3d), t(v2d), KH, t(elem, torch.int32), t(ri), t(rj), t(rlev))
    np.testing.assert_array_equal(qc.cpu().numpy(), qc0)
    _close(hx.cpu().numpy(), hx0)
