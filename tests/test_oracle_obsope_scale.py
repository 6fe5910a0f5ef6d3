"""The SCALE observation operator restatement (oracle/obs_operator_scale.c)
against closed forms.  Fields linear in (k, i, j) with log p linear in k make
phys2ijk and the interpolation exact, so H(x) is known in closed form:
scale/common/common_obs_scale.f90:262-334 (Trans_XtoY), :583-599 (prsadj),
:969-1075 (phys2ijk), :1254-1325 (itpl_2d / itpl_3d);
scale/obs/obsope_tools.f90:340-380, 602-608 (qc over members: the maximum)."""
import numpy as np
import pytest

from oracle import oracle as O

U, V, T, TV, Q, RH, PS = 2819, 2820, 3073, 3074, 3330, 3331, 14593
KH = 2


def linear_case(ne=3, nlonh=12, nlath=10, nlev=8, seed=0):
    """Member m: p = p0 exp(-h k) (k the 1-based level index of the halo
    domain), field n = c0 + c1 k + c2 i + c3 j (+ m), 2-D fields linear in (i, j)."""
    rng = np.random.default_rng(seed)
    nlevh = nlev + 2 * KH
    k = np.arange(1, nlevh + 1, dtype=np.float64)
    i = np.arange(1, nlonh + 1, dtype=np.float64)
    j = np.arange(1, nlath + 1, dtype=np.float64)
    J, I, K = np.meshgrid(j, i, k, indexing="ij")  # [nlath, nlonh, nlevh]
    coef = rng.uniform(-2, 2, (6, 4))
    coef2 = rng.uniform(-2, 2, (4, 3))
    v3d = np.zeros((ne, 6, nlath, nlonh, nlevh))
    v2d = np.zeros((ne, 4, nlath, nlonh))
    p0, h = 1.0e5, 0.15
    for m in range(ne):
        for n in range(5):
            c = coef[n]
            v3d[m, n] = c[0] + c[1] * K + c[2] * I + c[3] * J + m
        v3d[m, 5] = p0 * np.exp(-h * K)
        for n in range(4):
            c = coef2[n]
            v2d[m, n] = c[0] + c[1] * I[:, :, 0] + c[2] * J[:, :, 0] + 0.5 * m
    v2d[:, 0] += 9.0e4   # ps
    v2d[:, 1] += 280.0   # t2m
    v2d[:, 2] = 0.01     # q2m
    v2d[:, 3] = 10.0 * (1 + np.arange(ne))[:, None, None]  # topo per member
    return v3d, v2d, coef, coef2, p0, h


def rk_of(p, p0, h):
    return (np.log(p0) - np.log(p)) / h


def test_upper_air_interpolation_is_exact_for_linear_fields():
    v3d, v2d, coef, _, p0, h = linear_case()
    ne, nlev = v3d.shape[0], v3d.shape[-1] - 2 * KH
    ri = np.array([3.3, 5.0, 7.75, 2.5, 4.1, 6.6])
    rj = np.array([2.2, 4.0, 8.5, 3.5, 6.9, 5.5])
    # levels between rk = 3.5 and 8.5, inside [ks, top] = [3, 10]
    rks = np.array([3.5, 4.25, 6.0, 7.3, 8.5, 5.1])
    rlev = p0 * np.exp(-h * rks)
    elem = np.array([T, Q, RH, U, V, TV], np.int32)
    rotc = np.array([[1.0, 0.0], [1.0, 0.0], [1.0, 0.0], [0.8, 0.6], [0.6, -0.8], [1.0, 0.0]])
    hx, qc, qcm = O.scale_obsope(v3d, v2d, KH, elem, ri, rj, rlev, rotc)
    assert (qc == 0).all() and (qcm == 0).all()
    fvirt = 461.50 / 287.05 - 1.0
    for n in range(elem.size):
        rk = rk_of(rlev[n], p0, h)
        for m in range(ne):
            val = lambda v: coef[v, 0] + coef[v, 1] * rk + coef[v, 2] * ri[n] + coef[v, 3] * rj[n] + m
            if elem[n] == U:
                want = val(0) * rotc[n, 0] - val(1) * rotc[n, 1]
            elif elem[n] == V:
                want = val(0) * rotc[n, 1] + val(1) * rotc[n, 0]
            elif elem[n] == TV:
                want = val(2) * (1.0 + fvirt * val(3))
            else:
                want = val({T: 2, Q: 3, RH: 4}[elem[n]])
            assert abs(hx[n, m] - want) < 1e-9 * max(1.0, abs(want)), (n, m, hx[n, m], want)


def test_staggered_winds_read_half_a_cell_back():
    v3d, v2d, coef, _, p0, h = linear_case()
    rlev = np.full(2, p0 * np.exp(-h * 5.5))
    ri, rj = np.array([4.4, 6.2]), np.array([3.7, 5.9])
    hx, qc, _ = O.scale_obsope(v3d, v2d, KH, np.array([U, V], np.int32), ri, rj, rlev, stggrd=1)
    assert (qc == 0).all()
    rk = rk_of(rlev[0], p0, h)
    u = coef[0, 0] + coef[0, 1] * rk + coef[0, 2] * (ri[0] - 0.5) + coef[0, 3] * rj[0]
    v = coef[1, 0] + coef[1, 1] * rk + coef[1, 2] * ri[1] + coef[1, 3] * (rj[1] - 0.5)
    assert abs(hx[0, 0] - u) < 1e-9 and abs(hx[1, 0] - v) < 1e-9


def test_surface_pressure_height_adjustment_and_threshold():
    v3d, v2d, _, coef2, _, _ = linear_case(ne=2)
    ri, rj = np.array([4.25, 4.25]), np.array([6.5, 6.5])
    z = np.array([60.0, 250.0])  # observation heights; topo is 10 m (member 0) / 20 m (member 1)
    hx, qc, qcm = O.scale_obsope(v3d, v2d, KH, np.array([PS, PS], np.int32), ri, rj, z)
    for n in range(2):
        for m in range(2):
            lin = lambda v: coef2[v, 0] + coef2[v, 1] * ri[n] + coef2[v, 2] * rj[n]
            ps = lin(0) + 9.0e4 + 0.5 * m
            t = lin(1) + 280.0 + 0.5 * m
            dz = z[n] - 10.0 * (1 + m)
            tv = t * (1.0 + 0.608 * 0.01)
            want = ps * ((-5.0e-3 * dz + tv) / tv) ** (9.81 / (5.0e-3 * 287.05))
            assert abs(hx[n, m] - want) < 1e-9 * want
    # |dz| > 100 m: qc 10 (the value is still computed)
    assert (qcm[0] == 0).all() and (qcm[1] == 10).all() and qc.tolist() == [0, 10]


def test_rejections_and_qc_over_members():
    v3d, v2d, _, _, p0, h = linear_case(ne=3)
    nlonh, nlath = v3d.shape[3], v3d.shape[2]
    # member 2: the four lowest valid levels below ground in one column
    v3d[2, 5, 3, 3, KH:KH + 4] = -1.0
    top = v3d.shape[-1] - KH
    elem = np.array([T, T, T, T, 1234, T], np.int32)
    ri = np.array([0.5, 5.0, 5.0, 4.5, 8.0, 6.2])
    rj = np.array([5.0, 5.0, 5.0, 4.5, 8.0, 6.3])
    rlev = np.array([5e4, p0 * np.exp(-h * (top + 0.5)), p0 * np.exp(-h * (KH + 0.5)),
                     p0 * np.exp(-h * (KH + 3.5)), 5e4, p0 * np.exp(-h * 6.0)])
    hx, qc, qcm = O.scale_obsope(v3d, v2d, KH, elem, ri, rj, rlev)
    assert qc[0] == 22 and (hx[0] == 0).all()          # outside the domain
    assert qc[1] == 20 and (hx[1] == 0).all()          # above the top level
    assert qc[2] == 21                                  # below the lowest level
    # ks moved up in member 2 only (its column (4, 4), 1-based, holds the raised ground): too low there
    assert qcm[3].tolist() == [0, 0, 21] and qc[3] == 21
    assert qc[4] == 90 and (hx[4] == -9.99e33).all()   # unknown element
    assert qc[5] == 0
    assert nlonh > 5 and nlath > 5


@pytest.mark.parametrize("edge", [1.0, 12.0])
def test_domain_edges_stay_in_the_arrays(edge):
    """ri exactly 1 (the reference's stencil reads index 0 with weight 0) and
    ri = nlonh give the linear field's value."""
    v3d, v2d, coef, _, p0, h = linear_case()
    rlev = np.array([p0 * np.exp(-h * 6.5)])
    hx, qc, _ = O.scale_obsope(v3d, v2d, KH, np.array([T], np.int32), np.array([edge]), np.array([4.5]), rlev)
    rk = rk_of(rlev[0], p0, h)
    want = coef[2, 0] + coef[2, 1] * rk + coef[2, 2] * edge + coef[2, 3] * 4.5
    assert qc[0] == 0 and abs(hx[0, 0] - want) < 1e-9
