"""The continuous-batching server (letkf_server_*): jobs for domains of
different sizes, ensemble sizes and precisions, submitted together, must give
the same analyses as each job alone (bit for bit: every point is computed by
one CTA independently of the others), overlap on the device, respect the
device-memory budget and reuse resident domains."""
import numpy as np
import pytest

from letkf_gb300 import synthetic as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _regional(seed, nlon, nlat, nlev, ne, nobs, precision):
    from letkf_gb300.serve import PREC_MIXED

    dt = np.float32 if precision == PREC_MIXED else np.float64
    c = S.regional_case(seed, nlon=nlon, nlat=nlat, nlev=nlev, ne=ne, nobs=nobs, nvar=2, sigma_obs=9.0e3, dtype=dt)
    return dict(kind="sweep", case=c, precision=precision)


def _l96(seed, nx, ne, precision):
    rng = np.random.default_rng(seed)
    xf = 8.0 + rng.standard_normal((nx, ne))
    cell = np.arange(1, nx + 1, dtype=np.int32)
    hx = xf[cell - 1]
    m = hx.sum(1) / ne
    y = m + rng.standard_normal(nx)
    return dict(kind="l96", xf=xf, hdxf=hx - m[:, None], dep=y - m, cell=cell, precision=precision)


def _jobs():
    from letkf_gb300.serve import PREC_F64, PREC_MIXED

    return [_regional(1, 24, 20, 4, 20, 2500, PREC_MIXED), _l96(2, 40, 20, PREC_F64),
            _regional(3, 32, 24, 3, 64, 4000, PREC_MIXED), _l96(4, 20000, 32, PREC_MIXED),
            _regional(5, 16, 16, 3, 32, 1500, PREC_F64), _l96(6, 3000, 20, PREC_F64),
            _regional(7, 20, 20, 5, 48, 3000, PREC_MIXED)]


def _submit(srv, spec, domain=-1):
    if spec["kind"] == "l96":
        return srv.submit_l96(spec["xf"], spec["hdxf"], spec["dep"], spec["cell"], precision=spec["precision"],
                              domain=domain)
    c = spec["case"]
    obs = {k: c[k] for k in ("ri", "rj", "lev", "dat", "err", "cls")}
    return srv.submit_sweep(c["pri"], c["prj"], c["prlev"], S.scale_params(c), c["nlon"], c["nlat"], obs, c["hdxf"],
                            c["dep"], c["xb"], infl=np.full(c["pri"].size, 1.04), precision=spec["precision"],
                            domain=domain)


def test_results_are_the_same_alone_and_in_the_mix(cuda):
    from letkf_gb300.serve import Server

    specs = _jobs()
    alone = []
    with Server(nslots=1) as s1:
        for sp in specs:
            j = _submit(s1, sp)
            s1.wait(j)
            alone.append((j.xa.copy(), None if j.infl is None else j.infl.copy()))
    with Server(nslots=3) as s3:
        jobs = [_submit(s3, sp) for sp in specs]
        for j in jobs:
            assert s3.wait(j)["status"] == 0
        st = s3.stats()
    for (xa, infl), j in zip(alone, jobs):
        np.testing.assert_array_equal(j.xa, xa)
        if infl is not None:
            np.testing.assert_array_equal(j.infl, infl)
    assert st["completed"] == len(specs) and st["failed"] == 0
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"]
    assert st["points_per_s"] > 0
    # work of different jobs was on the device at the same time
    iv = [(j.result["t_start"], j.result["t_done"]) for j in jobs]
    assert any(a0 < b1 and b0 < a1 for i, (a0, a1) in enumerate(iv) for (b0, b1) in iv[i + 1:])


def test_memory_budget_admits_one_job_at_a_time(cuda):
    from letkf_gb300.serve import Server

    specs = _jobs()[:4]
    with Server(nslots=3) as probe:
        js = [_submit(probe, sp) for sp in specs]
        ref = []
        for j in js:
            probe.wait(j)
            ref.append(j.xa.copy())
        fps = [j.result["device_bytes"] for j in js]
    budget = int(max(fps) * 1.2)
    with Server(nslots=3, hbm_budget=budget) as srv:
        jobs = [_submit(srv, sp) for sp in specs]
        for j, r in zip(jobs, ref):
            srv.wait(j)
            np.testing.assert_array_equal(j.xa, r)
        st = srv.stats()
    assert st["peak_bytes"] <= budget
    assert st["completed"] == len(specs)


def test_job_larger_than_the_budget_fails_cleanly(cuda):
    from letkf_gb300.lib import LETKF_ERR_CAPACITY, LetkfError
    from letkf_gb300.serve import Server

    with Server(nslots=2, hbm_budget=1 << 20) as srv:
        big = _submit(srv, _jobs()[2])
        small = _submit(srv, _l96(9, 40, 20, 0))
        with pytest.raises(LetkfError) as e:
            srv.wait(big)
        assert e.value.status == LETKF_ERR_CAPACITY
        assert srv.wait(small)["status"] == 0
        assert srv.stats()["failed"] == 1


def test_resident_domain_is_reused_across_cycles(cuda):
    """Two analysis cycles of one domain key: the second job reuses the device
    state and equals a fresh run of the same inputs."""
    from letkf_gb300.serve import PREC_MIXED, Server

    sp = _regional(11, 24, 20, 3, 40, 2500, PREC_MIXED)
    with Server(nslots=2) as srv:
        j1 = _submit(srv, sp, domain=7)
        srv.wait(j1)
        sp2 = dict(sp)
        sp2["case"] = dict(sp["case"])
        sp2["case"]["xb"] = j1.xa.copy()            # the next cycle starts from this analysis
        j2 = _submit(srv, sp2, domain=7)
        srv.wait(j2)
        assert srv.stats()["resident_domains"] == 1
        fresh = _submit(srv, sp2)
        srv.wait(fresh)
        np.testing.assert_array_equal(j2.xa, fresh.xa)
        # another L96 domain under a new key joins the resident set
        j3 = _submit(srv, _l96(12, 500, 20, 0), domain=8)
        srv.wait(j3)
        assert srv.stats()["resident_domains"] == 2


def test_l96_job_matches_the_oracle(cuda):
    """FP64 plain form through the server within 1e-10 of the oracle
    (lorenz96/letkf/letkf.f90:217-265 with fixed inflation 1.05)."""
    from letkf_gb300.serve import PREC_F64, Server

    sp = _l96(13, 200, 20, PREC_F64)
    with Server(nslots=2) as srv:
        j = _submit(srv, sp)
        srv.wait(j)
    nx, ne = sp["xf"].shape
    h = np.eye(nx)
    xm = sp["xf"].sum(1) / ne
    ref = np.zeros_like(sp["xf"])
    for ix in range(1, nx + 1):
        idx, rl = O.l96_select(h, ix, 3.0)
        r = O.letkf_core(sp["hdxf"][idx], np.ones(idx.size), rl, sp["dep"][idx], 1.05)
        ref[ix - 1] = xm[ix - 1] + (sp["xf"][ix - 1] - xm[ix - 1]) @ r["trans"]
    err = np.abs(j.xa - ref).max() / np.abs(ref).max()
    assert err < 1e-10, err
