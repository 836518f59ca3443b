"""Serving: jobs submitted to the request loop while others run give the
same results they give alone (umcp_run on the job's mesh), whatever else
shares the device. Positions are compared bit for bit; energies to the FP32
form's 1e-6 (they are sums in a different order)."""
from __future__ import annotations

import time

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import GOLDEN, load_case

pytestmark = pytest.mark.gpu

E32 = 1e-6


@pytest.fixture(scope="module")
def ctx():
    return U.Context(0)


def _its():
    return [
        U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.00125, seed=31, stream=1),
        U.integrator(U.LANGEVIN, time_step=1e-15, gamma=10.0, seed=32, stream=2),
        U.integrator(U.BD_MEMBRANE, time_step=1e-15, gamma=10.0, seed=33, stream=3),
        U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.002, seed=34, stream=4),
    ]


JOBS = [  # (case, integrator index, step0, steps)
    ("ico3_deformed", 0, 0, 300),
    ("planar12_deformed", 1, 7, 90),
    ("ico2_lipids", 2, 0, 45),
    ("ico2_plain", 3, 100, 200),
    ("ico4_plain", 0, 5, 130),
    ("planar12_deformed", 3, 0, 64),
]


def _alone(ctx, case, it, step0, n, precision=U.FP32_CENTRED):
    plan, prm, _ = load_case(case, precision)
    m = U.Mesh(ctx, plan, prm)
    e = m.run(it, step0, n)
    return m.state_get()[0], e


def _submit_all(srv, its, gap_s=0.0):
    ids = []
    for case, k, step0, n in JOBS:
        _, prm, _ = load_case(case, U.FP32_CENTRED)
        ids.append(srv.submit(GOLDEN / f"{case}.mesh", prm, its[k], step0, n, keep_energies=True))
        if gap_s:
            time.sleep(gap_s)
    return ids


def _check_results(ctx, srv, ids, its):
    for jid, (case, k, step0, n) in zip(ids, JOBS):
        info = srv.job(jid)
        assert info.state == U.JOB_DONE and info.status == 0, info.message
        assert info.steps_done == n
        assert 0 <= info.t_submit <= info.t_admit <= info.t_done
        r, e = srv.fetch(jid)
        r0, e0 = _alone(ctx, case, its[k], step0, n)
        assert np.array_equal(r, r0), case
        assert np.max(np.abs(e - e0) / np.abs(e0)) <= E32


def test_jobs_in_the_mix_equal_their_alone_runs(ctx):
    its = _its()
    srv = U.Server(ctx, U.FP32_CENTRED, chunk_ms=2.0)
    ids = _submit_all(srv, its, gap_s=0.01)  # arrivals while earlier jobs run
    assert srv.wait_all(120.0)
    st = srv.stats()
    assert st.submitted == st.completed == len(JOBS) and st.failed == 0
    assert st.p50_latency_s > 0 and st.p99_latency_s >= st.p50_latency_s
    expected = 0
    for case, _, _, n in JOBS:
        expected += load_case(case, U.FP32_CENTRED)[0].nv * n
    assert st.vertex_steps == expected
    assert st.hbm_in_use_bytes == 0 and st.running == 0
    _check_results(ctx, srv, ids, its)
    srv.close()


def test_admission_respects_the_memory_budget(ctx):
    its = _its()
    biggest = max(load_case(c, U.FP32_CENTRED)[0].device_bytes(ctx, U.FP32_CENTRED, n) for c, _, _, n in JOBS)
    srv = U.Server(ctx, U.FP32_CENTRED, hbm_budget_bytes=biggest * 1.01, chunk_ms=2.0)
    ids = _submit_all(srv, its)
    assert srv.wait_all(120.0)
    st = srv.stats()
    assert st.completed == len(JOBS) and st.failed == 0
    assert st.hbm_peak_bytes <= biggest * 1.01
    # whenever a job was admitted, the footprints resident with it fit the budget
    infos = [srv.job(j) for j in ids]
    for a in infos:
        resident = [b for b in infos if b.t_admit <= a.t_admit < b.t_done]
        assert sum(b.device_bytes for b in resident) <= biggest * 1.01
    _check_results(ctx, srv, ids, its)
    srv.close()


def test_rejected_jobs_fail_alone(ctx):
    its = _its()
    small = load_case("ico2_plain", U.FP32_CENTRED)[0].device_bytes(ctx, U.FP32_CENTRED, 50)
    srv = U.Server(ctx, U.FP32_CENTRED, hbm_budget_bytes=small * 1.5)
    _, prm, _ = load_case("ico2_plain", U.FP32_CENTRED)
    _, prm4, _ = load_case("ico4_plain", U.FP32_CENTRED)
    ok = srv.submit(GOLDEN / "ico2_plain.mesh", prm, its[0], 0, 50)
    too_big = srv.submit(GOLDEN / "ico4_plain.mesh", prm4, its[0], 0, 50)
    missing = srv.submit(GOLDEN / "no_such.mesh", prm, its[0], 0, 50)
    assert srv.wait_all(60.0)
    assert srv.job(too_big).status == U.ERR_NOMEM
    assert srv.job(missing).status == 2 and b"no_such" in srv.job(missing).message
    info = srv.job(ok)
    assert info.status == 0 and info.steps_done == 50
    assert np.array_equal(srv.fetch(ok)[0], _alone(ctx, "ico2_plain", its[0], 0, 50)[0])
    srv.release(ok)
    with pytest.raises(U.UmcpError):
        srv.job(ok)
    srv.close()


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_footprint_matches_the_mesh(ctx, precision):
    for case in ("ico2_plain", "planar12_deformed", "ico4_plain"):
        plan, prm, _ = load_case(case, precision)
        m = U.Mesh(ctx, plan, prm)
        m.run(U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.00125, seed=1), 0, 37)
        assert plan.device_bytes(ctx, precision, 37) == m.info().device_bytes
