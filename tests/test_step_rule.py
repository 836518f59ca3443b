"""The overdamped BD step rule: r += -(D dt/kT) g + sqrt(2 D dt) xi is stable
while (D dt/kT) lambda_max < 2, lambda_max the largest eigenvalue of the
energy's Hessian. On a stiff vesicle (icosahedron subdivided 5x at R 55 A
with 0.01 R radial noise, kc 23.5 kT: edges of 1.8 A, lambda_max near 2.5e3
kcal/mol/A^2) the rule's step (the drift coefficient times lambda_max equal
to 1) runs, and 2.5 times it (6.25, past the linear bound of 2) diverges in
both arithmetic forms: the limit is the integrator's, not the precision's.
(Just past the bound the stiffest modes grow into the energy's nonlinear
range and can saturate, so the test does not sit at the bound itself.)"""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from umcp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_step_rule_separates_stable_and_unstable_steps(tmp_path):
    ctx = U.Context(0)
    path = tmp_path / "stiff.mesh"
    U.generate_icosphere(path, 5, 55.0, 0.55, 41)
    prm64 = U.params(kc=U.kc_from_kT(23.5), KA=0.215)
    plan = U.Plan(path, prm64)
    lam = W.hessian_lambda_max(U.Mesh(ctx, plan, prm64), plan.positions())
    assert 1e3 < lam < 1e4
    rms = W.stable_rms_step(lam)
    for precision in (U.FP64, U.FP32_CENTRED):
        prm = U.params(kc=U.kc_from_kT(23.5), KA=0.215, precision=precision)
        e = U.Mesh(ctx, U.Plan(path, prm), prm).run(W.bd_integrator(5, 0, rms), 0, 300)
        assert np.all(np.isfinite(e))
        it = W.bd_integrator(5, 0, 2.5 * rms)
        it.divergence_threshold = 1e5
        with pytest.raises(U.UmcpError, match="non-finite|diverged"):
            U.Mesh(ctx, U.Plan(path, prm), prm).run(it, 0, 300)
