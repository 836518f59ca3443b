"""Global area and volume restraints on the limit surface.

CPU: the oracle's gradient against central finite differences of its own
A, V and E_r. GPU: energy, gradient (including the box-scale slots), the
reported A and V, and restrained Langevin steps with the built mass, against
the oracle (plain FP64 path: 1e-10; FP32 form: 1e-6 in energy)."""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import load_case, rel_inf
from oracle import bridge as B
from oracle import restraints as OR

KA, KV = 0.2, 0.01


def _state(plan, seed=3, sigma=0.3, alpha=(1.01, 0.99, 1.02)):
    r = plan.positions()
    r[:-3] += np.random.default_rng(seed).normal(0, sigma, 3 * plan.nv)
    r[-3:] = alpha
    return r


def test_oracle_gradient_matches_finite_differences():
    plan, _, _ = load_case("ico2_plain")
    r = _state(plan)
    A0, V0 = OR.area_volume(plan, plan.positions())
    E, g, _, _ = OR.restraint(plan, r, KA, A0, KV, V0)
    rng = np.random.default_rng(0)
    for i in list(rng.choice(3 * plan.nv, 8, replace=False)) + [3 * plan.nv, 3 * plan.nv + 2]:
        h = 1e-5
        rp, rm = r.copy(), r.copy()
        rp[i] += h
        rm[i] -= h
        fd = (OR.restraint(plan, rp, KA, A0, KV, V0)[0] - OR.restraint(plan, rm, KA, A0, KV, V0)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g).max(), 1e-300), (i, fd, g[i])


def test_sphere_area_and_volume():
    plan, _, _ = load_case("ico4_plain")
    A, V = OR.area_volume(plan, plan.positions())
    R = 150.0
    assert abs(A - 4 * np.pi * R * R) <= 0.01 * 4 * np.pi * R * R
    assert abs(abs(V) - 4 / 3 * np.pi * R ** 3) <= 0.02 * 4 / 3 * np.pi * R ** 3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_restrained_energy_and_gradient_match_oracle(precision):
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico3_deformed", precision)
    mesh = U.Mesh(ctx, plan, prm)
    r = _state(plan)
    E0, g0 = mesh.energy_grad(r)
    mesh.restraints_set(K_area=KA, K_volume=KV)  # targets from the resident (reference) state
    A0, V0 = OR.area_volume(plan, plan.positions())
    E1, g1 = mesh.energy_grad(r)
    Er, gr, A, V = OR.restraint(plan, r, KA, A0, KV, V0)
    tol = 1e-10 if precision == U.FP64 else 1e-6
    a, v, e = mesh.restraints_get()
    assert abs(a - A) <= tol * A and abs(v - V) <= tol * abs(V)
    assert abs(e - Er) <= tol * max(Er, 1.0)
    assert abs((E1 - E0) - Er) <= tol * max(abs(E1), 1.0)
    gtol = 1e-10 if precision == U.FP64 else 2e-5
    assert rel_inf(g1 - g0, gr) <= gtol
    mesh.restraints_clear()
    E2, _ = mesh.energy_grad(r)
    assert E2 == E0


@pytest.mark.gpu
def test_restrained_langevin_with_mass_matches_oracle():
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    mesh.mass_build(plan)
    mesh.restraints_set(K_area=KA, area0=0.98 * OR.area_volume(plan, plan.positions())[0], K_volume=KV)
    A0 = 0.98 * OR.area_volume(plan, plan.positions())[0]
    V0 = OR.area_volume(plan, plan.positions())[1]
    it = U.integrator(U.LANGEVIN, time_step=1e-15, gamma=10.0, seed=5, stream=2, use_mass=1)
    e_gpu = mesh.run(it, 0, 3)
    r_gpu, _ = mesh.state_get()
    minv = mesh.mass_get()
    row_ptr = np.arange(0, plan.nv * plan.nv + 1, plan.nv, dtype=np.int32)
    cols = np.tile(np.arange(plan.nv, dtype=np.int32), plan.nv)
    O = B.Oracle(plan, prm)
    r = plan.positions()
    p = np.zeros(3 * plan.nv)
    for s in range(3):
        Er, gr, _, _ = OR.restraint(plan, r, KA, A0, KV, V0)
        assert abs(e_gpu[s] - (O.energy(r) + Er)) <= 1e-10 * abs(e_gpu[s])
        g = O.grad(r) + gr
        xi = B.noise(5, 2, s, plan.nv)
        rv = r[:-3].copy()
        B.step(U.LANGEVIN, 1e-15, 10.0, U.KCAL_MOL_PER_KT_298, 0.0, rv, p, g[:-3], xi,
               mass=(row_ptr, cols, minv.reshape(-1)))
        r[:-3] = rv
    assert np.max(np.abs(r_gpu - r)) <= 1e-9 * np.max(np.abs(r))


@pytest.mark.gpu
def test_volume_restraint_rejects_periodic_meshes_and_batches():
    ctx = U.Context(0)
    plan, prm, _ = load_case("planar12_deformed")
    mesh = U.Mesh(ctx, plan, prm)
    with pytest.raises(U.UmcpError, match="closed surface"):
        mesh.restraints_set(K_volume=KV)
    mesh.restraints_set(K_area=KA)
    b = U.Batch(ctx, U.FP64)
    with pytest.raises(U.UmcpError):
        b.add(mesh, U.integrator(U.OVERDAMPED_BD, D=0.001), 0, 10)
