"""The effective mass built from the limit surface (getSparseEffectiveMass,
src/modes.C:1719-1990, mass points of src/hd.C:417-481).

CPU: the planner's limit-point weights at the reference's own mass points,
and the oracle's assembly and inverse built on them, against the
reference's dump (tests/golden/<case>.mass.npz, made by make_golden.py
--mass from oracle/_ref). GPU: umcp_mass_build against the same M^-1, and a
Langevin run through the built M^-1 against the oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import GOLDEN, load_case
from oracle import mass as OM

CASES = ["ico2_plain", "planar12_deformed"]


def _gold(name):
    return dict(np.load(GOLDEN / f"{name}.mass.npz"))


def _as_dict(ids, coef):
    d = {}
    for i, c in zip(ids, coef):
        if c != 0.0:
            d[int(i)] = d.get(int(i), 0.0) + float(c)
    return d


@pytest.mark.parametrize("name", CASES)
def test_limit_point_weights_match_reference(name):
    plan, _, _ = load_case(name)
    g = _gold(name)
    assert len(g["pt_face"]) >= 132
    for f, n, u, v, ids, coef in zip(g["pt_face"], g["pt_n"], g["pt_u"], g["pt_v"], g["pt_ids"], g["pt_coef"]):
        mine = _as_dict(*plan.point_coeffs(int(f), float(u), float(v)))
        ref = _as_dict(ids[:n], coef[:n])
        for k in set(mine) | set(ref):  # weights below rounding may be exact zeros on one side only
            assert abs(mine.get(k, 0.0) - ref.get(k, 0.0)) <= 1e-12, (f, u, v, k)


@pytest.mark.parametrize("name", CASES)
def test_oracle_effective_mass_matches_reference(name):
    plan, _, _ = load_case(name)
    g = _gold(name)
    assert abs(OM.area0(plan) - g["area0"]) <= 1e-12 * g["area0"]
    assert abs(OM.mass_per_point(plan) - g["mass_per_pt"]) <= 1e-12 * g["mass_per_pt"]
    minv = OM.inverse(OM.effective_mass(plan))
    assert np.max(np.abs(minv - g["minv"])) <= 1e-10 * np.max(np.abs(g["minv"]))


def test_point_weights_partition_unity_and_bad_points_fail():
    plan, _, _ = load_case("ico3_deformed")
    for f in (0, plan.n_regular, plan.n_regular + plan.n_irregular - 1):
        for u, v in ((0.0, 0.0), (0.3, 0.3), (1.0, 0.0), (0.0, 1.0), (0.05, 0.02)):
            _, c = plan.point_coeffs(f, u, v)
            assert abs(c.sum() - 1.0) <= 1e-13
    with pytest.raises(U.UmcpError):
        plan.point_coeffs(plan.n_regular + plan.n_irregular, 0.1, 0.1)
    with pytest.raises(U.UmcpError):
        plan.point_coeffs(0, 0.8, 0.8)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_device_mass_build_matches_reference(name):
    ctx = U.Context(0)
    plan, prm, _ = load_case(name)
    mesh = U.Mesh(ctx, plan, prm)
    info = mesh.mass_build(plan)
    g = _gold(name)
    assert info.dense == 1 and info.nnz_inverse == plan.nv * plan.nv
    assert abs(info.mass_per_point - g["mass_per_pt"]) <= 1e-12 * g["mass_per_pt"]
    minv = mesh.mass_get()
    assert np.max(np.abs(minv - g["minv"])) <= 1e-10 * np.max(np.abs(g["minv"]))
    assert np.array_equal(minv, minv.T)
    # M is assembled on the device: its sparsity is the oracle's, the build is
    # deterministic, and the three phases are timed
    assert info.nnz_mass == np.count_nonzero(OM.effective_mass(plan))
    assert min(info.assembly_s, info.inverse_s, info.truncation_s) > 0
    info2 = mesh.mass_build(plan)
    assert info2.nnz_mass == info.nnz_mass and np.array_equal(mesh.mass_get(), minv)


@pytest.mark.gpu
def test_truncated_inverse_is_stored_sparse():
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico3_plain")
    mesh = U.Mesh(ctx, plan, prm)
    info = mesh.mass_build(plan, rel_tol=0.02)
    ref = OM.inverse(OM.effective_mass(plan), rel_tol=0.02)
    assert info.dense == 0 and info.nnz_inverse == np.count_nonzero(ref)
    got = mesh.mass_get()
    assert np.array_equal(got != 0, ref != 0)
    assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [U.LANGEVIN, U.BD_MEMBRANE])
def test_leapfrog_with_built_mass_matches_oracle(kind):
    from oracle import bridge as B

    ctx = U.Context(0)
    plan, prm, _ = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    mesh.mass_build(plan)
    minv = _gold("ico2_plain")["minv"]
    rows, cols = np.nonzero(np.ones_like(minv))
    row_ptr = np.arange(0, plan.nv * plan.nv + 1, plan.nv, dtype=np.int32)
    it = U.integrator(kind, time_step=1e-15, gamma=10.0, seed=5, stream=2, use_mass=1)
    mesh.run(it, 0, 4)
    r_gpu, p_gpu = mesh.state_get()
    O = B.Oracle(plan, prm)
    r = plan.positions()
    p = np.zeros(3 * plan.nv)
    for s in range(4):
        g = O.grad(r)
        xi = B.noise(5, 2, s, plan.nv)
        rv = r[:-3].copy()
        B.step(kind, 1e-15, 10.0, U.KCAL_MOL_PER_KT_298, 0.0, rv, p, g[:-3], xi,
               mass=(row_ptr, cols.astype(np.int32), minv.reshape(-1)))
        r[:-3] = rv
    assert np.max(np.abs(r_gpu - r)) <= 1e-9 * np.max(np.abs(r))
    assert np.max(np.abs(p_gpu - p)) <= 1e-9 * max(np.max(np.abs(p)), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("rel_tol", [1e-20, 0.02])
def test_precision_form_applies_the_inverse_in_fp32(rel_tol):
    """A mesh of the FP32 form keeps M^-1 rounded once to FP32 (dense, or CSR
    when truncation leaves it sparse) and applies it with compensated FP32
    sums: within 1e-6 of sum_j |M^-1_ij| |x_j| of the FP64 apply."""
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico3_plain")
    _, prm32, _ = load_case("ico3_plain", U.FP32_CENTRED)
    m64 = U.Mesh(ctx, plan, prm)
    i64 = m64.mass_build(plan, rel_tol=rel_tol)
    m32 = U.Mesh(ctx, plan, prm32)
    i32 = m32.mass_build(plan, rel_tol=rel_tol)
    assert (i32.dense, i32.nnz_inverse) == (i64.dense, i64.nnz_inverse) and i32.dense == (rel_tol < 0.01)
    # the stored form and its column bytes: none when dense, 16-bit columns in the FP32 CSR, 32-bit in FP64
    assert m32.info().mass_form == m64.info().mass_form == (1 if i32.dense else 2)
    assert (i32.column_bytes, i64.column_bytes) == ((0, 0) if i32.dense else (2 * i32.nnz_inverse, 4 * i64.nnz_inverse))
    g = m64.mass_get()
    assert np.array_equal(m32.mass_get(), g.astype(np.float32).astype(np.float64))
    rng = np.random.default_rng(3)
    vin = rng.normal(0, 1, 3 * plan.nv)
    base = rng.normal(0, 1, 3 * plan.nv)
    scalev = rng.uniform(0.5, 2.0, 3 * plan.nv)
    bound = (np.abs(g) @ np.abs(vin.reshape(-1, 3))).reshape(-1)
    for sv, scale, al in [(None, 1.0, (1, 1, 1)), (scalev, -0.7, (1.01, 0.98, 1.2))]:
        want = m64.mass_apply(vin, base.copy(), sv, scale, al)
        got = m32.mass_apply(vin, base.copy(), sv, scale, al)
        f = abs(scale) / np.min(np.asarray(al)) ** 2 * (1.0 if sv is None else sv.reshape(3, -1).T.reshape(-1))
        assert np.all(np.abs(got - want) <= 1e-6 * f * bound + 1e-12 * np.abs(base))
