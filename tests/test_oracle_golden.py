"""The oracle and the host planner against the reference's own outputs
(golden fixtures made by tests/golden/make_golden.py from the reference
sources compiled here). CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, load_case, rel_inf
from oracle import bridge as B

E_TOL = 1e-12   # relative; the restatement sums in a different order only
G_TOL = 1e-11   # max|dg| / max|g|


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_energy_matches_reference(name):
    plan, prm, gold = load_case(name)
    O = B.Oracle(plan, prm)
    E, t = O.energy(gold["r"], terms=True)
    assert abs(E - gold["E"]) <= E_TOL * abs(gold["E"])
    for got, want in zip(t, (gold["VA"], gold["VC"], gold["VR"])):
        assert abs(got - want) <= E_TOL * abs(gold["E"])


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_gradient_matches_reference(name):
    plan, prm, gold = load_case(name)
    g = B.Oracle(plan, prm).grad(gold["r"])
    assert rel_inf(g[:-3], gold["grad"][:-3]) <= G_TOL
    assert np.allclose(g[-3:], gold["grad"][-3:], rtol=1e-10, atol=1e-10 * np.abs(gold["grad"]).max())


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_face_energies_match_reference(name):
    plan, prm, gold = load_case(name)
    _, fe = B.Oracle(plan, prm).energy(gold["r"], per_face=True)
    # the engine lists regular faces then irregular ones, both in generatePlan order
    assert fe.shape == gold["face_energy"].shape
    assert np.max(np.abs(fe - gold["face_energy"])) <= 1e-11 * np.abs(gold["face_energy"]).max()


@pytest.mark.parametrize("name", [n for n in golden_cases() if "reg_cp" in np.load(f"tests/golden/{n}.npz")])
def test_planner_matches_reference_plan(name):
    plan, prm, gold = load_case(name)
    val, ring = plan.rings()
    assert np.array_equal(val, gold["valence"]) and np.array_equal(ring, gold["ring"])
    reg = plan.faces(0)
    assert np.array_equal(reg["cp"][:, :12], gold["reg_cp"])
    assert rel_inf(reg["g0"], gold["reg_g0"]) <= 1e-13
    b6 = plan.basis(6)
    # golden rows are [pt][kind][cp]
    assert np.max(np.abs(b6["rows"].transpose(1, 0, 2) - gold["reg_rows"])) <= 1e-14
    assert np.allclose(b6["weight"], gold["reg_w"], rtol=0, atol=1e-16)
    if "irr_cp" in gold:
        irr = plan.faces(1)
        assert np.array_equal(irr["cp"], gold["irr_cp"])
        assert rel_inf(irr["g0"], gold["irr_g0"]) <= 1e-12
        val0 = int(irr["valence"][0])
        b = plan.basis(val0)
        assert np.max(np.abs(b["rows"].transpose(1, 0, 2) - gold["irr_rows"])) <= 1e-11 * np.abs(gold["irr_rows"]).max()
        assert np.allclose(b["weight"], gold["irr_w"], rtol=1e-12)


def test_reference_fd_acceptance_on_oracle():
    """Central differences as the reference's own fdiff_check_grad judges them
    (src/grad.C:25-63: eps 1e-5, OK if relative error < 1e-3 or absolute < 1e-7)."""
    plan, prm, gold = load_case("ico2_lipids")
    O = B.Oracle(plan, prm)
    r = gold["r"].copy()
    g = O.grad(r)
    rng = np.random.default_rng(3)
    for i in rng.choice(3 * plan.nv, 40, replace=False):
        rp, rm = r.copy(), r.copy()
        rp[i] += 1e-5
        rm[i] -= 1e-5
        fd = (O.energy(rp) - O.energy(rm)) / 2e-5
        rel = 2 * abs(fd - g[i]) / (abs(fd) + abs(g[i]))
        assert rel < 1e-3 or abs(fd - g[i]) < 1e-7
