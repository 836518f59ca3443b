"""The oracle's own plan construction (oracle/planner.py), which lets the CPU
reference arm run without any engine code, pinned against the reference's
own plan dumps and outputs (tests/golden, written by the reference's code):

  control-point lists: identical; g0 at every point: to 1e-13 relative;
  energy with the reference's basis rows: to 1e-12 relative; gradient: to
  1e-11 of max|g|; the workload's vesicle generator: the committed mesh files
  (positions to 1e-12 relative, rings identical).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, rel_inf
from oracle import planner as P


def _surface(name):
    kv, lip = {}, []
    for ln in (GOLDEN / f"{name}.params").read_text().splitlines():
        f = ln.split()
        if not f:
            continue
        if f[0].lower() == "lipid":
            lip.append(ln)
        else:
            kv[f[0].lower()] = float(f[1])
    return P.Surface(P.read_mesh(GOLDEN / f"{name}.mesh"), kv.get("kc", 14.0), kv.get("ka", 0.215),
                     kv.get("kg", 0.0), kv.get("k_reg", 0.0), "\n".join(lip) if lip else None)


@pytest.mark.parametrize("name", [n for n in golden_cases() if "reg_cp" in np.load(GOLDEN / f"{n}.npz")])
def test_oracle_plan_matches_reference_plan(name):
    S = _surface(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    assert np.array_equal(S.reg_cp, gold["reg_cp"])
    assert np.max(np.abs(S.reg_g0 - gold["reg_g0"])) <= 1e-13 * np.abs(gold["reg_g0"]).max()
    if "irr_cp" in gold:
        assert np.array_equal(S.irr_cp[:, :11], gold["irr_cp"][:, :11])
        assert np.max(np.abs(S.irr_g0 - gold["irr_g0"])) <= 1e-13 * np.abs(gold["irr_g0"]).max()


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_plan_energy_and_gradient_match_reference(name):
    S = _surface(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    assert abs(S.energy(gold["r"]) - gold["E"]) <= 1e-12 * abs(gold["E"])
    assert rel_inf(S.grad(gold["r"]), gold["grad"]) <= 1e-11


@pytest.mark.parametrize("name,level,R,sigma,seed", [("ico2_plain", 2, 100.0, 1.0, 1001),
                                                     ("ico3_plain", 3, 100.0, 1.0, 1001),
                                                     ("ico4_plain", 4, 150.0, 1.5, 1004)])
def test_oracle_vesicle_generator_matches_mesh_files(name, level, R, sigma, seed):
    a, b = P.icosphere(level, R, sigma, seed), P.read_mesh(GOLDEN / f"{name}.mesh")
    assert a.rings == b.rings and np.array_equal(a.box, b.box)
    assert np.max(np.abs(a.r - b.r)) <= 1e-12 * np.abs(b.r).max()
