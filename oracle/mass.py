"""ORACLE - test infrastructure, not product code.

numpy restatement of the reference's effective mass (getSparseEffectiveMass,
src/modes.C:1719-1990, with the mass points of src/hd.C:417-481): mass
points on a (p+1)(p+2)/2 grid per face, mass per point from area0 (the
reference area as surface::area sums it, src/interpLib.C:4413-4601),
M = sum_k m c_k c_k^T, inverse by Cholesky,
rel_tol truncation. The limit-point weights c_k come from the engine's
planner (Plan.point_coeffs), which the tests pin separately against the
reference's own weights. Imported only by tests/.
"""
from __future__ import annotations

import numpy as np

AMU_PER_KG = 1.0 / 1.661e-27  # src/units.h:4


def area0(plan) -> float:
    """surface::area's area0: 0.5 g0 w over the regular faces' points plus
    g0 w over the irregular faces' points (src/interpLib.C:4413-4601)."""
    reg = plan.faces(0)
    a = float(np.sum(0.5 * reg["g0"].reshape(-1, 15) * plan.basis(6)["weight"][None, :]))
    if plan.n_irregular:
        irr = plan.faces(1)
        g0 = irr["g0"].reshape(-1, 16)
        for f in range(plan.n_irregular):
            a += float(np.sum(g0[f] * plan.basis(int(irr["valence"][f]))["weight"]))
    return a


def mass_per_point(plan, mass_scale: float = 5.0, plim: int = 10) -> float:
    ppf = (plim + 1) * (plim + 2) // 2
    mass_per_lipid = mass_scale * 1000 * 760.09 / 6.022e23 / 1000
    nfaces = plan.n_regular + plan.n_irregular
    return AMU_PER_KG * 2 * area0(plan) / nfaces / ppf * mass_per_lipid / 65.35


def effective_mass(plan, mass_scale: float = 5.0, plim: int = 10) -> np.ndarray:
    m = mass_per_point(plan, mass_scale, plim)
    M = np.zeros((plan.nv, plan.nv))
    for f in range(plan.n_regular + plan.n_irregular):
        for fi in range(plim + 1):
            for fj in range(plim + 1 - fi):
                ids, c = plan.point_coeffs(f, fi / plim, fj / plim)
                np.add.at(M, (ids[:, None], ids[None, :]), m * np.outer(c, c))
    return M


def inverse(M: np.ndarray, rel_tol: float = 1e-20) -> np.ndarray:
    L = np.linalg.cholesky(M)
    Li = np.linalg.inv(L)
    Minv = Li.T @ Li
    d = np.sqrt(np.abs(np.outer(np.diag(Minv), np.diag(Minv))))
    return np.where(np.abs(Minv) / d > rel_tol, Minv, 0.0)
