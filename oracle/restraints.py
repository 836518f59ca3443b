"""ORACLE - test infrastructure, not product code.

numpy restatement of the global area/volume restraint terms on the limit
surface (no reference counterpart as an energy: the reference only measures
area and volume, src/interpLib.C:4355, src/volume.C): at every quadrature
point of every face, with X the face's control points (lattice images
applied, box scales alpha),
  A = sum dudv w |Ru x Rv|,   V = 1/3 sum dudv w R.(Ru x Rv),
  E_r = 1/2 K_A (A - A0)^2 / A0 + 1/2 K_V (V - V0)^2,
and dE_r/dr (3 nv + 3: vertices, then the box scales). Basis rows and face
tables come from the engine's planner (pinned against the reference by the
golden tests). Imported only by tests/.
"""
from __future__ import annotations

import numpy as np


def _faces(plan):
    out = []
    for kind in (0, 1):
        F = plan.faces(kind)
        n = plan.n_regular if kind == 0 else plan.n_irregular
        for f in range(n):
            val = 6 if kind == 0 else int(F["valence"][f])
            ncp = val + 6
            out.append((F["cp"][f, :ncp], F["img"][f, :ncp, :].astype(float), val, 0.5 if kind == 0 else 1.0))
    return out


def area_volume(plan, r, grad=False):
    """A, V (and dA/dr, dV/dr over 3 nv + 3 entries when grad)."""
    nv = plan.nv
    alpha = r[3 * nv:3 * nv + 3]
    box = plan.box
    bases = {}
    A = V = 0.0
    gA = np.zeros(3 * nv + 3)
    gV = np.zeros(3 * nv + 3)
    for cp, img, val, dudv in _faces(plan):
        if val not in bases:
            bases[val] = plan.basis(val)
        b = bases[val]
        Y = r[:3 * nv].reshape(nv, 3)[cp] + img @ box  # unscaled, images applied
        X = Y * alpha[None, :]
        for p in range(len(b["weight"])):
            bw, bu, bv = b["rows"][0, p], b["rows"][1, p], b["rows"][2, p]
            R, Ru, Rv = bw @ X, bu @ X, bv @ X
            m = np.cross(Ru, Rv)
            g = np.linalg.norm(m)
            c = dudv * b["weight"][p]
            A += c * g
            V += c / 3.0 * R.dot(m)
            if grad:
                n = m / g
                dA_dRu, dA_dRv = c * np.cross(Rv, n), c * np.cross(n, Ru)
                dV_dR, dV_dRu, dV_dRv = c / 3.0 * m, c / 3.0 * np.cross(Rv, R), c / 3.0 * np.cross(R, Ru)
                GA = np.outer(bu, dA_dRu) + np.outer(bv, dA_dRv)  # dA/dX [ncp][3]
                GV = np.outer(bw, dV_dR) + np.outer(bu, dV_dRu) + np.outer(bv, dV_dRv)
                for x, v in enumerate(cp):
                    gA[3 * v:3 * v + 3] += GA[x] * alpha
                    gV[3 * v:3 * v + 3] += GV[x] * alpha
                gA[3 * nv:] += (GA * Y).sum(0)
                gV[3 * nv:] += (GV * Y).sum(0)
    return (A, V, gA, gV) if grad else (A, V)


def restraint(plan, r, KA, A0, KV, V0):
    """E_r and dE_r/dr."""
    A, V, gA, gV = area_volume(plan, r, grad=True)
    E = 0.5 * KA * (A - A0) ** 2 / A0 + 0.5 * KV * (V - V0) ** 2
    g = KA * (A - A0) / A0 * gA + KV * (V - V0) * gV
    return E, g, A, V
