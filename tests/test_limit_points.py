"""Limit-surface points and normals (surface::evaluateRNRM,
src/interpLib.C:7936) against the reference's own evaluation
(tests/golden/<case>.rnrm.npz from the reference-built oracle): regular and
irregular faces, box scales, periodic images."""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import GOLDEN, load_case


@pytest.mark.parametrize("name", ["ico2_lipids", "planar12_deformed"])
def test_points_and_normals_match_reference(name):
    plan, _, gold = load_case(name)
    rows = np.load(GOLDEN / f"{name}.rnrm.npz")["rows"]
    R, N = plan.evaluate(gold["r"], rows[:, 0].astype(int), rows[:, 1:3])
    scale = np.abs(rows[:, 3:6]).max()
    assert np.max(np.abs(R - rows[:, 3:6])) <= 1e-13 * scale
    assert np.max(np.abs(N - rows[:, 6:9])) <= 1e-12


def test_extraordinary_vertex_point_and_bad_queries():
    plan, _, gold = load_case("ico2_plain")
    f = plan.n_regular  # an irregular face: (0,0) is its valence-5 vertex
    R, N = plan.evaluate(gold["r"], [f], [(0.0, 0.0)])
    ids, c = plan.point_coeffs(f, 0.0, 0.0)
    r = gold["r"]
    assert np.allclose(R[0], sum(ci * r[3 * i:3 * i + 3] for i, ci in zip(ids, c)) * r[-3:], rtol=1e-14)
    assert np.all(np.isnan(N[0]))
    with pytest.raises(U.UmcpError):
        plan.evaluate(gold["r"], [plan.n_regular + plan.n_irregular], [(0.1, 0.1)])
