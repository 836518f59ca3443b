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


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ico2_lipids", "planar12_deformed"])
def test_device_limit_points_and_writer(tmp_path, name):
    """umcp_limit_points on the device equals the host evaluation (which the
    test above pins to the reference) at every face's lattice; the writer
    writes the reference's xyz layout with each face's three corners."""
    plan, prm, gold = load_case(name)
    ctx = U.Context(0)
    mesh = U.Mesh(ctx, plan, prm)
    mesh.state_set(gold["r"])
    plim = 3
    R, N = mesh.limit_points(plim)
    nf = plan.n_regular + plan.n_irregular
    uv = [(i / plim, j / plim) for i in range(plim + 1) for j in range(plim + 1 - i)]
    faces = np.repeat(np.arange(nf), len(uv))
    Rh, Nh = plan.evaluate(gold["r"], faces, np.tile(uv, (nf, 1)))
    assert np.max(np.abs(R.reshape(-1, 3) - Rh)) <= 1e-12 * np.abs(Rh).max()
    ok = np.isfinite(Nh)
    assert np.array_equal(ok, np.isfinite(N.reshape(-1, 3)))
    assert np.max(np.abs(N.reshape(-1, 3)[ok] - Nh[ok])) <= 1e-12
    out = tmp_path / "limit.xyz"
    mesh.write_limiting_surface(out)
    lines = out.read_text().splitlines()
    assert lines[0] == str(3 * nf) and lines[1] == "limiting surface" and len(lines) == 2 + 3 * nf
    corners = np.array([[float(x) for x in ln.split()[1:]] for ln in lines[2:]])
    Rc, _ = plan.evaluate(gold["r"], np.repeat(np.arange(nf), 3), np.tile([(0, 0), (0, 1), (1, 0)], (nf, 1)))
    assert all(ln.startswith("C ") for ln in lines[2:]) and np.max(np.abs(corners - Rc)) <= 5e-7
