"""Host-side logic of the engine library (no GPU needed): the C ABI loads and
exports every symbol include/umcp_gpu.h declares, mesh generation and parsing,
plan errors, parameter parsing."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import umcp_gb300 as U

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    text = (ROOT / "include" / "umcp_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(umcp_[a-z_0-9]+)\s*\(", text))


def test_library_exports_every_declared_symbol():
    lib = U.library()
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing
    assert declared_symbols() == set(U.exported_symbols())


def test_status_strings_and_last_error():
    lib = U.library()
    assert lib.umcp_status_string(0) == b"ok"
    h = C.c_void_p()
    st = lib.umcp_plan_from_file(b"/nonexistent/x.mesh", None, C.byref(h))
    assert st == 2 and b"cannot open" in lib.umcp_last_error()


def test_icosphere_counts(tmp_path):
    for level, nv in [(1, 42), (2, 162), (3, 642)]:
        p = tmp_path / f"i{level}.mesh"
        U.generate_icosphere(p, level, 50.0, 0.0, 1)
        plan = U.Plan(p)
        assert plan.nv == nv
        assert plan.n_regular + plan.n_irregular == 2 * nv - 4
        assert plan.n_irregular == 60
        r = plan.positions()[:-3].reshape(-1, 3)
        assert np.allclose(np.linalg.norm(r, axis=1), 50.0)


def test_planar_counts_and_periodic_images(tmp_path):
    p = tmp_path / "pl.mesh"
    U.generate_planar(p, 8, 8, 10.0, 20.0, 3)
    plan = U.Plan(p)
    assert plan.nv == 64 and plan.n_regular == 128 and plan.n_irregular == 0
    reg = plan.faces(0)
    assert np.abs(reg["img"]).max() == 1  # some one-rings wrap across the box


def test_noise_is_seeded(tmp_path):
    a, b, c = tmp_path / "a.mesh", tmp_path / "b.mesh", tmp_path / "c.mesh"
    U.generate_icosphere(a, 2, 100.0, 1.0, 5)
    U.generate_icosphere(b, 2, 100.0, 1.0, 5)
    U.generate_icosphere(c, 2, 100.0, 1.0, 6)
    assert a.read_text() == b.read_text() and a.read_text() != c.read_text()


def test_rejects_adjacent_irregular_vertices(tmp_path):
    p = tmp_path / "ico0.mesh"
    # a bare icosahedron: every vertex has valence 5, so faces touch two irregular corners
    lines = (ROOT / "tests" / "golden" / "ico2_plain.mesh").read_text().splitlines()[:4]
    phi = (1 + 5 ** 0.5) / 2
    pts = np.array([[0, 1, phi], [0, -1, phi], [0, 1, -phi], [0, -1, -phi], [1, phi, 0], [-1, phi, 0],
                    [1, -phi, 0], [-1, -phi, 0], [phi, 0, 1], [-phi, 0, 1], [phi, 0, -1], [-phi, 0, -1]])
    d = np.linalg.norm(pts[:, None] - pts[None], axis=2)
    rows = []
    for i in range(12):
        nb = [j for j in range(12) if abs(d[i, j] - 2.0) < 1e-9]
        # order the ring around the outward normal
        n = pts[i] / np.linalg.norm(pts[i])
        e1 = pts[nb[0]] - pts[i]
        e1 -= n * (e1 @ n)
        e2 = np.cross(n, e1)
        ang = [np.arctan2((pts[j] - pts[i]) @ e2, (pts[j] - pts[i]) @ e1) for j in nb]
        nb = [x for _, x in sorted(zip(ang, nb))]
        rows.append(f"{i} {pts[i][0]} {pts[i][1]} {pts[i][2]} 5 " + " ".join(map(str, nb)))
    p.write_text("\n".join(lines + rows) + "\n")
    with pytest.raises(U.UmcpError, match="illegal mesh"):
        U.Plan(p)


def test_rejects_bad_valence(tmp_path):
    src = (ROOT / "tests" / "golden" / "ico2_plain.mesh").read_text().splitlines()
    parts = src[4].split()
    parts[4] = "4"
    src[4] = " ".join(parts[:9])
    p = tmp_path / "bad.mesh"
    p.write_text("\n".join(src) + "\n")
    with pytest.raises(U.UmcpError, match="valence"):
        U.Plan(p)


def test_params_from_input_text():
    lib = U.library()
    p = U.params()
    buf = C.create_string_buffer(4096)
    txt = b"mesh x.mesh\nkc 20.5\nKA -1\nkg -2\nT 310\nlipid library Lo 68.3 0.01\nlipid outer Lo 1\n"
    assert lib.umcp_params_from_input(txt, C.byref(p), buf, 4096) == 0
    assert (p.kc, p.KA, p.kg, p.temperature) == (20.5, 0.215, -2.0, 310.0)
    assert b"lipid outer Lo 1" in buf.value


def test_lipid_directives_set_composition(tmp_path):
    mesh = ROOT / "tests" / "golden" / "ico2_lipids.mesh"
    prm = U.params(lipids="lipid library Lo 68.3 0.01\nlipid library Li 68.3 -0.01\nlipid outer Lo 1\nlipid inner Li 1\n")
    plan = U.Plan(mesh, prm)
    c0, apl = plan.lipids()
    assert list(c0) == [0.01, -0.01] and list(apl) == [68.3, 68.3]
    f = plan.faces(0)
    assert np.all(f["outer"][:, 1] == 0) and np.all(f["inner"][:, 0] == 0)
    assert np.all(f["outer"][:, 0] > 0) and np.all(f["inner"][:, 1] > 0)
