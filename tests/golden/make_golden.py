"""Generates the golden fixtures in this directory from the REFERENCE's own
code (oracle/_ref/ref_driver, built from the reference sources by
oracle/ref/Makefile). Run where the reference tree exists:

    python tests/golden/make_golden.py

Each case writes <name>.mesh (the input mesh, full-precision positions),
<name>.params (the reference's input keywords) and <name>.npz with the
reference's energy terms, gradient, evaluation positions, per-face energies
and, for small meshes, its plan tables (control points, basis rows, g0).

`--rnrm` writes <name>.rnrm.npz for RNRM_CASES: the reference's limit
points and normals on every face. `--sub6` writes sub6.npz: the reference's regular-patch subdivision
stencils. `--mass` writes <name>.mass.npz for the MASS_CASES instead, from the existing
mesh and params files: the reference's inverse effective mass (dense), its
mass per point and area0, and the limit-surface weights of the 66 mass
points of four faces (two regular, two irregular where there are any).
`--min` writes <name>.min.npz for MIN_CASES: the reference's own L-BFGS
minimization (100 iterations from the case's evaluation state), the energy
before and after every iteration and the final state.
"""
from __future__ import annotations

import sys
import zlib
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import umcp_gb300 as U  # noqa: E402
from oracle import bridge as B  # noqa: E402

KC20 = U.kc_from_kT(20.0)  # 20 kT at 298 K

# name, generator, params text, deformation (sigma of vertex displacement, alphas), keep plan tables
CASES = [
    ("ico2_plain", ("ico", 2, 100.0, 1.0, 1001), f"kc {KC20}\nKA 0.215\n", None, True),
    ("ico3_plain", ("ico", 3, 100.0, 1.0, 1001), f"kc {KC20}\nKA 0.215\n", None, False),
    ("ico3_deformed", ("ico", 3, 100.0, 1.0, 1001), f"kc {KC20}\nKA 0.215\nkg -3.0\nk_reg 0.5\n", (0.3, (1.01, 0.99, 1.02)), False),
    ("ico2_lipids", ("ico", 2, 60.0, 0.6, 7), f"kc {KC20}\nKA 0.215\nlipid library Lo 68.3 0.01\nlipid library Li 68.3 -0.01\n"
     "lipid outer Lo 1\nlipid inner Li 1\n", (0.2, (1.0, 1.0, 1.0)), False),
    ("planar12_deformed", ("planar", 12, 12, 10.0, 20.0, 1002), f"kc {KC20}\nKA 0.215\nk_reg 0.2\n", (0.05, (1.003, 0.998, 1.0)), True),
    ("ico4_plain", ("ico", 4, 150.0, 1.5, 1004), f"kc {KC20}\nKA 0.215\n", (0.2, (1.0, 1.0, 1.0)), False),
]


def _read_formulas(path: Path, nfaces: int, npt: int):
    raw = path.read_bytes()
    off = 0
    cps, g0, rows, w = [], [], [], []
    for _ in range(nfaces * npt):
        n, _tri = np.frombuffer(raw, dtype=np.int32, count=2, offset=off)
        off += 8
        cp = np.frombuffer(raw, dtype=np.int32, count=n, offset=off)
        off += 4 * n
        d3 = np.frombuffer(raw, dtype=np.float64, count=3, offset=off)
        off += 24
        off += 24 * n  # r_pbc
        rw = np.frombuffer(raw, dtype=np.float64, count=6 * n, offset=off).reshape(6, n)
        off += 48 * n
        cps.append(cp.copy())
        w.append(d3[0])
        g0.append(d3[1])
        rows.append(rw.copy())
    return cps, np.array(w), np.array(g0), rows


def make_case(name, gen, params_txt, deform, keep_plan, work: Path) -> None:
    mesh = HERE / f"{name}.mesh"
    if gen[0] == "ico":
        U.generate_icosphere(mesh, gen[1], gen[2], gen[3], gen[4])
    else:
        U.generate_planar(mesh, gen[1], gen[2], gen[3], gen[4], gen[5])
    (HERE / f"{name}.params").write_text(params_txt)
    plan = U.Plan(mesh)
    r = plan.positions()
    positions = None
    if deform is not None:
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        r[:-3] += rng.normal(0.0, deform[0], 3 * plan.nv)
        r[-3:] = deform[1]
        positions = work / f"{name}.r.bin"
        r.tofile(positions)
    prefix = work / name
    ref = B.reference_dump(mesh, HERE / f"{name}.params", positions, prefix)
    out = {
        "E": ref["E"], "VA": ref["VA"], "VC": ref["VC"], "VR": ref["VR"], "grad": ref["grad"], "r": ref["positions"],
        "face_energy": ref["face_energy"], "nf_faces": ref["nf_faces"], "nf_irr_faces": ref["nf_irr_faces"],
    }
    if keep_plan:
        cps, w, g0, rows = _read_formulas(Path(f"{prefix}.plan_reg.bin"), ref["nf_faces"], 15)
        out["reg_cp"] = np.array(cps[::15], dtype=np.int32)
        out["reg_g0"] = g0.reshape(-1, 15)
        out["reg_rows"] = np.array(rows[:15])  # the shared regular basis, [pt][kind][cp]
        out["reg_w"] = w[:15]
        if ref["nf_irr_faces"]:
            cps, w, g0, rows = _read_formulas(Path(f"{prefix}.plan_irr.bin"), ref["nf_irr_faces"], 16)
            out["irr_cp"] = np.array([np.pad(c, (0, 13 - len(c)), constant_values=-1) for c in cps[::16]], dtype=np.int32)
            out["irr_g0"] = g0.reshape(-1, 16)
            out["irr_rows"] = np.array(rows[:16])  # basis of the first irregular face's valence
            out["irr_w"] = w[:16]
        val, ring = [], []
        for line in Path(f"{prefix}.edges.txt").read_text().splitlines():
            f = [int(x) for x in line.split()]
            val.append(f[1])
            ring.extend(f[2:])
        out["valence"] = np.array(val, dtype=np.int32)
        out["ring"] = np.array(ring, dtype=np.int32)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: nv={plan.nv} E={ref['E']:.12g}")


MASS_CASES = ["ico2_plain", "planar12_deformed"]


RNRM_CASES = ["ico2_lipids", "planar12_deformed"]


MIN_CASES = ["ico2_lipids", "planar12_deformed"]


def make_min_case(name: str, work: Path) -> None:
    """The reference's minimization from the case's evaluation state."""
    r = np.load(HERE / f"{name}.npz")["r"]
    pos = work / f"{name}.r.bin"
    r.tofile(pos)
    ref = B.reference_min(HERE / f"{name}.mesh", HERE / f"{name}.params", pos, work / name)
    np.savez_compressed(HERE / f"{name}.min.npz", energies=ref["energies"], r=ref["r"])
    print(f"{name}: {len(ref['energies']) - 1} iterations, E {ref['energies'][0]:.12g} -> {ref['energies'][-1]:.12g}")


def make_rnrm(name: str, work: Path) -> None:
    """The reference's limit points and normals (evaluateRNRM) on every face of
    the case's evaluation state."""
    r = np.load(HERE / f"{name}.npz")["r"]
    pos = work / f"{name}.r.bin"
    r.tofile(pos)
    rows = B.reference_rnrm(HERE / f"{name}.mesh", HERE / f"{name}.params", pos, work / name)
    np.savez_compressed(HERE / f"{name}.rnrm.npz", rows=rows)
    print(f"{name}: {len(rows)} limit points")


def make_sub6(work: Path) -> None:
    """The reference's four regular-patch subdivision stencils (fast_sub6_k),
    as 12 x 12 matrices per child (the same for x, y and z)."""
    S = B.reference_sub6(work / "s")
    np.savez_compressed(HERE / "sub6.npz", stencils=S)
    print("sub6: 4 stencils")


def make_mass_case(name: str, work: Path) -> None:
    ref = B.reference_mass(HERE / f"{name}.mesh", HERE / f"{name}.params", work / name)
    pts = ref["points"]
    nreg = int(np.load(HERE / f"{name}.npz")["nf_faces"])
    faces = [0, 1] + ([nreg, nreg + 1] if pts["face"].max() >= nreg else [])
    keep = pts[np.isin(pts["face"], faces)]
    np.savez_compressed(HERE / f"{name}.mass.npz", minv=ref["minv"], mass_per_pt=ref["mass_per_pt"],
                        area0=ref["area0"], npts=ref["npts"], pt_face=keep["face"], pt_n=keep["n"], pt_u=keep["u"],
                        pt_v=keep["v"], pt_ids=keep["ids"], pt_coef=keep["coef"])
    print(f"{name}: mass per point {ref['mass_per_pt']:.12g}, {len(keep)} points kept")


def main() -> None:
    if not B.reference_available():
        raise SystemExit("reference-built oracle missing; build it with __graft_entry__.build() where the reference exists")
    with tempfile.TemporaryDirectory() as td:
        if "--rnrm" in sys.argv:
            for name in RNRM_CASES:
                make_rnrm(name, Path(td))
            return
        if "--sub6" in sys.argv:
            make_sub6(Path(td))
            return
        if "--min" in sys.argv:
            for name in MIN_CASES:
                make_min_case(name, Path(td))
            return
        if "--mass" in sys.argv:
            for name in MASS_CASES:
                make_mass_case(name, Path(td))
            return
        for case in CASES:
            make_case(*case, Path(td))


if __name__ == "__main__":
    main()
