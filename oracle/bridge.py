"""ORACLE - test infrastructure, not product code.

ctypes bridge to the oracle's C restatement (oracle/umcp_oracle.c) and to the
reference-built driver (oracle/_ref/ref_driver, present only where the
reference tree was available at build time). Imported only by tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline leg, always as the checker.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "lib" / "libumcp_oracle.so"
REF_DRIVER = HERE / "_ref" / "ref_driver"

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_B = C.POINTER(C.c_int8)


class OracleSurface(C.Structure):
    _fields_ = [
        ("nv", C.c_int), ("box", C.c_double * 9), ("kc", C.c_double), ("KA", C.c_double), ("kg", C.c_double),
        ("k_reg", C.c_double), ("ntypes", C.c_int), ("lipid_c0", _D),
        ("nreg", C.c_int), ("reg_cp", _I), ("reg_img", _B), ("reg_rows", _D), ("reg_w", _D),
        ("reg_g0", _D), ("reg_rr0", _D), ("reg_outer", _D), ("reg_inner", _D),
        ("nirr", C.c_int), ("irr_val", _I), ("irr_cp", _I), ("irr_img", _B), ("irr_rows5", _D), ("irr_rows7", _D),
        ("irr_w5", _D), ("irr_w7", _D), ("irr_g0", _D), ("irr_rr0", _D), ("irr_outer", _D), ("irr_inner", _D),
    ]


class StepParams(C.Structure):
    _fields_ = [
        ("mode", C.c_int), ("dt", C.c_double), ("gamma", C.c_double), ("kT", C.c_double), ("D", C.c_double),
        ("nrow", C.c_int), ("row_ptr", _I), ("col", _I), ("val", _D),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            raise ImportError(f"oracle library missing: {ORACLE_LIB}")
        L = C.CDLL(str(ORACLE_LIB))
        L.oracle_energy.argtypes = [C.POINTER(OracleSurface), _D, _D, _D]
        L.oracle_energy.restype = C.c_double
        L.oracle_grad.argtypes = [C.POINTER(OracleSurface), _D, _D]
        L.oracle_grad.restype = None
        L.oracle_energy_faces.argtypes = [C.POINTER(OracleSurface), _D, C.c_int, C.c_int]
        L.oracle_energy_faces.restype = C.c_double
        L.oracle_grad_faces.argtypes = [C.POINTER(OracleSurface), _D, _D, C.c_int, C.c_int]
        L.oracle_grad_faces.restype = None
        L.oracle_sparse_apply.argtypes = [C.c_int, _I, _I, _D, _D, C.c_double, _D, _D, _D]
        L.oracle_sparse_apply.restype = None
        L.oracle_step.argtypes = [C.POINTER(StepParams), C.c_int, _D, _D, _D, _D]
        L.oracle_step.restype = None
        L.oracle_noise.argtypes = [C.c_ulonglong, C.c_uint, C.c_ulonglong, C.c_int, _D]
        L.oracle_noise.restype = None
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_D)


class Oracle:
    """The oracle's view of one plan (the engine's planner output, which the
    tests separately pin against the reference's own plan dump)."""

    def __init__(self, plan, prm):
        self._keep = []
        s = OracleSurface()
        s.nv = plan.nv
        s.box[:] = plan.box.reshape(-1).tolist()
        s.kc, s.KA, s.kg, s.k_reg = prm.kc, prm.KA, prm.kg, prm.k_reg
        c0, _ = plan.lipids()
        s.ntypes = len(c0)
        s.lipid_c0 = self._k(c0)
        reg = plan.faces(0)
        s.nreg = plan.n_regular
        s.reg_cp = self._k(np.ascontiguousarray(reg["cp"][:, :12]), C.c_int)
        s.reg_img = self._k(np.ascontiguousarray(reg["img"][:, :12, :]), C.c_int8)
        b6 = plan.basis(6)
        s.reg_rows, s.reg_w = self._k(b6["rows"]), self._k(b6["weight"])
        s.reg_g0, s.reg_rr0 = self._k(reg["g0"]), self._k(reg["rr0"])
        s.reg_outer, s.reg_inner = self._k(reg["outer"]), self._k(reg["inner"])
        irr = plan.faces(1)
        s.nirr = plan.n_irregular
        s.irr_val = self._k(irr["valence"], C.c_int)
        s.irr_cp = self._k(irr["cp"], C.c_int)
        s.irr_img = self._k(irr["img"], C.c_int8)
        b5, b7 = plan.basis(5), plan.basis(7)
        s.irr_rows5, s.irr_rows7 = self._k(b5["rows"]), self._k(b7["rows"])
        s.irr_w5, s.irr_w7 = self._k(b5["weight"]), self._k(b7["weight"])
        s.irr_g0, s.irr_rr0 = self._k(irr["g0"]), self._k(irr["rr0"])
        s.irr_outer, s.irr_inner = self._k(irr["outer"]), self._k(irr["inner"])
        self.s = s
        self.nv = plan.nv

    def _k(self, a, ct=C.c_double):
        a = np.ascontiguousarray(a)
        self._keep.append(a)
        return a.ctypes.data_as(C.POINTER(ct))

    def energy(self, r, terms=False, per_face=False):
        r = np.ascontiguousarray(r, dtype=np.float64)
        t = np.zeros(3)
        fe = np.zeros(self.s.nreg + self.s.nirr) if per_face else None
        E = lib().oracle_energy(C.byref(self.s), _d(r), _d(t), _d(fe))
        out = [E]
        if terms:
            out.append(t)
        if per_face:
            out.append(fe)
        return out[0] if len(out) == 1 else tuple(out)

    @property
    def n_faces(self) -> int:
        return self.s.nreg + self.s.nirr

    def energy_grad_faces(self, r, f0, f1, g):
        """Energy of faces [f0, f1) and their gradient added into g."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        e = lib().oracle_energy_faces(C.byref(self.s), _d(r), f0, f1)
        lib().oracle_grad_faces(C.byref(self.s), _d(r), _d(g), f0, f1)
        return e

    def grad(self, r, g=None):
        r = np.ascontiguousarray(r, dtype=np.float64)
        if g is None:
            g = np.zeros(3 * self.nv + 3)
        lib().oracle_grad(C.byref(self.s), _d(r), _d(g))
        return g


def sparse_apply(row_ptr, col, val, vin, vout, scalev=None, scale=1.0, alphas=(1.0, 1.0, 1.0)):
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    a = np.asarray(alphas, dtype=np.float64)
    sv = None if scalev is None else np.ascontiguousarray(scalev, dtype=np.float64)
    lib().oracle_sparse_apply(len(row_ptr) - 1, row_ptr.ctypes.data_as(_I), col.ctypes.data_as(_I), _d(val), _d(sv),
                              scale, _d(a), _d(np.ascontiguousarray(vin, dtype=np.float64)), _d(vout))
    return vout


def noise(seed: int, stream: int, step: int, nv: int) -> np.ndarray:
    out = np.zeros(3 * nv)
    lib().oracle_noise(seed, stream, step, nv, _d(out))
    return out


def step(mode, dt, gamma, kT, D, r, p, g, xi, mass=None):
    sp = StepParams(mode, dt, gamma, kT, D, 0, None, None, None)
    keep = []
    if mass is not None:
        rp, cl, vl = (np.ascontiguousarray(x, dtype=t) for x, t in zip(mass, (np.int32, np.int32, np.float64)))
        keep += [rp, cl, vl]
        sp.nrow, sp.row_ptr, sp.col, sp.val = len(rp) - 1, rp.ctypes.data_as(_I), cl.ctypes.data_as(_I), _d(vl)
    lib().oracle_step(C.byref(sp), len(p) // 3, _d(r), _d(p), _d(np.ascontiguousarray(g, dtype=np.float64)),
                      _d(np.ascontiguousarray(xi, dtype=np.float64)))


def reference_available() -> bool:
    return REF_DRIVER.exists()


def reference_dump(mesh: Path, params_txt: Path, positions: Path | None, prefix: Path, timeout: float = 600) -> dict:
    """Runs the reference's own code on a mesh and returns its dump."""
    cmd = [str(REF_DRIVER), "dump", str(mesh), str(params_txt), str(positions) if positions else "-", str(prefix)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=timeout)
    out = {}
    for line in Path(f"{prefix}.energy.txt").read_text().splitlines():
        k, v = line.split()
        out[k] = float(v) if k in ("E", "VA", "VC", "VR") else int(v)
    out["grad"] = np.fromfile(f"{prefix}.grad.bin", dtype=np.float64)
    out["positions"] = np.fromfile(f"{prefix}.positions.bin", dtype=np.float64)
    out["face_energy"] = np.fromfile(f"{prefix}.face_energy.bin", dtype=np.float64)
    return out


def reference_min(mesh: Path, params_txt: Path, positions: Path, prefix: Path, timeout: float = 600) -> dict:
    """Runs the reference's own L-BFGS minimization (ref_driver min: src/l-bfgs.C
    driven as src/minimize.C drives it for one surface) and returns the energy
    before and after every iteration and the final state."""
    cmd = [str(REF_DRIVER), "min", str(mesh), str(params_txt), str(positions), str(prefix)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=timeout)
    return {"energies": np.fromfile(f"{prefix}.min_energy.bin", dtype=np.float64),
            "r": np.fromfile(f"{prefix}.min_positions.bin", dtype=np.float64)}


MASS_POINT = np.dtype([("face", "i4"), ("n", "i4"), ("u", "f8"), ("v", "f8"), ("ids", "i4", 13), ("coef", "f8", 13)])


def reference_mass(mesh: Path, params_txt: Path, prefix: Path, timeout: float = 600) -> dict:
    """Runs the reference's own mass-point setup and effective-mass inverse
    (ref_driver mass) and returns M^-1 (dense), the mass per point, area0 and
    every mass point's limit-surface weights."""
    cmd = [str(REF_DRIVER), "mass", str(mesh), str(params_txt), "-", str(prefix)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=timeout)
    out = {}
    for line in Path(f"{prefix}.mass.txt").read_text().splitlines():
        k, v = line.split()
        out[k] = float(v) if k in ("area0", "mass_per_pt") else int(v)
    minv = np.fromfile(f"{prefix}.minv.bin", dtype=np.float64)
    n = int(round(np.sqrt(minv.size)))
    out["minv"] = minv.reshape(n, n)
    out["points"] = np.fromfile(f"{prefix}.coef.bin", dtype=MASS_POINT)
    return out


def reference_sub6(prefix: Path, timeout: float = 60) -> np.ndarray:
    """The reference's fast_sub6_0..3 (ref_driver sub6) as S[child][out point][in point]."""
    subprocess.run([str(REF_DRIVER), "sub6", "-", "-", "-", str(prefix)], check=True, capture_output=True,
                   timeout=timeout)
    M = np.fromfile(f"{prefix}.sub6.bin", dtype=np.float64).reshape(4, 36, 36).transpose(0, 2, 1)
    for k in range(4):  # the same 12 x 12 stencil acts on x, y and z
        for c in range(3):
            for d in range(3):
                blk = M[k][c::3, d::3]
                assert np.array_equal(blk, M[k][0::3, 0::3] if c == d else np.zeros_like(blk))
    return M[:, 0::3, 0::3].copy()


def reference_rnrm(mesh: Path, params_txt: Path, positions: Path | None, prefix: Path, timeout: float = 600):
    """surface::evaluateRNRM of the reference at 7 fixed (u,v) on every face:
    rows of (face, u, v, R[3], N[3])."""
    cmd = [str(REF_DRIVER), "rnrm", str(mesh), str(params_txt), str(positions) if positions else "-", str(prefix)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=timeout)
    return np.fromfile(f"{prefix}.rnrm.bin", dtype=np.float64).reshape(-1, 9)


def reference_time(mesh: Path, params_txt: Path, n_calls: int, timeout: float = 600) -> dict:
    import json
    res = subprocess.run([str(REF_DRIVER), "time", str(mesh), str(params_txt), "-", str(n_calls)], check=True,
                         capture_output=True, text=True, timeout=timeout)
    return json.loads(res.stdout.strip().splitlines()[-1])
