"""GB300 engine for UMCP's membrane-surface hot path.

Python mirror of the reference's `struct surface` call surface over the C ABI
in include/umcp_gpu.h (ctypes, plain pointers): `Plan` is the host side of
loadLattice/generatePlan/setg0, `Mesh.energy`/`Mesh.grad` replace
surface::energy(r, NULL)/surface::grad(r, g) (grad ADDS into g, as the
reference's does), `Mesh.mass_apply` replaces AltSparseCartMatVecIncrScale
and `Mesh.run`/`Mesh.step_host` the dynamics loop body of hd.C.

The compute runs only in the CUDA library; if it is missing the import
fails loudly (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libumcp_gb300.so"

FP64 = 0
FP32_CENTRED = 1
OVERDAMPED_BD = 0
BD_MEMBRANE = 1
LANGEVIN = 2

ERR_NOMEM = 6
ERR_NONFINITE = 4
ERR_DIVERGED = 8

KCAL_MOL_PER_KT_298 = 0.592186663194  # kT at 298 K in kcal/mol (src/hd.C:142)

_STATUS = {
    0: "ok", 1: "invalid argument", 2: "i/o error", 3: "cuda error", 4: "non-finite energy",
    5: "device wait timed out", 6: "out of device memory", 7: "unsupported", 8: "diverged",
}


class UmcpError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    _fields_ = [
        ("kc", C.c_double), ("KA", C.c_double), ("kg", C.c_double), ("k_reg", C.c_double),
        ("temperature", C.c_double), ("precision", C.c_int), ("lipid_directives", C.c_char_p),
        ("face_kernel", C.c_int),
    ]


class PlanInfo(C.Structure):
    _fields_ = [
        ("nv", C.c_int), ("n_regular", C.c_int), ("n_irregular", C.c_int), ("n_lipid_types", C.c_int),
        ("box", C.c_double * 9),
    ]


class MeshInfo(C.Structure):
    _fields_ = [
        ("nv", C.c_int), ("n_faces", C.c_int), ("n_points", C.c_int), ("n_slots", C.c_int),
        ("kernels_per_step", C.c_int), ("kernels_per_step_mass", C.c_int), ("precision", C.c_int),
        ("device_bytes", C.c_longlong), ("h2d_bytes", C.c_longlong), ("mass_form", C.c_int),
    ]


class Integrator(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("time_step", C.c_double), ("gamma", C.c_double), ("D", C.c_double),
        ("seed", C.c_uint64), ("stream", C.c_uint32), ("divergence_threshold", C.c_double),
        ("use_mass", C.c_int),
    ]


class BatchOpts(C.Structure):
    _fields_ = [("tile_faces", C.c_int), ("blocks_per_sm", C.c_int), ("irr_tile_faces", C.c_int),
                ("tune_cache", C.c_char_p)]


class BatchInfo(C.Structure):
    _fields_ = [
        ("n_jobs", C.c_int), ("n_vertices", C.c_longlong), ("n_faces", C.c_longlong),
        ("n_tiles", C.c_int * 3), ("face_grid", C.c_int * 3), ("n_vertex_tiles", C.c_int),
        ("tile_faces", C.c_int), ("kernels_per_step", C.c_int), ("tuned_face_ms", C.c_double),
        ("irr_tile_faces", C.c_int), ("tune_source", C.c_int),
    ]


class Restraints(C.Structure):
    _fields_ = [("K_area", C.c_double), ("area0", C.c_double), ("K_volume", C.c_double), ("volume0", C.c_double)]


class MinimizeOpts(C.Structure):
    _fields_ = [("max_iterations", C.c_int), ("history", C.c_int), ("max_move", C.c_double)]


class MinimizeInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("evaluations", C.c_int), ("energy_initial", C.c_double),
                ("energy_final", C.c_double), ("grad_rms", C.c_double)]


class MassOpts(C.Structure):
    _fields_ = [("mass_scale", C.c_double), ("points_per_edge", C.c_int), ("rel_tol", C.c_double)]


class MassInfo(C.Structure):
    _fields_ = [
        ("area0", C.c_double), ("mass_per_point", C.c_double), ("points", C.c_longlong),
        ("nnz_mass", C.c_longlong), ("nnz_inverse", C.c_longlong), ("dense", C.c_int),
        ("assembly_s", C.c_double), ("inverse_s", C.c_double), ("truncation_s", C.c_double),
        ("column_bytes", C.c_longlong),
    ]


class ServerOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("hbm_budget_bytes", C.c_double), ("max_jobs", C.c_int), ("chunk_ms", C.c_double),
        ("builder_threads", C.c_int), ("tile_faces", C.c_int),
    ]


class JobDesc(C.Structure):
    _fields_ = [
        ("mesh_path", C.c_char_p), ("params", Params), ("it", Integrator), ("step0", C.c_uint64),
        ("n_steps", C.c_int64), ("keep_energies", C.c_int),
    ]


class JobInfo(C.Structure):
    _fields_ = [
        ("state", C.c_int), ("status", C.c_int), ("nv", C.c_int), ("steps_done", C.c_int64),
        ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double), ("device_bytes", C.c_double),
        ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double),
        ("message", C.c_char * 160),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
        ("queued", C.c_longlong), ("running", C.c_longlong), ("chunks", C.c_longlong),
        ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double), ("mean_latency_s", C.c_double),
        ("max_latency_s", C.c_double), ("vertex_steps", C.c_double), ("busy_s", C.c_double),
        ("vertex_steps_per_s", C.c_double), ("hbm_budget_bytes", C.c_double), ("hbm_in_use_bytes", C.c_double),
        ("hbm_peak_bytes", C.c_double), ("chunk_steps", C.c_int),
    ]


JOB_DONE = 4

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_I64 = C.POINTER(C.c_int64)
_I8 = C.POINTER(C.c_int8)
_VP = C.c_void_p

# name -> argument types; every function returns umcp_status (int) unless listed in _VOID/_STR.
_SIGNATURES = {
    "umcp_params_default": [C.POINTER(Params)],
    "umcp_params_from_input": [C.c_char_p, C.POINTER(Params), C.c_char_p, C.c_size_t],
    "umcp_mesh_generate_icosphere": [C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_char_p],
    "umcp_mesh_generate_planar": [C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_char_p],
    "umcp_plan_from_file": [C.c_char_p, C.POINTER(Params), C.POINTER(_VP)],
    "umcp_plan_set_reference": [_VP, _D],
    "umcp_plan_info_get": [_VP, C.POINTER(PlanInfo)],
    "umcp_plan_positions": [_VP, _D],
    "umcp_plan_rings": [_VP, _I, _I],
    "umcp_plan_faces": [_VP, C.c_int, _I, _I8, _I, _D, _D, _D, _D],
    "umcp_plan_basis": [_VP, C.c_int, _D, _D, _D, _D],
    "umcp_plan_lipids": [_VP, _D, _D],
    "umcp_plan_destroy": [_VP],
    "umcp_ctx_create": [C.c_int, C.POINTER(_VP)],
    "umcp_ctx_destroy": [_VP],
    "umcp_ctx_synchronize": [_VP],
    "umcp_ctx_stream": [_VP, C.POINTER(_VP)],
    "umcp_face_pass": [_VP],
    "umcp_mesh_info_get": [_VP, C.POINTER(MeshInfo)],
    "umcp_mesh_create": [_VP, _VP, C.POINTER(Params), C.POINTER(_VP)],
    "umcp_mesh_destroy": [_VP],
    "umcp_mesh_set_params": [_VP, C.POINTER(Params)],
    "umcp_energy": [_VP, _D, _D, _D],
    "umcp_grad": [_VP, _D, _D],
    "umcp_energy_grad": [_VP, _D, _D, _D],
    "umcp_energy_grad_device": [_VP, _VP, _VP, _VP],
    "umcp_energy_grad_static": [_VP, _VP, _VP, _VP],
    "umcp_mesh_check_status": [_VP],
    "umcp_mass_set": [_VP, C.c_int, _I, _I, _D],
    "umcp_mass_apply": [_VP, _D, _D, _D, C.c_double, _D],
    "umcp_mass_apply_device": [_VP, _VP, _VP, _VP, C.c_double, _D],
    "umcp_state_set": [_VP, _D, _D],
    "umcp_minimize": [_VP, C.POINTER(MinimizeOpts), _D, C.POINTER(MinimizeInfo)],
    "umcp_state_get": [_VP, _D, _D],
    "umcp_run": [_VP, C.POINTER(Integrator), C.c_uint64, C.c_int, _D],
    "umcp_run_async": [_VP, C.POINTER(Integrator), C.c_uint64, C.c_int],
    "umcp_step_host": [_VP, C.POINTER(Integrator), C.c_uint64, _D, _D, _D],
    "umcp_mesh_energies": [_VP, _D, C.c_int64],
    "umcp_subdivide_patches": [_VP, _VP, _VP, C.c_longlong],
    "umcp_subdivision_stencils": [_D],
    "umcp_restart_write": [_VP, C.c_char_p, C.c_int],
    "umcp_restart_read": [_VP, C.c_char_p, _I],
    "umcp_mass_build": [_VP, _VP, C.POINTER(MassOpts), C.POINTER(MassInfo)],
    "umcp_mass_get": [_VP, _D],
    "umcp_restraints_set": [_VP, C.POINTER(Restraints)],
    "umcp_restraints_get": [_VP, _D, _D, _D],
    "umcp_plan_point_coeffs": [_VP, C.c_int, C.c_double, C.c_double, _I, _D, _I],
    "umcp_plan_evaluate": [_VP, _D, C.c_int, _I, _D, _D, _D],
    "umcp_limit_points": [_VP, C.c_int, _D, _D],
    "umcp_write_limiting_surface": [_VP, C.c_char_p],
    "umcp_batch_create": [_VP, C.c_int, C.POINTER(BatchOpts), C.POINTER(_VP)],
    "umcp_batch_destroy": [_VP],
    "umcp_batch_add": [_VP, _VP, C.POINTER(Integrator), C.c_uint64, C.c_int64],
    "umcp_batch_remove": [_VP, _VP],
    "umcp_batch_run": [_VP, C.c_int],
    "umcp_batch_poll": [_VP, _I64, _I],
    "umcp_batch_job": [_VP, _VP, _I64, _I],
    "umcp_batch_info_get": [_VP, C.POINTER(BatchInfo)],
    "umcp_batch_face_pass": [_VP],
    "umcp_batch_step_host": [_VP, _VP, _VP, _VP, C.c_int],
    "umcp_ctx_mem_info": [_VP, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)],
    "umcp_plan_device_bytes": [_VP, _VP, C.c_int, C.c_int64, C.POINTER(C.c_size_t)],
    "umcp_server_create": [_VP, C.POINTER(ServerOpts), C.POINTER(_VP)],
    "umcp_server_destroy": [_VP],
    "umcp_server_submit": [_VP, C.POINTER(JobDesc), C.POINTER(C.c_uint64)],
    "umcp_server_wait": [_VP, C.c_uint64, C.c_double],
    "umcp_server_wait_all": [_VP, C.c_double],
    "umcp_server_job": [_VP, C.c_uint64, C.POINTER(JobInfo)],
    "umcp_server_fetch": [_VP, C.c_uint64, _D, _D],
    "umcp_server_release": [_VP, C.c_uint64],
    "umcp_server_stats_get": [_VP, C.POINTER(ServerStats)],
    "umcp_server_now": [_VP],
    "umcp_last_error": [],
    "umcp_status_string": [C.c_int],
}
_VOID = {"umcp_plan_destroy", "umcp_ctx_destroy", "umcp_mesh_destroy", "umcp_batch_destroy", "umcp_server_destroy"}
_DOUBLE = {"umcp_server_now"}
_STR = {"umcp_last_error", "umcp_status_string"}

_lib = None


def library() -> C.CDLL:
    """Loads the engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"umcp_gb300 engine library missing: {LIB_PATH} (run __graft_entry__.build())")
        lib = C.CDLL(str(LIB_PATH))
        for name, args in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = (None if name in _VOID else C.c_char_p if name in _STR else C.c_double if name in _DOUBLE
                          else C.c_int)
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return sorted(_SIGNATURES)


def _check(status: int) -> None:
    if status != 0:
        raise UmcpError(status, library().umcp_last_error().decode())


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _ip(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I)


SIMT = 0          # Params.face_kernel: the FP32 SIMT face kernel (default)
TENSOR_CORES = 1  # regular faces of the precision form through tcgen05 (kind::f16 MMAs on fp16 hi/lo splits)


def params(kc=14.0, KA=0.215, kg=0.0, k_reg=0.0, temperature=298.0, precision=FP64, lipids: str | None = None,
           face_kernel: int = SIMT) -> Params:
    p = Params()
    _check(library().umcp_params_default(C.byref(p)))
    p.kc, p.KA, p.kg, p.k_reg, p.temperature, p.precision = kc, KA, kg, k_reg, temperature, precision
    p.face_kernel = face_kernel
    p._lipid_bytes = lipids.encode() if lipids else None  # keep alive
    p.lipid_directives = p._lipid_bytes
    return p


def kc_from_kT(kc_kT: float, temperature: float = 298.0) -> float:
    """Bending modulus in kcal/mol for kc given in units of kT (src/hd.C:142-143)."""
    return kc_kT * KCAL_MOL_PER_KT_298 / 298.0 * temperature


def generate_icosphere(path: str | os.PathLike, level: int, R: float, sigma: float, seed: int) -> None:
    _check(library().umcp_mesh_generate_icosphere(level, R, sigma, seed, str(path).encode()))


def generate_planar(path: str | os.PathLike, nx: int, ny: int, a: float, kc_kT: float, seed: int) -> None:
    _check(library().umcp_mesh_generate_planar(nx, ny, a, kc_kT, seed, str(path).encode()))


class Plan:
    """Host-side plan of one mesh (loadLattice + generatePlan + lipids + setg0)."""

    def __init__(self, mesh_path: str | os.PathLike, prm: Params | None = None):
        self._h = C.c_void_p()
        self._prm = prm if prm is not None else params()
        _check(library().umcp_plan_from_file(str(mesh_path).encode(), C.byref(self._prm), C.byref(self._h)))
        info = PlanInfo()
        _check(library().umcp_plan_info_get(self._h, C.byref(info)))
        self.nv = info.nv
        self.n_regular = info.n_regular
        self.n_irregular = info.n_irregular
        self.n_lipid_types = info.n_lipid_types
        self.box = np.array(info.box[:], dtype=np.float64).reshape(3, 3)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.umcp_plan_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def device_bytes(self, ctx: "Context", precision: int, n_energies: int = 0) -> int:
        """Device bytes a Mesh of this plan holds (plus an n_energies-step energy record)."""
        b = C.c_size_t()
        _check(library().umcp_plan_device_bytes(self._h, ctx.handle, precision, n_energies, C.byref(b)))
        return b.value

    def point_coeffs(self, face: int, u: float, v: float) -> tuple[np.ndarray, np.ndarray]:
        """Limit-surface point (u,v) of a face as (vertex ids, weights)."""
        ids = np.zeros(13, dtype=np.int32)
        coef = np.zeros(13)
        n = C.c_int()
        _check(library().umcp_plan_point_coeffs(self._h, face, u, v, _ip(ids), _dp(coef), C.byref(n)))
        return ids[:n.value], coef[:n.value]

    def evaluate(self, r: np.ndarray, faces, uv) -> tuple[np.ndarray, np.ndarray]:
        """Limit-surface points and unit normals of state r at (face, u, v) queries."""
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        uv = np.ascontiguousarray(uv, dtype=np.float64).reshape(-1, 2)
        n = len(faces)
        R, N = np.zeros((n, 3)), np.zeros((n, 3))
        _check(library().umcp_plan_evaluate(self._h, _dp(np.ascontiguousarray(r, dtype=np.float64)), n, _ip(faces),
                                            _dp(uv), _dp(R), _dp(N)))
        return R, N

    def positions(self) -> np.ndarray:
        r = np.zeros(3 * self.nv + 3)
        _check(library().umcp_plan_positions(self._h, _dp(r)))
        return r

    def set_reference(self, r: np.ndarray) -> None:
        _check(library().umcp_plan_set_reference(self._h, _dp(np.ascontiguousarray(r, dtype=np.float64))))

    def rings(self) -> tuple[np.ndarray, np.ndarray]:
        val = np.zeros(self.nv, dtype=np.int32)
        _check(library().umcp_plan_rings(self._h, _ip(val), None))
        ring = np.zeros(int(val.sum()), dtype=np.int32)
        _check(library().umcp_plan_rings(self._h, None, _ip(ring)))
        return val, ring

    def faces(self, kind: int) -> dict:
        nf = self.n_irregular if kind else self.n_regular
        npt = 16 if kind else 15
        nt = self.n_lipid_types
        out = {
            "cp": np.zeros((nf, 13), dtype=np.int32), "img": np.zeros((nf, 13, 3), dtype=np.int8),
            "valence": np.zeros(nf, dtype=np.int32), "g0": np.zeros((nf, npt)), "rr0": np.zeros((nf, npt)),
            "outer": np.zeros((nf, nt)), "inner": np.zeros((nf, nt)),
        }
        _check(library().umcp_plan_faces(
            self._h, kind, _ip(out["cp"]), out["img"].ctypes.data_as(_I8), _ip(out["valence"]), _dp(out["g0"]),
            _dp(out["rr0"]), _dp(out["outer"]), _dp(out["inner"])))
        return out

    def basis(self, valence: int) -> dict:
        npt, ncp = (15, 12) if valence == 6 else (16, valence + 6)
        rows = np.zeros((6, npt, ncp))
        w, u, v = np.zeros(npt), np.zeros(npt), np.zeros(npt)
        _check(library().umcp_plan_basis(self._h, valence, _dp(rows), _dp(w), _dp(u), _dp(v)))
        return {"rows": rows, "weight": w, "u": u, "v": v}

    def lipids(self) -> tuple[np.ndarray, np.ndarray]:
        c0, apl = np.zeros(self.n_lipid_types), np.zeros(self.n_lipid_types)
        _check(library().umcp_plan_lipids(self._h, _dp(c0), _dp(apl)))
        return c0, apl


class Context:
    """One CUDA device and stream."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        _check(library().umcp_ctx_create(device, C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.umcp_ctx_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def synchronize(self) -> None:
        _check(library().umcp_ctx_synchronize(self._h))

    def mem_info(self) -> tuple[int, int]:
        f, t = C.c_size_t(), C.c_size_t()
        _check(library().umcp_ctx_mem_info(self._h, C.byref(f), C.byref(t)))
        return f.value, t.value

    def stream(self) -> int:
        """The cudaStream_t every engine call on this context is queued on."""
        s = C.c_void_p()
        _check(library().umcp_ctx_stream(self._h, C.byref(s)))
        return s.value or 0


class Mesh:
    """Device-resident surface; energy/grad mirror surface::energy/grad."""

    def __init__(self, ctx: Context, plan: Plan, prm: Params | None = None):
        self.ctx = ctx  # keep the context alive
        self.nv = plan.nv
        self._prm = prm if prm is not None else plan._prm
        self._h = C.c_void_p()
        _check(library().umcp_mesh_create(ctx.handle, plan.handle, C.byref(self._prm), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.umcp_mesh_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def info(self) -> MeshInfo:
        i = MeshInfo()
        _check(library().umcp_mesh_info_get(self._h, C.byref(i)))
        return i

    def face_pass(self) -> None:
        _check(library().umcp_face_pass(self._h))

    def set_params(self, prm: Params) -> None:
        self._prm = prm
        _check(library().umcp_mesh_set_params(self._h, C.byref(prm)))

    def energy(self, r: np.ndarray, terms: bool = False):
        r = np.ascontiguousarray(r, dtype=np.float64)
        E = C.c_double()
        t = np.zeros(3)
        _check(library().umcp_energy(self._h, _dp(r), C.byref(E), _dp(t)))
        return (E.value, t) if terms else E.value

    def grad(self, r: np.ndarray, g: np.ndarray) -> np.ndarray:
        """Adds dE/dr into g (3*nv+3), as surface::grad does."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        _check(library().umcp_grad(self._h, _dp(r), _dp(g)))
        return g

    def energy_grad(self, r: np.ndarray) -> tuple[float, np.ndarray]:
        r = np.ascontiguousarray(r, dtype=np.float64)
        g = np.zeros(3 * self.nv + 3)
        E = C.c_double()
        _check(library().umcp_energy_grad(self._h, _dp(r), C.byref(E), _dp(g)))
        return E.value, g

    def energy_grad_device(self, d_r: int, d_E: int, d_g: int) -> None:
        """Device-pointer energy+gradient (g accumulated), queued on the ctx stream."""
        _check(library().umcp_energy_grad_device(self._h, C.c_void_p(d_r), C.c_void_p(d_E), C.c_void_p(d_g)))

    def energy_grad_static(self, d_r: int, d_E: int, d_g: int) -> None:
        """As energy_grad_device, with all scratch in the library's static device
        array instead of the mesh's own buffers (no allocation at call time)."""
        _check(library().umcp_energy_grad_static(self._h, C.c_void_p(d_r), C.c_void_p(d_E), C.c_void_p(d_g)))

    def limit_points(self, plim: int, normals: bool = True) -> tuple[np.ndarray, np.ndarray | None]:
        """Limit points (and unit normals) of the resident state at every face's
        lattice (i/plim, j/plim), i + j <= plim: arrays [faces, points, 3]."""
        info = self.info()
        npts = (plim + 1) * (plim + 2) // 2
        R = np.zeros((info.n_faces, npts, 3))
        N = np.zeros((info.n_faces, npts, 3)) if normals else None
        _check(library().umcp_limit_points(self._h, plim, R.ctypes.data_as(_D),
                                           None if N is None else N.ctypes.data_as(_D)))
        return R, N

    def write_limiting_surface(self, path) -> None:
        """The reference's limiting-surface xyz file of the resident state."""
        _check(library().umcp_write_limiting_surface(self._h, str(path).encode()))

    def check_status(self) -> None:
        """Waits for the mesh's queued work; raises UmcpError if a kernel recorded
        a non-finite energy, a divergence or a timeout since the last check."""
        _check(library().umcp_mesh_check_status(self._h))

    def mass_set(self, row_ptr: np.ndarray, col: np.ndarray, val: np.ndarray) -> None:
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=np.float64)
        _check(library().umcp_mass_set(self._h, len(row_ptr) - 1, _ip(row_ptr), _ip(col), _dp(val)))

    def mass_apply(self, vin: np.ndarray, vout: np.ndarray, scalev: np.ndarray | None = None, scale: float = 1.0,
                   alphas=(1.0, 1.0, 1.0)) -> np.ndarray:
        a = np.asarray(alphas, dtype=np.float64)
        sv = None if scalev is None else np.ascontiguousarray(scalev, dtype=np.float64)
        _check(library().umcp_mass_apply(self._h, _dp(np.ascontiguousarray(vin, dtype=np.float64)), _dp(vout),
                                         _dp(sv), scale, _dp(a)))
        return vout

    def mass_apply_device(self, d_in: int, d_out: int, d_scalev: int = 0, scale: float = 1.0,
                          alphas=(1.0, 1.0, 1.0)) -> None:
        """out (+)= M^-1 in on device pointers (3 nv doubles each), queued on the context's stream."""
        a = np.asarray(alphas, dtype=np.float64)
        _check(library().umcp_mass_apply_device(self._h, C.c_void_p(d_in), C.c_void_p(d_out),
                                                C.c_void_p(d_scalev or None), scale, _dp(a)))

    def state_set(self, r: np.ndarray, p: np.ndarray | None = None) -> None:
        _check(library().umcp_state_set(self._h, _dp(np.ascontiguousarray(r, dtype=np.float64)),
                                        _dp(None if p is None else np.ascontiguousarray(p, dtype=np.float64))))

    def state_get(self) -> tuple[np.ndarray, np.ndarray]:
        r, p = np.zeros(3 * self.nv + 3), np.zeros(3 * self.nv)
        _check(library().umcp_state_get(self._h, _dp(r), _dp(p)))
        return r, p

    def run(self, it: Integrator, step0: int, n_steps: int, energies: bool = True):
        e = np.zeros(max(n_steps, 1)) if energies else None
        _check(library().umcp_run(self._h, C.byref(it), step0, n_steps, _dp(e)))
        return e[:n_steps] if energies else None

    def run_async(self, it: Integrator, step0: int, n_steps: int) -> None:
        _check(library().umcp_run_async(self._h, C.byref(it), step0, n_steps))

    def step_host(self, it: Integrator, step: int, r: np.ndarray, p: np.ndarray | None = None) -> float:
        E = C.c_double()
        _check(library().umcp_step_host(self._h, C.byref(it), step, _dp(r), _dp(p), C.byref(E)))
        return E.value

    def mass_build(self, plan: "Plan", mass_scale: float = 5.0, points_per_edge: int = 10,
                   rel_tol: float = 1e-20) -> MassInfo:
        """Builds and installs M^-1 from the limit surface (umcp_mass_build)."""
        info = MassInfo()
        opts = MassOpts(mass_scale, points_per_edge, rel_tol)
        _check(library().umcp_mass_build(self._h, plan.handle, C.byref(opts), C.byref(info)))
        return info

    def restraints_set(self, K_area: float = 0.0, area0: float = -1.0, K_volume: float = 0.0,
                       volume0: float = -1.0) -> None:
        """Global area/volume restraints (umcp_restraints_set); area0/volume0 < 0: the resident state's."""
        rs = Restraints(K_area, area0, K_volume, volume0)
        _check(library().umcp_restraints_set(self._h, C.byref(rs)))

    def minimize(self, max_iterations: int = 100, history: int = 0, max_move: float = 1.0):
        """L-BFGS over the vertex positions from the resident state
        (umcp_minimize; the reference's Simulation::minimize for a membrane).
        Returns (energies before and after each iteration, MinimizeInfo)."""
        e = np.zeros(max_iterations + 1)
        info = MinimizeInfo()
        _check(library().umcp_minimize(self._h, C.byref(MinimizeOpts(max_iterations, history, max_move)), _dp(e),
                                       C.byref(info)))
        return e[: info.iterations + 1], info

    def restraints_clear(self) -> None:
        _check(library().umcp_restraints_set(self._h, None))

    def restraints_get(self) -> tuple[float, float, float]:
        """(A, V, E_r) of the latest evaluation."""
        a, v, e = C.c_double(), C.c_double(), C.c_double()
        _check(library().umcp_restraints_get(self._h, C.byref(a), C.byref(v), C.byref(e)))
        return a.value, v.value, e.value

    def mass_get(self) -> np.ndarray:
        out = np.zeros((self.nv, self.nv))
        _check(library().umcp_mass_get(self._h, _dp(out)))
        return out

    def restart_write(self, path, seed: int = -1) -> None:
        _check(library().umcp_restart_write(self._h, str(path).encode(), seed))

    def restart_read(self, path) -> int:
        """Loads a restart file into the resident state; returns its seed (-1 if none)."""
        seed = C.c_int()
        _check(library().umcp_restart_read(self._h, str(path).encode(), C.byref(seed)))
        return seed.value

    def energies(self, n: int) -> np.ndarray:
        """The first n energies recorded by the latest run or batch job."""
        e = np.zeros(max(n, 1))
        _check(library().umcp_mesh_energies(self._h, _dp(e), n))
        return e[:n]


class Batch:
    """Many meshes of one context advanced together (umcp_batch_*). Each job
    behaves as Mesh.run(it, step0, n_steps) on its own mesh."""

    def __init__(self, ctx: Context, precision: int = FP64, tile_faces: int = 0, blocks_per_sm: int = 0,
                 irr_tile_faces: int = 0, tune_cache: str | os.PathLike | None = None):
        self.ctx = ctx  # keep the context alive; a job's mesh leaves the batch when it is destroyed
        self._h = C.c_void_p()
        self._cache = str(tune_cache).encode() if tune_cache else None  # keep alive
        opts = BatchOpts(tile_faces, blocks_per_sm, irr_tile_faces, self._cache)
        _check(library().umcp_batch_create(ctx.handle, precision, C.byref(opts), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.umcp_batch_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def add(self, mesh: Mesh, it: Integrator, step0: int, n_steps: int) -> None:
        _check(library().umcp_batch_add(self._h, mesh.handle, C.byref(it), step0, n_steps))

    def remove(self, mesh: Mesh) -> None:
        _check(library().umcp_batch_remove(self._h, mesh.handle))

    def run(self, n_steps: int) -> None:
        _check(library().umcp_batch_run(self._h, n_steps))

    def step_host(self, r_in, r_out, E, n_steps: int = 1) -> None:
        """Host-driven steps (umcp_batch_step_host): r_in / r_out / E are host
        arrays (float64, the jobs' 3*nv+3 states packed in add order / one
        energy per job) or raw host addresses (int, e.g. of pinned memory), or
        None."""
        def ptr(a):
            if a is None or isinstance(a, int):
                return C.c_void_p(a)
            assert a.dtype == np.float64 and a.flags.c_contiguous
            return C.c_void_p(a.ctypes.data)
        _check(library().umcp_batch_step_host(self._h, ptr(r_in), ptr(r_out), ptr(E), n_steps))

    def poll(self) -> tuple[np.ndarray, np.ndarray]:
        """(steps done, status) of every job, in add order."""
        n = self.info().n_jobs
        done = np.zeros(max(n, 1), dtype=np.int64)
        st = np.zeros(max(n, 1), dtype=np.int32)
        _check(library().umcp_batch_poll(self._h, done.ctypes.data_as(_I64), st.ctypes.data_as(_I)))
        return done[:n], st[:n]

    def job(self, mesh: Mesh) -> tuple[int, int]:
        done, st = C.c_int64(), C.c_int()
        _check(library().umcp_batch_job(self._h, mesh.handle, C.byref(done), C.byref(st)))
        return done.value, st.value

    def info(self) -> BatchInfo:
        i = BatchInfo()
        _check(library().umcp_batch_info_get(self._h, C.byref(i)))
        return i

    def face_pass(self) -> None:
        """Queues the face launches of one step only (for timing)."""
        _check(library().umcp_batch_face_pass(self._h))


def subdivision_stencils() -> np.ndarray:
    """S[child][out point][in point] of regular-patch Loop subdivision (4 x 12 x 12)."""
    S = np.zeros((4, 12, 12))
    _check(library().umcp_subdivision_stencils(_dp(S)))
    return S


def subdivide_patches(ctx: "Context", d_in: int, d_out: int, n: int) -> None:
    """Device-pointer batched subdivision: n x 36 doubles in, n x 4 x 36 out."""
    _check(library().umcp_subdivide_patches(ctx.handle, C.c_void_p(d_in), C.c_void_p(d_out), n))


def integrator(kind=OVERDAMPED_BD, time_step=1.0, gamma=0.0, D=0.0, seed=1, stream=0, divergence_threshold=0.0,
               use_mass=0) -> Integrator:
    return Integrator(kind, time_step, gamma, D, seed, stream, divergence_threshold, use_mass)


class Server:
    """Request loop over one batch (umcp_server_*): submit jobs from any thread,
    wait for them, fetch their final state and energies."""

    def __init__(self, ctx: Context, precision: int = FP32_CENTRED, hbm_budget_bytes: float = 0.0, max_jobs: int = 0,
                 chunk_ms: float = 0.0, builder_threads: int = 0, tile_faces: int = 0):
        self.ctx = ctx
        self._h = C.c_void_p()
        self._keep = {}  # id -> (path bytes, lipid bytes, nv) kept alive until the job is built
        opts = ServerOpts(precision, hbm_budget_bytes, max_jobs, chunk_ms, builder_threads, tile_faces)
        _check(library().umcp_server_create(ctx.handle, C.byref(opts), C.byref(self._h)))

    def close(self) -> None:
        if getattr(self, "_h", None) and _lib is not None:
            _lib.umcp_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def submit(self, mesh_path, prm: Params, it: Integrator, step0: int, n_steps: int,
               keep_energies: bool = False) -> int:
        path = str(mesh_path).encode()
        d = JobDesc(path, prm, it, step0, n_steps, int(keep_energies))
        jid = C.c_uint64()
        _check(library().umcp_server_submit(self._h, C.byref(d), C.byref(jid)))
        self._keep[jid.value] = path
        return jid.value

    def wait(self, jid: int, timeout_s: float = -1.0) -> bool:
        st = library().umcp_server_wait(self._h, jid, timeout_s)
        if st not in (0, 5):
            _check(st)
        return st == 0

    def wait_all(self, timeout_s: float = -1.0) -> bool:
        st = library().umcp_server_wait_all(self._h, timeout_s)
        if st not in (0, 5):
            _check(st)
        return st == 0

    def job(self, jid: int) -> JobInfo:
        i = JobInfo()
        _check(library().umcp_server_job(self._h, jid, C.byref(i)))
        return i

    def fetch(self, jid: int) -> tuple[np.ndarray, np.ndarray]:
        """(final r, kept energies) of a done job."""
        i = self.job(jid)
        r = np.zeros(3 * i.nv + 3)
        e = np.zeros(max(i.steps_done, 1))
        _check(library().umcp_server_fetch(self._h, jid, _dp(r), _dp(e)))
        return r, e[:i.steps_done]

    def release(self, jid: int) -> None:
        _check(library().umcp_server_release(self._h, jid))
        self._keep.pop(jid, None)

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(library().umcp_server_stats_get(self._h, C.byref(s)))
        return s

    def now(self) -> float:
        return library().umcp_server_now(self._h)
