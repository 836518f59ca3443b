"""Synthetic workloads of the membrane benchmarks: the mixed-vesicle batch
and the planar periodic membrane. Meshes are written in the .mesh format by
the engine's own generators and read back through Plan, exactly as a user's
mesh files would be.

Mixed vesicles (the batched benchmark): icosahedra Loop-subdivided 2-5 times
(162 / 642 / 2562 / 10,242 vertices), level drawn uniformly per vesicle,
radius log-uniform in 50-300 A, radial noise N(0, 0.01 R), kc uniform in
10-40 kT, spontaneous curvature c0 uniform in +-0.01 1/A carried by the lipid
library (c0 on the outer leaflet's lipid, -c0 on the inner one, APL 68.3 A^2;
the reference's only c0 channel). Overdamped BD with sqrt(2 D dt) = 0.05 A.
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

import umcp_gb300 as U

APL = 68.3
RMS_STEP_A = 0.05


def lipid_text(c0: float) -> str:
    return (f"lipid library Lo {APL} {c0!r}\nlipid library Li {APL} {-c0!r}\n"
            "lipid outer Lo 1\nlipid inner Li 1\n")


@dataclass
class VesicleSpec:
    index: int
    level: int
    radius: float
    sigma: float
    kc_kT: float
    c0: float
    seed: int


def vesicle_specs(n: int, seed: int, levels=(2, 3, 4, 5), r_range=(50.0, 300.0), noise_frac=0.01,
                  kc_range=(10.0, 40.0), c0_max=0.01) -> list[VesicleSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        level = int(rng.choice(levels))
        radius = float(math.exp(rng.uniform(math.log(r_range[0]), math.log(r_range[1]))))
        kc = float(rng.uniform(*kc_range))
        c0 = float(rng.uniform(-c0_max, c0_max))
        out.append(VesicleSpec(i, level, radius, noise_frac * radius, kc, c0, seed * 100003 + i))
    return out


def _build_vesicle(spec: VesicleSpec, tmpdir: Path, precision: int, temperature: float):
    path = tmpdir / f"vesicle_{spec.index}.mesh"
    U.generate_icosphere(path, spec.level, spec.radius, spec.sigma, spec.seed)
    prm = U.params(kc=U.kc_from_kT(spec.kc_kT, temperature), KA=0.215, temperature=temperature,
                   precision=precision, lipids=lipid_text(spec.c0))
    return U.Plan(path, prm), prm


def vesicle_plans(specs: list[VesicleSpec], tmpdir: Path, precision: int, temperature: float = 298.0,
                  threads: int | None = None):
    """(plan, params) per vesicle, built on host threads (the engine's plan
    builder runs without the interpreter lock)."""
    tmpdir.mkdir(parents=True, exist_ok=True)
    threads = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(lambda s: _build_vesicle(s, tmpdir, precision, temperature), specs))


def bd_integrator(seed: int, stream: int, rms_step: float):
    """Overdamped BD with sqrt(2 D dt) = rms_step (time_step 1, D = rms^2/2)."""
    return U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=rms_step * rms_step / 2.0, seed=seed, stream=stream)


def hessian_lambda_max(mesh, r: np.ndarray, iters: int = 30, eps: float = 1e-4) -> float:
    """Largest eigenvalue of the energy's Hessian in the vertex coordinates at
    state r (kcal/mol/A^2), by power iteration on central differences of the
    engine's gradient: H v ~ (g(r + eps v) - g(r - eps v)) / (2 eps)."""
    n = 3 * mesh.nv
    v = np.random.default_rng(1).normal(size=n)
    v /= np.linalg.norm(v)
    lam = 0.0
    for _ in range(iters):
        rp, rm = r.copy(), r.copy()
        rp[:n] += eps * v
        rm[:n] -= eps * v
        hv = (mesh.energy_grad(rp)[1][:n] - mesh.energy_grad(rm)[1][:n]) / (2.0 * eps)
        lam = float(v @ hv)
        v = hv / np.linalg.norm(hv)
    return lam


def stable_rms_step(lambda_max: float, temperature: float = 298.0) -> float:
    """The overdamped BD update r += -(D dt/kT) g + sqrt(2 D dt) xi is stable
    while (D dt/kT) lambda_max < 2 (the stiffest mode's drift overshoots
    beyond that); this returns the sqrt(2 D dt) that puts it at 1, half the
    limit: sqrt(2 kT / lambda_max)."""
    kT = U.KCAL_MOL_PER_KT_298 / 298.0 * temperature
    return math.sqrt(2.0 * kT / lambda_max)


def planar_plan(tmpdir: Path, nx: int, ny: int, seed: int, precision: int, kc_kT: float = 20.0,
                a: float = 10.0, temperature: float = 298.0):
    tmpdir.mkdir(parents=True, exist_ok=True)
    path = tmpdir / f"planar_{nx}x{ny}_{seed}.mesh"
    U.generate_planar(path, nx, ny, a, kc_kT, seed)
    prm = U.params(kc=U.kc_from_kT(kc_kT, temperature), KA=0.215, temperature=temperature, precision=precision)
    return U.Plan(path, prm), prm


AKMA_TIME_S = 0.04888e-12  # one AKMA time unit in seconds (the engine's time_step conversion)


def large_vesicle(tmpdir: Path, precision: int, level: int = 6, radius: float = 1000.0, sigma: float = 2.0,
                  kc_kT: float = 20.0, seed: int = 1004, temperature: float = 298.0):
    """The Langevin-with-mass workload: an icosahedron subdivided `level` times
    (40,962 vertices at 6), radius 1000 A, radial noise N(0, 2 A), kc 20 kT,
    c0 = 0."""
    tmpdir.mkdir(parents=True, exist_ok=True)
    path = tmpdir / "large_vesicle.mesh"
    U.generate_icosphere(path, level, radius, sigma, seed)
    prm = U.params(kc=U.kc_from_kT(kc_kT, temperature), KA=0.215, temperature=temperature, precision=precision)
    return U.Plan(path, prm), prm


def langevin_mass_integrator(mesh, nv: int, seed: int, rms_step: float = RMS_STEP_A, gamma_per_ps: float = 1.0,
                             temperature: float = 298.0, samples: int = 8):
    """Langevin leapfrog with the installed M^-1 and a time step whose thermal
    displacement sqrt(kT <M^-1_ii>) dt is rms_step; <M^-1_ii> is the mean
    diagonal entry over `samples` vertices spread over the mesh."""
    kT = U.KCAL_MOL_PER_KT_298 / 298.0 * temperature
    diag = []
    for i in np.linspace(0, nv - 1, samples).astype(int):
        e = np.zeros(3 * nv)
        e[3 * i] = 1.0
        out = np.zeros(3 * nv)
        mesh.mass_apply(e, out)
        diag.append(out[3 * i])
    minv = float(np.mean(diag))
    dt_akma = rms_step / math.sqrt(kT * minv)
    it = U.integrator(U.LANGEVIN, time_step=dt_akma * AKMA_TIME_S, gamma=gamma_per_ps * AKMA_TIME_S * 1e12,
                      seed=seed, divergence_threshold=1e5, use_mass=1)
    return it, minv, dt_akma
