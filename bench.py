#!/usr/bin/env python3
"""BD vertex-steps/s of the membrane-surface hot path on one GB300 (N GPUs:
one independent replica of the workload per GPU).

Headline workload (value): batched overdamped BD of 256 mixed vesicles in one
batch: icosahedra Loop-subdivided 2-5 times (162 / 642 / 2,562 / 10,242
vertices, level drawn per vesicle), radius log-uniform in 50-300 A, radial
noise N(0, 0.01 R), kc uniform in 10-40 kT, c0 uniform in +-0.01 1/A on the
lipid library; FP32 face-centred patch arithmetic with FP64 sums and FP64
position update; sqrt(2 D dt) = 0.02 A. One step advances every vesicle by
one BD step (energy, gradient, update): one face launch per patch type over
all vesicles, a per-vesicle energy sum and one fused gather + update.

  value     device-resident throughput: K steps between CUDA events on the
            engine's stream (the step inputs, about 0.4 GB of face tables and
            state, exceed the 129 MB L2, so no flush is needed).
  e2e       the same batch driven from the host through the public C ABI
            (umcp_batch_step_host), as the reference's loop holds its state
            on the host: every step all jobs' states go in from pinned host
            memory and the new states and energies come back; wall clock.
  admission the same vesicles as mesh files through the serving API
            (umcp_server_*): plans built, state uploaded, K steps, results
            copied back; wall clock from first submit to last result.
  roofline  the batch's face launches (the dominant kernels) timed alone with
            CUDA events: algorithmic bytes per launch / duration against the
            measured HBM copy bandwidth, and FP32 flop rate against the
            nominal FP32 SIMT rate.
  cpu_baseline  the oracle's C restatement of the reference path on one host
            core, a bounded sample of the same vesicles.
  variants  FP64 batched; the plain FP64 path one vesicle at a time; the
            FP32 form's relative error against FP64 on the same states; the
            128 x 128 planar membrane alone.
  serving   Poisson arrivals at 200 jobs/s over a window (default 1 s) of
            vesicles (levels 2-5, R 50-500 A) and planar patches (32-128 per
            side), kc 10-40 kT, steps log-uniform in 1e3-1e5; p50/p99 job
            latency and aggregate vertex-steps/s.

--impl reference runs the oracle's C restatement of the reference path on its
own plan of every vesicle (oracle/planner.py: no engine code is loaded), with
all host cores, vesicles dealt round robin over one process per core, as
independent reference runs would (the reference's own sources are not on the
GPU host).

Profiling modes (the commands behind the ncu summaries; no JSON line):
  --mode facepass   queues the per-face pass `--repeat` times after one
            energy+gradient call: on an --nx x --ny planar membrane (or an
            --icosphere level), or, with --vesicles N, the batched face
            launches over the first N vesicles of the benchmark workload after
            three batched BD steps at --tile-faces.
  --mode massapply  builds M^-1 on an icosahedral vesicle of --level (the
            reference's settings: 66 mass points per face, truncation 1e-20)
            and times --repeat applies with CUDA events after 3 untimed ones.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {
    "workload": "batched BD of 256 mixed vesicles (icosahedra subdivided 2-5x, 162-10,242 vertices each), "
                "FP32 face-centred",
    "n_vesicles": 256, "levels": [2, 3, 4, 5], "radius_A": [50.0, 300.0], "noise": "0.01 R",
    "kc_kT": [10.0, 40.0], "c0_per_A": [-0.01, 0.01], "KA": 0.215, "seed": 1003, "rms_step_A": 0.02,
    "quadrature": "15-point regular rule, 4x4 Gauss on irregular sub-triangles",
    "l2": "inputs larger than L2 (about 0.4 GB of face tables and state per step); no flush",
}
METRIC = "BD vertex-steps/s"
L2_BYTES = 129 * 1024 * 1024
SM_COUNT, FP32_LANES_PER_SM = 152, 128
# independent batches driven from host threads in the e2e measurement: one group's
# copies overlap another's step (256 vesicles: 1 group 740, 2: 822, 3: 894, 4: 875 M vertex-steps/s)
E2E_GROUPS = 3
E2E_REPEATS = 3  # K-step e2e runs; the median is reported
# DRAM bytes per face of the batched face launches, from the ncu capture of
# the first 64 vesicles of the workload at 512-face tiles (dram__bytes_read.sum
# + dram__bytes_write.sum of the regular and valence-5 launches: 86.48 +
# 26.64 + 2.79 + 0.01 MB over 392,960 faces); the benchmark's pass is scaled
# from it by its face count.
BATCH_FACE_DRAM_BYTES_PER_FACE = 115.92e6 / 392960


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--vesicles", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window of the serving run; 0 skips it")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--ref-seconds", type=float, default=60.0)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--e2e-groups", type=int, default=E2E_GROUPS,
                    help="independent batches (contexts, host threads) the e2e measurement drives the vesicles as")
    ap.add_argument("--mode", default="bench", choices=["bench", "facepass", "massapply", "geo"])
    ap.add_argument("--nx", type=int, default=512, help="facepass: planar membrane size")
    ap.add_argument("--ny", type=int, default=512)
    ap.add_argument("--icosphere", type=int, default=0, help="facepass: an icosahedral vesicle of this level instead")
    ap.add_argument("--level", type=int, default=5, help="massapply: Loop subdivisions of the icosahedron")
    ap.add_argument("--radius", type=float, default=1000.0, help="massapply: vesicle radius (A)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"], help="facepass / massapply")
    ap.add_argument("--repeat", type=int, default=3, help="facepass / massapply")
    ap.add_argument("--tile-faces", type=int, default=128, help="facepass with --vesicles")
    ap.add_argument("--face-kernel", default="simt", choices=["tc", "simt"],
                    help="facepass: regular faces of the FP32 form on the tensor cores or the SIMT kernel")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_seed(rank: int) -> int:
    """Seed of a rank's vesicle set: every rank is an independent replica of the workload."""
    return WORKLOAD["seed"] + 1000 * rank


def over_ranks(x: float, op: str, device) -> float:
    """x reduced over all ranks ("max" or "sum"), returned on every rank."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def face_pass_work(plans, esize: int) -> tuple[float, float, int]:
    """Algorithmic bytes and flops of one face pass over the given plans
    (vesicles: regular faces and valence-5 irregular faces).

    Bytes per face with c control points and q quadrature points: its packed
    control points and their slot destinations (2 x 4c), its gradient
    partials (3c x esize), g0 and the reference angle per point (2q x esize)
    and its composition (3 x esize); per vertex its position once (hi/lo
    pairs, 24 B in the FP32 form; 24 B of FP64 in the plain path) and, in the
    FP32 form, its displacement from the reference state (12 B).
    Flops per quadrature point: the five basis contractions over the c control
    points (5 x 3c FMA), the same contracted back onto them, and about 190
    for the pointwise energy and adjoint; in the FP32 form also the u and v
    rows contracted with the displacements (2 x 3c FMA) and about 30 for the
    area strain formed from them.
    """
    strain = esize == 4
    byts = flops = 0.0
    faces = 0
    for pi in plans:
        for nf, c, q in ((pi.n_regular, 12, 15), (pi.n_irregular, 11, 16)):
            byts += nf * (8 * c + 3 * c * esize + 2 * q * esize + 3 * esize)
            flops += nf * q * (2 * 2 * 5 * 3 * c + 190 + (2 * 2 * 3 * c + 30 if strain else 0))
            faces += nf
        byts += (36.0 if strain else 24.0) * pi.nv
    return byts, flops, faces


def build_vesicles(specs, tmpdir: Path, precision: int, ctx, U, W):
    pp = W.vesicle_plans(specs, tmpdir, precision)
    meshes = [U.Mesh(ctx, plan, prm) for plan, prm in pp]
    return pp, meshes


def time_batch(batch, ctx, stream, torch, K: int) -> float:
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    batch.run(K)
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def workload_config(specs) -> dict:
    """The workload's description: the same dict in both arms' lines."""
    nv = sum(10 * 4 ** s.level + 2 for s in specs)
    nf = sum(20 * 4 ** s.level for s in specs)
    return dict(WORKLOAD, n_vesicles=len(specs), vertices=nv, faces=nf)


def engine_mapped() -> bool:
    """Whether this process has the engine's shared library mapped (the CPU
    legs must not: they run the oracle's restatement alone)."""
    try:
        return "libumcp_gb300" in Path("/proc/self/maps").read_text()
    except OSError:
        return False


class OracleVesicles:
    """The workload's vesicles planned by the oracle (oracle/planner.py, no
    engine code): the vesicle generator, the reference's plan construction
    and setg0, the reference's basis rows; the topology is planned once per
    subdivision level (the generator's connectivity depends on the level only,
    and a vesicle's box of 3 R leaves every control point in its home image)."""

    def __init__(self):
        self.topology = {}

    def surface(self, s):
        from oracle import planner as OP
        from umcp_gb300 import kc_from_kT
        from umcp_gb300 import workloads as W

        m = OP.icosphere(s.level, s.radius, s.sigma, s.seed)
        return OP.Surface(m, kc_from_kT(s.kc_kT), 0.215, lipids=W.lipid_text(s.c0),
                          topology=self.topology.setdefault(s.level, {}))


def _oracle_bd_steps(systems, seconds: float, seed: int, rms: float):
    """Overdamped BD steps (energy + gradient + update, the oracle's C
    restatement) over the systems in turn for `seconds` (each at least once)."""
    from oracle import bridge as OB

    D_dt = rms * rms / 2.0
    kT = 0.592186663194
    steps, vs, t0 = 0, 0, time.perf_counter()
    while True:
        S, r, p, idx = systems[steps % len(systems)]
        S.energy(r)
        g = S.grad(r)
        xi = OB.noise(seed, idx, steps // len(systems), S.nv)
        rv = r[:-3].copy()
        OB.step(0, 1.0, 0.0, kT, D_dt, rv, p, g[:-3], xi)
        r[:-3] = rv
        steps += 1
        vs += S.nv
        el = time.perf_counter() - t0
        if el >= seconds and steps >= len(systems):
            return vs, el, steps


def cpu_port_sample(specs, seconds: float) -> dict:
    """Single-core oracle (restatement of the reference path, planned by the
    oracle itself): energy + gradient + BD update per step over one vesicle
    of each subdivision level of the workload, in turn, for about `seconds`."""
    chosen = [next(s for s in specs if s.level == lvl) for lvl in (2, 3, 4, 5) if any(s.level == lvl for s in specs)]
    ov = OracleVesicles()
    systems = []
    for s in chosen:
        S = ov.surface(s)
        systems.append((S, S.positions.copy(), np.zeros(3 * S.nv), s.index))
    vs, el, steps = _oracle_bd_steps(systems, seconds, WORKLOAD["seed"], WORKLOAD["rms_step_A"])
    levels = "/".join(str(s.level) for s in chosen)
    return {"value": vs / el, "unit": "vertex-steps/s", "cores": 1, "kind": "port",
            "sample": f"{steps} BD steps (energy+gradient+update), one vesicle per step in turn over one vesicle of "
                      f"each subdivision level ({levels}) of the same workload, one core, {el:.1f} s; the oracle's "
                      f"C restatement of the reference path on its own plan of each vesicle (the reference's "
                      f"sources are not on this host)"}


def serving_run(ctx, U, W, seconds: float, rate: float, seed: int, tmpdir: Path) -> dict:
    """Poisson stream of BD jobs into the serving loop; latency = submit to
    result on the host."""
    rng = np.random.default_rng(seed)
    arrivals, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        arrivals.append(t)
    jobs = []
    for i, ta in enumerate(arrivals):
        steps = int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e5)))))
        kc = float(rng.uniform(10.0, 40.0))
        if rng.random() < 0.5:
            level = int(rng.choice([2, 3, 4, 5]))
            R = float(math.exp(rng.uniform(math.log(50.0), math.log(500.0))))
            jobs.append(("vesicle", ta, steps, kc, (level, R, 0.01 * R, seed * 7919 + i)))
        else:
            n = int(rng.choice([32, 48, 64, 80, 96, 112, 128]))
            jobs.append(("planar", ta, steps, kc, (n, seed * 7919 + i)))
    tmpdir.mkdir(parents=True, exist_ok=True)

    def make(ij):
        i, (kind, ta, steps, kc, a) = ij
        path = tmpdir / f"job_{i}.mesh"
        if kind == "vesicle":
            U.generate_icosphere(path, a[0], a[1], a[2], a[3])
        else:
            U.generate_planar(path, a[0], a[0], 10.0, kc, a[1])
        return path

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        paths = list(ex.map(make, enumerate(jobs)))
    srv = U.Server(ctx, U.FP32_CENTRED, chunk_ms=25.0)
    ids = []
    t0 = time.perf_counter()
    for (kind, ta, steps, kc, _), path in zip(jobs, paths):
        d = ta - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        prm = U.params(kc=U.kc_from_kT(kc), KA=0.215, precision=U.FP32_CENTRED)
        ids.append(srv.submit(path, prm, W.bd_integrator(seed, len(ids), WORKLOAD["rms_step_A"]), 0, steps))
    srv.wait_all()
    wall = time.perf_counter() - t0
    st = srv.stats()
    infos = [srv.job(j) for j in ids]
    total_vs = sum(i.nv * i.steps_done for i in infos)
    out = {
        "jobs": len(ids), "failed": int(st.failed), "arrival_rate_per_s": rate, "window_s": seconds,
        "p50_latency_s": st.p50_latency_s, "p99_latency_s": st.p99_latency_s, "mean_latency_s": st.mean_latency_s,
        "max_latency_s": st.max_latency_s, "vertex_steps": total_vs, "wall_s": wall,
        "vertex_steps_per_s": total_vs / wall, "device_busy_vertex_steps_per_s": st.vertex_steps_per_s,
        "chunks": int(st.chunks), "hbm_peak_bytes": st.hbm_peak_bytes,
        "offered_vertex_steps_per_s": total_vs / seconds,
        "jobs_mix": "half vesicles (levels 2-5, R 50-500 A, noise 0.01 R), half planar patches "
                    "(32-128 per side, 10 A lattice, q^-4 heights); kc 10-40 kT; steps log-uniform 1e3-1e5; "
                    "BD sqrt(2 D dt) = 0.02 A; FP32 form with FP64 sums",
    }
    srv.close()
    return out


def planar_variant(ctx, U, W, torch, stream, tmpdir: Path, K: int) -> dict:
    plan, prm = W.planar_plan(tmpdir, 128, 128, 1002, U.FP32_CENTRED)
    mesh = U.Mesh(ctx, plan, prm)
    it = W.bd_integrator(1002, 0, 0.05)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    for s in range(5):
        mesh.run_async(it, s, 1)
    ctx.synchronize()
    st = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    for k in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        st[k].record(stream)
        mesh.run_async(it, 5 + k, 1)
        en[k].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    total = sum(a.elapsed_time(b) for a, b in zip(st, en)) / 1e3
    return {"workload": "planar periodic membrane 128x128 (16,384 vertices), one mesh, FP32, sqrt(2 D dt) = 0.05 A, "
                        "L2 flushed between steps",
            "vertex_steps_per_s": plan.nv * K / total, "ms_per_step": total * 1e3 / K, "steps": K}


FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal


def config1_variant(ctx, U, W, torch, stream, tmpdir: Path, K: int, peak_gbs: float) -> dict:
    """The plain FP64 method on one closed vesicle: an icosahedron subdivided
    3x (642 vertices, 1280 faces), R 100 A, radial noise N(0, 1 A) (seed
    1001), kc 20 kT, c0 0, T 298 K; one energy+gradient, then K overdamped BD
    steps with sqrt(2 D dt) = 0.05 A, timed with CUDA events on the engine's
    stream. Beside it the same vesicle on one host core through the oracle's
    C restatement (its own plan), 20 steps."""
    tmpdir.mkdir(parents=True, exist_ok=True)
    path = tmpdir / "config1.mesh"
    U.generate_icosphere(path, 3, 100.0, 1.0, 1001)
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=U.FP64)
    plan = U.Plan(path, prm)
    mesh = U.Mesh(ctx, plan, prm)
    E0, g0 = mesh.energy_grad(plan.positions())
    it = W.bd_integrator(1001, 0, 0.05)
    mesh.run(it, 0, 32, energies=False)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    mesh.run_async(it, 32, K)
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    r1, _ = mesh.state_get()
    byts, flops, _ = face_pass_work([plan], 8)
    # the same vesicle on one host core, the oracle's own plan
    from oracle import planner as OP

    S = OP.Surface(OP.icosphere(3, 100.0, 1.0, 1001), U.kc_from_kT(20.0), 0.215)
    Ecpu = S.energy(plan.positions())
    systems = [(S, S.positions.copy(), np.zeros(3 * S.nv), 0)]
    vs, el, nsteps = _oracle_bd_steps(systems, 0.0, 1001, 0.05)
    t0 = time.perf_counter()
    for _ in range(20):
        _oracle_bd_steps(systems, 0.0, 1001, 0.05)
    cpu_s = (time.perf_counter() - t0) / 20
    return {"workload": "plain FP64 path, one icosahedral vesicle subdivided 3x (642 vertices, 1280 faces), R 100 A, "
                        "radial noise N(0, 1 A), kc 20 kT, c0 0; one energy+gradient, then BD steps with "
                        "sqrt(2 D dt) = 0.05 A",
            "steps": K, "vertex_steps_per_s": plan.nv * K / sec, "ms_per_step": sec * 1e3 / K,
            "first_energy": E0, "first_energy_rel_err_vs_oracle": abs(E0 - Ecpu) / abs(Ecpu),
            "states_finite": bool(np.all(np.isfinite(r1))),
            "fp64_tflops": flops * K / sec / 1e12, "fp64_frac_of_nominal": flops * K / sec / 1e12 / FP64_NOMINAL_TFLOPS,
            "face_pass_bytes_per_step": byts, "hbm_gbs": byts * K / sec / 1e9, "hbm_frac": byts * K / sec / 1e9 / peak_gbs,
            "note": "the whole mesh's data (about 0.6 MB) stays in L2; one step is two face launches and a fused "
                    "gather-update, captured as CUDA graphs of 32 steps, so the step is launch- and latency-bound "
                    "rather than bound by FP64 issue or HBM",
            "cpu_oracle_1core": {"vertex_steps_per_s": plan.nv / cpu_s, "ms_per_step": cpu_s * 1e3, "cores": 1,
                                 "kind": "port", "sample": "20 BD steps after one untimed step"}}


def langevin_mass_variant(ctx, U, W, torch, stream, tmpdir: Path, K: int, peak_gbs: float) -> dict:
    """Langevin with the limit-surface mass matrix on a 40,962-vertex vesicle
    (icosahedron subdivided 6x, R 1000 A, noise N(0, 2 A), kc 20 kT, c0 0),
    global area and volume restraints (K_area 0.2 kcal/mol/A^2 on the total
    area, K_volume 0.01 kcal/mol/A^6 on the enclosed volume, targets the start
    state), gamma 1/ps, FP32 form with M^-1 applied in FP32 each step.

    The time step: a thermal displacement of 0.05 A per step would take
    dt = 0.05 / sqrt(kT <M^-1_ii>) (about 120 AKMA units here), far beyond the
    stability limits of the leapfrog with friction (gamma dt < 1) and of the
    volume restraint's breathing mode, whose frequency is
    omega = sqrt(K_volume A^2 / M_total); dt = 0.25 / omega is used, and the
    line states both."""
    t0 = time.perf_counter()
    plan, prm = W.large_vesicle(tmpdir, U.FP32_CENTRED)
    mesh = U.Mesh(ctx, plan, prm)
    t1 = time.perf_counter()
    mi = mesh.mass_build(plan)
    t2 = time.perf_counter()
    it_th, minv, dt_thermal = W.langevin_mass_integrator(mesh, plan.nv, 1004)
    omega = math.sqrt(0.01 * mi.area0 ** 2 / (mi.mass_per_point * mi.points))
    dt = min(dt_thermal, 0.25 / omega)
    it = U.integrator(U.LANGEVIN, time_step=dt * W.AKMA_TIME_S, gamma=it_th.gamma, seed=1004,
                      divergence_threshold=1e5, use_mass=1)
    mesh.restraints_set(K_area=0.2, K_volume=0.01)
    r0, _ = mesh.state_get()
    e_warm = mesh.run(it, 0, 32)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    mesh.run_async(it, 32, K)
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    energies = mesh.energies(K)
    r1, _ = mesh.state_get()
    # the M^-1 apply alone: the stored form's bytes (values, columns or runs, row pointers) and the vectors
    n3 = 3 * plan.nv
    a = torch.randn(n3, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    torch.cuda.synchronize()
    mesh.mass_apply_device(a.data_ptr(), b.data_ptr())
    reps = 20
    e0.record(stream)
    for _ in range(reps):
        mesh.mass_apply_device(a.data_ptr(), b.data_ptr())
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    ms_apply = e0.elapsed_time(e1) / reps
    apply_bytes = float(mass_apply_bytes(plan.nv, mi.nnz_inverse, bool(mi.dense), True, mi.column_bytes))
    gbs = apply_bytes / (ms_apply * 1e-3) / 1e9
    return {"workload": "Langevin with the limit-surface M^-1 on a 40,962-vertex vesicle (R 1000 A, noise 2 A, "
                        "kc 20 kT), area and volume restraints, gamma 1/ps, FP32 form",
            "vertex_steps_per_s": plan.nv * K / sec, "ms_per_step": sec * 1e3 / K, "steps": K,
            "energies_finite": bool(np.all(np.isfinite(energies)) and np.all(np.isfinite(e_warm))),
            "energy_first_last": [float(e_warm[0]), float(energies[-1])],
            "rms_displacement_A": float(np.sqrt(np.mean((r1[:-3] - r0[:-3]) ** 2))),
            "time_step_akma": dt, "thermal_0p05A_time_step_akma": dt_thermal, "volume_mode_omega_per_akma": omega,
            "plan_s": t1 - t0, "mass_build_s": t2 - t1,
            "mass_build_split_s": {"assembly": mi.assembly_s, "cholesky_inverse": mi.inverse_s,
                                   "truncation_and_storage": mi.truncation_s},
            "minv_dense": bool(mi.dense), "minv_nnz": int(mi.nnz_inverse),
            "minv_fill": mi.nnz_inverse / plan.nv ** 2,
            "minv_apply": {"ms": ms_apply, "bytes": apply_bytes, "gbs": gbs, "hbm_frac": gbs / peak_gbs,
                           "storage": ("FP32 dense" if mi.dense else "FP32 values, %s columns (CSR)"
                                       % ("uint16" if plan.nv <= 65536 else "int32")),
                           "column_bytes": int(mi.column_bytes)}}


def engine_arm(args) -> None:
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    import umcp_gb300 as U
    from umcp_gb300 import workloads as W

    tmp = Path(tempfile.mkdtemp(prefix="umcp_bench_"))
    ctx = U.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device(f"cuda:{local}"))
    specs = W.vesicle_specs(args.vesicles, replica_seed(rank))
    pp32, meshes32 = build_vesicles(specs, tmp / "fp32", U.FP32_CENTRED, ctx, U, W)
    nv_total = sum(m.nv for m in meshes32)
    K, Wu = args.steps, max(args.warmup, 3)
    batch = U.Batch(ctx, U.FP32_CENTRED)
    for i, m in enumerate(meshes32):
        # one step more than the run takes, so the jobs stay live for the face-pass timing below
        batch.add(m, W.bd_integrator(WORKLOAD["seed"], i, WORKLOAD["rms_step_A"]), 0, Wu + K + 1)
    batch.run(Wu)  # includes the tile-size timing at the first run
    batch.poll()
    info = batch.info()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        total_s = time_batch(batch, ctx, stream, torch, K)
        t_wall = time.perf_counter() - t_wall0
    nv_job = nv_total  # vertices of every rank's vesicles (the ranks' sets differ)
    if world > 1:
        torch.distributed.barrier()
        total_s = over_ranks(total_s, "max", f"cuda:{local}")  # the job's time is its slowest rank's
        nv_job = int(over_ranks(nv_total, "sum", f"cuda:{local}"))
    done, status = batch.poll()
    assert np.all(done == Wu + K) and np.all(status == 0), "a vesicle stopped early"
    value = nv_job * K / total_s

    # ---- roofline: the batch's face launches alone
    F = 30
    fs = [torch.cuda.Event(enable_timing=True) for _ in range(F)]
    fe = [torch.cuda.Event(enable_timing=True) for _ in range(F)]
    for i in range(F):
        fs[i].record(stream)
        batch.face_pass()
        fe[i].record(stream)
    ctx.synchronize()
    face_ms = float(np.mean([a.elapsed_time(b) for a, b in zip(fs, fe)]))
    plan_infos = [p for p, _ in pp32]
    byts, flops, nfaces = face_pass_work(plan_infos, 4)
    peaks = measured_peaks()
    achieved = byts / (face_ms / 1e3) / 1e9
    clocks = clk.summary()
    fp32_peak = SM_COUNT * FP32_LANES_PER_SM * 2 * (clocks.get("sm_mhz") or 2070.0) * 1e6 / 1e12

    out = {
        "metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": K, "warmup": Wu,
        "ms_per_step": total_s * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded vesicles generated on the host)",
        "config": workload_config(specs),
        "engine": {"parallelism": f"replicas x{world}" if world > 1 else "one GPU", "tile_faces": info.tile_faces,
                   "face_grid": list(info.face_grid)},
        "roofline": {"bound": "hbm", "limiter": "FP32 instruction issue (see compute): the HBM fraction is "
                     "small by design, the face work is ~40 flop per byte", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"],
                     "traffic": (BATCH_FACE_DRAM_BYTES_PER_FACE * nfaces) if BATCH_FACE_DRAM_BYTES_PER_FACE else None,
                     "kernel": "batch_face_tpf_kernel (regular faces) and batch_face_kernel (valence-5 and "
                               "valence-7 faces): the face launches of one step",
                     "launch_ms": face_ms, "algorithmic_bytes_per_launch": byts, "peak_source": peaks["source"],
                     "compute": {"fp32_tflops": flops / (face_ms / 1e3) / 1e12, "fp32_simt_peak_tflops": fp32_peak,
                                 "frac": flops / (face_ms / 1e3) / 1e12 / fp32_peak,
                                 "peak_note": "nominal FP32 SIMT rate at the sampled SM clock: "
                                              "152 SMs x 128 lanes x 2 flop x clock"}},
        "clocks": clocks,
        "gpu_launches": info.kernels_per_step * K,
        "wall_s_timed": t_wall,
    }
    if world > 1:
        out["engine"]["vertices_all_ranks"] = nv_job  # each rank its own replica set; config is rank 0's
    e32_first = np.array([m.energies(1)[0] for m in meshes32])
    del batch

    # ---- e2e: the same vesicles driven from the host (umcp_batch_step_host):
    # every step, all jobs' states go in from pinned host memory and the new
    # states and each job's energy come back. The vesicles are independent, so
    # they are driven as E2E_GROUPS batches, each on its own context (stream)
    # from its own host thread: one group's copies run while another computes.
    # Wall clock around K calls of every group.
    import threading

    groups = []
    ngroups = max(1, args.e2e_groups)
    for g in range(ngroups):
        gctx = ctx if g == 0 else U.Context(local)
        idx = list(range(g, len(meshes32), ngroups))
        gm = [meshes32[i] if g == 0 else U.Mesh(gctx, *pp32[i]) for i in idx]
        be = U.Batch(gctx, U.FP32_CENTRED, tile_faces=info.tile_faces)
        for k, m in zip(idx, gm):
            be.add(m, W.bd_integrator(WORKLOAD["seed"] + 7, k, WORKLOAD["rms_step_A"]), 0, Wu + E2E_REPEATS * K)
        npk = sum(3 * m.nv + 3 for m in gm)
        pack_t = torch.empty(npk, dtype=torch.float64, pin_memory=True)
        E_t = torch.empty(len(gm), dtype=torch.float64, pin_memory=True)
        pack_t.numpy()[:] = np.concatenate([m.state_get()[0] for m in gm])
        groups.append((gctx, gm, be, pack_t, E_t))

    def drive(grp, n):
        be, pack_t, E_t = grp[2], grp[3], grp[4]
        for _ in range(n):
            be.step_host(pack_t.data_ptr(), pack_t.data_ptr(), E_t.data_ptr(), 1)

    def drive_all(n):
        ths = [threading.Thread(target=drive, args=(grp, n)) for grp in groups]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    drive_all(Wu)
    walls = []
    for _ in range(E2E_REPEATS):  # the median of a few K-step runs: host threads make single runs noisy
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        drive_all(K)
        w = time.perf_counter() - t0
        walls.append(over_ranks(w, "max", f"cuda:{local}") if world > 1 else w)
    e2e_wall = float(np.median(walls))
    npack = 0
    for grp in groups:
        done_e, st_e = grp[2].poll()
        assert np.all(st_e == 0) and np.all(done_e == Wu + E2E_REPEATS * K) and np.all(np.isfinite(grp[4].numpy())), \
            "a job failed"
        npack += grp[3].numel()
    out["e2e"] = {"value": nv_job * K / e2e_wall, "unit": "vertex-steps/s",
                  "h2d_bytes_per_step": 8.0 * npack, "d2h_bytes_per_step": 8.0 * (npack + len(meshes32)),
                  "path": f"umcp_batch_step_host once per step: every job's state (positions and box scales, "
                          f"packed) copied in from pinned host memory, one batched step, the new states and each "
                          f"job's energy copied back; the {len(meshes32)} vesicles as {ngroups} batches "
                          f"(vesicle i in batch i mod {ngroups}), each on its own context from its own host thread, so "
                          f"one batch's copies overlap another's step; wall clock, median of {E2E_REPEATS} runs",
                  "groups": ngroups, "wall_s": e2e_wall, "wall_s_runs": walls}
    del groups

    if rank == 0 and world == 1:
        # ---- admission: the same vesicles submitted to the serving API as mesh files
        srv = U.Server(ctx, U.FP32_CENTRED, chunk_ms=50.0)
        t0 = time.perf_counter()
        ids = [srv.submit(tmp / "fp32" / f"vesicle_{s.index}.mesh", pp32[s.index][1],
                          W.bd_integrator(WORKLOAD["seed"], s.index, WORKLOAD["rms_step_A"]), 0, K) for s in specs]
        srv.wait_all()
        sub_wall = time.perf_counter() - t0
        jinfo = [srv.job(j) for j in ids]
        assert all(j.status == 0 and j.steps_done == K for j in jinfo), "a served vesicle failed"
        out["admission"] = {"vertex_steps_per_s": nv_total * K / sub_wall, "wall_s": sub_wall, "steps": K,
                            "last_admit_s": max(j.t_admit - j.t_submit for j in jinfo),
                            "path": "umcp_server_submit of the 256 mesh files (plans built on host threads, state "
                                    "uploaded), K steps batched, final states copied to the host; wall clock from "
                                    "the first submit to the last result"}
        srv.close()

        if not args.no_variants:
            var = {}
            # FP64 batch: same vesicles, same initial states
            pp64, meshes64 = build_vesicles(specs, tmp / "fp64", U.FP64, ctx, U, W)
            b64 = U.Batch(ctx, U.FP64)
            K64 = max(20, min(K, 200))
            for i, m in enumerate(meshes64):
                b64.add(m, W.bd_integrator(WORKLOAD["seed"], i, WORKLOAD["rms_step_A"]), 0, 3 + K64)
            b64.run(3)
            b64.poll()
            s64 = time_batch(b64, ctx, stream, torch, K64)
            e64_first = np.array([m.energies(1)[0] for m in meshes64])
            _, fl64, _ = face_pass_work([pl for pl, _ in pp64], 8)
            var["batched_fp64"] = {"vertex_steps_per_s": nv_total * K64 / s64, "steps": K64,
                                   "ms_per_step": s64 * 1e3 / K64,
                                   "fp64_tflops": fl64 * K64 / s64 / 1e12,
                                   "fp64_frac": fl64 * K64 / s64 / 1e12 / FP64_NOMINAL_TFLOPS,
                                   "fp64_peak_note": "face-pass flops of the whole step over its time, against the "
                                                     "nominal 1.25 TFLOP/s dense FP64 of a GB300: the plain path is "
                                                     "bound by the FP64 pipe, not by HBM"}
            del b64
            # FP32 form against FP64 on the same states: every vesicle, at its
            # reference state (where the area forces vanish and only rounding
            # would remain of them) and after the timed steps
            gmax, gl2, emax = [], [], []
            for k in range(len(specs)):
                for r in (pp32[k][0].positions(), meshes32[k].state_get()[0]):
                    E32_, g32 = meshes32[k].energy_grad(r)
                    E64_, g64 = meshes64[k].energy_grad(r)
                    gmax.append(float(np.max(np.abs(g32[:-3] - g64[:-3])) / np.max(np.abs(g64[:-3]))))
                    gl2.append(float(np.linalg.norm(g32[:-3] - g64[:-3]) / np.linalg.norm(g64[:-3])))
                    emax.append(abs(E32_ - E64_) / abs(E64_))
            var["fp32_rel_err"] = {"energy_max": max(emax),
                                   "energy_first_step_max": float(np.max(np.abs(e32_first - e64_first)
                                                                         / np.abs(e64_first))),
                                   "grad_max": max(gmax), "grad_l2_max": max(gl2),
                                   "grad_measure": "per vesicle max|g32-g64|/max|g64| and ||g32-g64||/||g64||, "
                                                   "largest over vesicles and states",
                                   "states": "each vesicle's reference state and its state after the timed steps",
                                   "vesicles": len(specs)}
            # plain FP64 path, one vesicle at a time
            tot_vs, tot_t = 0, 0.0
            for i, m in enumerate(meshes64):
                it = W.bd_integrator(WORKLOAD["seed"], i, WORKLOAD["rms_step_A"])
                m.run(it, 10**6, 32, energies=False)
                ctx.synchronize()
                t0 = time.perf_counter()
                m.run_async(it, 2 * 10**6, 32)
                ctx.synchronize()
                tot_t += time.perf_counter() - t0
                tot_vs += m.nv * 32
            var["plain_fp64_one_by_one"] = {"vertex_steps_per_s": tot_vs / tot_t,
                                            "how": "each vesicle alone on the single-mesh FP64 path, 32 steps "
                                                   "(one captured graph) after a warm-up, wall clock"}
            var["batched_fp32_over_plain_fp64"] = value / var["plain_fp64_one_by_one"]["vertex_steps_per_s"]
            del meshes64
            var["planar128_fp32"] = planar_variant(ctx, U, W, torch, stream, tmp / "planar", 300)
            var["config1_plain_fp64_642"] = config1_variant(ctx, U, W, torch, stream, tmp / "config1", 1000,
                                                            peaks["hbm_gbs"])
            var["langevin_mass_40962"] = langevin_mass_variant(ctx, U, W, torch, stream, tmp / "large", 2000,
                                                               peaks["hbm_gbs"])
            out["variants"] = var
        if args.serve_seconds > 0:
            out["serving"] = serving_run(ctx, U, W, args.serve_seconds, args.serve_rate, 1005, tmp / "serve")
            if "variants" in out:
                out["serving"]["over_plain_fp64_one_by_one"] = (
                    out["serving"]["vertex_steps_per_s"] / out["variants"]["plain_fp64_one_by_one"]["vertex_steps_per_s"])
        out["cpu_baseline"] = cpu_port_sample(specs, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


# ------------------------------------------------------------------ reference arm

def _ref_worker(job):
    """One host process of the reference arm: plans its vesicles with the
    oracle (no engine code), steps each once untimed, then steps them in turn
    for `seconds`. Returns (vertex-steps, seconds, steps, engine library mapped)."""
    specs, seconds, seed, rms = job
    ov = OracleVesicles()
    systems = []
    for s in specs:
        S = ov.surface(s)
        systems.append((S, S.positions.copy(), np.zeros(3 * S.nv), s.index))
    _oracle_bd_steps(systems, 0.0, seed, rms)
    vs, el, steps = _oracle_bd_steps(systems, seconds, seed, rms)
    return vs, el, steps, engine_mapped()


def reference_arm(args) -> None:
    """The reference path on the host cores: the oracle's C restatement of
    surface::energy / surface::grad and the BD update, on the oracle's own
    plan of every vesicle of the workload (one process per core, vesicles
    dealt round robin), for --ref-seconds. The reference's own build cannot
    run here: its sources are not on this host."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    from umcp_gb300 import workloads as W

    specs = W.vesicle_specs(args.vesicles, WORKLOAD["seed"])
    P = min(os.cpu_count() or 1, len(specs))
    per = [specs[i::P] for i in range(P)]
    seconds = max(5.0, args.ref_seconds)
    jobs = [(p, seconds, WORKLOAD["seed"], WORKLOAD["rms_step_A"]) for p in per]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(P) as pool:
        res = pool.map(_ref_worker, jobs)
    wall = time.perf_counter() - t0
    vs = sum(r[0] for r in res)
    el = max(r[1] for r in res)
    steps = sum(r[2] for r in res)
    mapped = engine_mapped() or any(r[3] for r in res)
    value = vs / el
    cfg = workload_config(specs)
    out = {
        "metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 1), "ms_per_step": cfg["vertices"] / value * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded vesicles generated on the host)",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": "vertex-steps/s", "cores": P, "kind": "port",
                         "sample": f"{P} processes, {len(specs)} vesicles dealt round robin ({len(per[0])} or fewer "
                                   f"each), every one planned by the oracle and stepped once untimed, then BD steps "
                                   f"(energy + gradient + update) of each process's vesicles in turn for "
                                   f"{seconds:.0f} s: {steps} steps in all, {wall:.0f} s wall. ms_per_step is one "
                                   f"step of the whole workload at that rate. The oracle's C restatement of the "
                                   f"reference path (the reference's sources are not on this host)."},
        "engine_library_mapped": bool(mapped),
        "e2e": {"value": value, "unit": "vertex-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ------------------------------------------------------------------ profiling modes

def _time_passes(ctx, face_pass, repeat: int) -> float:
    """Microseconds per face pass: `repeat` passes between two CUDA events on
    the context's stream (the first pass of a capture is the profiled one)."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda:0"))
    face_pass()  # untimed
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(repeat):
        face_pass()
    e1.record(stream)
    e1.synchronize()
    ctx.synchronize()
    return e0.elapsed_time(e1) * 1e3 / max(repeat, 1)


def facepass_mode(args) -> None:
    """The per-face pass alone (the dominant kernels), for ncu captures."""
    import umcp_gb300 as U
    from umcp_gb300 import workloads as W

    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    ctx = U.Context(0)
    if args.vesicles:
        with tempfile.TemporaryDirectory() as td:
            pp = W.vesicle_plans(W.vesicle_specs(args.vesicles, WORKLOAD["seed"]), Path(td), prec)
        meshes = [U.Mesh(ctx, plan, prm) for plan, prm in pp]
        batch = U.Batch(ctx, prec, tile_faces=args.tile_faces)
        for i, m in enumerate(meshes):
            batch.add(m, W.bd_integrator(WORKLOAD["seed"], i, WORKLOAD["rms_step_A"]), 0, 4)  # live after three steps
        batch.run(3)
        done, st = batch.poll()
        us = _time_passes(ctx, batch.face_pass, args.repeat)
        info = batch.info()
        print(f"vesicles={info.n_jobs} vertices={info.n_vertices} faces={info.n_faces} tiles={list(info.n_tiles)} "
              f"steps={int(done.min())} status={int(st.max())} face_pass_us={us:.1f}")
        return
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=prec,
                   face_kernel=U.TENSOR_CORES if args.face_kernel == "tc" else U.SIMT)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "m.mesh"
        if args.icosphere:
            U.generate_icosphere(path, args.icosphere, 1000.0, 2.0, 7)
        else:
            U.generate_planar(path, args.nx, args.ny, 10.0, 20.0, 7)
        plan = U.Plan(path, prm)
    mesh = U.Mesh(ctx, plan, prm)
    E, _ = mesh.energy_grad(plan.positions())
    us = _time_passes(ctx, mesh.face_pass, args.repeat)
    info = mesh.info()
    print(f"faces={info.n_faces} points={info.n_points} E={E:.10g} face_pass_us={us:.1f}")


def geo_mode(args) -> None:
    """Energy and gradient of one vesicle (icosahedron subdivided --level times,
    radius --radius) with and without the global area and volume restraints
    (K_area 0.2, K_volume 0.01), on the device: the restraint kernels' cost,
    and a launch sequence for their ncu captures. At the state's own targets
    the restraint gradient is zero and its kernel returns at once; with the
    targets 1% off (as under dynamics) it runs."""
    import torch
    import umcp_gb300 as U

    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    ctx = U.Context(0)
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=prec)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "v.mesh"
        U.generate_icosphere(path, args.level, args.radius, 2.0, 7)
        plan = U.Plan(path, prm)
    mesh = U.Mesh(ctx, plan, prm)
    d_r = torch.tensor(plan.positions(), dtype=torch.float64, device="cuda:0")
    d_E = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    d_g = torch.zeros(d_r.numel(), dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda:0"))
    torch.cuda.synchronize()

    def timed() -> float:
        mesh.energy_grad_device(d_r.data_ptr(), d_E.data_ptr(), d_g.data_ptr())  # untimed
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.repeat):
            mesh.energy_grad_device(d_r.data_ptr(), d_E.data_ptr(), d_g.data_ptr())
        e1.record(stream)
        e1.synchronize()
        ctx.synchronize()
        return e0.elapsed_time(e1) * 1e3 / max(args.repeat, 1)

    plain = timed()
    mesh.restraints_set(K_area=0.2, K_volume=0.01)
    restrained = timed()
    A, V, Er = mesh.restraints_get()
    mesh.restraints_set(K_area=0.2, area0=0.99 * A, K_volume=0.01, volume0=0.99 * V)
    active = timed()
    print(f"vertices={plan.nv} faces={mesh.info().n_faces} energy_grad_us={plain:.1f} "
          f"with_restraints_us={restrained:.1f} restraints_us={restrained - plain:.1f} "
          f"with_active_restraints_us={active:.1f} restraint_gradient_us={active - restrained:.1f} "
          f"A={A:.6f} V={V:.6f}")


def mass_apply_bytes(nrow: int, nnz: int, dense: bool, fp32: bool, column_bytes: int) -> int:
    """Algorithmic bytes of one apply, out += M^-1 in on 3 components per row:
    sparse, the values (4 per nonzero in FP32, 8 in FP64) and the stored
    columns (column_bytes: 4 or 2 per nonzero) plus, per row, the row pointer (4), the input
    gathered at least once (16 as the packed FP32 copy, 24 in FP64) and the
    output read and written (48); dense 4 (or 8) per entry plus the same per
    row without the pointer."""
    per_row = (0 if dense else 4) + (16 if fp32 else 24) + 48
    if dense:
        return (4 if fp32 else 8) * nrow * nrow + per_row * nrow
    return (4 if fp32 else 8) * nnz + column_bytes + per_row * nrow


def massapply_mode(args) -> None:
    """Times the effective-mass inverse apply (umcp_mass_apply_device)."""
    import torch

    import umcp_gb300 as U

    fp32 = args.precision == "fp32"
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=U.FP32_CENTRED if fp32 else U.FP64)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "vesicle.mesh"
        U.generate_icosphere(path, args.level, args.radius, 2.0, 7)
        plan = U.Plan(path, prm)
    ctx = U.Context(0)
    mesh = U.Mesh(ctx, plan, prm)
    info = mesh.mass_build(plan)
    nrow = mesh.nv
    dev = torch.device("cuda:0")
    x = torch.randn(3 * nrow, dtype=torch.float64, generator=torch.Generator().manual_seed(7)).to(dev)
    y = torch.zeros(3 * nrow, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    for _ in range(3):
        mesh.mass_apply_device(x.data_ptr(), y.data_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.repeat):
        mesh.mass_apply_device(x.data_ptr(), y.data_ptr())
    e1.record(stream)
    e1.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / max(args.repeat, 1)
    nbytes = mass_apply_bytes(nrow, info.nnz_inverse, bool(info.dense), fp32, info.column_bytes)
    fill = info.nnz_inverse / float(nrow * nrow)
    form = {1: "dense", 2: "csr"}[mesh.info().mass_form]
    print(f"rows={nrow} nnz={info.nnz_inverse} fill={fill:.3f} {form} {args.precision} "
          f"apply {us:.1f} us bytes={nbytes} ({nbytes / (us * 1e-6) / 1e9:.0f} GB/s) "
          f"finite={bool(torch.isfinite(y).all().item())}")


def main() -> None:
    args = parse_args()
    if args.mode == "facepass":
        facepass_mode(args)
    elif args.mode == "massapply":
        massapply_mode(args)
    elif args.mode == "geo":
        geo_mode(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        engine_arm(args)


if __name__ == "__main__":
    main()
