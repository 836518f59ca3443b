#!/usr/bin/env python3
"""BD vertex-steps/s of the membrane-surface hot path on one GB300 (or N, one
independent membrane replica per GPU).

Workload (one step = energy + gradient + overdamped BD update of the whole
membrane): the planar periodic membrane of 128 x 128 vertices (16,384
vertices, 32,768 faces, all valence 6), lattice spacing 10 A, q^-4 height
spectrum for kc = 20 kT, KA = 0.215, FP32 face-centred patch arithmetic with
FP64 sums and FP64 position update; BD step with sqrt(2 D dt) = 0.05 A.

  value   device-resident throughput: each timed step is bracketed by CUDA
          events on the engine's stream; L2 is flushed (a write larger than L2)
          between steps, outside the events.
  e2e     the same steps through the host-buffer C-ABI call umcp_step_host
          (state copied in and out every step), wall clock.
  roofline  the per-face pass (the dominant kernel) timed alone with CUDA
          events, algorithmic bytes per launch / duration against the measured
          HBM copy bandwidth; its FP32 flop rate is reported beside it.
  cpu_baseline  the oracle's C restatement of the reference path on one host
          core, a bounded sample of the same workload.

--impl reference runs the CPU restatement of the reference path (the
reference's own code cannot run here) with all host cores, faces partitioned
across processes as the reference's MPI runs partition them.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {
    "workload": "planar periodic membrane 128x128 (16384 vertices, 32768 faces), BD, FP32 face-centred",
    "nx": 128, "ny": 128, "lattice_A": 10.0, "kc_kT": 20.0, "KA": 0.215, "seed": 1002,
    "rms_step_A": 0.05, "quadrature": "15-point regular rule", "l2": "flushed between timed steps",
}
METRIC = "BD vertex-steps/s"
L2_BYTES = 129 * 1024 * 1024
KT298 = 0.592186663194
# DRAM bytes per face of one face pass, from the ncu capture of the 512x512
# membrane (dram__bytes_read.sum + dram__bytes_write.sum = 166.76 MB over
# 524,288 faces); the benchmark's pass is scaled from it by its face count.
FACE_PASS_DRAM_BYTES_PER_FACE = 166.757e6 / 524288
SM_COUNT, FP32_LANES_PER_SM = 152, 128


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_membrane(tmpdir: Path, seed: int):
    import umcp_gb300 as U

    path = tmpdir / f"membrane_{seed}.mesh"
    U.generate_planar(path, WORKLOAD["nx"], WORKLOAD["ny"], WORKLOAD["lattice_A"], WORKLOAD["kc_kT"], seed)
    return path


def bd_integrator(seed: int, stream: int):
    import umcp_gb300 as U

    D_dt = WORKLOAD["rms_step_A"] ** 2 / 2.0  # sqrt(2 D dt) = 0.05 A
    return U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=D_dt, seed=seed, stream=stream)


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
        return {"hbm_gbs": d.get("hbm_gbs"), "bf16_tflops": d.get("bf16_tflops"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def face_pass_work(info, esize: int) -> tuple[float, float]:
    """Algorithmic bytes and flops of one face pass.

    Bytes: every vertex position read once (24 B), per face its 12 packed
    control points (48 B), per quadrature point g0 and the reference angle
    (2 x esize), the face's composition (3 x esize), its gradient partials
    (12 x 3 x esize) and its six FP64 sums (48 B).
    Flops per quadrature point: the five basis contractions over 12 control
    points (5 x 12 x 3 FMA = 360), the pointwise energy and adjoint (190),
    the adjoint contracted back onto the 12 control points (360): 910.
    """
    nf, npts = info.n_faces, info.n_points
    ncp = 12
    byts = 24.0 * info.nv + nf * (4 * ncp + 3 * esize + ncp * 3 * esize + 48) + npts * 2 * esize
    flops = 910.0 * npts
    return byts, flops


def cpu_port_sample(mesh_path: Path, prm, seconds: float) -> dict:
    """Single-core oracle (restatement of the reference path) on the same
    membrane: energy + gradient + BD update per step, for about `seconds`."""
    import umcp_gb300 as U
    from oracle import bridge as OB

    plan = U.Plan(mesh_path, prm)
    O = OB.Oracle(plan, prm)
    r = plan.positions()
    p = np.zeros(3 * plan.nv)
    kT = KT298
    D_dt = WORKLOAD["rms_step_A"] ** 2 / 2.0
    steps, t0 = 0, time.perf_counter()
    while True:
        E = O.energy(r)
        g = O.grad(r)
        xi = OB.noise(1, 0, steps, plan.nv)
        rv = r[:-3].copy()
        OB.step(0, 1.0, 0.0, kT, D_dt, rv, p, g[:-3], xi)
        r[:-3] = rv
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    assert math.isfinite(E)
    return {"value": plan.nv * steps / el, "unit": "vertex-steps/s", "cores": 1, "kind": "port",
            "sample": f"{steps} full BD steps (energy+gradient+update) of the same {plan.nv}-vertex membrane on one "
                      f"core, {el:.1f} s; oracle C restatement of the reference path (the reference cannot be "
                      f"compiled on this host)"}


def engine_arm(args) -> None:
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    import umcp_gb300 as U

    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    prm = U.params(kc=U.kc_from_kT(WORKLOAD["kc_kT"]), KA=WORKLOAD["KA"], precision=prec)
    tmp = Path(tempfile.mkdtemp(prefix="umcp_bench_"))
    mesh_path = make_membrane(tmp, WORKLOAD["seed"] + rank)
    plan = U.Plan(mesh_path, prm)
    ctx = U.Context(local)
    mesh = U.Mesh(ctx, plan, prm)
    info = mesh.info()
    it = bd_integrator(seed=WORKLOAD["seed"], stream=rank)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device(f"cuda:{local}"))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    def l2_flush():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    step = 0
    for _ in range(max(args.warmup, 3)):
        l2_flush()
        mesh.run_async(it, step, 1)
        step += 1
    ctx.synchronize()

    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        for k in range(K):
            l2_flush()
            starts[k].record(stream)
            mesh.run_async(it, step, 1)
            stops[k].record(stream)
            step += 1
        ctx.synchronize()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if world > 1:
        torch.distributed.barrier()
    step_ms = np.array([a.elapsed_time(b) for a, b in zip(starts, stops)])
    total_s = float(step_ms.sum()) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    value = info.nv * K * world / total_s
    r_state, _ = mesh.state_get()
    assert np.all(np.isfinite(r_state)), "state became non-finite"

    # ---- roofline: the per-face pass alone
    F = 50
    fs = [torch.cuda.Event(enable_timing=True) for _ in range(F)]
    fe = [torch.cuda.Event(enable_timing=True) for _ in range(F)]
    for i in range(F):
        l2_flush()
        fs[i].record(stream)
        mesh.face_pass()
        fe[i].record(stream)
    ctx.synchronize()
    face_ms = float(np.mean([a.elapsed_time(b) for a, b in zip(fs, fe)]))
    esize = 4 if prec == U.FP32_CENTRED else 8
    byts, flops = face_pass_work(info, esize)
    peaks = measured_peaks()
    achieved = byts / (face_ms / 1e3) / 1e9

    # ---- e2e through the host-buffer C-ABI step
    r_host = plan.positions()
    n_e2e = max(1, args.e2e_steps)
    for s in range(3):
        mesh.step_host(it, 10**6 + s, r_host)
    t0 = time.perf_counter()
    for s in range(n_e2e):
        mesh.step_host(it, 2 * 10**6 + s, r_host)
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_val = info.nv * n_e2e * world / e2e_s

    clocks = clk.summary()
    fp32_peak = SM_COUNT * FP32_LANES_PER_SM * 2 * (clocks.get("sm_mhz") or 2070.0) * 1e6 / 1e12
    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_port_sample(mesh_path, U.params(kc=prm.kc, KA=prm.KA, precision=U.FP64), args.cpu_seconds)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": K,
            "warmup": max(args.warmup, 3), "ms_per_step": total_s * 1e3 / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == U.FP32_CENTRED else "f64",
            "data": "synthetic (seeded q^-4 membrane, generated on the host)",
            "config": dict(WORKLOAD, precision=args.precision, vertices=info.nv, faces=info.n_faces,
                           parallelism=f"replicas x{world}"),
            "e2e": {"value": e2e_val, "unit": "vertex-steps/s", "h2d_bytes_per_step": 8 * (3 * info.nv + 3),
                    "d2h_bytes_per_step": 8 * (3 * info.nv + 3) + 8},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"],
                         "traffic": FACE_PASS_DRAM_BYTES_PER_FACE * info.n_faces,
                         "kernel": "face_kernel (per-face pass)", "launch_ms": face_ms,
                         "algorithmic_bytes_per_launch": byts, "peak_source": peaks["source"],
                         "compute": {"fp32_tflops": flops / (face_ms / 1e3) / 1e12,
                                     "fp32_simt_peak_tflops": fp32_peak,
                                     "frac": flops / (face_ms / 1e3) / 1e12 / fp32_peak,
                                     "peak_note": "nominal FP32 SIMT rate at the sampled SM clock: "
                                                  "152 SMs x 128 lanes x 2 flop x clock"}},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": info.kernels_per_step * K,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------------------------ reference arm

def _ref_worker_init(mesh_path, kc, KA):
    global _W
    import umcp_gb300 as U
    from oracle import bridge as OB

    prm = U.params(kc=kc, KA=KA)
    plan = U.Plan(mesh_path, prm)
    _W = OB.Oracle(plan, prm)


def _ref_worker(job):
    r, f0, f1 = job
    g = np.zeros(len(r))
    e = _W.energy_grad_faces(r, f0, f1, g)
    return e, g


def reference_arm(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    import umcp_gb300 as U
    from oracle import bridge as OB

    prm = U.params(kc=U.kc_from_kT(WORKLOAD["kc_kT"]), KA=WORKLOAD["KA"])
    tmp = Path(tempfile.mkdtemp(prefix="umcp_ref_"))
    mesh_path = make_membrane(tmp, WORKLOAD["seed"])
    plan = U.Plan(mesh_path, prm)
    nfaces = plan.n_regular + plan.n_irregular
    cores = os.cpu_count() or 1
    P = cores
    r = plan.positions()
    p = np.zeros(3 * plan.nv)
    D_dt = WORKLOAD["rms_step_A"] ** 2 / 2.0
    ctx = mp.get_context("spawn")
    with ctx.Pool(P, initializer=_ref_worker_init, initargs=(str(mesh_path), prm.kc, prm.KA)) as pool:
        def one_step(s, nf):
            sb = np.linspace(0, nf, P + 1).astype(int)
            jobs = [(r, int(sb[i]), int(sb[i + 1])) for i in range(P)]
            res = pool.map(_ref_worker, jobs)
            g = sum(x[1] for x in res)
            xi = OB.noise(1, 0, s, plan.nv)
            rv = r[:-3].copy()
            OB.step(0, 1.0, 0.0, KT298, D_dt, rv, p, g[:-3], xi)
            r[:-3] = rv

        # Warm-up with whole-membrane steps; their time sizes the sample so the
        # timed run stays near two minutes: each timed step is the energy,
        # gradient and BD update of a fixed slice of the faces (all of them
        # when that fits), split over all host cores.
        t0 = time.perf_counter()
        for s in range(max(args.warmup, 1)):
            one_step(s, nfaces)
        t_full = (time.perf_counter() - t0) / max(args.warmup, 1)
        sample_faces = int(min(nfaces, max(P * 64, nfaces * 120.0 / max(args.steps * t_full, 1e-9))))
        t0 = time.perf_counter()
        for s in range(args.steps):
            one_step(100000 + s, sample_faces)
        el = time.perf_counter() - t0
    frac = sample_faces / nfaces
    value = plan.nv * frac * args.steps / el
    out = {
        "metric": METRIC, "value": value, "unit": "vertex-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 1), "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded q^-4 membrane, generated on the host)",
        "config": dict(WORKLOAD, precision="fp64", vertices=plan.nv, faces=nfaces, parallelism=f"{P} host processes"),
        "cpu_baseline": {"value": value, "unit": "vertex-steps/s", "cores": P, "kind": "port",
                         "sample": f"per step: energy+gradient of {sample_faces} of {nfaces} faces "
                                   f"({frac:.4f} of the membrane) split over {P} processes, plus the BD update; "
                                   f"vertex-steps counted pro rata. Oracle C restatement of the reference path "
                                   f"(the reference's own build needs its source tree, absent here)."},
        "e2e": {"value": value, "unit": "vertex-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main() -> None:
    args = parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        engine_arm(args)


if __name__ == "__main__":
    main()
