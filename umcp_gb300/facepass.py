"""Runs the per-face pass (the dominant kernel) on a synthetic membrane, for
profiling: `python -m umcp_gb300.facepass --nx 512 --ny 512 --precision fp32
--repeat 3`. The pass is queued `repeat` times after one energy+gradient call.

With --vesicles N it runs the batched face launches instead, over the first N
vesicles of the mixed-vesicle benchmark workload, after three batched BD
steps at a fixed tile size (--tile-faces): `python -m umcp_gb300.facepass
--vesicles 64 --tile-faces 128 --repeat 3`.
"""
from __future__ import annotations

import argparse
import tempfile
from pathlib import Path

import umcp_gb300 as U


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=512)
    ap.add_argument("--icosphere", type=int, default=0, help="use an icosahedral vesicle of this level instead")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--vesicles", type=int, default=0)
    ap.add_argument("--tile-faces", type=int, default=128)
    ap.add_argument("--face-kernel", default="simt", choices=["tc", "simt"],
                    help="regular faces of the FP32 form on the tensor cores or the SIMT kernel")
    args = ap.parse_args()
    if args.vesicles:
        return batch_main(args)
    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=prec,
                   face_kernel=U.TENSOR_CORES if args.face_kernel == "tc" else U.SIMT)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "m.mesh"
        if args.icosphere:
            U.generate_icosphere(path, args.icosphere, 1000.0, 2.0, 7)
        else:
            U.generate_planar(path, args.nx, args.ny, 10.0, 20.0, 7)
        plan = U.Plan(path, prm)
    ctx = U.Context(0)
    mesh = U.Mesh(ctx, plan, prm)
    E, _ = mesh.energy_grad(plan.positions())
    for _ in range(args.repeat):
        mesh.face_pass()
    ctx.synchronize()
    info = mesh.info()
    print(f"faces={info.n_faces} points={info.n_points} E={E:.10g}")


def batch_main(args) -> None:
    from umcp_gb300 import workloads as W

    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    ctx = U.Context(0)
    with tempfile.TemporaryDirectory() as td:
        pp = W.vesicle_plans(W.vesicle_specs(args.vesicles, 1003), Path(td), prec)
    meshes = [U.Mesh(ctx, plan, prm) for plan, prm in pp]
    batch = U.Batch(ctx, prec, tile_faces=args.tile_faces)
    for i, m in enumerate(meshes):
        batch.add(m, W.bd_integrator(1003, i), 0, 4)  # live after the three steps: the passes below do work
    batch.run(3)
    done, st = batch.poll()
    for _ in range(args.repeat):
        batch.face_pass()
    ctx.synchronize()
    info = batch.info()
    print(f"vesicles={info.n_jobs} vertices={info.n_vertices} faces={info.n_faces} tiles={list(info.n_tiles)} "
          f"steps={int(done.min())} status={int(st.max())}")


if __name__ == "__main__":
    main()
