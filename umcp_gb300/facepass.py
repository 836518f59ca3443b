"""Runs the per-face pass (the dominant kernel) on a synthetic membrane, for
profiling: `python -m umcp_gb300.facepass --nx 512 --ny 512 --precision fp32
--repeat 3`. The pass is queued `repeat` times after one energy+gradient call.
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
    args = ap.parse_args()
    prec = U.FP32_CENTRED if args.precision == "fp32" else U.FP64
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=prec)
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


if __name__ == "__main__":
    main()
