"""Applies the effective-mass inverse (umcp_mass_apply_device) on an
icosahedral vesicle, for profiling and timing: `python -m umcp_gb300.massapply
--level 5 --repeat 20`. M^-1 is built by umcp_mass_build at the reference's
settings (66 mass points per face, truncation 1e-20); then `repeat` applies
are timed with CUDA events on the context's stream, after 3 untimed ones.

Algorithmic bytes of one apply, out += M^-1 in on 3 components per row:
CSR 8 per nonzero (FP32 value and column; 12 in FP64) plus, per row, the row
pointer (4), the input gathered at least once (16 as the packed FP32 copy, 24
in FP64) and the output read and written (48); dense 4 (or 8) per entry plus
the same per row.
"""
from __future__ import annotations

import argparse
import tempfile
from pathlib import Path

import torch

import umcp_gb300 as U


def apply_bytes(nrow: int, nnz: int, dense: bool, fp32: bool) -> int:
    per_entry = (4 if fp32 else 8) if dense else (8 if fp32 else 12)
    entries = nrow * nrow if dense else nnz
    per_row = (0 if dense else 4) + (16 if fp32 else 24) + 48
    return per_entry * entries + per_row * nrow


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--level", type=int, default=5, help="Loop subdivisions of the icosahedron (5: 10,242 vertices)")
    ap.add_argument("--radius", type=float, default=1000.0)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--repeat", type=int, default=20)
    args = ap.parse_args()
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
    nbytes = apply_bytes(nrow, info.nnz_inverse, bool(info.dense), fp32)
    fill = info.nnz_inverse / float(nrow * nrow)
    print(f"rows={nrow} nnz={info.nnz_inverse} fill={fill:.3f} {'dense' if info.dense else 'csr'} {args.precision} "
          f"apply {us:.1f} us bytes={nbytes} ({nbytes / (us * 1e-6) / 1e9:.0f} GB/s) "
          f"finite={bool(torch.isfinite(y).all().item())}")


if __name__ == "__main__":
    main()
