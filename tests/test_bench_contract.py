"""bench.py on CPU: the reference arm's JSON line, and the algorithmic byte
counts behind the roofline entries.

The reference arm runs the oracle's C restatement of the reference path on the
host cores, on plans the oracle builds itself: the engine's library must not be
mapped in any of its processes. The byte counts are pinned to the figures the
GPU runs print for the benchmark workloads, so a change to a formula shows up
here before it reaches a bench line."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from umcp_gb300 import workloads as W  # noqa: E402


def test_reference_arm_prints_the_contract_line_without_the_engine():
    run = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--vesicles", "4", "--ref-seconds", "5",
                          "--steps", "2", "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=240)
    assert run.returncode == 0, run.stderr[-2000:]
    line = json.loads([x for x in run.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "vertex-steps/s"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["config"]["workload"] == bench.WORKLOAD["workload"] and line["config"]["n_vesicles"] == 4
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "vertex-steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["engine_library_mapped"] is False


def _vesicle_plan(level: int) -> SimpleNamespace:
    """Face and vertex counts of a Loop-subdivided icosahedron: 12 valence-5
    vertices, each with 5 irregular faces."""
    faces, nv = 20 * 4 ** level, 10 * 4 ** level + 2
    return SimpleNamespace(n_regular=faces - 60, n_irregular=60, nv=nv)


def test_face_pass_bytes_of_the_benchmark_batch():
    """The batch's algorithmic bytes per face launch (the roofline entry's
    algorithmic_bytes_per_launch of the 256-vesicle FP32 workload)."""
    plans = [_vesicle_plan(s.level) for s in W.vesicle_specs(256, bench.WORKLOAD["seed"])]
    byts, flops, faces = bench.face_pass_work(plans, 4)
    assert faces == 1646720 and sum(p.nv for p in plans) == 823872
    assert byts == 642054912.0
    # per point: the five contractions both ways, the displacement rows, the pointwise step and the strain
    assert flops == sum(p.n_regular * 15 * (720 + 190 + 144 + 30) + p.n_irregular * 16 * (660 + 190 + 132 + 30)
                        for p in plans)


def test_mass_apply_bytes_of_the_stored_forms():
    """M^-1 apply bytes: the 40,962-vertex truncated inverse as FP32 CSR with
    16-bit columns, and the 10,242-vertex inverse kept dense."""
    nnz = 414828282
    assert bench.mass_apply_bytes(40962, nnz, False, True, 2 * nnz) == 2491755108
    assert bench.mass_apply_bytes(10242, 79099782, True, True, 0) == 420249744
    # FP64 CSR: 8-byte values and 4-byte columns
    assert bench.mass_apply_bytes(100, 1000, False, False, 4000) == 12 * 1000 + (4 + 24 + 48) * 100
