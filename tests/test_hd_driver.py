"""Restart files in the reference's save format and the hd-style driver
(umcp_gb300/lib/hd_gb300): the t: lines, the save at the end, resuming
from a save, and the same trajectory as the library calls give."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import GOLDEN, load_case
from umcp_gb300 import build as UB

pytestmark = pytest.mark.gpu


def _lines(path):
    return path.read_text().splitlines()


def test_restart_round_trip_and_format(tmp_path):
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico2_plain")
    m = U.Mesh(ctx, plan, prm)
    m.run(U.integrator(U.LANGEVIN, time_step=1e-15, gamma=10.0, seed=4), 0, 5)
    r, p = m.state_get()
    f = tmp_path / "a.save"
    m.restart_write(f, seed=77)
    L = _lines(f)
    assert len(L) == 1 + plan.nv + 1 + 1
    assert len(L[0].split()) == 3 and all(len(x.split()) == 6 for x in L[1:-1]) and L[-1] == "seed 77"
    m2 = U.Mesh(ctx, plan, prm)
    assert m2.restart_read(f) == 77
    r2, p2 = m2.state_get()
    assert np.max(np.abs(r2 - r)) <= 5e-7 and np.max(np.abs(p2 - p)) <= 5e-7


def test_restart_reads_position_only_lines_and_particle_records(tmp_path):
    ctx = U.Context(0)
    plan, prm, _ = load_case("ico2_plain")
    r = plan.positions()
    r[:-3] += 0.25
    rows = ["1.0 1.0 1.0"] + [f"{r[3*v]:.6f} {r[3*v+1]:.6f} {r[3*v+2]:.6f}" for v in range(plan.nv)] + ["1.0 1.0 1.0"]
    rows += ["1", "203 0.549946 0.388415 0.0 0.0 0.0 0.0 0.0"]  # a particle record, as reference saves hold
    f = tmp_path / "b.save"
    f.write_text("\n".join(rows) + "\n")
    m = U.Mesh(ctx, plan, prm)
    assert m.restart_read(f) == -1
    r2, p2 = m.state_get()
    assert np.max(np.abs(r2 - r)) <= 5e-7 and not p2.any()


def test_driver_runs_saves_and_resumes(tmp_path):
    plan, prm, _ = load_case("ico2_plain")
    inp = tmp_path / "run.inp"
    params = (GOLDEN / "ico2_plain.params").read_text()
    inp.write_text(f"mesh {GOLDEN / 'ico2_plain.mesh'}\njobname {tmp_path / 'job'}\n{params}do_ld yes\n"
                   "time_step 1e-15\ngamma_langevin 10\nnsteps 3\no_lim 4\nseed 9\n")
    res = subprocess.run([str(UB.HD_EXE), str(inp)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    tl = [x for x in res.stdout.splitlines() if x.startswith("t: ")]
    assert len(tl) == 3 and " o: 2 " in tl[2] and "VMEM:" in tl[0]
    saved = tmp_path / "job.save"
    assert saved.exists() and not (tmp_path / "job_crash0.save").exists()
    # the same run through the library
    ctx = U.Context(0)
    m = U.Mesh(ctx, plan, prm)
    m.mass_build(plan)
    it = U.integrator(U.LANGEVIN, time_step=1e-15, gamma=10.0, seed=9, divergence_threshold=1e5, use_mass=1)
    for o in range(3):
        m.run(it, 4 * o, 4)
    r, _ = m.state_get()
    m2 = U.Mesh(ctx, plan, prm)
    assert m2.restart_read(saved) == 9
    assert np.max(np.abs(m2.state_get()[0] - r)) <= 5e-7
    # resume from the save for one more iteration
    res = subprocess.run([str(UB.HD_EXE), str(inp), f"load={saved}", "nsteps=1", f"jobname={tmp_path / 'job2'}"],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "Loaded" in res.stdout, res.stderr
    assert (tmp_path / "job2.save").exists()


def test_driver_minimizes_first_and_restarts_the_temperature_average(tmp_path):
    """nmin runs the reference's L-BFGS before the dynamics; nequil restarts
    AV_TEMP at that outer iteration; kv and planar_topology (inert on the
    membrane path) are accepted."""
    inp = tmp_path / "run.inp"
    params = (GOLDEN / "ico2_plain.params").read_text()
    inp.write_text(f"mesh {GOLDEN / 'ico2_plain.mesh'}\njobname {tmp_path / 'job'}\n{params}do_ld yes\n"
                   "time_step 1e-15\ngamma_langevin 10\nnsteps 4\no_lim 3\nseed 9\nnmin 1\nnequil 2\nkv 0.01\n"
                   "planar_topology no\n")
    res = subprocess.run([str(UB.HD_EXE), str(inp)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    assert "minimization 0:" in res.stdout
    tl = [x.split() for x in res.stdout.splitlines() if x.startswith("t: ")]
    temp = [float(x[x.index("TEMP:") + 1]) for x in tl]
    av = [float(x[x.index("AV_TEMP") + 1]) for x in tl]
    assert len(tl) == 4
    assert abs(av[1] - (temp[0] + temp[1]) / 2) <= 1e-6 * abs(av[1])
    assert abs(av[3] - (temp[2] + temp[3]) / 2) <= 1e-6 * abs(av[3])
