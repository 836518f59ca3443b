"""Batches: every job of a batch follows the trajectory its mesh takes when
run alone (umcp_run with the same integrator, first step and step count).

Positions and momenta are compared bit for bit: the per-face and per-vertex
arithmetic of the batch is the single-mesh path's, and the gradient partials
are summed per vertex in the same slot order. Energies are sums over tiles
instead of over the single-mesh grid's blocks, so they agree to rounding:
1e-12 relative in FP64, 1e-6 in the FP32 precision form.
"""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import load_case

pytestmark = pytest.mark.gpu

CASES = ["ico2_plain", "ico3_deformed", "planar12_deformed", "ico2_lipids"]
E_TOL = {U.FP64: 1e-12, U.FP32_CENTRED: 1e-6}


@pytest.fixture(scope="module")
def ctx():
    return U.Context(0)


def _integrators():
    return [
        U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.00125, seed=7, stream=1),
        U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.002, seed=7, stream=2),
        U.integrator(U.LANGEVIN, time_step=1e-15, gamma=10.0, seed=9, stream=3),
        U.integrator(U.BD_MEMBRANE, time_step=1e-15, gamma=10.0, seed=9, stream=4),
    ]


def _mesh(ctx, name, precision):
    plan, prm, _ = load_case(name, precision)
    return U.Mesh(ctx, plan, prm)


def _alone(ctx, name, precision, it, step0, n):
    m = _mesh(ctx, name, precision)
    e = m.run(it, step0, n)
    r, p = m.state_get()
    return r, p, e


def _check_job(mesh, ref, n, precision):
    r, p = mesh.state_get()
    assert np.array_equal(r, ref[0])
    assert np.array_equal(p, ref[1])
    e = mesh.energies(n)
    assert np.max(np.abs(e - ref[2][:n]) / np.abs(ref[2][:n])) <= E_TOL[precision]


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_batch_jobs_equal_their_alone_runs(ctx, precision):
    its = _integrators()
    batch = U.Batch(ctx, precision)
    meshes = []
    for k, name in enumerate(CASES):
        m = _mesh(ctx, name, precision)
        batch.add(m, its[k], 100 * k, 70)
        meshes.append(m)
    batch.run(70)  # two captured 32-step chunks and 6 single steps
    done, st = batch.poll()
    assert list(done) == [70] * len(CASES) and list(st) == [0] * len(CASES)
    info = batch.info()
    assert info.n_jobs == len(CASES) and info.tile_faces > 0 and info.tuned_face_ms > 0
    assert info.kernels_per_step == 4  # regular and valence-5 faces, reduce, gather + update
    for k, name in enumerate(CASES):
        _check_job(meshes[k], _alone(ctx, name, precision, its[k], 100 * k, 70), 70, precision)


def test_each_job_stops_at_its_own_step_count(ctx):
    its = _integrators()
    counts = [5, 37, 64, 0]
    batch = U.Batch(ctx, U.FP64)
    meshes = []
    for k, name in enumerate(CASES):
        m = _mesh(ctx, name, U.FP64)
        batch.add(m, its[k], 0, counts[k])
        meshes.append(m)
    batch.run(40)
    batch.run(40)
    done, _ = batch.poll()
    assert list(done) == counts
    for k, name in enumerate(CASES):
        if counts[k]:
            _check_job(meshes[k], _alone(ctx, name, U.FP64, its[k], 0, counts[k]), counts[k], U.FP64)


def test_tile_size_does_not_change_trajectories(ctx):
    it = _integrators()[0]
    finals = []
    for tf in (4, 6, 36, 512):  # 6: tiles that start off a 4-face boundary take the unstaged face loop
        batch = U.Batch(ctx, U.FP32_CENTRED, tile_faces=tf)
        m = _mesh(ctx, "ico3_deformed", U.FP32_CENTRED)
        batch.add(m, it, 0, 33)
        batch.run(33)
        assert batch.info().tile_faces == tf
        finals.append(m.state_get()[0])
    assert all(np.array_equal(finals[0], f) for f in finals[1:])


def test_jobs_join_and_leave_between_runs(ctx):
    its = _integrators()
    batch = U.Batch(ctx, U.FP64, tile_faces=32)
    a = _mesh(ctx, "ico2_plain", U.FP64)
    b = _mesh(ctx, "ico3_deformed", U.FP64)
    batch.add(a, its[0], 0, 60)
    batch.add(b, its[1], 0, 60)
    batch.run(20)
    c = _mesh(ctx, "planar12_deformed", U.FP64)
    batch.add(c, its[2], 5, 30)  # starts at the next run
    batch.remove(b)
    batch.run(40)
    assert batch.job(a) == (60, 0) and batch.job(c) == (30, 0)
    assert list(batch.poll()[0]) == [60, 30]
    _check_job(a, _alone(ctx, "ico2_plain", U.FP64, its[0], 0, 60), 60, U.FP64)
    _check_job(c, _alone(ctx, "planar12_deformed", U.FP64, its[2], 5, 30), 30, U.FP64)
    rb, _, _ = _alone(ctx, "ico3_deformed", U.FP64, its[1], 0, 20)
    assert np.array_equal(b.state_get()[0], rb)  # b kept the state of its 20 batched steps
    del c  # destroying a job's mesh removes the job
    batch.run(3)
    assert batch.info().n_jobs == 1


def test_a_diverging_job_stops_alone(ctx):
    its = _integrators()
    wild = U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=5.0, seed=2, divergence_threshold=10.0)
    batch = U.Batch(ctx, U.FP64)
    calm = _mesh(ctx, "ico3_deformed", U.FP64)
    bad = _mesh(ctx, "ico2_plain", U.FP64)
    batch.add(calm, its[0], 0, 40)
    batch.add(bad, wild, 0, 40)
    batch.run(40)
    done, st = batch.poll()
    assert done[0] == 40 and st[0] == 0
    assert st[1] == U.ERR_DIVERGED and 0 < done[1] < 40
    _check_job(calm, _alone(ctx, "ico3_deformed", U.FP64, its[0], 0, 40), 40, U.FP64)
    alone = _mesh(ctx, "ico2_plain", U.FP64)
    with pytest.raises(U.UmcpError, match="diverged"):
        alone.run(wild, 0, 40)
    # the flagged step records its energy and moves nothing, alone or batched
    assert np.array_equal(bad.state_get()[0], alone.state_get()[0])
    k = int(done[1])
    assert np.max(np.abs(bad.energies(k) - alone.energies(k)) / np.abs(alone.energies(k))) <= E_TOL[U.FP64]


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_host_driven_steps_follow_the_resident_run(ctx, precision):
    """umcp_batch_step_host: the jobs' states go in from one packed host
    array and come out after each call; the trajectory is the device-resident
    batch run's, bit for bit, and E holds each job's latest step energy. A
    state the caller changes between calls is the one the next step starts
    from. Page-locked and pageable host buffers give the same states."""
    torch = pytest.importorskip("torch")
    its = _integrators()[:2]
    names = ["ico2_plain", "ico3_deformed"]
    runs = []
    for host in (False, True, "pinned"):
        batch = U.Batch(ctx, precision)
        meshes = [_mesh(ctx, n, precision) for n in names]
        for k, m in enumerate(meshes):
            batch.add(m, its[k], 10 * k, 40)
        if host:
            pack = np.concatenate([m.state_get()[0] for m in meshes])
            E = np.zeros(len(meshes))
            if host == "pinned":
                pack_t = torch.from_numpy(pack).pin_memory()
                E_t = torch.zeros(len(meshes), dtype=torch.float64).pin_memory()
                pack, E = pack_t.numpy(), E_t.numpy()  # views of the page-locked memory
                for _ in range(20):
                    batch.step_host(pack_t.data_ptr(), pack_t.data_ptr(), E_t.data_ptr(), 2)
            else:
                for _ in range(20):
                    batch.step_host(pack, pack, E, 2)
            states = np.split(pack, np.cumsum([3 * m.nv + 3 for m in meshes])[:-1])
            assert all(np.array_equal(s, m.state_get()[0]) for s, m in zip(states, meshes))
            assert np.array_equal(E, [m.energies(40)[-1] for m in meshes])
        else:
            batch.run(40)
            states = [m.state_get()[0] for m in meshes]
        runs.append(states)
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            assert np.array_equal(a, b)
    # a changed state is picked up by the next call
    batch = U.Batch(ctx, precision)
    m = _mesh(ctx, "ico2_plain", precision)
    batch.add(m, its[0], 0, 5)
    r = m.state_get()[0]
    r[:-3] *= 1.001
    out = np.zeros_like(r)
    batch.step_host(r, out, None, 1)
    alone = _mesh(ctx, "ico2_plain", precision)
    alone.state_set(r)
    alone.run(its[0], 0, 1)
    assert np.array_equal(out, alone.state_get()[0])


def test_tuned_layout_is_cached_and_leaves_trajectories_unchanged(ctx, tmp_path):
    """The face launches' layout (regular and irregular tile sizes, blocks per
    SM) is timed at a batch's first run and written to the tune cache; a second
    batch of the same kind reads it instead of timing. A different layout
    groups the energy sums differently but the per-vertex gradient sums not at
    all, so positions are the same bit for bit."""
    import json

    cache = tmp_path / "tune.json"
    its = _integrators()
    runs = []
    for opts in ({"tune_cache": cache}, {"tune_cache": cache},
                 {"tile_faces": 128, "irr_tile_faces": 8, "blocks_per_sm": 2}):
        batch = U.Batch(ctx, U.FP32_CENTRED, **opts)
        meshes = [_mesh(ctx, n, U.FP32_CENTRED) for n in CASES]
        for k, m in enumerate(meshes):
            batch.add(m, its[k], 100 * k, 20)
        batch.run(20)
        runs.append((batch.info(), [m.state_get()[0] for m in meshes], [m.energies(20) for m in meshes]))
    (i1, r1, e1), (i2, r2, e2), (i3, r3, e3) = runs
    assert i1.tune_source == 1 and i2.tune_source == 2 and i3.tune_source == 0
    entries = json.loads(cache.read_text())
    assert len(entries) == 1
    (key, choice), = entries.items()
    assert "fp32" in key and choice["tile_faces"] == i1.tile_faces == i2.tile_faces
    assert choice["irr_tile_faces"] == i1.irr_tile_faces == i2.irr_tile_faces
    assert (i3.tile_faces, i3.irr_tile_faces, i3.face_grid[0]) == (128, 8, min(i1.face_grid[0], 2 * 152))
    for a, b, c in zip(r1, r2, r3):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    for a, c in zip(e1, e3):
        assert np.max(np.abs(a - c) / np.abs(a)) <= E_TOL[U.FP32_CENTRED]


def test_energy_call_between_runs_leaves_the_batch_trajectory(ctx):
    """An energy evaluation of a batch job's mesh at other positions (which
    takes the precision form's FP32 copies from those positions) between two
    runs does not change the batch's trajectory, whether the next step is a
    device-resident run or a host-driven step that passes the state back
    unchanged (whose unpacking keeps the copies of unchanged coordinates)."""
    it = _integrators()[0]
    runs = []
    for poke in (None, "run", "host"):
        batch = U.Batch(ctx, U.FP32_CENTRED)
        m = _mesh(ctx, "ico3_deformed", U.FP32_CENTRED)
        batch.add(m, it, 0, 10)
        batch.run(4)
        r = m.state_get()[0]
        if poke:
            r2 = r.copy()
            r2[:-3] += 0.3
            m.energy(r2)
        if poke == "host":
            batch.step_host(r, r, None, 1)
        else:
            batch.run(1)
        batch.run(5)
        runs.append(m.state_get()[0])
    assert np.array_equal(runs[0], runs[1]) and np.array_equal(runs[0], runs[2])
