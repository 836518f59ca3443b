"""GPU parity: the CUDA path through the C ABI against the reference's own
outputs (golden fixtures) and against the oracle at larger sizes.

Tolerances (written here, used below):
  FP64 plain path: energy |dE|/|E| <= 1e-10; gradient max|dg|/max|g| <= 1e-10.
  FP32 face-centred form: energy |dE|/|E| <= 1e-6; gradient max|dg|/max|g| <= 1e-6
  and ||dg||/||g|| <= 1e-6.
  FP32 form on the tensor-core kernel (an option, not the default): the same
  bounds (energy 1e-6, gradient 1e-6 in both norms).
  Integrator steps (FP64, same Philox draws as the oracle): positions to 1e-12
  of the largest coordinate.
"""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import golden_cases, load_case, rel_inf, rel_l2
from oracle import bridge as B

pytestmark = pytest.mark.gpu

E64, G64 = 1e-10, 1e-10
E32, G32 = 1e-6, 1e-6
GTC = 1e-6


@pytest.fixture(scope="module")
def ctx():
    return U.Context(0)


@pytest.mark.parametrize("name", golden_cases())
def test_fp64_energy_and_gradient_match_reference(ctx, name):
    plan, prm, gold = load_case(name)
    mesh = U.Mesh(ctx, plan, prm)
    E, t = mesh.energy(gold["r"], terms=True)
    assert abs(E - gold["E"]) <= E64 * abs(gold["E"])
    assert np.allclose(t, [gold["VA"], gold["VC"], gold["VR"]], rtol=0, atol=E64 * abs(gold["E"]))
    g = np.zeros(3 * plan.nv + 3)
    mesh.grad(gold["r"], g)
    assert rel_inf(g[:-3], gold["grad"][:-3]) <= G64
    assert np.allclose(g[-3:], gold["grad"][-3:], rtol=G64, atol=G64 * np.abs(gold["grad"]).max())


def test_grad_accumulates_like_the_reference(ctx):
    plan, prm, gold = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    g = np.ones(3 * plan.nv + 3)
    mesh.grad(gold["r"], g)
    assert rel_inf(g - 1.0, gold["grad"]) <= G64


@pytest.mark.parametrize("kind,size", [("ico", 5), ("planar", 48)])
def test_fp64_matches_oracle_at_larger_sizes(ctx, tmp_path, kind, size):
    path = tmp_path / "m.mesh"
    if kind == "ico":
        U.generate_icosphere(path, size, 300.0, 3.0, 77)
    else:
        U.generate_planar(path, size, size, 10.0, 20.0, 78)
    prm = U.params(kc=U.kc_from_kT(20.0), KA=0.215, kg=-1.0, k_reg=0.1)
    plan = U.Plan(path, prm)
    r = plan.positions()
    rng = np.random.default_rng(9)
    r[:-3] += rng.normal(0, 0.2, 3 * plan.nv)
    r[-3:] = (1.002, 0.999, 1.001)
    O = B.Oracle(plan, prm)
    mesh = U.Mesh(ctx, plan, prm)
    E, g = mesh.energy_grad(r)
    assert abs(E - O.energy(r)) <= E64 * abs(E)
    assert rel_inf(g, O.grad(r)) <= G64


def test_energy_grad_is_deterministic(ctx):
    plan, prm, gold = load_case("ico4_plain")
    mesh = U.Mesh(ctx, plan, prm)
    E1, g1 = mesh.energy_grad(gold["r"])
    E2, g2 = mesh.energy_grad(gold["r"])
    assert E1 == E2 and np.array_equal(g1, g2)


@pytest.mark.parametrize("name", golden_cases())
def test_fp32_centred_form_error_bound(ctx, name):
    plan, prm, gold = load_case(name, precision=U.FP32_CENTRED)
    mesh = U.Mesh(ctx, plan, prm)
    E, g = mesh.energy_grad(gold["r"])
    assert abs(E - gold["E"]) <= E32 * abs(gold["E"])
    assert rel_inf(g[:-3], gold["grad"][:-3]) <= G32
    assert rel_l2(g[:-3], gold["grad"][:-3]) <= G32


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_fp32_centred_form_on_benchmark_vesicles(ctx, tmp_path, level):
    """Vesicles of the batched benchmark (seed 1003; the first three of each
    subdivision level), at the reference state, where every area force is
    zero and any rounding of the strain is all that is left of it, and at a
    state displaced by N(0, 0.05 A): FP32 against the FP64 path."""
    from umcp_gb300 import workloads as W

    specs = [s for s in W.vesicle_specs(256, 1003) if s.level == level][:3]
    for s in specs:
        plan64, prm64 = W._build_vesicle(s, tmp_path, U.FP64, 298.0)
        plan32, prm32 = W._build_vesicle(s, tmp_path, U.FP32_CENTRED, 298.0)
        m64, m32 = U.Mesh(ctx, plan64, prm64), U.Mesh(ctx, plan32, prm32)
        r0 = plan64.positions()
        for sigma in (0.0, 0.05):
            r = r0.copy()
            r[:-3] += np.random.default_rng(s.seed).normal(0.0, sigma, 3 * plan64.nv)
            E64_, g64 = m64.energy_grad(r)
            E32_, g32 = m32.energy_grad(r)
            assert abs(E32_ - E64_) <= E32 * abs(E64_), (s, sigma)
            assert rel_inf(g32[:-3], g64[:-3]) <= G32, (s, sigma)
            assert rel_l2(g32[:-3], g64[:-3]) <= G32, (s, sigma)


def test_fp32_centred_form_on_the_planar_benchmark_membrane(ctx, tmp_path):
    path = tmp_path / "p128.mesh"
    U.generate_planar(path, 128, 128, 10.0, 20.0, 1002)
    prm64 = U.params(kc=U.kc_from_kT(20.0), KA=0.215)
    prm32 = U.params(kc=U.kc_from_kT(20.0), KA=0.215, precision=U.FP32_CENTRED)
    plan = U.Plan(path, prm64)
    r = plan.positions()
    r[:-3] += np.random.default_rng(4).normal(0, 0.05, 3 * plan.nv)
    E64_, g64 = U.Mesh(ctx, plan, prm64).energy_grad(r)
    E32_, g32 = U.Mesh(ctx, plan, prm32).energy_grad(r)
    assert abs(E32_ - E64_) <= E32 * abs(E64_)
    assert rel_inf(g32, g64) <= G32
    assert rel_l2(g32, g64) <= G32


def _oracle_run(plan, prm, r, mode, dt, gamma, D, seed, stream, nsteps, mass=None):
    O = B.Oracle(plan, prm)
    kT = 0.592186663194 / 298.0 * prm.temperature
    p = np.zeros(3 * plan.nv)
    r = r.copy()
    for s in range(nsteps):
        g = O.grad(r)
        xi = B.noise(seed, stream, s, plan.nv)
        rv = r[:-3].copy()
        B.step(mode, dt, gamma, kT, D, rv, p, g[:-3], xi, mass=mass)
        r[:-3] = rv
    return r, p


@pytest.mark.parametrize("kind", [U.OVERDAMPED_BD, U.BD_MEMBRANE, U.LANGEVIN])
def test_integrator_steps_match_oracle(ctx, kind):
    plan, prm, gold = load_case("ico3_plain")
    mesh = U.Mesh(ctx, plan, prm)
    r0 = plan.positions()
    if kind == U.OVERDAMPED_BD:
        it = U.integrator(kind, time_step=1.0, D=0.00125, seed=11, stream=3)
    else:
        it = U.integrator(kind, time_step=1e-15, gamma=10.0, seed=11, stream=3)
    mesh.state_set(r0)
    energies = mesh.run(it, 0, 5)
    r_gpu, p_gpu = mesh.state_get()
    r_ref, p_ref = _oracle_run(plan, prm, r0, kind, it.time_step, it.gamma, it.D, 11, 3, 5)
    assert np.max(np.abs(r_gpu - r_ref)) <= 1e-12 * np.abs(r_ref).max()
    assert np.max(np.abs(p_gpu - p_ref)) <= 1e-12 * max(np.abs(p_ref).max(), 1e-300)
    assert abs(energies[0] - B.Oracle(plan, prm).energy(r0)) <= E64 * energies[0]


def test_run_graph_chunks_equal_eager_steps(ctx):
    plan, prm, _ = load_case("ico2_plain")
    it = U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.00125, seed=5)
    a = U.Mesh(ctx, plan, prm)
    e_a = a.run(it, 0, 70)  # two captured chunks of 32 and 6 eager steps
    b = U.Mesh(ctx, plan, prm)
    e_b = np.array([b.run(it, s, 1)[0] for s in range(70)])
    assert np.array_equal(e_a, e_b)
    assert np.array_equal(a.state_get()[0], b.state_get()[0])


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_step_host_is_one_run_step(ctx, precision):
    plan, prm, _ = load_case("ico2_plain", precision)
    it = U.integrator(U.LANGEVIN, time_step=1e-15, gamma=0.001, seed=8)
    a = U.Mesh(ctx, plan, prm)
    a.run(it, 7, 2)  # the resident state (and its FP32 pairs) moves away from r
    r = plan.positions()
    p = np.zeros(3 * plan.nv)
    for s in range(3):
        a.step_host(it, s, r, p)
    b = U.Mesh(ctx, plan, prm)
    b.run(it, 0, 3)
    rb, pb = b.state_get()
    assert np.array_equal(r, rb) and np.array_equal(p, pb)


def _random_mass(nv, seed, fill=0.05):
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for i in range(nv):
        js = np.unique(np.concatenate([[i], rng.choice(nv, max(1, int(fill * nv)), replace=False)]))
        rows.append(len(js))
        cols.extend(js)
        vals.extend(rng.normal(0, 1, len(js)) + (js == i) * 5.0)
    row_ptr = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    return row_ptr, np.array(cols, dtype=np.int32), np.array(vals)


def test_mass_apply_matches_oracle(ctx):
    plan, prm, _ = load_case("ico3_plain")
    mesh = U.Mesh(ctx, plan, prm)
    rp, cl, vl = _random_mass(plan.nv, 2)
    mesh.mass_set(rp, cl, vl)
    rng = np.random.default_rng(1)
    vin = rng.normal(0, 1, 3 * plan.nv)
    base = rng.normal(0, 1, 3 * plan.nv)
    scalev = rng.uniform(0.5, 2.0, 3 * plan.nv)
    for sv, scale, al in [(None, 1.0, (1, 1, 1)), (scalev, -0.7, (1.01, 0.98, 1.2))]:
        got = mesh.mass_apply(vin, base.copy(), sv, scale, al)
        want = B.sparse_apply(rp, cl, vl, vin, base.copy(), sv, scale, al)
        assert np.max(np.abs(got - want)) <= 1e-13 * np.abs(want).max()


def test_leapfrog_with_mass_matches_oracle(ctx):
    plan, prm, _ = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    rp, cl, vl = _random_mass(plan.nv, 5, fill=0.2)
    vl = np.abs(vl) * 0.01
    mesh.mass_set(rp, cl, vl)
    r0 = plan.positions()
    for kind in (U.BD_MEMBRANE, U.LANGEVIN):
        it = U.integrator(kind, time_step=1e-15, gamma=10.0, seed=21, stream=1, use_mass=1)
        mesh.state_set(r0)
        mesh.run(it, 0, 3)
        r_gpu, p_gpu = mesh.state_get()
        r_ref, p_ref = _oracle_run(plan, prm, r0, kind, it.time_step, it.gamma, 0.0, 21, 1, 3, mass=(rp, cl, vl))
        assert np.max(np.abs(r_gpu - r_ref)) <= 1e-12 * np.abs(r_ref).max()


def test_nonfinite_energy_is_reported_and_context_survives(ctx):
    plan, prm, gold = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    r = gold["r"].copy()
    r[5] = np.nan
    with pytest.raises(U.UmcpError, match="non-finite"):
        mesh.energy(r)
    assert abs(mesh.energy(gold["r"]) - gold["E"]) <= E64 * abs(gold["E"])


def test_divergence_stops_the_run(ctx):
    plan, prm, _ = load_case("ico2_plain")
    mesh = U.Mesh(ctx, plan, prm)
    it = U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=5.0, seed=2, divergence_threshold=10.0)
    with pytest.raises(U.UmcpError, match="diverged"):
        mesh.run(it, 0, 40)


@pytest.mark.parametrize("name", ["ico3_deformed", "planar12_deformed", "ico4_plain", "ico2_lipids"])
def test_tensor_core_face_kernel_matches_reference(ctx, name):
    """The tcgen05 form of the regular-face pass (kind::f16 contractions on
    affine-centred control points) meets its bounds against the reference
    (energy as the precision form, gradient GTC) and is deterministic; its
    meshes run the same integrators."""
    plan, prm, gold = load_case(name, U.FP32_CENTRED)
    prm.face_kernel = U.TENSOR_CORES
    mesh = U.Mesh(ctx, plan, prm)
    r = gold["r"]
    E, g = mesh.energy_grad(r)
    assert abs(E - gold["E"]) <= E32 * abs(gold["E"])
    assert rel_inf(g[:-3], gold["grad"][:-3]) <= GTC and rel_l2(g[:-3], gold["grad"][:-3]) <= GTC
    E2, g2 = mesh.energy_grad(r)
    assert E2 == E and np.array_equal(g2, g)
    it = U.integrator(U.OVERDAMPED_BD, time_step=1.0, D=0.00125, seed=3)
    e = mesh.run(it, 0, 40)
    prm.face_kernel = U.SIMT
    e_simt = U.Mesh(ctx, plan, prm).run(it, 0, 40)
    assert np.all(np.isfinite(e)) and np.max(np.abs(e - e_simt)) <= 1e-5 * np.max(np.abs(e_simt))


def test_precision_form_mass_set_applies_in_fp32(ctx):
    """A CSR installed on a mesh of the FP32 form (FP32 values, 16-bit columns)
    applies within 1e-6 of sum_j |M_ij| |x_j| of the FP64 mesh's apply of the
    same CSR, on rows of every length mod 4, and reads back as installed."""
    plan, prm, _ = load_case("ico3_plain")
    _, prm32, _ = load_case("ico3_plain", U.FP32_CENTRED)
    m64, m32 = U.Mesh(ctx, plan, prm), U.Mesh(ctx, plan, prm32)
    rng = np.random.default_rng(5)
    rows, cols, vals = [], [], []
    for i in range(plan.nv):  # row lengths 1 .. 9, every residue mod 4
        js = np.unique(np.concatenate([[i], rng.choice(plan.nv, i % 9, replace=False)]))
        rows.append(len(js))
        cols.extend(js)
        vals.extend(rng.normal(0, 1, len(js)) + (js == i) * 5.0)
    rp = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    cl, vl = np.array(cols, dtype=np.int32), np.array(vals)
    assert len({int(n) % 4 for n in np.diff(rp)}) == 4
    m64.mass_set(rp, cl, vl)
    m32.mass_set(rp, cl, vl)
    vin = rng.normal(0, 1, 3 * plan.nv)
    base = rng.normal(0, 1, 3 * plan.nv)
    dense = np.zeros((plan.nv, plan.nv))
    for i in range(plan.nv):
        for k in range(rp[i], rp[i + 1]):
            dense[i, cl[k]] += vl[k]
    bound = (np.abs(dense) @ np.abs(vin.reshape(-1, 3))).reshape(-1)
    want = m64.mass_apply(vin, base.copy(), None, 1.0, (1, 1, 1))
    got = m32.mass_apply(vin, base.copy(), None, 1.0, (1, 1, 1))
    assert np.all(np.abs(got - want) <= 1e-6 * bound + 1e-12 * np.abs(base))
    assert np.array_equal(m32.mass_get(), dense.astype(np.float32).astype(np.float64))


def _run_rows(nv: int, rng) -> tuple:
    """CSR rows made of runs of consecutive columns, as a truncated inverse's
    rows are: a single run of up to 2,400 nonzeros, 40 one-column runs ahead
    of a long run, runs of random lengths in random order with a repeated
    column, and empty rows."""
    rows, cols = [], []
    for i in range(nv):
        kind = i % 4
        if i % 16 == 3:
            js = np.zeros(0, dtype=np.int64)
        elif kind == 0:
            n = 1 + (37 * i) % min(2400, nv - 1)
            a = int(rng.integers(0, nv - n))
            js = np.arange(a, a + n)
        elif kind == 1:
            a = int(rng.integers(0, nv - 400))
            js = np.concatenate([a + 2 * np.arange(40), a + 81 + np.arange(300)])
        else:
            parts = []
            for _ in range(int(rng.integers(2, 9))):
                n = int(rng.integers(1, 71))
                a = int(rng.integers(0, nv - n))
                parts.append(np.arange(a, a + n))
            parts.append(parts[0][:1])  # a repeated column
            js = np.concatenate([parts[k] for k in rng.permutation(len(parts))])
        rows.append(len(js))
        cols.extend(js)
    rp = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    return rp, np.array(cols, dtype=np.int32)


def test_precision_form_mass_apply_on_long_and_ragged_rows(ctx):
    """A CSR of rows of 0 to 2,400 nonzeros in runs of consecutive columns,
    installed on meshes of both forms: the FP32 apply (which asks L2 for the
    lines of long rows ahead of its loads) stays within 1e-6 of
    sum_j |M_ij| |x_j| of the FP64 apply, with and without the per-row scaling
    and alphas, and the CSR reads back as installed."""
    plan, prm, _ = load_case("ico4_plain")
    _, prm32, _ = load_case("ico4_plain", U.FP32_CENTRED)
    m64, m32 = U.Mesh(ctx, plan, prm), U.Mesh(ctx, plan, prm32)
    rng = np.random.default_rng(11)
    rp, cl = _run_rows(plan.nv, rng)
    assert np.diff(rp).max() > 32 * 40 and np.diff(rp).min() == 0
    vl = rng.normal(0, 1, len(cl))
    m64.mass_set(rp, cl, vl)
    m32.mass_set(rp, cl, vl)
    assert m32.info().mass_form == 2 and m64.info().mass_form == 2
    dense = np.zeros((plan.nv, plan.nv))
    np.add.at(dense, (np.repeat(np.arange(plan.nv), np.diff(rp)), cl), vl.astype(np.float32).astype(np.float64))
    vin = rng.normal(0, 1, 3 * plan.nv)
    base = rng.normal(0, 1, 3 * plan.nv)
    scalev = rng.uniform(0.5, 2.0, 3 * plan.nv)
    bound = (np.abs(dense) @ np.abs(vin.reshape(-1, 3))).reshape(-1)
    for sv, alphas in ((None, (1, 1, 1)), (scalev, (1.1, 0.9, 1.05))):
        want = m64.mass_apply(vin, base.copy(), sv, 0.7, alphas)
        got = m32.mass_apply(vin, base.copy(), sv, 0.7, alphas)
        scale_bound = 0.7 * 2.0 / 0.81 * bound  # scale x max scalev / min alpha^2
        assert np.all(np.abs(got - want) <= 1e-6 * scale_bound + 1e-12 * np.abs(base))
    assert np.array_equal(m32.mass_get(), dense)
