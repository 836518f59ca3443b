"""The allocation-free energy+gradient entry point (umcp_energy_grad_static),
for callers that cannot call cudaMalloc at the time they need the energy,
e.g. code running inside another framework's CUDA-graph capture. Its scratch
is the library's static device array; its results must equal those of the
allocating entry point (umcp_energy_grad_device) on the same inputs, call
after call, in both arithmetic forms and on the tensor-core face kernel. A
non-finite energy it meets is recorded in the mesh's status word
(umcp_mesh_check_status), as the allocating entry point's is. Collected last
so a failure here stops a -x run only after all other tests have run."""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import load_case, rel_inf

pytestmark = pytest.mark.gpu

# (energy, gradient) bounds, as in test_gpu_parity: FP64, the FP32 form, and
# the FP32 form on the tensor-core kernel
TOL = {(U.FP64, U.SIMT): (1e-10, 1e-10), (U.FP32_CENTRED, U.SIMT): (1e-6, 1e-6),
       (U.FP32_CENTRED, U.TENSOR_CORES): (1e-6, 1e-6)}


def _mesh(precision, face_kernel):
    plan, prm, gold = load_case("ico3_deformed", precision)
    prm.face_kernel = face_kernel
    ctx = U.Context(0)
    return ctx, plan, U.Mesh(ctx, plan, prm), gold


@pytest.mark.parametrize("precision,face_kernel", sorted(TOL))
def test_static_scratch_entry_matches_allocating_entry(precision, face_kernel):
    torch = pytest.importorskip("torch")
    ctx, plan, mesh, gold = _mesh(precision, face_kernel)
    n = 3 * plan.nv + 3
    d_r = torch.tensor(gold["r"], dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    e_tol, g_tol = TOL[(precision, face_kernel)]
    for call in range(2):
        d_E0 = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        d_g0 = torch.zeros(n, dtype=torch.float64, device="cuda:0")
        d_E1 = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        d_g1 = torch.zeros(n, dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        mesh.energy_grad_device(d_r.data_ptr(), d_E0.data_ptr(), d_g0.data_ptr())
        ctx.synchronize()
        mesh.energy_grad_static(d_r.data_ptr(), d_E1.data_ptr(), d_g1.data_ptr())
        mesh.check_status()
        E0, E1 = float(d_E0.item()), float(d_E1.item())
        g0, g1 = d_g0.cpu().numpy(), d_g1.cpu().numpy()
        assert np.isfinite(E1) and abs(E1 - E0) <= e_tol * abs(E0), (call, E0, E1)
        assert rel_inf(g1, g0) <= g_tol, call
        # and both against the reference's own values
        assert abs(E1 - gold["E"]) <= e_tol * abs(gold["E"])
        assert rel_inf(g1[:-3], gold["grad"][:-3]) <= g_tol


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_static_scratch_entry_reports_a_nonfinite_energy(precision):
    """A NaN coordinate gives a NaN energy; the next status check reports it,
    and a clean call afterwards (energy to the mesh's own slot) is clean."""
    torch = pytest.importorskip("torch")
    ctx, plan, mesh, gold = _mesh(precision, U.SIMT)
    r = gold["r"].copy()
    r[7] = np.nan
    d_bad = torch.tensor(r, dtype=torch.float64, device="cuda:0")
    d_good = torch.tensor(gold["r"], dtype=torch.float64, device="cuda:0")
    d_E = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    mesh.energy_grad_static(d_bad.data_ptr(), d_E.data_ptr(), 0)
    with pytest.raises(U.UmcpError, match="non-finite"):
        mesh.check_status()
    mesh.energy_grad_static(d_good.data_ptr(), 0, 0)
    mesh.check_status()
