"""The allocation-free energy+gradient entry point (umcp_energy_grad_static),
for callers that cannot call cudaMalloc at the time they need the energy,
e.g. code running inside another framework's CUDA-graph capture. Its scratch
is the library's static device array; its results must equal those of the
allocating entry point (umcp_energy_grad_device) on the same inputs, call
after call. Collected last so a failure here stops a -x run only after all
other tests have run."""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import load_case, rel_inf

pytestmark = pytest.mark.gpu

TOL = {U.FP64: (1e-10, 1e-10), U.FP32_CENTRED: (1e-6, 2e-5)}  # (energy, gradient), as in test_gpu_parity


@pytest.mark.parametrize("precision", [U.FP64, U.FP32_CENTRED])
def test_static_scratch_entry_matches_allocating_entry(precision):
    torch = pytest.importorskip("torch")
    plan, prm, gold = load_case("ico3_deformed", precision)
    ctx = U.Context(0)
    mesh = U.Mesh(ctx, plan, prm)
    n = 3 * plan.nv + 3
    d_r = torch.tensor(gold["r"], dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    e_tol, g_tol = TOL[precision]
    for call in range(2):
        d_E0 = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        d_g0 = torch.zeros(n, dtype=torch.float64, device="cuda:0")
        d_E1 = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        d_g1 = torch.zeros(n, dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        mesh.energy_grad_device(d_r.data_ptr(), d_E0.data_ptr(), d_g0.data_ptr())
        ctx.synchronize()
        mesh.energy_grad_static(d_r.data_ptr(), d_E1.data_ptr(), d_g1.data_ptr())
        ctx.synchronize()
        E0, E1 = float(d_E0.item()), float(d_E1.item())
        g0, g1 = d_g0.cpu().numpy(), d_g1.cpu().numpy()
        assert np.isfinite(E1) and abs(E1 - E0) <= e_tol * abs(E0), (call, E0, E1)
        assert rel_inf(g1, g0) <= g_tol, call
        # and both against the reference's own values
        assert abs(E1 - gold["E"]) <= e_tol * abs(gold["E"])
        assert rel_inf(g1[:-3], gold["grad"][:-3]) <= g_tol
