"""Regular-patch Loop subdivision (the reference's fast_sub6_0..3,
src/fast_mm.C): the stencils the engine derives from box-spline refinement
are the reference's exactly (tests/golden/sub6.npz, dumped by the
reference-built oracle); the batched device kernel applies them."""
from __future__ import annotations

import numpy as np
import pytest

import umcp_gb300 as U
from conftest import GOLDEN


def test_stencils_equal_the_reference():
    ref = np.load(GOLDEN / "sub6.npz")["stencils"]
    S = U.subdivision_stencils()
    assert np.array_equal(S, ref)
    assert np.allclose(S.sum(axis=2), 1.0)  # affine invariance


@pytest.mark.gpu
def test_device_subdivision_matches_stencils():
    import torch

    ctx = U.Context(0)
    rng = np.random.default_rng(1)
    n = 20000
    P = rng.normal(0, 10, (n, 12, 3))
    d_in = torch.tensor(P.reshape(n, 36), device="cuda", dtype=torch.float64)
    d_out = torch.zeros((n, 4, 36), device="cuda", dtype=torch.float64)
    torch.cuda.synchronize()
    U.subdivide_patches(ctx, d_in.data_ptr(), d_out.data_ptr(), n)
    ctx.synchronize()
    got = d_out.cpu().numpy().reshape(n, 4, 12, 3)
    want = np.einsum("kij,njc->nkic", U.subdivision_stencils(), P)
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
    # a patch subdivided twice through the device equals the stencil product
    d2 = torch.zeros((n * 4, 4, 36), device="cuda", dtype=torch.float64)
    U.subdivide_patches(ctx, d_out.data_ptr(), d2.data_ptr(), n * 4)
    ctx.synchronize()
    S = U.subdivision_stencils()
    two = d2.cpu().numpy().reshape(n, 4, 4, 12, 3)
    assert np.max(np.abs(two[:, 3, 0] - np.einsum("ij,jk,nkc->nic", S[0], S[3], P))) <= 1e-12 * np.max(np.abs(P))
