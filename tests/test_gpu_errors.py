"""Argument errors of the newer entry points come back as statuses before any work is
queued (HmrError from the Python layer), and the context stays usable afterwards."""
import ctypes

import numpy as np
import pytest


@pytest.mark.gpu
def test_argument_errors_are_reported(cuda):
    import torch
    from hamers_gb300 import _lib as L
    from hamers_gb300 import flow
    fm = flow.FlowModel("SINGLE_SPECIES", 2, [1.4])
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision="exact")
    eu = flow.Euler(rec)
    n = [8, 8]
    Q = torch.ones((4, 1, 16, 16), dtype=torch.float64, device="cuda")
    Q[3] = 2.5
    pc = flow.Patch(n, [0.1, 0.1], Q)
    pf = flow.Patch([4, 4], [0.05, 0.05], torch.ones_like(Q[:, :, :12, :12]).contiguous())
    # a fine box that is not aligned with the ratio
    with pytest.raises(L.HmrError) as e:
        flow.coarsenPatch(rec, pc, (0, 0), pf, (3, 2), (2, 2))
    assert e.value.code == L.HMR_ERR_ARGUMENT
    with pytest.raises(L.HmrError) as e:
        flow.refineGhosts(rec, pf, (4, 4), pc, (0, 0), (0, 2), Q, Q, 0.5)
    assert e.value.code == L.HMR_ERR_ARGUMENT
    with pytest.raises(L.HmrError) as e:
        flow.refineGhosts(rec, pf, (4, 4), pc, (0, 0), (2, 2), Q, Q, 1.5)
    assert e.value.code == L.HMR_ERR_ARGUMENT
    # Navier-Stokes entry points on an Euler context
    F = rec.allocateFlux(pc)
    with pytest.raises(ValueError):
        flow.DiffusiveFluxReconstructor(rec)
    g = pc.geometry()
    q, _k1 = L.ptr_array([Q[e].data_ptr() for e in range(4)])
    f, _k2 = L.ptr_array([t[e].data_ptr() for t in F for e in range(4)])
    assert rec._lib.hmr_diff_flux_patch(rec.ctx, ctypes.byref(g), q, 1e-3, f, None) == L.HMR_ERR_UNSUPPORTED
    # the context still works
    S = rec.allocateSource(pc)
    eu.fillGhosts(pc, [1, 1])
    eu.computeFluxesAndSourcesOnPatch(pc, F, S, 1e-3)
    torch.cuda.synchronize()
    assert all(np.isfinite(t.cpu().numpy()).all() for t in F)
    rec.close()
