"""Refluxing on the device against the oracle: the two-level step of test_oracle_reflux
(coarse step, two fine steps, flux-sum coarsening, synchronizeFluxes, coarsening of the
fine interior) through the C ABI, bitwise equal to the oracle (exact form) and
conserving the composite totals to rounding.  Also the three operators alone on random
data in 3D with an anisotropic ratio."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import reflux_case as R
from tests.test_oracle_reflux import A3, B3, G3, two_level_step


def _gpu_two_level():
    import torch
    from hamers_gb300 import flow
    fm = flow.FlowModel("SINGLE_SPECIES", 2, R.GAMMA)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision="exact")
    eu = flow.Euler(rec)
    nc, nf = [R.N, R.N], list(R.FN)
    dxc, dxf = 1.0 / R.N, 0.5 / R.N
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Qc = t(R.analytic_state(nc, [dxc, dxc], (0, 0)))
    Qf = t(R.analytic_state(nf, [dxf, dxf], R.FLO))
    pc, pf = flow.Patch(nc, [dxc, dxc], Qc), flow.Patch(nf, [dxf, dxf], Qf)
    flow.coarsenPatch(rec, pc, (0, 0), pf, R.FLO, R.RATIO)
    torch.cuda.synchronize()
    before = R.composite_totals(Qc.cpu().numpy(), Qf.cpu().numpy(), dxc, dxf)
    dt = 0.2 * dxc
    Qc_old = Qc.clone()
    Qc_old_np = Qc.cpu().numpy()

    def step(patch, dt, fill, Facc, Sacc):
        X = patch.data
        Qs, Fs, Ss = [], [], []
        for s in range(3):
            fill(X)
            Qs.append(X.clone())
            F = rec.allocateFlux(patch)
            S = rec.allocateSource(patch)
            eu.computeFluxesAndSourcesOnPatch(flow.Patch(patch.n, patch.dx, Qs[-1]), F, S, dt)
            Fs.append(F)
            Ss.append(S)
            eu.advanceSingleStepOnPatch(flow.Patch(patch.n, patch.dx, X), A3[s], B3[s], G3[s], Qs, Fs, Ss, Facc, Sacc)

    Fc = rec.allocateFlux(pc)
    Sc = rec.allocateSource(pc)
    step(pc, dt, lambda X: eu.fillGhosts(flow.Patch(nc, [dxc, dxc], X), [1, 1]), Fc, Sc)
    Ff = rec.allocateFlux(pf)
    Sf = rec.allocateSource(pf)

    def fill_fine(X):
        h = X.cpu().numpy()
        R.inject_ghosts(h, Qc_old_np)
        X.copy_(torch.from_numpy(h))

    for _ in range(2):
        step(pf, 0.5 * dt, fill_fine, Ff, Sf)
    flow.coarsenFluxSum(rec, pc, (0, 0), pf, R.FLO, R.RATIO, Ff, Fc)
    Qc.copy_(Qc_old)
    eu.synchronizeFluxes(pc, Fc, Sc)
    flow.coarsenPatch(rec, pc, (0, 0), pf, R.FLO, R.RATIO)
    torch.cuda.synchronize()
    after = R.composite_totals(Qc.cpu().numpy(), Qf.cpu().numpy(), dxc, dxf, covered=False)
    out = Qc.cpu().numpy()
    rec.close()
    return before, after, out


@pytest.mark.gpu
def test_two_level_reflux_matches_oracle_and_conserves(cuda):
    before, after, Qc = _gpu_two_level()
    assert np.all(np.abs(after - before) <= 1e-14 * np.abs(before)), (before, after)
    _, _, _, Qc_o = two_level_step(True)
    sl = (slice(None), 0, slice(4, -4), slice(4, -4))
    assert np.array_equal(Qc[sl], Qc_o[sl]), np.abs(Qc[sl] - Qc_o[sl]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("model", [O.MODEL_SINGLE_SPECIES, O.MODEL_FIVE_EQN_ALLAIRE], ids=["single", "five"])
def test_operators_alone_3d(cuda, model):
    import torch
    from hamers_gb300 import flow
    gam = [1.4] if model == O.MODEL_SINGLE_SPECIES else [1.4, 1.09]
    name = "SINGLE_SPECIES" if model == O.MODEL_SINGLE_SPECIES else "FIVE_EQN_ALLAIRE"
    cfg = O.Config(model, 3, gam)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", flow.FlowModel(name, 3, gam), precision="exact")
    eu = flow.Euler(rec)
    rng = np.random.default_rng(9)
    nc, clo = [10, 9, 8], [2, 3, 1]
    ratio = [2, 4, 2]
    flo, nf = [8, 20, 4], [8, 12, 10]       # coarse cells [4, 8) x [5, 8) x [2, 7): inside the coarse patch
    dx = [0.1, 0.12, 0.09]
    Qc = rng.standard_normal(O.ghost_shape(cfg, nc)) + 2.0
    Qf = rng.standard_normal(O.ghost_shape(cfg, nf)) + 2.0
    Fc = [rng.standard_normal(s) for s in O.flux_shapes(cfg, nc)]
    Ff = [rng.standard_normal(s) for s in O.flux_shapes(cfg, nf)]
    S = rng.standard_normal((cfg.neq, nc[2], nc[1], nc[0]))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    # flux sums
    Fc_o = [f.copy() for f in Fc]
    O.coarsen_fluxsum(cfg, ratio, nc, clo, nf, flo, Ff, Fc_o)
    tFc = [t(f) for f in Fc]
    pc, pf = flow.Patch(nc, dx, t(Qc)), flow.Patch(nf, [d / r for d, r in zip(dx, ratio)], t(Qf))
    flow.coarsenFluxSum(rec, pc, clo, pf, flo, ratio, [t(f) for f in Ff], tFc)
    torch.cuda.synchronize()
    for a in range(3):
        assert np.array_equal(tFc[a].cpu().numpy(), Fc_o[a])
    assert any(not np.array_equal(Fc_o[a], Fc[a]) for a in range(3))
    # synchronizeFluxes
    Qs = Qc.copy()
    O.sync_fluxes(cfg, nc, dx, Fc_o, S, Qs)
    tQ = t(Qc)
    eu.synchronizeFluxes(flow.Patch(nc, dx, tQ), tFc, t(S))
    torch.cuda.synchronize()
    sl = (slice(0, cfg.ncomp),) + (slice(4, -4),) * 3
    assert np.array_equal(tQ.cpu().numpy()[sl], Qs[sl])
    # coarsening of the fine interior
    Qo = Qc.copy()
    O.coarsen_cells(cfg, ratio, nc, clo, nf, flo, Qf, Qo)
    flow.coarsenPatch(rec, pc, clo, pf, flo, ratio)
    torch.cuda.synchronize()
    assert np.array_equal(pc.data.cpu().numpy(), Qo)
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_refine_ghosts_matches_oracle(cuda, dim):
    """Coarse-fine ghost cells (time interpolation + conservative linear refinement), bitwise."""
    import torch
    from hamers_gb300 import flow
    gam = [1.4, 1.67]
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, dim, gam)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", flow.FlowModel("FIVE_EQN_ALLAIRE", dim, gam),
                                           precision="exact")
    rng = np.random.default_rng(5 + dim)
    if dim == 2:
        cn, clo, ratio, flo, fn = [12, 10], [3, 2], [2, 4], [10, 12], [8, 12]
    else:
        cn, clo, ratio, flo, fn = [9, 8, 7], [1, 2, 0], [2, 4, 2], [6, 12, 2], [6, 8, 8]
    Qo = rng.standard_normal(O.ghost_shape(cfg, cn)) + 2.0
    Qn = rng.standard_normal(Qo.shape) + 2.0
    Qf = rng.standard_normal(O.ghost_shape(cfg, fn))
    theta = 0.37
    Qf_o = Qf.copy()
    O.refine_ghosts(cfg, ratio, fn, flo, cn, clo, Qo, Qn, theta, Qf_o)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pf = flow.Patch(fn, [0.1] * dim, t(Qf))
    pc = flow.Patch(cn, [0.1] * dim, t(Qo))
    flow.refineGhosts(rec, pf, flo, pc, clo, ratio, t(Qo), t(Qn), theta)
    torch.cuda.synchronize()
    got = pf.data.cpu().numpy()
    assert np.array_equal(got, Qf_o), np.abs(got - Qf_o).max()
    assert not np.array_equal(Qf_o, Qf)                     # some ghosts were covered and written
    rec.close()
