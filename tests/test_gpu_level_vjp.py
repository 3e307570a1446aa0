"""Batched adjoint: the VJP of a level substep over all patches at once (hmr_level_substep_vjp).

Every patch's result must be bitwise that of the per-patch VJP (hmr_rk_substep_vjp_patch) at the
same stage states, for all three SSPRK3 stages, uneven patch sizes, 2D and 3D, the three flow
models, and in groups of patches (a reverse-buffer budget that fits only a few patches at a
time).  The per-patch VJP itself is checked against the oracle's tangent in test_gpu_adjoint.py.
"""
import numpy as np
import pytest

from tests.helpers import noisy_shock_state, smooth_state
from tests.test_gpu_level import _patches
from tests.test_gpu_parity import IDS, VARIANTS, make

CASES = [VARIANTS[i] for i in (1, 2, 5, 7, 9)]
CASE_IDS = [IDS[i] for i in (1, 2, 5, 7, 9)]
NS_TRANSPORT = dict(species_mu=0.02, species_mu_v=0.005, species_c_p=3.5, species_Pr=0.72)


def _run(variant, budget=None, diffusive=None):
    """Batched and per-patch VJPs of the three substeps; diffusive: None (Euler) or the
    NavierStokes midpoint order (single species)."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = variant
    if diffusive is None:
        rec = make(model, dim, scheme, gam, "fast")
        eu = flow.Euler(rec)
    else:
        fm = flow.FlowModel("SINGLE_SPECIES", dim, gam, transport=NS_TRANSPORT)
        rec = flow.ConvectiveFluxReconstructor(
            "WCNS5_JS_HLLC_HLL", fm, precision="fast",
            diffusive_flux_reconstructor={2: "MIDPOINT_SECOND_ORDER", 4: "MIDPOINT_FOURTH_ORDER",
                                          6: "MIDPOINT_SIXTH_ORDER"}[diffusive])
        eu = flow.NavierStokes(rec)
    grow = rec.getPatchNumberOfGhostCells() - 4
    sizes, periodic = _patches(dim, 11)
    dt = 1.0e-3
    geoms, states = [], []
    for p, n in enumerate(sizes):
        gen = noisy_shock_state if p % 2 else smooth_state
        Q = gen(model, dim, [v + 2 * grow for v in n], seed=60 + p, species_gamma=gam)
        states.append(torch.from_numpy(Q).cuda())
        geoms.append((list(n), [1.0 / v for v in n]))
    lv = flow.BatchedLevel(rec, geoms)
    if budget is not None:
        lv._lib.hmr_level_set_vjp_budget(lv.level, int(budget))
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, periodic[p])
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    out = []
    for stage in range(3):
        lv.substep(stage, dt)   # forward: fills the ghosts of slot `stage`, writes the next slot
        torch.cuda.synchronize()
        lv.check()
        Qbo = [torch.randn(Q.shape, dtype=torch.float64, device="cuda", generator=gen) for Q in states]
        batched = [[torch.zeros_like(Q) for _ in range(stage + 1)] for Q in states]
        lv.substepVJP(stage, dt, Qbo, batched)
        per_patch = [[torch.zeros_like(Q) for _ in range(stage + 1)] for Q in states]
        for p, (n, dx) in enumerate(geoms):
            Qint = [lv.state(p, s).contiguous() for s in range(stage + 1)]
            rec.reserve(flow.Patch(n, dx, Qint[-1]))
            eu.substepVJP(flow.Patch(n, dx, Qint[-1]), stage, Qint, dt, Qbo[p], per_patch[p])
        torch.cuda.synchronize()
        out.append((batched, per_patch))
    lv.close()
    rec.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("variant", CASES, ids=CASE_IDS)
def test_batched_vjp_equals_per_patch_vjp(cuda, variant):
    rk3_alpha = [[1.0], [0.75, 0.25], [1.0 / 3.0, 0.0, 2.0 / 3.0]]
    for stage, (batched, per_patch) in enumerate(_run(variant)):
        for p, (b, q) in enumerate(zip(batched, per_patch)):
            for s in range(stage + 1):
                x, y = b[s].cpu().numpy(), q[s].cpu().numpy()
                assert np.array_equal(x, y), f"stage {stage} patch {p} slot {s}: max diff {np.abs(x - y).max()}"
                # a slot with a zero SSPRK3 weight that is not the stage's own has a zero adjoint
                assert (np.abs(x).max() > 0.0) == (rk3_alpha[stage][s] != 0.0 or s == stage)


@pytest.mark.gpu
def test_batched_vjp_in_groups_of_patches(cuda):
    """A budget that holds about two patches' reverse buffers: the level runs in several
    groups, with the same results."""
    variant = VARIANTS[5]
    for stage, (batched, per_patch) in enumerate(_run(variant, budget=2 * 40 * 40 * 1300)):
        for b, q in zip(batched, per_patch):
            for s in range(stage + 1):
                assert np.array_equal(b[s].cpu().numpy(), q[s].cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("variant", [VARIANTS[0], VARIANTS[2]], ids=[IDS[0], IDS[2]])
def test_batched_navier_stokes_vjp_equals_per_patch_vjp(cuda, variant, order):
    """NavierStokes contexts (single species, midpoint diffusive flux of each order; 5-ghost
    arrays at sixth order): the batched VJP is bitwise the per-patch one."""
    for stage, (batched, per_patch) in enumerate(_run(variant, diffusive=order)):
        for p, (b, q) in enumerate(zip(batched, per_patch)):
            for s in range(stage + 1):
                x, y = b[s].cpu().numpy(), q[s].cpu().numpy()
                assert np.array_equal(x, y), f"stage {stage} patch {p} slot {s}: max diff {np.abs(x - y).max()}"
