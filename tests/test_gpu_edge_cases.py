"""Edge cases of the patch geometry: patches one to three cells thick along an axis (the
stencils then read mostly ghost cells), strongly anisotropic spacing, and a single-cell patch.
Exact form bitwise to the oracle for the flux/source and for two SSPRK3 steps with
zero-gradient and periodic ghost fills."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import shock_state, smooth_state
from tests.test_gpu_parity import gpu_flux, make, ocfg

SHAPES_2D = [(1, 7), (2, 3), (3, 1), (1, 1), (17, 2)]
SHAPES_3D = [(1, 4, 3), (2, 1, 5), (3, 3, 1), (1, 1, 1)]
MODELS = [(O.MODEL_SINGLE_SPECIES, [1.4]), (O.MODEL_FIVE_EQN_ALLAIRE, [1.4, 1.67]),
          (O.MODEL_FOUR_EQN_CONSERVATIVE, None)]


def _gam(model, gam):
    from hamers_gb300 import problems as P
    return gam if gam is not None else P.FOUR_EQN_GAMMA


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [O.SCHEME_WCNS5_JS, O.SCHEME_WCNS6_LD], ids=["js", "ld"])
@pytest.mark.parametrize("model,gam", MODELS, ids=["single", "five", "four"])
def test_thin_patches_flux_bitwise(cuda, model, gam, scheme):
    gam = _gam(model, gam)
    for dim, shapes in ((2, SHAPES_2D), (3, SHAPES_3D)):
        cfg = ocfg(model, dim, gam, scheme)
        rec = make(model, dim, scheme, gam, "exact")
        for n in shapes:
            dx = [0.01 * (1 + 7 * d) for d in range(dim)]          # anisotropic spacing
            for label, Q in (("smooth", smooth_state(model, dim, n, seed=3, species_gamma=gam)),
                             ("shock", shock_state(model, dim, n, seed=4, species_gamma=gam))):
                Fo, So, st = O.conv_flux_source(cfg, n, dx, 1e-3, Q)
                Fg, Sg = gpu_flux(rec, n, dx, 1e-3, Q)
                for a in range(dim):
                    assert np.array_equal(Fg[a], Fo[a]), (n, label, a)
                assert np.array_equal(Sg, So), (n, label)
        rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("model,gam", MODELS, ids=["single", "five", "four"])
def test_thin_patches_rk3_bitwise(cuda, model, gam):
    import torch
    from hamers_gb300 import flow
    gam = _gam(model, gam)
    for dim, shapes in ((2, SHAPES_2D), (3, SHAPES_3D)):
        cfg = ocfg(model, dim, gam, O.SCHEME_WCNS6_LD)
        rec = make(model, dim, O.SCHEME_WCNS6_LD, gam, "exact")
        for n in shapes:
            for per in ([0] * dim, [1] * dim):
                dx = [1.0 / (4 + v) for v in n]
                Q = smooth_state(model, dim, n, seed=5, species_gamma=gam)
                Qo = Q.copy()
                O.fill_ghosts(cfg, n, per, Qo)
                O.rk3_advance(cfg, n, dx, 1e-3, per, 2, Qo)
                Qg = torch.from_numpy(Q).cuda()
                flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qg), per).advance(1e-3, nsteps=2)
                assert np.array_equal(Qg.cpu().numpy(), Qo), (n, per)
        rec.close()
