"""Pins the oracle's tangent (dual-number instantiation) to central differences of the oracle.

The reference has no derivative code; the GPU adjoint is checked against this
tangent, so the tangent itself is checked here: along a random direction, the
central difference of the oracle's substep converges to the tangent at second
order (truncation error ~h^2) away from kinks.
"""
import numpy as np
import pytest

from hamers_gb300 import problems as P
from oracle import oracle as O
from tests.helpers import smooth_state

CASES = [
    (O.MODEL_SINGLE_SPECIES, 2, O.SCHEME_WCNS5_JS, [1.4], None),
    (O.MODEL_SINGLE_SPECIES, 2, O.SCHEME_WCNS6_LD, [1.4], None),
    (O.MODEL_FOUR_EQN_CONSERVATIVE, 2, O.SCHEME_WCNS5_JS, P.FOUR_EQN_GAMMA, P.FOUR_EQN_R),
    (O.MODEL_FIVE_EQN_ALLAIRE, 2, O.SCHEME_WCNS5_JS, [1.4, 1.67], None),
    (O.MODEL_FIVE_EQN_ALLAIRE, 2, O.SCHEME_WCNS6_LD, [1.4, 1.67], None),
    (O.MODEL_SINGLE_SPECIES, 3, O.SCHEME_WCNS5_JS, [1.4], None),
    (O.MODEL_SINGLE_SPECIES, 2, O.SCHEME_WCNS5_Z, [1.4], None),
    (O.MODEL_FIVE_EQN_ALLAIRE, 2, O.SCHEME_WCNS5_Z, [1.4, 1.67], None),
    (O.MODEL_SINGLE_SPECIES, 2, O.SCHEME_WCNS6_CU_M2, [1.4], None),
    (O.MODEL_FOUR_EQN_CONSERVATIVE, 2, O.SCHEME_WCNS6_CU_M2, P.FOUR_EQN_GAMMA, P.FOUR_EQN_R),
]
SCHEME_IDS = {O.SCHEME_WCNS5_JS: "js", O.SCHEME_WCNS6_LD: "ld", O.SCHEME_WCNS5_Z: "z", O.SCHEME_WCNS6_CU_M2: "cu"}
IDS = ["%s-%dd-%s" % ({0: "single", 1: "four", 2: "five"}[m], d, SCHEME_IDS[s]) for m, d, s, _, _ in CASES]


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_tangent_matches_central_differences(case):
    model, dim, scheme, gam, R = case
    n = (12, 10) if dim == 2 else (8, 7, 6)
    dx = [0.1] * dim
    cfg = O.Config(model, dim, gam, scheme, species_R=R, grid_dx=dx)
    Q = smooth_state(model, dim, n, seed=3, species_gamma=gam)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(Q.shape) * np.abs(Q).mean(axis=(1, 2, 3), keepdims=True)
    dt = 1e-2
    _, dQ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q], [v])
    zero = np.zeros_like(v)
    errs = []
    for h in (1e-5, 1e-6):
        Qp, _ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q + h * v], [zero])
        Qm, _ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q - h * v], [zero])
        errs.append(np.abs((Qp - Qm) / (2 * h) - dQ).max() / np.abs(dQ).max())
    assert min(errs) < 2e-6, errs


@pytest.mark.parametrize("dim,order", [(2, 4), (3, 4), (2, 2)], ids=["2d-o4", "3d-o4", "2d-o2"])
def test_navier_stokes_tangent_matches_central_differences(dim, order):
    """The same check for the Navier-Stokes substep (diffusive flux included)."""
    n = (12, 10) if dim == 2 else (8, 7, 6)
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    tr = O.Transport(0.05, 3.5, 0.72, mu_v=0.01, order=order)
    Q = smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=4, species_gamma=[1.4])
    rng = np.random.default_rng(1)
    v = rng.standard_normal(Q.shape) * np.abs(Q).mean(axis=(1, 2, 3), keepdims=True)
    dx, dt = [0.1] * dim, 1e-2
    _, dQ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q], [v], transport=tr)
    zero = np.zeros_like(v)
    errs = []
    for h in (1e-5, 1e-6):
        Qp, _ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q + h * v], [zero], transport=tr)
        Qm, _ = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q - h * v], [zero], transport=tr)
        errs.append(np.abs((Qp - Qm) / (2 * h) - dQ).max() / np.abs(dQ).max())
    assert min(errs) < 2e-6, errs
    # and the diffusive part is really there: the Euler tangent differs
    _, dQe = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q], [v])
    assert np.abs(dQe - dQ).max() > 1e-6 * np.abs(dQ).max()
