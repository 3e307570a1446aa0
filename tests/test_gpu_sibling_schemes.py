"""WCNS5-Z and WCNS6-CU-M2: the sibling weight formulas on the same WCNS56 driver.

ConvectiveFluxReconstructorWCNS5-Z-HLLC-HLL.cpp:78-168 and
ConvectiveFluxReconstructorWCNS6-CU-M2-HLLC-HLL.cpp:112-228, checked against
the oracle the way WCNS5-JS / WCNS6-LD are: exact form bitwise (fluxes,
source, face counters), fast form within 1e-12 per call, SSPRK3 steps, and the
batched level.  WCNS6-CU-M2 scales its weights by the grid geometry's (coarsest
level's) spacing, which on a finer level differs from the patch's own; that
case is covered too.
"""
import numpy as np
import pytest

from hamers_gb300 import problems as P
from oracle import oracle as O
from tests.helpers import rel_err, smooth_state
from tests.test_gpu_parity import NAMES, gpu_flux, species_R, states

TOL_FAST = 1e-12
SCHEMES = {O.SCHEME_WCNS5_Z: "WCNS5_Z_HLLC_HLL", O.SCHEME_WCNS6_CU_M2: "WCNS6_CU_M2_HLLC_HLL"}

VARIANTS = [
    (O.MODEL_SINGLE_SPECIES, 2, (37, 29), [1.4]),
    (O.MODEL_SINGLE_SPECIES, 3, (13, 11, 9), [1.4]),
    (O.MODEL_FIVE_EQN_ALLAIRE, 2, (33, 27), [1.4, 1.67]),
    (O.MODEL_FIVE_EQN_ALLAIRE, 3, (12, 10, 9), [1.4, 1.09]),
    (O.MODEL_FOUR_EQN_CONSERVATIVE, 2, (31, 26), P.FOUR_EQN_GAMMA),
    (O.MODEL_FOUR_EQN_CONSERVATIVE, 3, (11, 10, 9), P.FOUR_EQN_GAMMA),
]
MID = {O.MODEL_SINGLE_SPECIES: "single", O.MODEL_FOUR_EQN_CONSERVATIVE: "four", O.MODEL_FIVE_EQN_ALLAIRE: "five"}
CASES = [(s,) + v for s in SCHEMES for v in VARIANTS]
IDS = ["%s-%s-%dd" % ("z" if s == O.SCHEME_WCNS5_Z else "cu", MID[m], d) for s, m, d, _, _ in CASES]


def ocfg(model, dim, gam, scheme, grid_dx):
    return O.Config(model, dim, gam, scheme, species_R=species_R(model), grid_dx=grid_dx)


def make(model, dim, scheme, gam, precision, grid_dx):
    from hamers_gb300 import flow
    fm = flow.FlowModel(NAMES[model], dim, gam, species_R=species_R(model))
    return flow.ConvectiveFluxReconstructor(SCHEMES[scheme], fm, precision=precision, grid_geometry=grid_dx)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_flux_source(cuda, case, precision):
    scheme, model, dim, n, gam = case
    dx = [1.0 / v for v in n]
    cfg = ocfg(model, dim, gam, scheme, dx)
    rec = make(model, dim, scheme, gam, precision, dx)
    dt = 1.3e-3
    for label, Q in states(model, dim, n, gam):
        Fo, So, st = O.conv_flux_source(cfg, n, dx, dt, Q)
        Fg, Sg = gpu_flux(rec, n, dx, dt, Q)
        for a in range(dim):
            if precision == "exact":
                assert np.array_equal(Fg[a], Fo[a]), f"{label}: axis {a} max diff {np.abs(Fg[a] - Fo[a]).max()}"
            else:
                err = rel_err(Fg[a], Fo[a])
                assert err <= TOL_FAST, f"{label}: flux axis {a} rel err {err:.3e}"
        if precision == "exact":
            assert np.array_equal(Sg, So), f"{label}: source differs"
        elif model == O.MODEL_FIVE_EQN_ALLAIRE:
            assert rel_err(Sg[-1:], So[-1:]) <= TOL_FAST
        assert rec.readCounters() == (st[1], st[2]), f"{label}: face counters"
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("model", [O.MODEL_SINGLE_SPECIES, O.MODEL_FIVE_EQN_ALLAIRE], ids=["single", "five"])
def test_cu_m2_uses_the_grid_geometry_spacing(cuda, model):
    """A patch of a level refined by 2 and 4: the weights take the coarse spacing (bitwise),
    and differ from a reconstructor given the patch's own spacing."""
    dim, n = 2, (24, 20)
    gam = [1.4] if model == O.MODEL_SINGLE_SPECIES else [1.4, 1.67]
    coarse = [0.1, 0.125]
    Q = states(model, dim, n, gam)[1][1]
    for ratio in (2, 4):
        dx = [v / ratio for v in coarse]
        cfg = ocfg(model, dim, gam, O.SCHEME_WCNS6_CU_M2, coarse)
        Fo, So, _ = O.conv_flux_source(cfg, n, dx, 1e-3, Q)
        rec = make(model, dim, O.SCHEME_WCNS6_CU_M2, gam, "exact", coarse)
        Fg, Sg = gpu_flux(rec, n, dx, 1e-3, Q)
        for a in range(dim):
            assert np.array_equal(Fg[a], Fo[a])
        assert np.array_equal(Sg, So)
        own = make(model, dim, O.SCHEME_WCNS6_CU_M2, gam, "exact", dx)
        Fw, _ = gpu_flux(own, n, dx, 1e-3, Q)
        assert any(not np.array_equal(Fw[a], Fo[a]) for a in range(dim))
        rec.close()
        own.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[i] for i in (0, 3, 6, 9)], ids=[IDS[i] for i in (0, 3, 6, 9)])
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_rk3_steps(cuda, case, precision):
    """Two SSPRK3 steps with periodic ghosts through the fused substep."""
    import torch
    from hamers_gb300 import flow
    scheme, model, dim, n, gam = case
    dx = [1.0 / v for v in n]
    cfg = ocfg(model, dim, gam, scheme, dx)
    rec = make(model, dim, scheme, gam, precision, dx)
    dt = 2.0e-3
    Q = smooth_state(model, dim, n, seed=3, species_gamma=gam)
    per = [1] * dim
    Qo = Q.copy()
    O.fill_ghosts(cfg, n, per, Qo)
    O.rk3_advance(cfg, n, dx, dt, per, 2, Qo)
    Qg = torch.from_numpy(Q).cuda()
    flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qg), per).advance(dt, nsteps=2)
    out = Qg.cpu().numpy()
    if precision == "exact":
        assert np.array_equal(out, Qo), f"max diff {np.abs(out - Qo).max()}"
    else:
        assert rel_err(out, Qo) <= 1e-9, f"rel err {rel_err(out, Qo):.3e}"
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[i] for i in (2, 5, 8, 11)], ids=[IDS[i] for i in (2, 5, 8, 11)])
def test_batched_level_exact(cuda, case):
    """Uneven patches of one level, one persistent kernel per substep, bitwise to the oracle."""
    import torch
    from hamers_gb300 import flow
    scheme, model, dim, _, gam = case
    rng = np.random.default_rng(21)
    if dim == 2:
        sizes = [(int(rng.integers(8, 30)), int(rng.integers(8, 30))) for _ in range(4)]
    else:
        sizes = [tuple(int(rng.integers(6, 13)) for _ in range(3)) for _ in range(3)]
    grid_dx = [0.05] * dim
    dt = 1.0e-3
    cfg = ocfg(model, dim, gam, scheme, grid_dx)
    rec = make(model, dim, scheme, gam, "exact", grid_dx)
    geoms, tens, expect = [], [], []
    for p, n in enumerate(sizes):
        dx = [1.0 / v for v in n]
        Q = smooth_state(model, dim, n, seed=30 + p, species_gamma=gam)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, [1] * dim, Qo)
        O.rk3_advance(cfg, n, dx, dt, [1] * dim, 1, Qo)
        geoms.append((list(n), dx))
        tens.append(torch.from_numpy(Q).cuda())
        expect.append(Qo)
    lv = flow.BatchedLevel(rec, geoms)
    for p, Q in enumerate(tens):
        lv.bind(p, Q)
        lv.set_periodic(p, [1] * dim)
    lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    sl = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
    for Q, Qo in zip(tens, expect):
        assert np.array_equal(Q.cpu().numpy()[sl], Qo[sl])
    lv.close()
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("stage", [0, 2])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_vjp_dot_product(cuda, case, stage):
    """The substep adjoint against the oracle's dual-number tangent: <w, J v> = <J^T w, v>."""
    import torch
    from hamers_gb300 import flow
    from tests.helpers import noisy_shock_state
    from tests.test_gpu_adjoint import SSP, TOL_DOT, _directions, _interior_mask
    scheme, model, dim, n, gam = case
    dx = [1.0 / v for v in n]
    cfg = ocfg(model, dim, gam, scheme, dx)
    eu = flow.Euler(make(model, dim, scheme, gam, "exact", dx))
    dt = 1.5e-3
    alpha, beta = SSP[stage]
    rng = np.random.default_rng(200 + stage)
    for label, gen in (("smooth", smooth_state), ("shock", noisy_shock_state)):
        Qs = [gen(model, dim, n, seed=50 + k, species_gamma=gam) for k in range(stage + 1)]
        O.fill_ghosts(cfg, n, [1] * dim, Qs[stage])
        V = [_directions(q, rng) for q in Qs]
        W = rng.standard_normal(Qs[0].shape) * _interior_mask(Qs[0].shape, dim)
        _, JV = O.tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Qs, V)
        lhs = float(np.sum(W * JV))
        scale = float(np.sum(np.abs(W * JV)))
        tQ = [torch.from_numpy(q).cuda() for q in Qs]
        tB = [torch.zeros_like(t) for t in tQ]
        eu.substepVJP(flow.Patch(n, dx, tQ[stage]), stage, tQ, dt, torch.from_numpy(W).cuda(), tB)
        torch.cuda.synchronize()
        rhs = float(sum(np.sum(b.cpu().numpy() * v) for b, v in zip(tB, V)))
        assert abs(lhs - rhs) <= TOL_DOT[label] * scale, f"{label}: {lhs:.16e} vs {rhs:.16e} scale {scale:.3e}"
