"""Navier-Stokes on the device: the midpoint diffusive flux and the NavierStokes stage
against the oracle (single species, second and fourth order, 2D and 3D).

Exact form bitwise (diffusive face fluxes, the general stage, SSPRK3 steps of the fused
substep); fast form within 1e-12 per call, like the convective path.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err, shock_state, smooth_state

TRANSPORT = dict(species_mu=0.02, species_mu_v=0.005, species_c_p=3.5, species_Pr=0.72)
CASES = [(2, 4, (37, 29)), (2, 2, (37, 29)), (3, 4, (13, 11, 9)), (3, 2, (12, 10, 9))]
IDS = ["2d-o4", "2d-o2", "3d-o4", "3d-o2"]
SCHEMES = {O.SCHEME_WCNS5_JS: "WCNS5_JS_HLLC_HLL", O.SCHEME_WCNS6_LD: "WCNS6_LD_HLLC_HLL"}


def transport(order):
    t = TRANSPORT
    return O.Transport(t["species_mu"], t["species_c_p"], t["species_Pr"], mu_v=t["species_mu_v"], order=order)


def make(dim, order, precision, scheme=O.SCHEME_WCNS5_JS):
    from hamers_gb300 import flow
    fm = flow.FlowModel("SINGLE_SPECIES", dim, [1.4], transport=TRANSPORT)
    name = "MIDPOINT_FOURTH_ORDER" if order == 4 else "MIDPOINT_SECOND_ORDER"
    rec = flow.ConvectiveFluxReconstructor(SCHEMES[scheme], fm, precision=precision, diffusive_flux_reconstructor=name)
    return flow.NavierStokes(rec)


def states(dim, n):
    return [("smooth", smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=11, species_gamma=[1.4])),
            ("shock", shock_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=12, species_gamma=[1.4]))]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_diffusive_flux(cuda, case, precision):
    import torch
    from hamers_gb300 import flow
    dim, order, n = case
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, precision)
    dx = [1.0 / (v + 3) for v in n]
    dt = 1.7e-3
    for label, Q in states(dim, n):
        Fo = O.diff_flux(cfg, transport(order), n, dx, dt, Q)
        patch = flow.Patch(n, dx, torch.from_numpy(Q).cuda())
        F = ns.rec.allocateFlux(patch)
        ns.diff.computeDiffusiveFluxOnPatch(patch, F, dt)
        torch.cuda.synchronize()
        for a in range(dim):
            got = F[a].cpu().numpy()
            if precision == "exact":
                assert np.array_equal(got, Fo[a]), f"{label} axis {a}: max diff {np.abs(got - Fo[a]).max()}"
            else:
                assert rel_err(got[1:], Fo[a][1:]) <= 1e-12, f"{label} axis {a}: {rel_err(got[1:], Fo[a][1:]):.3e}"
                assert not np.any(got[0])
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES[:3], ids=IDS[:3])
def test_navier_stokes_stage_general(cuda, case):
    """advanceSingleStepOnPatch of NavierStokes with three coefficient sets and accumulation."""
    import torch
    from hamers_gb300 import flow
    dim, order, n = case
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, "exact")
    dx = [1.0 / v for v in n]
    rng = np.random.default_rng(6)
    Qs = [smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=20 + k, species_gamma=[1.4]) for k in range(3)]
    Fs, Ds, Ss = [], [], []
    for k in range(3):
        F, S, _ = O.conv_flux_source(cfg, n, dx, 1e-3, Qs[k])
        Fs.append(F)
        Ds.append(O.diff_flux(cfg, transport(order), n, dx, 1e-3, Qs[k]))
        Ss.append(S + 1e-3 * rng.standard_normal(S.shape))
    alpha, beta, gamma = [0.3, 0.2, 0.5], [0.1, 0.25, 0.6], [0.2, 0.3, 0.5]
    Qo = O.rk_stage_ns(cfg, n, dx, alpha, beta, gamma, Qs, Fs, Ds, Ss)
    t = lambda arrs: [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
    out = torch.zeros_like(torch.from_numpy(Qs[0])).cuda()
    Fa = [torch.zeros(f.shape, dtype=torch.float64, device="cuda") for f in Fs[0]]
    Da = [torch.zeros(f.shape, dtype=torch.float64, device="cuda") for f in Fs[0]]
    Sa = torch.zeros(Ss[0].shape, dtype=torch.float64, device="cuda")
    ns.advanceSingleStepOnPatch(flow.Patch(n, dx, out), alpha, beta, gamma, t(Qs), [t(F) for F in Fs],
                                [t(D) for D in Ds], t(Ss), Fa, Da, Sa)
    torch.cuda.synchronize()
    sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
    assert np.array_equal(out.cpu().numpy()[sl], Qo[sl])
    for a in range(dim):
        exp_f = sum(g * F[a] for g, F in zip(gamma, Fs))
        exp_d = sum(g * D[a] for g, D in zip(gamma, Ds))
        assert np.allclose(Fa[a].cpu().numpy(), exp_f, rtol=1e-14, atol=1e-300)
        assert np.allclose(Da[a].cpu().numpy(), exp_d, rtol=1e-14, atol=1e-300)
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_navier_stokes_rk3_steps(cuda, case, precision):
    """Two SSPRK3 steps of the Navier-Stokes equations with periodic ghosts, fused substep."""
    import torch
    from hamers_gb300 import flow
    dim, order, n = case
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, precision)
    dx = [1.0 / v for v in n]
    dt = 1.5e-3
    Q = smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=13, species_gamma=[1.4])
    per = [1] * dim
    Qo = Q.copy()
    O.fill_ghosts(cfg, n, per, Qo)
    O.ns_rk3_advance(cfg, transport(order), n, dx, dt, per, 2, Qo)
    Qg = torch.from_numpy(Q).cuda()
    flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qg), per).advance(dt, nsteps=2)
    out = Qg.cpu().numpy()
    if precision == "exact":
        assert np.array_equal(out, Qo), f"max diff {np.abs(out - Qo).max()}"
    else:
        assert rel_err(out, Qo) <= 1e-9, f"rel err {rel_err(out, Qo):.3e}"
    # the diffusive terms are really there
    Qe = Q.copy()
    O.fill_ghosts(cfg, n, per, Qe)
    O.rk3_advance(cfg, n, dx, dt, per, 2, Qe)
    assert np.abs(Qe - Qo).max() > 1e-8
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("stage", [0, 2])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_navier_stokes_vjp_dot_product(cuda, case, stage):
    """The substep adjoint with the diffusive flux against the oracle's dual-number tangent."""
    import torch
    from hamers_gb300 import flow
    from tests.helpers import noisy_shock_state
    from tests.test_gpu_adjoint import SSP, TOL_DOT, _directions, _interior_mask
    dim, order, n = case
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, "exact")
    dx = [1.0 / v for v in n]
    dt = 1.5e-3
    alpha, beta = SSP[stage]
    rng = np.random.default_rng(300 + stage)
    for label, gen in (("smooth", smooth_state), ("shock", noisy_shock_state)):
        Qs = [gen(O.MODEL_SINGLE_SPECIES, dim, n, seed=60 + k, species_gamma=[1.4]) for k in range(stage + 1)]
        O.fill_ghosts(cfg, n, [1] * dim, Qs[stage])
        V = [_directions(q, rng) for q in Qs]
        W = rng.standard_normal(Qs[0].shape) * _interior_mask(Qs[0].shape, dim)
        _, JV = O.tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Qs, V, transport=transport(order))
        lhs = float(np.sum(W * JV))
        scale = float(np.sum(np.abs(W * JV)))
        tQ = [torch.from_numpy(q).cuda() for q in Qs]
        tB = [torch.zeros_like(t) for t in tQ]
        ns.substepVJP(flow.Patch(n, dx, tQ[stage]), stage, tQ, dt, torch.from_numpy(W).cuda(), tB)
        torch.cuda.synchronize()
        rhs = float(sum(np.sum(b.cpu().numpy() * v) for b, v in zip(tB, V)))
        assert abs(lhs - rhs) <= TOL_DOT[label] * scale, f"{label}: {lhs:.16e} vs {rhs:.16e} scale {scale:.3e}"
        # the diffusive part is in the adjoint: the Euler adjoint differs
        _, JVe = O.tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Qs, V)
        assert abs(float(np.sum(W * JVe)) - rhs) > 10 * TOL_DOT[label] * scale
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[0], CASES[2]], ids=[IDS[0], IDS[2]])
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_batched_level_navier_stokes(cuda, case, precision):
    """Uneven patches of one level in the persistent kernel with the diffusive phases: exact
    form bitwise to the oracle's NavierStokes steps per patch, fast form within 1e-9."""
    import torch
    from hamers_gb300 import flow
    dim, order, _ = case
    rng = np.random.default_rng(23)
    if dim == 2:
        sizes = [(int(rng.integers(6, 26)), int(rng.integers(6, 26))) for _ in range(4)]
    else:
        sizes = [tuple(int(rng.integers(5, 12)) for _ in range(3)) for _ in range(3)]
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, precision)
    dt = 1.0e-3
    geoms, tens, expect = [], [], []
    for p, n in enumerate(sizes):
        dx = [1.0 / v for v in n]
        Q = smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=40 + p, species_gamma=[1.4])
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, [1] * dim, Qo)
        O.ns_rk3_advance(cfg, transport(order), n, dx, dt, [1] * dim, 2, Qo)
        geoms.append((list(n), dx))
        tens.append(torch.from_numpy(Q).cuda())
        expect.append(Qo)
    lv = flow.BatchedLevel(ns.rec, geoms)
    for p, Q in enumerate(tens):
        lv.bind(p, Q)
        lv.set_periodic(p, [1] * dim)
    for _ in range(2):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    sl = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
    for Q, Qo in zip(tens, expect):
        got = Q.cpu().numpy()[sl]
        if precision == "exact":
            assert np.array_equal(got, Qo[sl]), np.abs(got - Qo[sl]).max()
        else:
            assert rel_err(got, Qo[sl]) <= 1e-9
    lv.close()
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[0], CASES[2]], ids=[IDS[0], IDS[2]])
def test_navier_stokes_stable_dt(cuda, case):
    """NavierStokes::computeSpectralRadiusesAndStableDtOnPatch: the acoustic and diffusive radii
    over the ghost box, bitwise; and the level's on-device dt = (1/(max + eps))*cfl."""
    import torch
    from hamers_gb300 import flow
    dim, order, n = case
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
    ns = make(dim, order, "exact")
    # a viscous case: the diffusive radius dominates on the finer axis
    dx = [1.0 / v for v in n]
    dx[0] *= 1e-3
    Q = smooth_state(O.MODEL_SINGLE_SPECIES, dim, n, seed=17, species_gamma=[1.4])
    want = O.spectral_radius(cfg, n, dx, Q, transport=transport(order))
    assert want > O.spectral_radius(cfg, n, dx, Q)
    got = ns.spectralRadius(flow.Patch(n, dx, torch.from_numpy(Q).cuda()))
    assert got == want
    lv = flow.BatchedLevel(ns.rec, [(list(n), dx)])
    Qg = torch.from_numpy(Q).cuda()
    lv.bind(0, Qg)
    lv.set_periodic(0, [1] * dim)
    lv.step_cfl(0.4)
    torch.cuda.synchronize()
    lv.check()
    assert lv.last_dt() == (1.0 / (want + 1e-15)) * 0.4
    lv.close()
    ns.rec.close()
