"""Navier-Stokes with the sixth-order midpoint diffusive flux on the device
(DiffusiveFluxReconstructorMidpointSixthOrder, 5 ghost cells) against the oracle, whose
sixth order is bitwise the reference's own code (tests/test_ref_oracle.py).

Exact form bitwise (diffusive face fluxes, the general NavierStokes stage, SSPRK3 steps of the
fused substep, the spectral radius over the 5-ghost box, reflecting and periodic ghost fills);
fast form within 1e-12 per flux and 1e-9 over two steps.  A sixth-order context reads and writes
5-ghost patch arrays everywhere, the batched level's included (uneven patches with their own
fills, and a tiled domain with the device ghost exchange, against the oracle), and the
substep VJP against the oracle's tangent.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err, shock_state, smooth_state

TRANSPORT = dict(species_mu=0.02, species_mu_v=0.005, species_c_p=3.5, species_Pr=0.72)
CASES = [(2, (37, 29)), (3, (13, 11, 9))]
IDS = ["2d", "3d"]
GH = 5


def transport():
    t = TRANSPORT
    return O.Transport(t["species_mu"], t["species_c_p"], t["species_Pr"], mu_v=t["species_mu_v"], order=6)


def make(dim, precision):
    from hamers_gb300 import flow
    fm = flow.FlowModel("SINGLE_SPECIES", dim, [1.4], transport=TRANSPORT)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=precision,
                                           diffusive_flux_reconstructor="MIDPOINT_SIXTH_ORDER")
    return flow.NavierStokes(rec)


def cfg_of(dim):
    return O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4], ghosts=GH)


def state(gen, dim, n, seed):
    """A state on the 5-ghost box of n (generated on n grown by one cell per side)."""
    return gen(O.MODEL_SINGLE_SPECIES, dim, [v + 2 for v in n], seed=seed, species_gamma=[1.4])


def interior(dim):
    return (slice(None),) + tuple(slice(GH, -GH) if a < dim else slice(None) for a in (2, 1, 0))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_diffusive_flux(cuda, case, precision):
    import torch
    from hamers_gb300 import flow
    dim, n = case
    cfg = cfg_of(dim)
    ns = make(dim, precision)
    assert ns.rec.getPatchNumberOfGhostCells() == GH
    assert ns.diff.getDiffusiveFluxNumberOfGhostCells() == GH
    dx = [1.0 / (v + 3) for v in n]
    dt = 1.7e-3
    for label, gen in (("smooth", smooth_state), ("shock", shock_state)):
        Q = state(gen, dim, n, 11)
        Fo = O.diff_flux(cfg, transport(), n, dx, dt, Q)
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
        # the convective flux of the same 5-ghost arrays is the 4-ghost one
        Fc, Sc, _ = O.conv_flux_source(cfg, n, dx, dt, Q)
        Fg = ns.rec.allocateFlux(patch)
        Sg = ns.rec.allocateSource(patch)
        ns.rec.computeConvectiveFluxAndSourceOnPatch(patch, Fg, Sg, dt)
        torch.cuda.synchronize()
        for a in range(dim):
            got = Fg[a].cpu().numpy()
            if precision == "exact":
                assert np.array_equal(got, Fc[a])
            else:
                assert rel_err(got[1:], Fc[a][1:]) <= 1e-12
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_stage_general(cuda, case):
    """NavierStokes::advanceSingleStepOnPatch with three coefficient sets, 5-ghost arrays."""
    import torch
    from hamers_gb300 import flow
    dim, n = case
    cfg = cfg_of(dim)
    ns = make(dim, "exact")
    dx = [1.0 / v for v in n]
    rng = np.random.default_rng(6)
    Qs = [state(smooth_state, dim, n, 20 + k) for k in range(3)]
    Fs, Ds, Ss = [], [], []
    for k in range(3):
        F, S, _ = O.conv_flux_source(cfg, n, dx, 1e-3, Qs[k])
        Fs.append(F)
        Ds.append(O.diff_flux(cfg, transport(), n, dx, 1e-3, Qs[k]))
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
    sl = interior(dim)
    assert np.array_equal(out.cpu().numpy()[sl], Qo[sl])
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_rk3_steps(cuda, case, precision):
    """Two SSPRK3 steps with the fused substep: periodic, and reflecting walls on the first axis."""
    import torch
    from hamers_gb300 import flow
    dim, n = case
    cfg = cfg_of(dim)
    ns = make(dim, precision)
    dx = [1.0 / v for v in n]
    dt = 1.5e-3
    for per in ([1] * dim, [3] + [1] * (dim - 1)):
        Q = state(smooth_state, dim, n, 13)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo)
        O.ns_rk3_advance(cfg, transport(), n, dx, dt, per, 2, Qo)
        Qg = torch.from_numpy(Q).cuda()
        flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qg), per).advance(dt, nsteps=2)
        out = Qg.cpu().numpy()
        if precision == "exact":
            assert np.array_equal(out, Qo), f"{per}: max diff {np.abs(out - Qo).max()}"
        else:
            assert rel_err(out, Qo) <= 1e-9, f"{per}: rel err {rel_err(out, Qo):.3e}"
        # the sixth-order terms are there: the fourth order gives another result
        tr4 = O.Transport(TRANSPORT["species_mu"], TRANSPORT["species_c_p"], TRANSPORT["species_Pr"],
                          mu_v=TRANSPORT["species_mu_v"], order=4)
        Q4 = Q.copy()
        O.fill_ghosts(cfg, n, per, Q4)
        O.ns_rk3_advance(cfg, tr4, n, dx, dt, per, 2, Q4)
        assert np.abs(Q4 - Qo).max() > 1e-14
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_spectral_radius_and_fills(cuda, case):
    """The spectral radius runs over the 5-ghost box; ghost fills (periodic, zero-gradient,
    reflecting) and the fill's adjoint use the 5-cell width."""
    import torch
    from hamers_gb300 import flow
    dim, n = case
    cfg = cfg_of(dim)
    ns = make(dim, "exact")
    dx = [1.0 / v for v in n]
    dx[0] *= 1e-3
    Q = state(smooth_state, dim, n, 17)
    want = O.spectral_radius(cfg, n, dx, Q, transport=transport())
    assert ns.spectralRadius(flow.Patch(n, dx, torch.from_numpy(Q).cuda())) == want
    rng = np.random.default_rng(4)
    for per in ([1] * dim, [0] * dim, [3] * dim, [3, 0, 1][:dim]):
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo)
        Qg = torch.from_numpy(Q.copy()).cuda()
        ns.fillGhosts(flow.Patch(n, dx, Qg), per)
        torch.cuda.synchronize()
        assert np.array_equal(Qg.cpu().numpy(), Qo), per
        v = rng.standard_normal(Q.shape)
        w = rng.standard_normal(Q.shape)
        Fv = v.copy()
        O.fill_ghosts(cfg, n, per, Fv)
        tw = torch.from_numpy(w).cuda()
        ns.fillGhostsVJP(flow.Patch(n, dx, tw), per)
        torch.cuda.synchronize()
        lhs, rhs = float(np.sum(w * Fv)), float(np.sum(tw.cpu().numpy() * v))
        assert abs(lhs - rhs) <= 1e-12 * float(np.sum(np.abs(w * Fv))), (per, lhs, rhs)
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_batched_level(cuda, case, precision):
    """Uneven patches of one level in the persistent kernel (5-ghost arrays, each patch with its
    own periodic or reflecting fill): exact form bitwise to the oracle's NavierStokes steps per
    patch, fast form within 1e-9."""
    import torch
    from hamers_gb300 import flow
    dim, _ = case
    rng = np.random.default_rng(29)
    if dim == 2:
        sizes = [(int(rng.integers(6, 26)), int(rng.integers(6, 26))) for _ in range(4)]
    else:
        sizes = [tuple(int(rng.integers(5, 12)) for _ in range(3)) for _ in range(3)]
    cfg = cfg_of(dim)
    ns = make(dim, precision)
    dt = 1.0e-3
    geoms, tens, expect, pers = [], [], [], []
    for p, n in enumerate(sizes):
        dx = [1.0 / v for v in n]
        per = [3 if (p + a) % 2 else 1 for a in range(dim)]
        Q = state(smooth_state, dim, n, 40 + p)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo)
        O.ns_rk3_advance(cfg, transport(), n, dx, dt, per, 2, Qo)
        geoms.append((list(n), dx))
        tens.append(torch.from_numpy(Q).cuda())
        expect.append(Qo)
        pers.append(per)
    lv = flow.BatchedLevel(ns.rec, geoms)
    for p, Q in enumerate(tens):
        assert tuple(Q.shape) == lv.shapes[p]
        lv.bind(p, Q)
        lv.set_periodic(p, pers[p])
    for _ in range(2):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    sl = interior(dim)
    for Q, Qo in zip(tens, expect):
        got = Q.cpu().numpy()[sl]
        if precision == "exact":
            assert np.array_equal(got, Qo[sl]), np.abs(got - Qo[sl]).max()
        else:
            assert rel_err(got, Qo[sl]) <= 1e-9
    lv.close()
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(2, (36, 30), (1, 3)), (3, (15, 13, 12), (3, 1, 1))], ids=["2d", "3d"])
def test_sixth_order_tiled_level_equals_one_patch(cuda, case):
    """A domain tiled by uneven patches (down to two cells wide), advanced by the batched
    substeps with the device ghost exchange over 5-cell halos, equals the oracle's single patch
    covering the domain, bitwise (exact form)."""
    import torch
    from hamers_gb300 import flow
    from tests.test_gpu_exchange import _tile
    dim, domain, periodic = case
    cfg = cfg_of(dim)
    dx = [1.0 / v for v in domain]
    dt, nsteps = 1.0e-3, 2
    Qfull = state(shock_state, dim, domain, 31)
    Qo = Qfull.copy()
    O.fill_ghosts(cfg, domain, list(periodic), Qo)
    O.ns_rk3_advance(cfg, transport(), domain, dx, dt, list(periodic), nsteps, Qo)
    rng = np.random.default_rng(9)
    segs = [_tile(domain[a], rng, 2, 13 if dim == 2 else 7) for a in range(dim)]
    starts = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(int) for s in segs]
    boxes = []
    for idx in np.ndindex(*[len(s) for s in segs]):
        boxes.append(([int(starts[a][idx[a]]) for a in range(dim)], [int(segs[a][idx[a]]) for a in range(dim)]))

    def block(Q, lo, n):
        sl = [slice(None)]
        for a in (2, 1, 0):
            sl.append(slice(lo[a] + GH, lo[a] + GH + n[a]) if a < dim else slice(None))
        return Q[tuple(sl)]

    inner = interior(dim)
    states = []
    for lo, n in boxes:
        Q = np.zeros((Qfull.shape[0],) + tuple(n[a] + 2 * GH if a < dim else 1 for a in (2, 1, 0)))
        Q[inner] = block(Qfull, lo, n)
        states.append(torch.from_numpy(Q).cuda())
    ns = make(dim, "exact")
    lv = flow.BatchedLevel(ns.rec, [(n, dx) for _, n in boxes])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
    lv.set_layout([lo for lo, _ in boxes], list(domain), list(periodic))
    for _ in range(nsteps):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    for (lo, n), Q in zip(boxes, states):
        got = Q.cpu().numpy()[inner]
        ref = block(Qo, lo, n)
        assert np.array_equal(got, ref), f"patch at {lo}: max diff {np.abs(got - ref).max()}"
    lv.close()
    ns.rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("stage", [0, 2])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_sixth_order_vjp_dot_product(cuda, case, stage):
    """The substep adjoint with the sixth-order diffusive flux (5-ghost arrays) against the
    oracle's dual-number tangent, <W, J V> = <J^T W, V>, in the tolerances of the Euler
    adjoint; and the diffusive part is in it (the fourth-order tangent differs)."""
    import torch
    from hamers_gb300 import flow
    from tests.helpers import noisy_shock_state
    from tests.test_gpu_adjoint import SSP, TOL_DOT, _directions
    dim, n = case
    cfg = cfg_of(dim)
    ns = make(dim, "exact")
    dx = [1.0 / v for v in n]
    dt = 1.5e-3
    alpha, beta = SSP[stage]
    rng = np.random.default_rng(500 + stage)
    mask = np.zeros((1,) + state(smooth_state, dim, n, 0).shape[1:], dtype=bool)
    mask[interior(dim)] = True
    tr4 = O.Transport(TRANSPORT["species_mu"], TRANSPORT["species_c_p"], TRANSPORT["species_Pr"],
                      mu_v=TRANSPORT["species_mu_v"], order=4)
    for label, gen in (("smooth", smooth_state), ("shock", noisy_shock_state)):
        Qs = [state(gen, dim, n, 60 + k) for k in range(stage + 1)]
        O.fill_ghosts(cfg, n, [1] * dim, Qs[stage])
        V = [_directions(q, rng) for q in Qs]
        W = rng.standard_normal(Qs[0].shape) * mask
        _, JV = O.tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Qs, V, transport=transport())
        lhs = float(np.sum(W * JV))
        scale = float(np.sum(np.abs(W * JV)))
        tQ = [torch.from_numpy(q).cuda() for q in Qs]
        tB = [torch.zeros_like(t) for t in tQ]
        ns.substepVJP(flow.Patch(n, dx, tQ[stage]), stage, tQ, dt, torch.from_numpy(W).cuda(), tB)
        torch.cuda.synchronize()
        rhs = float(sum(np.sum(b.cpu().numpy() * v) for b, v in zip(tB, V)))
        assert abs(lhs - rhs) <= TOL_DOT[label] * scale, f"{label}: {lhs:.16e} vs {rhs:.16e} scale {scale:.3e}"
        _, JV4 = O.tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Qs, V, transport=tr4)
        assert abs(float(np.sum(W * JV4)) - rhs) > 10 * TOL_DOT[label] * scale
    ns.rec.close()


@pytest.mark.gpu
def test_patch_arrays_must_match_the_ghost_width(cuda):
    """The library reads and writes the whole ghost box, so the Python layer refuses an array
    whose extent is not the context's ghost box (4-ghost arrays on a sixth-order context)."""
    import torch
    from hamers_gb300 import flow
    ns = make(2, "exact")
    n = (12, 10)
    Q4 = torch.from_numpy(smooth_state(O.MODEL_SINGLE_SPECIES, 2, n, seed=3, species_gamma=[1.4])).cuda()
    patch = flow.Patch(n, [0.1, 0.1], Q4)
    with pytest.raises(ValueError):
        ns.diff.computeDiffusiveFluxOnPatch(patch, ns.rec.allocateFlux(patch), 1e-3)
    with pytest.raises(ValueError):
        ns.fillGhosts(patch, [1, 1])
    Q5 = torch.from_numpy(state(smooth_state, 2, n, 3)).cuda()
    ns.fillGhosts(flow.Patch(n, [0.1, 0.1], Q5), [1, 1])
    ns.rec.close()
