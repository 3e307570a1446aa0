"""The hand-written adjoint (VJP) of the substep against the oracle's tangent.

The reference has no adjoint, so parity is defined by the dot-product identity
<w, J v> = <J^T w, v>: J v from the dual-number instantiation of the oracle
(pinned to central differences in test_oracle_tangent.py), J^T w from the
CUDA VJP, on the same branch of every discrete choice (the VJP recomputes the
forward in the reference's operation order, which is bitwise the oracle's).
A torch.autograd.Function wrapper (here, in the tests only) chains the VJPs of
several SSPRK3 steps and is compared with the checkpointed reverse sweep of
RungeKuttaLevelIntegrator and with the chained oracle tangent.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import noisy_shock_state, smooth_state, vortex_state
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg

# Relative to sum_i |w_i (J v)_i|: both sides are exact derivatives of the same branch,
# evaluated with different rounding, so the bound is set by the conditioning of the
# reference's formulas.  Two places amplify rounding: the HLLC-HLL blending weights
# depend on the direction of the velocity jump across a face, which on smooth data is
# a near-zero vector (derivatives ~ 1/|jump|, cancelling between the two sides), and
# near discontinuities the WCNS weights 1/(beta + eps)^p see smoothness indicators
# close to eps.
TOL_DOT = {"smooth": 1e-7, "shock": 1e-6}

SSP = [([1.0], 1.0), ([3.0 / 4.0, 1.0 / 4.0], 1.0 / 4.0), ([1.0 / 3.0, 0.0, 2.0 / 3.0], 2.0 / 3.0)]


def _interior_mask(shape, dim):
    m = np.zeros(shape, dtype=bool)
    sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
    m[sl] = True
    return m


def _directions(Q, rng):
    scale = np.abs(Q).mean(axis=(1, 2, 3), keepdims=True) + 1e-3
    return rng.standard_normal(Q.shape) * scale


@pytest.mark.gpu
@pytest.mark.parametrize("stage", [0, 1, 2])
@pytest.mark.parametrize("variant", VARIANTS, ids=IDS)
def test_vjp_dot_product(cuda, variant, stage):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    eu = flow.Euler(rec)
    dx = [1.0 / v for v in n]
    dt = 1.5e-3
    alpha, beta = SSP[stage]
    rng = np.random.default_rng(100 + stage)
    for label, gen in (("smooth", smooth_state), ("shock", noisy_shock_state)):
        Qs = [gen(model, dim, n, seed=20 + k, species_gamma=gam) for k in range(stage + 1)]
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
        assert abs(lhs - rhs) <= TOL_DOT[label] * scale, f"{label}: <w,Jv>={lhs:.16e} <J^T w,v>={rhs:.16e} scale {scale:.3e}"


# On the 2D Taylor-Green state (tests/helpers.py vortex_state: no face selects HLLC-HLL, no
# stencil is constant) neither ill-conditioned place is reached, and the identity holds to the
# rounding of an FP64 evaluation.  (The 3D form has w = 0 and mirror-symmetric faces, points
# where the reference's flux has no derivative; there the two sides agree to about 1e-5.)
TOL_DOT_VORTEX = 1e-11
VARIANTS_2D = [v for v in VARIANTS if v[1] == 2]
IDS_2D = [i for v, i in zip(VARIANTS, IDS) if v[1] == 2]


@pytest.mark.gpu
@pytest.mark.parametrize("stage", [0, 1, 2])
@pytest.mark.parametrize("variant", VARIANTS_2D, ids=IDS_2D)
def test_vjp_dot_product_tight_on_vortex(cuda, variant, stage):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = variant
    n = (24, 20) if dim == 2 else (12, 10, 8)
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    eu = flow.Euler(rec)
    dx = [1.0 / v for v in n]
    dt = 1.0e-3
    alpha, beta = SSP[stage]
    rng = np.random.default_rng(300 + stage)
    Qs = [vortex_state(model, dim, n, seed=50 + k, species_gamma=gam) for k in range(stage + 1)]
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
    assert abs(lhs - rhs) <= TOL_DOT_VORTEX * scale, \
        f"<w,Jv>={lhs:.16e} <J^T w,v>={rhs:.16e} rel {abs(lhs - rhs) / scale:.3e}"
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (0, 6, 9)], ids=[IDS[i] for i in (0, 6, 9)])
def test_fill_ghosts_vjp_dot_product(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    eu = flow.Euler(make(model, dim, scheme, gam, "exact"))
    rng = np.random.default_rng(7)
    for per in ([1] * dim, [0] * dim, [1, 0, 1][:dim]):
        v = rng.standard_normal(O.ghost_shape(cfg, n))
        w = rng.standard_normal(v.shape)
        Fv = v.copy()
        O.fill_ghosts(cfg, n, per, Fv)
        tw = torch.from_numpy(w).cuda()
        eu.fillGhostsVJP(flow.Patch(n, [1.0] * dim, tw), per)
        torch.cuda.synchronize()
        lhs, rhs = float(np.sum(w * Fv)), float(np.sum(tw.cpu().numpy() * v))
        assert abs(lhs - rhs) <= 1e-12 * float(np.sum(np.abs(w * Fv))), (per, lhs, rhs)


def _objective_grad(model, dim, nsp, Q):
    """J = 1/2 sum_interior rho |u|^2 and dJ/dQ (ghost box, interior only)."""
    m = _interior_mask(Q.shape, dim)
    iu = 1 if model == O.MODEL_SINGLE_SPECIES else nsp
    rho = Q[0] if model == O.MODEL_SINGLE_SPECIES else Q[:nsp].sum(axis=0)
    mom = Q[iu:iu + dim]
    u = mom / rho
    J = 0.5 * float(np.sum((mom * u).sum(axis=0) * m[0]))
    G = np.zeros_like(Q)
    ke = (u * u).sum(axis=0)
    if model == O.MODEL_SINGLE_SPECIES:
        G[0] = -0.5 * ke
    else:
        G[:nsp] = -0.5 * ke
    G[iu:iu + dim] = u
    return J, G * m


def _tangent_steps(cfg, n, dx, dt, per, nsteps, Q, dQ):
    """Chained oracle tangent of nsteps SSPRK3 steps with ghost fill (forward of advance())."""
    Q, dQ = Q.copy(), dQ.copy()
    for _ in range(nsteps):
        O.fill_ghosts(cfg, n, per, Q)
        O.fill_ghosts(cfg, n, per, dQ)
        st = [(Q, dQ)]
        for s in range(3):
            a, b = SSP[s]
            Qo, dQo = O.tangent_substep(cfg, n, dx, dt, s, a, b, [x for x, _ in st], [d for _, d in st])
            if s < 2:
                O.fill_ghosts(cfg, n, per, Qo)
                O.fill_ghosts(cfg, n, per, dQo)
                st.append((Qo, dQo))
            else:
                # the last substep writes the interior of the step's own buffer (ghosts are refilled next)
                m = _interior_mask(Q.shape, cfg.dim)
                Q = np.where(m, Qo, Q)
                dQ = np.where(m, dQo, dQ)
    O.fill_ghosts(cfg, n, per, Q)
    O.fill_ghosts(cfg, n, per, dQ)
    return Q, dQ


ADJ_CASES = [VARIANTS[i] for i in (0, 5, 9)]
ADJ_IDS = [IDS[i] for i in (0, 5, 9)]


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ADJ_CASES, ids=ADJ_IDS)
def test_checkpointed_adjoint_matches_chained_tangent(cuda, variant):
    """4 SSPRK3 steps, checkpoint every 2: <dJ/dQ0, v> from the reverse sweep vs dJ along v."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    nsp = len(gam)
    dx = [1.0 / v for v in n]
    dt, nsteps, per = 1.5e-3, 4, [1] * dim
    Q0 = smooth_state(model, dim, n, seed=5, species_gamma=gam)
    v = _directions(Q0, np.random.default_rng(11)) * _interior_mask(Q0.shape, dim)
    QF, dQF = _tangent_steps(cfg, n, dx, dt, per, nsteps, Q0, v)
    J, G = _objective_grad(model, dim, nsp, QF)
    dJ = float(np.sum(G * dQF))

    rec = make(model, dim, scheme, gam, "exact")
    tQ = torch.from_numpy(Q0).cuda()
    integ = flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, tQ), per)
    integ.advance(dt, nsteps=nsteps, checkpoint_every=2)
    assert np.array_equal(tQ.cpu().numpy(), QF)                  # exact form: bitwise forward
    grad = integ.adjoint(torch.from_numpy(G).cuda())
    torch.cuda.synchronize()
    got = float(np.sum(grad.cpu().numpy() * v))
    assert abs(got - dJ) <= 1e-10 * float(np.sum(np.abs(grad.cpu().numpy() * v))), (got, dJ)


class _Substep:
    """torch.autograd.Function wrappers of the substep and the ghost fill (test-only glue)."""

    @staticmethod
    def make(eu, n, dx, per):
        import torch
        from hamers_gb300 import flow

        class SubstepFn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, stage, dt, *Q):
                out = torch.zeros_like(Q[0])
                eu.substep(flow.Patch(n, dx, Q[stage]), stage, list(Q), dt, out)
                ctx.save_for_backward(*Q)
                ctx.stage, ctx.dt = stage, dt
                return out

            @staticmethod
            def backward(ctx, gout):
                Q = ctx.saved_tensors
                B = [torch.zeros_like(q) for q in Q]
                eu.substepVJP(flow.Patch(n, dx, Q[ctx.stage]), ctx.stage, list(Q), ctx.dt, gout.contiguous(), B)
                return (None, None) + tuple(B)

        class FillFn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, Q):
                out = Q.clone()
                eu.fillGhosts(flow.Patch(n, dx, out), per)
                return out

            @staticmethod
            def backward(ctx, gout):
                g = gout.clone()
                eu.fillGhostsVJP(flow.Patch(n, dx, g), per)
                return g

        return SubstepFn, FillFn


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ADJ_CASES, ids=ADJ_IDS)
def test_autograd_wrapper_and_finite_differences(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    nsp = len(gam)
    dx = [1.0 / v for v in n]
    n = tuple(v + (v % 2) for v in n)          # vortex_state wants even sizes
    dx = [1.0 / v for v in n]
    dt, nsteps, per = 1.5e-3, 3, [1] * dim
    rec = make(model, dim, scheme, gam, "exact")
    eu = flow.Euler(rec)
    SubstepFn, FillFn = _Substep.make(eu, n, dx, per)
    Q0 = vortex_state(model, dim, n, seed=6, species_gamma=gam)
    mask = torch.from_numpy(_interior_mask(Q0.shape, dim)).cuda()

    def run(Q):
        X = Q
        for _ in range(nsteps):
            X = FillFn.apply(X)
            Q1 = FillFn.apply(SubstepFn.apply(0, dt, X))
            Q2 = FillFn.apply(SubstepFn.apply(1, dt, X, Q1))
            X = torch.where(mask, SubstepFn.apply(2, dt, X, Q1, Q2), X)
        X = FillFn.apply(X)
        iu = 1 if model == O.MODEL_SINGLE_SPECIES else nsp
        rho = X[0] if model == O.MODEL_SINGLE_SPECIES else X[:nsp].sum(dim=0)
        mom = X[iu:iu + dim]
        return 0.5 * ((mom * mom).sum(dim=0) / rho * mask[0]).sum()

    x = torch.from_numpy(Q0).cuda().requires_grad_(True)
    J = run(x)
    J.backward()
    g_auto = x.grad.clone()

    # same gradient from the checkpointed reverse sweep
    tQ = torch.from_numpy(Q0).cuda()
    integ = flow.RungeKuttaLevelIntegrator(eu, flow.Patch(n, dx, tQ), per)
    integ.advance(dt, nsteps=nsteps, checkpoint_every=1)
    _, G = _objective_grad(model, dim, nsp, tQ.cpu().numpy())
    g_sweep = integ.adjoint(torch.from_numpy(G).cuda())
    scale = g_auto.abs().max().item()
    assert (g_auto - g_sweep).abs().max().item() <= 1e-12 * scale

    # central differences along smooth interior directions, away from kinks (the vortex
    # state has no HLLC-HLL faces; see vortex_state)
    rng = np.random.default_rng(3)
    with torch.no_grad():
        for _ in range(2):
            v = torch.from_numpy(_directions(Q0, rng)).cuda() * mask
            h = 1e-7
            fd = (run(x.detach() + h * v) - run(x.detach() - h * v)).item() / (2 * h)
            ad = (g_auto * v).sum().item()
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-12), (fd, ad)
