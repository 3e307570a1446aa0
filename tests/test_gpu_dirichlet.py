"""Dirichlet boundaries and symmetry planes on the device (HMR_FILL_DIRICHLET, the reference's
DIRICHLET condition of BasicCartesianBoundaryUtilities2/3 with EulerBoundaryConditions'
conservative boundary values; HMR_FILL_SYMMETRY, its SYMMETRY condition for every variable).

* the single-patch ghost fill equals the oracle's bitwise (the oracle's Dirichlet and symmetry
  fills are the reference's own, tests/test_ref_oracle.py), Dirichlet sides mixed with
  zero-gradient, periodic, reflecting and symmetry axes, for every flow model in 2D and 3D;
* two SSPRK3 steps of one patch with Dirichlet sides equal the oracle's bitwise (exact form);
* the adjoint of the fill passes the dot-product test <w, F v> = <F^T w, v> (F's linear part:
  Dirichlet ghost cells copy no cell);
* a level tiled by uneven patches with Dirichlet (and symmetry) domain faces, advanced by the batched substeps
  with the device ghost exchange, equals the oracle's single patch covering the domain bitwise,
  its fill adjoint passes the dot-product test and its reverse sweep gives the one patch's
  adjoint;
* values are per context, checked for their count and finiteness.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err, rough_state, shock_state, smooth_state, vortex_state
from tests.test_gpu_level_adjoint import _box, _inner, _layout, _level
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg
from tests.test_ref_oracle import dirichlet_values

PER_2D = ([4, 4], [4, 1], [3, 4], [0, 4], [5, 4], [5, 1])
PER_3D = ([4, 4, 4], [4, 0, 1], [1, 3, 4], [5, 4, 3])


def _pers(dim):
    return PER_2D if dim == 2 else PER_3D


def _set_values(rec, bv, dim):
    for a in range(dim):
        for side in (0, 1):
            rec.setDirichletValues(a, side, bv[2 * a + side])


@pytest.mark.gpu
@pytest.mark.parametrize("variant", VARIANTS, ids=IDS)
def test_dirichlet_fill_bitwise(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    bv = dirichlet_values(smooth_state(model, dim, n, seed=20, species_gamma=gam), dim, seed=7)
    _set_values(rec, bv, dim)
    eu = flow.Euler(rec)
    for per in _pers(dim):
        for Q in (smooth_state(model, dim, n, seed=21, species_gamma=gam),
                  rough_state(model, dim, n, seed=22, species_gamma=gam)):
            Qo = Q.copy()
            O.fill_ghosts(cfg, n, per, Qo, dirichlet=bv)
            Qg = torch.from_numpy(Q).cuda()
            eu.fillGhosts(flow.Patch(n, [1.0] * dim, Qg), per)
            torch.cuda.synchronize()
            assert np.array_equal(Qg.cpu().numpy(), Qo), per
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (1, 3, 5, 7, 9)], ids=[IDS[i] for i in (1, 3, 5, 7, 9)])
def test_dirichlet_rk3_bitwise(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    dx = [1.0 / v for v in n]
    bv = dirichlet_values(shock_state(model, dim, n, seed=24, species_gamma=gam), dim, seed=8)
    _set_values(rec, bv, dim)
    for per in _pers(dim)[:2]:
        Q = shock_state(model, dim, n, seed=23, species_gamma=gam)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo, dirichlet=bv)
        O.rk3_advance(cfg, n, dx, 1e-3, per, 2, Qo, dirichlet=bv)
        Qg = torch.from_numpy(Q).cuda()
        flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qg), per).advance(1e-3, nsteps=2)
        assert np.array_equal(Qg.cpu().numpy(), Qo), per
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (0, 6, 9)], ids=[IDS[i] for i in (0, 6, 9)])
def test_dirichlet_fill_vjp_dot_product(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    eu = flow.Euler(make(model, dim, scheme, gam, "exact"))   # values 0.0: F is linear
    rng = np.random.default_rng(8)
    for per in _pers(dim):
        v = rng.standard_normal(O.ghost_shape(cfg, n))
        w = rng.standard_normal(v.shape)
        Fv = v.copy()
        O.fill_ghosts(cfg, n, per, Fv, dirichlet=np.zeros((2 * dim, v.shape[0])))
        tw = torch.from_numpy(w).cuda()
        eu.fillGhostsVJP(flow.Patch(n, [1.0] * dim, tw), per)
        torch.cuda.synchronize()
        lhs, rhs = float(np.sum(w * Fv)), float(np.sum(tw.cpu().numpy() * v))
        assert abs(lhs - rhs) <= 1e-12 * float(np.sum(np.abs(w * Fv))), (per, lhs, rhs)


LEVEL_CASES = [(1, (30, 26), (4, 1)), (5, (28, 24), (4, 4)), (3, (13, 12, 11), (1, 4, 3)), (9, (26, 22), (3, 4)),
               (4, (30, 24), (5, 4)), (2, (12, 13, 11), (5, 1, 5))]
LEVEL_IDS = ["%s-%s" % (IDS[i], "".join(map(str, per))) for i, _, per in LEVEL_CASES]


@pytest.mark.gpu
@pytest.mark.parametrize("case", LEVEL_CASES, ids=LEVEL_IDS)
def test_tiled_level_dirichlet_equals_one_patch(cuda, case):
    import torch
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    cfg = ocfg(model, dim, gam, scheme)
    dx = [1.0 / v for v in domain]
    dt, nsteps = 1.0e-3, 2
    Qfull = shock_state(model, dim, domain, seed=29, species_gamma=gam)
    bv = dirichlet_values(Qfull[_inner(dim)], dim, seed=9)
    Qo = Qfull.copy()
    O.fill_ghosts(cfg, domain, list(periodic), Qo, dirichlet=bv)
    O.rk3_advance(cfg, domain, dx, dt, list(periodic), nsteps, Qo, dirichlet=bv)
    boxes = _layout(dim, domain, 3)
    rec = make(model, dim, scheme, gam, "exact")
    _set_values(rec, bv, dim)
    shape = lambda n: (Qfull.shape[0],) + tuple(n[a] + 8 if a < dim else 1 for a in (2, 1, 0))
    states = []
    for lo, n in boxes:
        Q = np.zeros(shape(n))
        Q[_inner(dim)] = _box(Qfull, lo, n, dim, False)
        states.append(torch.from_numpy(Q).cuda())
    lv = _level(rec, boxes, dx, domain, periodic, states)
    for _ in range(nsteps):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    for (lo, n), Q in zip(boxes, states):
        got = Q.cpu().numpy()[_inner(dim)]
        ref = _box(Qo, lo, n, dim, False)
        assert np.array_equal(got, ref), f"patch at {lo}: max diff {np.abs(got - ref).max()}"
    lv.close()
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", LEVEL_CASES, ids=LEVEL_IDS)
def test_level_dirichlet_fill_vjp_dot_product(cuda, case):
    import torch
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    cfg = ocfg(model, dim, gam, scheme)
    boxes = _layout(dim, domain, 3)
    rng = np.random.default_rng(17)
    shape = lambda n: (cfg.ncomp,) + tuple(n[a] + 8 if a < dim else 1 for a in (2, 1, 0))
    V = [rng.standard_normal(shape(n)) for _, n in boxes]
    W = [rng.standard_normal(shape(n)) for _, n in boxes]
    full = np.zeros(O.ghost_shape(cfg, domain))
    for (lo, n), v in zip(boxes, V):
        _box(full, lo, n, dim, False)[...] = v[_inner(dim)]
    O.fill_ghosts(cfg, domain, list(periodic), full, dirichlet=np.zeros((2 * dim, cfg.ncomp)))
    FV = [np.ascontiguousarray(_box(full, lo, n, dim, True)) for lo, n in boxes]
    rec = make(model, dim, scheme, gam, "exact")
    states = [torch.zeros(shape(n), dtype=torch.float64, device="cuda") for _, n in boxes]
    lv = _level(rec, boxes, [1.0 / v for v in domain], domain, periodic, states)
    tw = [torch.from_numpy(w.copy()).cuda() for w in W]
    lv.fillGhostsVJP(tw)
    torch.cuda.synchronize()
    lhs = sum(float(np.sum(w * fv)) for w, fv in zip(W, FV))
    rhs = sum(float(np.sum(t.cpu().numpy() * v)) for t, v in zip(tw, V))
    scale = sum(float(np.sum(np.abs(w * fv))) for w, fv in zip(W, FV))
    assert abs(lhs - rhs) <= 1e-13 * scale, (lhs, rhs)
    lv.close()
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", [LEVEL_CASES[0], LEVEL_CASES[2]], ids=[LEVEL_IDS[0], LEVEL_IDS[2]])
def test_level_dirichlet_reverse_sweep_equals_one_patch(cuda, case):
    """As tests/test_gpu_level_adjoint.py's sweep, with Dirichlet domain faces (single species,
    whose smooth and Taylor-Green states select no HLLC-HLL face)."""
    import torch
    from hamers_gb300 import flow
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    dx = [1.0 / v for v in domain]
    dt, nsteps, every = 1.0e-3, 4, 2
    Qfull = (vortex_state if dim == 2 else smooth_state)(model, dim, domain, seed=21, species_gamma=gam)
    bv = dirichlet_values(Qfull[_inner(dim)], dim, seed=10)
    boxes = _layout(dim, domain, 5)
    rng = np.random.default_rng(23)
    Wfull = np.zeros_like(Qfull)
    Wfull[_inner(dim)] = rng.standard_normal(Wfull[_inner(dim)].shape)
    rec = make(model, dim, scheme, gam, "exact")
    _set_values(rec, bv, dim)
    Qg = torch.from_numpy(Qfull.copy()).cuda()
    integ = flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(list(domain), dx, Qg), list(periodic))
    integ.advance(dt, nsteps=nsteps, checkpoint_every=every)
    g_one = integ.adjoint(torch.from_numpy(Wfull.copy()).cuda()).cpu().numpy()
    shape = lambda n: (Qfull.shape[0],) + tuple(n[a] + 8 if a < dim else 1 for a in (2, 1, 0))
    states = []
    for lo, n in boxes:
        Q = np.zeros(shape(n))
        Q[_inner(dim)] = _box(Qfull, lo, n, dim, False)
        states.append(torch.from_numpy(Q).cuda())
    lv = _level(rec, boxes, dx, domain, periodic, states)
    lv.advance(dt, nsteps=nsteps, checkpoint_every=every)
    Wp = []
    for lo, n in boxes:
        w = np.zeros(shape(n))
        w[_inner(dim)] = _box(Wfull, lo, n, dim, False)
        Wp.append(torch.from_numpy(w).cuda())
    g_lv = lv.adjoint(Wp)
    torch.cuda.synchronize()
    lv.check()
    got = np.zeros_like(Qfull)
    for (lo, n), gp in zip(boxes, g_lv):
        _box(got, lo, n, dim, False)[...] = gp.cpu().numpy()[_inner(dim)]
    err = rel_err(got[_inner(dim)], g_one[_inner(dim)])
    assert err <= 1e-12, f"level adjoint vs one patch: {err:.3e}"
    lv.close()
    rec.close()


@pytest.mark.gpu
def test_dirichlet_values_are_checked(cuda):
    model, dim, scheme, _, gam = VARIANTS[0]
    rec = make(model, dim, scheme, gam, "exact")
    with pytest.raises(ValueError):
        rec.setDirichletValues(0, 0, [1.0] * (rec.ncomp - 1))
    with pytest.raises(RuntimeError):
        rec.setDirichletValues(0, 0, [1.0, float("nan")] + [1.0] * (rec.ncomp - 2))
    with pytest.raises(RuntimeError):
        rec.setDirichletValues(dim, 0, [1.0] * rec.ncomp)
    with pytest.raises(RuntimeError):
        rec.setDirichletValues(0, 2, [1.0] * rec.ncomp)
    rec.setDirichletValues(1, 1, [1.0] * rec.ncomp)
    rec.close()
