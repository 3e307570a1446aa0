"""Adjoint over a whole level: the ghost fill's adjoint with a layout (hmr_level_fill_vjp) and
the checkpointed reverse sweep of the batched form (BatchedLevel.advance / adjoint).

* the fill's adjoint passes the dot-product test <w, F v> = <F^T w, v>, F being the level's
  ghost fill (neighbour and periodic-image copies, then the physical faces: zero-gradient and
  reflecting walls), evaluated on the CPU by the oracle's fill of the whole domain;
* a level tiled by uneven patches equals one patch covering the domain in the forward (exact
  form, bitwise), so its reverse sweep over several steps must give that patch's adjoint:
  the per-patch integrator's, to rounding (the fill's adjoint sums by atomic additions).

The 2D sweeps start from the Taylor-Green state (tests/helpers.py vortex_state), on which no
face selects HLLC-HLL.  Where the sensor does select it on smooth data, the blending weights
depend on the direction of a near-zero velocity jump and their derivatives (of order
1/|jump|) cancel between the two sides of the face, so summing a face's contributions per
tile instead of once changes the adjoint by far more than rounding: on the multi-species
smooth states of tests/helpers.py splitting the adjoint seed into the tiles' parts alone
moves the one-patch VJP by about 1e-5 of its size.  The 3D sweep (single species, odd
sizes) selects no HLLC-HLL face on its smooth state.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err, smooth_state, vortex_state
from tests.test_gpu_exchange import _tile
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg

G = 4
CASES = [(1, (30, 26), (1, 3)), (5, (28, 24), (3, 0)), (3, (13, 12, 11), (1, 3, 0)), (9, (26, 22), (1, 1))]
CASE_IDS = ["%s-%s" % (IDS[i], "".join(map(str, per))) for i, _, per in CASES]


def _layout(dim, domain, seed):
    rng = np.random.default_rng(seed)
    segs = [_tile(domain[a], rng, 2, 11 if dim == 2 else 6) for a in range(dim)]
    starts = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(int) for s in segs]
    boxes = []
    for idx in np.ndindex(*[len(s) for s in segs]):
        boxes.append(([int(starts[a][idx[a]]) for a in range(dim)], [int(segs[a][idx[a]]) for a in range(dim)]))
    return boxes


def _box(Q, lo, n, dim, ghosts):
    """The sub-array of a full-domain ghost-box array covering a patch (with or without its ghosts)."""
    g = G if ghosts else 0
    sl = [slice(None)]
    for a in (2, 1, 0):
        sl.append(slice(lo[a] + G - g, lo[a] + G + n[a] + g) if a < dim else slice(None))
    return Q[tuple(sl)]


def _inner(dim):
    return (slice(None),) + tuple(slice(G, -G) if a < dim else slice(None) for a in (2, 1, 0))


def _level(rec, boxes, dx, domain, periodic, states):
    from hamers_gb300 import flow
    lv = flow.BatchedLevel(rec, [(n, dx) for _, n in boxes])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
    lv.set_layout([lo for lo, _ in boxes], list(domain), list(periodic))
    return lv


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=CASE_IDS)
def test_level_fill_vjp_dot_product(cuda, case):
    import torch
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    cfg = ocfg(model, dim, gam, scheme)
    boxes = _layout(dim, domain, 3)
    rng = np.random.default_rng(17)
    shape = lambda n: (cfg.ncomp,) + tuple(n[a] + 2 * G if a < dim else 1 for a in (2, 1, 0))
    V = [rng.standard_normal(shape(n)) for _, n in boxes]
    W = [rng.standard_normal(shape(n)) for _, n in boxes]
    # F v: the patches' interiors assembled into the domain, filled as one patch, cut back out
    full = np.zeros(O.ghost_shape(cfg, domain))
    for (lo, n), v in zip(boxes, V):
        _box(full, lo, n, dim, False)[...] = v[_inner(dim)]
    O.fill_ghosts(cfg, domain, list(periodic), full)
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
@pytest.mark.parametrize("case", CASES, ids=CASE_IDS)
def test_level_reverse_sweep_equals_one_patch(cuda, case):
    import torch
    from hamers_gb300 import flow
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    dx = [1.0 / v for v in domain]
    dt, nsteps, every = 1.0e-3, 4, 2
    gen = vortex_state if dim == 2 else smooth_state
    Qfull = gen(model, dim, domain, seed=21, species_gamma=gam)
    boxes = _layout(dim, domain, 5)
    # objective: J = sum over the domain's interior of a seeded weight times the final state
    rng = np.random.default_rng(23)
    Wfull = np.zeros_like(Qfull)
    Wfull[_inner(dim)] = rng.standard_normal(Wfull[_inner(dim)].shape)

    rec = make(model, dim, scheme, gam, "exact")
    # one patch covering the domain, per-patch integrator
    Qg = torch.from_numpy(Qfull.copy()).cuda()
    integ = flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(list(domain), dx, Qg), list(periodic))
    integ.advance(dt, nsteps=nsteps, checkpoint_every=every)
    g_one = integ.adjoint(torch.from_numpy(Wfull.copy()).cuda()).cpu().numpy()
    final_one = Qg.cpu().numpy()

    # the tiled level
    shape = lambda n: (Qfull.shape[0],) + tuple(n[a] + 2 * G if a < dim else 1 for a in (2, 1, 0))
    states = []
    for lo, n in boxes:
        Q = np.zeros(shape(n))
        Q[_inner(dim)] = _box(Qfull, lo, n, dim, False)
        states.append(torch.from_numpy(Q).cuda())
    lv = _level(rec, boxes, dx, domain, periodic, states)
    lv.advance(dt, nsteps=nsteps, checkpoint_every=every)
    torch.cuda.synchronize()
    lv.check()
    for (lo, n), Q in zip(boxes, states):
        assert np.array_equal(Q.cpu().numpy()[_inner(dim)], _box(final_one, lo, n, dim, False))
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
    assert np.abs(g_one[_inner(dim)]).max() > 0.0
    lv.close()
    rec.close()
