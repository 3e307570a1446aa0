"""Reflecting (slip) walls on the device (HMR_FILL_REFLECT).

* the single-patch ghost fill equals the oracle's bitwise, with reflecting walls mixed with
  zero-gradient and periodic axes, for every flow model in 2D and 3D;
* two SSPRK3 steps of one patch in a reflecting box equal the oracle's bitwise (exact form);
* the adjoint of the fill passes the dot-product test <w, F v> = <F^T w, v>;
* a level tiled by uneven patches with reflecting domain faces, advanced by the batched
  substeps with the device ghost exchange, equals the oracle's single patch covering the
  domain bitwise (exact form);
* a reflecting axis narrower than the ghost width is rejected.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rough_state, shock_state, smooth_state
from tests.test_gpu_exchange import _tile
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg

PER_2D = ([3, 3], [3, 1], [0, 3])
PER_3D = ([3, 3, 3], [3, 0, 1], [1, 3, 0])


def _pers(dim):
    return PER_2D if dim == 2 else PER_3D


@pytest.mark.gpu
@pytest.mark.parametrize("variant", VARIANTS, ids=IDS)
def test_reflect_fill_bitwise(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    eu = flow.Euler(rec)
    for per in _pers(dim):
        for Q in (smooth_state(model, dim, n, seed=21, species_gamma=gam),
                  rough_state(model, dim, n, seed=22, species_gamma=gam)):
            Qo = Q.copy()
            O.fill_ghosts(cfg, n, per, Qo)
            Qg = torch.from_numpy(Q).cuda()
            eu.fillGhosts(flow.Patch(n, [1.0] * dim, Qg), per)
            torch.cuda.synchronize()
            assert np.array_equal(Qg.cpu().numpy(), Qo), per
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (1, 3, 5, 7, 9)], ids=[IDS[i] for i in (1, 3, 5, 7, 9)])
def test_reflect_box_rk3_bitwise(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    dx = [1.0 / v for v in n]
    for per in _pers(dim)[:2]:
        Q = shock_state(model, dim, n, seed=23, species_gamma=gam)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo)
        O.rk3_advance(cfg, n, dx, 1e-3, per, 2, Qo)
        Qg = torch.from_numpy(Q).cuda()
        flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qg), per).advance(1e-3, nsteps=2)
        assert np.array_equal(Qg.cpu().numpy(), Qo), per
    rec.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (0, 6, 9)], ids=[IDS[i] for i in (0, 6, 9)])
def test_reflect_fill_vjp_dot_product(cuda, variant):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    eu = flow.Euler(make(model, dim, scheme, gam, "exact"))
    rng = np.random.default_rng(8)
    for per in _pers(dim):
        v = rng.standard_normal(O.ghost_shape(cfg, n))
        w = rng.standard_normal(v.shape)
        Fv = v.copy()
        O.fill_ghosts(cfg, n, per, Fv)
        tw = torch.from_numpy(w).cuda()
        eu.fillGhostsVJP(flow.Patch(n, [1.0] * dim, tw), per)
        torch.cuda.synchronize()
        lhs, rhs = float(np.sum(w * Fv)), float(np.sum(tw.cpu().numpy() * v))
        assert abs(lhs - rhs) <= 1e-12 * float(np.sum(np.abs(w * Fv))), (per, lhs, rhs)


LEVEL_CASES = [(1, (36, 30), (3, 3)), (4, (34, 28), (3, 1)), (3, (15, 13, 12), (3, 1, 3)), (9, (32, 27), (0, 3))]
LEVEL_IDS = ["%s-%s" % (IDS[i], "".join(map(str, per))) for i, _, per in LEVEL_CASES]


@pytest.mark.gpu
@pytest.mark.parametrize("case", LEVEL_CASES, ids=LEVEL_IDS)
def test_tiled_level_reflect_equals_one_patch(cuda, case):
    import torch
    from hamers_gb300 import flow
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    cfg = ocfg(model, dim, gam, scheme)
    dx = [1.0 / v for v in domain]
    dt, nsteps = 1.0e-3, 2
    Qfull = shock_state(model, dim, domain, seed=29, species_gamma=gam)
    Qo = Qfull.copy()
    O.fill_ghosts(cfg, domain, list(periodic), Qo)
    O.rk3_advance(cfg, domain, dx, dt, list(periodic), nsteps, Qo)

    rng = np.random.default_rng(5)
    # patches as thin as one cell along a reflecting axis: their wall ghosts mirror cells of
    # the neighbouring patch, copied into their own ghost box by the exchange first
    segs = [_tile(domain[a], rng, 1 if dim == 2 else 2, 13 if dim == 2 else 7) for a in range(dim)]
    starts = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(int) for s in segs]
    boxes = []
    for idx in np.ndindex(*[len(s) for s in segs]):
        boxes.append(([int(starts[a][idx[a]]) for a in range(dim)], [int(segs[a][idx[a]]) for a in range(dim)]))

    def block(Q, lo, n):
        sl = [slice(None)]
        for a in (2, 1, 0):
            sl.append(slice(lo[a] + 4, lo[a] + 4 + n[a]) if a < dim else slice(None))
        return Q[tuple(sl)]

    inner = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
    states = []
    for lo, n in boxes:
        Q = np.zeros((Qfull.shape[0],) + tuple(n[a] + 8 if a < dim else 1 for a in (2, 1, 0)))
        Q[inner] = block(Qfull, lo, n)
        states.append(torch.from_numpy(Q).cuda())
    rec = make(model, dim, scheme, gam, "exact")
    lv = flow.BatchedLevel(rec, [(n, dx) for _, n in boxes])
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


@pytest.mark.gpu
def test_reflect_needs_ghost_width(cuda):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = VARIANTS[0]
    rec = make(model, dim, scheme, gam, "exact")
    eu = flow.Euler(rec)
    n = (3, 9)
    Qg = torch.from_numpy(smooth_state(model, dim, n, seed=1, species_gamma=gam)).cuda()
    with pytest.raises(RuntimeError):
        eu.fillGhosts(flow.Patch(n, [1.0] * dim, Qg), [3, 0])
    eu.fillGhosts(flow.Patch(n, [1.0] * dim, Qg), [0, 3])
    lv = flow.BatchedLevel(rec, [((3, 9), [0.1, 0.1])])
    with pytest.raises(RuntimeError):
        lv.set_periodic(0, [3, 1])
    with pytest.raises(RuntimeError):
        lv.set_layout([[0, 0]], [3, 9], [3, 0])
    lv.set_layout([[0, 0]], [3, 9], [0, 3])
    lv.close()
    rec.close()
