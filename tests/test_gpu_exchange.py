"""Device-resident ghost exchange between the patches of a level (hmr_level_set_layout).

A level tiled by uneven patches and advanced by the batched substeps, with ghost
cells copied from neighbouring patches and periodic images and zero-gradient at
the domain's other faces, must reproduce -- bitwise, in the exact form -- the
oracle's single patch covering the whole domain.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import smooth_state
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg

CASES = [(0, (40, 36), (0, 1)), (5, (34, 30), (1, 0)), (2, (16, 14, 12), (1, 1, 1)), (10, (15, 13, 12), (0, 1, 0))]
CASE_IDS = ["%s-%s" % (IDS[i], "".join(map(str, per))) for i, _, per in CASES]


def _tile(length, rng, lo=4, hi=13):
    segs, r = [], length
    while r > hi:
        s = int(rng.integers(lo, min(hi, r - lo) + 1))
        segs.append(s)
        r -= s
    segs.append(r)
    return segs


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=CASE_IDS)
def test_tiled_level_equals_one_patch(cuda, case):
    import torch
    from hamers_gb300 import flow
    vi, domain, periodic = case
    model, dim, scheme, _, gam = VARIANTS[vi]
    cfg = ocfg(model, dim, gam, scheme)
    dx = [1.0 / v for v in domain]
    dt, nsteps = 1.0e-3, 2
    Qfull = smooth_state(model, dim, domain, seed=17, species_gamma=gam)
    Qo = Qfull.copy()
    O.fill_ghosts(cfg, domain, list(periodic), Qo)
    O.rk3_advance(cfg, domain, dx, dt, list(periodic), nsteps, Qo)

    rng = np.random.default_rng(3)
    segs = [_tile(domain[a], rng, 4, 13 if dim == 2 else 7) for a in range(dim)]
    starts = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(int) for s in segs]
    boxes = []
    for idx in np.ndindex(*[len(s) for s in segs]):
        lo = [int(starts[a][idx[a]]) for a in range(dim)]
        n = [int(segs[a][idx[a]]) for a in range(dim)]
        boxes.append((lo, n))
    assert len(boxes) >= 6

    def block(Q, lo, n, ghosts):
        g = 4 if ghosts else 0
        sl = [slice(None)]
        for a in (2, 1, 0):
            if a < dim:
                sl.append(slice(lo[a] + 4 - g, lo[a] + 4 + n[a] + g))
            else:
                sl.append(slice(None))
        return Q[tuple(sl)]

    states = []
    for lo, n in boxes:
        shape = (Qfull.shape[0],) + tuple(n[a] + 8 if a < dim else 1 for a in (2, 1, 0))
        Q = np.zeros(shape)
        inner = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
        Q[inner] = block(Qfull, lo, n, False)
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
    inner = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
    for (lo, n), Q in zip(boxes, states):
        got = Q.cpu().numpy()[inner]
        ref = block(Qo, lo, n, False)
        assert np.array_equal(got, ref), f"patch at {lo}: max diff {np.abs(got - ref).max()}"
    lv.close()
