"""Golden fixtures of the convective path (tests/golden/convective_fixtures.npz).

The fixtures freeze the oracle's output on small seeded inputs for all 12
variants (see tests/golden/make_golden.py).  The CPU test checks that the
oracle still reproduces them bit for bit (x86 and Arm alike: the oracle is
built with -ffp-contract=off and uses only correctly rounded operations); the
GPU test checks the exact form of the CUDA path against the stored values
directly, without running the oracle.
"""
import os

import numpy as np
import pytest

from tests.golden import make_golden as G

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convective_fixtures.npz")
CASES = list(G.cases())
IDS = ["%s-%dd-%s" % (c[1], c[4], c[6]) for c in CASES]


@pytest.fixture(scope="module")
def golden():
    return np.load(FIXTURES)


def test_oracle_reproduces_golden_fixtures(golden):
    fresh = G.compute()
    assert sorted(fresh) == sorted(golden.files)
    for k in golden.files:
        assert np.array_equal(fresh[k], golden[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_exact_form_matches_golden_fixtures(cuda, golden, case):
    import torch
    from hamers_gb300 import flow
    model, mname, gam, R, dim, scheme, sname = case
    names = {0: "SINGLE_SPECIES", 1: "FOUR_EQN_CONSERVATIVE", 2: "FIVE_EQN_ALLAIRE"}
    fm = flow.FlowModel(names[model], dim, gam, species_R=R)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL" if scheme == 0 else "WCNS6_LD_HLLC_HLL", fm,
                                           precision="exact")
    for label in ("smooth", "shock"):
        key = f"{mname}_{dim}d_{sname}_{label}"
        n, Q = G.inputs(model, dim, gam, label)
        dx = [1.0 / v for v in n]
        patch = flow.Patch(n, dx, torch.from_numpy(Q).cuda())
        F, S = rec.allocateFlux(patch), rec.allocateSource(patch)
        rec.readCounters()
        rec.computeConvectiveFluxAndSourceOnPatch(patch, F, S, G.DT)
        torch.cuda.synchronize()
        for a in range(dim):
            assert np.array_equal(F[a].cpu().numpy(), golden[f"{key}_flux{a}"]), f"{key} flux {a}"
        assert np.array_equal(S.cpu().numpy(), golden[f"{key}_source"]), f"{key} source"
        assert tuple(rec.readCounters()) == tuple(golden[f"{key}_counters"]), f"{key} counters"
        Qs = torch.from_numpy(Q).cuda()
        integ = flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qs), [1] * dim)
        integ.advance(G.DT, nsteps=1)
        torch.cuda.synchronize()
        sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
        assert np.array_equal(Qs.cpu().numpy()[sl], golden[f"{key}_rk3"]), f"{key} rk3"
