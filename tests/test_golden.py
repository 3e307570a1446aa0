"""Golden fixtures of the convective path (tests/golden/convective_fixtures.npz).

The convective face fluxes and sources of all 24 variants are the output of the reference's own
code (its translation units compiled by oracle/refshim/Makefile) on small seeded inputs; the face
counters, the SSPRK3 steps and the Navier-Stokes fixtures are the oracle's (see
tests/golden/make_golden.py).  The CPU tests check that the oracle reproduces every fixture bit
for bit (x86 and Arm alike: it is built with -ffp-contract=off and uses only correctly rounded
operations) and, where the reference sources are present, that the reference's code still
produces the stored fluxes; the GPU test checks the exact form of the CUDA path against the
stored values directly, without running either.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden import make_golden as G

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convective_fixtures.npz")
CASES = list(G.cases())
IDS = ["%s-%dd-%s" % (c[1], c[4], c[6]) for c in CASES]


@pytest.fixture(scope="module")
def golden():
    return np.load(FIXTURES)


def test_oracle_reproduces_golden_fixtures(golden):
    fresh = G.compute(fluxes_from="oracle")
    assert sorted(fresh) == sorted(golden.files)
    for k in golden.files:
        assert np.array_equal(fresh[k], golden[k]), k


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
def test_reference_reproduces_golden_fluxes(golden):
    fresh = G.compute(fluxes_from="reference")
    for k in golden.files:
        if "_flux" in k or k.endswith("_source"):
            assert np.array_equal(fresh[k], golden[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_exact_form_matches_golden_fixtures(cuda, golden, case):
    import torch
    from hamers_gb300 import flow
    model, mname, gam, R, dim, scheme, sname = case
    names = {0: "SINGLE_SPECIES", 1: "FOUR_EQN_CONSERVATIVE", 2: "FIVE_EQN_ALLAIRE"}
    fm = flow.FlowModel(names[model], dim, gam, species_R=R)
    rname = {0: "WCNS5_JS_HLLC_HLL", 1: "WCNS6_LD_HLLC_HLL", 2: "WCNS5_Z_HLLC_HLL", 3: "WCNS6_CU_M2_HLLC_HLL"}[scheme]
    n0, _ = G.inputs(model, dim, gam, "smooth")
    rec = flow.ConvectiveFluxReconstructor(rname, fm, precision="exact", grid_geometry=[1.0 / v for v in n0])
    for label in G.LABELS:
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
        if label == "rough":
            continue
        Qs = torch.from_numpy(Q).cuda()
        integ = flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qs), [1] * dim)
        integ.advance(G.DT, nsteps=1)
        torch.cuda.synchronize()
        sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
        assert np.array_equal(Qs.cpu().numpy()[sl], golden[f"{key}_rk3"]), f"{key} rk3"


NS_CASES = list(G.ns_cases())


@pytest.mark.gpu
@pytest.mark.parametrize("case", NS_CASES, ids=["%dd-o%d" % c for c in NS_CASES])
def test_navier_stokes_matches_golden_fixtures(cuda, golden, case):
    import torch
    from hamers_gb300 import flow
    dim, order = case
    t = G.NS_TRANSPORT
    fm = flow.FlowModel("SINGLE_SPECIES", dim, [1.4], transport={
        "species_mu": t["mu"], "species_mu_v": t["mu_v"], "species_c_p": t["c_p"], "species_Pr": t["Pr"]})
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision="exact",
                                           diffusive_flux_reconstructor="MIDPOINT_FOURTH_ORDER" if order == 4
                                           else "MIDPOINT_SECOND_ORDER")
    ns = flow.NavierStokes(rec)
    for label in ("smooth", "shock"):
        key = f"ns_{dim}d_o{order}_{label}"
        n, Q = G.inputs(0, dim, [1.4], label)
        dx = [1.0 / v for v in n]
        patch = flow.Patch(n, dx, torch.from_numpy(Q).cuda())
        F = rec.allocateFlux(patch)
        ns.diff.computeDiffusiveFluxOnPatch(patch, F, G.DT)
        torch.cuda.synchronize()
        for a in range(dim):
            assert np.array_equal(F[a].cpu().numpy(), golden[f"{key}_dflux{a}"]), f"{key} flux {a}"
        Qs = torch.from_numpy(Q).cuda()
        flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qs), [1] * dim).advance(G.DT, nsteps=1)
        torch.cuda.synchronize()
        sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
        assert np.array_equal(Qs.cpu().numpy()[sl], golden[f"{key}_rk3"]), f"{key} rk3"
    rec.close()
