"""Generates the golden fixtures of the convective path.

The reference ships no golden flux vectors (its tests pin only the order of accuracy), so these
fixtures are made here on small seeded inputs.  For each of the 24 variants (model x dimension x
scheme: WCNS5-JS, WCNS6-LD, WCNS5-Z, WCNS6-CU-M2):

  * the dt-scaled face fluxes and the source of computeConvectiveFluxAndSourceOnPatch on a
    smooth, a shock and a rough (fallback-heavy) state come from the REFERENCE'S OWN CODE --
    its translation units compiled by oracle/refshim/Makefile into oracle/_ref/libhmr_ref.so;
  * the fallback and HLLC-HLL face counters (the reference does not count them) and the interior
    state after one SSPRK3 step with periodic ghost fill (smooth and shock states; the RK stage
    of Euler::advanceSingleStepOnPatch is not among the compiled units) come from the oracle.

For the Navier-Stokes path (single species, 2D/3D, second and fourth order) the diffusive face
fluxes and one NavierStokes SSPRK3 step come from the oracle.  The inputs are regenerated from
their seeds (tests/helpers.py, tests/test_ref_oracle.py).

    python tests/golden/make_golden.py      # rewrites tests/golden/convective_fixtures.npz
                                            # (needs the reference sources for the fluxes)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from hamers_gb300 import problems as P  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import rough_state, shock_state, smooth_state  # noqa: E402

OUT = os.path.join(HERE, "convective_fixtures.npz")

MODELS = [(O.MODEL_SINGLE_SPECIES, "single", [1.4], None),
          (O.MODEL_FOUR_EQN_CONSERVATIVE, "four", P.FOUR_EQN_GAMMA, P.FOUR_EQN_R),
          (O.MODEL_FIVE_EQN_ALLAIRE, "five", [1.4, 1.67], None)]
SIZES = {2: (8, 6), 3: (4, 4, 4)}
DT = 1.3e-3


SCHEMES = ((O.SCHEME_WCNS5_JS, "js"), (O.SCHEME_WCNS6_LD, "ld"), (O.SCHEME_WCNS5_Z, "z"),
           (O.SCHEME_WCNS6_CU_M2, "cu"))
NS_TRANSPORT = dict(mu=0.02, c_p=3.5, Pr=0.72, mu_v=0.005)


def cases():
    for model, mname, gam, R in MODELS:
        for dim in (2, 3):
            for scheme, sname in SCHEMES:
                yield model, mname, gam, R, dim, scheme, sname


def ns_cases():
    for dim in (2, 3):
        for order in (2, 4):
            yield dim, order


def ns_transport(order):
    t = NS_TRANSPORT
    return O.Transport(t["mu"], t["c_p"], t["Pr"], mu_v=t["mu_v"], order=order)


LABELS = ("smooth", "shock", "rough")


def inputs(model, dim, gam, label):
    n = SIZES[dim]
    gen = {"smooth": smooth_state, "shock": shock_state, "rough": rough_state}[label]
    return n, gen(model, dim, n, seed=7, species_gamma=gam)


def compute(fluxes_from="reference"):
    """All fixtures; the convective fluxes and sources from the reference's compiled code
    (fluxes_from="reference") or from the oracle ("oracle")."""
    out = {}
    for model, mname, gam, R, dim, scheme, sname in cases():
        for label in LABELS:
            key = f"{mname}_{dim}d_{sname}_{label}"
            n, Q = inputs(model, dim, gam, label)
            dx = [1.0 / v for v in n]
            cfg = O.Config(model, dim, gam, scheme, species_R=R, grid_dx=dx)
            F, S, st = O.conv_flux_source(cfg, n, dx, DT, Q)
            if fluxes_from == "reference":
                F, S = O.ref_conv_flux_source(cfg, n, dx, DT, Q)
            for a, f in enumerate(F):
                out[f"{key}_flux{a}"] = f
            out[f"{key}_source"] = S
            out[f"{key}_counters"] = np.array(st[1:], dtype=np.int64)
            if label == "rough":
                continue   # no time step: the rough state's sound speeds are far above this dt's CFL bound
            Qs = Q.copy()
            O.fill_ghosts(cfg, n, [1] * dim, Qs)
            O.rk3_advance(cfg, n, dx, DT, [1] * dim, 1, Qs)
            sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
            out[f"{key}_rk3"] = np.ascontiguousarray(Qs[sl])
    for dim, order in ns_cases():
        cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4])
        for label in ("smooth", "shock"):
            key = f"ns_{dim}d_o{order}_{label}"
            n, Q = inputs(O.MODEL_SINGLE_SPECIES, dim, [1.4], label)
            dx = [1.0 / v for v in n]
            for a, f in enumerate(O.diff_flux(cfg, ns_transport(order), n, dx, DT, Q)):
                out[f"{key}_dflux{a}"] = f
            Qs = Q.copy()
            O.fill_ghosts(cfg, n, [1] * dim, Qs)
            O.ns_rk3_advance(cfg, ns_transport(order), n, dx, DT, [1] * dim, 1, Qs)
            sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
            out[f"{key}_rk3"] = np.ascontiguousarray(Qs[sl])
    return out


if __name__ == "__main__":
    O.build()
    np.savez_compressed(OUT, **compute())
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
