"""Reflecting (slip) walls in the oracle's ghost fill.

The reference fills a REFLECT edge cell-by-cell from its mirror image across the
boundary face (BasicCartesianBoundaryUtilities2.cpp:349-395): the pivot of ghost
cell lo-1-d is interior cell lo+d, and the momentum component normal to the edge
is negated, the scalars copied (EulerBoundaryConditions.cpp:205-297 sends the
momentum to the vector routine and density/energy/fractions to the SYMMETRY one).
Corners are filled afterwards by the node conditions XREFLECT or YREFLECT
(:779-840), which mirror along one axis only, reading the edge ghost cells filled
before.  Either choice gives the same corner: the mirror image across both faces
with both normal components negated.  The oracle fills every ghost cell at once
from that composite rule; the first test restates the reference's two-pass
procedure in numpy and requires the two to agree for both corner conditions.

The remaining tests check the physics of the closed box: with reflecting walls on
every face no mass, species mass or energy crosses the boundary.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import shock_state, smooth_state
from tests.test_gpu_parity import ocfg

G = 4
MODELS = [(O.MODEL_SINGLE_SPECIES, [1.4]), (O.MODEL_FIVE_EQN_ALLAIRE, [1.4, 1.67]),
          (O.MODEL_FOUR_EQN_CONSERVATIVE, None)]


def _gam(gam):
    from hamers_gb300 import problems as P
    return gam if gam is not None else P.FOUR_EQN_GAMMA


def _mom0(model, nsp):
    return 1 if model == O.MODEL_SINGLE_SPECIES else nsp


def _reference_two_pass_2d(Q, n, mom0, corner_axis):
    """Edges (cells outside the box along one axis only), then corners by XREFLECT
    (corner_axis 0) or YREFLECT (1), as BasicCartesianBoundaryUtilities2 orders them."""
    Q = Q.copy()
    nx, ny = n
    gx = lambda i: i + G
    # x edges: ghost columns beside the interior rows
    for j in range(ny):
        for d in range(G):
            for i, piv in ((-1 - d, d), (nx + d, nx - 1 - d)):
                Q[:, 0, gx(j), gx(i)] = Q[:, 0, gx(j), gx(piv)]
                Q[mom0, 0, gx(j), gx(i)] = -Q[mom0, 0, gx(j), gx(piv)]
    # y edges
    for i in range(nx):
        for d in range(G):
            for j, piv in ((-1 - d, d), (ny + d, ny - 1 - d)):
                Q[:, 0, gx(j), gx(i)] = Q[:, 0, gx(piv), gx(i)]
                Q[mom0 + 1, 0, gx(j), gx(i)] = -Q[mom0 + 1, 0, gx(piv), gx(i)]
    # corners: mirror along corner_axis only, from the edge ghosts filled above
    for j in list(range(-G, 0)) + list(range(ny, ny + G)):
        for i in list(range(-G, 0)) + list(range(nx, nx + G)):
            if corner_axis == 0:
                pi = -1 - i if i < 0 else 2 * nx - 1 - i
                src = Q[:, 0, gx(j), gx(pi)].copy()
                src[mom0] = -src[mom0]
            else:
                pj = -1 - j if j < 0 else 2 * ny - 1 - j
                src = Q[:, 0, gx(pj), gx(i)].copy()
                src[mom0 + 1] = -src[mom0 + 1]
            Q[:, 0, gx(j), gx(i)] = src
    return Q


@pytest.mark.parametrize("model,gam", MODELS, ids=["single", "five", "four"])
def test_reflect_fill_matches_reference_procedure(model, gam):
    gam = _gam(gam)
    cfg = ocfg(model, 2, gam, O.SCHEME_WCNS6_LD)
    for n in ((9, 7), (4, 4), (12, 5)):
        Q = smooth_state(model, 2, n, seed=11, species_gamma=gam)
        mom0 = _mom0(model, len(gam))
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, [3, 3], Qo)
        for corner_axis in (0, 1):
            ref = _reference_two_pass_2d(Q, n, mom0, corner_axis)
            assert np.array_equal(Qo, ref), (n, corner_axis)


@pytest.mark.parametrize("model,gam", MODELS, ids=["single", "five", "four"])
def test_reflect_fill_3d_mixed_axes(model, gam):
    """3D: reflect, zero-gradient and periodic axes mixed; every ghost cell is the composite
    image (mirror / clamp / wrap per axis) with the normal momentum of each reflecting axis
    on which the cell lies outside negated."""
    gam = _gam(gam)
    cfg = ocfg(model, 3, gam, O.SCHEME_WCNS5_JS)
    n = (6, 5, 4)
    mom0 = _mom0(model, len(gam))
    for per in ([3, 0, 1], [1, 3, 3], [3, 3, 3]):
        Q = smooth_state(model, 3, n, seed=5, species_gamma=gam)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, per, Qo)

        def src(v, a):
            if 0 <= v < n[a]:
                return v
            if per[a] == 1:
                return v % n[a]
            if per[a] == 3:
                return -1 - v if v < 0 else 2 * n[a] - 1 - v
            return 0 if v < 0 else n[a] - 1

        for k in range(-G, n[2] + G):
            for j in range(-G, n[1] + G):
                for i in range(-G, n[0] + G):
                    c = (i, j, k)
                    if all(0 <= c[a] < n[a] for a in range(3)):
                        continue
                    v = Q[:, src(k, 2) + G, src(j, 1) + G, src(i, 0) + G].copy()
                    for a in range(3):
                        if per[a] == 3 and not 0 <= c[a] < n[a]:
                            v[mom0 + a] = -v[mom0 + a]
                    assert np.array_equal(Qo[:, k + G, j + G, i + G], v), (per, c)


def _totals(model, nsp, Q, dim):
    inner = (slice(None),) + tuple(slice(G, -G) if a < dim else slice(None) for a in (2, 1, 0))
    Qi = Q[inner]
    ne = 1 if model == O.MODEL_SINGLE_SPECIES else nsp
    return [float(np.sum(Qi[e])) for e in range(ne)] + [float(np.sum(Qi[ne + dim]))]


@pytest.mark.parametrize("scheme", [O.SCHEME_WCNS5_JS, O.SCHEME_WCNS6_LD], ids=["js", "ld"])
@pytest.mark.parametrize("model,gam", MODELS, ids=["single", "five", "four"])
def test_closed_box_conserves_mass_and_energy(model, gam, scheme):
    """A shock state in a box with reflecting walls on every face: three SSPRK3 steps leave
    the total (species) mass and the total energy unchanged to rounding.  Control: with
    zero-gradient (outflow) faces the same run changes them by far more."""
    gam = _gam(gam)
    nsp = len(gam)
    for dim, n in ((2, (24, 20)), (3, (10, 9, 8))):
        cfg = ocfg(model, dim, gam, scheme)
        dx = [1.0 / v for v in n]
        dt = 2.0e-3
        drift = {}
        for per in ([3] * dim, [0] * dim):
            Q = shock_state(model, dim, n, seed=2, species_gamma=gam)
            O.fill_ghosts(cfg, n, per, Q)
            t0 = _totals(model, nsp, Q, dim)
            O.rk3_advance(cfg, n, dx, dt, per, 3, Q)
            t1 = _totals(model, nsp, Q, dim)
            drift[per[0]] = max(abs(b - a) / abs(a) for a, b in zip(t0, t1))
        assert drift[3] <= 1e-13, (dim, drift)
        assert drift[0] > 1e3 * max(drift[3], 1e-16), (dim, drift)
