"""The oracle restatement against the reference's own code.

oracle/refshim/Makefile compiles the reference's hot-path translation units unmodified and in
place -- the WCNS56 driver and its WCNS5-JS / WCNS6-LD / WCNS5-Z / WCNS6-CU-M2 reconstructors
(src/flow/convective_flux_reconstructors/WCNS56/), the three flow models with their basic
utilities and HLLC / HLLC-HLL Riemann solvers (src/flow/flow_models/), the ideal-gas equation of
state and mixing rules (src/util/mixing_rules/), and the first-order derivative of the shock
sensor (src/util/derivatives/) -- against a stand-in for the SAMRAI API, into
oracle/_ref/libhmr_ref.so.  These tests run ConvectiveFluxReconstructorWCNS56::
computeConvectiveFluxAndSourceOnPatch from that library and the oracle's restatement on the
same inputs and require every face flux and source value to be bitwise equal.  They need the
reference sources (or a library built from them) and skip without them.
"""
import numpy as np
import pytest

from hamers_gb300 import problems as P
from oracle import oracle as O
from tests.helpers import noisy_shock_state, rough_state, shock_state, smooth_state, vortex_state

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")

MODELS = [(O.MODEL_SINGLE_SPECIES, "single", [1.4], None),
          (O.MODEL_FOUR_EQN_CONSERVATIVE, "four", list(P.FOUR_EQN_GAMMA), list(P.FOUR_EQN_R)),
          (O.MODEL_FIVE_EQN_ALLAIRE, "five", [1.4, 1.67], None)]
SCHEMES = [(O.SCHEME_WCNS5_JS, "js"), (O.SCHEME_WCNS6_LD, "ld"), (O.SCHEME_WCNS5_Z, "z"),
           (O.SCHEME_WCNS6_CU_M2, "cu")]
CASES = [(m, mn, g, r, d, s, sn) for (m, mn, g, r) in MODELS for d in (2, 3) for (s, sn) in SCHEMES]
IDS = ["%s-%dd-%s" % (c[1], c[4], c[6]) for c in CASES]


STATES = {"smooth": smooth_state, "shock": shock_state, "noisy": noisy_shock_state, "rough": rough_state}


def run_both(model, dim, gam, R, scheme, n, Q, dt=1.3e-3):
    dx = [1.0 / v for v in n]
    cfg = O.Config(model, dim, gam, scheme, species_R=R, grid_dx=dx)
    fo, so, stats = O.conv_flux_source(cfg, n, dx, dt, Q)
    fr, sr = O.ref_conv_flux_source(cfg, n, dx, dt, Q)
    return fo, so, fr, sr, stats


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oracle_is_bitwise_the_reference(case):
    model, _, gam, R, dim, scheme, _ = case
    n = [13, 11] if dim == 2 else [9, 8, 7]
    for label, gen in STATES.items():
        Q = gen(model, dim, n, seed=3, species_gamma=gam)
        fo, so, fr, sr, _ = run_both(model, dim, gam, R, scheme, n, Q)
        for a in range(dim):
            assert np.array_equal(fo[a], fr[a]), f"{label}: face flux of axis {a}"
        assert np.array_equal(so, sr), f"{label}: source"


def test_the_comparison_exercises_every_branch():
    """The states above reach the first-order fallback and the HLLC-HLL faces in every model."""
    for model, _, gam, R in MODELS:
        seen = [0, 0]
        for label in ("shock", "noisy", "rough"):
            n = [13, 11]
            Q = STATES[label](model, 2, n, seed=3, species_gamma=gam)
            _, _, _, _, stats = run_both(model, 2, gam, R, O.SCHEME_WCNS6_LD, n, Q)
            seen[0] += stats[1]
            seen[1] += stats[2]
        assert seen[0] > 0, f"model {model}: no fallback face"
        assert seen[1] > 0, f"model {model}: no HLLC-HLL face"


def test_default_workload_band_is_bitwise_the_reference():
    """The benchmark's 2D five-equation shock/interface problem (WCNS6-LD) at 96^2, whose
    Mach 1.5 shock and tanh interface hit the fallback and HLLC-HLL faces."""
    Q, dx, dt = P.shock_interface_2d(N=96, seed=1)
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, 2, [1.4, 1.67], O.SCHEME_WCNS6_LD)
    fo, so, stats = O.conv_flux_source(cfg, [96, 96], dx, dt, Q)
    fr, sr = O.ref_conv_flux_source(cfg, [96, 96], dx, dt, Q)
    assert stats[1] > 0 and stats[2] > 0
    for a in range(2):
        assert np.array_equal(fo[a], fr[a])
    assert np.array_equal(so, sr)


def test_source_is_accumulated_like_the_reference():
    """The source argument is added to (Euler.cpp zeroes it before the call), in both."""
    model, gam = O.MODEL_FIVE_EQN_ALLAIRE, [1.4, 1.67]
    n = [10, 9]
    dx = [0.1, 1.0 / 9]
    Q = smooth_state(model, 2, n, seed=4, species_gamma=gam)
    cfg = O.Config(model, 2, gam, O.SCHEME_WCNS5_JS)
    s0 = np.random.default_rng(1).standard_normal((cfg.neq, 1, 9, 10))
    _, so, _ = O.conv_flux_source(cfg, n, dx, 1e-3, Q, source=s0.copy())
    _, sr = O.ref_conv_flux_source(cfg, n, dx, 1e-3, Q, source=s0.copy())
    assert np.array_equal(so, sr) and not np.array_equal(so, s0)


def test_vortex_state_is_bitwise_the_reference():
    """The smooth periodic state of the finite-difference checks."""
    for model, _, gam, R in MODELS:
        for dim in (2, 3):
            n = [12, 10] if dim == 2 else [8, 6, 6]
            Q = vortex_state(model, dim, n, seed=2, species_gamma=gam)
            fo, so, fr, sr, _ = run_both(model, dim, gam, R, O.SCHEME_WCNS6_LD, n, Q)
            assert all(np.array_equal(a, b) for a, b in zip(fo, fr)) and np.array_equal(so, sr)


# ---------------------------------------------------------------------------
# Navier-Stokes: DiffusiveFluxReconstructorMidpointSecondOrder / FourthOrder / SixthOrder
# (src/flow/diffusive_flux_reconstructors/midpoint/) with FlowModelSingleSpecies's diffusive
# utilities, compiled from the reference's sources into the same library.
# ---------------------------------------------------------------------------
DIFF_CASES = [(d, o) for d in (2, 3) for o in (2, 4, 6)]


def _wider(gen, dim, n, extra, seed):
    """A state generated on n grown by `extra` cells per side: ghost width 4 + extra around n."""
    return gen(O.MODEL_SINGLE_SPECIES, dim, [v + 2 * extra for v in n], seed=seed, species_gamma=[1.4])


@pytest.mark.parametrize("dim,order", DIFF_CASES, ids=["%dd-o%d" % c for c in DIFF_CASES])
def test_oracle_diffusive_flux_is_bitwise_the_reference(dim, order):
    gh = 5 if order == 6 else 4
    n = [13, 11] if dim == 2 else [8, 7, 6]
    dx = [0.1, 0.07, 0.13][:dim]
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4], species_R=[287.0], ghosts=gh)
    tr = O.Transport(0.05, 1004.5, 0.72, mu_v=0.01, order=order, mu_kappa=0.07)
    for label, gen in (("smooth", smooth_state), ("shock", shock_state), ("rough", rough_state)):
        Q = _wider(gen, dim, n, gh - 4, seed=5)
        fo = O.diff_flux(cfg, tr, n, dx, 1.1e-3, Q)
        fr = O.ref_diff_flux(cfg, tr, n, dx, 1.1e-3, Q, ghosts=gh)
        for a in range(dim):
            assert np.array_equal(fo[a], fr[a]), f"{label}: diffusive flux of axis {a}"
            assert np.any(fo[a] != 0.0)


def test_oracle_wider_ghost_box_changes_nothing_else():
    """The convective flux and the second/fourth-order diffusive flux read at most 4 ghost cells:
    on a 5-ghost box they equal the 4-ghost results."""
    for dim, n in ((2, [13, 11]), (3, [8, 7, 6])):
        Q5 = _wider(shock_state, dim, n, 1, seed=8)
        inner = (slice(None),) + tuple(slice(1, -1) if a < dim else slice(None) for a in (2, 1, 0))
        Q4 = np.ascontiguousarray(Q5[inner])
        c5 = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4], species_R=[287.0], ghosts=5)
        c4 = O.Config(O.MODEL_SINGLE_SPECIES, dim, [1.4], species_R=[287.0])
        f5, s5, _ = O.conv_flux_source(c5, n, [0.1] * dim, 1e-3, Q5)
        f4, s4, _ = O.conv_flux_source(c4, n, [0.1] * dim, 1e-3, Q4)
        assert all(np.array_equal(a, b) for a, b in zip(f5, f4)) and np.array_equal(s5, s4)
        for order in (2, 4):
            tr = O.Transport(0.05, 1004.5, 0.72, mu_v=0.01, order=order)
            d5 = O.diff_flux(c5, tr, n, [0.1] * dim, 1e-3, Q5)
            d4 = O.diff_flux(c4, tr, n, [0.1] * dim, 1e-3, Q4)
            assert all(np.array_equal(a, b) for a, b in zip(d5, d4))


# ---------------------------------------------------------------------------
# Physical boundaries: the reference's EulerBoundaryConditions split (SCALAR variables SYMMETRY,
# the momentum REFLECT, at REFLECT walls) over its BasicCartesianBoundaryUtilities2 / 3
# (src/util/basic_boundary_conditions/), compiled into the same library, on a patch covering
# the domain with FLOW, REFLECT or SYMMETRY (mode 5, every variable) on every side.
# ---------------------------------------------------------------------------
BC_MODES = {2: ([3, 3], [0, 0], [3, 0], [0, 3], [5, 5], [5, 3], [0, 5]),
            3: ([3, 3, 3], [0, 0, 0], [3, 0, 3], [0, 3, 0], [3, 3, 0], [5, 5, 5], [5, 3, 0], [0, 5, 3])}


@pytest.mark.parametrize("model,mn,gam,R", MODELS, ids=[m[1] for m in MODELS])
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_ghost_fill_is_bitwise_the_reference(model, mn, gam, R, dim):
    n = [9, 7] if dim == 2 else [6, 5, 7]
    cfg = O.Config(model, dim, gam, O.SCHEME_WCNS5_JS, species_R=R)
    for mode in BC_MODES[dim]:
        for corner_axis in range(dim):   # every choice of the corners' X/Y/Z-prefixed condition
            Q = smooth_state(model, dim, n, seed=3, species_gamma=gam)
            Qo = Q.copy()
            O.fill_ghosts(cfg, n, mode, Qo)
            Qr = Q.copy()
            O.ref_fill_boundaries(cfg, n, mode, Qr, corner_axis)
            assert not np.array_equal(Qr, Q)
            assert np.array_equal(Qo, Qr), (mode, corner_axis)


# DIRICHLET sides (BasicCartesianBoundaryUtilities2.cpp:150-165 and the X/Y/Z-prefixed corner
# conditions, :679-710) with per-side conservative values, alone and beside FLOW and REFLECT.
DIRICHLET_MODES = {2: ([4, 4], [4, 0], [0, 4], [3, 4], [4, 3], [5, 4]),
                   3: ([4, 4, 4], [4, 0, 3], [0, 4, 0], [3, 3, 4], [0, 3, 4], [4, 5, 3])}


def dirichlet_values(Q, dim, seed):
    """Conservative values per side (2 dim rows, row 2 axis + high): interior cells of a physical
    state, so that each side's values are a consistent state of the model."""
    rng = np.random.default_rng(seed)
    flat = Q.reshape(Q.shape[0], -1)
    return np.ascontiguousarray(flat[:, rng.integers(0, flat.shape[1], 2 * dim)].T)


@pytest.mark.parametrize("model,mn,gam,R", MODELS, ids=[m[1] for m in MODELS])
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_dirichlet_fill_is_bitwise_the_reference(model, mn, gam, R, dim):
    n = [9, 7] if dim == 2 else [6, 5, 7]
    cfg = O.Config(model, dim, gam, O.SCHEME_WCNS5_JS, species_R=R)
    Q = smooth_state(model, dim, n, seed=3, species_gamma=gam)
    bv = dirichlet_values(Q, dim, seed=11)
    for mode in DIRICHLET_MODES[dim]:
        for corner_axis in range(dim):   # decides the corners without a Dirichlet side
            Qo = Q.copy()
            O.fill_ghosts(cfg, n, mode, Qo, dirichlet=bv)
            Qr = Q.copy()
            O.ref_fill_boundaries(cfg, n, mode, Qr, corner_axis, dirichlet=bv)
            assert not np.array_equal(Qr, Q)
            assert np.array_equal(Qo, Qr), (mode, corner_axis)
            # every ghost cell beyond a Dirichlet side holds one of the sides' values
            d = [a for a in range(dim) if mode[a] == 4]
            sl = (slice(None),) + tuple(slice(0, 4) if (2 - a) < dim and (2 - a) == d[0] else slice(None)
                                        for a in range(3))
            assert np.all(Qo[sl] == bv[2 * d[0]][:, None, None, None])
