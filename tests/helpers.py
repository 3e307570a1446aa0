"""Shared helpers of the test suite: problem set-ups and comparisons."""
import math

import numpy as np

from hamers_gb300 import problems as P
from oracle import oracle as O

GHOST = 4


def n3(n):
    return list(n) + [1] * (3 - len(n))


def smooth_state(model, dim, n, seed=0, amp=0.3, species_gamma=None):
    """A smooth but non-trivial state with every component varying (ghost box)."""
    rng = np.random.default_rng(seed)
    nn = n3(n)
    G = [nn[d] + 2 * GHOST if d < dim else 1 for d in range(3)]
    axes = [np.arange(G[d]) / max(1, nn[d]) for d in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    X = [x, y, z][:dim]

    def wave(k):
        ph = rng.uniform(0, 2 * math.pi, 3)
        return sum(np.sin(2 * math.pi * (d + 1) * X[d] + ph[d] + k) for d in range(dim))

    vel = [0.3 * wave(1 + k) for k in range(dim)]
    p = 1.0 + 0.2 * wave(7)
    if model == O.MODEL_SINGLE_SPECIES:
        rho = 1.0 + amp * wave(3) / dim
        return np.ascontiguousarray(P.single_species_state(rho, vel, p, (species_gamma or [1.4])[0]))
    if model == O.MODEL_FOUR_EQN_CONSERVATIVE:
        Y1 = 0.5 + 0.4 * np.tanh(2.0 * wave(5))
        rho = 1.0 + amp * wave(3) / dim
        return np.ascontiguousarray(P.four_eqn_state([rho * Y1, rho * (1.0 - Y1)], vel, p,
                                                     species_gamma or P.FOUR_EQN_GAMMA, P.FOUR_EQN_R))
    Z1 = 0.5 + 0.4 * np.tanh(2.0 * wave(5))
    return np.ascontiguousarray(P.five_eqn_state(Z1, 1.0 + 0.2 * wave(9), 3.0, vel, p,
                                                 tuple(species_gamma or [1.4, 1.67])))


def shock_state(model, dim, n, seed=0, species_gamma=None):
    """Discontinuous data: a pressure/density jump plus a shear layer (exercises HLLC-HLL and LD switches)."""
    rng = np.random.default_rng(seed)
    nn = n3(n)
    G = [nn[d] + 2 * GHOST if d < dim else 1 for d in range(3)]
    axes = [(np.arange(G[d]) - GHOST + 0.5) / max(1, nn[d]) for d in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    X = [x, y, z][:dim]
    front = 0.45 + 0.05 * np.sin(2 * math.pi * X[1])
    left = X[0] < front
    u = np.where(left, 0.8, -0.1) + 0.01 * rng.standard_normal(x.shape)
    v = np.where(X[1] < 0.5, 0.3, -0.3)
    vel = [u, v] + ([0.1 * np.sin(2 * math.pi * X[2])] if dim == 3 else [])
    p = np.where(left, 4.0, 1.0)
    if model == O.MODEL_SINGLE_SPECIES:
        rho = np.where(left, 2.5, 1.0)
        return np.ascontiguousarray(P.single_species_state(rho, vel, p, (species_gamma or [1.4])[0]))
    if model == O.MODEL_FOUR_EQN_CONSERVATIVE:
        Y1 = np.clip(np.where(X[0] < 0.6, 1.0 - 1e-6, 1e-6), 1e-8, 1 - 1e-8)
        rho = np.where(left, 2.0, 1.0) * (1.0 + 0.5 * (X[0] >= 0.6))
        return np.ascontiguousarray(P.four_eqn_state([rho * Y1, rho * (1.0 - Y1)], vel, p,
                                                     species_gamma or P.FOUR_EQN_GAMMA, P.FOUR_EQN_R))
    Z1 = np.clip(np.where(X[0] < 0.6, 1.0 - 1e-6, 1e-6), 1e-8, 1 - 1e-8)
    return np.ascontiguousarray(P.five_eqn_state(Z1, np.where(left, 2.0, 1.0), 3.0, vel, p,
                                                 tuple(species_gamma or [1.4, 1.67])))


def rough_state(model, dim, n, seed=0, species_gamma=None):
    """Cell-by-cell random data: density and pressure log-uniform over six decades (a uniform
    significand in [1, 2) times 2^-k, k = 0..19), velocity U[-2, 2], mass or volume fraction
    U[0, 1].  Reconstructed states of many faces leave their bounds, which sends those faces to
    the first-order fallback.  Only exact operations build the values (no exp or log, whose
    vectorised implementations differ between machines), so every machine makes the same bits."""
    rng = np.random.default_rng(seed)
    nn = list(n) + [1] * (3 - len(n))
    shape = tuple(nn[d] + 8 if d < dim else 1 for d in (2, 1, 0))

    def logu():
        return np.ldexp(rng.uniform(1.0, 2.0, shape), -rng.integers(0, 20, shape))

    rho, p = logu(), logu()
    vel = [rng.uniform(-2.0, 2.0, shape) for _ in range(dim)]
    if model == O.MODEL_SINGLE_SPECIES:
        return np.ascontiguousarray(P.single_species_state(rho, vel, p, (species_gamma or [1.4])[0]))
    frac = np.clip(rng.uniform(0.0, 1.0, shape), 1e-8, 1 - 1e-8)
    if model == O.MODEL_FOUR_EQN_CONSERVATIVE:
        return np.ascontiguousarray(P.four_eqn_state([rho * frac, rho * (1.0 - frac)], vel, p,
                                                     species_gamma or P.FOUR_EQN_GAMMA, P.FOUR_EQN_R))
    return np.ascontiguousarray(P.five_eqn_state(frac, rho, 3.0, vel, p, tuple(species_gamma or [1.4, 1.67])))


def rel_err(a, b):
    """max |a-b| / max(|b|, component scale), component scale = max |b| of that component."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    worst = 0.0
    for e in range(b.shape[0]):
        scale = max(np.abs(b[e]).max(), 1e-300)
        den = np.maximum(np.abs(b[e]), scale)
        worst = max(worst, float((np.abs(a[e] - b[e]) / den).max()))
    return worst


def noisy_shock_state(model, dim, n, seed=0, species_gamma=None, rel=1e-3):
    """shock_state with seeded relative noise on every conserved component.

    Piecewise-constant stencils leave the WCNS smoothness indicators at the
    rounding level of their expanded quadratic forms (~1e-16 |U|^2, the scale
    of HAMERS_EPSILON = 1e-15), where the reference's weights -- and any
    derivative of them -- are ill-conditioned; the noise keeps every stencil
    resolved for the derivative checks."""
    Q = shock_state(model, dim, n, seed=seed, species_gamma=species_gamma)
    rng = np.random.default_rng(seed + 1000)
    return np.ascontiguousarray(Q * (1.0 + rel * rng.standard_normal(Q.shape)))


def vortex_state(model, dim, n, seed=0, species_gamma=None):
    """Smooth periodic state with a Taylor-Green velocity field for the finite-difference checks.

    Each velocity component is scaled by 1/(n sin(2 pi/n)) of its own axis, so that
    the 2nd-order central dilatation of the shock sensor vanishes to rounding, and
    with even n on every axis no cell centre lies on a zero line of the vorticity:
    the sensor never selects HLLC-HLL (whose blending weights depend on the direction
    of the near-zero velocity jump across a face and have derivatives of order
    1/|jump|), and no stencil is constant (where the WCNS smoothness indicators are
    rounding noise of the size of HAMERS_EPSILON)."""
    rng = np.random.default_rng(seed)
    nn = n3(n)
    assert all(nn[d] % 2 == 0 for d in range(dim)), "vortex_state needs even sizes"
    G = [nn[d] + 2 * GHOST if d < dim else 1 for d in range(3)]
    axes = [2 * math.pi * (np.arange(G[d]) - GHOST + 0.5) / max(1, nn[d]) for d in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    ph = rng.uniform(0, 2 * math.pi, 3)
    cz = np.cos(z) if dim == 3 else 1.0
    sx = 1.0 / (nn[0] * math.sin(2 * math.pi / nn[0]))
    sy = 1.0 / (nn[1] * math.sin(2 * math.pi / nn[1]))
    vel = [2.0 * sx * np.sin(x) * np.cos(y) * cz, -2.0 * sy * np.cos(x) * np.sin(y) * cz]
    if dim == 3:
        vel.append(0.0 * x)
    p = 1.0 + 0.1 * np.cos(2 * x + ph[0]) * np.cos(y + ph[1])
    rho = 1.0 + 0.2 * np.sin(x + y + ph[2])
    if model == O.MODEL_SINGLE_SPECIES:
        return np.ascontiguousarray(P.single_species_state(rho, vel, p, (species_gamma or [1.4])[0]))
    Y1 = 0.5 + 0.3 * np.sin(x + ph[2]) * np.cos(y)
    if model == O.MODEL_FOUR_EQN_CONSERVATIVE:
        return np.ascontiguousarray(P.four_eqn_state([rho * Y1, rho * (1.0 - Y1)], vel, p,
                                                     species_gamma or P.FOUR_EQN_GAMMA, P.FOUR_EQN_R))
    return np.ascontiguousarray(P.five_eqn_state(Y1, rho, 3.0, vel, p, tuple(species_gamma or [1.4, 1.67])))
