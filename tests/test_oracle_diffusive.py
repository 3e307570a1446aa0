"""Pins the oracle's Navier-Stokes diffusive flux to the viscous terms it discretises.

The reference has no test of its diffusive fluxes, so the restatement of
DiffusiveFluxReconstructorMidpoint (second and fourth order, single species)
is checked against the continuous operator: for smooth periodic fields, the
divergence of the face fluxes, -sum_d (F_R - F_L)/(dt dx_d), converges to
  momentum  d_j tau_ij,  tau_ij = mu (d_j u_i + d_i u_j) + (mu_v - 2/3 mu) delta_ij div u
  energy    d_j (u_i tau_ij) + d_j (kappa d_j T),  kappa = c_p mu/Pr,  T = p/(rho R)
at the scheme's order (rate > 3.7 for fourth order, > 1.85 for second order),
with the exact terms from sympy.  Also: the mass flux is zero and a uniform
flow has no diffusive flux.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

sympy = pytest.importorskip("sympy")

GAMMA, R = 1.4, 1.0
TR = dict(mu=0.05, mu_v=0.02, c_p=3.5, Pr=0.72)


def _fields(dim):
    X = sympy.symbols("x y z")[:dim]
    s = [sympy.sin(2 * sympy.pi * (X[d] + 0.1 * d)) for d in range(dim)]
    c = [sympy.cos(2 * sympy.pi * (X[d] + 0.2 * d)) for d in range(dim)]
    rho = 1 + sympy.Rational(1, 5) * s[0] * (c[1] if dim > 1 else 1)
    vel = [sympy.Rational(1, 2) * s[(d + 1) % dim] * c[d] + sympy.Rational(1, 10) * d for d in range(dim)]
    p = 1 + sympy.Rational(1, 10) * c[0] * s[-1]
    return X, rho, vel, p


def _exact_rhs(dim, tr):
    X, rho, vel, p = _fields(dim)
    T = p / (rho * R)
    div = sum(sympy.diff(vel[d], X[d]) for d in range(dim))
    tau = [[tr["mu"] * (sympy.diff(vel[i], X[j]) + sympy.diff(vel[j], X[i])) +
            ((tr["mu_v"] - sympy.Rational(2, 3) * tr["mu"]) * div if i == j else 0) for j in range(dim)]
           for i in range(dim)]
    kappa = tr["c_p"] * tr["mu"] / tr["Pr"]
    mom = [sum(sympy.diff(tau[i][j], X[j]) for j in range(dim)) for i in range(dim)]
    en = sum(sympy.diff(sum(vel[i] * tau[i][j] for i in range(dim)) + kappa * sympy.diff(T, X[j]), X[j])
             for j in range(dim))
    return [sympy.lambdify(X, e, "numpy") for e in [sympy.Integer(0)] + mom + [en]]


def _state(dim, N):
    """Conserved state of the fields at the cell centres of the ghost box (ghost width 4)."""
    X, rho, vel, p = _fields(dim)
    f_rho = sympy.lambdify(X, rho, "numpy")
    f_vel = [sympy.lambdify(X, v, "numpy") for v in vel]
    f_p = sympy.lambdify(X, p, "numpy")
    h = 1.0 / N
    ax = (np.arange(N + 8) - 4 + 0.5) * h
    if dim == 2:
        y, x = np.meshgrid(ax, ax, indexing="ij")
        pts = (x, y)
    else:
        z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
        pts = (x, y, z)
    r = f_rho(*pts) * np.ones_like(pts[0])
    u = [f(*pts) * np.ones_like(pts[0]) for f in f_vel]
    pr = f_p(*pts) * np.ones_like(pts[0])
    E = pr / (GAMMA - 1) + 0.5 * r * sum(v * v for v in u)
    Q = np.stack([r] + [r * v for v in u] + [E])
    if dim == 2:
        Q = Q[:, None]
    return np.ascontiguousarray(Q), pts


def _divergence(cfg, n, dx, dt, F):
    dim = cfg.dim
    out = 0.0
    for a in range(dim):
        f = F[a]
        sl_r = [slice(None)] * 4
        sl_l = [slice(None)] * 4
        sl_r[3 - a] = slice(1, None)
        sl_l[3 - a] = slice(None, -1)
        out = out - (f[tuple(sl_r)] - f[tuple(sl_l)]) / dx[a]
    return out / dt


def _errors(dim, order, levels):
    rhs = _exact_rhs(dim, TR)
    errs = []
    for N in levels:
        cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [GAMMA], species_R=[R])
        tr = O.Transport(TR["mu"], TR["c_p"], TR["Pr"], mu_v=TR["mu_v"], order=order)
        Q, pts = _state(dim, N)
        n = [N] * dim
        dx = [1.0 / N] * dim
        dt = 0.37
        F = O.diff_flux(cfg, tr, n, dx, dt, Q)
        assert all(np.all(f[0] == 0.0) for f in F)
        div = _divergence(cfg, n, dx, dt, F)
        inner = tuple(slice(4, -4) for _ in range(dim))
        e = 0.0
        for q in range(dim + 2):
            got = div[q][0] if dim == 2 else div[q]
            exact = np.broadcast_to(rhs[q](*[p[inner] for p in pts]), got.shape)
            e = max(e, float(np.sqrt(np.mean((got - exact) ** 2))))
        errs.append(e)
    return errs


@pytest.mark.parametrize("dim,order,levels,rate", [(2, 4, [16, 32, 64], 3.7), (2, 2, [16, 32, 64], 1.85),
                                                   (3, 4, [8, 16, 32], 3.6), (3, 2, [8, 16, 32], 1.8)],
                         ids=["2d-o4", "2d-o2", "3d-o4", "3d-o2"])
def test_diffusive_flux_converges_to_viscous_terms(dim, order, levels, rate):
    errs = _errors(dim, order, levels)
    r = math.log2(errs[-2] / errs[-1])
    assert r > rate, (errs, r)


def test_uniform_flow_has_no_diffusive_flux():
    for dim in (2, 3):
        cfg = O.Config(O.MODEL_SINGLE_SPECIES, dim, [GAMMA])
        n = [6] * dim
        Q = np.zeros(O.ghost_shape(cfg, n))
        Q[0] = 1.3
        for d in range(dim):
            Q[1 + d] = 1.3 * (0.2 + 0.1 * d)
        Q[dim + 1] = 2.5 + 0.5 * 1.3 * sum((0.2 + 0.1 * d) ** 2 for d in range(dim))
        for order in (2, 4):
            F = O.diff_flux(cfg, O.Transport(0.1, 1.0, 0.7, order=order), n, [0.1] * dim, 1e-3, Q)
            assert max(float(np.abs(f).max()) for f in F) < 1e-13
