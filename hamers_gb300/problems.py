"""Initial conditions and workload definitions (host side, numpy).

Every state array uses the SAMRAI layout of the conserved variables of a
patch: shape (ncomp, G2, G1, G0), ghost width 4, x fastest.  Component order
follows the reference's conservative variables:

  single species  : rho, rho*u_k (dim), E
  four-eqn conservative: rho*Y_i (N), rho*u_k (dim), E
  five-eqn Allaire: Z_i*rho_i (N), rho*u_k (dim), E, Z_i (N, the last one is
                    stored as the reference's volume-fraction CellData does)

The problems are the reference's convergence problems
(problems/Euler/initial_conditions/ConvergenceSingleSpecies.cpp:77-99,
ConvergenceFiveEqnAllaire.cpp:100-125) and seeded synthetic stand-ins for the
benchmark workloads (a 2D periodic density wave, a shocked two-species
interface, 3D density blobs on uneven patches, the Taylor-Green vortex).
"""
import math

import numpy as np

GHOST = 4
MODEL_SINGLE_SPECIES = 0
MODEL_FOUR_EQN_CONSERVATIVE = 1
MODEL_FIVE_EQN_ALLAIRE = 2


def ncomp_of(model, dim, nspecies):
    if model == MODEL_SINGLE_SPECIES:
        return dim + 2
    if model == MODEL_FOUR_EQN_CONSERVATIVE:
        return nspecies + dim + 1
    return dim + 2 * nspecies + 1


def _grid(n, xlo, dx, dim):
    """Cell-centre coordinates over the ghost box, each (G2, G1, G0)."""
    axes = []
    for d in range(3):
        if d < dim:
            idx = np.arange(-GHOST, n[d] + GHOST, dtype=np.float64)
            axes.append(xlo[d] + (idx + 0.5) * dx[d])
        else:
            axes.append(np.zeros(1))
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return [x, y, z][:dim]


def single_species_state(rho, vel, p, gamma):
    """Conserved variables from primitives (ideal gas)."""
    dim = len(vel)
    out = np.empty((dim + 2,) + rho.shape)
    out[0] = rho
    ke = sum(v * v for v in vel)
    for k in range(dim):
        out[1 + k] = rho * vel[k]
    out[dim + 1] = p / (gamma - 1.0) + 0.5 * rho * ke
    return out


def five_eqn_state(Z1, rho1, rho2, vel, p, gammas):
    """Two-species five-equation (Allaire) conserved variables."""
    dim = len(vel)
    g1, g2 = gammas
    Z2 = 1.0 - Z1
    out = np.empty((dim + 5,) + Z1.shape)
    out[0] = Z1 * rho1
    out[1] = Z2 * rho2
    rho_m = out[0] + out[1]
    gamma_m = 1.0 / (Z1 / (g1 - 1.0) + Z2 / (g2 - 1.0)) + 1.0
    for k in range(dim):
        out[2 + k] = rho_m * vel[k]
    ke = sum(v * v for v in vel)
    out[2 + dim] = p / (gamma_m - 1.0) + 0.5 * rho_m * ke
    out[3 + dim] = Z1
    out[4 + dim] = Z2
    return out


def four_eqn_state(rho_Y, vel, p, gammas, Rs):
    """Four-equation (conservative) conserved variables from partial densities.

    Ideal-gas mixture with mass fractions: c_p = sum Y_i c_p,i, c_v = sum Y_i c_v,i,
    gamma = c_p/c_v, species c_p,i = gamma_i/(gamma_i-1) R_i, c_v,i = R_i/(gamma_i-1)
    (EquationOfStateMixingRulesIdealGas.cpp:107-120).
    """
    dim = len(vel)
    N = len(rho_Y)
    rho = sum(rho_Y)
    cp = sum(rY / rho * g / (g - 1.0) * R for rY, g, R in zip(rho_Y, gammas, Rs))
    cv = sum(rY / rho / (g - 1.0) * R for rY, g, R in zip(rho_Y, gammas, Rs))
    gamma_m = cp / cv
    out = np.empty((N + dim + 1,) + rho.shape)
    for si in range(N):
        out[si] = rho_Y[si]
    for k in range(dim):
        out[N + k] = rho * vel[k]
    ke = sum(v * v for v in vel)
    out[N + dim] = p / (gamma_m - 1.0) + 0.5 * rho * ke
    return out


FOUR_EQN_GAMMA = [1.6, 1.4]
FOUR_EQN_R = [1.0, 2.5]


# ---------------------------------------------------------------------------
# Convergence problems of the reference's CI (tests/*_convergence_test_*/convergence_test.py)
# ---------------------------------------------------------------------------
def convergence_problem(model, dim, N):
    """Density-wave (single) or volume-fraction-wave (five-eqn) advection on [-1,1]^dim.

    Returns (state, dx, dt, nsteps, exact(t) -> field on the interior, species_gamma);
    the four-equation variant advects a mass-fraction wave (field: rho*Y_1 at rho = 1).
    dt = 0.001*dx, 8 steps in 2D (1 in 3D) at N=8, doubled per refinement
    (convergence_test.py:18-23).
    """
    n = [N] * dim
    dx = [2.0 / N] * dim
    xlo = [-1.0] * dim
    X = _grid(n, xlo, dx, dim)
    s = sum(X)
    ones = [np.ones_like(s) for _ in range(dim)]
    level = int(round(math.log2(N / 8)))
    dt = 0.001 * (2.0 / 8) / 2 ** level
    nsteps = (8 if dim == 2 else 1) * 2 ** level
    if model == MODEL_SINGLE_SPECIES:
        rho = 1.0 + 0.5 * np.sin(math.pi * s)
        Q = single_species_state(rho, ones, 1.0, 1.4)
        gam = [1.4]

        def exact(t):
            Xi = _interior(X, dim)
            return 1.0 + 0.5 * np.sin(math.pi * (sum(Xi) - dim * t))
    elif model == MODEL_FOUR_EQN_CONSERVATIVE:
        # Mass-fraction wave at uniform density, velocity and pressure (the
        # reference has no four-equation convergence test; same set-up as its
        # five-equation one with mass instead of volume fractions).
        Y1 = 0.5 + 0.25 * np.sin(math.pi * s)
        Q = four_eqn_state([Y1, 1.0 - Y1], ones, 1.0, FOUR_EQN_GAMMA, FOUR_EQN_R)
        gam = list(FOUR_EQN_GAMMA)

        def exact(t):
            Xi = _interior(X, dim)
            return 0.5 + 0.25 * np.sin(math.pi * (sum(Xi) - dim * t))
    else:
        Z1 = 0.5 + 0.25 * np.sin(math.pi * s)
        Q = five_eqn_state(Z1, 2.0, 1.0, ones, 1.0, (1.6, 1.4))
        gam = [1.6, 1.4]

        def exact(t):
            Xi = _interior(X, dim)
            return 0.5 + 0.25 * np.sin(math.pi * (sum(Xi) - dim * t))
    return np.ascontiguousarray(Q), dx, dt, nsteps, exact, gam


def _interior(X, dim):
    sl = tuple([slice(GHOST, -GHOST) if d < dim else slice(None) for d in (2, 1, 0)])
    return [x[sl] for x in X]


def interior(Q, dim):
    sl = (slice(None),) + tuple([slice(GHOST, -GHOST) if d < dim else slice(None) for d in (2, 1, 0)])
    return Q[sl]


# ---------------------------------------------------------------------------
# Benchmark workloads
# ---------------------------------------------------------------------------
def density_wave_2d(N=256, amp=0.2, gamma=1.4, cfl=0.4):
    """2D single species on [0,1]^2, rho = 1 + amp*sin(2*pi*(x+y)), u=v=1, p=1, periodic.

    dt from the initial state at the given CFL (sum over directions of
    max(|u_d|+c)/dx_d, Euler::computeSpectralRadiusesAndStableDtOnPatch).
    """
    n = [N, N]
    dx = [1.0 / N, 1.0 / N]
    X = _grid(n, [0.0, 0.0], dx, 2)
    rho = 1.0 + amp * np.sin(2.0 * math.pi * (X[0] + X[1]))
    ones = [np.ones_like(rho), np.ones_like(rho)]
    Q = single_species_state(rho, ones, 1.0, gamma)
    c = np.sqrt(gamma * 1.0 / rho)
    dt = cfl / sum((1.0 + c).max() / d for d in dx)
    return np.ascontiguousarray(Q), dx, dt


def shock_interface_2d(N=1024, seed=1, gammas=(1.4, 1.67), density_ratio=3.0, mach=1.5,
                       modes=16, amp_max=0.02, cfl=0.4):
    """2D five-equation shock / perturbed-interface problem on [0,1]^2.

    Species 1 (gamma 1.4, density 1) on the left of a tanh interface at
    x_I(y) = 0.5 + sum_k a_k sin(2 pi k y + phi_k) (a_k ~ U[0, amp_max],
    phi_k ~ U[0, 2 pi), seeded), species 2 (density ratio 3) on the right,
    interface width 4 cells (0.05 -> 0.95), volume fraction clipped to
    [1e-8, 1-1e-8].  A Mach 1.5 shock at x = 0.25 moves right into species 1
    with the Rankine-Hugoniot post-shock state behind it.  Zero-gradient in
    x, periodic in y.
    """
    rng = np.random.default_rng(seed)
    a_k = rng.uniform(0.0, amp_max, modes)
    phi_k = rng.uniform(0.0, 2.0 * math.pi, modes)
    n = [N, N]
    dx = [1.0 / N, 1.0 / N]
    X = _grid(n, [0.0, 0.0], dx, 2)
    x, y = X
    xI = 0.5 + sum(a_k[k] * np.sin(2.0 * math.pi * (k + 1) * y + phi_k[k]) for k in range(modes))
    delta = 4.0 * dx[0] / (2.0 * math.atanh(0.9))
    Z1 = 0.5 * (1.0 - np.tanh((x - xI) / delta))
    Z1 = np.clip(Z1, 1e-8, 1.0 - 1e-8)
    rho1, rho2 = 1.0, density_ratio
    g1 = gammas[0]
    p0 = 1.0
    # Rankine-Hugoniot jump for a shock of Mach `mach` moving into gas 1 at rest.
    M2 = mach * mach
    p_s = p0 * (2.0 * g1 * M2 - (g1 - 1.0)) / (g1 + 1.0)
    rho_s = rho1 * (g1 + 1.0) * M2 / ((g1 - 1.0) * M2 + 2.0)
    c1 = math.sqrt(g1 * p0 / rho1)
    u_s = mach * c1 * (1.0 - rho1 / rho_s)
    shocked = x < 0.25
    u = np.where(shocked, u_s, 0.0)
    v = np.zeros_like(u)
    p = np.where(shocked, p_s, p0)
    r1 = np.where(shocked, rho_s, rho1)
    Q = five_eqn_state(Z1, r1, rho2, [u, v], p, gammas)
    rho_m = Q[0] + Q[1]
    gamma_m = 1.0 / (Z1 / (gammas[0] - 1.0) + (1.0 - Z1) / (gammas[1] - 1.0)) + 1.0
    c = np.sqrt(gamma_m * p / rho_m)
    dt = cfl / ((np.abs(u) + c).max() / dx[0] + (np.abs(v) + c).max() / dx[1])
    return np.ascontiguousarray(Q), dx, dt


def taylor_green_3d(N=128, mach=0.1, gamma=1.4, perturb=0.0, seed=3):
    """3D Taylor-Green vortex on [0, 2 pi)^3 (rho = 1, p0 = 1/(gamma M^2)).

    perturb > 0 adds smooth periodic modes of that amplitude (seeded phases) to every
    primitive variable.  The unperturbed vortex has w = 0 everywhere and mirror-symmetric
    states across the faces on its symmetry planes: constant WCNS stencils (smoothness
    indicators at HAMERS_EPSILON) and HLLC contact speeds of exactly zero, points where the
    reference's flux is not differentiable at the scale of a finite-difference step; the
    perturbed vortex is used where derivatives are checked by differences."""
    n = [N, N, N]
    dx = [2.0 * math.pi / N] * 3
    X = _grid(n, [0.0, 0.0, 0.0], dx, 3)
    x, y, z = X
    ph = np.random.default_rng(seed).uniform(0.0, 2.0 * math.pi, 10) if perturb else np.zeros(10)
    e = float(perturb)
    u = np.sin(x) * np.cos(y) * np.cos(z) + e * np.sin(x + 2.0 * y + ph[0]) * np.cos(z + ph[1])
    v = -np.cos(x) * np.sin(y) * np.cos(z) + e * np.cos(2.0 * x + ph[2]) * np.sin(y + z + ph[3])
    w = e * np.sin(x + ph[4]) * np.cos(y + ph[5]) * np.sin(2.0 * z + ph[6])
    p0 = 1.0 / (gamma * mach * mach)
    p = p0 + ((np.cos(2.0 * z) + 2.0) * (np.cos(2.0 * x) + np.cos(2.0 * y)) - 2.0) / 16.0 + \
        e * np.cos(x + y + z + ph[7])
    rho = 1.0 + e * np.sin(x + ph[8]) * np.sin(y + z + ph[9])
    Q = single_species_state(rho, [u, v, w], p, gamma)
    return np.ascontiguousarray(Q), dx


# Navier-Stokes Taylor-Green vortex at Re = 1600 (mu = 1/Re with the unit velocity and length
# of taylor_green_3d), Pr = 0.72, constant viscosity, no bulk viscosity, R = 1 so that
# c_p = gamma/(gamma - 1).  Keys are the reference's mixing-rule keys.
def taylor_green_transport(reynolds=1600.0, prandtl=0.72, gamma=1.4):
    return {"species_mu": 1.0 / reynolds, "species_mu_v": 0.0,
            "species_c_p": gamma / (gamma - 1.0), "species_Pr": prandtl}


def taylor_green_dt(Q, dx, gamma=1.4, cfl=0.4, mu=1.0 / 1600.0, prandtl=0.72):
    """Time step of the initial Taylor-Green state: cfl over the larger of the convective
    spectral radius max sum_d (|u_d| + c)/dx_d and the diffusive one 2 max(D)/dx^2 summed
    over the axes, D = max(4/3 mu, gamma mu/Pr)/rho (held fixed over the run)."""
    rho = Q[0]
    u = [Q[1 + d] / rho for d in range(3)]
    ke = 0.5 * rho * sum(v * v for v in u)
    p = (gamma - 1.0) * (Q[4] - ke)
    c = np.sqrt(gamma * p / rho)
    conv = sum((np.abs(u[d]) + c) / dx[d] for d in range(3)).max()
    D = max(4.0 / 3.0 * mu, gamma * mu / prandtl) / rho.min()
    diff = 2.0 * D * sum(1.0 / (h * h) for h in dx)
    return cfl / max(conv, diff)


def blobs_patches_3d(num_patches=512, side_lo=16, side_hi=64, seed=2, nblobs=32, gamma=1.4):
    """Uneven cubic 3D patches (side length U{lo..hi} per patch, seeded) holding a
    density field of 32 Gaussian blobs on [0,1]^3 with smoothed random
    velocity, p = 1.  Returns a list of (n[3], xlo[3], dx[3], state).  Half
    the patches sit on a level with twice the spacing of the other half
    (refinement ratio 2).
    """
    rng = np.random.default_rng(seed)
    amps = rng.uniform(0.0, 0.5, nblobs)
    widths = rng.uniform(0.02, 0.1, nblobs)
    centres = rng.uniform(0.0, 1.0, (nblobs, 3))
    patches = []
    for p_i in range(num_patches):
        n = [int(rng.integers(side_lo, side_hi + 1))] * 3
        level = 0 if p_i < num_patches // 2 else 1
        h = (1.0 / 256.0) / (2 ** level)
        xlo = [float(v) for v in rng.uniform(0.0, 1.0 - max(n) * h, 3)]
        dx = [h, h, h]
        X = _grid(n, xlo, dx, 3)
        rho = np.ones_like(X[0])
        for b in range(nblobs):
            r2 = sum((X[d] - centres[b, d]) ** 2 for d in range(3))
            rho = rho + amps[b] * np.exp(-r2 / widths[b] ** 2)
        vel = []
        for d in range(3):
            f = rng.uniform(-0.5, 0.5, X[0].shape)
            for _ in range(3):
                f = (np.roll(f, 1, 0) + f + np.roll(f, -1, 0)) / 3.0
                f = (np.roll(f, 1, 1) + f + np.roll(f, -1, 1)) / 3.0
                f = (np.roll(f, 1, 2) + f + np.roll(f, -1, 2)) / 3.0
            vel.append(f)
        Q = single_species_state(rho, vel, np.ones_like(rho), gamma)
        patches.append((n, xlo, dx, np.ascontiguousarray(Q)))
    return patches


def blobs_patches_3d_device(num_patches=512, side_lo=16, side_hi=64, seed=2, nblobs=32, gamma=1.4,
                            device="cuda"):
    """blobs_patches_3d evaluated with torch on the device (same recipe and seeds
    for the layout and the blobs, cubic patches with E[side^3] ~ 87k cells, ~44.6 M
    cells for 512 patches; the smoothed random velocity uses torch's generator).
    Returns a list of (n[3], dx[3], state tensor (5, G2, G1, G0))."""
    import torch
    rng = np.random.default_rng(seed)
    amps = rng.uniform(0.0, 0.5, nblobs)
    widths = rng.uniform(0.02, 0.1, nblobs)
    centres = rng.uniform(0.0, 1.0, (nblobs, 3))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    out = []
    for p_i in range(num_patches):
        n = [int(rng.integers(side_lo, side_hi + 1))] * 3
        level = 0 if p_i < num_patches // 2 else 1
        h = (1.0 / 256.0) / (2 ** level)
        xlo = [float(v) for v in rng.uniform(0.0, 1.0 - max(n) * h, 3)]
        axes = [xlo[d] + (torch.arange(-GHOST, n[d] + GHOST, device=device, dtype=torch.float64) + 0.5) * h
                for d in range(3)]
        z, y, x = torch.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        rho = torch.ones_like(x)
        for b in range(nblobs):
            r2 = (x - centres[b, 0]) ** 2 + (y - centres[b, 1]) ** 2 + (z - centres[b, 2]) ** 2
            rho = rho + amps[b] * torch.exp(-r2 / widths[b] ** 2)
        vel = []
        for d in range(3):
            f = torch.rand(x.shape, generator=gen, device=device, dtype=torch.float64) - 0.5
            for _ in range(3):
                for ax in range(3):
                    f = (torch.roll(f, 1, ax) + f + torch.roll(f, -1, ax)) / 3.0
            vel.append(f)
        Q = torch.empty((5,) + tuple(x.shape), dtype=torch.float64, device=device)
        Q[0] = rho
        for d in range(3):
            Q[1 + d] = rho * vel[d]
        Q[4] = 1.0 / (gamma - 1.0) + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2)
        out.append((n, [h, h, h], Q.contiguous()))
    return out


# ---------------------------------------------------------------------------
# 3D five-equation shock / perturbed interface on a 3-level layout of uneven patches
# ---------------------------------------------------------------------------
def _tile(length, lo, hi, rng):
    """Split `length` cells into segments of U{lo..hi} cells (the last one takes the rest)."""
    segs, r = [], int(length)
    while r > hi:
        s = int(rng.integers(lo, min(hi, r - lo) + 1))
        segs.append(s)
        r -= s
    segs.append(r)
    return segs


def amr_layout_3d(base=128, seed=4, side_lo=16, side_hi=64, x_ranges=((0.0, 1.0), (0.30, 0.70), (0.40, 0.60))):
    """Seeded 3-level layout on [0,1]^3 (refinement ratio 2): level l has base*2^l cells per unit
    length, covers x in x_ranges[l] (all of y and z) and is tiled by boxes whose side lengths along
    each axis are drawn from U{side_lo..side_hi}.  Returns a list of (level, lo[3], n[3], dx[3])
    with lo the box's first cell index at its level's resolution."""
    rng = np.random.default_rng(seed)
    out = []
    for lev, (x0, x1) in enumerate(x_ranges):
        N = base * 2 ** lev
        xlo, xhi = int(round(x0 * N)), int(round(x1 * N))
        axes = [_tile(xhi - xlo, side_lo, side_hi, rng), _tile(N, side_lo, side_hi, rng),
                _tile(N, side_lo, side_hi, rng)]
        starts = [np.concatenate([[0], np.cumsum(a)[:-1]]) for a in axes]
        dx = [1.0 / N] * 3
        for a0, s0 in zip(axes[0], starts[0]):
            for a1, s1 in zip(axes[1], starts[1]):
                for a2, s2 in zip(axes[2], starts[2]):
                    out.append((lev, [xlo + int(s0), int(s1), int(s2)], [int(a0), int(a1), int(a2)], dx))
    return out


def shock_interface_3d_modes(modes=64, seed=4, amp_max=0.01):
    """The 64-mode interface perturbation of the 3D shock/interface problem: amplitudes
    a_k ~ U[0, amp_max], wavenumbers (m_k, l_k) over an 8x8 grid, phases ~ U[0, 2 pi) (seeded)."""
    rng = np.random.default_rng(seed + 1)
    side = int(round(math.sqrt(modes)))
    ml = [(1 + k // side, 1 + k % side) for k in range(modes)]
    return rng.uniform(0.0, amp_max, modes), np.array(ml, dtype=np.float64), rng.uniform(0.0, 2 * math.pi, modes)


def shock_interface_3d_patch(lo, n, dx, amps, waves, phases, finest_dx, gammas=(1.4, 1.09),
                             density_ratio=3.0, mach=1.5):
    """Conserved variables (8, G2, G1, G0) of one patch's ghost box (torch, on the amplitudes'
    device, differentiable with respect to `amps`): species 1 (density 1) left of the interface
    x_I(y, z) = 0.5 + sum_k a_k sin(2 pi (m_k y + l_k z) + phi_k), species 2 (density ratio 3)
    right of it, tanh profile 4 finest cells wide, volume fraction clipped to [1e-8, 1 - 1e-8];
    a Mach 1.5 shock at x = 0.25 moving into species 1 with the Rankine-Hugoniot state behind it.
    Ghost cells hold the same analytic values (no fill needed)."""
    import torch
    dev, dt_ = amps.device, torch.float64
    idx = [torch.arange(-GHOST, n[d] + GHOST, device=dev, dtype=dt_) for d in range(3)]
    xs = [(lo[d] + idx[d] + 0.5) * dx[d] for d in range(3)]
    z, y, x = torch.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    w = torch.as_tensor(waves, device=dev, dtype=dt_)
    ph = torch.as_tensor(phases, device=dev, dtype=dt_)
    arg = 2.0 * math.pi * (w[:, 0, None, None] * y[:, :, 0][None] + w[:, 1, None, None] * z[:, :, 0][None]) \
        + ph[:, None, None]
    xI = 0.5 + (amps[:, None, None] * torch.sin(arg)).sum(dim=0)          # (G2, G1)
    delta = 4.0 * finest_dx / (2.0 * math.atanh(0.9))
    Z1 = 0.5 * (1.0 - torch.tanh((x - xI[:, :, None]) / delta))
    Z1 = torch.clamp(Z1, 1e-8, 1.0 - 1e-8)
    g1, g2 = gammas
    p0, rho1, rho2 = 1.0, 1.0, density_ratio
    M2 = mach * mach
    p_s = p0 * (2.0 * g1 * M2 - (g1 - 1.0)) / (g1 + 1.0)
    rho_s = rho1 * (g1 + 1.0) * M2 / ((g1 - 1.0) * M2 + 2.0)
    u_s = mach * math.sqrt(g1 * p0 / rho1) * (1.0 - rho1 / rho_s)
    shocked = x < 0.25
    u = torch.where(shocked, torch.full_like(x, u_s), torch.zeros_like(x))
    p = torch.where(shocked, torch.full_like(x, p_s), torch.full_like(x, p0))
    r1 = torch.where(shocked, torch.full_like(x, rho_s), torch.full_like(x, rho1))
    Z2 = 1.0 - Z1
    zr1, zr2 = Z1 * r1, Z2 * rho2
    rho = zr1 + zr2
    gamma_m = 1.0 / (Z1 / (g1 - 1.0) + Z2 / (g2 - 1.0)) + 1.0
    E = p / (gamma_m - 1.0) + 0.5 * rho * u * u
    zero = torch.zeros_like(x)
    return torch.stack([zr1, zr2, rho * u, zero, zero, E, Z1, Z2])
