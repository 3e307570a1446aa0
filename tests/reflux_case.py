"""Two-level periodic set-up shared by the refluxing tests (oracle on the CPU, and the
device path): a 2D coarse level of one periodic patch and one fine patch (refinement
ratio 2, time refinement 2) inside it.  Not a test module."""
import math

import numpy as np

from oracle import oracle as O

GAMMA = [1.4]
N = 16
FLO, FN = (8, 12), (16, 8)      # fine patch: level index of the first cell and size (ratio 2)
RATIO = (2, 2)


def analytic_state(n, dx, lo):
    G = [v + 8 for v in n]
    ax = [(np.arange(G[d]) - 4 + lo[d] + 0.5) * dx[d] for d in range(2)]
    y, x = np.meshgrid(ax[1], ax[0], indexing="ij")
    rho = 1.0 + 0.3 * np.sin(2 * math.pi * (x + 0.3 * y))
    u = 0.8 + 0.2 * np.cos(2 * math.pi * y)
    v = 0.5 - 0.3 * np.sin(2 * math.pi * x)
    p = 1.0 + 0.2 * np.cos(2 * math.pi * (x - y))
    E = p / (GAMMA[0] - 1) + 0.5 * rho * (u * u + v * v)
    return np.ascontiguousarray(np.stack([rho, rho * u, rho * v, E])[:, None])


def inject_ghosts(Qf, Qc):
    """Fine ghost cells from the coarse cell containing them (piecewise constant)."""
    G0, G1 = FN[0] + 8, FN[1] + 8
    for jj in range(G1):
        for ii in range(G0):
            i, j = ii - 4, jj - 4
            if 0 <= i < FN[0] and 0 <= j < FN[1]:
                continue
            ci = ((FLO[0] + i) // RATIO[0]) % N
            cj = ((FLO[1] + j) // RATIO[1]) % N
            Qf[:, 0, jj, ii] = Qc[:, 0, cj + 4, ci + 4]


def composite_totals(Qc, Qf, dxc, dxf, covered=True):
    tot = Qc[:, 0, 4:-4, 4:-4].sum(axis=(1, 2)) * dxc * dxc
    if covered:
        cov = Qc[:, 0, 4 + FLO[1] // 2: 4 + (FLO[1] + FN[1]) // 2, 4 + FLO[0] // 2: 4 + (FLO[0] + FN[0]) // 2]
        tot = tot - cov.sum(axis=(1, 2)) * dxc * dxc + Qf[:, 0, 4:-4, 4:-4].sum(axis=(1, 2)) * dxf * dxf
    return tot
