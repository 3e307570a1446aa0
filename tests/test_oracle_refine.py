"""Coarse-fine ghost cells restated in the oracle (linear time interpolation, conservative
linear refinement with monotonised-central slopes).  The operators are SAMRAI's and not in
the reference's tree, so they are pinned by their defining properties: the fine values of a
coarse cell average back to the coarse value, linear fields are reproduced exactly, the slopes
vanish at extrema, and theta picks the old / new state."""
import numpy as np
import pytest

from oracle import oracle as O

CFG = O.Config(O.MODEL_SINGLE_SPECIES, 2, [1.4])
CN, CLO = [12, 10], [0, 0]
FN, FLO, RATIO = [8, 6], [8, 6], [2, 2]      # fine cells [8, 16) x [6, 12): coarse [4, 8) x [3, 6)


def coarse_field(fun):
    G = [CN[0] + 8, CN[1] + 8]
    x = (np.arange(G[0]) - 4 + CLO[0] + 0.5)
    y = (np.arange(G[1]) - 4 + CLO[1] + 0.5)
    Y, X = np.meshgrid(y, x, indexing="ij")
    return np.ascontiguousarray(np.stack([fun(X, Y, q) for q in range(4)])[:, None])


def fine_centres():
    G = [FN[0] + 8, FN[1] + 8]
    x = (np.arange(G[0]) - 4 + FLO[0] + 0.5) / RATIO[0]
    y = (np.arange(G[1]) - 4 + FLO[1] + 0.5) / RATIO[1]
    Y, X = np.meshgrid(y, x, indexing="ij")
    return X, Y


def ghost_mask():
    m = np.ones((FN[1] + 8, FN[0] + 8), dtype=bool)
    m[4:-4, 4:-4] = False
    return m


def test_linear_fields_are_reproduced():
    lin = lambda X, Y, q: 1.0 + 0.3 * q + 0.25 * X - 0.4 * Y
    Qc = coarse_field(lin)
    Qf = np.zeros((4, 1, FN[1] + 8, FN[0] + 8))
    O.refine_ghosts(CFG, RATIO, FN, FLO, CN, CLO, Qc, Qc, 0.0, Qf)
    X, Y = fine_centres()
    m = ghost_mask()
    for q in range(4):
        assert np.allclose(Qf[q, 0][m], lin(X, Y, q)[m], rtol=0, atol=1e-13)
    assert np.all(Qf[:, 0, 4:-4, 4:-4] == 0.0)      # interior untouched


def test_conservative_and_monotone():
    rng = np.random.default_rng(2)
    Qc = rng.standard_normal((4, 1, CN[1] + 8, CN[0] + 8)) + 3.0
    Qf = np.zeros((4, 1, FN[1] + 8, FN[0] + 8))
    O.refine_ghosts(CFG, RATIO, FN, FLO, CN, CLO, Qc, Qc, 0.0, Qf)
    # coarse cells entirely made of fine ghost cells: the 2x2 blocks left of the fine patch
    for cj in range(3, 6):
        for ci in (2, 3):
            block = Qf[:, 0, 4 + (cj * 2 - FLO[1]): 6 + (cj * 2 - FLO[1]), 4 + (ci * 2 - FLO[0]): 6 + (ci * 2 - FLO[0])]
            assert np.allclose(block.mean(axis=(1, 2)), Qc[:, 0, 4 + cj, 4 + ci], rtol=1e-14, atol=0)
            # the fine values stay within the range of the coarse cell and its face neighbours
            nb = Qc[:, 0, [4 + cj, 4 + cj, 4 + cj, 3 + cj, 5 + cj], [4 + ci, 3 + ci, 5 + ci, 4 + ci, 4 + ci]]
            assert np.all(block.min(axis=(1, 2)) >= nb.min(axis=1) - 1e-12)
            assert np.all(block.max(axis=(1, 2)) <= nb.max(axis=1) + 1e-12)


@pytest.mark.parametrize("theta", [0.0, 1.0])
def test_time_interpolation_end_points(theta):
    rng = np.random.default_rng(4)
    Qo = rng.standard_normal((4, 1, CN[1] + 8, CN[0] + 8)) + 3.0
    Qn = rng.standard_normal(Qo.shape) + 3.0
    A = np.zeros((4, 1, FN[1] + 8, FN[0] + 8))
    B = np.zeros_like(A)
    O.refine_ghosts(CFG, RATIO, FN, FLO, CN, CLO, Qo, Qn, theta, A)
    O.refine_ghosts(CFG, RATIO, FN, FLO, CN, CLO, Qn if theta else Qo, Qn if theta else Qo, 0.0, B)
    assert np.array_equal(A, B)
