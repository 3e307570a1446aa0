"""Refluxing restated in the oracle: a coarse step, two fine steps, the flux-sum coarsening,
synchronizeFluxes and the coarsening of the fine interior conserve the composite totals of
every conserved variable to rounding; without the flux correction they do not.
(The reference's own tests run one level only, so this is a property check.)"""
import numpy as np

from oracle import oracle as O
from tests import reflux_case as R

A3 = [[1.0], [0.75, 0.25], [1.0 / 3.0, 0.0, 2.0 / 3.0]]
B3 = [[1.0], [0.0, 0.25], [0.0, 0.0, 2.0 / 3.0]]
G3 = [[1.0 / 6.0], [0.0, 1.0 / 6.0], [0.0, 0.0, 2.0 / 3.0]]


def rk3_accumulate(cfg, n, dx, dt, Q, fill, F_acc, S_acc):
    """One SSPRK3 step through the stage form, accumulating gamma-weighted fluxes and sources."""
    Qs, Fs, Ss = [], [], []
    X = Q.copy()
    for s in range(3):
        fill(X)
        Qs.append(X.copy())
        F, S, _ = O.conv_flux_source(cfg, n, dx, dt, Qs[-1])
        Fs.append(F)
        Ss.append(S)
        X = O.rk_stage(cfg, n, dx, A3[s], B3[s], G3[s], Qs, Fs, Ss, F_acc=F_acc, S_acc=S_acc)
    return X


def two_level_step(reflux):
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, 2, R.GAMMA)
    nc, nf = [R.N, R.N], list(R.FN)
    dxc, dxf = 1.0 / R.N, 0.5 / R.N
    Qc = R.analytic_state(nc, [dxc, dxc], (0, 0))
    Qf = R.analytic_state(nf, [dxf, dxf], R.FLO)
    O.coarsen_cells(cfg, R.RATIO, nc, (0, 0), nf, R.FLO, Qf, Qc)
    before = R.composite_totals(Qc, Qf, dxc, dxf)
    dt = 0.2 * dxc
    Qc_old = Qc.copy()
    Fc = [np.zeros(s) for s in O.flux_shapes(cfg, nc)]
    Sc = np.zeros((4, 1, R.N, R.N))
    Qc_new = rk3_accumulate(cfg, nc, [dxc, dxc], dt, Qc, lambda X: O.fill_ghosts(cfg, nc, [1, 1], X), Fc, Sc)
    Ff = [np.zeros(s) for s in O.flux_shapes(cfg, nf)]
    Sf = np.zeros((4, 1, nf[1], nf[0]))
    for _ in range(2):
        Qf = rk3_accumulate(cfg, nf, [dxf, dxf], 0.5 * dt, Qf, lambda X: R.inject_ghosts(X, Qc_old), Ff, Sf)
    if reflux:
        O.coarsen_fluxsum(cfg, R.RATIO, nc, (0, 0), nf, R.FLO, Ff, Fc)
        Qc = Qc_old.copy()
        O.sync_fluxes(cfg, nc, [dxc, dxc], Fc, Sc, Qc)
    else:
        Qc = Qc_new
    O.coarsen_cells(cfg, R.RATIO, nc, (0, 0), nf, R.FLO, Qf, Qc)
    after = R.composite_totals(Qc, Qf, dxc, dxf, covered=False)
    return before, after, Qc_new, Qc


def test_reflux_conserves_composite_totals():
    before, after, _, _ = two_level_step(True)
    assert np.all(np.abs(after - before) <= 1e-14 * np.abs(before)), (before, after)


def test_without_flux_correction_totals_drift():
    before, after, _, _ = two_level_step(False)
    assert np.any(np.abs(after - before) > 1e-9 * np.abs(before)), (before, after)


def test_sync_with_uncorrected_fluxes_redoes_the_coarse_step():
    """Away from the fine patch, synchronizeFluxes from the old state with the
    time-integrated fluxes reproduces the SSPRK3 result (to rounding)."""
    _, _, Qc_new, Qc = two_level_step(True)
    far = (slice(None), 0, slice(4, 4 + 4), slice(4, 4 + 4))
    assert np.allclose(Qc[far], Qc_new[far], rtol=1e-13, atol=0)
