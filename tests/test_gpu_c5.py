"""The 3-level 3D five-equation shock/interface configuration at a small scale.

Patches of all levels, with ghost cells supplied by the analytic initial state
(fill mode HMR_FILL_PROVIDED), advanced by one batched substep must equal the
per-patch substep (exact form: bitwise); the gradient of J = sum <w, Q_out>
with respect to the 64 interface-mode amplitudes, from the per-patch VJPs
chained through the differentiable initial condition, must match the oracle's
tangent along random amplitude directions.
"""
import numpy as np
import pytest

from hamers_gb300 import problems as P
from oracle import oracle as O

GAM = [1.4, 1.09]


def _setup(torch, flow, precision):
    layout = P.amr_layout_3d(base=8, seed=4, side_lo=4, side_hi=8)
    amps, waves, phases = P.shock_interface_3d_modes(64, seed=4)
    a = torch.tensor(amps, dtype=torch.float64, device="cuda")
    finest = min(dx[0] for _, _, _, dx in layout)
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 3, GAM)
    rec = flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision=precision)
    states = [P.shock_interface_3d_patch(lo, n, dx, a, waves, phases, finest).contiguous() for _, lo, n, dx in layout]
    return layout, (a, waves, phases, finest), rec, states


@pytest.mark.gpu
def test_batched_substep_with_provided_ghosts_equals_per_patch(cuda):
    import torch
    from hamers_gb300 import flow
    layout, _, rec, states = _setup(torch, flow, "exact")
    assert len(layout) >= 10 and len({lev for lev, _, _, _ in layout}) == 3
    dt = 1e-3
    eu = flow.Euler(rec)
    outs = []
    for (_, _, n, dx), Q in zip(layout, states):
        o = torch.zeros_like(Q)
        eu.substep(flow.Patch(n, dx, Q), 0, [Q], dt, o)
        outs.append(o)
    lv = flow.BatchedLevel(rec, [(n, dx) for _, _, n, dx in layout])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, [2, 2, 2])
    lv.substep(0, dt)
    torch.cuda.synchronize()
    lv.check()
    sl = (slice(None), slice(4, -4), slice(4, -4), slice(4, -4))
    for p, o in enumerate(outs):
        got = lv.state(p, 1)
        assert torch.equal(got[sl], o[sl]), f"patch {p}"
    lv.close()


@pytest.mark.gpu
def test_amplitude_gradient_matches_oracle_tangent(cuda):
    import torch
    from hamers_gb300 import flow
    layout, (a, waves, phases, finest), rec, states = _setup(torch, flow, "exact")
    dt = 1e-3
    eu = flow.Euler(rec)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(4)
    W = [torch.randn(Q.shape, dtype=torch.float64, device="cuda", generator=gen) for Q in states]
    a_req = a.clone().requires_grad_(True)
    grad = torch.zeros_like(a)
    for (_, lo, n, dx), Q, w in zip(layout, states, W):
        b = torch.zeros_like(Q)
        eu.substepVJP(flow.Patch(n, dx, Q), 0, [Q], dt, w, [b])
        Qa = P.shock_interface_3d_patch(lo, n, dx, a_req, waves, phases, finest)
        grad += torch.autograd.grad(Qa, a_req, grad_outputs=b)[0]
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, 3, GAM, O.SCHEME_WCNS6_LD)
    rng = np.random.default_rng(5)
    for _ in range(2):
        d = torch.tensor(rng.standard_normal(64), dtype=torch.float64, device="cuda")
        dJ, scale = 0.0, 0.0
        for (_, lo, n, dx), Q, w in zip(layout, states, W):
            _, dQ = torch.autograd.functional.jvp(
                lambda aa: P.shock_interface_3d_patch(lo, n, dx, aa, waves, phases, finest), (a,), (d,))
            _, JV = O.tangent_substep(cfg, n, dx, dt, 0, [1.0], 1.0, [Q.cpu().numpy()], [dQ.cpu().numpy()])
            prod = w.cpu().numpy() * JV
            dJ += float(prod.sum())
            scale += float(np.abs(prod).sum())
        got = float((grad * d).sum())
        assert abs(got - dJ) <= 1e-9 * scale, (got, dJ, scale)
