"""The benchmark workloads at their full sizes.  First the default one: 2D five-equation
Allaire, 1024 x 1024, WCNS6-LD + HLLC-HLL, a Mach 1.5 shock on a perturbed interface (seed 1):

* one flux/source call against the oracle on the whole patch (exact form bitwise, fast form
  within 1e-12; a flux component whose values on the whole axis are below 1e-6 of the axis's
  largest component -- the y-fluxes of mass and energy of a state with v = 0, the x-flux of a
  species held at volume fraction 1e-8 -- is measured against that largest component, since
  its own values are rounding noise of the other components' scale);
* the batched persistent kernel against the per-patch kernels over one SSPRK3 step: the same
  bits in either arithmetic form (every face and cell is computed by the same item code);
* conservation: with periodic ghosts on both axes, one SSPRK3 step leaves the totals of the
  conserved components (partial densities, momentum, energy) unchanged to rounding, because
  every face flux enters its two cells with opposite signs.

Then the uneven-patch workload (3D single species, 512 patches, 45 M cells) and the 3-level
workload (3D five-equation, 474 patches, 35.5 M cells): batched against per-patch, bit for bit;
and the Navier-Stokes Taylor-Green vortex at 128^3: conservation over ten steps.
"""
import numpy as np
import pytest

from hamers_gb300 import problems as P
from oracle import oracle as O
from tests.helpers import rel_err

N = 1024
GAMMA = [1.4, 1.67]
NCONS = 5          # Z_1 rho_1, Z_2 rho_2, rho u, rho v, E (the volume fractions are advected)
G = 4


@pytest.fixture(scope="module")
def c2():
    Q, dx, dt = P.shock_interface_2d(N=N, seed=1)
    return np.ascontiguousarray(Q), list(dx), float(dt)


def _axis_err(a, b):
    """max |a-b| / max(|b|, s_e), s_e = the component's max |b|, or the axis's largest
    component max where that is more than 1e6 times the component's own."""
    scales = [float(np.abs(b[e]).max()) for e in range(b.shape[0])]
    top = max(scales)
    worst = 0.0
    for e in range(b.shape[0]):
        s_e = scales[e] if scales[e] >= 1e-6 * top else top
        worst = max(worst, float((np.abs(a[e] - b[e]) / np.maximum(np.abs(b[e]), s_e)).max()))
    return worst


def _rec(precision):
    from hamers_gb300 import flow
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 2, GAMMA)
    return flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision=precision)


@pytest.mark.gpu
def test_full_size_flux_matches_oracle(cuda, c2):
    import torch
    from hamers_gb300 import flow
    Q, dx, dt = c2
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, 2, GAMMA, O.SCHEME_WCNS6_LD)
    Fo, So, _ = O.conv_flux_source(cfg, [N, N], dx, dt, Q)
    for precision in ("exact", "fast"):
        rec = _rec(precision)
        patch = flow.Patch([N, N], dx, torch.from_numpy(Q).cuda())
        F = rec.allocateFlux(patch)
        S = rec.allocateSource(patch)
        rec.computeConvectiveFluxAndSourceOnPatch(patch, F, S, dt)
        torch.cuda.synchronize()
        Fg = [f.cpu().numpy() for f in F]
        Sg = S.cpu().numpy()
        rec.close()
        for a in range(2):
            if precision == "exact":
                assert np.array_equal(Fg[a], Fo[a]), f"flux axis {a}"
            else:
                assert _axis_err(Fg[a], Fo[a]) <= 1e-12, f"flux axis {a}"
        if precision == "exact":
            assert np.array_equal(Sg, So)
        else:
            assert rel_err(Sg[-1:], So[-1:]) <= 1e-12


def _per_patch_step(rec, Q0, dx, dt, periodic):
    import torch
    from hamers_gb300 import flow
    eu = flow.Euler(rec)
    Qs = [torch.from_numpy(Q0).cuda(), torch.empty(Q0.shape, dtype=torch.float64, device="cuda"),
          torch.empty(Q0.shape, dtype=torch.float64, device="cuda")]
    views = [flow.Patch([N, N], dx, q) for q in Qs]
    for s in range(3):
        eu.fillGhosts(views[s], periodic)
        eu.substep(views[s], s, Qs[:s + 1], dt, Qs[0] if s == 2 else Qs[s + 1])
    torch.cuda.synchronize()
    return Qs[0].cpu().numpy()


def _batched_step(rec, Q0, dx, dt, periodic):
    import torch
    from hamers_gb300 import flow
    Q = torch.from_numpy(Q0).cuda()
    lv = flow.BatchedLevel(rec, [([N, N], dx)])
    lv.bind(0, Q)
    lv.set_periodic(0, periodic)
    lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    out = Q.cpu().numpy()
    lv.close()
    return out


def _interior(Q):
    return Q[:, 0, G:-G, G:-G]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_full_size_batched_equals_per_patch(cuda, c2, precision):
    Q, dx, dt = c2
    rec = _rec(precision)
    a = _per_patch_step(rec, Q, dx, dt, [0, 1])
    b = _batched_step(rec, Q, dx, dt, [0, 1])
    rec.close()
    assert np.array_equal(_interior(a), _interior(b))


@pytest.mark.gpu
def test_full_size_periodic_step_conserves_totals(cuda, c2):
    Q, dx, dt = c2
    rec = _rec("fast")
    out = _batched_step(rec, Q, dx, dt, [1, 1])
    rec.close()
    before, after = _interior(Q), _interior(out)
    assert np.isfinite(after).all()
    mom = float(np.sum(np.abs(before[2])) + np.sum(np.abs(before[3])))   # v = 0 initially
    for e in range(NCONS):
        t0 = np.sum(before[e], dtype=np.float64)
        t1 = np.sum(after[e], dtype=np.float64)
        scale = mom if e in (2, 3) else float(np.sum(np.abs(before[e])))
        assert abs(t1 - t0) <= 1e-12 * scale, (e, t0, t1)
    # the step did change the state (the shock and the interface moved)
    assert not np.array_equal(before, after)


@pytest.mark.gpu
def test_full_size_uneven_level_batched_equals_per_patch(cuda):
    """The uneven-patch workload at its full size (3D single species WCNS5-JS, 512 cubic
    patches of side 16-64 on 2 levels, 45 M cells, fast form): one SSPRK3 step of the batched
    level gives the same bits as the per-patch kernels, patch by patch (each patch's own
    zero-gradient ghosts in both forms)."""
    import torch
    from hamers_gb300 import flow
    patches = P.blobs_patches_3d_device(num_patches=512)
    fm = flow.FlowModel("SINGLE_SPECIES", 3, [1.4])
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision="fast")
    dt = 0.2 * min(dx[0] for _, dx, _ in patches) / 2.5
    Q0 = [Q.clone() for _, _, Q in patches]
    lv = flow.BatchedLevel(rec, [(n, dx) for n, dx, _ in patches])
    for i, (_, _, Q) in enumerate(patches):
        lv.bind(i, Q)
    lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    lv.close()
    batched = [Q.clone() for _, _, Q in patches]
    eu = flow.Euler(rec)
    for (n, dx, Q), q0 in zip(patches, Q0):
        Q.copy_(q0)
        Qs = [Q, torch.empty_like(Q), torch.empty_like(Q)]
        views = [flow.Patch(n, dx, q) for q in Qs]
        for s in range(3):
            eu.fillGhosts(views[s], [0, 0, 0])
            eu.substep(views[s], s, Qs[:s + 1], dt, Qs[0] if s == 2 else Qs[s + 1])
    torch.cuda.synchronize()
    rec.close()
    for (n, _, Q), b in zip(patches, batched):
        inner = (slice(None),) + tuple(slice(G, G + v) for v in (n[2], n[1], n[0]))
        assert torch.equal(Q[inner], b[inner]), n


@pytest.mark.gpu
def test_full_size_amr_substep_batched_equals_per_patch(cuda):
    """The 3-level workload at its full size (3D five-equation shock on a perturbed interface,
    474 uneven patches, 35.5 M cells, WCNS6-LD, fast form, ghosts from the analytic initial
    state): the first RK substep of the batched level (slot 1 of every patch) gives the same bits
    as the per-patch kernels."""
    import torch
    from hamers_gb300 import flow
    layout = P.amr_layout_3d(base=128, seed=4)
    amps, waves, phases = P.shock_interface_3d_modes(64, seed=4)
    a = torch.tensor(amps, dtype=torch.float64, device="cuda")
    finest = min(dx[0] for _, _, _, dx in layout)
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 3, [1.4, 1.09])
    rec = flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision="fast")
    states = [P.shock_interface_3d_patch(lo, n, dx, a, waves, phases, finest) for _, lo, n, dx in layout]
    dt = 0.4 * finest / (3.0 * 3.0)
    lv = flow.BatchedLevel(rec, [(n, dx) for _, _, n, dx in layout])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, [2, 2, 2])
    lv.substep(0, dt)
    torch.cuda.synchronize()
    lv.check()
    eu = flow.Euler(rec)
    out = None
    for p, ((_, _, n, dx), Q) in enumerate(zip(layout, states)):
        if out is None or out.shape != Q.shape:
            out = torch.empty_like(Q)
        eu.substep(flow.Patch(n, dx, Q), 0, [Q], dt, out)
        inner = (slice(None),) + tuple(slice(G, G + v) for v in (n[2], n[1], n[0]))
        assert torch.equal(out[inner], lv.state(p, 1)[inner]), (p, n)
    lv.close()
    rec.close()


@pytest.mark.gpu
def test_full_size_navier_stokes_step_conserves_totals(cuda):
    """The Navier-Stokes workload at its full size (Taylor-Green vortex 128^3, periodic, Mach 0.1,
    Re 1600, WCNS5-JS + HLLC-HLL + fourth-order midpoint diffusive flux, fast form): ten SSPRK3
    steps keep the totals of mass, momentum and energy to rounding (convective and diffusive
    face fluxes both enter their two cells with opposite signs), and the kinetic energy decays."""
    import torch
    from hamers_gb300 import flow
    N3 = 128
    Qnp, dx = P.taylor_green_3d(N3)
    tr = P.taylor_green_transport()
    dt = P.taylor_green_dt(Qnp[:, 4:-4, 4:-4, 4:-4], dx, mu=tr["species_mu"], prandtl=tr["species_Pr"])
    fm = flow.FlowModel("SINGLE_SPECIES", 3, [1.4], transport=tr)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision="fast",
                                           diffusive_flux_reconstructor="MIDPOINT_FOURTH_ORDER")
    Q = torch.from_numpy(np.ascontiguousarray(Qnp)).cuda()
    integ = flow.RungeKuttaLevelIntegrator(flow.NavierStokes(rec), flow.Patch([N3] * 3, dx, Q), [1, 1, 1])
    integ.advance(dt, nsteps=10)
    torch.cuda.synchronize()
    out = Q.cpu().numpy()
    rec.close()
    inner = (slice(None),) + (slice(G, -G),) * 3
    before, after = Qnp[inner], out[inner]
    assert np.isfinite(after).all()
    mom = float(sum(np.sum(np.abs(before[1 + d])) for d in range(3)))
    for e in range(5):
        scale = mom if 1 <= e <= 3 else float(np.sum(np.abs(before[e])))
        assert abs(np.sum(after[e]) - np.sum(before[e])) <= 1e-12 * scale, e
    ke0 = 0.5 * np.sum((before[1] ** 2 + before[2] ** 2 + before[3] ** 2) / before[0])
    ke1 = 0.5 * np.sum((after[1] ** 2 + after[2] ** 2 + after[3] ** 2) / after[0])
    assert ke1 < ke0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_c1_full_size_every_substep_matches_oracle(cuda, precision):
    """The 2D single-species workload at its full size (256^2 density wave, WCNS5-JS + HLLC-HLL,
    periodic, one SSPRK3 step at CFL 0.4): the flux and source of every substep's input state
    against the oracle's (exact form bitwise, fast form within 1e-12 per axis), the stage states
    advanced by the oracle; then the whole step through the per-patch integrator against the
    oracle's step."""
    import torch
    from hamers_gb300 import flow
    from tests.test_gpu_parity import gpu_flux
    n = [256, 256]
    Q, dx, dt = P.density_wave_2d(256)
    cfg = O.Config(O.MODEL_SINGLE_SPECIES, 2, [1.4], O.SCHEME_WCNS5_JS)
    fm = flow.FlowModel("SINGLE_SPECIES", 2, [1.4])
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=precision)
    per = [1, 1]
    X = np.ascontiguousarray(Q.copy())
    O.fill_ghosts(cfg, n, per, X)
    Qint, Fint, Sint = [X], [], []
    for s in range(3):
        Fo, So, _ = O.conv_flux_source(cfg, n, dx, dt, Qint[s])
        Fg, Sg = gpu_flux(rec, n, dx, dt, Qint[s])
        for a in range(2):
            if precision == "exact":
                assert np.array_equal(Fg[a], Fo[a]), f"substep {s} axis {a}"
            else:
                assert _axis_err(Fg[a], Fo[a]) <= 1e-12, f"substep {s} axis {a}: {_axis_err(Fg[a], Fo[a]):.3e}"
        Fint.append(Fo)
        Sint.append(So)
        Xn = O.rk_stage(cfg, n, dx, flow.RK3_ALPHA[s], flow.RK3_BETA[s], flow.RK3_GAMMA[s], Qint, Fint, Sint)
        O.fill_ghosts(cfg, n, per, Xn)
        Qint.append(Xn)
    Qg = torch.from_numpy(Q.copy()).cuda()
    flow.RungeKuttaLevelIntegrator(flow.Euler(rec), flow.Patch(n, dx, Qg), per).advance(dt, nsteps=1)
    got = Qg.cpu().numpy()[:, :, G:-G, G:-G]
    want = Qint[3][:, :, G:-G, G:-G]
    if precision == "exact":
        assert np.array_equal(got, want)
    else:
        assert rel_err(got, want) <= 1e-12
    rec.close()
