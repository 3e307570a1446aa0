"""Batched form: every patch of a level advanced by one persistent kernel per RK substep.

Checked against the oracle patch by patch (exact form: bitwise over two steps;
fast form: 1e-12 over one substep), with uneven patch sizes, periodic and
zero-gradient ghost fills, the launch-shape autotuner, the stable time step
computed on the device, and the bounded grid barrier's give-up path (a barrier that can never complete raises the level's
error flag within its time limit, and the level works again afterwards).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import rel_err, smooth_state
from tests.test_gpu_parity import IDS, VARIANTS, make, ocfg

LEVEL_CASES = [VARIANTS[i] for i in (0, 3, 5, 6, 9, 10)]
LEVEL_IDS = [IDS[i] for i in (0, 3, 5, 6, 9, 10)]


def _patches(dim, seed):
    rng = np.random.default_rng(seed)
    if dim == 2:
        sizes = [(int(rng.integers(8, 33)), int(rng.integers(8, 33))) for _ in range(5)]
    else:
        sizes = [tuple(int(rng.integers(6, 15)) for _ in range(3)) for _ in range(4)]
    periodic = [[int(rng.integers(0, 2)) for _ in range(dim)] for _ in sizes]
    return sizes, periodic


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["exact", "fast"])
@pytest.mark.parametrize("variant", LEVEL_CASES, ids=LEVEL_IDS)
def test_batched_level_matches_oracle(cuda, variant, precision):
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, precision)
    sizes, periodic = _patches(dim, 7)
    dt, nsteps = 1.0e-3, 2
    geoms, states, expect = [], [], []
    for p, n in enumerate(sizes):
        dx = [1.0 / v for v in n]
        Q = smooth_state(model, dim, n, seed=40 + p, species_gamma=gam)
        Qo = Q.copy()
        O.fill_ghosts(cfg, n, periodic[p], Qo)
        O.rk3_advance(cfg, n, dx, dt, periodic[p], nsteps, Qo)
        geoms.append((list(n), dx))
        states.append(torch.from_numpy(Q).cuda())
        expect.append(Qo)
    lv = flow.BatchedLevel(rec, geoms)
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, periodic[p])
    for _ in range(nsteps):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    sl = lambda d: (slice(None),) + tuple(slice(4, -4) if a < d else slice(None) for a in (2, 1, 0))
    for p, (Q, Qo) in enumerate(zip(states, expect)):
        got, ref = Q.cpu().numpy()[sl(dim)], Qo[sl(dim)]
        if precision == "exact":
            assert np.array_equal(got, ref), f"patch {p}: max diff {np.abs(got - ref).max()}"
        else:
            # several steps of the fast form drift once a last-bit difference flips a later
            # WCNS6-LD switch; the per-substep bound is checked below
            assert rel_err(got, ref) <= 1e-4, f"patch {p}: rel err {rel_err(got, ref):.3e}"
    if precision == "fast":
        # one substep from identical inputs: within the per-call bound of the fast form
        for p, n in enumerate(sizes):
            Q = torch.from_numpy(smooth_state(model, dim, n, seed=40 + p, species_gamma=gam)).cuda()
            states[p].copy_(Q)
        lv.substep(0, dt)
        torch.cuda.synchronize()
        lv.check()
        for p, n in enumerate(sizes):
            Q0 = smooth_state(model, dim, n, seed=40 + p, species_gamma=gam)
            O.fill_ghosts(cfg, n, periodic[p], Q0)
            F, S, _ = O.conv_flux_source(cfg, n, geoms[p][1], dt, Q0)
            Q1 = O.rk_stage(cfg, n, geoms[p][1], [1.0], [1.0], [0.0], [Q0], [F], [S])
            got = lv.state(p, 1).cpu().numpy()[sl(dim)]
            assert rel_err(got, Q1[sl(dim)]) <= 1e-12, f"patch {p}: substep rel err {rel_err(got, Q1[sl(dim)]):.3e}"
    lv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("vi", [5, 7], ids=[IDS[5], IDS[7]])
@pytest.mark.parametrize("precision", ["exact", "fast"])
def test_launch_shape_leaves_results_unchanged(cuda, precision, vi):
    """Every resident launch shape and work splitting gives the same bits (phase items are
    handed out in chunks from counters or by grid stride, and each item's arithmetic does not
    depend on which block runs it); shapes that cannot be resident, and unknown splittings, are
    rejected before any launch."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = VARIANTS[vi]
    rec = make(model, dim, scheme, gam, precision)
    sizes, periodic = _patches(dim, 13)
    dt = 1.0e-3
    Q0 = [smooth_state(model, dim, n, seed=80 + p, species_gamma=gam) for p, n in enumerate(sizes)]
    lv = flow.BatchedLevel(rec, [(list(n), [1.0 / v for v in n]) for n in sizes])
    states = [torch.from_numpy(q).cuda() for q in Q0]
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, periodic[p])
    for bad in ((256, 1), (96, 1), (64, 0), (128, 1000)):
        with pytest.raises(RuntimeError):
            lv.set_launch(*bad)
    for bad in ((3, 0), (0, 0), (1, 4), (2, -1)):
        with pytest.raises(RuntimeError):
            lv.set_work_split(*bad)
    results = []
    # launch shapes and work splittings (chunk widths of 1, 2, 4 blocks; grid-stride hand-out
    # of the cell-wise phases; faces sorted by their sensor, fast form)
    for shape, split in (((64, 1), (1, 0)), ((128, 1), (1, 0)), ((128, 2), (1, 0)), ((64, 3), (1, 0)),
                         ((128, 2), (2, 0)), ((64, 2), (4, 0)), ((128, 1), (1, 1)), ((64, 3), (4, 1)),
                         ((128, 2), (1, 2)), ((64, 3), (2, 3)), ((128, 1), (4, 2))):
        lv.set_launch(*shape)
        lv.set_work_split(*split)
        assert lv.work_split() == split
        for p, Q in enumerate(states):
            Q.copy_(torch.from_numpy(Q0[p]))
        lv.step(dt)
        torch.cuda.synchronize()
        lv.check()
        results.append([Q.cpu().numpy() for Q in states])
    lv.close()
    for other in results[1:]:
        for a, b in zip(results[0], other):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_autotuned_level_is_unchanged(cuda):
    """The autotuner only changes the launch shape: results stay bitwise equal (exact form)."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = VARIANTS[5]
    rec = make(model, dim, scheme, gam, "exact")
    sizes, periodic = _patches(dim, 11)
    dt = 1.0e-3
    Q0 = [smooth_state(model, dim, n, seed=60 + p, species_gamma=gam) for p, n in enumerate(sizes)]
    results = []
    for tune in (False, True):
        lv = flow.BatchedLevel(rec, [(list(n), [1.0 / v for v in n]) for n in sizes])
        states = [torch.from_numpy(q).cuda() for q in Q0]
        for p, Q in enumerate(states):
            lv.bind(p, Q)
            lv.set_periodic(p, periodic[p])
        if tune:
            shape = lv.autotune(dt)
            assert shape[0] in (64, 128) and shape[1] >= 1
            for p, Q in enumerate(states):
                Q.copy_(torch.from_numpy(Q0[p]))
        lv.step(dt)
        torch.cuda.synchronize()
        lv.check()
        results.append([Q.cpu().numpy() for Q in states])
        lv.close()
    for a, b in zip(*results):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_barrier_gives_up_within_its_limit_and_level_recovers(cuda):
    """A grid barrier that can never complete (one arrival short, on purpose and on the
    host's request) waits 2 ms, raises the level's error flag and lets every block leave;
    hmr_level_check reports HMR_ERR_BARRIER, and with the normal barrier the level steps again."""
    import time
    import torch
    from hamers_gb300 import _lib as L
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = VARIANTS[0]
    rec = make(model, dim, scheme, gam, "exact")
    sizes = [(16, 12), (9, 20)]
    dt = 1.0e-3
    Q0 = [smooth_state(model, dim, n, seed=80 + p, species_gamma=gam) for p, n in enumerate(sizes)]
    states = [torch.from_numpy(q).cuda() for q in Q0]
    lv = flow.BatchedLevel(rec, [(list(n), [1.0 / v for v in n]) for n in sizes])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
    lv.barrier_diagnostic(1, 2_000_000)
    t0 = time.perf_counter()
    lv.substep(0, dt)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(L.HmrError) as err:
        lv.check()
    assert err.value.code == L.HMR_ERR_BARRIER
    lv.check()                                   # the flag is cleared once reported
    lv.barrier_diagnostic(0, 2_000_000_000)
    for p, Q in enumerate(states):
        Q.copy_(torch.from_numpy(Q0[p]))
    lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    cfg = ocfg(model, dim, gam, scheme)
    for p, n in enumerate(sizes):
        Qo = Q0[p].copy()
        O.fill_ghosts(cfg, n, [0] * dim, Qo)
        O.rk3_advance(cfg, n, [1.0 / v for v in n], dt, [0] * dim, 1, Qo)
        sl = (slice(None),) + tuple(slice(4, -4) if a < dim else slice(None) for a in (2, 1, 0))
        assert np.array_equal(states[p].cpu().numpy()[sl], Qo[sl])
    lv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", LEVEL_CASES, ids=LEVEL_IDS)
def test_spectral_radius_matches_oracle(cuda, variant):
    """Euler::computeSpectralRadiusesAndStableDtOnPatch's max over the interior, bitwise."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, n, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    eu = flow.Euler(make(model, dim, scheme, gam, "exact"))
    dx = [1.0 / (v + 1) for v in n]
    Q = smooth_state(model, dim, n, seed=90, species_gamma=gam)
    got = eu.spectralRadius(flow.Patch(n, dx, torch.from_numpy(Q).cuda()))
    assert got == O.spectral_radius(cfg, n, dx, Q)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [VARIANTS[i] for i in (0, 6)], ids=[IDS[i] for i in (0, 6)])
def test_cfl_step_computes_dt_on_the_device(cuda, variant):
    """step_cfl: dt = min over patches of 1/spectral radius, times the CFL number, computed in
    the graph; the step equals a host-driven step with that dt (exact form, bitwise)."""
    import torch
    from hamers_gb300 import flow
    model, dim, scheme, _, gam = variant
    cfg = ocfg(model, dim, gam, scheme)
    rec = make(model, dim, scheme, gam, "exact")
    sizes, periodic = _patches(dim, 13)
    Q0 = [smooth_state(model, dim, n, seed=100 + p, species_gamma=gam) for p, n in enumerate(sizes)]
    geoms = [(list(n), [1.0 / (v + p) for v in n]) for p, n in enumerate(sizes)]
    cfl = 0.4
    dt = min(1.0 / O.spectral_radius(cfg, n, dx, q) for (n, dx), q in zip(geoms, Q0)) * cfl
    results = []
    for mode in ("cfl", "host"):
        lv = flow.BatchedLevel(rec, geoms)
        states = [torch.from_numpy(q).cuda() for q in Q0]
        for p, Q in enumerate(states):
            lv.bind(p, Q)
            lv.set_periodic(p, periodic[p])
        if mode == "cfl":
            lv.step_cfl(cfl)
            torch.cuda.synchronize()
            assert lv.last_dt() == dt
        else:
            lv.step(dt)
        torch.cuda.synchronize()
        lv.check()
        results.append([Q.cpu().numpy() for Q in states])
        lv.close()
    for a, b in zip(*results):
        assert np.array_equal(a, b)
