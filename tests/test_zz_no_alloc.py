"""hmr_rk_substep_patch_noalloc against hmr_rk_substep_patch, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device memory
where they call the substep (their device memory belongs to their own pool, or
a cudaMalloc/cudaFree would synchronise the device inside their time-step
loop).  It must give the same result as the allocating entry point on the same
inputs -- bitwise, since both run the same kernels in the same arithmetic
form -- on consecutive calls that reuse its one shared scratch array, and must
reject a patch too large for that array.  This file is collected last so that a
failure here leaves every other test already run; it also runs alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

from hamers_gb300 import _lib as L
from tests.helpers import shock_state, smooth_state

RK3_ALPHA = [[1.0, 0.0, 0.0], [0.75, 0.25, 0.0], [1.0 / 3.0, 0.0, 2.0 / 3.0]]
RK3_BETA = [1.0, 0.25, 2.0 / 3.0]


def config(lib, model, reconstructor, dim, nsp, gammas, precision):
    cfg = L.Config()
    assert lib.hmr_config_default(ctypes.byref(cfg), model, reconstructor, dim, nsp) == L.HMR_OK
    for s, g in enumerate(gammas):
        cfg.species_gamma[s] = g
    cfg.precision = precision
    return cfg


def geometry(n, dx):
    g = L.PatchGeometry()
    for d in range(3):
        g.n[d] = n[d] if d < len(n) else 1
        g.dx[d] = dx[d] if d < len(dx) else 1.0
    return g


def run_pair(lib, cfg, ncomp, n, dx, stage, states, dt):
    """Returns (allocating result, no-alloc result) of one substep, as numpy arrays."""
    import torch
    ctx = ctypes.c_void_p()
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_OK
    try:
        g = geometry(n, dx)
        Qs = [torch.from_numpy(q).cuda() for q in states[:stage + 1]]
        qi, _k1 = L.ptr_array2([[t[e].data_ptr() for e in range(ncomp)] for t in Qs])
        alpha = (ctypes.c_double * 3)(*RK3_ALPHA[stage])
        outs = []
        for fn in ("alloc", "noalloc"):
            out = torch.full_like(Qs[0], float("nan"))
            qo, _k2 = L.ptr_array([out[e].data_ptr() for e in range(ncomp)])
            if fn == "alloc":
                rc = lib.hmr_rk_substep_patch(ctx, ctypes.byref(g), stage, alpha, RK3_BETA[stage], qi, dt, qo, None)
            else:
                rc = lib.hmr_rk_substep_patch_noalloc(ctypes.byref(cfg), ctypes.byref(g), stage, alpha,
                                                      RK3_BETA[stage], qi, dt, qo, None)
            assert rc == L.HMR_OK, (fn, rc)
            torch.cuda.synchronize()
            outs.append(out.cpu().numpy())
        return outs
    finally:
        lib.hmr_ctx_destroy(ctx)


def interior(a, dim):
    sl = (slice(None),) + tuple(slice(4, -4) if d < dim else slice(None) for d in (2, 1, 0))
    return a[sl]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.HMR_PRECISION_EXACT, L.HMR_PRECISION_FAST], ids=["exact", "fast"])
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(cuda, precision):
    from hamers_gb300 import build
    build.build()
    lib = L.load()
    # Call 1: 2D five-equation WCNS6-LD, stage 1 (two input states).
    gam = [1.4, 1.67]
    cfg = config(lib, L.HMR_FIVE_EQN_ALLAIRE, L.HMR_WCNS6_LD_HLLC_HLL, 2, 2, gam, precision)
    n, dx = [61, 47], [1.0 / 61, 1.0 / 47]
    states = [shock_state(2, 2, n, seed=11, species_gamma=gam), smooth_state(2, 2, n, seed=12, species_gamma=gam)]
    a, b = run_pair(lib, cfg, 7, n, dx, 1, states, 1.0e-3)
    assert np.array_equal(interior(a, 2)[:6], interior(b, 2)[:6])
    assert np.array_equal(interior(a, 2), interior(b, 2))
    # Call 2, right after, reusing the shared scratch: 3D single species WCNS5-JS, stage 0.
    cfg = config(lib, L.HMR_SINGLE_SPECIES, L.HMR_WCNS5_JS_HLLC_HLL, 3, 1, [1.4], precision)
    n, dx = [19, 14, 11], [1.0 / 19, 1.0 / 14, 1.0 / 11]
    states = [shock_state(0, 3, n, seed=13)]
    a, b = run_pair(lib, cfg, 5, n, dx, 0, states, 1.0e-3)
    assert np.array_equal(interior(a, 3), interior(b, 3))
    assert not np.isnan(interior(b, 3)).any()


@pytest.mark.gpu
def test_noalloc_rejects_a_patch_larger_than_its_scratch(cuda):
    lib = L.load()
    cfg = config(lib, L.HMR_FIVE_EQN_ALLAIRE, L.HMR_WCNS6_LD_HLLC_HLL, 2, 2, [1.4, 1.67], L.HMR_PRECISION_FAST)
    g = geometry([398, 398], [1.0 / 398] * 2)
    dummy = (ctypes.POINTER(ctypes.c_double) * 7)()
    for e in range(7):
        dummy[e] = ctypes.cast(ctypes.c_void_p(8), ctypes.POINTER(ctypes.c_double))   # never dereferenced
    inner = ctypes.cast(dummy, L.DPP)
    outer = (L.DPP * 1)(inner)
    alpha = (ctypes.c_double * 3)(1.0, 0.0, 0.0)
    rc = lib.hmr_rk_substep_patch_noalloc(ctypes.byref(cfg), ctypes.byref(g), 0, alpha, 1.0,
                                          ctypes.cast(outer, L.DPPP), 1.0e-3, inner, None)
    assert rc == L.HMR_ERR_CAPACITY
    # A geometry whose sizes would overflow the scratch arithmetic is refused as an argument
    # error, before any size is computed from it.
    g = geometry([2**31 - 4, 16], [1.0e-9, 1.0 / 16])
    rc = lib.hmr_rk_substep_patch_noalloc(ctypes.byref(cfg), ctypes.byref(g), 0, alpha, 1.0,
                                          ctypes.cast(outer, L.DPPP), 1.0e-3, inner, None)
    assert rc == L.HMR_ERR_ARGUMENT
