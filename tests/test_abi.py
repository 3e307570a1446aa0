"""The C-ABI library loads and exports every symbol include/hmr.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

from hamers_gb300 import _lib as L
from hamers_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "hmr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^int\s+(hmr_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return L.load()


def test_header_and_binding_agree():
    assert declared_functions() == sorted(L.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_config_defaults_match_reference(lib):
    cfg = L.Config()
    assert lib.hmr_config_default(ctypes.byref(cfg), L.HMR_FIVE_EQN_ALLAIRE, L.HMR_WCNS6_LD_HLLC_HLL, 2, 2) == 0
    assert (cfg.constant_p, cfg.constant_q, cfg.constant_C, cfg.constant_alpha_tau) == (2, 4, 1.0e9, 35.0)
    assert cfg.precision == L.HMR_PRECISION_FAST


@pytest.mark.parametrize("field,value", [("dim", 1), ("dim", 4), ("num_species", 0), ("constant_p", 0),
                                         ("convective_flux_reconstructor", 7), ("precision", 9)])
def test_ctx_create_rejects_bad_config_before_touching_a_device(lib, field, value):
    cfg = L.Config()
    lib.hmr_config_default(ctypes.byref(cfg), L.HMR_SINGLE_SPECIES, L.HMR_WCNS5_JS_HLLC_HLL, 2, 1)
    setattr(cfg, field, value)
    ctx = ctypes.c_void_p()
    rc = lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx))
    assert rc in (L.HMR_ERR_ARGUMENT, L.HMR_ERR_UNSUPPORTED)
    assert not ctx.value


def test_null_arguments_are_rejected(lib):
    assert lib.hmr_ctx_create(None, None) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_ctx_destroy(None) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_conv_flux_source_patch(None, None, None, 0.0, None, None, None) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_level_destroy(None) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_level_set_launch(None, 128, 1) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_level_autotune(None, 1e-3, None, None, None) == L.HMR_ERR_ARGUMENT
    assert lib.hmr_level_fill_vjp(None, None, None) == L.HMR_ERR_ARGUMENT


def test_cu_m2_defaults_and_grid_spacing(lib):
    """WCNS6-CU-M2 defaults (WCNS6-CU-M2-HLLC-HLL.cpp:252-270: q 4, C 1000, Chi 1e8, epsilon 1e-8);
    its weights use the grid geometry's spacing, so a context without one is refused."""
    cfg = L.Config()
    assert lib.hmr_config_default(ctypes.byref(cfg), L.HMR_SINGLE_SPECIES, L.HMR_WCNS6_CU_M2_HLLC_HLL, 2, 1) == 0
    assert (cfg.constant_q, cfg.constant_C, cfg.constant_Chi, cfg.constant_epsilon) == (4, 1000.0, 1.0e8, 1.0e-8)
    ctx = ctypes.c_void_p()
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_ARGUMENT
    cfg.grid_dx[0], cfg.grid_dx[1] = 0.1, -0.1
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_ARGUMENT


def test_reconstructor_names_and_grid_geometry_requirement():
    from hamers_gb300 import flow
    fm = flow.FlowModel("SINGLE_SPECIES", 2, [1.4])
    with pytest.raises(ValueError):
        flow.ConvectiveFluxReconstructor("WCNS6_CU_M2_HLLC_HLL", fm)
    with pytest.raises(ValueError):
        flow.ConvectiveFluxReconstructor("WCNS6_TEST", fm)


def test_diffusive_flux_needs_single_species_and_valid_transport(lib):
    cfg = L.Config()
    lib.hmr_config_default(ctypes.byref(cfg), L.HMR_FIVE_EQN_ALLAIRE, L.HMR_WCNS5_JS_HLLC_HLL, 2, 2)
    cfg.diffusive_flux_reconstructor = L.HMR_MIDPOINT_FOURTH_ORDER
    cfg.species_mu, cfg.species_c_p, cfg.species_Pr, cfg.species_mu_kappa = 0.01, 1.0, 0.7, 0.01
    ctx = ctypes.c_void_p()
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_UNSUPPORTED
    lib.hmr_config_default(ctypes.byref(cfg), L.HMR_SINGLE_SPECIES, L.HMR_WCNS5_JS_HLLC_HLL, 3, 1)
    cfg.diffusive_flux_reconstructor = 8
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_UNSUPPORTED
    cfg.diffusive_flux_reconstructor = 3
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_UNSUPPORTED
    cfg.diffusive_flux_reconstructor = L.HMR_MIDPOINT_SECOND_ORDER
    cfg.species_Pr = 0.0
    assert lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)) == L.HMR_ERR_ARGUMENT
