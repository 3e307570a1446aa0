"""ctypes binding of libhmr_gb300.so (the C ABI declared in include/hmr.h).

The library is the only compute path: there is no CPU fallback.  Loading it
fails loudly when it has not been built; calls that need a GPU return
HMR_ERR_NO_DEVICE, which the wrappers raise as errors.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhmr_gb300.so")

HMR_MAX_SPECIES = 4
HMR_MAX_COMPONENTS = 12

HMR_OK = 0
HMR_ERR_ARGUMENT = -1
HMR_ERR_UNSUPPORTED = -2
HMR_ERR_NO_DEVICE = -3
HMR_ERR_STATE = -4
HMR_ERR_BARRIER = -5
HMR_ERR_CAPACITY = -6
HMR_FILL_ZERO_GRADIENT, HMR_FILL_PERIODIC, HMR_FILL_PROVIDED = 0, 1, 2

HMR_SINGLE_SPECIES = 0
HMR_FOUR_EQN_CONSERVATIVE = 1
HMR_FIVE_EQN_ALLAIRE = 2
HMR_WCNS5_JS_HLLC_HLL = 0
HMR_WCNS6_LD_HLLC_HLL = 1
HMR_WCNS5_Z_HLLC_HLL = 2
HMR_WCNS6_CU_M2_HLLC_HLL = 3
HMR_DIFFUSIVE_NONE = 0
HMR_MIDPOINT_SECOND_ORDER = 2
HMR_MIDPOINT_FOURTH_ORDER = 4
HMR_MIDPOINT_SIXTH_ORDER = 6
HMR_PRECISION_FAST = 0
HMR_PRECISION_EXACT = 1

# Every symbol include/hmr.h declares.
EXPORTS = [
    "hmr_config_default", "hmr_ctx_create", "hmr_ctx_destroy", "hmr_num_equations", "hmr_num_components",
    "hmr_num_ghosts", "hmr_num_patch_ghosts", "hmr_ctx_reserve", "hmr_read_counters", "hmr_conv_flux_source_patch",
    "hmr_rk_stage_patch", "hmr_rk_substep_patch", "hmr_fill_ghosts_patch", "hmr_level_create",
    "hmr_level_destroy", "hmr_level_bind_state", "hmr_level_set_periodic", "hmr_level_state",
    "hmr_level_substep", "hmr_level_step", "hmr_level_check", "hmr_level_barrier_diagnostic", "hmr_level_autotune", "hmr_level_set_launch",
    "hmr_rk_substep_patch_noalloc", "hmr_rk_substep_vjp_patch", "hmr_fill_ghosts_vjp_patch",
    "hmr_spectral_radius_patch", "hmr_level_step_cfl", "hmr_level_last_dt", "hmr_level_set_layout",
    "hmr_diff_flux_patch", "hmr_rk_stage_ns_patch", "hmr_coarsen_fluxsum_patch", "hmr_sync_fluxes_patch",
    "hmr_coarsen_patch", "hmr_refine_ghosts_patch", "hmr_level_substep_vjp", "hmr_level_fill_vjp",
    "hmr_level_set_vjp_budget", "hmr_level_set_work_split", "hmr_level_work_split", "hmr_set_dirichlet_values",
]


class Config(ctypes.Structure):
    _fields_ = [
        ("flow_model", ctypes.c_int),
        ("dim", ctypes.c_int),
        ("num_species", ctypes.c_int),
        ("species_gamma", ctypes.c_double * HMR_MAX_SPECIES),
        ("species_R", ctypes.c_double * HMR_MAX_SPECIES),
        ("convective_flux_reconstructor", ctypes.c_int),
        ("constant_p", ctypes.c_int),
        ("constant_q", ctypes.c_int),
        ("constant_C", ctypes.c_double),
        ("constant_alpha_tau", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("constant_Chi", ctypes.c_double),
        ("constant_epsilon", ctypes.c_double),
        ("grid_dx", ctypes.c_double * 3),
        ("diffusive_flux_reconstructor", ctypes.c_int),
        ("species_mu", ctypes.c_double),
        ("species_mu_v", ctypes.c_double),
        ("species_c_p", ctypes.c_double),
        ("species_Pr", ctypes.c_double),
        ("species_mu_kappa", ctypes.c_double),
    ]


class PatchGeometry(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("dx", ctypes.c_double * 3)]


DPP = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))   # double* const*
DPPP = ctypes.POINTER(DPP)                             # double* const* const*

_lib = None


class HmrError(RuntimeError):
    def __init__(self, where, code):
        names = {HMR_ERR_ARGUMENT: "HMR_ERR_ARGUMENT", HMR_ERR_UNSUPPORTED: "HMR_ERR_UNSUPPORTED",
                 HMR_ERR_NO_DEVICE: "HMR_ERR_NO_DEVICE", HMR_ERR_STATE: "HMR_ERR_STATE",
                 HMR_ERR_BARRIER: "HMR_ERR_BARRIER", HMR_ERR_CAPACITY: "HMR_ERR_CAPACITY"}
        super().__init__(f"{where} failed: {names.get(code, 'cudaError %d' % code)}")
        self.code = code


def check(where, code):
    if code != HMR_OK:
        raise HmrError(where, code)


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "or `python hamers_gb300/build.py`")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    cfgp = ctypes.POINTER(Config)
    gp = ctypes.POINTER(PatchGeometry)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    L.hmr_config_default.argtypes = [cfgp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.hmr_ctx_create.argtypes = [cfgp, ctypes.POINTER(vp)]
    L.hmr_ctx_destroy.argtypes = [vp]
    L.hmr_num_equations.argtypes = [vp]
    L.hmr_num_components.argtypes = [vp]
    L.hmr_num_ghosts.argtypes = [vp]
    L.hmr_num_patch_ghosts.argtypes = [vp]
    L.hmr_ctx_reserve.argtypes = [vp, gp]
    L.hmr_read_counters.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
    L.hmr_conv_flux_source_patch.argtypes = [vp, gp, DPP, ctypes.c_double, DPP, DPP, vp]
    L.hmr_rk_stage_patch.argtypes = [vp, gp, ctypes.c_int, dp, dp, dp, DPPP, DPPP, DPPP, DPP, DPP, DPP, vp]
    L.hmr_rk_substep_patch.argtypes = [vp, gp, ctypes.c_int, dp, ctypes.c_double, DPPP, ctypes.c_double, DPP, vp]
    L.hmr_fill_ghosts_patch.argtypes = [vp, gp, DPP, ip, vp]
    L.hmr_level_create.argtypes = [vp, ctypes.c_int, gp, ctypes.POINTER(vp)]
    L.hmr_level_destroy.argtypes = [vp]
    L.hmr_level_bind_state.argtypes = [vp, ctypes.c_int, DPP]
    L.hmr_level_state.argtypes = [vp, ctypes.c_int, ctypes.c_int, DPP]
    L.hmr_level_substep.argtypes = [vp, ctypes.c_int, ctypes.c_double, vp]
    L.hmr_level_set_periodic.argtypes = [vp, ctypes.c_int, ip]
    L.hmr_level_check.argtypes = [vp]
    L.hmr_level_barrier_diagnostic.argtypes = [vp, ctypes.c_uint, ctypes.c_ulonglong]
    L.hmr_level_step.argtypes = [vp, ctypes.c_double, vp]
    L.hmr_level_autotune.argtypes = [vp, ctypes.c_double, ip, ip, vp]
    L.hmr_level_set_launch.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.hmr_rk_substep_patch_noalloc.argtypes = [cfgp, gp, ctypes.c_int, dp, ctypes.c_double, DPPP,
                                               ctypes.c_double, DPP, vp]
    L.hmr_rk_substep_vjp_patch.argtypes = [vp, gp, ctypes.c_int, dp, ctypes.c_double, DPPP, ctypes.c_double,
                                           DPP, DPPP, vp]
    L.hmr_fill_ghosts_vjp_patch.argtypes = [vp, gp, DPP, ip, vp]
    L.hmr_level_substep_vjp.argtypes = [vp, ctypes.c_int, ctypes.c_double, DPPP, ctypes.POINTER(DPPP), vp]
    L.hmr_level_fill_vjp.argtypes = [vp, DPPP, vp]
    L.hmr_set_dirichlet_values.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp]
    L.hmr_level_set_vjp_budget.argtypes = [vp, ctypes.c_ulonglong]
    L.hmr_level_set_work_split.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.hmr_level_work_split.argtypes = [vp, ip, ip]
    L.hmr_spectral_radius_patch.argtypes = [vp, gp, DPP, dp, vp]
    L.hmr_level_step_cfl.argtypes = [vp, ctypes.c_double, vp]
    L.hmr_level_last_dt.argtypes = [vp, dp]
    L.hmr_level_set_layout.argtypes = [vp, ip, ip, ip]
    L.hmr_diff_flux_patch.argtypes = [vp, gp, DPP, ctypes.c_double, DPP, vp]
    L.hmr_coarsen_fluxsum_patch.argtypes = [vp, gp, ip, gp, ip, ip, DPP, DPP, vp]
    L.hmr_sync_fluxes_patch.argtypes = [vp, gp, DPP, DPP, DPP, DPP, vp]
    L.hmr_coarsen_patch.argtypes = [vp, gp, ip, gp, ip, ip, DPP, DPP, vp]
    L.hmr_refine_ghosts_patch.argtypes = [vp, gp, ip, gp, ip, ip, DPP, DPP, ctypes.c_double, DPP, vp]
    L.hmr_rk_stage_ns_patch.argtypes = [vp, gp, ctypes.c_int, dp, dp, dp, DPPP, DPPP, DPPP, DPPP, DPP, DPP, DPP,
                                        DPP, vp]
    for name in EXPORTS:
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def ptr_array(ptrs):
    """double* const* from a list of integer device addresses."""
    arr = (ctypes.POINTER(ctypes.c_double) * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = ctypes.cast(ctypes.c_void_p(int(p)), ctypes.POINTER(ctypes.c_double))
    return ctypes.cast(arr, DPP), arr


def ptr_array3(lists):
    """double* const* const* const* from a list of lists of pointer lists."""
    inner = [ptr_array2(p) for p in lists]
    outer = (DPPP * len(inner))()
    for i, (pp, _) in enumerate(inner):
        outer[i] = pp
    return ctypes.cast(outer, ctypes.POINTER(DPPP)), (outer, inner)


def ptr_array2(lists):
    """double* const* const* from a list of pointer lists."""
    inner = [ptr_array(p) for p in lists]
    outer = (DPP * len(inner))()
    for i, (pp, _) in enumerate(inner):
        outer[i] = pp
    return ctypes.cast(outer, DPPP), (outer, inner)
