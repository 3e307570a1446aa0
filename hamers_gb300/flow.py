"""Host-side mirror of the reference's patch-level interface, over the C ABI.

Names follow HAMeRS:
  FlowModel                     -- FlowModelManager + ideal-gas mixing rules
                                   (include/flow/flow_models/FlowModel.hpp:59-572)
  ConvectiveFluxReconstructor   -- ConvectiveFluxReconstructorManager product
                                   (include/flow/convective_flux_reconstructors/ConvectiveFluxReconstructor.hpp:23-124)
  Euler                         -- the RungeKuttaPatchStrategy of src/apps/Euler/Euler.cpp
                                   (computeFluxesAndSourcesOnPatch :904, advanceSingleStepOnPatch :1003)
  DiffusiveFluxReconstructor    -- DiffusiveFluxReconstructorMidpoint (second / fourth / sixth order)
                                   (src/flow/diffusive_flux_reconstructors/midpoint/DiffusiveFluxReconstructorMidpoint.cpp:38)
  NavierStokes                  -- the patch strategy of src/apps/Navier-Stokes/NavierStokes.cpp
                                   (computeFluxesAndSourcesOnPatch :1104, advanceSingleStepOnPatch :1249)
  RungeKuttaLevelIntegrator     -- SSPRK3 stage loop (RungeKuttaLevelIntegrator.cpp:1672-1748)
  BatchedLevel                  -- all patches of a level per substep in one persistent kernel

Patch data are torch tensors on the CUDA device in SAMRAI layout:
conserved variables (ncomp, G2, G1, G0) over the ghost box (ghost width 4; 5 with the
sixth-order diffusive flux, getPatchNumberOfGhostCells()),
face fluxes [axis] -> (neq, ...) and sources (neq, n2, n1, n0).  torch is used
for device memory and streams only; every computation runs in libhmr_gb300.so.
Errors from the library raise HmrError (argument errors are raised before any
work is queued, mirroring TBOX_ERROR in the reference).
"""
import ctypes

import torch

from . import _lib as L

GHOST = 4

_FLOW_MODELS = {
    "SINGLE_SPECIES": L.HMR_SINGLE_SPECIES,
    "FOUR_EQN_CONSERVATIVE": L.HMR_FOUR_EQN_CONSERVATIVE,
    "FIVE_EQN_ALLAIRE": L.HMR_FIVE_EQN_ALLAIRE,
}
_RECONSTRUCTORS = {
    "WCNS5_JS_HLLC_HLL": L.HMR_WCNS5_JS_HLLC_HLL,
    "WCNS6_LD_HLLC_HLL": L.HMR_WCNS6_LD_HLLC_HLL,
    "WCNS5_Z_HLLC_HLL": L.HMR_WCNS5_Z_HLLC_HLL,
    "WCNS6_CU_M2_HLLC_HLL": L.HMR_WCNS6_CU_M2_HLLC_HLL,
}

_DIFFUSIVE = {
    "MIDPOINT_SECOND_ORDER": L.HMR_MIDPOINT_SECOND_ORDER,
    "MIDPOINT_FOURTH_ORDER": L.HMR_MIDPOINT_FOURTH_ORDER,
    "MIDPOINT_SIXTH_ORDER": L.HMR_MIDPOINT_SIXTH_ORDER,
}

# SSPRK(3,3), RungeKuttaLevelIntegrator.cpp:3909-3927
RK3_ALPHA = [[1.0], [3.0 / 4.0, 1.0 / 4.0], [1.0 / 3.0, 0.0, 2.0 / 3.0]]

# ghost-fill mode per axis (hmr_fill_mode of include/hmr.h)
FILL_ZERO_GRADIENT, FILL_PERIODIC, FILL_PROVIDED, FILL_REFLECT, FILL_DIRICHLET, FILL_SYMMETRY = 0, 1, 2, 3, 4, 5
RK3_BETA = [[1.0], [0.0, 1.0 / 4.0], [0.0, 0.0, 2.0 / 3.0]]
RK3_GAMMA = [[1.0 / 6.0], [0.0, 1.0 / 6.0], [0.0, 0.0, 2.0 / 3.0]]


def _stream_ptr(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


class FlowModel:
    """Flow model selection: 'SINGLE_SPECIES', 'FOUR_EQN_CONSERVATIVE' or 'FIVE_EQN_ALLAIRE', ideal gas.

    transport (Navier-Stokes, single species): the reference's mixing-rule keys
      species_mu    Equation_of_shear_viscosity_mixing_rules (equation_of_shear_viscosity CONSTANT)
      species_mu_v  Equation_of_bulk_viscosity_mixing_rules (CONSTANT; default 0)
      species_c_p, species_Pr
                    Equation_of_thermal_conductivity_mixing_rules (PRANDTL: kappa = c_p mu/Pr,
                    with that block's own species_mu, given here as species_mu_kappa and
                    defaulting to species_mu)
    """

    def __init__(self, flow_model, dim, species_gamma, species_R=None, transport=None):
        if flow_model not in _FLOW_MODELS:
            raise ValueError(f"unknown flow model {flow_model!r}")
        self.name = flow_model
        self.model = _FLOW_MODELS[flow_model]
        self.dim = int(dim)
        self.species_gamma = [float(g) for g in species_gamma]
        self.num_species = len(self.species_gamma)
        self.species_R = [float(r) for r in (species_R or [1.0] * self.num_species)]
        self.transport = None
        if transport is not None:
            t = dict(transport)
            self.transport = {
                "species_mu": float(t["species_mu"]),
                "species_mu_v": float(t.get("species_mu_v", 0.0)),
                "species_c_p": float(t["species_c_p"]),
                "species_Pr": float(t["species_Pr"]),
                "species_mu_kappa": float(t.get("species_mu_kappa", t["species_mu"])),
            }

    def getNumberOfEquations(self):
        if self.model == L.HMR_SINGLE_SPECIES:
            return self.dim + 2
        if self.model == L.HMR_FOUR_EQN_CONSERVATIVE:
            return self.num_species + self.dim + 1
        return self.dim + 2 * self.num_species

    def getNumberOfComponents(self):
        return self.getNumberOfEquations() + (1 if self.model == L.HMR_FIVE_EQN_ALLAIRE else 0)


class Patch:
    """One patch: interior size n, spacing dx, conserved variables on the ghost box."""

    def __init__(self, n, dx, data):
        self.n = [int(v) for v in n]
        self.dx = [float(v) for v in dx]
        self.data = data

    def geometry(self):
        g = L.PatchGeometry()
        for d in range(3):
            g.n[d] = self.n[d] if d < len(self.n) else 1
            g.dx[d] = self.dx[d] if d < len(self.dx) else 1.0
        return g


def _comp_ptrs(t, ncomp):
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError("patch arrays must be contiguous float64 CUDA tensors")
    if t.shape[0] < ncomp:
        raise ValueError(f"expected {ncomp} components, got {t.shape[0]}")
    return [t[e].data_ptr() for e in range(ncomp)]


def _state_ptrs(rec, n, t):
    """Component pointers of a conserved-variable array over the ghost box of a patch of n
    interior cells; the library reads and writes the whole box, so its extent is checked
    against the context's ghost width (4, or 5 with the sixth-order diffusive flux)."""
    dim = rec.flow_model.dim
    gh = rec.ghosts
    want = tuple(int(n[a]) + 2 * gh if a < dim else 1 for a in (2, 1, 0))
    if tuple(t.shape[1:]) != want:
        raise ValueError(f"patch array of shape {tuple(t.shape)}: expected (ncomp,) + {want} "
                         f"(interior {list(n)[:dim]} with {gh} ghost cells per side)")
    return _comp_ptrs(t, rec.ncomp)


class ConvectiveFluxReconstructor:
    """WCNS5-JS / WCNS6-LD / WCNS5-Z / WCNS6-CU-M2 + HLLC-HLL reconstructor behind the C ABI.

    db keys follow the reference's input database: constant_p, constant_q,
    constant_C, constant_alpha_tau (ConvectiveFluxReconstructorWCNS6-LD-HLLC-HLL.cpp:343-361),
    constant_Chi, constant_epsilon (ConvectiveFluxReconstructorWCNS6-CU-M2-HLLC-HLL.cpp:252-270);
    keys left out take the scheme's defaults.
    grid_geometry: the grid geometry (an object with getDx(), or the spacing itself) of
    the coarsest level, as the reference passes CartesianGridGeometry to the reconstructor;
    WCNS6-CU-M2 scales its weights by that spacing and needs it, the others ignore it.
    precision: 'fast' (default, <= 1e-12 relative; <= 2e-15 c/|u_n| for the flux components
    proportional to a normal velocity below 1e-3 of the sound speed) or 'exact' (bitwise to the
    reference order).
    """

    def __init__(self, name, flow_model, db=None, precision="fast", grid_geometry=None,
                 diffusive_flux_reconstructor=None):
        if name not in _RECONSTRUCTORS:
            raise ValueError(f"unknown convective flux reconstructor {name!r}")
        if diffusive_flux_reconstructor is not None:
            if diffusive_flux_reconstructor not in _DIFFUSIVE:
                raise ValueError(f"unknown diffusive flux reconstructor {diffusive_flux_reconstructor!r}")
            if flow_model.transport is None:
                raise ValueError("a diffusive flux reconstructor needs the flow model's transport properties")
        db = db or {}
        lib = L.load()
        cfg = L.Config()
        L.check("hmr_config_default", lib.hmr_config_default(
            ctypes.byref(cfg), flow_model.model, _RECONSTRUCTORS[name], flow_model.dim, flow_model.num_species))
        for s in range(flow_model.num_species):
            cfg.species_gamma[s] = flow_model.species_gamma[s]
            cfg.species_R[s] = flow_model.species_R[s]
        for key, conv in (("constant_p", int), ("constant_q", int), ("constant_C", float),
                          ("constant_alpha_tau", float), ("constant_Chi", float), ("constant_epsilon", float)):
            if key in db:
                setattr(cfg, key, conv(db[key]))
        if grid_geometry is not None:
            dx = grid_geometry.getDx() if hasattr(grid_geometry, "getDx") else grid_geometry
            for d, v in enumerate(list(dx)[:3]):
                cfg.grid_dx[d] = float(v)
        elif name == "WCNS6_CU_M2_HLLC_HLL":
            raise ValueError("WCNS6_CU_M2_HLLC_HLL needs grid_geometry (its weights use the grid spacing)")
        if diffusive_flux_reconstructor is not None:
            cfg.diffusive_flux_reconstructor = _DIFFUSIVE[diffusive_flux_reconstructor]
            for key, v in flow_model.transport.items():
                setattr(cfg, key, v)
        self.diffusive = diffusive_flux_reconstructor
        cfg.precision = L.HMR_PRECISION_EXACT if precision == "exact" else L.HMR_PRECISION_FAST
        self.flow_model = flow_model
        self.name = name
        self.precision = precision
        self._lib = lib
        ctx = ctypes.c_void_p()
        L.check("hmr_ctx_create", lib.hmr_ctx_create(ctypes.byref(cfg), ctypes.byref(ctx)))
        self.ctx = ctx
        self.neq = lib.hmr_num_equations(ctx)
        self.ncomp = lib.hmr_num_components(ctx)
        self.ghosts = lib.hmr_num_patch_ghosts(ctx)

    def close(self):
        if self.ctx:
            self._lib.hmr_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def getConvectiveFluxNumberOfGhostCells(self):
        return self._lib.hmr_num_ghosts(self.ctx)

    def getPatchNumberOfGhostCells(self):
        """Ghost width of the patch arrays this context reads: 4, or 5 with the sixth-order
        diffusive flux (NavierStokes.cpp:317-349 takes the larger of the two widths)."""
        return self._lib.hmr_num_patch_ghosts(self.ctx)

    def setDirichletValues(self, axis, side, values):
        """Conservative values (ncomp) that ghost cells beyond the FILL_DIRICHLET side `side`
        (0 low, 1 high) of `axis` take in every fill of this context (the reference's DIRICHLET
        boundary data, EulerBoundaryConditions::readDirichletBoundaryDataEntry, already
        converted to conservative variables)."""
        v = [float(x) for x in values]
        if len(v) != self.ncomp:
            raise ValueError(f"expected {self.ncomp} conservative values, got {len(v)}")
        arr = (ctypes.c_double * len(v))(*v)
        L.check("hmr_set_dirichlet_values", self._lib.hmr_set_dirichlet_values(
            self.ctx, int(axis), int(side), ctypes.cast(arr, ctypes.POINTER(ctypes.c_double))))

    def allocateFlux(self, patch):
        dim = self.flow_model.dim
        n3 = list(patch.n) + [1] * (3 - len(patch.n))
        out = []
        for a in range(dim):
            e = [n3[d] + (1 if d == a else 0) for d in range(3)]
            out.append(torch.zeros((self.neq, e[2], e[1], e[0]), dtype=torch.float64, device=patch.data.device))
        return out

    def allocateSource(self, patch):
        n3 = list(patch.n) + [1] * (3 - len(patch.n))
        return torch.zeros((self.neq, n3[2], n3[1], n3[0]), dtype=torch.float64, device=patch.data.device)

    def reserve(self, patch):
        g = patch.geometry()
        L.check("hmr_ctx_reserve", self._lib.hmr_ctx_reserve(self.ctx, ctypes.byref(g)))

    def computeConvectiveFluxAndSourceOnPatch(self, patch, convective_flux, source, dt, stream=None):
        """dt-scaled face fluxes (overwritten) and advective source (+=)."""
        g = patch.geometry()
        q, _k1 = L.ptr_array(_state_ptrs(self, patch.n, patch.data))
        fptrs = []
        for a in range(self.flow_model.dim):
            fptrs += _comp_ptrs(convective_flux[a], self.neq)
        f, _k2 = L.ptr_array(fptrs)
        s, _k3 = L.ptr_array(_comp_ptrs(source, self.neq))
        L.check("hmr_conv_flux_source_patch", self._lib.hmr_conv_flux_source_patch(
            self.ctx, ctypes.byref(g), q, float(dt), f, s, _stream_ptr(stream)))

    def readCounters(self, reset=True):
        out = (ctypes.c_ulonglong * 2)()
        L.check("hmr_read_counters", self._lib.hmr_read_counters(self.ctx, out, 1 if reset else 0))
        return int(out[0]), int(out[1])


class Euler:
    """Patch strategy: flux + RK stage on one patch (src/apps/Euler/Euler.cpp)."""

    def __init__(self, reconstructor):
        self.rec = reconstructor
        self._lib = reconstructor._lib

    def computeFluxesAndSourcesOnPatch(self, patch, flux, source, dt, stream=None):
        source.zero_()   # Euler.cpp:916-932
        self.rec.computeConvectiveFluxAndSourceOnPatch(patch, flux, source, dt, stream)

    def advanceSingleStepOnPatch(self, patch, alpha, beta, gamma, Q_int, F_int, S_int,
                                 flux_acc=None, source_acc=None, stream=None):
        """Q = sum alpha_n Q_int[n] + beta_n (-div F_int[n] + S_int[n]) written into patch.data."""
        rec = self.rec
        nc = len(alpha)
        g = patch.geometry()
        a = (ctypes.c_double * nc)(*alpha)
        b = (ctypes.c_double * nc)(*beta)
        c = (ctypes.c_double * nc)(*gamma)
        qi, k1 = L.ptr_array2([_state_ptrs(rec, patch.n, t) for t in Q_int])
        fi, k2 = L.ptr_array2([sum((_comp_ptrs(f, rec.neq) for f in F), []) for F in F_int])
        si, k3 = L.ptr_array2([_comp_ptrs(t, rec.neq) for t in S_int])
        qo, k4 = L.ptr_array(_state_ptrs(rec, patch.n, patch.data))
        fa = sa = None
        keep = []
        if flux_acc is not None:
            fa, k5 = L.ptr_array(sum((_comp_ptrs(f, rec.neq) for f in flux_acc), []))
            sa, k6 = L.ptr_array(_comp_ptrs(source_acc, rec.neq))
            keep += [k5, k6]
        L.check("hmr_rk_stage_patch", self._lib.hmr_rk_stage_patch(
            rec.ctx, ctypes.byref(g), nc, a, b, c, qi, fi, si, qo, fa, sa, _stream_ptr(stream)))

    def synchronizeFluxes(self, patch, flux, source, stream=None, diffusive_flux=None):
        """Euler::synchronizeFluxes (Euler.cpp:1682): the coarse step redone from the old state in
        patch.data with the time-integrated (gamma-accumulated, reflux-corrected) fluxes."""
        rec = self.rec
        g = patch.geometry()
        q, k1 = L.ptr_array(_state_ptrs(rec, patch.n, patch.data))
        f, k2 = L.ptr_array(sum((_comp_ptrs(t, rec.neq) for t in flux[:rec.flow_model.dim]), []))
        d = None
        if diffusive_flux is not None:
            d, k3 = L.ptr_array(sum((_comp_ptrs(t, rec.neq) for t in diffusive_flux[:rec.flow_model.dim]), []))
        s_, k4 = L.ptr_array(_comp_ptrs(source, rec.neq))
        L.check("hmr_sync_fluxes_patch", self._lib.hmr_sync_fluxes_patch(
            rec.ctx, ctypes.byref(g), q, f, d, s_, _stream_ptr(stream)))

    def fillGhosts(self, patch, periodic, stream=None):
        """Ghost fill of one patch, mode per axis: FILL_ZERO_GRADIENT (0, the extrapolation
        boundary), FILL_PERIODIC (1), FILL_PROVIDED (2, left as supplied), FILL_REFLECT (3, a
        slip wall: mirror image with the normal momentum negated; needs >= 4 cells on the axis),
        FILL_DIRICHLET (4, the values of ConvectiveFluxReconstructor.setDirichletValues) or
        FILL_SYMMETRY (5, the mirror image of every variable as it is)."""
        g = patch.geometry()
        q, _k = L.ptr_array(_state_ptrs(self.rec, patch.n, patch.data))
        per = (ctypes.c_int * 3)(*(list(periodic) + [0] * (3 - len(periodic))))
        L.check("hmr_fill_ghosts_patch", self._lib.hmr_fill_ghosts_patch(
            self.rec.ctx, ctypes.byref(g), q, per, _stream_ptr(stream)))

    def substep(self, patch, stage, Q_int, dt, out, stream=None):
        """Fused flux + update of SSPRK3 stage `stage`: out = sum alpha Q_int + beta (-div F(Q_int[stage]) + S)."""
        rec = self.rec
        g = patch.geometry()
        alpha = (ctypes.c_double * 3)(*(RK3_ALPHA[stage] + [0.0] * (2 - stage)))
        qi, k1 = L.ptr_array2([_state_ptrs(rec, patch.n, t) for t in Q_int[:stage + 1]])
        qo, k2 = L.ptr_array(_state_ptrs(rec, patch.n, out))
        L.check("hmr_rk_substep_patch", self._lib.hmr_rk_substep_patch(
            rec.ctx, ctypes.byref(g), int(stage), alpha, RK3_BETA[stage][stage], qi, float(dt), qo,
            _stream_ptr(stream)))


    def substepVJP(self, patch, stage, Q_int, dt, Qbar_out, Qbar_int, stream=None):
        """Adjoint of substep(): accumulates into Qbar_int[n] (n <= stage, ghost boxes) the
        vector-Jacobian product of Qbar_out with the substep at the stage states Q_int."""
        rec = self.rec
        g = patch.geometry()
        alpha = (ctypes.c_double * 3)(*(RK3_ALPHA[stage] + [0.0] * (2 - stage)))
        qi, k1 = L.ptr_array2([_state_ptrs(rec, patch.n, t) for t in Q_int[:stage + 1]])
        qb, k2 = L.ptr_array(_state_ptrs(rec, patch.n, Qbar_out))
        qbi, k3 = L.ptr_array2([_state_ptrs(rec, patch.n, t) for t in Qbar_int[:stage + 1]])
        L.check("hmr_rk_substep_vjp_patch", self._lib.hmr_rk_substep_vjp_patch(
            rec.ctx, ctypes.byref(g), int(stage), alpha, RK3_BETA[stage][stage], qi, float(dt), qb, qbi,
            _stream_ptr(stream)))

    def spectralRadius(self, patch, out=None, stream=None):
        """Max over the interior of sum_d (|u_d| + c)/dx_d (Euler::computeSpectralRadiusesAndStableDtOnPatch);
        max-reduced into the device scalar `out` if given (running max), else returned (synchronises)."""
        g = patch.geometry()
        q, _k = L.ptr_array(_state_ptrs(self.rec, patch.n, patch.data))
        dst = out if out is not None else torch.zeros(1, dtype=torch.float64, device=patch.data.device)
        L.check("hmr_spectral_radius_patch", self._lib.hmr_spectral_radius_patch(
            self.rec.ctx, ctypes.byref(g), q, ctypes.cast(ctypes.c_void_p(dst.data_ptr()), ctypes.POINTER(ctypes.c_double)),
            _stream_ptr(stream)))
        return None if out is not None else float(dst.item())

    def fillGhostsVJP(self, patch, periodic, stream=None):
        """Adjoint of fillGhosts() applied to the adjoint array patch.data."""
        g = patch.geometry()
        q, _k = L.ptr_array(_state_ptrs(self.rec, patch.n, patch.data))
        per = (ctypes.c_int * 3)(*(list(periodic) + [0] * (3 - len(periodic))))
        L.check("hmr_fill_ghosts_vjp_patch", self._lib.hmr_fill_ghosts_vjp_patch(
            self.rec.ctx, ctypes.byref(g), q, per, _stream_ptr(stream)))


class DiffusiveFluxReconstructor:
    """MIDPOINT_SECOND_ORDER / _FOURTH_ORDER / _SIXTH_ORDER diffusive flux behind the C ABI.
    With the sixth order every patch array of the context carries 5 ghost cells
    (ConvectiveFluxReconstructor.getPatchNumberOfGhostCells).

    It runs in the context of a ConvectiveFluxReconstructor created with
    diffusive_flux_reconstructor=<name> (one context holds the whole
    Navier-Stokes configuration, so that the fused substep can use both)."""

    def __init__(self, convective):
        if convective.diffusive is None:
            raise ValueError("the convective reconstructor was created without a diffusive flux reconstructor")
        self.conv = convective
        self.name = convective.diffusive
        self._lib = convective._lib

    def getDiffusiveFluxNumberOfGhostCells(self):
        return {"MIDPOINT_SECOND_ORDER": 1, "MIDPOINT_FOURTH_ORDER": 3, "MIDPOINT_SIXTH_ORDER": 5}[self.name]

    def computeDiffusiveFluxOnPatch(self, patch, diffusive_flux, dt, stream=None):
        """dt-scaled diffusive face fluxes (overwritten), same layout as the convective flux."""
        rec = self.conv
        g = patch.geometry()
        q, _k1 = L.ptr_array(_state_ptrs(rec, patch.n, patch.data))
        f, _k2 = L.ptr_array(sum((_comp_ptrs(t, rec.neq) for t in diffusive_flux[:rec.flow_model.dim]), []))
        L.check("hmr_diff_flux_patch", self._lib.hmr_diff_flux_patch(
            rec.ctx, ctypes.byref(g), q, float(dt), f, _stream_ptr(stream)))


class NavierStokes(Euler):
    """Patch strategy of src/apps/Navier-Stokes/NavierStokes.cpp: convective + diffusive fluxes.

    The reconstructor's context carries the diffusive flux reconstructor; substep() is then
    NavierStokes's fused stage and RungeKuttaLevelIntegrator advances the Navier-Stokes
    equations."""

    def __init__(self, reconstructor):
        super().__init__(reconstructor)
        self.diff = DiffusiveFluxReconstructor(reconstructor)

    def computeFluxesAndSourcesOnPatch(self, patch, convective_flux, diffusive_flux, source, dt, stream=None):
        source.zero_()   # NavierStokes.cpp:1112-1126
        self.rec.computeConvectiveFluxAndSourceOnPatch(patch, convective_flux, source, dt, stream)
        self.diff.computeDiffusiveFluxOnPatch(patch, diffusive_flux, dt, stream)

    def advanceSingleStepOnPatch(self, patch, alpha, beta, gamma, Q_int, F_int, Fd_int, S_int,
                                 flux_acc=None, diff_flux_acc=None, source_acc=None, stream=None):
        """Q = sum alpha_n Q_int[n] + beta_n (-div (F_int[n] + Fd_int[n]) + S_int[n]) into patch.data."""
        rec = self.rec
        nc = len(alpha)
        g = patch.geometry()
        a = (ctypes.c_double * nc)(*alpha)
        b = (ctypes.c_double * nc)(*beta)
        c = (ctypes.c_double * nc)(*gamma)
        qi, k1 = L.ptr_array2([_state_ptrs(rec, patch.n, t) for t in Q_int])
        fi, k2 = L.ptr_array2([sum((_comp_ptrs(f, rec.neq) for f in F), []) for F in F_int])
        di, k3 = L.ptr_array2([sum((_comp_ptrs(f, rec.neq) for f in F), []) for F in Fd_int])
        si, k4 = L.ptr_array2([_comp_ptrs(t, rec.neq) for t in S_int])
        qo, k5 = L.ptr_array(_state_ptrs(rec, patch.n, patch.data))
        fa = da = sa = None
        keep = []
        if flux_acc is not None:
            fa, k6 = L.ptr_array(sum((_comp_ptrs(f, rec.neq) for f in flux_acc), []))
            da, k7 = L.ptr_array(sum((_comp_ptrs(f, rec.neq) for f in diff_flux_acc), []))
            sa, k8 = L.ptr_array(_comp_ptrs(source_acc, rec.neq))
            keep += [k6, k7, k8]
        L.check("hmr_rk_stage_ns_patch", self._lib.hmr_rk_stage_ns_patch(
            rec.ctx, ctypes.byref(g), nc, a, b, c, qi, fi, di, si, qo, fa, da, sa, _stream_ptr(stream)))


def _ivec(v, fill=0):
    return (ctypes.c_int * 3)(*((list(v) + [fill] * 3)[:3]))


def coarsenFluxSum(reconstructor, coarse, coarse_lo, fine, fine_lo, ratio, fine_flux, coarse_flux, stream=None):
    """Flux-sum coarsening of refluxing (RungeKuttaLevelIntegrator.cpp:2140-2160): on the outer
    sides of the fine patch, coarse faces take the mean of the fine faces they cover."""
    rec = reconstructor
    dim = rec.flow_model.dim
    gc, gf = coarse.geometry(), fine.geometry()
    ff, k1 = L.ptr_array(sum((_comp_ptrs(t, rec.neq) for t in fine_flux[:dim]), []))
    fc, k2 = L.ptr_array(sum((_comp_ptrs(t, rec.neq) for t in coarse_flux[:dim]), []))
    L.check("hmr_coarsen_fluxsum_patch", rec._lib.hmr_coarsen_fluxsum_patch(
        rec.ctx, ctypes.byref(gc), _ivec(coarse_lo), ctypes.byref(gf), _ivec(fine_lo), _ivec(ratio, 1),
        ff, fc, _stream_ptr(stream)))


def refineGhosts(reconstructor, fine, fine_lo, coarse, coarse_lo, ratio, coarse_old, coarse_new, theta,
                 stream=None):
    """Coarse-fine ghost cells of the fine patch from the coarse patch's states at the old and new
    time (coarse_old / coarse_new: ghost-box tensors, ghosts filled) at time fraction theta."""
    rec = reconstructor
    gf, gc = fine.geometry(), coarse.geometry()
    qo, k1 = L.ptr_array(_state_ptrs(rec, coarse.n, coarse_old))
    qn, k2 = L.ptr_array(_state_ptrs(rec, coarse.n, coarse_new))
    qf, k3 = L.ptr_array(_state_ptrs(rec, fine.n, fine.data))
    L.check("hmr_refine_ghosts_patch", rec._lib.hmr_refine_ghosts_patch(
        rec.ctx, ctypes.byref(gf), _ivec(fine_lo), ctypes.byref(gc), _ivec(coarse_lo), _ivec(ratio, 1),
        qo, qn, float(theta), qf, _stream_ptr(stream)))


def coarsenPatch(reconstructor, coarse, coarse_lo, fine, fine_lo, ratio, stream=None):
    """Coarsening of a fine patch's interior onto the coarse cells it covers (mean of the fine cells)."""
    rec = reconstructor
    gc, gf = coarse.geometry(), fine.geometry()
    qf, k1 = L.ptr_array(_state_ptrs(rec, fine.n, fine.data))
    qc, k2 = L.ptr_array(_state_ptrs(rec, coarse.n, coarse.data))
    L.check("hmr_coarsen_patch", rec._lib.hmr_coarsen_patch(
        rec.ctx, ctypes.byref(gc), _ivec(coarse_lo), ctypes.byref(gf), _ivec(fine_lo), _ivec(ratio, 1),
        qf, qc, _stream_ptr(stream)))


class RungeKuttaLevelIntegrator:
    """SSPRK3 on one patch with ghost fill between stages (per-patch form).

    advance(..., checkpoint_every=K) records the state every K steps;
    adjoint(Qbar) then runs the reverse sweep of that advance segment by
    segment, recomputing each segment's stage states from its checkpoint."""

    def __init__(self, euler, patch, periodic):
        self.euler = euler
        self.patch = patch
        self.periodic = list(periodic)
        self.stages = [torch.empty_like(patch.data) for _ in range(2)]
        self._record = None
        euler.rec.reserve(patch)

    def _step(self, Q0, Q1, Q2, dt, stream):
        p = self.patch
        views = [Patch(p.n, p.dx, Q) for Q in (Q0, Q1, Q2)]
        self.euler.fillGhosts(views[0], self.periodic, stream)
        self.euler.substep(views[0], 0, [Q0], dt, Q1, stream)
        self.euler.fillGhosts(views[1], self.periodic, stream)
        self.euler.substep(views[1], 1, [Q0, Q1], dt, Q2, stream)
        self.euler.fillGhosts(views[2], self.periodic, stream)
        self.euler.substep(views[2], 2, [Q0, Q1, Q2], dt, Q0, stream)

    def advance(self, dt, nsteps=1, stream=None, checkpoint_every=0):
        p = self.patch
        Q0, Q1, Q2 = p.data, self.stages[0], self.stages[1]
        if checkpoint_every:
            self._record = {"dt": dt, "nsteps": nsteps, "every": int(checkpoint_every),
                            "ckpt": {0: Q0.clone()}}
        for step in range(nsteps):
            self._step(Q0, Q1, Q2, dt, stream)
            if checkpoint_every and (step + 1) % checkpoint_every == 0 and step + 1 < nsteps:
                self._record["ckpt"][step + 1] = Q0.clone()
        self.euler.fillGhosts(Patch(p.n, p.dx, Q0), self.periodic, stream)

    def adjoint(self, Qbar, stream=None):
        """Reverse sweep of the last recorded advance.  Qbar: adjoint of the final state
        (ghost box); returns the adjoint of the initial state (ghost box, ghosts zero)."""
        rec = self._record
        if rec is None:
            raise RuntimeError("adjoint() needs a preceding advance(..., checkpoint_every=K)")
        p, eu, per, dt = self.patch, self.euler, self.periodic, rec["dt"]
        Xb = Qbar.clone()
        eu.fillGhostsVJP(Patch(p.n, p.dx, Xb), per, stream)          # final ghost fill
        starts = sorted(rec["ckpt"])
        ends = starts[1:] + [rec["nsteps"]]
        for s0, s1 in reversed(list(zip(starts, ends))):
            # recompute the segment, keeping every step's ghost-filled stage states
            X = rec["ckpt"][s0].clone()
            S1, S2 = torch.empty_like(X), torch.empty_like(X)
            saved = []
            for _ in range(s0, s1):
                views = [Patch(p.n, p.dx, Q) for Q in (X, S1, S2)]
                eu.fillGhosts(views[0], per, stream)
                eu.substep(views[0], 0, [X], dt, S1, stream)
                eu.fillGhosts(views[1], per, stream)
                eu.substep(views[1], 1, [X, S1], dt, S2, stream)
                eu.fillGhosts(views[2], per, stream)
                saved.append((X.clone(), S1.clone(), S2.clone()))
                eu.substep(views[2], 2, [X, S1, S2], dt, X, stream)
            for X0, X1, X2 in reversed(saved):
                view = Patch(p.n, p.dx, X0)
                Xn, B1, B2 = torch.zeros_like(Xb), torch.zeros_like(Xb), torch.zeros_like(Xb)
                eu.substepVJP(view, 2, [X0, X1, X2], dt, Xb, [Xn, B1, B2], stream)
                eu.fillGhostsVJP(Patch(p.n, p.dx, B2), per, stream)
                eu.substepVJP(view, 1, [X0, X1], dt, B2, [Xn, B1], stream)
                eu.fillGhostsVJP(Patch(p.n, p.dx, B1), per, stream)
                eu.substepVJP(view, 0, [X0], dt, B1, [Xn], stream)
                eu.fillGhostsVJP(Patch(p.n, p.dx, Xn), per, stream)
                Xb = Xn
        return Xb


class _DeviceArray:
    """A device FP64 array (pointer + shape) exposed through __cuda_array_interface__."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(int(v) for v in shape), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 3}


class BatchedLevel:
    """Every patch of a level advanced by one persistent kernel per SSPRK3 substep."""

    def __init__(self, reconstructor, geometries):
        self.rec = reconstructor
        self._lib = reconstructor._lib
        n = len(geometries)
        arr = (L.PatchGeometry * n)()
        self.shapes = []
        dim = reconstructor.flow_model.dim
        for i, (nn, dx) in enumerate(geometries):
            for d in range(3):
                arr[i].n[d] = nn[d] if d < dim else 1
                arr[i].dx[d] = dx[d] if d < dim else 1.0
            gh = reconstructor.getPatchNumberOfGhostCells()
            G = [nn[d] + 2 * gh if d < dim else 1 for d in range(3)]
            self.shapes.append((reconstructor.ncomp, G[2], G[1], G[0]))
        lv = ctypes.c_void_p()
        L.check("hmr_level_create", self._lib.hmr_level_create(reconstructor.ctx, n, arr, ctypes.byref(lv)))
        self.level = lv
        self.npatch = n
        self._bound = {}
        self._record = None

    def close(self):
        if self.level:
            self._lib.hmr_level_destroy(self.level)
            self.level = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind(self, patch, data):
        """Binds a patch's conserved-variable tensor (ncomp, G2, G1, G0) as its slot-0 state."""
        if tuple(data.shape) != self.shapes[patch]:
            raise ValueError(f"patch {patch}: expected shape {self.shapes[patch]}, got {tuple(data.shape)}")
        q, _k = L.ptr_array(_comp_ptrs(data, self.rec.ncomp))
        L.check("hmr_level_bind_state", self._lib.hmr_level_bind_state(self.level, int(patch), q))
        self._bound[patch] = data

    def _slot_views(self, patch, slot):
        """Writable tensor views, one per component, of a patch's stage-`slot` state."""
        return [torch.as_tensor(_DeviceArray(ptr, self.shapes[patch][1:]), device="cuda")
                for ptr in self.state_pointers(patch, slot)]

    def _load_slot(self, patch, slot, data):
        for e, v in enumerate(self._slot_views(patch, slot)):
            v.copy_(data[e])

    def state_pointers(self, patch, slot=0):
        arr = (ctypes.POINTER(ctypes.c_double) * self.rec.ncomp)()
        L.check("hmr_level_state", self._lib.hmr_level_state(
            self.level, int(patch), int(slot), ctypes.cast(arr, L.DPP)))
        return [ctypes.cast(arr[e], ctypes.c_void_p).value for e in range(self.rec.ncomp)]

    def state(self, patch, slot):
        """Tensor view (ncomp, G2, G1, G0) of a patch's stage-`slot` state (slot 0: the bound
        tensor; slots 1, 2: the intermediate stage states owned by the level)."""
        ptrs = self.state_pointers(patch, slot)
        comps = [torch.as_tensor(_DeviceArray(ptr, self.shapes[patch][1:]), device="cuda") for ptr in ptrs]
        return torch.stack(comps)

    def substep(self, stage, dt, stream=None):
        L.check("hmr_level_substep", self._lib.hmr_level_substep(self.level, int(stage), float(dt),
                                                                 _stream_ptr(stream)))

    def substepVJP(self, stage, dt, Qbar_out, Qbar_int, stream=None):
        """Adjoint of substep(stage, dt) over every patch, batched: for each patch p accumulates
        into Qbar_int[p][n] (n <= stage, ghost-box tensors) the vector-Jacobian product of
        Qbar_out[p] with the substep at the level's stage states (as the forward left them).
        Bitwise the per-patch Euler.substepVJP of each patch."""
        nc = self.rec.ncomp
        qb, k1 = L.ptr_array2([_comp_ptrs(t, nc) for t in Qbar_out])
        qbi, k2 = L.ptr_array3([[_comp_ptrs(t, nc) for t in slots[:stage + 1]] for slots in Qbar_int])
        L.check("hmr_level_substep_vjp", self._lib.hmr_level_substep_vjp(
            self.level, int(stage), float(dt), qb, qbi, _stream_ptr(stream)))

    def fillGhostsVJP(self, Qbar, stream=None):
        """Adjoint of the level's ghost fill (the exchange with the layout's physical faces, or
        each patch's own fill) applied to the adjoint tensors Qbar[p] (ghost boxes)."""
        nc = self.rec.ncomp
        qb, k1 = L.ptr_array2([_comp_ptrs(t, nc) for t in Qbar])
        L.check("hmr_level_fill_vjp", self._lib.hmr_level_fill_vjp(self.level, qb, _stream_ptr(stream)))

    def advance(self, dt, nsteps=1, stream=None, checkpoint_every=0):
        """nsteps level steps; with checkpoint_every=K the bound states are recorded every K
        steps for adjoint()."""
        if checkpoint_every:
            self._record = {"dt": dt, "nsteps": nsteps,
                            "ckpt": {0: [self._bound[p].clone() for p in range(self.npatch)]}}
        for step in range(nsteps):
            self.step(dt, stream)
            if checkpoint_every and (step + 1) % checkpoint_every == 0 and step + 1 < nsteps:
                self._record["ckpt"][step + 1] = [self._bound[p].clone() for p in range(self.npatch)]

    def adjoint(self, Qbar, stream=None):
        """Reverse sweep of the last recorded advance over the whole level: Qbar[p], the adjoint
        of patch p's final state (ghost box, interior read); returns the adjoints of the initial
        states (ghost boxes, the filled ghosts zero).  Each checkpoint segment is recomputed
        keeping every step's ghost-filled stage states, which are loaded back into the level's
        slots for the batched substep VJPs.  Overwrites the bound states."""
        rec = self._record
        if rec is None:
            raise RuntimeError("adjoint() needs a preceding advance(..., checkpoint_every=K)")
        np_, dt = self.npatch, rec["dt"]
        Xb = [q.clone() for q in Qbar]
        starts = sorted(rec["ckpt"])
        ends = starts[1:] + [rec["nsteps"]]
        for s0, s1 in reversed(list(zip(starts, ends))):
            for p in range(np_):
                self._bound[p].copy_(rec["ckpt"][s0][p])
            saved = []
            for _ in range(s0, s1):
                self.substep(0, dt, stream)
                X0 = [self._bound[p].clone() for p in range(np_)]
                self.substep(1, dt, stream)
                X1 = [torch.stack(self._slot_views(p, 1)).clone() for p in range(np_)]
                self.substep(2, dt, stream)
                X2 = [torch.stack(self._slot_views(p, 2)).clone() for p in range(np_)]
                saved.append((X0, X1, X2))
            for X0, X1, X2 in reversed(saved):
                for p in range(np_):
                    self._bound[p].copy_(X0[p])
                    self._load_slot(p, 1, X1[p])
                    self._load_slot(p, 2, X2[p])
                Xn = [torch.zeros_like(x) for x in Xb]
                B1 = [torch.zeros_like(x) for x in Xb]
                B2 = [torch.zeros_like(x) for x in Xb]
                self.substepVJP(2, dt, Xb, [[Xn[p], B1[p], B2[p]] for p in range(np_)], stream)
                self.fillGhostsVJP(B2, stream)
                self.substepVJP(1, dt, B2, [[Xn[p], B1[p]] for p in range(np_)], stream)
                self.fillGhostsVJP(B1, stream)
                self.substepVJP(0, dt, B1, [[Xn[p]] for p in range(np_)], stream)
                self.fillGhostsVJP(Xn, stream)
                Xb = Xn
        return Xb

    def set_layout(self, lo, domain, periodic):
        """Patch positions (first interior cell per patch, level index space), the domain's cells
        per axis and its boundary per axis (FILL_PERIODIC, FILL_ZERO_GRADIENT, FILL_REFLECT walls
        or FILL_DIRICHLET faces): enables the ghost exchange between patches."""
        dim = self.rec.flow_model.dim
        flat = []
        for p in range(self.npatch):
            flat += list(lo[p][:dim]) + [0] * (3 - dim)
        lo_a = (ctypes.c_int * len(flat))(*flat)
        dom = (ctypes.c_int * 3)(*(list(domain) + [1] * (3 - len(domain))))
        per = (ctypes.c_int * 3)(*(list(periodic) + [0] * (3 - len(periodic))))
        L.check("hmr_level_set_layout", self._lib.hmr_level_set_layout(self.level, lo_a, dom, per))

    def set_periodic(self, patch, periodic):
        per = (ctypes.c_int * 3)(*(list(periodic) + [0] * (3 - len(periodic))))
        L.check("hmr_level_set_periodic", self._lib.hmr_level_set_periodic(self.level, int(patch), per))

    def check(self):
        """Raises HmrError(HMR_ERR_BARRIER) if a persistent-kernel barrier gave up."""
        L.check("hmr_level_check", self._lib.hmr_level_check(self.level))

    def barrier_diagnostic(self, extra_arrivals, timeout_ns):
        L.check("hmr_level_barrier_diagnostic", self._lib.hmr_level_barrier_diagnostic(
            self.level, int(extra_arrivals), int(timeout_ns)))

    def step_cfl(self, cfl, stream=None):
        """One SSPRK3 step with dt = (1/max spectral radius)*cfl computed on the device
        from the current states (no host synchronisation)."""
        L.check("hmr_level_step_cfl", self._lib.hmr_level_step_cfl(self.level, float(cfl), _stream_ptr(stream)))

    def last_dt(self):
        dt = ctypes.c_double()
        L.check("hmr_level_last_dt", self._lib.hmr_level_last_dt(self.level, ctypes.byref(dt)))
        return dt.value

    def step(self, dt, stream=None):
        L.check("hmr_level_step", self._lib.hmr_level_step(self.level, float(dt), _stream_ptr(stream)))

    def set_launch(self, threads, blocks_per_sm):
        L.check("hmr_level_set_launch", self._lib.hmr_level_set_launch(self.level, int(threads), int(blocks_per_sm)))

    def set_work_split(self, chunk_blocks, mode=0):
        """Chunks of chunk_blocks (1, 2, 4) block widths per phase; mode bit 0: grid-stride
        hand-out of the cell-wise phases; bit 1 (fast form): faces sorted by their sensor, the
        HLLC ones in the fast form beside the HLLC-HLL ones in the exact form."""
        L.check("hmr_level_set_work_split", self._lib.hmr_level_set_work_split(self.level, int(chunk_blocks), int(mode)))

    def work_split(self):
        m, s_ = ctypes.c_int(), ctypes.c_int()
        L.check("hmr_level_work_split", self._lib.hmr_level_work_split(self.level, ctypes.byref(m), ctypes.byref(s_)))
        return m.value, s_.value

    def autotune(self, dt, stream=None):
        t = ctypes.c_int()
        b = ctypes.c_int()
        L.check("hmr_level_autotune", self._lib.hmr_level_autotune(
            self.level, float(dt), ctypes.byref(t), ctypes.byref(b), _stream_ptr(stream)))
        return t.value, b.value
