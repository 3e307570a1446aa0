"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's FP64 hot path on the CPU; it is the
checker for the GPU path and the CPU-baseline leg of bench.py.  Nothing in the
hamers_gb300 package imports this module.

Array conventions (SAMRAI layout, x fastest):
  state  : numpy (ncomp, G[2], G[1], G[0]) with G = n + 2*4 on the used axes
  flux   : list over axes a of numpy (neq, n2', n1', n0'), n grown by 1 along a
  source : numpy (neq, n2, n1, n0)
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhmr_oracle.so")
_TAN_PATH = os.path.join(_HERE, "_build", "libhmr_tangent.so")

MODEL_SINGLE_SPECIES = 0
MODEL_FOUR_EQN_CONSERVATIVE = 1
MODEL_FIVE_EQN_ALLAIRE = 2
SCHEME_WCNS5_JS = 0
SCHEME_WCNS6_LD = 1
SCHEME_WCNS5_Z = 2
SCHEME_WCNS6_CU_M2 = 3
GHOST = 4


class _Cfg(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("dim", ctypes.c_int), ("num_species", ctypes.c_int),
                ("scheme", ctypes.c_int), ("gamma", ctypes.c_double * 8), ("R", ctypes.c_double * 8),
                ("p", ctypes.c_int),
                ("q", ctypes.c_int), ("C", ctypes.c_double), ("alpha_tau", ctypes.c_double),
                ("Chi", ctypes.c_double), ("epsilon", ctypes.c_double), ("grid_dx", ctypes.c_double * 3),
                ("ghosts", ctypes.c_int)]


class _Transport(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("mu", ctypes.c_double), ("mu_v", ctypes.c_double),
                ("c_p", ctypes.c_double), ("Pr", ctypes.c_double), ("mu_kappa", ctypes.c_double)]


class Transport:
    """Navier-Stokes transport of a single-species patch: midpoint diffusive flux of
    the given order (2, 4, or 6 with a Config of ghosts=5), constant shear viscosity mu and bulk viscosity mu_v,
    Prandtl thermal conductivity c_p*mu_kappa/Pr (mu_kappa defaults to mu)."""

    def __init__(self, mu, c_p, Pr, mu_v=0.0, order=4, mu_kappa=None):
        self.order = int(order)
        self.mu, self.mu_v, self.c_p, self.Pr = float(mu), float(mu_v), float(c_p), float(Pr)
        self.mu_kappa = float(mu if mu_kappa is None else mu_kappa)

    def c(self):
        return _Transport(self.order, self.mu, self.mu_v, self.c_p, self.Pr, self.mu_kappa)


def build():
    """Compile the oracle library with its Makefile."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        lp = ctypes.POINTER(ctypes.c_long)
        cp = ctypes.POINTER(_Cfg)
        L.hmro_conv_flux_source.argtypes = [cp, ip, dp, ctypes.c_double, dp, dp, dp, lp]
        L.hmro_rk_stage.argtypes = [cp, ip, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.hmro_fill_ghosts.argtypes = [cp, ip, ip, dp]
        L.hmro_fill_ghosts_bv.argtypes = [cp, ip, ip, dp, dp]
        L.hmro_rk3_advance.argtypes = [cp, ip, dp, ctypes.c_double, ip, ctypes.c_int, dp, lp]
        L.hmro_rk3_advance_bv.argtypes = [cp, ip, dp, ctypes.c_double, ip, dp, ctypes.c_int, dp, lp]
        L.hmro_stage_threads.argtypes = [cp, ip, dp, ctypes.c_double, dp, ctypes.c_int]
        L.hmro_stage_threads.restype = ctypes.c_long
        L.hmro_spectral_radius.argtypes = [cp, ip, dp, dp]
        L.hmro_spectral_radius.restype = ctypes.c_double
        L.hmro_spectral_radius_ns.argtypes = [cp, ctypes.POINTER(_Transport), ip, dp, dp]
        L.hmro_spectral_radius_ns.restype = ctypes.c_double
        tp = ctypes.POINTER(_Transport)
        L.hmro_diff_flux.argtypes = [cp, tp, ip, dp, ctypes.c_double, dp, dp]
        L.hmro_rk_stage_ns.argtypes = [cp, ip, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
        L.hmro_ns_rk3_advance.argtypes = [cp, tp, ip, dp, ctypes.c_double, ip, ctypes.c_int, dp]
        L.hmro_sync_fluxes.argtypes = [cp, ip, dp, dp, dp, dp, dp]
        L.hmro_coarsen_fluxsum.argtypes = [cp, ip, ip, ip, ip, ip, dp, dp]
        L.hmro_coarsen_cells.argtypes = [cp, ip, ip, ip, ip, ip, dp, dp]
        L.hmro_refine_ghosts.argtypes = [cp, ip, ip, ip, ip, ip, dp, dp, ctypes.c_double, dp]
        L.hmro_num_eqn.argtypes = [cp]
        L.hmro_num_comp.argtypes = [cp]
        _lib = L
    return _lib


_tan = None


def tangent_lib():
    global _tan
    if _tan is None:
        if not os.path.exists(_TAN_PATH):
            build()
        L = ctypes.CDLL(_TAN_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.hmro_tangent_substep.argtypes = [ctypes.POINTER(_Cfg), ip, dp, ctypes.c_double, ctypes.c_int, dp,
                                           ctypes.c_double, dp, dp, dp, dp, ctypes.POINTER(_Transport)]
        _tan = L
    return _tan


class Config:
    """Flow model + scheme selection (mirrors the reference's input keys).

    C defaults to the scheme's own default (1e9 for WCNS6-LD, 1000 for
    WCNS6-CU-M2).  grid_dx is the grid geometry's (coarsest level's) spacing,
    which WCNS6-CU-M2's weights use on every level; it is required for that
    scheme and ignored by the others.
    """

    def __init__(self, model, dim, species_gamma, scheme=SCHEME_WCNS5_JS,
                 p=2, q=4, C=None, alpha_tau=35.0, species_R=None, Chi=1.0e8, epsilon=1.0e-8,
                 grid_dx=None, ghosts=GHOST):
        self.model = int(model)
        self.ghosts = int(ghosts)
        self.dim = int(dim)
        self.species_gamma = [float(g) for g in species_gamma]
        self.num_species = len(self.species_gamma)
        self.species_R = [float(r) for r in (species_R or [1.0] * self.num_species)]
        self.scheme = int(scheme)
        if C is None:
            C = 1000.0 if self.scheme == SCHEME_WCNS6_CU_M2 else 1.0e9
        self.p, self.q, self.C, self.alpha_tau = int(p), int(q), float(C), float(alpha_tau)
        self.Chi, self.epsilon = float(Chi), float(epsilon)
        self.grid_dx = None if grid_dx is None else [float(v) for v in grid_dx] + [1.0] * (3 - len(grid_dx))

    def c(self):
        if self.scheme == SCHEME_WCNS6_CU_M2 and self.grid_dx is None:
            raise ValueError("WCNS6-CU-M2 needs the grid geometry's spacing (grid_dx)")
        g = (ctypes.c_double * 8)(*(self.species_gamma + [0.0] * (8 - self.num_species)))
        r = (ctypes.c_double * 8)(*(self.species_R + [0.0] * (8 - self.num_species)))
        gd = (ctypes.c_double * 3)(*(self.grid_dx or [0.0, 0.0, 0.0]))
        return _Cfg(self.model, self.dim, self.num_species, self.scheme, g, r, self.p, self.q,
                    self.C, self.alpha_tau, self.Chi, self.epsilon, gd, self.ghosts)

    @property
    def neq(self):
        if self.model == MODEL_SINGLE_SPECIES:
            return self.dim + 2
        if self.model == MODEL_FOUR_EQN_CONSERVATIVE:
            return self.num_species + self.dim + 1
        return self.dim + 2 * self.num_species

    @property
    def ncomp(self):
        return self.neq + (1 if self.model == MODEL_FIVE_EQN_ALLAIRE else 0)


def _n3(n):
    n = list(n)
    return n + [1] * (3 - len(n))


def ghost_shape(cfg, n, ghosts=None):
    n3 = _n3(n)
    ghosts = cfg.ghosts if ghosts is None else ghosts
    G = [n3[d] + 2 * ghosts if d < cfg.dim else 1 for d in range(3)]
    return (cfg.ncomp, G[2], G[1], G[0])


def flux_shapes(cfg, n):
    n3 = _n3(n)
    out = []
    for a in range(cfg.dim):
        e = [n3[d] + (1 if d == a else 0) for d in range(3)]
        out.append((cfg.neq, e[2], e[1], e[0]))
    return out


_REF_DIR = os.path.join(_HERE, "_ref")
_REF_LIB_PATH = os.path.join(_REF_DIR, "libhmr_ref.so")
_REF_SRC = os.environ.get("HMR_REFERENCE_SRC", "/root/reference")
_ref_lib = None


def ref_available():
    """True when the reference's own translation units are built (oracle/_ref/libhmr_ref.so)
    or can be built here (the reference sources are present)."""
    return os.path.exists(_REF_LIB_PATH) or os.path.isdir(os.path.join(_REF_SRC, "src"))


def ref_lib():
    """The reference's hot path compiled from its own sources (refshim/Makefile): the checker
    of this oracle.  Builds it on first use when the reference sources are present."""
    global _ref_lib
    if _ref_lib is None:
        if os.path.isdir(os.path.join(_REF_SRC, "src")):
            subprocess.check_call(["make", "-s", "-j", str(os.cpu_count() or 1), "-C",
                                   os.path.join(_HERE, "refshim"), "REF=" + _REF_SRC])
        L = ctypes.CDLL(_REF_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.hmrref_conv_flux_source.argtypes = [ctypes.POINTER(_Cfg), ip, dp, ctypes.c_double, dp, dp, dp]
        L.hmrref_conv_flux_source.restype = ctypes.c_int
        L.hmrref_last_error.restype = ctypes.c_char_p
        L.hmrref_diff_flux.argtypes = [ctypes.POINTER(_Cfg), ctypes.POINTER(_Transport), ip, ctypes.c_int, dp,
                                       ctypes.c_double, dp, dp]
        L.hmrref_diff_flux.restype = ctypes.c_int
        L.hmrref_fill_boundaries.argtypes = [ctypes.POINTER(_Cfg), ip, ip, ctypes.c_int, dp]
        L.hmrref_fill_boundaries.restype = ctypes.c_int
        L.hmrref_fill_boundaries_bv.argtypes = [ctypes.POINTER(_Cfg), ip, ip, ctypes.c_int, dp, dp]
        L.hmrref_fill_boundaries_bv.restype = ctypes.c_int
        _ref_lib = L
    return _ref_lib


def ref_conv_flux_source(cfg, n, dx, dt, Q, source=None):
    """The reference's ConvectiveFluxReconstructorWCNS56::computeConvectiveFluxAndSourceOnPatch on
    one patch, same arguments and results as conv_flux_source (without the face statistics)."""
    n3 = _n3(n)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert Q.shape == ghost_shape(cfg, n)
    shapes = flux_shapes(cfg, n)
    flat = np.zeros(sum(int(np.prod(s)) for s in shapes))
    if source is None:
        source = np.zeros((cfg.neq, n3[2], n3[1], n3[0]))
    source = np.ascontiguousarray(source, dtype=np.float64)
    L = ref_lib()
    rc = L.hmrref_conv_flux_source(ctypes.byref(cfg.c()), _ip(n3), _dv(list(dx) + [1.0] * (3 - len(dx))),
                                   float(dt), _dp(Q), _dp(flat), _dp(source))
    if rc != 0:
        raise RuntimeError("reference: " + L.hmrref_last_error().decode())
    out, off = [], 0
    for s in shapes:
        m = int(np.prod(s))
        out.append(flat[off:off + m].reshape(s))
        off += m
    return out, source


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(v):
    return (ctypes.c_int * len(v))(*v)


def _dv(v):
    return (ctypes.c_double * len(v))(*v)


def conv_flux_source(cfg, n, dx, dt, Q, source=None):
    """computeConvectiveFluxAndSourceOnPatch: returns (flux list, source, stats)."""
    n3 = _n3(n)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert Q.shape == ghost_shape(cfg, n)
    shapes = flux_shapes(cfg, n)
    flat = np.zeros(sum(int(np.prod(s)) for s in shapes))
    if source is None:
        source = np.zeros((cfg.neq, n3[2], n3[1], n3[0]))
    source = np.ascontiguousarray(source, dtype=np.float64)
    stats = (ctypes.c_long * 3)()
    lib().hmro_conv_flux_source(ctypes.byref(cfg.c()), _ip(n3), _dv(list(dx) + [1.0] * (3 - len(dx))),
                                float(dt), _dp(Q), _dp(flat), _dp(source), stats)
    out, off = [], 0
    for s in shapes:
        m = int(np.prod(s))
        out.append(flat[off:off + m].reshape(s))
        off += m
    return out, source, (stats[0], stats[1], stats[2])


def rk_stage(cfg, n, dx, alpha, beta, gamma, Q_int, F_int, S_int, F_acc=None, S_acc=None):
    """advanceSingleStepOnPatch for one stage (len(alpha) coefficient sets)."""
    n3 = _n3(n)
    ns = len(alpha)
    Qi = np.ascontiguousarray(np.stack(Q_int), dtype=np.float64)
    Fi = np.ascontiguousarray(np.stack([np.concatenate([f.ravel() for f in F]) for F in F_int]))
    Si = np.ascontiguousarray(np.stack(S_int), dtype=np.float64)
    Qo = np.zeros(ghost_shape(cfg, n))
    fa = None
    if F_acc is not None:
        fa = np.ascontiguousarray(np.concatenate([f.ravel() for f in F_acc]))
    lib().hmro_rk_stage(ctypes.byref(cfg.c()), _ip(n3), _dv(list(dx) + [1.0] * (3 - len(dx))), ns,
                        _dv(alpha), _dv(beta), _dv(gamma), _dp(Qi), _dp(Fi), _dp(Si), _dp(Qo),
                        _dp(fa) if fa is not None else None,
                        _dp(S_acc) if S_acc is not None else None)
    if F_acc is not None:
        off = 0
        for f in F_acc:
            f.ravel()[:] = fa[off:off + f.size]
            off += f.size
    return Qo


def fill_ghosts(cfg, n, periodic, Q, dirichlet=None):
    """Ghost fill, mode per axis: 0 zero-gradient, 1 periodic, 3 reflecting wall, 4 Dirichlet
    (dirichlet: values per side, shape (2 dim, ncomp), row 2 axis + high), 5 symmetry plane."""
    assert Q.flags["C_CONTIGUOUS"] and Q.dtype == np.float64
    per = _ip(list(periodic) + [0] * (3 - len(periodic)))
    if dirichlet is None:
        lib().hmro_fill_ghosts(ctypes.byref(cfg.c()), _ip(_n3(n)), per, _dp(Q))
    else:
        bv = np.zeros((6, Q.shape[0]))
        d = np.asarray(dirichlet, dtype=np.float64)
        bv[:d.shape[0]] = d
        lib().hmro_fill_ghosts_bv(ctypes.byref(cfg.c()), _ip(_n3(n)), per, _dp(np.ascontiguousarray(bv)), _dp(Q))
    return Q


def rk3_advance(cfg, n, dx, dt, periodic, nsteps, Q, dirichlet=None):
    """nsteps SSPRK3 steps of one patch, in place; returns the face counters.  dirichlet: values
    of the Dirichlet sides (mode 4), as fill_ghosts takes them."""
    assert Q.flags["C_CONTIGUOUS"] and Q.dtype == np.float64
    stats = (ctypes.c_long * 3)()
    bv = np.zeros((6, Q.shape[0]))
    if dirichlet is not None:
        d = np.asarray(dirichlet, dtype=np.float64)
        bv[:d.shape[0]] = d
    lib().hmro_rk3_advance_bv(ctypes.byref(cfg.c()), _ip(_n3(n)), _dv(list(dx) + [1.0] * (3 - len(dx))),
                              float(dt), _ip(list(periodic) + [0] * (3 - len(periodic))), _dp(bv), int(nsteps),
                              _dp(Q), stats)
    return (stats[0], stats[1], stats[2])


def stage_threads(cfg, n, dx, dt, Q, nthreads):
    """One RK stage of a patch split into nthreads sub-patches; returns cells updated."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    return lib().hmro_stage_threads(ctypes.byref(cfg.c()), _ip(_n3(n)),
                                    _dv(list(dx) + [1.0] * (3 - len(dx))), float(dt), _dp(Q),
                                    int(nthreads))


def _split_flux(cfg, n, flat):
    out, off = [], 0
    for s in flux_shapes(cfg, n):
        m = int(np.prod(s))
        out.append(flat[off:off + m].reshape(s))
        off += m
    return out


def ref_fill_boundaries(cfg, n, mode, Q, corner_axis=0, dirichlet=None):
    """The reference's physical-boundary fill (EulerBoundaryConditions with
    BasicCartesianBoundaryUtilities2/3) of one patch covering the domain, in place: mode per
    axis 0 (FLOW), 3 (REFLECT), 5 (SYMMETRY) or 4 (DIRICHLET, values per side in dirichlet: shape
    (2 dim, ncomp), row 2 axis + high); corner_axis picks the axis of the X/Y/Z-prefixed corner
    conditions (a corner with a Dirichlet side takes the lowest Dirichlet axis's)."""
    assert Q.flags["C_CONTIGUOUS"] and Q.dtype == np.float64 and Q.shape == ghost_shape(cfg, n)
    L = ref_lib()
    per = _ip(list(mode) + [0] * (3 - len(mode)))
    if dirichlet is None:
        rc = L.hmrref_fill_boundaries(ctypes.byref(cfg.c()), _ip(_n3(n)), per, int(corner_axis), _dp(Q))
    else:
        bv = np.ascontiguousarray(dirichlet, dtype=np.float64)
        rc = L.hmrref_fill_boundaries_bv(ctypes.byref(cfg.c()), _ip(_n3(n)), per, int(corner_axis), _dp(bv), _dp(Q))
    if rc != 0:
        raise RuntimeError("reference: " + L.hmrref_last_error().decode())
    return Q


def ref_diff_flux(cfg, tr, n, dx, dt, Q, ghosts=4):
    """The reference's DiffusiveFluxReconstructorMidpoint::computeDiffusiveFluxOnPatch (single
    species) on one patch whose conservative variables carry `ghosts` ghost cells per side."""
    n3 = _n3(n)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert Q.shape == ghost_shape(cfg, n, ghosts)
    flat = np.zeros(sum(int(np.prod(s)) for s in flux_shapes(cfg, n)))
    L = ref_lib()
    rc = L.hmrref_diff_flux(ctypes.byref(cfg.c()), ctypes.byref(tr.c()), _ip(n3), int(ghosts),
                            _dv(list(dx) + [1.0] * (3 - len(dx))), float(dt), _dp(Q), _dp(flat))
    if rc != 0:
        raise RuntimeError("reference: " + L.hmrref_last_error().decode())
    return _split_flux(cfg, n, flat)


def diff_flux(cfg, tr, n, dx, dt, Q):
    """computeDiffusiveFluxOnPatch (single species): list of dt-scaled face fluxes per axis."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert Q.shape == ghost_shape(cfg, n)
    flat = np.zeros(sum(int(np.prod(s)) for s in flux_shapes(cfg, n)))
    r = lib().hmro_diff_flux(ctypes.byref(cfg.c()), ctypes.byref(tr.c()), _ip(_n3(n)),
                             _dv(list(dx) + [1.0] * (3 - len(dx))), float(dt), _dp(Q), _dp(flat))
    if r != 0:
        raise ValueError("the oracle's diffusive flux covers single-species patches, order 2 or 4 (or 6 with ghosts=5)")
    return _split_flux(cfg, n, flat)


def rk_stage_ns(cfg, n, dx, alpha, beta, gamma, Q_int, F_int, Fd_int, S_int):
    """NavierStokes::advanceSingleStepOnPatch for one stage."""
    ns = len(alpha)
    Qi = np.ascontiguousarray(np.stack(Q_int), dtype=np.float64)
    Fi = np.ascontiguousarray(np.stack([np.concatenate([f.ravel() for f in F]) for F in F_int]))
    Di = np.ascontiguousarray(np.stack([np.concatenate([f.ravel() for f in F]) for F in Fd_int]))
    Si = np.ascontiguousarray(np.stack(S_int), dtype=np.float64)
    Qo = np.zeros(ghost_shape(cfg, n))
    lib().hmro_rk_stage_ns(ctypes.byref(cfg.c()), _ip(_n3(n)), _dv(list(dx) + [1.0] * (3 - len(dx))), ns,
                           _dv(alpha), _dv(beta), _dv(gamma), _dp(Qi), _dp(Fi), _dp(Di), _dp(Si), _dp(Qo))
    return Qo


def ns_rk3_advance(cfg, tr, n, dx, dt, periodic, nsteps, Q):
    """nsteps SSPRK3 steps of the Navier-Stokes equations on one patch, in place."""
    assert Q.flags["C_CONTIGUOUS"] and Q.dtype == np.float64
    r = lib().hmro_ns_rk3_advance(ctypes.byref(cfg.c()), ctypes.byref(tr.c()), _ip(_n3(n)),
                                  _dv(list(dx) + [1.0] * (3 - len(dx))), float(dt),
                                  _ip(list(periodic) + [0] * (3 - len(periodic))), int(nsteps), _dp(Q))
    if r != 0:
        raise ValueError("the oracle's diffusive flux covers single-species patches, order 2 or 4 (or 6 with ghosts=5)")
    return Q


def _flat(F):
    return np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.float64).ravel() for f in F]))


def sync_fluxes(cfg, n, dx, F, S, Q, Fd=None):
    """synchronizeFluxes on one coarse patch: Q (ghost box, in place) += -div (F [+ Fd]) + S."""
    assert Q.flags["C_CONTIGUOUS"] and Q.dtype == np.float64
    fd = _flat(Fd) if Fd is not None else None
    lib().hmro_sync_fluxes(ctypes.byref(cfg.c()), _ip(_n3(n)), _dv(list(dx) + [1.0] * (3 - len(dx))),
                           _dp(_flat(F)), _dp(fd) if fd is not None else None,
                           _dp(np.ascontiguousarray(S, dtype=np.float64)), _dp(Q))
    return Q


def coarsen_fluxsum(cfg, ratio, cn, clo, fn, flo, Ff, Fc):
    """Flux-sum coarsening of a fine patch (at flo, size fn) onto a coarse patch (clo, cn); Fc in place."""
    flat = _flat(Fc)
    lib().hmro_coarsen_fluxsum(ctypes.byref(cfg.c()), _ip(_n3(ratio)), _ip(_n3(cn)), _ip(list(clo) + [0] * (3 - len(clo))),
                               _ip(_n3(fn)), _ip(list(flo) + [0] * (3 - len(flo))), _dp(_flat(Ff)), _dp(flat))
    off = 0
    for f in Fc:
        f.ravel()[:] = flat[off:off + f.size]
        off += f.size
    return Fc


def coarsen_cells(cfg, ratio, cn, clo, fn, flo, Qf, Qc):
    """Coarsen a fine patch's interior onto the covered cells of a coarse patch (Qc in place)."""
    assert Qc.flags["C_CONTIGUOUS"] and Qc.dtype == np.float64
    lib().hmro_coarsen_cells(ctypes.byref(cfg.c()), _ip(_n3(ratio)), _ip(_n3(cn)), _ip(list(clo) + [0] * (3 - len(clo))),
                             _ip(_n3(fn)), _ip(list(flo) + [0] * (3 - len(flo))),
                             _dp(np.ascontiguousarray(Qf, dtype=np.float64)), _dp(Qc))
    return Qc


def refine_ghosts(cfg, ratio, fn, flo, cn, clo, Qc_old, Qc_new, theta, Qf):
    """Coarse-fine ghost cells of the fine patch (flo, fn) from the coarse patch (clo, cn)
    at time fraction theta (linear time interpolation, conservative linear refinement); Qf in place."""
    assert Qf.flags["C_CONTIGUOUS"] and Qf.dtype == np.float64
    lib().hmro_refine_ghosts(ctypes.byref(cfg.c()), _ip(_n3(ratio)), _ip(_n3(fn)), _ip(list(flo) + [0] * (3 - len(flo))),
                             _ip(_n3(cn)), _ip(list(clo) + [0] * (3 - len(clo))),
                             _dp(np.ascontiguousarray(Qc_old, dtype=np.float64)),
                             _dp(np.ascontiguousarray(Qc_new, dtype=np.float64)), float(theta), _dp(Qf))
    return Qf


def tangent_substep(cfg, n, dx, dt, stage, alpha, beta, Q_int, dQ_int, transport=None):
    """Fused substep (hmr_rk_substep_patch's forward) and its tangent along dQ_int.

    Q_int, dQ_int: lists of stage+1 ghost-box states; returns (Q_out, dQ_out)
    over the ghost box (interior written, ghosts zero).  With a Transport the
    substep is NavierStokes's (diffusive flux included)."""
    shape = ghost_shape(cfg, n)
    Qi = np.ascontiguousarray(np.stack([np.asarray(q, dtype=np.float64) for q in Q_int[:stage + 1]]))
    dQi = np.ascontiguousarray(np.stack([np.asarray(q, dtype=np.float64) for q in dQ_int[:stage + 1]]))
    assert Qi.shape[1:] == shape and dQi.shape == Qi.shape
    Qo = np.zeros(shape)
    dQo = np.zeros(shape)
    tangent_lib().hmro_tangent_substep(ctypes.byref(cfg.c()), _ip(_n3(n)), _dv(list(dx) + [1.0] * (3 - len(dx))),
                                       float(dt), int(stage), _dv(list(alpha)[:stage + 1]), float(beta),
                                       _dp(Qi), _dp(dQi), _dp(Qo), _dp(dQo),
                                       ctypes.byref(transport.c()) if transport is not None else None)
    return Qo, dQo


def spectral_radius(cfg, n, dx, Q, transport=None):
    """Max over the ghost box of sum_d (|u_d| + c)/dx_d (the stable dt is (1/that)*CFL); with a
    Transport, NavierStokes's max of that and the diffusive radius (dt = (1/(that + eps))*CFL)."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    if transport is not None:
        return lib().hmro_spectral_radius_ns(ctypes.byref(cfg.c()), ctypes.byref(transport.c()), _ip(_n3(n)),
                                             _dv(list(dx) + [1.0] * (3 - len(dx))), _dp(Q))
    return lib().hmro_spectral_radius(ctypes.byref(cfg.c()), _ip(_n3(n)), _dv(list(dx) + [1.0] * (3 - len(dx))),
                                      _dp(Q))
