"""ctypes wrapper for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (``hydro_oracle.cpp``) is a double-precision C++ restatement of
hydro-cl-lua's generated OpenCL kernels for the Euler / Roe / PLM / Runge-Kutta
path.  Only the tests, the smoke check and the benchmark's CPU-baseline leg
import this module; the product library never does.

Parity anchoring: the reference itself cannot run here (no LuaJIT, no OpenCL
CPU platform), so the restatement is pinned by the density L1 errors recorded
in the reference's accuracy harness (``tests/test-order/schemes.lua``) and by
the eigen-basis identities the reference uses as diagnostics
(``hydro/solver/fvsolver.lua:396-527``); see ``tests/test_oracle_pins.py``.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
LIB_CONTRACT_PATH = os.path.join(BUILD_DIR, "liboracle_contract.so")
SRC = os.path.join(HERE, "hydro_oracle.cpp")

# Names in the order of the reference's limiter table (hydro/app.lua:614-635).
LIMITERS = [
    "donor cell", "Lax-Wendroff", "Beam-Warming", "Fromm", "CHARM", "HCUS",
    "HQUICK", "Koren", "minmod", "Oshker", "ospre", "smart", "Sweby", "UMIST",
    "van Albada 1", "van Albada 2", "van Leer", "monotized central",
    "superbee", "Barth-Jespersen",
    # not a row of the reference's table: the van Leer form of the comment at
    # hydro/app.lua:631, (r + |r|) / (1 + |r|)
    "van Leer (abs)",
]
# Explicit integrators (hydro/int/all.lua), in the oracle's numbering.
INTEGRATORS = [
    "forward Euler", "Runge-Kutta 2", "Runge-Kutta 2 Heun",
    "Runge-Kutta 2 Ralston", "Runge-Kutta 3", "Runge-Kutta 4",
    "Runge-Kutta 4, 3/8ths rule", "Runge-Kutta 2, TVD",
    "Runge-Kutta 2, non-TVD", "Runge-Kutta 3, TVD", "Runge-Kutta 4, TVD",
    "Runge-Kutta 4, non-TVD",
]
BOUNDARIES = {"none": 0, "periodic": 1, "mirror": 2, "freeflow": 3, "linear": 4, "quadratic": 5, "fixed": 6}
RECONS = {None: 0, False: 0, "piecewise constant": 1, "plm cons": 2, "plm prim": 3, "plm athena": 4}


def build(force=False, contract=False):
    """Compile the oracle with g++ (OpenMP).  The default build forbids FMA
    contraction (-ffp-contract=off): its order of operations is the
    reference's, term by term.  contract=True builds a second library that lets
    the compiler fuse multiply-adds (-ffp-contract=fast, with FMA instructions
    enabled on x86-64), as an OpenCL compiler may under FP_CONTRACT ON: the
    tests use it to bound how far such a build of the reference can drift from
    the contraction-free reading."""
    path = LIB_CONTRACT_PATH if contract else LIB_PATH
    if not force and os.path.exists(path) and os.path.getmtime(path) >= os.path.getmtime(SRC):
        return path
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    fp = ["-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []) if contract \
        else ["-ffp-contract=off"]
    cmd = ["g++", "-O3", "-std=c++17"] + fp + ["-fno-fast-math", "-fopenmp", "-shared", "-fPIC", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, path)
    return path


class OrDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("mins", ctypes.c_double * 3),
        ("maxs", ctypes.c_double * 3),
        ("boundary", ctypes.c_int * 6),
        ("flux_limiter", ctypes.c_int),
        ("recon", ctypes.c_int),
        ("slope_limiter", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("gamma", ctypes.c_double),
        ("rho_min", ctypes.c_double),
        ("p_min", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("fixed_dt", ctypes.c_double),
        ("flux", ctypes.c_int),
        ("hllc_method", ctypes.c_int),
        ("entropy_fix", ctypes.c_int),
        ("reserved0", ctypes.c_int),
        ("entropy_fix_factor", ctypes.c_double),
        ("fixed_cons", (ctypes.c_double * 5) * 6),
    ]

# flux names in the reference's vocabulary (hydro/flux/*.lua)
FLUXES = ["roe", "hll", "rusanov", "euler-hllc"]


_libs = {}


def lib(contract=False):
    if contract not in _libs:
        path = build(contract=contract)
        L = ctypes.CDLL(path)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.or_create.restype = vp
        L.or_create.argtypes = [ctypes.POINTER(OrDesc)]
        L.or_destroy.argtypes = [vp]
        L.or_num_cells.restype = ctypes.c_long
        L.or_num_cells.argtypes = [vp]
        for name in ("or_set_state_full", "or_get_state_full", "or_reset_state", "or_get_interior"):
            getattr(L, name).argtypes = [vp, dp]
        L.or_boundary.argtypes = [vp]
        L.or_constrain_u.argtypes = [vp]
        L.or_calc_dt.restype = ctypes.c_double
        L.or_calc_dt.argtypes = [vp]
        L.or_step.argtypes = [vp, ctypes.c_double]
        L.or_update.restype = ctypes.c_double
        L.or_update.argtypes = [vp]
        L.or_get_t.restype = ctypes.c_double
        L.or_get_t.argtypes = [vp]
        L.or_set_t.argtypes = [vp, ctypes.c_double]
        L.or_run_until.restype = ctypes.c_long
        L.or_run_until.argtypes = [vp, ctypes.c_double, ctypes.c_long]
        L.or_calc_deriv.argtypes = [vp, ctypes.c_double, dp]
        L.or_get_flux.argtypes = [vp, dp]
        L.or_roe_flux.argtypes = [ctypes.POINTER(OrDesc), dp, dp, ip, dp]
        L.or_interface_flux.argtypes = [ctypes.POINTER(OrDesc), dp, dp, ip, dp]
        L.or_eigen_basis.argtypes = [ctypes.POINTER(OrDesc), dp, dp, ip, dp, dp, dp]
        L.or_limiter.restype = ctypes.c_double
        L.or_limiter.argtypes = [ip, ctypes.c_double]
        L.or_num_threads.restype = ctypes.c_int
        L.or_set_plm_athena_recorded_edges.argtypes = [ip]
        _libs[contract] = L
    return _libs[contract]


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_desc(cfg):
    """Map a reference-style solver args table (a dict) onto the oracle descriptor."""
    d = OrDesc()
    dim = int(cfg["dim"])
    gs = cfg["gridSize"]
    if isinstance(gs, int):
        gs = [gs]
    mins = list(cfg.get("mins", [-1, -1, -1])) + [-1] * 3
    maxs = list(cfg.get("maxs", [1, 1, 1])) + [1] * 3
    d.dim = dim
    for k in range(3):
        d.n[k] = int(gs[k]) if k < dim else 1
        d.mins[k] = float(mins[k])
        d.maxs[k] = float(maxs[k])
    bnd = cfg.get("boundary", {}) or {}
    if isinstance(bnd, str):
        bnd = {k: bnd for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")}
    eq = cfg.get("eqnArgs", {}) or {}
    gamma = float(eq.get("heatCapacityRatio", 7.0 / 5.0))
    for k, name in enumerate(("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")):
        spec = bnd.get(name, "freeflow")
        if isinstance(spec, dict):
            cons = fixed_cons(spec, gamma)
            for f in range(5):
                d.fixed_cons[k][f] = cons[f]
            spec = spec["name"]
        d.boundary[k] = BOUNDARIES[spec]
    d.flux_limiter = LIMITERS.index(cfg.get("fluxLimiter", "donor cell"))
    d.recon = RECONS[cfg.get("usePLM", None)]
    d.slope_limiter = LIMITERS.index(cfg.get("slopeLimiter", "donor cell"))
    d.integrator = INTEGRATORS.index(cfg.get("integrator", "forward Euler"))
    eq = cfg.get("eqnArgs", {}) or {}
    d.gamma = float(eq.get("heatCapacityRatio", 7.0 / 5.0))
    d.rho_min = float(eq.get("rhoMin", 1e-7))
    d.p_min = float(eq.get("PMin", 1e-7))
    d.cfl = float(cfg.get("cfl", 0.5))
    d.fixed_dt = float(cfg.get("fixedDT", 0.0) or 0.0)
    d.flux = FLUXES.index(cfg.get("flux", "roe"))
    # euler-hllc's hllcMethod (default 2, euler-hllc.lua:19); 0 in the descriptor is that default
    d.hllc_method = int(cfg["hllcMethod"]) + 1 if "hllcMethod" in cfg else 0
    # hydro/flux/roe.lua:10-16
    d.entropy_fix = 1 if cfg.get("useEntropyFluxFix", False) else 0
    d.entropy_fix_factor = float(cfg.get("entropyFluxFixLimitingFactor", 0.2))
    return d


def fixed_cons(spec, gamma):
    """The constant state of a 'fixed' boundary side, {"name": "fixed", "cons":
    [rho, m.x, m.y, m.z, ETotal]} or {"name": "fixed", "prim": {"rho", "v",
    "P"}} (consFromPrim, hydro/eqn/euler.cl:163-173, ePot 0)."""
    if spec.get("name") != "fixed":
        return [0.0] * 5
    if "cons" in spec:
        return [float(c) for c in spec["cons"]]
    w = spec["prim"]
    rho, P = float(w["rho"]), float(w["P"])
    v = [float(c) for c in list(w.get("v", [0, 0, 0])) + [0.0] * 3][:3]
    return [rho, v[0] * rho, v[1] * rho, v[2] * rho,
            rho * (.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2])) + P / (gamma - 1.)]


class OracleSolver:
    """The oracle behind the reference's solver-args vocabulary."""

    def __init__(self, cfg, contract=False):
        self.cfg = dict(cfg)
        self.desc = make_desc(cfg)
        self.L = lib(contract)
        self.h = self.L.or_create(ctypes.byref(self.desc))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.dim = self.desc.dim
        self.n = [self.desc.n[k] for k in range(3)]
        self.gs = [self.n[k] + 4 if k < self.dim else 1 for k in range(3)]
        self.num_cells = int(self.L.or_num_cells(self.h))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.or_destroy(h)
            self.h = None

    # state I/O ---------------------------------------------------------
    def reset_state(self, cons_interior):
        """cons_interior: float64 array (..., 6) in x-fastest order, interior cells only."""
        a = np.ascontiguousarray(cons_interior, dtype=np.float64).reshape(-1, 6)
        assert a.shape[0] == self.n[0] * self.n[1] * self.n[2]
        self.L.or_reset_state(self.h, _ptr(a))

    def get_interior(self):
        out = np.empty((self.n[0] * self.n[1] * self.n[2], 6), dtype=np.float64)
        self.L.or_get_interior(self.h, _ptr(out))
        return out

    def get_full(self):
        out = np.empty((self.num_cells, 6), dtype=np.float64)
        self.L.or_get_state_full(self.h, _ptr(out))
        return out

    def set_full(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.num_cells, 6)
        self.L.or_set_state_full(self.h, _ptr(a))

    # the reference's solver verbs -----------------------------------------
    def boundary(self):
        self.L.or_boundary(self.h)

    def constrainU(self):
        self.L.or_constrain_u(self.h)

    def calcDT(self):
        return self.L.or_calc_dt(self.h)

    def step(self, dt):
        self.L.or_step(self.h, float(dt))

    def update(self):
        return self.L.or_update(self.h)

    @property
    def t(self):
        return self.L.or_get_t(self.h)

    @t.setter
    def t(self, v):
        self.L.or_set_t(self.h, float(v))

    def run_until(self, t_end, max_steps=1 << 40):
        return int(self.L.or_run_until(self.h, float(t_end), int(max_steps)))

    def calc_deriv(self, dt):
        out = np.empty((self.num_cells, 6), dtype=np.float64)
        self.L.or_calc_deriv(self.h, float(dt), _ptr(out))
        return out


def roe_flux(cfg, UL, UR, side):
    d = make_desc(cfg)
    a = np.ascontiguousarray(UL, dtype=np.float64)
    b = np.ascontiguousarray(UR, dtype=np.float64)
    out = np.empty(6)
    lib().or_roe_flux(ctypes.byref(d), _ptr(a), _ptr(b), int(side), _ptr(out))
    return out


def interface_flux(cfg, UL, UR, side):
    """The interface flux of cfg["flux"] (roe without a limiter, hll, rusanov)."""
    d = make_desc(cfg)
    a = np.ascontiguousarray(UL, dtype=np.float64)
    b = np.ascontiguousarray(UR, dtype=np.float64)
    out = np.empty(6)
    lib().or_interface_flux(ctypes.byref(d), _ptr(a), _ptr(b), int(side), _ptr(out))
    return out


def eigen_basis(cfg, UL, UR, side):
    d = make_desc(cfg)
    a = np.ascontiguousarray(UL, dtype=np.float64)
    b = np.ascontiguousarray(UR, dtype=np.float64)
    L = np.empty(25)
    R = np.empty(25)
    lam = np.empty(5)
    lib().or_eigen_basis(ctypes.byref(d), _ptr(a), _ptr(b), int(side), _ptr(L), _ptr(R), _ptr(lam))
    return L.reshape(5, 5), R.reshape(5, 5), lam


def limiter(name_or_index, r):
    idx = LIMITERS.index(name_or_index) if isinstance(name_or_index, str) else int(name_or_index)
    return lib().or_limiter(idx, float(r))


class plm_athena_recorded_edges:
    """Within this context "plm athena" assigns the cell's L state from its
    left-edge value and R from its right-edge value, as the revision that
    recorded the reference's 'plm-athena' errors did; outside it the oracle
    follows the current source, which swaps the two (plm.cl:877-878)."""

    def __enter__(self):
        lib().or_set_plm_athena_recorded_edges(1)
        return self

    def __exit__(self, *exc):
        lib().or_set_plm_athena_recorded_edges(0)
        return False


def num_threads():
    return int(lib().or_num_threads())
