"""Python host side of libhydrocuda: the reference's solver-args vocabulary over the C ABI.

hydro-cl-lua builds a solver from one Lua args table (hydro/solver/solverbase.lua:324-338,
hydro/solver/gridsolver.lua:98-104, hydro/solver/fvsolver.lua:201-206), e.g.

    FiniteVolumeSolver{dim=2, gridSize={1024,1024}, mins=..., maxs=..., boundary={xmin='periodic', ...},
                       flux='roe', fluxLimiter='donor cell', usePLM='plm cons', slopeLimiter='monotized central',
                       integrator='Runge-Kutta 3, TVD', cfl=.4, eqnArgs={...}}

``Solver(**args)`` takes the same keys and the same names, maps them onto
``hc_solver_desc`` and forwards the solver verbs (``boundary``, ``constrainU``,
``calcDT``, ``step``, ``update``) to ``libhydrocuda.so``.  Unknown names raise
``ValueError`` (the reference falls back to the first table entry with a
printed warning, solverbase.lua:795-812; failing loudly is safer for a
library).  There is no CPU fallback: if the CUDA library cannot be loaded or a
call fails, ``HydroCudaError`` is raised.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhydrocuda.so")

# hydro/app.lua:614-635, in table order
LIMITERS = [
    "donor cell", "Lax-Wendroff", "Beam-Warming", "Fromm", "CHARM", "HCUS",
    "HQUICK", "Koren", "minmod", "Oshker", "ospre", "smart", "Sweby", "UMIST",
    "van Albada 1", "van Albada 2", "van Leer", "monotized central",
    "superbee", "Barth-Jespersen",
    # beyond the reference's table: the van Leer form the reference keeps in a
    # comment (hydro/app.lua:631), equal to "van Leer" except at r = -1, where
    # the table's expression is 0/0
    "van Leer (abs)",
]
# hydro/int/all.lua (explicit integrators)
INTEGRATORS = [
    "forward Euler", "Runge-Kutta 2", "Runge-Kutta 2 Heun", "Runge-Kutta 2 Ralston",
    "Runge-Kutta 3", "Runge-Kutta 4", "Runge-Kutta 4, 3/8ths rule", "Runge-Kutta 2, TVD",
    "Runge-Kutta 2, non-TVD", "Runge-Kutta 3, TVD", "Runge-Kutta 4, TVD", "Runge-Kutta 4, non-TVD",
]
BOUNDARIES = {"none": 0, "periodic": 1, "mirror": 2, "freeflow": 3, "linear": 4, "quadratic": 5, "fixed": 6}
RECONS = {None: 0, False: 0, "piecewise constant": 1, "plm cons": 2, "plm prim": 3, "plm athena": 4}
# hydro/flux/*.lua names
FLUXES = ["roe", "hll", "rusanov", "euler-hllc"]
PRECISIONS = {"f64 plain": 0, "f64": 1, "f32": 2}
LAYOUTS = {"aos6": 0, "soa5": 1, "soa5_f32": 2}
SIDES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")

HC_OK = 0
ERRORS = {-1: "HC_ERR_INVALID", -2: "HC_ERR_CUDA", -3: "HC_ERR_NOMEM", -4: "HC_ERR_BUDGET",
          -5: "HC_ERR_NO_SLOT", -6: "HC_ERR_NONFINITE", -7: "HC_ERR_TIMEOUT", -8: "HC_ERR_STATE"}


class HydroCudaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


class SolverDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("n", ctypes.c_int * 3),
        ("mins", ctypes.c_double * 3), ("maxs", ctypes.c_double * 3),
        ("boundary", ctypes.c_int * 6),
        ("flux_limiter", ctypes.c_int), ("recon", ctypes.c_int), ("slope_limiter", ctypes.c_int),
        ("integrator", ctypes.c_int), ("precision", ctypes.c_int),
        ("gamma", ctypes.c_double), ("rho_min", ctypes.c_double), ("p_min", ctypes.c_double),
        ("cfl", ctypes.c_double), ("fixed_dt", ctypes.c_double),
        ("flux", ctypes.c_int), ("hllc_method", ctypes.c_int),
        ("entropy_fix", ctypes.c_int), ("reserved0", ctypes.c_int), ("entropy_fix_factor", ctypes.c_double),
        ("fixed_cons", (ctypes.c_double * 5) * 6),
    ]


class BatchDesc(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int), ("flux_limiter", ctypes.c_int), ("recon", ctypes.c_int),
        ("slope_limiter", ctypes.c_int), ("integrator", ctypes.c_int), ("max_slots", ctypes.c_int),
        ("hbm_budget", ctypes.c_size_t), ("flux", ctypes.c_int), ("hllc_method", ctypes.c_int),
    ]


class Done(ctypes.Structure):
    _fields_ = [("slot", ctypes.c_int), ("status", ctypes.c_int), ("tag", ctypes.c_ulonglong),
                ("steps", ctypes.c_longlong), ("t", ctypes.c_double)]


class BatchStats(ctypes.Structure):
    _fields_ = [("active", ctypes.c_int), ("occupied", ctypes.c_int), ("bytes_in_use", ctypes.c_size_t),
                ("tiles", ctypes.c_longlong), ("cells", ctypes.c_longlong), ("n_stages", ctypes.c_int),
                ("tile", (ctypes.c_int * 3) * 3), ("schedule", ctypes.c_int * 3), ("marching", ctypes.c_int * 3)]


class Init(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("reserved", ctypes.c_int), ("seed", ctypes.c_ulonglong),
                ("p", ctypes.c_double * 16)]


INIT_KINDS = {"sod": 0, "blast": 1, "quadrant": 2, "kelvin-helmholtz": 3}

# HC_DISPLAY_*: the reference's display variable names (hydro/eqn/euler.lua:240-260,
# the state fields of eqn.lua:913-915), vectors by component
DISPLAY_VARS = ["rho", "m x", "m y", "m z", "m mag", "ETotal", "ePot", "v x", "v y", "v z", "v mag", "P",
                "eInt", "eKin", "eTotal", "EInt", "EKin", "EPot", "S", "H", "h", "HTotal", "hTotal",
                "speed of sound", "Mach number", "temperature"]
RENDER_MODES = {"heatmap": 0, "volume": 1, "lic": 2, "slices": 3}
PALETTES = ["white-rainbow-black", "stripes", "blue", "paraview-red-grey-blue"]


class Render(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("var", ctypes.c_int), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("palette", ctypes.c_int), ("use_log", ctypes.c_int),
                ("value_min", ctypes.c_double), ("value_max", ctypes.c_double),
                ("bbox", ctypes.c_double * 4), ("slice_angle", ctypes.c_double * 4), ("fixed_z", ctypes.c_double),
                ("eye", ctypes.c_double * 3), ("fov_y", ctypes.c_double),
                ("alpha", ctypes.c_double), ("alpha_gamma", ctypes.c_double), ("num_isobars", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("use_isobars", ctypes.c_int), ("use_lighting", ctypes.c_int),
                ("lic_iter", ctypes.c_int), ("noise_size", ctypes.c_int), ("reserved", ctypes.c_int),
                ("noise_seed", ctypes.c_ulonglong), ("slice_axis", ctypes.c_int), ("num_slices", ctypes.c_int)]


def display_index(var):
    if isinstance(var, str):
        if var not in DISPLAY_VARS:
            raise ValueError("unknown display variable %r" % (var,))
        return DISPLAY_VARS.index(var)
    return int(var)


# every entry point of include/hydrocuda.h with its argument types
_vp, _dp, _ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
PROTOTYPES = {
    "hc_version": (ctypes.c_char_p, []),
    "hc_last_error": (ctypes.c_char_p, []),
    "hc_device_count": (_ip, [ctypes.POINTER(ctypes.c_int)]),
    "hc_context_create": (_ip, [_ip, ctypes.POINTER(_vp)]),
    "hc_context_destroy": (_ip, [_vp]),
    "hc_host_alloc": (_ip, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "hc_host_free": (_ip, [_vp]),
    "hc_init_defaults": (_ip, [_ip, ctypes.POINTER(Init)]),
    "hc_solver_create": (_ip, [_vp, ctypes.POINTER(SolverDesc), ctypes.POINTER(_vp)]),
    "hc_solver_destroy": (_ip, [_vp]),
    "hc_solver_reset_state": (_ip, [_vp, _vp, _ip]),
    "hc_solver_init_state": (_ip, [_vp, ctypes.POINTER(Init)]),
    "hc_solver_set_state": (_ip, [_vp, _vp, _ip, _ip]),
    "hc_solver_get_state": (_ip, [_vp, _vp, _ip, _ip]),
    "hc_solver_boundary": (_ip, [_vp]),
    "hc_solver_constrain_u": (_ip, [_vp]),
    "hc_solver_calc_dt": (_ip, [_vp, _dp]),
    "hc_solver_step": (_ip, [_vp, ctypes.c_double]),
    "hc_solver_update": (_ip, [_vp, _dp]),
    "hc_measure_fma": (_ip, [_ip, _dp]),
    "hc_solver_autotune": (_ip, [_vp, ctypes.c_char_p]),
    "hc_solver_stage": (_ip, [_vp, ctypes.c_double]),
    "hc_solver_num_stages": (_ip, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "hc_solver_get_slab": (_ip, [_vp, _ip, _ip, _dp]),
    "hc_solver_set_slab": (_ip, [_vp, _ip, _ip, _dp]),
    "hc_solver_run_until": (_ip, [_vp, ctypes.c_double, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "hc_solver_get_time": (_ip, [_vp, _dp]),
    "hc_solver_set_time": (_ip, [_vp, ctypes.c_double]),
    "hc_solver_conservation": (_ip, [_vp, _dp]),
    "hc_solver_status": (_ip, [_vp]),
    "hc_batch_create": (_ip, [_vp, ctypes.POINTER(BatchDesc), ctypes.POINTER(_vp)]),
    "hc_batch_destroy": (_ip, [_vp]),
    "hc_batch_admit": (_ip, [_vp, ctypes.POINTER(SolverDesc), _vp, _ip, ctypes.c_double, ctypes.c_longlong,
                             ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_admit_init": (_ip, [_vp, ctypes.POINTER(SolverDesc), ctypes.POINTER(Init), ctypes.c_double,
                                  ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_step": (_ip, [_vp, _ip, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_step_async": (_ip, [_vp, _ip]),
    "hc_batch_wait": (_ip, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_step_timed": (_ip, [_vp, _ip, _dp, _ip, _dp]),
    "hc_batch_poll": (_ip, [_vp, ctypes.POINTER(Done), _ip, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_list": (_ip, [_vp, ctypes.POINTER(Done), _ip, ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_fetch": (_ip, [_vp, _ip, _vp, _ip]),
    "hc_batch_admit_many": (_ip, [_vp, _ip, ctypes.POINTER(SolverDesc), ctypes.POINTER(_vp), _ip, _dp,
                                  ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_ulonglong),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "hc_batch_fetch_many": (_ip, [_vp, _ip, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_vp), _ip]),
    "hc_batch_retire": (_ip, [_vp, _ip]),
    "hc_batch_stats_get": (_ip, [_vp, ctypes.POINTER(BatchStats)]),
    "hc_batch_conservation": (_ip, [_vp, _ip, _dp]),
    "hc_batch_autotune": (_ip, [_vp, ctypes.c_char_p]),
    "hc_batch_set_schedule": (_ip, [_vp, _ip, _ip]),
    "hc_solver_display": (_ip, [_vp, _ip, _ip, _dp]),
    "hc_solver_display_range": (_ip, [_vp, _ip, _dp]),
    "hc_render_defaults": (_ip, [_ip, ctypes.POINTER(Render)]),
    "hc_solver_render": (_ip, [_vp, ctypes.POINTER(Render), _vp]),
    "hc_calc_dt_noalloc": (_ip, [ctypes.POINTER(SolverDesc), _vp, _vp, _vp]),
}

_lib = None


def load_library(path=None):
    """Loads libhydrocuda.so (building it first when it is missing); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location("hydrocuda_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(code):
    if code != HC_OK:
        raise HydroCudaError(code, _lib.hc_last_error().decode())


def measure_fma(precision="f32"):
    """The current device's FMA throughput in TFLOP/s (hc_measure_fma)."""
    L = load_library()
    v = ctypes.c_double()
    _check(L.hc_measure_fma(PRECISIONS[precision], ctypes.byref(v)))
    return v.value


def device_count():
    L = load_library()
    n = ctypes.c_int(0)
    _check(L.hc_device_count(ctypes.byref(n)))
    return n.value


class Context:
    """One CUDA device and the stream the solvers on it use."""

    def __init__(self, device=0):
        self.L = load_library()
        self.h = ctypes.c_void_p()
        _check(self.L.hc_context_create(int(device), ctypes.byref(self.h)))
        self.device = device

    def close(self):
        if self.h:
            self.L.hc_context_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _index(table, name, what):
    if isinstance(name, int):
        return name
    try:
        return table.index(name)
    except ValueError:
        raise ValueError("unknown %s %r" % (what, name))


def make_render(mode="heatmap", **kw):
    """hc_render with the reference's defaults for `mode`, updated from kw
    (var may be a display variable name, palette a palette name)."""
    L = load_library()
    r = Render()
    _check(L.hc_render_defaults(RENDER_MODES[mode], ctypes.byref(r)))
    for k, v in kw.items():
        if k == "var":
            v = display_index(v)
        elif k == "palette" and isinstance(v, str):
            v = PALETTES.index(v)
        elif k in ("use_log", "use_isobars", "use_lighting"):
            v = int(bool(v))
        if k in ("bbox", "slice_angle", "eye"):
            arr = getattr(r, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        elif not hasattr(r, k):
            raise ValueError("hc_render has no field %r" % (k,))
        else:
            setattr(r, k, v)
    return r


def make_init(kind, **params):
    """An initial condition for the device (hc_init).  kind: "sod" (rhoL, PL, rhoR,
    PR), "blast" (radius, Pin, Pout, rho), "quadrant" (q: 4 x (rho, vx, vy, P), as
    random_quadrants returns), "kelvin-helmholtz" (seed, noise); parameters not
    given keep the library's defaults.  The states equal those of sod_state,
    blast_state, quadrant_state and kelvin_helmholtz_state bit for bit."""
    L = load_library()
    ic = Init()
    _check(L.hc_init_defaults(INIT_KINDS[kind], ctypes.byref(ic)))
    names = {"sod": ("rhoL", "PL", "rhoR", "PR"), "blast": ("radius", "Pin", "Pout", "rho"),
             "kelvin-helmholtz": ("noise",), "quadrant": ()}[kind]
    for k, v in params.items():
        if k == "seed" and kind == "kelvin-helmholtz":
            ic.seed = int(v)
        elif k == "q" and kind == "quadrant":
            flat = [float(x) for quad in v for x in quad]
            if len(flat) != 16:
                raise ValueError("quadrant: q must hold 4 x (rho, vx, vy, P)")
            for i, x in enumerate(flat):
                ic.p[i] = x
        elif k in names:
            ic.p[names.index(k)] = float(v)
        else:
            raise ValueError("unknown parameter %r for %s" % (k, kind))
    return ic


def make_desc(args):
    """Maps a reference-style solver args dict onto hc_solver_desc."""
    d = SolverDesc()
    dim = int(args["dim"])
    if args.get("eqn", "euler") != "euler":
        raise ValueError("only eqn='euler' is provided")
    d.flux = _index(FLUXES, args.get("flux", "roe"), "flux")
    # euler-hllc's hllcMethod (0, 1, 2; the reference's default 2); 0 in the descriptor is that default
    d.hllc_method = int(args["hllcMethod"]) + 1 if "hllcMethod" in args else 0
    if args.get("coord", "cartesian") != "cartesian":
        raise ValueError("only coord='cartesian' is provided")
    gs = args["gridSize"]
    if isinstance(gs, (int, np.integer)):
        gs = [int(gs)]
    mins = list(args.get("mins", [-1, -1, -1])) + [-1.0] * 3
    maxs = list(args.get("maxs", [1, 1, 1])) + [1.0] * 3
    d.dim = dim
    for k in range(3):
        d.n[k] = int(gs[k]) if k < dim else 1
        d.mins[k] = float(mins[k])
        d.maxs[k] = float(maxs[k])
    bnd = args.get("boundary", {}) or {}
    if isinstance(bnd, str):
        bnd = {k: bnd for k in SIDES}
    eq = args.get("eqnArgs", {}) or {}
    for k, side in enumerate(SIDES):
        name = bnd.get(side, "freeflow")
        if isinstance(name, dict):
            # {"name": "fixed", "cons": [...]} or {"name": "fixed", "prim": {...}}
            cons = fixed_cons(name, float(eq.get("heatCapacityRatio", 7.0 / 5.0)))
            for f in range(5):
                d.fixed_cons[k][f] = cons[f]
            name = name["name"]
        if name not in BOUNDARIES:
            raise ValueError("unknown boundary %r" % name)
        d.boundary[k] = BOUNDARIES[name]
    d.flux_limiter = _index(LIMITERS, args.get("fluxLimiter", "donor cell"), "fluxLimiter")
    plm = args.get("usePLM", None)
    if plm not in RECONS:
        raise ValueError("unknown usePLM %r" % (plm,))
    d.recon = RECONS[plm]
    d.slope_limiter = _index(LIMITERS, args.get("slopeLimiter", "donor cell"), "slopeLimiter")
    d.integrator = _index(INTEGRATORS, args.get("integrator", "forward Euler"), "integrator")
    prec = args.get("precision", "f64 plain")
    if prec not in PRECISIONS:
        raise ValueError("unknown precision %r" % prec)
    d.precision = PRECISIONS[prec]
    eq = args.get("eqnArgs", {}) or {}
    d.gamma = float(eq.get("heatCapacityRatio", 7.0 / 5.0))
    d.rho_min = float(eq.get("rhoMin", 1e-7))
    d.p_min = float(eq.get("PMin", 1e-7))
    d.cfl = float(args.get("cfl", 0.5))
    d.fixed_dt = float(args.get("fixedDT", 0.0) or 0.0)
    # the Roe flux's entropy fix (hydro/flux/roe.lua:10-16)
    d.entropy_fix = 1 if args.get("useEntropyFluxFix", False) else 0
    d.entropy_fix_factor = float(args.get("entropyFluxFixLimitingFactor", 0.2))
    return d


def fixed_cons(spec, gamma):
    """The constant ghost state of a 'fixed' boundary side (the reference's
    BoundaryFixed takes generated fixedCode; here the state itself):
    {"name": "fixed", "cons": [rho, m.x, m.y, m.z, ETotal]} or
    {"name": "fixed", "prim": {"rho": r, "v": [vx, vy, vz], "P": p}} (consFromPrim)."""
    if spec.get("name") != "fixed":
        return [0.0] * 5
    if "cons" in spec:
        c = [float(x) for x in spec["cons"]]
        if len(c) != 5:
            raise ValueError("a fixed boundary's cons has 5 values")
        return c
    w = spec["prim"]
    v = [float(x) for x in list(w.get("v", [0, 0, 0])) + [0.0] * 3][:3]
    return [float(x) for x in cons_from_prim(float(w["rho"]), v[0], v[1], v[2], float(w["P"]), gamma)[0, :5]]


def interior_count(desc):
    n = 1
    for k in range(desc.dim):
        n *= desc.n[k]
    return n


def _as_layout(cons, layout, ncell):
    if layout == "aos6":
        a = np.ascontiguousarray(cons, dtype=np.float64).reshape(ncell, 6)
    elif layout == "soa5":
        a = np.ascontiguousarray(cons, dtype=np.float64).reshape(5, ncell)
    elif layout == "soa5_f32":
        a = np.ascontiguousarray(cons, dtype=np.float32).reshape(5, ncell)
    else:
        raise ValueError("unknown layout %r" % layout)
    return a


class Solver:
    """A 'cuda' FiniteVolumeSolver (eqn='euler', flux='roe') on one GPU."""

    def __init__(self, ctx=None, **args):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        self.args = dict(args)
        self.desc = make_desc(args)
        self.dim = self.desc.dim
        self.gridSize = [self.desc.n[k] for k in range(self.dim)]
        self.num_interior = interior_count(self.desc)
        self.numGhost = 2
        self.h = ctypes.c_void_p()
        _check(self.L.hc_solver_create(self.ctx.h, ctypes.byref(self.desc), ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.hc_solver_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # state ---------------------------------------------------------------
    def resetState(self, cons, layout="aos6"):
        """resetState with the given interior conserved state (applyInitCond's output)."""
        a = _as_layout(cons, layout, self.num_interior)
        _check(self.L.hc_solver_reset_state(self.h, a.ctypes.data, LAYOUTS[layout]))

    def initState(self, kind, **params):
        """resetState with the initial condition built on the device (see make_init)."""
        ic = make_init(kind, **params)
        _check(self.L.hc_solver_init_state(self.h, ctypes.byref(ic)))

    def setState(self, cons, layout="aos6", withGhosts=False):
        if withGhosts:
            a = np.ascontiguousarray(cons, dtype=np.float64)
        else:
            a = _as_layout(cons, layout, self.num_interior)
        _check(self.L.hc_solver_set_state(self.h, a.ctypes.data, LAYOUTS[layout], int(bool(withGhosts))))

    def getState(self, layout="aos6", withGhosts=False):
        if withGhosts:
            n = 1
            for k in range(self.dim):
                n *= self.gridSize[k] + 4
            out = np.empty((n, 6), dtype=np.float64)
        elif layout == "aos6":
            out = np.empty((self.num_interior, 6), dtype=np.float64)
        elif layout == "soa5":
            out = np.empty((5, self.num_interior), dtype=np.float64)
        else:
            out = np.empty((5, self.num_interior), dtype=np.float32)
        _check(self.L.hc_solver_get_state(self.h, out.ctypes.data, LAYOUTS[layout], int(bool(withGhosts))))
        return out

    # display ------------------------------------------------------------------
    def display(self, var, zeroBorder=False):
        """calcDisplayVarToBuffer: the display variable at every cell of the grid,
        ghosts included (shape: the grid with ghosts, z, y, x)."""
        shape = tuple(self.gridSize[k] + 4 for k in reversed(range(self.dim)))
        out = np.empty(shape, dtype=np.float64)
        _check(self.L.hc_solver_display(self.h, display_index(var), int(bool(zeroBorder)),
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def displayRange(self, var):
        """calcDisplayVarRangeAndAvgAndStdDev: (min, max, mean, standard deviation)."""
        out = (ctypes.c_double * 4)()
        _check(self.L.hc_solver_display_range(self.h, display_index(var), out))
        return tuple(out)

    def render(self, mode="heatmap", var="rho", **kw):
        """An RGBA8 image (height, width, 4) of the state: mode 'heatmap'
        (2d_heatmap.glsl), 'volume' (volumetric.glsl), 'lic'
        (vector_lic.glsl) or 'slices' (3d_slice.glsl); keyword arguments set
        hc_render fields."""
        r = make_render(mode, var=var, **kw)
        out = np.empty((r.height, r.width, 4), dtype=np.uint8)
        _check(self.L.hc_solver_render(self.h, ctypes.byref(r), out.ctypes.data))
        return out

    # the reference's solver verbs -------------------------------------------
    def boundary(self):
        _check(self.L.hc_solver_boundary(self.h))

    def constrainU(self):
        _check(self.L.hc_solver_constrain_u(self.h))

    def calcDT(self):
        dt = ctypes.c_double()
        _check(self.L.hc_solver_calc_dt(self.h, ctypes.byref(dt)))
        return dt.value

    def step(self, dt):
        _check(self.L.hc_solver_step(self.h, float(dt)))

    def update(self):
        dt = ctypes.c_double()
        _check(self.L.hc_solver_update(self.h, ctypes.byref(dt)))
        return dt.value

    def autotune(self, cache_path=None):
        """Picks the fused forms' fastest stage-kernel schedule for this grid
        (hc_solver_autotune); the solve is left as it was."""
        _check(self.L.hc_solver_autotune(self.h, cache_path.encode() if cache_path else None))

    # one grid cut into slabs (see hc_solver_stage in the header)
    @property
    def num_stages(self):
        n = ctypes.c_int()
        _check(self.L.hc_solver_num_stages(self.h, ctypes.byref(n)))
        return n.value

    def stage(self, dt):
        """The next Runge-Kutta stage of the update with the update's dt (hc_solver_stage)."""
        _check(self.L.hc_solver_stage(self.h, float(dt)))

    def _slab_cells(self, axis):
        n = 2
        for k in range(self.dim):
            if k != axis:
                n *= self.gridSize[k]
        return n

    def get_slab(self, axis, side):
        """The two interior layers next to face (axis, side) of the state the next stage reads,
        (cells, 6) float64 x-fastest over the two-layer slab."""
        out = np.empty((self._slab_cells(axis), 6), dtype=np.float64)
        _check(self.L.hc_solver_get_slab(self.h, int(axis), int(side), out.ctypes.data_as(_dp)))
        return out

    def set_slab(self, axis, side, cons):
        """Writes the two ghost layers beyond face (axis, side) of the state the next stage reads."""
        a = np.ascontiguousarray(cons, dtype=np.float64).reshape(self._slab_cells(axis), 6)
        _check(self.L.hc_solver_set_slab(self.h, int(axis), int(side), a.ctypes.data_as(_dp)))

    def run_until(self, t_end, max_steps=(1 << 62)):
        n = ctypes.c_longlong()
        _check(self.L.hc_solver_run_until(self.h, float(t_end), int(max_steps), ctypes.byref(n)))
        return n.value

    @property
    def t(self):
        v = ctypes.c_double()
        _check(self.L.hc_solver_get_time(self.h, ctypes.byref(v)))
        return v.value

    @t.setter
    def t(self, value):
        _check(self.L.hc_solver_set_time(self.h, float(value)))

    def conservation(self):
        s = (ctypes.c_double * 5)()
        _check(self.L.hc_solver_conservation(self.h, s))
        return np.array(list(s))

    def status(self):
        return self.L.hc_solver_status(self.h)


class Batch:
    """Many independent instances advanced together (continuous admission)."""

    def __init__(self, ctx=None, precision="f32", usePLM=None, slopeLimiter="donor cell",
                 fluxLimiter="donor cell", integrator="forward Euler", max_slots=1024,
                 hbm_budget=150 * (1 << 30), flux="roe", hllcMethod=None):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        d = BatchDesc()
        d.precision = PRECISIONS[precision]
        d.flux_limiter = _index(LIMITERS, fluxLimiter, "fluxLimiter")
        d.recon = RECONS[usePLM]
        d.slope_limiter = _index(LIMITERS, slopeLimiter, "slopeLimiter")
        d.integrator = _index(INTEGRATORS, integrator, "integrator")
        d.max_slots = int(max_slots)
        d.hbm_budget = int(hbm_budget)
        d.flux = _index(FLUXES, flux, "flux")
        d.hllc_method = int(hllcMethod) + 1 if hllcMethod is not None else 0
        self.desc = d
        self.scheme = dict(precision=precision, usePLM=usePLM, slopeLimiter=slopeLimiter,
                           fluxLimiter=fluxLimiter, integrator=integrator, flux=flux)
        if hllcMethod is not None:
            self.scheme["hllcMethod"] = hllcMethod
        self.h = ctypes.c_void_p()
        _check(self.L.hc_batch_create(self.ctx.h, ctypes.byref(d), ctypes.byref(self.h)))
        self.slot_desc = {}

    def close(self):
        if self.h:
            self.L.hc_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, args, cons, t_end, max_steps=0, tag=0, layout="aos6"):
        """Returns the slot; raises HydroCudaError (HC_ERR_BUDGET / HC_ERR_NO_SLOT) if refused."""
        a = dict(self.scheme)
        a.update(args)
        desc = make_desc(a)
        arr = _as_layout(cons, layout, interior_count(desc))
        slot = ctypes.c_int(-1)
        _check(self.L.hc_batch_admit(self.h, ctypes.byref(desc), arr.ctypes.data, LAYOUTS[layout],
                                     float(t_end), int(max_steps), int(tag), ctypes.byref(slot)))
        self.slot_desc[slot.value] = desc
        return slot.value

    def admit_many(self, items, layout="aos6"):
        """Admits every (args, cons, t_end, max_steps, tag) of `items` in one
        call (hc_batch_admit_many: one wait for all uploads).  Returns their
        slots; on a refusal raises HydroCudaError with `.slots` = the slots of
        the instances admitted before it (they stay admitted)."""
        n = len(items)
        descs = (SolverDesc * n)()
        ptrs = (_vp * n)()
        t_end = (ctypes.c_double * n)()
        steps = (ctypes.c_longlong * n)()
        tags = (ctypes.c_ulonglong * n)()
        keep = []
        for k, (args, cons, te, ms, tag) in enumerate(items):
            a = dict(self.scheme)
            a.update(args)
            descs[k] = make_desc(a)
            arr = _as_layout(cons, layout, interior_count(descs[k]))
            keep.append(arr)
            ptrs[k] = arr.ctypes.data
            t_end[k], steps[k], tags[k] = float(te), int(ms), int(tag)
        slots = (ctypes.c_int * max(n, 1))()
        got = ctypes.c_int(0)
        code = self.L.hc_batch_admit_many(self.h, n, descs, ptrs, LAYOUTS[layout], t_end, steps, tags, slots,
                                          ctypes.byref(got))
        out = [slots[k] for k in range(got.value)]
        for k, slot in enumerate(out):
            self.slot_desc[slot] = SolverDesc.from_buffer_copy(descs[k])
        if code != HC_OK:
            err = HydroCudaError(code, _lib.hc_last_error().decode())
            err.slots = out
            raise err
        return out

    def admit_init(self, args, kind, t_end, max_steps=0, tag=0, **params):
        """admit with the initial condition built on the device (see make_init)."""
        a = dict(self.scheme)
        a.update(args)
        desc = make_desc(a)
        ic = make_init(kind, **params)
        slot = ctypes.c_int(-1)
        _check(self.L.hc_batch_admit_init(self.h, ctypes.byref(desc), ctypes.byref(ic), float(t_end), int(max_steps),
                                          int(tag), ctypes.byref(slot)))
        self.slot_desc[slot.value] = desc
        return slot.value

    def try_admit_init(self, args, kind, t_end, max_steps=0, tag=0, **params):
        """Like admit_init, but returns None when the budget or the slot table refuses."""
        try:
            return self.admit_init(args, kind, t_end, max_steps, tag, **params)
        except HydroCudaError as e:
            if e.code in (-4, -5):
                return None
            raise

    def try_admit(self, args, cons, t_end, max_steps=0, tag=0, layout="aos6"):
        """Like admit, but returns None when the budget or the slot table refuses."""
        try:
            return self.admit(args, cons, t_end, max_steps, tag, layout)
        except HydroCudaError as e:
            if e.code in (-4, -5):
                return None
            raise

    def step(self, steps=1):
        n = ctypes.c_int()
        _check(self.L.hc_batch_step(self.h, int(steps), ctypes.byref(n)))
        return n.value

    def step_async(self, steps=1):
        """Queues `steps` updates and returns at once (hc_batch_step_async)."""
        _check(self.L.hc_batch_step_async(self.h, int(steps)))

    def wait(self):
        """Waits for queued work; returns the instances still stepping (hc_batch_wait)."""
        n = ctypes.c_int()
        _check(self.L.hc_batch_wait(self.h, ctypes.byref(n)))
        return n.value

    def step_timed(self, steps=1):
        """Steps with CUDA events around each stage kernel; returns (stage_ms list, total_ms)."""
        n = self.stats()["n_stages"]
        st = (ctypes.c_double * max(n, 1))()
        tot = ctypes.c_double(0.0)
        _check(self.L.hc_batch_step_timed(self.h, int(steps), st, n, ctypes.byref(tot)))
        return [st[i] for i in range(n)], tot.value

    def poll(self, cap=4096):
        arr = (Done * cap)()
        n = ctypes.c_int()
        _check(self.L.hc_batch_poll(self.h, arr, cap, ctypes.byref(n)))
        return [dict(slot=arr[i].slot, status=arr[i].status, tag=arr[i].tag, steps=arr[i].steps, t=arr[i].t)
                for i in range(n.value)]

    def list(self, cap=4096):
        """Every occupied slot, finished or not (hc_batch_list): slot, status so far, tag, updates, t."""
        arr = (Done * cap)()
        n = ctypes.c_int()
        _check(self.L.hc_batch_list(self.h, arr, cap, ctypes.byref(n)))
        return [dict(slot=arr[i].slot, status=arr[i].status, tag=arr[i].tag, steps=arr[i].steps, t=arr[i].t)
                for i in range(n.value)]

    def fetch(self, slot, layout="aos6", out=None):
        """The slot's interior state in `layout`; written into `out` when given
        (a C-contiguous array of the layout's dtype and size, e.g. a view of
        pinned host memory), else into a new array."""
        desc = self.slot_desc[slot]
        n = interior_count(desc)
        shape, dtype = {"aos6": ((n, 6), np.float64), "soa5": ((5, n), np.float64),
                        "soa5_f32": ((5, n), np.float32)}[layout]
        if out is None:
            out = np.empty(shape, dtype=dtype)
        elif out.dtype != dtype or out.size != shape[0] * shape[1] or not out.flags["C_CONTIGUOUS"] \
                or not out.flags["WRITEABLE"]:
            raise ValueError("fetch: out must be a writeable C-contiguous %s array of %d values" % (
                np.dtype(dtype).name, shape[0] * shape[1]))
        _check(self.L.hc_batch_fetch(self.h, int(slot), out.ctypes.data, LAYOUTS[layout]))
        return out

    def fetch_many(self, slots, layout="aos6", outs=None):
        """fetch of every slot in one call (hc_batch_fetch_many: one wait for
        all copies); `outs` as fetch's `out`, one per slot, or None."""
        n = len(slots)
        shapes = []
        for slot in slots:
            # a slot not in use is refused by the library, before any copy
            m = interior_count(self.slot_desc[slot]) if slot in self.slot_desc else 1
            shapes.append({"aos6": ((m, 6), np.float64), "soa5": ((5, m), np.float64),
                           "soa5_f32": ((5, m), np.float32)}[layout])
        if outs is None:
            outs = [np.empty(sh, dtype=dt) for sh, dt in shapes]
        for o, (sh, dt) in zip(outs, shapes):
            if o.dtype != dt or o.size != sh[0] * sh[1] or not o.flags["C_CONTIGUOUS"] or not o.flags["WRITEABLE"]:
                raise ValueError("fetch_many: each out must be a writeable C-contiguous %s array of %d values" % (
                    np.dtype(dt).name, sh[0] * sh[1]))
        cs = (ctypes.c_int * max(n, 1))(*[int(s) for s in slots])
        ptrs = (_vp * max(n, 1))(*[o.ctypes.data for o in outs])
        _check(self.L.hc_batch_fetch_many(self.h, n, cs, ptrs, LAYOUTS[layout]))
        return outs

    def retire(self, slot):
        _check(self.L.hc_batch_retire(self.h, int(slot)))
        self.slot_desc.pop(slot, None)

    def stats(self):
        s = BatchStats()
        _check(self.L.hc_batch_stats_get(self.h, ctypes.byref(s)))
        return dict(active=s.active, occupied=s.occupied, bytes_in_use=s.bytes_in_use, tiles=s.tiles, cells=s.cells,
                    n_stages=s.n_stages, tile=[list(s.tile[d]) for d in range(3)], schedule=list(s.schedule),
                    marching=[bool(m) for m in s.marching])

    def conservation(self, slot):
        s = (ctypes.c_double * 5)()
        _check(self.L.hc_batch_conservation(self.h, int(slot), s))
        return np.array(list(s))

    def set_schedule(self, dim, variant):
        """Pins the stage kernel's schedule for grids of dimension `dim` (the
        autotuner log's variant number)."""
        _check(self.L.hc_batch_set_schedule(self.h, int(dim), int(variant)))

    def autotune(self, cache_path=None):
        _check(self.L.hc_batch_autotune(self.h, cache_path.encode() if cache_path else None))


# ---------------------------------------------------------------------------
# initial states (host, FP64): prim -> cons as consFromPrim does
# (hydro/eqn/euler.cl:163-173), cell centres as coord.lua:1399-1440
# ---------------------------------------------------------------------------

class SplitMix64:
    """Seeded 64-bit generator (SplitMix64) with uniform doubles in [0, 1)."""

    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.s = int(seed) & self.MASK

    def next_u64(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def splitmix_uniform_array(seed, n, lo, hi):
    """n uniforms in [lo, hi) from SplitMix64(seed), vectorised (same values as SplitMix64.uniform)."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        z = (np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)) & M
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
    return lo + (hi - lo) * u


def cell_centers(desc_or_args):
    d = desc_or_args if isinstance(desc_or_args, SolverDesc) else make_desc(desc_or_args)
    axes = []
    for k in range(d.dim):
        N = d.n[k]
        i = np.arange(N, dtype=np.float64) + 2
        axes.append((i + .5 - 2) / N * (d.maxs[k] - d.mins[k]) + d.mins[k])
    return axes


def cons_from_prim(rho, vx, vy, vz, P, gamma):
    """AoS-6 conserved state (rho, m, ETotal, ePot = 0) in the reference's expression order."""
    rho = np.asarray(rho, dtype=np.float64)
    out = np.zeros(rho.shape + (6,), dtype=np.float64)
    out[..., 0] = rho
    out[..., 1] = vx * rho
    out[..., 2] = vy * rho
    out[..., 3] = vz * rho
    out[..., 4] = rho * (.5 * (vx * vx + vy * vy + vz * vz)) + P / (gamma - 1.)
    return out.reshape(-1, 6)


def _grid(d):
    axes = cell_centers(d)
    if d.dim == 1:
        return (axes[0],)
    return tuple(np.meshgrid(*axes, indexing="ij"))


def _xfast(a, dim):
    """meshgrid(indexing='ij') arrays are (x, y, z); cells are x-fastest."""
    return np.ascontiguousarray(np.transpose(a, tuple(range(dim))[::-1])).reshape(-1) if dim > 1 else a


def sod_state(args, rhoL=1.0, PL=1.0, rhoR=0.125, PR=0.1):
    """Sod shock tube (hydro/init/euler.lua:742-752): left where x < mid on every active axis."""
    d = make_desc(args)
    gamma = d.gamma
    X = _grid(d)
    left = np.ones_like(X[0], dtype=bool)
    for k in range(d.dim):
        mid = (d.mins[k] + d.maxs[k]) * .5
        left &= X[k] < mid
    rho = np.where(left, rhoL, rhoR)
    P = np.where(left, PL, PR)
    z = np.zeros_like(rho)
    return cons_from_prim(_xfast(rho, d.dim), _xfast(z, d.dim), _xfast(z, d.dim), _xfast(z, d.dim),
                          _xfast(P, d.dim), gamma)


def kelvin_helmholtz_state(args, seed=2, noise=0.01):
    """Sharp-band Kelvin-Helmholtz: |y| < .25 has rho = 2, vx = +.5; else rho = 1, vx = -.5;
    P = 2.5; vy = noise * U(-1, 1) per cell from SplitMix64(seed) in x-fastest cell order."""
    d = make_desc(args)
    X, Y = _grid(d)
    inside = np.abs(Y) < 0.25
    rho = _xfast(np.where(inside, 2.0, 1.0), 2)
    vx = _xfast(np.where(inside, 0.5, -0.5), 2)
    vy = noise * splitmix_uniform_array(seed, rho.size, -1.0, 1.0)
    P = np.full_like(rho, 2.5)
    return cons_from_prim(rho, vx, vy, np.zeros_like(rho), P, d.gamma)


def blast_state(args, radius=0.2, Pin=1.0, Pout=0.1, rho=1.0):
    """Spherical blast: rho = 1, v = 0, P = Pin where |x_cell|^2 < radius^2, else Pout."""
    d = make_desc(args)
    X = _grid(d)
    r2 = np.zeros_like(X[0])
    for k in range(d.dim):
        r2 = r2 + X[k] * X[k]
    P = _xfast(np.where(r2 < radius * radius, Pin, Pout), d.dim)
    r = np.full_like(P, rho)
    z = np.zeros_like(P)
    return cons_from_prim(r, z, z, z, P, d.gamma)


def quadrant_state(args, q):
    """Four-quadrant Riemann problem (hydro/init/euler.lua:249-283): q is a list of 4
    (rho, vx, vy, P) in the reference's quadrant order (x>mid,y>mid), (x<=mid,y>mid),
    (x<=mid,y<=mid), (x>mid,y<=mid)."""
    d = make_desc(args)
    X, Y = _grid(d)
    xm = (d.mins[0] + d.maxs[0]) * .5
    ym = (d.mins[1] + d.maxs[1]) * .5
    xp = X > xm
    yp = Y > ym
    idx = np.where(yp, np.where(xp, 0, 1), np.where(~xp, 2, 3))
    qa = np.asarray(q, dtype=np.float64)
    rho = _xfast(qa[idx, 0], 2)
    vx = _xfast(qa[idx, 1], 2)
    vy = _xfast(qa[idx, 2], 2)
    P = _xfast(qa[idx, 3], 2)
    return cons_from_prim(rho, vx, vy, np.zeros_like(rho), P, d.gamma)


def random_quadrants(rng):
    """Per-quadrant rho, P ~ U(0.1, 2), vx, vy ~ U(-1, 1) from a SplitMix64 stream."""
    q = []
    for _ in range(4):
        rho = rng.uniform(0.1, 2.0)
        P = rng.uniform(0.1, 2.0)
        vx = rng.uniform(-1.0, 1.0)
        vy = rng.uniform(-1.0, 1.0)
        q.append((rho, vx, vy, P))
    return q


def batched_quadrant_sizes(count=512, seed=4, lo=64, hi=512):
    """N per instance, log-uniform in [lo, hi] (rounded), from SplitMix64(seed)."""
    rng = SplitMix64(seed)
    return [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(count)]
