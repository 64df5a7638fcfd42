"""ctypes front end of the C++ oracle — TEST INFRASTRUCTURE ONLY.

The oracle (``oracle/cmdg_oracle.cpp``) is a CPU FP64 restatement of
ClimateMachine.jl's DGModel tendency, LSRK54 integrator and reductions.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module; the product library never does.

Parity status: pinned against the isentropic-vortex golden errors of
``test/Numerics/DGMethods/Euler/isentropicvortex.jl:105-106`` and the LSRK54
order of ``test/Numerics/ODESolvers/ode_tests_convergence.jl:41``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

# CLIMAParameters.jl 0.2.0 Earth values (Planet: gas_constant / molmass_dryair,
# kappa_d = 2/7, T_0, MSLP, grav; SubgridScale: inv_Pr_turb = 3, C_smag = 0.21).
_R_D = 8.3144598 / 28.97e-3
_KAPPA_D = 2 / 7
_CP_D = _R_D / _KAPPA_D
EARTH = dict(
    R_d=_R_D,
    cp_d=_CP_D,
    cv_d=_CP_D - _R_D,
    T_0=273.16,
    grav=9.81,
    MSLP=1.01325e5,
    inv_Pr_turb=3.0,
    C_smag=0.21,
    planet_radius=6.371e6,
)


class Brick(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("ne", ctypes.c_int * 3),
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("periodic", ctypes.c_int * 3),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("warp", ctypes.c_int),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("R_d", ctypes.c_double),
        ("cp_d", ctypes.c_double),
        ("cv_d", ctypes.c_double),
        ("T_0", ctypes.c_double),
        ("grav", ctypes.c_double),
        ("MSLP", ctypes.c_double),
        ("inv_Pr_turb", ctypes.c_double),
        ("numflux", ctypes.c_int),
        ("orientation", ctypes.c_int),
        ("gravity", ctypes.c_int),
        ("ref_state", ctypes.c_int),
        ("subtract_off", ctypes.c_int),
        ("profile", ctypes.c_int),
        ("T_surface", ctypes.c_double),
        ("T_min", ctypes.c_double),
        ("turbulence", ctypes.c_int),
        ("rho_nu", ctypes.c_double),
        ("with_divergence", ctypes.c_int),
        ("C_smag", ctypes.c_double),
        ("planet_radius", ctypes.c_double),
        ("hyperdiffusion", ctypes.c_int),
        ("tau_hyper", ctypes.c_double),
        ("hyper_direction", ctypes.c_int),
        ("mms", ctypes.c_int),
    ]


class Shell(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int),
        ("nhorz", ctypes.c_int),
        ("nvert", ctypes.c_int),
        ("r_inner", ctypes.c_double),
        ("r_outer", ctypes.c_double),
        ("bc_inner", ctypes.c_int),
        ("bc_outer", ctypes.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (portable flags, any host)."""
    src = os.path.join(HERE, "cmdg_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "_build/liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.c_double
        dp = ctypes.POINTER(ctypes.c_double)
        L.om_create.restype = P
        L.om_create.argtypes = [ctypes.POINTER(Brick), ctypes.POINTER(Params)]
        L.om_create_shell.restype = P
        L.om_create_shell.argtypes = [ctypes.POINTER(Shell), ctypes.POINTER(Params)]
        L.om_free.argtypes = [P]
        L.om_nelem.restype = ctypes.c_int64
        L.om_nelem.argtypes = [P]
        L.om_Np.argtypes = [P]
        L.om_ngradflux.argtypes = [P]
        for name in ("om_vgeo", "om_sgeo", "om_aux", "om_gradflux", "om_D", "om_lgl_nodes", "om_lgl_weights"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [P]
        for name in ("om_vmapM", "om_vmapP"):
            getattr(L, name).restype = ctypes.POINTER(ctypes.c_int64)
            getattr(L, name).argtypes = [P]
        L.om_elemtobndy.restype = ctypes.POINTER(ctypes.c_int)
        L.om_elemtobndy.argtypes = [P]
        L.om_set_threads.argtypes = [ctypes.c_int]
        L.om_tendency.argtypes = [P, dp, dp, D, D, D]
        L.om_gradient_pass.argtypes = [P, dp]
        L.om_hyper_pass.argtypes = [P, dp]
        L.om_set_mms.argtypes = [P, dp, dp]
        for name in ("om_hyper_grad", "om_hyper_div"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [P]
        L.om_lsrk54.argtypes = [P, dp, dp, D, D, ctypes.c_int]
        L.om_solve.restype = ctypes.c_int
        L.om_solve.argtypes = [P, dp, D, D, D]
        L.om_norm.restype = D
        L.om_norm.argtypes = [P, dp]
        L.om_euclidean_distance.restype = D
        L.om_euclidean_distance.argtypes = [P, dp, dp]
        L.om_field_l2.argtypes = [P, dp, dp, dp, dp]
        L.om_weightedsum.restype = D
        L.om_weightedsum.argtypes = [P, dp, ctypes.c_int]
        L.om_courant_dt.restype = D
        L.om_courant_dt.argtypes = [P, dp, D]
        L.om_init_vortex.argtypes = [P, dp, D, D, D, D, D, D, D, D]
        L.om_init_bubble.argtypes = [P, dp, D, D, D, D, D, D]
        L.om_init_rest.argtypes = [P, dp]
        L.om_filter_matrix.restype = ctypes.c_int
        L.om_filter_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, dp]
        ip = ctypes.POINTER(ctypes.c_int)
        L.om_apply_filter.argtypes = [P, dp, dp, dp, ctypes.c_int, ip, ctypes.c_int]
        L.om_apply_tmar.argtypes = [P, dp, ip, ctypes.c_int]
        L.om_apply_mp_filter.argtypes = [P, dp, dp, dp, ctypes.c_int, ip, ctypes.c_int]
        L.om_create_scalar_hyper.restype = P
        L.om_create_scalar_hyper.argtypes = [ctypes.POINTER(Brick), dp, ctypes.c_int]
        L.om_scalar_hyper_tendency.argtypes = [P, dp, dp, D, D]
        L.om_scalar_hyper_lsrk54.argtypes = [P, dp, dp, D, ctypes.c_int]
        L.om_lsrk54_scalar.restype = D
        L.om_lsrk54_scalar.argtypes = [D, D, D]
        L.om_linear_tendency.argtypes = [P, dp, dp, D, D]
        L.om_hevi_create.restype = P
        L.om_hevi_create.argtypes = [P, D, ctypes.c_int, ctypes.c_int]
        L.om_hevi_free.argtypes = [P]
        L.om_hevi_solve.argtypes = [P, dp, dp]
        L.om_hevi_alpha.restype = D
        L.om_hevi_alpha.argtypes = [P]
        L.om_hevi_bandwidth.argtypes = [P]
        L.om_hevi_step.argtypes = [P, dp, D, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> int:
    return lib().om_set_threads(n)


# Auxiliary field indices of the oracle's (Np, NAUX, nelem) aux array
AUX = dict(x=0, y=1, z=2, Phi=3, gPhi=4, rho_ref=7, p_ref=8, T_ref=9, rhoe_ref=10, theta_v=11, air_T=12, Delta=13,
           Delta_h=14)
NAUX = 15
VGEO = dict(xi1x1=0, xi2x1=1, xi3x1=2, xi1x2=3, xi2x2=4, xi3x2=5, xi1x3=6, xi2x3=7, xi3x3=8, M=9, MI=10, MH=11,
            x1=12, x2=13, x3=14, JcV=15)


class OracleModel:
    """A brick mesh + dry AtmosModel configuration evaluated by the oracle."""

    def __init__(self, N, ne=None, lo=None, hi=None, periodic=(1, 1, 1), bc_lo=(1, 1, 1), bc_hi=(2, 2, 2),
                 shell=None, **physics):
        """Brick (N, ne, lo, hi, periodic, bc_lo, bc_hi) or, with
        ``shell=dict(nhorz, nvert, r_inner, r_outer)``, a stacked
        equiangular cubed shell with walls at both radii."""
        p = Params()
        consts = dict(EARTH)
        consts.update({k: v for k, v in physics.items() if k in EARTH})
        for k in ("R_d", "cp_d", "cv_d", "T_0", "grav", "MSLP", "inv_Pr_turb", "planet_radius"):
            setattr(p, k, consts[k])
        p.numflux = {"rusanov": 0, "central": 1}[physics.get("numflux", "rusanov")]
        p.orientation = {"none": 0, "flat": 1, "sphere": 2}[physics.get("orientation", "none")]
        p.gravity = int(physics.get("gravity", False))
        p.ref_state = int(physics.get("ref_state", False))
        p.subtract_off = int(physics.get("subtract_off", True))
        p.profile = {"isothermal": 0, "dry_adiabatic": 1}[physics.get("profile", "dry_adiabatic")]
        p.T_surface = physics.get("T_surface", 300.0)
        p.T_min = physics.get("T_min", 0.0)
        p.turbulence = {"none": 0, "constant": 1, "smagorinsky": 2}[physics.get("turbulence", "none")]
        p.rho_nu = physics.get("rho_nu", 0.0)
        p.with_divergence = int(physics.get("with_divergence", False))
        p.C_smag = physics.get("C_smag", consts["C_smag"])
        p.hyperdiffusion = {"none": 0, "dry_biharmonic": 1}[physics.get("hyperdiffusion", "none")]
        p.tau_hyper = physics.get("tau_hyper", 0.0)
        p.hyper_direction = {"every": 0, "horizontal": 1}[physics.get("hyper_direction", "every")]
        p.mms = int(physics.get("mms", False))
        self.params, self.consts = p, consts
        self.L = lib()
        if shell is None:
            b = Brick()
            b.N = N
            for d in range(3):
                b.ne[d] = ne[d]
                b.lo[d] = lo[d]
                b.hi[d] = hi[d]
                b.periodic[d] = int(periodic[d])
                b.bc_lo[d] = bc_lo[d]
                b.bc_hi[d] = bc_hi[d]
            b.warp = int(physics.get("warp", 0))
            self.brick = b
            self.h = self.L.om_create(ctypes.byref(b), ctypes.byref(p))
        else:
            sh = Shell()
            sh.N = N
            sh.nhorz = shell["nhorz"]
            sh.nvert = shell["nvert"]
            sh.r_inner = shell["r_inner"]
            sh.r_outer = shell["r_outer"]
            sh.bc_inner = shell.get("bc_inner", 1)
            sh.bc_outer = shell.get("bc_outer", 2)
            self.shell = sh
            self.h = self.L.om_create_shell(ctypes.byref(sh), ctypes.byref(p))
            if not self.h:
                raise RuntimeError("oracle: cubed-shell construction failed")
        self.N = N
        self.Nq = N + 1
        self.Np = self.L.om_Np(self.h)
        self.nelem = self.L.om_nelem(self.h)
        self.nstate = 5

    def __del__(self):
        if getattr(self, "h", None):
            self.L.om_free(self.h)
            self.h = None

    # ------------------------------------------------------------ arrays
    def _view(self, fn, shape, ctype=np.float64):
        ptr = fn(self.h)
        n = int(np.prod(shape))
        buf = np.ctypeslib.as_array(ptr, shape=(n,))
        return np.array(buf, dtype=ctype, copy=True).reshape(shape)

    @property
    def vgeo(self):
        return self._view(self.L.om_vgeo, (self.nelem, 16, self.Np))

    @property
    def sgeo(self):
        return self._view(self.L.om_sgeo, (self.nelem, 6, self.Nq * self.Nq, 5))

    @property
    def aux(self):
        return self._view(self.L.om_aux, (self.nelem, NAUX, self.Np))

    @property
    def gradflux(self):
        ngf = self.L.om_ngradflux(self.h)
        return self._view(self.L.om_gradflux, (self.nelem, ngf, self.Np))

    @property
    def vmapM(self):
        return self._view(self.L.om_vmapM, (self.nelem, 6, self.Nq * self.Nq), np.int64)

    @property
    def vmapP(self):
        return self._view(self.L.om_vmapP, (self.nelem, 6, self.Nq * self.Nq), np.int64)

    @property
    def elemtobndy(self):
        return self._view(self.L.om_elemtobndy, (self.nelem, 6), np.int32)

    @property
    def D(self):
        # column-major (Julia) D[j, k] stored at j + Nq*k -> numpy [k, j]; return D[j, k]
        return self._view(self.L.om_D, (self.Nq, self.Nq)).T.copy()

    @property
    def lgl(self):
        return self._view(self.L.om_lgl_nodes, (self.Nq,)), self._view(self.L.om_lgl_weights, (self.Nq,))

    def state(self):
        return np.zeros((self.nelem, self.nstate, self.Np), dtype=np.float64)

    # ------------------------------------------------------------ ops
    def tendency(self, Q, t=0.0, alpha=1.0, beta=0.0, dQ=None):
        if dQ is None:
            dQ = self.state()
        self.L.om_tendency(self.h, _ptr(dQ), _ptr(Q), t, alpha, beta)
        return dQ

    def gradient_pass(self, Q):
        self.L.om_gradient_pass(self.h, _ptr(Q))
        return self.gradflux

    def set_mms(self, src, exact):
        """Source terms and InitStateBC state (nelem, 5, Np) for the next
        tendency of an mms model; the arrays must stay alive until then."""
        self._mms = (np.ascontiguousarray(src, dtype=np.float64), np.ascontiguousarray(exact, dtype=np.float64))
        self.L.om_set_mms(self.h, _ptr(self._mms[0]), _ptr(self._mms[1]))

    def hyper_pass(self, Q):
        """Hyperdiffusion passes of Q: returns (nu grad^3 (nelem, 12, Np),
        laplacians (nelem, 4, Np))."""
        self.L.om_hyper_pass(self.h, _ptr(Q))
        return (self._view(self.L.om_hyper_grad, (self.nelem, 12, self.Np)),
                self._view(self.L.om_hyper_div, (self.nelem, 4, self.Np)))

    def lsrk54(self, Q, dt, nsteps, t0=0.0, dQ=None):
        if dQ is None:
            dQ = self.state()
        self.L.om_lsrk54(self.h, _ptr(Q), _ptr(dQ), t0, dt, nsteps)
        return Q, dQ

    def solve(self, Q, dt, timeend, t0=0.0):
        return self.L.om_solve(self.h, _ptr(Q), t0, dt, timeend)

    def norm(self, Q):
        return self.L.om_norm(self.h, _ptr(Q))

    def euclidean_distance(self, A, B):
        return self.L.om_euclidean_distance(self.h, _ptr(A), _ptr(B))

    def field_l2(self, A, B):
        err = np.zeros(5)
        ref = np.zeros(5)
        self.L.om_field_l2(self.h, _ptr(A), _ptr(B), _ptr(err), _ptr(ref))
        return err, ref

    def weightedsum(self, Q, field):
        return self.L.om_weightedsum(self.h, _ptr(Q), field)

    def courant_dt(self, Q, CFL):
        return self.L.om_courant_dt(self.h, _ptr(Q), CFL)

    def init_vortex(self, t=0.0, p_inf=1e5, T_inf=300.0, translation_speed=150.0, translation_angle=np.pi / 4,
                    vortex_speed=50.0, R=1 / 200, L=1 / 20):
        Q = self.state()
        self.L.om_init_vortex(self.h, _ptr(Q), t, p_inf, T_inf, translation_speed, translation_angle, vortex_speed,
                              R, L)
        return Q

    def init_bubble(self, theta0=300.0, amp=2.0, rc=250.0, xc=1250.0, yc=1250.0, zc=350.0):
        Q = self.state()
        self.L.om_init_bubble(self.h, _ptr(Q), theta0, amp, rc, xc, yc, zc)
        return Q

    def init_rest(self):
        Q = self.state()
        self.L.om_init_rest(self.h, _ptr(Q))
        return Q

    def linear_tendency(self, Q, alpha=1.0, beta=0.0, dQ=None):
        """AtmosAcousticGravityLinearModel tendency in VerticalDirection."""
        if dQ is None:
            dQ = self.state()
        self.L.om_linear_tendency(self.h, _ptr(dQ), _ptr(Q), alpha, beta)
        return dQ


class OracleHevi:
    """ARK2GiraldoKellyConstantinescu (LowStorageVariant) of an OracleModel
    with the vertical AtmosAcousticGravityLinearModel solved implicitly by the
    column-wise banded LU (AdditiveRungeKuttaMethod.jl:413-538, 839-897;
    columnwise_lu_solver.jl)."""

    def __init__(self, model: OracleModel, dt: float, split_explicit_implicit: bool = False,
                 paperversion: bool = False):
        self.model = model
        self.L = model.L
        self.dt = float(dt)
        self.h = self.L.om_hevi_create(model.h, self.dt, int(split_explicit_implicit), int(paperversion))
        if not self.h:
            raise ValueError("oracle HEVI needs wall-bounded stacks and a hydrostatic reference state")
        self.alpha = self.L.om_hevi_alpha(self.h)
        self.bandwidth = self.L.om_hevi_bandwidth(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.om_hevi_free(self.h)
            self.h = None

    def solve(self, Qhat):
        """Q with Q - alpha L(Q) = Qhat."""
        Q = np.empty_like(Qhat)
        self.L.om_hevi_solve(self.h, _ptr(Q), _ptr(np.ascontiguousarray(Qhat)))
        return Q

    def step(self, Q, nsteps=1, t0=0.0):
        self.L.om_hevi_step(self.h, _ptr(Q), t0, nsteps)
        return Q


FILTER_KINDS = {"exponential": 0, "cutoff": 1, "boyd_vandeven": 2}


def filter_matrix(N, kind, Nc, s=32, alpha=None):
    """spectral_filter_matrix of the named filter, W[i, n] (row = output node)."""
    if alpha is None:
        alpha = -np.log(np.finfo(np.float64).eps)
    W = np.zeros((N + 1, N + 1))
    if lib().om_filter_matrix(N, FILTER_KINDS[kind], Nc, s, alpha, _ptr(W)):
        raise ValueError("bad filter arguments")
    return W


def _fields(fields):
    arr = (ctypes.c_int * len(fields))(*fields)
    return arr, len(fields)


def apply_filter(model, Q, Wh, Wv, direction="every", fields=(0, 1, 2, 3, 4)):
    d = {"every": 0, "horizontal": 1, "vertical": 2}[direction]
    arr, n = _fields(fields)
    Wh = np.ascontiguousarray(Wh, dtype=np.float64)
    Wv = np.ascontiguousarray(Wv, dtype=np.float64)
    lib().om_apply_filter(model.h, _ptr(Q), _ptr(Wh), _ptr(Wv), d, arr, n)
    return Q


def apply_mp_filter(model, Q, Wh, Wv, direction="every", fields=(0, 1, 2, 3, 4)):
    """MassPreservingCutoffFilter application (Filters.jl:542-606, 895-1065)."""
    arr, n = _fields(fields)
    Wh = np.ascontiguousarray(Wh, dtype=np.float64)
    Wv = np.ascontiguousarray(Wv, dtype=np.float64)
    lib().om_apply_mp_filter(model.h, _ptr(Q), _ptr(Wh), _ptr(Wv), {"every": 0, "horizontal": 1, "vertical": 2}[direction],
                             arr, n)
    return Q


def apply_tmar(model, Q, fields):
    arr, n = _fields(fields)
    lib().om_apply_tmar(model.h, _ptr(Q), arr, n)
    return Q


def lsrk54_scalar(q0: float, dt: float, timeend: float) -> float:
    """q' = q cos t integrated with the oracle's LSRK54 (exact: q0 exp(sin t))."""
    return lib().om_lsrk54_scalar(q0, dt, timeend)


class ScalarHyperdiffusion:
    """Constant-tensor scalar hyperdiffusion d rho/dt = -div(H grad lap rho)
    on a brick (the AdvectionDiffusion model of
    test/Numerics/DGMethods/advection_diffusion/periodic_3D_hyperdiffusion.jl),
    evaluated by the same hyperdiffusion passes as the AtmosModel closure."""

    def __init__(self, N, ne, lo, hi, H, periodic=(1, 1, 1), direction="every"):
        b = Brick()
        b.N = N
        for d in range(3):
            b.ne[d], b.lo[d], b.hi[d], b.periodic[d] = ne[d], lo[d], hi[d], int(periodic[d])
            b.bc_lo[d], b.bc_hi[d] = 1, 2
        self.L = lib()
        Hc = np.ascontiguousarray(np.asarray(H, dtype=np.float64).T.reshape(9))  # column-major
        self.brick = b
        self.h = self.L.om_create_scalar_hyper(ctypes.byref(b), _ptr(Hc), {"every": 0, "horizontal": 1}[direction])
        self.N, self.Nq = N, N + 1
        self.Np = self.L.om_Np(self.h)
        self.nelem = self.L.om_nelem(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.om_free(self.h)
            self.h = None

    @property
    def vgeo(self):
        ptr = self.L.om_vgeo(self.h)
        n = self.nelem * 16 * self.Np
        return np.array(np.ctypeslib.as_array(ptr, shape=(n,))).reshape(self.nelem, 16, self.Np)

    def state(self):
        return np.zeros((self.nelem, 1, self.Np), dtype=np.float64)

    def tendency(self, Q, alpha=1.0, beta=0.0, dQ=None):
        if dQ is None:
            dQ = self.state()
        self.L.om_scalar_hyper_tendency(self.h, _ptr(dQ), _ptr(Q), alpha, beta)
        return dQ

    def lsrk54(self, Q, dt, nsteps, dQ=None):
        if dQ is None:
            dQ = self.state()
        self.L.om_scalar_hyper_lsrk54(self.h, _ptr(Q), _ptr(dQ), dt, nsteps)
        return Q, dQ


# ---------------------------------------------------------------------------
# Element orders of the reference's brick topologies, restated in plain Python
# integers (src/Numerics/Mesh/BrickMesh.jl:40-90 hilbertcode, :112-150
# centroidtocode, :531-627 partition's sort by code; src/Numerics/Mesh/
# Topologies.jl:632-715 StackedBrickTopology's contiguous columns).

def hilbertcode(Y, bits=64):
    """Hilbert index of the coordinates Y (each `bits` bits wide) as
    len(Y) words, most significant first: Skilling's axes-to-transpose
    followed by the transposition of BrickMesh.jl:78-87."""
    X = [int(y) for y in Y]
    n = len(X)
    M = 1 << (bits - 1)
    Q = M
    for _ in range(bits - 1):
        P = Q - 1
        for i in range(n):
            if X[i] & Q:
                X[0] ^= P
            else:
                t = (X[0] ^ X[i]) & P
                X[0] ^= t
                X[i] ^= t
        Q >>= 1
    for i in range(1, n):
        X[i] ^= X[i - 1]
    t = 0
    Q = M
    for _ in range(bits - 1):
        if X[n - 1] & Q:
            t ^= Q - 1
        Q >>= 1
    X = [x ^ t for x in X]
    H = [0] * n
    for i in range(n):
        for j in range(bits):
            k = i * bits + j
            bit = (X[n - 1 - (k % n)] >> (k // n)) & 1
            H[n - 1 - i] |= bit << j
    return H


def centroidtocode(elemtocorner):
    """Codes (d, nelem) of the element centroids of elemtocorner (d, nvert,
    nelem), as centroidtocode computes them on one rank: the centroid scaled
    by the elements' bounding box to [0, 1], times 2^64 - 1, floored
    exactly (BrickMesh.jl:112-150)."""
    from fractions import Fraction

    etc = np.asarray(elemtocorner, dtype=np.float64)
    d, nvert, nelem = etc.shape
    cent = np.zeros((d, nelem))
    for v in range(nvert):  # the reference sums the corners in order
        cent += etc[:, v, :]
    cent = cent / nvert
    lo, hi = cent.min(axis=1), cent.max(axis=1)
    size = hi - lo
    if np.all(size == 0):
        size = np.ones(d)
    else:
        size = np.where(size == 0, size.max(), size)
    code = np.zeros((d, nelem), dtype=np.uint64)
    top = (1 << 64) - 1
    for e in range(nelem):
        c = (cent[:, e] - lo) / size
        X = [int(Fraction(float(ci)) * top) for ci in c]  # floor of an exact product
        code[:, e] = np.array(hilbertcode(X, 64), dtype=np.uint64)
    return code


def range_point(lo, hi, n, k):
    """The k-th point of range(lo, stop=hi, length=n+1): the exact
    (lo (n - k) + hi k) / n rounded once to the nearest double."""
    from fractions import Fraction

    if k == 0:
        return float(lo)
    if k == n:
        return float(hi)
    return float((Fraction(lo) * (n - k) + Fraction(hi) * k) / n)


def brick_corners(ne, lo, hi):
    """elemtocorner (d, 2^d, nelem) of brickmesh over the ranges
    range(lo, hi, length=ne+1), elements in Cartesian order (x fastest)."""
    d = len(ne)
    nelem = int(np.prod(ne))
    etc = np.zeros((d, 1 << d, nelem))
    for e in range(nelem):
        r = e
        idx = []
        for i in range(d):
            idx.append(r % ne[i])
            r //= ne[i]
        for v in range(1 << d):
            for i in range(d):
                k = idx[i] + ((v >> i) & 1)
                etc[i, v, e] = range_point(lo[i], hi[i], ne[i], k)
    return etc


def hilbert_order(ne, lo, hi):
    """Cartesian indices of the elements of a brick in BrickTopology's
    order (sorted by code, ties by original index)."""
    code = centroidtocode(brick_corners(ne, lo, hi))
    keys = [tuple(int(c) for c in code[:, e]) + (e,) for e in range(code.shape[1])]
    return [k[-1] for k in sorted(keys)]


def reference_element_order(ne, lo, hi, topology):
    """perm[e_ref] = index in the library's stacked order (e = iz + nz (ix +
    nx iy)) of the element the reference's topology numbers e_ref:
    "brick" (3D Hilbert order) or "stacked_brick" (2D Hilbert order of the
    base, columns contiguous)."""
    nx, ny, nz = ne
    lib = lambda ix, iy, iz: iz + nz * (ix + nx * iy)
    if topology == "brick":
        return np.array([lib(c % nx, (c // nx) % ny, c // (nx * ny)) for c in hilbert_order(ne, lo, hi)])
    cols = hilbert_order(ne[:2], lo[:2], hi[:2])
    return np.array([lib(c % nx, c // nx, iz) for c in cols for iz in range(nz)])
