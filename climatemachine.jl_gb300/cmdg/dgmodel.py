"""DGModel and grid objects over libcmdg.so.

``DGModel`` mirrors the SpaceDiscretization functor of the reference:
``dg(tendency, Q, param, t; increment)`` computes
``tendency = dQ/dt(Q) + increment * tendency``
(src/Numerics/DGMethods/SpaceDiscretization.jl:68-77,
src/Numerics/DGMethods/DGModel.jl:85-427).  State arrays are torch tensors on
the current CUDA device of shape (nelem, 5, Np) — the same memory as the
reference's column-major MPIStateArray ``.data[Np, nstate, nelem]``.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._lib import AtmosParams, BrickDesc, ShellDesc, call

NSTATE = 5


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dptr(t: torch.Tensor):
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("state arrays must be contiguous CUDA tensors")
    return ctypes.c_void_p(t.data_ptr())


def brick_desc(N, ne, lo, hi, periodicity=(True, True, True), boundary=((1, 2), (1, 2), (1, 2))) -> BrickDesc:
    d = BrickDesc()
    d.N = int(N)
    for k in range(3):
        d.ne[k] = int(ne[k])
        d.lo[k] = float(lo[k])
        d.hi[k] = float(hi[k])
        d.periodic[k] = int(bool(periodicity[k]))
        d.bc_lo[k] = int(boundary[k][0])
        d.bc_hi[k] = int(boundary[k][1])
    return d


def brick_element_order(ne, lo, hi, topology: str) -> np.ndarray:
    """perm[e_ref] = library (stacked x-then-y) index of the element that
    the reference's topology ("brick": BrickTopology, "stacked_brick":
    StackedBrickTopology) numbers e_ref; host only, needs no GPU
    (cmdg_brick_element_order)."""
    _lib.load()
    d = brick_desc(2, ne, lo, hi)  # the order does not depend on N
    perm = np.empty(int(ne[0]) * int(ne[1]) * int(ne[2]), dtype=np.int64)
    call("cmdg_brick_element_order", ctypes.byref(d), BrickGrid.TOPOLOGIES[topology],
         ctypes.c_void_p(perm.ctypes.data))
    return perm


class BrickGrid:
    """BrickTopology/StackedBrickTopology + DiscontinuousSpectralElementGrid
    (src/Numerics/Mesh/Topologies.jl:470-545,632; src/Numerics/Mesh/Grids.jl:267-414).

    Elements are ordered with the vertical index fastest, then the columns
    in x-then-y order (``topology="library"``) or along the 2D Hilbert curve
    of the reference's StackedBrickTopology (``topology="stacked_brick"``),
    or all along the 3D Hilbert curve of BrickTopology (``topology="brick"``;
    HEVI refuses this order, its column solves need contiguous columns).
    ``boundary`` gives the tags of the (lower, upper) faces of each
    non-periodic direction, as in the reference's ``boundary`` keyword.
    """

    TOPOLOGIES = {"library": _lib.CMDG_TOPOLOGY_LIBRARY, "brick": _lib.CMDG_TOPOLOGY_BRICK,
                  "stacked_brick": _lib.CMDG_TOPOLOGY_STACKED_BRICK}

    def __init__(self, N, ne, lo, hi, periodicity=(True, True, True), boundary=((1, 2), (1, 2), (1, 2)),
                 topology="library"):
        _lib.load()
        d = brick_desc(N, ne, lo, hi, periodicity, boundary)
        h = ctypes.c_void_p()
        call("cmdg_mesh_create_brick_ordered", ctypes.byref(d), self.TOPOLOGIES[topology], ctypes.byref(h))
        self.topology = topology
        self.h = h
        self.desc = d
        nelem = ctypes.c_int64()
        Np = ctypes.c_int()
        call("cmdg_mesh_info", self.h, ctypes.byref(nelem), ctypes.byref(Np))
        self.N, self.Nq, self.nelem, self.Np = int(N), int(N) + 1, nelem.value, Np.value
        self.ne = tuple(int(x) for x in ne)

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.cmdg_mesh_destroy(self.h)
            self.h = None

    def _sizes(self):
        nelem = ctypes.c_int64()
        Np = ctypes.c_int()
        call("cmdg_mesh_info", self.h, ctypes.byref(nelem), ctypes.byref(Np))
        return nelem.value, Np.value

    def coordinates(self) -> np.ndarray:
        xyz = np.empty((self.nelem, 3, self.Np), dtype=np.float64)
        call("cmdg_mesh_coordinates", self.h, ctypes.c_void_p(xyz.ctypes.data))
        return xyz

    def mass(self) -> np.ndarray:
        M = np.empty((self.nelem, self.Np), dtype=np.float64)
        call("cmdg_mesh_mass", self.h, ctypes.c_void_p(M.ctypes.data))
        return M


class CubedShellGrid(BrickGrid):
    """StackedCubedSphereTopology(nhorz, grid1d(r_inner, r_outer, nelem=nvert);
    boundary=(1, 2)) + DiscontinuousSpectralElementGrid(meshwarp =
    equiangular_cubed_sphere_warp) (src/Numerics/Mesh/Topologies.jl:1067-1305,
    1620-1760; src/Numerics/Mesh/Grids.jl:1028-1110), as
    AtmosGCMConfiguration builds it (src/Driver/driver_configs.jl:344-420).

    Columns are contiguous: element e = iz + nvert * h.
    """

    def __init__(self, N, nhorz, nvert, r_inner, r_outer, boundary=(1, 2)):
        _lib.load()
        d = ShellDesc()
        d.N, d.nhorz, d.nvert = int(N), int(nhorz), int(nvert)
        d.r_inner, d.r_outer = float(r_inner), float(r_outer)
        d.bc_inner, d.bc_outer = int(boundary[0]), int(boundary[1])
        h = ctypes.c_void_p()
        call("cmdg_mesh_create_shell", ctypes.byref(d), ctypes.byref(h))
        self.h = h
        self.desc = d
        self.nelem, self.Np = self._sizes()
        self.N, self.Nq = int(N), int(N) + 1
        self.ne = (6 * int(nhorz) * int(nhorz), 1, int(nvert))


class ArraysGrid(BrickGrid):
    """A mesh given by the reference's own DiscontinuousSpectralElementGrid
    arrays (src/Numerics/Mesh/Grids.jl:76-125, 559-638): vgeo (Np, 16,
    nelem), vmap+ (Nfp, 6, nelem, 1-based) and elemtobndy (6, nelem), passed
    here in numpy's C order of the same memory: (nelem, 16, Np),
    (nelem, 6, Nfp), (nelem, 6)."""

    def __init__(self, N, vgeo: np.ndarray, vmap_plus: np.ndarray, elemtobndy: np.ndarray):
        _lib.load()
        vg = np.ascontiguousarray(vgeo, dtype=np.float64)
        vp = np.ascontiguousarray(vmap_plus, dtype=np.int64)
        eb = np.ascontiguousarray(elemtobndy, dtype=np.int64)
        nelem = vg.shape[0]
        Nq = int(N) + 1
        if vg.shape != (nelem, 16, Nq**3) or vp.shape != (nelem, 6, Nq * Nq) or eb.shape != (nelem, 6):
            raise ValueError("grid arrays have inconsistent shapes")
        d = _lib.GridArrays()
        d.N, d.nelem = int(N), int(nelem)
        d.vgeo, d.vmap_plus, d.elemtobndy = vg.ctypes.data, vp.ctypes.data, eb.ctypes.data
        h = ctypes.c_void_p()
        call("cmdg_mesh_create_arrays", ctypes.byref(d), ctypes.byref(h))
        self.h = h
        self.desc = d
        self.nelem, self.Np = self._sizes()
        self.N, self.Nq = int(N), Nq
        self.ne = (int(nelem), 1, 1)


class DGModel:
    """DGModel(balance_law, grid, numerical_flux_first_order, ...) on the GPU.

    precision="fp64": plain Float64 state.
    precision="mixed": FP32 state perturbation about the FP64 hydrostatic
    reference state with an FP64 RK register (see ``to_perturbation``).
    diffusion_direction ("every" or "horizontal", the reference's
    ``diffusion_direction`` keyword): directions of the hyperdiffusion passes.
    """

    def __init__(self, balance_law, grid: BrickGrid, numerical_flux: str = "rusanov", precision: str = "fp64",
                 diffusion_direction: str = "every", direction: str = "every", state_auxiliary: "DGModel" = None):
        from .atmos import AtmosAcousticGravityLinearModel

        if isinstance(balance_law, AtmosAcousticGravityLinearModel):
            # DGModel(linearmodel, grid, ...; direction = VerticalDirection(),
            # state_auxiliary = dg.state_auxiliary): the linear operator on the
            # parent model's tables (no model of its own)
            if direction != "vertical" or not isinstance(state_auxiliary, DGModel):
                raise ValueError("the linear model runs in direction='vertical' with state_auxiliary=<its DGModel>")
            self.balance_law, self.grid, self.numerical_flux = balance_law, grid, numerical_flux
            self.precision, self.mixed, self.direction = "fp64", False, direction
            self.parent = state_auxiliary
            self.h = state_auxiliary.h
            self.device = state_auxiliary.device
            self._borrowed = True
            return
        if direction != "every" or state_auxiliary is not None:
            raise ValueError("the AtmosModel DGModel runs in every direction with its own auxiliary state")
        self.direction = direction
        self.balance_law = balance_law
        self.grid = grid
        self.numerical_flux = numerical_flux
        self.precision = precision
        self.mixed = precision == "mixed"
        p: AtmosParams = balance_law.c_params(numerical_flux)
        p.hyper_direction = {"every": _lib.CMDG_DIR_EVERY, "horizontal": _lib.CMDG_DIR_HORIZONTAL}[diffusion_direction]
        self._params = p
        h = ctypes.c_void_p()
        call("cmdg_model_create", grid.h, ctypes.byref(p), _lib.CMDG_MIXED if self.mixed else _lib.CMDG_FP64,
             ctypes.byref(h))
        self.h = h
        self.device = torch.device("cuda", torch.cuda.current_device())

    def __del__(self):
        if getattr(self, "_borrowed", False):
            return
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.cmdg_model_destroy(self.h)
            self.h = None

    @property
    def is_linear(self) -> bool:
        return getattr(self, "_borrowed", False)

    # ------------------------------------------------------------------ state
    @property
    def state_dtype(self):
        return torch.float32 if self.mixed else torch.float64

    def new_state(self, dtype=None) -> torch.Tensor:
        return torch.zeros((self.grid.nelem, NSTATE, self.grid.Np), dtype=dtype or self.state_dtype,
                           device=self.device)

    def init_ode_state(self, Q_host: np.ndarray) -> torch.Tensor:
        """Copies a host FP64 state (nelem, 5, Np) to the device in the model's
        own representation (FP64, or the FP32 perturbation for "mixed")."""
        Q64 = torch.from_numpy(np.ascontiguousarray(Q_host, dtype=np.float64)).to(self.device)
        if not self.mixed:
            return Q64
        return self.to_perturbation(Q64)

    def set_reference(self, aux7: np.ndarray):
        """Geopotential and reference state of a model on an ArraysGrid:
        (nelem, 7, Np) = Phi, dPhi/dx1..3, rho_ref, rhoe_ref, p_ref."""
        a = np.ascontiguousarray(aux7, dtype=np.float64)
        if a.shape != (self.grid.nelem, 7, self.grid.Np):
            raise ValueError(f"aux7 must be (nelem, 7, Np), got {a.shape}")
        call("cmdg_model_set_reference", self.h, ctypes.c_void_p(a.ctypes.data))

    def set_mms(self, src: torch.Tensor | None, wall: torch.Tensor | None, zero_enthalpy: bool = True):
        """Manufactured-solution terms of an FP64 model on an ArraysGrid
        (cmdg_model_set_mms): a source (nelem, 5, Np) added to the tendency,
        the InitStateBC wall state (nelem, 5, Np), and total_specific_enthalpy
        := 0.  The tensors stay referenced here; refill them in place between
        tendencies."""
        self._mms = (src, wall)
        call("cmdg_model_set_mms", self.h, _dptr(src) if src is not None else None,
             _dptr(wall) if wall is not None else None, int(zero_enthalpy))

    def reference_state(self) -> np.ndarray:
        out = np.empty((self.grid.nelem, 3, self.grid.Np), dtype=np.float64)
        call("cmdg_model_reference_state", self.h, ctypes.c_void_p(out.ctypes.data))
        return out

    def to_perturbation(self, Q64: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        Qp = self.new_state(torch.float32) if out is None else out
        call("cmdg_to_perturbation", self.h, _dptr(Qp), _dptr(Q64), _stream())
        return Qp

    def from_perturbation(self, Qp: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        Q64 = self.new_state(torch.float64) if out is None else out
        call("cmdg_from_perturbation", self.h, _dptr(Q64), _dptr(Qp), _stream())
        return Q64

    def full_state(self, Q: torch.Tensor) -> torch.Tensor:
        """FP64 full state of Q whatever the model's representation."""
        return self.from_perturbation(Q) if self.mixed else Q

    # ------------------------------------------------------------------ tendency
    def __call__(self, tendency, Q, param=None, t=0.0, alpha=None, beta=None, increment=False):
        """tendency = alpha * dQ/dt(Q) + beta * tendency; the 4-argument form
        is alpha = 1, beta = increment (SpaceDiscretization.jl:68-77)."""
        a = 1.0 if alpha is None else float(alpha)
        b = (1.0 if increment else 0.0) if beta is None else float(beta)
        if tendency.dtype != torch.float64:
            raise ValueError("the tendency / RK register is FP64 in every precision")
        if self.is_linear:
            call("cmdg_linear_tendency", self.h, _dptr(tendency), _dptr(Q), float(t), a, b, _stream())
            return tendency
        fn = "cmdg_tendency_mixed" if self.mixed else "cmdg_tendency"
        if Q.dtype != self.state_dtype:
            raise ValueError(f"state dtype {Q.dtype} does not match the model ({self.state_dtype})")
        call(fn, self.h, _dptr(tendency), _dptr(Q), float(t), a, b, _stream())
        return tendency

    def lsrk54_step(self, Q, dQ, t, dt, nsteps=1):
        fn = "cmdg_lsrk54_step_mixed" if self.mixed else "cmdg_lsrk54_step"
        call(fn, self.h, _dptr(Q), _dptr(dQ), float(t), float(dt), int(nsteps), _stream())

    def lsrk54_step_host(self, h_Q: torch.Tensor, Qp: torch.Tensor, dQ: torch.Tensor, t, dt, nsteps=1):
        """Mixed-precision steps of an FP64 state in pinned host memory
        (``h_Q.is_pinned()``): h_Q is copied to the device and converted to
        the FP32 perturbation Qp, stepped with the FP64 register dQ, and the
        FP64 result copied back into h_Q, ordered on the current stream."""
        if not self.mixed:
            raise ValueError("lsrk54_step_host needs a mixed-precision model")
        if h_Q.device.type != "cpu" or not h_Q.is_pinned() or h_Q.dtype != torch.float64 or not h_Q.is_contiguous():
            raise ValueError("h_Q must be a contiguous pinned FP64 host tensor")
        call("cmdg_lsrk54_step_mixed_host", self.h, ctypes.c_void_p(h_Q.data_ptr()), _dptr(Qp), _dptr(dQ), float(t),
             float(dt), int(nsteps), _stream())

    # ------------------------------------------------------------------ launch configuration
    KERNELS = {"node": 0, "column": 1, "lines": 2, "cluster": 3}

    def set_kernel(self, kind: str = "node", grid_ctas: int = -1):
        """Stage-kernel family ("node", "column", "lines" or "cluster") and
        grid: -1 = one CTA per element (the default), 0 = one wave of resident
        CTAs, n > 0 = n CTAs (the "lines" kernel always runs one CTA per
        element); for "cluster", grid_ctas is the cluster size, 2, 4 or 8
        adjacent elements whose shared faces read the neighbour from its
        CTA's shared memory."""
        call("cmdg_model_set_kernel", self.h, self.KERNELS[kind], int(grid_ctas))

    def get_kernel(self):
        k, g = ctypes.c_int(), ctypes.c_int()
        call("cmdg_model_get_kernel", self.h, ctypes.byref(k), ctypes.byref(g))
        return {v: n for n, v in self.KERNELS.items()}[k.value], g.value

    def autotune(self, reps: int = 20):
        """Times every launch candidate and keeps the fastest; returns the
        per-candidate ms/stage and the choice."""
        ms = (ctypes.c_double * 8)()
        n = ctypes.c_int()
        call("cmdg_model_autotune", self.h, int(reps), ms, 8, ctypes.byref(n), _stream())
        return list(ms)[: n.value], self.get_kernel()

    # ------------------------------------------------------------------ reductions
    def weighted_sums(self, Q, fields=(0, 4)):
        fl = (ctypes.c_int * len(fields))(*fields)
        out = (ctypes.c_double * len(fields))()
        fn = "cmdg_weighted_sums_mixed" if self.mixed else "cmdg_weighted_sums"
        call(fn, self.h, _dptr(Q), len(fields), fl, out, _stream())
        return list(out)

    def courant_dt(self, Q, CFL):
        dt = ctypes.c_double()
        call("cmdg_courant_dt", self.h, _dptr(self.full_state(Q)), float(CFL), ctypes.byref(dt), _stream())
        return dt.value

    def gradient_flux(self, Q) -> torch.Tensor:
        """Gradient-flux state (nelem, 10, Np) of Q: grad h_tot, S, N^2."""
        gf = torch.zeros((self.grid.nelem, 10, self.grid.Np), dtype=self.state_dtype, device=self.device)
        call("cmdg_gradient_flux", self.h, _dptr(gf), _dptr(Q), _stream())
        return gf

    def hyperdiffusive_state(self, Q) -> torch.Tensor:
        """Hyperdiffusive state of Q, word 3 c + d = nu_4 d/dx_d lap(c):
        (nelem, 9, Np) on a brick (c = u, v, h_tot; u_h has no vertical
        component), (nelem, 12, Np) on the cubed shell (c = u_h[0..2], h_tot)."""
        nw = 12 if isinstance(self.grid, CubedShellGrid) else 9
        hd = torch.zeros((self.grid.nelem, nw, self.grid.Np), dtype=self.state_dtype, device=self.device)
        call("cmdg_hyperdiffusive_state", self.h, _dptr(hd), _dptr(Q), _stream())
        return hd

    def status_word(self) -> int:
        st = ctypes.c_uint32()
        call("cmdg_status_word", self.h, ctypes.byref(st), _stream())
        return st.value


class RemainderDGModel:
    """remainder_DGModel(dg, (lineardg,)) (src/Numerics/DGMethods/remainder.jl):
    the tendency of the full model minus the linear one, evaluated as the full
    tendency followed by the linear tendency with alpha = -1."""

    def __init__(self, main: DGModel, subs):
        subs = tuple(subs)
        if len(subs) != 1 or not subs[0].is_linear or subs[0].parent is not main:
            raise ValueError("remainder_DGModel(dg, (lineardg,)) with the linear model of dg")
        self.main, self.subs = main, subs
        self.grid = main.grid

    def __call__(self, tendency, Q, param=None, t=0.0, increment=False):
        self.main(tendency, Q, param, t, increment=increment)
        self.subs[0](tendency, Q, param, t, alpha=-1.0, beta=1.0)
        return tendency


def remainder_DGModel(dg: DGModel, subs, **_kw) -> RemainderDGModel:
    return RemainderDGModel(dg, subs)


def _host(Q: torch.Tensor) -> np.ndarray:
    return Q.detach().to("cpu", torch.float64).numpy()


def norm(dg: DGModel, Q) -> float:
    """Weighted L2 norm sqrt(sum M q^2) (src/Arrays/MPIStateArrays.jl:583-606)."""
    q = _host(dg.full_state(Q))
    M = dg.grid.mass()
    return math.sqrt(float(np.sum(q * q * M[:, None, :])))


def euclidean_distance(dg: DGModel, A, B) -> float:
    """sqrt(sum M (A-B)^2) (src/Arrays/MPIStateArrays.jl:628-648)."""
    a = _host(dg.full_state(A))
    b = _host(dg.full_state(B)) if isinstance(B, torch.Tensor) else np.asarray(B)
    M = dg.grid.mass()
    return math.sqrt(float(np.sum((a - b) ** 2 * M[:, None, :])))


def weightedsum(dg: DGModel, Q, field: int) -> float:
    """Compensated sum M q[field] (src/Arrays/MPIStateArrays.jl:655-675)."""
    return dg.weighted_sums(Q, (field,))[0]
