"""Synthetic workloads: the configurations the benchmark and tests run.

Initial conditions are evaluated in FP64 on the host from the grid's node
coordinates (the reference evaluates its ``init_state_prognostic`` on the
nodes in the same way, src/Numerics/DGMethods/SpaceDiscretization.jl:79-148).

* ``isentropic_vortex``: test/Numerics/DGMethods/Euler/isentropicvortex_setup.jl
  (translation 150 m/s at pi/4, vortex speed 50, radius L/10, Mach-0.5 style
  advection), plus optional seeded uniform noise.
* ``rising_bubble``: dry rising thermal bubble about an isentropic
  (dry-adiabatic) hydrostatic background of potential temperature theta0,
  with a cos^2 bump of amplitude A and radius rc centred at (xc, yc, zc)
  (the structure of experiments/TestCase/risingbubble.jl:23-91).
* ``gcm_initial_state``: isothermal hydrostatic atmosphere on the cubed shell
  with a seeded zonal wind and a Gaussian temperature anomaly.
* ``les_initial_state``: stably stratified box with a seeded divergence-free
  k^-5/3 velocity field (SmagorinskyLilly LES).
"""
from __future__ import annotations

import math

import numpy as np

from .atmos import EARTH, AtmosModel, DryAdiabaticProfile, DryBiharmonic, HydrostaticState, IsothermalProfile
from .dgmodel import ArraysGrid, BrickGrid, CubedShellGrid, DGModel, brick_element_order


def isentropic_vortex(xyz: np.ndarray, t: float = 0.0, *, p_inf=1e5, T_inf=300.0, translation_speed=150.0,
                      translation_angle=math.pi / 4, vortex_speed=50.0, R=1 / 200, L=1 / 20, consts=EARTH,
                      noise=0.0, seed=0) -> np.ndarray:
    R_d, cp, cv, T0 = consts["R_d"], consts["cp_d"], consts["cv_d"], consts["T_0"]
    kappa = R_d / cp
    rho_inf = p_inf / (R_d * T_inf)
    uinf = np.array([translation_speed * math.cos(translation_angle), translation_speed * math.sin(translation_angle), 0.0])
    x = xyz.copy()
    for d in range(3):
        x[:, d, :] -= uinf[d] * t
        x[:, d, :] -= np.floor((x[:, d, :] + L) / (2 * L)) * (2 * L)
    r = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2)
    g = np.exp(-((r / R) ** 2) / 2)
    u = np.stack([uinf[0] - vortex_speed * x[:, 1] / R * g, uinf[1] + vortex_speed * x[:, 0] / R * g,
                  np.zeros_like(r)], axis=1)
    T = T_inf * (1 - kappa * vortex_speed**2 / 2 * rho_inf / p_inf * np.exp(-((r / R) ** 2)))
    p = p_inf * (T / T_inf) ** (1 / kappa)
    rho = p / (R_d * T)
    Q = np.empty((xyz.shape[0], 5, xyz.shape[2]))
    Q[:, 0] = rho
    Q[:, 1:4] = rho[:, None, :] * u
    Q[:, 4] = rho * (0.5 * np.sum(u * u, axis=1) + cv * (T - T0))
    if noise:
        rng = np.random.default_rng(seed)
        Q += rng.uniform(-noise, noise, size=Q.shape)
    return Q


def c1_vortex_state(xyz: np.ndarray, *, seed=2024, strength=5.0, mach=0.5, p_inf=1e5, T_inf=300.0,
                    consts=EARTH) -> np.ndarray:
    """The plain CPU-runnable configuration: on the periodic brick [0, 10]^3
    (4 x 4 x 4 elements, N = 4), an isentropic vortex of strength 5 and
    radius 1 (a tenth of the domain) at the centre, advected diagonally (at
    pi/4 in the x-y plane) at Mach 0.5, plus seeded uniform noise of
    amplitude 1e-6 on all five fields.  The vortex is the Gaussian vortex of
    isentropicvortex_setup.jl (test/Numerics/DGMethods/Euler) with its swirl
    speed set by the strength beta as in Shu's vortex,
    u_theta = beta e^(1/2) / (2 pi) sqrt(R_d T_inf) (r/R) exp(-r^2 / (2 R^2)),
    which makes its temperature drop kappa beta^2 e / (8 pi^2) T_inf at the
    centre."""
    R_d, cp, cv = consts["R_d"], consts["cp_d"], consts["cv_d"]
    c_inf = math.sqrt(cp / cv * R_d * T_inf)
    vortex_speed = strength * math.exp(0.5) / (2 * math.pi) * math.sqrt(R_d * T_inf)
    return isentropic_vortex(xyz - 5.0, 0.0, p_inf=p_inf, T_inf=T_inf, translation_speed=mach * c_inf,
                             translation_angle=math.pi / 4, vortex_speed=vortex_speed, R=1.0, L=5.0, consts=consts,
                             noise=1e-6, seed=seed)


def rising_bubble(xyz: np.ndarray, *, theta0=300.0, amp=2.0, rc=250.0, center=(1250.0, 1250.0, 350.0),
                  consts=EARTH) -> np.ndarray:
    R_d, cp, cv, T0, g, p0 = (consts[k] for k in ("R_d", "cp_d", "cv_d", "T_0", "grav", "MSLP"))
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    xc, yc, zc = center
    r = np.sqrt((x - xc) ** 2 + (y - yc) ** 2 + (z - zc) ** 2)
    dth = np.where(r <= rc, amp * np.cos(np.pi * r / (2 * rc)) ** 2, 0.0)
    th = theta0 + dth
    pi_ex = 1.0 - g / (cp * th) * z
    rho = p0 / (R_d * th) * pi_ex ** (cv / R_d)
    T = th * pi_ex
    Q = np.zeros((xyz.shape[0], 5, xyz.shape[2]))
    Q[:, 0] = rho
    Q[:, 4] = rho * (g * z + cv * (T - T0))
    return Q


def bubble_model(ne=(20, 20, 20), N=4, L=2500.0, precision="fp64", numerical_flux="rusanov"):
    """The dry rising-bubble configuration: [0, L]^3, periodic in x and y,
    FreeSlip/Insulating walls at the bottom and top, FlatOrientation + Gravity,
    HydrostaticState(DryAdiabaticProfile(300 K)), inviscid."""
    grid = BrickGrid(N, ne, (0.0, 0.0, 0.0), (L, L, L), periodicity=(True, True, False),
                     boundary=((0, 0), (0, 0), (1, 2)))
    model = AtmosModel(orientation="flat", gravity=True,
                       ref_state=HydrostaticState(DryAdiabaticProfile(300.0, 0.0), subtract_off=True))
    return DGModel(model, grid, numerical_flux=numerical_flux, precision=precision)


def lgl(N):
    """Legendre-Gauss-Lobatto nodes and weights on [-1, 1] (N + 1 points):
    the interior nodes are the roots of P_N', the weights 2 / (N (N+1) P_N^2)."""
    from numpy.polynomial import legendre as leg

    c = np.zeros(N + 1)
    c[N] = 1.0
    x = np.concatenate(([-1.0], np.sort(np.real(leg.legroots(leg.legder(c)))), [1.0]))
    return x, 2.0 / (N * (N + 1) * leg.legval(x, c) ** 2)


def brick_grid_arrays(N, ne, lo, hi, periodicity=(True, True, True), boundary=((1, 2), (1, 2), (1, 2)),
                      topology="brick"):
    """The reference's DiscontinuousSpectralElementGrid arrays of an affine
    brick, as a Julia caller holds them for cmdg_mesh_create_arrays:
    vgeo (nelem, 16, Np) with the fields of src/Numerics/Mesh/Grids.jl:76-92
    (dxi_d/dx_j, M = J w_i w_j w_k, MI, MH = w_i w_j J |dxi3/dx|, x1..x3,
    JcV = |dx/dxi3|), vmap+ (nelem, 6, Nfp; 1-based, the facing node of
    every face node through the face masks of Grids.jl:559-638, the node
    itself on a wall) and elemtobndy (nelem, 6), with the elements numbered
    as the reference's topology numbers them ("brick": BrickTopology's
    Hilbert order, "stacked_brick", or "library": columns with the vertical
    index fastest, then x, then y).  Host only (no GPU).

    Returns (vgeo, vmap_plus, elemtobndy, perm) with perm[e] the library
    (stacked) index of the reference's element e."""
    N, Nq = int(N), int(N) + 1
    Np, Nfp = Nq**3, Nq * Nq
    nx, ny, nz = (int(x) for x in ne)
    nelem = nx * ny * nz
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    h = (hi - lo) / np.array([nx, ny, nz], dtype=np.float64)
    perm = (np.arange(nelem, dtype=np.int64) if topology == "library"
            else brick_element_order((nx, ny, nz), lo, hi, topology))
    inv = np.empty_like(perm)
    inv[perm] = np.arange(nelem, dtype=np.int64)
    iz, ix, iy = perm % nz, (perm // nz) % nx, perm // (nz * nx)
    cell = (ix, iy, iz)

    xi, w = lgl(N)
    p = np.arange(Np).reshape(Nq, Nq, Nq)  # p[k, j, i] = i + Nq (j + Nq k)
    # face masks: faces 1/2 (j, k), 3/4 (i, k), 5/6 (i, j), first index fastest
    fmask = [p[:, :, 0].ravel(), p[:, :, N].ravel(), p[:, 0, :].ravel(), p[:, N, :].ravel(),
             p[0, :, :].ravel(), p[N, :, :].ravel()]
    ii, jj, kk = (p % Nq), (p // Nq) % Nq, p // Nfp
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()

    vgeo = np.zeros((nelem, 16, Np), dtype=np.float64)
    for d in range(3):
        vgeo[:, 4 * d, :] = 2.0 / h[d]
    J = h[0] * h[1] * h[2] / 8.0
    M = J * w[ii] * w[jj] * w[kk]
    vgeo[:, 9, :] = M
    vgeo[:, 10, :] = 1.0 / M
    vgeo[:, 11, :] = w[ii] * w[jj] * h[0] * h[1] / 4.0
    for d, (a, r) in enumerate(zip(cell, (ii, jj, kk))):
        vgeo[:, 12 + d, :] = lo[d] + h[d] * (a[:, None] + (xi[r][None, :] + 1.0) / 2.0)
    vgeo[:, 15, :] = h[2] / 2.0

    vmap = np.empty((nelem, 6, Nfp), dtype=np.int64)
    bndy = np.zeros((nelem, 6), dtype=np.int64)
    own = np.arange(nelem, dtype=np.int64)
    for f in range(6):
        d, side = f // 2, f % 2
        nb = [c.copy() for c in cell]
        nb[d] = cell[d] + (1 if side else -1)
        n_d = (nx, ny, nz)[d]
        if periodicity[d]:
            nb[d] %= n_d
            wall = np.zeros(nelem, dtype=bool)
        else:
            wall = (nb[d] < 0) | (nb[d] >= n_d)
            nb[d] = np.clip(nb[d], 0, n_d - 1)
        nb_ref = inv[nb[2] + nz * (nb[0] + nx * nb[1])]
        across = Np * nb_ref[:, None] + fmask[f ^ 1][None, :] + 1
        itself = Np * own[:, None] + fmask[f][None, :] + 1
        vmap[:, f, :] = np.where(wall[:, None], itself, across)
        bndy[:, f] = np.where(wall, int(boundary[d][side]), 0)
    return vgeo, vmap, bndy, perm


def bubble_arrays_model(ne=(20, 20, 20), N=4, L=2500.0, precision="fp64", topology="brick"):
    """The rising-bubble configuration of bubble_model run through the grid
    arrays a Julia caller passes (cmdg_mesh_create_arrays +
    cmdg_model_set_reference): the brick's arrays in the reference
    topology's element order, Phi = g z, grad Phi = (0, 0, g), and the
    reference state of the library's own hydrostatic solve on the same
    brick, permuted into that order.  Returns (model, perm, xyz) with xyz
    the node coordinates in the reference's order."""
    per, bnd = (True, True, False), ((0, 0), (0, 0), (1, 2))
    vgeo, vmap, bndy, perm = brick_grid_arrays(N, ne, (0.0, 0.0, 0.0), (L, L, L), per, bnd, topology)
    model = AtmosModel(orientation="flat", gravity=True,
                       ref_state=HydrostaticState(DryAdiabaticProfile(300.0, 0.0), subtract_off=True))
    lib = DGModel(model, BrickGrid(N, ne, (0.0, 0.0, 0.0), (L, L, L), periodicity=per, boundary=bnd))
    ref = lib.reference_state()[perm]
    del lib
    g = model.constants["grav"]
    xyz = np.ascontiguousarray(vgeo[:, 12:15, :])
    aux7 = np.zeros((vgeo.shape[0], 7, vgeo.shape[2]), dtype=np.float64)
    aux7[:, 0] = g * xyz[:, 2]
    aux7[:, 3] = g
    aux7[:, 4:7] = ref
    dg = DGModel(model, ArraysGrid(N, vgeo, vmap, bndy), precision=precision)
    dg.set_reference(aux7)
    return dg, perm, xyz


def hyper_bubble_model(ne=(20, 20, 20), N=4, L=2500.0, precision="fp64", tau=3600.0):
    """The rising-bubble configuration of bubble_model with DryBiharmonic(tau)
    horizontal hyperdiffusion (src/Common/TurbulenceClosures/
    TurbulenceClosures.jl:793-848)."""
    grid = BrickGrid(N, ne, (0.0, 0.0, 0.0), (L, L, L), periodicity=(True, True, False),
                     boundary=((0, 0), (0, 0), (1, 2)))
    model = AtmosModel(orientation="flat", gravity=True,
                       ref_state=HydrostaticState(DryAdiabaticProfile(300.0, 0.0), subtract_off=True),
                       hyperdiffusion=DryBiharmonic(tau))
    return DGModel(model, grid, numerical_flux="rusanov", precision=precision)


def bubble_ensemble_specs(n=64, seed=2024, L=2500.0):
    """Seeded members of the uneven rising-bubble ensemble: element counts per
    direction U{8..16}, N in U{3, 4, 5}, amplitude U[0.5, 3] K, radius
    U[150, 400] m, centred mid-domain 350 m above the bottom."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        ne = tuple(int(x) for x in rng.integers(8, 17, size=3))
        N = int(rng.integers(3, 6))
        amp = float(rng.uniform(0.5, 3.0))
        rc = float(rng.uniform(150.0, 400.0))
        specs.append(dict(ne=ne, N=N, amp=amp, rc=rc, center=(L / 2, L / 2, 350.0)))
    return specs


def bubble_member(spec, L=2500.0, precision="mixed"):
    """Model and FP64 initial state of one ensemble member."""
    dg = bubble_model(ne=spec["ne"], N=spec["N"], L=L, precision=precision)
    Q0 = rising_bubble(dg.grid.coordinates(), amp=spec["amp"], rc=spec["rc"], center=spec["center"])
    return dg, Q0


def gcm_shell_model(nhorz=12, nvert=6, N=4, H=30e3, precision="fp64", numerical_flux="rusanov", T_ref=285.0,
                    subtract_off=True, tau_hyper=None, diffusion_direction="horizontal"):
    """Dry shallow-atmosphere GCM on the stacked equiangular cubed shell:
    6 x nhorz^2 columns of nvert elements between the planet radius and a lid
    H above it, walls at both (AtmosGCMConfiguration's boundary = (1, 2)),
    SphericalOrientation + Gravity, HydrostaticState(IsothermalProfile(T_ref)),
    inviscid, with DryBiharmonic(tau_hyper) hyperdiffusion in the horizontal
    directions when tau_hyper is given (as experiments/AtmosGCM/heldsuarez.jl
    configures it: diffdir = HorizontalDirection())."""
    R = EARTH["planet_radius"]
    grid = CubedShellGrid(N, nhorz, nvert, R, R + H)
    model = AtmosModel(orientation="sphere", gravity=True,
                       ref_state=HydrostaticState(IsothermalProfile(T_ref), subtract_off=subtract_off),
                       hyperdiffusion=None if tau_hyper is None else DryBiharmonic(tau_hyper))
    return DGModel(model, grid, numerical_flux=numerical_flux, precision=precision,
                   diffusion_direction=diffusion_direction)


def gcm_initial_state(xyz: np.ndarray, *, seed=2024, T_ref=285.0, u_max=30.0, dT=1.0, radius=1.0e6, z_c=10e3,
                      z_w=5e3, consts=EARTH) -> np.ndarray:
    """Isothermal (T_ref) hydrostatic atmosphere with a seeded zonal wind and a
    Gaussian temperature anomaly, evaluated at the nodes.

    Wind: u_zonal = u_max cos(lat) (1 + sin(k lon + phase)) / 2 (0 .. u_max),
    k in {1, 2, 3} and phase from the seed, along the local east vector.
    Anomaly: dT exp(-(d / radius)^2 - ((z - z_c) / z_w)^2) with d the
    great-circle distance to a seeded centre.  The pressure keeps the
    hydrostatic profile p = MSLP exp(-g z / (R_d T_ref)) and rho = p / (R_d T)."""
    R_d, cv, T0, g, p0, a = (consts[k] for k in ("R_d", "cv_d", "T_0", "grav", "MSLP", "planet_radius"))
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, 4))
    phase = float(rng.uniform(0, 2 * np.pi))
    lon_c = float(rng.uniform(-np.pi, np.pi))
    lat_c = float(rng.uniform(-np.pi / 3, np.pi / 3))
    x, y, z3 = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    r = np.sqrt(x * x + y * y + z3 * z3)
    z = r - a
    lat = np.arcsin(z3 / r)
    lon = np.arctan2(y, x)
    u = u_max * np.cos(lat) * 0.5 * (1.0 + np.sin(k * lon + phase))
    cosd = np.sin(lat) * np.sin(lat_c) + np.cos(lat) * np.cos(lat_c) * np.cos(lon - lon_c)
    d = a * np.arccos(np.clip(cosd, -1.0, 1.0))
    T = T_ref + dT * np.exp(-((d / radius) ** 2) - ((z - z_c) / z_w) ** 2)
    p = p0 * np.exp(-g * z / (R_d * T_ref))
    rho = p / (R_d * T)
    Q = np.zeros((xyz.shape[0], 5, xyz.shape[2]))
    Q[:, 0] = rho
    Q[:, 1] = rho * (-np.sin(lon) * u)
    Q[:, 2] = rho * (np.cos(lon) * u)
    Q[:, 4] = rho * (cv * (T - T0) + 0.5 * u * u + g * z)
    return Q


def acoustic_wave_model(nhorz=10, nvert=5, N=5, H=10e3, T_ref=300.0, precision="fp64"):
    """The acoustic wave on the sphere of
    test/Numerics/DGMethods/Euler/acousticwave_1d_imex.jl: stacked cubed
    shell (nhorz x nhorz per cube face, nvert levels, lid H),
    SphericalOrientation + Gravity, HydrostaticState(IsothermalProfile(T_ref)),
    inviscid, Rusanov flux, walls at both radii.  precision="mixed" runs the
    explicit tendency of HEVI steps on the FP32 perturbation."""
    R = EARTH["planet_radius"]
    grid = CubedShellGrid(N, nhorz, nvert, R, R + H)
    model = AtmosModel(orientation="sphere", gravity=True, ref_state=HydrostaticState(IsothermalProfile(T_ref)))
    return DGModel(model, grid, numerical_flux="rusanov", precision=precision)


def acoustic_wave_state(xyz: np.ndarray, p_ref: np.ndarray, *, H=10e3, T_ref=300.0, alpha=3.0, gamma=100.0,
                        nv=1, consts=EARTH) -> np.ndarray:
    """AcousticWaveSetup (acousticwave_1d_imex.jl): at rest, T = T_ref and
    p = p_ref + gamma f(beta) sin(nv pi z / H), beta = min(1, alpha
    acos(cos(lat) cos(lon))), f = (1 + cos(pi beta)) / 2; rho = p / (R_d T),
    rhoe = rho (cv_d (T - T_0) + Phi).  xyz (nelem, 3, Np) node coordinates,
    p_ref (nelem, Np) the reference pressure."""
    g, a, R_d, cv, T0 = (consts[k] for k in ("grav", "planet_radius", "R_d", "cv_d", "T_0"))
    x, y, z3 = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    r = np.sqrt(x * x + y * y + z3 * z3)
    Phi = g * (r - a)
    lam = np.arctan2(y, x)
    phi = np.arcsin(z3 / r)
    z = Phi / g
    beta = np.minimum(1.0, alpha * np.arccos(np.cos(phi) * np.cos(lam)))
    f = (1 + np.cos(np.pi * beta)) / 2
    p = p_ref + gamma * f * np.sin(nv * np.pi * z / H)
    Q = np.zeros((xyz.shape[0], 5, xyz.shape[2]))
    rho = p / (R_d * T_ref)
    Q[:, 0] = rho
    Q[:, 4] = rho * (cv * (T_ref - T0) + Phi)
    return Q


def acoustic_wave_dt(H=10e3, nvert=5, N=5, T_ref=300.0, dt_factor=445, consts=EARTH):
    """dt of acousticwave_1d_imex.jl: dt_factor x the vertical acoustic
    element time over N^2, shortened to hit one hour exactly; and the number
    of steps in an hour."""
    cs = math.sqrt(consts["cp_d"] / consts["cv_d"] * consts["R_d"] * T_ref)
    dt = dt_factor * (H / nvert) / cs / N**2
    dt = 3600 / math.ceil(3600 / dt)
    return dt, math.ceil(3600 / dt)


def les_model(ne=(32, 32, 16), N=4, L=(3200.0, 3200.0, 1600.0), precision="fp64", theta0=300.0):
    """Compressible Navier-Stokes LES: SmagorinskyLilly (C_s = 0.21) on a
    brick periodic in x and y with FreeSlip/Insulating walls in z (a stratified
    state needs them), FlatOrientation + Gravity,
    HydrostaticState(DryAdiabaticProfile(theta0)), Rusanov flux."""
    grid = BrickGrid(N, ne, (0.0, 0.0, 0.0), L, periodicity=(True, True, False), boundary=((0, 0), (0, 0), (1, 2)))
    model = AtmosModel(orientation="flat", gravity=True,
                       ref_state=HydrostaticState(DryAdiabaticProfile(theta0, 0.0), subtract_off=True),
                       turbulence="smagorinsky", C_smag=EARTH["C_smag"])
    return DGModel(model, grid, numerical_flux="rusanov", precision=precision)


def les_initial_state(xyz: np.ndarray, L=(3200.0, 3200.0, 1600.0), *, seed=2024, theta0=300.0, N_bv=0.01,
                      u_rms=1.0, nmodes=48, consts=EARTH) -> np.ndarray:
    """Stably stratified (Brunt-Vaisala frequency N_bv) hydrostatic state,
    theta = theta0 exp(N_bv^2 z / g) with the matching Exner pressure, plus a
    seeded divergence-free velocity: the curl of a vector potential summed
    over nmodes Fourier modes periodic in x and y, amplitudes following a
    k^-5/3 energy spectrum, scaled to an rms speed u_rms."""
    R_d, cp, cv, T0, g, p0 = (consts[k] for k in ("R_d", "cp_d", "cv_d", "T_0", "grav", "MSLP"))
    rng = np.random.default_rng(seed)
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    u = np.zeros_like(x)
    v = np.zeros_like(x)
    w = np.zeros_like(x)
    for _ in range(nmodes):
        n = rng.integers(1, 9, size=2) * rng.choice([-1, 1], size=2)
        kz = float(rng.uniform(0.5, 8.0)) * np.pi / L[2]
        kv = np.array([2 * np.pi * n[0] / L[0], 2 * np.pi * n[1] / L[1], kz])
        kmag = float(np.linalg.norm(kv))
        a = rng.normal(size=3)
        a -= kv * (a @ kv) / kmag**2  # potential amplitude normal to k
        a *= kmag ** (-5.0 / 6.0 - 1.0) / np.linalg.norm(a)  # |u_k| ~ k^(-5/6): E(k) ~ k^-5/3
        ph = float(rng.uniform(0, 2 * np.pi))
        arg = kv[0] * x + kv[1] * y + kv[2] * z + ph
        c = np.cos(arg)
        # u = curl(a sin(k.x + phase)) = (k x a) cos(k.x + phase)
        cr = np.cross(kv, a)
        u += cr[0] * c
        v += cr[1] * c
        w += cr[2] * c
    scale = u_rms / np.sqrt(np.mean(u * u + v * v + w * w))
    u, v, w = u * scale, v * scale, w * scale
    S = N_bv**2 / g
    th = theta0 * np.exp(S * z)
    # hydrostatic Exner function for theta(z): dpi/dz = -g / (cp theta)
    pi_ex = 1.0 + g / (cp * theta0 * S) * (np.exp(-S * z) - 1.0)
    rho = p0 / (R_d * th) * pi_ex ** (cv / R_d)
    T = th * pi_ex
    Q = np.zeros((xyz.shape[0], 5, xyz.shape[2]))
    Q[:, 0] = rho
    Q[:, 1] = rho * u
    Q[:, 2] = rho * v
    Q[:, 3] = rho * w
    Q[:, 4] = rho * (cv * (T - T0) + 0.5 * (u * u + v * v + w * w) + g * z)
    return Q
