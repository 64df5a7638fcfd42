"""
    CMDG

Julia `ccall` shim over libcmdg.so (include/cmdg.h): a `SpaceDiscretization`
whose functor runs the GPU DG tendency, a `dostep!` method that runs a
whole LSRK54CarpenterKennedy step in one fused GPU call, and the HEVI pair:
the vertical acoustic-gravity linear model and an
ARK2GiraldoKellyConstantinescu solver whose column LU lives on the GPU.
`solve!`, callbacks and `invoke!` of ClimateMachine.jl are used unchanged.

State arrays are the reference's `MPIStateArray.data` (`(Np, nstate,
nelem)` CuArrays), passed by pointer.  Not exercised in this repository's
tests (there is no Julia toolchain here); the same ABI is exercised from
Python.
"""
module CMDG

using CUDA
using ClimateMachine.ODESolvers: LowStorageRungeKutta2N, AbstractODESolver
using ClimateMachine.Mesh.Grids: polynomialorders
import ClimateMachine.ODESolvers: dostep!
import ClimateMachine.DGMethods: SpaceDiscretization

const libcmdg = get(ENV, "CMDG_LIB", joinpath(@__DIR__, "..", "_build", "libcmdg.so"))

const CMDG_FP64 = Cint(0)
const CMDG_MIXED = Cint(1)
# element orders (cmdg_mesh_create_brick_ordered / cmdg_brick_element_order)
const CMDG_TOPOLOGY_LIBRARY = Cint(0)
const CMDG_TOPOLOGY_BRICK = Cint(1)
const CMDG_TOPOLOGY_STACKED_BRICK = Cint(2)

struct Brick
    N::Cint
    ne::NTuple{3, Cint}
    lo::NTuple{3, Cdouble}
    hi::NTuple{3, Cdouble}
    periodic::NTuple{3, Cint}
    bc_lo::NTuple{3, Cint}
    bc_hi::NTuple{3, Cint}
end

struct AtmosParams
    R_d::Cdouble
    cp_d::Cdouble
    cv_d::Cdouble
    T_0::Cdouble
    grav::Cdouble
    MSLP::Cdouble
    inv_Pr_turb::Cdouble
    numflux::Cint
    orientation::Cint
    gravity::Cint
    ref_state::Cint
    subtract_off::Cint
    profile::Cint
    T_surface::Cdouble
    T_min::Cdouble
    turbulence::Cint
    rho_nu::Cdouble
    with_divergence::Cint
    C_smag::Cdouble
    planet_radius::Cdouble   # SphericalOrientation
    hyperdiffusion::Cint     # 0 = NoHyperDiffusion, 1 = DryBiharmonic
    tau_hyper::Cdouble       # DryBiharmonic tau_timescale
    hyper_direction::Cint    # 0 = EveryDirection, 1 = HorizontalDirection (diffusion_direction)
end

check(rc::Cint) =
    rc == 0 || error(unsafe_string(ccall((:cmdg_last_error, libcmdg), Cstring, ())))

stream_handle() = CUDA.stream().handle

"""
    CMDGModel(brick::Brick, params::AtmosParams, grid, balance_law, state_auxiliary;
              precision = CMDG_FP64, topology = CMDG_TOPOLOGY_STACKED_BRICK)

GPU DG model on a brick whose elements are numbered as the reference's
topology numbers them: `CMDG_TOPOLOGY_STACKED_BRICK` (the default) for a
grid built with `StackedBrickTopology` (columns along the 2D Hilbert curve
of the horizontal base, each column contiguous), `CMDG_TOPOLOGY_BRICK` for
`BrickTopology` (every element along the 3D Hilbert curve), so `Q.data` of
that grid over the same ranges is passed unpermuted.  HEVI needs the
stacked order.  `grid`, `balance_law` and `state_auxiliary` are kept for the
reference's callbacks that read them.
"""
mutable struct CMDGModel{G, BL, A} <: SpaceDiscretization
    mesh::Ptr{Cvoid}
    model::Ptr{Cvoid}
    grid::G
    balance_law::BL
    state_auxiliary::A
end

function CMDGModel(brick::Brick, params::AtmosParams, grid, balance_law, state_auxiliary;
                   precision = CMDG_FP64, topology = CMDG_TOPOLOGY_STACKED_BRICK)
    mesh = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:cmdg_mesh_create_brick_ordered, libcmdg), Cint, (Ref{Brick}, Cint, Ref{Ptr{Cvoid}}),
                brick, Cint(topology), mesh))
    model = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:cmdg_model_create, libcmdg), Cint, (Ptr{Cvoid}, Ref{AtmosParams}, Cint, Ref{Ptr{Cvoid}}),
                mesh[], params, precision, model))
    dg = CMDGModel(mesh[], model[], grid, balance_law, state_auxiliary)
    finalizer(dg) do x
        ccall((:cmdg_model_destroy, libcmdg), Cint, (Ptr{Cvoid},), x.model)
        ccall((:cmdg_mesh_destroy, libcmdg), Cint, (Ptr{Cvoid},), x.mesh)
    end
    return dg
end

struct GridArrays
    N::Cint
    nelem::Int64
    vgeo::Ptr{Cdouble}
    vmap_plus::Ptr{Int64}
    elemtobndy::Ptr{Int64}
end

"""
    CMDGModel(dg::DGModel, params; precision = CMDG_FP64)

GPU model on the reference DGModel's own grid arrays and reference state:
`vgeo`, `vmap⁺`, `elemtobndy` of `dg.grid` and `Φ`, `∇Φ`, `ρ_ref`, `ρe_ref`,
`p_ref` of `dg.state_auxiliary` (cmdg_mesh_create_arrays +
cmdg_model_set_reference).  `aux_index` gives the aux columns of
orientation.Φ, the three components of orientation.∇Φ and ref_state.ρ,
ref_state.ρe and ref_state.p (`varsindices` of the model's Auxiliary vars).
"""
function CMDGModel(dg, params::AtmosParams, aux_index::NTuple{7, Int}; precision = CMDG_FP64)
    g = dg.grid
    N = Cint(polynomialorders(g)[1])
    vgeo = Array(g.vgeo)
    vmapP = Array{Int64}(Array(g.vmap⁺))
    e2b = Array{Int64}(Array(g.elemtobndy))
    nelem = Int64(size(vgeo, 3))
    arr = GridArrays(N, nelem, pointer(vgeo), pointer(vmapP), pointer(e2b))
    mesh = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve vgeo vmapP e2b begin
        check(ccall((:cmdg_mesh_create_arrays, libcmdg), Cint, (Ref{GridArrays}, Ref{Ptr{Cvoid}}), arr, mesh))
    end
    model = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:cmdg_model_create, libcmdg), Cint, (Ptr{Cvoid}, Ref{AtmosParams}, Cint, Ref{Ptr{Cvoid}}),
                mesh[], params, precision, model))
    aux7 = Array(Array(dg.state_auxiliary.data)[:, collect(aux_index), 1:nelem])
    check(ccall((:cmdg_model_set_reference, libcmdg), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), model[], aux7))
    cm = CMDGModel(mesh[], model[], g, dg.balance_law, dg.state_auxiliary)
    finalizer(cm) do x
        ccall((:cmdg_model_destroy, libcmdg), Cint, (Ptr{Cvoid},), x.model)
        ccall((:cmdg_mesh_destroy, libcmdg), Cint, (Ptr{Cvoid},), x.mesh)
    end
    return cm
end

# tendency .= α dQ/dt(Q) + β tendency   (DGModel.jl:85)
function (dg::CMDGModel)(tendency, Q, _, t, α, β)
    check(ccall((:cmdg_tendency, libcmdg), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Cdouble, Cdouble, Cdouble, Ptr{Cvoid}),
                dg.model, pointer(tendency.data), pointer(Q.data), t, α, β, stream_handle()))
end
(dg::CMDGModel)(tendency, Q, p, t; increment = false) = dg(tendency, Q, p, t, true, increment)

# one LSRK54 step as one library call (LowStorageRungeKuttaMethod.jl:102)
function dostep!(Q, lsrk::LowStorageRungeKutta2N{T, RT, AT, 5}, p, time) where {T, RT, AT}
    dg = lsrk.rhs!
    if !(dg isa CMDGModel)
        return invoke(dostep!, Tuple{Any, AbstractODESolver, Any, Any}, Q, lsrk, p, time)
    end
    check(ccall((:cmdg_lsrk54_step, libcmdg), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Cdouble, Cdouble, Cint, Ptr{Cvoid}),
                dg.model, pointer(Q.data), pointer(lsrk.dQ.data), time, lsrk.dt, 1, stream_handle()))
end

"""
    CMDGLinearModel(dg::CMDGModel)

`DGModel(AtmosAcousticGravityLinearModel(model), grid, ...; direction =
VerticalDirection(), state_auxiliary = dg.state_auxiliary)` on the GPU
(Atmos/Model/linear.jl): its functor is `cmdg_linear_tendency`.
"""
struct CMDGLinearModel <: SpaceDiscretization
    parent::CMDGModel
end
function (lm::CMDGLinearModel)(tendency, Q, _, t, α, β)
    check(ccall((:cmdg_linear_tendency, libcmdg), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Cdouble, Cdouble, Cdouble, Ptr{Cvoid}),
                lm.parent.model, pointer(tendency.data), pointer(Q.data), t, α, β, stream_handle()))
end
(lm::CMDGLinearModel)(tendency, Q, p, t; increment = false) = lm(tendency, Q, p, t, true, increment)

"""
    CMDGHEVI(dg::CMDGModel, dt; t0 = 0, split_explicit_implicit = false, paperversion = false,
             single_column = false)

Stands in for `ARK2GiraldoKellyConstantinescu(dg_or_rem_dg, lineardg,
LinearBackwardEulerSolver(ManyColumnLU() or SingleColumnLU()), Q; dt, t0,
split_explicit_implicit, paperversion)` (AdditiveRungeKuttaMethod.jl:
839-897): the column LU of the vertical linear model is assembled and
factored on the GPU at construction (`cmdg_hevi_create`) and each
`dostep!` is `cmdg_hevi_step`.  Carries the `dt`, `t`, `steps` fields that
`solve!` reads and updates.
"""
mutable struct CMDGHEVI <: AbstractODESolver
    hevi::Ptr{Cvoid}
    dg::CMDGModel
    dt::Float64
    t::Float64
    steps::Int
end
function CMDGHEVI(dg::CMDGModel, dt; t0 = 0, split_explicit_implicit = false, paperversion = false,
                  single_column = false)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:cmdg_hevi_create, libcmdg), Cint, (Ptr{Cvoid}, Cdouble, Cint, Cint, Cint, Ref{Ptr{Cvoid}}),
                dg.model, dt, split_explicit_implicit, paperversion, single_column, h))
    solver = CMDGHEVI(h[], dg, Float64(dt), Float64(t0), 0)
    finalizer(x -> ccall((:cmdg_hevi_destroy, libcmdg), Cint, (Ptr{Cvoid},), x.hevi), solver)
    return solver
end
function dostep!(Q, ark::CMDGHEVI, p, time)
    check(ccall((:cmdg_hevi_step, libcmdg), Cint, (Ptr{Cvoid}, CuPtr{Float64}, Cdouble, Cint, Ptr{Cvoid}),
                ark.hevi, pointer(Q.data), time, 1, stream_handle()))
end

"""Compensated Σ M q over `fields` (weightedsum, MPIStateArrays.jl:655)."""
function weighted_sums(dg::CMDGModel, Q, fields::Vector{Cint})
    out = zeros(Cdouble, length(fields))
    check(ccall((:cmdg_weighted_sums, libcmdg), Cint,
                (Ptr{Cvoid}, CuPtr{Float64}, Cint, Ptr{Cint}, Ptr{Cdouble}, Ptr{Cvoid}),
                dg.model, pointer(Q.data), length(fields), fields, out, stream_handle()))
    return out
end

end # module
