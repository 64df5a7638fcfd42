/*
 * cmdg.h — C ABI of libcmdg.so, a GB300 (sm_103a) implementation of
 * ClimateMachine.jl's DG spectral-element tendency and LSRK54 stage update
 * for the dry compressible AtmosModel.
 *
 * Conventions
 *   - Every entry point returns CMDG_OK (0) or a CMDG_ERR_* code and never
 *     throws; cmdg_last_error() gives a thread-local message for the last
 *     failure on the calling thread.
 *   - State arrays use the reference's MPIStateArray layout: column-major
 *     (Np, nstate, nelem) with nstate = 5 (rho, rhou, rhov, rhow, rhoe),
 *     Np = (N+1)^3, node index ijk = i + Nq*(j + Nq*k).
 *   - Pointers named d_* are device pointers (cudaMalloc'd or torch
 *     tensors); pointers named h_* are host pointers.  `stream` is a
 *     cudaStream_t passed as void* (NULL = legacy default stream).
 *   - The caller owns Q, dQ and every buffer it passes.  The library owns
 *     geometry, reference-state tables, scratch buffers and CUDA graphs.
 *   - One model is used by one stream at a time; calls on one model are not
 *     re-entrant.
 *   - Element ordering of generated brick meshes is "stacked": the vertical
 *     element index is fastest, then x, then y (columns contiguous, as in
 *     StackedBrickTopology, src/Numerics/Mesh/Topologies.jl:632, whose
 *     columns follow the Hilbert curve instead); cmdg_mesh_create_brick_ordered
 *     builds StackedBrickTopology's or BrickTopology's order instead.
 */
#ifndef CMDG_H
#define CMDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    CMDG_OK = 0,
    CMDG_ERR_ARG = 1,          /* invalid argument or size */
    CMDG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    CMDG_ERR_UNSUPPORTED = 3,  /* configuration not implemented */
    CMDG_ERR_NONFINITE = 4,    /* a kernel saw a non-finite value */
    CMDG_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    CMDG_ERR_ALLOC = 6,        /* device allocation failed */
    CMDG_ERR_STATE = 7         /* object used in the wrong state */
};

/* Arithmetic of a model.
 *   CMDG_FP64  : plain Float64, the reference's arithmetic.
 *   CMDG_MIXED : FP32 state perturbation q' = q - q_ref about an FP64
 *                hydrostatic reference state; FP64 RK register dQ; FP64
 *                reference subtraction; compensated FP64 sums. */
enum { CMDG_FP64 = 0, CMDG_MIXED = 1 };

/* Numerical flux for first-order terms */
enum { CMDG_FLUX_RUSANOV = 0, CMDG_FLUX_CENTRAL = 1 };
/* Orientation */
enum { CMDG_ORIENT_NONE = 0, CMDG_ORIENT_FLAT = 1, CMDG_ORIENT_SPHERE = 2 };
/* Reference-state temperature profile */
enum { CMDG_PROFILE_ISOTHERMAL = 0, CMDG_PROFILE_DRY_ADIABATIC = 1 };
/* Turbulence closure */
enum { CMDG_TURB_NONE = 0, CMDG_TURB_CONSTANT = 1, CMDG_TURB_SMAGORINSKY = 2 };
/* Hyperdiffusion (NoHyperDiffusion / DryBiharmonic,
 * src/Common/TurbulenceClosures/TurbulenceClosures.jl:793-848) */
enum { CMDG_HYPER_NONE = 0, CMDG_HYPER_DRY_BIHARMONIC = 1 };

/* Brick mesh (BrickTopology / StackedBrickTopology + DiscontinuousSpectralElementGrid,
 * src/Numerics/Mesh/Topologies.jl:470-545,632; src/Numerics/Mesh/Grids.jl:267-414). */
typedef struct {
    int N;              /* polynomial order, 1..7 (kernels instantiated for 2..5) */
    int ne[3];          /* elements in x, y, z */
    double lo[3];       /* domain lower corner */
    double hi[3];       /* domain upper corner */
    int periodic[3];    /* 1 = periodic */
    int bc_lo[3];       /* boundary tag of the lower face when not periodic (>0) */
    int bc_hi[3];       /* boundary tag of the upper face when not periodic (>0) */
} cmdg_brick_desc;

/* Dry AtmosModel parameters (src/Atmos/Model/AtmosModel.jl:242-375;
 * planet constants as CLIMAParameters.Planet supplies them). */
typedef struct {
    double R_d, cp_d, cv_d, T_0, grav, MSLP, inv_Pr_turb;
    int numflux;        /* CMDG_FLUX_* */
    int orientation;    /* CMDG_ORIENT_* */
    int gravity;        /* 1 = Gravity() source */
    int ref_state;      /* 1 = HydrostaticState */
    int subtract_off;   /* HydrostaticState.subtract_off */
    int profile;        /* CMDG_PROFILE_* */
    double T_surface;   /* isothermal T_virt, or dry-adiabatic surface temperature */
    double T_min;       /* dry-adiabatic minimum temperature */
    int turbulence;     /* CMDG_TURB_* (both closures on every mesh, FP64 and mixed) */
    double rho_nu;      /* ConstantDynamicViscosity rho*nu */
    int with_divergence;/* ConstantDynamicViscosity WithDivergence */
    double C_smag;      /* SmagorinskyLilly coefficient */
    double planet_radius; /* SphericalOrientation: Phi = grav (|x| - planet_radius) */
    int hyperdiffusion; /* CMDG_HYPER_* (brick meshes with FlatOrientation) */
    double tau_hyper;   /* DryBiharmonic tau_timescale (s) */
    int hyper_direction;/* diffusion_direction of the hyperdiffusion passes: CMDG_DIR_EVERY or
                           CMDG_DIR_HORIZONTAL (DGModel.jl:22-65, SpaceDiscretization.jl:731-1083) */
} cmdg_atmos_params;

/* Stacked equiangular cubed shell: 6 nhorz^2 columns of nvert elements
 * between radii r_inner and r_outer, walls (FreeSlip + Insulating) at both. */
typedef struct {
    int N;              /* polynomial order, 2..5 */
    int nhorz;          /* elements along each cube-face edge */
    int nvert;          /* elements per column */
    double r_inner, r_outer;
    int bc_inner, bc_outer; /* boundary tags (> 0) */
} cmdg_shell_desc;

typedef struct cmdg_mesh cmdg_mesh;
typedef struct cmdg_model cmdg_model;

/* Last error message of the calling thread (never NULL). */
const char* cmdg_last_error(void);

/* Library version string. */
const char* cmdg_version(void);

/* Builds a brick mesh and its geometry on the current device.
 * Replaces BrickTopology/StackedBrickTopology + DiscontinuousSpectralElementGrid
 * (src/Numerics/Mesh/Topologies.jl:470-545,632; src/Numerics/Mesh/Grids.jl:267-414). */
int cmdg_mesh_create_brick(const cmdg_brick_desc* desc, cmdg_mesh** out);

/* Element orders of the reference's brick topologies.
 *   CMDG_TOPOLOGY_LIBRARY        the library's stacked order: vertical index
 *                                fastest, then x, then y;
 *   CMDG_TOPOLOGY_BRICK          BrickTopology: all elements along the 3D
 *                                Hilbert curve through their centroids
 *                                (BrickMesh.partition, src/Numerics/Mesh/BrickMesh.jl:531-627,
 *                                codes from centroidtocode / hilbertcode, :40-150);
 *   CMDG_TOPOLOGY_STACKED_BRICK  StackedBrickTopology: the horizontal base
 *                                elements along the 2D Hilbert curve, each
 *                                column contiguous, vertical index fastest
 *                                (src/Numerics/Mesh/Topologies.jl:632-715). */
enum { CMDG_TOPOLOGY_LIBRARY = 0, CMDG_TOPOLOGY_BRICK = 1, CMDG_TOPOLOGY_STACKED_BRICK = 2 };

/* Host-only (needs no GPU): h_perm[e_ref] = the index, in the library's
 * stacked order, of the element that the given topology numbers e_ref
 * (0-based), for ne[0] ne[1] ne[2] entries.  A state in the reference's
 * order maps to the library's by moving element e_ref to h_perm[e_ref]. */
int cmdg_brick_element_order(const cmdg_brick_desc* desc, int topology, int64_t* h_perm);

/* A brick mesh whose elements are numbered in the reference's order, so
 * states in that order need no permutation: topology CMDG_TOPOLOGY_LIBRARY
 * (the same mesh as cmdg_mesh_create_brick), CMDG_TOPOLOGY_STACKED_BRICK
 * (columns along the 2D Hilbert curve; the bricks of AtmosLESConfiguration,
 * src/Driver/driver_configs.jl:213) or CMDG_TOPOLOGY_BRICK (every element
 * along the 3D Hilbert curve).  Every kernel reads an element's vertical
 * index from its neighbour row, so all three orders run the same kernels
 * with the same per-level tables; only HEVI, whose column solves need
 * contiguous columns, refuses a CMDG_TOPOLOGY_BRICK mesh (CMDG_ERR_UNSUPPORTED). */
int cmdg_mesh_create_brick_ordered(const cmdg_brick_desc* desc, int topology, cmdg_mesh** out);
/* Builds a stacked cubed-shell mesh: curvilinear geometry with the
 * curl-invariant metric terms.  Replaces StackedCubedSphereTopology +
 * DiscontinuousSpectralElementGrid(meshwarp = equiangular_cubed_sphere_warp)
 * (src/Numerics/Mesh/Topologies.jl:1067-1305,1620-1760;
 * src/Numerics/Mesh/Grids.jl:1028-1110; src/Numerics/Mesh/Metrics.jl:431-724). */
int cmdg_mesh_create_shell(const cmdg_shell_desc* desc, cmdg_mesh** out);

/* A mesh from the reference's own grid arrays (a DiscontinuousSpectralElementGrid
 * of any topology: warped bricks, cubed shells, ...), host arrays in Julia's
 * column-major layout:
 *   vgeo       (Np, 16, nelem) FP64: xi1x1, xi2x1, xi3x1, xi1x2, ..., xi3x3,
 *              M, MI, MH, x1, x2, x3, JcV (src/Numerics/Mesh/Grids.jl:76-125);
 *   vmap_plus  (Nfp, 6, nelem) 1-based global node index of the node facing
 *              each face node (Grids.jl:559-638; the face nodes are numbered
 *              by the reference's face masks, Grids.jl:580-597);
 *   elemtobndy (6, nelem) 0 on interior faces, the boundary tag (> 0) on
 *              walls (FreeSlip + Insulating).
 * Faces must be conforming (every node of a face faces one element). */
typedef struct {
    int N;                      /* polynomial order, 2..5 */
    int64_t nelem;
    const double* vgeo;
    const int64_t* vmap_plus;
    const int64_t* elemtobndy;
} cmdg_grid_arrays;
int cmdg_mesh_create_arrays(const cmdg_grid_arrays* desc, cmdg_mesh** out);
int cmdg_mesh_destroy(cmdg_mesh* mesh);
/* Sizes of a mesh. */
int cmdg_mesh_info(const cmdg_mesh* mesh, int64_t* nelem, int* Np);
/* Node coordinates into host memory, (Np, 3, nelem) column-major
 * (vgeo x1,x2,x3, src/Numerics/Mesh/Grids.jl:76-125). */
int cmdg_mesh_coordinates(const cmdg_mesh* mesh, double* h_xyz);
/* Nodal quadrature weights M = J w_i w_j w_k into host memory, (Np, nelem)
 * (vgeo M, src/Numerics/Mesh/Grids.jl:96-100). */
int cmdg_mesh_mass(const cmdg_mesh* mesh, double* h_M);

/* Builds a model (DGModel + AtmosModel) on a mesh; computes the orientation,
 * reference-state and closure auxiliary data.
 * Replaces DGModel(bl, grid, nf1, nf2, nfgrad) (src/Numerics/DGMethods/DGModel.jl:22-65)
 * with the dry AtmosModel auxiliary initialisation (src/Atmos/Model/AtmosModel.jl:908-925,
 * src/Atmos/Model/ref_state.jl:143-263). */
int cmdg_model_create(cmdg_mesh* mesh, const cmdg_atmos_params* params, int precision, cmdg_model** out);
int cmdg_model_destroy(cmdg_model* model);
/* Geopotential and reference state of a model on a mesh from grid arrays,
 * host (Np, 7, nelem) FP64: Phi, dPhi/dx1, dPhi/dx2, dPhi/dx3, rho_ref,
 * rhoe_ref, p_ref -- the reference's aux.orientation.Phi, aux.orientation.gradPhi
 * and aux.ref_state.(rho, rhoe, p) (src/Common/Orientations/Orientations.jl:57-136,
 * src/Atmos/Model/ref_state.jl:66-67).  Required before the first tendency
 * of such a model whose orientation, gravity or reference state uses them;
 * may be called again to replace them. */
int cmdg_model_set_reference(cmdg_model* model, const double* h_aux7);
/* Manufactured-solution runs on grid-arrays meshes (FP64 models): d_src, a
 * source (Np, 5, nelem) added to the tendency (the MMSSource of
 * test/Numerics/DGMethods/compressible_Navier_Stokes/mms_bc_atmos.jl:60-80);
 * d_wall, the wall state (Np, 5, nelem) used on every wall face node for the
 * first-order, gradient and one-sided second-order fluxes (InitStateBC,
 * src/Atmos/Model/bc_initstate.jl:12-26, NumericalFluxes.jl:872-966) in place
 * of FreeSlip + Insulating; zero_enthalpy = 1 sets total_specific_enthalpy to
 * zero in the gradient arguments (mms_bc_atmos.jl:45-48).  Device arrays owned
 * by the caller, read by every following tendency; NULL switches each off. */
int cmdg_model_set_mms(cmdg_model* model, const double* d_src, const double* d_wall, int zero_enthalpy);

/* Reference state at the nodes into host memory, (Np, 3, nelem):
 * rho_ref, rhoe_ref, p_ref (aux.ref_state, src/Atmos/Model/ref_state.jl:66-67). */
int cmdg_model_reference_state(const cmdg_model* model, double* h_ref);

/* Stage-kernel family of a model: CMDG_KERNEL_NODE (one thread per node,
 * all precisions), CMDG_KERNEL_COLUMN (one thread per vertical line of
 * nodes; mixed precision, N = 3..5; other models fall back to the node
 * kernel), CMDG_KERNEL_LINES (one thread per element line in the face and
 * contraction phase) or CMDG_KERNEL_CLUSTER (the node kernel in thread-block
 * clusters of grid_ctas = 2, 4 or 8 adjacent elements of an inviscid brick,
 * 1 x 1 x 2, 2 x 1 x 2 or 2 x 2 x 2 in x, y, z, whose shared faces read the
 * neighbour's staged state and flux from its CTA's shared memory; the
 * element counts must be even in the directions a cluster spans, else
 * CMDG_ERR_UNSUPPORTED).  For the node kernel, grid_ctas > 0 fixes the size
 * of its persistent grid, 0 = one wave of resident CTAs, -1 = no
 * persistence (one CTA per element, the default).  No counterpart in the
 * reference (the launch configuration of a KernelAbstractions kernel is
 * fixed, src/Numerics/DGMethods/SpaceDiscretization.jl:1120-1133). */
enum { CMDG_KERNEL_NODE = 0, CMDG_KERNEL_COLUMN = 1, CMDG_KERNEL_LINES = 2, CMDG_KERNEL_CLUSTER = 3 };
int cmdg_model_set_kernel(cmdg_model* model, int kernel_kind, int grid_ctas);
int cmdg_model_get_kernel(const cmdg_model* model, int* kernel_kind, int* grid_ctas);

/* Autotuner: times every (kernel family, grid) candidate of this model on a
 * scratch copy of the reference state for `reps` stage launches each, keeps
 * the fastest, and writes the number of candidates and their times (ms per
 * stage, candidate order: node kernel with a persistent grid of one wave of
 * resident CTAs, node kernel with one CTA per element, column kernel when the
 * model has one) to h_ms (capacity h_ms_len).
 * Allocates and frees two state-sized temporaries.  No counterpart in the
 * reference. */
int cmdg_model_autotune(cmdg_model* model, int reps, double* h_ms, int h_ms_len, int* n_candidates, void* stream);

/* One tendency evaluation in FP64:
 *   d_dQ = alpha * dQ/dt(d_Q) + beta * d_dQ
 * Replaces (dg::DGModel)(tendency, Q, _, t, alpha, beta)
 * (src/Numerics/DGMethods/DGModel.jl:85-427). */
int cmdg_tendency(cmdg_model* model, double* d_dQ, const double* d_Q, double t, double alpha, double beta,
                  void* stream);

/* nsteps LSRK54CarpenterKennedy steps of size dt in FP64, in place on d_Q;
 * d_dQ is the solver's RK register (zero before the first step, as the
 * reference's `fill!(dQ, 0)`).  The dry AtmosModel terms of the library do
 * not depend on time, so the stage times t + C_s dt of the reference
 * (LowStorageRungeKuttaMethod.jl:319-324) do not enter the kernels; a model
 * whose tendency takes terms that the caller refreshes at each stage time
 * (cmdg_model_set_mms) is refused with CMDG_ERR_STATE and is stepped stage by
 * stage with cmdg_tendency instead.
 * Replaces dostep!(Q, lsrk::LowStorageRungeKutta2N, p, time)
 * (src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:102-158, 293-327). */
int cmdg_lsrk54_step(cmdg_model* model, double* d_Q, double* d_dQ, double t, double dt, int nsteps, void* stream);

/* Allocation-free form of cmdg_lsrk54_step / cmdg_lsrk54_step_mixed, for
 * callers that cannot let the library allocate device memory: hosts whose
 * arena or pool allocator owns all of the device's memory, and hosts that
 * forbid allocation after start-up.  No counterpart in the reference.
 *   d_Q: double* for a CMDG_FP64 model, float* (the perturbation) for a
 *   CMDG_MIXED model; d_dQ: the FP64 RK register.
 *   The two stage buffers live in a fixed 48 MiB __device__ array.  It is
 *   reserved on a device when the first model is created there
 *   (cmdg_model_create looks its address up, which loads the module that
 *   holds it) and is held until the process exits; create the model before
 *   the host's arena takes the device's memory.  The call itself makes no
 *   cudaMalloc / cudaFree and reserves nothing.  States larger than 24 MiB are
 *   rejected with CMDG_ERR_ARG; the model's device must be current
 *   (CMDG_ERR_STATE otherwise).  Calls share the array: calls whose kernels
 *   overlap on the GPU race. */
int cmdg_lsrk54_step_noalloc(cmdg_model* model, void* d_Q, double* d_dQ, double t, double dt, int nsteps,
                             void* stream);

/* Ensembles.  A batch advances n mixed-precision brick models of any sizes
 * and polynomial orders N = 3..5 together.  Inviscid members are grouped by
 * order; each LSRK54 stage of a group is one launch of a tile-walking kernel
 * (a tile is a run of consecutive elements of one member), the groups' stage
 * chains run on their own streams, and the steps of a call are captured in one
 * CUDA graph (stream != NULL).  Members with a turbulence closure (LES
 * members: ConstantDynamicViscosity or SmagorinskyLilly) take the gradient
 * pass and the viscous stage kernel at every stage, member by member, on a
 * further branch of the same graph.  The batch owns two stage buffers per
 * member; a viscous member's gradient-flux buffer is its model's.
 * No counterpart in the reference (there, ensemble members are separate
 * solver runs). */
typedef struct cmdg_batch cmdg_batch;
int cmdg_batch_create(cmdg_model* const* models, int n, cmdg_batch** out);
int cmdg_batch_destroy(cmdg_batch* batch);
/* Tiling of the members of order N (0 = every order): tile_elems elements per
 * tile; grid_ctas -1 = one CTA per tile, 0 = one wave of resident CTAs,
 * n > 0 = n CTAs. */
int cmdg_batch_set_tiling(cmdg_batch* batch, int N, int tile_elems, int grid_ctas);
int cmdg_batch_get_tiling(const cmdg_batch* batch, int N, int* tile_elems, int* grid_ctas);
/* nsteps LSRK54 steps of every member; h_Q, h_dQ, h_dt: host arrays of n
 * device state pointers (FP32 perturbations), n device RK registers and n
 * time steps.  Same per-member semantics as cmdg_lsrk54_step_mixed. */
int cmdg_batch_lsrk54_step(cmdg_batch* batch, void* const* h_Q, double* const* h_dQ, const double* h_dt, int nsteps,
                           void* stream);
/* Kernel family of the inviscid members:
 *   CMDG_BATCH_PER_ORDER  one tile-walking launch per order and stage, the
 *                         orders on independent branches (tiling per order:
 *                         cmdg_batch_set_tiling);
 *   CMDG_BATCH_PERSISTENT one launch per stage of one persistent kernel over
 *                         tiles of every order with one CTA shape:
 *                         cta_threads 128 (two N = 3 elements, one N = 4
 *                         element, one N = 5 element at two nodes per thread
 *                         per CTA pass) or 256 (four, two and one, a thread
 *                         per node); tile_elems elements per tile; grid_ctas
 *                         -1 = one CTA per tile, 0 = one wave of resident
 *                         CTAs, n > 0 = n CTAs.
 * cmdg_batch_get_kernel returns the family and the persistent tiling. */
enum { CMDG_BATCH_PER_ORDER = 0, CMDG_BATCH_PERSISTENT = 1 };
int cmdg_batch_set_kernel(cmdg_batch* batch, int family, int cta_threads, int tile_elems, int grid_ctas);
int cmdg_batch_get_kernel(const cmdg_batch* batch, int* family, int* cta_threads, int* tile_elems, int* grid_ctas);
/* Autotuner: times `reps` stage launches of every candidate on copies of the
 * members' states (the states are not changed; the RK registers are
 * overwritten, which the next step ignores): per order tile_elems {1, 2, 4,
 * 8, 16} x grid {one CTA per tile, one wave of resident CTAs}, keeping each
 * order's fastest, then the whole per-order family; and the persistent kernel
 * over cta_threads {128, 256} x tile_elems {1, 2, 4, 8} x grid {one CTA per
 * tile, one wave}.  Keeps the faster family with its fastest tiling.  h_ms
 * receives ms per stage launch: [order 3, 4, 5][10 per-order candidates] (0
 * for an order without members), the 16 persistent candidates, the whole
 * per-order family (n_candidates = 47). */
int cmdg_batch_autotune(cmdg_batch* batch, void* const* h_Q, double* const* h_dQ, int reps, double* h_ms,
                        int h_ms_len, int* n_candidates, void* stream);

/* Filters applied to a state between steps (src/Numerics/Mesh/Filters.jl).
 * cmdg_filter_matrix: spectral_filter_matrix of an ExponentialFilter
 * (sigma = exp(-alpha eta^s)), CutoffFilter (sigma = 0) or
 * BoydVandevenFilter, (N+1)^2 doubles, row i = output node i
 * (Filters.jl:114-128, 172-306); host only.
 * cmdg_apply_filter: applies the horizontal matrix along xi1 and xi2 and the
 * vertical one along xi3 (direction CMDG_DIR_*) to the listed fields of a
 * model's state in place (FP64 state, or the FP32 perturbation of a mixed
 * model, to which the FP64 change of the reference state under the filter
 * is added) — Filters.apply!(Q, fields, grid, filter; direction)
 * (:408-505).  Any mesh, FP64 and mixed (the filters act along the element
 * lines).
 * cmdg_apply_tmar: TMARFilter on the listed fields (:369-407, 794-892).
 * cmdg_apply_mp_filter: MassPreservingCutoffFilter (:309-345, 542-606,
 * 895-1065) with the cutoff matrices of cmdg_filter_matrix (the identity for
 * Nc > N): a horizontal pass (xi1, xi2) and/or a vertical pass (xi3), each
 * followed by the per-element shift that restores sum M q of every listed
 * field; any mesh; a mixed model's FP32 perturbation is filtered through an
 * FP64 copy of its full state (the masses are those of the full state). */
enum { CMDG_FILTER_EXPONENTIAL = 0, CMDG_FILTER_CUTOFF = 1, CMDG_FILTER_BOYD_VANDEVEN = 2 };
enum { CMDG_DIR_EVERY = 0, CMDG_DIR_HORIZONTAL = 1, CMDG_DIR_VERTICAL = 2 };
int cmdg_filter_matrix(int N, int kind, int Nc, int s, double alpha, double* h_W);
int cmdg_apply_filter(cmdg_model* model, void* d_Q, const double* h_Wh, const double* h_Wv, int direction,
                      const int* h_fields, int nfields, void* stream);
int cmdg_apply_tmar(cmdg_model* model, void* d_Q, const int* h_fields, int nfields, void* stream);
int cmdg_apply_mp_filter(cmdg_model* model, void* d_Q, const double* h_Wh, const double* h_Wv, int direction,
                         const int* h_fields, int nfields, void* stream);

/* HEVI (horizontally explicit, vertically implicit) stepping of FP64 states,
 * for models with a hydrostatic reference state on wall-bounded element
 * stacks: a cubed shell, a brick non-periodic in z, or a mesh from grid
 * arrays whose elements are in stacked order (element e = v + nz h, walls at
 * both ends of every stack, found from vmap_plus / elemtobndy; the
 * reference state must be set first).  The linear operator,
 * the column LU and the ARK stage algebra are FP64; a mixed-precision model
 * evaluates the explicit tendency on the FP32 perturbation of each stage
 * state (cmdg_tendency_mixed semantics), an FP64 model in FP64.
 *
 * cmdg_linear_tendency: d_dQ = alpha * L(d_Q) + beta * d_dQ, the tendency of
 * AtmosAcousticGravityLinearModel(model) as a DGModel in VerticalDirection
 * sharing the model's auxiliary state (src/Atmos/Model/linear.jl:1-57,
 * 150-262; src/Atmos/Model/linear_tendencies.jl; DGModel.jl:85-427 with
 * direction = VerticalDirection()): fluxes rho u, p_L I,
 * (rhoe_ref + p_ref) / rho_ref rho u with p_L = rho R_d T_0 + R_d / cv_d
 * (rhoe - rho Phi), source -rho grad Phi, Rusanov flux at the reference
 * sound speed on faces 5 and 6.  d_dQ must not alias d_Q.
 *
 * cmdg_hevi_create: ARK2GiraldoKellyConstantinescu(dg, lineardg,
 * LinearBackwardEulerSolver(ManyColumnLU()), Q; dt, split_explicit_implicit,
 * paperversion, variant = LowStorageVariant())
 * (src/Numerics/ODESolvers/AdditiveRungeKuttaMethod.jl:839-897, 413-538):
 * builds and LU-factors, without pivoting, the banded matrix of
 * Q - alpha L(Q), alpha = dt (1 - 1/sqrt(2)), for every vertical node line
 * (src/Numerics/SystemSolvers/columnwise_lu_solver.jl:92-158, 228-488).
 * single_column = 1 is SingleColumnLU(): one factorization (the first
 * line's) serves every line; refused with CMDG_ERR_ARG unless all column
 * matrices agree to 1e-10 (e.g. an affine brick with level-dependent
 * coefficients).  Owns the factors and seven state-sized FP64 buffers.
 * cmdg_hevi_solve: besolver!(Q, Qhat, alpha): d_Q = d_Qhat + alpha L(d_Q)
 * (BackwardEulerSolvers.jl; linearsolve! columnwise_lu_solver.jl:110-127,
 * 615-780); d_Q may alias d_Qhat.
 * cmdg_hevi_step: nsteps ARK2 steps of d_Q (dostep!, :413-538); the explicit
 * part is the model's full tendency (split_explicit_implicit = 0) or the
 * remainder full - linear (1, remainder_DGModel).
 * cmdg_hevi_info: the implicit coefficient alpha, the band half-width
 * 5 (N+1) - 1 and the number of vertical lines.
 * A solver refers to its model: destroy the solver before the model. */
typedef struct cmdg_hevi cmdg_hevi;
int cmdg_linear_tendency(cmdg_model* model, double* d_dQ, const double* d_Q, double t, double alpha, double beta,
                         void* stream);
int cmdg_hevi_create(cmdg_model* model, double dt, int split_explicit_implicit, int paperversion, int single_column,
                     cmdg_hevi** out);
int cmdg_hevi_destroy(cmdg_hevi* hevi);
int cmdg_hevi_info(const cmdg_hevi* hevi, double* alpha, int* bandwidth, int64_t* nline);
int cmdg_hevi_solve(cmdg_hevi* hevi, double* d_Q, const double* d_Qhat, void* stream);
int cmdg_hevi_step(cmdg_hevi* hevi, double* d_Q, double t, int nsteps, void* stream);

/* Mixed precision: converts an FP64 state to the FP32 perturbation
 * q' = q - q_ref (the subtraction is done in FP64) and back.
 * No counterpart in the reference (the reference state lives in aux.ref_state,
 * src/Atmos/Model/ref_state.jl:66-67). */
int cmdg_to_perturbation(cmdg_model* model, float* d_Qp, const double* d_Q, void* stream);
int cmdg_from_perturbation(cmdg_model* model, double* d_Q, const float* d_Qp, void* stream);

/* Mixed-precision tendency: d_dQ (FP64) = alpha * dQ/dt(q_ref + d_Qp) + beta * d_dQ.
 * Same semantics as cmdg_tendency (src/Numerics/DGMethods/DGModel.jl:85-427). */
int cmdg_tendency_mixed(cmdg_model* model, double* d_dQ, const float* d_Qp, double t, double alpha, double beta,
                        void* stream);

/* Mixed-precision LSRK54 steps: FP32 perturbation state d_Qp, FP64 RK register d_dQ.
 * Same semantics as cmdg_lsrk54_step
 * (src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:102-158). */
int cmdg_lsrk54_step_mixed(cmdg_model* model, float* d_Qp, double* d_dQ, double t, double dt, int nsteps,
                           void* stream);

/* Mixed-precision LSRK54 steps of an FP64 state h_Q (Np, 5, nelem) held in
 * page-locked host memory (cudaHostAlloc / cudaMallocHost /
 * cudaHostRegister; anything else is refused with CMDG_ERR_ARG): h_Q is
 * copied over the host link into an FP64 device copy and converted to the
 * FP32 perturbation d_Qp, nsteps steps advance it with the FP64 register
 * d_dQ, and the FP64 result is copied back into h_Q.  The copies run on a
 * stream of the model's own in element chunks, each overlapping the
 * conversion of its neighbour, and are ordered after the earlier work of
 * `stream` and before its later work (synchronize it before reading h_Q).
 * The first call allocates the device copy (state-sized) and that stream.
 * The dostep! of a reference solver whose state lives in host memory
 * (src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:102-158). */
int cmdg_lsrk54_step_mixed_host(cmdg_model* model, double* h_Q, float* d_Qp, double* d_dQ, double t, double dt,
                                int nsteps, void* stream);

/* Compensated weighted sums sum_nodes M * Q[:, field, :] for nfields fields
 * (FP64 state), result into host memory; double-double accumulation.
 * Replaces weightedsum(Q, states) (src/Arrays/MPIStateArrays.jl:655-675). */
int cmdg_weighted_sums(cmdg_model* model, const double* d_Q, int nfields, const int* h_fields, double* h_out,
                       void* stream);
/* The same for a mixed-precision perturbation state: sum M*(q_ref + q'). */
int cmdg_weighted_sums_mixed(cmdg_model* model, const float* d_Qp, int nfields, const int* h_fields, double* h_out,
                             void* stream);

/* Time step from the nondiffusive Courant number (host-side evaluation of a
 * device state): dt = CFL / max_nodes((|u| + c_s) / dx_min).
 * Replaces calculate_dt (src/Numerics/DGMethods/DGMethods.jl:79-83,
 * src/Numerics/DGMethods/SpaceDiscretization.jl:307-365). */
int cmdg_courant_dt(cmdg_model* model, const double* d_Q, double CFL, double* h_dt, void* stream);

/* Gradient-flux state of d_Q (the diffusive pass that precedes every
 * tendency of a model with a turbulence closure) into d_gf, column-major
 * (Np, 10, nelem) in the model's precision: grad h_tot (3), S = sym(grad u)
 * as S11, S21, S31, S22, S32, S33, and N^2 (zero for ConstantDynamicViscosity).
 * Replaces launch_volume_gradients! + launch_interface_gradients! filling
 * dg.state_gradient_flux (src/Numerics/DGMethods/SpaceDiscretization.jl:502-728,
 * src/Numerics/DGMethods/DGModel.jl:132-230). */
int cmdg_gradient_flux(cmdg_model* model, void* d_gf, const void* d_Q, void* stream);

/* Hyperdiffusive state of d_Q (the passes that precede every tendency of a
 * model with DryBiharmonic hyperdiffusion) into d_hd, column-major in the
 * model's precision: word 3 c + d holds nu_4 d/dx_d (laplacian of c),
 * nu_4 = (Delta_h/2)^4/2/tau.  Brick: (Np, 9, nelem), c = u, v, h_tot (the
 * horizontal velocity u_h of a flat brick has no vertical component); cubed
 * shell: (Np, 12, nelem), c = u_h[0], u_h[1], u_h[2], h_tot.  d_hd must
 * hold that many words.
 * Replaces the hyperdiffusive part of launch_volume_gradients! +
 * launch_interface_gradients!, launch_volume_divergence_of_gradients! +
 * launch_interface_divergence_of_gradients! and
 * launch_volume_gradients_of_laplacians! +
 * launch_interface_gradients_of_laplacians! filling Qhypervisc_grad
 * (src/Numerics/DGMethods/SpaceDiscretization.jl:502-1090,
 * src/Numerics/DGMethods/DGModel.jl:132-301). */
int cmdg_hyperdiffusive_state(cmdg_model* model, void* d_hd, const void* d_Q, void* stream);

/* Device status word accumulated by the kernels since the last call;
 * reading clears it.
 *   bit 0: a kernel saw a non-finite tendency;
 *   bit 1: a bounded wait of the persistent stage kernel (grid_ctas >= 0) for
 *          its staging copies gave up (the CTA carried on with the shared
 *          buffer as it was, so the stage's results are not valid, waited
 *          again, bounded, for its copies in flight and returned; the
 *          context stays usable).
 * Replaces checked_wait's error flag (src/Arrays/MPIStateArrays.jl:910-936). */
int cmdg_status_word(cmdg_model* model, uint32_t* h_status, void* stream);

/* Test hook of the bounded waits (bit 1 of the status word) that makes them
 * run out without a fault: with skip_copies = 1 the persistent stage kernel
 * arms its staging barriers with the bytes of each element's copies but
 * issues no copy, so every wait gives up after wait_polls polls (0 = the
 * default limit of 65536).  skip_copies = 0, wait_polls = 0 restores normal
 * operation.  No counterpart in the reference. */
int cmdg_model_set_staging_test(cmdg_model* model, int skip_copies, int wait_polls);

#ifdef __cplusplus
}
#endif

#endif /* CMDG_H */
