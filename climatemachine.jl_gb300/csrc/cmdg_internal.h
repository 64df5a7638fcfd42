// Internal declarations shared by the libcmdg translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/cmdg.h"

namespace cmdg {

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

#define CMDG_CUDA_CHECK(call)                                                                       \
    do {                                                                                            \
        cudaError_t _e = (call);                                                                    \
        if (_e != cudaSuccess) {                                                                    \
            ::cmdg::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
            return CMDG_ERR_CUDA;                                                                   \
        }                                                                                           \
    } while (0)

#define CMDG_ARG_CHECK(cond, ...)           \
    do {                                    \
        if (!(cond)) {                      \
            ::cmdg::set_error(__VA_ARGS__); \
            return CMDG_ERR_ARG;            \
        }                                   \
    } while (0)

constexpr int NSTATE = 5;
// neighbour table row per element: 6 face neighbours (or -tag), vertical index, spare
constexpr int NBR_STRIDE = 8;
// stage-kernel families: one thread per node, one thread per vertical line
// of nodes, or one thread per node for the fluxes and one per element line
// for the face fluxes and contractions
enum { KERNEL_NODE = 0, KERNEL_COLUMN = 1, KERNEL_LINES = 2, KERNEL_CLUSTER = 3 };
constexpr int MIN_N = 2;
constexpr int MAX_N = 5;

// per vertical node level ("lvl") table columns (FP64 and FP32 copies)
enum LevelField {
    LV_PHI = 0,     // gravitational potential Phi = g z
    LV_GPHIZ,       // DG derivative dPhi/dz (the only non-zero component on a brick)
    LV_RHO_REF,     // reference density
    LV_P_REF,       // reference pressure
    LV_RHOE_REF,    // reference total energy density
    LV_CRHO,        // R_d T_0 - (R_d/cv_d) Phi : pressure coefficient of rho
    LV_HREF,        // rhoe_ref + p_ref : reference total enthalpy density
    LV_PAD,         // unused: rows are 8 wide so a row loads with 128-bit accesses
    LV_NFIELDS
};

// per vertical node level rows used by the diffusive passes (8 wide)
enum ViscLevelField {
    VV_THV_REF = 0,  // reference virtual potential temperature
    VV_DTHV_REF,     // its DG derivative along z (volume + central face terms)
    VV_HT_REF,       // reference total specific enthalpy (rhoe_ref + p_ref) / rho_ref
    VV_DHT_REF,      // its DG derivative along z
    VV_P_REF,        // reference pressure (duplicate of LV_P_REF, for the same row)
    VV_RHO_REF,      // reference density
    VV_PAD0,
    VV_PAD1,
    VV_NFIELDS
};

// gradient-flux words per node: grad h_tot (3), S = sym(grad u) (6), N^2 (Smagorinsky)
constexpr int NGF = 10;
// second-order flux words per node on bricks: F2[d][s] of fields s = 1..4 in
// the three directions, word 4 d + s - 1
constexpr int NF2 = 12;
// element chunks of a host-memory state: each chunk's copy over the host
// link overlaps the conversion of the one before it
constexpr int HOST_CHUNKS = 4;

// Physical constants in the form the kernels use them.
struct Physics {
    double R_d, cv_d, gamma, gm1, T_0, grav, inv_cv;
    int numflux, gravity, ref_state, subtract_off, turbulence;
    // diffusive terms (TurbulenceClosures.jl): rho*nu, WithDivergence, C_smag, 1/Pr_t,
    // kappa = R_d/cp_d and MSLP for theta_v
    double rho_nu, C_smag, inv_Pr_turb, kappa, MSLP;
    int with_divergence;
};

// mesh kinds: affine brick, stacked cubed shell (curvilinear, per-node
// metrics), or a mesh given by the reference's grid arrays (per-node metrics,
// reference state and facing nodes)
enum { MESH_BRICK = 0, MESH_SHELL = 1, MESH_ARRAYS = 2 };

// per-node geometry of a curvilinear mesh, (Np, CG_NFIELDS, nelem) on the host
enum CurvGeoField {
    CG_XI = 0,       // curl-invariant dxi_d/dx_j, 9 words: d-major (d = 0..2, then j = 0..2)
    CG_J = 9,        // det(dx/dxi)
    CG_M = 10,       // J w_i w_j w_k
    CG_DXMIN = 11,   // distance to the nearest neighbouring node along the element lines
    CG_NFIELDS = 12
};
// per-node kernel geometry of a model on a curvilinear mesh, (Np, KG_NFIELDS, nelem)
enum KernelGeoField {
    KG_JXI = 0,      // J dxi_d/dx_j, 9 words, d-major
    KG_INVJ = 9,
    KG_GPHI = 10,    // DG gradient of the geopotential, 3 words
    KG_DRHO = 13,    // reference density at the node minus its level value
    KG_DRHOE = 14,   // reference total energy at the node minus its level value
    KG_DCRHO = 15,   // pressure coefficient R_d T_0 - (R_d/cv_d) Phi at the node minus its level value
    KG_DPREF = 16,   // reference pressure at the node minus its level value
    KG_NFIELDS = 17
};

struct Mesh {
    int kind = MESH_BRICK;
    cmdg_brick_desc desc;
    cmdg_shell_desc shell;
    int N = 0, Nq = 0, Np = 0, Nfp = 0;
    int64_t nelem = 0;
    int nz = 0;                      // elements per column
    int nlev = 0;                    // vertical node levels = nz * Nq
    std::vector<double> xi, omega;   // LGL nodes / weights
    std::vector<double> D;           // D[j*Nq + k] = d l_k / d xi at xi_j
    std::vector<double> Dhat;        // Dhat[i*Nq + n] = D[n][i] w_n / w_i (weak-form volume operator)
    std::vector<double> emetric;     // [nelem][3] dxi_d/dx_d (affine brick)
    std::vector<int> nbr;            // [nelem][NBR_STRIDE]: 6 neighbours (or -tag), vertical index ez, spare
    std::vector<double> zlev;        // [nlev] node height of each vertical level
    std::vector<double> dzlev;       // [nlev] dz/dxi3 derivative helper (xi3x3 per level)
    // curvilinear meshes: node coordinates (Np, 3, nelem) and geometry (Np, CG_NFIELDS, nelem);
    // zlev holds the radius of each level, and nbr[7] the horizontal face
    // orientation codes (4 bits per face: neighbour face 0..3, bit 2 = the
    // in-face horizontal index runs reversed)
    std::vector<double> xyz, cgeo;
    // brick meshes: column order (col_at[h] = ix + nx iy of the h-th column)
    // and its topology (CMDG_TOPOLOGY_LIBRARY or CMDG_TOPOLOGY_STACKED_BRICK)
    // (empty in BrickTopology order, whose columns are not contiguous), and
    // the (ix, iy, iz) of every element
    std::vector<int> col_at;
    std::vector<int> ijk;
    int topology = CMDG_TOPOLOGY_LIBRARY;
    // grid-arrays meshes: the facing node of every face node, (Nfp, 6, nelem)
    std::vector<int> fpart;
    int* d_fpart = nullptr;
    // device copies
    double* d_emetric = nullptr;
    float* d_emetric32 = nullptr;
    int* d_nbr = nullptr;
};

struct GraphKey {
    const void* Q;
    const void* dQ;
    double dt;
    int nsteps;
    void* stream;
    bool operator<(const GraphKey& o) const {
        return std::tie(Q, dQ, dt, nsteps, stream) < std::tie(o.Q, o.dQ, o.dt, o.nsteps, o.stream);
    }
};

struct Model {
    Mesh* mesh = nullptr;
    cmdg_atmos_params prm;
    Physics ph;
    int precision = CMDG_FP64;
    std::vector<double> lvl64;       // [nlev][LV_NFIELDS]
    std::vector<float> lvl32;        // [nlev][LV_NFIELDS]
    std::vector<float> jump32;       // [nz][2] FP64-computed ref jumps (rho, rhoe) across the bottom face of level ez
    double* d_lvl64 = nullptr;
    float* d_lvl32 = nullptr;
    float* d_jump32 = nullptr;
    double* d_Dhat64 = nullptr;
    float* d_Dhat32 = nullptr;
    unsigned* d_status = nullptr;
    void* d_scratch = nullptr;       // two state-sized stage buffers (S1, S2) for the fused stage kernels
    size_t scratch_bytes = 0;
    std::vector<double> lvv64;       // [nlev][VV_NFIELDS] diffusive-pass reference rows
    double* d_lvv64 = nullptr;
    float* d_lvv32 = nullptr;
    void* d_gf = nullptr;            // gradient-flux state (Np, NGF, nelem) in the model's precision
    double* d_red = nullptr;         // reduction partials
    size_t red_len = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    double* d_geo64 = nullptr;       // curvilinear meshes: (Np, KG_NFIELDS, nelem)
    float* d_geo32 = nullptr;
    double* d_mass = nullptr;        // curvilinear meshes: M per node
    std::vector<double> ref64;       // curvilinear meshes: (Np, 2, nelem) rho_ref, rhoe_ref per node
    double* d_ref64 = nullptr;
    double* d_dxmin = nullptr;       // curvilinear meshes: nearest-node distance per node
    std::vector<float> filter_corr;  // mixed precision: vertical-filter change of the reference state per level
    float* d_filter_corr = nullptr;
    // mixed precision on other meshes: the reference state as a full FP64
    // state, a scratch copy for its filtered values, and the per-node change
    double* d_filter_ref64 = nullptr;
    double* d_mp_scratch = nullptr;  // mixed models: FP64 full state for the mass-preserving filter
    float* d_filter_corr_node = nullptr;
    double* d_omega = nullptr;       // LGL weights on the device (TMAR filter)
    void* d_hd = nullptr;            // hyperdiffusion: gradient, then nu grad^3, (Np, 9, nelem)
    void* d_hlap = nullptr;          // hyperdiffusion: laplacians (Np, 3, nelem)
    std::vector<double> glap_ref64;  // [nlev] DG d/dz of the laplacian of the reference h_tot
    float* d_glap_ref = nullptr;
    void* d_nu4 = nullptr;           // cubed shell: nu_4 per node, (Np, nelem), model precision
    float* d_hglap_ref = nullptr;    // cubed shell, mixed: nu_4 grad lap h_ref per node, (Np, 3, nelem)
    float* d_vgref = nullptr;        // cubed shell, viscous, mixed: grad h_ref per node, (Np, 3, nelem)
    double* d_sdelta = nullptr;      // cubed shell, SmagorinskyLilly: length scale per node (Np, nelem)
    // grid-arrays meshes: per-node kernel geometry on the host, per-node p_ref,
    // FP64-computed reference jumps (rho, rhoe) per face node, reference set?
    std::vector<double> arrays_geo, pref64;
    float* d_fjump = nullptr;
    bool has_reference = false;
    // linear (acoustic-gravity) model in VerticalDirection: per-node table
    // (Np, 10, nelem) and bottom/top face table (Nfp, 4, 2, nelem), FP64
    double* d_lin64 = nullptr;
    double* d_linface64 = nullptr;
    int lin_nz = 0;                  // grid-arrays meshes: elements per stack found for the linear model
    // grid-arrays meshes, FP64: caller-owned source and InitStateBC wall state
    // (Np, 5, nelem) device arrays, and the zero-enthalpy override
    const double* mms_src = nullptr;
    const double* mms_wall = nullptr;
    int mms_zero_h = 0;
    int grid_ctas = -1;              // stage-kernel grid: -1 = one CTA per element (the measured best
                                     // on GB300), 0 = one wave of resident CTAs, n > 0 = n CTAs
    int kernel_kind = 0;             // KERNEL_NODE, KERNEL_COLUMN, KERNEL_LINES or KERNEL_CLUSTER
    int* d_cl_elem = nullptr;        // KERNEL_CLUSTER: element of each CTA, clusters of cl_size adjacent elements
    int cl_size = 0;
    int device = -1;                 // CUDA device current when the model was created
    void* noalloc_stage = nullptr;   // device address of the allocation-free stage array on that device
    // stepping a state held in host memory: its FP64 device copy, the stream
    // of the host-link copies and the events that order them against the
    // conversions on the caller's stream (fork, HOST_CHUNKS copies in,
    // HOST_CHUNKS conversions out, join)
    double* d_host_stage = nullptr;
    cudaStream_t host_copy_stream = nullptr;
    cudaEvent_t host_ev[2 * HOST_CHUNKS + 2] = {};
    // test hook of the persistent stage kernel's bounded waits: when
    // staging_skip_copies is set the kernel arms its staging barriers without
    // issuing the copies, and every wait gives up after wait_polls polls
    int staging_skip_copies = 0;
    int wait_polls = 0;              // 0 = the default limit
};

// host-side setup (mesh.cpp, shell_mesh.cpp)
int build_brick(const cmdg_brick_desc* desc, Mesh* m, int topology = CMDG_TOPOLOGY_LIBRARY);
// element orders of the reference's brick topologies (order.cpp): Hilbert
// index of n coordinates of `bits` bits (n words, most significant first),
// the codes of element centroids (d x nelem), and the column order of a brick
void hilbert_code(const uint64_t* Y, int n, int bits, uint64_t* H);
void centroid_codes(const double* centroids, int d, int64_t nelem, std::vector<uint64_t>& code);
int brick_column_order(const cmdg_brick_desc& b, int topology, std::vector<int>& col_at);
int build_shell(const cmdg_shell_desc* desc, Mesh* m);
int build_arrays(const cmdg_grid_arrays* desc, Mesh* m);
int init_arrays_tables(Model* md);
int set_arrays_reference(Model* md, const double* aux7);
void lgl_derivative(Mesh* m);
int init_shell_tables(Model* md);
// virtual temperature and pressure of the reference profile at height z
void temperature_profile(const cmdg_atmos_params& p, double z, double& Tv, double& pres);
void lgl_nodes(int N, std::vector<double>& x, std::vector<double>& w);
int init_model_tables(Model* md);
int init_viscous_tables(Model* md);

// kernel launchers (stage.cu)
struct LaunchArgs {
    const void* Qin;
    void* Qout;
    double* dQ;
    double alpha, beta;      // tendency mode
    double rka, rkb_dt;      // stage mode: A_s applied to the previous increment, B_s dt
    int mode;                // 0 = tendency, 1 = RK stage
    int first_stage = 0;     // stage 1: the register is not read (A_1 = 0)
    int last_stage = 0;      // stage 5: the register is not written
    int remainder = 0;       // tendency mode on a mixed cubed shell: f - l of the vertical linear model
};
int launch_stage(Model* md, const LaunchArgs& a, cudaStream_t s);
// curvilinear stage kernel (shell.cu)
int launch_shell_stage(Model* md, const LaunchArgs& a, cudaStream_t s);
// whether launch_shell_stage can form the remainder f - l of the vertical
// acoustic-gravity linear model (mixed, inviscid, subtracted reference state)
bool shell_remainder_supported(const Model* md);
// grid-arrays stage kernel (arrays.cu)
int launch_arrays_stage(Model* md, const LaunchArgs& a, cudaStream_t s);
// LSRK54CarpenterKennedy A and B coefficient arrays (5 entries each)
void lsrk54_coefficients(const double** A, const double** B);
// CMDG_ERR_STATE (with the message set) for a model whose tendency depends on
// terms the caller refreshes at every stage time, which fused steps cannot honour
int check_fused_stepping(const Model* md);
// allocation-free stepping (noalloc.cu): device address of the fixed stage
// array on the current device, looked up when a model is created
int noalloc_stage_address(void** out);

// diffusive passes (viscous.cu): gradient flux of Qin (NGF words per node;
// with flux, the second-order flux rows it gives, NF2 words) into gf_out,
// then the stage kernel with second-order fluxes
int launch_gradient(Model* md, const void* Qin, void* gf_out, cudaStream_t s, bool flux = false);
int launch_viscous_stage(Model* md, const LaunchArgs& a, cudaStream_t s);

// hyperdiffusion (hyper.cu): reference rows and buffers, the three passes of
// Qin into hd_out (nu grad^3, (Np, 9, nelem)), and the stage with them
int init_hyper_tables(Model* md);
int launch_hyper_passes(Model* md, const void* Qin, void* hd_out, cudaStream_t s);
int launch_hyper_stage(Model* md, const LaunchArgs& a, cudaStream_t s);
// the same passes on the cubed shell (hyper_shell.cu): tables, then Qin into
// hd_out (nu grad^3 of u_h[0..2], h_tot, (Np, 12, nelem))
int init_shell_hyper_tables(Model* md);
int launch_shell_hyper_passes(Model* md, const void* Qin, void* hd_out, cudaStream_t s);
// ConstantDynamicViscosity on the cubed shell (hyper_shell.cu): the gradient
// buffer (grad u, grad h_tot, (Np, 12, nelem)) and, mixed, grad h_ref; the
// gradient pass of Qin into gout
int init_shell_visc_tables(Model* md);
// mixed precision: the FP64 gradients of the reference h_tot (and theta_v)
// per node into md->d_vgref (the viscous pass on the reference state at rest)
int visc_reference_gradients(Model* md);
int launch_shell_visc_gradient(Model* md, const void* Qin, void* gout, cudaStream_t s);

// reductions / conversions (reduce.cu)
// Qp = FP32 perturbation of Q about the reference state; Qd, if given, the
// FP64 perturbation
// elements [e0, e1) only (e1 < 0: to the last element)
int launch_to_perturbation(Model* md, float* Qp, const double* Q, cudaStream_t s, double* Qd = nullptr,
                           int64_t e0 = 0, int64_t e1 = -1);
int launch_from_perturbation(Model* md, double* Q, const float* Qp, cudaStream_t s, int64_t e0 = 0,
                             int64_t e1 = -1);
int weighted_sums(Model* md, const void* Q, bool mixed, int nfields, const int* fields, double* out, cudaStream_t s);
int courant_dt(Model* md, const double* Q, double CFL, double* dt, cudaStream_t s);
void release_quad(const Model* md);

}  // namespace cmdg

struct cmdg_mesh {
    cmdg::Mesh m;
};
struct cmdg_model {
    cmdg::Model m;
};
