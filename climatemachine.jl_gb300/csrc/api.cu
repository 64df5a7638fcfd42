// C ABI of libcmdg.so: object lifetime, argument checking, LSRK54 stepping
// with CUDA-graph capture, and the thin wrappers over the kernels.
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "cmdg_internal.h"

namespace cmdg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

const char* last_error() { return g_err; }

// LSRK54CarpenterKennedy 2N-storage coefficients (Carpenter & Kennedy 1994,
// NASA TM-109112), exact rationals as in
// src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:302-324.
static const double LSRK_A[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                                 -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
static const double LSRK_B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                                 1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                                 2277821191437.0 / 14882151754819.0};

// Two state-sized scratch buffers: the five stages of a step run
// Q -> S1 -> S2 -> S1 -> S2 -> Q, so every stage reads one buffer and writes
// another and the step ends in the caller's Q without a copy.
static int ensure_scratch(Model* md) {
    const Mesh& m = *md->mesh;
    const size_t elt = md->precision == CMDG_MIXED ? sizeof(float) : sizeof(double);
    const size_t need = 2 * (size_t)m.nelem * NSTATE * m.Np * elt;
    if (md->scratch_bytes >= need) return CMDG_OK;
    if (md->d_scratch) cudaFree(md->d_scratch);
    md->d_scratch = nullptr;
    md->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&md->d_scratch, need);
    if (e != cudaSuccess) {
        set_error("scratch allocation of %zu bytes failed: %s", need, cudaGetErrorString(e));
        return CMDG_ERR_ALLOC;
    }
    md->scratch_bytes = need;
    return CMDG_OK;
}

// Issues 5*nsteps fused stage kernels on stream s (stage buffers
// Q -> S1 -> S2 -> S1 -> S2 -> Q for every step).
static int issue_steps(Model* md, void* Q, double* dQ, double dt, int nsteps, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    const size_t elt = md->precision == CMDG_MIXED ? sizeof(float) : sizeof(double);
    const size_t bytes = (size_t)m.nelem * NSTATE * m.Np * elt;
    char* S1 = static_cast<char*>(md->d_scratch);
    char* S2 = S1 + bytes;
    void* const order[6] = {Q, S1, S2, S1, S2, Q};
    for (int step = 0; step < nsteps; ++step) {
        for (int st = 0; st < 5; ++st) {
            LaunchArgs a;
            a.Qin = order[st];
            a.Qout = order[st + 1];
            a.dQ = dQ;
            a.alpha = 1.0;
            a.beta = 1.0;
            a.rka = LSRK_A[st];
            a.rkb_dt = LSRK_B[st] * dt;
            a.mode = 1;
            a.first_stage = (st == 0);
            a.last_stage = (st == 4);
            int rc = launch_stage(md, a, s);
            if (rc) return rc;
        }
    }
    return CMDG_OK;
}

// The fused steps run five stages with no host work between them, so a term
// the caller refreshes at every stage time t + C_s dt cannot enter them.
int check_fused_stepping(const Model* md) {
    if (md->mms_src != nullptr || md->mms_wall != nullptr) {
        set_error("the model's manufactured-solution source or wall state is refreshed by the caller at each stage "
                  "time; step it stage by stage (cmdg_tendency at t + C_s dt), not with the fused LSRK54 steps");
        return CMDG_ERR_STATE;
    }
    return CMDG_OK;
}

static int run_steps(Model* md, void* Q, double* dQ, double dt, int nsteps, cudaStream_t s) {
    int rc = check_fused_stepping(md);
    if (rc) return rc;
    rc = ensure_scratch(md);
    if (rc) return rc;
    if (s == nullptr || nsteps > 64) return issue_steps(md, Q, dQ, dt, nsteps, s);
    // capture once per (Q, dQ, dt, nsteps, stream), replay afterwards
    GraphKey key{Q, dQ, dt, nsteps, (void*)s};
    auto it = md->graphs.find(key);
    if (it == md->graphs.end()) {
        cudaGraph_t g;
        CMDG_CUDA_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        rc = issue_steps(md, Q, dQ, dt, nsteps, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc) return rc;
        if (ce != cudaSuccess) {
            set_error("graph capture failed: %s", cudaGetErrorString(ce));
            return CMDG_ERR_CUDA;
        }
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            set_error("graph instantiate failed: %s", cudaGetErrorString(ce));
            return CMDG_ERR_CUDA;
        }
        if (md->graphs.size() > 32) {
            for (auto& kv : md->graphs) cudaGraphExecDestroy(kv.second);
            md->graphs.clear();
        }
        it = md->graphs.emplace(key, ex).first;
    }
    CMDG_CUDA_CHECK(cudaGraphLaunch(it->second, s));
    return CMDG_OK;
}

void lsrk54_coefficients(const double** A, const double** B) {
    *A = LSRK_A;
    *B = LSRK_B;
}

static int check_model(const cmdg_model* model) {
    if (!model) {
        set_error("model is NULL");
        return CMDG_ERR_ARG;
    }
    return CMDG_OK;
}

}  // namespace cmdg

using namespace cmdg;

extern "C" {

const char* cmdg_last_error(void) { return cmdg::last_error(); }

const char* cmdg_version(void) { return "cmdg 0.1 (sm_103a)"; }

int cmdg_mesh_create_brick(const cmdg_brick_desc* desc, cmdg_mesh** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    cmdg_mesh* mh = new cmdg_mesh();
    int rc = build_brick(desc, &mh->m);
    if (rc) {
        if (mh->m.d_emetric) cudaFree(mh->m.d_emetric);
        if (mh->m.d_nbr) cudaFree(mh->m.d_nbr);
        if (mh->m.d_emetric32) cudaFree(mh->m.d_emetric32);
        delete mh;
        return rc;
    }
    *out = mh;
    return CMDG_OK;
}

int cmdg_mesh_create_brick_ordered(const cmdg_brick_desc* desc, int topology, cmdg_mesh** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    CMDG_ARG_CHECK(topology == CMDG_TOPOLOGY_LIBRARY || topology == CMDG_TOPOLOGY_STACKED_BRICK ||
                       topology == CMDG_TOPOLOGY_BRICK,
                   "unknown topology order %d", topology);
    cmdg_mesh* mh = new cmdg_mesh();
    int rc = build_brick(desc, &mh->m, topology);
    if (rc) {
        if (mh->m.d_emetric) cudaFree(mh->m.d_emetric);
        if (mh->m.d_nbr) cudaFree(mh->m.d_nbr);
        if (mh->m.d_emetric32) cudaFree(mh->m.d_emetric32);
        delete mh;
        return rc;
    }
    *out = mh;
    return CMDG_OK;
}

int cmdg_mesh_create_shell(const cmdg_shell_desc* desc, cmdg_mesh** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    cmdg_mesh* mh = new cmdg_mesh();
    int rc = build_shell(desc, &mh->m);
    if (rc) {
        if (mh->m.d_nbr) cudaFree(mh->m.d_nbr);
        delete mh;
        return rc;
    }
    *out = mh;
    return CMDG_OK;
}

int cmdg_mesh_create_arrays(const cmdg_grid_arrays* desc, cmdg_mesh** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    cmdg_mesh* mh = new cmdg_mesh();
    int rc = build_arrays(desc, &mh->m);
    if (rc) {
        cudaFree(mh->m.d_nbr);
        cudaFree(mh->m.d_fpart);
        delete mh;
        return rc;
    }
    *out = mh;
    return CMDG_OK;
}

int cmdg_mesh_destroy(cmdg_mesh* mesh) {
    if (!mesh) return CMDG_OK;
    cudaFree(mesh->m.d_emetric);
    cudaFree(mesh->m.d_nbr);
    cudaFree(mesh->m.d_emetric32);
    cudaFree(mesh->m.d_fpart);
    delete mesh;
    return CMDG_OK;
}

int cmdg_mesh_info(const cmdg_mesh* mesh, int64_t* nelem, int* Np) {
    CMDG_ARG_CHECK(mesh != nullptr, "mesh is NULL");
    if (nelem) *nelem = mesh->m.nelem;
    if (Np) *Np = mesh->m.Np;
    return CMDG_OK;
}

int cmdg_mesh_coordinates(const cmdg_mesh* mesh, double* h_xyz) {
    CMDG_ARG_CHECK(mesh != nullptr && h_xyz != nullptr, "NULL argument");
    const Mesh& m = mesh->m;
    const int Nq = m.Nq, Np = m.Np;
    if (m.kind != MESH_BRICK) {
        std::memcpy(h_xyz, m.xyz.data(), sizeof(double) * m.xyz.size());
        return CMDG_OK;
    }
    for (int64_t e = 0; e < m.nelem; ++e) {
        const int64_t idx[3] = {m.ijk[(size_t)e * 3 + 0], m.ijk[(size_t)e * 3 + 1], m.ijk[(size_t)e * 3 + 2]};
        for (int d = 0; d < 3; ++d) {
            const double lo = m.desc.lo[d], hi = m.desc.hi[d];
            const int n = m.desc.ne[d];
            const double a = (double)(((long double)lo * (n - idx[d]) + (long double)hi * idx[d]) / n);
            const double b = (double)(((long double)lo * (n - idx[d] - 1) + (long double)hi * (idx[d] + 1)) / n);
            for (int node = 0; node < Np; ++node) {
                const int ijk[3] = {node % Nq, (node / Nq) % Nq, node / (Nq * Nq)};
                h_xyz[((size_t)e * 3 + d) * Np + node] = a + (m.xi[ijk[d]] + 1) * 0.5 * (b - a);
            }
        }
    }
    return CMDG_OK;
}

int cmdg_mesh_mass(const cmdg_mesh* mesh, double* h_M) {
    CMDG_ARG_CHECK(mesh != nullptr && h_M != nullptr, "NULL argument");
    const Mesh& m = mesh->m;
    const int Nq = m.Nq, Np = m.Np;
    if (m.kind != MESH_BRICK) {
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int node = 0; node < Np; ++node)
                h_M[(size_t)e * Np + node] = m.cgeo[((size_t)e * CG_NFIELDS + CG_M) * Np + node];
        return CMDG_OK;
    }
    for (int64_t e = 0; e < m.nelem; ++e) {
        const double J = 1.0 / (m.emetric[3 * e] * m.emetric[3 * e + 1] * m.emetric[3 * e + 2]);
        for (int node = 0; node < Np; ++node) {
            const int i = node % Nq, j = (node / Nq) % Nq, k = node / (Nq * Nq);
            h_M[(size_t)e * Np + node] = J * (m.omega[i] * m.omega[j] * m.omega[k]);
        }
    }
    return CMDG_OK;
}

int cmdg_model_create(cmdg_mesh* mesh, const cmdg_atmos_params* p, int precision, cmdg_model** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    CMDG_ARG_CHECK(mesh != nullptr && p != nullptr, "NULL argument");
    CMDG_ARG_CHECK(precision == CMDG_FP64 || precision == CMDG_MIXED, "unknown precision %d", precision);
    CMDG_ARG_CHECK(p->numflux == CMDG_FLUX_RUSANOV || p->numflux == CMDG_FLUX_CENTRAL, "unknown numerical flux %d",
                   p->numflux);
    const bool shell = mesh->m.kind == MESH_SHELL;
    const bool arrays = mesh->m.kind == MESH_ARRAYS;
    if (arrays) {
        CMDG_ARG_CHECK(p->hyperdiffusion == CMDG_HYPER_NONE, "no hyperdiffusion on grid-arrays meshes");
        CMDG_ARG_CHECK(p->orientation >= CMDG_ORIENT_NONE && p->orientation <= CMDG_ORIENT_SPHERE,
                       "unknown orientation %d", p->orientation);
    } else if (shell) {
        CMDG_ARG_CHECK(p->orientation == CMDG_ORIENT_NONE || p->orientation == CMDG_ORIENT_SPHERE,
                       "orientation %d is not available on a cubed shell", p->orientation);
        CMDG_ARG_CHECK(p->turbulence == CMDG_TURB_NONE || p->hyperdiffusion == CMDG_HYPER_NONE,
                       "the cubed-shell kernels run viscosity or hyperdiffusion, not both");
        CMDG_ARG_CHECK(p->orientation != CMDG_ORIENT_SPHERE || p->planet_radius > 0, "planet_radius must be positive");
    } else {
        CMDG_ARG_CHECK(p->orientation == CMDG_ORIENT_NONE || p->orientation == CMDG_ORIENT_FLAT,
                       "orientation %d is not available on a brick", p->orientation);
    }
    CMDG_ARG_CHECK(p->R_d > 0 && p->cv_d > 0 && p->cp_d > 0, "gas constants must be positive");
    CMDG_ARG_CHECK(p->turbulence == CMDG_TURB_NONE || p->turbulence == CMDG_TURB_CONSTANT ||
                       p->turbulence == CMDG_TURB_SMAGORINSKY,
                   "unknown turbulence closure %d", p->turbulence);
    CMDG_ARG_CHECK(p->turbulence != CMDG_TURB_SMAGORINSKY || p->orientation != CMDG_ORIENT_NONE,
                   "SmagorinskyLilly needs an orientation (its buoyancy correction uses grad Phi)");
    CMDG_ARG_CHECK(p->hyperdiffusion == CMDG_HYPER_NONE || p->hyperdiffusion == CMDG_HYPER_DRY_BIHARMONIC,
                   "unknown hyperdiffusion %d", p->hyperdiffusion);
    if (p->hyperdiffusion != CMDG_HYPER_NONE) {
        CMDG_ARG_CHECK(p->orientation == (shell ? CMDG_ORIENT_SPHERE : CMDG_ORIENT_FLAT),
                       "DryBiharmonic needs %s (u_h = (I - khat khat') u)",
                       shell ? "SphericalOrientation on a cubed shell" : "FlatOrientation on a brick");
        CMDG_ARG_CHECK(p->tau_hyper > 0, "DryBiharmonic tau_timescale must be positive");
        CMDG_ARG_CHECK(p->hyper_direction == CMDG_DIR_EVERY || p->hyper_direction == CMDG_DIR_HORIZONTAL,
                       "hyperdiffusion direction %d: EveryDirection or HorizontalDirection", p->hyper_direction);
    }
    cmdg_model* mo = new cmdg_model();
    Model& md = mo->m;
    md.mesh = &mesh->m;
    md.prm = *p;
    md.precision = precision;
    md.ph.R_d = p->R_d;
    md.ph.cv_d = p->cv_d;
    md.ph.gamma = p->cp_d / p->cv_d;
    md.ph.gm1 = p->R_d / p->cv_d;
    md.ph.T_0 = p->T_0;
    md.ph.grav = p->grav;
    md.ph.inv_cv = 1.0 / p->cv_d;
    md.ph.numflux = p->numflux;
    md.ph.gravity = p->gravity;
    md.ph.ref_state = p->ref_state;
    md.ph.subtract_off = p->subtract_off;
    md.ph.turbulence = p->turbulence;
    md.ph.rho_nu = p->rho_nu;
    md.ph.C_smag = p->C_smag;
    md.ph.inv_Pr_turb = p->inv_Pr_turb;
    md.ph.kappa = p->R_d / p->cp_d;
    md.ph.MSLP = p->MSLP;
    md.ph.with_divergence = p->with_divergence;
    int rc = init_model_tables(&md);
    if (rc == CMDG_OK && shell) rc = init_shell_tables(&md);
    if (rc == CMDG_OK && arrays) rc = init_arrays_tables(&md);
    if (rc == CMDG_OK && !shell && !arrays &&
        (p->turbulence != CMDG_TURB_NONE || p->hyperdiffusion != CMDG_HYPER_NONE))
        rc = init_viscous_tables(&md);
    if (rc == CMDG_OK && p->hyperdiffusion != CMDG_HYPER_NONE)
        rc = shell ? init_shell_hyper_tables(&md) : init_hyper_tables(&md);
    if (rc == CMDG_OK && (shell || arrays) && p->turbulence != CMDG_TURB_NONE) rc = init_shell_visc_tables(&md);
    if (rc == CMDG_OK) {
        cudaError_t e = cudaMalloc(&md.d_status, sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMemset(md.d_status, 0, sizeof(unsigned));
        if (e != cudaSuccess) {
            set_error("status word allocation failed: %s", cudaGetErrorString(e));
            rc = CMDG_ERR_CUDA;
        }
    }
    if (rc == CMDG_OK) {
        cudaError_t e = cudaGetDevice(&md.device);
        if (e != cudaSuccess) {
            set_error("cudaGetDevice failed: %s", cudaGetErrorString(e));
            rc = CMDG_ERR_CUDA;
        }
    }
    // set-up of the allocation-free stepping: loading the module that holds
    // its fixed stage array reserves the array on this device now, while the
    // library may still allocate, not at the first allocation-free call
    if (rc == CMDG_OK) rc = noalloc_stage_address(&md.noalloc_stage);
    if (rc) {
        cmdg_model_destroy(mo);
        return rc;
    }
    *out = mo;
    return CMDG_OK;
}

int cmdg_model_destroy(cmdg_model* model) {
    if (!model) return CMDG_OK;
    Model& md = model->m;
    for (auto& kv : md.graphs) cudaGraphExecDestroy(kv.second);
    cudaFree(md.d_lvl64);
    cudaFree(md.d_lvl32);
    cudaFree(md.d_jump32);
    cudaFree(md.d_Dhat64);
    cudaFree(md.d_Dhat32);
    cudaFree(md.d_status);
    cudaFree(md.d_scratch);
    cudaFree(md.d_cl_elem);
    cudaFree(md.d_red);
    cudaFree(md.d_lvv64);
    cudaFree(md.d_lvv32);
    cudaFree(md.d_gf);
    cudaFree(md.d_hd);
    cudaFree(md.d_hlap);
    cudaFree(md.d_glap_ref);
    cudaFree(md.d_nu4);
    cudaFree(md.d_hglap_ref);
    cudaFree(md.d_vgref);
    cudaFree(md.d_sdelta);
    cudaFree(md.d_fjump);
    cudaFree(md.d_geo64);
    cudaFree(md.d_geo32);
    cudaFree(md.d_mass);
    cudaFree(md.d_dxmin);
    cudaFree(md.d_ref64);
    cudaFree(md.d_filter_corr);
    cudaFree(md.d_filter_ref64);
    cudaFree(md.d_mp_scratch);
    cudaFree(md.d_host_stage);
    for (cudaEvent_t e : md.host_ev)
        if (e) cudaEventDestroy(e);
    if (md.host_copy_stream) cudaStreamDestroy(md.host_copy_stream);
    cudaFree(md.d_filter_corr_node);
    cudaFree(md.d_omega);
    cudaFree(md.d_lin64);
    cudaFree(md.d_linface64);
    release_quad(&md);
    delete model;
    return CMDG_OK;
}

int cmdg_model_reference_state(const cmdg_model* model, double* h_ref) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(h_ref != nullptr, "NULL output");
    const Model& md = model->m;
    const Mesh& m = *md.mesh;
    const bool pernode = !md.ref64.empty(), pernode_p = !md.pref64.empty();
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int node = 0; node < m.Np; ++node) {
            const int lev = m.nbr[(size_t)e * NBR_STRIDE + 6] * m.Nq + node / m.Nfp;
            const double* L = &md.lvl64[(size_t)lev * LV_NFIELDS];
            h_ref[((size_t)e * 3 + 0) * m.Np + node] = pernode ? md.ref64[((size_t)e * 2 + 0) * m.Np + node] : L[LV_RHO_REF];
            h_ref[((size_t)e * 3 + 1) * m.Np + node] = pernode ? md.ref64[((size_t)e * 2 + 1) * m.Np + node] : L[LV_RHOE_REF];
            h_ref[((size_t)e * 3 + 2) * m.Np + node] = pernode_p ? md.pref64[(size_t)e * m.Np + node] : L[LV_P_REF];
        }
    return CMDG_OK;
}

int cmdg_model_set_mms(cmdg_model* model, const double* d_src, const double* d_wall, int zero_enthalpy) {
    int rc = check_model(model);
    if (rc) return rc;
    Model& md = model->m;
    CMDG_ARG_CHECK(md.mesh->kind == MESH_ARRAYS && md.precision == CMDG_FP64,
                   "sources and InitStateBC wall states are set on FP64 models on grid-arrays meshes");
    md.mms_src = d_src;
    md.mms_wall = d_wall;
    md.mms_zero_h = zero_enthalpy ? 1 : 0;
    for (auto& kv : md.graphs) cudaGraphExecDestroy(kv.second);
    md.graphs.clear();
    return CMDG_OK;
}

int cmdg_model_set_reference(cmdg_model* model, const double* h_aux7) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(h_aux7 != nullptr, "NULL aux");
    CMDG_ARG_CHECK(model->m.mesh->kind == MESH_ARRAYS,
                   "cmdg_model_set_reference applies to models on grid-arrays meshes (the generated meshes build "
                   "their reference state)");
    CMDG_CUDA_CHECK(cudaDeviceSynchronize());  // no stage may be reading the tables being replaced
    return set_arrays_reference(&model->m, h_aux7);
}

int cmdg_tendency(cmdg_model* model, double* d_dQ, const double* d_Q, double t, double alpha, double beta,
                  void* stream) {
    (void)t;
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(model->m.precision == CMDG_FP64, "cmdg_tendency needs an FP64 model");
    CMDG_ARG_CHECK(d_dQ != nullptr && d_Q != nullptr, "NULL state");
    LaunchArgs a{d_Q, nullptr, d_dQ, alpha, beta, 0.0, 0.0, 0, 0, 0};
    return launch_stage(&model->m, a, (cudaStream_t)stream);
}

int cmdg_tendency_mixed(cmdg_model* model, double* d_dQ, const float* d_Qp, double t, double alpha, double beta,
                        void* stream) {
    (void)t;
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(model->m.precision == CMDG_MIXED, "cmdg_tendency_mixed needs a mixed-precision model");
    CMDG_ARG_CHECK(d_dQ != nullptr && d_Qp != nullptr, "NULL state");
    LaunchArgs a{d_Qp, nullptr, d_dQ, alpha, beta, 0.0, 0.0, 0, 0, 0};
    return launch_stage(&model->m, a, (cudaStream_t)stream);
}

int cmdg_lsrk54_step(cmdg_model* model, double* d_Q, double* d_dQ, double t, double dt, int nsteps, void* stream) {
    (void)t;
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(model->m.precision == CMDG_FP64, "cmdg_lsrk54_step needs an FP64 model");
    CMDG_ARG_CHECK(d_Q != nullptr && d_dQ != nullptr, "NULL state");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    CMDG_ARG_CHECK(std::isfinite(dt) && dt > 0, "dt must be positive and finite");
    if (nsteps == 0) return CMDG_OK;
    return run_steps(&model->m, d_Q, d_dQ, dt, nsteps, (cudaStream_t)stream);
}

int cmdg_lsrk54_step_mixed(cmdg_model* model, float* d_Qp, double* d_dQ, double t, double dt, int nsteps,
                           void* stream) {
    (void)t;
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(model->m.precision == CMDG_MIXED, "cmdg_lsrk54_step_mixed needs a mixed-precision model");
    CMDG_ARG_CHECK(d_Qp != nullptr && d_dQ != nullptr, "NULL state");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    CMDG_ARG_CHECK(std::isfinite(dt) && dt > 0, "dt must be positive and finite");
    if (nsteps == 0) return CMDG_OK;
    return run_steps(&model->m, d_Qp, d_dQ, dt, nsteps, (cudaStream_t)stream);
}

namespace cmdg {
// FP64 device copy of a host-memory state, the copy stream and its events,
// made on first use with the model's device current
static int ensure_host_staging(Model* md) {
    const Mesh& m = *md->mesh;
    if (!md->host_copy_stream)
        CMDG_CUDA_CHECK(cudaStreamCreateWithFlags(&md->host_copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : md->host_ev)
        if (!e) CMDG_CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!md->d_host_stage)
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_host_stage, sizeof(double) * NSTATE * m.Np * (size_t)m.nelem));
    return CMDG_OK;
}
}  // namespace cmdg

int cmdg_lsrk54_step_mixed_host(cmdg_model* model, double* h_Q, float* d_Qp, double* d_dQ, double t, double dt,
                                int nsteps, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(model->m.precision == CMDG_MIXED, "cmdg_lsrk54_step_mixed_host needs a mixed-precision model");
    CMDG_ARG_CHECK(h_Q != nullptr && d_Qp != nullptr && d_dQ != nullptr, "NULL state");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    CMDG_ARG_CHECK(std::isfinite(dt) && dt > 0, "dt must be positive and finite");
    // the host state must be page-locked, so the copies run asynchronously on the copy engines
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, h_Q);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("h_Q: %s", cudaGetErrorString(e));
        return CMDG_ERR_ARG;
    }
    CMDG_ARG_CHECK(attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr,
                   "h_Q must be page-locked host memory (cudaHostAlloc, cudaMallocHost or cudaHostRegister)");
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    if ((rc = ensure_host_staging(md))) return rc;
    const cudaStream_t s = (cudaStream_t)stream, cs = md->host_copy_stream;
    double* stage = md->d_host_stage;
    cudaEvent_t* ev = md->host_ev;  // [0] fork, [1..K] copied in, [K+1..2K] converted out, [2K+1] join
    const size_t per_elem = (size_t)NSTATE * m.Np;
    auto chunk = [&](int k, int64_t& e0, int64_t& e1) {
        e0 = m.nelem * k / HOST_CHUNKS;
        e1 = m.nelem * (k + 1) / HOST_CHUNKS;
    };
    // host -> device on the copy stream, chunk by chunk, after the caller's earlier work;
    // each chunk's conversion on the caller's stream overlaps the next chunk's copy
    CMDG_CUDA_CHECK(cudaEventRecord(ev[0], s));
    CMDG_CUDA_CHECK(cudaStreamWaitEvent(cs, ev[0], 0));
    for (int k = 0; k < HOST_CHUNKS; ++k) {
        int64_t e0, e1;
        chunk(k, e0, e1);
        if (e1 > e0)
            CMDG_CUDA_CHECK(cudaMemcpyAsync(stage + e0 * per_elem, h_Q + e0 * per_elem,
                                            (size_t)(e1 - e0) * per_elem * sizeof(double), cudaMemcpyHostToDevice,
                                            cs));
        CMDG_CUDA_CHECK(cudaEventRecord(ev[1 + k], cs));
    }
    for (int k = 0; k < HOST_CHUNKS; ++k) {
        int64_t e0, e1;
        chunk(k, e0, e1);
        CMDG_CUDA_CHECK(cudaStreamWaitEvent(s, ev[1 + k], 0));
        if ((rc = launch_to_perturbation(md, d_Qp, stage, s, nullptr, e0, e1))) return rc;
    }
    if (nsteps > 0 && (rc = cmdg_lsrk54_step_mixed(model, d_Qp, d_dQ, t, dt, nsteps, stream))) return rc;
    // device -> host: each converted chunk is copied back while the next converts
    for (int k = 0; k < HOST_CHUNKS; ++k) {
        int64_t e0, e1;
        chunk(k, e0, e1);
        if ((rc = launch_from_perturbation(md, stage, d_Qp, s, e0, e1))) return rc;
        CMDG_CUDA_CHECK(cudaEventRecord(ev[1 + HOST_CHUNKS + k], s));
        CMDG_CUDA_CHECK(cudaStreamWaitEvent(cs, ev[1 + HOST_CHUNKS + k], 0));
        if (e1 > e0)
            CMDG_CUDA_CHECK(cudaMemcpyAsync(h_Q + e0 * per_elem, stage + e0 * per_elem,
                                            (size_t)(e1 - e0) * per_elem * sizeof(double), cudaMemcpyDeviceToHost,
                                            cs));
    }
    // the caller's stream resumes after the last copy back
    CMDG_CUDA_CHECK(cudaEventRecord(ev[1 + 2 * HOST_CHUNKS], cs));
    CMDG_CUDA_CHECK(cudaStreamWaitEvent(s, ev[1 + 2 * HOST_CHUNKS], 0));
    return CMDG_OK;
}

int cmdg_to_perturbation(cmdg_model* model, float* d_Qp, const double* d_Q, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_Qp != nullptr && d_Q != nullptr, "NULL state");
    return launch_to_perturbation(&model->m, d_Qp, d_Q, (cudaStream_t)stream);
}

int cmdg_from_perturbation(cmdg_model* model, double* d_Q, const float* d_Qp, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_Qp != nullptr && d_Q != nullptr, "NULL state");
    return launch_from_perturbation(&model->m, d_Q, d_Qp, (cudaStream_t)stream);
}

int cmdg_weighted_sums(cmdg_model* model, const double* d_Q, int nfields, const int* h_fields, double* h_out,
                       void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_Q && h_fields && h_out && nfields > 0, "bad arguments");
    return weighted_sums(&model->m, d_Q, false, nfields, h_fields, h_out, (cudaStream_t)stream);
}

int cmdg_weighted_sums_mixed(cmdg_model* model, const float* d_Qp, int nfields, const int* h_fields, double* h_out,
                             void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_Qp && h_fields && h_out && nfields > 0, "bad arguments");
    return weighted_sums(&model->m, d_Qp, true, nfields, h_fields, h_out, (cudaStream_t)stream);
}

int cmdg_courant_dt(cmdg_model* model, const double* d_Q, double CFL, double* h_dt, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_Q && h_dt && CFL > 0, "bad arguments");
    return courant_dt(&model->m, d_Q, CFL, h_dt, (cudaStream_t)stream);
}

int cmdg_gradient_flux(cmdg_model* model, void* d_gf, const void* d_Q, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(d_gf != nullptr && d_Q != nullptr, "NULL buffer");
    CMDG_ARG_CHECK(model->m.prm.turbulence != CMDG_TURB_NONE, "the model has no diffusive terms");
    CMDG_ARG_CHECK(model->m.mesh->kind == MESH_BRICK, "cmdg_gradient_flux exposes the brick gradient-flux layout");
    return launch_gradient(&model->m, d_Q, d_gf, (cudaStream_t)stream);
}

int cmdg_model_set_staging_test(cmdg_model* model, int skip_copies, int wait_polls) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(wait_polls >= 0, "wait_polls must be >= 0");
    Model& md = model->m;
    md.staging_skip_copies = skip_copies ? 1 : 0;
    md.wait_polls = wait_polls;
    // captured graphs hold the old launch parameters
    for (auto& kv : md.graphs) cudaGraphExecDestroy(kv.second);
    md.graphs.clear();
    return CMDG_OK;
}

int cmdg_status_word(cmdg_model* model, uint32_t* h_status, void* stream) {
    int rc = check_model(model);
    if (rc) return rc;
    CMDG_ARG_CHECK(h_status != nullptr, "NULL output");
    cudaStream_t s = (cudaStream_t)stream;
    CMDG_CUDA_CHECK(cudaMemcpyAsync(h_status, model->m.d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CMDG_CUDA_CHECK(cudaMemsetAsync(model->m.d_status, 0, sizeof(unsigned), s));
    CMDG_CUDA_CHECK(cudaStreamSynchronize(s));
    return CMDG_OK;
}

}  // extern "C"
