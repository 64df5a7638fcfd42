// Launch-configuration selection for the fused stage kernels: explicit
// setting, and a timing autotuner over the candidates of a model.
#include <cstring>
#include <vector>

#include "cmdg_internal.h"

namespace {

struct Candidate {
    int kind;
    int grid;  // 0 = one wave of resident CTAs (persistent), n > 0 = n CTAs, -1 = one CTA per element
};

}  // namespace

namespace cmdg {

// The element of every CTA of the cluster kernel: clusters of CL adjacent
// elements of a brick (2 x 2 x 2 in x, y, z for CL = 8, 2 x 1 x 2 for 4,
// 1 x 1 x 2 for 2), cluster rank bit 0 = upper in z, bit 1 = upper in x,
// bit 2 = upper in y; clusters ordered z fastest, then x, then y, whatever
// the mesh's element numbering.  Needs an inviscid brick whose element
// counts are even in the directions the cluster spans.
int build_cluster_map(Model* md, int CL) {
    const Mesh& m = *md->mesh;
    CMDG_ARG_CHECK(CL == 2 || CL == 4 || CL == 8, "cluster size must be 2, 4 or 8, got %d", CL);
    if (m.kind != MESH_BRICK || m.ijk.empty() || md->prm.turbulence != CMDG_TURB_NONE ||
        md->prm.hyperdiffusion != CMDG_HYPER_NONE) {
        set_error("the cluster kernel runs inviscid models on bricks");
        return CMDG_ERR_UNSUPPORTED;
    }
    const int nx = m.desc.ne[0], ny = m.desc.ne[1], nz = m.desc.ne[2];
    if (nz % 2 || (CL >= 4 && nx % 2) || (CL == 8 && ny % 2)) {
        set_error("clusters of %d elements need even element counts in the directions they span (%d x %d x %d)", CL,
                  nx, ny, nz);
        return CMDG_ERR_UNSUPPORTED;
    }
    const int sx = CL >= 4 ? 2 : 1, sy = CL == 8 ? 2 : 1;
    std::vector<int> elem_at((size_t)m.nelem, -1);  // element at library index iz + nz (ix + nx iy)
    for (int64_t e = 0; e < m.nelem; ++e)
        elem_at[(size_t)m.ijk[(size_t)e * 3 + 2] +
                (size_t)nz * ((size_t)m.ijk[(size_t)e * 3 + 0] + (size_t)nx * m.ijk[(size_t)e * 3 + 1])] = (int)e;
    std::vector<int> map((size_t)m.nelem);
    size_t b = 0;
    for (int by = 0; by < ny / sy; ++by)
        for (int bx = 0; bx < nx / sx; ++bx)
            for (int bz = 0; bz < nz / 2; ++bz)
                for (int r = 0; r < CL; ++r) {
                    const int iz = 2 * bz + (r & 1);
                    const int ix = sx * bx + (CL >= 4 ? (r >> 1) & 1 : 0);
                    const int iy = sy * by + (CL == 8 ? (r >> 2) & 1 : 0);
                    map[b++] = elem_at[(size_t)iz + (size_t)nz * ((size_t)ix + (size_t)nx * iy)];
                }
    if (md->d_cl_elem) cudaFree(md->d_cl_elem);
    md->d_cl_elem = nullptr;
    md->cl_size = 0;
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_cl_elem, sizeof(int) * map.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_cl_elem, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice));
    md->cl_size = CL;
    return CMDG_OK;
}

}  // namespace cmdg

extern "C" int cmdg_model_set_kernel(cmdg_model* model, int kernel_kind, int grid_ctas) {
    using namespace cmdg;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    CMDG_ARG_CHECK(kernel_kind == KERNEL_NODE || kernel_kind == KERNEL_COLUMN || kernel_kind == KERNEL_LINES ||
                       kernel_kind == KERNEL_CLUSTER,
                   "unknown kernel kind %d", kernel_kind);
    CMDG_ARG_CHECK(grid_ctas >= -1, "grid_ctas must be >= -1");
    if (kernel_kind == KERNEL_CLUSTER) {
        const int rc = build_cluster_map(&model->m, grid_ctas);
        if (rc) return rc;
    }
    model->m.kernel_kind = kernel_kind;
    model->m.grid_ctas = grid_ctas;
    // captured step graphs embed the old launch configuration
    for (auto& kv : model->m.graphs) cudaGraphExecDestroy(kv.second);
    model->m.graphs.clear();
    return CMDG_OK;
}

extern "C" int cmdg_model_get_kernel(const cmdg_model* model, int* kernel_kind, int* grid_ctas) {
    using namespace cmdg;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    if (kernel_kind) *kernel_kind = model->m.kernel_kind;
    if (grid_ctas) *grid_ctas = model->m.grid_ctas;
    return CMDG_OK;
}

extern "C" int cmdg_model_autotune(cmdg_model* model, int reps, double* h_ms, int h_ms_len, int* n_candidates,
                                   void* stream) {
    using namespace cmdg;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    CMDG_ARG_CHECK(reps >= 1 && reps <= 10000, "reps must be in [1, 10000]");
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    const bool mixed = md->precision == CMDG_MIXED;
    const size_t n = (size_t)m.nelem * NSTATE * m.Np;
    const size_t elt = mixed ? sizeof(float) : sizeof(double);
    cudaStream_t s = (cudaStream_t)stream;

    // a physically valid scratch state: the reference state (zero perturbation)
    std::vector<unsigned char> host(n * elt, 0);
    if (!mixed) {
        double* h = reinterpret_cast<double*>(host.data());
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int node = 0; node < m.Np; ++node) {
                const int lev = m.nbr[(size_t)e * NBR_STRIDE + 6] * m.Nq + node / m.Nfp;
                const double* L = &md->lvl64[(size_t)lev * LV_NFIELDS];
                const bool ref = md->prm.ref_state != 0;
                h[((size_t)e * NSTATE + 0) * m.Np + node] = ref ? L[LV_RHO_REF] : 1.0;
                h[((size_t)e * NSTATE + 4) * m.Np + node] = ref ? L[LV_RHOE_REF] : 2.5e5;
            }
    }
    void *Qa = nullptr, *Qb = nullptr;
    double* dQ = nullptr;
    int rc = CMDG_OK;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    const int saved_kind = md->kernel_kind, saved_grid = md->grid_ctas;
    std::vector<Candidate> cands = {{KERNEL_NODE, 0}, {KERNEL_NODE, -1}, {KERNEL_LINES, -1}};
    // one kernel family for viscous models and for curvilinear meshes
    if (md->prm.turbulence != CMDG_TURB_NONE || md->prm.hyperdiffusion != CMDG_HYPER_NONE || m.kind != MESH_BRICK)
        cands = {{KERNEL_NODE, -1}};
    else {
        if (mixed && m.N >= 3 && m.N <= 5) cands.push_back({KERNEL_COLUMN, 0});
        // thread-block clusters of adjacent elements, where the element counts allow them
        const int nx = m.desc.ne[0], ny = m.desc.ne[1], nz = m.desc.ne[2];
        if (nz % 2 == 0) {
            cands.push_back({KERNEL_CLUSTER, 2});
            if (nx % 2 == 0) cands.push_back({KERNEL_CLUSTER, 4});
            if (nx % 2 == 0 && ny % 2 == 0) cands.push_back({KERNEL_CLUSTER, 8});
        }
    }
    std::vector<double> ms(cands.size(), 0.0);
    auto fail = [&](cudaError_t e, const char* what) {
        set_error("autotune: %s: %s", what, cudaGetErrorString(e));
        rc = CMDG_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&Qa, n * elt)) != cudaSuccess) fail(e, "allocation");
    if (!rc && (e = cudaMalloc(&Qb, n * elt)) != cudaSuccess) fail(e, "allocation");
    if (!rc && (e = cudaMalloc((void**)&dQ, n * sizeof(double))) != cudaSuccess) fail(e, "allocation");
    if (!rc && (e = cudaMemcpy(Qa, host.data(), n * elt, cudaMemcpyHostToDevice)) != cudaSuccess) fail(e, "copy");
    if (!rc && (e = cudaMemset(dQ, 0, n * sizeof(double))) != cudaSuccess) fail(e, "memset");
    if (!rc && (e = cudaEventCreate(&t0)) != cudaSuccess) fail(e, "event");
    if (!rc && (e = cudaEventCreate(&t1)) != cudaSuccess) fail(e, "event");
    for (size_t ci = 0; ci < cands.size() && !rc; ++ci) {
        if (cands[ci].kind == KERNEL_CLUSTER && (rc = build_cluster_map(md, cands[ci].grid))) break;
        md->kernel_kind = cands[ci].kind;
        md->grid_ctas = cands[ci].grid;
        LaunchArgs a;
        a.dQ = dQ;
        a.alpha = a.beta = 1.0;
        a.rka = 0.5;
        a.rkb_dt = 0.0;  // the scratch state does not change
        a.mode = 1;
        a.first_stage = 0;
        a.last_stage = 0;
        for (int r = -2; r < reps && !rc; ++r) {
            if (r == 0 && (e = cudaEventRecord(t0, s)) != cudaSuccess) fail(e, "event record");
            a.Qin = (r & 1) ? Qb : Qa;
            a.Qout = (r & 1) ? Qa : Qb;
            rc = launch_stage(md, a, s);
        }
        if (rc) break;
        if ((e = cudaEventRecord(t1, s)) != cudaSuccess) { fail(e, "event record"); break; }
        if ((e = cudaEventSynchronize(t1)) != cudaSuccess) { fail(e, "event sync"); break; }
        float elapsed = 0;
        cudaEventElapsedTime(&elapsed, t0, t1);
        ms[ci] = elapsed / reps;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (Qa) cudaFree(Qa);
    if (Qb) cudaFree(Qb);
    if (dQ) cudaFree(dQ);
    if (rc) {
        md->kernel_kind = saved_kind;
        md->grid_ctas = saved_grid;
        return rc;
    }
    size_t best = 0;
    for (size_t ci = 1; ci < cands.size(); ++ci)
        if (ms[ci] < ms[best]) best = ci;
    if (cands[best].kind == KERNEL_CLUSTER && (rc = build_cluster_map(md, cands[best].grid))) {
        md->kernel_kind = saved_kind;
        md->grid_ctas = saved_grid;
        return rc;
    }
    md->kernel_kind = cands[best].kind;
    md->grid_ctas = cands[best].grid;
    for (auto& kv : md->graphs) cudaGraphExecDestroy(kv.second);
    md->graphs.clear();
    if (n_candidates) *n_candidates = (int)cands.size();
    for (int i = 0; h_ms && i < h_ms_len && i < (int)cands.size(); ++i) h_ms[i] = ms[i];
    // the scratch runs may have flagged nothing; clear the word anyway
    cudaMemsetAsync(md->d_status, 0, sizeof(unsigned), s);
    return CMDG_OK;
}
