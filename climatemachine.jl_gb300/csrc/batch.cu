// Ensembles of models advanced together, by one of two kernel families:
//   per order  the members are grouped by polynomial order; each LSRK54
//              stage of a group is one launch of the tile-walking node kernel
//              of that order (stage.cu), so members of uneven size share the
//              GPU without a launch per member.  Members are independent, so
//              the groups' stage chains run on their own streams: captured as
//              one CUDA graph they are three independent branches that the
//              GPU overlaps, joined at the end of the call;
//   persistent one launch per stage of the line kernel (stage_lines.cu) over
//              one list of tiles of every order, with one CTA shape for all
//              orders: its size sets the elements per CTA pass and the nodes
//              per thread of each order.
// cmdg_batch_autotune times both families over their tilings (elements per
// tile, grid, and the persistent kernel's CTA size) and keeps the fastest.
//
// Members with a turbulence closure (the LES members of a viscous ensemble)
// take the gradient pass and the viscous stage kernel at every stage; their
// stage chains, one launch pair per member and stage, run on a fourth branch
// of the same graph.
//
// There is no counterpart in the reference, which advances one DGModel per
// solver (ensembles there are separate runs).
#include <algorithm>
#include <cstring>
#include <vector>

#include "dg_common.cuh"

namespace cmdg {

constexpr int BATCH_NMIN = 3, BATCH_NMAX = 5, BATCH_NGROUPS = BATCH_NMAX - BATCH_NMIN + 1;

struct Group {
    int N = 0;
    int tile_elems = 1;
    int grid = -1;                  // -1 = one CTA per tile, 0 = one wave of resident CTAs, n > 0 = n CTAs
    BatchTile* d_tiles = nullptr;
    int ntiles = 0;
    cudaStream_t stream = nullptr;  // side stream of the group's stage chain
    cudaEvent_t join = nullptr;
};

enum { FAMILY_PER_ORDER = 0, FAMILY_PERSISTENT = 1 };

// the persistent line kernel's tiling: every inviscid member's elements
struct Unified {
    int cta_threads = 128;          // 128 or 256
    int tile_elems = 2;
    int grid = 0;                   // -1 = one CTA per tile, 0 = one wave of resident CTAs, n > 0 = n CTAs
    BatchTile* d_tiles = nullptr;
    int ntiles = 0;
    EnsDhat dhat;                   // Dhat of the orders 3, 4, 5 in FP32
};

struct Batch {
    std::vector<Model*> members;
    int family = FAMILY_PER_ORDER;
    Unified uni;
    std::vector<void*> scratch;     // two stage buffers per member (one allocation each)
    std::vector<size_t> state_bytes;
    KParams* d_params = nullptr;    // [5 stages][members]
    Group groups[BATCH_NGROUPS];
    // members with a turbulence closure, stepped member by member on their own branch
    std::vector<int> viscous;
    cudaStream_t visc_stream = nullptr;
    cudaEvent_t visc_join = nullptr;
    cudaEvent_t fork = nullptr;
    // the parameters currently on the device
    std::vector<const void*> cur_Q;
    std::vector<const void*> cur_dQ;
    std::vector<double> cur_dt;
    cudaGraphExec_t graph = nullptr;
    int graph_nsteps = 0;
    void* graph_stream = nullptr;
};

static void drop_graph(Batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

// Tiles of one order: members interleaved, tile_elems consecutive elements each.
static int build_tiles(Batch* b, Group& g) {
    std::vector<BatchTile> tiles;
    std::vector<int64_t> pos(b->members.size(), 0);
    bool more = true;
    while (more) {
        more = false;
        for (size_t m = 0; m < b->members.size(); ++m) {
            const Mesh& mesh = *b->members[m]->mesh;
            if (mesh.N != g.N || pos[m] >= mesh.nelem || b->members[m]->prm.turbulence != CMDG_TURB_NONE) continue;
            const int64_t e1 = std::min<int64_t>(mesh.nelem, pos[m] + g.tile_elems);
            tiles.push_back(BatchTile{(int)m, (int)pos[m], (int)e1, mesh.N});
            pos[m] = e1;
            more = true;
        }
    }
    if (g.d_tiles) cudaFree(g.d_tiles);
    g.d_tiles = nullptr;
    g.ntiles = 0;
    if (tiles.empty()) return CMDG_OK;
    CMDG_CUDA_CHECK(cudaMalloc(&g.d_tiles, sizeof(BatchTile) * tiles.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(g.d_tiles, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice));
    g.ntiles = (int)tiles.size();
    return CMDG_OK;
}

// Tiles of every order for the persistent kernel: members interleaved,
// tile_elems consecutive elements each, the largest orders first.
static int build_unified_tiles(Batch* b) {
    Unified& u = b->uni;
    std::vector<BatchTile> tiles;
    for (int N = BATCH_NMAX; N >= BATCH_NMIN; --N) {
        std::vector<int64_t> pos(b->members.size(), 0);
        bool more = true;
        while (more) {
            more = false;
            for (size_t m = 0; m < b->members.size(); ++m) {
                const Mesh& mesh = *b->members[m]->mesh;
                if (mesh.N != N || pos[m] >= mesh.nelem || b->members[m]->prm.turbulence != CMDG_TURB_NONE) continue;
                const int64_t e1 = std::min<int64_t>(mesh.nelem, pos[m] + u.tile_elems);
                tiles.push_back(BatchTile{(int)m, (int)pos[m], (int)e1, N});
                pos[m] = e1;
                more = true;
            }
        }
    }
    if (u.d_tiles) cudaFree(u.d_tiles);
    u.d_tiles = nullptr;
    u.ntiles = 0;
    if (tiles.empty()) return CMDG_OK;
    CMDG_CUDA_CHECK(cudaMalloc(&u.d_tiles, sizeof(BatchTile) * tiles.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(u.d_tiles, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice));
    u.ntiles = (int)tiles.size();
    return CMDG_OK;
}

static int unified_grid(const Unified& u) {
    int grid = u.grid > 0 ? u.grid : u.grid == 0 ? ens_lines_resident_ctas(u.cta_threads) : u.ntiles;
    if (grid <= 0) grid = 1;
    return std::min(grid, u.ntiles);
}

static void build_dhat(EnsDhat& d) {
    float* rows[3] = {d.d3, d.d4, d.d5};
    for (int N = BATCH_NMIN; N <= BATCH_NMAX; ++N) {
        Mesh m;
        m.N = N;
        m.Nq = N + 1;
        lgl_derivative(&m);
        for (int i = 0; i < m.Nq * m.Nq; ++i) rows[N - BATCH_NMIN][i] = (float)m.Dhat[i];
    }
}

static int grid_of(const Group& g) {
    int grid = g.grid > 0 ? g.grid : g.grid == 0 ? batch_resident_ctas(g.N) : g.ntiles;
    if (grid <= 0) grid = 1;
    return std::min(grid, g.ntiles);
}

// Uploads the per-stage launch parameters of every member when the state
// pointers or time steps differ from the ones on the device.
static int upload_params(Batch* b, void* const* Q, double* const* dQ, const double* dt, bool force) {
    const size_t n = b->members.size();
    bool same = !force && b->cur_Q.size() == n;
    for (size_t m = 0; same && m < n; ++m)
        same = b->cur_Q[m] == Q[m] && b->cur_dQ[m] == dQ[m] && b->cur_dt[m] == dt[m];
    if (same) return CMDG_OK;
    const double *A, *B;
    lsrk54_coefficients(&A, &B);
    std::vector<KParams> host(5 * n);
    for (size_t m = 0; m < n; ++m) {
        char* S1 = static_cast<char*>(b->scratch[m]);
        char* S2 = S1 + b->state_bytes[m];
        void* const order[6] = {Q[m], S1, S2, S1, S2, Q[m]};
        for (int st = 0; st < 5; ++st) {
            LaunchArgs a;
            a.Qin = order[st];
            a.Qout = order[st + 1];
            a.dQ = dQ[m];
            a.alpha = a.beta = 1.0;
            a.rka = A[st];
            a.rkb_dt = B[st] * dt[m];
            a.mode = 1;
            a.first_stage = st == 0;
            a.last_stage = st == 4;
            host[st * n + m] = make_params(b->members[m], a);
        }
    }
    CMDG_CUDA_CHECK(cudaMemcpy(b->d_params, host.data(), sizeof(KParams) * host.size(), cudaMemcpyHostToDevice));
    b->cur_Q.assign(Q, Q + n);
    b->cur_dQ.assign(dQ, dQ + n);
    b->cur_dt.assign(dt, dt + n);
    drop_graph(b);
    return CMDG_OK;
}

static int launch_error(cudaError_t e) {
    set_error("ensemble stage launch failed: %s", cudaGetErrorString(e));
    return CMDG_ERR_CUDA;
}

// nsteps steps of every group: the first non-empty group on s, the others on
// their side streams, forked from and joined back into s.
static int issue(Batch* b, int nsteps, cudaStream_t s) {
    const size_t n = b->members.size();
    bool first = true;
    cudaError_t e = cudaEventRecord(b->fork, s);
    if (e != cudaSuccess) return launch_error(e);
    std::vector<Group*> joined;
    if (b->family == FAMILY_PERSISTENT && b->uni.ntiles) {
        const int grid = unified_grid(b->uni);
        for (int step = 0; step < nsteps; ++step)
            for (int st = 0; st < 5; ++st)
                if ((e = launch_ens_lines(b->d_params + st * n, b->uni.d_tiles, b->uni.ntiles, b->uni.cta_threads,
                                          grid, b->uni.dhat, s)) != cudaSuccess)
                    return launch_error(e);
        first = false;
    }
    for (Group& g : b->groups) {
        if (!g.ntiles || b->family != FAMILY_PER_ORDER) continue;
        cudaStream_t gs = first ? s : g.stream;
        if (!first) {
            if ((e = cudaStreamWaitEvent(gs, b->fork, 0)) != cudaSuccess) return launch_error(e);
            joined.push_back(&g);
        }
        first = false;
        const int grid = grid_of(g);
        for (int step = 0; step < nsteps; ++step)
            for (int st = 0; st < 5; ++st)
                if ((e = launch_batch_stage(b->d_params + st * n, g.d_tiles, g.ntiles, g.N, grid, gs)) != cudaSuccess)
                    return launch_error(e);
    }
    if (!b->viscous.empty()) {
        cudaStream_t vs = first ? s : b->visc_stream;
        if (!first && (e = cudaStreamWaitEvent(vs, b->fork, 0)) != cudaSuccess) return launch_error(e);
        const double *A, *B;
        lsrk54_coefficients(&A, &B);
        for (int step = 0; step < nsteps; ++step)
            for (int st = 0; st < 5; ++st)
                for (int m : b->viscous) {
                    char* S1 = static_cast<char*>(b->scratch[m]);
                    char* S2 = S1 + b->state_bytes[m];
                    void* Q = const_cast<void*>(b->cur_Q[m]);
                    void* const order[6] = {Q, S1, S2, S1, S2, Q};
                    LaunchArgs a;
                    a.Qin = order[st];
                    a.Qout = order[st + 1];
                    a.dQ = const_cast<double*>(static_cast<const double*>(b->cur_dQ[m]));
                    a.alpha = a.beta = 1.0;
                    a.rka = A[st];
                    a.rkb_dt = B[st] * b->cur_dt[m];
                    a.mode = 1;
                    a.first_stage = st == 0;
                    a.last_stage = st == 4;
                    const int rc = launch_stage(b->members[m], a, vs);
                    if (rc) return rc;
                }
        if (!first) {
            if ((e = cudaEventRecord(b->visc_join, vs)) != cudaSuccess) return launch_error(e);
            if ((e = cudaStreamWaitEvent(s, b->visc_join, 0)) != cudaSuccess) return launch_error(e);
        }
    }
    for (Group* g : joined) {
        if ((e = cudaEventRecord(g->join, g->stream)) != cudaSuccess) return launch_error(e);
        if ((e = cudaStreamWaitEvent(s, g->join, 0)) != cudaSuccess) return launch_error(e);
    }
    return CMDG_OK;
}

static void release(Batch* b) {
    for (void* p : b->scratch) cudaFree(p);
    if (b->d_params) cudaFree(b->d_params);
    for (Group& g : b->groups) {
        if (g.d_tiles) cudaFree(g.d_tiles);
        if (g.stream) cudaStreamDestroy(g.stream);
        if (g.join) cudaEventDestroy(g.join);
    }
    if (b->uni.d_tiles) cudaFree(b->uni.d_tiles);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->visc_stream) cudaStreamDestroy(b->visc_stream);
    if (b->visc_join) cudaEventDestroy(b->visc_join);
    drop_graph(b);
    delete b;
}

}  // namespace cmdg

struct cmdg_batch {
    cmdg::Batch* b;
};

using namespace cmdg;

extern "C" int cmdg_batch_create(cmdg_model* const* models, int n, cmdg_batch** out) {
    CMDG_ARG_CHECK(out != nullptr, "output pointer is NULL");
    *out = nullptr;
    CMDG_ARG_CHECK(models != nullptr && n > 0, "need at least one member");
    for (int m = 0; m < n; ++m) {
        CMDG_ARG_CHECK(models[m] != nullptr, "member %d is NULL", m);
        const Model& md = models[m]->m;
        CMDG_ARG_CHECK(md.precision == CMDG_MIXED, "member %d: ensembles run the mixed-precision path", m);
        CMDG_ARG_CHECK(md.mesh->N >= BATCH_NMIN && md.mesh->N <= BATCH_NMAX,
                       "member %d: N=%d outside the ensemble range [3, 5]", m, md.mesh->N);
        CMDG_ARG_CHECK(md.prm.hyperdiffusion == CMDG_HYPER_NONE, "member %d: ensembles run without hyperdiffusion",
                       m);
        CMDG_ARG_CHECK(md.mesh->kind == MESH_BRICK, "member %d: ensembles run on brick meshes", m);
    }
    Batch* b = new Batch();
    for (int m = 0; m < n; ++m) {
        b->members.push_back(&models[m]->m);
        if (models[m]->m.prm.turbulence != CMDG_TURB_NONE) b->viscous.push_back(m);
    }
    int rc = CMDG_OK;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        set_error("ensemble %s failed: %s", what, cudaGetErrorString(e));
        rc = e == cudaErrorMemoryAllocation ? CMDG_ERR_ALLOC : CMDG_ERR_CUDA;
    };
    for (int m = 0; m < n && !rc; ++m) {
        const Mesh& mesh = *b->members[m]->mesh;
        const size_t bytes = ((size_t)mesh.nelem * NSTATE * mesh.Np * sizeof(float) + 255) / 256 * 256;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, 2 * bytes);
        if (e != cudaSuccess) {
            cuda_fail(e, "scratch allocation");
            break;
        }
        b->scratch.push_back(p);
        b->state_bytes.push_back(bytes);
    }
    cudaError_t e;
    if (!rc && (e = cudaMalloc(&b->d_params, sizeof(KParams) * 5 * n)) != cudaSuccess) cuda_fail(e, "allocation");
    if (!rc && (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) cuda_fail(e, "event");
    if (!rc && (e = cudaStreamCreateWithFlags(&b->visc_stream, cudaStreamNonBlocking)) != cudaSuccess)
        cuda_fail(e, "stream");
    if (!rc && (e = cudaEventCreateWithFlags(&b->visc_join, cudaEventDisableTiming)) != cudaSuccess)
        cuda_fail(e, "event");
    for (int gi = 0; gi < BATCH_NGROUPS && !rc; ++gi) {
        Group& g = b->groups[gi];
        g.N = BATCH_NMIN + gi;
        if ((e = cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking)) != cudaSuccess) cuda_fail(e, "stream");
        if (!rc && (e = cudaEventCreateWithFlags(&g.join, cudaEventDisableTiming)) != cudaSuccess)
            cuda_fail(e, "event");
        if (!rc) rc = build_tiles(b, g);
    }
    if (!rc) {
        build_dhat(b->uni.dhat);
        rc = build_unified_tiles(b);
    }
    if (rc) {
        release(b);
        return rc;
    }
    *out = new cmdg_batch{b};
    return CMDG_OK;
}

extern "C" int cmdg_batch_set_kernel(cmdg_batch* batch, int family, int cta_threads, int tile_elems, int grid_ctas) {
    CMDG_ARG_CHECK(batch != nullptr, "batch is NULL");
    CMDG_ARG_CHECK(family == FAMILY_PER_ORDER || family == FAMILY_PERSISTENT, "unknown ensemble kernel family %d",
                   family);
    Batch* b = batch->b;
    drop_graph(b);
    b->family = family;
    if (family == FAMILY_PERSISTENT) {
        CMDG_ARG_CHECK(cta_threads == 128 || cta_threads == 256, "cta_threads must be 128 or 256");
        CMDG_ARG_CHECK(tile_elems >= 1 && tile_elems <= 4096, "tile_elems must be in [1, 4096]");
        CMDG_ARG_CHECK(grid_ctas >= -1, "grid_ctas must be >= -1");
        Unified& u = b->uni;
        u.cta_threads = cta_threads;
        u.grid = grid_ctas;
        if (tile_elems != u.tile_elems) {
            u.tile_elems = tile_elems;
            return build_unified_tiles(b);
        }
    }
    return CMDG_OK;
}

extern "C" int cmdg_batch_get_kernel(const cmdg_batch* batch, int* family, int* cta_threads, int* tile_elems,
                                     int* grid_ctas) {
    CMDG_ARG_CHECK(batch != nullptr, "batch is NULL");
    const Batch* b = batch->b;
    if (family) *family = b->family;
    if (cta_threads) *cta_threads = b->uni.cta_threads;
    if (tile_elems) *tile_elems = b->uni.tile_elems;
    if (grid_ctas) *grid_ctas = b->uni.grid;
    return CMDG_OK;
}

extern "C" int cmdg_batch_destroy(cmdg_batch* batch) {
    if (!batch) return CMDG_OK;
    release(batch->b);
    delete batch;
    return CMDG_OK;
}

extern "C" int cmdg_batch_set_tiling(cmdg_batch* batch, int N, int tile_elems, int grid_ctas) {
    CMDG_ARG_CHECK(batch != nullptr, "batch is NULL");
    CMDG_ARG_CHECK(N == 0 || (N >= BATCH_NMIN && N <= BATCH_NMAX), "N must be 0 (all orders) or in [3, 5]");
    CMDG_ARG_CHECK(tile_elems >= 1 && tile_elems <= 4096, "tile_elems must be in [1, 4096]");
    CMDG_ARG_CHECK(grid_ctas >= -1, "grid_ctas must be >= -1");
    Batch* b = batch->b;
    drop_graph(b);
    for (Group& g : b->groups) {
        if (N && g.N != N) continue;
        g.grid = grid_ctas;
        if (tile_elems != g.tile_elems) {
            g.tile_elems = tile_elems;
            int rc = build_tiles(b, g);
            if (rc) return rc;
        }
    }
    return CMDG_OK;
}

extern "C" int cmdg_batch_get_tiling(const cmdg_batch* batch, int N, int* tile_elems, int* grid_ctas) {
    CMDG_ARG_CHECK(batch != nullptr, "batch is NULL");
    CMDG_ARG_CHECK(N >= BATCH_NMIN && N <= BATCH_NMAX, "N must be in [3, 5]");
    const Group& g = batch->b->groups[N - BATCH_NMIN];
    if (tile_elems) *tile_elems = g.tile_elems;
    if (grid_ctas) *grid_ctas = g.grid;
    return CMDG_OK;
}

extern "C" int cmdg_batch_lsrk54_step(cmdg_batch* batch, void* const* h_Q, double* const* h_dQ, const double* h_dt,
                                      int nsteps, void* stream) {
    CMDG_ARG_CHECK(batch != nullptr && h_Q != nullptr && h_dQ != nullptr && h_dt != nullptr, "NULL argument");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    Batch* b = batch->b;
    for (size_t m = 0; m < b->members.size(); ++m) {
        CMDG_ARG_CHECK(h_Q[m] != nullptr && h_dQ[m] != nullptr, "member %zu: NULL state", m);
        CMDG_ARG_CHECK(h_dt[m] > 0 && h_dt[m] < 1e300, "member %zu: dt must be positive and finite", m);
    }
    if (nsteps == 0) return CMDG_OK;
    int rc = upload_params(b, h_Q, h_dQ, h_dt, false);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (s == nullptr || nsteps > 64) return issue(b, nsteps, s);
    if (!b->graph || b->graph_nsteps != nsteps || b->graph_stream != stream) {
        drop_graph(b);
        cudaGraph_t g;
        CMDG_CUDA_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        rc = issue(b, nsteps, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) {
            set_error("ensemble graph capture failed: %s", cudaGetErrorString(ce));
            return CMDG_ERR_CUDA;
        }
        ce = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            b->graph = nullptr;
            set_error("ensemble graph instantiate failed: %s", cudaGetErrorString(ce));
            return CMDG_ERR_CUDA;
        }
        b->graph_nsteps = nsteps;
        b->graph_stream = stream;
    }
    CMDG_CUDA_CHECK(cudaGraphLaunch(b->graph, s));
    return CMDG_OK;
}

// One stage launch of the per-order family, every group on its branch as in
// issue(), with the parameters of stage index 1.
static cudaError_t per_order_stage(Batch* b, cudaStream_t s) {
    const size_t n = b->members.size();
    cudaError_t e = cudaEventRecord(b->fork, s);
    if (e != cudaSuccess) return e;
    bool first = true;
    std::vector<Group*> joined;
    for (Group& g : b->groups) {
        if (!g.ntiles) continue;
        cudaStream_t gs = first ? s : g.stream;
        if (!first) {
            if ((e = cudaStreamWaitEvent(gs, b->fork, 0)) != cudaSuccess) return e;
            joined.push_back(&g);
        }
        first = false;
        if ((e = launch_batch_stage(b->d_params + n, g.d_tiles, g.ntiles, g.N, grid_of(g), gs)) != cudaSuccess)
            return e;
    }
    for (Group* g : joined) {
        if ((e = cudaEventRecord(g->join, g->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s, g->join, 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Autotuner.  On stage launches that leave the members' states unchanged
// (B dt = 0 on copies of the states; the RK register is overwritten, which
// the next step ignores because stage 1 does not read it) it times
//   the per-order family: for each order tile_elems in {1, 2, 4, 8, 16} x
//   grid in {one CTA per tile, one wave of resident CTAs}, keeping each
//   order's fastest, then the whole family (every order's launch on its
//   branch);
//   the persistent family: CTA size in {128, 256} threads (elements per CTA
//   pass and nodes per thread of each order follow from it) x tile_elems in
//   {1, 2, 4, 8} x grid in {one CTA per tile, one wave of resident CTAs};
// and keeps the faster family with its fastest tiling.  h_ms receives ms per
// stage launch: [order 3, 4, 5][10 per-order candidates] (0 for an order
// without members), then the 16 persistent candidates, then the whole
// per-order family; n_candidates = 47.
extern "C" int cmdg_batch_autotune(cmdg_batch* batch, void* const* h_Q, double* const* h_dQ, int reps, double* h_ms,
                                   int h_ms_len, int* n_candidates, void* stream) {
    CMDG_ARG_CHECK(batch != nullptr && h_Q != nullptr && h_dQ != nullptr, "NULL argument");
    CMDG_ARG_CHECK(reps >= 1 && reps <= 1000, "reps must be in [1, 1000]");
    Batch* b = batch->b;
    const size_t n = b->members.size();
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<double> unit_dt(n, 1.0);
    int rc = upload_params(b, h_Q, h_dQ, unit_dt.data(), true);
    if (rc) return rc;
    {
        std::vector<KParams> host(n);
        CMDG_CUDA_CHECK(cudaMemcpy(host.data(), b->d_params + n, sizeof(KParams) * n, cudaMemcpyDeviceToHost));
        for (auto& P : host) {
            P.rkb_dt = 0.0;
            P.rkb_dt32 = 0.0f;
        }
        CMDG_CUDA_CHECK(cudaMemcpy(b->d_params + n, host.data(), sizeof(KParams) * n, cudaMemcpyHostToDevice));
        for (size_t m = 0; m < n; ++m)
            CMDG_CUDA_CHECK(cudaMemcpyAsync(b->scratch[m], h_Q[m], b->state_bytes[m], cudaMemcpyDeviceToDevice, s));
    }
    const int tiles[5] = {1, 2, 4, 8, 16};
    const int grids[2] = {-1, 0};
    constexpr int NC = 10, NU = 16, NTOT = BATCH_NGROUPS * NC + NU + 1;
    std::vector<double> ms(NTOT, 0.0);
    cudaEvent_t t0, t1;
    CMDG_CUDA_CHECK(cudaEventCreate(&t0));
    CMDG_CUDA_CHECK(cudaEventCreate(&t1));
    // times `reps` launches of fn (after one untimed launch), in ms per launch
    auto time_it = [&](auto fn, double& out) -> int {
        cudaError_t e = cudaSuccess;
        for (int r = -1; r < reps && e == cudaSuccess; ++r) {
            if (r == 0) cudaEventRecord(t0, s);
            e = fn();
        }
        cudaEventRecord(t1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(t1);
        if (e != cudaSuccess) return launch_error(e);
        float el = 0;
        cudaEventElapsedTime(&el, t0, t1);
        out = el / reps;
        return CMDG_OK;
    };
    for (int gi = 0; gi < BATCH_NGROUPS && !rc; ++gi) {
        Group& g = b->groups[gi];
        if (!g.ntiles) continue;
        int best_tile = g.tile_elems, best_grid = g.grid;
        double best = 1e300;
        for (int c = 0; c < NC && !rc; ++c) {
            g.tile_elems = tiles[c / 2];
            g.grid = grids[c % 2];
            if ((rc = build_tiles(b, g))) break;
            const int grid = grid_of(g);
            rc = time_it([&] { return launch_batch_stage(b->d_params + n, g.d_tiles, g.ntiles, g.N, grid, s); },
                         ms[gi * NC + c]);
            if (!rc && ms[gi * NC + c] < best) {
                best = ms[gi * NC + c];
                best_tile = g.tile_elems;
                best_grid = g.grid;
            }
        }
        g.tile_elems = best_tile;
        g.grid = best_grid;
        const int rc2 = build_tiles(b, g);
        if (!rc) rc = rc2;
    }
    double per_order = 0;
    bool any_tiles = false;
    for (const Group& g : b->groups) any_tiles |= g.ntiles > 0;
    if (!rc && any_tiles) {
        rc = time_it([&] { return per_order_stage(b, s); }, ms[BATCH_NGROUPS * NC + NU]);
        per_order = ms[BATCH_NGROUPS * NC + NU];
    }
    // the persistent family
    Unified& u = b->uni;
    const int u_threads[2] = {128, 256}, u_tiles[4] = {1, 2, 4, 8};
    int best_threads = u.cta_threads, best_tile = u.tile_elems, best_grid = u.grid;
    double best_u = 1e300;
    for (int c = 0; c < NU && !rc && u.ntiles; ++c) {
        u.cta_threads = u_threads[c / 8];
        u.tile_elems = u_tiles[(c / 2) % 4];
        u.grid = grids[c % 2];
        if ((rc = build_unified_tiles(b))) break;
        const int grid = unified_grid(u);
        double& out = ms[BATCH_NGROUPS * NC + c];
        rc = time_it([&] { return launch_ens_lines(b->d_params + n, u.d_tiles, u.ntiles, u.cta_threads, grid, u.dhat, s); },
                     out);
        if (!rc && out < best_u) {
            best_u = out;
            best_threads = u.cta_threads;
            best_tile = u.tile_elems;
            best_grid = u.grid;
        }
    }
    u.cta_threads = best_threads;
    u.tile_elems = best_tile;
    u.grid = best_grid;
    const int rc3 = build_unified_tiles(b);
    if (!rc) rc = rc3;
    if (!rc && any_tiles) b->family = (u.ntiles && best_u < per_order) ? FAMILY_PERSISTENT : FAMILY_PER_ORDER;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    b->cur_Q.clear();  // the next step re-uploads its real parameters
    drop_graph(b);
    for (Model* md : b->members) cudaMemsetAsync(md->d_status, 0, sizeof(unsigned), s);
    if (n_candidates) *n_candidates = NTOT;
    for (int i = 0; h_ms && i < h_ms_len && i < (int)ms.size(); ++i) h_ms[i] = ms[i];
    return rc;
}
