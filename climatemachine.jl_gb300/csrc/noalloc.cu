// Allocation-free LSRK54 stepping.
//
// cmdg_lsrk54_step needs two state-sized stage buffers and allocates them
// with cudaMalloc on its first call.  Some callers cannot allow that: a host
// whose memory-pool or arena allocator owns all of the device's memory (a
// cudaMalloc from the library would fail or fragment the arena), and hosts
// that forbid any allocation after start-up.  cmdg_lsrk54_step_noalloc serves
// them: the two stage buffers live in one file-scope __device__ array whose
// size is fixed when the library is loaded, so a call allocates nothing.
//
// The array is CMDG_NOALLOC_MAX_BYTES (48 MiB) on every GPU that loads the
// library, held until the process exits; a state of up to half of it
// (24 MiB) can be stepped.  Every call shares the array: the stage buffers
// are written in full by each stage before any stage reads them, so nothing
// in it has to start at zero, but two calls whose kernels overlap on the GPU
// (on different streams, or from different threads) race on it.
#include <mutex>

#include "cmdg_internal.h"

namespace {

constexpr size_t NOALLOC_MAX_BYTES = (size_t)48 << 20;
constexpr size_t NOALLOC_ALIGN = 256;
constexpr int MAX_DEVICES = 64;

// Both stage buffers.  In host code this name is only a handle for
// cudaGetSymbolAddress, never a device address.
__device__ __align__(256) unsigned char g_noalloc_stage[NOALLOC_MAX_BYTES];

void* g_stage_addr[MAX_DEVICES] = {};
std::mutex g_stage_mutex;

// Device address of g_noalloc_stage on the current device, looked up once
// per device (the first call on a device does this set-up).
int stage_address(void** out) {
    int dev = 0;
    CMDG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) {
        cmdg::set_error("device ordinal %d is beyond the %d devices the allocation-free path tracks", dev,
                        MAX_DEVICES);
        return CMDG_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    if (g_stage_addr[dev] == nullptr) {
        void* p = nullptr;
        CMDG_CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_stage));
        g_stage_addr[dev] = p;
    }
    *out = g_stage_addr[dev];
    return CMDG_OK;
}

}  // namespace

extern "C" int cmdg_lsrk54_step_noalloc(cmdg_model* model, void* d_Q, double* d_dQ, double t, double dt, int nsteps,
                                        void* stream) {
    (void)t;
    using namespace cmdg;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    CMDG_ARG_CHECK(d_Q != nullptr && d_dQ != nullptr, "NULL state");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    CMDG_ARG_CHECK(dt > 0 && dt < 1e300, "dt must be positive and finite");
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    const size_t elt = md->precision == CMDG_MIXED ? sizeof(float) : sizeof(double);
    const size_t bytes = (size_t)m.nelem * NSTATE * m.Np * elt;
    const size_t slot = (bytes + NOALLOC_ALIGN - 1) / NOALLOC_ALIGN * NOALLOC_ALIGN;
    CMDG_ARG_CHECK(2 * slot <= NOALLOC_MAX_BYTES,
                   "state of %zu bytes exceeds the allocation-free limit of %zu bytes per stage buffer "
                   "(two buffers in a fixed %zu-byte device array); use cmdg_lsrk54_step",
                   bytes, NOALLOC_MAX_BYTES / 2, NOALLOC_MAX_BYTES);
    if (nsteps == 0) return CMDG_OK;
    void* base = nullptr;
    int rc = stage_address(&base);
    if (rc) return rc;
    char* S1 = static_cast<char*>(base);
    char* S2 = S1 + slot;
    const double *A, *B;
    lsrk54_coefficients(&A, &B);
    void* const order[6] = {d_Q, S1, S2, S1, S2, d_Q};
    for (int step = 0; step < nsteps; ++step) {
        for (int st = 0; st < 5; ++st) {
            LaunchArgs a;
            a.Qin = order[st];
            a.Qout = order[st + 1];
            a.dQ = d_dQ;
            a.alpha = 1.0;
            a.beta = 1.0;
            a.rka = A[st];
            a.rkb_dt = B[st] * dt;
            a.mode = 1;
            a.first_stage = (st == 0);
            a.last_stage = (st == 4);
            rc = launch_stage(md, a, (cudaStream_t)stream);
            if (rc) return rc;
        }
    }
    return CMDG_OK;
}
