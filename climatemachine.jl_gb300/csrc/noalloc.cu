// Allocation-free LSRK54 stepping.
//
// cmdg_lsrk54_step needs two state-sized stage buffers and allocates them
// with cudaMalloc on its first call.  Some callers cannot allow that: a host
// whose memory-pool or arena allocator owns all of the device's memory (a
// cudaMalloc from the library would fail or fragment the arena), and hosts
// that forbid any allocation after start-up.  cmdg_lsrk54_step_noalloc serves
// them: the two stage buffers live in one file-scope __device__ array of a
// fixed size, so a call allocates nothing.
//
// The array is CMDG_NOALLOC_MAX_BYTES (48 MiB) on every GPU where a model is
// created, held until the process exits; a state of up to half of it
// (24 MiB) can be stepped.  The CUDA runtime loads this file's module, and
// with it reserves the array, when its symbol is first looked up; that
// look-up is part of model creation (cmdg_model_create, which allocates
// anyway), so the array is reserved before the host hands its memory to an
// arena, and the allocation-free call itself reserves nothing.  Every call
// shares the array: the stage buffers are written in full by each stage
// before any stage reads them, so nothing in it has to start at zero, but two
// calls whose kernels overlap on the GPU (on different streams, or from
// different threads) race on it.
#include "cmdg_internal.h"

namespace {

constexpr size_t NOALLOC_MAX_BYTES = (size_t)48 << 20;
constexpr size_t NOALLOC_ALIGN = 256;

// Both stage buffers.  In host code this name is only a handle for
// cudaGetSymbolAddress, never a device address.
__device__ __align__(256) unsigned char g_noalloc_stage[NOALLOC_MAX_BYTES];

}  // namespace

namespace cmdg {

// Set-up, with the model's device current: the device address of the array.
// A model created after a device reset looks it up again, so no address
// outlives the context it belongs to longer than the models of that context.
int noalloc_stage_address(void** out) {
    void* p = nullptr;
    CMDG_CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_stage));
    *out = p;
    return CMDG_OK;
}

}  // namespace cmdg

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
    int rc = check_fused_stepping(md);
    if (rc) return rc;
    int dev = -1;
    CMDG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev != md->device || md->noalloc_stage == nullptr) {
        set_error("the model was created on device %d; make it current (now %d) before stepping", md->device, dev);
        return CMDG_ERR_STATE;
    }
    if (nsteps == 0) return CMDG_OK;
    char* S1 = static_cast<char*>(md->noalloc_stage);
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
