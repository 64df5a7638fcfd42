// Device-side building blocks shared by the fused stage kernels: kernel
// parameters, precision-dependent constants, IEEE-754 conversions on the
// integer pipe, per-level reference-state rows, dry-air thermodynamics and
// first-order fluxes of the AtmosModel, and planar shared-memory records.
#pragma once

#include "cmdg_internal.h"

namespace cmdg {

// Arguments of one stage-kernel launch (passed by value: the parameter bank).
struct KParams {
    const void* Qin;
    void* Qout;
    double* dQ;
    const double* emetric;
    const int* nbr;
    const double* lvl64;
    const float* lvl32;
    const float* jump32;
    const void* Dhat;
    unsigned* status;
    int nelem, nz;
    const float* emetric32;
    double alpha, beta, rka, rkb_dt;
    double inv_w0;
    float rkb_dt32, inv_w032, gm132, gamma32;
    int first_stage, last_stage;
    Physics ph;
    // weak-form derivative Dhat[i][n] = D[n][i] w_n / w_i (row-major, N <= MAX_N),
    // in the parameter bank so compile-time indexed reads cost no instruction
    float DhatC32[(MAX_N + 1) * (MAX_N + 1)];
    double DhatC64[(MAX_N + 1) * (MAX_N + 1)];
    // diffusive passes: gradient-flux state, reference rows, strong-form D
    // (D[j][k] = d l_k / d xi at xi_j), FP32 copies of the closure constants
    void* gf;
    const double* lvv64;
    const float* lvv32;
    float DC32[(MAX_N + 1) * (MAX_N + 1)];
    double DC64[(MAX_N + 1) * (MAX_N + 1)];
    float rho_nu32, C_smag32, inv_Pr32, kappa32, MSLP32, grav32;
    // curvilinear meshes: per-node kernel geometry (Np, KG_NFIELDS, nelem) in
    // the working precision
    const void* geo;
    // hyperdiffusion: gradient / hyperdiffusive state (Np, 9, nelem),
    // laplacians (Np, 3, nelem), the FP64-computed z-gradient of the laplacian
    // of the reference h_tot per level (mixed precision) and tau
    void* hd;
    void* hlap;
    const float* glap_ref32;
    double inv_tau_hyper;
    float inv_tau_hyper32;
    // cubed shell: nu_4 per node (working precision) and, mixed, the FP64
    // reference part nu_4 grad lap h_ref per node (Np, 3, nelem)
    const void* nu4;
    const float* hglap_ref32;
    // cubed shell with ConstantDynamicViscosity, mixed: the FP64-computed
    // gradient of the reference h_tot per node (Np, 3, nelem); the viscous
    // gradient pass writes grad u, grad h_tot (Np, 12, nelem) into gf
    const float* vgref32;
    const double* sdelta;  // cubed shell, SmagorinskyLilly: length scale per node (Np, nelem)
    // grid-arrays meshes, FP64 (cmdg_model_set_mms): a source added to the
    // tendency, the InitStateBC wall state, both (Np, 5, nelem) or NULL, and
    // total_specific_enthalpy := 0 in the gradient arguments
    const double* mms_src;
    const double* mms_wall;
    int mms_zero_h;
    int hyper_horizontal;  // 1: the passes run in the horizontal directions only (HorizontalDirection)
    // grid-arrays meshes: facing node of each face node (Nfp, 6, nelem) and
    // the FP64-computed reference jumps (rho, rhoe) per face node
    const int* fpart;
    const float* fjump;
    // bounded waits of the persistent stage kernel: poll limit (0 = default)
    // and the test hook that arms the staging barriers without issuing the
    // copies, so that every wait runs out (cmdg_model_set_staging_test)
    int wait_polls;
    // cluster kernel: the element of each CTA (clusters of adjacent elements)
    const int* cl_elem;
    int staging_skip_copies;
};

// A run of consecutive elements [e0, e1) of ensemble member `member`, of
// polynomial order N.
struct BatchTile {
    int member, e0, e1, N;
};
// Ensemble stage launch over the tiles of one polynomial order N (3..5) with
// `grid` CTAs, and the number of CTAs of that order resident on the device
// (stage.cu).
cudaError_t launch_batch_stage(const KParams* d_params, const BatchTile* d_tiles, int ntiles, int N, int grid,
                               cudaStream_t s);
int batch_resident_ctas(int N);

// Builds the launch arguments of a model (stage.cu).
KParams make_params(Model* md, const LaunchArgs& a);
// Column-kernel launcher (column.cu); returns cudaErrorNotSupported when no
// column instantiation exists for the model's N.
cudaError_t launch_column(const KParams& P, int N, bool mixed, int mode, int grid, cudaStream_t s);
// Line-kernel launcher (stage_lines.cu), one CTA per element; returns
// cudaErrorNotSupported for an N without an instantiation.
cudaError_t launch_lines(const KParams& P, int N, bool mixed, int mode, cudaStream_t s);
// Weak-form derivative Dhat of the orders 3, 4 and 5 in FP32, passed by value
// to the ensemble kernel (row-major, Dhat[i][n] = D[n][i] w_n / w_i).
struct EnsDhat {
    float d3[16];
    float d4[25];
    float d5[36];
};
// Ensemble stage launch of the persistent line kernel over tiles of every
// order (mixed precision, stage mode) with cta_threads = 128 or 256, and the
// number of its CTAs resident on the device (stage_lines.cu).
cudaError_t launch_ens_lines(const KParams* d_params, const BatchTile* d_tiles, int ntiles, int cta_threads, int grid,
                             const EnsDhat& D, cudaStream_t s);
int ens_lines_resident_ctas(int cta_threads);

namespace {


// Constants in the working precision R, read without a run-time FP64->FP32
// conversion (on this GPU such conversions issue on the FP64 pipe).
template <typename R>
struct KConst;
template <>
struct KConst<double> {
    static __device__ __forceinline__ double gm1(const KParams& P) { return P.ph.gm1; }
    static __device__ __forceinline__ double gamma(const KParams& P) { return P.ph.gamma; }
    static __device__ __forceinline__ double inv_w0(const KParams& P) { return P.inv_w0; }
    static __device__ __forceinline__ double rkb_dt(const KParams& P) { return P.rkb_dt; }
    static __device__ __forceinline__ double metric(const KParams& P, int e, int d) { return P.emetric[3 * e + d]; }
    static __device__ __forceinline__ double inv_tau(const KParams& P) { return P.inv_tau_hyper; }
};
template <>
struct KConst<float> {
    static __device__ __forceinline__ float gm1(const KParams& P) { return P.gm132; }
    static __device__ __forceinline__ float gamma(const KParams& P) { return P.gamma32; }
    static __device__ __forceinline__ float inv_w0(const KParams& P) { return P.inv_w032; }
    static __device__ __forceinline__ float rkb_dt(const KParams& P) { return P.rkb_dt32; }
    static __device__ __forceinline__ float metric(const KParams& P, int e, int d) { return P.emetric32[3 * e + d]; }
    static __device__ __forceinline__ float inv_tau(const KParams& P) { return P.inv_tau_hyper32; }
};

// FP32 -> FP64 by IEEE-754 field arithmetic on the integer pipe (on this GPU
// the F2F conversion instructions issue on the FP64 pipe).  Exact for normal
// numbers and zero; an FP32 subnormal (|f| < 2^-126) maps to a value of the
// same sign below 2^-126, and a non-finite input to a value beyond the FP32
// range (non-finite tendencies are reported through the status word before
// they reach this conversion).
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u;
    const unsigned mag = b & 0x7FFFFFFFu;
    const unsigned hi = (mag == 0u) ? sign : (sign | ((mag >> 3) + (896u << 20)));
    return __hiloint2double((int)hi, (int)(mag << 29));
}

// FP64 -> FP32 by IEEE-754 field arithmetic on the integer pipe, rounding to
// nearest, ties to even (the IEEE default, so the stage increments carry no
// directed bias).  The FP64 significand keeps its top 23 bits; the 29 bits
// dropped, plus 2^28 - 1 plus the kept value's lowest bit, carry one into the
// kept value exactly when they exceed half an FP32 ulp, or equal it with the
// kept value odd; a carry out of the significand steps the exponent (up to an
// infinity past the largest FP32 value).  Magnitudes under 2^-126 flush to a
// signed zero; magnitudes beyond the FP32 range, infinities and NaNs give an
// infinity.  Used for the stage increment only, which is small next to the
// state it is added to.
__device__ __forceinline__ float f64_to_f32_bits(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned mag = hi & 0x7FFFFFFFu;
    unsigned kept = ((mag - (896u << 20)) << 3) | (lo >> 29);
    kept += ((lo & 0x1FFFFFFFu) + 0x0FFFFFFFu + (kept & 1u)) >> 29;
    unsigned bits = sign | kept;
    bits = (mag < (897u << 20)) ? sign : bits;
    bits = (mag >= (1151u << 20)) ? (sign | 0x7F800000u) : bits;
    return __uint_as_float(bits);
}

template <typename R>
struct Level {
    R rho_ref, p_ref, href, crho, gphiz;
};

template <typename R>
__device__ __forceinline__ Level<R> load_level(const KParams& P, int lev);

static_assert(LV_NFIELDS == 8 && LV_GPHIZ == 1 && LV_RHO_REF == 2 && LV_P_REF == 3 && LV_CRHO == 5 && LV_HREF == 6,
              "level rows are read as vectors");

template <>
__device__ __forceinline__ Level<double> load_level<double>(const KParams& P, int lev) {
    const double2* L = reinterpret_cast<const double2*>(P.lvl64 + (size_t)lev * LV_NFIELDS);
    const double2 a = __ldg(L), b = __ldg(L + 1), c = __ldg(L + 2), d = __ldg(L + 3);
    Level<double> l;
    l.gphiz = a.y;
    l.rho_ref = b.x;
    l.p_ref = b.y;
    l.crho = c.y;
    l.href = d.x;
    return l;
}

template <>
__device__ __forceinline__ Level<float> load_level<float>(const KParams& P, int lev) {
    const float4* L = reinterpret_cast<const float4*>(P.lvl32 + (size_t)lev * LV_NFIELDS);
    const float4 a = __ldg(L), b = __ldg(L + 1);
    Level<float> l;
    l.gphiz = a.y;
    l.rho_ref = a.z;
    l.p_ref = a.w;
    l.crho = b.y;
    l.href = b.z;
    return l;
}

// Reciprocal and square root in the working precision: correctly rounded in
// FP64; the hardware approximations (a few ulp) in FP32, where every other
// operation already carries FP32 rounding.
__device__ __forceinline__ double rcp_r(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp_r(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_r(float x) { return x * rsqrtf(x); }

// Pointwise thermodynamics of dry air (PhaseDry: T = T0 + e_int/cv, p = rho R T,
// c = sqrt(gamma R T)) for a conserved state q, which is the full state
// (R = double) or the perturbation about the reference state (MIXED).
template <typename R, bool MIXED>
struct Thermo {
    R rinv;   // 1 / rho
    R u[3];   // velocity
    R pflux;  // pressure entering the momentum flux (p - p_ref with subtract_off)
    R H;      // rhoe + p
    R c;      // sound speed
};

template <typename R, bool MIXED>
__device__ __forceinline__ Thermo<R, MIXED> thermo(const R q[NSTATE], const Level<R>& lv, const KParams& P) {
    Thermo<R, MIXED> t;
    const Physics& ph = P.ph;
    const R gm1 = KConst<R>::gm1(P), gamma = KConst<R>::gamma(P);
    R rho = MIXED ? (lv.rho_ref + q[0]) : q[0];
    t.rinv = rcp_r(rho);
    t.u[0] = q[1] * t.rinv;
    t.u[1] = q[2] * t.rinv;
    t.u[2] = q[3] * t.rinv;
    R ke2 = q[1] * t.u[0] + q[2] * t.u[1] + q[3] * t.u[2];
    R p;
    if (MIXED) {
        // p' = gm1 (rhoe' - ke/2) + rho' crho ; p = p_ref + p'
        R pp = gm1 * (q[4] - R(0.5) * ke2) + q[0] * lv.crho;
        p = lv.p_ref + pp;
        t.pflux = (ph.ref_state && ph.subtract_off) ? pp : p;
        t.H = lv.href + (q[4] + pp);
    } else {
        p = gm1 * (q[4] - R(0.5) * ke2) + rho * lv.crho;
        t.pflux = (ph.ref_state && ph.subtract_off) ? (p - lv.p_ref) : p;
        t.H = q[4] + p;
    }
    t.c = sqrt_r(gamma * p * t.rinv);
    return t;
}

// first-order flux component in direction d for field s
template <typename R, bool MIXED>
__device__ __forceinline__ R flux_d(const R q[NSTATE], const Thermo<R, MIXED>& t, int d, int s) {
    if (s == 0) return q[1 + d];
    if (s == 4) return t.u[d] * t.H;
    return q[1 + d] * t.u[s - 1] + ((s - 1 == d) ? t.pflux : R(0));
}

// component d (0, 1, 2; a run-time value) of a 3-vector without indexing a
// local array, so the values stay in registers
template <typename R>
__device__ __forceinline__ R pick3(int d, R a, R b, R c) {
    return d == 0 ? a : (d == 1 ? b : c);
}

// normal first-order flux F_d (all 5 fields) for a face normal to xi_d
template <typename R, bool MIXED>
__device__ __forceinline__ void normal_flux(const R q[NSTATE], const Thermo<R, MIXED>& t, int d, R sgn, R F[NSTATE]) {
    const R mn = pick3(d, q[1], q[2], q[3]);
    const R un = pick3(d, t.u[0], t.u[1], t.u[2]);
    F[0] = sgn * mn;
    F[1] = sgn * (mn * t.u[0] + (d == 0 ? t.pflux : R(0)));
    F[2] = sgn * (mn * t.u[1] + (d == 1 ? t.pflux : R(0)));
    F[3] = sgn * (mn * t.u[2] + (d == 2 ? t.pflux : R(0)));
    F[4] = sgn * (un * t.H);
}


// Planar shared-memory records of five fields for n nodes: fields 0..3 in a
// plane of 16-byte vectors (float4; two double2 planes in FP64) and field 4
// in a scalar plane.  A warp reading or writing consecutive records touches
// consecutive 16-byte (and 4/8-byte) words, so the accesses are free of bank
// conflicts; a record still moves with one 128-bit and one 32-bit access in
// FP32.  Plane offsets are kept 16-byte aligned (planar_words).
template <typename R>
struct Planar5;
template <>
struct Planar5<float> {
    static __device__ __forceinline__ void ld(const float* base, int n, int i, float v[NSTATE]) {
        const float4 a = reinterpret_cast<const float4*>(base)[i];
        v[0] = a.x;
        v[1] = a.y;
        v[2] = a.z;
        v[3] = a.w;
        v[4] = base[4 * n + i];
    }
    static __device__ __forceinline__ void st(float* base, int n, int i, const float v[NSTATE]) {
        reinterpret_cast<float4*>(base)[i] = make_float4(v[0], v[1], v[2], v[3]);
        base[4 * n + i] = v[4];
    }
};
template <>
struct Planar5<double> {
    static __device__ __forceinline__ void ld(const double* base, int n, int i, double v[NSTATE]) {
        const double2 a = reinterpret_cast<const double2*>(base)[i];
        const double2 b = reinterpret_cast<const double2*>(base + 2 * n)[i];
        v[0] = a.x;
        v[1] = a.y;
        v[2] = b.x;
        v[3] = b.y;
        v[4] = base[4 * n + i];
    }
    static __device__ __forceinline__ void st(double* base, int n, int i, const double v[NSTATE]) {
        reinterpret_cast<double2*>(base)[i] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(base + 2 * n)[i] = make_double2(v[2], v[3]);
        base[4 * n + i] = v[4];
    }
};
// Bulk asynchronous global->shared copies (the TMA engine, cp.async.bulk)
// completing on a shared-memory mbarrier: one thread issues a contiguous
// copy of a multiple of 16 bytes between 16-byte-aligned addresses and arms
// the barrier with the byte count; the consumers wait on the barrier's
// phase.  Every wait is bounded: after the limit the caller records an error
// and carries on (its shared-memory reads then see stale data, never
// out-of-bounds addresses).
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same buffers
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// waits for the phase of `parity` to complete; false after `polls` polls
// (2^16 when polls <= 0; each poll may suspend the thread for a
// hardware-defined interval)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int polls) {
    const int limit = polls > 0 ? polls : (1 << 16);
    for (int i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// words of R taken by `words` words rounded up to 16 bytes
template <typename R>
constexpr int planar_pad(int words) {
    return (int)(((size_t)words * sizeof(R) + 15) / 16 * 16 / sizeof(R));
}
// pair of values per node (sound speed, 1/rho) as an 8- or 16-byte vector plane
template <typename R>
struct Pair;
template <>
struct Pair<float> {
    using V = float2;
    static __device__ __forceinline__ V make(float a, float b) { return make_float2(a, b); }
};
template <>
struct Pair<double> {
    using V = double2;
    static __device__ __forceinline__ V make(double a, double b) { return make_double2(a, b); }
};

}  // namespace
}  // namespace cmdg
