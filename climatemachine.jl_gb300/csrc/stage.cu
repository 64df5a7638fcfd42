// Fused DG tendency + LSRK stage kernels for brick meshes (sm_103a).
//
// One CTA owns one element for a whole stage:
//   phase 1  every node loads its state (coalesced), evaluates the dry
//            AtmosModel thermodynamics and its first-order flux in the three
//            directions and stages them in shared memory;
//   phase 2  every face node (6 (N+1)^2 of them) gathers the neighbour's
//            state at the matching node, forms the Rusanov (or central)
//            flux F*.n and stores it lifted, vMI*sM*F*, in shared memory;
//   phase 3  every node contracts the staged fluxes with the weak-form
//            derivative Dhat = M^-1 D^T M along xi1, xi2, xi3, subtracts its
//            face terms, adds gravity and finishes either the tendency
//            T = alpha*dQ/dt + beta*T or the LSRK 2N stage update.  The
//            register holds the unscaled stage increment:
//            dq_s = dQ/dt(Q_{s-1}) + A_s dq_{s-1}, Q_s = Q_{s-1} + B_s dt dq_s,
//            which is the reference's dQ <- dQ/dt + dQ; Q <- Q + B_s dt dQ;
//            dQ <- A_{s+1} dQ with the A-scaling moved into the next stage
//            (one FMA per DOF; A_1 = 0, so stage 1 does not read the register
//            and stage 5 does not write it).
// The state is read from one buffer and the stage's new state written to
// another, so neighbouring elements never see a half-updated state.
//
// Algorithm restated from src/Numerics/DGMethods/DGModel_kernels.jl:64-548
// (volume_tendency!, H and V), :588-901 (dgsem_interface_tendency!),
// src/Numerics/DGMethods/NumericalFluxes.jl:219-340 (Rusanov / central),
// src/Atmos/Model/{tendencies_mass.jl:7-9, tendencies_momentum.jl:13-29,60-72,
// tendencies_energy.jl:7-21, AtmosModel.jl:776-796, bc_momentum.jl:25-34} and
// src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:102-158.
//
// On an affine brick element the contravariant flux M xi_d . F reduces to
// J w_i w_j w_k (2/dx_d) F_d, so the volume term at node (i,j,k) is
// (2/dx_1) sum_n Dhat[i][n] F_1(n,j,k) + ... with Dhat[i][n] = D[n][i] w_n / w_i,
// and the lift vMI*sM on a face normal to xi_d is (2/dx_d) / w_0.
//
// Precision: R = double (plain FP64) or R = float (mixed).  In the mixed
// form the state held in memory is the FP32 perturbation q' = q - q_ref about
// the FP64 hydrostatic reference state; pressure is formed directly as the
// perturbation p' = (R/cv)(rhoe' - |rhou|^2/(2 rho)) + rho' (R T0 - (R/cv) Phi),
// which is exact algebra for dry air (T = T0 + e_int/cv, p = rho R T), the
// reference-state jump across vertical faces enters the Rusanov penalty
// from an FP64-computed table, and the RK register dQ stays FP64.
#include "cmdg_internal.h"

namespace cmdg {
namespace {

template <int N>
struct Dims {
    static constexpr int Nq = N + 1;
    static constexpr int Nfp = Nq * Nq;
    static constexpr int Np = Nq * Nq * Nq;
    static constexpr int NF = 6 * Nfp;
    static constexpr int NT = (((Np > NF) ? Np : NF) + 31) / 32 * 32;
    // resident CTAs per SM requested for the FP32 kernels (register budget
    // 65536 / (NT * MIN_CTAS): 64, 56, 51 and 58 registers for N = 2..5)
    static constexpr int MIN_CTAS = N == 2 ? 16 : N == 3 ? 12 : N == 4 ? 8 : 5;
};

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
};

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
};
template <>
struct KConst<float> {
    static __device__ __forceinline__ float gm1(const KParams& P) { return P.gm132; }
    static __device__ __forceinline__ float gamma(const KParams& P) { return P.gamma32; }
    static __device__ __forceinline__ float inv_w0(const KParams& P) { return P.inv_w032; }
    static __device__ __forceinline__ float rkb_dt(const KParams& P) { return P.rkb_dt32; }
    static __device__ __forceinline__ float metric(const KParams& P, int e, int d) { return P.emetric32[3 * e + d]; }
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

// FP64 -> FP32 by IEEE-754 field arithmetic on the integer pipe, rounding
// toward zero (error below one FP32 ulp).  Magnitudes under 2^-126 flush to a
// signed zero; magnitudes beyond the FP32 range, infinities and NaNs give an
// infinity.  Used for the stage increment only, which is small next to the
// state it is added to.
__device__ __forceinline__ float f64_to_f32_bits(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned mag = hi & 0x7FFFFFFFu;
    unsigned bits = sign | (((mag - (896u << 20)) << 3) | (lo >> 29));
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

template <>
__device__ __forceinline__ Level<double> load_level<double>(const KParams& P, int lev) {
    const double* L = P.lvl64 + (size_t)lev * LV_NFIELDS;
    Level<double> l;
    l.rho_ref = L[LV_RHO_REF];
    l.p_ref = L[LV_P_REF];
    l.href = L[LV_HREF];
    l.crho = L[LV_CRHO];
    l.gphiz = L[LV_GPHIZ];
    return l;
}

template <>
__device__ __forceinline__ Level<float> load_level<float>(const KParams& P, int lev) {
    const float* L = P.lvl32 + (size_t)lev * LV_NFIELDS;
    Level<float> l;
    l.rho_ref = L[LV_RHO_REF];
    l.p_ref = L[LV_P_REF];
    l.href = L[LV_HREF];
    l.crho = L[LV_CRHO];
    l.gphiz = L[LV_GPHIZ];
    return l;
}

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
    t.rinv = R(1) / rho;
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
    t.c = sqrt(gamma * p * t.rinv);
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

template <int N>
__device__ __forceinline__ int face_node(int f, int a, int b) {
    constexpr int Nq = N + 1;
    switch (f) {
        case 0: return 0 + Nq * (a + Nq * b);
        case 1: return N + Nq * (a + Nq * b);
        case 2: return a + Nq * (0 + Nq * b);
        case 3: return a + Nq * (N + Nq * b);
        case 4: return a + Nq * (b + Nq * 0);
        default: return a + Nq * (b + Nq * N);
    }
}

// Shared-memory record of one node or face node: the five fields packed
// contiguously (plus two spare slots) so a record moves with 128-bit accesses.
template <typename R>
struct Slot {
    static constexpr int W = 8;  // record width in elements of R
};

template <typename R>
__device__ __forceinline__ void ld5(const R* p, R v[NSTATE]);
template <>
__device__ __forceinline__ void ld5<float>(const float* p, float v[NSTATE]) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
    v[4] = p[4];
}
template <>
__device__ __forceinline__ void ld5<double>(const double* p, double v[NSTATE]) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    const double2 b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
    v[4] = p[4];
}
template <typename R>
__device__ __forceinline__ void st5(R* p, const R v[NSTATE]);
template <>
__device__ __forceinline__ void st5<float>(float* p, const float v[NSTATE]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    p[4] = v[4];
}
template <>
__device__ __forceinline__ void st5<double>(double* p, const double v[NSTATE]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
    p[4] = v[4];
}

template <int N, typename R>
struct Smem {
    static constexpr int Nq = N + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq, W = Slot<R>::W;
    // node records: q (5), sound speed (slot 5), 1/rho (slot 6)
    static constexpr int NODE = 0;
    // volume fluxes by direction
    static constexpr int FLUX = NODE + Np * W;
    // lifted face fluxes
    static constexpr int FACE = FLUX + 3 * Np * W;
    static constexpr int DMAT = FACE + 6 * Nfp * W;
    static constexpr int TOTAL = DMAT + Nq * Nq;
    static constexpr size_t BYTES = sizeof(R) * TOTAL;
};

template <int N, typename R, bool MIXED, int MODE>
__global__ void __launch_bounds__(Dims<N>::NT, MIXED ? Dims<N>::MIN_CTAS : 1) stage_kernel(const KParams P) {
    using Dm = Dims<N>;
    using SM = Smem<N, R>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, W = SM::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const sm = reinterpret_cast<R*>(smem_raw);
    R* const s_node = sm + SM::NODE;
    R* const s_F = sm + SM::FLUX;
    R* const s_fs = sm + SM::FACE;
    R* const s_D = sm + SM::DMAT;

    const int e = blockIdx.x;
    const int t = threadIdx.x;
    const int ez = e % P.nz;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    const Physics& ph = P.ph;
    const bool node_thread = t < Np;
    const bool face_thread = t < 6 * Nfp;
    const bool read_reg = (MODE == 0) ? (P.beta != 0) : !P.first_stage;
    const size_t ebase = (size_t)e * NSTATE * Np;

    // ---------------- issue every global load of this thread up front:
    // own node state and RK register, then the neighbour state at this
    // thread's face node (its latency overlaps the volume work below)
    R q[NSTATE];
    double dq_old[NSTATE];
    if (node_thread) {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = Qin[ebase + s * Np + t];
        if (read_reg) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) dq_old[s] = P.dQ[ebase + s * Np + t];
        }
    }
    int f = 0, fn = 0, d = 0, vM = 0, nb = -1, levp = 0;
    R qp[NSTATE];
    if (face_thread) {
        f = t / Nfp;
        fn = t - f * Nfp;
        const int fa = fn % Nq, fb = fn / Nq;
        d = f >> 1;
        vM = face_node<N>(f, fa, fb);
        nb = P.nbr[6 * e + f];
        if (nb >= 0) {
            const int vP = face_node<N>(f ^ 1, fa, fb);
            levp = (nb % P.nz) * Nq + vP / Nfp;
            const size_t nbase = (size_t)nb * NSTATE * Np + vP;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = Qin[nbase + s * Np];
        } else {
            levp = ez * Nq + vM / Nfp;
        }
    }
    if (t < Nq * Nq) s_D[t] = static_cast<const R*>(P.Dhat)[t];
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};

    // ---------------- phase 1: node thermodynamics and volume fluxes
    R gsrc = 0;
    if (node_thread) {
        const Level<R> lv = load_level<R>(P, ez * Nq + t / Nfp);
        const Thermo<R, MIXED> th = thermo<R, MIXED>(q, lv, P);
        R* rec = s_node + t * W;
        st5<R>(rec, q);
        rec[5] = th.c;
        rec[6] = th.rinv;
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
            R F[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(q, th, dd, s);
            st5<R>(s_F + (dd * Np + t) * W, F);
        }
        if (ph.gravity) {
            R rho_s = MIXED ? ((ph.ref_state && ph.subtract_off) ? q[0] : lv.rho_ref + q[0])
                            : ((ph.ref_state && ph.subtract_off) ? q[0] - lv.rho_ref : q[0]);
            gsrc = -rho_s * lv.gphiz;
        }
    }
    __syncthreads();

    // ---------------- phase 2: one numerical flux per face node
    if (face_thread) {
        const R sgn = (f & 1) ? R(1) : R(-1);
        R qm[NSTATE], Fm[NSTATE], Fp[NSTATE], jr[NSTATE] = {0, 0, 0, 0, 0};
        const R* rec = s_node + vM * W;
        ld5<R>(rec, qm);
        const R c_m = rec[5], ri_m = rec[6];
        ld5<R>(s_F + (d * Np + vM) * W, Fm);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) Fm[s] *= sgn;
        const R lam_m = fabs(pick3(d, qm[1], qm[2], qm[3]) * ri_m) + c_m;
        if (nb >= 0) {
            if (MIXED && d == 2 && ph.numflux == CMDG_FLUX_RUSANOV) {
                // reference-state jump q_ref(-) - q_ref(+) across a vertical face
                if (f == 4) {
                    jr[0] = (R)P.jump32[2 * ez + 0];
                    jr[4] = (R)P.jump32[2 * ez + 1];
                } else {
                    const int ea = (ez + 1) % P.nz;
                    jr[0] = -(R)P.jump32[2 * ea + 0];
                    jr[4] = -(R)P.jump32[2 * ea + 1];
                }
            }
        } else {
            // Impenetrable(FreeSlip) + Insulating wall: rhou+ = rhou- - 2 (rhou-.n) n
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
            qp[1] = (d == 0) ? -qm[1] : qm[1];
            qp[2] = (d == 1) ? -qm[2] : qm[2];
            qp[3] = (d == 2) ? -qm[3] : qm[3];
        }
        const Level<R> lvp = load_level<R>(P, levp);
        const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
        normal_flux<R, MIXED>(qp, thp, d, sgn, Fp);
        const R lam_p = fabs(pick3(d, thp.u[0], thp.u[1], thp.u[2])) + thp.c;
        const R lift = pick3(d, xi[0], xi[1], xi[2]) * KConst<R>::inv_w0(P);
        const R hmw = (ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
        const R hl = R(0.5) * lift, pl = hmw * lift;
        R fs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) fs[s] = hl * (Fm[s] + Fp[s]) + pl * ((qm[s] - qp[s]) + jr[s]);
        st5<R>(s_fs + (f * Nfp + fn) * W, fs);
    }
    __syncthreads();

    // ---------------- phase 3: volume contraction, face terms, source, update
    int bad = 0;
    if (node_thread) {
        const int i = t % Nq, j = (t / Nq) % Nq, k = t / Nfp;
        R acc1[NSTATE] = {0, 0, 0, 0, 0}, acc2[NSTATE] = {0, 0, 0, 0, 0}, acc3[NSTATE] = {0, 0, 0, 0, 0};
        const R* F1 = s_F + (0 * Np + Nq * (j + Nq * k)) * W;      // line along xi1
        const R* F2 = s_F + (1 * Np + i + Nq * Nq * k) * W;        // line along xi2 (stride Nq)
        const R* F3 = s_F + (2 * Np + i + Nq * j) * W;             // line along xi3 (stride Nfp)
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            R v1[NSTATE], v2[NSTATE], v3[NSTATE];
            ld5<R>(F1 + n * W, v1);
            ld5<R>(F2 + n * Nq * W, v2);
            ld5<R>(F3 + n * Nfp * W, v3);
            const R d1 = s_D[i * Nq + n], d2 = s_D[j * Nq + n], d3 = s_D[k * Nq + n];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                acc1[s] = fma(d1, v1[s], acc1[s]);
                acc2[s] = fma(d2, v2[s], acc2[s]);
                acc3[s] = fma(d3, v3[s], acc3[s]);
            }
        }
        R rhs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) rhs[s] = xi[0] * acc1[s] + xi[1] * acc2[s] + xi[2] * acc3[s];
        // face terms (vMI sM F*, lifted in phase 2), in face order 1..6
        const int fidx[6] = {j + Nq * k, j + Nq * k, i + Nq * k, i + Nq * k, i + Nq * j, i + Nq * j};
        const bool on[6] = {i == 0, i == N, j == 0, j == N, k == 0, k == N};
#pragma unroll
        for (int ff = 0; ff < 6; ++ff) {
            if (on[ff]) {
                R v[NSTATE];
                ld5<R>(s_fs + (ff * Nfp + fidx[ff]) * W, v);
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) rhs[s] -= v[s];
            }
        }
        rhs[3] += gsrc;
        const R rkb_dt = KConst<R>::rkb_dt(P);
        R* Qout = static_cast<R*>(P.Qout);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) {
            if (!isfinite(rhs[s])) bad = 1;
            const size_t idx = ebase + s * Np + t;
            if (MODE == 0) {
                double out = P.alpha * (double)rhs[s];
                if (read_reg) out = fma(P.beta, dq_old[s], out);
                P.dQ[idx] = out;
            } else {
                // unscaled 2N register: dq_s = rhs_s + A_s dq_{s-1}  (A_1 = 0)
                double dq;
                if (MIXED) {
                    // one FP64 FMA per DOF; the conversions run on the integer pipe
                    if (read_reg) {
                        dq = fma(P.rka, dq_old[s], f32_to_f64_bits((float)rhs[s]));
                        Qout[idx] = fma(rkb_dt, (R)f64_to_f32_bits(dq), q[s]);
                    } else {
                        dq = f32_to_f64_bits((float)rhs[s]);
                        Qout[idx] = fma(rkb_dt, rhs[s], q[s]);
                    }
                } else {
                    dq = read_reg ? fma(P.rka, dq_old[s], (double)rhs[s]) : (double)rhs[s];
                    Qout[idx] = (R)fma(P.rkb_dt, dq, (double)q[s]);
                }
                if (!P.last_stage) P.dQ[idx] = dq;
            }
        }
    }
    if (__syncthreads_or(bad) && t == 0) atomicOr(P.status, 1u);
}

template <int N, typename R, bool MIXED, int MODE>
cudaError_t launch_mode(const KParams& P, cudaStream_t s) {
    constexpr size_t bytes = Smem<N, R>::BYTES;
    if (bytes > 48 * 1024) {
        // opt in to more than 48 KB of dynamic shared memory, once per device
        static unsigned long long configured = 0;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (!(configured & (1ull << (dev & 63)))) {
            e = cudaFuncSetAttribute(stage_kernel<N, R, MIXED, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)bytes);
            if (e != cudaSuccess) return e;
            configured |= 1ull << (dev & 63);
        }
    }
    stage_kernel<N, R, MIXED, MODE><<<(unsigned)P.nelem, Dims<N>::NT, bytes, s>>>(P);
    return cudaGetLastError();
}

template <int N, typename R, bool MIXED>
cudaError_t launch_typed(const KParams& P, int mode, cudaStream_t s) {
    return mode == 0 ? launch_mode<N, R, MIXED, 0>(P, s) : launch_mode<N, R, MIXED, 1>(P, s);
}

template <int N>
cudaError_t launch_N(const KParams& P, bool mixed, int mode, cudaStream_t s) {
    return mixed ? launch_typed<N, float, true>(P, mode, s) : launch_typed<N, double, false>(P, mode, s);
}

}  // namespace

int launch_stage(Model* md, const LaunchArgs& a, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    KParams P;
    P.Qin = a.Qin;
    P.Qout = a.Qout;
    P.dQ = a.dQ;
    P.emetric = m.d_emetric;
    P.nbr = m.d_nbr;
    P.lvl64 = md->d_lvl64;
    P.lvl32 = md->d_lvl32;
    P.jump32 = md->d_jump32;
    const bool mixed = md->precision == CMDG_MIXED;
    P.Dhat = mixed ? (const void*)md->d_Dhat32 : (const void*)md->d_Dhat64;
    P.status = md->d_status;
    P.nelem = (int)m.nelem;
    P.nz = m.nz;
    P.alpha = a.alpha;
    P.beta = a.beta;
    P.rka = a.rka;
    P.rkb_dt = a.rkb_dt;
    P.first_stage = a.first_stage;
    P.last_stage = a.last_stage;
    P.inv_w0 = 1.0 / m.omega[0];
    P.emetric32 = m.d_emetric32;
    P.rkb_dt32 = (float)a.rkb_dt;
    P.inv_w032 = (float)P.inv_w0;
    P.gm132 = (float)md->ph.gm1;
    P.gamma32 = (float)md->ph.gamma;
    P.ph = md->ph;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_N<2>(P, mixed, a.mode, s); break;
        case 3: err = launch_N<3>(P, mixed, a.mode, s); break;
        case 4: err = launch_N<4>(P, mixed, a.mode, s); break;
        case 5: err = launch_N<5>(P, mixed, a.mode, s); break;
        default: set_error("no kernel instantiated for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
