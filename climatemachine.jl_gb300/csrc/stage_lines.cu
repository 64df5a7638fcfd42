// Line-per-thread fused DG tendency + LSRK stage kernel for brick meshes
// (sm_103a), FP32 mixed and FP64.
//
// A CTA works on EPI elements at a time, each with a sub-block of TPE
// threads (TPE >= the element's 3 (N+1)^2 lines; a thread owns NPT nodes):
//   phase 1  every node thread loads its state (coalesced), evaluates the dry
//            AtmosModel thermodynamics, and stores in shared memory its
//            state, (c, 1/rho, pressure of the momentum flux, rhoe + p) and
//            its three directional first-order fluxes, each already scaled by
//            the element's metric 2/dx_d;
//   phase 2  each of the 3 (N+1)^2 element lines (xi_d line L) is one thread:
//            it forms the numerical fluxes (Rusanov or central) of the two
//            face nodes at its ends from the end nodes' staged states and
//            the neighbours' states (loaded at the start of the element),
//            then, field by field, reads the N+1 staged fluxes along the line,
//            contracts them with the weak-form derivative
//            Dhat[i][n] = D[n][i] w_n / w_i (compile-time indices: the
//            coefficients come from the kernel's parameter bank), subtracts
//            the lifted face fluxes at the two ends and writes the line's
//            N+1 derivative values back in place;
//   phase 3  every node thread sums its three directional derivatives, adds
//            gravity and finishes the tendency T = alpha dQ/dt + beta T or
//            the LSRK 2N stage update (unscaled register, as in stage.cu).
// The face flux of a face node is formed once, by the thread of the line
// that ends there, and never goes through shared memory; each staged flux is
// read once per contraction (by its line's thread) instead of once per node
// of the line.  Shared planes are node-major scalar planes, so the node
// threads' stores and loads are consecutive, and a line thread's reads of
// one position along consecutive lines are strided by 1, N+1 or (N+1)^2.
//
// One model: one CTA of roundup32((N+1)^3) threads per element (EPI = NPT = 1).
// Ensembles: one persistent launch per stage over a list of tiles of all
// orders, with one CTA shape for every order: 128 threads run two N = 3
// elements, one N = 4 element, or one N = 5 element at two nodes per thread;
// 256 threads run four N = 3, two N = 4 or one N = 5 element, a thread per
// node (the autotuner's choice).
//
// Arithmetic restated from src/Numerics/DGMethods/DGModel_kernels.jl:64-548
// (volume_tendency!), :588-901 (dgsem_interface_tendency!),
// src/Numerics/DGMethods/NumericalFluxes.jl:219-340 (Rusanov / central) and
// src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:102-158; the terms
// are those of the node kernel in stage.cu, summed in a different order.
#include <type_traits>

#include "dg_common.cuh"

namespace cmdg {
namespace {

template <int N>
struct LDims {
    static constexpr int Nq = N + 1;
    static constexpr int Nfp = Nq * Nq;
    static constexpr int Np = Nq * Nfp;
    static constexpr int NL = 3 * Nfp;  // element lines
    static constexpr int NT = (Np + 31) / 32 * 32;
    // resident CTAs per SM the register budget is set for (one model)
    static constexpr int MIN_CTAS = N == 2 ? 16 : N == 3 ? 16 : N == 4 ? 8 : 4;
    static constexpr int MIN_CTAS64 = N == 5 ? 2 : N == 4 ? 4 : 6;
};

// Work split of a CTA of NT threads over elements of order N: EPI elements
// at a time, TPE threads per element, NPT nodes per thread -- as many
// elements as fit with a thread per node, else one element with several
// nodes per thread (every line still needs a thread of its own).
template <int N, int NT>
struct LSplit {
    static constexpr int Np = LDims<N>::Np;
    static constexpr int TPE_NODE = (Np + 31) / 32 * 32;
    static constexpr int EPI = NT / TPE_NODE >= 4 ? 4 : (NT / TPE_NODE >= 2 ? 2 : 1);
    static constexpr int TPE = NT / EPI;
    static constexpr int NPT = (Np + TPE - 1) / TPE;
    static_assert(TPE >= LDims<N>::NL, "a sub-block needs one thread per element line");
};

// node-major scalar planes of Np words per element: 15 directional fluxes
// (d major, field minor), 5 state fields, 4 auxiliary values per node
template <int N, typename R>
struct LSmem {
    static constexpr int Np = LDims<N>::Np;
    static constexpr int PS = Np;
    static constexpr int FLUX = 0;
    static constexpr int NODE = FLUX + 15 * PS;
    static constexpr int AUX = NODE + 5 * PS;
    static constexpr int TOTAL = AUX + 4 * PS;  // words per element
    static constexpr size_t BYTES = sizeof(R) * TOTAL;
};
enum { AUX_C = 0, AUX_RINV = 1, AUX_PFLUX = 2, AUX_H = 3 };

// Weak-form derivative coefficients with compile-time indices, read from a
// kernel parameter (the constant bank): a model's own launch parameters, or,
// for the ensemble kernel whose launch parameters sit in global memory, the
// per-order table passed with the launch.
template <typename R>
struct DhatOfModel;
template <>
struct DhatOfModel<float> {
    const KParams& P;
    __device__ __forceinline__ float operator()(int idx) const { return P.DhatC32[idx]; }
};
template <>
struct DhatOfModel<double> {
    const KParams& P;
    __device__ __forceinline__ double operator()(int idx) const { return P.DhatC64[idx]; }
};
template <int N>
struct DhatOfOrder {
    const EnsDhat& D;
    __device__ __forceinline__ float operator()(int idx) const {
        return N == 3 ? D.d3[idx] : (N == 4 ? D.d4[idx] : D.d5[idx]);
    }
};

// node index of position n along line L of direction d; a line's index is
// the in-face index of its end nodes on the faces normal to xi_d (the
// reference's face-mask numbering, src/Numerics/Mesh/Grids.jl:580-597)
template <int N>
__device__ __forceinline__ int line_node(int d, int L, int n) {
    constexpr int Nq = N + 1;
    return d == 0 ? n + Nq * L : (d == 1 ? (L % Nq) + Nq * n + Nq * Nq * (L / Nq) : L + Nq * Nq * n);
}

// One pass over element e (or none when e < 0) by a sub-block of TPE threads
// (local index lt), NPT nodes per thread, with the element's shared planes
// at sm.  Every thread of the CTA calls it with the same barrier sequence.
template <int N, typename R, bool MIXED, int MODE, int TPE, int NPT, class DH>
__device__ __forceinline__ int lines_element(const KParams& P, const DH& dhat, R* sm, int e, int lt) {
    using Dm = LDims<N>;
    using SM = LSmem<N, R>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, PS = SM::PS;
    constexpr int ESTRIDE = NSTATE * Np;
    R* const s_F = sm + SM::FLUX;
    R* const s_q = sm + SM::NODE;
    R* const s_a = sm + SM::AUX;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    R* __restrict__ Qout = static_cast<R*>(P.Qout);
    const Physics& ph = P.ph;
    const bool active = e >= 0;
    const bool line_thread = active && lt < Dm::NL;
    const bool read_reg = (MODE == 0) ? (P.beta != 0) : !P.first_stage;

    // line thread: direction ld, line L; its end nodes on faces 2 ld (side 0)
    // and 2 ld + 1 (side 1), and the matching nodes of the neighbours
    const int ld = line_thread ? lt / Nfp : 0;
    const int L = line_thread ? lt - ld * Nfp : 0;
    const int vM0 = line_node<N>(ld, L, 0), vM1 = line_node<N>(ld, L, N);
    const int kM0 = vM0 / Nfp, kM1 = vM1 / Nfp;

    const int* nbr = P.nbr + NBR_STRIDE * (active ? e : 0);
    const int ez = active ? __ldg(nbr + 6) : 0;
    // ---------------- loads, all issued before any arithmetic
    R q[NPT][NSTATE];
    const size_t ebase = (size_t)(active ? e : 0) * ESTRIDE;
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int node = lt + k * TPE;
        if (active && node < Np) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) q[k][s] = Qin[ebase + s * Np + node];
        }
    }
    // neighbour states at the line's two end nodes (the node of the
    // neighbour on the opposite face: vM1 for side 0, vM0 for side 1)
    int nb0 = -1, nb1 = -1;
    R qp0[NSTATE], qp1[NSTATE];
    if (line_thread) {
        nb0 = __ldg(nbr + 2 * ld);
        nb1 = __ldg(nbr + 2 * ld + 1);
        if (nb0 >= 0) {
            const R* qn = Qin + (size_t)nb0 * ESTRIDE + vM1;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp0[s] = qn[s * Np];
        }
        if (nb1 >= 0) {
            const R* qn = Qin + (size_t)nb1 * ESTRIDE + vM0;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp1[s] = qn[s * Np];
        }
    }
    R xi[3] = {R(0), R(0), R(0)};
    if (active) {
        xi[0] = KConst<R>::metric(P, e, 0);
        xi[1] = KConst<R>::metric(P, e, 1);
        xi[2] = KConst<R>::metric(P, e, 2);
    }

    // ---------------- phase 1: node thermodynamics and scaled volume fluxes
    R gsrc[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int node = lt + k * TPE;
        gsrc[k] = 0;
        if (active && node < Np) {
            const Level<R> lv = load_level<R>(P, ez * Nq + node / Nfp);
            const Thermo<R, MIXED> th = thermo<R, MIXED>(q[k], lv, P);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) s_q[s * PS + node] = q[k][s];
            s_a[AUX_C * PS + node] = th.c;
            s_a[AUX_RINV * PS + node] = th.rinv;
            s_a[AUX_PFLUX * PS + node] = th.pflux;
            s_a[AUX_H * PS + node] = th.H;
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int s = 0; s < NSTATE; ++s)
                    s_F[(dd * NSTATE + s) * PS + node] = xi[dd] * flux_d<R, MIXED>(q[k], th, dd, s);
            if (ph.gravity) {
                R rho_s = MIXED ? ((ph.ref_state && ph.subtract_off) ? q[k][0] : lv.rho_ref + q[k][0])
                                : ((ph.ref_state && ph.subtract_off) ? q[k][0] - lv.rho_ref : q[k][0]);
                gsrc[k] = -rho_s * lv.gphiz;
            }
        }
    }
    __syncthreads();

    // ---------------- phase 2: face fluxes at the line's ends, line contraction
    if (line_thread) {
        const R lift = pick3(ld, xi[0], xi[1], xi[2]) * KConst<R>::inv_w0(P);
        R fs0[NSTATE], fs1[NSTATE];
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int vM = side ? vM1 : vM0;
            const int nb = side ? nb1 : nb0;
            const R sgn = side ? R(1) : R(-1);
            R qm[NSTATE], qp[NSTATE], Fm[NSTATE], Fp[NSTATE], jr[NSTATE] = {0, 0, 0, 0, 0};
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qm[s] = s_q[s * PS + vM];
            const R c_m = s_a[AUX_C * PS + vM], ri_m = s_a[AUX_RINV * PS + vM];
            const R pf_m = s_a[AUX_PFLUX * PS + vM], H_m = s_a[AUX_H * PS + vM];
            // minus-side normal flux sgn F_d from the staged state
            {
                const R mn = pick3(ld, qm[1], qm[2], qm[3]);
                const R un = mn * ri_m;
                Fm[0] = sgn * mn;
                Fm[1] = sgn * (mn * (qm[1] * ri_m) + (ld == 0 ? pf_m : R(0)));
                Fm[2] = sgn * (mn * (qm[2] * ri_m) + (ld == 1 ? pf_m : R(0)));
                Fm[3] = sgn * (mn * (qm[3] * ri_m) + (ld == 2 ? pf_m : R(0)));
                Fm[4] = sgn * (un * H_m);
            }
            const R lam_m = fabs(pick3(ld, qm[1], qm[2], qm[3]) * ri_m) + c_m;
            int ezp = ez;
            const int kM = side ? kM1 : kM0;
            int kP = kM;
            if (nb >= 0) {
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) qp[s] = side ? qp1[s] : qp0[s];
                if (ld == 2) {
                    // vertical neighbour: one element below (side 0) or above (side 1), periodic wrap
                    ezp = ez + (side ? 1 : -1);
                    ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
                    kP = side ? 0 : N;
                    if (MIXED && ph.numflux == CMDG_FLUX_RUSANOV) {
                        // reference-state jump q_ref(-) - q_ref(+) across the face
                        const int ej = side ? ezp : ez;
                        const R sj = side ? R(-1) : R(1);
                        jr[0] = sj * (R)P.jump32[2 * ej + 0];
                        jr[4] = sj * (R)P.jump32[2 * ej + 1];
                    }
                }
            } else {
                // Impenetrable(FreeSlip) + Insulating wall: rhou+ = rhou- - 2 (rhou-.n) n
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
                qp[1] = (ld == 0) ? -qm[1] : qm[1];
                qp[2] = (ld == 1) ? -qm[2] : qm[2];
                qp[3] = (ld == 2) ? -qm[3] : qm[3];
            }
            const Level<R> lvp = load_level<R>(P, ezp * Nq + kP);
            const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
            normal_flux<R, MIXED>(qp, thp, ld, sgn, Fp);
            const R lam_p = fabs(pick3(ld, thp.u[0], thp.u[1], thp.u[2])) + thp.c;
            const R hmw = (ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
            const R hl = R(0.5) * lift, pl = hmw * lift;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                const R v = hl * (Fm[s] + Fp[s]) + pl * ((qm[s] - qp[s]) + jr[s]);
                if (side) fs1[s] = v;
                else fs0[s] = v;
            }
        }
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) {
            R* plane = s_F + (ld * NSTATE + s) * PS;
            R v[Nq], out[Nq];
#pragma unroll
            for (int n = 0; n < Nq; ++n) v[n] = plane[line_node<N>(ld, L, n)];
#pragma unroll
            for (int i = 0; i < Nq; ++i) {
                R acc = dhat(i * Nq) * v[0];
#pragma unroll
                for (int n = 1; n < Nq; ++n) acc = fma(dhat(i * Nq + n), v[n], acc);
                out[i] = acc;
            }
            out[0] -= fs0[s];
            out[N] -= fs1[s];
#pragma unroll
            for (int i = 0; i < Nq; ++i) plane[line_node<N>(ld, L, i)] = out[i];
        }
    }
    __syncthreads();

    // ---------------- phase 3: sum of the directions, source, update
    int bad = 0;
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int node = lt + k * TPE;
        if (!(active && node < Np)) continue;
        double dq_old[NSTATE];
        if (read_reg) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) dq_old[s] = P.dQ[ebase + s * Np + node];
        }
        R rhs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s)
            rhs[s] = s_F[s * PS + node] + s_F[(NSTATE + s) * PS + node] + s_F[(2 * NSTATE + s) * PS + node];
        rhs[3] += gsrc[k];
        const R rkb_dt = KConst<R>::rkb_dt(P);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) {
            if (!isfinite(rhs[s])) bad = 1;
            const size_t idx = ebase + s * Np + node;
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
                        Qout[idx] = fma(rkb_dt, (R)f64_to_f32_bits(dq), q[k][s]);
                    } else {
                        dq = f32_to_f64_bits((float)rhs[s]);
                        Qout[idx] = fma(rkb_dt, rhs[s], q[k][s]);
                    }
                } else {
                    dq = read_reg ? fma(P.rka, dq_old[s], (double)rhs[s]) : (double)rhs[s];
                    Qout[idx] = (R)fma(P.rkb_dt, dq, (double)q[k][s]);
                }
                if (!P.last_stage) P.dQ[idx] = dq;
            }
        }
    }
    return bad;
}

// One model: one CTA per element.
template <int N, typename R, bool MIXED, int MODE>
__global__ void __launch_bounds__(LDims<N>::NT, MIXED ? LDims<N>::MIN_CTAS : LDims<N>::MIN_CTAS64)
    lines_kernel(const KParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const DhatOfModel<R> dh{P};
    const int bad = lines_element<N, R, MIXED, MODE, LDims<N>::NT, 1>(P, dh, reinterpret_cast<R*>(smem_raw),
                                                                       blockIdx.x, threadIdx.x);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(P.status, 1u);
}

// Ensembles: tiles of every order, EPI elements of a tile at a time.
template <int N, int NT>
__device__ __forceinline__ int lines_tile(const KParams& P, const EnsDhat& D, unsigned char* smem_raw, int e0,
                                          int e1) {
    using S = LSplit<N, NT>;
    const int sb = threadIdx.x / S::TPE, lt = threadIdx.x - sb * S::TPE;
    float* sm = reinterpret_cast<float*>(smem_raw) + sb * LSmem<N, float>::TOTAL;
    const DhatOfOrder<N> dh{D};
    int bad = 0;
    for (int e = e0; e < e1; e += S::EPI) {
        const int me = e + sb < e1 ? e + sb : -1;
        bad |= lines_element<N, float, true, 1, S::TPE, S::NPT>(P, dh, sm, me, lt);
        __syncthreads();  // the next elements' phase 1 overwrites these planes
    }
    return bad;
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == 128 ? 6 : 3)
    ens_lines_kernel(const KParams* __restrict__ params, const BatchTile* __restrict__ tiles, int ntiles,
                     const __grid_constant__ EnsDhat D) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int bad = 0;
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const BatchTile T = tiles[it];
        const KParams& P = params[T.member];
        int b = 0;
        switch (T.N) {
            case 3: b = lines_tile<3, NT>(P, D, smem_raw, T.e0, T.e1); break;
            case 4: b = lines_tile<4, NT>(P, D, smem_raw, T.e0, T.e1); break;
            case 5: b = lines_tile<5, NT>(P, D, smem_raw, T.e0, T.e1); break;
            default: break;
        }
        if (__syncthreads_or(b) && threadIdx.x == 0) atomicOr(P.status, 1u);
        bad |= b;
    }
    (void)bad;
}

template <int NT>
constexpr size_t ens_smem_bytes() {
    constexpr size_t a = LSplit<3, NT>::EPI * LSmem<3, float>::BYTES;
    constexpr size_t b = LSplit<4, NT>::EPI * LSmem<4, float>::BYTES;
    constexpr size_t c = LSplit<5, NT>::EPI * LSmem<5, float>::BYTES;
    return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

template <int N, typename R, bool MIXED, int MODE>
cudaError_t launch_lines_mode(const KParams& P, cudaStream_t s) {
    constexpr size_t bytes = LSmem<N, R>::BYTES;
    if (bytes > 48 * 1024) {
        static unsigned long long configured = 0;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (!(configured & (1ull << (dev & 63)))) {
            e = cudaFuncSetAttribute(lines_kernel<N, R, MIXED, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)bytes);
            if (e != cudaSuccess) return e;
            configured |= 1ull << (dev & 63);
        }
    }
    lines_kernel<N, R, MIXED, MODE><<<(unsigned)P.nelem, LDims<N>::NT, bytes, s>>>(P);
    return cudaGetLastError();
}

template <int NT>
cudaError_t launch_ens_NT(const KParams* d_params, const BatchTile* d_tiles, int ntiles, int grid, const EnsDhat& D,
                          cudaStream_t s) {
    constexpr size_t bytes = ens_smem_bytes<NT>();
    static_assert(bytes <= 48 * 1024, "the ensemble kernel's planes fit the default shared-memory window");
    ens_lines_kernel<NT><<<(unsigned)grid, NT, bytes, s>>>(d_params, d_tiles, ntiles, D);
    return cudaGetLastError();
}

template <int NT>
int ens_resident() {
    int dev = 0, per_sm = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ens_lines_kernel<NT>, NT, ens_smem_bytes<NT>()) !=
        cudaSuccess)
        return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return per_sm * sms;
}

}  // namespace

cudaError_t launch_lines(const KParams& P, int N, bool mixed, int mode, cudaStream_t s) {
    auto go = [&](auto nt) -> cudaError_t {
        constexpr int NN = decltype(nt)::value;
        if (mixed) return mode == 0 ? launch_lines_mode<NN, float, true, 0>(P, s) : launch_lines_mode<NN, float, true, 1>(P, s);
        return mode == 0 ? launch_lines_mode<NN, double, false, 0>(P, s) : launch_lines_mode<NN, double, false, 1>(P, s);
    };
    switch (N) {
        case 2: return go(std::integral_constant<int, 2>{});
        case 3: return go(std::integral_constant<int, 3>{});
        case 4: return go(std::integral_constant<int, 4>{});
        case 5: return go(std::integral_constant<int, 5>{});
        default: return cudaErrorNotSupported;
    }
}

cudaError_t launch_ens_lines(const KParams* d_params, const BatchTile* d_tiles, int ntiles, int cta_threads, int grid,
                             const EnsDhat& D, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    if (cta_threads == 128) return launch_ens_NT<128>(d_params, d_tiles, ntiles, grid, D, s);
    if (cta_threads == 256) return launch_ens_NT<256>(d_params, d_tiles, ntiles, grid, D, s);
    return cudaErrorInvalidValue;
}

int ens_lines_resident_ctas(int cta_threads) {
    return cta_threads == 128 ? ens_resident<128>() : cta_threads == 256 ? ens_resident<256>() : 0;
}

}  // namespace cmdg
