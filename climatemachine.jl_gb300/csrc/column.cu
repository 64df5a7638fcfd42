// Column-per-thread fused DG tendency + LSRK stage kernel for brick meshes
// (sm_103a, FP32 mixed-precision path).
//
// Work decomposition: a CTA holds EPB elements; the (N+1)^2 threads of an
// element each own one vertical line of N+1 nodes (i, j, 0..N) — the same
// (i, j) workgroup shape as the reference's volume_tendency!
// (src/Numerics/DGMethods/DGModel_kernels.jl:64-309, a thread per (i, j)
// walking k).  Everything along xi3 stays in registers:
//   phase A  load the line's state (coalesced across threads), evaluate
//            thermodynamics and fluxes of its N+1 nodes, stage the xi1/xi2
//            fluxes in shared memory, contract the xi3 fluxes with Dhat
//            (compile-time indices: the coefficients come from the parameter
//            bank), and form the bottom/top face fluxes of the line from the
//            vertical neighbours' states;
//   phase B  each thread forms the numerical flux at in-face node c of the
//            four horizontal faces (balanced: 4 per thread), and contracts the
//            staged xi1/xi2 fluxes along the two lines through each of its
//            nodes;
//   phase C  lines on a horizontal face subtract the lifted face fluxes of
//            their nodes; gravity; tendency or LSRK 2N stage update.
// Two barriers per element.  The arithmetic (fluxes, Rusanov flux, lift
// vMI sM = (2/dx_d)/w_0, Dhat = M^-1 D^T M, unscaled 2N register with one
// FP64 FMA per DOF) is that of the node-per-thread kernel in stage.cu; only
// the mapping of work to threads differs.
#include "dg_common.cuh"

namespace cmdg {
namespace {

// elements per CTA for each N (threads = EPB (N+1)^2, kept near a multiple of 32)
template <int N>
struct ColCfg;
template <>
struct ColCfg<3> {
    static constexpr int EPB = 8;  // 128 threads
    static constexpr int MIN_CTAS = 4;
};
template <>
struct ColCfg<4> {
    static constexpr int EPB = 5;  // 125 threads
    static constexpr int MIN_CTAS = 5;
};
template <>
struct ColCfg<5> {
    static constexpr int EPB = 4;  // 144 threads
    static constexpr int MIN_CTAS = 3;
};

template <int N, typename R>
struct ColSmem {
    static constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    // per element, planar five-field records (Planar5): xi1 and xi2 fluxes,
    // states and (c, 1/rho) of the horizontal-face nodes, then the lifted
    // horizontal face fluxes in place of those states
    static constexpr int F1 = 0;
    static constexpr int F2 = F1 + planar_pad<R>(5 * Np);
    static constexpr int NODE = F2 + planar_pad<R>(5 * Np);
    static constexpr int CR = NODE + planar_pad<R>(5 * 4 * Nfp);
    // the lifted face flux of in-face node c replaces that node's record: the
    // thread that reads the record is the one that writes the flux
    static constexpr int FACE = NODE;
    static constexpr int PER_ELEM = CR + planar_pad<R>(2 * 4 * Nfp);
    static constexpr int DMAT = ColCfg<N>::EPB * PER_ELEM;
    static constexpr int TOTAL = DMAT + Nq * Nq;
    static constexpr size_t BYTES = sizeof(R) * TOTAL;
};

template <typename R>
__device__ __forceinline__ R dhat_c(const KParams& P, int idx);
template <>
__device__ __forceinline__ float dhat_c<float>(const KParams& P, int idx) {
    return P.DhatC32[idx];
}
template <>
__device__ __forceinline__ double dhat_c<double>(const KParams& P, int idx) {
    return P.DhatC64[idx];
}

// Numerical flux F*.n (Rusanov or central) of one face node, lifted:
// out = lift * (1/2 (Fm + Fp) + 1/2 max(lam_m, lam_p) ((qm - qp) + jr)).
template <typename R, bool MIXED>
__device__ __forceinline__ void face_flux(const KParams& P, const R qm[NSTATE], const R Fm[NSTATE], R lam_m,
                                          const R qp_in[NSTATE], bool wall, const Level<R>& lvp, int d, R sgn,
                                          const R jr[NSTATE], R lift, R out[NSTATE]) {
    R qp[NSTATE];
    if (wall) {
        // Impenetrable(FreeSlip) + Insulating wall: rhou+ = rhou- - 2 (rhou-.n) n
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
        qp[1 + d] = -qm[1 + d];
    } else {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qp_in[s];
    }
    const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
    R Fp[NSTATE];
    normal_flux<R, MIXED>(qp, thp, d, sgn, Fp);
    const R lam_p = fabs(thp.u[d]) + thp.c;
    const R hmw = (P.ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
    const R hl = R(0.5) * lift, pl = hmw * lift;
#pragma unroll
    for (int s = 0; s < NSTATE; ++s) out[s] = hl * (Fm[s] + Fp[s]) + pl * ((qm[s] - qp[s]) + jr[s]);
}

template <int N, typename R, bool MIXED, int MODE>
__global__ void __launch_bounds__(ColCfg<N>::EPB*(N + 1) * (N + 1), ColCfg<N>::MIN_CTAS) column_kernel(const KParams P) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, EPB = ColCfg<N>::EPB, NH = 4 * Nfp;
    constexpr int ESTRIDE = NSTATE * Np;
    using CS = ColSmem<N, R>;
    using PL = Planar5<R>;
    using CRV = typename Pair<R>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const sm = reinterpret_cast<R*>(smem_raw);

    const int lt = threadIdx.x;
    const int el = lt / Nfp;
    const int c = lt - el * Nfp;
    const int ci = c % Nq, cj = c / Nq;
    const int e_raw = blockIdx.x * EPB + el;
    const bool valid = e_raw < P.nelem;
    const int e = valid ? e_raw : P.nelem - 1;
    R* const sF1 = sm + el * CS::PER_ELEM + CS::F1;
    R* const sF2 = sm + el * CS::PER_ELEM + CS::F2;
    R* const sNode = sm + el * CS::PER_ELEM + CS::NODE;
    CRV* const sCR = reinterpret_cast<CRV*>(sm + el * CS::PER_ELEM + CS::CR);
    R* const sFace = sm + el * CS::PER_ELEM + CS::FACE;
    R* const sD = sm + CS::DMAT;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    const Physics& ph = P.ph;
    const bool read_reg = (MODE == 0) ? (P.beta != 0) : !P.first_stage;
    if (lt < Nq * Nq) sD[lt] = dhat_c<R>(P, lt);

    // ---------------- loads: element row, own line
    const int4 nb03 = __ldg(reinterpret_cast<const int4*>(P.nbr + NBR_STRIDE * e));
    const int4 nb45 = __ldg(reinterpret_cast<const int4*>(P.nbr + NBR_STRIDE * e + 4));
    const int nbf[4] = {nb03.x, nb03.y, nb03.z, nb03.w};
    const int nbb = nb45.x, nbt = nb45.y, ez = nb45.z;
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};
    const R* qe = Qin + (size_t)e * ESTRIDE + c;

    // ---------------- phase A: line thermodynamics and fluxes; the xi3
    // contraction is accumulated node by node (acc[m] += Dhat[m][k] F3(k)),
    // so only one line node's xi3 flux is live at a time
    R acc[Nq][NSTATE];
#pragma unroll
    for (int m = 0; m < Nq; ++m)
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) acc[m][s] = 0;
    R gsrc[Nq];
    R qend[2][NSTATE], Fend[2][NSTATE], c_end[2], ri_end[2];
#pragma unroll
    for (int k = 0; k < Nq; ++k) {
        R qk[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qk[s] = qe[s * Np + k * Nfp];
        const Level<R> lv = load_level<R>(P, ez * Nq + k);
        const Thermo<R, MIXED> th = thermo<R, MIXED>(qk, lv, P);
        const int node = c + k * Nfp;
        R F[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(qk, th, 0, s);
        PL::st(sF1, Np, node, F);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(qk, th, 1, s);
        PL::st(sF2, Np, node, F);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(qk, th, 2, s);
#pragma unroll
        for (int m = 0; m < Nq; ++m)
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) acc[m][s] = fma(dhat_c<R>(P, m * Nq + k), F[s], acc[m][s]);
        if (k == 0 || k == N) {
            const int side = k == 0 ? 0 : 1;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                qend[side][s] = qk[s];
                Fend[side][s] = F[s];
            }
            c_end[side] = th.c;
            ri_end[side] = th.rinv;
        }
        // node records of horizontal-face nodes, at their in-face index
        int ri = -1;
        if (ci == 0) ri = 0 * Nfp + cj + Nq * k;
        if (ci == N) ri = 1 * Nfp + cj + Nq * k;
        if (ri >= 0) {
            PL::st(sNode, NH, ri, qk);
            sCR[ri] = Pair<R>::make(th.c, th.rinv);
        }
        ri = -1;
        if (cj == 0) ri = 2 * Nfp + ci + Nq * k;
        if (cj == N) ri = 3 * Nfp + ci + Nq * k;
        if (ri >= 0) {
            PL::st(sNode, NH, ri, qk);
            sCR[ri] = Pair<R>::make(th.c, th.rinv);
        }
        gsrc[k] = 0;
        if (ph.gravity) {
            R rho_s = MIXED ? ((ph.ref_state && ph.subtract_off) ? qk[0] : lv.rho_ref + qk[0])
                            : ((ph.ref_state && ph.subtract_off) ? qk[0] - lv.rho_ref : qk[0]);
            gsrc[k] = -rho_s * lv.gphiz;
        }
    }
#pragma unroll
    for (int m = 0; m < Nq; ++m)
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) acc[m][s] *= xi[2];
    // bottom (face 5 of the reference, xi3 = -1) and top (face 6) of the line
    {
        const R lift3 = xi[2] * KConst<R>::inv_w0(P);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int k = side ? N : 0;
            const R sgn = side ? R(1) : R(-1);
            const int nbv = side ? nbt : nbb;
            R Fm[NSTATE], qv[NSTATE], jr[NSTATE] = {0, 0, 0, 0, 0};
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) Fm[s] = sgn * Fend[side][s];
            const R lam_m = fabs(qend[side][3] * ri_end[side]) + c_end[side];
            int lev_p = ez * Nq + k;
            if (nbv >= 0) {
                const R* qn = Qin + (size_t)nbv * ESTRIDE + c + (side ? 0 : N * Nfp);
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) qv[s] = qn[s * Np];
                int ezp = ez + (side ? 1 : -1);
                ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
                lev_p = ezp * Nq + (side ? 0 : N);
                if (MIXED && ph.numflux == CMDG_FLUX_RUSANOV) {
                    const int ej = side ? ezp : ez;
                    const R sj = side ? R(-1) : R(1);
                    jr[0] = sj * (R)P.jump32[2 * ej + 0];
                    jr[4] = sj * (R)P.jump32[2 * ej + 1];
                }
            }
            const Level<R> lvp = load_level<R>(P, lev_p);
            R fs[NSTATE];
            face_flux<R, MIXED>(P, qend[side], Fm, lam_m, qv, nbv < 0, lvp, 2, sgn, jr, lift3, fs);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) acc[k][s] -= fs[s];
        }
    }
    __syncthreads();

    // ---------------- phase B: horizontal faces (in-face node c of faces 1-4), xi1/xi2 terms
    {
        const int ca = c % Nq, cb = c / Nq;
        const int vPh[4] = {N + Nq * c, Nq * c, ca + Nq * (N + Nq * cb), ca + Nq * (Nq * cb)};
        const int vMh[4] = {Nq * c, N + Nq * c, ca + Nfp * cb, ca + Nq * N + Nfp * cb};
        const R inv_w0 = KConst<R>::inv_w0(P);
        const Level<R> lvh = load_level<R>(P, ez * Nq + cb);
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const int d = f >> 1;
            const R sgn = (f & 1) ? R(1) : R(-1);
            R qh[NSTATE];
            if (nbf[f] >= 0) {
                const R* qn = Qin + (size_t)nbf[f] * ESTRIDE + vPh[f];
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) qh[s] = qn[s * Np];
            }
            R qm[NSTATE], Fm[NSTATE];
            PL::ld(sNode, NH, f * Nfp + c, qm);
            const CRV cr = sCR[f * Nfp + c];
            const R c_m = cr.x, ri_m = cr.y;
            PL::ld(d == 0 ? sF1 : sF2, Np, vMh[f], Fm);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) Fm[s] *= sgn;
            const R lam_m = fabs(qm[1 + d] * ri_m) + c_m;
            const R jr[NSTATE] = {0, 0, 0, 0, 0};
            R fs[NSTATE];
            face_flux<R, MIXED>(P, qm, Fm, lam_m, qh, nbf[f] < 0, lvh, d, sgn, jr, xi[d] * inv_w0, fs);
            PL::st(sFace, NH, f * Nfp + c, fs);
        }
        R Di[Nq], Dj[Nq];
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            Di[n] = sD[ci * Nq + n];
            Dj[n] = sD[cj * Nq + n];
        }
#pragma unroll
        for (int k = 0; k < Nq; ++k) {
            R c1[NSTATE] = {0, 0, 0, 0, 0}, c2[NSTATE] = {0, 0, 0, 0, 0};
            const int L1 = Nq * (cj + Nq * k), L2 = ci + Nfp * k;
#pragma unroll
            for (int n = 0; n < Nq; ++n) {
                R v1[NSTATE], v2[NSTATE];
                PL::ld(sF1, Np, L1 + n, v1);
                PL::ld(sF2, Np, L2 + n * Nq, v2);
#pragma unroll
                for (int s = 0; s < NSTATE; ++s) {
                    c1[s] = fma(Di[n], v1[s], c1[s]);
                    c2[s] = fma(Dj[n], v2[s], c2[s]);
                }
            }
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) acc[k][s] += xi[0] * c1[s] + xi[1] * c2[s];
        }
    }
    __syncthreads();

    // ---------------- phase C: horizontal face terms, source, update (the
    // line's state and RK register are read here, where they are used)
    int bad = 0;
    const size_t ebase = (size_t)e * ESTRIDE + c;
#pragma unroll
    for (int k = 0; k < Nq; ++k) {
        auto sub_face = [&](int f, int idx) {
            R v[NSTATE];
            PL::ld(sFace, NH, f * Nfp + idx, v);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) acc[k][s] -= v[s];
        };
        if (ci == 0) sub_face(0, cj + Nq * k);
        if (ci == N) sub_face(1, cj + Nq * k);
        if (cj == 0) sub_face(2, ci + Nq * k);
        if (cj == N) sub_face(3, ci + Nq * k);
        acc[k][3] += gsrc[k];
    }
    if (valid) {
        const R rkb_dt = KConst<R>::rkb_dt(P);
        R* Qout = static_cast<R*>(P.Qout);
#pragma unroll
        for (int k = 0; k < Nq; ++k) {
            R qk[NSTATE];
            double dq_old[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                qk[s] = qe[s * Np + k * Nfp];
                if (read_reg) dq_old[s] = P.dQ[ebase + s * Np + k * Nfp];
            }
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                const R rhs = acc[k][s];
                if (!isfinite(rhs)) bad = 1;
                const size_t idx = ebase + s * Np + k * Nfp;
                if (MODE == 0) {
                    double out = P.alpha * (double)rhs;
                    if (read_reg) out = fma(P.beta, dq_old[s], out);
                    P.dQ[idx] = out;
                } else {
                    double dq;
                    if (MIXED) {
                        if (read_reg) {
                            dq = fma(P.rka, dq_old[s], f32_to_f64_bits((float)rhs));
                            Qout[idx] = fma(rkb_dt, (R)f64_to_f32_bits(dq), qk[s]);
                        } else {
                            dq = f32_to_f64_bits((float)rhs);
                            Qout[idx] = fma(rkb_dt, rhs, qk[s]);
                        }
                    } else {
                        dq = read_reg ? fma(P.rka, dq_old[s], (double)rhs) : (double)rhs;
                        Qout[idx] = (R)fma(P.rkb_dt, dq, (double)qk[s]);
                    }
                    if (!P.last_stage) P.dQ[idx] = dq;
                }
            }
        }
    }
    // one pass per CTA: no barrier at the end, one vote per warp
    if (__any_sync(0xffffffffu, bad) && (lt & 31) == 0) atomicOr(P.status, 1u);
}

template <int N, int MODE>
cudaError_t launch_col(const KParams& P, cudaStream_t s) {
    using CS = ColSmem<N, float>;
    constexpr int EPB = ColCfg<N>::EPB;
    constexpr size_t bytes = CS::BYTES;
    static unsigned long long configured = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (bytes > 48 * 1024 && !(configured & (1ull << (dev & 63)))) {
        e = cudaFuncSetAttribute(column_kernel<N, float, true, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)bytes);
        if (e != cudaSuccess) return e;
        configured |= 1ull << (dev & 63);
    }
    const unsigned grid = (unsigned)((P.nelem + EPB - 1) / EPB);
    column_kernel<N, float, true, MODE><<<grid, EPB * (N + 1) * (N + 1), bytes, s>>>(P);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_col_mode(const KParams& P, int mode, cudaStream_t s) {
    return mode == 0 ? launch_col<N, 0>(P, s) : launch_col<N, 1>(P, s);
}

}  // namespace

cudaError_t launch_column(const KParams& P, int N, bool mixed, int mode, int grid, cudaStream_t s) {
    (void)grid;
    if (!mixed) return cudaErrorNotSupported;
    switch (N) {
        case 3: return launch_col_mode<3>(P, mode, s);
        case 4: return launch_col_mode<4>(P, mode, s);
        case 5: return launch_col_mode<5>(P, mode, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace cmdg
