// Device code shared by the diffusive passes (viscous.cu) and the
// hyperdiffusion passes (hyper.cu) on brick meshes: thread layout, closure
// constants in the working precision, the diffusive reference rows, the
// gradient arguments, the second-order flux of the turbulence closures and
// the fused stage kernel with second-order fluxes.
#pragma once

#include "dg_common.cuh"

namespace cmdg {
namespace {

template <int N>
struct VDims {
    static constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, NF = 6 * Nfp;
    static constexpr int NT = (((Np > NF) ? Np : NF) + 31) / 32 * 32;
};

template <typename R>
struct VConst;
template <>
struct VConst<double> {
    static __device__ __forceinline__ double rho_nu(const KParams& P) { return P.ph.rho_nu; }
    static __device__ __forceinline__ double C_smag(const KParams& P) { return P.ph.C_smag; }
    static __device__ __forceinline__ double inv_Pr(const KParams& P) { return P.ph.inv_Pr_turb; }
    static __device__ __forceinline__ double kappa(const KParams& P) { return P.ph.kappa; }
    static __device__ __forceinline__ double MSLP(const KParams& P) { return P.ph.MSLP; }
    static __device__ __forceinline__ double grav(const KParams& P) { return P.ph.grav; }
    static __device__ __forceinline__ double R_d(const KParams& P) { return P.ph.R_d; }
    static __device__ __forceinline__ double D(const KParams& P, int i) { return P.DC64[i]; }
};
template <>
struct VConst<float> {
    static __device__ __forceinline__ float rho_nu(const KParams& P) { return P.rho_nu32; }
    static __device__ __forceinline__ float C_smag(const KParams& P) { return P.C_smag32; }
    static __device__ __forceinline__ float inv_Pr(const KParams& P) { return P.inv_Pr32; }
    static __device__ __forceinline__ float kappa(const KParams& P) { return P.kappa32; }
    static __device__ __forceinline__ float MSLP(const KParams& P) { return P.MSLP32; }
    static __device__ __forceinline__ float grav(const KParams& P) { return P.grav32; }
    static __device__ __forceinline__ float R_d(const KParams& P) { return (float)P.ph.R_d; }
    static __device__ __forceinline__ float D(const KParams& P, int i) { return P.DC32[i]; }
};

template <typename R>
struct VLevel {
    R thv_ref, dthv_ref, ht_ref, dht_ref, p_ref, rho_ref;
};
template <typename R>
__device__ __forceinline__ VLevel<R> load_vlevel(const KParams& P, int lev);
template <>
__device__ __forceinline__ VLevel<double> load_vlevel<double>(const KParams& P, int lev) {
    const double2* L = reinterpret_cast<const double2*>(P.lvv64 + (size_t)lev * VV_NFIELDS);
    const double2 a = __ldg(L), b = __ldg(L + 1), c = __ldg(L + 2);
    return VLevel<double>{a.x, a.y, b.x, b.y, c.x, c.y};
}
template <>
__device__ __forceinline__ VLevel<float> load_vlevel<float>(const KParams& P, int lev) {
    const float4* L = reinterpret_cast<const float4*>(P.lvv32 + (size_t)lev * VV_NFIELDS);
    const float4 a = __ldg(L), b = __ldg(L + 1);
    return VLevel<float>{a.x, a.y, a.z, a.w, b.x, b.y};
}

__device__ __forceinline__ double pow_r(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float pow_r(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double log1p_r(double x) { return log1p(x); }
__device__ __forceinline__ double expm1_r(double x) { return expm1(x); }
// FP32 log(1 + x) and exp(y) - 1 for the mixed path's relative
// perturbations (T'/T_ref, p'/p_ref, and their theta_v combination), which
// are almost always below 1/32 in magnitude: there the truncated Taylor
// series (Mercator's series x - x^2/2 + ... - x^6/6; y + y^2/2 + ... +
// y^5/120) in Horner form, whose first omitted terms are below 2e-10 of
// the value, far under FP32 rounding; elsewhere the library functions.
__device__ __forceinline__ float log1p_r(float x) {
    if (fabsf(x) < 0.03125f) {
        float h = fmaf(-x, 1.0f / 6.0f, 0.2f);
        h = fmaf(-x, h, 0.25f);
        h = fmaf(-x, h, 1.0f / 3.0f);
        h = fmaf(-x, h, 0.5f);
        h = fmaf(-x, h, 1.0f);
        return x * h;
    }
    return log1pf(x);
}
__device__ __forceinline__ float expm1_r(float y) {
    if (fabsf(y) < 0.03125f) {
        float h = fmaf(y, 1.0f / 120.0f, 1.0f / 24.0f);
        h = fmaf(y, h, 1.0f / 6.0f);
        h = fmaf(y, h, 0.5f);
        h = fmaf(y, h, 1.0f);
        return y * h;
    }
    return expm1f(y);
}
// weak-form derivative coefficient Dhat[i] from the kernel's parameter bank
// (a constant-cache read with the thread's row index, no shared memory)
template <typename R>
__device__ __forceinline__ R dhat_p(const KParams& P, int i);
template <>
__device__ __forceinline__ float dhat_p<float>(const KParams& P, int i) {
    return P.DhatC32[i];
}
template <>
__device__ __forceinline__ double dhat_p<double>(const KParams& P, int i) {
    return P.DhatC64[i];
}
// spacing to the next representable value above x >= 0 (Julia's eps(x))
__device__ __forceinline__ double ulp_r(double x) { return __longlong_as_double(__double_as_longlong(x) + 1) - x; }
__device__ __forceinline__ float ulp_r(float x) { return __int_as_float(__float_as_int(x) + 1) - x; }

// Gradient arguments G = (u, v, w, h_tot, theta_v) of a node; in the mixed
// form with a reference state, G[3] and G[4] are perturbations.
template <typename R, bool MIXED, bool SMAG>
__device__ __forceinline__ void grad_args(const KParams& P, const R q[NSTATE], const Level<R>& lv,
                                          const VLevel<R>& vv, R G[5]) {
    const Physics& ph = P.ph;
    const R gm1 = KConst<R>::gm1(P);
    const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
    const R rinv = MIXED ? rcp_r(rho) : R(1) / rho;
    G[0] = q[1] * rinv;
    G[1] = q[2] * rinv;
    G[2] = q[3] * rinv;
    const R ke2 = q[1] * G[0] + q[2] * G[1] + q[3] * G[2];
    G[4] = 0;
    if (MIXED && ph.ref_state) {
        const R pp = gm1 * (q[4] - R(0.5) * ke2) + q[0] * lv.crho;  // p'
        const R Hp = q[4] + pp;                                       // H' = rhoe' + p'
        G[3] = (Hp * vv.rho_ref - lv.href * q[0]) * (rinv * rcp_r(vv.rho_ref));
        if (SMAG) {
            const R ipr = rcp_r(vv.p_ref);
            const R rT = (pp * vv.rho_ref - vv.p_ref * q[0]) * (rinv * ipr);
            const R lnr = log1p_r(rT) - VConst<R>::kappa(P) * log1p_r(pp * ipr);
            G[4] = vv.thv_ref * expm1_r(lnr);
        }
    } else {
        const R p = gm1 * (q[4] - R(0.5) * ke2) + rho * lv.crho;
        G[3] = (q[4] + p) * rinv;
        if (SMAG) {
            const R T = p * rinv / VConst<R>::R_d(P);
            G[4] = T / pow_r(p / VConst<R>::MSLP(P), VConst<R>::kappa(P));
        }
    }
}

template <typename R, int TURB>
__device__ __forceinline__ void flux2(const KParams& P, R rho, R rinv, const R ru[3], const R gf[NGF],
                                      const R khat[3], R Delta, R F[3][NSTATE]);

// brick form: khat = (0, 0, khat_z)
template <typename R, int TURB>
__device__ __forceinline__ void flux2(const KParams& P, R rho, R rinv, const R ru[3], const R gf[NGF], R khat_z,
                                      R Delta, R F[3][NSTATE]) {
    const R khat[3] = {R(0), R(0), khat_z};
    flux2<R, TURB>(P, rho, rinv, ru, gf, khat, Delta, F);
}

// Second-order flux rows F[d][s] (fields 1..4; field 0 has none).
template <typename R, int TURB>
__device__ __forceinline__ void flux2(const KParams& P, R rho, R rinv, const R ru[3], const R gf[NGF],
                                      const R khat[3], R Delta, R F[3][NSTATE]) {
    const R S[3][3] = {{gf[3], gf[4], gf[5]}, {gf[4], gf[6], gf[7]}, {gf[5], gf[7], gf[8]}};
    R nu[3], tau[3][3];
    const R invPr = VConst<R>::inv_Pr(P);
    if (TURB == CMDG_TURB_CONSTANT) {
        const R nu0 = VConst<R>::rho_nu(P) * rinv;
        nu[0] = nu[1] = nu[2] = nu0;
        const R trS = S[0][0] + S[1][1] + S[2][2];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                tau[r][c] = (-2 * nu0) * S[r][c];
                if (P.ph.with_divergence && r == c) tau[r][c] += (2 * nu0 / 3) * trS;
            }
    } else {
        const R norm2 = S[0][0] * S[0][0] + 2 * (S[1][0] * S[1][0]) + 2 * (S[2][0] * S[2][0]) + S[1][1] * S[1][1] +
                        2 * (S[2][1] * S[2][1]) + S[2][2] * S[2][2];
        const R normS = sqrt(2 * norm2);
        const R Ri = gf[9] / (normS * normS + ulp_r(normS));
        const R fb2 = sqrt(fmin(fmax(R(1) - Ri * invPr, R(0)), R(1)));
        const R cd = VConst<R>::C_smag(P) * Delta;
        const R nu0 = normS * (cd * cd) + R(1e-5);
        // nu_v = khat (nu . khat), nu_h = nu0 - nu_v, nu = nu_h + nu_v fb2
        const R dnk = nu0 * khat[0] + nu0 * khat[1] + nu0 * khat[2];
        const R nv[3] = {khat[0] * dnk, khat[1] * dnk, khat[2] * dnk};
#pragma unroll
        for (int c = 0; c < 3; ++c) nu[c] = (nu0 - nv[c]) + nv[c] * fb2;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) tau[r][c] = -2 * nu[r] * S[r][c];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        F[d][0] = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) F[d][1 + c] = tau[d][c] * rho;
        const R Dt = (TURB == CMDG_TURB_CONSTANT ? nu[0] : nu[d]) * invPr;
        F[d][4] = (tau[d][0] * ru[0] + tau[d][1] * ru[1] + tau[d][2] * ru[2]) + (-Dt * gf[d]) * rho;
    }
}

// Hyperdiffusive flux rows (HyperdiffViscousFlux, HyperdiffEnthalpyFlux;
// src/Atmos/Model/tendencies_momentum.jl:51-54, tendencies_energy.jl:40-48)
// added to F: hd holds nu grad^3 of (u, v, h_tot) as words 3 c + d (the
// vertical component of u_h = (I - khat khat') u vanishes on a flat brick).
template <typename R>
__device__ __forceinline__ void add_hyper_flux(R rho, const R ru[3], const R hd[9], R F[3][NSTATE]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        F[d][1] += rho * hd[d];
        F[d][2] += rho * hd[3 + d];
        F[d][4] += (hd[d] * ru[0] + hd[3 + d] * ru[1]) + hd[6 + d] * rho;
    }
}

// Stage kernel with second-order fluxes: TURB = the turbulence closure
// (CMDG_TURB_NONE only together with HYPER), HYPER = DryBiharmonic
// hyperdiffusion, whose state nu grad^3 (Np, 9, nelem) is read from P.hd.
// Resident CTAs per SM the FP32 stage kernel is compiled for.  N = 4: 6
// with a closure (measured on the Smagorinsky LES: 183 us per stage against
// 195 us at the compiler's choice of 90 registers, 4 CTAs) and with
// hyperdiffusion alone (64 registers; on the hyperdiffusion bubble 0.528 ms
// per step against 0.547 ms at 5 CTAs and 0.587 ms at 4); 5 with both (72
// registers, where 6 would spill).  N = 5 (224 threads): 4, 72 registers
// (at 6 the closure kernels spilled 160-184 bytes).  FP64: the compiler's
// choice.
template <int N, typename R, int TURB, bool HYPER>
constexpr int vstage_min_ctas() {
    if (sizeof(R) != 4) return 1;
    if (N == 5) return 4;
    return (HYPER && TURB != CMDG_TURB_NONE) ? 5 : 6;
}

template <int N, typename R, bool MIXED, int MODE, int TURB, bool HYPER>
__global__ void __launch_bounds__(VDims<N>::NT, vstage_min_ctas<N, R, TURB, HYPER>())
    viscous_stage_kernel(const KParams P) {
    using Dm = VDims<N>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, NFN = 6 * Nfp, P5N = planar_pad<R>(5 * Np);
    constexpr int ESTRIDE = NSTATE * Np;
    using PL = Planar5<R>;
    using CRV = typename Pair<R>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_node = reinterpret_cast<R*>(smem_raw);                      // planar records: q
    CRV* const s_cr = reinterpret_cast<CRV*>(s_node + P5N);                 // (c, 1/rho)
    R* const s_F = s_node + P5N + planar_pad<R>(2 * Np);                    // total flux, 3 directions
    R* const s_fs = s_F + 3 * P5N;                                          // lifted face flux

    const int e = blockIdx.x, t = threadIdx.x;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    R* __restrict__ Qout = static_cast<R*>(P.Qout);
    const R* __restrict__ GF = static_cast<const R*>(P.gf);
    const R* __restrict__ HDS = static_cast<const R*>(P.hd);
    constexpr bool VISC = TURB != CMDG_TURB_NONE;
    const Physics& ph = P.ph;
    const bool node_thread = t < Np, face_thread = t < 6 * Nfp;
    const bool read_reg = (MODE == 0) ? (P.beta != 0) : !P.first_stage;
    const int* nbr = P.nbr + NBR_STRIDE * e;
    const int ez = __ldg(nbr + 6);
    const int nk = node_thread ? t / Nfp : 0;
    const int nj = node_thread ? (t - nk * Nfp) / Nq : 0;
    const int ni = node_thread ? t - nk * Nfp - nj * Nq : 0;
    const int f = face_thread ? t / Nfp : 0;
    const int fn = face_thread ? t - f * Nfp : 0;
    const int fd = f >> 1, fside = f & 1, oside = fside ^ 1;
    const int fa = fn % Nq, fb = fn / Nq;
    const int vM = fd == 0 ? fside * N + Nq * fn : (fd == 1 ? fa + Nq * (fside * N + Nq * fb) : fn + Nfp * (fside * N));
    const int vP = fd == 0 ? oside * N + Nq * fn : (fd == 1 ? fa + Nq * (oside * N + Nq * fb) : fn + Nfp * (oside * N));
    const R sgn = fside ? R(1) : R(-1);

    // record of this node in the direction-d flux plane (contraction index slowest)
    auto dir_rec = [&](int d) {
        return d == 0 ? ni * Nfp + (nj + Nq * nk) : (d == 1 ? nj * Nfp + (ni + Nq * nk) : t);
    };

    const size_t ebase = (size_t)e * ESTRIDE + t;
    R q[NSTATE], f2[NF2], hd[9];
    double dq_old[NSTATE];
    if (node_thread) {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = Qin[ebase + s * Np];
        if (VISC) {
            // the node's second-order flux rows, formed by the gradient pass
            const R* g = GF + (size_t)e * NF2 * Np + t;
#pragma unroll
            for (int w = 0; w < NF2; ++w) f2[w] = g[(size_t)w * Np];
        }
        if (HYPER) {
#pragma unroll
            for (int w = 0; w < 9; ++w) hd[w] = HDS[(size_t)e * 9 * Np + w * Np + t];
        }
        if (read_reg) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) dq_old[s] = P.dQ[ebase + s * Np];
        }
    }
    const int nb = face_thread ? __ldg(nbr + f) : -1;
    R qp[NSTATE], f2p[4], hdp[3];
    int ezp = ez;
    if (nb >= 0) {
        const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
        if (VISC) {
            // the neighbour's second-order flux row normal to the face
            const R* gn = GF + (size_t)nb * NF2 * Np + (size_t)(4 * fd) * Np + vP;
#pragma unroll
            for (int w = 0; w < 4; ++w) f2p[w] = gn[(size_t)w * Np];
        }
        if (HYPER) {
            // the neighbour's nu grad^3 components normal to the face
            const R* hn = HDS + (size_t)nb * 9 * Np + (size_t)fd * Np + vP;
#pragma unroll
            for (int c = 0; c < 3; ++c) hdp[c] = hn[(size_t)c * 3 * Np];
        }
        if (fd == 2) {
            ezp = ez + (fside ? 1 : -1);
            ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
        }
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};

    // phase 1: node thermodynamics, total (first + second order) volume flux
    R gsrc = 0;
    if (node_thread) {
        const Level<R> lv = load_level<R>(P, ez * Nq + nk);
        const Thermo<R, MIXED> th = thermo<R, MIXED>(q, lv, P);
        PL::st(s_node, Np, t, q);
        s_cr[t] = Pair<R>::make(th.c, th.rinv);
        R F2[3][NSTATE] = {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}};
        const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
        const R ru[3] = {q[1], q[2], q[3]};
        if (VISC) {
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int s = 1; s < NSTATE; ++s) F2[dd][s] = f2[4 * dd + s - 1];
        }
        if (HYPER) add_hyper_flux<R>(rho, ru, hd, F2);
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
            R F[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(q, th, dd, s) + F2[dd][s];
            PL::st(s_F + dd * P5N, Np, dir_rec(dd), F);
        }
        if (ph.gravity) {
            R rho_s = MIXED ? ((ph.ref_state && ph.subtract_off) ? q[0] : lv.rho_ref + q[0])
                            : ((ph.ref_state && ph.subtract_off) ? q[0] - lv.rho_ref : q[0]);
            gsrc = -rho_s * lv.gphiz;
        }
    }
    __syncthreads();

    // phase 2: numerical flux per face node (Rusanov/central + central second order)
    if (face_thread) {
        R qm[NSTATE], Fm[NSTATE], Fp[NSTATE], jr[NSTATE] = {0, 0, 0, 0, 0};
        PL::ld(s_node, Np, vM, qm);
        const CRV cr = s_cr[vM];
        const R c_m = cr.x, ri_m = cr.y;
        const R lam_m = fabs(pick3(fd, qm[1], qm[2], qm[3]) * ri_m) + c_m;
        const Level<R> lvm = load_level<R>(P, ez * Nq + vM / Nfp);
        if (nb >= 0) {
            PL::ld(s_F + fd * P5N, Np, fside * N * Nfp + fn, Fm);  // dir_rec(fd) of vM
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) Fm[s] *= sgn;
            if (MIXED && fd == 2 && ph.numflux == CMDG_FLUX_RUSANOV) {
                const int ej = fside ? ezp : ez;
                const R sj = fside ? R(-1) : R(1);
                jr[0] = sj * (R)P.jump32[2 * ej + 0];
                jr[4] = sj * (R)P.jump32[2 * ej + 1];
            }
        } else {
            // walls: first-order flux only on both sides
            const Thermo<R, MIXED> thm = thermo<R, MIXED>(qm, lvm, P);
            normal_flux<R, MIXED>(qm, thm, fd, sgn, Fm);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
            qp[1] = (fd == 0) ? -qm[1] : qm[1];
            qp[2] = (fd == 1) ? -qm[2] : qm[2];
            qp[3] = (fd == 2) ? -qm[3] : qm[3];
        }
        const Level<R> lvp = nb >= 0 ? load_level<R>(P, ezp * Nq + vP / Nfp) : lvm;
        const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
        normal_flux<R, MIXED>(qp, thp, fd, sgn, Fp);
        if (nb >= 0) {
            const R rho = MIXED ? lvp.rho_ref + qp[0] : qp[0];
            const R ru[3] = {qp[1], qp[2], qp[3]};
            if (VISC) {
#pragma unroll
                for (int s = 1; s < NSTATE; ++s) Fp[s] += sgn * f2p[s - 1];
            }
            if (HYPER) {
                Fp[1] += sgn * (rho * hdp[0]);
                Fp[2] += sgn * (rho * hdp[1]);
                Fp[4] += sgn * ((hdp[0] * ru[0] + hdp[1] * ru[1]) + hdp[2] * rho);
            }
        }
        const R lam_p = fabs(pick3(fd, thp.u[0], thp.u[1], thp.u[2])) + thp.c;
        const R lift = pick3(fd, xi[0], xi[1], xi[2]) * KConst<R>::inv_w0(P);
        const R hmw = (ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
        const R hl = R(0.5) * lift, pl = hmw * lift;
        R fs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) fs[s] = hl * (Fm[s] + Fp[s]) + pl * ((qm[s] - qp[s]) + jr[s]);
        PL::st(s_fs, NFN, f * Nfp + fn, fs);
    }
    __syncthreads();

    // phase 3: volume contraction, face terms, source, update
    int bad = 0;
    if (node_thread) {
        R acc1[NSTATE] = {0, 0, 0, 0, 0}, acc2[NSTATE] = {0, 0, 0, 0, 0}, acc3[NSTATE] = {0, 0, 0, 0, 0};
        const int L1 = nj + Nq * nk, L2 = ni + Nq * nk, L3 = ni + Nq * nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            R v1[NSTATE], v2[NSTATE], v3[NSTATE];
            PL::ld(s_F, Np, L1 + n * Nfp, v1);
            PL::ld(s_F + P5N, Np, L2 + n * Nfp, v2);
            PL::ld(s_F + 2 * P5N, Np, L3 + n * Nfp, v3);
            const R d1 = dhat_p<R>(P, ni * Nq + n), d2 = dhat_p<R>(P, nj * Nq + n), d3 = dhat_p<R>(P, nk * Nq + n);
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
        auto sub_face = [&](int ff, int idx) {
            R v[NSTATE];
            PL::ld(s_fs, NFN, ff * Nfp + idx, v);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) rhs[s] -= v[s];
        };
        if (ni == 0) sub_face(0, nj + Nq * nk);
        if (ni == N) sub_face(1, nj + Nq * nk);
        if (nj == 0) sub_face(2, ni + Nq * nk);
        if (nj == N) sub_face(3, ni + Nq * nk);
        if (nk == 0) sub_face(4, ni + Nq * nj);
        if (nk == N) sub_face(5, ni + Nq * nj);
        rhs[3] += gsrc;
        const R rkb_dt = KConst<R>::rkb_dt(P);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) {
            if (!isfinite(rhs[s])) bad = 1;
            const size_t idx = ebase + s * Np;
            if (MODE == 0) {
                double out = P.alpha * (double)rhs[s];
                if (read_reg) out = fma(P.beta, dq_old[s], out);
                P.dQ[idx] = out;
            } else {
                double dq;
                if (MIXED) {
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
    // one pass per CTA: no barrier at the end, one vote per warp
    if (__any_sync(0xffffffffu, bad) && (t & 31) == 0) atomicOr(P.status, 1u);
}

template <typename K>
cudaError_t opt_in(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}


// Launches the stage kernel with second-order fluxes for closure `turb`.
template <int N, typename R, bool MIXED, int MODE, bool HYPER>
cudaError_t launch_vstage_typed(const KParams& P, int turb, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    constexpr size_t bytes =
        sizeof(R) * (4 * planar_pad<R>(5 * Np) + planar_pad<R>(2 * Np) + planar_pad<R>(30 * Nfp) + Nq * Nq);
    cudaError_t e;
    if (turb == CMDG_TURB_SMAGORINSKY) {
        auto k = viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_SMAGORINSKY, HYPER>;
        if ((e = opt_in(k, bytes)) != cudaSuccess) return e;
        k<<<P.nelem, VDims<N>::NT, bytes, s>>>(P);
    } else if (turb == CMDG_TURB_CONSTANT) {
        auto k = viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_CONSTANT, HYPER>;
        if ((e = opt_in(k, bytes)) != cudaSuccess) return e;
        k<<<P.nelem, VDims<N>::NT, bytes, s>>>(P);
    } else {
        if constexpr (HYPER) {
            auto k = viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_NONE, true>;
            if ((e = opt_in(k, bytes)) != cudaSuccess) return e;
            k<<<P.nelem, VDims<N>::NT, bytes, s>>>(P);
        } else {
            return cudaErrorInvalidValue;
        }
    }
    return cudaGetLastError();
}

template <int N, bool HYPER>
cudaError_t launch_vstage_N(const KParams& P, bool mixed, int mode, int turb, cudaStream_t s) {
    if (mixed)
        return mode == 0 ? launch_vstage_typed<N, float, true, 0, HYPER>(P, turb, s)
                         : launch_vstage_typed<N, float, true, 1, HYPER>(P, turb, s);
    return mode == 0 ? launch_vstage_typed<N, double, false, 0, HYPER>(P, turb, s)
                     : launch_vstage_typed<N, double, false, 1, HYPER>(P, turb, s);
}

}  // namespace
}  // namespace cmdg
