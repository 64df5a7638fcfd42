// Diffusive passes of the DG tendency on brick meshes (sm_103a):
//
//  * gradient kernel: the auxiliary gradient of G = (u, v, w, h_tot[, theta_v])
//    in strong form, Sigma = D G + M^-1 L Mf (G* - n G-), with the central
//    gradient flux G* = n (G- + G+)/2 on interior faces and G* = n G+ of the
//    FreeSlip boundary state on walls, transformed into the gradient-flux
//    words grad h_tot, S = sym(grad u) and N^2 = grad theta_v . grad Phi /
//    theta_v (volume_gradients! and dgsem_interface_gradients!,
//    src/Numerics/DGMethods/DGModel_kernels.jl:934-1651;
//    compute_gradient_argument!/compute_gradient_flux!,
//    src/Atmos/Model/AtmosModel.jl:622-744, src/Atmos/Model/energy.jl:20-59,
//    src/Common/TurbulenceClosures/TurbulenceClosures.jl:351-362, 446-470);
//  * viscous stage kernel: the fused tendency + LSRK stage kernel of stage.cu
//    with the second-order flux added to the volume flux and the central
//    second-order numerical flux on interior faces (zero on FreeSlip /
//    Insulating walls, src/Atmos/Model/boundaryconditions.jl:113-185), for
//    ConstantDynamicViscosity and SmagorinskyLilly (turbulence_tensors,
//    TurbulenceClosures.jl:199-225, 368-404, 472-505; ViscousStress,
//    ViscousFlux, DiffEnthalpyFlux, src/Atmos/Model/tendencies_momentum.jl:37-42,
//    tendencies_energy.jl:27-31, 51-56).
//
// Mixed precision: h_tot and theta_v are carried as FP32 perturbations about
// the level's FP64 reference values, formed without cancellation:
//   h' = (H' rho_ref - H_ref rho') / (rho rho_ref),  H = rhoe + p,
//   theta_v' = theta_v_ref expm1(log1p(T'/T_ref) - kappa log1p(p'/p_ref)),
//   T'/T_ref = (p' rho_ref - p_ref rho') / (rho p_ref);
// their reference parts enter through FP64-computed DG z-derivatives.
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
__device__ __forceinline__ float log1p_r(float x) { return log1pf(x); }
__device__ __forceinline__ double expm1_r(double x) { return expm1(x); }
__device__ __forceinline__ float expm1_r(float x) { return expm1f(x); }
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
    const R rinv = R(1) / rho;
    G[0] = q[1] * rinv;
    G[1] = q[2] * rinv;
    G[2] = q[3] * rinv;
    const R ke2 = q[1] * G[0] + q[2] * G[1] + q[3] * G[2];
    G[4] = 0;
    if (MIXED && ph.ref_state) {
        const R pp = gm1 * (q[4] - R(0.5) * ke2) + q[0] * lv.crho;  // p'
        const R Hp = q[4] + pp;                                       // H' = rhoe' + p'
        G[3] = (Hp * vv.rho_ref - lv.href * q[0]) * (rinv / vv.rho_ref);
        if (SMAG) {
            const R rT = (pp * vv.rho_ref - vv.p_ref * q[0]) * (rinv / vv.p_ref);
            const R lnr = log1p_r(rT) - VConst<R>::kappa(P) * log1p_r(pp / vv.p_ref);
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

template <int N, typename R, bool MIXED, bool SMAG>
__global__ void __launch_bounds__(VDims<N>::NT) gradient_kernel(const KParams P, const void* Qv, R* __restrict__ gf) {
    using Dm = VDims<N>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, NFN = 6 * Nfp;
    constexpr int ESTRIDE = NSTATE * Np;
    using PL = Planar5<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_q = reinterpret_cast<R*>(smem_raw);      // planar records: states
    R* const s_G = s_q + planar_pad<R>(5 * Np);            // gradient arguments
    R* const s_dG = s_G + planar_pad<R>(5 * Np);           // face terms
    R* const s_D = s_dG + planar_pad<R>(5 * NFN);          // strong-form D

    const int e = blockIdx.x, t = threadIdx.x;
    const R* __restrict__ Qin = static_cast<const R*>(Qv);
    const bool node_thread = t < Np, face_thread = t < 6 * Nfp;
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
    if (t < Nq * Nq) s_D[t] = VConst<R>::D(P, t);

    R q[NSTATE], qp[NSTATE];
    if (node_thread) {
        const R* qe = Qin + (size_t)e * ESTRIDE + t;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = qe[s * Np];
    }
    const int nb = face_thread ? __ldg(nbr + f) : -1;
    int levp = ez * Nq + vM / Nfp;
    if (nb >= 0) {
        const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
        int ezp = ez;
        if (fd == 2) {
            ezp = ez + (fside ? 1 : -1);
            ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
        }
        levp = ezp * Nq + vP / Nfp;
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};

    // phase 1: gradient arguments of the element's nodes
    if (node_thread) {
        const int lev = ez * Nq + nk;
        R G[5];
        grad_args<R, MIXED, SMAG>(P, q, load_level<R>(P, lev), load_vlevel<R>(P, lev), G);
        PL::st(s_q, Np, t, q);
        PL::st(s_G, Np, t, G);
    }
    __syncthreads();

    // phase 2: face terms lift n (G+ - G-) c, c = 1/2 inside, 1 on walls
    if (face_thread) {
        R Gm[5], Gp[5];
        PL::ld(s_G, Np, vM, Gm);
        R c;
        if (nb >= 0) {
            grad_args<R, MIXED, SMAG>(P, qp, load_level<R>(P, levp), load_vlevel<R>(P, levp), Gp);
            c = R(0.5);
        } else {
            // FreeSlip state for the gradient flux: rhou+ = rhou- - (rhou-.n) n
            R qb[NSTATE];
            PL::ld(s_q, Np, vM, qb);
            qb[1 + 0] = fd == 0 ? R(0) : qb[1];
            qb[1 + 1] = fd == 1 ? R(0) : qb[2];
            qb[1 + 2] = fd == 2 ? R(0) : qb[3];
            grad_args<R, MIXED, SMAG>(P, qb, load_level<R>(P, levp), load_vlevel<R>(P, levp), Gp);
            c = R(1);
        }
        const R sgn = fside ? R(1) : R(-1);
        const R w = c * sgn * pick3(fd, xi[0], xi[1], xi[2]) * KConst<R>::inv_w0(P);
        R out[5];
#pragma unroll
        for (int g = 0; g < 5; ++g) out[g] = w * (Gp[g] - Gm[g]);
        PL::st(s_dG, NFN, f * Nfp + fn, out);
    }
    __syncthreads();

    // phase 3: volume gradient (strong form), face terms, reference part, transform
    if (node_thread) {
        R g1[5] = {0, 0, 0, 0, 0}, g2[5] = {0, 0, 0, 0, 0}, g3[5] = {0, 0, 0, 0, 0};
        const int L1 = Nq * (nj + Nq * nk), L2 = ni + Nfp * nk, L3 = ni + Nq * nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            R v1[5], v2[5], v3[5];
            PL::ld(s_G, Np, L1 + n, v1);
            PL::ld(s_G, Np, L2 + n * Nq, v2);
            PL::ld(s_G, Np, L3 + n * Nfp, v3);
            const R d1 = s_D[ni * Nq + n], d2 = s_D[nj * Nq + n], d3 = s_D[nk * Nq + n];
#pragma unroll
            for (int g = 0; g < 5; ++g) {
                g1[g] = fma(d1, v1[g], g1[g]);
                g2[g] = fma(d2, v2[g], g2[g]);
                g3[g] = fma(d3, v3[g], g3[g]);
            }
        }
#pragma unroll
        for (int g = 0; g < 5; ++g) {
            g1[g] *= xi[0];
            g2[g] *= xi[1];
            g3[g] *= xi[2];
        }
        auto add = [&](int ff, int idx, R* gd) {
            R v[5];
            PL::ld(s_dG, NFN, ff * Nfp + idx, v);
#pragma unroll
            for (int g = 0; g < 5; ++g) gd[g] += v[g];
        };
        if (ni == 0) add(0, nj + Nq * nk, g1);
        if (ni == N) add(1, nj + Nq * nk, g1);
        if (nj == 0) add(2, ni + Nq * nk, g2);
        if (nj == N) add(3, ni + Nq * nk, g2);
        if (nk == 0) add(4, ni + Nq * nj, g3);
        if (nk == N) add(5, ni + Nq * nj, g3);
        const int lev = ez * Nq + nk;
        const VLevel<R> vv = load_vlevel<R>(P, lev);
        R thv = 0;
        if (SMAG) {
            thv = s_G[4 * Np + t];
        }
        if (MIXED && P.ph.ref_state) {
            g3[3] += vv.dht_ref;
            if (SMAG) {
                g3[4] += vv.dthv_ref;
                thv += vv.thv_ref;
            }
        }
        R out[NGF];
        out[0] = g1[3];
        out[1] = g2[3];
        out[2] = g3[3];
        out[3] = g1[0];
        out[4] = (g2[0] + g1[1]) / R(2);
        out[5] = (g3[0] + g1[2]) / R(2);
        out[6] = g2[1];
        out[7] = (g3[1] + g2[2]) / R(2);
        out[8] = g3[2];
        out[9] = SMAG ? (g3[4] * load_level<R>(P, lev).gphiz) / thv : R(0);
        R* o = gf + (size_t)e * NGF * Np + t;
#pragma unroll
        for (int s = 0; s < NGF; ++s) o[s * Np] = out[s];
    }
}

// Second-order flux rows F[d][s] (fields 1..4; field 0 has none).
template <typename R, int TURB>
__device__ __forceinline__ void flux2(const KParams& P, R rho, R rinv, const R ru[3], const R gf[NGF], R khat_z,
                                      R Delta, R F[3][NSTATE]) {
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
        // nu_v = khat (nu . khat), nu_h = nu0 - nu_v, nu = nu_h + nu_v fb2 (khat = (0, 0, khat_z) on a brick)
        const R dnk = nu0 * khat_z;
        const R nv[3] = {R(0), R(0), khat_z * dnk};
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

template <typename R>
__device__ __forceinline__ void ld_gf(const R* gf, size_t base, int Np, R out[NGF]) {
#pragma unroll
    for (int s = 0; s < NGF; ++s) out[s] = gf[base + (size_t)s * Np];
}

template <int N, typename R, bool MIXED, int MODE, int TURB>
// FP32: 6 resident CTAs per SM (measured on the Smagorinsky LES: 183 us per
// stage against 195 us at the compiler's choice of 90 registers, 4 CTAs)
__global__ void __launch_bounds__(VDims<N>::NT, (sizeof(R) == 4 ? 6 : 1)) viscous_stage_kernel(const KParams P) {
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
    R* const s_D = s_fs + planar_pad<R>(5 * NFN);                           // Dhat

    const int e = blockIdx.x, t = threadIdx.x;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    R* __restrict__ Qout = static_cast<R*>(P.Qout);
    const R* __restrict__ GF = static_cast<const R*>(P.gf);
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
    if (t < Nq * Nq) s_D[t] = static_cast<const R*>(P.Dhat)[t];

    const size_t ebase = (size_t)e * ESTRIDE + t;
    R q[NSTATE], g[NGF];
    double dq_old[NSTATE];
    if (node_thread) {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = Qin[ebase + s * Np];
        ld_gf<R>(GF, (size_t)e * NGF * Np + t, Np, g);
        if (read_reg) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) dq_old[s] = P.dQ[ebase + s * Np];
        }
    }
    const int nb = face_thread ? __ldg(nbr + f) : -1;
    R qp[NSTATE], gp[NGF];
    int ezp = ez;
    if (nb >= 0) {
        const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
        ld_gf<R>(GF, (size_t)nb * NGF * Np + vP, Np, gp);
        if (fd == 2) {
            ezp = ez + (fside ? 1 : -1);
            ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
        }
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};
    // Smagorinsky filter width, lengthscale = 2 / (cbrt(det dxi/dx) N) (src/Numerics/Mesh/Geometry.jl:121-122)
    const R Delta = R(2) / (cbrt(xi[0] * xi[1] * xi[2]) * R(N));

    // phase 1: node thermodynamics, total (first + second order) volume flux
    R gsrc = 0;
    if (node_thread) {
        const Level<R> lv = load_level<R>(P, ez * Nq + nk);
        const Thermo<R, MIXED> th = thermo<R, MIXED>(q, lv, P);
        PL::st(s_node, Np, t, q);
        s_cr[t] = Pair<R>::make(th.c, th.rinv);
        R F2[3][NSTATE];
        const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
        const R ru[3] = {q[1], q[2], q[3]};
        flux2<R, TURB>(P, rho, th.rinv, ru, g, lv.gphiz / VConst<R>::grav(P), Delta, F2);
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
            R F[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) F[s] = flux_d<R, MIXED>(q, th, dd, s) + F2[dd][s];
            PL::st(s_F + dd * P5N, Np, t, F);
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
            PL::ld(s_F + fd * P5N, Np, vM, Fm);
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
            R F2[3][NSTATE];
            const R rho = MIXED ? lvp.rho_ref + qp[0] : qp[0];
            const R ru[3] = {qp[1], qp[2], qp[3]};
            flux2<R, TURB>(P, rho, thp.rinv, ru, gp, lvp.gphiz / VConst<R>::grav(P), Delta, F2);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) Fp[s] += sgn * pick3(fd, F2[0][s], F2[1][s], F2[2][s]);
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
        const int L1 = Nq * (nj + Nq * nk), L2 = ni + Nfp * nk, L3 = ni + Nq * nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            R v1[NSTATE], v2[NSTATE], v3[NSTATE];
            PL::ld(s_F, Np, L1 + n, v1);
            PL::ld(s_F + P5N, Np, L2 + n * Nq, v2);
            PL::ld(s_F + 2 * P5N, Np, L3 + n * Nfp, v3);
            const R d1 = s_D[ni * Nq + n], d2 = s_D[nj * Nq + n], d3 = s_D[nk * Nq + n];
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

template <int N, typename R, bool MIXED>
cudaError_t launch_grad_typed(const KParams& P, const void* Q, void* gf, int turb, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    constexpr size_t bytes = sizeof(R) * (2 * planar_pad<R>(5 * Np) + planar_pad<R>(30 * Nfp) + Nq * Nq);
    cudaError_t e;
    if (turb == CMDG_TURB_SMAGORINSKY) {
        if ((e = opt_in(gradient_kernel<N, R, MIXED, true>, bytes)) != cudaSuccess) return e;
        gradient_kernel<N, R, MIXED, true><<<P.nelem, VDims<N>::NT, bytes, s>>>(P, Q, static_cast<R*>(gf));
    } else {
        if ((e = opt_in(gradient_kernel<N, R, MIXED, false>, bytes)) != cudaSuccess) return e;
        gradient_kernel<N, R, MIXED, false><<<P.nelem, VDims<N>::NT, bytes, s>>>(P, Q, static_cast<R*>(gf));
    }
    return cudaGetLastError();
}

template <int N, typename R, bool MIXED, int MODE>
cudaError_t launch_vstage_typed(const KParams& P, int turb, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    constexpr size_t bytes =
        sizeof(R) * (4 * planar_pad<R>(5 * Np) + planar_pad<R>(2 * Np) + planar_pad<R>(30 * Nfp) + Nq * Nq);
    cudaError_t e;
    if (turb == CMDG_TURB_SMAGORINSKY) {
        if ((e = opt_in(viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_SMAGORINSKY>, bytes)) != cudaSuccess) return e;
        viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_SMAGORINSKY><<<P.nelem, VDims<N>::NT, bytes, s>>>(P);
    } else {
        if ((e = opt_in(viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_CONSTANT>, bytes)) != cudaSuccess) return e;
        viscous_stage_kernel<N, R, MIXED, MODE, CMDG_TURB_CONSTANT><<<P.nelem, VDims<N>::NT, bytes, s>>>(P);
    }
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_grad_N(const KParams& P, const void* Q, void* gf, bool mixed, int turb, cudaStream_t s) {
    return mixed ? launch_grad_typed<N, float, true>(P, Q, gf, turb, s)
                 : launch_grad_typed<N, double, false>(P, Q, gf, turb, s);
}

template <int N>
cudaError_t launch_vstage_N(const KParams& P, bool mixed, int mode, int turb, cudaStream_t s) {
    if (mixed)
        return mode == 0 ? launch_vstage_typed<N, float, true, 0>(P, turb, s)
                         : launch_vstage_typed<N, float, true, 1>(P, turb, s);
    return mode == 0 ? launch_vstage_typed<N, double, false, 0>(P, turb, s)
                     : launch_vstage_typed<N, double, false, 1>(P, turb, s);
}

}  // namespace

int launch_gradient(Model* md, const void* Qin, void* gf_out, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    LaunchArgs a;
    a.Qin = Qin;
    a.Qout = nullptr;
    a.dQ = nullptr;
    a.alpha = a.beta = a.rka = a.rkb_dt = 0;
    a.mode = 0;
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    const int turb = md->prm.turbulence;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_grad_N<2>(P, Qin, gf_out, mixed, turb, s); break;
        case 3: err = launch_grad_N<3>(P, Qin, gf_out, mixed, turb, s); break;
        case 4: err = launch_grad_N<4>(P, Qin, gf_out, mixed, turb, s); break;
        case 5: err = launch_grad_N<5>(P, Qin, gf_out, mixed, turb, s); break;
        default: set_error("no gradient kernel for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("gradient kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

int launch_viscous_stage(Model* md, const LaunchArgs& a, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    // gradient pass of this stage's input state, then the tendency / stage update
    int rc = launch_gradient(md, a.Qin, md->d_gf, s);
    if (rc) return rc;
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    const int turb = md->prm.turbulence;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_vstage_N<2>(P, mixed, a.mode, turb, s); break;
        case 3: err = launch_vstage_N<3>(P, mixed, a.mode, turb, s); break;
        case 4: err = launch_vstage_N<4>(P, mixed, a.mode, turb, s); break;
        case 5: err = launch_vstage_N<5>(P, mixed, a.mode, turb, s); break;
        default: set_error("no viscous stage kernel for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("viscous stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
