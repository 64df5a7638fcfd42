// Hyperdiffusion passes on the stacked cubed shell (sm_103a): the three
// passes of hyper.cu with per-node geometry, for the DryBiharmonic closure
// with SphericalOrientation (src/Common/TurbulenceClosures/
// TurbulenceClosures.jl:793-848):
//
//  * shell_hyper_grad_kernel: gradients of the GradientLaplacian states
//    u_h = (I - khat khat') u (khat = grad Phi / g at the node, three
//    components on a sphere) and h_tot, strong form dxi_d/dx_j dG/dxi_d with
//    the interface correction vMI sM n_j c (G+ - G-), c = 1/2 inside and 1 on
//    walls with the FreeSlip gradient state (volume_gradients!,
//    dgsem_interface_gradients!, DGModel_kernels.jl:934-1651);
//  * shell_hyper_div_kernel: laplacians -J^-1 Dhat (J dxi_d/dx . grad G)
//    plus vMI sM (grad G- + grad G+) . n / 2, grad G+ = grad G- on walls
//    (DGModel_kernels.jl:2132-2495, NumericalFluxes.jl:720-730);
//  * shell_hyper_glap_kernel: nu_4 grad(lap) in strong form with
//    vMI sM n (lap+ - lap-)/2 inside, zero on walls (DGModel_kernels.jl:
//    2525-3000, NumericalFluxes.jl:768-790), nu_4 per node from
//    lengthscale_horizontal (src/Numerics/Mesh/Geometry.jl:129-151).
//
// The normals, surface Jacobians and lift weights come from J dxi_d/dx at the
// face node, as in the cubed-shell stage kernel (Metrics.jl:431-724).  In
// mixed precision the FP32 passes carry h' = h_tot - h_ref(node); the
// reference part nu_4 grad lap h_ref is computed once by the FP64 passes on
// the reference state at rest (the passes are linear in their argument) and
// added in the last pass.
#include <algorithm>
#include <cmath>

#include "shell_common.cuh"
#include "viscous_common.cuh"

namespace cmdg {
namespace {

template <int N>
struct ShellIdx {
    static constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    int ni, nj, nk, f, fn, fd, fside, vM, kM;
    bool node, face;
    __device__ __forceinline__ explicit ShellIdx(int t) {
        node = t < Np;
        face = t < 6 * Nfp;
        nk = node ? t / Nfp : 0;
        nj = node ? (t - nk * Nfp) / Nq : 0;
        ni = node ? t - nk * Nfp - nj * Nq : 0;
        f = face ? t / Nfp : 0;
        fn = face ? t - f * Nfp : 0;
        fd = f >> 1;
        fside = f & 1;
        const int fa = fn % Nq, fb = fn / Nq;
        vM = fd == 0 ? fside * N + Nq * fn : (fd == 1 ? fa + Nq * (fside * N + Nq * fb) : fn + Nfp * (fside * N));
        kM = vM / Nfp;
    }
    __device__ __forceinline__ int on_face(int ff) const {
        return ff < 2 ? nj + Nq * nk : (ff < 4 ? ni + Nq * nk : ni + Nq * nj);
    }
};

// Unit outward normal, and the lift weight vMI sM = |J dxi_fd/dx| / (J w_0),
// of face node vM (face direction fd, sign sgn) from the element's kernel
// geometry g.
template <typename R>
__device__ __forceinline__ R shell_face_normal(const KParams& P, const R* g, int Np, int fd, R sgn, int vM, R nv[3]) {
    const R j0 = g[(KG_JXI + fd * 3 + 0) * Np + vM];
    const R j1 = g[(KG_JXI + fd * 3 + 1) * Np + vM];
    const R j2 = g[(KG_JXI + fd * 3 + 2) * Np + vM];
    const R sJ = sqrt_r(j0 * j0 + j1 * j1 + j2 * j2);
    const R rs = rcp_r(sJ);
    nv[0] = sgn * j0 * rs;
    nv[1] = sgn * j1 * rs;
    nv[2] = sgn * j2 * rs;
    return sJ * g[KG_INVJ * Np + vM] * KConst<R>::inv_w0(P);
}

// GradientLaplacian arguments (u_h[0..2], h_tot) of a state at a node with
// reference row lv (per-node parts included) and geometry g; in the mixed
// form h_tot is the perturbation h' = (H' rho_ref - H_ref rho') / (rho rho_ref)
// PROJECT = false: the gradient arguments of the diffusive closures, u and
// h_tot (AtmosModel.jl:622-650, energy.jl:20-31)
// NA = 5 adds theta_v = T / (p / MSLP)^kappa (SmagorinskyLilly's N^2,
// TurbulenceClosures.jl:446-454); in the mixed form the perturbation
// theta_v' = theta_v_ref expm1(log1p(T'/T_ref) - kappa log1p(p'/p_ref)),
// formed without cancelling against the reference value
template <typename R, bool MIXED, bool PROJECT = true, int NA = 4>
__device__ __forceinline__ void shell_hyper_args(const KParams& P, const R q[NSTATE], const Level<R>& lv, const R* g,
                                                 int Np, int n, R H[NA]) {
    const R gm1 = KConst<R>::gm1(P);
    const R ig = R(1) / VConst<R>::grav(P);
    const R k[3] = {g[(KG_GPHI + 0) * Np + n] * ig, g[(KG_GPHI + 1) * Np + n] * ig, g[(KG_GPHI + 2) * Np + n] * ig};
    const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
    const R rinv = R(1) / rho;
    const R u[3] = {q[1] * rinv, q[2] * rinv, q[3] * rinv};
    const R ku = k[0] * u[0] + k[1] * u[1] + k[2] * u[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) H[c] = PROJECT ? u[c] - k[c] * ku : u[c];
    const R ke2 = q[1] * u[0] + q[2] * u[1] + q[3] * u[2];
    if (MIXED && P.ph.ref_state) {
        const R pp = gm1 * (q[4] - R(0.5) * ke2) + q[0] * lv.crho;
        H[3] = ((q[4] + pp) * lv.rho_ref - lv.href * q[0]) * (rinv / lv.rho_ref);
        if (NA == 5) {
            const R kappa = VConst<R>::kappa(P);
            const R rT = (pp * lv.rho_ref - lv.p_ref * q[0]) * (rinv / lv.p_ref);  // T'/T_ref
            const R lnr = log1p_r(rT) - kappa * log1p_r(pp / lv.p_ref);
            const R T_ref = lv.p_ref / (lv.rho_ref * VConst<R>::R_d(P));
            const R thv_ref = T_ref / pow_r(lv.p_ref / VConst<R>::MSLP(P), kappa);
            H[NA - 1] = thv_ref * expm1_r(lnr);
        }
    } else {
        const R p = gm1 * (q[4] - R(0.5) * ke2) + rho * lv.crho;
        H[3] = (q[4] + p) * rinv;
        if (NA == 5) {
            const R T = p * rinv / VConst<R>::R_d(P);
            H[NA - 1] = T / pow_r(p / VConst<R>::MSLP(P), VConst<R>::kappa(P));
        }
    }
    if (P.mms_zero_h) H[3] = R(0);  // total_specific_enthalpy := 0 (mms_bc_atmos.jl:45-48)
}

// strong-form gradient of 4 node fields s_X[4][Np] at this node thread,
// dxi_d/dx_j dX/dxi_d, plus the staged face terms s_dF[(3 s + j) NFN + face node]
template <int N, typename R, int NA = 4>
__device__ __forceinline__ void shell_strong_gradient(const ShellIdx<N>& x, const R* s_X, const R* s_dF, const R* s_D,
                                                      const R* g, int t, bool horiz, R out[3 * NA]) {
    constexpr int Nq = N + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq, NFN = 6 * Nfp;
    R a[NA][3];
#pragma unroll
    for (int s = 0; s < NA; ++s) a[s][0] = a[s][1] = a[s][2] = R(0);
    const int L1 = Nq * (x.nj + Nq * x.nk), L2 = x.ni + Nfp * x.nk, L3 = x.ni + Nq * x.nj;
#pragma unroll
    for (int n = 0; n < Nq; ++n) {
        const R d1 = s_D[x.ni * Nq + n], d2 = s_D[x.nj * Nq + n], d3 = s_D[x.nk * Nq + n];
#pragma unroll
        for (int s = 0; s < NA; ++s) {
            a[s][0] = fma(d1, s_X[s * Np + L1 + n], a[s][0]);
            a[s][1] = fma(d2, s_X[s * Np + L2 + n * Nq], a[s][1]);
            a[s][2] = fma(d3, s_X[s * Np + L3 + n * Nfp], a[s][2]);
        }
    }
    R Jx[9];
#pragma unroll
    for (int w = 0; w < 9; ++w) Jx[w] = g[(KG_JXI + w) * Np + t];
    const R iJ = g[KG_INVJ * Np + t];
    if (horiz) {  // HorizontalDirection: no xi3 derivative
#pragma unroll
        for (int s = 0; s < NA; ++s) a[s][2] = R(0);
    }
#pragma unroll
    for (int s = 0; s < NA; ++s)
#pragma unroll
        for (int j = 0; j < 3; ++j) out[3 * s + j] = iJ * (Jx[j] * a[s][0] + Jx[3 + j] * a[s][1] + Jx[6 + j] * a[s][2]);
    auto add = [&](int ff) {
        const int idx = ff * Nfp + x.on_face(ff);
#pragma unroll
        for (int w = 0; w < 3 * NA; ++w) out[w] += s_dF[w * NFN + idx];
    };
    if (x.ni == 0) add(0);
    if (x.ni == N) add(1);
    if (x.nj == 0) add(2);
    if (x.nj == N) add(3);
    if (x.nk == 0) add(4);
    if (x.nk == N) add(5);
}

// level and kernel geometry of the node across face x.f (nb >= 0)
template <int N>
__device__ __forceinline__ int shell_partner_level(const ShellIdx<N>& x, int ez, int vP) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq;
    const int ezp = x.fd == 2 ? ez + (x.fside ? 1 : -1) : ez;
    return ezp * Nq + vP / Nfp;
}

// ARRAYS: a grid-arrays mesh (per-node reference values, facing node from
// the partner table) instead of the cubed shell (levels, orientation codes)
template <int N, typename R, bool MIXED, bool PROJECT = true, int NA = 4, bool ARRAYS = false>
__global__ void __launch_bounds__(ShellDims<N>::NT) shell_hyper_grad_kernel(const KParams P, const void* Qv,
                                                                            R* __restrict__ hg) {
    using Ix = ShellIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp, ESTRIDE = NSTATE * Np;
    constexpr int GSTRIDE = KG_NFIELDS * Np;
    using PL = Planar5<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_q = reinterpret_cast<R*>(smem_raw);  // planar records: states
    R* const s_H = s_q + planar_pad<R>(5 * Np);      // [NA][Np] arguments
    R* const s_dF = s_H + NA * Np;                   // [3 NA][NFN] lifted face terms
    R* const s_D = s_dF + 3 * NA * NFN;              // strong-form D

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const R* __restrict__ Qin = static_cast<const R*>(Qv);
    const R* __restrict__ geo = static_cast<const R*>(P.geo);
    const R* ge = geo + (size_t)e * GSTRIDE;
    const int* nbr = P.nbr + NBR_STRIDE * e;
    const int ez = __ldg(nbr + 6);
    if (t < Nq * Nq) s_D[t] = VConst<R>::D(P, t);
    R q[NSTATE], qp[NSTATE];
    if (x.node) {
        const R* qe = Qin + (size_t)e * ESTRIDE + t;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = qe[s * Np];
    }
    const int nb = x.face ? __ldg(nbr + x.f) : -1;
    const int vP = nb < 0 ? x.vM
                   : ARRAYS ? __ldg(P.fpart + ((size_t)e * 6 + x.f) * Nfp + x.fn)
                            : shell_partner<N>(nbr, x.f, x.fn);
    if (nb >= 0) {
        const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
    }
    if (x.node) {
        R H[NA];
        const Level<R> lv = ARRAYS ? node_ref<R>(P, ge, Np, t) : shell_level<R, MIXED>(P, ge, Np, t, ez * Nq + x.nk);
        shell_hyper_args<R, MIXED, PROJECT, NA>(P, q, lv, ge, Np, t, H);
        PL::st(s_q, Np, t, q);
#pragma unroll
        for (int s = 0; s < NA; ++s) s_H[s * Np + t] = H[s];
    }
    __syncthreads();

    if (x.face) {
        R nv[3], Hp[NA], c;
        R lift = shell_face_normal<R>(P, ge, Np, x.fd, x.fside ? R(1) : R(-1), x.vM, nv);
        if (PROJECT && P.hyper_horizontal && x.fd == 2) lift = R(0);  // HorizontalDirection: no xi3 face terms
        if (nb >= 0) {
            const R* gp = geo + (size_t)nb * GSTRIDE;
            const Level<R> lvp = ARRAYS ? node_ref<R>(P, gp, Np, vP)
                                        : shell_level<R, MIXED>(P, gp, Np, vP, shell_partner_level<N>(x, ez, vP));
            shell_hyper_args<R, MIXED, PROJECT, NA>(P, qp, lvp, gp, Np, vP, Hp);
            c = R(0.5);
        } else {
            R qb[NSTATE];
            if (ARRAYS && P.mms_wall) {
                // InitStateBC: the caller's wall state (bc_initstate.jl:12-26)
                const double* w = P.mms_wall + (size_t)e * ESTRIDE + x.vM;
#pragma unroll
                for (int cc = 0; cc < NSTATE; ++cc) qb[cc] = (R)w[cc * Np];
            } else {
                // FreeSlip state of the gradient flux: rhou+ = rhou- - (rhou-.n) n
                PL::ld(s_q, Np, x.vM, qb);
                const R mn = qb[1] * nv[0] + qb[2] * nv[1] + qb[3] * nv[2];
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) qb[1 + cc] -= mn * nv[cc];
            }
            const Level<R> lvm =
                ARRAYS ? node_ref<R>(P, ge, Np, x.vM) : shell_level<R, MIXED>(P, ge, Np, x.vM, ez * Nq + x.kM);
            shell_hyper_args<R, MIXED, PROJECT, NA>(P, qb, lvm, ge, Np, x.vM, Hp);
            c = R(1);
        }
#pragma unroll
        for (int s = 0; s < NA; ++s) {
            const R dh = c * lift * (Hp[s] - s_H[s * Np + x.vM]);
#pragma unroll
            for (int j = 0; j < 3; ++j) s_dF[(3 * s + j) * NFN + t] = dh * nv[j];
        }
    }
    __syncthreads();

    if (x.node) {
        R g[3 * NA];
        shell_strong_gradient<N, R, NA>(x, s_H, s_dF, s_D, ge, t, PROJECT && P.hyper_horizontal != 0, g);
        R* o = hg + (size_t)e * 3 * NA * Np + t;
#pragma unroll
        for (int w = 0; w < 3 * NA; ++w) o[w * Np] = g[w];
    }
}

template <int N, typename R>
__global__ void __launch_bounds__(ShellDims<N>::NT) shell_hyper_div_kernel(const KParams P, const R* __restrict__ hg,
                                                                           R* __restrict__ hl) {
    using Ix = ShellIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp, GSTRIDE = KG_NFIELDS * Np;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_G = reinterpret_cast<R*>(smem_raw);  // [12][Np] gradients
    R* const s_Ft = s_G + 12 * Np;                   // [3][4][Np] J dxi_d/dx . grad G_s
    R* const s_dF = s_Ft + 12 * Np;                  // [4][NFN] lifted face terms
    R* const s_Dh = s_dF + 4 * NFN;                  // weak-form Dhat

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const R* __restrict__ geo = static_cast<const R*>(P.geo);
    const R* ge = geo + (size_t)e * GSTRIDE;
    const int* nbr = P.nbr + NBR_STRIDE * e;
    if (t < Nq * Nq) s_Dh[t] = static_cast<const R*>(P.Dhat)[t];
    if (x.node) {
        const R* gn = hg + (size_t)e * 12 * Np + t;
        R G[12];
#pragma unroll
        for (int w = 0; w < 12; ++w) {
            G[w] = gn[w * Np];
            s_G[w * Np + t] = G[w];
        }
        R Jx[9];
#pragma unroll
        for (int w = 0; w < 9; ++w) Jx[w] = ge[(KG_JXI + w) * Np + t];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int s = 0; s < 4; ++s)
                s_Ft[(d * 4 + s) * Np + t] =
                    Jx[3 * d + 0] * G[3 * s + 0] + Jx[3 * d + 1] * G[3 * s + 1] + Jx[3 * d + 2] * G[3 * s + 2];
    }
    const int nb = x.face ? __ldg(nbr + x.f) : -1;
    R Gp[12];
    if (nb >= 0) {
        const int vP = shell_partner<N>(nbr, x.f, x.fn);
        const R* gq = hg + (size_t)nb * 12 * Np + vP;
#pragma unroll
        for (int w = 0; w < 12; ++w) Gp[w] = gq[(size_t)w * Np];
    }
    __syncthreads();

    if (x.face) {
        R nv[3];
        R lift = shell_face_normal<R>(P, ge, Np, x.fd, x.fside ? R(1) : R(-1), x.vM, nv);
        if (P.hyper_horizontal && x.fd == 2) lift = R(0);  // HorizontalDirection: no terms on the xi3 faces
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            R acc = 0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const R Gm = s_G[(3 * s + j) * Np + x.vM];
                acc += ((nb >= 0 ? Gp[3 * s + j] : Gm) + Gm) * (nv[j] / R(2));
            }
            s_dF[s * NFN + t] = lift * acc;
        }
    }
    __syncthreads();

    if (x.node) {
        R a[4] = {0, 0, 0, 0}, av[4] = {0, 0, 0, 0};
        const int L1 = Nq * (x.nj + Nq * x.nk), L2 = x.ni + Nfp * x.nk, L3 = x.ni + Nq * x.nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            const R d1 = s_Dh[x.ni * Nq + n], d2 = s_Dh[x.nj * Nq + n], d3 = s_Dh[x.nk * Nq + n];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                a[s] = fma(d1, s_Ft[(0 * 4 + s) * Np + L1 + n], fma(d2, s_Ft[(1 * 4 + s) * Np + L2 + n * Nq], a[s]));
                av[s] = fma(d3, s_Ft[(2 * 4 + s) * Np + L3 + n * Nfp], av[s]);
            }
        }
        if (!P.hyper_horizontal) {
#pragma unroll
            for (int s = 0; s < 4; ++s) a[s] += av[s];
        }
        const R iJ = ge[KG_INVJ * Np + t];
        R lap[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) lap[s] = -iJ * a[s];
        auto add = [&](int ff) {
            const int idx = ff * Nfp + x.on_face(ff);
#pragma unroll
            for (int s = 0; s < 4; ++s) lap[s] += s_dF[s * NFN + idx];
        };
        if (x.ni == 0) add(0);
        if (x.ni == N) add(1);
        if (x.nj == 0) add(2);
        if (x.nj == N) add(3);
        if (x.nk == 0) add(4);
        if (x.nk == N) add(5);
        R* o = hl + (size_t)e * 4 * Np + t;
#pragma unroll
        for (int s = 0; s < 4; ++s) o[s * Np] = lap[s];
    }
}

template <int N, typename R, bool MIXED>
__global__ void __launch_bounds__(ShellDims<N>::NT) shell_hyper_glap_kernel(const KParams P, const R* __restrict__ hl,
                                                                            R* __restrict__ hd) {
    using Ix = ShellIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp, GSTRIDE = KG_NFIELDS * Np;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_L = reinterpret_cast<R*>(smem_raw);  // [4][Np] laplacians
    R* const s_dF = s_L + 4 * Np;                    // [12][NFN] lifted face terms
    R* const s_D = s_dF + 12 * NFN;                  // strong-form D

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const R* __restrict__ geo = static_cast<const R*>(P.geo);
    const R* ge = geo + (size_t)e * GSTRIDE;
    const int* nbr = P.nbr + NBR_STRIDE * e;
    if (t < Nq * Nq) s_D[t] = VConst<R>::D(P, t);
    if (x.node) {
        const R* ln = hl + (size_t)e * 4 * Np + t;
#pragma unroll
        for (int s = 0; s < 4; ++s) s_L[s * Np + t] = ln[s * Np];
    }
    const int nb = x.face ? __ldg(nbr + x.f) : -1;
    R Lp[4];
    if (nb >= 0) {
        const int vP = shell_partner<N>(nbr, x.f, x.fn);
        const R* lq = hl + (size_t)nb * 4 * Np + vP;
#pragma unroll
        for (int s = 0; s < 4; ++s) Lp[s] = lq[(size_t)s * Np];
    }
    __syncthreads();

    if (x.face) {
        R nv[3];
        R lift = shell_face_normal<R>(P, ge, Np, x.fd, x.fside ? R(1) : R(-1), x.vM, nv);
        if (P.hyper_horizontal && x.fd == 2) lift = R(0);  // HorizontalDirection: no terms on the xi3 faces
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const R dl = nb >= 0 ? lift * (Lp[s] - s_L[s * Np + x.vM]) / R(2) : R(0);
#pragma unroll
            for (int j = 0; j < 3; ++j) s_dF[(3 * s + j) * NFN + t] = dl * nv[j];
        }
    }
    __syncthreads();

    if (x.node) {
        R g[12];
        shell_strong_gradient<N, R>(x, s_L, s_dF, s_D, ge, t, P.hyper_horizontal != 0, g);
        const R nu4 = static_cast<const R*>(P.nu4)[(size_t)e * Np + t];
        R* o = hd + (size_t)e * 12 * Np + t;
#pragma unroll
        for (int w = 0; w < 12; ++w) {
            R v = nu4 * g[w];
            if (MIXED && w >= 9) v += P.hglap_ref32[((size_t)e * 3 + (w - 9)) * Np + t];
            o[w * Np] = v;
        }
    }
}

template <int N, typename R, bool MIXED>
cudaError_t launch_shell_passes_typed(const KParams& P, const void* Q, void* hd, void* hl, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, NFN = 6 * Nfp, NT = ShellDims<N>::NT;
    constexpr size_t b1 = sizeof(R) * (planar_pad<R>(5 * Np) + 4 * Np + 12 * NFN + Nq * Nq);
    constexpr size_t b2 = sizeof(R) * (24 * Np + 4 * NFN + Nq * Nq);
    constexpr size_t b3 = sizeof(R) * (4 * Np + 12 * NFN + Nq * Nq);
    cudaError_t e;
    if ((e = opt_in(shell_hyper_grad_kernel<N, R, MIXED>, b1)) != cudaSuccess) return e;
    if ((e = opt_in(shell_hyper_div_kernel<N, R>, b2)) != cudaSuccess) return e;
    if ((e = opt_in(shell_hyper_glap_kernel<N, R, MIXED>, b3)) != cudaSuccess) return e;
    R* g = static_cast<R*>(hd);
    R* l = static_cast<R*>(hl);
    shell_hyper_grad_kernel<N, R, MIXED><<<P.nelem, NT, b1, s>>>(P, Q, g);
    shell_hyper_div_kernel<N, R><<<P.nelem, NT, b2, s>>>(P, g, l);
    shell_hyper_glap_kernel<N, R, MIXED><<<P.nelem, NT, b3, s>>>(P, l, g);
    return cudaGetLastError();
}

// the viscous gradient pass: grad u, grad h_tot (Np, 12, nelem)
template <int N, typename R, bool MIXED, int NA, bool ARRAYS = false>
cudaError_t launch_shell_visc_typed(const KParams& P, const void* Q, void* gout, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, NFN = 6 * Nfp, NT = ShellDims<N>::NT;
    constexpr size_t b1 = sizeof(R) * (planar_pad<R>(5 * Np) + NA * Np + 3 * NA * NFN + Nq * Nq);
    cudaError_t e;
    if ((e = opt_in(shell_hyper_grad_kernel<N, R, MIXED, false, NA, ARRAYS>, b1)) != cudaSuccess) return e;
    shell_hyper_grad_kernel<N, R, MIXED, false, NA, ARRAYS><<<P.nelem, NT, b1, s>>>(P, Q, static_cast<R*>(gout));
    return cudaGetLastError();
}

// grid-arrays meshes: grad u, grad h_tot (and grad theta_v with smag); the
// mixed form differentiates the perturbations
template <int N>
cudaError_t launch_arrays_visc_N(const KParams& P, bool mixed, bool smag, const void* Q, void* gout, cudaStream_t s) {
    if (mixed)
        return smag ? launch_shell_visc_typed<N, float, true, 5, true>(P, Q, gout, s)
                    : launch_shell_visc_typed<N, float, true, 4, true>(P, Q, gout, s);
    return smag ? launch_shell_visc_typed<N, double, false, 5, true>(P, Q, gout, s)
                : launch_shell_visc_typed<N, double, false, 4, true>(P, Q, gout, s);
}

cudaError_t launch_arrays_visc(const KParams& P, int N, bool mixed, bool smag, const void* Q, void* gout,
                               cudaStream_t s) {
    switch (N) {
        case 2: return launch_arrays_visc_N<2>(P, mixed, smag, Q, gout, s);
        case 3: return launch_arrays_visc_N<3>(P, mixed, smag, Q, gout, s);
        case 4: return launch_arrays_visc_N<4>(P, mixed, smag, Q, gout, s);
        case 5: return launch_arrays_visc_N<5>(P, mixed, smag, Q, gout, s);
        default: return cudaErrorInvalidValue;
    }
}

// grad u, grad h_tot (12 words); with smag also grad theta_v (15 words)
cudaError_t launch_shell_visc(const KParams& P, int N, bool mixed, bool smag, const void* Q, void* gout,
                              cudaStream_t s) {
    if (smag) {
        switch (N) {
            case 2: return mixed ? launch_shell_visc_typed<2, float, true, 5>(P, Q, gout, s)
                                 : launch_shell_visc_typed<2, double, false, 5>(P, Q, gout, s);
            case 3: return mixed ? launch_shell_visc_typed<3, float, true, 5>(P, Q, gout, s)
                                 : launch_shell_visc_typed<3, double, false, 5>(P, Q, gout, s);
            case 4: return mixed ? launch_shell_visc_typed<4, float, true, 5>(P, Q, gout, s)
                                 : launch_shell_visc_typed<4, double, false, 5>(P, Q, gout, s);
            case 5: return mixed ? launch_shell_visc_typed<5, float, true, 5>(P, Q, gout, s)
                                 : launch_shell_visc_typed<5, double, false, 5>(P, Q, gout, s);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (N) {
        case 2: return mixed ? launch_shell_visc_typed<2, float, true, 4>(P, Q, gout, s)
                             : launch_shell_visc_typed<2, double, false, 4>(P, Q, gout, s);
        case 3: return mixed ? launch_shell_visc_typed<3, float, true, 4>(P, Q, gout, s)
                             : launch_shell_visc_typed<3, double, false, 4>(P, Q, gout, s);
        case 4: return mixed ? launch_shell_visc_typed<4, float, true, 4>(P, Q, gout, s)
                             : launch_shell_visc_typed<4, double, false, 4>(P, Q, gout, s);
        case 5: return mixed ? launch_shell_visc_typed<5, float, true, 4>(P, Q, gout, s)
                             : launch_shell_visc_typed<5, double, false, 4>(P, Q, gout, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_shell_passes(const KParams& P, int N, bool mixed, const void* Q, void* hd, void* hl,
                                cudaStream_t s) {
    switch (N) {
        case 2: return mixed ? launch_shell_passes_typed<2, float, true>(P, Q, hd, hl, s)
                             : launch_shell_passes_typed<2, double, false>(P, Q, hd, hl, s);
        case 3: return mixed ? launch_shell_passes_typed<3, float, true>(P, Q, hd, hl, s)
                             : launch_shell_passes_typed<3, double, false>(P, Q, hd, hl, s);
        case 4: return mixed ? launch_shell_passes_typed<4, float, true>(P, Q, hd, hl, s)
                             : launch_shell_passes_typed<4, double, false>(P, Q, hd, hl, s);
        case 5: return mixed ? launch_shell_passes_typed<5, float, true>(P, Q, hd, hl, s)
                             : launch_shell_passes_typed<5, double, false>(P, Q, hd, hl, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

// nu_4 per node from the curl-invariant metric (lengthscale_horizontal:
// |columns 1 and 2 of (dxi/dx)^-1| 2/N, averaged), the buffers of the
// passes, and in mixed precision the FP64 reference part nu_4 grad lap h_ref.
int init_shell_hyper_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const int Np = m.Np, N = m.N;
    const size_t nn = (size_t)m.nelem * Np;
    const bool mixed = md->precision == CMDG_MIXED;
    std::vector<double> nu4(nn);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            const double* G = &m.cgeo[(size_t)e * CG_NFIELDS * Np];
            auto X = [&](int w) { return G[(CG_XI + w) * Np + n]; };
            const double a = X(0), b = X(1), c = X(2), d = X(3), f = X(4), g = X(5), h = X(6), i = X(7), j = X(8);
            const double det = a * (f * j - g * i) - b * (d * j - g * h) + c * (d * i - f * h);
            const double c1[3] = {(f * j - g * i) / det, -(d * j - g * h) / det, (d * i - f * h) / det};
            const double c2[3] = {-(b * j - c * i) / det, (a * j - c * h) / det, -(a * i - b * h) / det};
            const double D1 = std::sqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]) * 2 / N;
            const double D2 = std::sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]) * 2 / N;
            const double hh = (D1 + D2) / 2 / 2;
            nu4[(size_t)e * Np + n] = hh * hh * hh * hh / 2 / md->prm.tau_hyper;
        }
    const size_t elt = mixed ? sizeof(float) : sizeof(double);
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_hd, nn * 12 * elt));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_hlap, nn * 4 * elt));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_nu4, nn * elt));
    if (mixed) {
        std::vector<float> n32(nu4.begin(), nu4.end());
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_nu4, n32.data(), nn * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_nu4, nu4.data(), nn * sizeof(double), cudaMemcpyHostToDevice));
    }
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_hglap_ref, nn * 3 * sizeof(float)));
    CMDG_CUDA_CHECK(cudaMemset(md->d_hglap_ref, 0, nn * 3 * sizeof(float)));
    if (!mixed || !md->prm.ref_state) return CMDG_OK;

    // FP64 passes over the reference state at rest: rho_ref, 0, 0, 0, rhoe_ref per node
    std::vector<double> qref(nn * NSTATE, 0.0);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            qref[((size_t)e * NSTATE + 0) * Np + n] = md->ref64[((size_t)e * 2 + 0) * Np + n];
            qref[((size_t)e * NSTATE + 4) * Np + n] = md->ref64[((size_t)e * 2 + 1) * Np + n];
        }
    double *dq = nullptr, *dhd = nullptr, *dhl = nullptr, *dnu = nullptr;
    auto release = [&]() {
        cudaFree(dq);
        cudaFree(dhd);
        cudaFree(dhl);
        cudaFree(dnu);
    };
    cudaError_t ce = cudaMalloc(&dq, nn * NSTATE * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&dhd, nn * 12 * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&dhl, nn * 4 * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&dnu, nn * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMemcpy(dq, qref.data(), nn * NSTATE * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(dnu, nu4.data(), nn * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        LaunchArgs a;
        a.Qin = dq;
        a.Qout = nullptr;
        a.dQ = nullptr;
        a.alpha = a.beta = a.rka = a.rkb_dt = 0;
        a.mode = 0;
        KParams P = make_params(md, a);
        P.Dhat = md->d_Dhat64;
        P.geo = md->d_geo64;
        P.nu4 = dnu;
        P.hglap_ref32 = nullptr;
        ce = launch_shell_passes(P, N, false, dq, dhd, dhl, 0);
        if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    }
    std::vector<double> hd64;
    if (ce == cudaSuccess) {
        hd64.resize(nn * 12);
        ce = cudaMemcpy(hd64.data(), dhd, nn * 12 * sizeof(double), cudaMemcpyDeviceToHost);
    }
    release();
    if (ce != cudaSuccess) {
        set_error("reference hyperdiffusion pass failed: %s", cudaGetErrorString(ce));
        return CMDG_ERR_CUDA;
    }
    std::vector<float> ref32(nn * 3);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int j = 0; j < 3; ++j)
            for (int n = 0; n < Np; ++n)
                ref32[((size_t)e * 3 + j) * Np + n] = (float)hd64[((size_t)e * 12 + 9 + j) * Np + n];
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_hglap_ref, ref32.data(), nn * 3 * sizeof(float), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

int launch_shell_hyper_passes(Model* md, const void* Qin, void* hd_out, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    LaunchArgs a;
    a.Qin = Qin;
    a.Qout = nullptr;
    a.dQ = nullptr;
    a.alpha = a.beta = a.rka = a.rkb_dt = 0;
    a.mode = 0;
    const KParams P = make_params(md, a);
    const cudaError_t err = launch_shell_passes(P, m.N, md->precision == CMDG_MIXED, Qin, hd_out, md->d_hlap, s);
    if (err != cudaSuccess) {
        set_error("cubed-shell hyperdiffusion pass launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

// The gradient buffer of the viscous pass and, in mixed precision, the
// FP64 gradients of the reference h_tot and, with SmagorinskyLilly, of the
// reference theta_v (the viscous pass on the reference state at rest: u = 0,
// h_tot = h_ref, theta_v = theta_v_ref; the pass is linear in its
// arguments), per node (Np, 3 or 6, nelem).
int init_shell_visc_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const int Np = m.Np;
    const size_t nn = (size_t)m.nelem * Np;
    const bool mixed = md->precision == CMDG_MIXED;
    const bool smag = md->prm.turbulence == CMDG_TURB_SMAGORINSKY;
    const size_t elt = mixed ? sizeof(float) : sizeof(double);
    const int ngw = smag ? 15 : 12;
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_gf, nn * ngw * elt));
    CMDG_CUDA_CHECK(cudaMemset(md->d_gf, 0, nn * ngw * elt));
    if (smag) {
        // Smagorinsky length scale 2 / (cbrt(det(dxi/dx)) N) per node (Geometry.jl:121-122)
        std::vector<double> delta(nn);
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int n = 0; n < Np; ++n) {
                const double* G = &m.cgeo[(size_t)e * CG_NFIELDS * Np];
                auto X = [&](int w) { return G[(CG_XI + w) * Np + n]; };
                // rows d = xi_d, columns j = x_j
                const double a = X(0), b = X(1), c = X(2), d = X(3), f = X(4), g = X(5), h = X(6), i = X(7), j = X(8);
                const double det = a * (f * j - g * i) - b * (d * j - g * h) + c * (d * i - f * h);
                delta[(size_t)e * Np + n] = 2 / (std::cbrt(det) * std::max(1, m.N));
            }
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_sdelta, nn * sizeof(double)));
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_sdelta, delta.data(), nn * sizeof(double), cudaMemcpyHostToDevice));
    }
    const int nref = smag ? 6 : 3;
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_vgref, nn * nref * sizeof(float)));
    CMDG_CUDA_CHECK(cudaMemset(md->d_vgref, 0, nn * nref * sizeof(float)));
    // a mesh from grid arrays takes its reference state later, from
    // cmdg_model_set_reference, which computes these gradients then
    if (!mixed || !md->prm.ref_state || m.kind == MESH_ARRAYS) return CMDG_OK;
    return visc_reference_gradients(md);
}

// In mixed precision, the FP64 gradients of the reference h_tot (and
// theta_v) per node into md->d_vgref: the FP64 viscous gradient pass on the
// reference state at rest.
int visc_reference_gradients(Model* md) {
    const Mesh& m = *md->mesh;
    const int Np = m.Np;
    const size_t nn = (size_t)m.nelem * Np;
    const bool smag = md->prm.turbulence == CMDG_TURB_SMAGORINSKY;
    const int ngw = smag ? 15 : 12, nref = smag ? 6 : 3;
    std::vector<double> qref(nn * NSTATE, 0.0);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            qref[((size_t)e * NSTATE + 0) * Np + n] = md->ref64[((size_t)e * 2 + 0) * Np + n];
            qref[((size_t)e * NSTATE + 4) * Np + n] = md->ref64[((size_t)e * 2 + 1) * Np + n];
        }
    double *dq = nullptr, *dg = nullptr;
    cudaError_t ce = cudaMalloc(&dq, nn * NSTATE * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&dg, nn * ngw * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMemcpy(dq, qref.data(), nn * NSTATE * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        LaunchArgs a;
        a.Qin = dq;
        a.Qout = nullptr;
        a.dQ = nullptr;
        a.alpha = a.beta = a.rka = a.rkb_dt = 0;
        a.mode = 0;
        KParams P = make_params(md, a);
        P.Dhat = md->d_Dhat64;
        P.geo = md->d_geo64;
        ce = m.kind == MESH_ARRAYS ? launch_arrays_visc(P, m.N, false, smag, dq, dg, 0)
                                   : launch_shell_visc(P, m.N, false, smag, dq, dg, 0);
        if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    }
    std::vector<double> g64;
    if (ce == cudaSuccess) {
        g64.resize(nn * ngw);
        ce = cudaMemcpy(g64.data(), dg, nn * ngw * sizeof(double), cudaMemcpyDeviceToHost);
    }
    cudaFree(dq);
    cudaFree(dg);
    if (ce != cudaSuccess) {
        set_error("reference viscous gradient pass failed: %s", cudaGetErrorString(ce));
        return CMDG_ERR_CUDA;
    }
    // words 9..11 of the pass: grad h_tot; 12..14 with SmagorinskyLilly: grad theta_v
    std::vector<float> ref32(nn * nref);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int j = 0; j < nref; ++j)
            for (int n = 0; n < Np; ++n)
                ref32[((size_t)e * nref + j) * Np + n] = (float)g64[((size_t)e * ngw + 9 + j) * Np + n];
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_vgref, ref32.data(), nn * nref * sizeof(float), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

int launch_shell_visc_gradient(Model* md, const void* Qin, void* gout, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    LaunchArgs a;
    a.Qin = Qin;
    a.Qout = nullptr;
    a.dQ = nullptr;
    a.alpha = a.beta = a.rka = a.rkb_dt = 0;
    a.mode = 0;
    const KParams P = make_params(md, a);
    const bool smag = md->prm.turbulence == CMDG_TURB_SMAGORINSKY;
    const cudaError_t err = m.kind == MESH_ARRAYS
                                ? launch_arrays_visc(P, m.N, md->precision == CMDG_MIXED, smag, Qin, gout, s)
                                : launch_shell_visc(P, m.N, md->precision == CMDG_MIXED, smag, Qin, gout, s);
    if (err != cudaSuccess) {
        set_error("cubed-shell viscous gradient pass launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
