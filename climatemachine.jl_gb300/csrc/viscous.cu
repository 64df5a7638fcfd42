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
#include "viscous_common.cuh"

namespace cmdg {
namespace {

// FLUX: instead of the NGF gradient-flux words, write the second-order flux
// rows F2[d][1..4] they give at the node (NF2 words, word 4 d + s - 1), which
// is all the viscous stage kernel needs of them: the stage then evaluates
// the closure once per node here instead of at its nodes and again at every
// face node for the neighbour, and gathers 4 words per neighbour face node
// instead of NGF.  The neighbour's flux carries its own element's filter
// width, as the reference's per-node auxiliary Delta does.
// FP32 at N = 4: 9 resident CTAs per SM (40 registers, no spills; measured
// on the Smagorinsky LES: 0.765 ms per step against 0.783 ms at the
// compiler's 48 registers, 8 CTAs)
template <int N, typename R>
constexpr int grad_min_ctas() {
    return (sizeof(R) == 4 && N == 4) ? 9 : 1;
}

template <int N, typename R, bool MIXED, bool SMAG, bool FLUX>
__global__ void __launch_bounds__(VDims<N>::NT, grad_min_ctas<N, R>())
    gradient_kernel(const KParams P, const void* Qv, R* __restrict__ gf) {
    using Dm = VDims<N>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, NFN = 6 * Nfp;
    constexpr int ESTRIDE = NSTATE * Np;
    using PL = Planar5<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_q = reinterpret_cast<R*>(smem_raw);      // planar records: states
    R* const s_G = s_q + planar_pad<R>(5 * Np);            // gradient arguments
    R* const s_dG = s_G + planar_pad<R>(5 * Np);           // face terms
    // strong-form D in shared memory: each thread indexes it by its own node
    // coordinates, which from the parameter bank would be divergent
    // constant-cache reads (on the LES that pipe ran 59% busy; shared reads
    // made the step 1.1% faster)
    R* const s_D = s_dG + planar_pad<R>(5 * NFN);
    if (threadIdx.x < Nq * Nq) s_D[threadIdx.x] = VConst<R>::D(P, threadIdx.x);

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
        const Level<R> lv = load_level<R>(P, lev);
        out[9] = SMAG ? (g3[4] * lv.gphiz) / thv : R(0);
        if (FLUX) {
            const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
            const R ru[3] = {q[1], q[2], q[3]};
            // Smagorinsky filter width, lengthscale = 2 / (cbrt(det dxi/dx) N) (src/Numerics/Mesh/Geometry.jl:121-122)
            const R Delta = R(2) / (cbrt(xi[0] * xi[1] * xi[2]) * R(N));
            R F2[3][NSTATE];
            flux2<R, SMAG ? CMDG_TURB_SMAGORINSKY : CMDG_TURB_CONSTANT>(P, rho, rcp_r(rho), ru, out,
                                                                      lv.gphiz / VConst<R>::grav(P), Delta, F2);
            R* o = gf + (size_t)e * NF2 * Np + t;
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int s = 1; s < NSTATE; ++s) o[(4 * d + s - 1) * Np] = F2[d][s];
        } else {
            R* o = gf + (size_t)e * NGF * Np + t;
#pragma unroll
            for (int s = 0; s < NGF; ++s) o[s * Np] = out[s];
        }
    }
}


template <int N, typename R, bool MIXED, bool SMAG, bool FLUX>
cudaError_t launch_grad_kernel(const KParams& P, const void* Q, void* gf, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    constexpr size_t bytes = sizeof(R) * (2 * planar_pad<R>(5 * Np) + planar_pad<R>(30 * Nfp) + Nq * Nq);
    auto k = gradient_kernel<N, R, MIXED, SMAG, FLUX>;
    cudaError_t e;
    if ((e = opt_in(k, bytes)) != cudaSuccess) return e;
    k<<<P.nelem, VDims<N>::NT, bytes, s>>>(P, Q, static_cast<R*>(gf));
    return cudaGetLastError();
}

template <int N, typename R, bool MIXED>
cudaError_t launch_grad_typed(const KParams& P, const void* Q, void* gf, int turb, bool flux, cudaStream_t s) {
    if (turb == CMDG_TURB_SMAGORINSKY)
        return flux ? launch_grad_kernel<N, R, MIXED, true, true>(P, Q, gf, s)
                    : launch_grad_kernel<N, R, MIXED, true, false>(P, Q, gf, s);
    return flux ? launch_grad_kernel<N, R, MIXED, false, true>(P, Q, gf, s)
                : launch_grad_kernel<N, R, MIXED, false, false>(P, Q, gf, s);
}

template <int N>
cudaError_t launch_grad_N(const KParams& P, const void* Q, void* gf, bool mixed, int turb, bool flux,
                          cudaStream_t s) {
    return mixed ? launch_grad_typed<N, float, true>(P, Q, gf, turb, flux, s)
                 : launch_grad_typed<N, double, false>(P, Q, gf, turb, flux, s);
}

}  // namespace

int launch_gradient(Model* md, const void* Qin, void* gf_out, cudaStream_t s, bool flux) {
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
        case 2: err = launch_grad_N<2>(P, Qin, gf_out, mixed, turb, flux, s); break;
        case 3: err = launch_grad_N<3>(P, Qin, gf_out, mixed, turb, flux, s); break;
        case 4: err = launch_grad_N<4>(P, Qin, gf_out, mixed, turb, flux, s); break;
        case 5: err = launch_grad_N<5>(P, Qin, gf_out, mixed, turb, flux, s); break;
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
    // gradient pass of this stage's input state (its second-order flux rows),
    // then the tendency / stage update
    int rc = launch_gradient(md, a.Qin, md->d_gf, s, true);
    if (rc) return rc;
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    const int turb = md->prm.turbulence;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_vstage_N<2, false>(P, mixed, a.mode, turb, s); break;
        case 3: err = launch_vstage_N<3, false>(P, mixed, a.mode, turb, s); break;
        case 4: err = launch_vstage_N<4, false>(P, mixed, a.mode, turb, s); break;
        case 5: err = launch_vstage_N<5, false>(P, mixed, a.mode, turb, s); break;
        default: set_error("no viscous stage kernel for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("viscous stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
