// Hyperdiffusion passes of the DG tendency on brick meshes (sm_103a), for
// the AtmosModel's DryBiharmonic closure
// (src/Common/TurbulenceClosures/TurbulenceClosures.jl:793-848) with
// FlatOrientation, so that u_h = (I - khat khat') u = (u, v, 0):
//
//  * hyper_grad_kernel: gradients of the GradientLaplacian states (u, v,
//    h_tot) in strong form with the central interface correction
//    vMI sM (G* - n G-), G* = n (G- + G+)/2 inside and n G+ of the FreeSlip
//    gradient boundary state on walls (volume_gradients!,
//    dgsem_interface_gradients!, src/Numerics/DGMethods/DGModel_kernels.jl:
//    934-1651);
//  * hyper_div_kernel: their laplacians in weak form,
//    M^-1 (D^T M grad G + L^T Mf (grad G)*) with the central penalty
//    (grad G- + grad G+)' n / 2, grad G+ = grad G- on walls
//    (volume_divergence_of_gradients!, interface_divergence_of_gradients!,
//    DGModel_kernels.jl:2132-2495; NumericalFluxes.jl:720-730;
//    src/Atmos/Model/boundaryconditions.jl:88-95);
//  * hyper_glap_kernel: the hyperdiffusive state nu_4 grad(lap), strong form
//    with the interface term n (lap+ - lap-)/2, zero on walls
//    (volume_gradients_of_laplacians!, interface_gradients_of_laplacians!,
//    DGModel_kernels.jl:2525-3000; NumericalFluxes.jl:768-790), with
//    nu_4 = (Delta_h/2)^4 / 2 / tau and Delta_h the mean horizontal node
//    spacing (lengthscale_horizontal, src/Numerics/Mesh/Geometry.jl:129-151);
//  * the stage kernel of viscous_common.cuh with the hyperdiffusive fluxes
//    rho nu grad^3 u_h and nu grad^3 u_h . rho u + rho nu grad^3 h_tot added
//    to the second-order flux on both sides of interior faces.
//
// Every pass is linear in its input, so in mixed precision the FP32 passes
// carry the perturbation h' of h_tot alone; the reference part
// grad(lap h_ref), a function of the vertical level on a brick, is computed
// once in FP64 on the host and added to nu grad^3 h_tot.
#include "viscous_common.cuh"

namespace cmdg {
namespace {

// thread indices of a node / face-node thread of a one-CTA-per-element pass
template <int N>
struct HypIdx {
    static constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    int ni, nj, nk, f, fn, fd, fside, vM, vP;
    bool node, face;
    __device__ __forceinline__ explicit HypIdx(int t) {
        node = t < Np;
        face = t < 6 * Nfp;
        nk = node ? t / Nfp : 0;
        nj = node ? (t - nk * Nfp) / Nq : 0;
        ni = node ? t - nk * Nfp - nj * Nq : 0;
        f = face ? t / Nfp : 0;
        fn = face ? t - f * Nfp : 0;
        fd = f >> 1;
        fside = f & 1;
        const int oside = fside ^ 1, fa = fn % Nq, fb = fn / Nq;
        vM = fd == 0 ? fside * N + Nq * fn : (fd == 1 ? fa + Nq * (fside * N + Nq * fb) : fn + Nfp * (fside * N));
        vP = fd == 0 ? oside * N + Nq * fn : (fd == 1 ? fa + Nq * (oside * N + Nq * fb) : fn + Nfp * (oside * N));
    }
    // face-node index of face ff at this node thread's position on it
    __device__ __forceinline__ int on_face(int ff) const {
        return ff < 2 ? nj + Nq * nk : (ff < 4 ? ni + Nq * nk : ni + Nq * nj);
    }
};

// the GradientLaplacian arguments (u, v, h_tot) of a state; h_tot is the
// perturbation h' in the mixed form with a reference state
template <typename R, bool MIXED>
__device__ __forceinline__ void hyper_args(const KParams& P, const R q[NSTATE], int lev, R H[3]) {
    R G[5];
    grad_args<R, MIXED, false>(P, q, load_level<R>(P, lev), load_vlevel<R>(P, lev), G);
    H[0] = G[0];
    H[1] = G[1];
    H[2] = G[3];
}

template <int N, typename R, bool MIXED>
__global__ void __launch_bounds__(VDims<N>::NT) hyper_grad_kernel(const KParams P, const void* Qv,
                                                                  R* __restrict__ hg) {
    using Ix = HypIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp, ESTRIDE = NSTATE * Np;
    using PL = Planar5<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_q = reinterpret_cast<R*>(smem_raw);  // planar records: states
    R* const s_H = s_q + planar_pad<R>(5 * Np);      // [3][Np] arguments
    R* const s_dH = s_H + 3 * Np;                    // [3][NFN] lifted face terms
    R* const s_D = s_dH + 3 * NFN;                   // strong-form D

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const R* __restrict__ Qin = static_cast<const R*>(Qv);
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
    int levp = ez * Nq + x.vM / Nfp;
    if (nb >= 0) {
        const R* qn = Qin + (size_t)nb * ESTRIDE + x.vP;
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
        int ezp = ez;
        if (x.fd == 2) {
            ezp = ez + (x.fside ? 1 : -1);
            ezp = ezp < 0 ? ezp + P.nz : (ezp >= P.nz ? ezp - P.nz : ezp);
        }
        levp = ezp * Nq + x.vP / Nfp;
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};
    // HorizontalDirection: no xi3 derivatives and no xi3-face terms
    const R xz = P.hyper_horizontal ? R(0) : xi[2];

    if (x.node) {
        R H[3];
        hyper_args<R, MIXED>(P, q, ez * Nq + x.nk, H);
        PL::st(s_q, Np, t, q);
#pragma unroll
        for (int s = 0; s < 3; ++s) s_H[s * Np + t] = H[s];
    }
    __syncthreads();

    // face terms c n (H+ - H-) lifted, c = 1/2 inside, 1 on walls
    if (x.face) {
        R Hp[3], c;
        if (nb >= 0) {
            hyper_args<R, MIXED>(P, qp, levp, Hp);
            c = R(0.5);
        } else {
            // FreeSlip state of the gradient flux: rhou+ = rhou- - (rhou-.n) n
            R qb[NSTATE];
            PL::ld(s_q, Np, x.vM, qb);
            if (x.fd == 0) qb[1] = R(0);
            if (x.fd == 1) qb[2] = R(0);
            if (x.fd == 2) qb[3] = R(0);
            hyper_args<R, MIXED>(P, qb, levp, Hp);
            c = R(1);
        }
        const R sgn = x.fside ? R(1) : R(-1);
        const R w = c * sgn * pick3(x.fd, xi[0], xi[1], xz) * KConst<R>::inv_w0(P);
#pragma unroll
        for (int s = 0; s < 3; ++s) s_dH[s * NFN + t] = w * (Hp[s] - s_H[s * Np + x.vM]);
    }
    __syncthreads();

    if (x.node) {
        R g1[3] = {0, 0, 0}, g2[3] = {0, 0, 0}, g3[3] = {0, 0, 0};
        const int L1 = Nq * (x.nj + Nq * x.nk), L2 = x.ni + Nfp * x.nk, L3 = x.ni + Nq * x.nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            const R d1 = s_D[x.ni * Nq + n], d2 = s_D[x.nj * Nq + n], d3 = s_D[x.nk * Nq + n];
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                g1[s] = fma(d1, s_H[s * Np + L1 + n], g1[s]);
                g2[s] = fma(d2, s_H[s * Np + L2 + n * Nq], g2[s]);
                g3[s] = fma(d3, s_H[s * Np + L3 + n * Nfp], g3[s]);
            }
        }
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            g1[s] *= xi[0];
            g2[s] *= xi[1];
            g3[s] *= xz;
        }
        auto add = [&](int ff, R* gd) {
            const int idx = ff * Nfp + x.on_face(ff);
#pragma unroll
            for (int s = 0; s < 3; ++s) gd[s] += s_dH[s * NFN + idx];
        };
        if (x.ni == 0) add(0, g1);
        if (x.ni == N) add(1, g1);
        if (x.nj == 0) add(2, g2);
        if (x.nj == N) add(3, g2);
        if (x.nk == 0) add(4, g3);
        if (x.nk == N) add(5, g3);
        R* o = hg + (size_t)e * 9 * Np + t;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            o[(3 * s + 0) * Np] = g1[s];
            o[(3 * s + 1) * Np] = g2[s];
            o[(3 * s + 2) * Np] = g3[s];
        }
    }
}

template <int N, typename R>
__global__ void __launch_bounds__(VDims<N>::NT) hyper_div_kernel(const KParams P, const R* __restrict__ hg,
                                                                 R* __restrict__ hl) {
    using Ix = HypIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_G = reinterpret_cast<R*>(smem_raw);  // [9][Np] gradients
    R* const s_dF = s_G + 9 * Np;                    // [3][NFN] lifted face terms
    R* const s_Dh = s_dF + 3 * NFN;                  // weak-form Dhat

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const int* nbr = P.nbr + NBR_STRIDE * e;
    if (t < Nq * Nq) s_Dh[t] = static_cast<const R*>(P.Dhat)[t];
    if (x.node) {
        const R* ge = hg + (size_t)e * 9 * Np + t;
#pragma unroll
        for (int w = 0; w < 9; ++w) s_G[w * Np + t] = ge[w * Np];
    }
    const int nb = x.face ? __ldg(nbr + x.f) : -1;
    R Gp[3];
    if (nb >= 0) {
        // the neighbour's gradient components normal to the face
        const R* gn = hg + (size_t)nb * 9 * Np + (size_t)x.fd * Np + x.vP;
#pragma unroll
        for (int s = 0; s < 3; ++s) Gp[s] = gn[(size_t)s * 3 * Np];
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};
    // HorizontalDirection: no xi3 derivatives and no xi3-face terms
    const R xz = P.hyper_horizontal ? R(0) : xi[2];
    __syncthreads();

    if (x.face) {
        const R sgn = x.fside ? R(1) : R(-1);
        const R w = sgn * pick3(x.fd, xi[0], xi[1], xz) * KConst<R>::inv_w0(P);
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            const R Gm = s_G[(3 * s + x.fd) * Np + x.vM];
            s_dF[s * NFN + t] = w * ((nb >= 0 ? Gp[s] : Gm) + Gm) / R(2);
        }
    }
    __syncthreads();

    if (x.node) {
        R a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0}, a3[3] = {0, 0, 0};
        const int L1 = Nq * (x.nj + Nq * x.nk), L2 = x.ni + Nfp * x.nk, L3 = x.ni + Nq * x.nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            const R d1 = s_Dh[x.ni * Nq + n], d2 = s_Dh[x.nj * Nq + n], d3 = s_Dh[x.nk * Nq + n];
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                a1[s] = fma(d1, s_G[(3 * s + 0) * Np + L1 + n], a1[s]);
                a2[s] = fma(d2, s_G[(3 * s + 1) * Np + L2 + n * Nq], a2[s]);
                a3[s] = fma(d3, s_G[(3 * s + 2) * Np + L3 + n * Nfp], a3[s]);
            }
        }
        R lap[3];
#pragma unroll
        for (int s = 0; s < 3; ++s) lap[s] = -(xi[0] * a1[s] + xi[1] * a2[s] + xz * a3[s]);
        auto add = [&](int ff) {
            const int idx = ff * Nfp + x.on_face(ff);
#pragma unroll
            for (int s = 0; s < 3; ++s) lap[s] += s_dF[s * NFN + idx];
        };
        if (x.ni == 0) add(0);
        if (x.ni == N) add(1);
        if (x.nj == 0) add(2);
        if (x.nj == N) add(3);
        if (x.nk == 0) add(4);
        if (x.nk == N) add(5);
        R* o = hl + (size_t)e * 3 * Np + t;
#pragma unroll
        for (int s = 0; s < 3; ++s) o[s * Np] = lap[s];
    }
}

template <int N, typename R, bool MIXED>
__global__ void __launch_bounds__(VDims<N>::NT) hyper_glap_kernel(const KParams P, const R* __restrict__ hl,
                                                                  R* __restrict__ hd) {
    using Ix = HypIdx<N>;
    constexpr int Nq = Ix::Nq, Np = Ix::Np, Nfp = Ix::Nfp, NFN = 6 * Nfp;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const s_L = reinterpret_cast<R*>(smem_raw);  // [3][Np] laplacians
    R* const s_dL = s_L + 3 * Np;                    // [3][NFN] lifted face terms
    R* const s_D = s_dL + 3 * NFN;                   // strong-form D

    const int e = blockIdx.x, t = threadIdx.x;
    const Ix x(t);
    const int* nbr = P.nbr + NBR_STRIDE * e;
    const int ez = __ldg(nbr + 6);
    if (t < Nq * Nq) s_D[t] = VConst<R>::D(P, t);
    if (x.node) {
        const R* le = hl + (size_t)e * 3 * Np + t;
#pragma unroll
        for (int s = 0; s < 3; ++s) s_L[s * Np + t] = le[s * Np];
    }
    const int nb = x.face ? __ldg(nbr + x.f) : -1;
    R Lp[3];
    if (nb >= 0) {
        const R* ln = hl + (size_t)nb * 3 * Np + x.vP;
#pragma unroll
        for (int s = 0; s < 3; ++s) Lp[s] = ln[(size_t)s * Np];
    }
    const R xi[3] = {KConst<R>::metric(P, e, 0), KConst<R>::metric(P, e, 1), KConst<R>::metric(P, e, 2)};
    // HorizontalDirection: no xi3 derivatives and no xi3-face terms
    const R xz = P.hyper_horizontal ? R(0) : xi[2];
    // nu_4 = (Delta_h / 2)^4 / 2 / tau, Delta_h = (2/(N xi1x1) + 2/(N xi2x2)) / 2 on an affine brick,
    // in the working precision (FP64 divisions would dominate an FP32 pass)
    const R h2 = (R(2) / (R(N) * xi[0]) + R(2) / (R(N) * xi[1])) / R(4);
    const R nu4 = h2 * h2 * h2 * h2 / R(2) * KConst<R>::inv_tau(P);
    __syncthreads();

    if (x.face) {
        const R sgn = x.fside ? R(1) : R(-1);
        const R w = sgn * pick3(x.fd, xi[0], xi[1], xz) * KConst<R>::inv_w0(P);
#pragma unroll
        for (int s = 0; s < 3; ++s)
            s_dL[s * NFN + t] = nb >= 0 ? w * (Lp[s] - s_L[s * Np + x.vM]) / R(2) : R(0);
    }
    __syncthreads();

    if (x.node) {
        R g1[3] = {0, 0, 0}, g2[3] = {0, 0, 0}, g3[3] = {0, 0, 0};
        const int L1 = Nq * (x.nj + Nq * x.nk), L2 = x.ni + Nfp * x.nk, L3 = x.ni + Nq * x.nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            const R d1 = s_D[x.ni * Nq + n], d2 = s_D[x.nj * Nq + n], d3 = s_D[x.nk * Nq + n];
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                g1[s] = fma(d1, s_L[s * Np + L1 + n], g1[s]);
                g2[s] = fma(d2, s_L[s * Np + L2 + n * Nq], g2[s]);
                g3[s] = fma(d3, s_L[s * Np + L3 + n * Nfp], g3[s]);
            }
        }
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            g1[s] *= xi[0];
            g2[s] *= xi[1];
            g3[s] *= xz;
        }
        auto add = [&](int ff, R* gd) {
            const int idx = ff * Nfp + x.on_face(ff);
#pragma unroll
            for (int s = 0; s < 3; ++s) gd[s] += s_dL[s * NFN + idx];
        };
        if (x.ni == 0) add(0, g1);
        if (x.ni == N) add(1, g1);
        if (x.nj == 0) add(2, g2);
        if (x.nj == N) add(3, g2);
        if (x.nk == 0) add(4, g3);
        if (x.nk == N) add(5, g3);
        if (MIXED) g3[2] += P.glap_ref32[ez * Nq + x.nk];
        R* o = hd + (size_t)e * 9 * Np + t;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            o[(3 * s + 0) * Np] = nu4 * g1[s];
            o[(3 * s + 1) * Np] = nu4 * g2[s];
            o[(3 * s + 2) * Np] = nu4 * g3[s];
        }
    }
}

template <int N, typename R, bool MIXED>
cudaError_t launch_passes_typed(const KParams& P, const void* Q, void* hd, void* hl, cudaStream_t s) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, NFN = 6 * Nfp, NT = VDims<N>::NT;
    constexpr size_t b1 = sizeof(R) * (planar_pad<R>(5 * Np) + 3 * Np + 3 * NFN + Nq * Nq);
    constexpr size_t b2 = sizeof(R) * (9 * Np + 3 * NFN + Nq * Nq);
    constexpr size_t b3 = sizeof(R) * (3 * Np + 3 * NFN + Nq * Nq);
    cudaError_t e;
    if ((e = opt_in(hyper_grad_kernel<N, R, MIXED>, b1)) != cudaSuccess) return e;
    if ((e = opt_in(hyper_div_kernel<N, R>, b2)) != cudaSuccess) return e;
    if ((e = opt_in(hyper_glap_kernel<N, R, MIXED>, b3)) != cudaSuccess) return e;
    R* g = static_cast<R*>(hd);
    R* l = static_cast<R*>(hl);
    hyper_grad_kernel<N, R, MIXED><<<P.nelem, NT, b1, s>>>(P, Q, g);
    hyper_div_kernel<N, R><<<P.nelem, NT, b2, s>>>(P, g, l);
    hyper_glap_kernel<N, R, MIXED><<<P.nelem, NT, b3, s>>>(P, l, g);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_passes_N(const KParams& P, const void* Q, void* hd, void* hl, bool mixed, cudaStream_t s) {
    return mixed ? launch_passes_typed<N, float, true>(P, Q, hd, hl, s)
                 : launch_passes_typed<N, double, false>(P, Q, hd, hl, s);
}

}  // namespace

// Reference rows of the mixed-precision passes: with gz = the DG z-gradient
// of the reference h_tot (VV_DHT_REF), lap = its weak-form divergence with
// the central penalty (walls: the minus side on both sides) and
// glap = the strong DG z-derivative of lap with the n (lap+ - lap-)/2
// interface term (zero on walls) -- the brick's column restatement of the
// three passes applied to a field that varies with z only.
int init_hyper_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const int Nq = m.Nq, N = m.N, nz = m.nz, nlev = m.nlev;
    const bool zper = m.desc.periodic[2] != 0;
    const double inv_w0 = 1.0 / m.omega[0];
    std::vector<double> gz(nlev), lap(nlev);
    // HorizontalDirection: h_ref depends on z only, its horizontal derivatives vanish
    const bool horiz = md->prm.hyper_direction == CMDG_DIR_HORIZONTAL;
    for (int lev = 0; lev < nlev; ++lev) gz[lev] = horiz ? 0.0 : md->lvv64[(size_t)lev * VV_NFIELDS + VV_DHT_REF];
    auto below = [&](int ez) { return ez > 0 ? ez - 1 : (zper ? nz - 1 : -1); };
    auto above = [&](int ez) { return ez + 1 < nz ? ez + 1 : (zper ? 0 : -1); };
    for (int lev = 0; lev < nlev; ++lev) {
        const int ez = lev / Nq, k = lev % Nq;
        const double dz = m.dzlev[lev], lift = dz * inv_w0;
        double a = 0;
        for (int n = 0; n < Nq; ++n) a += m.Dhat[k * Nq + n] * gz[ez * Nq + n];
        double v = -dz * a;
        if (k == 0) {
            const int eb = below(ez);
            const double gp = eb >= 0 ? gz[eb * Nq + N] : gz[lev];
            v += lift * (-1.0) * (gp + gz[lev]) / 2;
        }
        if (k == N) {
            const int et = above(ez);
            const double gp = et >= 0 ? gz[et * Nq] : gz[lev];
            v += lift * (1.0) * (gp + gz[lev]) / 2;
        }
        lap[lev] = v;
    }
    md->glap_ref64.assign(nlev, 0.0);
    for (int lev = 0; lev < nlev; ++lev) {
        const int ez = lev / Nq, k = lev % Nq;
        const double dz = m.dzlev[lev], lift = dz * inv_w0;
        double a = 0;
        for (int n = 0; n < Nq; ++n) a += m.D[k * Nq + n] * lap[ez * Nq + n];
        double v = dz * a;
        if (k == 0) {
            const int eb = below(ez);
            if (eb >= 0) v += lift * (-1.0) * (lap[eb * Nq + N] - lap[lev]) / 2;
        }
        if (k == N) {
            const int et = above(ez);
            if (et >= 0) v += lift * (1.0) * (lap[et * Nq] - lap[lev]) / 2;
        }
        md->glap_ref64[lev] = v;
    }
    std::vector<float> g32(md->glap_ref64.begin(), md->glap_ref64.end());
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_glap_ref, sizeof(float) * nlev));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_glap_ref, g32.data(), sizeof(float) * nlev, cudaMemcpyHostToDevice));
    const size_t elt = md->precision == CMDG_MIXED ? sizeof(float) : sizeof(double);
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_hd, (size_t)m.nelem * 9 * m.Np * elt));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_hlap, (size_t)m.nelem * 3 * m.Np * elt));
    return CMDG_OK;
}

int launch_hyper_passes(Model* md, const void* Qin, void* hd_out, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    LaunchArgs a;
    a.Qin = Qin;
    a.Qout = nullptr;
    a.dQ = nullptr;
    a.alpha = a.beta = a.rka = a.rkb_dt = 0;
    a.mode = 0;
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_passes_N<2>(P, Qin, hd_out, md->d_hlap, mixed, s); break;
        case 3: err = launch_passes_N<3>(P, Qin, hd_out, md->d_hlap, mixed, s); break;
        case 4: err = launch_passes_N<4>(P, Qin, hd_out, md->d_hlap, mixed, s); break;
        case 5: err = launch_passes_N<5>(P, Qin, hd_out, md->d_hlap, mixed, s); break;
        default: set_error("no hyperdiffusion kernels for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("hyperdiffusion pass launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

int launch_hyper_stage(Model* md, const LaunchArgs& a, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    int rc = launch_hyper_passes(md, a.Qin, md->d_hd, s);
    if (rc) return rc;
    const int turb = md->prm.turbulence;
    if (turb != CMDG_TURB_NONE && (rc = launch_gradient(md, a.Qin, md->d_gf, s, true))) return rc;
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_vstage_N<2, true>(P, mixed, a.mode, turb, s); break;
        case 3: err = launch_vstage_N<3, true>(P, mixed, a.mode, turb, s); break;
        case 4: err = launch_vstage_N<4, true>(P, mixed, a.mode, turb, s); break;
        case 5: err = launch_vstage_N<5, true>(P, mixed, a.mode, turb, s); break;
        default: set_error("no hyperdiffusive stage kernel for N=%d", m.N); return CMDG_ERR_UNSUPPORTED;
    }
    if (err != cudaSuccess) {
        set_error("hyperdiffusive stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg

extern "C" int cmdg_hyperdiffusive_state(cmdg_model* model, void* d_hd, const void* d_Q, void* stream) {
    using namespace cmdg;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    CMDG_ARG_CHECK(d_hd != nullptr && d_Q != nullptr, "NULL buffer");
    CMDG_ARG_CHECK(model->m.prm.hyperdiffusion != CMDG_HYPER_NONE, "the model has no hyperdiffusion");
    if (model->m.mesh->kind == MESH_SHELL)
        return launch_shell_hyper_passes(&model->m, d_Q, d_hd, (cudaStream_t)stream);
    return launch_hyper_passes(&model->m, d_Q, d_hd, (cudaStream_t)stream);
}
