// Viscous fluxes on curvilinear meshes (cubed shell, grid arrays): the
// gradient-flux words from the curvilinear gradient pass's output and the
// second-order flux rows of a node (TurbulenceClosures.jl:199-225, 240-252,
// 368-404, 446-505; tendencies_momentum.jl:37-42; tendencies_energy.jl:27-31,
// 51-56).
#pragma once

#include "shell_common.cuh"
#include "viscous_common.cuh"

namespace cmdg {
namespace {

// gradient-flux words [grad h_tot (3), S11, S21, S31, S22, S32, S33, N^2]
// from the shell viscous pass's grad u, grad h_tot (and grad theta_v with
// SmagorinskyLilly) at node n of element e with state q and reference row
// lv (compute_gradient_flux!, TurbulenceClosures.jl:240-252, 446-470;
// energy.jl:10-11)
template <typename R, bool MIXED, int VT>
__device__ __forceinline__ void shell_gf(const KParams& P, int64_t e, int n, int Np, const R q[NSTATE],
                                         const Level<R>& lv, R gf[NGF]) {
    constexpr int NW = VT == CMDG_TURB_SMAGORINSKY ? 15 : 12;
    const R* g = static_cast<const R*>(P.gf) + (size_t)e * NW * Np + n;
    R G[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) G[w] = g[w * Np];
#pragma unroll
    for (int d = 0; d < 3; ++d) gf[d] = G[9 + d];
    // mixed: the pass differentiated the perturbations h' (and theta_v');
    // add the FP64-computed gradients of the reference parts
    constexpr int NREF = VT == CMDG_TURB_SMAGORINSKY ? 6 : 3;
    if (MIXED && P.ph.ref_state) {
        const float* r = P.vgref32 + (size_t)e * NREF * Np + n;
#pragma unroll
        for (int d = 0; d < 3; ++d) gf[d] += (R)r[d * Np];
        if (VT == CMDG_TURB_SMAGORINSKY) {
#pragma unroll
            for (int d = 0; d < 3; ++d) G[12 + (NW == 15 ? d : 0)] += (R)r[(3 + d) * Np];
        }
    }
    gf[3] = G[0];
    gf[4] = (G[1] + G[3]) / 2;
    gf[5] = (G[2] + G[6]) / 2;
    gf[6] = G[4];
    gf[7] = (G[5] + G[7]) / 2;
    gf[8] = G[8];
    if (NGF > 9) gf[NGF - 1] = 0;
    if (VT == CMDG_TURB_SMAGORINSKY) {
        // N^2 = grad theta_v . grad Phi / theta_v, theta_v of the node's state
        const R* ge = static_cast<const R*>(P.geo) + (size_t)e * KG_NFIELDS * Np;
        const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
        const R rinv = R(1) / rho;
        const R ke2 = (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) * rinv;
        // p = p_ref + p' in the mixed form (q holds the perturbation)
        const R p = MIXED ? lv.p_ref + (KConst<R>::gm1(P) * (q[4] - R(0.5) * ke2) + q[0] * lv.crho)
                          : KConst<R>::gm1(P) * (q[4] - R(0.5) * ke2) + rho * lv.crho;
        const R T = p * rinv / VConst<R>::R_d(P);
        const R thv = T / pow_r(p / VConst<R>::MSLP(P), VConst<R>::kappa(P));
        gf[9] = (G[12] * ge[(KG_GPHI + 0) * Np + n] + G[13] * ge[(KG_GPHI + 1) * Np + n] +
                 G[14] * ge[(KG_GPHI + 2) * Np + n]) /
                thv;
    }
}

// viscous flux rows of a node (VT = the closure), khat = grad Phi / g and the
// Smagorinsky length scale at the node for SmagorinskyLilly
template <typename R, bool MIXED, int VT>
__device__ __forceinline__ void shell_visc_flux(const KParams& P, int64_t e, int n, int Np, const R q[NSTATE],
                                                const Level<R>& lv, R rinv, R F[3][NSTATE]) {
    R gf[NGF];
    shell_gf<R, MIXED, VT>(P, e, n, Np, q, lv, gf);
    const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
    const R ru[3] = {q[1], q[2], q[3]};
    if (VT == CMDG_TURB_SMAGORINSKY) {
        const R* ge = static_cast<const R*>(P.geo) + (size_t)e * KG_NFIELDS * Np;
        const R ig = R(1) / VConst<R>::grav(P);
        const R khat[3] = {ge[(KG_GPHI + 0) * Np + n] * ig, ge[(KG_GPHI + 1) * Np + n] * ig,
                           ge[(KG_GPHI + 2) * Np + n] * ig};
        flux2<R, CMDG_TURB_SMAGORINSKY>(P, rho, rinv, ru, gf, khat, (R)P.sdelta[(size_t)e * Np + n], F);
    } else {
        flux2<R, CMDG_TURB_CONSTANT>(P, rho, rinv, ru, gf, R(0), R(0), F);
    }
}

}  // namespace
}  // namespace cmdg
