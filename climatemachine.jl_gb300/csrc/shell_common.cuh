// Device helpers shared by the cubed-shell kernels (shell.cu, hyper_shell.cu):
// thread layout, the node across a face (vertical faces: the element above or
// below, same in-face index; horizontal faces: through the face-orientation
// code of the connectivity row) and the reference state of a node (level row
// plus the node's own part).
#pragma once

#include "dg_common.cuh"

namespace cmdg {
namespace {

template <int N>
struct ShellDims {
    static constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp, NF = 6 * Nfp;
    static constexpr int NT = (((Np > NF) ? Np : NF) + 31) / 32 * 32;
    static constexpr int MIN_CTAS = N == 2 ? 12 : N == 3 ? 8 : N == 4 ? 6 : 4;
    static constexpr int MIN_CTAS64 = N == 5 ? 2 : 3;
};

// Volume node of the neighbour across face f (0..5) matching in-face node fn
// (a = fn % Nq, b = fn / Nq) of this element; nbr is the element's
// connectivity row (word 7: 4-bit orientation code per horizontal face:
// neighbour face in bits 0-1, bit 2 = the in-face horizontal index runs
// reversed).
template <int N>
__device__ __forceinline__ int shell_partner(const int* nbr, int f, int fn) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq;
    const int fd = f >> 1, fside = f & 1, fa = fn % Nq, fb = fn / Nq;
    if (fd == 2) return fn + Nfp * (fside ? 0 : N);
    const unsigned code = ((unsigned)__ldg(nbr + 7) >> (4 * f)) & 15u;
    const int f2 = (int)(code & 3u);
    const int a2 = (code & 4u) ? N - fa : fa;
    const int side2 = (f2 & 1) ? N : 0;
    return (f2 < 2) ? side2 + Nq * (a2 + Nq * fb) : a2 + Nq * (side2 + Nq * fb);
}

// Reference state at node n of an element with kernel geometry g (Np nodes
// per element): the level row of level lev plus the node's per-node parts
// (in FP64 also the rounding-sized pressure and pressure-coefficient parts,
// which are below FP32 resolution).
template <typename R, bool MIXED>
__device__ __forceinline__ Level<R> shell_level(const KParams& P, const R* g, int Np, int n, int lev) {
    Level<R> lv = load_level<R>(P, lev);
    if (!MIXED) lv.crho += g[KG_DCRHO * Np + n];
    if (P.ph.ref_state) {
        lv.rho_ref += g[KG_DRHO * Np + n];
        lv.href += g[KG_DRHOE * Np + n];
        if (!MIXED) {
            const R dp = g[KG_DPREF * Np + n];
            lv.p_ref += dp;
            lv.href += dp;
        }
    }
    return lv;
}

}  // namespace
// reference state of node n from the per-node tables of a grid-arrays mesh
// (zero without a reference state; the pressure coefficient always)
template <typename R>
__device__ __forceinline__ Level<R> node_ref(const KParams& P, const R* g, int Np, int n) {
    Level<R> lv;
    lv.crho = g[KG_DCRHO * Np + n];
    lv.gphiz = R(0);
    if (P.ph.ref_state) {
        lv.rho_ref = g[KG_DRHO * Np + n];
        lv.p_ref = g[KG_DPREF * Np + n];
        lv.href = g[KG_DRHOE * Np + n] + lv.p_ref;
    } else {
        lv.rho_ref = lv.p_ref = lv.href = R(0);
    }
    return lv;
}

}  // namespace cmdg
