// Fused DG tendency + LSRK stage kernel for curvilinear (cubed-shell) meshes.
//
// The brick kernel's three phases with per-node geometry: one CTA owns one
// element for a whole stage;
//   phase 1  every node evaluates the thermodynamics and first-order flux of
//            its state and stages the contravariant fluxes
//            Ft_d = J (dxi_d/dx) . F, d = 1..3, in shared memory, and forms
//            the gravity source -rho grad(Phi) with the DG gradient of Phi;
//   phase 2  every face node takes the outward normal n = +-J dxi_d/dx / |.|
//            and surface Jacobian |J dxi_d/dx| of its own volume node, the
//            interior normal flux F.n = +-Ft_d / |J dxi_d/dx| from phase 1,
//            gathers the neighbour's state at the matching node (horizontal
//            faces through the face-orientation code of the connectivity
//            row; walls reflect the normal momentum,
//            rho u+ = rho u- - 2 (rho u- . n) n), and stores the lifted
//            Rusanov or central flux vMI sM F* = |J dxi_d/dx| / (J w_0) F*;
//   phase 3  every node contracts Ft_d with the weak-form derivative Dhat,
//            scales by 1/J, subtracts its face terms, adds the source and
//            finishes the tendency or the LSRK 2N stage update.
// With M = J w_i w_j w_k this is M^-1 D^T M (dxi_d/dx . F) of
// src/Numerics/DGMethods/DGModel_kernels.jl:64-548 and the interface term of
// :588-901 (NumericalFluxes.jl:219-340; bc_momentum.jl:25-34), with the
// geometry of src/Numerics/Mesh/Metrics.jl:431-724 (normals and sJ from
// J dxi_d/dx at the face node) and Grids.jl:1068-1096.
//
// The geopotential and reference pressure are per vertical level (every node
// of a level has the same radius); the reference density and energy are the
// level row plus a per-node difference (the discrete hydrostatic balance on
// curved elements varies along a level).  In mixed precision the
// reference-state jump q_ref(-) - q_ref(+) in the Rusanov penalty is the
// FP64-computed level jump across vertical faces plus the difference of the
// two nodes' per-node parts.
#include "shell_common.cuh"
#include "visc_curv.cuh"

namespace cmdg {
namespace {

template <int N, typename R>
struct ShellSmem {
    static constexpr int Nq = N + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq;
    // planar five-field records (Planar5) as in the brick kernel
    static constexpr int P5N = planar_pad<R>(5 * Np);
    static constexpr int NODE = 0;
    static constexpr int CR = NODE + P5N;
    static constexpr int FLUX = CR + planar_pad<R>(2 * Np);
    static constexpr int FACE = FLUX + 3 * P5N;
    static constexpr int DMAT = FACE + planar_pad<R>(5 * 6 * Nfp);
    static constexpr int TOTAL = DMAT + Nq * Nq;
    static constexpr size_t BYTES = sizeof(R) * TOTAL;
};

// HYPER: DryBiharmonic hyperdiffusion, whose state nu grad^3 (Np, 12, nelem;
// word 3 c + d = nu d/dx_d lap(u_h[c]), 9 + d = nu d/dx_d lap(h_tot)) is read
// from P.hd: the hyperdiffusive fluxes (tendencies_momentum.jl:51-54,
// tendencies_energy.jl:40-48) join the volume flux and, with the neighbour's
// state, the central second-order interface flux; walls carry the
// first-order flux only (boundaryconditions.jl:113-185).
//
// VISC: ConstantDynamicViscosity, whose gradient state grad u, grad h_tot
// (Np, 12, nelem; word 3 c + d = d u_c / dx_d, 9 + d = d h_tot / dx_d, in
// mixed precision d h' / dx_d with the FP64 grad h_ref added here) is read
// from P.gf: the viscous fluxes tau rho, tau . rho u - D_t grad h_tot rho
// (tendencies_momentum.jl:37-42, tendencies_energy.jl:27-31, 51-56;
// TurbulenceClosures.jl:199-225, 368-404) join the volume flux and, with
// the neighbour's state, the central second-order interface flux; walls
// carry the first-order flux only.
//
// REM (mixed, tendency mode, inviscid, subtract_off): the remainder f - l of
// the vertical AtmosAcousticGravityLinearModel evaluated on the FP32
// perturbation q' (src/Atmos/Model/linear.jl:103-190, the
// remainder_DGModel of src/Numerics/DGMethods/remainder.jl).  The linear
// model's terms cancel before rounding: in xi3 the volume flux is
// J dxi3/dx . (F - F_L) with F - F_L = (0, rho u u - (R/cv) ke I,
// rho u ((rhoe' + p') rho_ref - h_ref rho') / (rho rho_ref)) -- p' - p_L' =
// -(R/cv) ke exactly, h_ref = rhoe_ref + p_ref -- the gravity sources cancel,
// and the faces normal to xi3 carry the central flux of F - F_L with the
// penalty (lambda - c_L)/2 on the perturbation jump plus lambda/2 on the
// reference jump (c_L: the larger reference sound speed, the linear model's
// Rusanov speed).  The stiff vertical acoustic terms are then applied in
// FP64 by the linear kernel, so FP32 rounding no longer enters them.
//
// Resident CTAs per SM of the FP32 kernel: the inviscid one ShellDims'
// MIN_CTAS; with hyperdiffusion alone at N = 4, 5 (72 registers; the mixed
// GCM with horizontal DryBiharmonic steps in 0.595 ms against 0.612 ms at 4
// and 0.629 ms at 6, which spills); 4 with a closure (24-56 bytes of
// spills at 5) and with hyperdiffusion at other N.
template <int N, typename R, bool MIXED, int MODE, bool HYPER, int VT, bool REM = false>
__global__ void __launch_bounds__(ShellDims<N>::NT,
                                  MIXED ? (HYPER && VT == 0 && N == 4 ? 5
                                                                      : (HYPER || VT != 0 ? 4 : ShellDims<N>::MIN_CTAS))
                                        : ShellDims<N>::MIN_CTAS64)
    shell_stage_kernel(const KParams P) {
    static_assert(!REM || (MIXED && MODE == 0 && !HYPER && VT == CMDG_TURB_NONE),
                  "the remainder form is a mixed inviscid tendency");
    constexpr bool VISC = VT != CMDG_TURB_NONE;
    using Dm = ShellDims<N>;
    using SM = ShellSmem<N, R>;
    constexpr int Nq = Dm::Nq, Np = Dm::Np, Nfp = Dm::Nfp, NFN = 6 * Nfp;
    constexpr int ESTRIDE = NSTATE * Np, GSTRIDE = KG_NFIELDS * Np;
    using PL = Planar5<R>;
    using CRV = typename Pair<R>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const sm = reinterpret_cast<R*>(smem_raw);
    R* const s_node = sm + SM::NODE;
    CRV* const s_cr = reinterpret_cast<CRV*>(sm + SM::CR);
    R* const s_F = sm + SM::FLUX;
    R* const s_fs = sm + SM::FACE;
    R* const s_D = sm + SM::DMAT;

    const int t = threadIdx.x;
    const int e = blockIdx.x;
    const R* __restrict__ Qin = static_cast<const R*>(P.Qin);
    R* __restrict__ Qout = static_cast<R*>(P.Qout);
    const R* __restrict__ ge = static_cast<const R*>(P.geo) + (size_t)e * GSTRIDE;
    const Physics& ph = P.ph;
    const bool node_thread = t < Np;
    const bool face_thread = t < 6 * Nfp;
    const bool read_reg = (MODE == 0) ? (P.beta != 0) : !P.first_stage;

    const int nk = node_thread ? t / Nfp : 0;
    const int nj = node_thread ? (t - nk * Nfp) / Nq : 0;
    const int ni = node_thread ? t - nk * Nfp - nj * Nq : 0;
    const int f = face_thread ? t / Nfp : 0;
    const int fn = face_thread ? t - f * Nfp : 0;
    const int fd = f >> 1, fside = f & 1;
    const int fa = fn % Nq, fb = fn / Nq;
    const int vM = fd == 0 ? fside * N + Nq * fn : (fd == 1 ? fa + Nq * (fside * N + Nq * fb) : fn + Nfp * (fside * N));
    const int kM = vM / Nfp;
    const R sgn = fside ? R(1) : R(-1);

    if (t < Nq * Nq) s_D[t] = static_cast<const R*>(P.Dhat)[t];
    const int* nbr = P.nbr + NBR_STRIDE * e;
    const int ez = __ldg(nbr + 6);
    const size_t ebase = (size_t)e * ESTRIDE + t;

    // ---------------- phase 1: node thermodynamics, contravariant fluxes, gravity
    R q[NSTATE], src[3] = {0, 0, 0}, invJ = 0;
    double dq_old[NSTATE];
    if (node_thread) {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) q[s] = Qin[ebase + s * Np];
        if (read_reg) {
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) dq_old[s] = P.dQ[ebase + s * Np];
        }
        R Jx[9];
#pragma unroll
        for (int w = 0; w < 9; ++w) Jx[w] = ge[(KG_JXI + w) * Np + t];
        invJ = ge[KG_INVJ * Np + t];
        Level<R> lv = load_level<R>(P, ez * Nq + nk);
        if (ph.ref_state) {
            // the reference density varies along a level on curved elements
            lv.rho_ref += ge[KG_DRHO * Np + t];
            lv.href += ge[KG_DRHOE * Np + t];
            if (!MIXED) {
                // rounding-sized per-node parts, below FP32 resolution
                const R dp = ge[KG_DPREF * Np + t];
                lv.p_ref += dp;
                lv.href += dp;
            }
        }
        if (!MIXED) lv.crho += ge[KG_DCRHO * Np + t];
        const Thermo<R, MIXED> th = thermo<R, MIXED>(q, lv, P);
        PL::st(s_node, Np, t, q);
        s_cr[t] = Pair<R>::make(th.c, th.rinv);
        R F0[NSTATE], F1[NSTATE], F2[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) {
            F0[s] = flux_d<R, MIXED>(q, th, 0, s);
            F1[s] = flux_d<R, MIXED>(q, th, 1, s);
            F2[s] = flux_d<R, MIXED>(q, th, 2, s);
        }
        if (HYPER) {
            const R* hn = static_cast<const R*>(P.hd) + (size_t)e * 12 * Np + t;
            R hd[12];
#pragma unroll
            for (int w = 0; w < 12; ++w) hd[w] = hn[w * Np];
            const R rho = MIXED ? lv.rho_ref + q[0] : q[0];
            auto add_hyper = [&](R(&F)[NSTATE], int d) {
#pragma unroll
                for (int c = 0; c < 3; ++c) F[1 + c] += rho * hd[3 * c + d];
                F[4] += (hd[d] * q[1] + hd[3 + d] * q[2] + hd[6 + d] * q[3]) + hd[9 + d] * rho;
            };
            add_hyper(F0, 0);
            add_hyper(F1, 1);
            add_hyper(F2, 2);
        }
        if (VISC) {
            R Fv[3][NSTATE];
            shell_visc_flux<R, MIXED, VT>(P, e, t, Np, q, lv, th.rinv, Fv);
#pragma unroll
            for (int s2 = 0; s2 < NSTATE; ++s2) {
                F0[s2] += Fv[0][s2];
                F1[s2] += Fv[1][s2];
                F2[s2] += Fv[2][s2];
            }
        }
        if (REM) {
            // xi1, xi2: the full flux; xi3: the rows of F - F_L
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                R Ft[NSTATE];
#pragma unroll
                for (int s = 0; s < NSTATE; ++s)
                    Ft[s] = Jx[d * 3 + 0] * F0[s] + Jx[d * 3 + 1] * F1[s] + Jx[d * 3 + 2] * F2[s];
                PL::st(s_F + d * SM::P5N, Np, t, Ft);
            }
            const R pke = KConst<R>::gm1(P) * R(0.5) * (q[1] * th.u[0] + q[2] * th.u[1] + q[3] * th.u[2]);
            const R hrem = ((q[4] + th.pflux) * lv.rho_ref - lv.href * q[0]) * th.rinv * rcp_r(lv.rho_ref);
            R Ft[NSTATE];
            Ft[0] = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c)
                Ft[1 + c] = Jx[6] * (q[1] * th.u[c]) + Jx[7] * (q[2] * th.u[c]) + Jx[8] * (q[3] * th.u[c]) -
                            Jx[6 + c] * pke;
            Ft[4] = (Jx[6] * q[1] + Jx[7] * q[2] + Jx[8] * q[3]) * hrem;
            PL::st(s_F + 2 * SM::P5N, Np, t, Ft);
        } else {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                R Ft[NSTATE];
#pragma unroll
                for (int s = 0; s < NSTATE; ++s)
                    Ft[s] = Jx[d * 3 + 0] * F0[s] + Jx[d * 3 + 1] * F1[s] + Jx[d * 3 + 2] * F2[s];
                PL::st(s_F + d * SM::P5N, Np, t, Ft);
            }
        }
        if (ph.gravity && !REM) {
            const R rho_s = MIXED ? ((ph.ref_state && ph.subtract_off) ? q[0] : lv.rho_ref + q[0])
                                  : ((ph.ref_state && ph.subtract_off) ? q[0] - lv.rho_ref : q[0]);
#pragma unroll
            for (int c = 0; c < 3; ++c) src[c] = -rho_s * ge[(KG_GPHI + c) * Np + t];
        }
    }
    __syncthreads();

    // ---------------- phase 2: one numerical flux per face node
    if (face_thread) {
        const R j0 = ge[(KG_JXI + fd * 3 + 0) * Np + vM];
        const R j1 = ge[(KG_JXI + fd * 3 + 1) * Np + vM];
        const R j2 = ge[(KG_JXI + fd * 3 + 2) * Np + vM];
        const R iJm = ge[KG_INVJ * Np + vM];
        const R sJ = sqrt_r(j0 * j0 + j1 * j1 + j2 * j2);
        const R rs = rcp_r(sJ);
        const R nv[3] = {sgn * j0 * rs, sgn * j1 * rs, sgn * j2 * rs};
        R qm[NSTATE], Fm[NSTATE], qp[NSTATE], Fp[NSTATE], jr[NSTATE] = {0, 0, 0, 0, 0};
        PL::ld(s_node, Np, vM, qm);
        const CRV cr = s_cr[vM];
        const R c_m = cr.x, ri_m = cr.y;
        PL::ld(s_F + fd * SM::P5N, Np, vM, Fm);
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) Fm[s] *= sgn * rs;
        const R mn_m = qm[1] * nv[0] + qm[2] * nv[1] + qm[3] * nv[2];
        const R lam_m = fabs(mn_m * ri_m) + c_m;
        const int nb = __ldg(nbr + f);
        int ezp = ez, kP = kM;
        const R* gp = ge;  // geometry of the node across the face (own node on a wall)
        int vP = vM;
        if (nb >= 0) {
            if (fd == 2) {
                kP = fside ? 0 : N;
                vP = fn + Nfp * kP;
                ezp = ez + (fside ? 1 : -1);
                if (MIXED && ph.numflux == CMDG_FLUX_RUSANOV) {
                    const int ej = fside ? ezp : ez;
                    const R sj = fside ? R(-1) : R(1);
                    jr[0] = sj * (R)P.jump32[2 * ej + 0];
                    jr[4] = sj * (R)P.jump32[2 * ej + 1];
                }
            } else {
                vP = shell_partner<N>(nbr, f, fn);
            }
            const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
            gp = static_cast<const R*>(P.geo) + (size_t)nb * GSTRIDE;
        } else {
            // Impenetrable(FreeSlip) + Insulating wall
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
#pragma unroll
            for (int c = 0; c < 3; ++c) qp[1 + c] = qm[1 + c] - R(2) * mn_m * nv[c];
            if (HYPER || VISC) {
                // the staged flux holds the second-order part too: walls take the first-order one
                const Level<R> lvm = shell_level<R, MIXED>(P, ge, Np, vM, ez * Nq + kM);
                const Thermo<R, MIXED> thm = thermo<R, MIXED>(qm, lvm, P);
                Fm[0] = mn_m;
#pragma unroll
                for (int c = 0; c < 3; ++c) Fm[1 + c] = mn_m * thm.u[c] + thm.pflux * nv[c];
                Fm[4] = mn_m * thm.rinv * thm.H;
            }
        }
        Level<R> lvp = load_level<R>(P, ezp * Nq + kP);
        if (!MIXED) lvp.crho += gp[KG_DCRHO * Np + vP];
        if (ph.ref_state) {
            const R drp = gp[KG_DRHO * Np + vP], dep = gp[KG_DRHOE * Np + vP];
            lvp.rho_ref += drp;
            lvp.href += dep;
            if (!MIXED) {
                const R dpp = gp[KG_DPREF * Np + vP];
                lvp.p_ref += dpp;
                lvp.href += dpp;
            }
            if (MIXED && ph.numflux == CMDG_FLUX_RUSANOV) {
                // per-node part of the reference jump q_ref(-) - q_ref(+)
                jr[0] += ge[KG_DRHO * Np + vM] - drp;
                jr[4] += ge[KG_DRHOE * Np + vM] - dep;
            }
        }
        const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
        const R mn_p = qp[1] * nv[0] + qp[2] * nv[1] + qp[3] * nv[2];
        const R un_p = mn_p * thp.rinv;
        Fp[0] = mn_p;
#pragma unroll
        for (int c = 0; c < 3; ++c) Fp[1 + c] = mn_p * thp.u[c] + thp.pflux * nv[c];
        Fp[4] = un_p * thp.H;
        R cL = 0;  // REM, faces normal to xi3: the linear model's Rusanov speed
        if (REM && fd == 2) {
            // F - F_L of the node across the face (or of the reflected state on a wall)
            const R pke_p = KConst<R>::gm1(P) * R(0.5) * (qp[1] * thp.u[0] + qp[2] * thp.u[1] + qp[3] * thp.u[2]);
            const R hrem_p =
                ((qp[4] + thp.pflux) * lvp.rho_ref - lvp.href * qp[0]) * thp.rinv * rcp_r(lvp.rho_ref);
            Fp[0] = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) Fp[1 + c] = mn_p * thp.u[c] - pke_p * nv[c];
            Fp[4] = mn_p * hrem_p;
            const Level<R> lvm = shell_level<R, MIXED>(P, ge, Np, vM, ez * Nq + kM);
            const R gam = KConst<R>::gamma(P);
            cL = fmax(sqrt_r(gam * lvm.p_ref * rcp_r(lvm.rho_ref)), sqrt_r(gam * lvp.p_ref * rcp_r(lvp.rho_ref)));
        }
        if (HYPER && nb >= 0) {
            // neighbour's hyperdiffusive flux . n
            const R* hn = static_cast<const R*>(P.hd) + (size_t)nb * 12 * Np + vP;
            R hn_n[4];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                hn_n[c] = nv[0] * hn[(3 * c + 0) * Np] + nv[1] * hn[(3 * c + 1) * Np] + nv[2] * hn[(3 * c + 2) * Np];
            const R rho_p = MIXED ? lvp.rho_ref + qp[0] : qp[0];
#pragma unroll
            for (int c = 0; c < 3; ++c) Fp[1 + c] += rho_p * hn_n[c];
            Fp[4] += (hn_n[0] * qp[1] + hn_n[1] * qp[2] + hn_n[2] * qp[3]) + hn_n[3] * rho_p;
        }
        if (VISC && nb >= 0) {
            // neighbour's viscous flux . n
            R Fv[3][NSTATE];
            shell_visc_flux<R, MIXED, VT>(P, nb, vP, Np, qp, lvp, thp.rinv, Fv);
#pragma unroll
            for (int s2 = 0; s2 < NSTATE; ++s2) Fp[s2] += nv[0] * Fv[0][s2] + nv[1] * Fv[1][s2] + nv[2] * Fv[2][s2];
        }
        const R lam_p = fabs(un_p) + thp.c;
        const R lift = sJ * iJm * KConst<R>::inv_w0(P);
        const R hmw = (ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
        const R hl = R(0.5) * lift, pl = hmw * lift;
        // REM: the linear model's penalty cL/2 on the perturbation jump comes off
        const R pq = (REM && fd == 2) ? (hmw - R(0.5) * cL) * lift : pl;
        R fs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) fs[s] = hl * (Fm[s] + Fp[s]) + (pq * (qm[s] - qp[s]) + pl * jr[s]);
        PL::st(s_fs, NFN, f * Nfp + fn, fs);
    }
    __syncthreads();

    // ---------------- phase 3: volume contraction, face terms, source, update
    int bad = 0;
    if (node_thread) {
        R acc[NSTATE] = {0, 0, 0, 0, 0};
        const int L1 = Nq * (nj + Nq * nk), L2 = ni + Nfp * nk, L3 = ni + Nq * nj;
#pragma unroll
        for (int n = 0; n < Nq; ++n) {
            R v1[NSTATE], v2[NSTATE], v3[NSTATE];
            PL::ld(s_F, Np, L1 + n, v1);
            PL::ld(s_F + SM::P5N, Np, L2 + n * Nq, v2);
            PL::ld(s_F + 2 * SM::P5N, Np, L3 + n * Nfp, v3);
            const R d1 = s_D[ni * Nq + n], d2 = s_D[nj * Nq + n], d3 = s_D[nk * Nq + n];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) acc[s] = fma(d1, v1[s], fma(d2, v2[s], fma(d3, v3[s], acc[s])));
        }
        R rhs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) rhs[s] = invJ * acc[s];
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
#pragma unroll
        for (int c = 0; c < 3; ++c) rhs[1 + c] += src[c];
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
    // one CTA per element: no barrier at the end, one vote per warp
    if (__any_sync(0xffffffffu, bad) && (t & 31) == 0) atomicOr(P.status, 1u);
}

template <int N, typename R, bool MIXED, int MODE, bool HYPER, int VT, bool REM = false>
cudaError_t launch_shell_typed(const KParams& P, cudaStream_t s) {
    constexpr size_t bytes = ShellSmem<N, R>::BYTES;
    static unsigned long long configured = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!(configured & (1ull << (dev & 63)))) {
        e = cudaFuncSetAttribute(shell_stage_kernel<N, R, MIXED, MODE, HYPER, VT, REM>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        configured |= 1ull << (dev & 63);
    }
    shell_stage_kernel<N, R, MIXED, MODE, HYPER, VT, REM><<<(unsigned)P.nelem, ShellDims<N>::NT, bytes, s>>>(P);
    return cudaGetLastError();
}

template <int N, bool HYPER, int VT>
cudaError_t launch_shell_N(const KParams& P, bool mixed, int mode, cudaStream_t s) {
    if (mixed)
        return mode == 0 ? launch_shell_typed<N, float, true, 0, HYPER, VT>(P, s)
                         : launch_shell_typed<N, float, true, 1, HYPER, VT>(P, s);
    return mode == 0 ? launch_shell_typed<N, double, false, 0, HYPER, VT>(P, s)
                     : launch_shell_typed<N, double, false, 1, HYPER, VT>(P, s);
}

// hyperdiffusion and viscosity are exclusive on the shell (cmdg_model_create)
template <int N>
cudaError_t launch_shell_N(const KParams& P, bool mixed, int mode, bool hyper, int turb, cudaStream_t s) {
    if (hyper) return launch_shell_N<N, true, CMDG_TURB_NONE>(P, mixed, mode, s);
    if (turb == CMDG_TURB_CONSTANT) return launch_shell_N<N, false, CMDG_TURB_CONSTANT>(P, mixed, mode, s);
    if (turb == CMDG_TURB_SMAGORINSKY) return launch_shell_N<N, false, CMDG_TURB_SMAGORINSKY>(P, mixed, mode, s);
    return launch_shell_N<N, false, CMDG_TURB_NONE>(P, mixed, mode, s);
}

}  // namespace

bool shell_remainder_supported(const Model* md) {
    return md->mesh->kind == MESH_SHELL && md->precision == CMDG_MIXED && md->prm.ref_state &&
           md->prm.subtract_off && md->prm.gravity && md->prm.hyperdiffusion == CMDG_HYPER_NONE &&
           md->prm.turbulence == CMDG_TURB_NONE && md->mms_src == nullptr;
}

int launch_shell_stage(Model* md, const LaunchArgs& a, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    const bool hyper = md->prm.hyperdiffusion != CMDG_HYPER_NONE;
    const bool visc = md->prm.turbulence != CMDG_TURB_NONE;
    if (a.remainder) {
        if (!shell_remainder_supported(md) || a.mode != 0) {
            set_error("the remainder tendency is built for mixed inviscid cubed-shell models with a subtracted "
                      "hydrostatic reference state");
            return CMDG_ERR_UNSUPPORTED;
        }
        const KParams P = make_params(md, a);
        cudaError_t err;
        switch (m.N) {
            case 2: err = launch_shell_typed<2, float, true, 0, false, CMDG_TURB_NONE, true>(P, s); break;
            case 3: err = launch_shell_typed<3, float, true, 0, false, CMDG_TURB_NONE, true>(P, s); break;
            case 4: err = launch_shell_typed<4, float, true, 0, false, CMDG_TURB_NONE, true>(P, s); break;
            case 5: err = launch_shell_typed<5, float, true, 0, false, CMDG_TURB_NONE, true>(P, s); break;
            default:
                set_error("no cubed-shell stage kernel for N=%d", m.N);
                return CMDG_ERR_ARG;
        }
        if (err != cudaSuccess) {
            set_error("cubed-shell remainder kernel launch failed: %s", cudaGetErrorString(err));
            return CMDG_ERR_CUDA;
        }
        return CMDG_OK;
    }
    if (hyper) {
        const int rc = launch_shell_hyper_passes(md, a.Qin, md->d_hd, s);
        if (rc) return rc;
    }
    if (visc) {
        const int rc = launch_shell_visc_gradient(md, a.Qin, md->d_gf, s);
        if (rc) return rc;
    }
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_shell_N<2>(P, mixed, a.mode, hyper, md->prm.turbulence, s); break;
        case 3: err = launch_shell_N<3>(P, mixed, a.mode, hyper, md->prm.turbulence, s); break;
        case 4: err = launch_shell_N<4>(P, mixed, a.mode, hyper, md->prm.turbulence, s); break;
        case 5: err = launch_shell_N<5>(P, mixed, a.mode, hyper, md->prm.turbulence, s); break;
        default:
            set_error("no cubed-shell stage kernel for N=%d", m.N);
            return CMDG_ERR_ARG;
    }
    if (err != cudaSuccess) {
        set_error("cubed-shell stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
