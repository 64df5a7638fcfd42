// Fused DG tendency + LSRK stage kernel for meshes given by the reference's
// own grid arrays (cmdg_mesh_create_arrays): the cubed-shell kernel's three
// phases with everything per node -- J dxi_d/dx, 1/J, grad Phi and the
// reference state (rho_ref, rhoe_ref, p_ref and the pressure coefficient
// R_d T_0 - (R_d/cv_d) Phi) -- the node facing each face node read from a
// partner table built from vmap+ (Grids.jl:559-638), and, in mixed
// precision, the reference-state jump q_ref(-) - q_ref(+) of the Rusanov
// penalty from an FP64-computed per-face-node table.  Algorithm as in
// shell.cu: src/Numerics/DGMethods/DGModel_kernels.jl:64-548 and :588-901,
// NumericalFluxes.jl:219-340, bc_momentum.jl:25-34, Metrics.jl:431-724.
#include "shell_common.cuh"
#include "visc_curv.cuh"

namespace cmdg {
namespace {

template <typename K>
cudaError_t opt_in_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int N, typename R>
struct ArraysSmem {
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

// VT: the turbulence closure (FP64 or mixed; mixed adds the FP64-computed
// gradients of the reference h_tot and theta_v): the viscous fluxes of the curvilinear
// gradient pass's output join the volume flux and, with the facing node's
// state, the central second-order interface flux; walls carry the
// first-order flux only.
//
// Resident CTAs per SM of the FP32 kernel: ShellDims' MIN_CTAS, but 4 with a
// closure at N = 4 (93-96 registers, no spills; at 6 the closure
// kernels spilled 24-116 bytes; a mixed Smagorinsky LES of 24 x 24 x 12
// elements through grid arrays steps in 0.762 ms against 0.766 ms).
template <int N, typename R, bool MIXED, int MODE, int VT = CMDG_TURB_NONE>
__global__ void __launch_bounds__(ShellDims<N>::NT,
                                  MIXED ? (VT != CMDG_TURB_NONE && N == 4 ? 4 : ShellDims<N>::MIN_CTAS)
                                        : ShellDims<N>::MIN_CTAS64)
    arrays_stage_kernel(const KParams P) {
    constexpr bool VISC = VT != CMDG_TURB_NONE;
    using Dm = ShellDims<N>;
    using SM = ArraysSmem<N, R>;
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
    const R sgn = fside ? R(1) : R(-1);

    if (t < Nq * Nq) s_D[t] = static_cast<const R*>(P.Dhat)[t];
    const int* nbr = P.nbr + NBR_STRIDE * e;
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
        const Level<R> lv = node_ref<R>(P, ge, Np, t);
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
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            R Ft[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) Ft[s] = Jx[d * 3 + 0] * F0[s] + Jx[d * 3 + 1] * F1[s] + Jx[d * 3 + 2] * F2[s];
            PL::st(s_F + d * SM::P5N, Np, t, Ft);
        }
        if (ph.gravity) {
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
        const R* gp = ge;  // geometry of the node across the face (own node on a wall)
        int vP = vM;
        if (nb >= 0) {
            vP = __ldg(P.fpart + ((size_t)e * 6 + f) * Nfp + fn);
            const R* qn = Qin + (size_t)nb * ESTRIDE + vP;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qn[s * Np];
            gp = static_cast<const R*>(P.geo) + (size_t)nb * GSTRIDE;
            if (MIXED && ph.ref_state && ph.numflux == CMDG_FLUX_RUSANOV) {
                // FP64-computed reference jump q_ref(-) - q_ref(+) at this face node
                const float2 j = __ldg(reinterpret_cast<const float2*>(P.fjump) + ((size_t)e * 6 + f) * Nfp + fn);
                jr[0] = (R)j.x;
                jr[4] = (R)j.y;
            }
        } else if (P.mms_wall) {
            // InitStateBC: the caller's wall state (bc_initstate.jl:12-26)
            const double* w = P.mms_wall + (size_t)e * ESTRIDE + vM;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = (R)w[s * Np];
            if (VISC) {
                const Level<R> lvm = node_ref<R>(P, ge, Np, vM);
                const Thermo<R, MIXED> thm = thermo<R, MIXED>(qm, lvm, P);
                Fm[0] = mn_m;
#pragma unroll
                for (int c = 0; c < 3; ++c) Fm[1 + c] = mn_m * thm.u[c] + thm.pflux * nv[c];
                Fm[4] = mn_m * thm.rinv * thm.H;
            }
        } else {
            // Impenetrable(FreeSlip) + Insulating wall
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) qp[s] = qm[s];
#pragma unroll
            for (int c = 0; c < 3; ++c) qp[1 + c] = qm[1 + c] - R(2) * mn_m * nv[c];
            if (VISC) {
                // the staged flux holds the second-order part too: walls take the first-order one
                const Level<R> lvm = node_ref<R>(P, ge, Np, vM);
                const Thermo<R, MIXED> thm = thermo<R, MIXED>(qm, lvm, P);
                Fm[0] = mn_m;
#pragma unroll
                for (int c = 0; c < 3; ++c) Fm[1 + c] = mn_m * thm.u[c] + thm.pflux * nv[c];
                Fm[4] = mn_m * thm.rinv * thm.H;
            }
        }
        const Level<R> lvp = node_ref<R>(P, gp, Np, vP);
        const Thermo<R, MIXED> thp = thermo<R, MIXED>(qp, lvp, P);
        const R mn_p = qp[1] * nv[0] + qp[2] * nv[1] + qp[3] * nv[2];
        const R un_p = mn_p * thp.rinv;
        Fp[0] = mn_p;
#pragma unroll
        for (int c = 0; c < 3; ++c) Fp[1 + c] = mn_p * thp.u[c] + thp.pflux * nv[c];
        Fp[4] = un_p * thp.H;
        if (VISC && nb >= 0) {
            // facing node's viscous flux . n
            R Fv[3][NSTATE];
            shell_visc_flux<R, MIXED, VT>(P, nb, vP, Np, qp, lvp, thp.rinv, Fv);
#pragma unroll
            for (int s2 = 0; s2 < NSTATE; ++s2) Fp[s2] += nv[0] * Fv[0][s2] + nv[1] * Fv[1][s2] + nv[2] * Fv[2][s2];
        } else if (VISC && P.mms_wall) {
            // InitStateBC second order: the one-sided flux of the wall state with
            // the interior gradient state (NumericalFluxes.jl:872-966); the face
            // term halves Fm + Fp, hence twice the flux here
            R Fv[3][NSTATE];
            shell_visc_flux<R, MIXED, VT>(P, e, vM, Np, qp, lvp, thp.rinv, Fv);
#pragma unroll
            for (int s2 = 0; s2 < NSTATE; ++s2)
                Fp[s2] += R(2) * (nv[0] * Fv[0][s2] + nv[1] * Fv[1][s2] + nv[2] * Fv[2][s2]);
        }
        const R lam_p = fabs(un_p) + thp.c;
        const R lift = sJ * iJm * KConst<R>::inv_w0(P);
        const R hmw = (ph.numflux == CMDG_FLUX_RUSANOV) ? R(0.5) * fmax(lam_m, lam_p) : R(0);
        const R hl = R(0.5) * lift, pl = hmw * lift;
        R fs[NSTATE];
#pragma unroll
        for (int s = 0; s < NSTATE; ++s) fs[s] = hl * (Fm[s] + Fp[s]) + pl * ((qm[s] - qp[s]) + jr[s]);
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
        if (P.mms_src) {
            // the caller's source term (MMSSource, mms_bc_atmos.jl:60-80)
            const double* sp = P.mms_src + ebase;
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) rhs[s] += (R)sp[s * Np];
        }
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

template <int N, typename R, bool MIXED, int MODE, int VT>
cudaError_t launch_arrays_typed(const KParams& P, cudaStream_t s) {
    constexpr size_t bytes = ArraysSmem<N, R>::BYTES;
    cudaError_t e = opt_in_smem(arrays_stage_kernel<N, R, MIXED, MODE, VT>, bytes);
    if (e != cudaSuccess) return e;
    arrays_stage_kernel<N, R, MIXED, MODE, VT><<<(unsigned)P.nelem, ShellDims<N>::NT, bytes, s>>>(P);
    return cudaGetLastError();
}

// closures run FP64 on grid-arrays meshes (cmdg_model_create)
template <int N, int VT>
cudaError_t launch_arrays_VT(const KParams& P, bool mixed, int mode, cudaStream_t s) {
    if (mixed)
        return mode == 0 ? launch_arrays_typed<N, float, true, 0, VT>(P, s) : launch_arrays_typed<N, float, true, 1, VT>(P, s);
    return mode == 0 ? launch_arrays_typed<N, double, false, 0, VT>(P, s)
                     : launch_arrays_typed<N, double, false, 1, VT>(P, s);
}

template <int N>
cudaError_t launch_arrays_N(const KParams& P, bool mixed, int mode, int turb, cudaStream_t s) {
    if (turb == CMDG_TURB_CONSTANT) return launch_arrays_VT<N, CMDG_TURB_CONSTANT>(P, mixed, mode, s);
    if (turb == CMDG_TURB_SMAGORINSKY) return launch_arrays_VT<N, CMDG_TURB_SMAGORINSKY>(P, mixed, mode, s);
    return launch_arrays_VT<N, CMDG_TURB_NONE>(P, mixed, mode, s);
}

}  // namespace

int launch_arrays_stage(Model* md, const LaunchArgs& a, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    const int turb = md->prm.turbulence;
    if (turb != CMDG_TURB_NONE) {
        const int rc = launch_shell_visc_gradient(md, a.Qin, md->d_gf, s);
        if (rc) return rc;
    }
    const KParams P = make_params(md, a);
    const bool mixed = md->precision == CMDG_MIXED;
    cudaError_t err;
    switch (m.N) {
        case 2: err = launch_arrays_N<2>(P, mixed, a.mode, turb, s); break;
        case 3: err = launch_arrays_N<3>(P, mixed, a.mode, turb, s); break;
        case 4: err = launch_arrays_N<4>(P, mixed, a.mode, turb, s); break;
        case 5: err = launch_arrays_N<5>(P, mixed, a.mode, turb, s); break;
        default:
            set_error("no grid-arrays stage kernel for N=%d", m.N);
            return CMDG_ERR_ARG;
    }
    if (err != cudaSuccess) {
        set_error("grid-arrays stage kernel launch failed: %s", cudaGetErrorString(err));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}

}  // namespace cmdg
