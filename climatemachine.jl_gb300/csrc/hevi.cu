// HEVI time stepping (sm_103a): the AtmosAcousticGravityLinearModel
// as a DGModel in VerticalDirection, its column-wise banded LU, and
// ARK2GiraldoKellyConstantinescu in the LowStorageVariant.
//
//   linear operator   Atmos/Model/linear.jl:1-57, 150-160, 242-262;
//                     Atmos/Model/linear_tendencies.jl (Advect,
//                     LinearPressureGradient, LinearEnergyFlux, Gravity);
//                     vertical volume kernel DGModel_kernels.jl:312-548 and the
//                     interface kernel on faces 5-6 (:588-901) with the Rusanov
//                     flux (NumericalFluxes.jl:223-285) at the reference sound
//                     speed and FreeSlip/Insulating walls.
//   implicit solve    LinearBackwardEulerSolver(ManyColumnLU())
//                     (ODESolvers/BackwardEulerSolvers.jl; SystemSolvers/
//                     columnwise_lu_solver.jl:92-127, 129-158, 228-488,
//                     555-780): the banded matrix of Q - alpha L(Q) per vertical
//                     line, from the operator applied to unit states, factored
//                     without pivoting (Golub & Van Loan Alg. 4.3.1) and solved
//                     by band forward / back substitution (Alg. 4.3.2, 4.3.3).
//   ARK scheme        ODESolvers/AdditiveRungeKuttaMethod.jl:413-538 (stage
//                     and solution updates :559-662), tableau :839-897.
//
// Precision: the state, the ARK stage algebra, the linear operator and the
// column LU are FP64.  The explicit tendency is FP64 on an FP64 model, or
// the mixed kernels (FP32 perturbation about the FP64 reference state, FP64
// output) on a mixed model: GB300's FP64 pipe is narrow and the explicit
// tendency is the larger part of a step.
//
// GPU mapping.  A vertical line is the (i, j) node column of one element
// stack: nz elements x Nq levels x 5 states = n unknowns, r = s + 5 (k + Nq v).
// The linear operator is evaluated one thread per (element, i, j): its Nq
// nodes' fluxes stay in registers, the xi3 weak derivative and both faces of
// the line are formed by the same thread, so the kernel needs no shared
// memory and no barrier.  The band storage is line-fastest,
// AB[(b * n + col) * nline + line] with band row b = bw + row - col, so that
// the thread-per-line factorization and substitutions read it coalesced.
// One thread per line keeps every lane of GB300's narrow FP64 pipe busy;
// the substitutions skip the band entries that the element coupling makes
// exact zeros (see fwd_len / bwd_len).
#include <cmath>
#include <vector>

#include "cmdg_internal.h"

namespace cmdg {

namespace {

// per-node table of the linear operator, (Np, LT_NFIELDS, nelem)
enum LinField {
    LT_MX0 = 0,  // M dxi3/dx_c, 3 words
    LT_MI = 3,   // 1 / M
    LT_CRHO = 4, // pressure coefficient of rho: R_d T_0 - (R_d / cv_d) Phi
    LT_H = 5,    // (rhoe_ref + p_ref) / rho_ref
    LT_G0 = 6,   // DG gradient of the geopotential, 3 words
    LT_C = 9,    // reference sound speed
    LT_NFIELDS = 10
};
// per face node of the bottom (side 0, face 5) and top (side 1, face 6) of
// each element: unit normal (3) and lift vMI sM, (Nfp, 4, 2, nelem)
constexpr int LF_NFIELDS = 4;

struct LinParams {
    const double* Q;
    double* T;
    const double* lt;
    const double* lf;
    int64_t nelem;
    int nz;
    double alpha, beta;
    double kv;       // R_d / cv_d: p_L = kv rhoe + crho rho
    double D[64];    // D[kk * Nq + k] = d l_k / dxi at xi_kk
};

struct LinNode {
    double q[5];
    double pL, h, c;
};

__device__ __forceinline__ void lin_normal_flux(const LinNode& a, const double n[3], double F[5]) {
    const double un = a.q[1] * n[0] + a.q[2] * n[1] + a.q[3] * n[2];
    F[0] = un;
    F[1] = a.pL * n[0];
    F[2] = a.pL * n[1];
    F[3] = a.pL * n[2];
    F[4] = a.h * un;
}

template <int Nq>
__device__ __forceinline__ void lin_load(const LinParams& P, int64_t e, int node, LinNode& a) {
    constexpr int Np = Nq * Nq * Nq;
    const double* Qe = P.Q + (size_t)e * 5 * Np;
    const double* L = P.lt + (size_t)e * LT_NFIELDS * Np;
#pragma unroll
    for (int s = 0; s < 5; ++s) a.q[s] = Qe[s * Np + node];
    // linearized_air_pressure rho R_d T_0 + R_d / cv_d (rhoe - rho Phi), grouped
    // as R_d / cv_d rhoe + (R_d T_0 - R_d / cv_d Phi) rho
    a.pL = P.kv * a.q[4] + L[LT_CRHO * Np + node] * a.q[0];
    a.h = L[LT_H * Np + node];
    a.c = L[LT_C * Np + node];
}

// Rusanov flux of the linear model across one face node; qP from the facing
// node, or the FreeSlip reflection of qM on a wall (aux+ = aux-).
__device__ __forceinline__ void lin_face(const LinNode& M, const LinNode* P, const double n[3], double fl[5]) {
    LinNode W;
    if (P == nullptr) {
        W = M;
        const double dn = M.q[1] * n[0] + M.q[2] * n[1] + M.q[3] * n[2];
#pragma unroll
        for (int c = 0; c < 3; ++c) W.q[1 + c] = M.q[1 + c] - 2 * dn * n[c];
        P = &W;
    }
    double FM[5], FP[5];
    lin_normal_flux(M, n, FM);
    lin_normal_flux(*P, n, FP);
    const double mw = fmax(M.c, P->c);
#pragma unroll
    for (int s = 0; s < 5; ++s) fl[s] = (FM[s] + FP[s]) * 0.5 + mw * (M.q[s] - P->q[s]) * 0.5;
}

template <int Nq>
__global__ void __launch_bounds__(128) linear_tendency_kernel(const LinParams P) {
    constexpr int Nfp = Nq * Nq, Np = Nfp * Nq;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t e = tid / Nfp;
    const int ij = (int)(tid % Nfp);
    if (e >= P.nelem) return;
    const double* L = P.lt + (size_t)e * LT_NFIELDS * Np;
    double F3[Nq][5], rho[Nq];
#pragma unroll
    for (int k = 0; k < Nq; ++k) {
        const int node = ij + Nfp * k;
        LinNode a;
        lin_load<Nq>(P, e, node, a);
        const double m0 = L[(LT_MX0 + 0) * Np + node], m1 = L[(LT_MX0 + 1) * Np + node],
                     m2 = L[(LT_MX0 + 2) * Np + node];
        F3[k][0] = m0 * a.q[1] + m1 * a.q[2] + m2 * a.q[3];
        F3[k][1] = m0 * a.pL;
        F3[k][2] = m1 * a.pL;
        F3[k][3] = m2 * a.pL;
        F3[k][4] = m0 * (a.h * a.q[1]) + m1 * (a.h * a.q[2]) + m2 * (a.h * a.q[3]);
        rho[k] = a.q[0];
    }
    // face fluxes of the bottom (k = 0) and top (k = Nq - 1) nodes of the line
    double flb[5], flt[5];
    const int ez = (int)(e % P.nz);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const int k = side ? Nq - 1 : 0;
        const double* F = P.lf + ((size_t)e * 2 + side) * LF_NFIELDS * Nfp;
        const double n[3] = {F[ij], F[Nfp + ij], F[2 * Nfp + ij]};
        LinNode M, Pn;
        lin_load<Nq>(P, e, ij + Nfp * k, M);
        const bool wall = side ? (ez == P.nz - 1) : (ez == 0);
        if (!wall) lin_load<Nq>(P, side ? e + 1 : e - 1, ij + Nfp * (Nq - 1 - k), Pn);
        lin_face(M, wall ? nullptr : &Pn, n, side ? flt : flb);
    }
    double* Te = P.T + (size_t)e * 5 * Np;
#pragma unroll
    for (int k = 0; k < Nq; ++k) {
        const int node = ij + Nfp * k;
        const double MI = L[LT_MI * Np + node];
        double lv[5];
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            double acc = 0;
#pragma unroll
            for (int kk = 0; kk < Nq; ++kk) acc += MI * P.D[kk * Nq + k] * F3[kk][s];
            lv[s] = acc;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) lv[1 + c] += -rho[k] * L[(LT_G0 + c) * Np + node];
        const double* F = P.lf + ((size_t)e * 2 + (k == 0 ? 0 : 1)) * LF_NFIELDS * Nfp;
        const double lift = F[3 * Nfp + ij];
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            double v = (P.beta != 0) ? P.alpha * lv[s] + P.beta * Te[s * Np + node] : P.alpha * lv[s];
            if (k == 0) v -= P.alpha * lift * flb[s];
            if (k == Nq - 1) v -= P.alpha * lift * flt[s];
            Te[s * Np + node] = v;
        }
    }
}

struct LineMap {
    int64_t nline;
    int nz, n;
};

// state index of unknown r of line `line`
template <int Nq>
__device__ __forceinline__ size_t line_index(const LineMap& lm, int64_t line, int r) {
    constexpr int Nfp = Nq * Nq, Np = Nfp * Nq;
    const int s = r % 5, k = (r / 5) % Nq, v = r / (5 * Nq);
    const int64_t col = line / Nfp;
    const int ij = (int)(line % Nfp);
    const int64_t e = v + (int64_t)lm.nz * col;
    return ((size_t)e * 5 + s) * Np + ij + Nfp * k;
}

// unit states of one assembly sweep: 1 at (level k, state s) of every node
// column of every element whose stack level is vi mod 3
template <int Nq>
__global__ void unit_state_kernel(double* E, int64_t nelem, int nz, int vi, int k, int s) {
    constexpr int Nfp = Nq * Nq, Np = Nfp * Nq;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nelem * 5 * Np) return;
    const int64_t e = tid / (5 * Np);
    const int rem = (int)(tid % (5 * Np));
    const int st = rem / Np, node = rem % Np;
    E[tid] = (((e % nz) % 3) == vi && st == s && node / Nfp == k) ? 1.0 : 0.0;
}

// column (vs, k, s) of the EulerOperator Q + eps L(Q) into the band storage;
// one thread per (line, row)
template <int Nq>
__global__ void band_scatter_kernel(const double* E, const double* R, double* AB, LineMap lm, int bw, int vi,
                                    int k, int s, double eps, unsigned* err) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= lm.nline * lm.n) return;
    const int64_t line = tid % lm.nline;
    const int row = (int)(tid / lm.nline);
    const int v = row / (5 * Nq);
    int vs = -1;
    for (int d = -1; d <= 1; ++d)
        if (v + d >= 0 && v + d < lm.nz && (v + d) % 3 == vi) vs = v + d;
    if (vs < 0) return;
    const int col = s + 5 * (k + Nq * vs);
    const size_t idx = line_index<Nq>(lm, line, row);
    const double val = E[idx] + eps * R[idx];
    if (abs(row - col) <= bw)
        AB[((size_t)(bw + row - col) * lm.n + col) * lm.nline + line] = val;
    else if (val != 0)
        atomicOr(err, 1u);
}

__device__ __forceinline__ double& band_at(double* AB, const LineMap& lm, int bw, int64_t line, int row, int col) {
    return AB[((size_t)(bw + row - col) * lm.n + col) * lm.nline + line];
}

// band_lu! without pivoting, one thread per line
__global__ void band_lu_kernel(double* AB, LineMap lm, int bw, unsigned* err) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= lm.nline) return;
    const int n = lm.n;
    for (int kk = 0; kk < n; ++kk) {
        const double Aq = band_at(AB, lm, bw, line, kk, kk);
        if (!(Aq != 0) || !isfinite(Aq)) atomicOr(err, 2u);
        for (int ii = 1; ii <= bw && kk + ii < n; ++ii) band_at(AB, lm, bw, line, kk + ii, kk) /= Aq;
        for (int jj = 1; jj <= bw && kk + jj < n; ++jj) {
            const double Ajj = band_at(AB, lm, bw, line, kk, kk + jj);
            for (int ii = 1; ii <= bw && kk + ii < n; ++ii)
                band_at(AB, lm, bw, line, kk + ii, kk + jj) -= band_at(AB, lm, bw, line, kk + ii, kk) * Ajj;
        }
    }
}

// Structure of the factors.  The vertical operator couples the unknowns of
// one element densely and neighbouring elements only through their facing
// nodes: the bottom layer (k = 0, 5 unknowns, block positions 0..4) of
// element v + 1 and the top layer of element v.  With block size
// NB = 5 (N + 1) = bw + 1, the LU factors of a column at block position p
// then have their non-zero band entries in contiguous runs:
//   L(j + i, j), i = 1 .. fwd_len(p) = bw - max(0, p - 5)
//   U(j - i, j), i = 1 .. bwd_len(p) = p < 5 ? bw : p
// (the sub-diagonal block A(v+1, v) U(v, v)^-1 has rows only in the bottom
// layer of v + 1; the super-diagonal block L(v, v)^-1 A(v, v+1) columns only
// there).  Every other band entry is an exact zero, which
// band_pattern_kernel verifies after the factorization.
__host__ __device__ constexpr int fwd_len(int p, int bw) { return bw - (p > 5 ? p - 5 : 0); }
__host__ __device__ constexpr int bwd_len(int p, int bw) { return p < 5 ? bw : p; }

// checks the zero pattern and turns the pivots into their reciprocals (the
// back substitution multiplies)
__global__ void band_pattern_kernel(double* AB, LineMap lm, int bw, unsigned* err) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= lm.nline) return;
    const int nb = bw + 1;
    bool bad = false;
    for (int col = 0; col < lm.n; ++col) {
        const int p = col % nb;
        for (int i = fwd_len(p, bw) + 1; i <= bw; ++i) bad |= band_at(AB, lm, bw, line, col + i, col) != 0;
        for (int i = bwd_len(p, bw) + 1; i <= bw; ++i) bad |= band_at(AB, lm, bw, line, col - i, col) != 0;
        double& d = band_at(AB, lm, bw, line, col, col);
        d = 1.0 / d;
    }
    if (bad) atomicOr(err, 4u);
}

// SingleColumnLU: every line's factors must equal the first line's to
// rounding (entries within 1e-10 of the larger of the entry and the pivot
// row's scale); copies the first line's factors out
__global__ void band_single_kernel(const double* AB, double* AB1, LineMap lm, int bw, unsigned* err) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= lm.nline) return;
    const int nb = 2 * bw + 1;
    bool bad = false;
    for (int b = 0; b < nb; ++b)
        for (int col = 0; col < lm.n; ++col) {
            const size_t i0 = ((size_t)b * lm.n + col) * lm.nline;
            const double v = AB[i0 + line], v0 = AB[i0];
            const double scale = fabs(v0) + fabs(1.0 / AB[((size_t)bw * lm.n + col) * lm.nline]);
            bad |= !(fabs(v - v0) <= 1e-10 * scale);
            if (line == 0) AB1[(size_t)b * lm.n + col] = v0;
        }
    if (bad) atomicOr(err, 8u);
}

// one warp per CTA: the column count is small (a few warps per SM), so the
// grid is spread evenly over the SMs
constexpr int SOLVE_THREADS = 32;

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// columns ahead whose factor entries are prefetched into L2
constexpr int SOLVE_PREFETCH = 3;

// band_forward! then band_back! (Golub & Van Loan Alg. 4.3.2, 4.3.3), one
// thread per line (all lanes do useful FP64 work), the factors read
// coalesced across neighbouring lines.  The window of bw + 1 right-hand-side
// values (the reference's l_b) is a register ring: row r lives in slot
// r mod NB, and the loop over the NB positions of an element block is
// unrolled, so every slot index and every run length is a compile-time
// constant and only the structurally non-zero band entries are touched.
// The factor entries SOLVE_PREFETCH columns ahead are prefetched into L2 (a
// column count of a few warps per SM leaves nothing else to hide the DRAM
// latency).  y is a state-sized scratch; out may alias b; accumulate adds
// x to out.
template <int Nq>
__global__ void __launch_bounds__(SOLVE_THREADS) band_solve_kernel(const double* __restrict__ AB, const double* b,
                                                                   double* __restrict__ y, double* out, LineMap lm,
                                                                   int accumulate, int single) {
    constexpr int NB = 5 * Nq, BW = NB - 1;
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= lm.nline) return;
    const int n = lm.n, nz = lm.nz;
    // column and band-row strides: one factorization per line, or the
    // first line's for all (SingleColumnLU)
    const size_t NL = single ? 1 : (size_t)lm.nline, RS = (size_t)n * NL;
    const double* A = single ? AB : AB + line;
    double w[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) w[i] = b[line_index<Nq>(lm, line, i)];
    for (int d = 0; d < SOLVE_PREFETCH && d < n; ++d)
        for (int i = 1; i <= BW; ++i) prefetch_l2(A + (size_t)(BW + i) * RS + (size_t)d * NL);
    for (int v = 0; v < nz; ++v) {
#pragma unroll
        for (int p = 0; p < NB; ++p) {
            const int jj = v * NB + p;
            if (jj + SOLVE_PREFETCH < n) {
                const double* Ap = A + (size_t)(jj + SOLVE_PREFETCH) * NL;
#pragma unroll
                for (int i = 1; i <= BW; ++i)
                    if (i <= fwd_len((p + SOLVE_PREFETCH) % NB, BW)) prefetch_l2(Ap + (size_t)(BW + i) * RS);
            }
            const double* Aj = A + (size_t)jj * NL;
            const double w0 = w[p];
#pragma unroll
            for (int i = 1; i <= BW; ++i)
                if (i <= fwd_len(p, BW)) w[(p + i) % NB] -= Aj[(size_t)(BW + i) * RS] * w0;
            y[line_index<Nq>(lm, line, jj)] = w0;
            w[p] = (jj + NB < n) ? b[line_index<Nq>(lm, line, jj + NB)] : 0.0;
        }
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) w[BW - i] = y[line_index<Nq>(lm, line, n - 1 - i)];
    for (int d = 0; d < SOLVE_PREFETCH && d < n; ++d)
        for (int i = 0; i <= BW; ++i) prefetch_l2(A + (size_t)(BW - i) * RS + (size_t)(n - 1 - d) * NL);
    for (int v = nz - 1; v >= 0; --v) {
#pragma unroll
        for (int p = NB - 1; p >= 0; --p) {
            const int jj = v * NB + p;
            if (jj - SOLVE_PREFETCH >= 0) {
                const double* Ap = A + (size_t)(jj - SOLVE_PREFETCH) * NL;
#pragma unroll
                for (int i = 0; i <= BW; ++i)
                    if (i <= bwd_len((p + NB - SOLVE_PREFETCH) % NB, BW)) prefetch_l2(Ap + (size_t)(BW - i) * RS);
            }
            const double* Aj = A + (size_t)jj * NL;
            const double x = w[p] * Aj[(size_t)BW * RS];  // reciprocal pivot
#pragma unroll
            for (int i = 1; i <= BW; ++i)
                if (i <= bwd_len(p, BW)) w[(p - i + NB) % NB] -= Aj[(size_t)(BW - i) * RS] * x;
            const size_t o = line_index<Nq>(lm, line, jj);
            out[o] = accumulate ? out[o] + x : x;
            w[p] = (jj - NB >= 0) ? y[line_index<Nq>(lm, line, jj - NB)] : 0.0;
        }
    }
}

// stage_update!(::LowStorageVariant) (AdditiveRungeKuttaMethod.jl:559-601)
struct StageCoef {
    const double* S[2];   // Qstages[1] = Q, Qstages[2]
    const double* R[2];
    double rk[2], dtAe[2];
    int nprev;
};

__global__ void ark_stage_kernel(const double* __restrict__ Q, StageCoef c, double* Sis, double* Qhat, size_t len) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (size_t)gridDim.x * blockDim.x) {
        double qh = Q[i], qs = -0.0;
        for (int js = 0; js < c.nprev; ++js) {
            const double common = c.rk[js] * c.S[js][i];
            qh += common + c.dtAe[js] * c.R[js][i];
            qs -= common;
        }
        Sis[i] = qs;
        Qhat[i] = qh;
    }
}

// solution_update!(::LowStorageVariant) (:642-662)
__global__ void ark_solution_kernel(double* Q, const double* R0, const double* R1, const double* R2, double b0,
                                    double b1, double b2, size_t len) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (size_t)gridDim.x * blockDim.x) {
        double q = Q[i];
        q += b0 * R0[i];
        q += b1 * R1[i];
        q += b2 * R2[i];
        Q[i] = q;
    }
}

// Elements per wall-bounded stack of a grid-arrays mesh, 0 when its
// elements are not stacked: element e = v + nz h, face 5 (xi3 = -1) of level
// 0 and face 6 of level nz - 1 on walls, and between levels the facing node
// of node (i, j) of one face being node (i, j) of the other
// (StackedBrickTopology / StackedCubedSphereTopology order).
int arrays_stack_height(const Mesh& m) {
    const int Nfp = m.Nfp, Nq = m.Nq;
    const int* row0 = &m.nbr[0];
    if (row0[4] >= 0) return 0;
    int nz = 1;
    for (int64_t e = 0; m.nbr[(size_t)e * NBR_STRIDE + 5] >= 0; ++e) {
        if (m.nbr[(size_t)e * NBR_STRIDE + 5] != e + 1 || e + 1 >= m.nelem) return 0;
        ++nz;
    }
    if (m.nelem % nz != 0) return 0;
    for (int64_t e = 0; e < m.nelem; ++e) {
        const int v = (int)(e % nz);
        const int* row = &m.nbr[(size_t)e * NBR_STRIDE];
        if ((v == 0) != (row[4] < 0) || (v == nz - 1) != (row[5] < 0)) return 0;
        if (v > 0 && row[4] != e - 1) return 0;
        if (v < nz - 1 && row[5] != e + 1) return 0;
        for (int fn = 0; fn < Nfp; ++fn) {
            if (v > 0 && m.fpart[((size_t)e * 6 + 4) * Nfp + fn] != fn + Nfp * (Nq - 1)) return 0;
            if (v < nz - 1 && m.fpart[((size_t)e * 6 + 5) * Nfp + fn] != fn) return 0;
        }
    }
    return nz;
}

int stack_height(const Model* md) {
    const Mesh& m = *md->mesh;
    if (m.kind == MESH_SHELL) return m.nz;
    // a brick in BrickTopology's Hilbert order (no column order) has no stacks
    if (m.kind == MESH_BRICK && !m.desc.periodic[2] && !m.col_at.empty()) return m.nz;
    if (m.kind == MESH_ARRAYS) return md->lin_nz;
    return 0;
}

// per-node and per-face tables of the linear operator (FP64, host-built)
int init_linear_tables(Model* md) {
    if (md->d_lin64) return CMDG_OK;
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    CMDG_ARG_CHECK(p.ref_state != 0, "AtmosAcousticGravityLinearModel needs a model with a reference state");
    if (m.kind == MESH_ARRAYS) {
        if (!md->has_reference) {
            set_error("set the reference state (cmdg_model_set_reference) before the linear model");
            return CMDG_ERR_STATE;
        }
        md->lin_nz = arrays_stack_height(m);
        if (md->lin_nz == 0) {
            set_error("the vertical linear model needs stacked elements with walls at both ends of each stack "
                      "(StackedBrickTopology / StackedCubedSphereTopology order)");
            return CMDG_ERR_UNSUPPORTED;
        }
    }
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, nz = m.kind == MESH_ARRAYS ? md->lin_nz : m.nz;
    const int64_t nelem = m.nelem;
    std::vector<double> lt((size_t)nelem * LT_NFIELDS * Np), lf((size_t)nelem * 2 * LF_NFIELDS * Nfp);
    const double cs2 = p.cp_d / p.cv_d * p.R_d;
    const double inv_w0 = 1.0 / m.omega[0];
    std::vector<double> geo;
    if (m.kind == MESH_SHELL) {
        geo.resize((size_t)nelem * KG_NFIELDS * Np);
        CMDG_CUDA_CHECK(cudaMemcpy(geo.data(), md->d_geo64, sizeof(double) * geo.size(), cudaMemcpyDeviceToHost));
    } else if (m.kind == MESH_ARRAYS) {
        geo = md->arrays_geo;
    }
    for (int64_t e = 0; e < nelem; ++e) {
        const int ez = (int)(e % nz);
        double* T = &lt[(size_t)e * LT_NFIELDS * Np];
        double* F = &lf[(size_t)e * 2 * LF_NFIELDS * Nfp];
        if (m.kind == MESH_BRICK) {
            const double* em = &m.emetric[(size_t)e * 3];
            const double J = 1.0 / (em[0] * em[1] * em[2]);
            for (int n = 0; n < Np; ++n) {
                const int i = n % Nq, j = (n / Nq) % Nq, k = n / Nfp;
                const double* L = &md->lvl64[(size_t)(ez * Nq + k) * LV_NFIELDS];
                const double M = J * m.omega[i] * m.omega[j] * m.omega[k];
                T[(LT_MX0 + 0) * Np + n] = 0.0;
                T[(LT_MX0 + 1) * Np + n] = 0.0;
                T[(LT_MX0 + 2) * Np + n] = M * em[2];
                T[LT_MI * Np + n] = 1.0 / M;
                T[LT_CRHO * Np + n] = p.R_d * p.T_0 - (p.R_d / p.cv_d) * L[LV_PHI];
                T[LT_G0 * Np + n] = 0.0;
                T[(LT_G0 + 1) * Np + n] = 0.0;
                T[(LT_G0 + 2) * Np + n] = L[LV_GPHIZ];
                const double rho = L[LV_RHO_REF], pr = L[LV_P_REF];
                T[LT_H * Np + n] = (L[LV_RHOE_REF] + pr) / rho;
                T[LT_C * Np + n] = std::sqrt(cs2 * (pr / (p.R_d * rho)));
            }
            for (int side = 0; side < 2; ++side)
                for (int ij = 0; ij < Nfp; ++ij) {
                    double* Fs = F + (size_t)side * LF_NFIELDS * Nfp;
                    Fs[ij] = 0.0;
                    Fs[Nfp + ij] = 0.0;
                    Fs[2 * Nfp + ij] = side ? 1.0 : -1.0;
                    Fs[3 * Nfp + ij] = std::fabs(em[2]) * inv_w0;
                }
        } else {
            const double* G = &m.cgeo[(size_t)e * CG_NFIELDS * Np];
            const double* X = &m.xyz[(size_t)e * 3 * Np];
            const double* K = &geo[(size_t)e * KG_NFIELDS * Np];
            for (int n = 0; n < Np; ++n) {
                const double M = G[CG_M * Np + n];
                for (int c = 0; c < 3; ++c) T[(LT_MX0 + c) * Np + n] = M * G[(CG_XI + 6 + c) * Np + n];
                T[LT_MI * Np + n] = 1.0 / M;
                for (int c = 0; c < 3; ++c) T[(LT_G0 + c) * Np + n] = K[(KG_GPHI + c) * Np + n];
                double pr;
                if (m.kind == MESH_ARRAYS) {
                    // the caller's geopotential (as its pressure coefficient) and reference pressure
                    T[LT_CRHO * Np + n] = K[KG_DCRHO * Np + n];
                    pr = md->pref64[(size_t)e * Np + n];
                } else {
                    const double r = std::sqrt(X[n] * X[n] + X[Np + n] * X[Np + n] + X[2 * Np + n] * X[2 * Np + n]);
                    const double phi = (p.orientation == CMDG_ORIENT_SPHERE) ? p.grav * (r - p.planet_radius) : 0.0;
                    T[LT_CRHO * Np + n] = p.R_d * p.T_0 - (p.R_d / p.cv_d) * phi;
                    double Tv;
                    temperature_profile(p, phi / p.grav, Tv, pr);
                }
                const double rho = md->ref64[((size_t)e * 2 + 0) * Np + n];
                const double rhoe = md->ref64[((size_t)e * 2 + 1) * Np + n];
                T[LT_H * Np + n] = (rhoe + pr) / rho;
                T[LT_C * Np + n] = std::sqrt(cs2 * (pr / (p.R_d * rho)));
            }
            for (int side = 0; side < 2; ++side)
                for (int ij = 0; ij < Nfp; ++ij) {
                    const int vM = ij + Nfp * (side ? Nq - 1 : 0);
                    const double j0 = K[(KG_JXI + 6) * Np + vM], j1 = K[(KG_JXI + 7) * Np + vM],
                                 j2 = K[(KG_JXI + 8) * Np + vM];
                    const double sJ = std::sqrt(j0 * j0 + j1 * j1 + j2 * j2);
                    const double sg = side ? 1.0 : -1.0;
                    double* Fs = F + (size_t)side * LF_NFIELDS * Nfp;
                    Fs[ij] = sg * j0 / sJ;
                    Fs[Nfp + ij] = sg * j1 / sJ;
                    Fs[2 * Nfp + ij] = sg * j2 / sJ;
                    Fs[3 * Nfp + ij] = sJ * K[KG_INVJ * Np + vM] * inv_w0;
                }
        }
    }
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_lin64, sizeof(double) * lt.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_lin64, lt.data(), sizeof(double) * lt.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_linface64, sizeof(double) * lf.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_linface64, lf.data(), sizeof(double) * lf.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

template <int Nq>
int launch_linear_N(Model* md, const double* Q, double* T, double alpha, double beta, cudaStream_t s) {
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    LinParams P{};
    P.Q = Q;
    P.T = T;
    P.lt = md->d_lin64;
    P.lf = md->d_linface64;
    P.nelem = m.nelem;
    P.nz = stack_height(md);
    P.alpha = alpha;
    P.beta = beta;
    P.kv = p.R_d / p.cv_d;
    for (int i = 0; i < Nq * Nq; ++i) P.D[i] = m.D[i];
    const int64_t threads = m.nelem * (int64_t)m.Nfp;
    linear_tendency_kernel<Nq><<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(P);
    CMDG_CUDA_CHECK(cudaGetLastError());
    return CMDG_OK;
}

}  // namespace

int launch_linear_tendency(Model* md, const double* Q, double* T, double alpha, double beta, cudaStream_t s) {
    int rc = init_linear_tables(md);
    if (rc) return rc;
    CMDG_ARG_CHECK(stack_height(md) > 0,
                   "the vertical linear model needs walls at the bottom and top of each column (non-periodic z)");
    switch (md->mesh->N) {
        case 2: return launch_linear_N<3>(md, Q, T, alpha, beta, s);
        case 3: return launch_linear_N<4>(md, Q, T, alpha, beta, s);
        case 4: return launch_linear_N<5>(md, Q, T, alpha, beta, s);
        case 5: return launch_linear_N<6>(md, Q, T, alpha, beta, s);
        default:
            set_error("the linear model is instantiated for N = 2..5");
            return CMDG_ERR_UNSUPPORTED;
    }
}

// ARK2GiraldoKellyConstantinescu with the column LU
struct Hevi {
    Model* md = nullptr;
    double dt = 0, alpha = 0;
    int split = 0;
    double Ae[3][3], Ai[3][3], B[3], C[3];
    LineMap lm{};
    int bw = 0;
    size_t len = 0;
    double* d_AB = nullptr;   // band matrix, then its LU factors (reciprocal pivots), line-fastest
    int single = 0;           // SingleColumnLU: d_AB1 holds the first line's factors, (2 bw + 1, n)
    double* d_AB1 = nullptr;
    double* d_buf = nullptr;  // S1, S2, R0, R1, R2, Qhat, Y
    float* d_Sp = nullptr;    // mixed models: FP32 perturbation of the stage state
    int rem = 0;              // mixed cubed shell: explicit part from the fused remainder f - l
    double* d_lref = nullptr; // rem with split: l(q_ref), the linear tendency of the reference state
    unsigned* d_err = nullptr;
    double* S(int i) const { return d_buf + (size_t)(i - 1) * len; }          // i = 1, 2
    double* R(int i) const { return d_buf + (size_t)(2 + i) * len; }          // i = 0..2
    double* Qhat() const { return d_buf + 5 * len; }
    double* Y() const { return d_buf + 6 * len; }
};

namespace {

template <int Nq>
int hevi_assemble_N(Hevi* h, cudaStream_t s) {
    Model* md = h->md;
    const Mesh& m = *md->mesh;
    double* E = h->Y();
    double* R = h->Qhat();
    const size_t len = h->len;
    const double eps = -h->alpha;
    const int64_t ntot = h->lm.nline * h->lm.n;
    for (int vi = 0; vi < 3 && vi < h->lm.nz; ++vi)
        for (int k = 0; k < Nq; ++k)
            for (int st = 0; st < 5; ++st) {
                unit_state_kernel<Nq><<<(unsigned)((len + 255) / 256), 256, 0, s>>>(E, m.nelem, h->lm.nz, vi, k, st);
                int rc = launch_linear_N<Nq>(md, E, R, 1.0, 0.0, s);
                if (rc) return rc;
                band_scatter_kernel<Nq><<<(unsigned)((ntot + 255) / 256), 256, 0, s>>>(E, R, h->d_AB, h->lm, h->bw, vi,
                                                                                       k, st, eps, h->d_err);
                CMDG_CUDA_CHECK(cudaGetLastError());
            }
    band_lu_kernel<<<(unsigned)((h->lm.nline + 127) / 128), 128, 0, s>>>(h->d_AB, h->lm, h->bw, h->d_err);
    CMDG_CUDA_CHECK(cudaGetLastError());
    band_pattern_kernel<<<(unsigned)((h->lm.nline + 127) / 128), 128, 0, s>>>(h->d_AB, h->lm, h->bw, h->d_err);
    CMDG_CUDA_CHECK(cudaGetLastError());
    if (h->single) {
        band_single_kernel<<<(unsigned)((h->lm.nline + 127) / 128), 128, 0, s>>>(h->d_AB, h->d_AB1, h->lm, h->bw,
                                                                                h->d_err);
        CMDG_CUDA_CHECK(cudaGetLastError());
    }
    return CMDG_OK;
}

int hevi_assemble(Hevi* h, cudaStream_t s) {
    switch (h->md->mesh->N) {
        case 2: return hevi_assemble_N<3>(h, s);
        case 3: return hevi_assemble_N<4>(h, s);
        case 4: return hevi_assemble_N<5>(h, s);
        default: return hevi_assemble_N<6>(h, s);
    }
}

template <int Nq>
int hevi_solve_N(Hevi* h, const double* b, double* out, int accumulate, cudaStream_t s) {
    const unsigned grid = (unsigned)((h->lm.nline + SOLVE_THREADS - 1) / SOLVE_THREADS);
    band_solve_kernel<Nq><<<grid, SOLVE_THREADS, 0, s>>>(h->single ? h->d_AB1 : h->d_AB, b, h->Y(), out, h->lm,
                                                         accumulate, h->single);
    CMDG_CUDA_CHECK(cudaGetLastError());
    return CMDG_OK;
}

int hevi_solve(Hevi* h, const double* b, double* out, int accumulate, cudaStream_t s) {
    switch (h->md->mesh->N) {
        case 2: return hevi_solve_N<3>(h, b, out, accumulate, s);
        case 3: return hevi_solve_N<4>(h, b, out, accumulate, s);
        case 4: return hevi_solve_N<5>(h, b, out, accumulate, s);
        default: return hevi_solve_N<6>(h, b, out, accumulate, s);
    }
}

__global__ void axpy_kernel(double* __restrict__ y, double a, const double* __restrict__ x, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}

unsigned elementwise_grid(size_t len);

// rhs!: the full tendency, or the remainder f - l when split.  A mixed
// model evaluates the explicit tendency on the FP32 perturbation of the FP64
// stage state (FP64 output); the ARK algebra and the solve stay FP64.  On a
// cubed shell the mixed tendency is split further: the fused remainder
// kernel forms f - l on the FP32 perturbation q' (the stiff vertical
// acoustic terms cancel before rounding) and the linear kernel adds l of the
// FP64 perturbation Q - q_ref, so f = (f - l)(q') + l(Q - q_ref); when the
// step is split, f - l(Q) = (f - l)(q') - l(q_ref), l(q_ref) formed once.
int hevi_rhs(Hevi* h, double* R, const double* Q, cudaStream_t s) {
    int rc;
    if (h->rem) {
        double* Qd = h->Y();  // free between the solve and the next stage
        rc = launch_to_perturbation(h->md, h->d_Sp, Q, s, Qd);
        if (rc) return rc;
        LaunchArgs a{h->d_Sp, nullptr, R, 1.0, 0.0, 0.0, 0.0, 0, 0, 0};
        a.remainder = 1;
        rc = launch_stage(h->md, a, s);
        if (rc) return rc;
        if (!h->split) return launch_linear_tendency(h->md, Qd, R, 1.0, 1.0, s);
        axpy_kernel<<<elementwise_grid(h->len), 256, 0, s>>>(R, -1.0, h->d_lref, h->len);
        CMDG_CUDA_CHECK(cudaGetLastError());
        return CMDG_OK;
    }
    if (h->md->precision == CMDG_MIXED) {
        rc = launch_to_perturbation(h->md, h->d_Sp, Q, s);
        if (rc) return rc;
        LaunchArgs a{h->d_Sp, nullptr, R, 1.0, 0.0, 0.0, 0.0, 0, 0, 0};
        rc = launch_stage(h->md, a, s);
    } else {
        LaunchArgs a{Q, nullptr, R, 1.0, 0.0, 0.0, 0.0, 0, 0, 0};
        rc = launch_stage(h->md, a, s);
    }
    if (rc) return rc;
    if (h->split) return launch_linear_tendency(h->md, Q, R, -1.0, 1.0, s);
    return CMDG_OK;
}

unsigned elementwise_grid(size_t len) {
    const size_t want = (len + 255) / 256;
    return (unsigned)(want < 152u * 16u ? want : 152u * 16u);
}

int hevi_step(Hevi* h, double* Q, cudaStream_t s) {
    const double dt = h->dt;
    const double* Sst[3] = {Q, h->S(1), h->S(2)};
    int rc = hevi_rhs(h, h->R(0), Q, s);
    if (rc) return rc;
    for (int is = 1; is < 3; ++is) {
        StageCoef c{};
        c.nprev = is;
        for (int js = 0; js < is; ++js) {
            c.S[js] = Sst[js];
            c.R[js] = h->R(js);
            c.rk[js] = h->split ? h->Ai[is][js] / h->Ai[is][is] : (h->Ai[is][js] - h->Ae[is][js]) / h->Ai[is][is];
            c.dtAe[js] = dt * h->Ae[is][js];
        }
        ark_stage_kernel<<<elementwise_grid(h->len), 256, 0, s>>>(Q, c, h->S(is), h->Qhat(), h->len);
        CMDG_CUDA_CHECK(cudaGetLastError());
        rc = hevi_solve(h, h->Qhat(), h->S(is), 1, s);
        if (rc) return rc;
        rc = hevi_rhs(h, h->R(is), h->S(is), s);
        if (rc) return rc;
    }
    if (h->split)
        for (int is = 0; is < 3; ++is) {
            rc = launch_linear_tendency(h->md, Sst[is], h->R(is), 1.0, 1.0, s);
            if (rc) return rc;
        }
    ark_solution_kernel<<<elementwise_grid(h->len), 256, 0, s>>>(Q, h->R(0), h->R(1), h->R(2), h->B[0] * dt,
                                                                  h->B[1] * dt, h->B[2] * dt, h->len);
    CMDG_CUDA_CHECK(cudaGetLastError());
    return CMDG_OK;
}

}  // namespace

}  // namespace cmdg

struct cmdg_hevi {
    cmdg::Hevi h;
};

using namespace cmdg;

extern "C" {

int cmdg_linear_tendency(cmdg_model* model, double* d_dQ, const double* d_Q, double t, double alpha, double beta,
                         void* stream) {
    (void)t;
    CMDG_ARG_CHECK(model != nullptr, "model is NULL");
    CMDG_ARG_CHECK(d_dQ != nullptr && d_Q != nullptr, "NULL state");
    CMDG_ARG_CHECK(d_dQ != d_Q, "the tendency must not alias the state");
    return launch_linear_tendency(&model->m, d_Q, d_dQ, alpha, beta, (cudaStream_t)stream);
}

int cmdg_hevi_create(cmdg_model* model, double dt, int split_explicit_implicit, int paperversion, int single_column,
                     cmdg_hevi** out) {
    CMDG_ARG_CHECK(model != nullptr && out != nullptr, "NULL argument");
    *out = nullptr;
    CMDG_ARG_CHECK(std::isfinite(dt) && dt > 0, "dt must be positive and finite");
    Model* md = &model->m;
    int rc = init_linear_tables(md);
    if (rc) return rc;
    const Mesh& m = *md->mesh;
    const int nz = stack_height(md);
    if (nz <= 0) {
        set_error("HEVI needs wall-bounded element stacks (a cubed shell, or a brick non-periodic in z in column order)");
        return CMDG_ERR_UNSUPPORTED;
    }
    if (m.N < 2 || m.N > 5) {
        set_error("HEVI is instantiated for N = 2..5");
        return CMDG_ERR_UNSUPPORTED;
    }
    cmdg_hevi* ho = new cmdg_hevi();
    Hevi* h = &ho->h;
    h->md = md;
    h->dt = dt;
    h->split = split_explicit_implicit ? 1 : 0;
    h->single = single_column ? 1 : 0;
    const double s2 = std::sqrt(2.0);
    const double a32 = paperversion ? (3 + 2 * s2) / 6 : 0.5;
    const double Ae[3][3] = {{0, 0, 0}, {2 - s2, 0, 0}, {1 - a32, a32, 0}};
    const double Ai[3][3] = {{0, 0, 0}, {1 - 1 / s2, 1 - 1 / s2, 0}, {1 / (2 * s2), 1 / (2 * s2), 1 - 1 / s2}};
    const double B[3] = {1 / (2 * s2), 1 / (2 * s2), 1 - 1 / s2}, C[3] = {0, 2 - s2, 1};
    for (int i = 0; i < 3; ++i) {
        h->B[i] = B[i];
        h->C[i] = C[i];
        for (int j = 0; j < 3; ++j) {
            h->Ae[i][j] = Ae[i][j];
            h->Ai[i][j] = Ai[i][j];
        }
    }
    h->alpha = dt * h->Ai[1][1];
    h->lm.nz = nz;
    h->lm.n = 5 * m.Nq * nz;
    h->lm.nline = (m.nelem / nz) * m.Nfp;
    h->bw = 5 * m.Nq - 1;
    h->len = (size_t)m.nelem * 5 * m.Np;
    const size_t ab = (size_t)(2 * h->bw + 1) * h->lm.n * h->lm.nline;
    cudaError_t e1 = cudaMalloc(&h->d_AB, sizeof(double) * ab);
    cudaError_t e2 = cudaMalloc(&h->d_buf, sizeof(double) * 7 * h->len);
    cudaError_t e3 = cudaMalloc(&h->d_err, sizeof(unsigned));
    cudaError_t e4 = md->precision == CMDG_MIXED ? cudaMalloc(&h->d_Sp, sizeof(float) * h->len) : cudaSuccess;
    cudaError_t e5 = h->single ? cudaMalloc(&h->d_AB1, sizeof(double) * (2 * h->bw + 1) * h->lm.n) : cudaSuccess;
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess || e5 != cudaSuccess) {
        cudaGetLastError();
        cmdg_hevi_destroy(ho);
        set_error("HEVI: device allocation of %zu bytes failed", sizeof(double) * (ab + 7 * h->len));
        return CMDG_ERR_ALLOC;
    }
    cudaStream_t s = 0;
    rc = CMDG_OK;
    if (cudaMemsetAsync(h->d_AB, 0, sizeof(double) * ab, s) != cudaSuccess ||
        cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), s) != cudaSuccess) {
        set_error("HEVI: cudaMemsetAsync failed");
        rc = CMDG_ERR_CUDA;
    }
    if (!rc) rc = hevi_assemble(h, s);
    unsigned err = 0;
    if (!rc && cudaMemcpy(&err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error("HEVI: reading the assembly status failed");
        rc = CMDG_ERR_CUDA;
    }
    if (!rc && (err & 7u)) {
        set_error((err & 1u)   ? "HEVI: the linear operator couples unknowns outside the column band"
                  : (err & 2u) ? "HEVI: zero or non-finite pivot in the column LU"
                               : "HEVI: the column LU factors have non-zeros outside the element-coupling pattern");
        rc = CMDG_ERR_NONFINITE;
    }
    if (!rc && (err & 8u)) {
        set_error("HEVI: SingleColumnLU needs identical column matrices (use ManyColumnLU on this mesh)");
        rc = CMDG_ERR_ARG;
    }
    if (!rc && shell_remainder_supported(md)) {
        h->rem = 1;
        if (h->split) {
            // l(q_ref): the reference state as a full state (zero perturbation)
            if (cudaMalloc(&h->d_lref, sizeof(double) * h->len) != cudaSuccess) {
                cudaGetLastError();
                set_error("HEVI: device allocation of %zu bytes failed", sizeof(double) * h->len);
                rc = CMDG_ERR_ALLOC;
            }
            if (!rc && cudaMemsetAsync(h->d_Sp, 0, sizeof(float) * h->len, s) != cudaSuccess) {
                set_error("HEVI: cudaMemsetAsync failed");
                rc = CMDG_ERR_CUDA;
            }
            if (!rc) rc = launch_from_perturbation(md, h->Y(), h->d_Sp, s);
            if (!rc) rc = launch_linear_tendency(md, h->Y(), h->d_lref, 1.0, 0.0, s);
            if (!rc && cudaStreamSynchronize(s) != cudaSuccess) {
                set_error("HEVI: forming the reference state's linear tendency failed");
                rc = CMDG_ERR_CUDA;
            }
        }
    }
    if (rc) {
        cmdg_hevi_destroy(ho);
        return rc;
    }
    if (h->single) {  // only the first line's factors are kept
        cudaFree(h->d_AB);
        h->d_AB = nullptr;
    }
    *out = ho;
    return CMDG_OK;
}

int cmdg_hevi_destroy(cmdg_hevi* hevi) {
    if (!hevi) return CMDG_OK;
    cudaFree(hevi->h.d_AB);
    cudaFree(hevi->h.d_AB1);
    cudaFree(hevi->h.d_buf);
    cudaFree(hevi->h.d_Sp);
    cudaFree(hevi->h.d_lref);
    cudaFree(hevi->h.d_err);
    delete hevi;
    return CMDG_OK;
}

int cmdg_hevi_info(const cmdg_hevi* hevi, double* alpha, int* bandwidth, int64_t* nline) {
    CMDG_ARG_CHECK(hevi != nullptr, "hevi is NULL");
    if (alpha) *alpha = hevi->h.alpha;
    if (bandwidth) *bandwidth = hevi->h.bw;
    if (nline) *nline = hevi->h.lm.nline;
    return CMDG_OK;
}

int cmdg_hevi_solve(cmdg_hevi* hevi, double* d_Q, const double* d_Qhat, void* stream) {
    CMDG_ARG_CHECK(hevi != nullptr && d_Q != nullptr && d_Qhat != nullptr, "NULL argument");
    return hevi_solve(&hevi->h, d_Qhat, d_Q, 0, (cudaStream_t)stream);
}

int cmdg_hevi_step(cmdg_hevi* hevi, double* d_Q, double t, int nsteps, void* stream) {
    (void)t;
    CMDG_ARG_CHECK(hevi != nullptr && d_Q != nullptr, "NULL argument");
    CMDG_ARG_CHECK(nsteps >= 0, "nsteps must be >= 0");
    for (int i = 0; i < nsteps; ++i) {
        int rc = hevi_step(&hevi->h, d_Q, (cudaStream_t)stream);
        if (rc) return rc;
    }
    return CMDG_OK;
}

}  // extern "C"
