// Filters applied to a state between steps (src/Numerics/Mesh/Filters.jl):
// spectral filters (ExponentialFilter, CutoffFilter, BoydVandevenFilter) and
// the TMAR nonnegativity filter.
//
// Spectral: W = V diag(Sigma) V^-1 with V the Legendre Vandermonde matrix at
// the LGL points (spectral_filter_matrix, Filters.jl:114-128); applied in
// place along xi1 and xi2 with the horizontal matrix and along xi3 with the
// vertical one (kernel_apply_filter! through apply_async!, :440-505,
// :651-790).  One CTA per element stages the filtered fields in shared
// memory and sweeps the three directions with a barrier between sweeps.
// Mixed precision filters the FP32 perturbation and adds the FP64-computed
// change of the reference state under the filter, W q_ref - q_ref: on a
// brick whose horizontal filter keeps constants, per vertical node level (a
// level function is left unchanged by the horizontal filter, whose constant
// mode has Sigma_0 = 1); otherwise (cubed shells and grid arrays, whose
// reference state varies along a level, or a horizontal filter that does not
// keep constants) per node, by the FP64 filter applied to the reference
// state itself.
//
// TMAR (kernel_apply_TMAR_filter!, :794-892): per element and field,
// r = sum(M q) / sum(M max(q, 0)) (0 when sum(M q) <= 0), q <- r q where
// q >= 0 and 0 elsewhere, on the full state.
#include <cmath>
#include <vector>

#include "cmdg_internal.h"

namespace cmdg {

static int filter_matrix(int N, int kind, int Nc, int s, double alpha, std::vector<double>& W) {
    const int Nq = N + 1;
    std::vector<double> r, w;
    lgl_nodes(N, r, w);
    // Legendre Vandermonde V[i][n] = P_n(r_i) (the normalisation cancels in V diag V^-1)
    std::vector<double> V((size_t)Nq * Nq);
    for (int i = 0; i < Nq; ++i) {
        double pm = 0.0, p = 1.0;
        for (int n = 0; n < Nq; ++n) {
            V[(size_t)i * Nq + n] = p;
            const double pn = ((2 * n + 1) * r[i] * p - n * pm) / (n + 1);
            pm = p;
            p = pn;
        }
    }
    std::vector<double> sig(Nq, 1.0);
    for (int n = Nc; n <= N; ++n) {
        const double eta = (N == Nc) ? 0.0 : (double)(n - Nc) / (N - Nc);
        if (kind == CMDG_FILTER_EXPONENTIAL) {
            sig[n] = std::exp(-alpha * std::pow(eta, s));
        } else if (kind == CMDG_FILTER_CUTOFF) {
            sig[n] = 0.0;
        } else {
            const double a = 2 * std::fabs(eta) - 1;
            const double chi = (a == 0) ? 1.0 : std::sqrt(-std::log1p(-a * a) / (a * a));
            sig[n] = std::erfc(std::sqrt((double)s) * chi * a) / 2;
        }
    }
    // W V = V diag(sig): W^T = V^-T (V diag sig)^T, Gauss-Jordan with partial pivoting
    std::vector<double> A((size_t)Nq * Nq), B((size_t)Nq * Nq);
    for (int i = 0; i < Nq; ++i)
        for (int j = 0; j < Nq; ++j) {
            A[(size_t)i * Nq + j] = V[(size_t)j * Nq + i];
            B[(size_t)i * Nq + j] = V[(size_t)j * Nq + i] * sig[i];
        }
    for (int c = 0; c < Nq; ++c) {
        int piv = c;
        for (int i = c + 1; i < Nq; ++i)
            if (std::fabs(A[(size_t)i * Nq + c]) > std::fabs(A[(size_t)piv * Nq + c])) piv = i;
        for (int j = 0; j < Nq; ++j) {
            std::swap(A[(size_t)c * Nq + j], A[(size_t)piv * Nq + j]);
            std::swap(B[(size_t)c * Nq + j], B[(size_t)piv * Nq + j]);
        }
        const double d = A[(size_t)c * Nq + c];
        if (d == 0) return CMDG_ERR_ARG;
        for (int j = 0; j < Nq; ++j) {
            A[(size_t)c * Nq + j] /= d;
            B[(size_t)c * Nq + j] /= d;
        }
        for (int i = 0; i < Nq; ++i) {
            if (i == c) continue;
            const double f = A[(size_t)i * Nq + c];
            for (int j = 0; j < Nq; ++j) {
                A[(size_t)i * Nq + j] -= f * A[(size_t)c * Nq + j];
                B[(size_t)i * Nq + j] -= f * B[(size_t)c * Nq + j];
            }
        }
    }
    W.assign((size_t)Nq * Nq, 0.0);
    for (int i = 0; i < Nq; ++i)
        for (int j = 0; j < Nq; ++j) W[(size_t)i * Nq + j] = B[(size_t)j * Nq + i];
    return CMDG_OK;
}

namespace {

constexpr int FNQ = MAX_N + 1;

struct FilterArgs {
    void* Q;
    const float* corr;        // mixed: [nlev][2] level corrections for rho, rhoe (or NULL)
    const float* corr_node;   // mixed: [nelem][2][Np] node corrections for rho, rhoe (or NULL)
    double Wh64[FNQ * FNQ], Wv64[FNQ * FNQ];
    float Wh32[FNQ * FNQ], Wv32[FNQ * FNQ];
    const int* nbr;           // neighbour rows: entry 6 is the element's vertical index
    int horizontal, vertical;
    unsigned field_mask;
};

template <typename R>
struct FW;
template <>
struct FW<double> {
    static __device__ __forceinline__ double h(const FilterArgs& A, int i) { return A.Wh64[i]; }
    static __device__ __forceinline__ double v(const FilterArgs& A, int i) { return A.Wv64[i]; }
};
template <>
struct FW<float> {
    static __device__ __forceinline__ float h(const FilterArgs& A, int i) { return A.Wh32[i]; }
    static __device__ __forceinline__ float v(const FilterArgs& A, int i) { return A.Wv32[i]; }
};

template <int N, typename R>
__global__ void __launch_bounds__(((N + 1) * (N + 1) * (N + 1) + 31) / 32 * 32)
    spectral_filter_kernel(const FilterArgs A) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    __shared__ R s_q[NSTATE][Np];
    const int e = blockIdx.x, t = threadIdx.x;
    const bool node = t < Np;
    const int k = t / Nfp, j = (t - k * Nfp) / Nq, i = t - k * Nfp - j * Nq;
    R* Q = static_cast<R*>(A.Q) + (size_t)e * NSTATE * Np;
    R v[NSTATE];
#pragma unroll
    for (int s = 0; s < NSTATE; ++s)
        if (node && ((A.field_mask >> s) & 1u)) v[s] = Q[s * Np + t];
    auto sweep = [&](int d) {
#pragma unroll
        for (int s = 0; s < NSTATE; ++s)
            if (node && ((A.field_mask >> s) & 1u)) s_q[s][t] = v[s];
        __syncthreads();
        if (node) {
            const int row = d == 0 ? i : (d == 1 ? j : k);
            const int base = d == 0 ? Nq * (j + Nq * k) : (d == 1 ? i + Nfp * k : i + Nq * j);
            const int st = d == 0 ? 1 : (d == 1 ? Nq : Nfp);
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                if (!((A.field_mask >> s) & 1u)) continue;
                R acc = 0;
#pragma unroll
                for (int n = 0; n < Nq; ++n) {
                    const R w = d == 2 ? FW<R>::v(A, row * Nq + n) : FW<R>::h(A, row * Nq + n);
                    acc = fma(w, s_q[s][base + n * st], acc);
                }
                v[s] = acc;
            }
        }
        __syncthreads();
    };
    if (A.horizontal) {
        sweep(0);
        sweep(1);
    }
    if (A.vertical) sweep(2);
    if (!node) return;
    if (A.corr) {
        const int lev = __ldg(A.nbr + (size_t)e * NBR_STRIDE + 6) * Nq + k;
        if (A.field_mask & 1u) v[0] += (R)A.corr[2 * lev + 0];
        if (A.field_mask & 16u) v[4] += (R)A.corr[2 * lev + 1];
    }
    if (A.corr_node) {
        const float* c = A.corr_node + (size_t)e * 2 * Np + t;
        if (A.field_mask & 1u) v[0] += (R)c[0];
        if (A.field_mask & 16u) v[4] += (R)c[Np];
    }
#pragma unroll
    for (int s = 0; s < NSTATE; ++s)
        if ((A.field_mask >> s) & 1u) Q[s * Np + t] = v[s];
}

template <int N, typename R>
cudaError_t launch_filter_N(const FilterArgs& A, int64_t nelem, cudaStream_t s) {
    constexpr int Np = (N + 1) * (N + 1) * (N + 1);
    spectral_filter_kernel<N, R><<<(unsigned)nelem, (Np + 31) / 32 * 32, 0, s>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_filter(const FilterArgs& A, int N, bool fp32, int64_t nelem, cudaStream_t s) {
    switch (N) {
        case 2: return fp32 ? launch_filter_N<2, float>(A, nelem, s) : launch_filter_N<2, double>(A, nelem, s);
        case 3: return fp32 ? launch_filter_N<3, float>(A, nelem, s) : launch_filter_N<3, double>(A, nelem, s);
        case 4: return fp32 ? launch_filter_N<4, float>(A, nelem, s) : launch_filter_N<4, double>(A, nelem, s);
        default: return fp32 ? launch_filter_N<5, float>(A, nelem, s) : launch_filter_N<5, double>(A, nelem, s);
    }
}

// corr[e][c][n] = W q_ref - q_ref of rho (c = 0) and rhoe (c = 1), from the
// filtered FP64 reference state Wq and the reference state q
__global__ void node_correction_kernel(float* __restrict__ corr, const double* __restrict__ Wq,
                                       const double* __restrict__ q, int64_t nelem, int Np) {
    const int64_t total = nelem * 2 * Np;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / (2 * Np);
        const int c = (int)((i / Np) % 2), n = (int)(i % Np);
        const size_t src = ((size_t)e * NSTATE + (c ? 4 : 0)) * Np + n;
        corr[i] = (float)(Wq[src] - q[src]);
    }
}

// TMAR: one CTA per element; sums of M q and M max(q, 0) in FP64
template <int N, typename R, bool MIXED>
__global__ void __launch_bounds__(256) tmar_kernel(void* Qv, const double* emetric, const double* mnode,
                                                   const double* w, const double* lvl, const double* refn, const int* nbr,
                                                   unsigned field_mask) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    __shared__ double red[2][256];
    const int e = blockIdx.x, t = threadIdx.x;
    R* Q = static_cast<R*>(Qv) + (size_t)e * NSTATE * Np;
    for (int s = 0; s < NSTATE; ++s) {
        if (!((field_mask >> s) & 1u)) continue;
        double a = 0, b = 0;
        for (int n = t; n < Np; n += blockDim.x) {
            const int i = n % Nq, j = (n / Nq) % Nq, k = n / Nfp;
            const double M = mnode ? mnode[(size_t)e * Np + n]
                                   : (1.0 / (emetric[3 * e] * emetric[3 * e + 1] * emetric[3 * e + 2])) *
                                         (w[i] * w[j] * w[k]);
            double q = (double)Q[s * Np + n];
            if (MIXED && (s == 0 || s == 4)) {
                q += refn ? refn[((size_t)e * 2 + (s == 4)) * Np + n]
                          : lvl[(size_t)(nbr[(size_t)e * NBR_STRIDE + 6] * Nq + k) * LV_NFIELDS + (s == 0 ? LV_RHO_REF : LV_RHOE_REF)];
            }
            a += M * q;
            b += M * (q >= 0 ? q : 0.0);
        }
        red[0][t] = a;
        red[1][t] = b;
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (t < off) {
                red[0][t] += red[0][t + off];
                red[1][t] += red[1][t + off];
            }
            __syncthreads();
        }
        const double sum = red[0][0], sumc = red[1][0];
        const double r = sum > 0 ? sum / sumc : 0.0;
        for (int n = t; n < Np; n += blockDim.x) {
            const int k = n / Nfp;
            double ref = 0;
            if (MIXED && (s == 0 || s == 4))
                ref = refn ? refn[((size_t)e * 2 + (s == 4)) * Np + n]
                           : lvl[(size_t)(nbr[(size_t)e * NBR_STRIDE + 6] * Nq + k) * LV_NFIELDS + (s == 0 ? LV_RHO_REF : LV_RHOE_REF)];
            const double q = (double)Q[s * Np + n] + ref;
            Q[s * Np + n] = (R)((q >= 0 ? r * q : 0.0) - ref);
        }
        __syncthreads();
    }
}

// MassPreservingCutoffFilter pass (Filters.jl:895-1065), FP64: one CTA per
// element; the filtered fields are swept along xi1 and xi2 (horizontal) or
// xi3 (vertical) with W in shared memory, then shifted by the element's lost
// mass (sum M q_before - sum M q_after) / sum M, the three sums reduced in
// the CTA.
template <int N>
__global__ void __launch_bounds__(((N + 1) * (N + 1) * (N + 1) + 31) / 32 * 32)
    mp_filter_kernel(double* Qv, const double* emetric, const double* mnode, const double* w, const FilterArgs A) {
    constexpr int Nq = N + 1, Nfp = Nq * Nq, Np = Nq * Nfp;
    constexpr int NT = (Np + 31) / 32 * 32;
    constexpr int NW = NT / 32;
    __shared__ double s_q[Np];
    __shared__ double red[3][NW];
    const int e = blockIdx.x, t = threadIdx.x;
    const bool node = t < Np;
    const int k = t / Nfp, j = (t - k * Nfp) / Nq, i = t - k * Nfp - j * Nq;
    double* Q = Qv + (size_t)e * NSTATE * Np;
    const double M = !node ? 0.0
                     : mnode ? mnode[(size_t)e * Np + t]
                             : (1.0 / (emetric[3 * e] * emetric[3 * e + 1] * emetric[3 * e + 2])) *
                                   (w[i] * w[j] * w[k]);
    auto sweep = [&](double v, int d) {
        if (node) s_q[t] = v;
        __syncthreads();
        double acc = 0;
        if (node) {
            const int row = d == 0 ? i : (d == 1 ? j : k);
            const int base = d == 0 ? Nq * (j + Nq * k) : (d == 1 ? i + Nfp * k : i + Nq * j);
            const int st = d == 0 ? 1 : (d == 1 ? Nq : Nfp);
#pragma unroll
            for (int n = 0; n < Nq; ++n)
                acc += (d == 2 ? A.Wv64[row * Nq + n] : A.Wh64[row * Nq + n]) * s_q[base + n * st];
        }
        __syncthreads();
        return acc;
    };
    for (int s = 0; s < NSTATE; ++s) {
        if (!((A.field_mask >> s) & 1u)) continue;
        const double q = node ? Q[s * Np + t] : 0.0;
        double v = q;
        if (A.horizontal) {
            v = sweep(v, 0);
            v = sweep(v, 1);
        } else {
            v = sweep(v, 2);
        }
        // three sums: warp shuffles, then the warps' partials
        double r0 = M * q, r1 = M * v, r2 = M;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            r0 += __shfl_down_sync(0xffffffffu, r0, off);
            r1 += __shfl_down_sync(0xffffffffu, r1, off);
            r2 += __shfl_down_sync(0xffffffffu, r2, off);
        }
        if ((t & 31) == 0) {
            red[0][t >> 5] = r0;
            red[1][t >> 5] = r1;
            red[2][t >> 5] = r2;
        }
        __syncthreads();
        if (t == 0) {
            for (int wi = 1; wi < NW; ++wi) {
                red[0][0] += red[0][wi];
                red[1][0] += red[1][wi];
                red[2][0] += red[2][wi];
            }
        }
        __syncthreads();
        const double Minv = 1 / red[2][0];
        if (node) Q[s * Np + t] = v + Minv * (red[0][0] - red[1][0]);
        __syncthreads();
    }
}

}  // namespace

static int field_mask_of(const int* fields, int nfields, unsigned* mask) {
    *mask = 0;
    for (int f = 0; f < nfields; ++f) {
        CMDG_ARG_CHECK(fields[f] >= 0 && fields[f] < NSTATE, "field index %d out of range", fields[f]);
        *mask |= 1u << fields[f];
    }
    return CMDG_OK;
}

}  // namespace cmdg

using namespace cmdg;

extern "C" int cmdg_filter_matrix(int N, int kind, int Nc, int s, double alpha, double* h_W) {
    CMDG_ARG_CHECK(h_W != nullptr, "NULL output");
    CMDG_ARG_CHECK(N >= 1 && N <= 15, "N must be in [1, 15]");
    CMDG_ARG_CHECK(Nc >= 0 && Nc <= N, "Nc must be in [0, N]");
    CMDG_ARG_CHECK(kind == CMDG_FILTER_EXPONENTIAL || kind == CMDG_FILTER_CUTOFF || kind == CMDG_FILTER_BOYD_VANDEVEN,
                   "unknown filter kind %d", kind);
    CMDG_ARG_CHECK(kind == CMDG_FILTER_CUTOFF || (s > 0 && s % 2 == 0), "the filter order s must be even and positive");
    std::vector<double> W;
    int rc = filter_matrix(N, kind, Nc, s, alpha, W);
    if (rc) {
        set_error("singular Vandermonde matrix");
        return rc;
    }
    for (size_t i = 0; i < W.size(); ++i) h_W[i] = W[i];
    return CMDG_OK;
}

extern "C" int cmdg_apply_filter(cmdg_model* model, void* d_Q, const double* h_Wh, const double* h_Wv, int direction,
                                 const int* h_fields, int nfields, void* stream) {
    CMDG_ARG_CHECK(model != nullptr && d_Q != nullptr && h_fields != nullptr, "NULL argument");
    CMDG_ARG_CHECK(direction >= CMDG_DIR_EVERY && direction <= CMDG_DIR_VERTICAL, "unknown direction %d", direction);
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    const bool horiz = direction != CMDG_DIR_VERTICAL, vert = direction != CMDG_DIR_HORIZONTAL;
    CMDG_ARG_CHECK(!horiz || h_Wh != nullptr, "horizontal filter matrix is NULL");
    CMDG_ARG_CHECK(!vert || h_Wv != nullptr, "vertical filter matrix is NULL");
    FilterArgs A{};
    int rc = field_mask_of(h_fields, nfields, &A.field_mask);
    if (rc) return rc;
    const int Nq = m.Nq;
    A.Q = d_Q;
    A.nbr = m.d_nbr;
    A.horizontal = horiz;
    A.vertical = vert;
    for (int i = 0; i < Nq * Nq; ++i) {
        A.Wh64[i] = horiz ? h_Wh[i] : 0.0;
        A.Wv64[i] = vert ? h_Wv[i] : 0.0;
        A.Wh32[i] = (float)A.Wh64[i];
        A.Wv32[i] = (float)A.Wv64[i];
    }
    const bool mixed = md->precision == CMDG_MIXED;
    cudaStream_t s = (cudaStream_t)stream;
    // the reference state's change under the filter: per level on a brick
    // whose horizontal filter keeps constants (Sigma_0 = 1), else per node
    bool keeps_constants = true;
    for (int i = 0; horiz && i < Nq; ++i) {
        double rs = 0;
        for (int n = 0; n < Nq; ++n) rs += h_Wh[i * Nq + n];
        keeps_constants = keeps_constants && std::fabs(rs - 1.0) < 1e-12;
    }
    const bool ref_fields = mixed && md->prm.ref_state && (A.field_mask & 17u);
    if (ref_fields && (m.kind != MESH_BRICK || !keeps_constants)) {
        // W q_ref - q_ref per node, FP64: the filter applied to the reference
        // state itself (zero perturbation, as a full FP64 state)
        const size_t len = (size_t)m.nelem * NSTATE * m.Np;
        if (!md->d_filter_ref64) {
            float* zero = nullptr;
            CMDG_CUDA_CHECK(cudaMalloc(&md->d_filter_ref64, sizeof(double) * 2 * len));
            CMDG_CUDA_CHECK(cudaMalloc(&md->d_filter_corr_node, sizeof(float) * 2 * (size_t)m.nelem * m.Np));
            CMDG_CUDA_CHECK(cudaMalloc(&zero, sizeof(float) * len));
            cudaError_t ez = cudaMemsetAsync(zero, 0, sizeof(float) * len, s);
            rc = ez == cudaSuccess ? launch_from_perturbation(md, md->d_filter_ref64, zero, s) : CMDG_ERR_CUDA;
            if (cudaStreamSynchronize(s) != cudaSuccess && rc == CMDG_OK) rc = CMDG_ERR_CUDA;
            cudaFree(zero);
            if (rc) {
                set_error("filter: forming the reference state failed");
                return rc;
            }
        }
        double* Wq = md->d_filter_ref64 + len;
        CMDG_CUDA_CHECK(cudaMemcpyAsync(Wq, md->d_filter_ref64, sizeof(double) * len, cudaMemcpyDeviceToDevice, s));
        FilterArgs R = A;
        R.Q = Wq;
        R.corr = nullptr;
        R.corr_node = nullptr;
        R.field_mask = A.field_mask & 17u;
        CMDG_CUDA_CHECK(launch_filter(R, m.N, false, m.nelem, s));
        const int64_t total = m.nelem * 2 * (int64_t)m.Np;
        node_correction_kernel<<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16), 256, 0, s>>>(
            md->d_filter_corr_node, Wq, md->d_filter_ref64, m.nelem, m.Np);
        CMDG_CUDA_CHECK(cudaGetLastError());
        A.corr_node = md->d_filter_corr_node;
    } else if (ref_fields && vert) {
        // W_v q_ref - q_ref per level, FP64
        md->filter_corr.assign((size_t)m.nlev * 2, 0.0f);
        for (int ez = 0; ez < m.nz; ++ez)
            for (int k = 0; k < Nq; ++k)
                for (int c = 0; c < 2; ++c) {
                    const int f = c == 0 ? LV_RHO_REF : LV_RHOE_REF;
                    double acc = 0;
                    for (int n = 0; n < Nq; ++n) acc += h_Wv[k * Nq + n] * md->lvl64[(size_t)(ez * Nq + n) * LV_NFIELDS + f];
                    md->filter_corr[(size_t)(ez * Nq + k) * 2 + c] =
                        (float)(acc - md->lvl64[(size_t)(ez * Nq + k) * LV_NFIELDS + f]);
                }
        if (!md->d_filter_corr) CMDG_CUDA_CHECK(cudaMalloc(&md->d_filter_corr, sizeof(float) * md->filter_corr.size()));
        CMDG_CUDA_CHECK(cudaMemcpyAsync(md->d_filter_corr, md->filter_corr.data(), sizeof(float) * md->filter_corr.size(),
                                        cudaMemcpyHostToDevice, s));
        A.corr = md->d_filter_corr;
    }
    const cudaError_t e = launch_filter(A, m.N, mixed, m.nelem, s);
    if (e != cudaSuccess) {
        set_error("filter launch failed: %s", cudaGetErrorString(e));
        return CMDG_ERR_CUDA;
    }
    if (A.corr) CMDG_CUDA_CHECK(cudaStreamSynchronize(s));  // the host table may be rewritten by the next call
    return CMDG_OK;
}

extern "C" int cmdg_apply_mp_filter(cmdg_model* model, void* d_state, const double* h_Wh, const double* h_Wv,
                                    int direction, const int* h_fields, int nfields, void* stream) {
    CMDG_ARG_CHECK(model != nullptr && d_state != nullptr && h_fields != nullptr, "NULL argument");
    CMDG_ARG_CHECK(direction >= CMDG_DIR_EVERY && direction <= CMDG_DIR_VERTICAL, "unknown direction %d", direction);
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    cudaStream_t s = (cudaStream_t)stream;
    // a mixed model's FP32 perturbation is filtered through an FP64 copy of
    // the full state: the element masses are those of the full state
    const bool mixed = md->precision == CMDG_MIXED;
    double* d_Q = static_cast<double*>(d_state);
    if (mixed) {
        if (!md->d_mp_scratch) {
            CMDG_CUDA_CHECK(cudaMalloc(&md->d_mp_scratch, sizeof(double) * (size_t)m.nelem * NSTATE * m.Np));
        }
        d_Q = md->d_mp_scratch;
        const int rc0 = launch_from_perturbation(md, d_Q, static_cast<const float*>(d_state), s);
        if (rc0) return rc0;
    }
    const bool horiz = direction != CMDG_DIR_VERTICAL, vert = direction != CMDG_DIR_HORIZONTAL;
    CMDG_ARG_CHECK(!horiz || h_Wh != nullptr, "horizontal filter matrix is NULL");
    CMDG_ARG_CHECK(!vert || h_Wv != nullptr, "vertical filter matrix is NULL");
    FilterArgs A{};
    int rc = field_mask_of(h_fields, nfields, &A.field_mask);
    if (rc) return rc;
    const int Nq = m.Nq;
    A.Q = d_Q;
    A.nbr = m.d_nbr;
    for (int i = 0; i < Nq * Nq; ++i) {
        A.Wh64[i] = horiz ? h_Wh[i] : 0.0;
        A.Wv64[i] = vert ? h_Wv[i] : 0.0;
    }
    if (!md->d_omega) {
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_omega, sizeof(double) * m.omega.size()));
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_omega, m.omega.data(), sizeof(double) * m.omega.size(), cudaMemcpyHostToDevice));
    }
    const double* mnode = m.kind == MESH_BRICK ? nullptr : md->d_mass;
    CMDG_ARG_CHECK(m.kind == MESH_BRICK || mnode != nullptr, "no mass matrix on this mesh");
    // horizontal pass, then vertical pass, each with its own mass restoration
    for (int pass = 0; pass < 2; ++pass) {
        if ((pass == 0 && !horiz) || (pass == 1 && !vert)) continue;
        A.horizontal = pass == 0;
        A.vertical = pass == 1;
        switch (m.N) {
            case 2: mp_filter_kernel<2><<<(unsigned)m.nelem, 32, 0, s>>>(d_Q, m.d_emetric, mnode, md->d_omega, A); break;
            case 3: mp_filter_kernel<3><<<(unsigned)m.nelem, 64, 0, s>>>(d_Q, m.d_emetric, mnode, md->d_omega, A); break;
            case 4: mp_filter_kernel<4><<<(unsigned)m.nelem, 128, 0, s>>>(d_Q, m.d_emetric, mnode, md->d_omega, A); break;
            default: mp_filter_kernel<5><<<(unsigned)m.nelem, 224, 0, s>>>(d_Q, m.d_emetric, mnode, md->d_omega, A); break;
        }
        CMDG_CUDA_CHECK(cudaGetLastError());
    }
    if (mixed) return launch_to_perturbation(md, static_cast<float*>(d_state), d_Q, s);
    return CMDG_OK;
}

extern "C" int cmdg_apply_tmar(cmdg_model* model, void* d_Q, const int* h_fields, int nfields, void* stream) {
    CMDG_ARG_CHECK(model != nullptr && d_Q != nullptr && h_fields != nullptr, "NULL argument");
    Model* md = &model->m;
    const Mesh& m = *md->mesh;
    unsigned mask;
    int rc = field_mask_of(h_fields, nfields, &mask);
    if (rc) return rc;
    if (!md->d_omega) {
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_omega, sizeof(double) * m.omega.size()));
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_omega, m.omega.data(), sizeof(double) * m.omega.size(), cudaMemcpyHostToDevice));
    }
    const double* d_w = md->d_omega;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    const bool mixed = md->precision == CMDG_MIXED;
    if (e == cudaSuccess) {
#define CMDG_TMAR(NN)                                                                                            \
    if (mixed)                                                                                                   \
        tmar_kernel<NN, float, true><<<(unsigned)m.nelem, 256, 0, s>>>(d_Q, m.d_emetric, md->d_mass, d_w,        \
                                                                       md->d_lvl64, md->d_ref64, m.d_nbr, mask);   \
    else                                                                                                         \
        tmar_kernel<NN, double, false><<<(unsigned)m.nelem, 256, 0, s>>>(d_Q, m.d_emetric, md->d_mass, d_w,      \
                                                                         md->d_lvl64, md->d_ref64, m.d_nbr, mask);
        switch (m.N) {
            case 2: CMDG_TMAR(2) break;
            case 3: CMDG_TMAR(3) break;
            case 4: CMDG_TMAR(4) break;
            default: CMDG_TMAR(5) break;
        }
#undef CMDG_TMAR
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_error("TMAR filter failed: %s", cudaGetErrorString(e));
        return CMDG_ERR_CUDA;
    }
    return CMDG_OK;
}
