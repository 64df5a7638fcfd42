// Element-wise conversions and global reductions of libcmdg.
//
//  * to/from perturbation: q' = q - q_ref evaluated in FP64 and rounded to
//    FP32 (and back), the reference state taken per vertical node level, or
//    per node on a curvilinear mesh.
//  * compensated weighted sums: sum_nodes M q in double-double (TwoSum /
//    TwoProd) per block, block partials summed on the host in double-double
//    (weightedsum, src/Arrays/MPIStateArrays.jl:655-675, which accumulates in
//    DoubleFloat{Float64}).
//  * nondiffusive Courant number (src/Numerics/DGMethods/SpaceDiscretization.jl:307-365,
//    src/Atmos/Model/courant.jl, minimum node distance src/Numerics/Mesh/Grids.jl:1228-1334).
#include <algorithm>
#include <cmath>

#include "cmdg_internal.h"

namespace cmdg {
namespace {

// level row of a node: the element's vertical index (entry 6 of its
// neighbour row, so any element order works) times Nq plus the node's k
__device__ __forceinline__ int node_level(int64_t e, int node, const int* nbr, int Nq, int Nfp) {
    return __ldg(nbr + (size_t)e * NBR_STRIDE + 6) * Nq + node / Nfp;
}

// reference value of field s at a node: per-node table (curvilinear meshes) or level row
__device__ __forceinline__ double ref_value(const double* lvl, const double* refn, int64_t e, int node, int s,
                                            int Np, const int* nbr, int Nq) {
    if (s != 0 && s != 4) return 0.0;
    if (refn) return refn[((size_t)e * 2 + (s == 4)) * Np + node];
    const double* L = lvl + (size_t)node_level(e, node, nbr, Nq, Nq * Nq) * LV_NFIELDS;
    return (s == 0) ? L[LV_RHO_REF] : L[LV_RHOE_REF];
}

// One CTA per element of [e_first, e_end) (grid-stride over elements), one
// thread per node; each thread issues its five loads before converting, and
// no index needs a division.
// Qp = FP32 perturbation Q - q_ref; Qd (if not NULL) = the FP64 perturbation
__global__ void to_perturbation_kernel(float* __restrict__ Qp, double* __restrict__ Qd, const double* __restrict__ Q,
                                       const double* lvl, const double* refn, int64_t e_first, int64_t e_end, int Np,
                                       int Nq, const int* nbr) {
    for (int64_t e = e_first + blockIdx.x; e < e_end; e += gridDim.x)
        for (int node = threadIdx.x; node < Np; node += blockDim.x) {
            const size_t base = (size_t)e * NSTATE * Np + node;
            double v[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) v[s] = Q[base + (size_t)s * Np];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) {
                const double d = v[s] - ref_value(lvl, refn, e, node, s, Np, nbr, Nq);
                Qp[base + (size_t)s * Np] = (float)d;
                if (Qd) Qd[base + (size_t)s * Np] = d;
            }
        }
}

__global__ void from_perturbation_kernel(double* __restrict__ Q, const float* __restrict__ Qp, const double* lvl,
                                         const double* refn, int64_t e_first, int64_t e_end, int Np, int Nq,
                                         const int* nbr) {
    for (int64_t e = e_first + blockIdx.x; e < e_end; e += gridDim.x)
        for (int node = threadIdx.x; node < Np; node += blockDim.x) {
            const size_t base = (size_t)e * NSTATE * Np + node;
            float v[NSTATE];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s) v[s] = Qp[base + (size_t)s * Np];
#pragma unroll
            for (int s = 0; s < NSTATE; ++s)
                Q[base + (size_t)s * Np] = ref_value(lvl, refn, e, node, s, Np, nbr, Nq) + (double)v[s];
        }
}

struct dd {
    double hi, lo;
};

__device__ __forceinline__ dd dd_add(dd a, dd b) {
    double s = a.hi + b.hi;
    double bp = s - a.hi;
    double err = (a.hi - (s - bp)) + (b.hi - bp);
    err += a.lo + b.lo;
    double hi = s + err;
    return dd{hi, err - (hi - s)};
}

__device__ __forceinline__ dd two_prod(double a, double b) {
    double p = a * b;
    return dd{p, fma(a, b, -p)};
}

// Block partial (hi, lo) of sum M * q over all nodes for one field.
// M = J w_i w_j w_k with J = (dx/2)(dy/2)(dz/2) = 1/(xi1 xi2 xi3) on an affine
// brick element, or the per-node M of a curvilinear mesh (mnode != NULL).
template <bool MIXED>
__global__ void weighted_sum_kernel(const void* Qv, int field, const double* emetric, const double* w, const double* lvl,
                                    int64_t nelem, int Np, int Nq, const int* nbr, const double* mnode, const double* refn,
                                    double* partial) {
    const int Nfp = Nq * Nq;
    dd acc{0.0, 0.0};
    const int64_t total = nelem * Np;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int node = (int)(idx % Np);
        const int64_t e = idx / Np;
        const int i = node % Nq, j = (node / Nq) % Nq, k = node / Nfp;
        const double M = mnode ? mnode[idx]
                               : (1.0 / (emetric[3 * e] * emetric[3 * e + 1] * emetric[3 * e + 2])) * (w[i] * w[j] * w[k]);
        const size_t qi = ((size_t)e * NSTATE + field) * Np + node;
        double qv;
        if (MIXED) {
            const double ref = ref_value(lvl, refn, e, node, field, Np, nbr, Nq);
            // sum M*ref + M*q' as two exact products
            acc = dd_add(acc, two_prod(M, ref));
            qv = (double)static_cast<const float*>(Qv)[qi];
        } else {
            qv = static_cast<const double*>(Qv)[qi];
        }
        acc = dd_add(acc, two_prod(M, qv));
    }
    __shared__ double sh[2][256];
    sh[0][threadIdx.x] = acc.hi;
    sh[1][threadIdx.x] = acc.lo;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            dd a{sh[0][threadIdx.x], sh[1][threadIdx.x]};
            dd b{sh[0][threadIdx.x + off], sh[1][threadIdx.x + off]};
            dd c = dd_add(a, b);
            sh[0][threadIdx.x] = c.hi;
            sh[1][threadIdx.x] = c.lo;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = sh[0][0];
        partial[2 * blockIdx.x + 1] = sh[1][0];
    }
}

// max over nodes of (|u| + c) / dx_min with dx_min the distance to the
// nearest neighbouring node of the same element along xi1, xi2 or xi3.
// geo (grid-arrays meshes): per-node kernel geometry whose KG_DCRHO plane holds
// the node's pressure coefficient; otherwise the level row's
__global__ void courant_kernel(const double* __restrict__ Q, const double* emetric, const double* xi, const double* lvl,
                               Physics ph, int64_t nelem, int Np, int Nq, const int* nbr, const double* dxmin,
                               const double* geo, double* partial) {
    const int Nfp = Nq * Nq;
    double best = 0.0;
    const int64_t total = nelem * Np;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int node = (int)(idx % Np);
        const int64_t e = idx / Np;
        const int ijk[3] = {node % Nq, (node / Nq) % Nq, node / Nfp};
        double md = INFINITY;
        if (dxmin) {
            md = dxmin[idx];
        } else {
            for (int d = 0; d < 3; ++d) {
                const double h = 2.0 / emetric[3 * e + d];
                const int a = ijk[d];
                if (a > 0) md = fmin(md, 0.5 * h * (xi[a] - xi[a - 1]));
                if (a < Nq - 1) md = fmin(md, 0.5 * h * (xi[a + 1] - xi[a]));
            }
        }
        const double* L = lvl + (size_t)node_level(e, node, nbr, Nq, Nfp) * LV_NFIELDS;
        double q[NSTATE];
        for (int s = 0; s < NSTATE; ++s) q[s] = Q[((size_t)e * NSTATE + s) * Np + node];
        const double rinv = 1.0 / q[0];
        const double u0 = q[1] * rinv, u1 = q[2] * rinv, u2 = q[3] * rinv;
        const double ke2 = q[1] * u0 + q[2] * u1 + q[3] * u2;
        const double crho = geo ? geo[((size_t)e * KG_NFIELDS + KG_DCRHO) * Np + node] : L[LV_CRHO];
        const double p = ph.gm1 * (q[4] - 0.5 * ke2) + q[0] * crho;
        const double c = sqrt(ph.gamma * p * rinv);
        best = fmax(best, (sqrt(u0 * u0 + u1 * u1 + u2 * u2) + c) / md);
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = best;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int CONVERT_CTAS = 152 * 16;  // state conversions: 16 resident 128-thread CTAs per SM
constexpr int RED_THREADS = 256;

int ensure_red(Model* md) {
    if (md->d_red == nullptr) {
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_red, sizeof(double) * 2 * RED_BLOCKS));
        md->red_len = 2 * RED_BLOCKS;
    }
    return CMDG_OK;
}

// Weights w and nodes xi on the device, kept per model.
struct DeviceQuad {
    double* w = nullptr;
    double* xi = nullptr;
};
std::map<const Model*, DeviceQuad> g_quad;

int quad(Model* md, DeviceQuad& out) {
    auto it = g_quad.find(md);
    if (it != g_quad.end()) {
        out = it->second;
        return CMDG_OK;
    }
    DeviceQuad q;
    const Mesh& m = *md->mesh;
    CMDG_CUDA_CHECK(cudaMalloc(&q.w, sizeof(double) * m.Nq));
    CMDG_CUDA_CHECK(cudaMalloc(&q.xi, sizeof(double) * m.Nq));
    CMDG_CUDA_CHECK(cudaMemcpy(q.w, m.omega.data(), sizeof(double) * m.Nq, cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(q.xi, m.xi.data(), sizeof(double) * m.Nq, cudaMemcpyHostToDevice));
    g_quad[md] = q;
    out = q;
    return CMDG_OK;
}

}  // namespace

void release_quad(const Model* md) {
    auto it = g_quad.find(md);
    if (it == g_quad.end()) return;
    cudaFree(it->second.w);
    cudaFree(it->second.xi);
    g_quad.erase(it);
}

int launch_to_perturbation(Model* md, float* Qp, const double* Q, cudaStream_t s, double* Qd, int64_t e0,
                           int64_t e1) {
    const Mesh& m = *md->mesh;
    if (e1 < 0) e1 = m.nelem;
    if (e1 <= e0) return CMDG_OK;
    const unsigned grid = (unsigned)std::min<int64_t>(e1 - e0, CONVERT_CTAS);
    to_perturbation_kernel<<<grid, 128, 0, s>>>(Qp, Qd, Q, md->d_lvl64, md->d_ref64, e0, e1, m.Np, m.Nq, m.d_nbr);
    CMDG_CUDA_CHECK(cudaGetLastError());
    return CMDG_OK;
}

int launch_from_perturbation(Model* md, double* Q, const float* Qp, cudaStream_t s, int64_t e0, int64_t e1) {
    const Mesh& m = *md->mesh;
    if (e1 < 0) e1 = m.nelem;
    if (e1 <= e0) return CMDG_OK;
    const unsigned grid = (unsigned)std::min<int64_t>(e1 - e0, CONVERT_CTAS);
    from_perturbation_kernel<<<grid, 128, 0, s>>>(Q, Qp, md->d_lvl64, md->d_ref64, e0, e1, m.Np, m.Nq, m.d_nbr);
    CMDG_CUDA_CHECK(cudaGetLastError());
    return CMDG_OK;
}

static void host_dd_add(double& hi, double& lo, double bhi, double blo) {
    double s = hi + bhi;
    double bp = s - hi;
    double err = (hi - (s - bp)) + (bhi - bp);
    err += lo + blo;
    double h = s + err;
    lo = err - (h - s);
    hi = h;
}

int weighted_sums(Model* md, const void* Q, bool mixed, int nfields, const int* fields, double* out, cudaStream_t s) {
    int rc = ensure_red(md);
    if (rc) return rc;
    DeviceQuad dq;
    if ((rc = quad(md, dq))) return rc;
    const Mesh& m = *md->mesh;
    std::vector<double> h(2 * RED_BLOCKS);
    for (int f = 0; f < nfields; ++f) {
        CMDG_ARG_CHECK(fields[f] >= 0 && fields[f] < NSTATE, "field index %d out of range", fields[f]);
        if (mixed)
            weighted_sum_kernel<true><<<RED_BLOCKS, RED_THREADS, 0, s>>>(Q, fields[f], m.d_emetric, dq.w, md->d_lvl64,
                                                                        m.nelem, m.Np, m.Nq, m.d_nbr, md->d_mass,
                                                                        md->d_ref64, md->d_red);
        else
            weighted_sum_kernel<false><<<RED_BLOCKS, RED_THREADS, 0, s>>>(Q, fields[f], m.d_emetric, dq.w, md->d_lvl64,
                                                                         m.nelem, m.Np, m.Nq, m.d_nbr, md->d_mass,
                                                                        md->d_ref64, md->d_red);
        CMDG_CUDA_CHECK(cudaGetLastError());
        CMDG_CUDA_CHECK(cudaMemcpyAsync(h.data(), md->d_red, sizeof(double) * 2 * RED_BLOCKS, cudaMemcpyDeviceToHost, s));
        CMDG_CUDA_CHECK(cudaStreamSynchronize(s));
        double hi = 0, lo = 0;
        for (int b = 0; b < RED_BLOCKS; ++b) host_dd_add(hi, lo, h[2 * b], h[2 * b + 1]);
        out[f] = hi + lo;
    }
    return CMDG_OK;
}

int courant_dt(Model* md, const double* Q, double CFL, double* dt, cudaStream_t s) {
    int rc = ensure_red(md);
    if (rc) return rc;
    DeviceQuad dq;
    if ((rc = quad(md, dq))) return rc;
    const Mesh& m = *md->mesh;
    courant_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(Q, m.d_emetric, dq.xi, md->d_lvl64, md->ph, m.nelem, m.Np, m.Nq,
                                                     m.d_nbr, md->d_dxmin,
                                                     m.kind == MESH_ARRAYS ? md->d_geo64 : nullptr, md->d_red);
    CMDG_CUDA_CHECK(cudaGetLastError());
    std::vector<double> h(RED_BLOCKS);
    CMDG_CUDA_CHECK(cudaMemcpyAsync(h.data(), md->d_red, sizeof(double) * RED_BLOCKS, cudaMemcpyDeviceToHost, s));
    CMDG_CUDA_CHECK(cudaStreamSynchronize(s));
    double best = 0;
    for (double v : h) best = std::max(best, v);
    CMDG_ARG_CHECK(best > 0 && std::isfinite(best), "Courant reduction produced %g", best);
    *dt = CFL / best;
    return CMDG_OK;
}

}  // namespace cmdg
