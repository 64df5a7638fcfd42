// Host-side set-up of meshes given by the reference's own grid arrays
// (DiscontinuousSpectralElementGrid.vgeo, vmap+, elemtobndy; src/Numerics/
// Mesh/Grids.jl:76-125, 559-638) and of the per-node model tables on them.
//
// The geometry is taken as given: the curl-invariant metric terms
// dxi_d/dx_j and M of vgeo (J = M / (w_i w_j w_k)), the node coordinates,
// and the facing node of every face node from vmap+.  The geopotential, its
// DG gradient and the hydrostatic reference state are the caller's aux
// values (cmdg_model_set_reference), so a model on such a mesh evaluates the
// reference's tendency on the reference's own discrete state.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "cmdg_internal.h"

namespace cmdg {

int build_arrays(const cmdg_grid_arrays* d, Mesh* m) {
    CMDG_ARG_CHECK(d != nullptr, "grid-arrays descriptor is NULL");
    CMDG_ARG_CHECK(d->N >= MIN_N && d->N <= MAX_N, "polynomial order N=%d outside the built range [%d, %d]", d->N,
                   MIN_N, MAX_N);
    CMDG_ARG_CHECK(d->nelem > 0 && d->nelem < ((int64_t)1 << 28), "nelem=%lld out of range", (long long)d->nelem);
    CMDG_ARG_CHECK(d->vgeo != nullptr && d->vmap_plus != nullptr && d->elemtobndy != nullptr, "NULL grid array");
    m->kind = MESH_ARRAYS;
    std::memset(&m->desc, 0, sizeof(m->desc));
    m->N = d->N;
    m->Nq = d->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = d->nelem;
    m->nz = 1;
    m->nlev = m->Nq;
    lgl_derivative(m);
    const int N = m->N, Nq = m->Nq, Np = m->Np, Nfp = m->Nfp;
    const int64_t nelem = m->nelem;
    constexpr int NVG = 16;  // vgeo fields (Grids.jl:76-92)
    m->xyz.assign((size_t)nelem * 3 * Np, 0.0);
    m->cgeo.assign((size_t)nelem * CG_NFIELDS * Np, 0.0);
    for (int64_t e = 0; e < nelem; ++e) {
        const double* V = d->vgeo + (size_t)e * NVG * Np;
        double* G = &m->cgeo[(size_t)e * CG_NFIELDS * Np];
        double* X = &m->xyz[(size_t)e * 3 * Np];
        for (int n = 0; n < Np; ++n) {
            // vgeo field d + 3 j holds dxi_d/dx_j; CG_XI is d-major
            for (int dd = 0; dd < 3; ++dd)
                for (int j = 0; j < 3; ++j) G[(CG_XI + 3 * dd + j) * Np + n] = V[(dd + 3 * j) * Np + n];
            const int i = n % Nq, jj = (n / Nq) % Nq, k = n / Nfp;
            const double M = V[9 * Np + n];
            CMDG_ARG_CHECK(M > 0 && std::isfinite(M), "vgeo: M must be positive at element %lld node %d", (long long)e,
                           n);
            G[CG_M * Np + n] = M;
            G[CG_J * Np + n] = M / (m->omega[i] * m->omega[jj] * m->omega[k]);
            for (int c = 0; c < 3; ++c) X[c * Np + n] = V[(12 + c) * Np + n];
        }
        // nearest node along the element lines
        for (int n = 0; n < Np; ++n) {
            const int i = n % Nq, jj = (n / Nq) % Nq, k = n / Nfp;
            double best = INFINITY;
            auto dist = [&](int o) {
                double s = 0;
                for (int c = 0; c < 3; ++c) {
                    const double dx = X[c * Np + n] - X[c * Np + o];
                    s += dx * dx;
                }
                best = std::min(best, std::sqrt(s));
            };
            if (i > 0) dist(n - 1);
            if (i < N) dist(n + 1);
            if (jj > 0) dist(n - Nq);
            if (jj < N) dist(n + Nq);
            if (k > 0) dist(n - Nfp);
            if (k < N) dist(n + Nfp);
            G[CG_DXMIN * Np + n] = best;
        }
    }
    // connectivity: neighbour element per face (or -tag) and the facing node of every face node
    auto face_node = [&](int f, int fn) {
        const int fd = f >> 1, side = (f & 1) ? N : 0, a = fn % Nq, b = fn / Nq;
        return fd == 0 ? side + Nq * fn : (fd == 1 ? a + Nq * (side + Nq * b) : fn + Nfp * side);
    };
    m->nbr.assign((size_t)nelem * NBR_STRIDE, 0);
    m->fpart.assign((size_t)nelem * 6 * Nfp, 0);
    const int64_t nnode = nelem * Np;
    for (int64_t e = 0; e < nelem; ++e) {
        int* row = &m->nbr[(size_t)e * NBR_STRIDE];
        for (int f = 0; f < 6; ++f) {
            const int64_t tag = d->elemtobndy[e * 6 + f];
            int* part = &m->fpart[((size_t)e * 6 + f) * Nfp];
            if (tag != 0) {
                CMDG_ARG_CHECK(tag > 0 && tag < (1 << 30), "elemtobndy: bad tag %lld", (long long)tag);
                row[f] = -(int)tag;
                for (int fn = 0; fn < Nfp; ++fn) part[fn] = face_node(f, fn);
                continue;
            }
            int64_t e2 = -1;
            for (int fn = 0; fn < Nfp; ++fn) {
                const int64_t id = d->vmap_plus[(e * 6 + f) * Nfp + fn] - 1;
                CMDG_ARG_CHECK(id >= 0 && id < nnode, "vmap_plus: index %lld out of range", (long long)(id + 1));
                const int64_t ee = id / Np;
                if (fn == 0) e2 = ee;
                CMDG_ARG_CHECK(ee == e2, "element %lld face %d: the face nodes face different elements", (long long)e,
                               f);
                part[fn] = (int)(id % Np);
            }
            row[f] = (int)e2;
        }
        row[6] = 0;
        row[7] = 0;
    }
    m->zlev.assign(m->nlev, 0.0);
    m->dzlev.assign(m->nlev, 0.0);
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_nbr, sizeof(int) * m->nbr.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_nbr, m->nbr.data(), sizeof(int) * m->nbr.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_fpart, sizeof(int) * m->fpart.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_fpart, m->fpart.data(), sizeof(int) * m->fpart.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

namespace {

// uploads the per-node kernel geometry (FP64 and FP32 copies), replacing any earlier copy
int upload_arrays_geo(Model* md, const std::vector<double>& geo) {
    std::vector<float> g32(geo.begin(), geo.end());
    if (!md->d_geo64) CMDG_CUDA_CHECK(cudaMalloc(&md->d_geo64, sizeof(double) * geo.size()));
    if (!md->d_geo32) CMDG_CUDA_CHECK(cudaMalloc(&md->d_geo32, sizeof(float) * g32.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_geo64, geo.data(), sizeof(double) * geo.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_geo32, g32.data(), sizeof(float) * g32.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

}  // namespace

// Per-node tables of a model on a grid-arrays mesh before its reference is
// set: J dxi/dx, 1/J, a zero geopotential and reference state (pressure
// coefficient R_d T_0), M and the nearest-node distance, zero reference jumps.
int init_arrays_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const int Np = m.Np, Nfp = m.Nfp;
    const int64_t nelem = m.nelem;
    md->arrays_geo.assign((size_t)nelem * KG_NFIELDS * Np, 0.0);
    std::vector<double> mass((size_t)nelem * Np), dxmin((size_t)nelem * Np);
    const double crho0 = md->prm.R_d * md->prm.T_0;
    for (int64_t e = 0; e < nelem; ++e) {
        const double* G = &m.cgeo[(size_t)e * CG_NFIELDS * Np];
        double* K = &md->arrays_geo[(size_t)e * KG_NFIELDS * Np];
        for (int n = 0; n < Np; ++n) {
            const double J = G[CG_J * Np + n];
            for (int w = 0; w < 9; ++w) K[(KG_JXI + w) * Np + n] = J * G[(CG_XI + w) * Np + n];
            K[KG_INVJ * Np + n] = 1.0 / J;
            K[KG_DCRHO * Np + n] = crho0;
            mass[(size_t)e * Np + n] = G[CG_M * Np + n];
            dxmin[(size_t)e * Np + n] = G[CG_DXMIN * Np + n];
        }
    }
    int rc = upload_arrays_geo(md, md->arrays_geo);
    if (rc) return rc;
    md->ref64.assign((size_t)nelem * 2 * Np, 0.0);
    md->pref64.assign((size_t)nelem * Np, 0.0);
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_ref64, sizeof(double) * md->ref64.size()));
    CMDG_CUDA_CHECK(cudaMemset(md->d_ref64, 0, sizeof(double) * md->ref64.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_fjump, sizeof(float) * 2 * (size_t)nelem * 6 * Nfp));
    CMDG_CUDA_CHECK(cudaMemset(md->d_fjump, 0, sizeof(float) * 2 * (size_t)nelem * 6 * Nfp));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_mass, sizeof(double) * mass.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_dxmin, sizeof(double) * dxmin.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_mass, mass.data(), sizeof(double) * mass.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_dxmin, dxmin.data(), sizeof(double) * dxmin.size(), cudaMemcpyHostToDevice));
    md->has_reference = false;
    return CMDG_OK;
}

// The caller's geopotential, its gradient and the reference state, (Np, 7, nelem).
int set_arrays_reference(Model* md, const double* aux7) {
    // a filter's cached copy of the reference state belongs to the old one
    cudaFree(md->d_filter_ref64);
    md->d_filter_ref64 = nullptr;
    cudaFree(md->d_filter_corr_node);
    md->d_filter_corr_node = nullptr;
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    const int Np = m.Np, Nfp = m.Nfp;
    const int64_t nelem = m.nelem;
    std::vector<double>& geo = md->arrays_geo;
    for (int64_t e = 0; e < nelem; ++e) {
        double* K = &geo[(size_t)e * KG_NFIELDS * Np];
        const double* A = aux7 + (size_t)e * 7 * Np;
        for (int n = 0; n < Np; ++n) {
            for (int w = 0; w < 7; ++w)
                CMDG_ARG_CHECK(std::isfinite(A[w * Np + n]), "aux: non-finite value at element %lld node %d",
                               (long long)e, n);
            const double phi = A[0 * Np + n];
            for (int c = 0; c < 3; ++c) K[(KG_GPHI + c) * Np + n] = p.gravity || p.orientation ? A[(1 + c) * Np + n] : 0.0;
            K[KG_DCRHO * Np + n] = p.R_d * p.T_0 - (p.R_d / p.cv_d) * phi;
            const double rho = p.ref_state ? A[4 * Np + n] : 0.0, rhoe = p.ref_state ? A[5 * Np + n] : 0.0,
                         pr = p.ref_state ? A[6 * Np + n] : 0.0;
            K[KG_DRHO * Np + n] = rho;
            K[KG_DRHOE * Np + n] = rhoe;
            K[KG_DPREF * Np + n] = pr;
            md->ref64[((size_t)e * 2 + 0) * Np + n] = rho;
            md->ref64[((size_t)e * 2 + 1) * Np + n] = rhoe;
            md->pref64[(size_t)e * Np + n] = pr;
        }
    }
    // reference jumps q_ref(-) - q_ref(+) at every face node, in FP64
    std::vector<float> jump((size_t)2 * nelem * 6 * Nfp, 0.0f);
    const int N = m.N, Nq = m.Nq;
    for (int64_t e = 0; e < nelem; ++e)
        for (int f = 0; f < 6; ++f) {
            const int e2 = m.nbr[(size_t)e * NBR_STRIDE + f];
            if (e2 < 0) continue;
            for (int fn = 0; fn < Nfp; ++fn) {
                const int fd = f >> 1, side = (f & 1) ? N : 0, a = fn % Nq, b = fn / Nq;
                const int vM = fd == 0 ? side + Nq * fn : (fd == 1 ? a + Nq * (side + Nq * b) : fn + Nfp * side);
                const int vP = m.fpart[((size_t)e * 6 + f) * Nfp + fn];
                const size_t j = ((size_t)e * 6 + f) * Nfp + fn;
                for (int s = 0; s < 2; ++s)
                    jump[2 * j + s] = (float)(md->ref64[((size_t)e * 2 + s) * Np + vM] -
                                              md->ref64[((size_t)e2 * 2 + s) * Np + vP]);
            }
        }
    int rc = upload_arrays_geo(md, geo);
    if (rc) return rc;
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_ref64, md->ref64.data(), sizeof(double) * md->ref64.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_fjump, jump.data(), sizeof(float) * jump.size(), cudaMemcpyHostToDevice));
    md->has_reference = true;
    // mixed precision with a closure: the FP64 gradients of the reference
    // h_tot (and theta_v) that the stage kernel adds to the perturbation's
    if (md->precision == CMDG_MIXED && p.turbulence != CMDG_TURB_NONE && p.ref_state) {
        rc = visc_reference_gradients(md);
        if (rc) return rc;
    }
    // the linear model's tables hold the previous reference state
    cudaFree(md->d_lin64);
    cudaFree(md->d_linface64);
    md->d_lin64 = nullptr;
    md->d_linface64 = nullptr;
    for (auto& kv : md->graphs) cudaGraphExecDestroy(kv.second);
    md->graphs.clear();
    return CMDG_OK;
}

}  // namespace cmdg
