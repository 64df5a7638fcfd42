// Host-side set-up of brick meshes and the per-level model tables.
//
// A brick element is affine, so its metric terms are three constants
// dxi_d/dx_d = 2 / dx_d; the curl-invariant metric of
// src/Numerics/Mesh/Metrics.jl:431-724 reduces to exactly these values on
// such elements (up to rounding).  Reference-state, geopotential and their
// DG derivatives depend only on the height of a node on a brick, so they are
// tabulated per vertical node level instead of per node.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "cmdg_internal.h"

namespace cmdg {

// Legendre-Gauss-Lobatto nodes (ascending) and weights by Newton iteration on
// x P_N(x) - P_{N-1}(x) = 0 with the Legendre recurrence (the rule that
// GaussQuadrature.legendre(T, N+1, both) returns, src/Numerics/Mesh/Elements.jl:11-14).
void lgl_nodes(int N, std::vector<double>& x, std::vector<double>& w) {
    const int Nq = N + 1;
    std::vector<long double> r(Nq);
    for (int i = 0; i < Nq; ++i) r[i] = -std::cos((long double)M_PI * i / N);
    auto legendre = [N](long double s, long double& PN, long double& PNm1) {
        long double a = 1, b = s;
        for (int k = 2; k <= N; ++k) {
            long double c = ((2 * k - 1) * s * b - (k - 1) * a) / k;
            a = b;
            b = c;
        }
        PN = b;
        PNm1 = a;
    };
    for (int it = 0; it < 200; ++it) {
        long double worst = 0;
        for (int i = 1; i < N; ++i) {
            long double PN, PNm1;
            legendre(r[i], PN, PNm1);
            long double step = (r[i] * PN - PNm1) / (Nq * PN);
            r[i] -= step;
            worst = std::max(worst, std::fabs(step));
        }
        if (worst < 1e-30L) break;
    }
    x.resize(Nq);
    w.resize(Nq);
    for (int i = 0; i < Nq; ++i) {
        long double s = (i == 0) ? -1.0L : (i == N) ? 1.0L : 0.5L * (r[i] - r[N - i]);
        long double PN, PNm1;
        legendre(s, PN, PNm1);
        x[i] = (double)s;
        w[i] = (double)(2.0L / ((long double)N * Nq * PN * PN));
    }
    if (N % 2 == 0) x[N / 2] = 0.0;
}

// LGL nodes and weights, the barycentric differentiation matrix
// (src/Numerics/Mesh/Elements.jl:34-82) and the weak-form operator Dhat.
void lgl_derivative(Mesh* m) {
    const int Nq = m->Nq;
    lgl_nodes(m->N, m->xi, m->omega);
    // barycentric differentiation matrix (src/Numerics/Mesh/Elements.jl:34-82)
    std::vector<double> wb(Nq, 1.0);
    for (int j = 0; j < Nq; ++j) {
        for (int i = 0; i < Nq; ++i)
            if (i != j) wb[j] *= (m->xi[j] - m->xi[i]);
        wb[j] = 1.0 / wb[j];
    }
    m->D.assign(Nq * Nq, 0.0);
    for (int j = 0; j < Nq; ++j)
        for (int k = 0; k < Nq; ++k) {
            if (j == k) {
                double s = 0;
                for (int l = 0; l < Nq; ++l)
                    if (l != k) s += 1.0 / (m->xi[k] - m->xi[l]);
                m->D[j * Nq + k] = s;
            } else {
                m->D[j * Nq + k] = (wb[k] / wb[j]) / (m->xi[j] - m->xi[k]);
            }
        }
    m->Dhat.assign(Nq * Nq, 0.0);
    for (int i = 0; i < Nq; ++i)
        for (int n = 0; n < Nq; ++n) m->Dhat[i * Nq + n] = m->D[n * Nq + i] * m->omega[n] / m->omega[i];
}

static double blend(double a, double b, int n, int i) {
    return (double)(((long double)a * (n - i) + (long double)b * i) / n);
}

int build_brick(const cmdg_brick_desc* d, Mesh* m, int topology) {
    CMDG_ARG_CHECK(d != nullptr, "brick descriptor is NULL");
    CMDG_ARG_CHECK(d->N >= MIN_N && d->N <= MAX_N, "polynomial order N=%d outside the built range [%d, %d]", d->N,
                   MIN_N, MAX_N);
    for (int k = 0; k < 3; ++k) {
        CMDG_ARG_CHECK(d->ne[k] >= 1, "ne[%d]=%d must be >= 1", k, d->ne[k]);
        CMDG_ARG_CHECK(d->hi[k] > d->lo[k], "hi[%d] must exceed lo[%d]", k, k);
        CMDG_ARG_CHECK(d->periodic[k] || (d->bc_lo[k] > 0 && d->bc_hi[k] > 0),
                       "non-periodic direction %d needs positive boundary tags", k);
    }
    const int64_t nelem = (int64_t)d->ne[0] * d->ne[1] * d->ne[2];
    CMDG_ARG_CHECK(nelem < (int64_t)1 << 31, "too many elements (%lld)", (long long)nelem);
    m->desc = *d;
    m->N = d->N;
    m->Nq = d->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = nelem;
    m->nz = d->ne[2];
    m->nlev = m->nz * m->Nq;
    const int Nq = m->Nq;

    lgl_derivative(m);

    m->emetric.assign(nelem * 3, 0.0);
    m->nbr.assign(nelem * NBR_STRIDE, 0);
    const int nx = d->ne[0], ny = d->ne[1], nz = d->ne[2];
    // element numbering: columns contiguous (vertical index fastest) in x-then-y
    // order or in the reference's StackedBrickTopology order, or every
    // element along BrickTopology's Hilbert curve (no contiguous columns)
    m->topology = topology;
    std::vector<int64_t> eid_of((size_t)nelem);  // element id of library index iz + nz (ix + nx iy)
    if (topology == CMDG_TOPOLOGY_BRICK) {
        std::vector<int64_t> perm((size_t)nelem);
        int rc = cmdg_brick_element_order(d, CMDG_TOPOLOGY_BRICK, perm.data());
        if (rc) return rc;
        for (int64_t p = 0; p < nelem; ++p) eid_of[(size_t)perm[p]] = p;
        m->col_at.clear();
    } else {
        int rc = brick_column_order(*d, topology, m->col_at);
        if (rc) return rc;
        std::vector<int> col_pos(m->col_at.size());
        for (size_t h = 0; h < m->col_at.size(); ++h) col_pos[m->col_at[h]] = (int)h;
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix)
                for (int iz = 0; iz < nz; ++iz)
                    eid_of[(size_t)iz + (size_t)nz * ((size_t)ix + (size_t)nx * iy)] =
                        (int64_t)iz + (int64_t)nz * (int64_t)col_pos[(size_t)ix + (size_t)nx * iy];
    }
    auto eid = [&](int ix, int iy, int iz) {
        return eid_of[(size_t)iz + (size_t)nz * ((size_t)ix + (size_t)nx * iy)];
    };
    m->ijk.assign((size_t)nelem * 3, 0);
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix)
            for (int iz = 0; iz < nz; ++iz) {
                int64_t e = eid(ix, iy, iz);
                m->ijk[(size_t)e * 3 + 0] = ix;
                m->ijk[(size_t)e * 3 + 1] = iy;
                m->ijk[(size_t)e * 3 + 2] = iz;
                int idx[3] = {ix, iy, iz};
                for (int dd = 0; dd < 3; ++dd) {
                    double a = blend(d->lo[dd], d->hi[dd], d->ne[dd], idx[dd]);
                    double b = blend(d->lo[dd], d->hi[dd], d->ne[dd], idx[dd] + 1);
                    m->emetric[e * 3 + dd] = 2.0 / (b - a);
                }
                for (int f = 0; f < 6; ++f) {
                    int dd = f / 2, side = f % 2;
                    int nb[3] = {ix, iy, iz};
                    nb[dd] += side ? 1 : -1;
                    int val;
                    if (nb[dd] < 0 || nb[dd] >= d->ne[dd]) {
                        if (d->periodic[dd]) {
                            nb[dd] = (nb[dd] + d->ne[dd]) % d->ne[dd];
                            val = (int)eid(nb[0], nb[1], nb[2]);
                        } else {
                            val = -(side ? d->bc_hi[dd] : d->bc_lo[dd]);
                        }
                    } else {
                        val = (int)eid(nb[0], nb[1], nb[2]);
                    }
                    m->nbr[e * NBR_STRIDE + f] = val;
                }
                m->nbr[e * NBR_STRIDE + 6] = iz;
            }
    m->zlev.assign(m->nlev, 0.0);
    m->dzlev.assign(m->nlev, 0.0);
    for (int ez = 0; ez < nz; ++ez) {
        double a = blend(d->lo[2], d->hi[2], nz, ez), b = blend(d->lo[2], d->hi[2], nz, ez + 1);
        for (int k = 0; k < Nq; ++k) {
            m->zlev[ez * Nq + k] = a + (m->xi[k] + 1) * 0.5 * (b - a);
            m->dzlev[ez * Nq + k] = 2.0 / (b - a);
        }
    }
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_emetric, sizeof(double) * m->emetric.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_nbr, sizeof(int) * m->nbr.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_emetric, m->emetric.data(), sizeof(double) * m->emetric.size(),
                               cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_nbr, m->nbr.data(), sizeof(int) * m->nbr.size(), cudaMemcpyHostToDevice));
    std::vector<float> em32(m->emetric.begin(), m->emetric.end());
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_emetric32, sizeof(float) * em32.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_emetric32, em32.data(), sizeof(float) * em32.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

// Temperature profiles (Thermodynamics.TemperatureProfiles: IsothermalProfile,
// DryAdiabaticProfile) as used by HydrostaticState (src/Atmos/Model/ref_state.jl:70-82).
void temperature_profile(const cmdg_atmos_params& p, double z, double& Tv, double& pres) {
    if (p.profile == CMDG_PROFILE_ISOTHERMAL) {
        Tv = p.T_surface;
        pres = p.MSLP * std::exp(-z * p.grav / (p.R_d * Tv));
    } else {
        const double Gamma = p.grav / p.cp_d;
        Tv = std::max(p.T_surface - Gamma * z, p.T_min);
        pres = std::pow(Tv / p.T_surface, p.grav / (p.R_d * Gamma));
        if (Tv == p.T_min) {
            const double z_top = (p.T_surface - p.T_min) / Gamma;
            const double H_min = p.R_d * p.T_min / p.grav;
            pres *= std::exp(-(z - z_top) / H_min);
        }
        pres *= p.MSLP;
    }
}

// Per-level tables: geopotential and its DG derivative (src/Common/Orientations/Orientations.jl:101-136,
// 246-258), hydrostatic reference state in discrete balance (src/Atmos/Model/ref_state.jl:143-185:
// p and rho from the profile, rho replaced by -(dp/dz)_DG / (dPhi/dz)_DG, then T and rhoe).
int init_model_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    const int Nq = m.Nq, nz = m.nz, nlev = m.nlev;
    md->lvl64.assign((size_t)nlev * LV_NFIELDS, 0.0);
    auto L = [&](int lev, int f) -> double& { return md->lvl64[(size_t)lev * LV_NFIELDS + f]; };
    std::vector<double> pz(nlev, 0.0), rz(nlev, 0.0);
    for (int lev = 0; lev < nlev; ++lev) {
        const double z = m.zlev[lev];
        // z: height on a brick, radius on a cubed shell
        L(lev, LV_PHI) = (p.orientation == CMDG_ORIENT_FLAT)     ? p.grav * z
                         : (p.orientation == CMDG_ORIENT_SPHERE) ? p.grav * (z - p.planet_radius)
                                                                 : 0.0;
    }
    // element-local DG derivative along a column
    auto ddz = [&](const std::vector<double>& f, int lev) {
        const int ez = lev / Nq, k = lev % Nq;
        double s = 0;
        for (int n = 0; n < Nq; ++n) s += m.D[k * Nq + n] * f[ez * Nq + n];
        return m.dzlev[lev] * s;
    };
    std::vector<double> phi(nlev);
    for (int lev = 0; lev < nlev; ++lev) phi[lev] = L(lev, LV_PHI);
    for (int lev = 0; lev < nlev; ++lev) L(lev, LV_GPHIZ) = ddz(phi, lev);
    // (a mesh from grid arrays takes its reference state per node from the caller)
    if (p.ref_state && m.kind != MESH_ARRAYS) {
        CMDG_ARG_CHECK(p.orientation == CMDG_ORIENT_FLAT || p.orientation == CMDG_ORIENT_SPHERE,
                       "a hydrostatic reference state needs an orientation");
        for (int lev = 0; lev < nlev; ++lev) {
            double Tv, pres;
            temperature_profile(p, L(lev, LV_PHI) / p.grav, Tv, pres);
            pz[lev] = pres;
        }
        for (int lev = 0; lev < nlev; ++lev) {
            const double rho = -ddz(pz, lev) / L(lev, LV_GPHIZ);
            const double T = pz[lev] / (p.R_d * rho);
            L(lev, LV_RHO_REF) = rho;
            L(lev, LV_P_REF) = pz[lev];
            L(lev, LV_RHOE_REF) = rho * ((0.0 + L(lev, LV_PHI)) + p.cv_d * (T - p.T_0));
        }
    }
    const double gm1 = p.R_d / p.cv_d;
    for (int lev = 0; lev < nlev; ++lev) {
        L(lev, LV_CRHO) = p.R_d * p.T_0 - gm1 * L(lev, LV_PHI);
        L(lev, LV_HREF) = L(lev, LV_RHOE_REF) + L(lev, LV_P_REF);
    }
    md->lvl32.resize(md->lvl64.size());
    for (size_t i = 0; i < md->lvl64.size(); ++i) md->lvl32[i] = (float)md->lvl64[i];
    // reference-state jumps across the bottom face of each element level (FP64 difference)
    md->jump32.assign((size_t)nz * 2, 0.0f);
    for (int ez = 0; ez < nz; ++ez) {
        int below = ez - 1;
        if (below < 0) {
            if (!m.desc.periodic[2]) continue;
            below = nz - 1;
        }
        const int lm = ez * Nq, lp = below * Nq + (Nq - 1);
        md->jump32[ez * 2 + 0] = (float)(L(lm, LV_RHO_REF) - L(lp, LV_RHO_REF));
        md->jump32[ez * 2 + 1] = (float)(L(lm, LV_RHOE_REF) - L(lp, LV_RHOE_REF));
    }
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_lvl64, sizeof(double) * md->lvl64.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_lvl32, sizeof(float) * md->lvl32.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_jump32, sizeof(float) * md->jump32.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_lvl64, md->lvl64.data(), sizeof(double) * md->lvl64.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_lvl32, md->lvl32.data(), sizeof(float) * md->lvl32.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_jump32, md->jump32.data(), sizeof(float) * md->jump32.size(), cudaMemcpyHostToDevice));
    std::vector<float> dh32(m.Dhat.size());
    for (size_t i = 0; i < dh32.size(); ++i) dh32[i] = (float)m.Dhat[i];
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_Dhat64, sizeof(double) * m.Dhat.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_Dhat32, sizeof(float) * dh32.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_Dhat64, m.Dhat.data(), sizeof(double) * m.Dhat.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_Dhat32, dh32.data(), sizeof(float) * dh32.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

}  // namespace cmdg

namespace cmdg {

// Reference-state rows of the diffusive passes: theta_v_ref, h_tot_ref and
// their DG z-derivatives, volume D plus the central face terms of
// dgsem_interface_gradients! (src/Numerics/DGMethods/DGModel_kernels.jl:1365-1651;
// zero jump on walls, where the boundary state of the reference state equals it).
int init_viscous_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    const int Nq = m.Nq, nz = m.nz, nlev = m.nlev, N = m.N;
    md->lvv64.assign((size_t)nlev * VV_NFIELDS, 0.0);
    auto V = [&](int lev, int f) -> double& { return md->lvv64[(size_t)lev * VV_NFIELDS + f]; };
    auto L = [&](int lev, int f) { return md->lvl64[(size_t)lev * LV_NFIELDS + f]; };
    const double kappa = p.R_d / p.cp_d;
    std::vector<double> thv(nlev), ht(nlev);
    for (int lev = 0; lev < nlev; ++lev) {
        const double rho = L(lev, LV_RHO_REF), pr = L(lev, LV_P_REF);
        if (p.ref_state && rho > 0) {
            const double T = pr / (p.R_d * rho);
            thv[lev] = T / std::pow(pr / p.MSLP, kappa);
            ht[lev] = (L(lev, LV_RHOE_REF) + pr) / rho;
        } else {
            thv[lev] = 0.0;
            ht[lev] = 0.0;
        }
        V(lev, VV_THV_REF) = thv[lev];
        V(lev, VV_HT_REF) = ht[lev];
        V(lev, VV_P_REF) = pr;
        V(lev, VV_RHO_REF) = rho;
    }
    const double inv_w0 = 1.0 / m.omega[0];
    auto ddz = [&](const std::vector<double>& f, int lev) {
        const int ez = lev / Nq, k = lev % Nq;
        double s = 0;
        for (int n = 0; n < Nq; ++n) s += m.D[k * Nq + n] * f[ez * Nq + n];
        double g = m.dzlev[lev] * s;
        const double lift = m.dzlev[lev] * inv_w0;
        if (k == 0) {  // bottom face, n_z = -1
            int eb = ez - 1;
            if (eb < 0) eb = m.desc.periodic[2] ? nz - 1 : -1;
            if (eb >= 0) g += lift * (-1.0) * (f[eb * Nq + N] - f[lev]) * 0.5;
        }
        if (k == N) {  // top face, n_z = +1
            int et = ez + 1;
            if (et >= nz) et = m.desc.periodic[2] ? 0 : -1;
            if (et >= 0) g += lift * (1.0) * (f[et * Nq + 0] - f[lev]) * 0.5;
        }
        return g;
    };
    for (int lev = 0; lev < nlev; ++lev) {
        V(lev, VV_DTHV_REF) = ddz(thv, lev);
        V(lev, VV_DHT_REF) = ddz(ht, lev);
    }
    std::vector<float> v32(md->lvv64.begin(), md->lvv64.end());
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_lvv64, sizeof(double) * md->lvv64.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_lvv32, sizeof(float) * v32.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_lvv64, md->lvv64.data(), sizeof(double) * md->lvv64.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_lvv32, v32.data(), sizeof(float) * v32.size(), cudaMemcpyHostToDevice));
    if (p.turbulence != CMDG_TURB_NONE) {
        const size_t elt = md->precision == CMDG_MIXED ? sizeof(float) : sizeof(double);
        // the stages' gradient pass writes the NF2 second-order flux words
        const size_t words = std::max(NGF, NF2);
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_gf, (size_t)m.nelem * words * m.Np * elt));
        CMDG_CUDA_CHECK(cudaMemset(md->d_gf, 0, (size_t)m.nelem * words * m.Np * elt));
    }
    return CMDG_OK;
}

}  // namespace cmdg
