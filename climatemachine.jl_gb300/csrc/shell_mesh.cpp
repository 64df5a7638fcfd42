// Host-side set-up of stacked cubed-shell meshes and their model tables.
//
// Topology: the six blocks of the developed net of cubedshellmesh
// (src/Numerics/Mesh/Topologies.jl:1150-1240) placed on the faces of the cube
// [-1, 1]^3 through their vertex lattice, stacked radially with contiguous
// columns (Topologies.jl:1620-1760): element e = iz + nvert * h.  Node
// coordinates: trilinear blend of the element corners (Metrics.jl:85-121),
// then the equiangular warp node by node (Topologies.jl:1265-1305; Grids.jl:
// 1050-1056).  Geometry: dx/dxi by the LGL derivative (Metrics.jl:215-270),
// curl-invariant metric terms, J and the face normals (Metrics.jl:431-724).
//
// On this mesh every node of one vertical level sits on the same radius (the
// warp keeps the radius of the blended cube point), so the geopotential and
// the hydrostatic reference state stay per-level tables as on a brick; the
// metric terms and the DG gradient of the geopotential are per node.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <utility>

#include "cmdg_internal.h"

namespace cmdg {

namespace {

double radius_blend(double a, double b, int n, int i) {
    return (double)(((long double)a * (n - i) + (long double)b * i) / n);
}

// (a, b, c) on the cube of half-width R = max(|a|, |b|, |c|) -> sphere of radius R
void equiangular(double& a, double& b, double& c) {
    const double A = std::fabs(a), B = std::fabs(b), C = std::fabs(c);
    const double R = std::max(std::max(A, B), C);
    const int face = (A >= B && A >= C) ? 0 : (B >= C ? 1 : 2);
    auto gnomonic = [](double sR, double xi, double eta, double& z1, double& z2, double& z3) {
        const double X = std::tan(M_PI * xi / 4), Y = std::tan(M_PI * eta / 4);
        z1 = sR / std::sqrt(X * X + Y * Y + 1);
        z2 = X * z1;
        z3 = Y * z1;
    };
    double x1, x2, x3;
    if (face == 0) gnomonic(a < 0 ? -R : R, b / a, c / a, x1, x2, x3);
    else if (face == 1) gnomonic(b < 0 ? -R : R, a / b, c / b, x2, x1, x3);
    else gnomonic(c < 0 ? -R : R, b / c, a / c, x3, x2, x1);
    a = x1;
    b = x2;
    c = x3;
}

}  // namespace

int build_shell(const cmdg_shell_desc* d, Mesh* m) {
    CMDG_ARG_CHECK(d != nullptr, "shell descriptor is NULL");
    CMDG_ARG_CHECK(d->N >= MIN_N && d->N <= MAX_N, "polynomial order N=%d outside the built range [%d, %d]", d->N,
                   MIN_N, MAX_N);
    CMDG_ARG_CHECK(d->nhorz >= 1 && d->nvert >= 1, "nhorz and nvert must be >= 1");
    CMDG_ARG_CHECK(d->r_inner > 0 && d->r_outer > d->r_inner, "need 0 < r_inner < r_outer");
    CMDG_ARG_CHECK(d->bc_inner > 0 && d->bc_outer > 0, "boundary tags must be positive");
    const int Ne = d->nhorz, nv = d->nvert;
    const int64_t nbase = 6LL * Ne * Ne, nelem = nbase * nv;
    CMDG_ARG_CHECK(nelem < (int64_t)1 << 28, "too many elements (%lld)", (long long)nelem);
    m->kind = MESH_SHELL;
    std::memset(&m->desc, 0, sizeof(m->desc));
    m->shell = *d;
    m->N = d->N;
    m->Nq = d->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = nelem;
    m->nz = nv;
    m->nlev = nv * m->Nq;
    lgl_derivative(m);
    const int N = m->N, Nq = m->Nq, Np = m->Np;

    // base elements: lattice vertex ids and cube coordinates of their 4 corners
    std::vector<int64_t> vid(nbase * 4);
    std::vector<double> vcube(nbase * 12);
    for (int64_t h = 0; h < nbase; ++h) {
        const int i = (int)(h % Ne), j = (int)((h / Ne) % Ne), blk = (int)(h / ((int64_t)Ne * Ne));
        for (int v = 0; v < 4; ++v) {
            const int ix = i + (v & 1), jx = j + (v >> 1);  // 0-based lattice indices along the block
            int L[3];
            switch (blk) {
                case 0: L[0] = 0; L[1] = Ne - ix; L[2] = jx; break;
                case 1: L[0] = ix; L[1] = 0; L[2] = jx; break;
                case 2: L[0] = Ne; L[1] = ix; L[2] = jx; break;
                case 3: L[0] = ix; L[1] = jx; L[2] = Ne; break;
                case 4: L[0] = ix; L[1] = Ne; L[2] = Ne - jx; break;
                default: L[0] = ix; L[1] = Ne - jx; L[2] = 0; break;
            }
            vid[h * 4 + v] = L[0] + (int64_t)(Ne + 1) * (L[1] + (int64_t)(Ne + 1) * L[2]);
            for (int c = 0; c < 3; ++c) vcube[(h * 4 + v) * 3 + c] = (double)(2 * L[c] - Ne) / Ne;
        }
    }
    std::vector<double> rr(nv + 1);
    for (int k = 0; k <= nv; ++k) rr[k] = radius_blend(d->r_inner, d->r_outer, nv, k);

    // coordinates and geometry
    m->xyz.assign((size_t)nelem * 3 * Np, 0.0);
    m->cgeo.assign((size_t)nelem * CG_NFIELDS * Np, 0.0);
    auto Dm = [&](int j, int k) { return m->D[j * Nq + k]; };
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t h = e / nv;
        const int iz = (int)(e % nv);
        double c[3][8];
        for (int v = 0; v < 4; ++v)
            for (int q = 0; q < 3; ++q) {
                c[q][v] = vcube[(h * 4 + v) * 3 + q] * rr[iz];
                c[q][4 + v] = vcube[(h * 4 + v) * 3 + q] * rr[iz + 1];
            }
        double* X = &m->xyz[(size_t)e * 3 * Np];
        for (int q = 0; q < 3; ++q)
            for (int k = 0; k < Nq; ++k)
                for (int j = 0; j < Nq; ++j)
                    for (int i = 0; i < Nq; ++i) {
                        const double a1 = 1 - m->xi[i], b1 = 1 + m->xi[i];
                        const double a2 = 1 - m->xi[j], b2 = 1 + m->xi[j];
                        const double a3 = 1 - m->xi[k], b3 = 1 + m->xi[k];
                        X[q * Np + i + Nq * (j + Nq * k)] =
                            (a1 * a2 * a3 * c[q][0] + b1 * a2 * a3 * c[q][1] + a1 * b2 * a3 * c[q][2] +
                             b1 * b2 * a3 * c[q][3] + a1 * a2 * b3 * c[q][4] + b1 * a2 * b3 * c[q][5] +
                             a1 * b2 * b3 * c[q][6] + b1 * b2 * b3 * c[q][7]) / 8;
                    }
        for (int n = 0; n < Np; ++n) equiangular(X[n], X[Np + n], X[2 * Np + n]);
        // dx_q/dxi_r
        std::vector<double> Xr(9 * Np, 0.0);  // [q*3 + r][node]
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    const int ijk = i + Nq * (j + Nq * k);
                    for (int q = 0; q < 3; ++q) {
                        double s0 = 0, s1 = 0, s2 = 0;
                        for (int n = 0; n < Nq; ++n) {
                            s0 += Dm(i, n) * X[q * Np + n + Nq * (j + Nq * k)];
                            s1 += Dm(j, n) * X[q * Np + i + Nq * (n + Nq * k)];
                            s2 += Dm(k, n) * X[q * Np + i + Nq * (j + Nq * n)];
                        }
                        Xr[(q * 3 + 0) * Np + ijk] = s0;
                        Xr[(q * 3 + 1) * Np + ijk] = s1;
                        Xr[(q * 3 + 2) * Np + ijk] = s2;
                    }
                }
        // curl-invariant form (Kopriva 2006, eq. 37): products x_a dx_b/dxi_r - x_b dx_a/dxi_r
        std::vector<double> J(Np), yz(3 * Np), zx(3 * Np), xy(3 * Np);
        for (int n = 0; n < Np; ++n) {
            auto xr = [&](int q, int r) { return Xr[(q * 3 + r) * Np + n]; };
            J[n] = xr(0, 0) * (xr(1, 1) * xr(2, 2) - xr(2, 1) * xr(1, 2)) +
                   xr(1, 0) * (xr(2, 1) * xr(0, 2) - xr(0, 1) * xr(2, 2)) +
                   xr(2, 0) * (xr(0, 1) * xr(1, 2) - xr(1, 1) * xr(0, 2));
            const double x1 = X[n], x2 = X[Np + n], x3 = X[2 * Np + n];
            for (int r = 0; r < 3; ++r) {
                yz[r * Np + n] = x2 * xr(2, r) - x3 * xr(1, r);
                zx[r * Np + n] = x3 * xr(0, r) - x1 * xr(2, r);
                xy[r * Np + n] = x1 * xr(1, r) - x2 * xr(0, r);
            }
        }
        double* G = &m->cgeo[(size_t)e * CG_NFIELDS * Np];
        const std::vector<double>* P3[3] = {&yz, &zx, &xy};  // component j = 0, 1, 2
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    const int ijk = i + Nq * (j + Nq * k);
                    for (int comp = 0; comp < 3; ++comp) {
                        const std::vector<double>& Pv = *P3[comp];
                        double g1 = 0, g2 = 0, g3 = 0;  // xi1, xi2, xi3 rows of component comp
                        for (int n = 0; n < Nq; ++n) {
                            const int l = n + Nq * (j + Nq * k);  // along xi1
                            g2 -= Dm(i, n) * Pv[2 * Np + l];
                            g3 += Dm(i, n) * Pv[1 * Np + l];
                        }
                        for (int n = 0; n < Nq; ++n) {
                            const int l = i + Nq * (n + Nq * k);  // along xi2
                            g1 += Dm(j, n) * Pv[2 * Np + l];
                            g3 -= Dm(j, n) * Pv[0 * Np + l];
                        }
                        for (int n = 0; n < Nq; ++n) {
                            const int l = i + Nq * (j + Nq * n);  // along xi3
                            g1 -= Dm(k, n) * Pv[1 * Np + l];
                            g2 += Dm(k, n) * Pv[0 * Np + l];
                        }
                        const double JI2 = 1 / (2 * J[ijk]);
                        G[(CG_XI + 0 * 3 + comp) * Np + ijk] = g1 * JI2;
                        G[(CG_XI + 1 * 3 + comp) * Np + ijk] = g2 * JI2;
                        G[(CG_XI + 2 * 3 + comp) * Np + ijk] = g3 * JI2;
                    }
                    G[CG_J * Np + ijk] = J[ijk];
                    G[CG_M * Np + ijk] = J[ijk] * (m->omega[k] * m->omega[j] * m->omega[i]);
                    // nearest neighbouring node along the three element lines
                    double md = INFINITY;
                    auto dist = [&](int o) {
                        double s = 0;
                        for (int q = 0; q < 3; ++q) {
                            const double dx = X[q * Np + ijk] - X[q * Np + o];
                            s += dx * dx;
                        }
                        md = std::min(md, std::sqrt(s));
                    };
                    if (i > 0) dist(ijk - 1);
                    if (i < N) dist(ijk + 1);
                    if (j > 0) dist(ijk - Nq);
                    if (j < N) dist(ijk + Nq);
                    if (k > 0) dist(ijk - Nq * Nq);
                    if (k < N) dist(ijk + Nq * Nq);
                    G[CG_DXMIN * Np + ijk] = md;
                }
    }

    // connectivity: horizontal neighbours share the two lattice vertices of a face
    const int fv[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
    std::map<std::pair<int64_t, int64_t>, std::vector<std::pair<int64_t, int>>> edges;
    for (int64_t h = 0; h < nbase; ++h)
        for (int f = 0; f < 4; ++f) {
            const int64_t a = vid[h * 4 + fv[f][0]], b = vid[h * 4 + fv[f][1]];
            edges[{std::min(a, b), std::max(a, b)}].push_back({h, f});
        }
    std::vector<int64_t> hn(nbase * 4, -1);
    std::vector<int> hf(nbase * 4, -1);
    for (auto& kv : edges) {
        CMDG_ARG_CHECK(kv.second.size() == 2, "cubed shell: an element edge is not shared by exactly two elements");
        const auto a = kv.second[0], b = kv.second[1];
        hn[a.first * 4 + a.second] = b.first;
        hf[a.first * 4 + a.second] = b.second;
        hn[b.first * 4 + b.second] = a.first;
        hf[b.first * 4 + b.second] = a.second;
    }
    // volume node of horizontal face f at in-face (a = horizontal index, b = k)
    auto face_node = [&](int f, int a, int b) {
        const int side = (f & 1) ? N : 0;
        return (f < 2) ? side + Nq * (a + Nq * b) : a + Nq * (side + Nq * b);
    };
    m->nbr.assign((size_t)nelem * NBR_STRIDE, 0);
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t h = e / nv;
        const int iz = (int)(e % nv);
        int* row = &m->nbr[(size_t)e * NBR_STRIDE];
        unsigned code = 0;
        for (int f = 0; f < 4; ++f) {
            const int64_t e2 = hn[h * 4 + f] * nv + iz;
            const int f2 = hf[h * 4 + f];
            row[f] = (int)e2;
            // orientation: does in-face index a meet a' = a or a' = N - a?
            int rev = -1;
            for (int r = 0; r < 2 && rev < 0; ++r) {
                bool ok = true;
                for (int b = 0; b < Nq && ok; ++b)
                    for (int a = 0; a < Nq && ok; ++a) {
                        const int v1 = face_node(f, a, b), v2 = face_node(f2, r ? N - a : a, b);
                        double s = 0;
                        for (int q = 0; q < 3; ++q) {
                            const double dx = m->xyz[((size_t)e * 3 + q) * Np + v1] - m->xyz[((size_t)e2 * 3 + q) * Np + v2];
                            s += dx * dx;
                        }
                        ok = s <= 1e-18 * d->r_outer * d->r_outer;
                    }
                if (ok) rev = r;
            }
            CMDG_ARG_CHECK(rev >= 0, "cubed shell: face nodes of element %lld face %d do not match", (long long)e, f);
            code |= (unsigned)(f2 | (rev << 2)) << (4 * f);
        }
        row[4] = iz > 0 ? (int)(e - 1) : -d->bc_inner;
        row[5] = iz < nv - 1 ? (int)(e + 1) : -d->bc_outer;
        row[6] = iz;
        row[7] = (int)code;
    }
    m->zlev.assign(m->nlev, 0.0);
    m->dzlev.assign(m->nlev, 0.0);
    for (int ez = 0; ez < nv; ++ez)
        for (int k = 0; k < Nq; ++k) {
            m->zlev[ez * Nq + k] = ((1 - m->xi[k]) * rr[ez] + (1 + m->xi[k]) * rr[ez + 1]) / 2;
            m->dzlev[ez * Nq + k] = 2.0 / (rr[ez + 1] - rr[ez]);
        }
    CMDG_CUDA_CHECK(cudaMalloc(&m->d_nbr, sizeof(int) * m->nbr.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(m->d_nbr, m->nbr.data(), sizeof(int) * m->nbr.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

// Neighbour node across face f of element e at face node fn (in-face index
// a + Nq * b as the stage kernel numbers it): the element and volume node on
// the other side, or (e, own node) on a wall.
static void neighbour_node(const Mesh& m, int64_t e, int f, int fn, int64_t& e2, int& v2) {
    const int N = m.N, Nq = m.Nq, Nfp = m.Nfp;
    const int fd = f >> 1, side = (f & 1) ? N : 0;
    const int a = fn % Nq, b = fn / Nq;
    const int vM = fd == 0 ? side + Nq * fn : (fd == 1 ? a + Nq * (side + Nq * b) : fn + Nfp * side);
    const int* row = &m.nbr[(size_t)e * NBR_STRIDE];
    if (row[f] < 0) {
        e2 = e;
        v2 = vM;
        return;
    }
    e2 = row[f];
    if (fd == 2) {
        v2 = fn + Nfp * ((f & 1) ? 0 : N);
        return;
    }
    const unsigned code = ((unsigned)row[7] >> (4 * f)) & 15u;
    const int f2 = (int)(code & 3u), a2 = (code & 4u) ? N - a : a, side2 = (f2 & 1) ? N : 0;
    v2 = (f2 < 2) ? side2 + Nq * (a2 + Nq * b) : a2 + Nq * (side2 + Nq * b);
}

// Per-node tables of a model on a cubed shell:
//  * J dxi/dx and 1/J;
//  * Phi = g (|x| - planet_radius) (Orientations.jl:161-175) and its DG
//    gradient taken element-locally as auxiliary_field_gradient! does
//    (DGModel_kernels.jl:3097-3232: strong derivative along each xi line
//    mapped by the metric terms);
//  * the hydrostatic reference state in discrete balance (ref_state.jl:
//    70-185, 204-263): p from the profile at altitude Phi / g, grad p as the
//    DG tendency of the flux -p I with central interface fluxes (walls take
//    the interior value), rho = -k.grad p / k.grad Phi with k = grad Phi / g,
//    T = p / (R_d rho), rhoe = rho (Phi + cv_d (T - T_0)).  On curved
//    elements the weak-form gradient differs from the element-wise strong one
//    by the polynomial aliasing of (J dxi/dx) p, so the reference density
//    varies from node to node along a level; the kernels read the level row
//    plus the per-node difference (KG_DRHO, KG_DRHOE, and for the FP64
//    kernel KG_DPREF and KG_DCRHO, which are rounding-sized);
//  * M and the nearest-node distance for the reductions.
int init_shell_tables(Model* md) {
    const Mesh& m = *md->mesh;
    const cmdg_atmos_params& p = md->prm;
    const int N = m.N, Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    const int64_t nelem = m.nelem;
    std::vector<double> geo((size_t)nelem * KG_NFIELDS * Np, 0.0);
    std::vector<double> mass((size_t)nelem * Np), dxmin((size_t)nelem * Np);
    std::vector<double> phi((size_t)nelem * Np), pres((size_t)nelem * Np, 0.0);
    for (int64_t e = 0; e < nelem; ++e) {
        const double* G = &m.cgeo[(size_t)e * CG_NFIELDS * Np];
        const double* X = &m.xyz[(size_t)e * 3 * Np];
        double* K = &geo[(size_t)e * KG_NFIELDS * Np];
        for (int n = 0; n < Np; ++n) {
            const double J = G[CG_J * Np + n];
            for (int w = 0; w < 9; ++w) K[(KG_JXI + w) * Np + n] = J * G[(CG_XI + w) * Np + n];
            K[KG_INVJ * Np + n] = 1.0 / J;
            mass[(size_t)e * Np + n] = G[CG_M * Np + n];
            dxmin[(size_t)e * Np + n] = G[CG_DXMIN * Np + n];
            const double r = std::sqrt(X[n] * X[n] + X[Np + n] * X[Np + n] + X[2 * Np + n] * X[2 * Np + n]);
            const double ph = (p.orientation == CMDG_ORIENT_SPHERE) ? p.grav * (r - p.planet_radius) : 0.0;
            phi[(size_t)e * Np + n] = ph;
            if (p.ref_state) {
                double Tv, pr;
                temperature_profile(p, ph / p.grav, Tv, pr);
                pres[(size_t)e * Np + n] = pr;
            }
        }
        const double* ph = &phi[(size_t)e * Np];
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    const int ijk = i + Nq * (j + Nq * k);
                    double G1 = 0, G2 = 0, G3 = 0;
                    for (int n = 0; n < Nq; ++n) {
                        G1 += m.D[i * Nq + n] * ph[n + Nq * (j + Nq * k)];
                        G2 += m.D[j * Nq + n] * ph[i + Nq * (n + Nq * k)];
                        G3 += m.D[k * Nq + n] * ph[i + Nq * (j + Nq * n)];
                    }
                    for (int c = 0; c < 3; ++c) {
                        const double hz = G[(CG_XI + 0 * 3 + c) * Np + ijk] * G1 + G[(CG_XI + 1 * 3 + c) * Np + ijk] * G2;
                        K[(KG_GPHI + c) * Np + ijk] = hz + G[(CG_XI + 2 * 3 + c) * Np + ijk] * G3;
                    }
                }
    }
    // the node's own geopotential differs from its level value by rounding of
    // the radius; the FP64 kernel reads the difference of the pressure
    // coefficient so that its pressure matches the per-node reference state
    for (int64_t e = 0; e < nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            const int lev = (int)(e % m.nz) * Nq + n / Nfp;
            const double* L = &md->lvl64[(size_t)lev * LV_NFIELDS];
            const double crho = p.R_d * p.T_0 - (p.R_d / p.cv_d) * phi[(size_t)e * Np + n];
            geo[((size_t)e * KG_NFIELDS + KG_DCRHO) * Np + n] = crho - L[LV_CRHO];
        }
    if (p.ref_state) {
        md->ref64.assign((size_t)nelem * 2 * Np, 0.0);
        const double inv_w0 = 1.0 / m.omega[0];
        std::vector<double> gp(3 * Np);
        for (int64_t e = 0; e < nelem; ++e) {
            const double* K = &geo[(size_t)e * KG_NFIELDS * Np];
            const double* pe = &pres[(size_t)e * Np];
            // volume term: -(1/J) sum_d Dhat_d (J xi_d,s p)
            for (int k = 0; k < Nq; ++k)
                for (int j = 0; j < Nq; ++j)
                    for (int i = 0; i < Nq; ++i) {
                        const int ijk = i + Nq * (j + Nq * k);
                        for (int c = 0; c < 3; ++c) {
                            double acc = 0;
                            for (int n = 0; n < Nq; ++n) {
                                const int l1 = n + Nq * (j + Nq * k), l2 = i + Nq * (n + Nq * k), l3 = i + Nq * (j + Nq * n);
                                acc += m.Dhat[i * Nq + n] * (K[(KG_JXI + 0 * 3 + c) * Np + l1] * pe[l1]);
                                acc += m.Dhat[j * Nq + n] * (K[(KG_JXI + 1 * 3 + c) * Np + l2] * pe[l2]);
                                acc += m.Dhat[k * Nq + n] * (K[(KG_JXI + 2 * 3 + c) * Np + l3] * pe[l3]);
                            }
                            gp[c * Np + ijk] = -K[KG_INVJ * Np + ijk] * acc;
                        }
                    }
            // interface term: - lift (F*.n) with F* = (F- + F+)/2, F = -p I
            for (int f = 0; f < 6; ++f)
                for (int fn = 0; fn < Nfp; ++fn) {
                    const int fd = f >> 1, a = fn % Nq, b = fn / Nq, side = (f & 1) ? N : 0;
                    const int vM = fd == 0 ? side + Nq * fn : (fd == 1 ? a + Nq * (side + Nq * b) : fn + Nfp * side);
                    int64_t e2;
                    int v2;
                    neighbour_node(m, e, f, fn, e2, v2);
                    const double j0 = K[(KG_JXI + fd * 3 + 0) * Np + vM], j1 = K[(KG_JXI + fd * 3 + 1) * Np + vM],
                                 j2 = K[(KG_JXI + fd * 3 + 2) * Np + vM];
                    const double sJ = std::sqrt(j0 * j0 + j1 * j1 + j2 * j2);
                    const double sg = (f & 1) ? 1.0 : -1.0;
                    const double nv[3] = {sg * j0 / sJ, sg * j1 / sJ, sg * j2 / sJ};
                    const double lift = sJ * K[KG_INVJ * Np + vM] * inv_w0;
                    const double pm = pe[vM], pp = pres[(size_t)e2 * Np + v2];
                    for (int c = 0; c < 3; ++c) gp[c * Np + vM] += lift * ((pm + pp) * 0.5) * nv[c];
                }
            for (int n = 0; n < Np; ++n) {
                const double g0 = K[(KG_GPHI + 0) * Np + n], g1 = K[(KG_GPHI + 1) * Np + n], g2 = K[(KG_GPHI + 2) * Np + n];
                const double kk[3] = {g0 / p.grav, g1 / p.grav, g2 / p.grav};
                const double num = kk[0] * gp[n] + kk[1] * gp[Np + n] + kk[2] * gp[2 * Np + n];
                const double den = kk[0] * g0 + kk[1] * g1 + kk[2] * g2;
                const double rho = -num / den;
                const double T = pe[n] / (p.R_d * rho);
                const double rhoe = rho * ((0.0 + phi[(size_t)e * Np + n]) + p.cv_d * (T - p.T_0));
                md->ref64[((size_t)e * 2 + 0) * Np + n] = rho;
                md->ref64[((size_t)e * 2 + 1) * Np + n] = rhoe;
                const int lev = (int)(e % m.nz) * Nq + n / Nfp;
                const double* L = &md->lvl64[(size_t)lev * LV_NFIELDS];
                double* Kw = &geo[(size_t)e * KG_NFIELDS * Np];
                Kw[KG_DRHO * Np + n] = rho - L[LV_RHO_REF];
                Kw[KG_DRHOE * Np + n] = rhoe - L[LV_RHOE_REF];
                Kw[KG_DPREF * Np + n] = pe[n] - L[LV_P_REF];
            }
        }
        CMDG_CUDA_CHECK(cudaMalloc(&md->d_ref64, sizeof(double) * md->ref64.size()));
        CMDG_CUDA_CHECK(cudaMemcpy(md->d_ref64, md->ref64.data(), sizeof(double) * md->ref64.size(),
                                   cudaMemcpyHostToDevice));
    }
    std::vector<float> geo32(geo.begin(), geo.end());
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_geo64, sizeof(double) * geo.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_geo32, sizeof(float) * geo32.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_mass, sizeof(double) * mass.size()));
    CMDG_CUDA_CHECK(cudaMalloc(&md->d_dxmin, sizeof(double) * dxmin.size()));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_geo64, geo.data(), sizeof(double) * geo.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_geo32, geo32.data(), sizeof(float) * geo32.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_mass, mass.data(), sizeof(double) * mass.size(), cudaMemcpyHostToDevice));
    CMDG_CUDA_CHECK(cudaMemcpy(md->d_dxmin, dxmin.data(), sizeof(double) * dxmin.size(), cudaMemcpyHostToDevice));
    return CMDG_OK;
}

}  // namespace cmdg
