// cmdg oracle — TEST INFRASTRUCTURE ONLY.
//
// A plain-C++ FP64 restatement of ClimateMachine.jl's DG spectral-element
// tendency for the dry AtmosModel (DGModel volume/interface kernels, gradient,
// diffusive and hyperdiffusion passes), its LSRK54CarpenterKennedy
// integrator, the HEVI scheme (vertical acoustic-gravity linear model, column
// LU, ARK2GiraldoKellyConstantinescu), the modal filters, the brick and
// stacked cubed-shell geometry it runs on and the weighted reductions used
// to report errors.
//
// It is the checker for the CUDA library: only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load it.  Nothing in the product path
// links, loads or calls this file.
//
// Parity status: pinned.  The isentropic-vortex golden errors of
// test/Numerics/DGMethods/Euler/isentropicvortex.jl:105-106, the
// manufactured-solution Navier-Stokes golden error of
// test/Numerics/DGMethods/compressible_Navier_Stokes/mms_bc_atmos.jl:232-235
// (viscous path, warped brick), the 3D hyperdiffusion golden errors of
// test/Numerics/DGMethods/advection_diffusion/periodic_3D_hyperdiffusion.jl,
// the LSRK54 convergence order of
// test/Numerics/ODESolvers/ode_tests_convergence.jl:41, the discrete
// hydrostatic balance of test/Atmos/Model/discrete_hydrostatic_balance.jl
// (LES brick and GCM cubed shell) and the HEVI acoustic-wave golden norm of
// test/Numerics/DGMethods/Euler/acousticwave_1d_imex.jl (vertical linear
// model, column LU, ARK2GiraldoKellyConstantinescu, vertical filter) are
// reproduced by tests/test_oracle_pins.py; the filters by
// tests/test_filters_cpu.py against test/Numerics/Mesh/filter.jl.
//
// Every function cites the reference file:line (paths relative to the
// ClimateMachine.jl project root) whose algorithm it restates.  Third-party
// arithmetic that lives outside the reference tree is restated from its
// published definitions:
//   * Thermodynamics.jl 0.5.1  — PhaseDry T(e_int), p, c_s, h_tot, theta_v
//   * CLIMAParameters.jl 0.2.0 — R_d, cp_d, cv_d, T_0, grav, MSLP, ... (set by
//                                 the caller through om_params)
//   * GaussQuadrature.jl 0.5.5 — Legendre-Gauss-Lobatto nodes and weights
//   * DoubleFloats.jl 1.1.18   — compensated (double-double) weighted sums
//
// Layouts follow the reference exactly (all column-major as in Julia):
//   Q, dQ   : (Np, nstate, nelem)           MPIStateArrays.jl:98
//   vgeo    : (Np, 16, nelem)               Grids.jl:76-125
//   sgeo    : (5, Nfp, 6, nelem)            Grids.jl:129-146
//   vmap-/+ : (Nfp, 6, nelem), 0-based      Grids.jl:559-638
// Element ordering is "stacked": the vertical index is fastest, then x, then
// y (columns contiguous, like StackedBrickTopology, Topologies.jl:632).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// ----------------------------------------------------------------------------
// Public parameter blocks (mirrored by oracle/oracle.py)
// ----------------------------------------------------------------------------
typedef struct {
    int N;                    // polynomial order (same in all directions)
    int ne[3];                // elements in x, y, z
    double lo[3], hi[3];      // domain extents
    int periodic[3];          // 1 = periodic in that direction
    int bc_lo[3], bc_hi[3];   // boundary tags for non-periodic faces (>0)
    int warp;                 // 0 = none; 1 = the 3D mesh warp of test/Numerics/DGMethods/
                              // compressible_Navier_Stokes/mms_bc_atmos.jl:268-276
} om_brick;

typedef struct {
    // CLIMAParameters.jl 0.2.0 planet / SGS constants
    double R_d, cp_d, cv_d, T_0, grav, MSLP, inv_Pr_turb;
    int numflux;        // 0 = Rusanov (NumericalFluxes.jl:219-285), 1 = central (:298-340)
    int orientation;    // 0 = NoOrientation, 1 = FlatOrientation, 2 = SphericalOrientation
                        // (Orientations.jl:138-150, 246-258, 161-175)
    int gravity;        // 1 = Gravity() source (tendencies_momentum.jl:60-72)
    int ref_state;      // 0 = NoReferenceState, 1 = HydrostaticState (ref_state.jl:36-60)
    int subtract_off;   // HydrostaticState.subtract_off
    int profile;        // 0 = Isothermal, 1 = DryAdiabatic (Thermodynamics.TemperatureProfiles)
    double T_surface;   // isothermal T_virt or dry-adiabatic T_surface
    double T_min;       // dry-adiabatic T_min_ref
    int turbulence;     // 0 = inviscid, 1 = ConstantDynamicViscosity, 2 = SmagorinskyLilly
    double rho_nu;      // dynamic viscosity for turbulence==1
    int with_divergence;// WithDivergence for turbulence==1
    double C_smag;      // Smagorinsky coefficient for turbulence==2
    double planet_radius; // SphericalOrientation: Phi = g (|x| - planet_radius)
    int hyperdiffusion; // 0 = NoHyperDiffusion, 1 = DryBiharmonic (TurbulenceClosures.jl:793-848)
    double tau_hyper;   // DryBiharmonic.tau_timescale
    int hyper_direction;// DGModel diffusion_direction of the hyperdiffusion passes:
                        // 0 = EveryDirection, 1 = HorizontalDirection (SpaceDiscretization.jl:731-1083)
    int mms;            // 1 = the manufactured-solution AtmosModel of mms_bc_atmos.jl: source terms
                        // and InitStateBC wall states supplied per node (om_set_mms), and
                        // total_specific_enthalpy overridden to zero (mms_bc_atmos.jl:45-48)
} om_params;

// StackedCubedSphereTopology (Topologies.jl:1620-1760) over a
// CubedShellTopology (Topologies.jl:1067-1240) with the equiangular warp
// (Topologies.jl:1254-1305); radial element edges grid1d(r_inner, r_outer,
// nelem = nvert) (Topologies.jl:2001).
typedef struct {
    int N;
    int nhorz;                // elements per cube-face edge
    int nvert;                // elements per stack
    double r_inner, r_outer;
    int bc_inner, bc_outer;   // boundary tags (> 0)
} om_shell;

}  // extern "C"

namespace {

constexpr int NVGEO = 16;
enum { XI1X1 = 0, XI2X1, XI3X1, XI1X2, XI2X2, XI3X2, XI1X3, XI2X3, XI3X3, VM, VMI, VMH, VX1, VX2, VX3, VJCV };
constexpr int NSGEO = 5;
enum { SN1 = 0, SN2, SN3, SSM, SVMI };
// auxiliary fields per node (own ordering; content as AtmosModel.jl:465-481)
enum { AX = 0, AY, AZ, APHI, AGPX, AGPY, AGPZ, ARHO_REF, AP_REF, AT_REF, ARHOE_REF, ATHV, AAIRT, ADELTA, AHDELTA, NAUX };
constexpr int NS = 5;   // rho, rhou(3), rhoe

struct Model {
    int kind = 0;                            // 0 = brick, 1 = stacked cubed shell
    om_brick mesh;
    om_shell shell;
    om_params prm;
    int N, Nq, Np, Nfp;
    int64_t nelem;
    std::vector<double> xi, omega, D;       // D[j + Nq*k] = D[j,k] (column-major)
    std::vector<double> vgeo, sgeo, aux;
    std::vector<int64_t> vmapM, vmapP;
    std::vector<int> elemtobndy;
    std::vector<int64_t> elemtoelem;
    int ngf;                                 // gradient-flux words per node
    std::vector<double> gradflux;            // (Np, ngf, nelem)
    // hyperdiffusion: Qhypervisc_grad (Np, 12, nelem) holds grad(u_h, h_tot)
    // after the gradient pass and nu grad^3 (u_h, h_tot) after the gradients
    // of the laplacians; Qhypervisc_div (Np, 4, nelem) the laplacians
    std::vector<double> hgrad, hdiv;
    int ngl = 4;                             // GradientLaplacian states per node
    const double* mms_src = nullptr;         // mms: source terms at the nodes, (Np, 5, nelem)
    const double* mms_exact = nullptr;       // mms: InitStateBC state at the nodes, (Np, 5, nelem)
    int law = 0;                             // 0 = AtmosModel, 1 = scalar constant-tensor hyperdiffusion
    double Hten[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // law 1: tensor H, column-major
};

// ----------------------------------------------------------------------------
// Legendre-Gauss-Lobatto points and weights.
// Elements.jl:11-14 calls GaussQuadrature.legendre(T, N+1, both); restated as
// Newton iteration on (1-x^2) P_N'(x) with the Legendre three-term recurrence,
// weights 2 / (N (N+1) P_N(x)^2), nodes ascending from -1 to 1.
// ----------------------------------------------------------------------------
void lgl(int N, std::vector<double>& x, std::vector<double>& w) {
    int Nq = N + 1;
    x.assign(Nq, 0.0);
    w.assign(Nq, 0.0);
    std::vector<long double> xl(Nq), P(Nq * Nq);
    for (int i = 0; i < Nq; ++i) xl[i] = -cosl(3.14159265358979323846264338327950288L * i / N);
    for (int it = 0; it < 100; ++it) {
        long double maxd = 0;
        for (int i = 0; i < Nq; ++i) {
            long double p0 = 1, p1 = xl[i], pm = 0;
            // P_N and P_{N-1} at x
            long double Pn = p1, Pnm1 = p0;
            if (N == 1) { Pn = p1; Pnm1 = p0; }
            for (int k = 2; k <= N; ++k) {
                pm = ((2 * k - 1) * xl[i] * p1 - (k - 1) * p0) / k;
                p0 = p1; p1 = pm;
                Pn = p1; Pnm1 = p0;
            }
            long double dx = (xl[i] * Pn - Pnm1) / (Nq * Pn);
            xl[i] -= dx;
            maxd = std::max(maxd, fabsl(dx));
        }
        if (maxd < 1e-30L) break;
    }
    for (int i = 0; i < Nq; ++i) {
        long double s = 0.5L * (xl[i] - xl[N - i]);
        long double p0 = 1, p1 = s, Pn = s;
        for (int k = 2; k <= N; ++k) {
            long double pm = ((2 * k - 1) * s * p1 - (k - 1) * p0) / k;
            p0 = p1; p1 = pm; Pn = p1;
        }
        x[i] = (double)s;
        w[i] = (double)(2.0L / ((long double)N * Nq * Pn * Pn));
    }
    x[0] = -1.0; x[N] = 1.0;
    if (N % 2 == 0) x[N / 2] = 0.0;
}

// Barycentric weights and spectral differentiation matrix, Elements.jl:34-82.
void spectral_derivative(const std::vector<double>& r, std::vector<double>& D) {
    int Np = (int)r.size();
    std::vector<double> wb(Np, 1.0);
    for (int j = 0; j < Np; ++j) {
        for (int i = 0; i < Np; ++i)
            if (i != j) wb[j] = wb[j] * (r[j] - r[i]);
        wb[j] = 1.0 / wb[j];
    }
    D.assign(Np * Np, 0.0);
    for (int k = 0; k < Np; ++k)
        for (int j = 0; j < Np; ++j) {
            if (k == j) {
                for (int l = 0; l < Np; ++l)
                    if (l != k) D[j + Np * k] = D[j + Np * k] + 1.0 / (r[k] - r[l]);
            } else {
                D[j + Np * k] = (wb[k] / wb[j]) / (r[j] - r[k]);
            }
        }
}

inline double Dm(const Model& m, int j, int k) { return m.D[j + m.Nq * k]; }
inline double& VG(Model& m, int64_t e, int f, int n) { return m.vgeo[(e * NVGEO + f) * m.Np + n]; }
inline double VGc(const Model& m, int64_t e, int f, int n) { return m.vgeo[(e * NVGEO + f) * m.Np + n]; }
inline double& SG(Model& m, int64_t e, int face, int n, int s) { return m.sgeo[((e * 6 + face) * m.Nfp + n) * NSGEO + s]; }
inline double SGc(const Model& m, int64_t e, int face, int n, int s) { return m.sgeo[((e * 6 + face) * m.Nfp + n) * NSGEO + s]; }
inline double& AUX(Model& m, int64_t e, int a, int n) { return m.aux[(e * NAUX + a) * m.Np + n]; }
inline double AUXc(const Model& m, int64_t e, int a, int n) { return m.aux[(e * NAUX + a) * m.Np + n]; }

// Julia-style range(a, stop=b, length=n+1) value i (correctly rounded blend).
double range_value(double a, double b, int n, int i) {
    long double v = ((long double)a * (n - i) + (long double)b * i) / n;
    return (double)v;
}

// Face node masks, Grids.jl:580-597: fmask[f][n] -> volume node index.
void face_masks(int Nq, std::vector<std::vector<int>>& fmask) {
    fmask.assign(6, std::vector<int>(Nq * Nq));
    for (int b = 0; b < Nq; ++b)
        for (int a = 0; a < Nq; ++a) {
            int n = a + Nq * b;
            fmask[0][n] = 0 + Nq * (a + Nq * b);           // i = 1, (j, k)
            fmask[1][n] = (Nq - 1) + Nq * (a + Nq * b);    // i = Nq
            fmask[2][n] = a + Nq * (0 + Nq * b);           // j = 1, (i, k)
            fmask[3][n] = a + Nq * ((Nq - 1) + Nq * b);    // j = Nq
            fmask[4][n] = a + Nq * (b + Nq * 0);           // k = 1, (i, j)
            fmask[5][n] = a + Nq * (b + Nq * (Nq - 1));    // k = Nq
        }
}

// ----------------------------------------------------------------------------
// Brick topology + grid.
//  * element corners and trilinear blend: Metrics.jl:85-121 (creategrid!)
//  * connectivity / boundary tags: Topologies.jl:470-545, BrickMesh.jl:827,1096
//  * vmap-/+ (orientation 1 only on a brick): Grids.jl:559-638
//  * dx/dxi by D: Metrics.jl:215-270; curl-invariant metric, J, normals,
//    surface Jacobian: Metrics.jl:431-724; M, MI, sM, vMI: Grids.jl:1068-1096
// ----------------------------------------------------------------------------
int64_t elem_index(const om_brick& b, int ix, int iy, int iz) {
    return (int64_t)iz + (int64_t)b.ne[2] * ((int64_t)ix + (int64_t)b.ne[0] * iy);
}

void alloc_geometry(Model& m) {
    m.vgeo.assign((size_t)m.nelem * NVGEO * m.Np, 0.0);
    m.sgeo.assign((size_t)m.nelem * 6 * m.Nfp * NSGEO, 0.0);
    m.vmapM.assign((size_t)m.nelem * 6 * m.Nfp, 0);
    m.vmapP.assign((size_t)m.nelem * 6 * m.Nfp, 0);
    m.elemtobndy.assign((size_t)m.nelem * 6, 0);
    m.elemtoelem.assign((size_t)m.nelem * 6, 0);
}

// Node coordinates of element e from its 8 corners (trilinear blend,
// Metrics.jl:85-121), an optional mesh warp applied node by node
// (Grids.jl:1050-1056), then dx/dxi (Metrics.jl:215-270), the curl-invariant
// metric terms, J, normals and surface Jacobian (Metrics.jl:431-724) and
// M, MI, sM, vMI (Grids.jl:1068-1096).
void element_geometry(Model& m, int64_t e, const double c[3][8], void (*warp)(double&, double&, double&)) {
    int N = m.N, Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    std::vector<std::vector<int>> fmask;
    face_masks(Nq, fmask);
    const std::vector<double>& xi = m.xi;
    {
        std::vector<double> X[3], Xr[3][3];
        for (int d = 0; d < 3; ++d) {
            X[d].assign(Np, 0.0);
            for (int q = 0; q < 3; ++q) Xr[d][q].assign(Np, 0.0);
        }
        // trilinear blend, Metrics.jl:100-118
        for (int d = 0; d < 3; ++d)
            for (int k = 0; k < Nq; ++k)
                for (int j = 0; j < Nq; ++j)
                    for (int i = 0; i < Nq; ++i) {
                        double a1 = 1 - xi[i], b1 = 1 + xi[i];
                        double a2 = 1 - xi[j], b2 = 1 + xi[j];
                        double a3 = 1 - xi[k], b3 = 1 + xi[k];
                        X[d][i + Nq * (j + Nq * k)] =
                            (a1 * a2 * a3 * c[d][0] + b1 * a2 * a3 * c[d][1] + a1 * b2 * a3 * c[d][2] +
                             b1 * b2 * a3 * c[d][3] + a1 * a2 * b3 * c[d][4] + b1 * a2 * b3 * c[d][5] +
                             a1 * b2 * b3 * c[d][6] + b1 * b2 * b3 * c[d][7]) / 8;
                    }
        if (warp)
            for (int n = 0; n < Np; ++n) warp(X[0][n], X[1][n], X[2][n]);
        // dx/dxi, Metrics.jl:246-266
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    for (int d = 0; d < 3; ++d) {
                        for (int n = 0; n < Nq; ++n) Xr[d][0][ijk] += Dm(m, i, n) * X[d][n + Nq * (j + Nq * k)];
                        for (int n = 0; n < Nq; ++n) Xr[d][1][ijk] += Dm(m, j, n) * X[d][i + Nq * (n + Nq * k)];
                        for (int n = 0; n < Nq; ++n) Xr[d][2][ijk] += Dm(m, k, n) * X[d][i + Nq * (j + Nq * n)];
                    }
                }
        // curl-invariant metric terms, Metrics.jl:490-606
        std::vector<double> J(Np), yz[3], zx[3], xy[3];
        for (int q = 0; q < 3; ++q) { yz[q].resize(Np); zx[q].resize(Np); xy[q].resize(Np); }
        double* x1 = X[0].data(); double* x2 = X[1].data(); double* x3 = X[2].data();
        for (int n = 0; n < Np; ++n) {
            double x1r = Xr[0][0][n], x1s = Xr[0][1][n], x1t = Xr[0][2][n];
            double x2r = Xr[1][0][n], x2s = Xr[1][1][n], x2t = Xr[1][2][n];
            double x3r = Xr[2][0][n], x3s = Xr[2][1][n], x3t = Xr[2][2][n];
            VG(m, e, VJCV, n) = std::hypot(std::hypot(x1t, x2t), x3t);
            J[n] = x1r * (x2s * x3t - x3s * x2t) + x2r * (x3s * x1t - x1s * x3t) + x3r * (x1s * x2t - x2s * x1t);
            yz[0][n] = x2[n] * x3r - x3[n] * x2r; yz[1][n] = x2[n] * x3s - x3[n] * x2s; yz[2][n] = x2[n] * x3t - x3[n] * x2t;
            zx[0][n] = x3[n] * x1r - x1[n] * x3r; zx[1][n] = x3[n] * x1s - x1[n] * x3s; zx[2][n] = x3[n] * x1t - x1[n] * x3t;
            xy[0][n] = x1[n] * x2r - x2[n] * x1r; xy[1][n] = x1[n] * x2s - x2[n] * x1s; xy[2][n] = x1[n] * x2t - x2[n] * x1t;
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // xi1x1 xi2x1 xi3x1 xi1x2 ... (vgeo order)
                    for (int n = 0; n < Nq; ++n) {
                        int nj = n + Nq * (j + Nq * k);
                        g[XI2X1] -= Dm(m, i, n) * yz[2][nj];
                        g[XI3X1] += Dm(m, i, n) * yz[1][nj];
                        g[XI2X2] -= Dm(m, i, n) * zx[2][nj];
                        g[XI3X2] += Dm(m, i, n) * zx[1][nj];
                        g[XI2X3] -= Dm(m, i, n) * xy[2][nj];
                        g[XI3X3] += Dm(m, i, n) * xy[1][nj];
                    }
                    for (int n = 0; n < Nq; ++n) {
                        int in = i + Nq * (n + Nq * k);
                        g[XI1X1] += Dm(m, j, n) * yz[2][in];
                        g[XI3X1] -= Dm(m, j, n) * yz[0][in];
                        g[XI1X2] += Dm(m, j, n) * zx[2][in];
                        g[XI3X2] -= Dm(m, j, n) * zx[0][in];
                        g[XI1X3] += Dm(m, j, n) * xy[2][in];
                        g[XI3X3] -= Dm(m, j, n) * xy[0][in];
                    }
                    for (int n = 0; n < Nq; ++n) {
                        int ij = i + Nq * (j + Nq * n);
                        g[XI1X1] -= Dm(m, k, n) * yz[1][ij];
                        g[XI2X1] += Dm(m, k, n) * yz[0][ij];
                        g[XI1X2] -= Dm(m, k, n) * zx[1][ij];
                        g[XI2X2] += Dm(m, k, n) * zx[0][ij];
                        g[XI1X3] -= Dm(m, k, n) * xy[1][ij];
                        g[XI2X3] += Dm(m, k, n) * xy[0][ij];
                    }
                    double JI2 = 1 / (2 * J[ijk]);
                    for (int q = 0; q < 9; ++q) VG(m, e, q, ijk) = g[q] * JI2;
                    VG(m, e, VX1, ijk) = x1[ijk];
                    VG(m, e, VX2, ijk) = x2[ijk];
                    VG(m, e, VX3, ijk) = x3[ijk];
                }
        // surface terms, Metrics.jl:660-722 (uses J before the omega scaling)
        for (int f = 0; f < 6; ++f) {
            int d = f / 2;
            double sgn = (f % 2) ? 1.0 : -1.0;
            int c1 = (d == 0) ? XI1X1 : (d == 1) ? XI2X1 : XI3X1;
            int c2 = (d == 0) ? XI1X2 : (d == 1) ? XI2X2 : XI3X2;
            int c3 = (d == 0) ? XI1X3 : (d == 1) ? XI2X3 : XI3X3;
            for (int n = 0; n < Nfp; ++n) {
                int v = fmask[f][n];
                double n1 = sgn * J[v] * VG(m, e, c1, v);
                double n2 = sgn * J[v] * VG(m, e, c2, v);
                double n3 = sgn * J[v] * VG(m, e, c3, v);
                double sJ = std::hypot(std::hypot(n1, n2), n3);
                SG(m, e, f, n, SN1) = n1 / sJ;
                SG(m, e, f, n, SN2) = n2 / sJ;
                SG(m, e, f, n, SN3) = n3 / sJ;
                SG(m, e, f, n, SSM) = sJ;
            }
        }
        // mass matrix and surface mass, Grids.jl:1068-1096
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double Mw = m.omega[k] * m.omega[j] * m.omega[i];
                    VG(m, e, VM, ijk) = J[ijk] * Mw;
                    VG(m, e, VMI, ijk) = 1 / VG(m, e, VM, ijk);
                    VG(m, e, VMH, ijk) = 0;  // diagnostics only
                }
        for (int f = 0; f < 6; ++f)
            for (int bb = 0; bb < Nq; ++bb)
                for (int a = 0; a < Nq; ++a) {
                    int n = a + Nq * bb;
                    SG(m, e, f, n, SVMI) = VG(m, e, VMI, fmask[f][n]);
                    SG(m, e, f, n, SSM) *= m.omega[a] * m.omega[bb];
                }
        (void)N;
    }
}


// The 3D mesh warp of mms_bc_atmos.jl:268-276.
void mms_warp(double& x1, double& x2, double& x3) {
    const double a = x1, b = x2, c = x3;
    x1 = a + (a - 0.5) * std::cos(2 * M_PI * b * c) / 4;
    x2 = b + std::exp(std::sin(2 * M_PI * (a * b + c))) / 20;
    x3 = c + a / 4 + b * b / 2 + std::sin(a * b * c);
}

void build_geometry(Model& m) {
    const om_brick& b = m.mesh;
    int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    int64_t nelem = m.nelem;
    alloc_geometry(m);
    std::vector<std::vector<int>> fmask;
    face_masks(Nq, fmask);

    // connectivity
    for (int iy = 0; iy < b.ne[1]; ++iy)
        for (int ix = 0; ix < b.ne[0]; ++ix)
            for (int iz = 0; iz < b.ne[2]; ++iz) {
                int64_t e = elem_index(b, ix, iy, iz);
                int idx[3] = {ix, iy, iz};
                for (int f = 0; f < 6; ++f) {
                    int d = f / 2, side = f % 2;
                    int nb[3] = {idx[0], idx[1], idx[2]};
                    nb[d] += side ? 1 : -1;
                    int64_t e2 = e;
                    int f2 = f;
                    int tag = 0;
                    if (nb[d] < 0 || nb[d] >= b.ne[d]) {
                        if (b.periodic[d]) {
                            nb[d] = (nb[d] + b.ne[d]) % b.ne[d];
                            e2 = elem_index(b, nb[0], nb[1], nb[2]);
                            f2 = f ^ 1;
                        } else {
                            tag = side ? b.bc_hi[d] : b.bc_lo[d];
                            if (tag <= 0) tag = 1;
                        }
                    } else {
                        e2 = elem_index(b, nb[0], nb[1], nb[2]);
                        f2 = f ^ 1;
                    }
                    m.elemtobndy[e * 6 + f] = tag;
                    m.elemtoelem[e * 6 + f] = e2;
                    for (int n = 0; n < Nfp; ++n) {
                        m.vmapM[(e * 6 + f) * Nfp + n] = e * Np + fmask[f][n];
                        m.vmapP[(e * 6 + f) * Nfp + n] = e2 * Np + fmask[f2][n];
                    }
                }
            }

    std::vector<double> xg[3];
    for (int d = 0; d < 3; ++d) {
        xg[d].resize(b.ne[d] + 1);
        for (int i = 0; i <= b.ne[d]; ++i) xg[d][i] = range_value(b.lo[d], b.hi[d], b.ne[d], i);
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nelem; ++e) {
        int64_t iz = e % b.ne[2];
        int64_t ix = (e / b.ne[2]) % b.ne[0];
        int64_t iy = e / ((int64_t)b.ne[2] * b.ne[0]);
        double c[3][8];
        for (int v = 0; v < 8; ++v) {
            int bi = v & 1, bj = (v >> 1) & 1, bk = (v >> 2) & 1;
            c[0][v] = xg[0][ix + bi];
            c[1][v] = xg[1][iy + bj];
            c[2][v] = xg[2][iz + bk];
        }
        element_geometry(m, e, c, b.warp == 1 ? mms_warp : nullptr);
    }
}

// Equiangular cubed-sphere warp, Topologies.jl:1265-1305 (Ronchi, Iacono and
// Paolucci 1996): a point (a, b, c) on the cube of half-width
// R = max(|a|, |b|, |c|) goes to the sphere of radius R; the face is the
// first coordinate of largest magnitude.
void equiangular_warp(double& a, double& b, double& c) {
    const double R = std::max(std::max(std::fabs(a), std::fabs(b)), std::fabs(c));
    auto f = [](double sR, double xi, double eta, double& z1, double& z2, double& z3) {
        const double X = std::tan(M_PI * xi / 4), Y = std::tan(M_PI * eta / 4);
        z1 = sR / std::sqrt(X * X + Y * Y + 1);
        z2 = X * z1;
        z3 = Y * z1;
    };
    const double A = std::fabs(a), B = std::fabs(b), C = std::fabs(c);
    const int fdim = (A >= B && A >= C) ? 1 : (B >= C ? 2 : 3);
    double x1, x2, x3;
    if (fdim == 1 && a < 0) f(-R, b / a, c / a, x1, x2, x3);
    else if (fdim == 2 && b < 0) f(-R, a / b, c / b, x2, x1, x3);
    else if (fdim == 1 && a > 0) f(R, b / a, c / a, x1, x2, x3);
    else if (fdim == 2 && b > 0) f(R, a / b, c / b, x2, x1, x3);
    else if (fdim == 3 && c > 0) f(R, b / c, a / c, x3, x2, x1);
    else f(-R, b / c, a / c, x3, x2, x1);
    a = x1;
    b = x2;
    c = x3;
}

// Stacked cubed shell.  Base elements follow cubedshellmesh (Topologies.jl:
// 1150-1240): CartesianIndices((Ne, Ne, 6)), the six blocks of the developed
// net mapped onto the faces of the cube [-1, 1]^3 by their vertex lattice
// points; stacks are contiguous, element e = iz + nvert * h (Topologies.jl:
// 1680-1700; the reference's space-filling-curve renumbering is a
// permutation and is not applied).  Lower corners are the base vertices times
// r_j, upper corners times r_{j+1}.  Horizontal neighbours share two lattice
// vertices; face-node maps vmapP match node coordinates (the reference builds
// the same map from elemtoordr, Grids.jl:559-638).
void build_shell_geometry(Model& m) {
    const om_shell& sh = m.shell;
    const int Ne = sh.nhorz, nv = sh.nvert, Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    alloc_geometry(m);
    std::vector<std::vector<int>> fmask;
    face_masks(Nq, fmask);
    const int64_t nbase = 6LL * Ne * Ne;
    // lattice vertex ids and cube coordinates of the 4 base vertices
    std::vector<int64_t> bvert(nbase * 4);
    std::vector<double> bcoord(nbase * 4 * 3);
    for (int64_t h = 0; h < nbase; ++h) {
        const int i = (int)(h % Ne) + 1, j = (int)((h / Ne) % Ne) + 1, blck = (int)(h / ((int64_t)Ne * Ne)) + 1;
        for (int n = 1; n <= 4; ++n) {
            const int ix = i + (n - 1) % 2, jx = j + (n - 1) / 2;
            int L[3];
            switch (blck) {
                case 1: L[0] = 1; L[1] = Ne + 2 - ix; L[2] = jx; break;
                case 2: L[0] = ix; L[1] = 1; L[2] = jx; break;
                case 3: L[0] = Ne + 1; L[1] = ix; L[2] = jx; break;
                case 4: L[0] = ix; L[1] = jx; L[2] = Ne + 1; break;
                case 5: L[0] = ix; L[1] = Ne + 1; L[2] = Ne + 2 - jx; break;
                default: L[0] = ix; L[1] = Ne + 2 - jx; L[2] = 1; break;
            }
            bvert[h * 4 + n - 1] = (L[0] - 1) + (int64_t)(Ne + 1) * ((L[1] - 1) + (int64_t)(Ne + 1) * (L[2] - 1));
            for (int d = 0; d < 3; ++d) bcoord[(h * 4 + n - 1) * 3 + d] = (double)(2 * (L[d] - 1) - Ne) / Ne;
        }
    }
    std::vector<double> rr(nv + 1);
    for (int k = 0; k <= nv; ++k) rr[k] = range_value(sh.r_inner, sh.r_outer, nv, k);
    // horizontal neighbours: base faces 1..4 are vertex pairs (1,3), (2,4), (1,2), (3,4)
    const int fv[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
    std::map<std::pair<int64_t, int64_t>, std::vector<std::pair<int64_t, int>>> edges;
    for (int64_t h = 0; h < nbase; ++h)
        for (int f = 0; f < 4; ++f) {
            int64_t a = bvert[h * 4 + fv[f][0]], b = bvert[h * 4 + fv[f][1]];
            edges[{std::min(a, b), std::max(a, b)}].push_back({h, f});
        }
    std::vector<int64_t> hn(nbase * 4);
    std::vector<int> hf(nbase * 4);
    for (auto& kv : edges) {
        if (kv.second.size() != 2) throw std::runtime_error("cubed shell: an edge without exactly two elements");
        auto a = kv.second[0], b = kv.second[1];
        hn[a.first * 4 + a.second] = b.first; hf[a.first * 4 + a.second] = b.second;
        hn[b.first * 4 + b.second] = a.first; hf[b.first * 4 + b.second] = a.second;
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        const int64_t h = e / nv;
        const int iz = (int)(e % nv);
        double c[3][8];
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) {
                c[d][v] = bcoord[(h * 4 + v) * 3 + d] * rr[iz];
                c[d][4 + v] = bcoord[(h * 4 + v) * 3 + d] * rr[iz + 1];
            }
        element_geometry(m, e, c, equiangular_warp);
    }
    for (int64_t e = 0; e < m.nelem; ++e) {
        const int64_t h = e / nv;
        const int iz = (int)(e % nv);
        for (int f = 0; f < 6; ++f) {
            int64_t e2 = e;
            int f2 = f, tag = 0;
            if (f < 4) {
                e2 = hn[h * 4 + f] * nv + iz;
                f2 = hf[h * 4 + f];
            } else if (f == 4) {
                if (iz == 0) tag = sh.bc_inner > 0 ? sh.bc_inner : 1;
                else { e2 = e - 1; f2 = 5; }
            } else {
                if (iz == nv - 1) tag = sh.bc_outer > 0 ? sh.bc_outer : 1;
                else { e2 = e + 1; f2 = 4; }
            }
            m.elemtobndy[e * 6 + f] = tag;
            m.elemtoelem[e * 6 + f] = e2;
            for (int n = 0; n < Nfp; ++n) {
                const int vM = fmask[f][n];
                m.vmapM[(e * 6 + f) * Nfp + n] = e * Np + vM;
                if (tag) {
                    m.vmapP[(e * 6 + f) * Nfp + n] = e * Np + vM;
                    continue;
                }
                // the neighbour's face node at the same physical point
                double best = INFINITY;
                int vb = -1;
                for (int n2 = 0; n2 < Nfp; ++n2) {
                    const int v2 = fmask[f2][n2];
                    double d2 = 0;
                    for (int d = 0; d < 3; ++d) {
                        const double dx = VGc(m, e, VX1 + d, vM) - VGc(m, e2, VX1 + d, v2);
                        d2 += dx * dx;
                    }
                    if (d2 < best) { best = d2; vb = v2; }
                }
                if (best > 1e-16 * sh.r_outer * sh.r_outer) throw std::runtime_error("cubed shell: unmatched face node");
                m.vmapP[(e * 6 + f) * Nfp + n] = e2 * Np + vb;
            }
        }
    }
}

// ----------------------------------------------------------------------------
// Thermodynamics (Thermodynamics.jl 0.5.1, dry air), as called from
// Atmos/Model/thermo_states.jl:67-77 and moisture.jl:32-45.
// ----------------------------------------------------------------------------
struct Thermo {
    double e_int, T, p;
};

// internal energy from the conserved state (moisture.jl:35-45)
inline double internal_energy(double rho, double rhoe, const double rhou[3], double Phi) {
    double ke2 = rhou[0] * rhou[0] + rhou[1] * rhou[1] + rhou[2] * rhou[2];
    return (1 / rho) * (rhoe - ke2 / (2 * rho)) - Phi;
}

inline Thermo phase_dry(const om_params& p, double rho, double rhoe, const double rhou[3], double Phi) {
    Thermo t;
    t.e_int = internal_energy(rho, rhoe, rhou, Phi);
    t.T = p.T_0 + t.e_int / p.cv_d;
    t.p = p.R_d * rho * t.T;
    return t;
}

inline double soundspeed(const om_params& p, double T) { return std::sqrt(p.cp_d / p.cv_d * p.R_d * T); }

// theta_v for dry air: T / (p / MSLP)^(R_d / cp_d)
inline double virtual_pottemp(const om_params& p, double T, double pres) {
    return (p.R_d / p.R_d) * (T / std::pow(pres / p.MSLP, p.R_d / p.cp_d));
}

// ----------------------------------------------------------------------------
// Temperature profiles (Thermodynamics.TemperatureProfiles 0.5.1) and the
// hydrostatic reference state, ref_state.jl:70-141, 143-185, 204-263.
// ----------------------------------------------------------------------------
void profile(const om_params& p, double z, double& Tv, double& pres) {
    if (p.profile == 0) {  // IsothermalProfile
        Tv = p.T_surface;
        pres = p.MSLP * std::exp(-z * p.grav / (p.R_d * Tv));
    } else {               // DryAdiabaticProfile
        double Gamma = p.grav / p.cp_d;
        Tv = std::max(p.T_surface - Gamma * z, p.T_min);
        pres = std::pow(Tv / p.T_surface, p.grav / (p.R_d * Gamma));
        if (Tv == p.T_min) {
            double z_top = (p.T_surface - p.T_min) / Gamma;
            double H_min = p.R_d * p.T_min / p.grav;
            pres *= std::exp(-(z - z_top) / H_min);
        }
        pres *= p.MSLP;
    }
}

// Element-local derivative of an aux field, DGModel_kernels.jl:3097-3232
// (auxiliary_field_gradient!, SpaceDiscretization.jl:391-483): horizontal
// pass then vertical pass added.
void aux_field_gradient(Model& m, int ain, int aout) {
    int Nq = m.Nq;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double G1 = 0, G2 = 0, G3 = 0;
                    for (int n = 0; n < Nq; ++n) {
                        G1 += Dm(m, i, n) * AUX(m, e, ain, n + Nq * (j + Nq * k));
                        G2 += Dm(m, j, n) * AUX(m, e, ain, i + Nq * (n + Nq * k));
                    }
                    for (int n = 0; n < Nq; ++n) G3 += Dm(m, k, n) * AUX(m, e, ain, i + Nq * (j + Nq * n));
                    double gh[3], gv[3];
                    gh[0] = VG(m, e, XI1X1, ijk) * G1 + VG(m, e, XI2X1, ijk) * G2;
                    gh[1] = VG(m, e, XI1X2, ijk) * G1 + VG(m, e, XI2X2, ijk) * G2;
                    gh[2] = VG(m, e, XI1X3, ijk) * G1 + VG(m, e, XI2X3, ijk) * G2;
                    gv[0] = VG(m, e, XI3X1, ijk) * G3;
                    gv[1] = VG(m, e, XI3X2, ijk) * G3;
                    gv[2] = VG(m, e, XI3X3, ijk) * G3;
                    for (int q = 0; q < 3; ++q) AUX(m, e, aout + q, ijk) = gh[q] + gv[q];
                }
    }
}

// ∇reference_pressure: DG tendency of PressureGradientModel (flux = -p I,
// central flux, boundary state = interior), ref_state.jl:204-263, evaluated
// with the volume/interface kernels of DGModel_kernels.jl:64-548, 588-901.
void ref_pressure_gradient(Model& m, std::vector<double>& gp /* (Np,3,nelem) */) {
    int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    gp.assign((size_t)m.nelem * 3 * Np, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> F1(Np * 3), F2(Np * 3), F3(Np * 3);
        for (int n = 0; n < Np; ++n) {
            double p = AUX(m, e, AP_REF, n);
            double M = VG(m, e, VM, n);
            // flux[:, s] = -p * e_s  -> F[d, s] = -p delta_ds
            for (int s = 0; s < 3; ++s) {
                double Fd[3] = {0, 0, 0};
                Fd[s] = -p;
                F1[n * 3 + s] = M * (VG(m, e, XI1X1, n) * Fd[0] + VG(m, e, XI1X2, n) * Fd[1] + VG(m, e, XI1X3, n) * Fd[2]);
                F2[n * 3 + s] = M * (VG(m, e, XI2X1, n) * Fd[0] + VG(m, e, XI2X2, n) * Fd[1] + VG(m, e, XI2X3, n) * Fd[2]);
                F3[n * 3 + s] = M * (VG(m, e, XI3X1, n) * Fd[0] + VG(m, e, XI3X2, n) * Fd[1] + VG(m, e, XI3X3, n) * Fd[2]);
            }
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double MI = VG(m, e, VMI, ijk);
                    for (int s = 0; s < 3; ++s) {
                        double th = 0, tv = 0;
                        for (int n = 0; n < Nq; ++n) {
                            th += MI * Dm(m, n, i) * F1[(n + Nq * (j + Nq * k)) * 3 + s];
                            th += MI * Dm(m, n, j) * F2[(i + Nq * (n + Nq * k)) * 3 + s];
                        }
                        for (int n = 0; n < Nq; ++n) tv += MI * Dm(m, n, k) * F3[(i + Nq * (j + Nq * n)) * 3 + s];
                        gp[(e * 3 + s) * Np + ijk] = th + tv;
                    }
                }
        for (int f = 0; f < 6; ++f)
            for (int n = 0; n < Nfp; ++n) {
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                if (m.elemtobndy[e * 6 + f] != 0) { eP = e; vP = vM; }
                double nv[3] = {SG(m, e, f, n, SN1), SG(m, e, f, n, SN2), SG(m, e, f, n, SN3)};
                double pM = AUX(m, e, AP_REF, vM), pP = AUX(m, eP, AP_REF, vP);
                double sM = SG(m, e, f, n, SSM), vMI = SG(m, e, f, n, SVMI);
                for (int s = 0; s < 3; ++s) {
                    // central: (F- + F+)' * (n / 2); F[d, s] = -p delta_ds
                    double fl = (-pM + -pP) * (nv[s] / 2);
                    gp[(e * 3 + s) * Np + vM] -= vMI * sM * fl;
                }
            }
    }
}

void init_aux(Model& m) {
    const om_params& p = m.prm;
    int Np = m.Np;
    m.aux.assign((size_t)m.nelem * NAUX * Np, 0.0);
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            AUX(m, e, AX, n) = VG(m, e, VX1, n);
            AUX(m, e, AY, n) = VG(m, e, VX2, n);
            AUX(m, e, AZ, n) = VG(m, e, VX3, n);
        }
    // Orientation: Phi = g z (FlatOrientation, Orientations.jl:246-258) or
    // g (|x| - planet_radius) (SphericalOrientation, :161-175), grad Phi by DG
    if (p.orientation == 1 || p.orientation == 2) {
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int n = 0; n < Np; ++n) {
                if (p.orientation == 1) {
                    AUX(m, e, APHI, n) = p.grav * AUX(m, e, AZ, n);
                } else {
                    const double x = AUX(m, e, AX, n), y = AUX(m, e, AY, n), z = AUX(m, e, AZ, n);
                    AUX(m, e, APHI, n) = p.grav * (std::sqrt(x * x + y * y + z * z) - p.planet_radius);
                }
            }
        aux_field_gradient(m, APHI, AGPX);
    }
    // Hydrostatic reference state (ref_state.jl:143-185)
    if (p.ref_state == 1) {
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int n = 0; n < Np; ++n) {
                double z = AUX(m, e, APHI, n) / p.grav;  // altitude = Phi / g
                double Tv, pres;
                profile(p, z, Tv, pres);
                AUX(m, e, AP_REF, n) = pres;
                AUX(m, e, ARHO_REF, n) = pres / (Tv * p.R_d);
            }
        std::vector<double> gp;
        ref_pressure_gradient(m, gp);
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int n = 0; n < Np; ++n) {
                double gP[3] = {AUX(m, e, AGPX, n), AUX(m, e, AGPY, n), AUX(m, e, AGPZ, n)};
                double k[3] = {gP[0] / p.grav, gP[1] / p.grav, gP[2] / p.grav};
                double dp[3] = {gp[(e * 3 + 0) * Np + n], gp[(e * 3 + 1) * Np + n], gp[(e * 3 + 2) * Np + n]};
                double num = k[0] * dp[0] + k[1] * dp[1] + k[2] * dp[2];
                double den = k[0] * gP[0] + k[1] * gP[1] + k[2] * gP[2];
                AUX(m, e, ARHO_REF, n) = -num / den;
            }
        for (int64_t e = 0; e < m.nelem; ++e)
            for (int n = 0; n < Np; ++n) {
                double rho = AUX(m, e, ARHO_REF, n), pres = AUX(m, e, AP_REF, n);
                double T = pres / (p.R_d * rho);  // PhaseDry_ρp
                AUX(m, e, AT_REF, n) = T;
                double e_pot = AUX(m, e, APHI, n);
                AUX(m, e, ARHOE_REF, n) = rho * ((0.0 + e_pot) + p.cv_d * (T - p.T_0));
            }
    }
    // Smagorinsky length scale, Geometry.jl:121-122 (2 / (cbrt(det(dxi/dx)) N))
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < Np; ++n) {
            double a = VG(m, e, XI1X1, n), b = VG(m, e, XI1X2, n), c = VG(m, e, XI1X3, n);
            double d = VG(m, e, XI2X1, n), f = VG(m, e, XI2X2, n), g = VG(m, e, XI2X3, n);
            double h = VG(m, e, XI3X1, n), i = VG(m, e, XI3X2, n), j = VG(m, e, XI3X3, n);
            // invJ = [xi1x1 xi1x2 xi1x3; xi2x1 ...; xi3x1 ...]
            double det = a * (f * j - g * i) - b * (d * j - g * h) + c * (d * i - f * h);
            AUX(m, e, ADELTA, n) = 2 / (std::cbrt(det) * std::max(1, m.N));
            // lengthscale_horizontal, Geometry.jl:129-151: the columns dx/dxi_1 and
            // dx/dxi_2 of invJ^-1 (cofactors / det), their lengths 2/N, averaged
            double c1[3] = {(f * j - g * i) / det, -(d * j - g * h) / det, (d * i - f * h) / det};
            double c2[3] = {-(b * j - c * i) / det, (a * j - c * h) / det, -(a * i - b * h) / det};
            double D1 = std::sqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]) * 2 / m.N;
            double D2 = std::sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2]) * 2 / m.N;
            AUX(m, e, AHDELTA, n) = (D1 + D2) / 2;
        }
}

// ----------------------------------------------------------------------------
// Model pointwise functions (AtmosModel, dry, TotalEnergy, Compressible).
// ----------------------------------------------------------------------------
struct NodeAux {
    double Phi, gPhi[3], rho_ref, p_ref, thv, Delta;
};

inline NodeAux node_aux(const Model& m, int64_t e, int n) {
    NodeAux a;
    a.Phi = AUXc(m, e, APHI, n);
    a.gPhi[0] = AUXc(m, e, AGPX, n);
    a.gPhi[1] = AUXc(m, e, AGPY, n);
    a.gPhi[2] = AUXc(m, e, AGPZ, n);
    a.rho_ref = AUXc(m, e, ARHO_REF, n);
    a.p_ref = AUXc(m, e, AP_REF, n);
    a.thv = AUXc(m, e, ATHV, n);
    a.Delta = AUXc(m, e, ADELTA, n);
    return a;
}

// First-order flux F[d][s] (atmos_tendencies.jl:9-45; tendencies_mass.jl:7-9,
// tendencies_momentum.jl:13-29, tendencies_energy.jl:7-21).
void flux_first_order(const om_params& p, const double q[NS], const NodeAux& a, double F[3][NS]) {
    double rho = q[0];
    const double* ru = q + 1;
    double rhoe = q[4];
    Thermo t = phase_dry(p, rho, rhoe, ru, a.Phi);
    double pres = t.p;
    double pg = (p.ref_state == 1 && p.subtract_off) ? (pres - a.p_ref) : pres;
    for (int d = 0; d < 3; ++d) {
        double u_d = ru[d] / rho;
        F[d][0] = ru[d];
        for (int c = 0; c < 3; ++c) F[d][1 + c] = ru[d] * (ru[c] / rho) + (c == d ? pg : 0.0);
        F[d][4] = u_d * rhoe + u_d * pres;
    }
}

// Gradient-flux layout per node: [dh_tot(3), S11,S21,S31,S22,S32,S33, (N2)]
// (AtmosModel.jl:447-461, energy.jl:10-11, TurbulenceClosures.jl:347-362,446-470)

// Second-order flux (tendencies_momentum.jl:37-42, tendencies_energy.jl:27-31,
// 51-56; turbulence_tensors TurbulenceClosures.jl:199-225, 368-404, 472-505).
//
// With hyperdiffusion, hd holds the node's nu grad^3 words (3 c + d for
// u_h[c], 9 + d for h_tot) and the fluxes HyperdiffViscousFlux and
// HyperdiffEnthalpyFlux are added (tendencies_momentum.jl:51-54,
// tendencies_energy.jl:40-48).
void hyper_flux(const double q[NS], const double* hd, double F[3][NS]) {
    double rho = q[0];
    const double* ru = q + 1;
    for (int d = 0; d < 3; ++d) {
        for (int c = 0; c < 3; ++c) F[d][1 + c] += rho * hd[3 * c + d];
        F[d][4] += (hd[d] * ru[0] + hd[3 + d] * ru[1] + hd[6 + d] * ru[2]) + hd[9 + d] * rho;
    }
}

void flux_second_order(const Model& m, const double q[NS], const double* gf, const NodeAux& a, double F[3][NS],
                       const double* hd = nullptr) {
    const om_params& p = m.prm;
    for (int d = 0; d < 3; ++d)
        for (int s = 0; s < NS; ++s) F[d][s] = 0;
    if (p.turbulence == 0) {
        if (hd) hyper_flux(q, hd, F);
        return;
    }
    double rho = q[0];
    const double* ru = q + 1;
    double S[3][3] = {{gf[3], gf[4], gf[5]}, {gf[4], gf[6], gf[7]}, {gf[5], gf[7], gf[8]}};
    double nu[3], Dt[3];
    double tau[3][3];
    if (p.turbulence == 1) {
        double nu0 = p.rho_nu / rho;
        double Dt0 = nu0 * p.inv_Pr_turb;
        for (int c = 0; c < 3; ++c) { nu[c] = nu0; Dt[c] = Dt0; }
        double trS = S[0][0] + S[1][1] + S[2][2];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                tau[r][c] = (-2 * nu0) * S[r][c];
                if (p.with_divergence && r == c) tau[r][c] += (2 * nu0 / 3) * trS;
            }
    } else {
        // SmagorinskyLilly
        double norm2 = S[0][0] * S[0][0] + 2 * (S[1][0] * S[1][0]) + 2 * (S[2][0] * S[2][0]) + S[1][1] * S[1][1] +
                       2 * (S[2][1] * S[2][1]) + S[2][2] * S[2][2];
        double normS = std::sqrt(2 * norm2);
        double khat[3] = {a.gPhi[0] / p.grav, a.gPhi[1] / p.grav, a.gPhi[2] / p.grav};
        double N2 = gf[9];
        double epsn = normS == 0 ? 4.9406564584124654e-324 : std::nextafter(normS, INFINITY) - normS;
        double Ri = N2 / (normS * normS + epsn);
        double fb2 = std::sqrt(std::min(std::max(1.0 - Ri * p.inv_Pr_turb, 0.0), 1.0));
        double cd = p.C_smag * a.Delta;
        double nu0 = normS * (cd * cd) + 1e-5;
        double dnk = nu0 * khat[0] + nu0 * khat[1] + nu0 * khat[2];
        for (int c = 0; c < 3; ++c) {
            double nv = khat[c] * dnk;
            double nh = nu0 - nv;
            nu[c] = nh + nv * fb2;
            Dt[c] = nu[c] * p.inv_Pr_turb;
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) tau[r][c] = -2 * nu[r] * S[r][c];
    }
    // momentum: tau * rho ; energy: tau * rhou + (-D_t .* grad h_tot) * rho
    for (int d = 0; d < 3; ++d) {
        for (int c = 0; c < 3; ++c) F[d][1 + c] = tau[d][c] * rho;
        double tr = tau[d][0] * ru[0] + tau[d][1] * ru[1] + tau[d][2] * ru[2];
        F[d][4] = tr + (-Dt[d] * gf[d]) * rho;
    }
    if (hd) hyper_flux(q, hd, F);
}

// Gravity source (tendencies_momentum.jl:64-72)
void source(const om_params& p, const double q[NS], const NodeAux& a, double S[NS]) {
    for (int s = 0; s < NS; ++s) S[s] = 0;
    if (!p.gravity) return;
    double r = (p.ref_state == 1 && p.subtract_off) ? (q[0] - a.rho_ref) : q[0];
    for (int c = 0; c < 3; ++c) S[1 + c] = -r * a.gPhi[c];
}

// wavespeed (AtmosModel.jl:776-796)
inline double wavespeed(const om_params& p, const double n[3], const double q[NS], const NodeAux& a) {
    double rinv = 1 / q[0];
    double u[3] = {rinv * q[1], rinv * q[2], rinv * q[3]};
    double uN = std::fabs(n[0] * u[0] + n[1] * u[1] + n[2] * u[2]);
    Thermo t = phase_dry(p, q[0], q[4], q + 1, a.Phi);
    return uN + soundspeed(p, t.T);
}

// Gradient argument (AtmosModel.jl:622-650, energy.jl:20-31,
// TurbulenceClosures.jl:446-454): u, h_tot, [theta_v]
int ngrad_args(const om_params& p) { return p.turbulence == 2 ? 5 : 4; }
void gradient_argument(const om_params& p, const double q[NS], double Phi, double thv, double G[5]) {
    double rinv = 1 / q[0];
    G[0] = rinv * q[1]; G[1] = rinv * q[2]; G[2] = rinv * q[3];
    Thermo t = phase_dry(p, q[0], q[4], q + 1, Phi);
    double e_tot = q[4] * (1 / q[0]);
    G[3] = p.mms ? 0.0 : e_tot + p.R_d * t.T;  // mms: total_specific_enthalpy := 0
    G[4] = thv;
}

// compute_gradient_flux!: linear map of grad G -> gradient-flux words
void gradient_flux(const om_params& p, const double gG[3][5], const NodeAux& a, double* gf) {
    gf[0] = gG[0][3]; gf[1] = gG[1][3]; gf[2] = gG[2][3];
    // symmetrize(grad u): X[i,j] = d u_j / d x_i (Grad layout (3, ngrad))
    gf[3] = gG[0][0];
    gf[4] = (gG[1][0] + gG[0][1]) / 2;
    gf[5] = (gG[2][0] + gG[0][2]) / 2;
    gf[6] = gG[1][1];
    gf[7] = (gG[2][1] + gG[1][2]) / 2;
    gf[8] = gG[2][2];
    if (p.turbulence == 2)
        gf[9] = (gG[0][4] * a.gPhi[0] + gG[1][4] * a.gPhi[1] + gG[2][4] * a.gPhi[2]) / a.thv;
}

// FreeSlip boundary state for first-order fluxes (bc_momentum.jl:25-34)
inline void bc_state_first(const double qM[NS], const double n[3], double qP[NS]) {
    for (int s = 0; s < NS; ++s) qP[s] = qM[s];
    double dn = qM[1] * n[0] + qM[2] * n[1] + qM[3] * n[2];
    for (int c = 0; c < 3; ++c) qP[1 + c] -= 2 * dn * n[c];
}
// FreeSlip boundary state for the gradient flux (bc_momentum.jl:35-43)
inline void bc_state_grad(const double qM[NS], const double n[3], double qP[NS]) {
    for (int s = 0; s < NS; ++s) qP[s] = qM[s];
    double dn = qM[1] * n[0] + qM[2] * n[1] + qM[3] * n[2];
    for (int c = 0; c < 3; ++c) qP[1 + c] -= dn * n[c];
}

inline void load_q(const Model& m, const double* Q, int64_t e, int n, double q[NS]) {
    for (int s = 0; s < NS; ++s) q[s] = Q[(e * NS + s) * m.Np + n];
}

// update_auxiliary_state!: DryModel theta_v, air_T (moisture.jl:58-68)
void update_aux(Model& m, const double* Q) {
    const om_params& p = m.prm;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e)
        for (int n = 0; n < m.Np; ++n) {
            double q[NS];
            load_q(m, Q, e, n, q);
            Thermo t = phase_dry(p, q[0], q[4], q + 1, AUX(m, e, APHI, n));
            AUX(m, e, ATHV, n) = virtual_pottemp(p, t.T, t.p);
            AUX(m, e, AAIRT, n) = t.T;
        }
}

// Gradient passes: volume_gradients! (DGModel_kernels.jl:934-1328, H then V
// incremented) and dgsem_interface_gradients! (:1365-1651, faces 1-4 then 5-6).
void gradient_pass(Model& m, const double* Q) {
    const om_params& p = m.prm;
    int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, ngf = m.ngf, ng = ngrad_args(p);
    m.gradflux.assign((size_t)m.nelem * ngf * Np, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> G(Np * 5);
        for (int n = 0; n < Np; ++n) {
            double q[NS];
            load_q(m, Q, e, n, q);
            gradient_argument(p, q, AUXc(m, e, APHI, n), AUXc(m, e, ATHV, n), &G[n * 5]);
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double gH[3][5], gV[3][5];
                    for (int s = 0; s < ng; ++s) {
                        double G1 = 0, G2 = 0, G3 = 0;
                        for (int n = 0; n < Nq; ++n) {
                            G1 += Dm(m, i, n) * G[(n + Nq * (j + Nq * k)) * 5 + s];
                            G2 += Dm(m, j, n) * G[(i + Nq * (n + Nq * k)) * 5 + s];
                            G3 += Dm(m, k, n) * G[(i + Nq * (j + Nq * n)) * 5 + s];
                        }
                        gH[0][s] = VGc(m, e, XI1X1, ijk) * G1 + VGc(m, e, XI2X1, ijk) * G2;
                        gH[1][s] = VGc(m, e, XI1X2, ijk) * G1 + VGc(m, e, XI2X2, ijk) * G2;
                        gH[2][s] = VGc(m, e, XI1X3, ijk) * G1 + VGc(m, e, XI2X3, ijk) * G2;
                        gV[0][s] = VGc(m, e, XI3X1, ijk) * G3;
                        gV[1][s] = VGc(m, e, XI3X2, ijk) * G3;
                        gV[2][s] = VGc(m, e, XI3X3, ijk) * G3;
                    }
                    NodeAux a = node_aux(m, e, ijk);
                    double gfH[10], gfV[10];
                    gradient_flux(p, gH, a, gfH);
                    gradient_flux(p, gV, a, gfV);
                    for (int s = 0; s < ngf; ++s) m.gradflux[(e * ngf + s) * Np + ijk] = gfH[s] + gfV[s];
                }
        for (int f = 0; f < 6; ++f)
            for (int n = 0; n < Nfp; ++n) {
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                int tag = m.elemtobndy[e * 6 + f];
                if (tag != 0) { eP = e; vP = vM; }
                double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                double qM[NS], qP[NS], GM[5], GP[5];
                load_q(m, Q, e, vM, qM);
                NodeAux aM = node_aux(m, e, vM);
                gradient_argument(p, qM, aM.Phi, aM.thv, GM);
                double Gs[3][5];
                if (tag == 0) {
                    load_q(m, Q, eP, vP, qP);
                    NodeAux aP = node_aux(m, eP, vP);
                    gradient_argument(p, qP, aP.Phi, aP.thv, GP);
                    for (int d = 0; d < 3; ++d)
                        for (int s = 0; s < ng; ++s) Gs[d][s] = nv[d] * (GP[s] + GM[s]) / 2;
                } else {
                    if (p.mms) load_q(m, m.mms_exact, e, vM, qP);  // InitStateBC (bc_initstate.jl:12-26)
                    else bc_state_grad(qM, nv, qP);
                    // boundary_state! refreshes aux+ (theta_v) from state+
                    Thermo t = phase_dry(p, qP[0], qP[4], qP + 1, aM.Phi);
                    double thvP = virtual_pottemp(p, t.T, t.p);
                    gradient_argument(p, qP, aM.Phi, thvP, GP);
                    for (int d = 0; d < 3; ++d)
                        for (int s = 0; s < ng; ++s) Gs[d][s] = nv[d] * GP[s];
                }
                double nG[3][5];
                for (int d = 0; d < 3; ++d)
                    for (int s = 0; s < ng; ++s) nG[d][s] = nv[d] * GM[s];
                double gfs[10], gfm[10];
                gradient_flux(p, Gs, aM, gfs);
                gradient_flux(p, nG, aM, gfm);
                for (int s = 0; s < ngf; ++s) m.gradflux[(e * ngf + s) * Np + vM] += vMI * sM * (gfs[s] - gfm[s]);
            }
    }
}

// ----------------------------------------------------------------------------
// Hyperdiffusion passes (DGModel.jl:200-301), shared by the AtmosModel's
// DryBiharmonic closure (TurbulenceClosures.jl:793-848; GradientLaplacian
// states s = u_h[0..2], h_tot) and the constant-tensor scalar hyperdiffusion
// of test/Numerics/DGMethods/advection_diffusion (one state, rho).
// Qhypervisc_grad word 3 s + d holds d/dx_d of state s (first the gradient,
// later the hyperdiffusive state), Qhypervisc_div word s its laplacian.
// ----------------------------------------------------------------------------

// compute_gradient_argument! (TurbulenceClosures.jl:813-827):
// u_h = (I - khat khat') u with khat = grad Phi / g, and h_tot.
void hyper_argument(const om_params& p, const double G[5], const NodeAux& a, double H[4]) {
    double k[3] = {a.gPhi[0] / p.grav, a.gPhi[1] / p.grav, a.gPhi[2] / p.grav};
    for (int r = 0; r < 3; ++r) {
        double acc = 0;
        for (int c = 0; c < 3; ++c) acc += ((r == c ? 1.0 : 0.0) - k[r] * k[c]) * G[c];
        H[r] = acc;
    }
    H[3] = G[3];
}

inline double& HG(Model& m, int64_t e, int w, int n) { return m.hgrad[(e * 3 * m.ngl + w) * m.Np + n]; }
inline double HGc(const Model& m, int64_t e, int w, int n) { return m.hgrad[(e * 3 * m.ngl + w) * m.Np + n]; }
inline double& HD(Model& m, int64_t e, int s, int n) { return m.hdiv[(e * m.ngl + s) * m.Np + n]; }
inline double HDc(const Model& m, int64_t e, int s, int n) { return m.hdiv[(e * m.ngl + s) * m.Np + n]; }

// GradientLaplacian arguments of node n of element e (the minus-side state)
void node_hyper_args(const Model& m, const double* Q, int64_t e, int n, double* H) {
    if (m.law == 1) {
        H[0] = Q[e * m.Np + n];  // compute_gradient_argument!: transform.rho = state.rho
        return;
    }
    double q[NS], G[5];
    load_q(m, Q, e, n, q);
    NodeAux a = node_aux(m, e, n);
    gradient_argument(m.prm, q, a.Phi, a.thv, G);
    hyper_argument(m.prm, G, a, H);
}

// Gradients of the GradientLaplacian states into Qhypervisc_grad: the
// strong-form volume gradient (volume_gradients!, DGModel_kernels.jl:1083-1098,
// horizontal then vertical increment) and the central interface correction
// vMI sM (G* - n G-) (dgsem_interface_gradients!, :1618-1627), with
// G* = n G+ of the FreeSlip gradient boundary state on walls.
void hyper_gradient_pass(Model& m, const double* Q) {
    const om_params& p = m.prm;
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, ngl = m.ngl;
    const bool horiz = p.hyper_direction == 1;
    const int nface = horiz ? 4 : 6;
    m.hgrad.assign((size_t)m.nelem * 3 * ngl * Np, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> H(Np * ngl);
        for (int n = 0; n < Np; ++n) node_hyper_args(m, Q, e, n, &H[n * ngl]);
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    for (int s = 0; s < ngl; ++s) {
                        double G1 = 0, G2 = 0, G3 = 0;
                        for (int n = 0; n < Nq; ++n) {
                            G1 += Dm(m, i, n) * H[(n + Nq * (j + Nq * k)) * ngl + s];
                            G2 += Dm(m, j, n) * H[(i + Nq * (n + Nq * k)) * ngl + s];
                            G3 += Dm(m, k, n) * H[(i + Nq * (j + Nq * n)) * ngl + s];
                        }
                        for (int d = 0; d < 3; ++d) {
                            double gH = VGc(m, e, XI1X1 + 3 * d, ijk) * G1 + VGc(m, e, XI2X1 + 3 * d, ijk) * G2;
                            double gV = VGc(m, e, XI3X1 + 3 * d, ijk) * G3;
                            HG(m, e, 3 * s + d, ijk) = horiz ? gH : gH + gV;
                        }
                    }
                }
        for (int f = 0; f < nface; ++f)
            for (int n = 0; n < Nfp; ++n) {
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                int tag = m.elemtobndy[e * 6 + f];
                double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                const double* HM = &H[vM * ngl];
                double HP[4], Hs[3][4];
                if (tag == 0) {
                    node_hyper_args(m, Q, eP, vP, HP);
                    for (int d = 0; d < 3; ++d)
                        for (int s = 0; s < ngl; ++s) Hs[d][s] = nv[d] * (HP[s] + HM[s]) / 2;
                } else {
                    double qM[NS], qP[NS], G[5];
                    load_q(m, Q, e, vM, qM);
                    bc_state_grad(qM, nv, qP);
                    NodeAux aM = node_aux(m, e, vM);
                    gradient_argument(p, qP, aM.Phi, aM.thv, G);
                    hyper_argument(p, G, aM, HP);
                    for (int d = 0; d < 3; ++d)
                        for (int s = 0; s < ngl; ++s) Hs[d][s] = nv[d] * HP[s];
                }
                for (int s = 0; s < ngl; ++s)
                    for (int d = 0; d < 3; ++d) HG(m, e, 3 * s + d, vM) += vMI * sM * (Hs[d][s] - nv[d] * HM[s]);
            }
    }
}

// Laplacians Qhypervisc_div = M^-1 (D^T M grad G + sum_f L^T Mf (grad G)*):
// volume_divergence_of_gradients! (DGModel_kernels.jl:2132-2330, horizontal
// then vertical increment) and interface_divergence_of_gradients!
// (:2360-2495) with the central penalty (grad G+ + grad G-)' n / 2
// (NumericalFluxes.jl:720-730); on walls grad G+ = grad G-
// (src/Atmos/Model/boundaryconditions.jl:88-95).
void hyper_divergence_pass(Model& m) {
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, ngl = m.ngl;
    const bool horiz = m.prm.hyper_direction == 1;
    const int nface = horiz ? 4 : 6;
    m.hdiv.assign((size_t)m.nelem * ngl * Np, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> S1(Np * ngl), S2(Np * ngl), S3(Np * ngl);
        for (int n = 0; n < Np; ++n) {
            double M = VGc(m, e, VM, n);
            for (int s = 0; s < ngl; ++s) {
                double G1 = HGc(m, e, 3 * s + 0, n), G2 = HGc(m, e, 3 * s + 1, n), G3 = HGc(m, e, 3 * s + 2, n);
                S1[n * ngl + s] = M * (VGc(m, e, XI1X1, n) * G1 + VGc(m, e, XI1X2, n) * G2 + VGc(m, e, XI1X3, n) * G3);
                S2[n * ngl + s] = M * (VGc(m, e, XI2X1, n) * G1 + VGc(m, e, XI2X2, n) * G2 + VGc(m, e, XI2X3, n) * G3);
                S3[n * ngl + s] = M * (VGc(m, e, XI3X1, n) * G1 + VGc(m, e, XI3X2, n) * G2 + VGc(m, e, XI3X3, n) * G3);
            }
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double MI = VGc(m, e, VMI, ijk);
                    for (int s = 0; s < ngl; ++s) {
                        double lh = 0, lv = 0;
                        for (int n = 0; n < Nq; ++n) {
                            lh -= MI * Dm(m, n, i) * S1[(n + Nq * (j + Nq * k)) * ngl + s];
                            lh -= MI * Dm(m, n, j) * S2[(i + Nq * (n + Nq * k)) * ngl + s];
                        }
                        for (int n = 0; n < Nq; ++n) lv -= MI * Dm(m, n, k) * S3[(i + Nq * (j + Nq * n)) * ngl + s];
                        HD(m, e, s, ijk) = horiz ? lh : lh + lv;
                    }
                }
        for (int f = 0; f < nface; ++f)
            for (int n = 0; n < Nfp; ++n) {
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                int tag = m.elemtobndy[e * 6 + f];
                if (tag != 0) { eP = e; vP = vM; }
                double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                for (int s = 0; s < ngl; ++s) {
                    double acc = 0;
                    for (int d = 0; d < 3; ++d)
                        acc += (HGc(m, eP, 3 * s + d, vP) + HGc(m, e, 3 * s + d, vM)) * (nv[d] / 2);
                    HD(m, e, s, vM) += vMI * sM * acc;
                }
            }
    }
}

// transform_post_gradient_laplacian! of a gradient g (word 3 s + d) at a node:
// DryBiharmonic nu_4 g with nu_4 = (Delta_h / 2)^4 / 2 / tau
// (TurbulenceClosures.jl:829-848), or eta = H g for the constant tensor H
// (test/Numerics/DGMethods/advection_diffusion/advection_diffusion_model.jl:310-326).
void hyper_transform(const Model& m, int64_t e, int n, const double* g, double* out) {
    if (m.law == 1) {
        for (int d = 0; d < 3; ++d) out[d] = m.Hten[d] * g[0] + m.Hten[d + 3] * g[1] + m.Hten[d + 6] * g[2];
        return;
    }
    double h = AUXc(m, e, AHDELTA, n) / 2;
    double nu4 = h * h * h * h / 2 / m.prm.tau_hyper;
    for (int w = 0; w < 12; ++w) out[w] = nu4 * g[w];
}

// Hyperdiffusive state into Qhypervisc_grad: volume_gradients_of_laplacians!
// (DGModel_kernels.jl:2525-2845; horizontal kernel writes T(grad_H lap), the
// vertical one adds T(grad_V lap)) and interface_gradients_of_laplacians!
// adding T(n (lap+ - lap-) / 2) (NumericalFluxes.jl:768-790); zero on walls
// where lap+ = lap-.
void hyper_gradlap_pass(Model& m) {
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, ngl = m.ngl, nw = 3 * m.ngl;
    const bool horiz = m.prm.hyper_direction == 1;
    const int nface = horiz ? 4 : 6;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double gH[12], gV[12], tH[12], tV[12];
                    for (int s = 0; s < ngl; ++s) {
                        double L1 = 0, L2 = 0, L3 = 0;
                        for (int n = 0; n < Nq; ++n) {
                            L1 += Dm(m, i, n) * HDc(m, e, s, n + Nq * (j + Nq * k));
                            L2 += Dm(m, j, n) * HDc(m, e, s, i + Nq * (n + Nq * k));
                            L3 += Dm(m, k, n) * HDc(m, e, s, i + Nq * (j + Nq * n));
                        }
                        for (int d = 0; d < 3; ++d) {
                            gH[3 * s + d] = VGc(m, e, XI1X1 + 3 * d, ijk) * L1 + VGc(m, e, XI2X1 + 3 * d, ijk) * L2;
                            gV[3 * s + d] = VGc(m, e, XI3X1 + 3 * d, ijk) * L3;
                        }
                    }
                    hyper_transform(m, e, ijk, gH, tH);
                    hyper_transform(m, e, ijk, gV, tV);
                    for (int w = 0; w < nw; ++w) HG(m, e, w, ijk) = horiz ? tH[w] : tH[w] + tV[w];
                }
        for (int f = 0; f < nface; ++f)
            for (int n = 0; n < Nfp; ++n) {
                if (m.elemtobndy[e * 6 + f] != 0) continue;
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                double G[12], T[12];
                for (int s = 0; s < ngl; ++s) {
                    double dl = HDc(m, eP, s, vP) - HDc(m, e, s, vM);
                    for (int d = 0; d < 3; ++d) G[3 * s + d] = nv[d] * dl / 2;
                }
                hyper_transform(m, e, vM, G, T);
                for (int w = 0; w < nw; ++w) HG(m, e, w, vM) += vMI * sM * T[w];
            }
    }
}

void hyper_passes(Model& m, const double* Q) {
    hyper_gradient_pass(m, Q);
    hyper_divergence_pass(m);
    hyper_gradlap_pass(m);
}

// Tendency of the constant-tensor scalar hyperdiffusion model
// (periodic_3D_hyperdiffusion.jl with advection = diffusion = false):
// d rho/dt = -div(eta), eta = H grad(lap rho); weak-form volume divergence
// (DGModel_kernels.jl:64-300) and the central second-order numerical flux
// (eta- + eta+)' n / 2 (NumericalFluxes.jl:670-715).
void scalar_hyper_tendency(Model& m, double* T, const double* Q, double alpha, double beta) {
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
    // HorizontalDirection: the model direction restricts the tendency too
    const bool horiz = m.prm.hyper_direction == 1;
    const int nface = horiz ? 4 : 6;
    hyper_passes(m, Q);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> F1(Np), F2(Np), F3(Np);
        for (int n = 0; n < Np; ++n) {
            double M = VGc(m, e, VM, n);
            double F[3] = {HGc(m, e, 0, n), HGc(m, e, 1, n), HGc(m, e, 2, n)};
            F1[n] = M * (VGc(m, e, XI1X1, n) * F[0] + VGc(m, e, XI1X2, n) * F[1] + VGc(m, e, XI1X3, n) * F[2]);
            F2[n] = M * (VGc(m, e, XI2X1, n) * F[0] + VGc(m, e, XI2X2, n) * F[1] + VGc(m, e, XI2X3, n) * F[2]);
            F3[n] = M * (VGc(m, e, XI3X1, n) * F[0] + VGc(m, e, XI3X2, n) * F[1] + VGc(m, e, XI3X3, n) * F[2]);
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double MI = VGc(m, e, VMI, ijk);
                    double lh = 0, lv = 0;
                    for (int n = 0; n < Nq; ++n) {
                        lh += MI * Dm(m, n, i) * F1[n + Nq * (j + Nq * k)];
                        lh += MI * Dm(m, n, j) * F2[i + Nq * (n + Nq * k)];
                    }
                    for (int n = 0; n < Nq; ++n) lv += MI * Dm(m, n, k) * F3[i + Nq * (j + Nq * n)];
                    if (horiz) lv = 0;
                    size_t idx = (size_t)e * Np + ijk;
                    double Th = (beta != 0) ? alpha * lh + beta * T[idx] : alpha * lh;
                    T[idx] = alpha * lv + Th;
                }
        for (int f = 0; f < nface; ++f)
            for (int n = 0; n < Nfp; ++n) {
                int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
                int vM = (int)(idM % Np);
                int64_t eP = idP / Np; int vP = (int)(idP % Np);
                double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                double fl = 0;
                for (int d = 0; d < 3; ++d) fl += (HGc(m, e, d, vM) + HGc(m, eP, d, vP)) * (nv[d] / 2);
                T[(size_t)e * Np + vM] -= alpha * vMI * sM * fl;
            }
    }
}

// Numerical flux F*.n at one face node: Rusanov/central first order
// (NumericalFluxes.jl:219-340, boundary wrapper :163-205) plus central
// second order (:668-715; zero on FreeSlip/Insulating walls,
// Atmos/Model/boundaryconditions.jl:113-185).
void face_flux(const Model& m, const double* Q, int64_t e, int f, int n, double fl[NS]) {
    const om_params& p = m.prm;
    int Np = m.Np, Nfp = m.Nfp, ngf = m.ngf;
    int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
    int vM = (int)(idM % Np);
    int64_t eP = idP / Np; int vP = (int)(idP % Np);
    int tag = m.elemtobndy[e * 6 + f];
    if (tag != 0) { eP = e; vP = vM; }
    double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
    double qM[NS], qP[NS];
    load_q(m, Q, e, vM, qM);
    NodeAux aM = node_aux(m, e, vM);
    NodeAux aP = node_aux(m, eP, vP);
    if (tag == 0) load_q(m, Q, eP, vP, qP);
    else if (p.mms) load_q(m, m.mms_exact, e, vM, qP);  // InitStateBC (bc_initstate.jl:12-26)
    else bc_state_first(qM, nv, qP);
    for (int s = 0; s < NS; ++s) fl[s] = 0;
    double FM[3][NS], FP[3][NS];
    flux_first_order(p, qM, aM, FM);
    flux_first_order(p, qP, aP, FP);
    for (int s = 0; s < NS; ++s) {
        double acc = 0;
        for (int d = 0; d < 3; ++d) acc += (FM[d][s] + FP[d][s]) * (nv[d] / 2);
        fl[s] += acc;
    }
    if (p.numflux == 0) {
        double wM = wavespeed(p, nv, qM, aM), wP = wavespeed(p, nv, qP, aP);
        double mw = std::max(wM, wP);
        for (int s = 0; s < NS; ++s) fl[s] += mw * (qM[s] - qP[s]) / 2;
    }
    if ((p.turbulence != 0 || p.hyperdiffusion != 0) && tag == 0) {
        double gfM[10] = {0}, gfP[10] = {0}, hdM[12], hdP[12];
        if (p.turbulence != 0) {
            const double* gM = &m.gradflux[0];
            for (int s = 0; s < ngf; ++s) {
                gfM[s] = gM[(e * ngf + s) * Np + vM];
                gfP[s] = gM[(eP * ngf + s) * Np + vP];
            }
        }
        if (p.hyperdiffusion != 0)
            for (int w = 0; w < 12; ++w) {
                hdM[w] = HGc(m, e, w, vM);
                hdP[w] = HGc(m, eP, w, vP);
            }
        const bool hyp = p.hyperdiffusion != 0;
        flux_second_order(m, qM, gfM, aM, FM, hyp ? hdM : nullptr);
        flux_second_order(m, qP, gfP, aP, FP, hyp ? hdP : nullptr);
        for (int s = 0; s < NS; ++s) {
            double acc = 0;
            for (int d = 0; d < 3; ++d) acc += (FM[d][s] + FP[d][s]) * (nv[d] / 2);
            fl[s] += acc;
        }
    } else if (p.mms && p.turbulence != 0 && tag != 0) {
        // InitStateBC second order: the one-sided flux of the boundary state
        // with the interior gradient flux (NumericalFluxes.jl:872-966)
        double gfM[10] = {0};
        for (int s = 0; s < ngf; ++s) gfM[s] = m.gradflux[(e * ngf + s) * Np + vM];
        flux_second_order(m, qP, gfM, aM, FP, nullptr);
        for (int s = 0; s < NS; ++s) {
            double acc = 0;
            for (int d = 0; d < 3; ++d) acc += FP[d][s] * nv[d];
            fl[s] += acc;
        }
    }
}

// Full tendency, DGModel.jl:85-427: T = alpha * dQ/dt(Q) + beta * T.
void tendency(Model& m, double* T, const double* Q, double t, double alpha, double beta) {
    (void)t;
    const om_params& p = m.prm;
    int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp, ngf = m.ngf;
    update_aux(m, Q);
    if (p.turbulence != 0) gradient_pass(m, Q);
    if (p.hyperdiffusion != 0) hyper_passes(m, Q);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> F1(Np * NS), F2(Np * NS), F3(Np * NS), Src(Np * NS);
        for (int n = 0; n < Np; ++n) {
            double q[NS];
            load_q(m, Q, e, n, q);
            NodeAux a = node_aux(m, e, n);
            double F[3][NS], G[3][NS];
            flux_first_order(p, q, a, F);
            if (p.turbulence != 0 || p.hyperdiffusion != 0) {
                double gf[10] = {0}, hd[12];
                if (p.turbulence != 0)
                    for (int s = 0; s < ngf; ++s) gf[s] = m.gradflux[(e * ngf + s) * Np + n];
                if (p.hyperdiffusion != 0)
                    for (int w = 0; w < 12; ++w) hd[w] = HGc(m, e, w, n);
                flux_second_order(m, q, gf, a, G, p.hyperdiffusion != 0 ? hd : nullptr);
                for (int d = 0; d < 3; ++d)
                    for (int s = 0; s < NS; ++s) F[d][s] += G[d][s];
            }
            double M = VGc(m, e, VM, n);
            for (int s = 0; s < NS; ++s) {
                F1[n * NS + s] = M * (VGc(m, e, XI1X1, n) * F[0][s] + VGc(m, e, XI1X2, n) * F[1][s] + VGc(m, e, XI1X3, n) * F[2][s]);
                F2[n * NS + s] = M * (VGc(m, e, XI2X1, n) * F[0][s] + VGc(m, e, XI2X2, n) * F[1][s] + VGc(m, e, XI2X3, n) * F[2][s]);
                F3[n * NS + s] = M * (VGc(m, e, XI3X1, n) * F[0][s] + VGc(m, e, XI3X2, n) * F[1][s] + VGc(m, e, XI3X3, n) * F[2][s]);
            }
            source(p, q, a, &Src[n * NS]);
            if (p.mms)  // MMSSource (mms_bc_atmos.jl:60-80)
                for (int s = 0; s < NS; ++s) Src[n * NS + s] += m.mms_src[(e * NS + s) * Np + n];
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double MI = VGc(m, e, VMI, ijk);
                    for (int s = 0; s < NS; ++s) {
                        // horizontal kernel (DGModel_kernels.jl:282-295)
                        double lh = 0;
                        for (int n = 0; n < Nq; ++n) {
                            lh += MI * Dm(m, n, i) * F1[(n + Nq * (j + Nq * k)) * NS + s];
                            lh += MI * Dm(m, n, j) * F2[(i + Nq * (n + Nq * k)) * NS + s];
                        }
                        // vertical kernel (:504-513, 519-524)
                        double lv = 0;
                        for (int kk = 0; kk < Nq; ++kk) lv += MI * Dm(m, kk, k) * F3[(i + Nq * (j + Nq * kk)) * NS + s];
                        lv += Src[ijk * NS + s];
                        size_t idx = (size_t)(e * NS + s) * Np + ijk;
                        double Th = (beta != 0) ? alpha * lh + beta * T[idx] : alpha * lh;
                        T[idx] = alpha * lv + Th;
                    }
                }
        // interface kernel (faces 1-4, then 5-6), DGModel_kernels.jl:893-896
        for (int f = 0; f < 6; ++f)
            for (int n = 0; n < Nfp; ++n) {
                double fl[NS];
                face_flux(m, Q, e, f, n, fl);
                int vM = (int)(m.vmapM[(e * 6 + f) * Nfp + n] % Np);
                double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                for (int s = 0; s < NS; ++s) T[(size_t)(e * NS + s) * Np + vM] -= alpha * vMI * sM * fl[s];
            }
    }
}

// LSRK54CarpenterKennedy coefficients, LowStorageRungeKuttaMethod.jl:302-324
const double RKA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                       -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double RKB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                       1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                       2277821191437.0 / 14882151754819.0};
const double RKC[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                       2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

// dostep!, LowStorageRungeKuttaMethod.jl:102-158
void lsrk_step(Model& m, double* Q, double* dQ, double time, double dt) {
    size_t len = (size_t)m.nelem * NS * m.Np;
    for (int s = 0; s < 5; ++s) {
        tendency(m, dQ, Q, time + RKC[s] * dt, 1.0, 1.0);
        double a = RKA[(s + 1) % 5], b = RKB[s];
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < len; ++i) {
            Q[i] += b * dt * dQ[i];
            dQ[i] *= a;
        }
    }
}

// ----------------------------------------------------------------------------
// HEVI: AtmosAcousticGravityLinearModel as a DGModel in VerticalDirection
// (Atmos/Model/linear.jl:1-57, 150-160, 242-262; linear_tendencies.jl;
// linear_atmos_tendencies.jl), the column-wise banded LU of
// SystemSolvers/columnwise_lu_solver.jl and ARK2GiraldoKellyConstantinescu in
// its LowStorageVariant (ODESolvers/AdditiveRungeKuttaMethod.jl:413-538,
// 603-662, 839-897).
// ----------------------------------------------------------------------------
struct LinAux {
    double Phi, gPhi[3], h_ref, c_ref;
};

inline LinAux lin_aux(const Model& m, int64_t e, int n) {
    LinAux a;
    a.Phi = AUXc(m, e, APHI, n);
    a.gPhi[0] = AUXc(m, e, AGPX, n);
    a.gPhi[1] = AUXc(m, e, AGPY, n);
    a.gPhi[2] = AUXc(m, e, AGPZ, n);
    // LinearEnergyFlux: (ref.rhoe + ref.p) / ref.rho (linear_tendencies.jl:62-71)
    a.h_ref = (AUXc(m, e, ARHOE_REF, n) + AUXc(m, e, AP_REF, n)) / AUXc(m, e, ARHO_REF, n);
    // wavespeed(::AtmosLinearModel) = soundspeed_air(ref.T) (linear.jl:150-160)
    a.c_ref = soundspeed(m.prm, AUXc(m, e, AT_REF, n));
    return a;
}

// linearized_air_pressure of a dry state (linear.jl:18-37, 49-57)
inline double linearized_pressure(const om_params& p, double rho, double rhoe, double Phi) {
    const double rho_epot = rho * Phi;
    return rho * p.R_d * p.T_0 + p.R_d / p.cv_d * (rhoe - rho_epot);
}

// First-order flux of the linear model: Advect, LinearPressureGradient,
// LinearEnergyFlux (linear_tendencies.jl:8-11, 21-27, 62-71).
void linear_flux(const om_params& p, const double q[NS], const LinAux& a, double F[3][NS]) {
    const double pL = linearized_pressure(p, q[0], q[4], a.Phi);
    for (int d = 0; d < 3; ++d) {
        F[d][0] = q[1 + d];
        for (int c = 0; c < 3; ++c) F[d][1 + c] = (c == d) ? pL : 0.0;
        F[d][4] = a.h_ref * q[1 + d];
    }
}

// Rusanov flux of the linear model across face f at face node n of element e
// (NumericalFluxes.jl:223-285 with the linear wavespeed; FreeSlip/Insulating
// boundary state on walls, boundaryconditions.jl:60-95, bc_momentum.jl:25-34).
void linear_face_flux(const Model& m, const double* Q, int64_t e, int f, int n, double fl[NS]) {
    const om_params& p = m.prm;
    const int Np = m.Np, Nfp = m.Nfp;
    const int64_t idM = m.vmapM[(e * 6 + f) * Nfp + n], idP = m.vmapP[(e * 6 + f) * Nfp + n];
    const int vM = (int)(idM % Np);
    int64_t eP = idP / Np;
    int vP = (int)(idP % Np);
    const int tag = m.elemtobndy[e * 6 + f];
    if (tag != 0) { eP = e; vP = vM; }
    const double nv[3] = {SGc(m, e, f, n, SN1), SGc(m, e, f, n, SN2), SGc(m, e, f, n, SN3)};
    double qM[NS], qP[NS];
    load_q(m, Q, e, vM, qM);
    if (tag == 0) load_q(m, Q, eP, vP, qP);
    else bc_state_first(qM, nv, qP);
    const LinAux aM = lin_aux(m, e, vM), aP = lin_aux(m, eP, vP);
    double FM[3][NS], FP[3][NS];
    linear_flux(p, qM, aM, FM);
    linear_flux(p, qP, aP, FP);
    const double mw = std::max(aM.c_ref, aP.c_ref);
    for (int s = 0; s < NS; ++s) {
        double acc = 0;
        for (int d = 0; d < 3; ++d) acc += (FM[d][s] + FP[d][s]) * (nv[d] / 2);
        fl[s] = acc + mw * (qM[s] - qP[s]) / 2;
    }
}

// lineardg(T, Q; alpha, beta): T = alpha * L(Q) + beta * T with the vertical
// volume kernel (DGModel_kernels.jl:312-548: M xi3 . F, M^-1 D^T, the
// Gravity source -rho grad Phi of linear_tendencies.jl:33-45) and the
// interface kernel on faces 5 and 6 (:588-901).
void linear_tendency(Model& m, double* T, const double* Q, double alpha, double beta) {
    const om_params& p = m.prm;
    const int Nq = m.Nq, Np = m.Np, Nfp = m.Nfp;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m.nelem; ++e) {
        std::vector<double> F3(Np * NS), Src(Np * NS);
        for (int n = 0; n < Np; ++n) {
            double q[NS];
            load_q(m, Q, e, n, q);
            const LinAux a = lin_aux(m, e, n);
            double F[3][NS];
            linear_flux(p, q, a, F);
            const double M = VGc(m, e, VM, n);
            for (int s = 0; s < NS; ++s)
                F3[n * NS + s] = M * (VGc(m, e, XI3X1, n) * F[0][s] + VGc(m, e, XI3X2, n) * F[1][s] + VGc(m, e, XI3X3, n) * F[2][s]);
            Src[n * NS + 0] = 0;
            for (int c = 0; c < 3; ++c) Src[n * NS + 1 + c] = -q[0] * a.gPhi[c];
            Src[n * NS + 4] = 0;
        }
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    const int ijk = i + Nq * (j + Nq * k);
                    const double MI = VGc(m, e, VMI, ijk);
                    for (int s = 0; s < NS; ++s) {
                        double lv = 0;
                        for (int kk = 0; kk < Nq; ++kk) lv += MI * Dm(m, kk, k) * F3[(i + Nq * (j + Nq * kk)) * NS + s];
                        lv += Src[ijk * NS + s];
                        const size_t idx = (size_t)(e * NS + s) * Np + ijk;
                        T[idx] = (beta != 0) ? alpha * lv + beta * T[idx] : alpha * lv;
                    }
                }
        for (int f = 4; f < 6; ++f)
            for (int n = 0; n < Nfp; ++n) {
                double fl[NS];
                linear_face_flux(m, Q, e, f, n, fl);
                const int vM = (int)(m.vmapM[(e * 6 + f) * Nfp + n] % Np);
                const double sM = SGc(m, e, f, n, SSM), vMI = SGc(m, e, f, n, SVMI);
                for (int s = 0; s < NS; ++s) T[(size_t)(e * NS + s) * Np + vM] -= alpha * vMI * sM * fl[s];
            }
    }
}

// Elements per vertical stack; 0 when the mesh has no wall-bounded columns.
int stack_height(const Model& m) {
    if (m.kind == 1) return m.shell.nvert;
    if (m.kind == 0 && m.law == 0 && !m.mesh.periodic[2]) return m.mesh.ne[2];
    return 0;
}

// ARK2GiraldoKellyConstantinescu (AdditiveRungeKuttaMethod.jl:839-897) with a
// LinearBackwardEulerSolver(ManyColumnLU()) (BackwardEulerSolvers.jl,
// columnwise_lu_solver.jl).  One banded matrix per vertical line (i, j) of
// each stack; unknown r = s + 5 (k + Nq v) of stack level v; bandwidths
// p = q = 5 Nq - 1 (eband = 1, columnwise_lu_solver.jl:56-74).
struct Hevi {
    Model* m = nullptr;
    double dt = 0, alpha = 0;
    int split = 0;
    double Ae[3][3], Ai[3][3], B[3], C[3];
    int nvert = 0, n = 0, bw = 0;
    int64_t nline = 0;
    std::vector<double> AB;    // line-major; A(row, col) at [(line * (2 bw + 1) + bw + row - col) * n + col]
    std::vector<double> S1, S2, R0, R1, R2, Qhat, Qtt;
};

inline size_t line_state_index(const Hevi& h, int64_t line, int r) {
    const Model& m = *h.m;
    const int Nq = m.Nq, Nfp = m.Nfp;
    const int s = r % NS, k = (r / NS) % Nq, v = r / (NS * Nq);
    const int64_t col = line / Nfp;
    const int ij = (int)(line % Nfp);
    const int64_t e = v + (int64_t)h.nvert * col;
    return (size_t)(e * NS + s) * m.Np + ij + Nfp * k;
}

inline double& band(Hevi& h, int64_t line, int row, int col) {
    return h.AB[((size_t)line * (2 * h.bw + 1) + h.bw + row - col) * h.n + col];
}

// banded_matrix of the EulerOperator Q - alpha L(Q) (columnwise_lu_solver.jl:
// 228-312, 404-488: the operator applied to unit states, one per (element
// level mod 2 eband + 1, k, s)), then band_lu! (:129-158, 555-600; Golub &
// Van Loan Algorithm 4.3.1 without pivoting).
void hevi_factorize(Hevi& h) {
    Model& m = *h.m;
    const int Nq = m.Nq, Nfp = m.Nfp, Np = m.Np;
    const size_t len = (size_t)m.nelem * NS * Np;
    h.n = NS * Nq * h.nvert;
    h.bw = NS * Nq - 1;
    h.nline = (m.nelem / h.nvert) * Nfp;
    h.AB.assign((size_t)h.nline * (2 * h.bw + 1) * h.n, 0.0);
    std::vector<double> E(len), R(len);
    const double eps = -h.alpha;
    for (int vi = 0; vi < 3 && vi < h.nvert; ++vi)
        for (int k = 0; k < Nq; ++k)
            for (int s = 0; s < NS; ++s) {
                std::fill(E.begin(), E.end(), 0.0);
                for (int64_t e = 0; e < m.nelem; ++e)
                    if ((e % h.nvert) % 3 == vi)
                        for (int ij = 0; ij < Nfp; ++ij) E[(size_t)(e * NS + s) * Np + ij + Nfp * k] = 1.0;
                linear_tendency(m, R.data(), E.data(), 1.0, 0.0);
                for (int64_t line = 0; line < h.nline; ++line)
                    for (int v = 0; v < h.nvert; ++v) {
                        int vs = -1;
                        for (int d = -1; d <= 1; ++d)
                            if (v + d >= 0 && v + d < h.nvert && (v + d) % 3 == vi) vs = v + d;
                        if (vs < 0) continue;
                        const int col = s + NS * (k + Nq * vs);
                        for (int r = NS * Nq * v; r < NS * Nq * (v + 1); ++r) {
                            const size_t idx = line_state_index(h, line, r);
                            const double val = E[idx] + eps * R[idx];  // EulerOperator: Q + eps L(Q)
                            if (std::abs(r - col) <= h.bw) band(h, line, r, col) = val;
                            else if (val != 0) throw std::runtime_error("HEVI: coupling outside the band");
                        }
                    }
            }
    const int n = h.n, bw = h.bw;
#pragma omp parallel for schedule(static)
    for (int64_t line = 0; line < h.nline; ++line)
        for (int kk = 0; kk < n; ++kk) {
            const double Aq = band(h, line, kk, kk);
            for (int ii = 1; ii <= bw && kk + ii < n; ++ii) band(h, line, kk + ii, kk) /= Aq;
            for (int jj = 1; jj <= bw && kk + jj < n; ++jj) {
                const double Ajj = band(h, line, kk, kk + jj);
                for (int ii = 1; ii <= bw && kk + ii < n; ++ii)
                    band(h, line, kk + ii, kk + jj) -= band(h, line, kk + ii, kk) * Ajj;
            }
        }
}

// linearsolve! of the factorization: Q .= Qrhs, band_forward!, band_back!
// (columnwise_lu_solver.jl:110-127, 615-690, 704-780).
void hevi_solve(Hevi& h, double* Q, const double* Qrhs) {
    Model& m = *h.m;
    const size_t len = (size_t)m.nelem * NS * m.Np;
    if (Q != Qrhs) std::memcpy(Q, Qrhs, len * sizeof(double));
    const int n = h.n, bw = h.bw;
#pragma omp parallel for schedule(static)
    for (int64_t line = 0; line < h.nline; ++line) {
        std::vector<double> b(n);
        for (int r = 0; r < n; ++r) b[r] = Q[line_state_index(h, line, r)];
        for (int jj = 0; jj < n; ++jj)
            for (int ii = 1; ii <= bw && jj + ii < n; ++ii) b[jj + ii] -= band(h, line, jj + ii, jj) * b[jj];
        for (int jj = n - 1; jj >= 0; --jj) {
            b[jj] /= band(h, line, jj, jj);
            for (int ii = 1; ii <= bw && jj - ii >= 0; ++ii) b[jj - ii] -= band(h, line, jj - ii, jj) * b[jj];
        }
        for (int r = 0; r < n; ++r) Q[line_state_index(h, line, r)] = b[r];
    }
}

// rhs!: the full tendency, or the remainder f - l when split (remainder.jl)
void hevi_rhs(Hevi& h, double* R, const double* Q, double t) {
    tendency(*h.m, R, Q, t, 1.0, 0.0);
    if (h.split) linear_tendency(*h.m, R, Q, -1.0, 1.0);
}

// dostep!(Q, ark, ::LowStorageVariant, p, time) (AdditiveRungeKuttaMethod.jl:413-538)
void hevi_step(Hevi& h, double* Q, double time) {
    Model& m = *h.m;
    const size_t len = (size_t)m.nelem * NS * m.Np;
    const double dt = h.dt;
    double* Sst[3] = {Q, h.S1.data(), h.S2.data()};
    double* Rst[3] = {h.R0.data(), h.R1.data(), h.R2.data()};
    hevi_rhs(h, Rst[0], Sst[0], time + h.C[0] * dt);
    for (int is = 1; is < 3; ++is) {
        const double stagetime = time + h.C[is] * dt;
        double rk[3];
        for (int js = 0; js < is; ++js)
            rk[js] = h.split ? h.Ai[is][js] / h.Ai[is][is] : (h.Ai[is][js] - h.Ae[is][js]) / h.Ai[is][is];
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < len; ++i) {
            double qh = Q[i], qs = -0.0;
            for (int js = 0; js < is; ++js) {
                const double common = rk[js] * Sst[js][i];
                qh += common + dt * h.Ae[is][js] * Rst[js][i];
                qs -= common;
            }
            Sst[is][i] = qs;
            h.Qhat[i] = qh;
            h.Qtt[i] = qh;
        }
        hevi_solve(h, h.Qtt.data(), h.Qhat.data());
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < len; ++i) Sst[is][i] += h.Qtt[i];
        hevi_rhs(h, Rst[is], Sst[is], stagetime);
    }
    if (h.split)
        for (int is = 0; is < 3; ++is) linear_tendency(m, Rst[is], Sst[is], 1.0, 1.0);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < len; ++i)
        for (int is = 0; is < 3; ++is) Q[i] += h.B[is] * dt * Rst[is][i];
}

// TwoSum-based double-double accumulate (DoubleFloats.jl semantics)
struct DD {
    double hi = 0, lo = 0;
    void add(double x) {
        double s = hi + x;
        double bp = s - hi;
        double err = (hi - (s - bp)) + (x - bp);
        lo += err;
        double s2 = s + lo;
        lo = lo - (s2 - s);
        hi = s2;
    }
};

// exact product as a double-double then added
inline void dd_add_prod(DD& acc, double a, double b) {
    double p = a * b;
    double e = std::fma(a, b, -p);
    acc.add(p);
    acc.add(e);
}

}  // namespace

extern "C" {

typedef struct Model om_model;

om_model* om_create(const om_brick* b, const om_params* p) {
    Model* m = new Model();
    m->mesh = *b;
    m->prm = *p;
    m->N = b->N;
    m->Nq = b->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = (int64_t)b->ne[0] * b->ne[1] * b->ne[2];
    m->ngf = p->turbulence == 2 ? 10 : 9;
    lgl(m->N, m->xi, m->omega);
    spectral_derivative(m->xi, m->D);
    build_geometry(*m);
    init_aux(*m);
    return m;
}

om_model* om_create_shell(const om_shell* sh, const om_params* p) {
    Model* m = new Model();
    m->kind = 1;
    m->shell = *sh;
    std::memset(&m->mesh, 0, sizeof(m->mesh));
    m->prm = *p;
    m->N = sh->N;
    m->Nq = sh->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = 6LL * sh->nhorz * sh->nhorz * sh->nvert;
    m->ngf = p->turbulence == 2 ? 10 : 9;
    lgl(m->N, m->xi, m->omega);
    spectral_derivative(m->xi, m->D);
    try {
        build_shell_geometry(*m);
    } catch (const std::exception&) {
        delete m;
        return nullptr;
    }
    init_aux(*m);
    return m;
}

// Constant-tensor scalar hyperdiffusion on a brick (one state per node,
// layout (Np, 1, nelem)); H column-major 3x3.
om_model* om_create_scalar_hyper(const om_brick* b, const double* H, int direction) {
    om_params p;
    std::memset(&p, 0, sizeof(p));
    p.hyper_direction = direction;
    Model* m = new Model();
    m->mesh = *b;
    m->prm = p;
    m->law = 1;
    m->ngl = 1;
    for (int i = 0; i < 9; ++i) m->Hten[i] = H[i];
    m->N = b->N;
    m->Nq = b->N + 1;
    m->Np = m->Nq * m->Nq * m->Nq;
    m->Nfp = m->Nq * m->Nq;
    m->nelem = (int64_t)b->ne[0] * b->ne[1] * b->ne[2];
    m->ngf = 9;
    lgl(m->N, m->xi, m->omega);
    spectral_derivative(m->xi, m->D);
    build_geometry(*m);
    init_aux(*m);
    return m;
}

void om_scalar_hyper_tendency(om_model* m, double* dQ, const double* Q, double alpha, double beta) {
    scalar_hyper_tendency(*m, dQ, Q, alpha, beta);
}

// nsteps LSRK54 steps (LowStorageRungeKuttaMethod.jl:102-158) of the scalar model
void om_scalar_hyper_lsrk54(om_model* m, double* Q, double* dQ, double dt, int nsteps) {
    size_t len = (size_t)m->nelem * m->Np;
    for (int it = 0; it < nsteps; ++it)
        for (int s = 0; s < 5; ++s) {
            scalar_hyper_tendency(*m, dQ, Q, 1.0, 1.0);
            double a = RKA[(s + 1) % 5], b = RKB[s];
            for (size_t i = 0; i < len; ++i) {
                Q[i] += b * dt * dQ[i];
                dQ[i] *= a;
            }
        }
}

void om_free(om_model* m) { delete m; }

int64_t om_nelem(const om_model* m) { return m->nelem; }
int om_Np(const om_model* m) { return m->Np; }
int om_naux(void) { return NAUX; }
int om_ngradflux(const om_model* m) { return m->ngf; }
const double* om_vgeo(const om_model* m) { return m->vgeo.data(); }
const double* om_sgeo(const om_model* m) { return m->sgeo.data(); }
const double* om_aux(const om_model* m) { return m->aux.data(); }
const double* om_gradflux(const om_model* m) { return m->gradflux.data(); }
const int64_t* om_vmapM(const om_model* m) { return m->vmapM.data(); }
const int64_t* om_vmapP(const om_model* m) { return m->vmapP.data(); }
const int* om_elemtobndy(const om_model* m) { return m->elemtobndy.data(); }
const double* om_D(const om_model* m) { return m->D.data(); }
const double* om_lgl_nodes(const om_model* m) { return m->xi.data(); }
const double* om_lgl_weights(const om_model* m) { return m->omega.data(); }

int om_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

void om_tendency(om_model* m, double* dQ, const double* Q, double t, double alpha, double beta) {
    tendency(*m, dQ, Q, t, alpha, beta);
}

// Gradient-flux pass only (for parity of the diffusive pass)
void om_gradient_pass(om_model* m, const double* Q) {
    update_aux(*m, Q);
    gradient_pass(*m, Q);
}

// Manufactured-solution inputs of the next tendency (Np, 5, nelem): source
// terms and the InitStateBC state at the nodes, at the tendency's time.
void om_set_mms(om_model* m, const double* src, const double* exact) {
    m->mms_src = src;
    m->mms_exact = exact;
}

// Hyperdiffusion passes only: afterwards om_hyper_grad holds nu grad^3
// (Np, 12, nelem) and om_hyper_div the laplacians (Np, 4, nelem).
void om_hyper_pass(om_model* m, const double* Q) {
    update_aux(*m, Q);
    hyper_passes(*m, Q);
}
const double* om_hyper_grad(const om_model* m) { return m->hgrad.data(); }
const double* om_hyper_div(const om_model* m) { return m->hdiv.data(); }

// nsteps LSRK54 steps of size dt from time t0 (dQ is the solver's register)
void om_lsrk54(om_model* m, double* Q, double* dQ, double t0, double dt, int nsteps) {
    double time = t0;
    for (int i = 0; i < nsteps; ++i) {
        lsrk_step(*m, Q, dQ, time, dt);
        time += dt;
    }
}

// solve!(Q, lsrk; timeend) with adjustfinalstep, ODESolvers.jl:49-158.
// Returns the number of steps taken.
int om_solve(om_model* m, double* Q, double t0, double dt, double timeend) {
    size_t len = (size_t)m->nelem * NS * m->Np;
    std::vector<double> dQ(len, 0.0);
    double time = t0;
    int step = 0;
    while (time < timeend) {
        ++step;
        double h = dt;
        bool final_step = false;
        if (time + h > timeend) { h = timeend - time; final_step = true; }
        lsrk_step(*m, Q, dQ.data(), time, h);
        time = final_step ? timeend : time + h;
    }
    return step;
}

// Scalar ODE q' = q cos(t) integrated by the same LSRK54 coefficients and
// solve! loop (test/Numerics/ODESolvers/ode_tests_convergence.jl:15-44).
double om_lsrk54_scalar(double q0, double dt, double timeend) {
    double Q = q0, dQ = 0.0, time = 0.0;
    while (time < timeend) {
        double h = dt;
        bool final_step = false;
        if (time + h > timeend) { h = timeend - time; final_step = true; }
        for (int s = 0; s < 5; ++s) {
            dQ += Q * std::cos(time + RKC[s] * h);
            Q += RKB[s] * h * dQ;
            dQ *= RKA[(s + 1) % 5];
        }
        time = final_step ? timeend : time + h;
    }
    return Q;
}

// Weighted L2 norm sqrt(sum M Q^2), MPIStateArrays.jl:583-606
typedef struct Hevi om_hevi;

// AtmosAcousticGravityLinearModel tendency in VerticalDirection
void om_linear_tendency(om_model* m, double* dQ, const double* Q, double alpha, double beta) {
    linear_tendency(*m, dQ, Q, alpha, beta);
}

// ARK2GiraldoKellyConstantinescu(dg, lineardg, LinearBackwardEulerSolver(ManyColumnLU()), Q;
// dt, split_explicit_implicit, paperversion); NULL when the mesh has no wall-bounded stacks.
om_hevi* om_hevi_create(om_model* m, double dt, int split, int paperversion) {
    const int nv = stack_height(*m);
    if (nv <= 0 || m->law != 0 || m->prm.ref_state != 1) return nullptr;
    Hevi* h = new Hevi();
    h->m = m;
    h->dt = dt;
    h->split = split;
    h->nvert = nv;
    const double s2 = std::sqrt(2.0);
    const double a32 = paperversion ? (3 + 2 * s2) / 6 : 0.5;
    const double Ae[3][3] = {{0, 0, 0}, {2 - s2, 0, 0}, {1 - a32, a32, 0}};
    const double Ai[3][3] = {{0, 0, 0}, {1 - 1 / s2, 1 - 1 / s2, 0}, {1 / (2 * s2), 1 / (2 * s2), 1 - 1 / s2}};
    const double B[3] = {1 / (2 * s2), 1 / (2 * s2), 1 - 1 / s2}, C[3] = {0, 2 - s2, 1};
    std::memcpy(h->Ae, Ae, sizeof(Ae));
    std::memcpy(h->Ai, Ai, sizeof(Ai));
    std::memcpy(h->B, B, sizeof(B));
    std::memcpy(h->C, C, sizeof(C));
    h->alpha = dt * h->Ai[1][1];
    const size_t len = (size_t)m->nelem * NS * m->Np;
    for (auto* v : {&h->S1, &h->S2, &h->R0, &h->R1, &h->R2, &h->Qhat, &h->Qtt}) v->assign(len, 0.0);
    try {
        hevi_factorize(*h);
    } catch (const std::exception&) {
        delete h;
        return nullptr;
    }
    return h;
}

void om_hevi_free(om_hevi* h) { delete h; }

// besolver!(Q, Qhat, alpha): Q = Qhat + alpha L(Q) by the factorization
void om_hevi_solve(om_hevi* h, double* Q, const double* Qhat) { hevi_solve(*h, Q, Qhat); }

double om_hevi_alpha(const om_hevi* h) { return h->alpha; }
int om_hevi_bandwidth(const om_hevi* h) { return h->bw; }

void om_hevi_step(om_hevi* h, double* Q, double t0, int nsteps) {
    for (int i = 0; i < nsteps; ++i) hevi_step(*h, Q, t0 + i * h->dt);
}

double om_norm(const om_model* m, const double* Q) {
    double acc = 0;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int s = 0; s < NS; ++s)
            for (int n = 0; n < m->Np; ++n) {
                double q = Q[(e * NS + s) * m->Np + n];
                acc += VGc(*m, e, VM, n) * q * q;
            }
    return std::sqrt(acc);
}

// euclidean_distance (MPIStateArrays.jl:628-648)
double om_euclidean_distance(const om_model* m, const double* A, const double* B) {
    double acc = 0;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int s = 0; s < NS; ++s)
            for (int n = 0; n < m->Np; ++n) {
                size_t i = (size_t)(e * NS + s) * m->Np + n;
                double d = A[i] - B[i];
                acc += d * d * VGc(*m, e, VM, n);
            }
    return std::sqrt(acc);
}

// Per-field weighted L2 of A-B and of B (for relative errors)
void om_field_l2(const om_model* m, const double* A, const double* B, double* err, double* ref) {
    for (int s = 0; s < NS; ++s) { err[s] = 0; ref[s] = 0; }
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int s = 0; s < NS; ++s)
            for (int n = 0; n < m->Np; ++n) {
                size_t i = (size_t)(e * NS + s) * m->Np + n;
                double M = VGc(*m, e, VM, n);
                double d = A[i] - B[i];
                err[s] += d * d * M;
                ref[s] += B[i] * B[i] * M;
            }
    for (int s = 0; s < NS; ++s) { err[s] = std::sqrt(err[s]); ref[s] = std::sqrt(ref[s]); }
}

// weightedsum (compensated), MPIStateArrays.jl:655-675
double om_weightedsum(const om_model* m, const double* Q, int field) {
    DD acc;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int n = 0; n < m->Np; ++n) dd_add_prod(acc, Q[(e * NS + field) * m->Np + n], VGc(*m, e, VM, n));
    return acc.hi + acc.lo;
}

// Pointwise nondiffusive Courant number max over nodes with dt = 1
// (SpaceDiscretization.jl:307-365, Atmos/Model/courant.jl, Grids.jl:1228-1334);
// calculate_dt = CFL / max (DGMethods.jl:79-83).
double om_courant_dt(const om_model* m, const double* Q, double CFL) {
    int Nq = m->Nq, Np = m->Np;
    double cmax = -INFINITY;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int k = 0; k < Nq; ++k)
            for (int j = 0; j < Nq; ++j)
                for (int i = 0; i < Nq; ++i) {
                    int ijk = i + Nq * (j + Nq * k);
                    double x[3] = {VGc(*m, e, VX1, ijk), VGc(*m, e, VX2, ijk), VGc(*m, e, VX3, ijk)};
                    double md = INFINITY;
                    auto nd = [&](int ii, int jj, int kk) {
                        int o = ii + Nq * (jj + Nq * kk);
                        double dx = x[0] - VGc(*m, e, VX1, o), dy = x[1] - VGc(*m, e, VX2, o), dz = x[2] - VGc(*m, e, VX3, o);
                        md = std::min(md, std::sqrt(dx * dx + dy * dy + dz * dz));
                    };
                    if (i > 0) nd(i - 1, j, k);
                    if (i < Nq - 1) nd(i + 1, j, k);
                    if (j > 0) nd(i, j - 1, k);
                    if (j < Nq - 1) nd(i, j + 1, k);
                    if (k > 0) nd(i, j, k - 1);
                    if (k < Nq - 1) nd(i, j, k + 1);
                    double q[NS];
                    load_q(*m, Q, e, ijk, q);
                    double u[3] = {q[1] / q[0], q[2] / q[0], q[3] / q[0]};
                    double nu = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                    Thermo t = phase_dry(m->prm, q[0], q[4], q + 1, AUXc(*m, e, APHI, ijk));
                    double c = 1.0 * (nu + soundspeed(m->prm, t.T)) / md;
                    cmax = std::max(cmax, c);
                }
    return CFL / cmax;
}

// Isentropic vortex initial condition,
// test/Numerics/DGMethods/Euler/isentropicvortex_setup.jl:1-62
void om_init_vortex(const om_model* m, double* Q, double t, double p_inf, double T_inf, double translation_speed,
                    double translation_angle, double vortex_speed, double R, double L) {
    const om_params& p = m->prm;
    double rho_inf = p_inf / (p.R_d * T_inf);
    double kappa = p.R_d / p.cp_d;
    double uinf[3] = {translation_speed * std::cos(translation_angle), translation_speed * std::sin(translation_angle), 0};
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int n = 0; n < m->Np; ++n) {
            double x[3] = {VGc(*m, e, VX1, n), VGc(*m, e, VX2, n), VGc(*m, e, VX3, n)};
            for (int d = 0; d < 3; ++d) {
                x[d] -= uinf[d] * t;
                x[d] -= std::floor((x[d] + L) / (2 * L)) * (2 * L);
            }
            double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
            double du_x = -vortex_speed * x[1] / R * std::exp(-((r / R) * (r / R)) / 2);
            double du_y = vortex_speed * x[0] / R * std::exp(-((r / R) * (r / R)) / 2);
            double u[3] = {uinf[0] + du_x, uinf[1] + du_y, uinf[2] + 0};
            double T = T_inf * (1 - kappa * (vortex_speed * vortex_speed) / 2 * rho_inf / p_inf * std::exp(-((r / R) * (r / R))));
            double pres = p_inf * std::pow(T / T_inf, 1.0 / kappa);
            double rho = pres / (p.R_d * T);
            double e_kin = (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / 2;
            double* q = Q;
            q[(e * NS + 0) * m->Np + n] = rho;
            for (int c = 0; c < 3; ++c) q[(e * NS + 1 + c) * m->Np + n] = rho * u[c];
            q[(e * NS + 4) * m->Np + n] = rho * ((e_kin + 0.0) + p.cv_d * (T - p.T_0));
        }
}

// Rising thermal bubble about a hydrostatic background of potential
// temperature theta0 (experiments/TestCase/risingbubble.jl:23-91, with a
// cos^2 bump): theta = theta0 + A cos^2(pi r / (2 rc)) for r <= rc.
void om_init_bubble(const om_model* m, double* Q, double theta0, double amp, double rc, double xc, double yc,
                    double zc) {
    const om_params& p = m->prm;
    double R = p.R_d, cp = p.cp_d, cv = p.cv_d;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int n = 0; n < m->Np; ++n) {
            double x = VGc(*m, e, VX1, n), y = VGc(*m, e, VX2, n), z = VGc(*m, e, VX3, n);
            double r = std::sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc) + (z - zc) * (z - zc));
            double dth = 0;
            if (r <= rc) {
                double c = std::cos(M_PI * r / (2 * rc));
                dth = amp * c * c;
            }
            double th = theta0 + dth;
            double pi_ex = 1.0 - p.grav / (cp * th) * z;
            double rho = p.MSLP / (R * th) * std::pow(pi_ex, cv / R);
            double T = th * pi_ex;
            double e_pot = AUXc(*m, e, APHI, n);
            Q[(e * NS + 0) * m->Np + n] = rho;
            for (int c = 1; c < 4; ++c) Q[(e * NS + c) * m->Np + n] = 0;
            Q[(e * NS + 4) * m->Np + n] = rho * ((0.0 + e_pot) + cv * (T - p.T_0));
        }
}

// ----------------------------------------------------------------------------
// Filters (src/Numerics/Mesh/Filters.jl).
// ----------------------------------------------------------------------------
// spectral_filter_matrix (Filters.jl:114-128): W = V diag(Sigma) V^-1 with V
// the orthonormal Legendre polynomials at the LGL points (GaussQuadrature
// orthonormal_poly: P~_n = sqrt((2n+1)/2) P_n) and Sigma_n = 1 for n < Nc,
// sigma((n - Nc)/(N - Nc)) for n >= Nc.  kind 0 = ExponentialFilter
// (sigma = exp(-alpha eta^s), :172-213), 1 = CutoffFilter (sigma = 0,
// :275-306), 2 = BoydVandevenFilter (sigma = erfc(sqrt(s) chi a)/2,
// a = 2|eta| - 1, chi = sqrt(-log1p(-a^2)/a^2) or 1, :231-269).  W is written
// row-major: W[i*Nq + n] multiplies node n for output node i.
int om_filter_matrix(int N, int kind, int Nc, int s, double alpha, double* W) {
    if (N < 1 || Nc < 0 || Nc > N) return -1;
    const int Nq = N + 1;
    std::vector<double> r, w;
    lgl(N, r, w);
    std::vector<double> V((size_t)Nq * Nq), Sig(Nq, 1.0);
    for (int i = 0; i < Nq; ++i) {
        double p0 = 1.0, p1 = r[i];
        for (int n = 0; n < Nq; ++n) {
            double pn;
            if (n == 0) pn = 1.0;
            else if (n == 1) pn = r[i];
            else {
                pn = ((2 * n - 1) * r[i] * p1 - (n - 1) * p0) / n;
                p0 = p1;
                p1 = pn;
            }
            V[(size_t)i * Nq + n] = std::sqrt((2.0 * n + 1) / 2) * pn;
        }
    }
    for (int n = Nc; n <= N; ++n) {
        const double eta = (N == Nc) ? 0.0 : (double)(n - Nc) / (N - Nc);
        double sg;
        if (kind == 0) sg = std::exp(-alpha * std::pow(eta, s));
        else if (kind == 1) sg = 0.0;
        else {
            const double a = 2 * std::fabs(eta) - 1;
            const double chi = (a == 0) ? 1.0 : std::sqrt(-std::log1p(-a * a) / (a * a));
            sg = std::erfc(std::sqrt((double)s) * chi * a) / 2;
        }
        Sig[n] = sg;
    }
    // W = V diag(Sig) V^-1: solve W V = V diag(Sig) row by row (Gauss-Jordan on V^T)
    std::vector<double> A((size_t)Nq * Nq), B((size_t)Nq * Nq);
    for (int i = 0; i < Nq; ++i)
        for (int j = 0; j < Nq; ++j) {
            A[(size_t)i * Nq + j] = V[(size_t)j * Nq + i];            // V^T
            B[(size_t)i * Nq + j] = V[(size_t)j * Nq + i] * Sig[i];   // (V diag Sig)^T
        }
    // solve V^T W^T = (V diag Sig)^T with partial pivoting
    for (int c = 0; c < Nq; ++c) {
        int piv = c;
        for (int i = c + 1; i < Nq; ++i)
            if (std::fabs(A[(size_t)i * Nq + c]) > std::fabs(A[(size_t)piv * Nq + c])) piv = i;
        for (int j = 0; j < Nq; ++j) {
            std::swap(A[(size_t)c * Nq + j], A[(size_t)piv * Nq + j]);
            std::swap(B[(size_t)c * Nq + j], B[(size_t)piv * Nq + j]);
        }
        const double d = A[(size_t)c * Nq + c];
        for (int j = 0; j < Nq; ++j) {
            A[(size_t)c * Nq + j] /= d;
            B[(size_t)c * Nq + j] /= d;
        }
        for (int i = 0; i < Nq; ++i) {
            if (i == c) continue;
            const double f = A[(size_t)i * Nq + c];
            if (f == 0) continue;
            for (int j = 0; j < Nq; ++j) {
                A[(size_t)i * Nq + j] -= f * A[(size_t)c * Nq + j];
                B[(size_t)i * Nq + j] -= f * B[(size_t)c * Nq + j];
            }
        }
    }
    for (int i = 0; i < Nq; ++i)
        for (int j = 0; j < Nq; ++j) W[(size_t)i * Nq + j] = B[(size_t)j * Nq + i];
    return 0;
}

// kernel_apply_filter! (Filters.jl:651-790) through apply_async!
// (:440-505): horizontal pass (xi1 then xi2 with Wh) then vertical pass (xi3
// with Wv), each a sum over the line in place; direction 0 = every,
// 1 = horizontal, 2 = vertical; fields: the filtered state indices.
void om_apply_filter(const om_model* m, double* Q, const double* Wh, const double* Wv, int direction,
                     const int* fields, int nfields) {
    const int Nq = m->Nq, Np = m->Np;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->nelem; ++e) {
        std::vector<double> a(Np), b(Np);
        for (int fi = 0; fi < nfields; ++fi) {
            double* q = Q + ((size_t)e * NS + fields[fi]) * Np;
            for (int n = 0; n < Np; ++n) a[n] = q[n];
            auto pass = [&](const double* W, int d) {
                for (int k = 0; k < Nq; ++k)
                    for (int j = 0; j < Nq; ++j)
                        for (int i = 0; i < Nq; ++i) {
                            const int ijk = i + Nq * (j + Nq * k);
                            const int row = d == 0 ? i : (d == 1 ? j : k);
                            double acc = 0;
                            for (int n = 0; n < Nq; ++n) {
                                const int src = d == 0 ? n + Nq * (j + Nq * k)
                                                       : (d == 1 ? i + Nq * (n + Nq * k) : i + Nq * (j + Nq * n));
                                acc += W[row * Nq + n] * a[src];
                            }
                            b[ijk] = acc;
                        }
                a.swap(b);
            };
            if (direction == 0 || direction == 1) {
                pass(Wh, 0);
                pass(Wh, 1);
            }
            if (direction == 0 || direction == 2) pass(Wv, 2);
            for (int n = 0; n < Np; ++n) q[n] = a[n];
        }
    }
}

// MassPreservingCutoffFilter (Filters.jl:316-345, 542-606, 895-1065): one
// pass per direction class (horizontal: xi1 then xi2 with Wh; vertical: xi3
// with Wv; both for every direction, horizontal first), each followed by
// the shift that restores the element's mass-weighted integral of every
// filtered field: q += (sum M q_before - sum M q_after) / sum M.
void om_apply_mp_filter(const om_model* m, double* Q, const double* Wh, const double* Wv, int direction,
                        const int* fields, int nfields) {
    const int Nq = m->Nq, Np = m->Np;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->nelem; ++e) {
        std::vector<double> a(Np), b(Np);
        double Ms = 0;
        for (int n = 0; n < Np; ++n) Ms += VGc(*m, e, VM, n);
        for (int pass = 0; pass < 2; ++pass) {
            const bool horiz = pass == 0;
            if (horiz && direction == 2) continue;
            if (!horiz && direction == 1) continue;
            for (int fi = 0; fi < nfields; ++fi) {
                double* q = Q + ((size_t)e * NS + fields[fi]) * Np;
                double before = 0;
                for (int n = 0; n < Np; ++n) {
                    a[n] = q[n];
                    before += VGc(*m, e, VM, n) * q[n];
                }
                auto sweep = [&](const double* W, int d) {
                    for (int k = 0; k < Nq; ++k)
                        for (int j = 0; j < Nq; ++j)
                            for (int i = 0; i < Nq; ++i) {
                                const int ijk = i + Nq * (j + Nq * k);
                                const int row = d == 0 ? i : (d == 1 ? j : k);
                                double acc = 0;
                                for (int n = 0; n < Nq; ++n) {
                                    const int src = d == 0 ? n + Nq * (j + Nq * k)
                                                           : (d == 1 ? i + Nq * (n + Nq * k) : i + Nq * (j + Nq * n));
                                    acc += W[row * Nq + n] * a[src];
                                }
                                b[ijk] = acc;
                            }
                    a.swap(b);
                };
                if (horiz) {
                    sweep(Wh, 0);
                    sweep(Wh, 1);
                } else {
                    sweep(Wv, 2);
                }
                double after = 0;
                for (int n = 0; n < Np; ++n) after += VGc(*m, e, VM, n) * a[n];
                const double Minv = 1 / Ms;
                for (int n = 0; n < Np; ++n) q[n] = a[n] + Minv * (before - after);
            }
        }
    }
}

// TMARFilter, kernel_apply_TMAR_filter! (Filters.jl:794-892): per element
// and field, r = sum(M q) / sum(M max(q, 0)) (0 when sum(M q) <= 0) and
// q <- r q where q >= 0, 0 elsewhere.
void om_apply_tmar(const om_model* m, double* Q, const int* fields, int nfields) {
    const int Np = m->Np;
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int fi = 0; fi < nfields; ++fi) {
            double* q = Q + ((size_t)e * NS + fields[fi]) * Np;
            double MJQ = 0, MJQc = 0;
            for (int n = 0; n < Np; ++n) {
                const double M = VGc(*m, e, VM, n);
                MJQ += M * q[n];
                MJQc += M * (q[n] >= 0 ? q[n] : 0.0);
            }
            const double r = MJQ > 0 ? MJQ / MJQc : 0.0;
            for (int n = 0; n < Np; ++n) q[n] = q[n] >= 0 ? r * q[n] : 0.0;
        }
}

// Rest state equal to the reference state (discrete_hydrostatic_balance.jl:25-30)
void om_init_rest(const om_model* m, double* Q) {
    for (int64_t e = 0; e < m->nelem; ++e)
        for (int n = 0; n < m->Np; ++n) {
            Q[(e * NS + 0) * m->Np + n] = AUXc(*m, e, ARHO_REF, n);
            for (int c = 1; c < 4; ++c) Q[(e * NS + c) * m->Np + n] = 0;
            Q[(e * NS + 4) * m->Np + n] = AUXc(*m, e, ARHOE_REF, n);
        }
}

}  // extern "C"
