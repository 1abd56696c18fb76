// MOL (method-of-lines) advection of the predictor-corrector scheme: the
// face-normal velocities extrapolated before the MAC projection and the
// conservative convective term from upwinded, MC-limited face states.
//
// Restates MOL::ExtrapVelToFaces (AMReX-Hydro; called from
// src/equation_systems/icns/icns_advection.H:501-527) and
// mol::compute_convective_fluxes / mol::compute_convective_rate
// (src/convection/incflo_mol_fluxes.cpp:9-268, driven by
// icns_advection.H:531-594 with q = rho u), with AMReX's order-2
// monotonized-central slopes (amrex_calc_{x,y,z}slope and their _extdir forms).
//
// Every face state is computed once: one thread per face forms the two
// one-sided states of all three components, the divergence pass reads the
// nine face-flux arrays and, in the predictor, also forms predictor_rhs.
#include <cfloat>

#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

// MC slope of a cell from its two neighbours.  edge = -1 / +1 marks the cell
// next to a low / high ext_dir or hoextrap domain face, whose ghost holds the
// face value: the central difference becomes the one-sided quadratic
// (q+ + 3 q0 - 4 qb)/3 or (4 qb - 3 q0 - q-)/3.
__device__ inline double mc_slope(double qm, double q0, double qp, int edge) {
    const double dl = 2.0 * (q0 - qm), dr = 2.0 * (qp - q0);
    double dc = 0.5 * (qp - qm);
    if (edge < 0) dc = (qp + 3.0 * q0 - 4.0 * qm) / 3.0;
    else if (edge > 0) dc = (4.0 * qp - 3.0 * q0 - qm) / 3.0;
    double s = fmin(fabs(dl), fmin(fabs(dc), fabs(dr)));
    if (!(dr * dl > 0.0)) s = 0.0;
    return dc > 0.0 ? s : -s;
}

// Every velocity component is ext_dir (normal) or hoextrap (tangential) at a
// z wall, so the one-sided slope applies in the first and last cell layers.
__device__ inline int z_edge(const Grid& g, int d, int k) {
    if (d != 2 || g.zper) return 0;
    return k == 0 ? -1 : (k == g.nz - 1 ? 1 : 0);
}

// States of component n on the d-face at the low side of cell (i, j, k):
// qmns extrapolated from the cell below, qpls from the cell above.
__device__ inline void mol_states(const VelFP& q, const Grid& g, int d, int n, int i, int j, int k, double& qmns, double& qpls) {
    const int e0 = d == 0, e1 = d == 1, e2 = d == 2;
    const double a = q(n, i - 2 * e0, j - 2 * e1, k - 2 * e2);
    const double b = q(n, i - e0, j - e1, k - e2);
    const double c = q(n, i, j, k);
    const double e = q(n, i + e0, j + e1, k + e2);
    const int kd = d == 0 ? i : (d == 1 ? j : k);
    qmns = b + 0.5 * mc_slope(a, b, c, z_edge(g, d, kd - 1));
    qpls = c - 0.5 * mc_slope(b, c, e, z_edge(g, d, kd));
}

// ExtrapVelToFaces choice: zero where the states diverge or their mean is
// below small_vel = 1e-10, else the upwind state
__device__ inline double mol_pick(double umns, double upls) {
    if (umns < 0.0 && upls > 0.0) return 0.0;
    const double avg = 0.5 * (upls + umns);
    if (fabs(avg) < 1.0e-10) return 0.0;
    return avg >= 0.0 ? umns : upls;
}

// One thread per (i, j, k) of the z-face layers: the x, y and z faces at the
// low side of the cell (z walls: the face takes the ghost value 0).
__global__ void k_mol_extrap(Grid g, const double* vel, double* um, double* vm, double* wm) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long M = (long long)g.nx * g.ny * nzfaces(g);
    if (t >= M) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const VelFP V{vel, g, 1.0};
    double mn, pl;
    if (k < g.nz) {
        mol_states(V, g, 0, 0, i, j, k, mn, pl);
        um[t] = mol_pick(mn, pl);
        mol_states(V, g, 1, 1, i, j, k, mn, pl);
        vm[t] = mol_pick(mn, pl);
    }
    if (!g.zper && (k == 0 || k == g.nz)) {
        wm[t] = 0.0;
    } else {
        mol_states(V, g, 2, 2, i, j, k, mn, pl);
        wm[t] = mol_pick(mn, pl);
    }
}

__device__ inline bool face_cell(const Grid& g, int d, long long t, int& i, int& j, int& k) {
    const long long M = (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz);
    if (t >= M) return false;
    i = (int)(t % g.nx);
    const long long r = t / g.nx;
    j = (int)(r % g.ny);
    k = (int)(r / g.ny);
    return true;
}

// Fluxes of rho u through the d-faces: the MC-limited states upwinded with
// the MAC velocity (their mean where |u_mac| <= FLT_EPSILON); on a z wall the
// normal component takes the ghost (boundary) value 0.
__global__ void k_mol_flux(Grid g, int d, const double* vel, const double* mac, double rho, double* F0, double* F1, double* F2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_cell(g, d, t, i, j, k)) return;
    const VelFP Q{vel, g, rho};
    const double u = mac[t];
    const double small_vel = (double)FLT_EPSILON;
    const bool wall = d == 2 && !g.zper && (k == 0 || k == g.nz);
    double* F[3] = {F0, F1, F2};
    for (int n = 0; n < 3; ++n) {
        double qs = 0.0;
        if (!(wall && n == 2)) {
            double mn, pl;
            mol_states(Q, g, d, n, i, j, k, mn, pl);
            qs = u > small_vel ? mn : (u < -small_vel ? pl : 0.5 * (mn + pl));
        }
        F[n][t] = qs * u;
    }
}

struct MolFlux {
    const double* p[9];
};

// conv = sum_d dxinv_d (F_lo - F_hi); mode 1 also forms predictor_rhs with
// fstate Old: vel = (rho u_old + dt (conv + src + divtau_old)) / rho
__global__ void k_mol_div(Grid g, MolFlux F, double* conv, int mode, const double* vo, const double* src, const double* dold,
                          double* vel, double dt, double rho) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long xp = fidx(g, 0, i + 1, j, k), yp = fidx(g, 1, i, j + 1, k);
    const long long zm = fidx(g, 2, i, j, k), zp = fidx(g, 2, i, j, k + 1);
    const long long N = g.N;
    for (int n = 0; n < 3; ++n) {
        const double c = (g.idx * (F.p[n][t] - F.p[n][xp])) + (g.idy * (F.p[3 + n][t] - F.p[3 + n][yp])) +
                         (g.idz * (F.p[6 + n][zm] - F.p[6 + n][zp]));
        conv[n * N + t] = c;
        if (mode == 1) vel[n * N + t] = (rho * vo[n * N + t] + dt * (c + src[n * N + t] + dold[n * N + t])) * (1.0 / rho);
    }
}

inline long long nfaces_d(const Grid& g, int d) { return (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz); }

}  // namespace

void launch_mol_extrap(Ctx& c, const Grid& g, const double* vel, double* const mac[3]) {
    const long long M = (long long)g.nx * g.ny * nzfaces(g);
    KS_LAUNCH(c, k_mol_extrap, nblocks(M, BS), BS, 8.0 * (3.0 * g.N + 2.0 * g.N + M), g, vel, mac[0], mac[1], mac[2]);
}

void launch_mol_advection(Ctx& c, const Grid& g, const double* vel, const double* const mac[3], double rho, double* const fl[9],
                          double* conv, int mode, const double* vel_old, const double* src, const double* dold, double* vel_out,
                          double dt) {
    for (int d = 0; d < 3; ++d) {
        const double nf = (double)nfaces_d(g, d);
        KS_LAUNCH(c, k_mol_flux, nblocks(nfaces_d(g, d), BS), BS, 8.0 * (3.0 * g.N + 4.0 * nf), g, d, vel, mac[d], rho, fl[3 * d],
                  fl[3 * d + 1], fl[3 * d + 2]);
    }
    MolFlux F;
    for (int m = 0; m < 9; ++m) F.p[m] = fl[m];
    const double nfz = (double)nfaces_d(g, 2);
    const double bytes = 8.0 * (6.0 * g.N + 3.0 * nfz + 3.0 * g.N + (mode == 1 ? 12.0 * g.N : 0.0));
    KS_LAUNCH(c, k_mol_div, nblocks(g.N, BS), BS, bytes, g, F, conv, mode, vel_old, src, dold, vel_out, dt, rho);
}

}  // namespace ks
