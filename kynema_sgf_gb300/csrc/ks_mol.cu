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
// FP64 issue is the bound, so every cell's slope is computed once per
// component (a few more at segment ends) and every face state once: the x-face
// kernel passes slopes between neighbouring lanes of a warp, the y- and z-face
// kernels march along columns.
// The divergence pass reads the nine face-flux arrays and, in the predictor,
// also forms predictor_rhs.
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

// ExtrapVelToFaces choice: zero where the states diverge or their mean is
// below small_vel = 1e-10, else the upwind state
__device__ inline double mol_pick(double umns, double upls) {
    if (umns < 0.0 && upls > 0.0) return 0.0;
    const double avg = 0.5 * (upls + umns);
    if (fabs(avg) < 1.0e-10) return 0.0;
    return avg >= 0.0 ? umns : upls;
}

// compute_convective_fluxes choice: the upwind state, the mean of both where
// |u_mac| <= small_vel = FLT_EPSILON
__device__ inline double mol_upwind(double u, double qmns, double qpls) {
    const double small_vel = (double)FLT_EPSILON;
    return u > small_vel ? qmns : (u < -small_vel ? qpls : 0.5 * (qmns + qpls));
}

__device__ inline double* pick3(int n, double* a, double* b, double* c) { return n == 0 ? a : (n == 1 ? b : c); }

// The face kernels come in three kinds: KIND 0 extrapolates the normal velocity
// component d of u to the d-faces (ExtrapVelToFaces, written to mac); KIND 1
// forms the fluxes of rho u (three components, upwinded with mac) through
// them; KIND 2 the fluxes of rho s for a cell scalar s (AdvOp_MOL.H:38-118),
// hoextrap at z walls like a tangential component.  Each computes the MC slope of every cell once per component: the
// x kernel takes the slope of cell i - 1 from the neighbouring lane of its warp,
// the y and z kernels march along a column of MOL_CHUNK faces and carry it.

// x faces: each warp covers 31 consecutive faces of one x row.  Lane l forms
// the slope of cell i = 31 s + l - 1 (s: the warp's segment of the row);
// lanes 1..31 take the slope of cell i - 1 from the lane below and form face i.
// Every lane does the same work, so no lane's extra slope stalls the others.
constexpr int XSEG = 31;
template <int KIND>
__global__ void k_mol_x(Grid g, const double* vel, double rho, const double* mac, double* o0, double* o1, double* o2) {
    const int nseg = (g.nx + XSEG - 1) / XSEG;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long rows = (long long)g.ny * g.nz;
    if (w >= rows * nseg) return;  // whole warps leave together
    const long long row = w / nseg;
    const int i = (int)(w % nseg) * XSEG + lane - 1;
    const int j = (int)(row % g.ny), k = (int)(row / g.ny);
    const bool face = lane > 0 && i < g.nx;
    const int ic = min(i, g.nx - 1);  // lanes past the row end read in range and write nothing
    const long long t = ((long long)k * g.ny + j) * g.nx + (face ? i : 0);
    const VelFP Q{vel, g, KIND ? rho : 1.0};
    const double u = (KIND && face) ? mac[t] : 0.0;
    constexpr int nend = KIND == 1 ? 3 : 1;
    for (int n = 0; n < nend; ++n) {
        const double b = Q(n, ic - 1, j, k), c = Q(n, ic, j, k), e = Q(n, ic + 1, j, k);
        const double s0 = mc_slope(b, c, e, 0);
        const double sm = __shfl_up_sync(0xffffffffu, s0, 1);
        if (!face) continue;
        const double qmns = b + 0.5 * sm, qpls = c - 0.5 * s0;
        if (KIND == 0) o0[t] = mol_pick(qmns, qpls);
        else pick3(n, o0, o1, o2)[t] = mol_upwind(u, qmns, qpls) * u;
    }
}

constexpr int MOL_CHUNK = 16;

// y faces: one thread per (i, k, chunk of MOL_CHUNK faces along y)
template <int KIND>
__global__ void k_mol_y(Grid g, const double* vel, double rho, const double* mac, double* o0, double* o1, double* o2) {
    const int nch = (g.ny + MOL_CHUNK - 1) / MOL_CHUNK;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.nx * g.nz * nch) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int k = (int)(r % g.nz), ch = (int)(r / g.nz);
    const int j0 = ch * MOL_CHUNK, j1 = min(j0 + MOL_CHUNK, g.ny);
    const VelFP Q{vel, g, KIND ? rho : 1.0};
    const int nbeg = KIND == 0 ? 1 : 0, nend = KIND == 0 ? 2 : (KIND == 1 ? 3 : 1);
    for (int n = nbeg; n < nend; ++n) {
        double qb = Q(n, i, j0 - 1, k), qc = Q(n, i, j0, k);
        double sb = mc_slope(Q(n, i, j0 - 2, k), qb, qc, 0);
        for (int j = j0; j < j1; ++j) {
            const double qe = Q(n, i, j + 1, k);
            const double sc = mc_slope(qb, qc, qe, 0);
            const double qmns = qb + 0.5 * sb, qpls = qc - 0.5 * sc;
            const long long f = cidx(g, i, j, k);
            if (KIND == 0) o0[f] = mol_pick(qmns, qpls);
            else pick3(n, o0, o1, o2)[f] = mol_upwind(mac[f], qmns, qpls) * mac[f];
            qb = qc;
            qc = qe;
            sb = sc;
        }
    }
}

// z faces: one thread per (i, j, chunk of MOL_CHUNK face layers); on a wall
// face the normal component takes the ghost (boundary) value 0
template <int KIND>
__global__ void k_mol_z(Grid g, const double* vel, double rho, const double* mac, double* o0, double* o1, double* o2) {
    const int nzf = nzfaces(g);
    const int nch = (nzf + MOL_CHUNK - 1) / MOL_CHUNK;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.nx * g.ny * nch) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), ch = (int)(r / g.ny);
    const int k0 = ch * MOL_CHUNK, k1 = min(k0 + MOL_CHUNK, nzf);
    const VelFP Q{vel, g, KIND ? rho : 1.0};
    const int nbeg = KIND == 0 ? 2 : 0, nend = KIND == 2 ? 1 : 3;
    for (int n = nbeg; n < nend; ++n) {
        double qb = Q(n, i, j, k0 - 1), qc = Q(n, i, j, k0);
        double sb = mc_slope(Q(n, i, j, k0 - 2), qb, qc, z_edge(g, 2, k0 - 1));
        for (int k = k0; k < k1; ++k) {
            const double qe = Q(n, i, j, k + 1);
            const double sc = mc_slope(qb, qc, qe, z_edge(g, 2, k));
            const double qmns = qb + 0.5 * sb, qpls = qc - 0.5 * sc;
            const long long f = fidx(g, 2, i, j, k);
            const bool wall = !g.zper && (k == 0 || k == g.nz);
            if (KIND == 0) {
                o0[f] = wall ? 0.0 : mol_pick(qmns, qpls);
            } else {
                const double u = mac[f];
                pick3(n, o0, o1, o2)[f] = ((wall && n == 2) ? 0.0 : mol_upwind(u, qmns, qpls)) * u;
            }
            qb = qc;
            qc = qe;
            sb = sc;
        }
    }
}

struct MolFlux {
    const double* p[9];
};

// conv = sum_d dxinv_d (F_lo - F_hi); mode 1 also forms predictor_rhs with
// fstate Old, vel = (rho u_old + dt (conv + src + fac divtau_old)) / rho; mode 2
// corrector_rhs without the new diffusion term (Crank-Nicolson / implicit),
// vel = (rho u_old + dt (0.5 (conv_old + conv) + fac divtau_old + src)) / rho
__global__ void k_mol_div(Grid g, MolFlux F, int nc, double* conv, int mode, const double* vo, const double* src, const double* dold,
                          const double* conv_o, double* vel, double dt, double rho, double fac, double irho) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const unsigned ut = (unsigned)t, r = ut / (unsigned)g.nx;
    const int i = (int)(ut - r * (unsigned)g.nx);
    const int k = (int)(r / (unsigned)g.ny), j = (int)(r - (unsigned)k * (unsigned)g.ny);
    const long long xp = fidx(g, 0, i + 1, j, k), yp = fidx(g, 1, i, j + 1, k);
    const long long zm = fidx(g, 2, i, j, k), zp = fidx(g, 2, i, j, k + 1);
    const long long N = g.N;
    for (int n = 0; n < nc; ++n) {
        const double c = (g.idx * (F.p[n][t] - F.p[n][xp])) + (g.idy * (F.p[3 + n][t] - F.p[3 + n][yp])) +
                         (g.idz * (F.p[6 + n][zm] - F.p[6 + n][zp]));
        conv[n * N + t] = c;
        const long long m = n * N + t;
        if (mode == 1) vel[m] = (rho * vo[m] + dt * (c + src[m] + fac * dold[m])) * irho;
        else if (mode == 2) vel[m] = (rho * vo[m] + dt * (0.5 * (conv_o[m] + c) + fac * dold[m] + src[m])) * irho;
    }
}

inline long long nfaces_d(const Grid& g, int d) { return (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz); }

}  // namespace

template <int KIND>
static void mol_faces(Ctx& c, const Grid& g, const double* vel, double rho, const double* const mac[3], double* const out[9]) {
    const double nc = KIND == 1 ? 3.0 : 1.0;  // components read and written per face
    const long long ty = (long long)g.nx * g.nz * ((g.ny + MOL_CHUNK - 1) / MOL_CHUNK);
    const long long tz = (long long)g.nx * g.ny * ((nzfaces(g) + MOL_CHUNK - 1) / MOL_CHUNK);
    const double nfz = (double)nfaces_d(g, 2);
    auto o = [&](int d, int n) { return out[KIND == 1 ? 3 * d + n : d]; };
    const double* m0 = KIND ? mac[0] : nullptr;
    const double* m1 = KIND ? mac[1] : nullptr;
    const double* m2 = KIND ? mac[2] : nullptr;
    const long long tx = 32LL * g.ny * g.nz * ((g.nx + XSEG - 1) / XSEG);
    KS_LAUNCH(c, k_mol_x<KIND>, nblocks(tx, BS), BS, 8.0 * (2.0 * nc + KIND) * g.N, g, vel, rho, m0, o(0, 0), o(0, 1), o(0, 2));
    KS_LAUNCH(c, k_mol_y<KIND>, nblocks(ty, BS), BS, 8.0 * (2.0 * nc + KIND) * g.N, g, vel, rho, m1, o(1, 0), o(1, 1), o(1, 2));
    KS_LAUNCH(c, k_mol_z<KIND>, nblocks(tz, BS), BS, 8.0 * (nc * g.N + (nc + KIND) * nfz), g, vel, rho, m2, o(2, 0), o(2, 1),
              o(2, 2));
}

void launch_mol_extrap(Ctx& c, const Grid& g, const double* vel, double* const mac[3]) {
    double* out[9] = {mac[0], mac[1], mac[2], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    mol_faces<0>(c, g, vel, 1.0, nullptr, out);
}

void launch_mol_advection(Ctx& c, const Grid& g, const double* vel, const double* const mac[3], double rho, double* const fl[9],
                          double* conv, int mode, const double* vel_old, const double* src, const double* dold, const double* conv_old,
                          double* vel_out, double dt, double fac) {
    mol_faces<1>(c, g, vel, rho, mac, fl);
    MolFlux F;
    for (int m = 0; m < 9; ++m) F.p[m] = fl[m];
    const double nfz = (double)nfaces_d(g, 2);
    const double bytes = 8.0 * (6.0 * g.N + 3.0 * nfz + 3.0 * g.N + (mode == 1 ? 12.0 * g.N : (mode == 2 ? 15.0 * g.N : 0.0)));
    KS_LAUNCH(c, k_mol_div, nblocks(g.N, BS), BS, bytes, g, F, 3, conv, mode, vel_old, src, dold, conv_old, vel_out, dt, rho, fac, 1.0 / rho);
}

void launch_mol_scalar_advection(Ctx& c, const Grid& g, const double* s, const double* const mac[3], double rho, double* const fl[3],
                                 double* conv) {
    double* out[9] = {fl[0], fl[1], fl[2], nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    mol_faces<2>(c, g, s, rho, mac, out);
    MolFlux F;
    for (int m = 0; m < 9; ++m) F.p[m] = nullptr;
    F.p[0] = fl[0];
    F.p[3] = fl[1];
    F.p[6] = fl[2];
    const double nfz = (double)nfaces_d(g, 2);
    KS_LAUNCH(c, k_mol_div, nblocks(g.N, BS), BS, 8.0 * (3.0 * g.N + nfz), g, F, 1, conv, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0,
              rho, 0.0, 1.0 / rho);
}

}  // namespace ks
