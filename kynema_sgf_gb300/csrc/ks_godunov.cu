// Godunov PPM advection: pre-MAC extrapolation of the normal face velocities
// and post-MAC conservative fluxes with their divergence.
//
// Restates the unsplit Godunov method with corner-transport corrections used
// by AMReX-Hydro (called from src/equation_systems/icns/icns_advection.H:
// 211-216 ExtrapVelToFaces, 359-373 ComputeFluxesOnBoxFromState, 418-422
// ComputeDivergence): Colella-Woodward PPM with van Leer limited edge values,
// traces over the characteristic domain of dependence, transverse terms with
// dt/6 (velocity form) or dt/3 (conservative form) corner factors, forces
// added after the transverse step, upwinding with AMReX-Hydro's small_vel.
//
// Each stage is one kernel over faces of one direction; intermediate face
// states live in HBM between stages.
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

__device__ inline double vls(double a, double b, double c) {
    const double dsc = 0.5 * (c - a), dsl = 2.0 * (b - a), dsr = 2.0 * (c - b);
    return (dsl * dsr > 0.0) ? copysign(fmin(fabs(dsc), fmin(fabs(dsl), fabs(dsr))), dsc) : 0.0;
}
__device__ inline double clipe(double e, double a, double b) { return fmin(fmax(e, fmin(a, b)), fmax(a, b)); }

// limited PPM edge values of the cell at q[2] (q[0..4] = cells c-2..c+2);
// zw = number of cells of a wall-bounded z line (else -1), c = cell index.
__device__ inline void ppm_edges(const double* q, int c, int zw, double& sm, double& sp) {
    const bool w = zw > 0;
    if (w && c == 0) sm = q[1];
    else if (w && c == 1) sm = clipe(-0.2 * q[0] + 0.75 * q[1] + 0.5 * q[2] - 0.05 * q[3], q[1], q[2]);
    else if (w && c == zw - 1) sm = clipe(-0.2 * q[3] + 0.75 * q[2] + 0.5 * q[1] - 0.05 * q[0], q[2], q[1]);
    else sm = clipe(0.5 * (q[1] + q[2]) - (1.0 / 6.0) * (vls(q[1], q[2], q[3]) - vls(q[0], q[1], q[2])), q[1], q[2]);
    if (w && c == zw - 1) sp = q[3];
    else if (w && c == zw - 2) sp = clipe(-0.2 * q[4] + 0.75 * q[3] + 0.5 * q[2] - 0.05 * q[1], q[3], q[2]);
    else if (w && c == 0) sp = clipe(-0.2 * q[1] + 0.75 * q[2] + 0.5 * q[3] - 0.05 * q[4], q[2], q[3]);
    else sp = clipe(0.5 * (q[2] + q[3]) - (1.0 / 6.0) * (vls(q[2], q[3], q[4]) - vls(q[1], q[2], q[3])), q[2], q[3]);
    const double s0 = q[2];
    if ((sp - s0) * (s0 - sm) <= 0.0) {
        sp = s0;
        sm = s0;
    } else if (fabs(sp - s0) >= 2.0 * fabs(sm - s0)) {
        sp = 3.0 * s0 - 2.0 * sm;
    } else if (fabs(sm - s0) >= 2.0 * fabs(sp - s0)) {
        sm = 3.0 * s0 - 2.0 * sp;
    }
}

struct FaceVel {  // face-centred advection velocities (post-MAC)
    const double* f[3];
};

// Trace of component n of cell (i,j,k) along d: the value on its high face
// (want_hi) or low face.  MODE 0 uses the cell velocity component d as the
// characteristic speed, MODE 1 the face velocities.
template <int MODE>
__device__ inline double cell_trace(const Grid& g, const VelFP& q, const VelFP& vc, const FaceVel& fv, int n, int d, int i, int j, int k,
                                    double dt, bool want_hi) {
    double a[5];
    for (int m = -2; m <= 2; ++m) a[m + 2] = q(n, i + (d == 0) * m, j + (d == 1) * m, k + (d == 2) * m);
    const int c = d == 0 ? i : (d == 1 ? j : k);
    const int zw = (d == 2 && !g.zper) ? g.nz : -1;
    double sm, sp;
    ppm_edges(a, c, zw, sm, sp);
    const double s0 = a[2];
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    const double dtdx = dt / hd(g, d);
    if (MODE == 0) {
        const double u = vc(d, i, j, k);
        const double sig = fabs(u) * dtdx;
        if (want_hi) return (u > kSmallVel) ? sp - 0.5 * sig * ((sp - sm) - (1.0 - 2.0 / 3.0 * sig) * s6) : s0;
        return (u < -kSmallVel) ? sm + 0.5 * sig * ((sp - sm) + (1.0 - 2.0 / 3.0 * sig) * s6) : s0;
    } else {
        if (want_hi) {
            const double up = fv.f[d][fidx(g, d, i + (d == 0), j + (d == 1), k + (d == 2))];
            const double sig = fabs(up) * dtdx;
            return (up > kSmallVel) ? sp - 0.5 * sig * ((sp - sm) - (1.0 - 2.0 / 3.0 * sig) * s6) : s0;
        }
        const double um = fv.f[d][fidx(g, d, i, j, k)];
        const double sig = fabs(um) * dtdx;
        return (um < -kSmallVel) ? sm + 0.5 * sig * ((sp - sm) + (1.0 - 2.0 / 3.0 * sig) * s6) : s0;
    }
}

// Wall face treatment (SetZEdgeBCs): tangential components take the interior
// state, the normal component is zero on both sides.
__device__ inline void zbc(const Grid& g, int k, int n, double& lo, double& hi) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) { lo = 0.0; hi = 0.0; } else lo = hi;
    } else if (k == g.nz) {
        if (n == 2) { lo = 0.0; hi = 0.0; } else hi = lo;
    }
}

// lo/hi states of component n on the d-face at the low side of cell (i,j,k)
template <int MODE>
__device__ inline void face_states(const Grid& g, const VelFP& q, const VelFP& vc, const FaceVel& fv, int n, int d, int i, int j, int k,
                                   double dt, double& lo, double& hi) {
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    lo = 0.0;
    hi = 0.0;
    if (!wl) lo = cell_trace<MODE>(g, q, vc, fv, n, d, i - (d == 0), j - (d == 1), k - (d == 2), dt, true);
    if (!wh) hi = cell_trace<MODE>(g, q, vc, fv, n, d, i, j, k, dt, false);
    if (d == 2) zbc(g, k, n, lo, hi);
}

__device__ inline double upwind(double vel, double lo, double hi) {
    const double st = (vel >= 0.0) ? lo : hi;
    const double fu = (fabs(vel) < kSmallVel) ? 0.0 : 1.0;
    return fu * st + (1.0 - fu) * 0.5 * (lo + hi);
}
__device__ inline double riemann(double lo, double hi) {
    const double st = (lo + hi >= 0.0) ? lo : hi;
    const bool ltm = (lo <= 0.0 && hi >= 0.0) || (fabs(lo + hi) < kSmallVel);
    return ltm ? 0.0 : st;
}

__device__ inline bool face_of(const Grid& g, int d, long long t, int& i, int& j, int& k) {
    const int nzl = (d == 2) ? nzfaces(g) : g.nz;
    const long long M = (long long)g.nx * g.ny * nzl;
    if (t >= M) return false;
    i = (int)(t % g.nx);
    const long long r = t / g.nx;
    j = (int)(r % g.ny);
    k = (int)(r / g.ny);
    return true;
}

inline long long nfaces(const Grid& g, int d) { return (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz); }

// ---- pre-MAC stage 1: advective velocities and upwinded transverse states
__global__ void k_pm_faces(Grid g, int d, const double* vel, double dt, double* ad, double* e1, double* e2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, 1.0};
    FaceVel fv{};
    double lo[3], hi[3];
    for (int n = 0; n < 3; ++n) face_states<0>(g, q, q, fv, n, d, i, j, k, dt, lo[n], hi[n]);
    const double a = riemann(lo[d], hi[d]);
    const long long f = fidx(g, d, i, j, k);
    ad[f] = a;
    const int n1 = (d + 1) % 3, n2 = (d + 2) % 3;
    e1[f] = upwind(a, lo[n1], hi[n1]);
    e2[f] = upwind(a, lo[n2], hi[n2]);
}

// ---- pre-MAC stage 2: a-face states of component n corrected along b
__global__ void k_pm_trans(Grid g, int a, int b, int n, const double* vel, double dt, const double* ad_a, const double* ad_b,
                           const double* edge_b, double* out) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    VelFP q{vel, g, 1.0};
    FaceVel fv{};
    double l, h;
    face_states<0>(g, q, q, fv, n, a, i, j, k, dt, l, h);
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    const double cb = dt / (6.0 * hd(g, b));
    const int eb0 = (b == 0), eb1 = (b == 1), eb2 = (b == 2);
    if (!wh) {
        const long long f0 = fidx(g, b, i, j, k), f1 = fidx(g, b, i + eb0, j + eb1, k + eb2);
        h -= cb * (ad_b[f1] + ad_b[f0]) * (edge_b[f1] - edge_b[f0]);
    }
    if (!wl) {
        const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
        const long long f0 = fidx(g, b, ci, cj, ck), f1 = fidx(g, b, ci + eb0, cj + eb1, ck + eb2);
        l -= cb * (ad_b[f1] + ad_b[f0]) * (edge_b[f1] - edge_b[f0]);
    }
    if (a == 2) zbc(g, k, n, l, h);
    const long long f = fidx(g, a, i, j, k);
    out[f] = upwind(ad_a[f], l, h);
}

// ---- pre-MAC stage 3: final normal velocity on d-faces
__global__ void k_pm_final(Grid g, int d, const double* vel, const double* forces, double dt, const double* ad0, const double* ad1,
                           const double* ad2, const double* T1, const double* T2, double* mac) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, 1.0};
    CellFO F{forces, g};
    FaceVel fv{};
    const double* ad[3] = {ad0, ad1, ad2};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const double c1 = dt / (4.0 * hd(g, b1)), c2 = dt / (4.0 * hd(g, b2));
    double lo, hi;
    face_states<0>(g, q, q, fv, d, d, i, j, k, dt, lo, hi);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    auto side = [&](int ci, int cj, int ck, double base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        double s = base;
        s -= c1 * (ad[b1][p1] + ad[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (ad[b2][p2] + ad[b2][m2]) * (T2[p2] - T2[m2]);
        s += 0.5 * dt * F(d, ci, cj, ck);
        return s;
    };
    double stl = 0.0, sth = 0.0;
    if (!wl) stl = side(i - (d == 0), j - (d == 1), k - (d == 2), lo);
    if (!wh) sth = side(i, j, k, hi);
    if (d == 2) zbc(g, k, d, stl, sth);
    mac[fidx(g, d, i, j, k)] = riemann(stl, sth);
}

// ---- post-MAC stage 1: upwinded states of all components on a-faces
__global__ void k_adv_faces(Grid g, int a, const double* vel, double rho, FaceVel fv, double dt, double* e0, double* e1, double* e2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    VelFP q{vel, g, rho};
    const long long f = fidx(g, a, i, j, k);
    const double um = fv.f[a][f];
    double* e[3] = {e0, e1, e2};
    for (int n = 0; n < 3; ++n) {
        double lo, hi;
        face_states<1>(g, q, q, fv, n, a, i, j, k, dt, lo, hi);
        e[n][f] = upwind(um, lo, hi);
    }
}

// ---- post-MAC stage 2: a-face states corrected along b (conservative form)
__global__ void k_adv_trans(Grid g, int a, int b, const double* vel, double rho, FaceVel fv, double dt, const double* E0, const double* E1,
                            const double* E2, double* o0, double* o1, double* o2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    VelFP q{vel, g, rho};
    const double* E[3] = {E0, E1, E2};
    double* o[3] = {o0, o1, o2};
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    const double cb = dt / (3.0 * hd(g, b));
    const double* vb = fv.f[b];
    const long long f = fidx(g, a, i, j, k);
    const double ua = fv.f[a][f];
    const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
    const long long h0 = fidx(g, b, i, j, k), h1 = fidx(g, b, i + (b == 0), j + (b == 1), k + (b == 2));
    const long long l0 = fidx(g, b, ci, cj, ck), l1 = fidx(g, b, ci + (b == 0), cj + (b == 1), ck + (b == 2));
    for (int n = 0; n < 3; ++n) {
        double l, h;
        face_states<1>(g, q, q, fv, n, a, i, j, k, dt, l, h);
        if (!wh) {
            const double vp = vb[h1], vm = vb[h0];
            h += -cb * (vp * E[n][h1] - vm * E[n][h0]) + cb * q(n, i, j, k) * (vp - vm);
        }
        if (!wl) {
            const double vp = vb[l1], vm = vb[l0];
            l += -cb * (vp * E[n][l1] - vm * E[n][l0]) + cb * q(n, ci, cj, ck) * (vp - vm);
        }
        if (a == 2) zbc(g, k, n, l, h);
        o[n][f] = upwind(ua, l, h);
    }
}

// ---- post-MAC stage 3: final states and fluxes on d-faces
__global__ void k_adv_flux(Grid g, int d, const double* vel, const double* forces, double rho, FaceVel fv, double dt, const double* T10,
                           const double* T11, const double* T12, const double* T20, const double* T21, const double* T22, double* F0,
                           double* F1, double* F2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, rho};
    CellFO Fo{forces, g};
    const double* T1[3] = {T10, T11, T12};
    const double* T2[3] = {T20, T21, T22};
    double* Fl[3] = {F0, F1, F2};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const double c1 = dt / (2.0 * hd(g, b1)), c2 = dt / (2.0 * hd(g, b2));
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, d, i, j, k);
    const double um = fv.f[d][f];
    for (int n = 0; n < 3; ++n) {
        double lo, hi;
        face_states<1>(g, q, q, fv, n, d, i, j, k, dt, lo, hi);
        auto side = [&](int ci, int cj, int ck, double base) {
            const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
            const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
            const double v1p = fv.f[b1][p1], v1m = fv.f[b1][m1], v2p = fv.f[b2][p2], v2m = fv.f[b2][m2];
            const double qc = q(n, ci, cj, ck);
            double s = base;
            s -= c1 * (T1[n][p1] * v1p - T1[n][m1] * v1m);
            s -= c2 * (T2[n][p2] * v2p - T2[n][m2] * v2m);
            s += c1 * qc * (v1p - v1m);
            s += c2 * qc * (v2p - v2m);
            s += 0.5 * dt * (rho * Fo(n, ci, cj, ck));
            return s;
        };
        double stl = 0.0, sth = 0.0;
        if (!wl) stl = side(i - (d == 0), j - (d == 1), k - (d == 2), lo);
        if (!wh) sth = side(i, j, k, hi);
        if (d == 2) zbc(g, k, n, stl, sth);
        double st = (um >= 0.0) ? stl : sth;
        if (fabs(um) < kSmallVel) st = 0.5 * (stl + sth);
        Fl[n][f] = um * st;
    }
}

struct FluxPtrs {
    const double* p[9];
};
__global__ void k_adv_div_s(Grid g, FluxPtrs F, double* conv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long xp = fidx(g, 0, i + 1, j, k), yp = fidx(g, 1, i, j + 1, k), zp = fidx(g, 2, i, j, k + 1), zm = fidx(g, 2, i, j, k);
    for (int n = 0; n < 3; ++n)
        conv[n * g.N + t] = -((F.p[n][xp] - F.p[n][t]) / g.dx + (F.p[3 + n][yp] - F.p[3 + n][t]) / g.dy +
                              (F.p[6 + n][zp] - F.p[6 + n][zm]) / g.dz);
}

}  // namespace


void launch_premac(Ctx& c, const Grid& g, const double* vel, const double* forces, double dt, GodunovBufs& B, double* mac[3]) {
    const double B8 = 8.0;
    for (int d = 0; d < 3; ++d) {
        const int n1 = (d + 1) % 3, n2 = (d + 2) % 3;
        const double nf = (double)nfaces(g, d);
        KS_LAUNCH(c, k_pm_faces, nblocks(nfaces(g, d), BS), BS, B8 * (3.0 * g.N + 3.0 * nf), g, d, vel, dt, B.ad[d], B.edge[d][n1],
                  B.edge[d][n2]);
    }
    // (a, b, n): states on a-faces of component n corrected along b
    const int tp[6][3] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    for (auto& p : tp) {
        const int a = p[0], b = p[1], n = p[2];
        const double bytes = B8 * (2.0 * g.N + 2.0 * nfaces(g, a) + 2.0 * nfaces(g, b));
        KS_LAUNCH(c, k_pm_trans, nblocks(nfaces(g, a), BS), BS, bytes, g, a, b, n, vel, dt, B.ad[a], B.ad[b], B.edge[b][n], B.tr[a][b][0]);
    }
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (2.0 * g.N + 2.0 * nfaces(g, d) + 2.0 * nfaces(g, b1) + 2.0 * nfaces(g, b2));
        KS_LAUNCH(c, k_pm_final, nblocks(nfaces(g, d), BS), BS, bytes, g, d, vel, forces, dt, B.ad[0], B.ad[1], B.ad[2], B.tr[b1][b2][0],
                  B.tr[b2][b1][0], mac[d]);
    }
}

void launch_advection(Ctx& c, const Grid& g, const double* vel, const double* forces, const double* mac[3], double dt, double rho,
                      GodunovBufs& B, double* conv) {
    const double B8 = 8.0;
    FaceVel fv{{mac[0], mac[1], mac[2]}};
    for (int a = 0; a < 3; ++a)
        KS_LAUNCH(c, k_adv_faces, nblocks(nfaces(g, a), BS), BS, B8 * (3.0 * g.N + 4.0 * nfaces(g, a)), g, a, vel, rho, fv, dt, B.edge[a][0],
                  B.edge[a][1], B.edge[a][2]);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            const double bytes = B8 * (3.0 * g.N + 4.0 * nfaces(g, a) + 4.0 * nfaces(g, b));
            KS_LAUNCH(c, k_adv_trans, nblocks(nfaces(g, a), BS), BS, bytes, g, a, b, vel, rho, fv, dt, B.edge[b][0], B.edge[b][1],
                      B.edge[b][2], B.tr[a][b][0], B.tr[a][b][1], B.tr[a][b][2]);
        }
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (6.0 * g.N + 4.0 * nfaces(g, d) + 4.0 * nfaces(g, b1) + 4.0 * nfaces(g, b2));
        KS_LAUNCH(c, k_adv_flux, nblocks(nfaces(g, d), BS), BS, bytes, g, d, vel, forces, rho, fv, dt, B.tr[b1][b2][0], B.tr[b1][b2][1],
                  B.tr[b1][b2][2], B.tr[b2][b1][0], B.tr[b2][b1][1], B.tr[b2][b1][2], B.flux[d][0], B.flux[d][1], B.flux[d][2]);
    }
    FluxPtrs F;
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < 3; ++n) F.p[d * 3 + n] = B.flux[d][n];
    KS_LAUNCH(c, k_adv_div_s, nblocks(g.N, BS), BS, B8 * (9.0 * g.N + 3.0 * g.N), g, F, conv);
}

}  // namespace ks
