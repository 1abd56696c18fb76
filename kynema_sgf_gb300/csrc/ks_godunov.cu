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
// FP64 arithmetic is the scarce resource on GB300, so nothing is computed
// twice: the unlimited PPM edge value of every face is computed once
// (k_edges), the left/right traces of every face once per stage (k_faces) and
// stored; the transverse and final stages only read them.  Post-MAC states of
// rho*u are rho times the traces of u (the PPM limiter and the traces are
// homogeneous of degree one in the advected field).
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

__device__ inline double vls(double a, double b, double c) {
    const double dsc = 0.5 * (c - a), dsl = 2.0 * (b - a), dsr = 2.0 * (c - b);
    return (dsl * dsr > 0.0) ? copysign(fmin(fabs(dsc), fmin(fabs(dsl), fabs(dsr))), dsc) : 0.0;
}
__device__ inline double clipe(double e, double a, double b) { return fmin(fmax(e, fmin(a, b)), fmax(a, b)); }

struct Dt {  // dt / h along x, y, z
    double v[3];
};

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

// ---- unlimited PPM edge values on the d-faces (face at the low side of the
// cell of the same index), 3 components.  Wall-bounded z: the wall faces take
// the boundary (ghost) value, the faces one cell inside the one-sided
// fourth-order formula, clipped to the two adjacent cells.
__global__ void k_edges(Grid g, int d, const double* vel, double* e0, double* e1, double* e2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, 1.0};
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wall = (d == 2 && !g.zper);
    double* e[3] = {e0, e1, e2};
    const long long f = fidx(g, d, i, j, k);
    for (int n = 0; n < 3; ++n) {
        double v;
        if (wall && k == 0) {
            v = q(n, i, j, -1);
        } else if (wall && k == g.nz) {
            v = q(n, i, j, g.nz);
        } else if (wall && k == 1) {
            const double b = q(n, i, j, -1), q0 = q(n, i, j, 0), q1 = q(n, i, j, 1), q2 = q(n, i, j, 2);
            v = clipe(-0.2 * b + 0.75 * q0 + 0.5 * q1 - 0.05 * q2, q0, q1);
        } else if (wall && k == g.nz - 1) {
            const int t0 = g.nz - 1;
            const double b = q(n, i, j, g.nz), q0 = q(n, i, j, t0), q1 = q(n, i, j, t0 - 1), q2 = q(n, i, j, t0 - 2);
            v = clipe(-0.2 * b + 0.75 * q0 + 0.5 * q1 - 0.05 * q2, q0, q1);
        } else {
            const double am = q(n, i - 2 * di, j - 2 * dj, k - 2 * dk), a0 = q(n, i - di, j - dj, k - dk);
            const double a1 = q(n, i, j, k), a2 = q(n, i + di, j + dj, k + dk);
            v = clipe(0.5 * (a0 + a1) - (1.0 / 6.0) * (vls(a0, a1, a2) - vls(am, a0, a1)), a0, a1);
        }
        e[n][f] = v;
    }
}

// limited parabola of a cell: (sm, sp) from its two stored edges and s0
__device__ inline void cw84(double s0, double& sm, double& sp) {
    if ((sp - s0) * (s0 - sm) <= 0.0) {
        sp = s0;
        sm = s0;
    } else if (fabs(sp - s0) >= 2.0 * fabs(sm - s0)) {
        sp = 3.0 * s0 - 2.0 * sm;
    } else if (fabs(sm - s0) >= 2.0 * fabs(sp - s0)) {
        sm = 3.0 * s0 - 2.0 * sp;
    }
}

// average of the limited parabola over the part of the cell that crosses its
// high (trace_hi) or low (trace_lo) face in dt, sig = |u| dt / h
__device__ inline double trace_hi(double sm, double s0, double sp, double sig) {
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    return sp - 0.5 * sig * ((sp - sm) - (1.0 - 2.0 / 3.0 * sig) * s6);
}
__device__ inline double trace_lo(double sm, double s0, double sp, double sig) {
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    return sm + 0.5 * sig * ((sp - sm) + (1.0 - 2.0 / 3.0 * sig) * s6);
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

struct P3 {
    double* p[3];
};
struct C3 {
    const double* p[3];
};

// ---- stage 1 of both passes: left/right states of all components on d-faces.
// MODE 0 (pre-MAC): the characteristic speed is the cell velocity component d;
// MODE 1 (post-MAC): the face velocities; states are scaled by rho.
// Pre-MAC also writes the Riemann-solved advective velocity and the states of
// the two transverse components upwinded with it; post-MAC writes the states of
// all three components upwinded with the MAC velocity.
template <int MODE>
__global__ void k_faces(Grid g, int d, const double* vel, C3 E, Dt dtdx, double rho, const double* umac_d, P3 LO, P3 HI, double* ad,
                        P3 edge) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, 1.0};
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, d, i, j, k);
    const long long fm = fidx(g, d, i - di, j - dj, k - dk), fp = fidx(g, d, i + di, j + dj, k + dk);
    const double s = dtdx.v[d];
    // characteristic speeds: cell velocities (pre-MAC) or the face velocities
    // of the low / high face of each cell (post-MAC)
    double ul = 0.0, uh = 0.0, umf = 0.0;
    if (MODE == 0) {
        if (!wl) ul = q(d, i - di, j - dj, k - dk);
        if (!wh) uh = q(d, i, j, k);
    } else {
        umf = umac_d[f];
        ul = umf;  // high face of cell c - e_d
        uh = umf;  // low face of cell c
    }
    double lo[3], hi[3];
    for (int n = 0; n < 3; ++n) {
        double l = 0.0, h = 0.0;
        if (!wl) {  // high-side trace of cell c - e_d
            const double s0 = q(n, i - di, j - dj, k - dk);
            double sm = E.p[n][fm], sp = E.p[n][f];
            cw84(s0, sm, sp);
            l = (ul > kSmallVel) ? trace_hi(sm, s0, sp, fabs(ul) * s) : s0;
        }
        if (!wh) {  // low-side trace of cell c
            const double s0 = q(n, i, j, k);
            double sm = E.p[n][f], sp = E.p[n][fp];
            cw84(s0, sm, sp);
            h = (uh < -kSmallVel) ? trace_lo(sm, s0, sp, fabs(uh) * s) : s0;
        }
        if (MODE == 1) {
            l *= rho;
            h *= rho;
        }
        if (d == 2) zbc(g, k, n, l, h);
        lo[n] = l;
        hi[n] = h;
        LO.p[n][f] = l;
        HI.p[n][f] = h;
    }
    if (MODE == 0) {
        const double a = riemann(lo[d], hi[d]);
        ad[f] = a;
        for (int n = 0; n < 3; ++n)
            if (n != d) edge.p[n][f] = upwind(a, lo[n], hi[n]);
    } else {
        for (int n = 0; n < 3; ++n) edge.p[n][f] = upwind(umf, lo[n], hi[n]);
    }
}

// ---- pre-MAC stage 2: a-face states of component n corrected along b
__global__ void k_pm_trans(Grid g, int a, int b, int n, double cb, const double* lo_an, const double* hi_an, const double* ad_a,
                           const double* ad_b, const double* edge_b, double* out) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    const long long f = fidx(g, a, i, j, k);
    double l = lo_an[f], h = hi_an[f];
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
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
    out[f] = upwind(ad_a[f], l, h);
}

// ---- pre-MAC stage 3: final normal velocity on d-faces
__global__ void k_pm_final(Grid g, int d, const double* lo_dd, const double* hi_dd, const double* forces, double dt, double c1, double c2,
                           C3 AD, const double* T1, const double* T2, double* mac) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    CellFO F{forces, g};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const long long f = fidx(g, d, i, j, k);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    auto side = [&](int ci, int cj, int ck, double base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        double s = base;
        s -= c1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        s += 0.5 * dt * F(d, ci, cj, ck);
        return s;
    };
    double stl = 0.0, sth = 0.0;
    if (!wl) stl = side(i - (d == 0), j - (d == 1), k - (d == 2), lo_dd[f]);
    if (!wh) sth = side(i, j, k, hi_dd[f]);
    if (d == 2) zbc(g, k, d, stl, sth);
    mac[f] = riemann(stl, sth);
}

// ---- post-MAC stage 2: a-face states corrected along b (conservative form)
__global__ void k_adv_trans(Grid g, int a, int b, const double* vel, double rho, double cb, const double* ua, const double* vb, C3 LO,
                            C3 HI, C3 E, P3 out) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    VelFP q{vel, g, rho};
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, a, i, j, k);
    const double u = ua[f];
    const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
    const long long h0 = fidx(g, b, i, j, k), h1 = fidx(g, b, i + (b == 0), j + (b == 1), k + (b == 2));
    const long long l0 = fidx(g, b, ci, cj, ck), l1 = fidx(g, b, ci + (b == 0), cj + (b == 1), ck + (b == 2));
    double vhp = 0.0, vhm = 0.0, vlp = 0.0, vlm = 0.0;
    if (!wh) { vhp = vb[h1]; vhm = vb[h0]; }
    if (!wl) { vlp = vb[l1]; vlm = vb[l0]; }
    for (int n = 0; n < 3; ++n) {
        double l = LO.p[n][f], h = HI.p[n][f];
        if (!wh) h += -cb * (vhp * E.p[n][h1] - vhm * E.p[n][h0]) + cb * q(n, i, j, k) * (vhp - vhm);
        if (!wl) l += -cb * (vlp * E.p[n][l1] - vlm * E.p[n][l0]) + cb * q(n, ci, cj, ck) * (vlp - vlm);
        if (a == 2) zbc(g, k, n, l, h);
        out.p[n][f] = upwind(u, l, h);
    }
}

// ---- post-MAC stage 3: final states and fluxes on d-faces
__global__ void k_adv_flux(Grid g, int d, const double* vel, const double* forces, double rho, double dt, double c1, double c2, C3 U,
                           C3 LO, C3 HI, C3 T1, C3 T2, P3 Fl) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFP q{vel, g, rho};
    CellFO Fo{forces, g};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, d, i, j, k);
    const double um = U.p[d][f];
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const long long lp1 = fidx(g, b1, li + (b1 == 0), lj + (b1 == 1), lk + (b1 == 2)), lm1 = fidx(g, b1, li, lj, lk);
    const long long lp2 = fidx(g, b2, li + (b2 == 0), lj + (b2 == 1), lk + (b2 == 2)), lm2 = fidx(g, b2, li, lj, lk);
    const long long hp1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), hm1 = fidx(g, b1, i, j, k);
    const long long hp2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), hm2 = fidx(g, b2, i, j, k);
    double l1p = 0, l1m = 0, l2p = 0, l2m = 0, h1p = 0, h1m = 0, h2p = 0, h2m = 0;
    if (!wl) { l1p = U.p[b1][lp1]; l1m = U.p[b1][lm1]; l2p = U.p[b2][lp2]; l2m = U.p[b2][lm2]; }
    if (!wh) { h1p = U.p[b1][hp1]; h1m = U.p[b1][hm1]; h2p = U.p[b2][hp2]; h2m = U.p[b2][hm2]; }
    for (int n = 0; n < 3; ++n) {
        double stl = 0.0, sth = 0.0;
        if (!wl) {
            const double qc = q(n, li, lj, lk);
            double s = LO.p[n][f];
            s -= c1 * (T1.p[n][lp1] * l1p - T1.p[n][lm1] * l1m);
            s -= c2 * (T2.p[n][lp2] * l2p - T2.p[n][lm2] * l2m);
            s += c1 * qc * (l1p - l1m);
            s += c2 * qc * (l2p - l2m);
            s += 0.5 * dt * (rho * Fo(n, li, lj, lk));
            stl = s;
        }
        if (!wh) {
            const double qc = q(n, i, j, k);
            double s = HI.p[n][f];
            s -= c1 * (T1.p[n][hp1] * h1p - T1.p[n][hm1] * h1m);
            s -= c2 * (T2.p[n][hp2] * h2p - T2.p[n][hm2] * h2m);
            s += c1 * qc * (h1p - h1m);
            s += c2 * qc * (h2p - h2m);
            s += 0.5 * dt * (rho * Fo(n, i, j, k));
            sth = s;
        }
        if (d == 2) zbc(g, k, n, stl, sth);
        double st = (um >= 0.0) ? stl : sth;
        if (fabs(um) < kSmallVel) st = 0.5 * (stl + sth);
        Fl.p[n][f] = um * st;
    }
}

struct FluxPtrs {
    const double* p[9];
};
__global__ void k_adv_div(Grid g, FluxPtrs F, double* conv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long xp = fidx(g, 0, i + 1, j, k), yp = fidx(g, 1, i, j + 1, k), zp = fidx(g, 2, i, j, k + 1), zm = fidx(g, 2, i, j, k);
    const double ix = 1.0 / g.dx, iy = 1.0 / g.dy, iz = 1.0 / g.dz;
    for (int n = 0; n < 3; ++n)
        conv[n * g.N + t] = -((F.p[n][xp] - F.p[n][t]) * ix + (F.p[3 + n][yp] - F.p[3 + n][t]) * iy + (F.p[6 + n][zp] - F.p[6 + n][zm]) * iz);
}

}  // namespace

void launch_premac(Ctx& c, const Grid& g, const double* vel, const double* forces, double dt, GodunovBufs& B, double* mac[3]) {
    const double B8 = 8.0;
    const Dt dtdx{{dt / g.dx, dt / g.dy, dt / g.dz}};
    for (int d = 0; d < 3; ++d)
        KS_LAUNCH(c, k_edges, nblocks(nfaces(g, d), BS), BS, B8 * (3.0 * g.N + 3.0 * nfaces(g, d)), g, d, vel, B.edge[d][0], B.edge[d][1],
                  B.edge[d][2]);
    for (int d = 0; d < 3; ++d) {
        C3 E{{B.edge[d][0], B.edge[d][1], B.edge[d][2]}};
        P3 LO{{B.lo[d][0], B.lo[d][1], B.lo[d][2]}}, HI{{B.hi[d][0], B.hi[d][1], B.hi[d][2]}};
        P3 ED{{B.tedge[d][0], B.tedge[d][1], B.tedge[d][2]}};
        const double nf = (double)nfaces(g, d);
        KS_LAUNCH(c, k_faces<0>, nblocks(nfaces(g, d), BS), BS, B8 * (3.0 * g.N + 12.0 * nf), g, d, vel, E, dtdx, 1.0, nullptr, LO, HI,
                  B.ad[d], ED);
    }
    // (a, b, n): states on a-faces of component n corrected along b
    const int tp[6][3] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    for (auto& p : tp) {
        const int a = p[0], b = p[1], n = p[2];
        const double bytes = B8 * (4.0 * nfaces(g, a) + 2.0 * nfaces(g, b));
        const double cb = dt / (6.0 * hd(g, b));
        KS_LAUNCH(c, k_pm_trans, nblocks(nfaces(g, a), BS), BS, bytes, g, a, b, n, cb, B.lo[a][n], B.hi[a][n], B.ad[a], B.ad[b],
                  B.tedge[b][n], B.tr[a][b][0]);
    }
    C3 AD{{B.ad[0], B.ad[1], B.ad[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (1.0 * g.N + 4.0 * nfaces(g, d) + 2.0 * nfaces(g, b1) + 2.0 * nfaces(g, b2));
        const double c1 = dt / (4.0 * hd(g, b1)), c2 = dt / (4.0 * hd(g, b2));
        KS_LAUNCH(c, k_pm_final, nblocks(nfaces(g, d), BS), BS, bytes, g, d, B.lo[d][d], B.hi[d][d], forces, dt, c1, c2, AD,
                  B.tr[b1][b2][0], B.tr[b2][b1][0], mac[d]);
    }
}

void launch_advection(Ctx& c, const Grid& g, const double* vel, const double* forces, const double* mac[3], double dt, double rho,
                      GodunovBufs& B, double* conv) {
    const double B8 = 8.0;
    const Dt dtdx{{dt / g.dx, dt / g.dy, dt / g.dz}};
    // the unlimited edge values of the pre-MAC pass are reused (same field)
    for (int a = 0; a < 3; ++a) {
        C3 E{{B.edge[a][0], B.edge[a][1], B.edge[a][2]}};
        P3 LO{{B.lo[a][0], B.lo[a][1], B.lo[a][2]}}, HI{{B.hi[a][0], B.hi[a][1], B.hi[a][2]}};
        P3 ED{{B.tedge[a][0], B.tedge[a][1], B.tedge[a][2]}};
        KS_LAUNCH(c, k_faces<1>, nblocks(nfaces(g, a), BS), BS, B8 * (3.0 * g.N + 13.0 * nfaces(g, a)), g, a, vel, E, dtdx, rho, mac[a],
                  LO, HI, nullptr, ED);
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            const double bytes = B8 * (3.0 * g.N + 10.0 * nfaces(g, a) + 4.0 * nfaces(g, b));
            C3 LO{{B.lo[a][0], B.lo[a][1], B.lo[a][2]}}, HI{{B.hi[a][0], B.hi[a][1], B.hi[a][2]}};
            C3 E{{B.tedge[b][0], B.tedge[b][1], B.tedge[b][2]}};
            P3 O{{B.tr[a][b][0], B.tr[a][b][1], B.tr[a][b][2]}};
            KS_LAUNCH(c, k_adv_trans, nblocks(nfaces(g, a), BS), BS, bytes, g, a, b, vel, rho, dt / (3.0 * hd(g, b)), mac[a], mac[b], LO,
                      HI, E, O);
        }
    C3 U{{mac[0], mac[1], mac[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (6.0 * g.N + 10.0 * nfaces(g, d) + 4.0 * nfaces(g, b1) + 4.0 * nfaces(g, b2));
        C3 LO{{B.lo[d][0], B.lo[d][1], B.lo[d][2]}}, HI{{B.hi[d][0], B.hi[d][1], B.hi[d][2]}};
        C3 T1{{B.tr[b1][b2][0], B.tr[b1][b2][1], B.tr[b1][b2][2]}}, T2{{B.tr[b2][b1][0], B.tr[b2][b1][1], B.tr[b2][b1][2]}};
        P3 F{{B.flux[d][0], B.flux[d][1], B.flux[d][2]}};
        KS_LAUNCH(c, k_adv_flux, nblocks(nfaces(g, d), BS), BS, bytes, g, d, vel, forces, rho, dt, dt / (2.0 * hd(g, b1)),
                  dt / (2.0 * hd(g, b2)), U, LO, HI, T1, T2, F);
    }
    FluxPtrs F;
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < 3; ++n) F.p[d * 3 + n] = B.flux[d][n];
    KS_LAUNCH(c, k_adv_div, nblocks(g.N, BS), BS, B8 * (9.0 * g.N + 3.0 * g.N), g, F, conv);
}

}  // namespace ks
