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

template <typename T>
__device__ inline T vls(T a, T b, T c) {
    const T dsc = T(0.5) * (c - a), dsl = T(2) * (b - a), dsr = T(2) * (c - b);
    return (dsl * dsr > T(0)) ? copysign(fmin(fabs(dsc), fmin(fabs(dsl), fabs(dsr))), dsc) : T(0);
}
template <typename T>
__device__ inline T clipe(T e, T a, T b) { return fmin(fmax(e, fmin(a, b)), fmax(a, b)); }

template <typename T>
struct Dt {  // dt / h along x, y, z
    T v[3];
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
template <typename T, int NC = 3>
__global__ void k_edges(Grid g, int d, const double* vel, T* e0, T* e1, T* e2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFPT<T> q{vel, g, T(1)};
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wall = (d == 2 && !g.zper);
    T* e[3] = {e0, e1, e2};
    const long long f = fidx(g, d, i, j, k);
    for (int n = 0; n < NC; ++n) {
        T v;
        if (wall && k == 0) {
            v = q(n, i, j, -1);
        } else if (wall && k == g.nz) {
            v = q(n, i, j, g.nz);
        } else if (wall && k == 1) {
            const T b = q(n, i, j, -1), q0 = q(n, i, j, 0), q1 = q(n, i, j, 1), q2 = q(n, i, j, 2);
            v = clipe(T(-0.2) * b + T(0.75) * q0 + T(0.5) * q1 - T(0.05) * q2, q0, q1);
        } else if (wall && k == g.nz - 1) {
            const int t0 = g.nz - 1;
            const T b = q(n, i, j, g.nz), q0 = q(n, i, j, t0), q1 = q(n, i, j, t0 - 1), q2 = q(n, i, j, t0 - 2);
            v = clipe(T(-0.2) * b + T(0.75) * q0 + T(0.5) * q1 - T(0.05) * q2, q0, q1);
        } else {
            const T am = q(n, i - 2 * di, j - 2 * dj, k - 2 * dk), a0 = q(n, i - di, j - dj, k - dk);
            const T a1 = q(n, i, j, k), a2 = q(n, i + di, j + dj, k + dk);
            v = clipe(T(0.5) * (a0 + a1) - T(1.0 / 6.0) * (vls(a0, a1, a2) - vls(am, a0, a1)), a0, a1);
        }
        e[n][f] = v;
    }
}

// limited parabola of a cell: (sm, sp) from its two stored edges and s0
template <typename T>
__device__ inline void cw84(T s0, T& sm, T& sp) {
    if ((sp - s0) * (s0 - sm) <= T(0)) {
        sp = s0;
        sm = s0;
    } else if (fabs(sp - s0) >= T(2) * fabs(sm - s0)) {
        sp = T(3) * s0 - T(2) * sm;
    } else if (fabs(sm - s0) >= T(2) * fabs(sp - s0)) {
        sm = T(3) * s0 - T(2) * sp;
    }
}

// average of the limited parabola over the part of the cell that crosses its
// high (trace_hi) or low (trace_lo) face in dt, sig = |u| dt / h
template <typename T>
__device__ inline T trace_hi(T sm, T s0, T sp, T sig) {
    const T s6 = T(6) * s0 - T(3) * (sm + sp);
    return sp - T(0.5) * sig * ((sp - sm) - (T(1) - T(2.0 / 3.0) * sig) * s6);
}
template <typename T>
__device__ inline T trace_lo(T sm, T s0, T sp, T sig) {
    const T s6 = T(6) * s0 - T(3) * (sm + sp);
    return sm + T(0.5) * sig * ((sp - sm) + (T(1) - T(2.0 / 3.0) * sig) * s6);
}

// Wall face treatment (SetZEdgeBCs): tangential components take the interior
// state, the normal component is zero on both sides.
template <typename T>
__device__ inline void zbc(const Grid& g, int k, int n, T& lo, T& hi) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) { lo = T(0); hi = T(0); } else lo = hi;
    } else if (k == g.nz) {
        if (n == 2) { lo = T(0); hi = T(0); } else hi = lo;
    }
}

template <typename T>
__device__ inline T upwind(T vel, T lo, T hi) {
    const T st = (vel >= T(0)) ? lo : hi;
    const T fu = (fabs(vel) < T(kSmallVel)) ? T(0) : T(1);
    return fu * st + (T(1) - fu) * T(0.5) * (lo + hi);
}
template <typename T>
__device__ inline T riemann(T lo, T hi) {
    const T st = (lo + hi >= T(0)) ? lo : hi;
    const bool ltm = (lo <= T(0) && hi >= T(0)) || (fabs(lo + hi) < T(kSmallVel));
    return ltm ? T(0) : st;
}

template <typename T>
struct P3 {
    T* p[3];
};
template <typename T>
struct C3 {
    const T* p[3];
};

// ---- stage 1 of both passes: left/right states of all components on d-faces.
// MODE 0 (pre-MAC): the characteristic speed is the cell velocity component d;
// MODE 1 (post-MAC): the face velocities; states are scaled by rho.
// Pre-MAC also writes the Riemann-solved advective velocity and the states of
// the two transverse components upwinded with it; post-MAC writes the states of
// all three components upwinded with the MAC velocity.
template <int MODE, typename T, int NC = 3>
__global__ void k_faces(Grid g, int d, const double* vel, C3<T> E, Dt<T> dtdx, T rho, const double* umac_d, P3<T> LO, P3<T> HI, T* ad,
                        P3<T> edge) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFPT<T> q{vel, g, T(1)};
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, d, i, j, k);
    const long long fm = fidx(g, d, i - di, j - dj, k - dk), fp = fidx(g, d, i + di, j + dj, k + dk);
    const T s = dtdx.v[d];
    // characteristic speeds: cell velocities (pre-MAC) or the face velocities
    // of the low / high face of each cell (post-MAC)
    T ul = T(0), uh = T(0), umf = T(0);
    if (MODE == 0) {
        if (!wl) ul = q(d, i - di, j - dj, k - dk);
        if (!wh) uh = q(d, i, j, k);
    } else {
        umf = (T)umac_d[f];
        ul = umf;  // high face of cell c - e_d
        uh = umf;  // low face of cell c
    }
    T lo[3], hi[3];
    for (int n = 0; n < NC; ++n) {
        T l = T(0), h = T(0);
        if (!wl) {  // high-side trace of cell c - e_d
            const T s0 = q(n, i - di, j - dj, k - dk);
            T sm = E.p[n][fm], sp = E.p[n][f];
            cw84(s0, sm, sp);
            l = (ul > T(kSmallVel)) ? trace_hi(sm, s0, sp, fabs(ul) * s) : s0;
        }
        if (!wh) {  // low-side trace of cell c
            const T s0 = q(n, i, j, k);
            T sm = E.p[n][f], sp = E.p[n][fp];
            cw84(s0, sm, sp);
            h = (uh < -T(kSmallVel)) ? trace_lo(sm, s0, sp, fabs(uh) * s) : s0;
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
        const T a = riemann(lo[d], hi[d]);
        ad[f] = a;
        for (int n = 0; n < 3; ++n)
            if (n != d) edge.p[n][f] = upwind(a, lo[n], hi[n]);
    } else {
        for (int n = 0; n < NC; ++n) edge.p[n][f] = upwind(umf, lo[n], hi[n]);
    }
}

// ---- pre-MAC stage 2: a-face states of component n corrected along b
template <typename T>
__global__ void k_pm_trans(Grid g, int a, int b, int n, T cb, const T* lo_an, const T* hi_an, const T* ad_a, const T* ad_b, const T* edge_b,
                           T* out) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    const long long f = fidx(g, a, i, j, k);
    T l = lo_an[f], h = hi_an[f];
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
template <typename T>
__global__ void k_pm_final(Grid g, int d, const T* lo_dd, const T* hi_dd, const double* forces, T dt, T c1, T c2, C3<T> AD, const T* T1,
                           const T* T2, double* mac) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    CellFOT<T> F{forces, g};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const long long f = fidx(g, d, i, j, k);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    auto side = [&](int ci, int cj, int ck, T base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        T s = base;
        s -= c1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        s += T(0.5) * dt * F(d, ci, cj, ck);
        return s;
    };
    T stl = T(0), sth = T(0);
    if (!wl) stl = side(i - (d == 0), j - (d == 1), k - (d == 2), lo_dd[f]);
    if (!wh) sth = side(i, j, k, hi_dd[f]);
    if (d == 2) zbc(g, k, d, stl, sth);
    mac[f] = (double)riemann(stl, sth);
}

// ---- post-MAC stage 2 for both transverse directions of the a-faces in one
// pass: the face states, the two adjacent cell values and the MAC velocity are
// loaded once for the corrections along b1 = a+1 and b2 = a+2 (each is the
// k_adv_trans arithmetic).
template <typename T, int NC = 3>
__global__ void __launch_bounds__(256, 2) k_adv_trans2(Grid g, int a, const double* vel, T rho, T cb1, T cb2, const double* ua,
                                                       const double* vb1, const double* vb2, C3<T> LO, C3<T> HI, C3<T> E1, C3<T> E2,
                                                       P3<T> out1, P3<T> out2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, a, t, i, j, k)) return;
    VelFPT<T> q{vel, g, rho};
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, a, i, j, k);
    const T u = (T)ua[f];
    const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
    const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
    auto fc = [&](int b, int ii, int jj, int kk, long long& m, long long& p) {
        m = fidx(g, b, ii, jj, kk);
        p = fidx(g, b, ii + (b == 0), jj + (b == 1), kk + (b == 2));
    };
    long long h0a, h1a, l0a, l1a, h0b, h1b, l0b, l1b;
    fc(b1, i, j, k, h0a, h1a);
    fc(b1, ci, cj, ck, l0a, l1a);
    fc(b2, i, j, k, h0b, h1b);
    fc(b2, ci, cj, ck, l0b, l1b);
    T vhp1 = T(0), vhm1 = T(0), vlp1 = T(0), vlm1 = T(0), vhp2 = T(0), vhm2 = T(0), vlp2 = T(0), vlm2 = T(0);
    if (!wh) {
        vhp1 = (T)vb1[h1a];
        vhm1 = (T)vb1[h0a];
        vhp2 = (T)vb2[h1b];
        vhm2 = (T)vb2[h0b];
    }
    if (!wl) {
        vlp1 = (T)vb1[l1a];
        vlm1 = (T)vb1[l0a];
        vlp2 = (T)vb2[l1b];
        vlm2 = (T)vb2[l0b];
    }
    for (int n = 0; n < NC; ++n) {
        const T l0 = LO.p[n][f], h0 = HI.p[n][f];
        const T qh = wh ? T(0) : q(n, i, j, k), ql = wl ? T(0) : q(n, ci, cj, ck);
        T l = l0, h = h0;
        if (!wh) h += -cb1 * (vhp1 * E1.p[n][h1a] - vhm1 * E1.p[n][h0a]) + cb1 * qh * (vhp1 - vhm1);
        if (!wl) l += -cb1 * (vlp1 * E1.p[n][l1a] - vlm1 * E1.p[n][l0a]) + cb1 * ql * (vlp1 - vlm1);
        if (a == 2) zbc(g, k, n, l, h);
        out1.p[n][f] = upwind(u, l, h);
        l = l0;
        h = h0;
        if (!wh) h += -cb2 * (vhp2 * E2.p[n][h1b] - vhm2 * E2.p[n][h0b]) + cb2 * qh * (vhp2 - vhm2);
        if (!wl) l += -cb2 * (vlp2 * E2.p[n][l1b] - vlm2 * E2.p[n][l0b]) + cb2 * ql * (vlp2 - vlm2);
        if (a == 2) zbc(g, k, n, l, h);
        out2.p[n][f] = upwind(u, l, h);
    }
}

// ---- post-MAC stage 3: final states and fluxes on d-faces
// The forces enter scaled by rho for the velocity (forces = (src + divtau) / rho)
// and as they are for a scalar (NC = 1: forces = src + diff, AdvOp_Godunov.H:114-329).
template <typename T, int NC = 3>
__global__ void __launch_bounds__(256, 3) k_adv_flux(Grid g, int d, const double* vel, const double* forces, T rho, T dt, T c1, T c2,
                                                     C3<double> U, C3<T> LO, C3<T> HI, C3<T> T1, C3<T> T2, P3<T> Fl) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_of(g, d, t, i, j, k)) return;
    VelFPT<T> q{vel, g, rho};
    CellFOT<T> Fo{forces, g};
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = fidx(g, d, i, j, k);
    const T um = (T)U.p[d][f];
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const long long lp1 = fidx(g, b1, li + (b1 == 0), lj + (b1 == 1), lk + (b1 == 2)), lm1 = fidx(g, b1, li, lj, lk);
    const long long lp2 = fidx(g, b2, li + (b2 == 0), lj + (b2 == 1), lk + (b2 == 2)), lm2 = fidx(g, b2, li, lj, lk);
    const long long hp1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), hm1 = fidx(g, b1, i, j, k);
    const long long hp2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), hm2 = fidx(g, b2, i, j, k);
    T l1p = 0, l1m = 0, l2p = 0, l2m = 0, h1p = 0, h1m = 0, h2p = 0, h2m = 0;
    if (!wl) { l1p = (T)U.p[b1][lp1]; l1m = (T)U.p[b1][lm1]; l2p = (T)U.p[b2][lp2]; l2m = (T)U.p[b2][lm2]; }
    if (!wh) { h1p = (T)U.p[b1][hp1]; h1m = (T)U.p[b1][hm1]; h2p = (T)U.p[b2][hp2]; h2m = (T)U.p[b2][hm2]; }
    for (int n = 0; n < NC; ++n) {
        T stl = T(0), sth = T(0);
        if (!wl) {
            const T qc = q(n, li, lj, lk);
            T s = LO.p[n][f];
            s -= c1 * (T1.p[n][lp1] * l1p - T1.p[n][lm1] * l1m);
            s -= c2 * (T2.p[n][lp2] * l2p - T2.p[n][lm2] * l2m);
            s += c1 * qc * (l1p - l1m);
            s += c2 * qc * (l2p - l2m);
            s += T(0.5) * dt * ((NC == 3 ? rho : T(1)) * Fo(n, li, lj, lk));
            stl = s;
        }
        if (!wh) {
            const T qc = q(n, i, j, k);
            T s = HI.p[n][f];
            s -= c1 * (T1.p[n][hp1] * h1p - T1.p[n][hm1] * h1m);
            s -= c2 * (T2.p[n][hp2] * h2p - T2.p[n][hm2] * h2m);
            s += c1 * qc * (h1p - h1m);
            s += c2 * qc * (h2p - h2m);
            s += T(0.5) * dt * ((NC == 3 ? rho : T(1)) * Fo(n, i, j, k));
            sth = s;
        }
        if (d == 2) zbc(g, k, n, stl, sth);
        T st = (um >= T(0)) ? stl : sth;
        if (fabs(um) < T(kSmallVel)) st = T(0.5) * (stl + sth);
        Fl.p[n][f] = um * st;
    }
}

template <typename T>
struct FluxPtrs {
    const T* p[9];
};
template <typename T, int NC = 3>
__global__ void k_adv_div(Grid g, FluxPtrs<T> F, double* conv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long xp = fidx(g, 0, i + 1, j, k), yp = fidx(g, 1, i, j + 1, k), zp = fidx(g, 2, i, j, k + 1), zm = fidx(g, 2, i, j, k);
    const T ix = T(g.idx), iy = T(g.idy), iz = T(g.idz);
    for (int n = 0; n < NC; ++n)
        conv[n * g.N + t] =
            (double)(-((F.p[n][xp] - F.p[n][t]) * ix + (F.p[3 + n][yp] - F.p[3 + n][t]) * iy + (F.p[6 + n][zp] - F.p[6 + n][zm]) * iz));
}

}  // namespace

template <typename T>
static T* tp(void* p) {
    return static_cast<T*>(p);
}

template <typename T>
static void premac_t(Ctx& c, const Grid& g, const double* vel, const double* forces, double dt, GodunovBufs& B, double* mac[3]) {
    const double BT = (double)sizeof(T), B8 = 8.0;
    const Dt<T> dtdx{{T(dt / g.dx), T(dt / g.dy), T(dt / g.dz)}};
    for (int d = 0; d < 3; ++d)
        KS_LAUNCH(c, k_edges<T>, nblocks(nfaces(g, d), BS), BS, B8 * 3.0 * g.N + BT * 3.0 * nfaces(g, d), g, d, vel, tp<T>(B.edge[d][0]),
                  tp<T>(B.edge[d][1]), tp<T>(B.edge[d][2]));
    for (int d = 0; d < 3; ++d) {
        C3<T> E{{tp<T>(B.edge[d][0]), tp<T>(B.edge[d][1]), tp<T>(B.edge[d][2])}};
        P3<T> LO{{tp<T>(B.lo[d][0]), tp<T>(B.lo[d][1]), tp<T>(B.lo[d][2])}}, HI{{tp<T>(B.hi[d][0]), tp<T>(B.hi[d][1]), tp<T>(B.hi[d][2])}};
        P3<T> ED{{tp<T>(B.tedge[d][0]), tp<T>(B.tedge[d][1]), tp<T>(B.tedge[d][2])}};
        const double nf = (double)nfaces(g, d);
        KS_LAUNCH(c, (k_faces<0, T>), nblocks(nfaces(g, d), BS), BS, B8 * 3.0 * g.N + BT * 12.0 * nf, g, d, vel, E, dtdx, T(1), nullptr,
                  LO, HI, tp<T>(B.ad[d]), ED);
    }
    // (a, b, n): states on a-faces of component n corrected along b
    const int tpl[6][3] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    for (auto& p : tpl) {
        const int a = p[0], b = p[1], n = p[2];
        const double bytes = BT * (4.0 * nfaces(g, a) + 2.0 * nfaces(g, b));
        const T cb = T(dt / (6.0 * hd(g, b)));
        KS_LAUNCH(c, k_pm_trans<T>, nblocks(nfaces(g, a), BS), BS, bytes, g, a, b, n, cb, tp<T>(B.lo[a][n]), tp<T>(B.hi[a][n]),
                  tp<T>(B.ad[a]), tp<T>(B.ad[b]), tp<T>(B.tedge[b][n]), tp<T>(B.tr[a][b][0]));
    }
    C3<T> AD{{tp<T>(B.ad[0]), tp<T>(B.ad[1]), tp<T>(B.ad[2])}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (1.0 * g.N + nfaces(g, d)) + BT * (3.0 * nfaces(g, d) + 2.0 * nfaces(g, b1) + 2.0 * nfaces(g, b2));
        const T c1 = T(dt / (4.0 * hd(g, b1))), c2 = T(dt / (4.0 * hd(g, b2)));
        KS_LAUNCH(c, k_pm_final<T>, nblocks(nfaces(g, d), BS), BS, bytes, g, d, tp<T>(B.lo[d][d]), tp<T>(B.hi[d][d]), forces, T(dt), c1, c2,
                  AD, tp<T>(B.tr[b1][b2][0]), tp<T>(B.tr[b2][b1][0]), mac[d]);
    }
}

template <typename T>
static void advection_t(Ctx& c, const Grid& g, const double* vel, const double* forces, const double* mac[3], double dt, double rho,
                        GodunovBufs& B, double* conv) {
    const double BT = (double)sizeof(T), B8 = 8.0;
    const Dt<T> dtdx{{T(dt / g.dx), T(dt / g.dy), T(dt / g.dz)}};
    // the unlimited edge values of the pre-MAC pass are reused (same field)
    for (int a = 0; a < 3; ++a) {
        C3<T> E{{tp<T>(B.edge[a][0]), tp<T>(B.edge[a][1]), tp<T>(B.edge[a][2])}};
        P3<T> LO{{tp<T>(B.lo[a][0]), tp<T>(B.lo[a][1]), tp<T>(B.lo[a][2])}}, HI{{tp<T>(B.hi[a][0]), tp<T>(B.hi[a][1]), tp<T>(B.hi[a][2])}};
        P3<T> ED{{tp<T>(B.tedge[a][0]), tp<T>(B.tedge[a][1]), tp<T>(B.tedge[a][2])}};
        KS_LAUNCH(c, (k_faces<1, T>), nblocks(nfaces(g, a), BS), BS, B8 * (3.0 * g.N + nfaces(g, a)) + BT * 12.0 * nfaces(g, a), g, a, vel,
                  E, dtdx, T(rho), mac[a], LO, HI, (T*)nullptr, ED);
    }
    for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        const double na = (double)nfaces(g, a), nt = (double)(nfaces(g, b1) + nfaces(g, b2));
        const double bytes = B8 * (3.0 * g.N + na + nt) + BT * (12.0 * na + 3.0 * nt);
        C3<T> LO{{tp<T>(B.lo[a][0]), tp<T>(B.lo[a][1]), tp<T>(B.lo[a][2])}}, HI{{tp<T>(B.hi[a][0]), tp<T>(B.hi[a][1]), tp<T>(B.hi[a][2])}};
        C3<T> E1{{tp<T>(B.tedge[b1][0]), tp<T>(B.tedge[b1][1]), tp<T>(B.tedge[b1][2])}};
        C3<T> E2{{tp<T>(B.tedge[b2][0]), tp<T>(B.tedge[b2][1]), tp<T>(B.tedge[b2][2])}};
        P3<T> O1{{tp<T>(B.tr[a][b1][0]), tp<T>(B.tr[a][b1][1]), tp<T>(B.tr[a][b1][2])}};
        P3<T> O2{{tp<T>(B.tr[a][b2][0]), tp<T>(B.tr[a][b2][1]), tp<T>(B.tr[a][b2][2])}};
        KS_LAUNCH(c, k_adv_trans2<T>, nblocks(nfaces(g, a), BS), BS, bytes, g, a, vel, T(rho), T(dt / (3.0 * hd(g, b1))),
                  T(dt / (3.0 * hd(g, b2))), mac[a], mac[b1], mac[b2], LO, HI, E1, E2, O1, O2);
    }
    C3<double> U{{mac[0], mac[1], mac[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = B8 * (6.0 * g.N + nfaces(g, d) + nfaces(g, b1) + nfaces(g, b2)) +
                             BT * (9.0 * nfaces(g, d) + 3.0 * nfaces(g, b1) + 3.0 * nfaces(g, b2));
        C3<T> LO{{tp<T>(B.lo[d][0]), tp<T>(B.lo[d][1]), tp<T>(B.lo[d][2])}}, HI{{tp<T>(B.hi[d][0]), tp<T>(B.hi[d][1]), tp<T>(B.hi[d][2])}};
        C3<T> T1{{tp<T>(B.tr[b1][b2][0]), tp<T>(B.tr[b1][b2][1]), tp<T>(B.tr[b1][b2][2])}};
        C3<T> T2{{tp<T>(B.tr[b2][b1][0]), tp<T>(B.tr[b2][b1][1]), tp<T>(B.tr[b2][b1][2])}};
        P3<T> F{{tp<T>(B.flux[d][0]), tp<T>(B.flux[d][1]), tp<T>(B.flux[d][2])}};
        KS_LAUNCH(c, k_adv_flux<T>, nblocks(nfaces(g, d), BS), BS, bytes, g, d, vel, forces, T(rho), T(dt), T(dt / (2.0 * hd(g, b1))),
                  T(dt / (2.0 * hd(g, b2))), U, LO, HI, T1, T2, F);
    }
    FluxPtrs<T> F;
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < 3; ++n) F.p[d * 3 + n] = tp<T>(B.flux[d][n]);
    KS_LAUNCH(c, k_adv_div<T>, nblocks(g.N, BS), BS, BT * 9.0 * g.N + B8 * 3.0 * g.N, g, F, conv);
}

// Godunov fluxes of rho s for a cell scalar s (hoextrap at z walls, like a
// tangential velocity component) with the forces fs = src + diff, and conv =
// -div(flux) (AdvOp_Godunov.H:114-329).  FP64; edges[3] holds the scalar's
// unlimited edge values; the other face arrays are the component-0 slots of B.
void launch_scalar_advection(Ctx& c, const Grid& g, const double* s, const double* fs, const double* mac[3], double dt, double rho,
                             double* const edges[3], GodunovBufs& B, double* conv) {
    using T = double;
    const double B8 = 8.0;
    const Dt<T> dtdx{{dt / g.dx, dt / g.dy, dt / g.dz}};
    for (int d = 0; d < 3; ++d)
        KS_LAUNCH(c, (k_edges<T, 1>), nblocks(nfaces(g, d), BS), BS, B8 * (g.N + nfaces(g, d)), g, d, s, edges[d], nullptr, nullptr);
    for (int a = 0; a < 3; ++a) {
        C3<T> E{{edges[a], nullptr, nullptr}};
        P3<T> LO{{tp<T>(B.lo[a][0]), nullptr, nullptr}}, HI{{tp<T>(B.hi[a][0]), nullptr, nullptr}};
        P3<T> ED{{tp<T>(B.tedge[a][0]), nullptr, nullptr}};
        KS_LAUNCH(c, (k_faces<1, T, 1>), nblocks(nfaces(g, a), BS), BS, B8 * (g.N + 5.0 * nfaces(g, a)), g, a, s, E, dtdx, T(rho), mac[a], LO,
                  HI, (T*)nullptr, ED);
    }
    for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        const double na = (double)nfaces(g, a), nt = (double)(nfaces(g, b1) + nfaces(g, b2));
        C3<T> LO{{tp<T>(B.lo[a][0]), nullptr, nullptr}}, HI{{tp<T>(B.hi[a][0]), nullptr, nullptr}};
        C3<T> E1{{tp<T>(B.tedge[b1][0]), nullptr, nullptr}}, E2{{tp<T>(B.tedge[b2][0]), nullptr, nullptr}};
        P3<T> O1{{tp<T>(B.tr[a][b1][0]), nullptr, nullptr}}, O2{{tp<T>(B.tr[a][b2][0]), nullptr, nullptr}};
        KS_LAUNCH(c, (k_adv_trans2<T, 1>), nblocks(nfaces(g, a), BS), BS, B8 * (g.N + 5.0 * na + 2.0 * nt), g, a, s, T(rho),
                  T(dt / (3.0 * hd(g, b1))), T(dt / (3.0 * hd(g, b2))), mac[a], mac[b1], mac[b2], LO, HI, E1, E2, O1, O2);
    }
    C3<double> U{{mac[0], mac[1], mac[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        C3<T> LO{{tp<T>(B.lo[d][0]), nullptr, nullptr}}, HI{{tp<T>(B.hi[d][0]), nullptr, nullptr}};
        C3<T> T1{{tp<T>(B.tr[b1][b2][0]), nullptr, nullptr}}, T2{{tp<T>(B.tr[b2][b1][0]), nullptr, nullptr}};
        P3<T> F{{tp<T>(B.flux[d][0]), nullptr, nullptr}};
        const double bytes = B8 * (2.0 * g.N + 4.0 * nfaces(g, d) + 2.0 * (nfaces(g, b1) + nfaces(g, b2)));
        KS_LAUNCH(c, (k_adv_flux<T, 1>), nblocks(nfaces(g, d), BS), BS, bytes, g, d, s, fs, T(rho), T(dt), T(dt / (2.0 * hd(g, b1))),
                  T(dt / (2.0 * hd(g, b2))), U, LO, HI, T1, T2, F);
    }
    FluxPtrs<T> F;
    for (int m = 0; m < 9; ++m) F.p[m] = nullptr;
    for (int d = 0; d < 3; ++d) F.p[3 * d] = tp<T>(B.flux[d][0]);
    KS_LAUNCH(c, (k_adv_div<T, 1>), nblocks(g.N, BS), BS, B8 * (3.0 * g.N + g.N), g, F, conv);
}

void launch_premac(Ctx& c, const Grid& g, const double* vel, const double* forces, double dt, GodunovBufs& B, double* mac[3], int fp32) {
    if (fp32) premac_t<float>(c, g, vel, forces, dt, B, mac);
    else premac_t<double>(c, g, vel, forces, dt, B, mac);
}

void launch_advection(Ctx& c, const Grid& g, const double* vel, const double* forces, const double* mac[3], double dt, double rho,
                      GodunovBufs& B, double* conv, int fp32) {
    if (fp32) advection_t<float>(c, g, vel, forces, mac, dt, rho, B, conv);
    else advection_t<double>(c, g, vel, forces, mac, dt, rho, B, conv);
}

}  // namespace ks
