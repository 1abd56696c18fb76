// Reverse (adjoint) kernels of the advance, FP64.
//
// Every forward pass y = K(x) gets a kernel that accumulates x_bar += (dK/dx)^T
// y_bar at the forward linearisation point.  The PPM limiter, clipping,
// Riemann and upwind selections are re-evaluated from the stored forward
// values and frozen (their derivatives are the derivatives of the selected
// branch).  Inputs that several outputs read are accumulated with atomicAdd.
// Boundary handling mirrors the forward kernels: x/y periodic; z periodic or
// walls, where the forward reads fill-patch ghosts (high-order extrapolation
// of the tangential components, zero normal component) for Godunov, odd/even
// reflections or the wall-model shift for diffusion, and replaces wall-face
// states (zbc); the reverse scatters every ghost read back onto the interior
// cells it was built from.
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;
constexpr double kSV = kSmallVel;

__device__ inline void aadd(double* p, double v) {
    if ((dbits(v) & kMag)) atomicAdd(p, v);
}

// faces of direction d, the same index domain as the forward kernels
__device__ inline bool face_at(const Grid& g, int d, long long t, int& i, int& j, int& k) {
    const int nzl = (d == 2) ? nzfaces(g) : g.nz;
    const long long M = (long long)g.nx * g.ny * nzl;
    if (t >= M) return false;
    const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
    i = (int)(u - r * (unsigned)g.nx);
    k = (int)(r / (unsigned)g.ny);
    j = (int)(r - (unsigned)k * (unsigned)g.ny);
    return true;
}
inline long long nfaces(const Grid& g, int d) { return (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz); }

// velocity read with the Godunov fill-patch ghosts (VelFPT, scale 1) and its adjoint
__device__ inline double Q(const Grid& g, const double* u, int n, int i, int j, int k) {
    const VelFPT<double> q{u, g, 1.0};
    return q(n, i, j, k);
}
__device__ inline void Qb(const Grid& g, double* ub, int n, int i, int j, int k, double v) {
    if (!(dbits(v) & kMag)) return;
    i = wrapn(i, g.nx);
    j = wrapn(j, g.ny);
    double* c = ub + (long long)n * g.N;
    if (g.zper) {
        atomicAdd(c + cidx(g, i, j, wrapn(k, g.nz)), v);
        return;
    }
    if (k < 0 || k >= g.nz) {  // ghost = (15 q0 - 10 q1 + 3 q2) / 8 of the nearest cells; normal component 0
        if (n == 2) return;
        const int k0 = k < 0 ? 0 : g.nz - 1, s = k < 0 ? 1 : -1;
        atomicAdd(c + cidx(g, i, j, k0), 1.875 * v);
        atomicAdd(c + cidx(g, i, j, k0 + s), -1.25 * v);
        atomicAdd(c + cidx(g, i, j, k0 + 2 * s), 0.375 * v);
        return;
    }
    atomicAdd(c + cidx(g, i, j, k), v);
}

// wall-face state replacement of the forward (zbc) and its adjoint
__device__ inline void zbc_fwd(const Grid& g, int k, int n, double& lo, double& hi) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) lo = hi = 0.0; else lo = hi;
    } else if (k == g.nz) {
        if (n == 2) lo = hi = 0.0; else hi = lo;
    }
}
__device__ inline void zbc_rev(const Grid& g, int k, int n, double& lb, double& hb) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) {
            lb = hb = 0.0;
        } else {
            hb += lb;
            lb = 0.0;
        }
    } else if (k == g.nz) {
        if (n == 2) {
            lb = hb = 0.0;
        } else {
            lb += hb;
            hb = 0.0;
        }
    }
}

// ---- van Leer slope: value and the coefficients of (a, b, c)
__device__ inline double vls_d(double a, double b, double c, double& ca, double& cb, double& cc) {
    const double dsc = 0.5 * (c - a), dsl = 2.0 * (b - a), dsr = 2.0 * (c - b);
    ca = cb = cc = 0.0;
    if (!isame_sign(dsl, dsr)) return 0.0;
    // magnitudes compared on the integer pipe (non-negative doubles order like their bits)
    const long long ac = dbits(dsc) & kMag, al = dbits(dsl) & kMag, ar = dbits(dsr) & kMag;
    if (ac <= (al < ar ? al : ar)) {
        ca = -0.5;
        cc = 0.5;
        return dsc;
    }
    if (al <= ar) {
        ca = -2.0;
        cb = 2.0;
        return dsl;
    }
    cb = -2.0;
    cc = 2.0;
    return dsr;
}

// adjoint of clip(e, a, b) = min(max(e, min(a, b)), max(a, b)) given the
// adjoint of the result: returns the adjoint of e; adds to those of a, b.
// The selections order -0 below +0 (the integer-pipe comparisons of
// ks_common.cuh), as the forward clip does, so a signed-zero tie routes the
// adjoint to the operand the forward selected.
__device__ inline double clip_rev(double e, double a, double b, double rb, double& ga, double& gb) {
    const double lo = imin(a, b), hi = imax(a, b);
    if (ilt(hi, imax(e, lo))) {
        if (!ilt(a, b)) ga += rb; else gb += rb;
        return 0.0;
    }
    if (ilt(e, lo)) {
        if (!ilt(b, a)) ga += rb; else gb += rb;
        return 0.0;
    }
    return rb;
}

// ---- reverse of the unlimited PPM edges on d-faces (k_edges)
template <typename TI>
__global__ void k_adj_edges(Grid g, int d, const double* u, const double* Eb0, const double* Eb1, const double* Eb2, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wall = (d == 2 && !g.zper);
    const double* Eb[3] = {Eb0, Eb1, Eb2};
    for (int n = 0; n < 3; ++n) {
        const double eb = Eb[n][t];
        if (!(dbits(eb) & kMag)) continue;
        if (wall && (k == 0 || k == g.nz)) {  // the wall face takes the ghost value
            Qb(g, ub, n, i, j, k == 0 ? -1 : g.nz, eb);
            continue;
        }
        if (wall && (k == 1 || k == g.nz - 1)) {  // one-sided fourth order, clipped to the adjacent cells
            const int kb = (k == 1) ? -1 : g.nz, k0 = (k == 1) ? 0 : g.nz - 1, s = (k == 1) ? 1 : -1;
            const double b = (TI)Q(g, u, n, i, j, kb), q0 = (TI)Q(g, u, n, i, j, k0), q1 = (TI)Q(g, u, n, i, j, k0 + s),
                         q2 = (TI)Q(g, u, n, i, j, k0 + 2 * s);
            const double e = -0.2 * b + 0.75 * q0 + 0.5 * q1 - 0.05 * q2;
            double g0 = 0.0, g1 = 0.0;
            const double ebar = clip_rev(e, q0, q1, eb, g0, g1);
            Qb(g, ub, n, i, j, kb, -0.2 * ebar);
            Qb(g, ub, n, i, j, k0, 0.75 * ebar + g0);
            Qb(g, ub, n, i, j, k0 + s, 0.5 * ebar + g1);
            Qb(g, ub, n, i, j, k0 + 2 * s, -0.05 * ebar);
            continue;
        }
        const double am = (TI)Q(g, u, n, i - 2 * di, j - 2 * dj, k - 2 * dk), a0 = (TI)Q(g, u, n, i - di, j - dj, k - dk);
        const double a1 = (TI)Q(g, u, n, i, j, k), a2 = (TI)Q(g, u, n, i + di, j + dj, k + dk);
        double c1a, c1b, c1c, c0a, c0b, c0c;
        const double s1 = vls_d(a0, a1, a2, c1a, c1b, c1c);
        const double s0 = vls_d(am, a0, a1, c0a, c0b, c0c);
        const double e = 0.5 * (a0 + a1) - (1.0 / 6.0) * (s1 - s0);
        double gm = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
        const double ebar = clip_rev(e, a0, a1, eb, g0, g1);
        if ((dbits(ebar) & kMag)) {
            g0 += 0.5 * ebar;
            g1 += 0.5 * ebar;
            const double ds1 = -ebar / 6.0, ds0 = ebar / 6.0;
            g0 += ds1 * c1a;
            g1 += ds1 * c1b;
            g2 += ds1 * c1c;
            gm += ds0 * c0a;
            g0 += ds0 * c0b;
            g1 += ds0 * c0c;
        }
        Qb(g, ub, n, i - 2 * di, j - 2 * dj, k - 2 * dk, gm);
        Qb(g, ub, n, i - di, j - dj, k - dk, g0);
        Qb(g, ub, n, i, j, k, g1);
        Qb(g, ub, n, i + di, j + dj, k + dk, g2);
    }
}

// ---- reverse of the CW84 limiter + trace.  Given the adjoint tb of the trace
// value, accumulate into the adjoints of sm_in, s0, sp_in and return the
// adjoint of sig.
__device__ inline double rev_trace(bool hi_side, double smi, double s0, double spi, double sig, double tb, double& gsm, double& gs0,
                                   double& gsp) {
    double sm = smi, sp = spi;
    int cs = 0;
    // the forward's CW84 decisions (k_ppm_*: cw84), on the integer pipe
    const double dp = sp - s0, dm = s0 - sm;
    if (!isame_sign(dp, dm)) {
        cs = 1;
        sp = s0;
        sm = s0;
    } else if (!iabs_lt2(dp, 2.0 * dm)) {
        cs = 2;
        sp = s0 + 2.0 * dm;
    } else if (!iabs_lt2(dm, 2.0 * dp)) {
        cs = 3;
        sm = s0 - 2.0 * dp;
    }
    const double Bf = 1.0 - 2.0 / 3.0 * sig;
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    double dsm, dsp, ds0, dsig;
    if (hi_side) {
        dsp = 1.0 - 0.5 * sig * (1.0 + 3.0 * Bf);
        dsm = 0.5 * sig * (1.0 - 3.0 * Bf);
        ds0 = 3.0 * sig * Bf;
        dsig = -0.5 * ((sp - sm) - Bf * s6) - (1.0 / 3.0) * sig * s6;
    } else {
        dsm = 1.0 - 0.5 * sig * (1.0 + 3.0 * Bf);
        dsp = 0.5 * sig * (1.0 - 3.0 * Bf);
        ds0 = 3.0 * sig * Bf;
        dsig = 0.5 * ((sp - sm) + Bf * s6) - (1.0 / 3.0) * sig * s6;
    }
    double bsm = dsm * tb, bsp = dsp * tb, bs0 = ds0 * tb;
    if (cs == 1) {
        bs0 += bsm + bsp;
        bsm = 0.0;
        bsp = 0.0;
    } else if (cs == 2) {
        bs0 += 3.0 * bsp;
        bsm += -2.0 * bsp;
        bsp = 0.0;
    } else if (cs == 3) {
        bs0 += 3.0 * bsm;
        bsp += -2.0 * bsm;
        bsm = 0.0;
    }
    gsm += bsm;
    gsp += bsp;
    gs0 += bs0;
    return dsig * tb;
}

__device__ inline void rev_upwind(double vel, double ob, double& lb, double& hb) {
    if (!iabs_lt(vel, kSV)) {
        if (ige0(vel)) lb += ob; else hb += ob;
    } else {
        lb += 0.5 * ob;
        hb += 0.5 * ob;
    }
}
__device__ inline void rev_riemann(double lo, double hi, double ob, double& lb, double& hb) {
    const double sum = lo + hi;
    const bool ltm = (ile0(lo) && ige0(hi)) || iabs_lt(sum, kSV);
    if (ltm) return;
    if (ige0(sum)) lb += ob; else hb += ob;
}

struct A3 {
    double* p[3];
};
struct K3 {
    const double* p[3];
};
// forward intermediates, stored in FP64 or FP32 (TI)
template <typename TI>
struct KI {
    const TI* p[3];
};

// ---- reverse of k_faces (both passes).  MODE 0: pre-MAC (cell speed), the
// adjoints of ad and of the upwinded transverse states are folded in here;
// MODE 1: post-MAC (face speed, rho scaling), upwinded states folded in.
template <int MODE, typename TI>
__global__ void k_adj_faces(Grid g, int d, const double* u, KI<TI> E, double s, double rho, const double* umac_d, KI<TI> LO, KI<TI> HI,
                            const TI* ad, K3 LOb, K3 HIb, const double* adb, K3 TEb, A3 Eb, double* ub, double* umacb_d) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = t;
    const long long fm = fidx(g, d, i - di, j - dj, k - dk), fp = fidx(g, d, i + di, j + dj, k + dk);
    double lb[3], hb[3];
    for (int n = 0; n < 3; ++n) {
        lb[n] = LOb.p[n][f];
        hb[n] = HIb.p[n][f];
    }
    double ul = 0.0, uh = 0.0;
    if (MODE == 0) {
        if (!wl) ul = (TI)Q(g, u, d, i - di, j - dj, k - dk);
        if (!wh) uh = (TI)Q(g, u, d, i, j, k);
        rev_riemann(LO.p[d][f], HI.p[d][f], adb[f], lb[d], hb[d]);
        const double a = ad[f];
        for (int n = 0; n < 3; ++n)
            if (n != d) rev_upwind(a, TEb.p[n][f], lb[n], hb[n]);
    } else {
        const double umf = (TI)umac_d[f];
        ul = uh = umf;
        for (int n = 0; n < 3; ++n) rev_upwind(umf, TEb.p[n][f], lb[n], hb[n]);
    }
    if (d == 2)
        for (int n = 0; n < 3; ++n) zbc_rev(g, k, n, lb[n], hb[n]);
    const double scale = (MODE == 1) ? (double)(TI)rho : 1.0;
    const double sT = (TI)s;
    double gul = 0.0, guh = 0.0;
    for (int n = 0; n < 3; ++n) {
        const double tl = lb[n] * scale, th = hb[n] * scale;
        if (!wl && (dbits(tl) & kMag)) {  // high-side trace of cell c - e_d
            double gsm = 0.0, gs0 = 0.0, gsp = 0.0;
            const double s0 = (TI)Q(g, u, n, i - di, j - dj, k - dk);
            if (dbits(ul) > dbits(kSV)) {
                const double bsig = rev_trace(true, E.p[n][fm], s0, E.p[n][f], (TI)(iabs(ul) * sT), tl, gsm, gs0, gsp);
                gul += bsig * s * (ige0(ul) ? 1.0 : -1.0);
            } else {
                gs0 += tl;
            }
            aadd(&Eb.p[n][fm], gsm);
            aadd(&Eb.p[n][f], gsp);
            Qb(g, ub, n, i - di, j - dj, k - dk, gs0);
        }
        if (!wh && (dbits(th) & kMag)) {  // low-side trace of cell c
            double gsm = 0.0, gs0 = 0.0, gsp = 0.0;
            const double s0 = (TI)Q(g, u, n, i, j, k);
            if (okey(uh) < okey(-kSV)) {
                const double bsig = rev_trace(false, E.p[n][f], s0, E.p[n][fp], (TI)(iabs(uh) * sT), th, gsm, gs0, gsp);
                guh += bsig * s * (ige0(uh) ? 1.0 : -1.0);
            } else {
                gs0 += th;
            }
            aadd(&Eb.p[n][f], gsm);
            aadd(&Eb.p[n][fp], gsp);
            Qb(g, ub, n, i, j, k, gs0);
        }
    }
    if (MODE == 0) {
        if (!wl) Qb(g, ub, d, i - di, j - dj, k - dk, gul);
        if (!wh) Qb(g, ub, d, i, j, k, guh);
    } else {
        aadd(&umacb_d[f], gul + guh);
    }
}

// ---- reverse of k_pm_trans (a, b, n)
template <typename TI>
__global__ void k_adj_pm_trans(Grid g, int a, int b, int n, double cb, const TI* ad_a, const TI* ad_b, const TI* edge_b, const double* outb,
                               double* lo_anb, double* hi_anb, double* ad_bb, double* edge_bb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, a, t, i, j, k)) return;
    const long long f = t;
    const double ob = outb[f];
    if (!(dbits(ob) & kMag)) return;
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    double lb = 0.0, hb = 0.0;
    rev_upwind(ad_a[f], ob, lb, hb);
    if (a == 2) zbc_rev(g, k, n, lb, hb);
    lo_anb[f] += lb;
    hi_anb[f] += hb;
    const int e0 = (b == 0), e1 = (b == 1), e2 = (b == 2);
    if (!wh && (dbits(hb) & kMag)) {
        const long long f0 = fidx(g, b, i, j, k), f1 = fidx(g, b, i + e0, j + e1, k + e2);
        const double S = (double)ad_b[f1] + ad_b[f0], Dd = (double)edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], -cb * Dd * hb);
        aadd(&ad_bb[f0], -cb * Dd * hb);
        aadd(&edge_bb[f1], -cb * S * hb);
        aadd(&edge_bb[f0], cb * S * hb);
    }
    if (!wl && (dbits(lb) & kMag)) {
        const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
        const long long f0 = fidx(g, b, ci, cj, ck), f1 = fidx(g, b, ci + e0, cj + e1, ck + e2);
        const double S = (double)ad_b[f1] + ad_b[f0], Dd = (double)edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], -cb * Dd * lb);
        aadd(&ad_bb[f0], -cb * Dd * lb);
        aadd(&edge_bb[f1], -cb * S * lb);
        aadd(&edge_bb[f0], cb * S * lb);
    }
}

// forces with the first-order extrapolated ghosts of CellFOT and the adjoint
__device__ inline long long cell_fo(const Grid& g, int i, int j, int k) {
    i = wrapn(i, g.nx);
    j = wrapn(j, g.ny);
    if (g.zper) k = wrapn(k, g.nz);
    else k = k < 0 ? 0 : (k >= g.nz ? g.nz - 1 : k);
    return cidx(g, i, j, k);
}

// ---- reverse of k_pm_final (d)
template <typename TI>
__global__ void k_adj_pm_final(Grid g, int d, double dt, double c1, double c2, const TI* lo_dd, const TI* hi_dd, KI<TI> AD, const TI* T1,
                               const TI* T2, const double* forces, const double* macb, double* lo_ddb, double* hi_ddb, A3 ADb, double* T1b,
                               double* T2b, double* forcesb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    if (d == 2 && !g.zper && (k == 0 || k == g.nz)) return;  // wall faces: the normal velocity is 0 whatever the input
    const long long f = t;
    const double mb = macb[f];
    if (!(dbits(mb) & kMag)) return;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    auto side_val = [&](int ci, int cj, int ck, double base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        // the forward's sum in its own precision (decides the Riemann branch)
        const TI tc1 = (TI)c1, tc2 = (TI)c2;
        TI s = (TI)base;
        s -= tc1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= tc2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        s += TI(0.5) * (TI)dt * (TI)forces[d * g.N + cell_fo(g, ci, cj, ck)];
        return (double)s;
    };
    auto side_rev = [&](int ci, int cj, int ck, double sb) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        const double S1 = (double)AD.p[b1][p1] + AD.p[b1][m1], D1 = (double)T1[p1] - T1[m1];
        const double S2 = (double)AD.p[b2][p2] + AD.p[b2][m2], D2 = (double)T2[p2] - T2[m2];
        aadd(&ADb.p[b1][p1], -c1 * D1 * sb);
        aadd(&ADb.p[b1][m1], -c1 * D1 * sb);
        aadd(&T1b[p1], -c1 * S1 * sb);
        aadd(&T1b[m1], c1 * S1 * sb);
        aadd(&ADb.p[b2][p2], -c2 * D2 * sb);
        aadd(&ADb.p[b2][m2], -c2 * D2 * sb);
        aadd(&T2b[p2], -c2 * S2 * sb);
        aadd(&T2b[m2], c2 * S2 * sb);
        aadd(&forcesb[d * g.N + cell_fo(g, ci, cj, ck)], 0.5 * dt * sb);
    };
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const double stl = side_val(li, lj, lk, lo_dd[f]), sth = side_val(i, j, k, hi_dd[f]);
    double bl = 0.0, bh = 0.0;
    rev_riemann(stl, sth, mb, bl, bh);
    if ((dbits(bl) & kMag)) {
        lo_ddb[f] += bl;
        side_rev(li, lj, lk, bl);
    }
    if ((dbits(bh) & kMag)) {
        hi_ddb[f] += bh;
        side_rev(i, j, k, bh);
    }
}

// ---- reverse of k_adv_trans (a, b): out_n = upwind(u_a; l, h),
// h = HI + (-cb (vp E(h1) - vm E(h0)) + cb q(c) (vp - vm)), l likewise at c - e_a
template <typename TI>
__global__ void k_adj_adv_trans(Grid g, int a, int b, const double* u, double rho, double cb, const double* ua, const double* vb, KI<TI> E,
                                K3 Ob, A3 LOb, A3 HIb, A3 Ebb, double* vbb, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, a, t, i, j, k)) return;
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    const long long f = t;
    const double uaf = (TI)ua[f];
    const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
    const long long h0 = fidx(g, b, i, j, k), h1 = fidx(g, b, i + (b == 0), j + (b == 1), k + (b == 2));
    const long long l0 = fidx(g, b, ci, cj, ck), l1 = fidx(g, b, ci + (b == 0), cj + (b == 1), ck + (b == 2));
    double vhp = 0.0, vhm = 0.0, vlp = 0.0, vlm = 0.0;
    if (!wh) {
        vhp = (TI)vb[h1];
        vhm = (TI)vb[h0];
    }
    if (!wl) {
        vlp = (TI)vb[l1];
        vlm = (TI)vb[l0];
    }
    double gvhp = 0.0, gvhm = 0.0, gvlp = 0.0, gvlm = 0.0;
    for (int n = 0; n < 3; ++n) {
        const double ob = Ob.p[n][f];
        if (!(dbits(ob) & kMag)) continue;
        double lb = 0.0, hb = 0.0;
        rev_upwind(uaf, ob, lb, hb);
        if (a == 2) zbc_rev(g, k, n, lb, hb);
        LOb.p[n][f] += lb;
        HIb.p[n][f] += hb;
        if (!wh && (dbits(hb) & kMag)) {
            const double qc = (TI)rho * (TI)Q(g, u, n, i, j, k);
            aadd(&Ebb.p[n][h1], -cb * vhp * hb);
            aadd(&Ebb.p[n][h0], cb * vhm * hb);
            gvhp += (-cb * E.p[n][h1] + cb * qc) * hb;
            gvhm += (cb * E.p[n][h0] - cb * qc) * hb;
            Qb(g, ub, n, i, j, k, rho * cb * (vhp - vhm) * hb);
        }
        if (!wl && (dbits(lb) & kMag)) {
            const double qc = (TI)rho * (TI)Q(g, u, n, ci, cj, ck);
            aadd(&Ebb.p[n][l1], -cb * vlp * lb);
            aadd(&Ebb.p[n][l0], cb * vlm * lb);
            gvlp += (-cb * E.p[n][l1] + cb * qc) * lb;
            gvlm += (cb * E.p[n][l0] - cb * qc) * lb;
            Qb(g, ub, n, ci, cj, ck, rho * cb * (vlp - vlm) * lb);
        }
    }
    aadd(&vbb[h1], gvhp);
    aadd(&vbb[h0], gvhm);
    aadd(&vbb[l1], gvlp);
    aadd(&vbb[l0], gvlm);
}

// ---- reverse of k_adv_flux (d) with the flux adjoint Fb given
template <typename TI>
__global__ void k_adj_adv_flux(Grid g, int d, const double* u, const double* forces, double rho, double dt, double c1, double c2, K3 Uf,
                               KI<TI> LO, KI<TI> HI, KI<TI> T1, KI<TI> T2, K3 Fb, A3 Ufb, A3 LOb, A3 HIb, A3 T1b, A3 T2b, double* ub,
                               double* forcesb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = t;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const double um = (TI)Uf.p[d][f];
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const long long lp1 = fidx(g, b1, li + (b1 == 0), lj + (b1 == 1), lk + (b1 == 2)), lm1 = fidx(g, b1, li, lj, lk);
    const long long lp2 = fidx(g, b2, li + (b2 == 0), lj + (b2 == 1), lk + (b2 == 2)), lm2 = fidx(g, b2, li, lj, lk);
    const long long hp1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), hm1 = fidx(g, b1, i, j, k);
    const long long hp2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), hm2 = fidx(g, b2, i, j, k);
    double l1p = 0, l1m = 0, l2p = 0, l2m = 0, h1p = 0, h1m = 0, h2p = 0, h2m = 0;
    if (!wl) {
        l1p = (TI)Uf.p[b1][lp1];
        l1m = (TI)Uf.p[b1][lm1];
        l2p = (TI)Uf.p[b2][lp2];
        l2m = (TI)Uf.p[b2][lm2];
    }
    if (!wh) {
        h1p = (TI)Uf.p[b1][hp1];
        h1m = (TI)Uf.p[b1][hm1];
        h2p = (TI)Uf.p[b2][hp2];
        h2m = (TI)Uf.p[b2][hm2];
    }
    double gum = 0, gl1p = 0, gl1m = 0, gl2p = 0, gl2m = 0, gh1p = 0, gh1m = 0, gh2p = 0, gh2m = 0;
    const long long cl = wl ? 0 : cell_fo(g, li, lj, lk);
    const long long ch = wh ? 0 : cell_fo(g, i, j, k);
    for (int n = 0; n < 3; ++n) {
        const double fb = Fb.p[n][f];
        if (!(dbits(fb) & kMag)) continue;
        // the forward's face states in its own precision (decide the upwind branch)
        const TI tr = (TI)rho, tc1 = (TI)c1, tc2 = (TI)c2, thd = TI(0.5) * (TI)dt;
        double ql = 0.0, qh = 0.0, stl = 0.0, sth = 0.0;
        if (!wl) {
            const TI q = tr * (TI)u[n * g.N + cl];
            ql = q;
            TI s_ = LO.p[n][f];
            s_ -= tc1 * (T1.p[n][lp1] * (TI)l1p - T1.p[n][lm1] * (TI)l1m);
            s_ -= tc2 * (T2.p[n][lp2] * (TI)l2p - T2.p[n][lm2] * (TI)l2m);
            s_ += tc1 * q * (TI)(l1p - l1m);
            s_ += tc2 * q * (TI)(l2p - l2m);
            s_ += thd * (tr * (TI)forces[n * g.N + cl]);
            stl = s_;
        }
        if (!wh) {
            const TI q = tr * (TI)u[n * g.N + ch];
            qh = q;
            TI s_ = HI.p[n][f];
            s_ -= tc1 * (T1.p[n][hp1] * (TI)h1p - T1.p[n][hm1] * (TI)h1m);
            s_ -= tc2 * (T2.p[n][hp2] * (TI)h2p - T2.p[n][hm2] * (TI)h2m);
            s_ += tc1 * q * (TI)(h1p - h1m);
            s_ += tc2 * q * (TI)(h2p - h2m);
            s_ += thd * (tr * (TI)forces[n * g.N + ch]);
            sth = s_;
        }
        double zl = stl, zh = sth;
        if (d == 2) zbc_fwd(g, k, n, zl, zh);
        double st, bl = 0.0, bh = 0.0;
        if (iabs_lt(um, kSV)) {
            st = 0.5 * (zl + zh);
            bl = bh = 0.5 * um * fb;
        } else if (ige0(um)) {
            st = zl;
            bl = um * fb;
        } else {
            st = zh;
            bh = um * fb;
        }
        gum += st * fb;
        if (d == 2) zbc_rev(g, k, n, bl, bh);
        if (!wl && (dbits(bl) & kMag)) {
            LOb.p[n][f] += bl;
            aadd(&T1b.p[n][lp1], -c1 * l1p * bl);
            aadd(&T1b.p[n][lm1], c1 * l1m * bl);
            aadd(&T2b.p[n][lp2], -c2 * l2p * bl);
            aadd(&T2b.p[n][lm2], c2 * l2m * bl);
            gl1p += (-c1 * T1.p[n][lp1] + c1 * ql) * bl;
            gl1m += (c1 * T1.p[n][lm1] - c1 * ql) * bl;
            gl2p += (-c2 * T2.p[n][lp2] + c2 * ql) * bl;
            gl2m += (c2 * T2.p[n][lm2] - c2 * ql) * bl;
            aadd(&ub[n * g.N + cl], rho * (c1 * (l1p - l1m) + c2 * (l2p - l2m)) * bl);
            aadd(&forcesb[n * g.N + cl], 0.5 * dt * rho * bl);
        }
        if (!wh && (dbits(bh) & kMag)) {
            HIb.p[n][f] += bh;
            aadd(&T1b.p[n][hp1], -c1 * h1p * bh);
            aadd(&T1b.p[n][hm1], c1 * h1m * bh);
            aadd(&T2b.p[n][hp2], -c2 * h2p * bh);
            aadd(&T2b.p[n][hm2], c2 * h2m * bh);
            gh1p += (-c1 * T1.p[n][hp1] + c1 * qh) * bh;
            gh1m += (c1 * T1.p[n][hm1] - c1 * qh) * bh;
            gh2p += (-c2 * T2.p[n][hp2] + c2 * qh) * bh;
            gh2m += (c2 * T2.p[n][hm2] - c2 * qh) * bh;
            aadd(&ub[n * g.N + ch], rho * (c1 * (h1p - h1m) + c2 * (h2p - h2m)) * bh);
            aadd(&forcesb[n * g.N + ch], 0.5 * dt * rho * bh);
        }
    }
    aadd(&Ufb.p[d][f], gum);
    aadd(&Ufb.p[b1][lp1], gl1p);
    aadd(&Ufb.p[b1][lm1], gl1m);
    aadd(&Ufb.p[b2][lp2], gl2p);
    aadd(&Ufb.p[b2][lm2], gl2m);
    aadd(&Ufb.p[b1][hp1], gh1p);
    aadd(&Ufb.p[b1][hm1], gh1m);
    aadd(&Ufb.p[b2][hp2], gh2p);
    aadd(&Ufb.p[b2][hm2], gh2m);
}

// ---- reverse of conv = -div F on d-faces: Fb(f) = (convb(cell above f) - convb(cell below f)) / h_d
__global__ void k_adj_div(Grid g, int d, const double* convb, double* F0, double* F1, double* F2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const bool has_hi = !(d == 2 && !g.zper && k == g.nz), has_lo = !(d == 2 && !g.zper && k == 0);
    const long long ch = has_hi ? cidx(g, i, j, k) : 0;
    const long long cl = has_lo ? cidx(g, wrapn(i - (d == 0), g.nx), wrapn(j - (d == 1), g.ny), g.zper ? wrapn(k - (d == 2), g.nz) : k - (d == 2)) : 0;
    const double ih = ihd(g, d);
    double* F[3] = {F0, F1, F2};
    for (int n = 0; n < 3; ++n)
        F[n][t] = ((has_hi ? convb[n * g.N + ch] : 0.0) - (has_lo ? convb[n * g.N + cl] : 0.0)) * ih;
}

// ---- tensor diffusion: the velocity seen by the flux stencil (VelDiff of the
// forward) and its adjoint
__device__ inline double Vd(const Grid& g, const double* v, const double* wg, int n, int i, int j, int k) {
    i = wrapn(i, g.nx);
    j = wrapn(j, g.ny);
    const double* c = v + (long long)n * g.N;
    if (g.zper) return c[cidx(g, i, j, wrapn(k, g.nz))];
    if (k < 0) {
        const double q0 = c[cidx(g, i, j, 0)];
        if (n == 2) return -q0;
        if (g.zlo == ZWALLMODEL) return q0 - wg[(long long)n * g.nx * g.ny + (long long)j * g.nx + i] * g.dz;
        return q0;
    }
    if (k >= g.nz) {
        const double q0 = c[cidx(g, i, j, g.nz - 1)];
        return n == 2 ? -q0 : q0;
    }
    return c[cidx(g, i, j, k)];
}
__device__ inline void Vdb(const Grid& g, double* ub, double* wgb, int n, int i, int j, int k, double v) {
    if (!(dbits(v) & kMag)) return;
    i = wrapn(i, g.nx);
    j = wrapn(j, g.ny);
    double* c = ub + (long long)n * g.N;
    if (g.zper) {
        atomicAdd(c + cidx(g, i, j, wrapn(k, g.nz)), v);
        return;
    }
    if (k < 0) {
        if (n == 2) {
            atomicAdd(c + cidx(g, i, j, 0), -v);
            return;
        }
        if (g.zlo == ZWALLMODEL && wgb) atomicAdd(wgb + (long long)n * g.nx * g.ny + (long long)j * g.nx + i, -v * g.dz);
        atomicAdd(c + cidx(g, i, j, 0), v);
        return;
    }
    if (k >= g.nz) {
        atomicAdd(c + cidx(g, i, j, g.nz - 1), n == 2 ? -v : v);
        return;
    }
    atomicAdd(c + cidx(g, i, j, k), v);
}

// ---- tiled form of k_adj_tau.  A block owns the faces at the low side of a
// TX x TY x TZ tile of cells (plus the top wall faces when the tile holds the
// last cell layer), stages the diffusion velocity (VelDiff ghosts included),
// mu_eff and the divergence adjoint of the tile and a one-cell halo in shared
// memory, scatters the face contributions into shared accumulators over the
// same box, and flushes them with one global atomic per box cell, mapping
// ghost positions back to the cells (and wall-model gradients) they come from.
constexpr int ATX = 32, ATY = 4, ATZ = 4;
constexpr int AHX = ATX + 2, AHY = ATY + 2, AHZ = ATZ + 2;
constexpr int ANH = AHX * AHY * AHZ;
constexpr size_t ADJ_TAU_SMEM = sizeof(double) * 11 * (size_t)ANH;

__global__ void __launch_bounds__(ATX* ATY* ATZ) k_adj_tau_tile(Grid g, const double* vel, const double* mu, const double* wg,
                                                                const double* db, double s, double* ub, double* mub, double* wgb) {
    extern __shared__ double sm[];
    double* sV = sm;              // [3][box]
    double* sD = sm + 3 * ANH;    // [3][box] divergence adjoint (cells in the domain, else 0)
    double* sM = sm + 6 * ANH;    // [box]
    double* aU = sm + 7 * ANH;    // [3][box] accumulated velocity adjoint
    double* aM = sm + 10 * ANH;   // [box] accumulated viscosity adjoint
    const int i0 = blockIdx.x * ATX, j0 = blockIdx.y * ATY, k0 = blockIdx.z * ATZ;
    const int tid = threadIdx.x, nthr = ATX * ATY * ATZ;
    auto hb = [](int hx, int hy, int hz) { return (hz * AHY + hy) * AHX + hx; };
    for (int h = tid; h < ANH; h += nthr) {
        const int hx = h % AHX, hy = (h / AHX) % AHY, hz = h / (AHX * AHY);
        const int gi = ((i0 + hx - 1) % g.nx + g.nx) % g.nx, gj = ((j0 + hy - 1) % g.ny + g.ny) % g.ny;
        int gk = k0 + hz - 1;
        const bool inz = g.zper || (gk >= 0 && gk < g.nz);
        if (g.zper) gk = (gk % g.nz + g.nz) % g.nz;
        for (int n = 0; n < 3; ++n) sV[n * ANH + h] = Vd(g, vel, wg, n, gi, gj, gk);
        const int kk = g.zper ? gk : (gk < 0 ? 0 : (gk >= g.nz ? g.nz - 1 : gk));
        const long long c = cidx(g, gi, gj, kk);
        sM[h] = mu[c];
        for (int n = 0; n < 3; ++n) {
            sD[n * ANH + h] = inz ? s * db[n * g.N + c] : 0.0;
            aU[n * ANH + h] = 0.0;
        }
        aM[h] = 0.0;
    }
    __syncthreads();
    const double ih[3] = {g.idx, g.idy, g.idz};
    const bool top = !g.zper && k0 + ATZ >= g.nz;  // this tile also owns the top wall faces
    const int nface = 3 * nthr + (top ? ATX * ATY : 0);
    for (int q = tid; q < nface; q += nthr) {
        int d, tx, ty, tz;
        if (q < 3 * nthr) {
            d = q / nthr;
            const int r = q % nthr;
            tx = r % ATX;
            ty = (r / ATX) % ATY;
            tz = r / (ATX * ATY);
        } else {
            d = 2;
            const int r = q - 3 * nthr;
            tx = r % ATX;
            ty = r / ATX;
            tz = g.nz - k0;  // face k = nz
        }
        const int gi = i0 + tx, gj = j0 + ty, gk = k0 + tz;
        if (gi >= g.nx || gj >= g.ny) continue;
        if (q < 3 * nthr && gk >= g.nz) continue;
        const int e0 = (d == 0), e1 = (d == 1), e2 = (d == 2);
        const int hx = tx + 1, hy = ty + 1, hz = tz + 1;     // cell above the face
        const int mx = hx - e0, my = hy - e1, mz = hz - e2;  // cell below
        const bool has_hi = !(d == 2 && !g.zper && gk == g.nz), has_lo = !(d == 2 && !g.zper && gk == 0);
        double Fb[3];
        bool any = false;
        for (int n = 0; n < 3; ++n) {
            Fb[n] = ((has_lo ? sD[n * ANH + hb(mx, my, mz)] : 0.0) - (has_hi ? sD[n * ANH + hb(hx, hy, hz)] : 0.0)) * ih[d];
            any = any || (dbits(Fb[n]) & kMag);
        }
        if (!any) continue;
        double mf;
        if (!has_lo) mf = sM[hb(hx, hy, hz)];
        else if (!has_hi) mf = sM[hb(mx, my, mz)];
        else mf = 0.5 * (sM[hb(mx, my, mz)] + sM[hb(hx, hy, hz)]);
        double gr[3][3];
        for (int n = 0; n < 3; ++n) {
            const double* v = sV + n * ANH;
            for (int m = 0; m < 3; ++m) {
                if (m == d) {
                    gr[m][n] = (v[hb(hx, hy, hz)] - v[hb(mx, my, mz)]) * ih[m];
                } else {
                    const int f0 = (m == 0), f1 = (m == 1), f2 = (m == 2);
                    gr[m][n] = 0.25 *
                               (v[hb(hx + f0, hy + f1, hz + f2)] + v[hb(mx + f0, my + f1, mz + f2)] - v[hb(hx - f0, hy - f1, hz - f2)] -
                                v[hb(mx - f0, my - f1, mz - f2)]) *
                               ih[m];
                }
            }
        }
        const double dv = gr[0][0] + gr[1][1] + gr[2][2];
        double mfb = 0.0, dvb = 0.0;
        double grb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int n = 0; n < 3; ++n) {
            const double Sn = (n == d) ? (2.0 * gr[d][d] - (2.0 / 3.0) * dv) : (gr[d][n] + gr[n][d]);
            mfb += Fb[n] * Sn;
            const double sb = mf * Fb[n];
            if (n == d) {
                grb[d][d] += 2.0 * sb;
                dvb += -(2.0 / 3.0) * sb;
            } else {
                grb[d][n] += sb;
                grb[n][d] += sb;
            }
        }
        for (int m = 0; m < 3; ++m) grb[m][m] += dvb;
        if (!has_lo) atomicAdd(&aM[hb(hx, hy, hz)], mfb);
        else if (!has_hi) atomicAdd(&aM[hb(mx, my, mz)], mfb);
        else {
            atomicAdd(&aM[hb(mx, my, mz)], 0.5 * mfb);
            atomicAdd(&aM[hb(hx, hy, hz)], 0.5 * mfb);
        }
        for (int n = 0; n < 3; ++n) {
            double* a = aU + n * ANH;
            for (int m = 0; m < 3; ++m) {
                const double b = grb[m][n];
                if (!(dbits(b) & kMag)) continue;
                if (m == d) {
                    atomicAdd(&a[hb(hx, hy, hz)], b * ih[m]);
                    atomicAdd(&a[hb(mx, my, mz)], -b * ih[m]);
                } else {
                    const int f0 = (m == 0), f1 = (m == 1), f2 = (m == 2);
                    const double w = 0.25 * b * ih[m];
                    atomicAdd(&a[hb(hx + f0, hy + f1, hz + f2)], w);
                    atomicAdd(&a[hb(mx + f0, my + f1, mz + f2)], w);
                    atomicAdd(&a[hb(hx - f0, hy - f1, hz - f2)], -w);
                    atomicAdd(&a[hb(mx - f0, my - f1, mz - f2)], -w);
                }
            }
        }
    }
    __syncthreads();
    // flush: box positions to cells (ghost positions through the diffusion ghost rules)
    for (int h = tid; h < ANH; h += nthr) {
        const int hx = h % AHX, hy = (h / AHX) % AHY, hz = h / (AHX * AHY);
        const int gi = ((i0 + hx - 1) % g.nx + g.nx) % g.nx, gj = ((j0 + hy - 1) % g.ny + g.ny) % g.ny;
        const int gk = k0 + hz - 1;
        for (int n = 0; n < 3; ++n) Vdb(g, ub, wgb, n, gi, gj, gk, aU[n * ANH + h]);
        if (mub && (dbits(aM[h]) & kMag)) {
            if (g.zper || (gk >= 0 && gk < g.nz)) atomicAdd(&mub[cidx(g, gi, gj, g.zper ? (gk % g.nz + g.nz) % g.nz : gk)], aM[h]);
        }
    }
}

// ---- reverse of the Smagorinsky viscosity mu_eff = mu + rho fac |S|(u)
__global__ void k_adj_smag(Grid g, const double* vel, const double* mub, double rho, double fac, double* ub) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const double mb = mub[t];
    if (!(dbits(mb) & kMag)) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    double a = 0.5, b = 0.0, c = -0.5;
    if (!g.zper && k == 0) {
        a = 1.0 / 3.0;
        b = 1.0;
        c = -4.0 / 3.0;
    }
    if (!g.zper && k == g.nz - 1) {
        a = 4.0 / 3.0;
        b = -1.0;
        c = -1.0 / 3.0;
    }
    double gx[3], gy[3], gz[3];
    for (int n = 0; n < 3; ++n) {
        gx[n] = 0.5 * (Q(g, vel, n, i + 1, j, k) - Q(g, vel, n, i - 1, j, k)) * g.idx;
        gy[n] = 0.5 * (Q(g, vel, n, i, j + 1, k) - Q(g, vel, n, i, j - 1, k)) * g.idy;
        gz[n] = (a * Q(g, vel, n, i, j, k + 1) + b * Q(g, vel, n, i, j, k) + c * Q(g, vel, n, i, j, k - 1)) * g.idz;
    }
    const double S = sqrt(2.0 * gx[0] * gx[0] + 2.0 * gy[1] * gy[1] + 2.0 * gz[2] * gz[2] + (gy[0] + gx[1]) * (gy[0] + gx[1]) +
                          (gz[1] + gy[2]) * (gz[1] + gy[2]) + (gx[2] + gz[0]) * (gx[2] + gz[0]));
    if (!(S > 0.0)) return;
    const double q = rho * fac * mb / S;
    double gxb[3] = {2.0 * q * gx[0], 0.0, 0.0}, gyb[3] = {0.0, 2.0 * q * gy[1], 0.0}, gzb[3] = {0.0, 0.0, 2.0 * q * gz[2]};
    const double t1 = q * (gy[0] + gx[1]), t2 = q * (gz[1] + gy[2]), t3 = q * (gx[2] + gz[0]);
    gyb[0] += t1;
    gxb[1] += t1;
    gzb[1] += t2;
    gyb[2] += t2;
    gxb[2] += t3;
    gzb[0] += t3;
    for (int n = 0; n < 3; ++n) {
        Qb(g, ub, n, i + 1, j, k, 0.5 * g.idx * gxb[n]);
        Qb(g, ub, n, i - 1, j, k, -0.5 * g.idx * gxb[n]);
        Qb(g, ub, n, i, j + 1, k, 0.5 * g.idy * gyb[n]);
        Qb(g, ub, n, i, j - 1, k, -0.5 * g.idy * gyb[n]);
        Qb(g, ub, n, i, j, k + 1, a * g.idz * gzb[n]);
        Qb(g, ub, n, i, j, k, b * g.idz * gzb[n]);
        Qb(g, ub, n, i, j, k - 1, c * g.idz * gzb[n]);
    }
}

__device__ inline double block_sum(double v, double* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// ---- reverse of the Moeng wall stress (k_wall_grad), local part.  wg =
// tau rho / mu_eff of the first cell layer, tau_x = ut2 ((u - um0) vm +
// |u_h| um0) / vm^2 (tau_y likewise with v, um1).  Accumulates the first-layer
// velocity and viscosity adjoints and block sums of the adjoints of the plane
// means um0, um1, vm and of ut2 = u_tau^2.
__global__ void k_adj_wall_local(Grid g, const double* vel, const double* mueff, const double* wgb, double ut2, double um0, double um1,
                                 double vm, double rho, double* ub, double* mub, double* parts, int np) {
    __shared__ double sh[256];
    const long long M = (long long)g.nx * g.ny;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const double u = vel[t], v = vel[g.N + t];
        const double ws = sqrt(u * u + v * v), iws = ws > 0.0 ? 1.0 / ws : 0.0;
        const double m = mueff[t];
        const double c = ut2 / (vm * vm);
        const double tx = ((u - um0) * vm + ws * um0) * c, ty = ((v - um1) * vm + ws * um1) * c;
        const double bx = wgb[t] * rho / m, by = wgb[M + t] * rho / m;
        if (!(dbits(bx) & kMag) && !(dbits(by) & kMag)) continue;
        mub[t] += -(bx * tx + by * ty) / m;
        ub[t] += bx * c * (vm + um0 * u * iws) + by * c * um1 * u * iws;
        ub[g.N + t] += by * c * (vm + um1 * v * iws) + bx * c * um0 * v * iws;
        s0 += bx * c * (ws - vm);
        s1 += by * c * (ws - vm);
        s2 += ut2 * (bx * (-(u - um0) / (vm * vm) - 2.0 * ws * um0 / (vm * vm * vm)) +
                     by * (-(v - um1) / (vm * vm) - 2.0 * ws * um1 / (vm * vm * vm)));
        s3 += (bx * tx + by * ty) / ut2;
    }
    s0 = block_sum(s0, sh);
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    s3 = block_sum(s3, sh);
    if (threadIdx.x == 0) {
        parts[blockIdx.x] = s0;
        parts[np + blockIdx.x] = s1;
        parts[2 * np + blockIdx.x] = s2;
        parts[3 * np + blockIdx.x] = s3;
    }
}

// plane means um0 = <u>, um1 = <v>, vm = <|u_h|> of the first layer: spread
// their adjoints (already divided by nx ny) back to the cells
__global__ void k_adj_wall_global(Grid g, const double* vel, double bu, double bv, double bm, double* ub) {
    const long long M = (long long)g.nx * g.ny;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    const double u = vel[t], v = vel[g.N + t];
    const double ws = sqrt(u * u + v * v), iws = ws > 0.0 ? 1.0 / ws : 0.0;
    ub[t] += bu + bm * u * iws;
    ub[g.N + t] += bv + bm * v * iws;
}

// ---- reverse of the Coriolis source src = rho (C u): u_bar += rho C^T src_bar
__global__ void k_adj_coriolis(Grid g, const double* srcb, Scalars s, double* ub) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const long long N = g.N;
    double fb[3];
    for (int n = 0; n < 3; ++n) fb[n] = s.rho * srcb[n * N + t];
    const double aeb = fb[0] * s.east[0] + fb[1] * s.east[1] + fb[2] * s.east[2];
    const double anb = fb[0] * s.north[0] + fb[1] * s.north[1] + fb[2] * s.north[2];
    const double aub = fb[0] * s.up[0] + fb[1] * s.up[1] + fb[2] * s.up[2];
    const double unb = s.corfac * s.sinphi * aeb;
    const double uub = -s.hfac * s.corfac * s.cosphi * aeb;
    const double ueb = -s.corfac * s.sinphi * anb + s.hfac * s.corfac * s.cosphi * aub;
    for (int n = 0; n < 3; ++n) ub[n * N + t] += ueb * s.east[n] + unb * s.north[n] + uub * s.up[n];
}

// ---- nodal projection adjoint: out = ub + Gn psi
__global__ void k_adj_nodal_post(Grid g, const double* psi, const double* ub, double* out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    auto P = [&](int a, int b, int c) {
        return psi[((long long)(g.zper ? wrapn(c, g.nz) : c) * g.ny + wrapn(b, g.ny)) * g.nx + wrapn(a, g.nx)];
    };
    double gx = 0, gy = 0, gz = 0;
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b) {
            gx += P(i + 1, j + b, k + c) - P(i, j + b, k + c);
            gy += P(i + b, j + 1, k + c) - P(i + b, j, k + c);
            gz += P(i + b, j + c, k + 1) - P(i + b, j + c, k);
        }
    out[t] = ub[t] + 0.25 * gx * g.idx;
    out[g.N + t] = ub[g.N + t] + 0.25 * gy * g.idy;
    out[2 * g.N + t] = ub[2 * g.N + t] + 0.25 * gz * g.idz;
}

// ---- elementwise helpers
__global__ void k_axpby(long long n, double a, const double* x, double b, const double* y, double* out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) out[t] = a * x[t] + b * y[t];
}

// objective: J = (1/M) sum_box 0.5 |u|^2 ; its gradient u/M in the box
__global__ void k_objective(Grid g, const double* u, int lo0, int lo1, int lo2, int hi0, int hi1, int hi2, double invM, double* ub,
                            double* parts) {
    __shared__ double sh[256];
    double s = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.nx);
        const long long r = t / g.nx;
        const int j = (int)(r % g.ny), k = (int)(r / g.ny);
        const bool in = i >= lo0 && i <= hi0 && j >= lo1 && j <= hi1 && k >= lo2 && k <= hi2;
        for (int n = 0; n < 3; ++n) {
            const double v = u[n * g.N + t];
            if (in) s += 0.5 * v * v;
            if (ub) ub[n * g.N + t] = in ? v * invM : 0.0;
        }
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) parts[blockIdx.x] = s * invM;
}

// disk adjoint: partial sums over the cut-off box of  sum_x (actb(x) . n) B(x),
// B(x) = sum_points w_p g3(x - p) with the per-point weights w_p in pts[4p+3]
__global__ void k_act_adj_dot(Grid g, const double* actb, const double* pts, int npts, double ax0, double ax1, double ax2, double eps, double x0,
                              double y0, double z0, int lo0, int lo1, int lo2, int n0, int n1, int n2, double* parts) {
    __shared__ double sh[256];
    double acc = 0.0;
    const long long M = (long long)n0 * n1 * n2;
    const double gfac = 0.17958712212516656 / (eps * eps * eps);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(t % n0);
        const long long r = t / n0;
        const int b = (int)(r % n1), c = (int)(r / n1);
        const int i = lo0 + a, j = lo1 + b, k = lo2 + c;
        const double x = x0 + (i + 0.5) * g.dx, y = y0 + (j + 0.5) * g.dy, z = z0 + (k + 0.5) * g.dz;
        double s = 0;
        for (int m = 0; m < npts; ++m) {
            const double rx = (pts[4 * m] - x) / eps, ry = (pts[4 * m + 1] - y) / eps, rz = (pts[4 * m + 2] - z) / eps;
            const double r2 = rx * rx + ry * ry + rz * rz;
            if (r2 < 16.0) s += gfac * exp(-rx * rx - ry * ry - rz * rz) * pts[4 * m + 3];
        }
        const long long cc = cidx(g, i, j, k);
        acc += s * (actb[cc] * ax0 + actb[g.N + cc] * ax1 + actb[2 * g.N + cc] * ax2);
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) parts[blockIdx.x] = acc;
}

// scatter of the sampled-velocity adjoint to the trilinear corners
__global__ void k_act_sample_adj(Grid g, const double* pts, const double* wb, int npts, double x0, double y0, double z0, double* ub) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double fx = (pts[3 * p] - x0 - 0.5 * g.dx) / g.dx;
    const double fy = (pts[3 * p + 1] - y0 - 0.5 * g.dy) / g.dy;
    const double fz = (pts[3 * p + 2] - z0 - 0.5 * g.dz) / g.dz;
    const int i = (int)floor(fx), j = (int)floor(fy), k = (int)floor(fz);
    const double wx = fx - i, wy = fy - j, wz = fz - k;
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                const double w = (a ? wx : 1 - wx) * (b ? wy : 1 - wy) * (c ? wz : 1 - wz);
                for (int n = 0; n < 3; ++n) Qb(g, ub, n, i + a, j + b, k + c, w * wb[3 * p + n]);
            }
}

}  // namespace

// ---------------------------------------------------------------- launchers
constexpr double B8 = 8.0;

template <typename TI>
static const TI* ti(void* p) {
    return static_cast<const TI*>(p);
}

void launch_adj_edges(Ctx& c, const Grid& g, int d, const double* u, double* const Eb[3], double* ub, int fp32) {
    const long long nf = nfaces(g, d);
    if (fp32)
        KS_LAUNCH(c, k_adj_edges<float>, nblocks(nf, BS), BS, B8 * (3.0 * nf + 6.0 * g.N), g, d, u, Eb[0], Eb[1], Eb[2], ub);
    else
        KS_LAUNCH(c, k_adj_edges<double>, nblocks(nf, BS), BS, B8 * (3.0 * nf + 6.0 * g.N), g, d, u, Eb[0], Eb[1], Eb[2], ub);
}

template <typename TI>
static void adj_faces_t(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                        const double* umac_d) {
    KI<TI> E{{ti<TI>(B.edge[d][0]), ti<TI>(B.edge[d][1]), ti<TI>(B.edge[d][2])}};
    KI<TI> LO{{ti<TI>(B.lo[d][0]), ti<TI>(B.lo[d][1]), ti<TI>(B.lo[d][2])}}, HI{{ti<TI>(B.hi[d][0]), ti<TI>(B.hi[d][1]), ti<TI>(B.hi[d][2])}};
    K3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    K3 TEb{{A.tedge[d][0], A.tedge[d][1], A.tedge[d][2]}};
    A3 Eb{{A.edge[d][0], A.edge[d][1], A.edge[d][2]}};
    const double s = dt * ihd(g, d);
    const long long nf = nfaces(g, d);
    const double bytes = B8 * (6.0 * g.N + 13.0 * nf) + sizeof(TI) * 9.0 * nf;
    if (mode == 0)
        KS_LAUNCH(c, (k_adj_faces<0, TI>), nblocks(nf, BS), BS, bytes, g, d, u, E, s, rho, nullptr, LO, HI, ti<TI>(B.ad[d]), LOb, HIb, A.ad[d], TEb,
                  Eb, A.u, nullptr);
    else
        KS_LAUNCH(c, (k_adj_faces<1, TI>), nblocks(nf, BS), BS, bytes, g, d, u, E, s, rho, umac_d, LO, HI, (const TI*)nullptr, LOb, HIb, nullptr,
                  TEb, Eb, A.u, A.umac[d]);
}
void launch_adj_faces(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                      const double* umac_d, int fp32) {
    if (fp32) adj_faces_t<float>(c, g, d, mode, u, B, A, dt, rho, umac_d);
    else adj_faces_t<double>(c, g, d, mode, u, B, A, dt, rho, umac_d);
}

template <typename TI>
static void adj_pm_trans_t(Ctx& c, const Grid& g, int a, int b, int n, double dt, const GodunovBufs& B, const AdjBufs& A) {
    const double cb = dt / (6.0 * hd(g, b));
    const long long na = nfaces(g, a), nb = nfaces(g, b);
    KS_LAUNCH(c, k_adj_pm_trans<TI>, nblocks(na, BS), BS, B8 * (3.0 * na + 2.0 * nb) + sizeof(TI) * (na + 2.0 * nb), g, a, b, n, cb,
              ti<TI>(B.ad[a]), ti<TI>(B.ad[b]), ti<TI>(B.tedge[b][n]), A.tr[a][b][0], A.lo[a][n], A.hi[a][n], A.ad[b], A.tedge[b][n]);
}
void launch_adj_pm_trans(Ctx& c, const Grid& g, int a, int b, int n, double dt, const GodunovBufs& B, const AdjBufs& A, int fp32) {
    if (fp32) adj_pm_trans_t<float>(c, g, a, b, n, dt, B, A);
    else adj_pm_trans_t<double>(c, g, a, b, n, dt, B, A);
}

template <typename TI>
static void adj_pm_final_t(Ctx& c, const Grid& g, int d, double dt, const GodunovBufs& B, const double* forces, const AdjBufs& A) {
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    KI<TI> AD{{ti<TI>(B.ad[0]), ti<TI>(B.ad[1]), ti<TI>(B.ad[2])}};
    A3 ADb{{A.ad[0], A.ad[1], A.ad[2]}};
    const long long nf = nfaces(g, d);
    KS_LAUNCH(c, k_adj_pm_final<TI>, nblocks(nf, BS), BS, B8 * (2.0 * g.N + 3.0 * nf + 3.0 * (nfaces(g, b1) + nfaces(g, b2))) +
              sizeof(TI) * (2.0 * nf + 2.0 * (nfaces(g, b1) + nfaces(g, b2))), g, d, dt, dt / (4.0 * hd(g, b1)), dt / (4.0 * hd(g, b2)),
              ti<TI>(B.lo[d][d]), ti<TI>(B.hi[d][d]), AD, ti<TI>(B.tr[b1][b2][0]), ti<TI>(B.tr[b2][b1][0]), forces, A.umac[d], A.lo[d][d],
              A.hi[d][d], ADb, A.tr[b1][b2][0], A.tr[b2][b1][0], A.forces);
}
void launch_adj_pm_final(Ctx& c, const Grid& g, int d, double dt, const GodunovBufs& B, const double* forces, const AdjBufs& A, int fp32) {
    if (fp32) adj_pm_final_t<float>(c, g, d, dt, B, forces, A);
    else adj_pm_final_t<double>(c, g, d, dt, B, forces, A);
}

template <typename TI>
static void adj_adv_trans_t(Ctx& c, const Grid& g, int a, int b, const double* u, double rho, double dt, const double* const mac[3],
                            const GodunovBufs& B, const AdjBufs& A) {
    KI<TI> E{{ti<TI>(B.tedge[b][0]), ti<TI>(B.tedge[b][1]), ti<TI>(B.tedge[b][2])}};
    K3 Ob{{A.tr[a][b][0], A.tr[a][b][1], A.tr[a][b][2]}};
    A3 LOb{{A.lo[a][0], A.lo[a][1], A.lo[a][2]}}, HIb{{A.hi[a][0], A.hi[a][1], A.hi[a][2]}};
    A3 Ebb{{A.tedge[b][0], A.tedge[b][1], A.tedge[b][2]}};
    const long long na = nfaces(g, a), nb = nfaces(g, b);
    KS_LAUNCH(c, k_adj_adv_trans<TI>, nblocks(na, BS), BS, B8 * (6.0 * g.N + 10.0 * na + 5.0 * nb) + sizeof(TI) * 3.0 * nb, g, a, b, u, rho,
              dt / (3.0 * hd(g, b)), mac[a], mac[b], E, Ob, LOb, HIb, Ebb, A.umac[b], A.u);
}
void launch_adj_adv_trans(Ctx& c, const Grid& g, int a, int b, const double* u, double rho, double dt, const double* const mac[3],
                          const GodunovBufs& B, const AdjBufs& A, int fp32) {
    if (fp32) adj_adv_trans_t<float>(c, g, a, b, u, rho, dt, mac, B, A);
    else adj_adv_trans_t<double>(c, g, a, b, u, rho, dt, mac, B, A);
}

template <typename TI>
static void adj_adv_flux_t(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                           const GodunovBufs& B, const AdjBufs& A) {
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    K3 Uf{{mac[0], mac[1], mac[2]}};
    KI<TI> LO{{ti<TI>(B.lo[d][0]), ti<TI>(B.lo[d][1]), ti<TI>(B.lo[d][2])}}, HI{{ti<TI>(B.hi[d][0]), ti<TI>(B.hi[d][1]), ti<TI>(B.hi[d][2])}};
    KI<TI> T1{{ti<TI>(B.tr[b1][b2][0]), ti<TI>(B.tr[b1][b2][1]), ti<TI>(B.tr[b1][b2][2])}};
    KI<TI> T2{{ti<TI>(B.tr[b2][b1][0]), ti<TI>(B.tr[b2][b1][1]), ti<TI>(B.tr[b2][b1][2])}};
    K3 Fb{{A.flux[d][0], A.flux[d][1], A.flux[d][2]}};
    A3 Ufb{{A.umac[0], A.umac[1], A.umac[2]}};
    A3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    A3 T1b{{A.tr[b1][b2][0], A.tr[b1][b2][1], A.tr[b1][b2][2]}}, T2b{{A.tr[b2][b1][0], A.tr[b2][b1][1], A.tr[b2][b1][2]}};
    const long long nf = nfaces(g, d), nt = nfaces(g, b1) + nfaces(g, b2);
    KS_LAUNCH(c, k_adj_adv_flux<TI>, nblocks(nf, BS), BS, B8 * (12.0 * g.N + 10.0 * nf + 8.0 * nt) + sizeof(TI) * (6.0 * nf + 6.0 * nt), g, d, u,
              forces, rho, dt, dt / (2.0 * hd(g, b1)), dt / (2.0 * hd(g, b2)), Uf, LO, HI, T1, T2, Fb, Ufb, LOb, HIb, T1b, T2b, A.u, A.forces);
}
void launch_adj_adv_flux(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                         const GodunovBufs& B, const AdjBufs& A, int fp32) {
    if (fp32) adj_adv_flux_t<float>(c, g, d, u, forces, rho, dt, mac, B, A);
    else adj_adv_flux_t<double>(c, g, d, u, forces, rho, dt, mac, B, A);
}
void launch_adj_div(Ctx& c, const Grid& g, const double* convb, const AdjBufs& A) {
    for (int d = 0; d < 3; ++d) {
        const long long nf = nfaces(g, d);
        KS_LAUNCH(c, k_adj_div, nblocks(nf, BS), BS, B8 * (3.0 * g.N + 3.0 * nf), g, d, convb, A.flux[d][0], A.flux[d][1], A.flux[d][2]);
    }
}
void launch_adj_tau(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, const double* divtau_b, double s, double* ub,
                    double* mub, double* wgb) {
    cudaFuncSetAttribute(k_adj_tau_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ADJ_TAU_SMEM);
    const dim3 grid((g.nx + ATX - 1) / ATX, (g.ny + ATY - 1) / ATY, (g.nz + ATZ - 1) / ATZ);
    KS_LAUNCH_SMEM(c, k_adj_tau_tile, grid, ATX * ATY * ATZ, ADJ_TAU_SMEM, B8 * 14.0 * g.N, g, vel, mueff, wg, divtau_b, s, ub, mub, wgb);
}
void launch_adj_smag(Ctx& c, const Grid& g, const double* vel, const double* mub, const Scalars& s, double* ub) {
    KS_LAUNCH(c, k_adj_smag, nblocks(g.N, BS), BS, B8 * 7.0 * g.N, g, vel, mub, s.rho, s.smag_fac, ub);
}
void launch_adj_wall_local(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wgb, double ut2, double um0, double um1,
                           double vm, double rho, double* ub, double* mub, double* parts, int* np) {
    const long long M = (long long)g.nx * g.ny;
    *np = (int)std::min<long long>(1216, (M + 255) / 256);
    KS_LAUNCH(c, k_adj_wall_local, *np, 256, B8 * 9.0 * M, g, vel, mueff, wgb, ut2, um0, um1, vm, rho, ub, mub, parts, *np);
}
void launch_adj_wall_global(Ctx& c, const Grid& g, const double* vel, double bu, double bv, double bm, double* ub) {
    const long long M = (long long)g.nx * g.ny;
    KS_LAUNCH(c, k_adj_wall_global, nblocks(M, BS), BS, B8 * 6.0 * M, g, vel, bu, bv, bm, ub);
}
void launch_adj_coriolis(Ctx& c, const Grid& g, const double* srcb, const Scalars& s, double* ub) {
    KS_LAUNCH(c, k_adj_coriolis, nblocks(g.N, BS), BS, B8 * 9.0 * g.N, g, srcb, s, ub);
}
void launch_adj_nodal_post(Ctx& c, const Grid& g, const double* psi, const double* ub, double* out) {
    KS_LAUNCH(c, k_adj_nodal_post, nblocks(g.N, BS), BS, B8 * 7.0 * g.N, g, psi, ub, out);
}
void launch_axpby(Ctx& c, long long n, double a, const double* x, double b, const double* y, double* out) {
    KS_LAUNCH(c, k_axpby, nblocks(n, BS), BS, B8 * 3.0 * n, n, a, x, b, y, out);
}
void launch_objective(Ctx& c, const Grid& g, const double* u, const int lo[3], const int hi[3], double invM, double* ub, double* parts, int* np) {
    *np = 1216;
    KS_LAUNCH(c, k_objective, *np, 256, B8 * 6.0 * g.N, g, u, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], invM, ub, parts);
}
void launch_act_adj_dot(Ctx& c, const Grid& g, const double* actb, const double* pts, int npts, const double ax[3], double eps, const double plo[3],
                        const int lo[3], const int hi[3], double* parts, int* np) {
    const int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
    *np = 1216;
    KS_LAUNCH(c, k_act_adj_dot, *np, 256, B8 * 3.0 * n0 * n1 * n2, g, actb, pts, npts, ax[0], ax[1], ax[2], eps, plo[0], plo[1], plo[2], lo[0],
              lo[1], lo[2], n0, n1, n2, parts);
}
void launch_act_sample_adj(Ctx& c, const Grid& g, const double* pts, const double* wb, int npts, const double plo[3], double* ub) {
    KS_LAUNCH(c, k_act_sample_adj, nblocks(npts, 64), 64, B8 * 30.0 * npts, g, pts, wb, npts, plo[0], plo[1], plo[2], ub);
}

}  // namespace ks
