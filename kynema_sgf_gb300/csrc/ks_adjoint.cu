// Reverse (adjoint) kernels of the advance, FP64, triply periodic grids.
//
// Every forward pass y = K(x) gets a kernel that accumulates x_bar += (dK/dx)^T
// y_bar at the forward linearisation point.  The PPM limiter, clipping,
// Riemann and upwind selections are re-evaluated from the stored forward
// values and frozen (their derivatives are the derivatives of the selected
// branch).  Inputs that several outputs read are accumulated with atomicAdd.
// Passes that are linear and self-adjoint on periodic grids reuse the forward
// kernels (tensor diffusion with constant viscosity, MAC projection); the
// nodal projection uses D^T = -G and G^T = -D of its divergence / gradient
// pair (ks_host.cpp).
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;
constexpr double kSV = kSmallVel;

__device__ inline void aadd(double* p, double v) {
    if (v != 0.0) atomicAdd(p, v);
}

__device__ inline bool face3(const Grid& g, long long t, int& i, int& j, int& k) {
    if (t >= g.N) return false;
    i = (int)(t % g.nx);
    const long long r = t / g.nx;
    j = (int)(r % g.ny);
    k = (int)(r / g.ny);
    return true;
}

// cell value of velocity component n (periodic)
__device__ inline double U(const Grid& g, const double* u, int n, int i, int j, int k) {
    return u[n * g.N + cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), wrapn(k, g.nz))];
}
__device__ inline double* Ub(const Grid& g, double* u, int n, int i, int j, int k) {
    return u + n * g.N + cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), wrapn(k, g.nz));
}

// ---- van Leer slope: value and the coefficients of (a, b, c)
__device__ inline double vls_d(double a, double b, double c, double& ca, double& cb, double& cc) {
    const double dsc = 0.5 * (c - a), dsl = 2.0 * (b - a), dsr = 2.0 * (c - b);
    ca = cb = cc = 0.0;
    if (!(dsl * dsr > 0.0)) return 0.0;
    const double ac = fabs(dsc), al = fabs(dsl), ar = fabs(dsr);
    if (ac <= fmin(al, ar)) {
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

// ---- reverse of the unlimited PPM edge on d-faces (k_edges):
// E = clip(0.5(a0+a1) - (vl(a0,a1,a2) - vl(am,a0,a1))/6, a0, a1)
__global__ void k_adj_edges(Grid g, int d, const double* u, const double* Eb0, const double* Eb1, const double* Eb2, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const double* Eb[3] = {Eb0, Eb1, Eb2};
    for (int n = 0; n < 3; ++n) {
        const double eb = Eb[n][t];
        if (eb == 0.0) continue;
        const double am = U(g, u, n, i - 2 * di, j - 2 * dj, k - 2 * dk), a0 = U(g, u, n, i - di, j - dj, k - dk);
        const double a1 = U(g, u, n, i, j, k), a2 = U(g, u, n, i + di, j + dj, k + dk);
        double c1a, c1b, c1c, c0a, c0b, c0c;
        const double s1 = vls_d(a0, a1, a2, c1a, c1b, c1c);
        const double s0 = vls_d(am, a0, a1, c0a, c0b, c0c);
        const double e = 0.5 * (a0 + a1) - (1.0 / 6.0) * (s1 - s0);
        const double lo = fmin(a0, a1), hi = fmax(a0, a1);
        double gm = 0, g0 = 0, g1 = 0, g2 = 0;
        const double r = fmax(e, lo);
        if (r > hi) {  // clipped to the larger neighbour
            if (a0 >= a1) g0 += eb; else g1 += eb;
        } else if (e < lo) {  // clipped to the smaller neighbour
            if (a0 <= a1) g0 += eb; else g1 += eb;
        } else {
            g0 += 0.5 * eb;
            g1 += 0.5 * eb;
            const double ds1 = -eb / 6.0, ds0 = eb / 6.0;
            g0 += ds1 * c1a;
            g1 += ds1 * c1b;
            g2 += ds1 * c1c;
            gm += ds0 * c0a;
            g0 += ds0 * c0b;
            g1 += ds0 * c0c;
        }
        aadd(Ub(g, ub, n, i - 2 * di, j - 2 * dj, k - 2 * dk), gm);
        aadd(Ub(g, ub, n, i - di, j - dj, k - dk), g0);
        aadd(Ub(g, ub, n, i, j, k), g1);
        aadd(Ub(g, ub, n, i + di, j + dj, k + dk), g2);
    }
}

// ---- reverse of the CW84 limiter + trace.  Given the adjoint tb of the trace
// value (after any rho scaling), accumulate into sm_in, s0, sp_in adjoints and
// return the adjoint of sig.
__device__ inline double rev_trace(bool hi_side, double smi, double s0, double spi, double sig, double tb, double& gsm, double& gs0,
                                   double& gsp) {
    // forward limiter with case record
    double sm = smi, sp = spi;
    int cs = 0;
    if ((sp - s0) * (s0 - sm) <= 0.0) {
        cs = 1;
        sp = s0;
        sm = s0;
    } else if (fabs(sp - s0) >= 2.0 * fabs(sm - s0)) {
        cs = 2;
        sp = 3.0 * s0 - 2.0 * sm;
    } else if (fabs(sm - s0) >= 2.0 * fabs(sp - s0)) {
        cs = 3;
        sm = 3.0 * s0 - 2.0 * sp;
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
    // reverse the limiter
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
    const bool fu = !(fabs(vel) < kSV);
    if (fu) {
        if (vel >= 0.0) lb += ob; else hb += ob;
    } else {
        lb += 0.5 * ob;
        hb += 0.5 * ob;
    }
}
__device__ inline void rev_riemann(double lo, double hi, double ob, double& lb, double& hb) {
    const bool ltm = (lo <= 0.0 && hi >= 0.0) || (fabs(lo + hi) < kSV);
    if (ltm) return;
    if (lo + hi >= 0.0) lb += ob; else hb += ob;
}

struct A3 {
    double* p[3];
};
struct K3 {
    const double* p[3];
};

// ---- reverse of k_faces (both passes).  MODE 0: pre-MAC (cell speed), the
// adjoints of ad and of the upwinded transverse states are folded in here;
// MODE 1: post-MAC (face speed, rho scaling), upwinded states folded in.
template <int MODE>
__global__ void k_adj_faces(Grid g, int d, const double* u, K3 E, double s, double rho, const double* umac_d, K3 LO, K3 HI, const double* ad,
                            K3 LOb, K3 HIb, const double* adb, K3 TEb, A3 Eb, double* ub, double* umacb_d) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const long long f = t;
    const long long fm = fidx(g, d, i - di, j - dj, k - dk), fp = fidx(g, d, i + di, j + dj, k + dk);
    double lb[3], hb[3];
    for (int n = 0; n < 3; ++n) {
        lb[n] = LOb.p[n][f];
        hb[n] = HIb.p[n][f];
    }
    double ul, uh, umf = 0.0;
    if (MODE == 0) {
        ul = U(g, u, d, i - di, j - dj, k - dk);
        uh = U(g, u, d, i, j, k);
        const double a = ad[f];
        rev_riemann(LO.p[d][f], HI.p[d][f], adb[f], lb[d], hb[d]);
        for (int n = 0; n < 3; ++n)
            if (n != d) rev_upwind(a, TEb.p[n][f], lb[n], hb[n]);
    } else {
        umf = umac_d[f];
        ul = uh = umf;
        for (int n = 0; n < 3; ++n) rev_upwind(umf, TEb.p[n][f], lb[n], hb[n]);
    }
    const double scale = (MODE == 1) ? rho : 1.0;
    double gul = 0.0, guh = 0.0;
    for (int n = 0; n < 3; ++n) {
        // low side: high-face trace of cell c - e_d
        const double tl = lb[n] * scale, th = hb[n] * scale;
        double gsm = 0, gs0 = 0, gsp = 0;
        if (tl != 0.0) {
            const double s0 = U(g, u, n, i - di, j - dj, k - dk);
            if (ul > kSV) {
                const double sig = fabs(ul) * s;
                const double bsig = rev_trace(true, E.p[n][fm], s0, E.p[n][f], sig, tl, gsm, gs0, gsp);
                gul += bsig * s * (ul >= 0.0 ? 1.0 : -1.0);
            } else {
                gs0 += tl;
            }
            aadd(&Eb.p[n][fm], gsm);
            aadd(&Eb.p[n][f], gsp);
            aadd(Ub(g, ub, n, i - di, j - dj, k - dk), gs0);
        }
        gsm = gs0 = gsp = 0;
        if (th != 0.0) {
            const double s0 = U(g, u, n, i, j, k);
            if (uh < -kSV) {
                const double sig = fabs(uh) * s;
                const double bsig = rev_trace(false, E.p[n][f], s0, E.p[n][fp], sig, th, gsm, gs0, gsp);
                guh += bsig * s * (uh >= 0.0 ? 1.0 : -1.0);
            } else {
                gs0 += th;
            }
            aadd(&Eb.p[n][f], gsm);
            aadd(&Eb.p[n][fp], gsp);
            aadd(Ub(g, ub, n, i, j, k), gs0);
        }
    }
    if (MODE == 0) {
        aadd(Ub(g, ub, d, i - di, j - dj, k - dk), gul);
        aadd(Ub(g, ub, d, i, j, k), guh);
    } else {
        aadd(&umacb_d[f], gul + guh);
    }
}

// ---- reverse of k_pm_trans (a, b, n)
__global__ void k_adj_pm_trans(Grid g, int a, int b, double cb, const double* ad_a, const double* ad_b, const double* edge_b, const double* lo_an,
                               const double* hi_an, const double* outb, double* lo_anb, double* hi_anb, double* ad_bb, double* edge_bb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const long long f = t;
    const double ob = outb[f];
    if (ob == 0.0) return;
    double lb = 0, hb = 0;
    rev_upwind(ad_a[f], ob, lb, hb);
    lo_anb[f] += lb;
    hi_anb[f] += hb;
    const int e0 = (b == 0), e1 = (b == 1), e2 = (b == 2);
    {
        const long long f0 = fidx(g, b, i, j, k), f1 = fidx(g, b, i + e0, j + e1, k + e2);
        const double S = ad_b[f1] + ad_b[f0], Dd = edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], -cb * Dd * hb);
        aadd(&ad_bb[f0], -cb * Dd * hb);
        aadd(&edge_bb[f1], -cb * S * hb);
        aadd(&edge_bb[f0], cb * S * hb);
    }
    {
        const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
        const long long f0 = fidx(g, b, ci, cj, ck), f1 = fidx(g, b, ci + e0, cj + e1, ck + e2);
        const double S = ad_b[f1] + ad_b[f0], Dd = edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], -cb * Dd * lb);
        aadd(&ad_bb[f0], -cb * Dd * lb);
        aadd(&edge_bb[f1], -cb * S * lb);
        aadd(&edge_bb[f0], cb * S * lb);
    }
}

// ---- reverse of k_pm_final (d)
__global__ void k_adj_pm_final(Grid g, int d, double dt, double c1, double c2, const double* lo_dd, const double* hi_dd, K3 AD, const double* T1,
                               const double* T2, const double* forces, const double* macb, double* lo_ddb, double* hi_ddb, A3 ADb,
                               double* T1b, double* T2b, double* forcesb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const long long f = t;
    const double mb = macb[f];
    if (mb == 0.0) return;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    auto side_val = [&](int ci, int cj, int ck, double base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        double s = base;
        s -= c1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        s += 0.5 * dt * forces[d * g.N + cidx(g, wrapn(ci, g.nx), wrapn(cj, g.ny), wrapn(ck, g.nz))];
        return s;
    };
    auto side_rev = [&](int ci, int cj, int ck, double sb) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        const double S1 = AD.p[b1][p1] + AD.p[b1][m1], D1 = T1[p1] - T1[m1];
        const double S2 = AD.p[b2][p2] + AD.p[b2][m2], D2 = T2[p2] - T2[m2];
        aadd(&ADb.p[b1][p1], -c1 * D1 * sb);
        aadd(&ADb.p[b1][m1], -c1 * D1 * sb);
        aadd(&T1b[p1], -c1 * S1 * sb);
        aadd(&T1b[m1], c1 * S1 * sb);
        aadd(&ADb.p[b2][p2], -c2 * D2 * sb);
        aadd(&ADb.p[b2][m2], -c2 * D2 * sb);
        aadd(&T2b[p2], -c2 * S2 * sb);
        aadd(&T2b[m2], c2 * S2 * sb);
        aadd(&forcesb[d * g.N + cidx(g, wrapn(ci, g.nx), wrapn(cj, g.ny), wrapn(ck, g.nz))], 0.5 * dt * sb);
    };
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const double stl = side_val(li, lj, lk, lo_dd[f]), sth = side_val(i, j, k, hi_dd[f]);
    double bl = 0, bh = 0;
    rev_riemann(stl, sth, mb, bl, bh);
    if (bl != 0.0) {
        lo_ddb[f] += bl;
        side_rev(li, lj, lk, bl);
    }
    if (bh != 0.0) {
        hi_ddb[f] += bh;
        side_rev(i, j, k, bh);
    }
}

// ---- reverse of k_adv_trans (a, b): out_n = upwind(u_a; l, h),
// h = HI + (-cb (vp E(h1) - vm E(h0)) + cb q(c) (vp - vm)), l likewise at c - e_a
__global__ void k_adj_adv_trans(Grid g, int a, int b, const double* u, double rho, double cb, const double* ua, const double* vb, K3 E, K3 Ob,
                                A3 LOb, A3 HIb, A3 Ebb, double* vbb, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const long long f = t;
    const double uaf = ua[f];
    const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
    const long long h0 = fidx(g, b, i, j, k), h1 = fidx(g, b, i + (b == 0), j + (b == 1), k + (b == 2));
    const long long l0 = fidx(g, b, ci, cj, ck), l1 = fidx(g, b, ci + (b == 0), cj + (b == 1), ck + (b == 2));
    const double vhp = vb[h1], vhm = vb[h0], vlp = vb[l1], vlm = vb[l0];
    double gvhp = 0, gvhm = 0, gvlp = 0, gvlm = 0;
    for (int n = 0; n < 3; ++n) {
        const double ob = Ob.p[n][f];
        if (ob == 0.0) continue;
        double lb = 0, hb = 0;
        rev_upwind(uaf, ob, lb, hb);
        LOb.p[n][f] += lb;
        HIb.p[n][f] += hb;
        if (hb != 0.0) {
            const double qc = rho * U(g, u, n, i, j, k);
            aadd(&Ebb.p[n][h1], -cb * vhp * hb);
            aadd(&Ebb.p[n][h0], cb * vhm * hb);
            gvhp += (-cb * E.p[n][h1] + cb * qc) * hb;
            gvhm += (cb * E.p[n][h0] - cb * qc) * hb;
            aadd(Ub(g, ub, n, i, j, k), rho * cb * (vhp - vhm) * hb);
        }
        if (lb != 0.0) {
            const double qc = rho * U(g, u, n, ci, cj, ck);
            aadd(&Ebb.p[n][l1], -cb * vlp * lb);
            aadd(&Ebb.p[n][l0], cb * vlm * lb);
            gvlp += (-cb * E.p[n][l1] + cb * qc) * lb;
            gvlm += (cb * E.p[n][l0] - cb * qc) * lb;
            aadd(Ub(g, ub, n, ci, cj, ck), rho * cb * (vlp - vlm) * lb);
        }
    }
    aadd(&vbb[h1], gvhp);
    aadd(&vbb[h0], gvhm);
    aadd(&vbb[l1], gvlp);
    aadd(&vbb[l0], gvlm);
}

// ---- reverse of k_adv_flux (d) with the flux adjoint Fb given
__global__ void k_adj_adv_flux(Grid g, int d, const double* u, const double* forces, double rho, double dt, double c1, double c2, K3 Uf, K3 LO,
                               K3 HI, K3 T1, K3 T2, K3 Fb, A3 Ufb, A3 LOb, A3 HIb, A3 T1b, A3 T2b, double* ub, double* forcesb) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    const long long f = t;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const double um = Uf.p[d][f];
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const long long lp1 = fidx(g, b1, li + (b1 == 0), lj + (b1 == 1), lk + (b1 == 2)), lm1 = fidx(g, b1, li, lj, lk);
    const long long lp2 = fidx(g, b2, li + (b2 == 0), lj + (b2 == 1), lk + (b2 == 2)), lm2 = fidx(g, b2, li, lj, lk);
    const long long hp1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), hm1 = fidx(g, b1, i, j, k);
    const long long hp2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), hm2 = fidx(g, b2, i, j, k);
    const double l1p = Uf.p[b1][lp1], l1m = Uf.p[b1][lm1], l2p = Uf.p[b2][lp2], l2m = Uf.p[b2][lm2];
    const double h1p = Uf.p[b1][hp1], h1m = Uf.p[b1][hm1], h2p = Uf.p[b2][hp2], h2m = Uf.p[b2][hm2];
    double gum = 0, gl1p = 0, gl1m = 0, gl2p = 0, gl2m = 0, gh1p = 0, gh1m = 0, gh2p = 0, gh2m = 0;
    const long long cl = cidx(g, wrapn(li, g.nx), wrapn(lj, g.ny), wrapn(lk, g.nz));
    const long long ch = cidx(g, i, j, k);
    for (int n = 0; n < 3; ++n) {
        const double fb = Fb.p[n][f];
        if (fb == 0.0) continue;
        const double ql = rho * u[n * g.N + cl], qh = rho * u[n * g.N + ch];
        double stl = LO.p[n][f];
        stl -= c1 * (T1.p[n][lp1] * l1p - T1.p[n][lm1] * l1m);
        stl -= c2 * (T2.p[n][lp2] * l2p - T2.p[n][lm2] * l2m);
        stl += c1 * ql * (l1p - l1m);
        stl += c2 * ql * (l2p - l2m);
        stl += 0.5 * dt * (rho * forces[n * g.N + cl]);
        double sth = HI.p[n][f];
        sth -= c1 * (T1.p[n][hp1] * h1p - T1.p[n][hm1] * h1m);
        sth -= c2 * (T2.p[n][hp2] * h2p - T2.p[n][hm2] * h2m);
        sth += c1 * qh * (h1p - h1m);
        sth += c2 * qh * (h2p - h2m);
        sth += 0.5 * dt * (rho * forces[n * g.N + ch]);
        double st, bl = 0, bh = 0;
        if (fabs(um) < kSV) {
            st = 0.5 * (stl + sth);
            bl = bh = 0.5 * um * fb;
        } else if (um >= 0.0) {
            st = stl;
            bl = um * fb;
        } else {
            st = sth;
            bh = um * fb;
        }
        gum += st * fb;
        if (bl != 0.0) {
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
        if (bh != 0.0) {
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

// ---- reverse of conv = -div F: Fb_d,n(f) = (convb(c_f) - convb(c_f - e_d)) / h_d
__global__ void k_adj_div(Grid g, const double* convb, A3 F0, A3 F1, A3 F2) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face3(g, t, i, j, k)) return;
    A3* F[3] = {&F0, &F1, &F2};
    const double ih[3] = {g.idx, g.idy, g.idz};
    for (int d = 0; d < 3; ++d) {
        const long long cm = cidx(g, wrapn(i - (d == 0), g.nx), wrapn(j - (d == 1), g.ny), wrapn(k - (d == 2), g.nz));
        for (int n = 0; n < 3; ++n) F[d]->p[n][t] = (convb[n * g.N + t] - convb[n * g.N + cm]) * ih[d];
    }
}

// ---- nodal projection adjoint: out = ub + G psi
__global__ void k_adj_nodal_post(Grid g, const double* psi, const double* ub, double* out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    face3(g, t, i, j, k);
    auto P = [&](int a, int b, int c) { return psi[cidx(g, wrapn(a, g.nx), wrapn(b, g.ny), wrapn(c, g.nz))]; };
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
    double s = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        face3(g, t, i, j, k);
        const bool in = i >= lo0 && i <= hi0 && j >= lo1 && j <= hi1 && k >= lo2 && k <= hi2;
        for (int n = 0; n < 3; ++n) {
            const double v = u[n * g.N + t];
            if (in) s += 0.5 * v * v;
            if (ub) ub[n * g.N + t] = in ? v * invM : 0.0;
        }
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) parts[blockIdx.x] = sh[0] * invM;
}

// disk adjoint: partial sums over the cut-off box of  sum_x (actb(x) . n) B(x),
// B(x) = sum_points w_p g3(x - p) with the per-point weights w_p in pts[4p+3]
__global__ void k_act_adj_dot(Grid g, const double* actb, const double* pts, int npts, double ax0, double ax1, double ax2, double eps, double x0,
                              double y0, double z0, int lo0, int lo1, int lo2, int n0, int n1, int n2, double* parts) {
    double acc = 0.0;
    const long long M = (long long)n0 * n1 * n2;
    const double gfac = 0.17958712212516656 / (eps * eps * eps);
    const double ie = 1.0 / eps;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(t % n0);
        const long long r = t / n0;
        const int b = (int)(r % n1), c = (int)(r / n1);
        const int i = lo0 + a, j = lo1 + b, k = lo2 + c;
        const double x = x0 + (i + 0.5) * g.dx, y = y0 + (j + 0.5) * g.dy, z = z0 + (k + 0.5) * g.dz;
        double s = 0;
        for (int m = 0; m < npts; ++m) {
            const double rx = (pts[4 * m] - x) * ie, ry = (pts[4 * m + 1] - y) * ie, rz = (pts[4 * m + 2] - z) * ie;
            const double r2 = rx * rx + ry * ry + rz * rz;
            if (r2 < 16.0) s += gfac * exp(-r2) * pts[4 * m + 3];
        }
        const long long cc = cidx(g, i, j, k);
        acc += s * (actb[cc] * ax0 + actb[g.N + cc] * ax1 + actb[2 * g.N + cc] * ax2);
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) parts[blockIdx.x] = sh[0];
}

// scatter of the sampled-velocity adjoint to the trilinear corners
__global__ void k_act_sample_adj(Grid g, const double* pts, const double* wb, int npts, double x0, double y0, double z0, double* ub) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double fx = (pts[3 * p] - x0 - 0.5 * g.dx) * g.idx;
    const double fy = (pts[3 * p + 1] - y0 - 0.5 * g.dy) * g.idy;
    const double fz = (pts[3 * p + 2] - z0 - 0.5 * g.dz) * g.idz;
    const int i = (int)floor(fx), j = (int)floor(fy), k = (int)floor(fz);
    const double wx = fx - i, wy = fy - j, wz = fz - k;
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                const double w = (a ? wx : 1 - wx) * (b ? wy : 1 - wy) * (c ? wz : 1 - wz);
                for (int n = 0; n < 3; ++n) aadd(Ub(g, ub, n, i + a, j + b, k + c), w * wb[3 * p + n]);
            }
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_adj_edges(Ctx& c, const Grid& g, int d, const double* u, double* const Eb[3], double* ub) {
    KS_LAUNCH(c, k_adj_edges, nblocks(g.N, BS), BS, 8.0 * 7 * g.N, g, d, u, Eb[0], Eb[1], Eb[2], ub);
}
void launch_adj_faces(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                      const double* umac_d) {
    K3 E{{(double*)B.edge[d][0], (double*)B.edge[d][1], (double*)B.edge[d][2]}};
    K3 LO{{(double*)B.lo[d][0], (double*)B.lo[d][1], (double*)B.lo[d][2]}}, HI{{(double*)B.hi[d][0], (double*)B.hi[d][1], (double*)B.hi[d][2]}};
    K3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    K3 TEb{{A.tedge[d][0], A.tedge[d][1], A.tedge[d][2]}};
    A3 Eb{{A.edge[d][0], A.edge[d][1], A.edge[d][2]}};
    const double s = dt * ihd(g, d);
    if (mode == 0)
        KS_LAUNCH(c, k_adj_faces<0>, nblocks(g.N, BS), BS, 8.0 * 30 * g.N, g, d, u, E, s, rho, nullptr, LO, HI, (const double*)B.ad[d], LOb,
                  HIb, A.ad[d], TEb, Eb, A.u, nullptr);
    else
        KS_LAUNCH(c, k_adj_faces<1>, nblocks(g.N, BS), BS, 8.0 * 30 * g.N, g, d, u, E, s, rho, umac_d, LO, HI, nullptr, LOb, HIb, nullptr, TEb,
                  Eb, A.u, A.umac[d]);
}
void launch_adj_pm_trans(Ctx& c, const Grid& g, int a, int b, int n, double dt, const GodunovBufs& B, const AdjBufs& A) {
    const double cb = dt / (6.0 * hd(g, b));
    KS_LAUNCH(c, k_adj_pm_trans, nblocks(g.N, BS), BS, 8.0 * 10 * g.N, g, a, b, cb, (const double*)B.ad[a], (const double*)B.ad[b],
              (const double*)B.tedge[b][n], (const double*)B.lo[a][n], (const double*)B.hi[a][n], A.tr[a][b][0], A.lo[a][n], A.hi[a][n], A.ad[b],
              A.tedge[b][n]);
}
void launch_adj_pm_final(Ctx& c, const Grid& g, int d, double dt, const GodunovBufs& B, const double* forces, const AdjBufs& A) {
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    K3 AD{{(double*)B.ad[0], (double*)B.ad[1], (double*)B.ad[2]}};
    A3 ADb{{A.ad[0], A.ad[1], A.ad[2]}};
    KS_LAUNCH(c, k_adj_pm_final, nblocks(g.N, BS), BS, 8.0 * 14 * g.N, g, d, dt, dt / (4.0 * hd(g, b1)), dt / (4.0 * hd(g, b2)),
              (const double*)B.lo[d][d], (const double*)B.hi[d][d], AD, (const double*)B.tr[b1][b2][0], (const double*)B.tr[b2][b1][0], forces,
              A.umac[d], A.lo[d][d], A.hi[d][d], ADb, A.tr[b1][b2][0], A.tr[b2][b1][0], A.forces);
}
void launch_adj_adv_trans(Ctx& c, const Grid& g, int a, int b, const double* u, double rho, double dt, const double* const mac[3],
                          const GodunovBufs& B, const AdjBufs& A) {
    K3 E{{(double*)B.tedge[b][0], (double*)B.tedge[b][1], (double*)B.tedge[b][2]}};
    K3 Ob{{A.tr[a][b][0], A.tr[a][b][1], A.tr[a][b][2]}};
    A3 LOb{{A.lo[a][0], A.lo[a][1], A.lo[a][2]}}, HIb{{A.hi[a][0], A.hi[a][1], A.hi[a][2]}};
    A3 Ebb{{A.tedge[b][0], A.tedge[b][1], A.tedge[b][2]}};
    KS_LAUNCH(c, k_adj_adv_trans, nblocks(g.N, BS), BS, 8.0 * 24 * g.N, g, a, b, u, rho, dt / (3.0 * hd(g, b)), mac[a], mac[b], E, Ob, LOb, HIb,
              Ebb, A.umac[b], A.u);
}
void launch_adj_adv_flux(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                         const GodunovBufs& B, const AdjBufs& A) {
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    K3 Uf{{mac[0], mac[1], mac[2]}};
    K3 LO{{(double*)B.lo[d][0], (double*)B.lo[d][1], (double*)B.lo[d][2]}}, HI{{(double*)B.hi[d][0], (double*)B.hi[d][1], (double*)B.hi[d][2]}};
    K3 T1{{(double*)B.tr[b1][b2][0], (double*)B.tr[b1][b2][1], (double*)B.tr[b1][b2][2]}};
    K3 T2{{(double*)B.tr[b2][b1][0], (double*)B.tr[b2][b1][1], (double*)B.tr[b2][b1][2]}};
    K3 Fb{{A.flux[d][0], A.flux[d][1], A.flux[d][2]}};
    A3 Ufb{{A.umac[0], A.umac[1], A.umac[2]}};
    A3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    A3 T1b{{A.tr[b1][b2][0], A.tr[b1][b2][1], A.tr[b1][b2][2]}}, T2b{{A.tr[b2][b1][0], A.tr[b2][b1][1], A.tr[b2][b1][2]}};
    KS_LAUNCH(c, k_adj_adv_flux, nblocks(g.N, BS), BS, 8.0 * 40 * g.N, g, d, u, forces, rho, dt, dt / (2.0 * hd(g, b1)), dt / (2.0 * hd(g, b2)),
              Uf, LO, HI, T1, T2, Fb, Ufb, LOb, HIb, T1b, T2b, A.u, A.forces);
}
void launch_adj_div(Ctx& c, const Grid& g, const double* convb, const AdjBufs& A) {
    A3 F0{{A.flux[0][0], A.flux[0][1], A.flux[0][2]}}, F1{{A.flux[1][0], A.flux[1][1], A.flux[1][2]}},
        F2{{A.flux[2][0], A.flux[2][1], A.flux[2][2]}};
    KS_LAUNCH(c, k_adj_div, nblocks(g.N, BS), BS, 8.0 * 15 * g.N, g, convb, F0, F1, F2);
}
void launch_adj_nodal_post(Ctx& c, const Grid& g, const double* psi, const double* ub, double* out) {
    KS_LAUNCH(c, k_adj_nodal_post, nblocks(g.N, BS), BS, 8.0 * 7 * g.N, g, psi, ub, out);
}
void launch_axpby(Ctx& c, long long n, double a, const double* x, double b, const double* y, double* out) {
    KS_LAUNCH(c, k_axpby, nblocks(n, BS), BS, 24.0 * n, n, a, x, b, y, out);
}
void launch_objective(Ctx& c, const Grid& g, const double* u, const int lo[3], const int hi[3], double invM, double* ub, double* parts, int* np) {
    *np = 1216;
    KS_LAUNCH(c, k_objective, *np, 256, 8.0 * 6 * g.N, g, u, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], invM, ub, parts);
}
void launch_act_adj_dot(Ctx& c, const Grid& g, const double* actb, const double* pts, int npts, const double ax[3], double eps, const double plo[3],
                        const int lo[3], const int hi[3], double* parts, int* np) {
    const int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
    *np = 1216;
    KS_LAUNCH(c, k_act_adj_dot, *np, 256, 8.0 * 3 * n0 * n1 * n2, g, actb, pts, npts, ax[0], ax[1], ax[2], eps, plo[0], plo[1], plo[2], lo[0], lo[1],
              lo[2], n0, n1, n2, parts);
}
void launch_act_sample_adj(Ctx& c, const Grid& g, const double* pts, const double* wb, int npts, const double plo[3], double* ub) {
    KS_LAUNCH(c, k_act_sample_adj, nblocks(npts, 64), 64, 8.0 * 30 * npts, g, pts, wb, npts, plo[0], plo[1], plo[2], ub);
}

}  // namespace ks
