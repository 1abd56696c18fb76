// Reverse (adjoint) kernels of the advance.  Adjoint arrays are FP64; each
// pass computes in its forward pass's precision (TI / A: double, or float for
// the mixed-precision form's FP32 passes).
//
// Every forward pass y = K(x) gets a kernel (or a pair) that accumulates
// x_bar += (dK/dx)^T y_bar at the forward linearisation point.  The PPM
// limiter, clipping, Riemann and upwind selections are re-evaluated from the
// stored forward values and frozen (their derivatives are the derivatives of
// the selected branch).  Inputs that several outputs read are accumulated
// either in gather form, each adjoint value owned by one thread that collects
// the terms of the outputs reading it (the post-MAC stages, the PPM edges and
// face stage, Smagorinsky; one FP64 add per owned value), or with atomicAdd
// (the pre-MAC transverse / final stages, the wall faces, the diffusion
// tile's flush).  Boundary handling mirrors the forward kernels: x/y periodic; z periodic or
// walls, where the forward reads fill-patch ghosts (high-order extrapolation
// of the tangential components, zero normal component) for Godunov, odd/even
// reflections or the wall-model shift for diffusion, and replaces wall-face
// states (zbc); the reverse scatters every ghost read back onto the interior
// cells it was built from.
#include "ks_decide.cuh"
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

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

// velocity read with the Godunov fill-patch ghosts (VelFPT, scale 1) in the
// arithmetic type A of the pass, and its adjoint (FP64 accumulation)
template <typename A = double>
__device__ inline A Q(const Grid& g, const double* u, int n, int i, int j, int k) {
    const VelFPT<A, double> q{u, g, A(1)};
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
template <typename A>
__device__ inline void zbc_fwd(const Grid& g, int k, int n, A& lo, A& hi) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) lo = hi = A(0); else lo = hi;
    } else if (k == g.nz) {
        if (n == 2) lo = hi = A(0); else hi = lo;
    }
}
template <typename A>
__device__ inline void zbc_rev(const Grid& g, int k, int n, A& lb, A& hb) {
    if (g.zper) return;
    if (k == 0) {
        if (n == 2) {
            lb = hb = A(0);
        } else {
            hb += lb;
            lb = A(0);
        }
    } else if (k == g.nz) {
        if (n == 2) {
            lb = hb = A(0);
        } else {
            lb += hb;
            hb = A(0);
        }
    }
}

// ---- van Leer slope (the forward's vls, ks_godunov.cu): value and the
// coefficients of (a, b, c), with the forward's branch order
template <typename A>
__device__ inline A vls_d(A a, A b, A c, A& ca, A& cb, A& cc) {
    const A dsc = A(0.5) * (c - a), dsl = A(2) * (b - a), dsr = A(2) * (c - b);
    ca = cb = cc = A(0);
    if (!same_sign(dsl, dsr)) return A(0);
    const bool left = abs_lt(dsl, dsr);  // forward: m = |dsl| < |dsr| ? dsl : dsr
    if (abs_lt(dsc, left ? dsl : dsr)) {
        ca = A(-0.5);
        cc = A(0.5);
        return dsc;
    }
    if (left) {
        ca = A(-2);
        cb = A(2);
        return dsl;
    }
    cb = A(-2);
    cc = A(2);
    return dsr;
}

// adjoint of clip(e, a, b) = min(max(e, min(a, b)), max(a, b)) given the
// adjoint of the result: returns the adjoint of e; adds to those of a, b.
// The selections are the forward's (ks_decide.cuh): for FP64 they order -0
// below +0, so a signed-zero tie routes the adjoint to the operand the
// forward selected.
template <typename A>
__device__ inline A clip_rev(A e, A a, A b, A rb, A& ga, A& gb) {
    const A lo = min2(a, b), hi = max2(a, b);
    if (lt(hi, max2(e, lo))) {
        if (!lt(a, b)) ga += rb; else gb += rb;
        return A(0);
    }
    if (lt(e, lo)) {
        if (!lt(b, a)) ga += rb; else gb += rb;
        return A(0);
    }
    return rb;
}

// adjoints of the four cells of an interior d-face's unlimited edge
// e = (a0 + a1) / 2 - (s1 - s0) / 6 (s the van Leer slopes), clipped to
// [a0, a1], given the edge's adjoint eb: g[0..3] for cells am, a0, a1, a2
template <typename A>
__device__ inline void edge_rev(A am, A a0, A a1, A a2, A eb, A g[4]) {
    A c1a, c1b, c1c, c0a, c0b, c0c;
    const A s1 = vls_d(a0, a1, a2, c1a, c1b, c1c);
    const A s0 = vls_d(am, a0, a1, c0a, c0b, c0c);
    const A e = A(0.5) * (a0 + a1) - A(1.0 / 6.0) * (s1 - s0);
    g[0] = g[1] = g[2] = g[3] = A(0);
    const A ebar = clip_rev(e, a0, a1, eb, g[1], g[2]);
    if (nonzero(ebar)) {
        g[1] += A(0.5) * ebar;
        g[2] += A(0.5) * ebar;
        const A ds1 = -ebar * A(1.0 / 6.0), ds0 = ebar * A(1.0 / 6.0);
        g[1] += ds1 * c1a;
        g[2] += ds1 * c1b;
        g[3] += ds1 * c1c;
        g[0] += ds0 * c0a;
        g[1] += ds0 * c0b;
        g[2] += ds0 * c0c;
    }
}

// the reverse of one d-face's edge, scattered with atomics (the wall faces and
// the one-sided faces next to them, every face of a short wall-bounded column)
template <typename A>
__device__ inline void edge_rev_scatter(const Grid& g, int d, const double* u, const double* const Eb[3], int i, int j, int k, long long t,
                                        double* ub) {
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wall = (d == 2 && !g.zper);
    for (int n = 0; n < 3; ++n) {
        const double eb64 = Eb[n][t];
        if (!(dbits(eb64) & kMag)) continue;
        if (wall && (k == 0 || k == g.nz)) {  // the wall face takes the ghost value
            Qb(g, ub, n, i, j, k == 0 ? -1 : g.nz, eb64);
            continue;
        }
        const A eb = (A)eb64;
        if (wall && (k == 1 || k == g.nz - 1)) {  // one-sided fourth order, clipped to the adjacent cells
            const int kb = (k == 1) ? -1 : g.nz, k0 = (k == 1) ? 0 : g.nz - 1, s = (k == 1) ? 1 : -1;
            const A b = Q<A>(g, u, n, i, j, kb), q0 = Q<A>(g, u, n, i, j, k0), q1 = Q<A>(g, u, n, i, j, k0 + s),
                    q2 = Q<A>(g, u, n, i, j, k0 + 2 * s);
            const A e = A(-0.2) * b + A(0.75) * q0 + A(0.5) * q1 - A(0.05) * q2;
            A g0 = A(0), g1 = A(0);
            const A ebar = clip_rev(e, q0, q1, eb, g0, g1);
            Qb(g, ub, n, i, j, kb, (double)(A(-0.2) * ebar));
            Qb(g, ub, n, i, j, k0, (double)(A(0.75) * ebar + g0));
            Qb(g, ub, n, i, j, k0 + s, (double)(A(0.5) * ebar + g1));
            Qb(g, ub, n, i, j, k0 + 2 * s, (double)(A(-0.05) * ebar));
            continue;
        }
        A gr[4];
        edge_rev(Q<A>(g, u, n, i - 2 * di, j - 2 * dj, k - 2 * dk), Q<A>(g, u, n, i - di, j - dj, k - dk), Q<A>(g, u, n, i, j, k),
                 Q<A>(g, u, n, i + di, j + dj, k + dk), eb, gr);
        Qb(g, ub, n, i - 2 * di, j - 2 * dj, k - 2 * dk, (double)gr[0]);
        Qb(g, ub, n, i - di, j - dj, k - dk, (double)gr[1]);
        Qb(g, ub, n, i, j, k, (double)gr[2]);
        Qb(g, ub, n, i + di, j + dj, k + dk, (double)gr[3]);
    }
}

// ---- reverse of the unlimited PPM edges on d-faces (k_edges).  TI is the
// forward's precision and the arithmetic type of the reverse pass.
// Scatter form over all d-faces (short wall-bounded columns) ...
template <typename TI>
__global__ void k_adj_edges(Grid g, int d, const double* u, const double* Eb0, const double* Eb1, const double* Eb2, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const double* Eb[3] = {Eb0, Eb1, Eb2};
    edge_rev_scatter<TI>(g, d, u, Eb, i, j, k, t, ub);
}

// ... or over the face layers 0, 1, nz - 1, nz of a wall-bounded z (nz >= 4)
template <typename TI>
__global__ void k_adj_edges_wall(Grid g, const double* u, const double* Eb0, const double* Eb1, const double* Eb2, double* ub) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long M = (long long)g.nx * g.ny;
    if (t >= 4 * M) return;
    const int layer = (int)(t / M), r = (int)(t - layer * M);
    const int k = layer < 2 ? layer : g.nz - 3 + layer, j = r / g.nx, i = r - j * g.nx;
    const double* Eb[3] = {Eb0, Eb1, Eb2};
    edge_rev_scatter<TI>(g, 2, u, Eb, i, j, k, cidx(g, i, j, k), ub);
}

// ... with every other face gathered per cell: cell c is a2, a1, a0, am of the
// d-faces c - 1, c, c + 1, c + 2 (face m reads cells m - 2 .. m + 1); the
// thread re-evaluates those four faces' slopes and clips from the seven cells
// c - 3 .. c + 3 (cheap in the pass precision) and owns the cell's adjoint.
// With a wall-bounded z only the faces 2 .. nz - 2 are gathered.
template <typename TI>
__global__ void __launch_bounds__(256, 2) k_adj_edges_gather(Grid g, int d, const double* u, const double* Eb0, const double* Eb1, const double* Eb2, double* ub) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;  // the x-face domain is the cell domain
    const bool wall = (d == 2 && !g.zper);
    const int c = d == 0 ? i : (d == 1 ? j : k), nd = d == 0 ? g.nx : (d == 1 ? g.ny : g.nz);
    const long long st = d == 0 ? 1 : (d == 1 ? (long long)g.nx : (long long)g.nx * g.ny);
    const long long base = t - (long long)c * st;  // the cell's column at d-index 0
    const double* Eb[3] = {Eb0, Eb1, Eb2};
    for (int n = 0; n < 3; ++n) {
        const double* un = u + n * g.N;
        A q[7];  // cells c - 3 .. c + 3 (wrapped; unused where a wall cuts the column)
        for (int s = -3; s <= 3; ++s) {
            int m = c + s;
            if (wall) m = m < 0 ? 0 : (m >= nd ? nd - 1 : m);
            else m = m < 0 ? m + nd : (m >= nd ? m - nd : m);
            q[s + 3] = (A)un[base + m * st];
        }
        A acc = A(0);
        for (int o = -1; o <= 2; ++o) {  // face m = c + o; the cell is its cell m + 1 - (o + 1) ... role 2 - o
            int m = c + o;
            if (wall) {
                if (m < 2 || m > nd - 2) continue;
            } else {
                m = m < 0 ? m + nd : (m >= nd ? m - nd : m);
            }
            const double eb64 = Eb[n][base + m * st];
            if (!(dbits(eb64) & kMag)) continue;
            A gr[4];
            edge_rev(q[o + 1], q[o + 2], q[o + 3], q[o + 4], (A)eb64, gr);
            acc += gr[2 - o];
        }
        if (nonzero(acc)) ub[n * g.N + t] += (double)acc;
    }
}

// ---- reverse of the CW84 limiter + trace.  Given the adjoint tb of the trace
// value, accumulate into the adjoints of sm_in, s0, sp_in and return the
// adjoint of sig.
template <typename A>
__device__ inline A rev_trace(bool hi_side, A smi, A s0, A spi, A sig, A tb, A& gsm, A& gs0, A& gsp) {
    A sm = smi, sp = spi;
    int cs = 0;
    // the forward's CW84 decisions (k_ppm_*: cw84)
    const A dp = sp - s0, dm = s0 - sm;
    if (!same_sign(dp, dm)) {
        cs = 1;
        sp = s0;
        sm = s0;
    } else if (!abs_lt(dp, A(2) * dm)) {
        cs = 2;
        sp = s0 + A(2) * dm;
    } else if (!abs_lt(dm, A(2) * dp)) {
        cs = 3;
        sm = s0 - A(2) * dp;
    }
    const A Bf = A(1) - A(2.0 / 3.0) * sig;
    const A s6 = A(6) * s0 - A(3) * (sm + sp);
    A dsm, dsp, ds0, dsig;
    if (hi_side) {
        dsp = A(1) - A(0.5) * sig * (A(1) + A(3) * Bf);
        dsm = A(0.5) * sig * (A(1) - A(3) * Bf);
        ds0 = A(3) * sig * Bf;
        dsig = A(-0.5) * ((sp - sm) - Bf * s6) - A(1.0 / 3.0) * sig * s6;
    } else {
        dsm = A(1) - A(0.5) * sig * (A(1) + A(3) * Bf);
        dsp = A(0.5) * sig * (A(1) - A(3) * Bf);
        ds0 = A(3) * sig * Bf;
        dsig = A(0.5) * ((sp - sm) + Bf * s6) - A(1.0 / 3.0) * sig * s6;
    }
    A bsm = dsm * tb, bsp = dsp * tb, bs0 = ds0 * tb;
    if (cs == 1) {
        bs0 += bsm + bsp;
        bsm = A(0);
        bsp = A(0);
    } else if (cs == 2) {
        bs0 += A(3) * bsp;
        bsm += A(-2) * bsp;
        bsp = A(0);
    } else if (cs == 3) {
        bs0 += A(3) * bsm;
        bsp += A(-2) * bsm;
        bsm = A(0);
    }
    gsm += bsm;
    gsp += bsp;
    gs0 += bs0;
    return dsig * tb;
}

template <typename A>
__device__ inline void rev_upwind(A vel, A ob, A& lb, A& hb) {
    if (!below_small_abs(vel)) {
        if (ge0(vel)) lb += ob; else hb += ob;
    } else {
        lb += A(0.5) * ob;
        hb += A(0.5) * ob;
    }
}
template <typename A>
__device__ inline void rev_riemann(A lo, A hi, A ob, A& lb, A& hb) {
    const A sum = lo + hi;
    const bool ltm = (le0(lo) && ge0(hi)) || below_small_abs(sum);
    if (ltm) return;
    if (ge0(sum)) lb += ob; else hb += ob;
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
// Arithmetic in the forward's precision TI; adjoint arrays FP64.
template <int MODE, typename TI>
__global__ void k_adj_faces(Grid g, int d, const double* u, KI<TI> E, double s, double rho, const double* umac_d, KI<TI> LO, KI<TI> HI,
                            const TI* ad, K3 LOb, K3 HIb, const double* adb, K3 TEb, A3 Eb, double* ub, double* umacb_d) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = t;
    const long long fm = fidx(g, d, i - di, j - dj, k - dk), fp = fidx(g, d, i + di, j + dj, k + dk);
    A lb[3], hb[3];
    for (int n = 0; n < 3; ++n) {
        lb[n] = (A)LOb.p[n][f];
        hb[n] = (A)HIb.p[n][f];
    }
    A ul = A(0), uh = A(0);
    if (MODE == 0) {
        if (!wl) ul = Q<A>(g, u, d, i - di, j - dj, k - dk);
        if (!wh) uh = Q<A>(g, u, d, i, j, k);
        rev_riemann(LO.p[d][f], HI.p[d][f], (A)adb[f], lb[d], hb[d]);
        const A a = ad[f];
        for (int n = 0; n < 3; ++n)
            if (n != d) rev_upwind(a, (A)TEb.p[n][f], lb[n], hb[n]);
    } else {
        const A umf = (A)umac_d[f];
        ul = uh = umf;
        for (int n = 0; n < 3; ++n) rev_upwind(umf, (A)TEb.p[n][f], lb[n], hb[n]);
    }
    if (d == 2)
        for (int n = 0; n < 3; ++n) zbc_rev(g, k, n, lb[n], hb[n]);
    const A scale = (MODE == 1) ? (A)rho : A(1);
    const A sT = (A)s;
    A gul = A(0), guh = A(0);
    for (int n = 0; n < 3; ++n) {
        const A tl = lb[n] * scale, th = hb[n] * scale;
        if (!wl && nonzero(tl)) {  // high-side trace of cell c - e_d
            A gsm = A(0), gs0 = A(0), gsp = A(0);
            const A s0 = Q<A>(g, u, n, i - di, j - dj, k - dk);
            if (above_small(ul)) {
                const A bsig = rev_trace(true, E.p[n][fm], s0, E.p[n][f], absv(ul) * sT, tl, gsm, gs0, gsp);
                gul += bsig * sT * (ge0(ul) ? A(1) : A(-1));
            } else {
                gs0 += tl;
            }
            aadd(&Eb.p[n][fm], (double)gsm);
            aadd(&Eb.p[n][f], (double)gsp);
            Qb(g, ub, n, i - di, j - dj, k - dk, (double)gs0);
        }
        if (!wh && nonzero(th)) {  // low-side trace of cell c
            A gsm = A(0), gs0 = A(0), gsp = A(0);
            const A s0 = Q<A>(g, u, n, i, j, k);
            if (below_msmall(uh)) {
                const A bsig = rev_trace(false, E.p[n][f], s0, E.p[n][fp], absv(uh) * sT, th, gsm, gs0, gsp);
                guh += bsig * sT * (ge0(uh) ? A(1) : A(-1));
            } else {
                gs0 += th;
            }
            aadd(&Eb.p[n][f], (double)gsm);
            aadd(&Eb.p[n][fp], (double)gsp);
            Qb(g, ub, n, i, j, k, (double)gs0);
        }
    }
    if (MODE == 0) {
        if (!wl) Qb(g, ub, d, i - di, j - dj, k - dk, (double)gul);
        if (!wh) Qb(g, ub, d, i, j, k, (double)guh);
    } else {
        aadd(&umacb_d[f], (double)(gul + guh));
    }
}

// ---- gather form of k_adj_faces.  A cell's value and the edges of its two
// d-faces are read by exactly two traces: its high-side trace at the face
// above (adjoint lb of that face) and its low-side trace at the face below
// (hb).  The per-cell pass re-forms the state adjoints of its two faces
// (LOb / HIb with the Riemann / upwind reverse and the wall rule, as
// k_adj_faces), reverses the two traces, owns the cell's velocity adjoint
// (before the MAC projection also that of its advective component), and
// keeps the edge adjoints of its lower and upper face (G[0..2], G[3..5]) and,
// after the MAC projection, the MAC-velocity adjoints (G[6], G[7]); the
// per-face pass gathers them.  Needs at least 2 cells along d.
template <int MODE, typename TI>
__device__ inline void face_state_rev(const Grid& g, int d, long long f, int kf, const KI<TI>& LO, const KI<TI>& HI, const TI* ad, const K3& LOb,
                                      const K3& HIb, const double* adb, const K3& TEb, const double* umac_d, TI lb[3], TI hb[3]) {
    using A = TI;
    for (int n = 0; n < 3; ++n) {
        lb[n] = (A)LOb.p[n][f];
        hb[n] = (A)HIb.p[n][f];
    }
    if (MODE == 0) {
        rev_riemann(LO.p[d][f], HI.p[d][f], (A)adb[f], lb[d], hb[d]);
        const A a = ad[f];
        for (int n = 0; n < 3; ++n)
            if (n != d) rev_upwind(a, (A)TEb.p[n][f], lb[n], hb[n]);
    } else {
        const A umf = (A)umac_d[f];
        for (int n = 0; n < 3; ++n) rev_upwind(umf, (A)TEb.p[n][f], lb[n], hb[n]);
    }
    if (d == 2)
        for (int n = 0; n < 3; ++n) zbc_rev(g, kf, n, lb[n], hb[n]);
}

template <int MODE, typename TI>
__global__ void __launch_bounds__(256, 2) k_adj_faces_cells(Grid g, int d, const double* u, KI<TI> E, double s, double rho, const double* umac_d,
                                                            KI<TI> LO, KI<TI> HI, const TI* ad, K3 LOb, K3 HIb, const double* adb, K3 TEb,
                                                            double* ub, TI* G) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;  // the x-face domain is the cell domain
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
    const long long flo = fidx(g, d, i, j, k), fhi = fidx(g, d, i + di, j + dj, k + dk);
    A lbH[3], hbH[3], lbL[3], hbL[3];
    face_state_rev<MODE, TI>(g, d, fhi, k + dk, LO, HI, ad, LOb, HIb, adb, TEb, umac_d, lbH, hbH);
    face_state_rev<MODE, TI>(g, d, flo, k, LO, HI, ad, LOb, HIb, adb, TEb, umac_d, lbL, hbL);
    const A scale = (MODE == 1) ? (A)rho : A(1), sT = (A)s;
    A uhi, ulo;  // the trace speeds: the cell's own advective component, or the MAC velocity of each face
    if (MODE == 0) uhi = ulo = Q<A>(g, u, d, i, j, k);
    else {
        uhi = (A)umac_d[fhi];
        ulo = (A)umac_d[flo];
    }
    A guh = A(0), gul = A(0);
    for (int n = 0; n < 3; ++n) {
        A gsm = A(0), gs0 = A(0), gsp = A(0);
        const A s0 = Q<A>(g, u, n, i, j, k);
        const A tl = lbH[n] * scale;  // high-side trace (at the face above)
        if (nonzero(tl)) {
            if (above_small(uhi)) {
                const A bsig = rev_trace(true, E.p[n][flo], s0, E.p[n][fhi], absv(uhi) * sT, tl, gsm, gs0, gsp);
                guh += bsig * sT * (ge0(uhi) ? A(1) : A(-1));
            } else {
                gs0 += tl;
            }
        }
        const A th = hbL[n] * scale;  // low-side trace (at the face below)
        if (nonzero(th)) {
            if (below_msmall(ulo)) {
                const A bsig = rev_trace(false, E.p[n][flo], s0, E.p[n][fhi], absv(ulo) * sT, th, gsm, gs0, gsp);
                gul += bsig * sT * (ge0(ulo) ? A(1) : A(-1));
            } else {
                gs0 += th;
            }
        }
        G[n * g.N + t] = gsm;
        G[(3 + n) * g.N + t] = gsp;
        if (nonzero(gs0)) ub[n * g.N + t] += (double)gs0;
    }
    if (MODE == 0) {
        const A gu = guh + gul;
        if (nonzero(gu)) ub[d * g.N + t] += (double)gu;
    } else {
        G[6 * g.N + t] = gul;
        G[7 * g.N + t] = guh;
    }
}

template <int MODE, typename TI>
__global__ void k_adj_faces_gather(Grid g, int d, const TI* G, A3 Eb, double* umacb_d) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const bool walls = d == 2 && !g.zper;
    const bool hasm = !(walls && k == 0), hasp = !(walls && k == g.nz);
    const long long cp = hasp ? cidx(g, i, j, k) : 0;
    const long long cm = hasm ? cidx(g, wrapn(i - (d == 0), g.nx), wrapn(j - (d == 1), g.ny), g.zper ? wrapn(k - (d == 2), g.nz) : k - (d == 2)) : 0;
    for (int n = 0; n < 3; ++n) {  // the upper edge terms of the cell below, the lower ones of the cell above
        const A v = (hasm ? G[(3 + n) * g.N + cm] : A(0)) + (hasp ? G[n * g.N + cp] : A(0));
        if (nonzero(v)) Eb.p[n][t] += (double)v;
    }
    if (MODE == 1) {
        const A w = (hasm ? G[7 * g.N + cm] : A(0)) + (hasp ? G[6 * g.N + cp] : A(0));
        if (nonzero(w)) umacb_d[t] += (double)w;
    }
}

// ---- reverse of k_pm_trans (a, b, n)
template <typename TI>
__global__ void k_adj_pm_trans(Grid g, int a, int b, int n, double cb64, const TI* ad_a, const TI* ad_b, const TI* edge_b, const double* outb,
                               double* lo_anb, double* hi_anb, double* ad_bb, double* edge_bb) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, a, t, i, j, k)) return;
    const long long f = t;
    const double ob64 = outb[f];
    if (!(dbits(ob64) & kMag)) return;
    const A ob = (A)ob64, cb = (A)cb64;
    const bool wl = (a == 2 && !g.zper && k == 0), wh = (a == 2 && !g.zper && k == g.nz);
    A lb = A(0), hb = A(0);
    rev_upwind(ad_a[f], ob, lb, hb);
    if (a == 2) zbc_rev(g, k, n, lb, hb);
    lo_anb[f] += (double)lb;
    hi_anb[f] += (double)hb;
    const int e0 = (b == 0), e1 = (b == 1), e2 = (b == 2);
    if (!wh && nonzero(hb)) {
        const long long f0 = fidx(g, b, i, j, k), f1 = fidx(g, b, i + e0, j + e1, k + e2);
        const A S = ad_b[f1] + ad_b[f0], Dd = edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], (double)(-cb * Dd * hb));
        aadd(&ad_bb[f0], (double)(-cb * Dd * hb));
        aadd(&edge_bb[f1], (double)(-cb * S * hb));
        aadd(&edge_bb[f0], (double)(cb * S * hb));
    }
    if (!wl && nonzero(lb)) {
        const int ci = i - (a == 0), cj = j - (a == 1), ck = k - (a == 2);
        const long long f0 = fidx(g, b, ci, cj, ck), f1 = fidx(g, b, ci + e0, cj + e1, ck + e2);
        const A S = ad_b[f1] + ad_b[f0], Dd = edge_b[f1] - edge_b[f0];
        aadd(&ad_bb[f1], (double)(-cb * Dd * lb));
        aadd(&ad_bb[f0], (double)(-cb * Dd * lb));
        aadd(&edge_bb[f1], (double)(-cb * S * lb));
        aadd(&edge_bb[f0], (double)(cb * S * lb));
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
__global__ void k_adj_pm_final(Grid g, int d, double dt, double c1_64, double c2_64, const TI* lo_dd, const TI* hi_dd, KI<TI> AD, const TI* T1,
                               const TI* T2, const double* forces, const double* macb, double* lo_ddb, double* hi_ddb, A3 ADb, double* T1b,
                               double* T2b, double* forcesb) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    if (d == 2 && !g.zper && (k == 0 || k == g.nz)) return;  // wall faces: the normal velocity is 0 whatever the input
    const long long f = t;
    const double mb64 = macb[f];
    if (!(dbits(mb64) & kMag)) return;
    const A mb = (A)mb64, c1 = (A)c1_64, c2 = (A)c2_64, hdt = A(0.5) * (A)dt;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    auto side_val = [&](int ci, int cj, int ck, A base) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        // the forward's sum in its own precision (decides the Riemann branch)
        A s = base;
        s -= c1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        s += hdt * (A)forces[d * g.N + cell_fo(g, ci, cj, ck)];
        return s;
    };
    auto side_rev = [&](int ci, int cj, int ck, A sb) {
        const long long p1 = fidx(g, b1, ci + (b1 == 0), cj + (b1 == 1), ck + (b1 == 2)), m1 = fidx(g, b1, ci, cj, ck);
        const long long p2 = fidx(g, b2, ci + (b2 == 0), cj + (b2 == 1), ck + (b2 == 2)), m2 = fidx(g, b2, ci, cj, ck);
        const A S1 = AD.p[b1][p1] + AD.p[b1][m1], D1 = T1[p1] - T1[m1];
        const A S2 = AD.p[b2][p2] + AD.p[b2][m2], D2 = T2[p2] - T2[m2];
        aadd(&ADb.p[b1][p1], (double)(-c1 * D1 * sb));
        aadd(&ADb.p[b1][m1], (double)(-c1 * D1 * sb));
        aadd(&T1b[p1], (double)(-c1 * S1 * sb));
        aadd(&T1b[m1], (double)(c1 * S1 * sb));
        aadd(&ADb.p[b2][p2], (double)(-c2 * D2 * sb));
        aadd(&ADb.p[b2][m2], (double)(-c2 * D2 * sb));
        aadd(&T2b[p2], (double)(-c2 * S2 * sb));
        aadd(&T2b[m2], (double)(c2 * S2 * sb));
        aadd(&forcesb[d * g.N + cell_fo(g, ci, cj, ck)], (double)(hdt * sb));
    };
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const A stl = side_val(li, lj, lk, lo_dd[f]), sth = side_val(i, j, k, hi_dd[f]);
    A bl = A(0), bh = A(0);
    rev_riemann(stl, sth, mb, bl, bh);
    if (nonzero(bl)) {
        lo_ddb[f] += (double)bl;
        side_rev(li, lj, lk, bl);
    }
    if (nonzero(bh)) {
        hi_ddb[f] += (double)bh;
        side_rev(i, j, k, bh);
    }
}

// ---- reverse of the post-MAC stages 2 and 3 (k_adv_trans_x/col,
// k_adv_flux_x/col) in gather form.  The forward gives every face state its
// cell's correction, corr(c) = hdt F(c) + q(c) r(c) - c1 x1(c) - c2 x2(c)
// (stage 3; r = rho (c1 (v1+ - v1-) + c2 (v2+ - v2-)), x_b = T_b(+) v_b+ -
// T_b(-) v_b- over the b faces of c) or the pair corr_b(c) = q(c) rho cb
// (v_b+ - v_b-) - cb (v_b+ E_b(+) - v_b- E_b(-)) (stage 2).  The reverse:
//  - per d-face, the upwind selection's adjoints of the two states (bl, bh)
//    and of the advective velocity (k_adj_flux_faces, stage 3 only);
//  - per cell, the adjoint of its correction, cb(c) = bl(face above) +
//    bh(face below), and what the cell owns: the velocity and forces
//    adjoints, the state adjoints of its low face (k_adj_*_cells); cb is kept
//    per cell, in the pass precision;
//  - per transverse face, the adjoints of T_b / E_b and of the MAC velocity
//    there, gathered from cb of its two cells (k_adj_*_bfaces).
// Every adjoint is written by the one thread that owns it: no atomics.  The
// arithmetic is the pass precision's, and each owned value takes one FP64
// add: FP64 issues at 1/64 of the FP32 rate, and an FP64 atomic's add runs in
// L2, so a gather form that summed its terms in FP64 on the SM (as the
// accumulations of a scatter form would) was slower than the atomics.

// stage 3, per d-face: gum = sum_n st_n fb_n (the upwinded state), and the
// face's LO / HI adjoints
template <typename TI>
__global__ void k_adj_flux_faces(Grid g, int d, const double* u, const double* forces, double rho64, double dt64, double c1_64, double c2_64,
                                 K3 Uf, KI<TI> LO, KI<TI> HI, KI<TI> T1, KI<TI> T2, K3 Fb, double* Udb, A3 LOb, A3 HIb) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, d, t, i, j, k)) return;
    const bool wl = (d == 2 && !g.zper && k == 0), wh = (d == 2 && !g.zper && k == g.nz);
    const long long f = t;
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const A um = (A)Uf.p[d][f];
    const A rho = (A)rho64, c1 = (A)c1_64, c2 = (A)c2_64, hdt = A(0.5) * (A)dt64;
    const int li = i - (d == 0), lj = j - (d == 1), lk = k - (d == 2);
    const long long lp1 = fidx(g, b1, li + (b1 == 0), lj + (b1 == 1), lk + (b1 == 2)), lm1 = fidx(g, b1, li, lj, lk);
    const long long lp2 = fidx(g, b2, li + (b2 == 0), lj + (b2 == 1), lk + (b2 == 2)), lm2 = fidx(g, b2, li, lj, lk);
    const long long hp1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), hm1 = fidx(g, b1, i, j, k);
    const long long hp2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), hm2 = fidx(g, b2, i, j, k);
    A l1p = A(0), l1m = A(0), l2p = A(0), l2m = A(0), h1p = A(0), h1m = A(0), h2p = A(0), h2m = A(0);
    if (!wl) {
        l1p = (A)Uf.p[b1][lp1];
        l1m = (A)Uf.p[b1][lm1];
        l2p = (A)Uf.p[b2][lp2];
        l2m = (A)Uf.p[b2][lm2];
    }
    if (!wh) {
        h1p = (A)Uf.p[b1][hp1];
        h1m = (A)Uf.p[b1][hm1];
        h2p = (A)Uf.p[b2][hp2];
        h2m = (A)Uf.p[b2][hm2];
    }
    A gum = A(0);
    const long long cl = wl ? 0 : cell_fo(g, li, lj, lk);
    const long long ch = wh ? 0 : cell_fo(g, i, j, k);
    for (int n = 0; n < 3; ++n) {
        const double fb64 = Fb.p[n][f];
        if (!(dbits(fb64) & kMag)) continue;
        const A fb = (A)fb64;
        // the forward's face states in its own precision (the upwind branch is
        // set by um alone; the states enter gum)
        A stl = A(0), sth = A(0);
        if (!wl) {
            const A q = rho * (A)u[n * g.N + cl];
            A s_ = LO.p[n][f];
            s_ -= c1 * (T1.p[n][lp1] * l1p - T1.p[n][lm1] * l1m);
            s_ -= c2 * (T2.p[n][lp2] * l2p - T2.p[n][lm2] * l2m);
            s_ += c1 * q * (l1p - l1m);
            s_ += c2 * q * (l2p - l2m);
            s_ += hdt * (rho * (A)forces[n * g.N + cl]);
            stl = s_;
        }
        if (!wh) {
            const A q = rho * (A)u[n * g.N + ch];
            A s_ = HI.p[n][f];
            s_ -= c1 * (T1.p[n][hp1] * h1p - T1.p[n][hm1] * h1m);
            s_ -= c2 * (T2.p[n][hp2] * h2p - T2.p[n][hm2] * h2m);
            s_ += c1 * q * (h1p - h1m);
            s_ += c2 * q * (h2p - h2m);
            s_ += hdt * (rho * (A)forces[n * g.N + ch]);
            sth = s_;
        }
        A zl = stl, zh = sth;
        if (d == 2) zbc_fwd(g, k, n, zl, zh);
        A st, bl = A(0), bh = A(0);
        if (below_small_abs(um)) {
            st = A(0.5) * (zl + zh);
            bl = bh = A(0.5) * um * fb;
        } else if (ge0(um)) {
            st = zl;
            bl = um * fb;
        } else {
            st = zh;
            bh = um * fb;
        }
        gum += st * fb;
        if (d == 2) zbc_rev(g, k, n, bl, bh);
        if (!wl) LOb.p[n][f] += (double)bl;
        if (!wh) HIb.p[n][f] += (double)bh;
    }
    if (nonzero(gum)) Udb[f] += (double)gum;
}

// adjoints (bl, bh) of the two states of a d-face of stage 3 (the upwind
// selection by um, then the wall rule)
template <typename A>
__device__ inline void flux_state_rev(const Grid& g, int d, int k, int n, A um, A fb, A& bl, A& bh) {
    bl = bh = A(0);
    if (below_small_abs(um)) bl = bh = A(0.5) * um * fb;
    else if (ge0(um)) bl = um * fb;
    else bh = um * fb;
    if (d == 2) zbc_rev(g, k, n, bl, bh);
}

// stage 3, per cell: cb = bl(face above) + bh(face below); the velocity and
// forces adjoints of the cell; cb kept in CB (3 components)
template <typename TI>
__global__ void k_adj_flux_cells(Grid g, int d, double rho64, double dt64, double c1_64, double c2_64, K3 Uf, K3 Fb, double* ub, double* forcesb,
                                 TI* CB) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;  // the x-face domain is the cell domain
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const long long flo = fidx(g, d, i, j, k), fhi = fidx(g, d, i + (d == 0), j + (d == 1), k + (d == 2));
    const A ulo = (A)Uf.p[d][flo], uhi = (A)Uf.p[d][fhi];
    const long long p1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), m1 = fidx(g, b1, i, j, k);
    const long long p2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), m2 = fidx(g, b2, i, j, k);
    const A rho = (A)rho64, c1 = (A)c1_64, c2 = (A)c2_64, hdt = A(0.5) * (A)dt64;
    const A r = rho * (c1 * ((A)Uf.p[b1][p1] - (A)Uf.p[b1][m1]) + c2 * ((A)Uf.p[b2][p2] - (A)Uf.p[b2][m2]));
    for (int n = 0; n < 3; ++n) {
        A bl, bh, dl, dh;
        flux_state_rev(g, d, k, n, ulo, (A)Fb.p[n][flo], dl, bh);
        flux_state_rev(g, d, k + 1, n, uhi, (A)Fb.p[n][fhi], bl, dh);
        const A cb = bh + bl;
        CB[n * g.N + t] = cb;
        if (nonzero(cb)) {
            ub[n * g.N + t] += (double)(r * cb);
            forcesb[n * g.N + t] += (double)(hdt * rho * cb);
        }
    }
}

// stage 3 / stage 2, per b-face: the faces' T_b (E_b) and MAC velocity
// adjoints from cb of the cells below (c-, the face is its high b face) and
// above (c+, its low b face):
//   Tb_n += c v (cb_n(c+) - cb_n(c-)),
//   vb += c sum_n (T_n (cb_n(c+) - cb_n(c-)) + rho (q_n(c-) cb_n(c-) - q_n(c+) cb_n(c+)))
// (c = c_b of stage 3, cb of stage 2).  CB holds the cb of this b.
template <typename TI>
__global__ void k_adj_bfaces(Grid g, int b, const double* u, double rho64, double c64, const double* vb, KI<TI> T, const TI* CB, A3 Tb,
                             double* vbb) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, b, t, i, j, k)) return;
    const bool walls = b == 2 && !g.zper;
    const bool hasm = !(walls && k == 0), hasp = !(walls && k == g.nz);
    const long long f = t;
    const long long cp = hasp ? cidx(g, i, j, k) : 0;
    const long long cm = hasm ? cidx(g, wrapn(i - (b == 0), g.nx), wrapn(j - (b == 1), g.ny), g.zper ? wrapn(k - (b == 2), g.nz) : k - (b == 2)) : 0;
    const A c = (A)c64, rho = (A)rho64, v = (A)vb[f];
    A gv = A(0);
    for (int n = 0; n < 3; ++n) {
        const A bp = hasp ? CB[n * g.N + cp] : A(0), bm = hasm ? CB[n * g.N + cm] : A(0);
        if (!nonzero(bp) && !nonzero(bm)) continue;
        const A e = T.p[n][f];
        Tb.p[n][f] += (double)(c * v * (bp - bm));
        const A qm = hasm ? rho * (A)u[n * g.N + cm] : A(0), qp = hasp ? rho * (A)u[n * g.N + cp] : A(0);
        gv += (c * qm - c * e) * bm + (c * e - c * qp) * bp;
    }
    if (nonzero(gv)) vbb[f] += (double)gv;
}

// stage 2 for the a-faces, per cell: the adjoints of its two corrections (one
// per transverse direction), cb_k = lb_k(face above) + hb_k(face below) from
// the upwind selections of outputs O1 (along b1) and O2 (along b2); the
// velocity adjoint of the cell; the LO / HI adjoints of its low a-face (and
// of the top wall face from the cells under it).  CB holds cb_1 then cb_2.
template <typename TI>
__global__ void k_adj_trans_cells(Grid g, int a, double rho64, double cb1_64, double cb2_64, const double* ua, const double* v1, const double* v2,
                                  K3 O1b, K3 O2b, A3 LOb, A3 HIb, double* ub, TI* CB) {
    using A = TI;
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;
    const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
    const bool top = a == 2 && !g.zper && k + 1 == g.nz;  // the face above is the top wall face
    const long long flo = fidx(g, a, i, j, k), fhi = fidx(g, a, i + (a == 0), j + (a == 1), k + (a == 2));
    const A ulo = (A)ua[flo], uhi = (A)ua[fhi];
    const long long p1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), m1 = fidx(g, b1, i, j, k);
    const long long p2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), m2 = fidx(g, b2, i, j, k);
    const A rho = (A)rho64;
    const A w1 = rho * (A)cb1_64 * ((A)v1[p1] - (A)v1[m1]), w2 = rho * (A)cb2_64 * ((A)v2[p2] - (A)v2[m2]);
    A ubs[3];
    for (int n = 0; n < 3; ++n) {
        A l1 = A(0), h1 = A(0), l2 = A(0), h2 = A(0), L1 = A(0), H1 = A(0), L2 = A(0), H2 = A(0);
        rev_upwind(ulo, (A)O1b.p[n][flo], l1, h1);  // face below
        rev_upwind(ulo, (A)O2b.p[n][flo], l2, h2);
        rev_upwind(uhi, (A)O1b.p[n][fhi], L1, H1);  // face above
        rev_upwind(uhi, (A)O2b.p[n][fhi], L2, H2);
        if (a == 2) {
            zbc_rev(g, k, n, l1, h1);
            zbc_rev(g, k, n, l2, h2);
            zbc_rev(g, k + 1, n, L1, H1);
            zbc_rev(g, k + 1, n, L2, H2);
        }
        const A sl = l1 + l2, sh = h1 + h2;
        if (nonzero(sl)) LOb.p[n][flo] += (double)sl;
        if (nonzero(sh)) HIb.p[n][flo] += (double)sh;
        if (top) {
            LOb.p[n][fhi] += (double)(L1 + L2);
            HIb.p[n][fhi] += (double)(H1 + H2);
        }
        const A cb1 = h1 + L1, cb2 = h2 + L2;
        CB[n * g.N + t] = cb1;
        CB[(3 + n) * g.N + t] = cb2;
        ubs[n] = w1 * cb1 + w2 * cb2;
    }
    for (int n = 0; n < 3; ++n)
        if (nonzero(ubs[n])) ub[n * g.N + t] += (double)ubs[n];
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
// shared memory of the reverse diffusion tile: FP64 accumulators (4 per box
// cell) and the staged values in the arithmetic type A (7 per box cell)
template <typename A>
constexpr size_t adj_tau_smem() { return sizeof(A) * 11 * (size_t)ANH; }

// A: arithmetic of the face terms and of the tile's shared-memory
// accumulators, double, or float for the reverse of the mixed-precision
// form's FP32 diffusion (native FP32 shared-memory atomics; each tile
// position sums a few dozen face terms); the flush adds them to the FP64
// adjoints.
template <typename A>
__global__ void __launch_bounds__(ATX* ATY* ATZ) k_adj_tau_tile(Grid g, const double* vel, const double* mu, const double* wg,
                                                                const double* db, double s, double* ub, double* mub, double* wgb) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    A* aU = reinterpret_cast<A*>(sm_raw);  // [3][box] accumulated velocity adjoint
    A* aM = aU + 3 * ANH;                  // [box] accumulated viscosity adjoint
    A* sV = aM + ANH;                      // [3][box]
    A* sD = sV + 3 * ANH;                            // [3][box] divergence adjoint (cells in the domain, else 0)
    A* sM = sV + 6 * ANH;                            // [box]
    const int i0 = blockIdx.x * ATX, j0 = blockIdx.y * ATY, k0 = blockIdx.z * ATZ;
    const int tid = threadIdx.x, nthr = ATX * ATY * ATZ;
    auto hb = [](int hx, int hy, int hz) { return (hz * AHY + hy) * AHX + hx; };
    const A sA = (A)s;
    for (int h = tid; h < ANH; h += nthr) {
        const int hx = h % AHX, hy = (h / AHX) % AHY, hz = h / (AHX * AHY);
        const int gi = ((i0 + hx - 1) % g.nx + g.nx) % g.nx, gj = ((j0 + hy - 1) % g.ny + g.ny) % g.ny;
        int gk = k0 + hz - 1;
        const bool inz = g.zper || (gk >= 0 && gk < g.nz);
        if (g.zper) gk = (gk % g.nz + g.nz) % g.nz;
        for (int n = 0; n < 3; ++n) sV[n * ANH + h] = (A)Vd(g, vel, wg, n, gi, gj, gk);
        const int kk = g.zper ? gk : (gk < 0 ? 0 : (gk >= g.nz ? g.nz - 1 : gk));
        const long long c = cidx(g, gi, gj, kk);
        sM[h] = (A)mu[c];
        for (int n = 0; n < 3; ++n) {
            sD[n * ANH + h] = inz ? sA * (A)db[n * g.N + c] : A(0);
            aU[n * ANH + h] = A(0);
        }
        aM[h] = A(0);
    }
    __syncthreads();
    const A ih[3] = {(A)g.idx, (A)g.idy, (A)g.idz};
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
        A Fb[3];
        bool any = false;
        for (int n = 0; n < 3; ++n) {
            Fb[n] = ((has_lo ? sD[n * ANH + hb(mx, my, mz)] : A(0)) - (has_hi ? sD[n * ANH + hb(hx, hy, hz)] : A(0))) * ih[d];
            any = any || nonzero(Fb[n]);
        }
        if (!any) continue;
        A mf;
        if (!has_lo) mf = sM[hb(hx, hy, hz)];
        else if (!has_hi) mf = sM[hb(mx, my, mz)];
        else mf = A(0.5) * (sM[hb(mx, my, mz)] + sM[hb(hx, hy, hz)]);
        A gr[3][3];
        for (int n = 0; n < 3; ++n) {
            const A* v = sV + n * ANH;
            for (int m = 0; m < 3; ++m) {
                if (m == d) {
                    gr[m][n] = (v[hb(hx, hy, hz)] - v[hb(mx, my, mz)]) * ih[m];
                } else {
                    const int f0 = (m == 0), f1 = (m == 1), f2 = (m == 2);
                    gr[m][n] = A(0.25) *
                               (v[hb(hx + f0, hy + f1, hz + f2)] + v[hb(mx + f0, my + f1, mz + f2)] - v[hb(hx - f0, hy - f1, hz - f2)] -
                                v[hb(mx - f0, my - f1, mz - f2)]) *
                               ih[m];
                }
            }
        }
        const A dv = gr[0][0] + gr[1][1] + gr[2][2];
        A mfb = A(0), dvb = A(0);
        A grb[3][3] = {{A(0), A(0), A(0)}, {A(0), A(0), A(0)}, {A(0), A(0), A(0)}};
        for (int n = 0; n < 3; ++n) {
            const A Sn = (n == d) ? (A(2) * gr[d][d] - A(2.0 / 3.0) * dv) : (gr[d][n] + gr[n][d]);
            mfb += Fb[n] * Sn;
            const A sb = mf * Fb[n];
            if (n == d) {
                grb[d][d] += A(2) * sb;
                dvb += A(-2.0 / 3.0) * sb;
            } else {
                grb[d][n] += sb;
                grb[n][d] += sb;
            }
        }
        for (int m = 0; m < 3; ++m) grb[m][m] += dvb;
        if (!has_lo) atomicAdd(&aM[hb(hx, hy, hz)], mfb);
        else if (!has_hi) atomicAdd(&aM[hb(mx, my, mz)], mfb);
        else {
            const A hm = A(0.5) * mfb;
            atomicAdd(&aM[hb(mx, my, mz)], hm);
            atomicAdd(&aM[hb(hx, hy, hz)], hm);
        }
        for (int n = 0; n < 3; ++n) {
            A* a = aU + n * ANH;
            for (int m = 0; m < 3; ++m) {
                const A b = grb[m][n];
                if (!nonzero(b)) continue;
                if (m == d) {
                    const A w = b * ih[m];
                    atomicAdd(&a[hb(hx, hy, hz)], w);
                    atomicAdd(&a[hb(mx, my, mz)], -w);
                } else {
                    const int f0 = (m == 0), f1 = (m == 1), f2 = (m == 2);
                    const A w = A(0.25) * b * ih[m];
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
        for (int n = 0; n < 3; ++n) Vdb(g, ub, wgb, n, gi, gj, gk, (double)aU[n * ANH + h]);
        if (mub && nonzero(aM[h])) {
            if (g.zper || (gk >= 0 && gk < g.nz)) atomicAdd(&mub[cidx(g, gi, gj, g.zper ? (gk % g.nz + g.nz) % g.nz : gk)], (double)aM[h]);
        }
    }
}

// ---- reverse of the Smagorinsky viscosity mu_eff = mu + rho fac |S|(u), in
// the arithmetic type of the forward's strain rate (A)
template <typename A>
__global__ void k_adj_smag(Grid g, const double* vel, const double* mub, double rho, double fac, double* ub) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const double mb = mub[t];
    if (!(dbits(mb) & kMag)) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    A a = A(0.5), b = A(0), c = A(-0.5);
    if (!g.zper && k == 0) {
        a = A(1.0 / 3.0);
        b = A(1);
        c = A(-4.0 / 3.0);
    }
    if (!g.zper && k == g.nz - 1) {
        a = A(4.0 / 3.0);
        b = A(-1);
        c = A(-1.0 / 3.0);
    }
    const A hx = A(0.5 * g.idx), hy = A(0.5 * g.idy), iz = (A)g.idz;
    A gx[3], gy[3], gz[3];
    for (int n = 0; n < 3; ++n) {
        gx[n] = hx * (Q<A>(g, vel, n, i + 1, j, k) - Q<A>(g, vel, n, i - 1, j, k));
        gy[n] = hy * (Q<A>(g, vel, n, i, j + 1, k) - Q<A>(g, vel, n, i, j - 1, k));
        gz[n] = (a * Q<A>(g, vel, n, i, j, k + 1) + b * Q<A>(g, vel, n, i, j, k) + c * Q<A>(g, vel, n, i, j, k - 1)) * iz;
    }
    const A S = sqrt(A(2) * gx[0] * gx[0] + A(2) * gy[1] * gy[1] + A(2) * gz[2] * gz[2] + (gy[0] + gx[1]) * (gy[0] + gx[1]) +
                     (gz[1] + gy[2]) * (gz[1] + gy[2]) + (gx[2] + gz[0]) * (gx[2] + gz[0]));
    if (!(S > A(0))) return;
    const A q = (A)(rho * fac * mb) / S;
    A gxb[3] = {A(2) * q * gx[0], A(0), A(0)}, gyb[3] = {A(0), A(2) * q * gy[1], A(0)}, gzb[3] = {A(0), A(0), A(2) * q * gz[2]};
    const A t1 = q * (gy[0] + gx[1]), t2 = q * (gz[1] + gy[2]), t3 = q * (gx[2] + gz[0]);
    gyb[0] += t1;
    gxb[1] += t1;
    gzb[1] += t2;
    gyb[2] += t2;
    gxb[2] += t3;
    gzb[0] += t3;
    for (int n = 0; n < 3; ++n) {
        const double wx = (double)(hx * gxb[n]), wy = (double)(hy * gyb[n]);
        Qb(g, ub, n, i + 1, j, k, wx);
        Qb(g, ub, n, i - 1, j, k, -wx);
        Qb(g, ub, n, i, j + 1, k, wy);
        Qb(g, ub, n, i, j - 1, k, -wy);
        Qb(g, ub, n, i, j, k + 1, (double)(a * iz * gzb[n]));
        Qb(g, ub, n, i, j, k, (double)(b * iz * gzb[n]));
        Qb(g, ub, n, i, j, k - 1, (double)(c * iz * gzb[n]));
    }
}

// Gather form of k_adj_smag (nz >= 4 or a periodic z): the first pass writes
// each cell's gradient adjoints, scaled by their stencil factors, W = (hx gxb,
// hy gyb, iz gzb) (zeros where the cell has none); the second lets every cell
// collect what the stencils of its neighbours give it:
//   ub += W_x(i-1) - W_x(i+1) + W_y(j-1) - W_y(j+1)
//       + a(k-1) W_z(k-1) + b(k) W_z(k) + c(k+1) W_z(k+1)
// (a, b, c the z stencil of each layer, one-sided at walls), and, at a wall,
// the ghost term of the wall layer's one-sided stencil through the ghost's
// extrapolation (15 q0 - 10 q1 + 3 q2) / 8 onto the three layers next to it
// (the normal component's ghost is 0).
template <typename A>
__device__ inline void smag_zcoef(const Grid& g, int k, A& a, A& b, A& c) {
    a = A(0.5);
    b = A(0);
    c = A(-0.5);
    if (!g.zper && k == 0) {
        a = A(1.0 / 3.0);
        b = A(1);
        c = A(-4.0 / 3.0);
    }
    if (!g.zper && k == g.nz - 1) {
        a = A(4.0 / 3.0);
        b = A(-1);
        c = A(-1.0 / 3.0);
    }
}

template <typename A>
__global__ void k_adj_smag_w(Grid g, const double* vel, const double* mub, double rho, double fac, A* W) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;
    const double mb = mub[t];
    A gxb[3] = {A(0), A(0), A(0)}, gyb[3] = {A(0), A(0), A(0)}, gzb[3] = {A(0), A(0), A(0)};
    const A hx = A(0.5 * g.idx), hy = A(0.5 * g.idy), iz = (A)g.idz;
    if (dbits(mb) & kMag) {
        A a, b, c;
        smag_zcoef(g, k, a, b, c);
        const long long sy = g.nx, sz = (long long)g.nx * g.ny;
        const long long xm = t + (i == 0 ? g.nx - 1 : -1), xp = t + (i + 1 == g.nx ? 1 - g.nx : 1);
        const long long ym = t + (j == 0 ? (long long)(g.ny - 1) * sy : -sy), yp = t + (j + 1 == g.ny ? -(long long)(g.ny - 1) * sy : sy);
        const long long zm = t + (k == 0 ? (long long)(g.nz - 1) * sz : -sz), zp = t + (k + 1 == g.nz ? -(long long)(g.nz - 1) * sz : sz);
        const bool glo = !g.zper && k == 0, ghi = !g.zper && k + 1 == g.nz;  // the z neighbour is a wall ghost
        A gx[3], gy[3], gz[3];
        for (int n = 0; n < 3; ++n) {
            const double* v = vel + n * g.N;
            gx[n] = hx * ((A)v[xp] - (A)v[xm]);
            gy[n] = hy * ((A)v[yp] - (A)v[ym]);
            // fill-patch ghost (VelFPT): the normal component 0, the others
            // (15 q0 - 10 q1 + 3 q2) / 8 from the three cells next to the wall
            A qm, qp;
            if (glo) qm = n == 2 ? A(0) : A(0.125) * (A(15) * (A)v[t] - A(10) * (A)v[t + sz] + A(3) * (A)v[t + 2 * sz]);
            else qm = (A)v[zm];
            if (ghi) qp = n == 2 ? A(0) : A(0.125) * (A(15) * (A)v[t] - A(10) * (A)v[t - sz] + A(3) * (A)v[t - 2 * sz]);
            else qp = (A)v[zp];
            gz[n] = (a * qp + b * (A)v[t] + c * qm) * iz;
        }
        const A S = sqrt(A(2) * gx[0] * gx[0] + A(2) * gy[1] * gy[1] + A(2) * gz[2] * gz[2] + (gy[0] + gx[1]) * (gy[0] + gx[1]) +
                         (gz[1] + gy[2]) * (gz[1] + gy[2]) + (gx[2] + gz[0]) * (gx[2] + gz[0]));
        if (S > A(0)) {
            const A q = (A)(rho * fac * mb) / S;
            gxb[0] = A(2) * q * gx[0];
            gyb[1] = A(2) * q * gy[1];
            gzb[2] = A(2) * q * gz[2];
            const A t1 = q * (gy[0] + gx[1]), t2 = q * (gz[1] + gy[2]), t3 = q * (gx[2] + gz[0]);
            gyb[0] += t1;
            gxb[1] += t1;
            gzb[1] += t2;
            gyb[2] += t2;
            gxb[2] += t3;
            gzb[0] += t3;
        }
    }
    for (int n = 0; n < 3; ++n) {
        W[n * g.N + t] = hx * gxb[n];
        W[(3 + n) * g.N + t] = hy * gyb[n];
        W[(6 + n) * g.N + t] = iz * gzb[n];
    }
}

template <typename A>
__global__ void k_adj_smag_gather(Grid g, const A* W, double* ub) {
    int i, j, k;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (!face_at(g, 0, t, i, j, k)) return;
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long xm = t + (i == 0 ? g.nx - 1 : -1), xp = t + (i + 1 == g.nx ? 1 - g.nx : 1);
    const long long ym = t + (j == 0 ? (long long)(g.ny - 1) * sy : -sy), yp = t + (j + 1 == g.ny ? -(long long)(g.ny - 1) * sy : sy);
    const bool hasm = g.zper || k > 0, hasp = g.zper || k + 1 < g.nz;
    const long long zm = t + (k == 0 ? (long long)(g.nz - 1) * sz : -sz), zp = t + (k + 1 == g.nz ? -(long long)(g.nz - 1) * sz : sz);
    A a, b, c, am, bm, cm, ap, bp, cp;
    smag_zcoef(g, k, a, b, c);
    smag_zcoef(g, k == 0 ? g.nz - 1 : k - 1, am, bm, cm);
    smag_zcoef(g, k + 1 == g.nz ? 0 : k + 1, ap, bp, cp);
    const bool walls = !g.zper;
    const A gw[3] = {A(1.875), A(-1.25), A(0.375)};
    for (int n = 0; n < 3; ++n) {
        const A* Wx = W + n * g.N;
        const A* Wy = W + (3 + n) * g.N;
        const A* Wz = W + (6 + n) * g.N;
        A acc = (Wx[xm] - Wx[xp]) + (Wy[ym] - Wy[yp]) + b * Wz[t];
        if (hasm) acc += am * Wz[zm];
        if (hasp) acc += cp * Wz[zp];
        if (walls && n != 2) {
            const long long col = t - (long long)k * sz;
            if (k <= 2) {  // the bottom wall layer's ghost (its c term)
                A a0, b0, c0;
                smag_zcoef(g, 0, a0, b0, c0);
                acc += gw[k] * c0 * Wz[col];
            }
            if (k >= g.nz - 3) {  // the top wall layer's ghost (its a term)
                A a1, b1, c1;
                smag_zcoef(g, g.nz - 1, a1, b1, c1);
                acc += gw[g.nz - 1 - k] * a1 * Wz[col + (long long)(g.nz - 1) * sz];
            }
        }
        if (nonzero(acc)) ub[n * g.N + t] += (double)acc;
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

template <typename TI>
static void adj_edges_t(Ctx& c, const Grid& g, int d, const double* u, double* const Eb[3], double* ub) {
    const long long nf = nfaces(g, d);
    const int nd = d == 0 ? g.nx : (d == 1 ? g.ny : g.nz);
    if (nd < 4) {  // the gather's window of 7 cells wraps more than once
        KS_LAUNCH(c, k_adj_edges<TI>, nblocks(nf, BS), BS, B8 * (3.0 * nf + 6.0 * g.N), g, d, u, Eb[0], Eb[1], Eb[2], ub);
        return;
    }
    KS_LAUNCH(c, k_adj_edges_gather<TI>, nblocks(g.N, BS), BS, B8 * (3.0 * nf + 6.0 * g.N), g, d, u, Eb[0], Eb[1], Eb[2], ub);
    if (d == 2 && !g.zper) {
        const long long M = 4LL * g.nx * g.ny;
        KS_LAUNCH(c, k_adj_edges_wall<TI>, nblocks(M, BS), BS, B8 * 3.0 * (M + 4.0 * M), g, u, Eb[0], Eb[1], Eb[2], ub);
    }
}
void launch_adj_edges(Ctx& c, const Grid& g, int d, const double* u, double* const Eb[3], double* ub, int fp32) {
    if (fp32) adj_edges_t<float>(c, g, d, u, Eb, ub);
    else adj_edges_t<double>(c, g, d, u, Eb, ub);
}

template <typename TI>
static void adj_faces_t(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                        const double* umac_d, double* scratch) {
    KI<TI> E{{ti<TI>(B.edge[d][0]), ti<TI>(B.edge[d][1]), ti<TI>(B.edge[d][2])}};
    KI<TI> LO{{ti<TI>(B.lo[d][0]), ti<TI>(B.lo[d][1]), ti<TI>(B.lo[d][2])}}, HI{{ti<TI>(B.hi[d][0]), ti<TI>(B.hi[d][1]), ti<TI>(B.hi[d][2])}};
    K3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    K3 TEb{{A.tedge[d][0], A.tedge[d][1], A.tedge[d][2]}};
    A3 Eb{{A.edge[d][0], A.edge[d][1], A.edge[d][2]}};
    const double s = dt * ihd(g, d);
    const long long nf = nfaces(g, d);
    const double bytes = B8 * (6.0 * g.N + 13.0 * nf) + sizeof(TI) * 9.0 * nf;
    const int nd = d == 0 ? g.nx : (d == 1 ? g.ny : g.nz);
    if (scratch && nd >= 2) {  // gather form
        TI* G = reinterpret_cast<TI*>(scratch);
        const double cb = B8 * (6.0 * g.N + 2.0 * 12.0 * nf) + sizeof(TI) * (2.0 * 9.0 * nf + 8.0 * g.N);
        const double fb = B8 * 2.0 * 4.0 * nf + sizeof(TI) * 8.0 * g.N;
        if (mode == 0) {
            KS_LAUNCH(c, (k_adj_faces_cells<0, TI>), nblocks(g.N, BS), BS, cb, g, d, u, E, s, rho, nullptr, LO, HI, ti<TI>(B.ad[d]), LOb, HIb,
                      A.ad[d], TEb, A.u, G);
            KS_LAUNCH(c, (k_adj_faces_gather<0, TI>), nblocks(nf, BS), BS, fb, g, d, (const TI*)G, Eb, nullptr);
        } else {
            KS_LAUNCH(c, (k_adj_faces_cells<1, TI>), nblocks(g.N, BS), BS, cb, g, d, u, E, s, rho, umac_d, LO, HI, (const TI*)nullptr, LOb, HIb,
                      nullptr, TEb, A.u, G);
            KS_LAUNCH(c, (k_adj_faces_gather<1, TI>), nblocks(nf, BS), BS, fb, g, d, (const TI*)G, Eb, A.umac[d]);
        }
        return;
    }
    if (mode == 0)
        KS_LAUNCH(c, (k_adj_faces<0, TI>), nblocks(nf, BS), BS, bytes, g, d, u, E, s, rho, nullptr, LO, HI, ti<TI>(B.ad[d]), LOb, HIb, A.ad[d], TEb,
                  Eb, A.u, nullptr);
    else
        KS_LAUNCH(c, (k_adj_faces<1, TI>), nblocks(nf, BS), BS, bytes, g, d, u, E, s, rho, umac_d, LO, HI, (const TI*)nullptr, LOb, HIb, nullptr,
                  TEb, Eb, A.u, A.umac[d]);
}
void launch_adj_faces(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                      const double* umac_d, double* scratch, int fp32) {
    if (fp32) adj_faces_t<float>(c, g, d, mode, u, B, A, dt, rho, umac_d, scratch);
    else adj_faces_t<double>(c, g, d, mode, u, B, A, dt, rho, umac_d, scratch);
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
static void adj_adv_trans_t(Ctx& c, const Grid& g, int a, const double* u, double rho, double dt, const double* const mac[3],
                            const GodunovBufs& B, const AdjBufs& A, double* CB) {
    const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
    const double cb1 = dt / (3.0 * hd(g, b1)), cb2 = dt / (3.0 * hd(g, b2));
    K3 O1b{{A.tr[a][b1][0], A.tr[a][b1][1], A.tr[a][b1][2]}}, O2b{{A.tr[a][b2][0], A.tr[a][b2][1], A.tr[a][b2][2]}};
    A3 LOb{{A.lo[a][0], A.lo[a][1], A.lo[a][2]}}, HIb{{A.hi[a][0], A.hi[a][1], A.hi[a][2]}};
    const double na = (double)nfaces(g, a), N = (double)g.N;
    KS_LAUNCH(c, k_adj_trans_cells<TI>, nblocks(g.N, BS), BS, B8 * (2.0 * na + 4.0 * N + 12.0 * na + 12.0 * na + 6.0 * N + 6.0 * N), g, a, rho,
              cb1, cb2, mac[a], mac[b1], mac[b2], O1b, O2b, LOb, HIb, A.u, reinterpret_cast<TI*>(CB));
    for (int q = 0; q < 2; ++q) {
        const int b = q == 0 ? b1 : b2;
        const double nb = (double)nfaces(g, b);
        KI<TI> E{{ti<TI>(B.tedge[b][0]), ti<TI>(B.tedge[b][1]), ti<TI>(B.tedge[b][2])}};
        A3 Eb{{A.tedge[b][0], A.tedge[b][1], A.tedge[b][2]}};
        KS_LAUNCH(c, k_adj_bfaces<TI>, nblocks(nfaces(g, b), BS), BS, B8 * (12.0 * N + 2.0 * nb + 6.0 * nb) + sizeof(TI) * 3.0 * nb, g, b, u, rho,
                  q == 0 ? cb1 : cb2, mac[b], E, reinterpret_cast<const TI*>(CB) + 3LL * q * g.N, Eb, A.umac[b]);
    }
}
void launch_adj_adv_trans(Ctx& c, const Grid& g, int a, const double* u, double rho, double dt, const double* const mac[3],
                          const GodunovBufs& B, const AdjBufs& A, double* CB, int fp32) {
    if (fp32) adj_adv_trans_t<float>(c, g, a, u, rho, dt, mac, B, A, CB);
    else adj_adv_trans_t<double>(c, g, a, u, rho, dt, mac, B, A, CB);
}

template <typename TI>
static void adj_adv_flux_t(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                           const GodunovBufs& B, const AdjBufs& A, double* CB) {
    const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
    const double c1 = dt / (2.0 * hd(g, b1)), c2 = dt / (2.0 * hd(g, b2));
    K3 Uf{{mac[0], mac[1], mac[2]}};
    KI<TI> LO{{ti<TI>(B.lo[d][0]), ti<TI>(B.lo[d][1]), ti<TI>(B.lo[d][2])}}, HI{{ti<TI>(B.hi[d][0]), ti<TI>(B.hi[d][1]), ti<TI>(B.hi[d][2])}};
    KI<TI> T1{{ti<TI>(B.tr[b1][b2][0]), ti<TI>(B.tr[b1][b2][1]), ti<TI>(B.tr[b1][b2][2])}};
    KI<TI> T2{{ti<TI>(B.tr[b2][b1][0]), ti<TI>(B.tr[b2][b1][1]), ti<TI>(B.tr[b2][b1][2])}};
    K3 Fb{{A.flux[d][0], A.flux[d][1], A.flux[d][2]}};
    A3 LOb{{A.lo[d][0], A.lo[d][1], A.lo[d][2]}}, HIb{{A.hi[d][0], A.hi[d][1], A.hi[d][2]}};
    A3 T1b{{A.tr[b1][b2][0], A.tr[b1][b2][1], A.tr[b1][b2][2]}}, T2b{{A.tr[b2][b1][0], A.tr[b2][b1][1], A.tr[b2][b1][2]}};
    const double nf = (double)nfaces(g, d), nt = (double)(nfaces(g, b1) + nfaces(g, b2)), N = (double)g.N;
    KS_LAUNCH(c, k_adj_flux_faces<TI>, nblocks(nfaces(g, d), BS), BS, B8 * (6.0 * N + 5.0 * nf + 8.0 * nt + 7.0 * nf) + sizeof(TI) * (6.0 * nf + 6.0 * nt),
              g, d, u, forces, rho, dt, c1, c2, Uf, LO, HI, T1, T2, Fb, A.umac[d], LOb, HIb);
    KS_LAUNCH(c, k_adj_flux_cells<TI>, nblocks(g.N, BS), BS, B8 * (2.0 * nf + 6.0 * nf + nt + 12.0 * N) + sizeof(TI) * 3.0 * N, g, d, rho, dt, c1,
              c2, Uf, Fb, A.u, A.forces, reinterpret_cast<TI*>(CB));
    for (int q = 0; q < 2; ++q) {
        const int b = q == 0 ? b1 : b2;
        const double nb = (double)nfaces(g, b);
        KS_LAUNCH(c, k_adj_bfaces<TI>, nblocks(nfaces(g, b), BS), BS, B8 * (12.0 * N + 2.0 * nb + 6.0 * nb) + sizeof(TI) * 3.0 * nb, g, b, u, rho,
                  q == 0 ? c1 : c2, mac[b], q == 0 ? T1 : T2, reinterpret_cast<const TI*>(CB), q == 0 ? T1b : T2b, A.umac[b]);
    }
}
void launch_adj_adv_flux(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                         const GodunovBufs& B, const AdjBufs& A, double* CB, int fp32) {
    if (fp32) adj_adv_flux_t<float>(c, g, d, u, forces, rho, dt, mac, B, A, CB);
    else adj_adv_flux_t<double>(c, g, d, u, forces, rho, dt, mac, B, A, CB);
}
void launch_adj_div(Ctx& c, const Grid& g, const double* convb, const AdjBufs& A) {
    for (int d = 0; d < 3; ++d) {
        const long long nf = nfaces(g, d);
        KS_LAUNCH(c, k_adj_div, nblocks(nf, BS), BS, B8 * (3.0 * g.N + 3.0 * nf), g, d, convb, A.flux[d][0], A.flux[d][1], A.flux[d][2]);
    }
}
void launch_adj_tau(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, const double* divtau_b, double s, double* ub,
                    double* mub, double* wgb, int fp32) {
    const dim3 grid((g.nx + ATX - 1) / ATX, (g.ny + ATY - 1) / ATY, (g.nz + ATZ - 1) / ATZ);
    if (fp32) {
        cudaFuncSetAttribute(k_adj_tau_tile<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_tau_smem<float>());
        KS_LAUNCH_SMEM(c, k_adj_tau_tile<float>, grid, ATX * ATY * ATZ, adj_tau_smem<float>(), B8 * 14.0 * g.N, g, vel, mueff, wg, divtau_b, s,
                       ub, mub, wgb);
    } else {
        cudaFuncSetAttribute(k_adj_tau_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_tau_smem<double>());
        KS_LAUNCH_SMEM(c, k_adj_tau_tile<double>, grid, ATX * ATY * ATZ, adj_tau_smem<double>(), B8 * 14.0 * g.N, g, vel, mueff, wg, divtau_b, s,
                       ub, mub, wgb);
    }
}
template <typename A>
static void adj_smag_t(Ctx& c, const Grid& g, const double* vel, const double* mub, const Scalars& s, double* ub, double* scratch) {
    if (!scratch || (!g.zper && g.nz < 4)) {
        KS_LAUNCH(c, k_adj_smag<A>, nblocks(g.N, BS), BS, B8 * 7.0 * g.N, g, vel, mub, s.rho, s.smag_fac, ub);
        return;
    }
    A* W = reinterpret_cast<A*>(scratch);
    KS_LAUNCH(c, k_adj_smag_w<A>, nblocks(g.N, BS), BS, B8 * 4.0 * g.N + sizeof(A) * 9.0 * g.N, g, vel, mub, s.rho, s.smag_fac, W);
    KS_LAUNCH(c, k_adj_smag_gather<A>, nblocks(g.N, BS), BS, B8 * 6.0 * g.N + sizeof(A) * 9.0 * g.N, g, (const A*)W, ub);
}
void launch_adj_smag(Ctx& c, const Grid& g, const double* vel, const double* mub, const Scalars& s, double* ub, double* scratch, int fp32) {
    if (fp32) adj_smag_t<float>(c, g, vel, mub, s, ub, scratch);
    else adj_smag_t<double>(c, g, vel, mub, s, ub, scratch);
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
