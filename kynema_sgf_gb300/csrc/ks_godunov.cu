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
// FP64 issue is the scarce resource on GB300 (every FP64 instruction,
// compares and min/max included, issues at 1/64 of the FP32 rate), so nothing
// is computed twice and no FP64 instruction makes a decision: every cell's
// slope, unlimited edge and limited parabola is formed once per component and
// pass (k_ppm_x / k_ppm_col), the face states are stored, and the transverse
// and final stages only read them; signs, comparisons, minima and maxima are
// taken on the integer pipe (ks_common.cuh).  Post-MAC states of rho*u are rho
// times the traces of u (the PPM limiter and the traces are homogeneous of
// degree one in the advected field).
#include "ks_decide.cuh"
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

inline long long nfaces(const Grid& g, int d) { return (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz); }

// van Leer limited slope of the middle cell of (a, b, c):
// copysign(min(|dsc|, |dsl|, |dsr|), dsc) where dsl dsr > 0, else 0
template <typename T>
__device__ inline T vls(T a, T b, T c) {
    const T dsc = T(0.5) * (c - a), dsl = T(2) * (b - a), dsr = T(2) * (c - b);
    if (!same_sign(dsl, dsr)) return T(0);
    T m = abs_lt(dsl, dsr) ? dsl : dsr;
    m = abs_lt(dsc, m) ? dsc : m;
    return mag_sign(m, dsc);
}

// unlimited PPM edge value between cells with values a0, a1 and slopes s0, s1,
// clipped to the two cells
template <typename T>
__device__ inline T ppm_edge(T a0, T a1, T s0, T s1) {
    return clip2(T(0.5) * (a0 + a1) - T(1.0 / 6.0) * (s1 - s0), a0, a1);
}

// Edge value on the face with index k along d from the cell values
// a(k-2), a(k-1), a(k), a(k+1) and the slopes s(k-1), s(k).  Wall-bounded z:
// the wall faces take the boundary (ghost) value, the faces one cell inside
// the one-sided fourth-order formula clipped to the two adjacent cells.
template <typename T>
__device__ inline T edge_at(bool walls, int k, int nz, T am2, T am1, T a0, T ap1, T sm1, T s0) {
    if (walls) {
        if (k == 0) return am1;
        if (k == nz) return a0;
        if (k == 1) return clip2(T(-0.2) * am2 + T(0.75) * am1 + T(0.5) * a0 - T(0.05) * ap1, am1, a0);
        if (k == nz - 1) return clip2(T(-0.2) * ap1 + T(0.75) * a0 + T(0.5) * am1 - T(0.05) * am2, a0, am1);
    }
    return ppm_edge(am1, a0, sm1, s0);
}

// limited parabola of a cell (Colella-Woodward 1984): (sm, sp) from its two
// edges and the cell value s0.  3 s0 - 2 sm = s0 + 2 (s0 - sm), and
// 3 s0 - 2 sp = s0 - 2 (sp - s0).
template <typename T>
__device__ inline void cw84(T s0, T& sm, T& sp) {
    const T dp = sp - s0, dm = s0 - sm;
    if (!same_sign(dp, dm)) {
        sp = s0;
        sm = s0;
        return;
    }
    const T dp2 = T(2) * dp, dm2 = T(2) * dm;
    if (!abs_lt(dp, dm2)) sp = s0 + dm2;
    else if (!abs_lt(dm, dp2)) sm = s0 - dp2;
}

// Average of the limited parabola (sm, s0, sp) over the part of the cell that
// crosses its high face (hi = true) or low face in dt, sig = |u| dt / h:
//   high: sp - h D + h g s6,   low: sm + h D + h g s6,
// h = sig / 2, g = 1 - 2 sig / 3, D = sp - sm, s6 = 6 s0 - 3 (sm + sp).
template <typename T>
struct TraceCoef {
    T h, hg;
    __device__ inline TraceCoef(T sig) {
        h = T(0.5) * sig;
        hg = h * (T(1) - T(2.0 / 3.0) * sig);
    }
};
template <typename T>
__device__ inline T ppm_trace(bool hi, T sm, T s0, T sp, const TraceCoef<T>& c) {
    const T D = sp - sm, s6 = T(6) * s0 - T(3) * (sm + sp);
    return c.hg * s6 + (neg_if(hi, c.h) * D + (hi ? sp : sm));
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

// upwind state with AMReX-Hydro's small_vel: the mean of both states where
// |vel| < small_vel
template <typename T>
__device__ inline T upwind(T vel, T lo, T hi) {
    if (below_small_abs(vel)) return T(0.5) * (lo + hi);
    return ge0(vel) ? lo : hi;
}
template <typename T>
__device__ inline T riemann(T lo, T hi) {
    const T sum = lo + hi;
    const bool ltm = (le0(lo) && ge0(hi)) || below_small_abs(sum);
    return ltm ? T(0) : (ge0(sum) ? lo : hi);
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
// MODE 0 (pre-MAC): the characteristic speed of a cell is its velocity
// component d, so one trace per cell (its downwind face; the other face
// takes the cell value).  Computes the unlimited edges from the slopes and
// stores them (reused by the post-MAC pass), writes the left/right states, the
// Riemann-solved advective velocity and the two transverse components
// upwinded with it.
// MODE 1 (post-MAC): the speed is the MAC velocity of the face, so one trace
// per face (from its upwind cell); states are scaled by rho and all NC
// components are upwinded with the MAC velocity.  EDGES = 0 reads the stored
// unlimited edges, EDGES = 1 computes them (a scalar's only pass).
//
// Every cell's slope, edge and limited parabola is computed once per
// component: the y and z kernels march along a column of faces and carry
// them, the x kernel passes them between neighbouring lanes of a warp.
template <typename T>
struct PpmArgs {
    Grid g;
    int d;
    const T* vel;   // advected field(s), NC components of N
    const T* umac;  // MAC velocity on d-faces (MODE 1)
};

template <typename T, int NC>
struct PpmOut {
    T* E[3];   // unlimited edges (MODE 0 writes them for the adjoint)
    T* PM[3];  // limited parabola (sm, sp) of every cell (MODE 0 writes, MODE 1 EDGES = 0 reads)
    T* PP[3];
    T* LO[3];  // left / right states
    T* HI[3];
    T* TE[3];  // upwinded states
    T* ad;     // advective velocity (MODE 0)
};

// the face states of one component on the face between cells with the
// limited parabolas (pm, p0, pp) (low cell) and (qm, q0, qp) (high cell)
// for the MAC velocity u (MODE 1)
template <typename T>
__device__ inline void face_states_mac(T u, T s, T pm, T p0, T pp, T qm, T q0, T qp, T& l, T& h) {
    l = p0;
    h = q0;
    const bool up = above_small(u), dn = below_msmall(u);
    if (up || dn) {
        const TraceCoef<T> c(absv(u) * s);
        const T t = ppm_trace(up, up ? pm : qm, up ? p0 : q0, up ? pp : qp, c);
        if (up) l = t;
        else h = t;
    }
}

// a[n] for a run-time n without addressing the register array
template <typename T, int NC>
__device__ inline T sel(const T (&a)[NC], int n) {
    T r = a[0];
#pragma unroll
    for (int m = 1; m < NC; ++m)
        if (n == m) r = a[m];
    return r;
}

// y (d = 1) and z (d = 2) faces: one thread per (i, transverse index, chunk of
// faces along d).  Face m lies between cells m-1 and m.
template <typename T, int NC, int MODE, int EDGES>
__global__ void __launch_bounds__(256) k_ppm_col(PpmArgs<T> A, T s, T rho, PpmOut<T, NC> O, int chunk) {
    const Grid& g = A.g;
    const int d = A.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nx) return;
    const bool walls = (d == 2 && !g.zper);
    const int nl = d == 1 ? g.ny : g.nz;  // cells along d
    const int nf = walls ? g.nz + 1 : nl;  // faces along d
    const int no = d == 1 ? g.nz : g.ny;
    const int o = blockIdx.y % no, ch = blockIdx.y / no;
    const int m0 = ch * chunk, m1 = min(m0 + chunk, nf);
    if (m0 >= m1) return;
    VelFPT<T, T> q{A.vel, g, T(1)};
    auto val = [&](int n, int m) -> T {
        if (!walls) m = ((m % nl) + nl) % nl;
        return d == 1 ? q(n, i, m, o) : q(n, i, o, m);
    };
    auto fid = [&](int m) -> long long { return d == 1 ? fidx(g, 1, i, m, o) : fidx(g, 2, i, o, m); };
    auto cellid = [&](int m) -> long long { return d == 1 ? cidx(g, i, m, o) : cidx(g, i, o, m); };  // 0 <= m < nl
    // per component at face m: a(m-1), a(m), a(m+1), the slope s(m), the edge
    // e(m), and cell m-1's high-face trace (MODE 0) or limited parabola (MODE 1)
    T am1[NC], a0[NC], ap1[NC], sl0[NC], e0[NC], lo0[NC], pm[NC], pp[NC];
    {
        T u = T(0);
        if (MODE == 0) u = val(d, m0 - 1);
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            T em1;
            am1[n] = val(n, m0 - 1);
            a0[n] = val(n, m0);
            if (MODE == 1 && !EDGES) {
                // the stored limited parabola of cell m0 - 1 (none below a wall)
                if (walls && m0 == 0) {
                    pm[n] = am1[n];
                    pp[n] = am1[n];
                } else {
                    const long long cm = cellid(((m0 - 1) % nl + nl) % nl);
                    pm[n] = O.PM[n][cm];
                    pp[n] = O.PP[n][cm];
                }
                continue;
            } else {
                const T x3 = val(n, m0 - 3), x2 = val(n, m0 - 2);
                ap1[n] = val(n, m0 + 1);
                const T s2 = vls(x3, x2, am1[n]), s1 = vls(x2, am1[n], a0[n]);
                sl0[n] = vls(am1[n], a0[n], ap1[n]);
                em1 = edge_at(walls, m0 - 1, g.nz, x3, x2, am1[n], a0[n], s2, s1);
                e0[n] = edge_at(walls, m0, g.nz, x2, am1[n], a0[n], ap1[n], s1, sl0[n]);
            }
            T sm = em1, sp = e0[n];
            cw84(am1[n], sm, sp);
            pm[n] = sm;
            pp[n] = sp;
            lo0[n] = am1[n];
            if (MODE == 0 && above_small(u)) lo0[n] = ppm_trace(true, sm, am1[n], sp, TraceCoef<T>(absv(u) * s));
        }
    }
    for (int m = m0; m < m1; ++m) {
        const long long f = fid(m);
        T e1[NC], ap2[NC], s1[NC];
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            if (MODE == 1 && !EDGES) {
                ap1[n] = val(n, m + 1);
            } else {
                ap2[n] = val(n, m + 2);
                s1[n] = vls(a0[n], ap1[n], ap2[n]);
                e1[n] = edge_at(walls, m + 1, g.nz, am1[n], a0[n], ap1[n], ap2[n], sl0[n], s1[n]);
            }
        }
        T lo[NC], hi[NC];
        if (MODE == 0) {
            const T u = sel(a0, d);  // cell m's velocity component d
            const bool up = above_small(u), dn = below_msmall(u);
            const TraceCoef<T> c(absv(u) * s);
#pragma unroll
            for (int n = 0; n < NC; ++n) {
                T sm = e0[n], sp = e1[n];
                cw84(a0[n], sm, sp);
                if (m < nl) {  // the post-MAC pass reads the limited parabola of every cell
                    O.PM[n][cellid(m)] = sm;
                    O.PP[n][cellid(m)] = sp;
                }
                T h = a0[n], lnext = a0[n];
                if (up || dn) {
                    const T t = ppm_trace(up, sm, a0[n], sp, c);
                    if (up) lnext = t;
                    else h = t;
                }
                lo[n] = lo0[n];
                hi[n] = h;
                lo0[n] = lnext;
            }
        } else {
            const T u = (T)A.umac[f];
#pragma unroll
            for (int n = 0; n < NC; ++n) {
                T sm, sp;
                if (MODE == 1 && !EDGES) {
                    if (m < nl) {
                        sm = O.PM[n][cellid(m)];
                        sp = O.PP[n][cellid(m)];
                    } else {  // the ghost cell above a wall: its state is replaced below
                        sm = a0[n];
                        sp = a0[n];
                    }
                } else {
                    sm = e0[n];
                    sp = e1[n];
                    cw84(a0[n], sm, sp);
                }
                T l, h;
                face_states_mac(u, s, pm[n], am1[n], pp[n], sm, a0[n], sp, l, h);
                lo[n] = rho * l;
                hi[n] = rho * h;
                pm[n] = sm;
                pp[n] = sp;
            }
        }
        if (walls) {
#pragma unroll
            for (int n = 0; n < NC; ++n) {
                if (m == 0) lo[n] = T(0);
                if (m == g.nz) hi[n] = T(0);
                zbc(g, m, n, lo[n], hi[n]);
            }
        }
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            O.LO[n][f] = lo[n];
            O.HI[n][f] = hi[n];
            if (MODE == 0) O.E[n][f] = e0[n];
        }
        if (MODE == 0) {
            const T a = riemann(sel(lo, d), sel(hi, d));
            O.ad[f] = a;
#pragma unroll
            for (int n = 0; n < NC; ++n)
                if (n != d) O.TE[n][f] = upwind(a, lo[n], hi[n]);
        } else {
            const T u = (T)A.umac[f];
#pragma unroll
            for (int n = 0; n < NC; ++n) O.TE[n][f] = upwind(u, lo[n], hi[n]);
        }
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            am1[n] = a0[n];
            a0[n] = ap1[n];
            if (!(MODE == 1 && !EDGES)) {
                e0[n] = e1[n];
                ap1[n] = ap2[n];
                sl0[n] = s1[n];
            }
        }
    }
}

// x faces: each warp covers XF consecutive faces of one x row; lane l holds
// cell c = XF seg + l - H.  Computed edges (H = 2, XF = 29): every lane forms
// its cell's slope, lanes >= 1 the edge of face c with the slope of lane l-1,
// lanes 1..30 their cell's parabola with the edge of lane l+1, lanes 2..30 the
// states of face c.  Stored edges (H = 1, XF = 31): every lane reads both
// edges of its cell and forms its parabola; lanes 1..31 form face c.  Every
// lane does the same work, so no lane's extra cell stalls the others.
template <typename T, int NC, int MODE, int EDGES>
__global__ void __launch_bounds__(256) k_ppm_x(PpmArgs<T> A, T s, T rho, PpmOut<T, NC> O) {
    constexpr bool LOADE = (MODE == 1 && !EDGES);
    constexpr int H = LOADE ? 1 : 2, XF = LOADE ? 31 : 29;
    const Grid& g = A.g;
    const int nseg = (g.nx + XF - 1) / XF;
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long rows = (long long)g.ny * g.nz;
    if (w >= rows * nseg) return;  // whole warps leave together
    const int row = (int)(w / nseg), seg = (int)(w % nseg);
    const int c = seg * XF + lane - H;
    const bool own = lane >= H && lane <= (LOADE ? 31 : 30) && c < g.nx;
    auto wx = [&](int x) { return ((x % g.nx) + g.nx) % g.nx; };
    const long long rb = (long long)row * g.nx;  // row base: cells and x faces share the index
    const long long fc = rb + wx(c);
    auto ld = [&](int n, int x) -> T { return (T)A.vel[n * g.N + rb + wx(x)]; };
    const unsigned FULL = 0xffffffffu;
    T lo[NC], hi[NC], ev[NC];
    T u = T(0);
    if (MODE == 0) u = ld(0, c);
    else u = (T)A.umac[fc];
    const bool up = above_small(u), dn = below_msmall(u);
    const TraceCoef<T> tc(absv(u) * s);
    T pmv[NC], ppv[NC];
    for (int n = 0; n < NC; ++n) {
        const T a0 = ld(n, c);
        T am1, sm, sp;
        if (LOADE) {  // the limited parabola of the lane's cell, stored by the pre-MAC pass
            sm = O.PM[n][fc];
            sp = O.PP[n][fc];
            am1 = __shfl_up_sync(FULL, a0, 1);
            ev[n] = T(0);
        } else {
            am1 = ld(n, c - 1);
            const T ap1 = ld(n, c + 1);
            const T sl = vls(am1, a0, ap1);
            const T slm = __shfl_up_sync(FULL, sl, 1);
            const T e0 = ppm_edge(am1, a0, slm, sl);
            const T e1 = __shfl_down_sync(FULL, e0, 1);
            ev[n] = e0;
            sm = e0;
            sp = e1;
            cw84(a0, sm, sp);
        }
        pmv[n] = sm;
        ppv[n] = sp;
        if (MODE == 0) {
            T h = a0, lnext = a0;
            if (up || dn) {
                const T t = ppm_trace(up, sm, a0, sp, tc);
                if (up) lnext = t;
                else h = t;
            }
            lo[n] = __shfl_up_sync(FULL, lnext, 1);
            hi[n] = h;
        } else {
            const T pm = __shfl_up_sync(FULL, sm, 1), pp = __shfl_up_sync(FULL, sp, 1);
            T l, h;
            face_states_mac(u, s, pm, am1, pp, sm, a0, sp, l, h);
            lo[n] = rho * l;
            hi[n] = rho * h;
        }
    }
    if (!own) return;
#pragma unroll
    for (int n = 0; n < NC; ++n) {
        O.LO[n][fc] = lo[n];
        O.HI[n][fc] = hi[n];
        if (MODE == 0) {  // x faces and cells share the index: face c is owned with cell c
            O.E[n][fc] = ev[n];
            O.PM[n][fc] = pmv[n];
            O.PP[n][fc] = ppv[n];
        }
    }
    if (MODE == 0) {
        const T a = riemann(lo[0], hi[0]);
        O.ad[fc] = a;
#pragma unroll
        for (int n = 1; n < NC; ++n) O.TE[n][fc] = upwind(a, lo[n], hi[n]);
    } else {
#pragma unroll
        for (int n = 0; n < NC; ++n) O.TE[n][fc] = upwind(u, lo[n], hi[n]);
    }
}

// ---- stages 2 and 3 of both passes by cells.  In each stage a face state is
// its stage-1 (or stage-2) value plus a correction that depends only on the
// cell it is traced from (its value, forces, and the advective / MAC
// velocities and states on its own transverse faces).  The low-side state of
// face c + e_d and the high-side state of face c share it, so the kernels
// below form each cell's corrections once: x faces take the low cell's from
// the previous lane of the warp (lane 0 and the periodic wrap form their
// own); y and z faces march a chunk of 16 faces along d and carry it.
//
// An op supplies T, K (values per cell), the grid g and face direction d,
//   cell(i, j, k, c[K]): the cell's corrections,
//   face(f, kf, wl, wh, cl[K], ch[K]): the face's output from the low and
//     high cells' corrections (kf the face's z index, wl / wh a wall face
//     without a cell below / above).
template <typename Op>
__global__ void __launch_bounds__(256, sizeof(typename Op::T) == 4 ? 3 : 2) k_cf_x(Op op) {
    using T = typename Op::T;
    constexpr int K = Op::K;
    const Grid& g = op.g;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t < g.N;
    int i = 0, j = 0, k = 0;
    T ch[K], cl[K];
    for (int n = 0; n < K; ++n) ch[n] = T(0);
    if (live) {
        const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
        i = (int)(u - r * (unsigned)g.nx);
        k = (int)(r / (unsigned)g.ny);
        j = (int)(r - (unsigned)k * (unsigned)g.ny);
        op.cell(i, j, k, ch);
    }
    for (int n = 0; n < K; ++n) cl[n] = __shfl_up_sync(0xffffffffu, ch[n], 1);
    if (!live) return;
    if ((threadIdx.x & 31) == 0 || i == 0) op.cell(i == 0 ? g.nx - 1 : i - 1, j, k, cl);
    op.face(t, k, false, false, cl, ch);
}

template <typename Op>
__global__ void __launch_bounds__(128) k_cf_col(Op op, int chunk) {
    using T = typename Op::T;
    constexpr int K = Op::K;
    const Grid& g = op.g;
    const int d = op.d;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.nx) return;
    const int nf = d == 1 ? g.ny : nzfaces(g);
    const int no = d == 1 ? g.nz : g.ny;
    const int o = (int)(blockIdx.y % (unsigned)no), chn = (int)(blockIdx.y / (unsigned)no);
    const int m0 = chn * chunk, m1 = min(m0 + chunk, nf);
    if (m0 >= m1) return;
    const bool walls = d == 2 && !g.zper;
    const int ncell = d == 1 ? g.ny : g.nz;
    auto cellc = [&](int m, T c[K]) {  // cell m along d (periodic wrap)
        m = m < 0 ? m + ncell : (m >= ncell ? m - ncell : m);
        if (d == 1) op.cell(i, m, o, c);
        else op.cell(i, o, m, c);
    };
    T cl[K], ch[K];
    for (int n = 0; n < K; ++n) cl[n] = ch[n] = T(0);
    if (!(walls && m0 == 0)) cellc(m0 - 1, cl);
    for (int m = m0; m < m1; ++m) {
        const bool wl = walls && m == 0, wh = walls && m == g.nz;
        if (!wh) cellc(m, ch);
        const long long f = d == 1 ? fidx(g, 1, i, m, o) : fidx(g, 2, i, o, m);
        op.face(f, m, wl, wh, cl, ch);
        for (int n = 0; n < K; ++n) cl[n] = ch[n];
    }
}

template <typename Op>
static void launch_cf(Ctx& c, const char* name_x, const char* name_col, const Op& op, double bytes) {
    const Grid& g = op.g;
    if (op.d == 0) {
        KS_LAUNCH_NAMED(c, name_x, k_cf_x<Op>, nblocks(g.N, 256), 256, bytes, op);
    } else {
        constexpr int chunk = 16;
        const int nf = op.d == 1 ? g.ny : nzfaces(g), no = op.d == 1 ? g.nz : g.ny;
        const int bx = g.nx >= 128 ? 128 : 32 * ((g.nx + 31) / 32);
        const dim3 grid((unsigned)((g.nx + bx - 1) / bx), (unsigned)(no * ((nf + chunk - 1) / chunk)));
        KS_LAUNCH_NAMED(c, name_col, k_cf_col<Op>, grid, bx, bytes, op, chunk);
    }
}

// pre-MAC stage 2: the a-face states of component n corrected along b,
// corr(c) = cb (ad_b+ + ad_b-) (E_b+ - E_b-) over the b faces of c (velocity
// form, dt/6 corner factor); out = upwind(ad_a; lo - corr(c - e_a), hi - corr(c))
template <typename T_>
struct PmTransOp {
    using T = T_;
    static constexpr int K = 1;
    Grid g;
    int d, b, n;
    T cb;
    const T *lo, *hi, *ad_a, *ad_b, *edge_b;
    T* out;
    __device__ inline void cell(int i, int j, int k, T c[1]) const {
        const long long f0 = fidx(g, b, i, j, k), f1 = fidx(g, b, i + (b == 0), j + (b == 1), k + (b == 2));
        c[0] = cb * (ad_b[f1] + ad_b[f0]) * (edge_b[f1] - edge_b[f0]);
    }
    __device__ inline void face(long long f, int kf, bool wl, bool wh, const T cl[1], const T ch[1]) const {
        T l = lo[f], h = hi[f];
        if (!wl) l -= cl[0];
        if (!wh) h -= ch[0];
        if (d == 2) zbc(g, kf, n, l, h);
        out[f] = upwind(ad_a[f], l, h);
    }
};

// pre-MAC stage 3: the normal velocity on d-faces,
// corr(c) = 0.5 dt F_d(c) - c1 (ad_b1+ + ad_b1-) (T1+ - T1-) - c2 (...)
// over the b1 / b2 faces of c (T_b the stage-2 states of component d on the
// b faces corrected along the other direction); mac = riemann(lo + corr(c -
// e_d), hi + corr(c))
template <typename T_>
struct PmFinalOp {
    using T = T_;
    static constexpr int K = 1;
    Grid g;
    int d, b1, b2;
    T hdt, c1, c2;
    const T *lo, *hi, *forces;
    C3<T> AD;
    const T *T1, *T2;
    double* mac;
    __device__ inline void cell(int i, int j, int k, T c[1]) const {
        const long long p1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), m1 = fidx(g, b1, i, j, k);
        const long long p2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), m2 = fidx(g, b2, i, j, k);
        const CellFOT<T, T> F{forces, g};
        T s = hdt * F(d, i, j, k);
        s -= c1 * (AD.p[b1][p1] + AD.p[b1][m1]) * (T1[p1] - T1[m1]);
        s -= c2 * (AD.p[b2][p2] + AD.p[b2][m2]) * (T2[p2] - T2[m2]);
        c[0] = s;
    }
    __device__ inline void face(long long f, int kf, bool wl, bool wh, const T cl[1], const T ch[1]) const {
        T stl = wl ? T(0) : lo[f] + cl[0], sth = wh ? T(0) : hi[f] + ch[0];
        if (d == 2) zbc(g, kf, d, stl, sth);
        mac[f] = (double)riemann(stl, sth);
    }
};

// post-MAC stage 2: the a-face states corrected along both transverse
// directions b1 = a+1 and b2 = a+2 (conservative form, dt/3 corner factors),
//   corr_b(c) = q(c) rho cb (v_b+ - v_b-) - cb (v_b+ E_b(+) - v_b- E_b(-))
// over the b faces of c; c[0..NC) the corrections along b1, c[NC..2NC) along b2
template <typename T_, int NC>
struct AdvTransOp {
    using T = T_;
    static constexpr int K = 2 * NC;
    Grid g;
    int d, b1, b2;
    const T* vel;
    T rho, cb1, cb2;
    const T *ua, *vb1, *vb2;
    C3<T> LO, HI, E1, E2;
    P3<T> O1, O2;
    __device__ inline void cell(int i, int j, int k, T c[K]) const {
        const long long p1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), m1 = fidx(g, b1, i, j, k);
        const long long p2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), m2 = fidx(g, b2, i, j, k);
        const T v1p = (T)vb1[p1], v1m = (T)vb1[m1], v2p = (T)vb2[p2], v2m = (T)vb2[m2];
        const T r1 = rho * cb1 * (v1p - v1m), r2 = rho * cb2 * (v2p - v2m);
        const VelFPT<T, T> q{vel, g, T(1)};
        for (int n = 0; n < NC; ++n) {
            const T qc = q(n, i, j, k);
            c[n] = qc * r1 - cb1 * (v1p * E1.p[n][p1] - v1m * E1.p[n][m1]);
            c[NC + n] = qc * r2 - cb2 * (v2p * E2.p[n][p2] - v2m * E2.p[n][m2]);
        }
    }
    __device__ inline void face(long long f, int kf, bool wl, bool wh, const T cl[K], const T ch[K]) const {
        const T u = (T)ua[f];
        const bool usmall = below_small_abs(u), upos = ge0(u);
        auto pick = [&](T l, T h) { return usmall ? T(0.5) * (l + h) : (upos ? l : h); };
        for (int n = 0; n < NC; ++n) {
            const T l0 = LO.p[n][f], h0 = HI.p[n][f];
            T l = wl ? l0 : l0 + cl[n], h = wh ? h0 : h0 + ch[n];
            if (d == 2) zbc(g, kf, n, l, h);
            O1.p[n][f] = pick(l, h);
            l = wl ? l0 : l0 + cl[NC + n];
            h = wh ? h0 : h0 + ch[NC + n];
            if (d == 2) zbc(g, kf, n, l, h);
            O2.p[n][f] = pick(l, h);
        }
    }
};

// post-MAC stage 3: final states and fluxes on d-faces.  The forces enter
// scaled by rho for the velocity (forces = (src + divtau) / rho) and as they
// are for a scalar (NC = 1: forces = src + diff, AdvOp_Godunov.H:114-329):
//   corr(c) = hdt forces(c) + (q(c) r(c) - c1 x1(c) - c2 x2(c)),
//   r = rho (c1 (v1+ - v1-) + c2 (v2+ - v2-)),  x_b = T_b(+) v_b+ - T_b(-) v_b-
template <typename T_, int NC>
struct AdvFluxOp {
    using T = T_;
    static constexpr int K = NC;
    Grid g;
    int d, b1, b2;
    const T *vel, *forces;
    T rho, hdt, c1, c2;
    C3<T> U, T1, T2, LO, HI;
    P3<T> Fl;
    __device__ inline void cell(int i, int j, int k, T c[K]) const {
        const long long p1 = fidx(g, b1, i + (b1 == 0), j + (b1 == 1), k + (b1 == 2)), m1 = fidx(g, b1, i, j, k);
        const long long p2 = fidx(g, b2, i + (b2 == 0), j + (b2 == 1), k + (b2 == 2)), m2 = fidx(g, b2, i, j, k);
        const T v1p = (T)U.p[b1][p1], v1m = (T)U.p[b1][m1], v2p = (T)U.p[b2][p2], v2m = (T)U.p[b2][m2];
        const T r = rho * (c1 * (v1p - v1m) + c2 * (v2p - v2m));
        const VelFPT<T, T> q{vel, g, T(1)};
        const CellFOT<T, T> Fo{forces, g};
        for (int n = 0; n < NC; ++n) {
            const T x1 = T1.p[n][p1] * v1p - T1.p[n][m1] * v1m, x2 = T2.p[n][p2] * v2p - T2.p[n][m2] * v2m;
            c[n] = hdt * Fo(n, i, j, k) + ((q(n, i, j, k) * r - c1 * x1) - c2 * x2);
        }
    }
    __device__ inline void face(long long f, int kf, bool wl, bool wh, const T cl[K], const T ch[K]) const {
        const T um = (T)U.p[d][f];
        const bool usmall = below_small_abs(um), upos = ge0(um);
        for (int n = 0; n < NC; ++n) {
            T stl = wl ? T(0) : LO.p[n][f] + cl[n];
            T sth = wh ? T(0) : HI.p[n][f] + ch[n];
            if (d == 2) zbc(g, kf, n, stl, sth);
            const T st = usmall ? T(0.5) * (stl + sth) : (upos ? stl : sth);
            Fl.p[n][f] = um * st;
        }
    }
};

template <typename T>
struct FluxPtrs {
    const T* p[9];
};
template <typename T, int NC = 3>
__global__ void k_adv_div(Grid g, FluxPtrs<T> F, double* conv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
    const int i = (int)(u - r * (unsigned)g.nx);
    const int k = (int)(r / (unsigned)g.ny), j = (int)(r - (unsigned)k * (unsigned)g.ny);
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

// stage 1 on the d-faces: the x kernel for d = 0, the column march otherwise
constexpr int PPM_CHUNK = 32;
template <typename T, int NC, int MODE, int EDGES>
static void launch_ppm(Ctx& c, const Grid& g, int d, const T* vel, const T* umac, double dt, double rho, const PpmOut<T, NC>& O,
                       double bytes) {
    const PpmArgs<T> A{g, d, vel, umac};
    const T s = T(dt / hd(g, d));
    if (d == 0) {
        constexpr int XF = (MODE == 1 && !EDGES) ? 31 : 29;
        const long long warps = (long long)g.ny * g.nz * ((g.nx + XF - 1) / XF);
        KS_LAUNCH(c, (k_ppm_x<T, NC, MODE, EDGES>), nblocks(warps * 32, BS), BS, bytes, A, s, T(rho), O);
    } else {
        const int nf = (d == 2) ? nzfaces(g) : g.ny;
        const int nch = (nf + PPM_CHUNK - 1) / PPM_CHUNK, chunk = (nf + nch - 1) / nch;
        const int bx = g.nx >= BS ? BS : 32 * ((g.nx + 31) / 32);
        const dim3 grid((unsigned)((g.nx + bx - 1) / bx), (unsigned)((d == 1 ? g.nz : g.ny) * nch));
        KS_LAUNCH(c, (k_ppm_col<T, NC, MODE, EDGES>), grid, bx, bytes, A, s, T(rho), O, chunk);
    }
}

template <typename T>
static void premac_t(Ctx& c, const Grid& g, const T* vel, const T* forces, double dt, GodunovBufs& B, double* mac[3]) {
    const double BT = (double)sizeof(T), B8 = 8.0;
    for (int d = 0; d < 3; ++d) {
        PpmOut<T, 3> O{};
        for (int n = 0; n < 3; ++n) {
            O.E[n] = tp<T>(B.edge[d][n]);
            O.PM[n] = tp<T>(B.pm[d][n]);
            O.PP[n] = tp<T>(B.pp[d][n]);
            O.LO[n] = tp<T>(B.lo[d][n]);
            O.HI[n] = tp<T>(B.hi[d][n]);
            O.TE[n] = tp<T>(B.tedge[d][n]);
        }
        O.ad = tp<T>(B.ad[d]);
        launch_ppm<T, 3, 0, 1>(c, g, d, vel, (const T*)nullptr, dt, 1.0, O, BT * 3.0 * g.N + BT * 12.0 * nfaces(g, d));
    }
    // (a, b, n): states on a-faces of component n corrected along b
    const int tpl[6][3] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    for (auto& p : tpl) {
        const int a = p[0], b = p[1], n = p[2];
        const double bytes = BT * (4.0 * nfaces(g, a) + 2.0 * nfaces(g, b));
        const PmTransOp<T> op{g, a, b, n, T(dt / (6.0 * hd(g, b))), tp<T>(B.lo[a][n]), tp<T>(B.hi[a][n]), tp<T>(B.ad[a]), tp<T>(B.ad[b]),
                              tp<T>(B.tedge[b][n]), tp<T>(B.tr[a][b][0])};
        launch_cf(c, "k_pm_trans_x", "k_pm_trans_col", op, bytes);
    }
    C3<T> AD{{tp<T>(B.ad[0]), tp<T>(B.ad[1]), tp<T>(B.ad[2])}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = BT * (1.0 * g.N + 3.0 * nfaces(g, d) + 2.0 * nfaces(g, b1) + 2.0 * nfaces(g, b2)) + B8 * nfaces(g, d);
        const PmFinalOp<T> op{g, d, b1, b2, T(0.5) * T(dt), T(dt / (4.0 * hd(g, b1))), T(dt / (4.0 * hd(g, b2))), tp<T>(B.lo[d][d]),
                              tp<T>(B.hi[d][d]), forces, AD, tp<T>(B.tr[b1][b2][0]), tp<T>(B.tr[b2][b1][0]), mac[d]};
        launch_cf(c, "k_pm_final_x", "k_pm_final_col", op, bytes);
    }
}

template <typename T>
static void advection_t(Ctx& c, const Grid& g, const T* vel, const T* forces, const T* const mac[3], double dt, double rho,
                        GodunovBufs& B, double* conv) {
    const double BT = (double)sizeof(T), B8 = 8.0;
    // the limited parabolas of the pre-MAC pass are reused (same field)
    for (int a = 0; a < 3; ++a) {
        PpmOut<T, 3> O{};
        for (int n = 0; n < 3; ++n) {
            O.E[n] = tp<T>(B.edge[a][n]);
            O.PM[n] = tp<T>(B.pm[a][n]);
            O.PP[n] = tp<T>(B.pp[a][n]);
            O.LO[n] = tp<T>(B.lo[a][n]);
            O.HI[n] = tp<T>(B.hi[a][n]);
            O.TE[n] = tp<T>(B.tedge[a][n]);
        }
        launch_ppm<T, 3, 1, 0>(c, g, a, vel, mac[a], dt, rho, O, BT * (3.0 * g.N + nfaces(g, a)) + BT * 12.0 * nfaces(g, a));
    }
    for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        const double na = (double)nfaces(g, a), nt = (double)(nfaces(g, b1) + nfaces(g, b2));
        const double bytes = BT * (3.0 * g.N + na + nt) + BT * (12.0 * na + 3.0 * nt);
        C3<T> LO{{tp<T>(B.lo[a][0]), tp<T>(B.lo[a][1]), tp<T>(B.lo[a][2])}}, HI{{tp<T>(B.hi[a][0]), tp<T>(B.hi[a][1]), tp<T>(B.hi[a][2])}};
        C3<T> E1{{tp<T>(B.tedge[b1][0]), tp<T>(B.tedge[b1][1]), tp<T>(B.tedge[b1][2])}};
        C3<T> E2{{tp<T>(B.tedge[b2][0]), tp<T>(B.tedge[b2][1]), tp<T>(B.tedge[b2][2])}};
        P3<T> O1{{tp<T>(B.tr[a][b1][0]), tp<T>(B.tr[a][b1][1]), tp<T>(B.tr[a][b1][2])}};
        P3<T> O2{{tp<T>(B.tr[a][b2][0]), tp<T>(B.tr[a][b2][1]), tp<T>(B.tr[a][b2][2])}};
        const AdvTransOp<T, 3> op{g, a, b1, b2, vel, T(rho), T(dt / (3.0 * hd(g, b1))), T(dt / (3.0 * hd(g, b2))), mac[a], mac[b1], mac[b2],
                                  LO, HI, E1, E2, O1, O2};
        launch_cf(c, "k_adv_trans_x", "k_adv_trans_col", op, bytes);
    }
    C3<T> U{{mac[0], mac[1], mac[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double bytes = BT * (6.0 * g.N + nfaces(g, d) + nfaces(g, b1) + nfaces(g, b2)) +
                             BT * (9.0 * nfaces(g, d) + 3.0 * nfaces(g, b1) + 3.0 * nfaces(g, b2));
        C3<T> LO{{tp<T>(B.lo[d][0]), tp<T>(B.lo[d][1]), tp<T>(B.lo[d][2])}}, HI{{tp<T>(B.hi[d][0]), tp<T>(B.hi[d][1]), tp<T>(B.hi[d][2])}};
        C3<T> T1{{tp<T>(B.tr[b1][b2][0]), tp<T>(B.tr[b1][b2][1]), tp<T>(B.tr[b1][b2][2])}};
        C3<T> T2{{tp<T>(B.tr[b2][b1][0]), tp<T>(B.tr[b2][b1][1]), tp<T>(B.tr[b2][b1][2])}};
        P3<T> F{{tp<T>(B.flux[d][0]), tp<T>(B.flux[d][1]), tp<T>(B.flux[d][2])}};
        const AdvFluxOp<T, 3> op{g, d, b1, b2, vel, forces, T(rho), T(0.5) * T(dt) * T(rho), T(dt / (2.0 * hd(g, b1))), T(dt / (2.0 * hd(g, b2))),
                                 U, T1, T2, LO, HI, F};
        launch_cf(c, "k_adv_flux_x", "k_adv_flux_col", op, bytes);
    }
    FluxPtrs<T> F;
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < 3; ++n) F.p[d * 3 + n] = tp<T>(B.flux[d][n]);
    KS_LAUNCH(c, k_adv_div<T>, nblocks(g.N, BS), BS, BT * 9.0 * g.N + B8 * 3.0 * g.N, g, F, conv);
}

// Godunov fluxes of rho s for a cell scalar s (hoextrap at z walls, like a
// tangential velocity component) with the forces fs = src + diff, and conv =
// -div(flux) (AdvOp_Godunov.H:114-329).  FP64; the face arrays are the
// component-0 slots of B.
void launch_scalar_advection(Ctx& c, const Grid& g, const double* s, const double* fs, const double* const mac[3], double dt, double rho,
                             GodunovBufs& B, double* conv) {
    using T = double;
    const double B8 = 8.0;
    for (int a = 0; a < 3; ++a) {
        PpmOut<T, 1> O{};
        O.LO[0] = tp<T>(B.lo[a][0]);
        O.HI[0] = tp<T>(B.hi[a][0]);
        O.TE[0] = tp<T>(B.tedge[a][0]);
        launch_ppm<T, 1, 1, 1>(c, g, a, s, mac[a], dt, rho, O, B8 * (g.N + 4.0 * nfaces(g, a)));
    }
    for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        const double na = (double)nfaces(g, a), nt = (double)(nfaces(g, b1) + nfaces(g, b2));
        C3<T> LO{{tp<T>(B.lo[a][0]), nullptr, nullptr}}, HI{{tp<T>(B.hi[a][0]), nullptr, nullptr}};
        C3<T> E1{{tp<T>(B.tedge[b1][0]), nullptr, nullptr}}, E2{{tp<T>(B.tedge[b2][0]), nullptr, nullptr}};
        P3<T> O1{{tp<T>(B.tr[a][b1][0]), nullptr, nullptr}}, O2{{tp<T>(B.tr[a][b2][0]), nullptr, nullptr}};
        const AdvTransOp<T, 1> op{g, a, b1, b2, s, T(rho), T(dt / (3.0 * hd(g, b1))), T(dt / (3.0 * hd(g, b2))), mac[a], mac[b1], mac[b2],
                                  LO, HI, E1, E2, O1, O2};
        launch_cf(c, "k_scalar_trans_x", "k_scalar_trans_col", op, B8 * (g.N + 5.0 * na + 2.0 * nt));
    }
    C3<double> U{{mac[0], mac[1], mac[2]}};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        C3<T> LO{{tp<T>(B.lo[d][0]), nullptr, nullptr}}, HI{{tp<T>(B.hi[d][0]), nullptr, nullptr}};
        C3<T> T1{{tp<T>(B.tr[b1][b2][0]), nullptr, nullptr}}, T2{{tp<T>(B.tr[b2][b1][0]), nullptr, nullptr}};
        P3<T> F{{tp<T>(B.flux[d][0]), nullptr, nullptr}};
        const double bytes = B8 * (2.0 * g.N + 4.0 * nfaces(g, d) + 2.0 * (nfaces(g, b1) + nfaces(g, b2)));
        const AdvFluxOp<T, 1> op{g, d, b1, b2, s, fs, T(rho), T(0.5) * T(dt), T(dt / (2.0 * hd(g, b1))), T(dt / (2.0 * hd(g, b2))), U, T1, T2,
                                 LO, HI, F};
        launch_cf(c, "k_scalar_flux_x", "k_scalar_flux_col", op, bytes);
    }
    FluxPtrs<T> F;
    for (int m = 0; m < 9; ++m) F.p[m] = nullptr;
    for (int d = 0; d < 3; ++d) F.p[3 * d] = tp<T>(B.flux[d][0]);
    KS_LAUNCH(c, (k_adv_div<T, 1>), nblocks(g.N, BS), BS, B8 * (3.0 * g.N + g.N), g, F, conv);
}

// FP64 -> FP32 copy of an array (the mixed-precision advection reads FP32
// copies of its inputs: a conversion per load would cost an FP64 issue slot)
__global__ void k_to_single(const double* __restrict__ a, float* __restrict__ b, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) b[t] = (float)a[t];
}
static void to_single(Ctx& c, const double* a, float* b, long long n) {
    const long long nb = (n + BS - 1) / BS;
    KS_LAUNCH(c, k_to_single, (unsigned)(nb < 152 * 16 ? nb : 152 * 16), BS, 12.0 * n, a, b, n);
}

void launch_premac(Ctx& c, const Grid& g, const double* vel, const double* forces, double dt, GodunovBufs& B, double* mac[3], int fp32,
                   GodunovIn32* in32) {
    if (fp32) {
        to_single(c, vel, in32->vel, 3 * g.N);
        to_single(c, forces, in32->forces, 3 * g.N);
        premac_t<float>(c, g, in32->vel, in32->forces, dt, B, mac);
    } else {
        premac_t<double>(c, g, vel, forces, dt, B, mac);
    }
}

void launch_advection(Ctx& c, const Grid& g, const double* vel, const double* forces, const double* mac[3], double dt, double rho,
                      GodunovBufs& B, double* conv, int fp32, GodunovIn32* in32) {
    if (fp32) {
        // vel and forces: the FP32 copies made by launch_premac of the same step
        for (int d = 0; d < 3; ++d) to_single(c, mac[d], in32->mac[d], nfaces(g, d));
        const float* m32[3] = {in32->mac[0], in32->mac[1], in32->mac[2]};
        advection_t<float>(c, g, in32->vel, in32->forces, m32, dt, rho, B, conv);
    } else {
        advection_t<double>(c, g, vel, forces, mac, dt, rho, B, conv);
    }
}

}  // namespace ks
