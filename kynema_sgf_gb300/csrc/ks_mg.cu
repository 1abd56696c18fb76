// Geometric multigrid kernels for the two Poisson problems of the step.
//
// MAC projection (cell-centred, 7-point, beta = 1/rho0): red-black
// Gauss-Seidel with the exact local solve at Neumann z walls, residual with a
// max-norm partial, 8-cell average restriction, piecewise-constant
// prolongation (2- or 4-cell averages where the hierarchy is semicoarsened),
// single-CTA bottom sweeps.
//
// Nodal projection (node-centred, 27-point Q1 finite-element Laplacian times
// sigma = dt/rho0): weighted Jacobi, residual, full-weighting restriction
// (the transpose of trilinear prolongation over 8), trilinear prolongation,
// single-CTA bottom sweeps.  Wall-bounded z uses mirror images of the
// node values about the boundary node plane.
#include <cstdint>

#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;
constexpr int MAXPARTS = 1216;

template <int OPMAX>
__device__ inline double bred(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const double x = __shfl_down_sync(0xffffffffu, v, o);
        v = OPMAX ? nmax(v, x) : v + x;
    }
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : (OPMAX ? -1.0e300 : 0.0);
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) {
            const double x = __shfl_down_sync(0xffffffffu, v, o);
            v = OPMAX ? nmax(v, x) : v + x;
        }
    return v;
}

inline int parts_for(long long n) {
    long long b = (n + BS - 1) / BS;
    return (int)(b < MAXPARTS ? (b < 1 ? 1 : b) : MAXPARTS);
}

// Index maps use 32-bit arithmetic (every level holds fewer than 2^31
// points): a 64-bit division costs as much issue as the FP64 work of these
// light kernels.
__device__ inline void split3(unsigned t, unsigned nx, unsigned ny, int& i, int& j, int& k) {
    const unsigned r = t / nx;
    i = (int)(t - r * nx);
    k = (int)(r / ny);
    j = (int)(r - (unsigned)k * ny);
}

// running maximum of |x|: FP64 on the integer pipe (NaN kept), FP32 compares
template <typename T>
struct MaxAbs;
template <>
struct MaxAbs<double> {
    long long b = 0;
    __device__ inline void add(double x) { b = imax_abs(b, x); }
    __device__ inline double get() const { return bitsd(b); }
};
template <>
struct MaxAbs<float> {
    float m = 0.0f;
    __device__ inline void add(float x) { m = (x != x) ? x : fmaxf(m, fabsf(x)); }
    __device__ inline double get() const { return (double)m; }
};

// ---------------------------------------------------------------- cell-centred
template <typename T>
__device__ inline int ci3(const CCLevelT<T>& L, int i, int j, int k) { return (k * L.ny + j) * L.nx + i; }

// Weighted neighbour sum S = sum_m (w_m / d) p_m of the cell's class
// (interior, wall-adjacent, single layer; Neumann walls drop a z neighbour).
// The operator is beta * laplacian = dg * (p - S), dg = -beta d.
template <typename T>
__device__ inline T cc_nsum(const CCLevelT<T>& L, const T* p, int i, int j, int k, int& cls) {
    const int ip = i + 1 == L.nx ? 0 : i + 1, im = i == 0 ? L.nx - 1 : i - 1;
    const int jp = j + 1 == L.ny ? 0 : j + 1, jm = j == 0 ? L.ny - 1 : j - 1;
    cls = (L.zper || (k > 0 && k < L.nz - 1)) ? 0 : (L.nz == 1 ? 2 : 1);
    T zs;
    if (L.zper) zs = p[ci3(L, i, j, k == 0 ? L.nz - 1 : k - 1)] + p[ci3(L, i, j, k + 1 == L.nz ? 0 : k + 1)];
    else zs = (k > 0 ? p[ci3(L, i, j, k - 1)] : T(0)) + (k < L.nz - 1 ? p[ci3(L, i, j, k + 1)] : T(0));
    return L.gs[cls][0] * (p[ci3(L, ip, j, k)] + p[ci3(L, im, j, k)]) + L.gs[cls][1] * (p[ci3(L, i, jp, k)] + p[ci3(L, i, jm, k)]) +
           L.gs[cls][2] * zs;
}

// Gauss-Seidel point update solved for the new value:
// dg (p - S) = rhs  =>  p = rhs / dg + S
template <typename T>
__device__ inline T cc_gs_point(const CCLevelT<T>& L, const T* p, int i, int j, int k, T rhs) {
    int cls;
    const T S = cc_nsum(L, p, i, j, k, cls);
    return L.inv_diag[cls] * rhs + S;
}

// Red-black Gauss-Seidel half-sweep (cells with (i + j + k) % 2 == color),
// z-marching: thread (i2, j) owns the cell pair (2 i2, 2 i2 + 1) of row j and
// walks k through a chunk of the column, updating the pair member of the
// sweep's colour at each k.  The per-class weights are scalars selected by the
// layer's class, the neighbour offsets are formed once per thread: about 30
// instructions per update where a thread-per-cell launch spends ~300 on index
// maps and indexed parameter loads (it is instruction-bound, in FP32 as in
// FP64).  The level's x extent is even (coarsening keeps it a multiple of 4).
template <typename T>
struct CCCoef {  // per class (interior, wall-adjacent, single layer): w_x / d, w_y / d, w_z / d, 1 / dg, dg
    T gx0, gx1, gx2, gy0, gy1, gy2, gz0, gz1, gz2, iv0, iv1, iv2, dg0, dg1, dg2;
};
template <typename T>
inline CCCoef<T> cc_coef(const CCLevelT<T>& L) {
    return CCCoef<T>{L.gs[0][0], L.gs[1][0], L.gs[2][0], L.gs[0][1], L.gs[1][1], L.gs[2][1], L.gs[0][2], L.gs[1][2],
                     L.gs[2][2], L.inv_diag[0], L.inv_diag[1], L.inv_diag[2], L.dg[0], L.dg[1], L.dg[2]};
}
template <typename T>
__global__ void k_cc_gsrb(CCLevelT<T> L, CCCoef<T> w, int color, int kc) {
    const int i2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (i2 >= (L.nx >> 1)) return;
    const int j = blockIdx.y;
    const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, L.nz);
    const int sy = L.nx, sz = L.nx * L.ny;
    const int dyp = (j + 1 == L.ny ? -j : 1) * sy, dym = (j == 0 ? L.ny - 1 : -1) * sy;
    T* p = L.phi;
    const T* rhs = L.rhs;
    // The values one update needs: its right-hand side, the x and y neighbour
    // pair sums and the z neighbour sum (all of the other colour, which this
    // half-sweep does not write).  They are loaded one layer ahead, before the
    // store of the current layer, so the loads of layer k + 1 overlap the
    // FP64 work of layer k.
    struct Upd {
        int c;
        T r, sx, sy, sz;
    };
    auto fetch = [&](int k) {
        Upd u;
        const int i = 2 * i2 + ((j + k + color) & 1);
        u.c = k * sz + j * sy + i;
        const int dxp = i + 1 == L.nx ? 1 - L.nx : 1, dxm = i == 0 ? L.nx - 1 : -1;
        u.r = rhs[u.c];
        u.sx = p[u.c + dxp] + p[u.c + dxm];
        u.sy = p[u.c + dyp] + p[u.c + dym];
        if (L.zper) {
            const int kp = k + 1 == L.nz ? 0 : k + 1, km = k == 0 ? L.nz - 1 : k - 1;
            u.sz = p[u.c + (kp - k) * sz] + p[u.c + (km - k) * sz];
        } else {
            u.sz = (k == 0 ? T(0) : p[u.c - sz]) + (k + 1 == L.nz ? T(0) : p[u.c + sz]);
        }
        return u;
    };
    Upd cur = fetch(k0);
    for (int k = k0; k < k1; ++k) {
        Upd nxt = cur;
        if (k + 1 < k1) nxt = fetch(k + 1);
        T gx = w.gx0, gy = w.gy0, gz = w.gz0, iv = w.iv0;
        if (!L.zper && (k == 0 || k + 1 == L.nz)) {
            const bool one = L.nz == 1;
            gx = one ? w.gx2 : w.gx1;
            gy = one ? w.gy2 : w.gy1;
            gz = one ? w.gz2 : w.gz1;
            iv = one ? w.iv2 : w.iv1;
        }
        p[cur.c] = iv * cur.r + (gx * cur.sx + gy * cur.sy + gz * cur.sz);
        cur = nxt;
    }
}

// residual with block maxima of its magnitude; with r32 (defect correction of
// the mixed-precision form) it goes to the FP32 cycle's right-hand side r32,
// whose solution z32 starts at zero, instead of L.res.  Grid-stride over
// (i, j, chunk of kc layers) columns marching in k, with the class weights
// selected from scalars (as in k_cc_gsrb).  zc = 0 / 1: the cells of that
// colour, (i + j + k) & 1 == zc, were the last half-sweep's, whose update
// solved their equations with their (other-colour) neighbours unchanged, so
// their residual is zero to rounding: it is written as 0 without the
// stencil.  A thread then owns the cell pair (2 i2, 2 i2 + 1) of a row, as in
// k_cc_gsrb, so that every lane of a warp evaluates the same colour (half the
// FP64 work); zc = -1: every cell is evaluated.
template <typename T>
__global__ void k_cc_resid(CCLevelT<T> L, CCCoef<T> w, int kc, double* parts, float* r32, float* z32, int zc) {
    const int sy = L.nx, sz = L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    if (zc >= 0) {
        const int hx = L.nx >> 1;
        const unsigned M2 = (unsigned)(hx * L.ny * nch);
        MaxAbs<T> mx;
        const T* p = L.phi;
        for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M2; t += gridDim.x * blockDim.x) {
            int i2, j, ch;
            split3(t, (unsigned)hx, (unsigned)L.ny, i2, j, ch);
            const int dyp = (j + 1 == L.ny ? -j : 1) * sy, dym = (j == 0 ? L.ny - 1 : -1) * sy;
            const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
            for (int k = k0; k < k1; ++k) {
                const int o = (j + k + 1 - zc) & 1;  // the pair member of the evaluated colour 1 - zc
                const int i = 2 * i2 + o, c = k * sz + j * sy + i;
                const int dxp = i + 1 == L.nx ? 1 - L.nx : 1, dxm = i == 0 ? L.nx - 1 : -1;
                const T sx = p[c + dxp] + p[c + dxm];
                const T syv = p[c + dyp] + p[c + dym];
                T szv;
                if (L.zper) {
                    const int kp = k + 1 == L.nz ? 0 : k + 1, km = k == 0 ? L.nz - 1 : k - 1;
                    szv = p[c + (kp - k) * sz] + p[c + (km - k) * sz];
                } else {
                    szv = (k == 0 ? T(0) : p[c - sz]) + (k + 1 == L.nz ? T(0) : p[c + sz]);
                }
                T gx = w.gx0, gy = w.gy0, gz = w.gz0, dg = w.dg0;
                if (!L.zper && (k == 0 || k + 1 == L.nz)) {
                    const bool one = L.nz == 1;
                    gx = one ? w.gx2 : w.gx1;
                    gy = one ? w.gy2 : w.gy1;
                    gz = one ? w.gz2 : w.gz1;
                    dg = one ? w.dg2 : w.dg1;
                }
                const T S = gx * sx + gy * syv + gz * szv;
                const T v = L.rhs[c] - dg * (p[c] - S);
                L.res[c] = v;
                L.res[c + 1 - 2 * o] = T(0);  // the other member
                mx.add(v);
            }
        }
        const double m = bred<1>(mx.get());
        if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
        return;
    }
    const unsigned M = (unsigned)(sz * nch);
    MaxAbs<T> mx;
    const T* p = L.phi;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        int i, j, ch;
        split3(t, (unsigned)L.nx, (unsigned)L.ny, i, j, ch);
        const int dxp = i + 1 == L.nx ? 1 - L.nx : 1, dxm = i == 0 ? L.nx - 1 : -1;
        const int dyp = (j + 1 == L.ny ? -j : 1) * sy, dym = (j == 0 ? L.ny - 1 : -1) * sy;
        const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
        // the loads of layer k + 1 are issued before the stores of layer k
        struct Ld {
            T r, pc, sx, sy, sz;
        };
        auto fetch = [&](int k) {
            Ld u;
            const int c = k * sz + j * sy + i;
            u.r = L.rhs[c];
            u.pc = p[c];
            u.sx = p[c + dxp] + p[c + dxm];
            u.sy = p[c + dyp] + p[c + dym];
            if (L.zper) {
                const int kp = k + 1 == L.nz ? 0 : k + 1, km = k == 0 ? L.nz - 1 : k - 1;
                u.sz = p[c + (kp - k) * sz] + p[c + (km - k) * sz];
            } else {
                u.sz = (k == 0 ? T(0) : p[c - sz]) + (k + 1 == L.nz ? T(0) : p[c + sz]);
            }
            return u;
        };
        Ld cur = fetch(k0);
        for (int k = k0; k < k1; ++k) {
            Ld nxt = cur;
            if (k + 1 < k1) nxt = fetch(k + 1);
            const int c = k * sz + j * sy + i;
            T gx = w.gx0, gy = w.gy0, gz = w.gz0, dg = w.dg0;
            if (!L.zper && (k == 0 || k + 1 == L.nz)) {
                const bool one = L.nz == 1;
                gx = one ? w.gx2 : w.gx1;
                gy = one ? w.gy2 : w.gy1;
                gz = one ? w.gz2 : w.gz1;
                dg = one ? w.dg2 : w.dg1;
            }
            const T S = gx * cur.sx + gy * cur.sy + gz * cur.sz;
            const T v = cur.r - dg * (cur.pc - S);
            cur = nxt;
            if (r32) {
                r32[c] = (float)v;
                z32[c] = 0.0f;
            } else {
                L.res[c] = v;
            }
            mx.add(v);
        }
    }
    const double m = bred<1>(mx.get());
    if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
}

// layers per thread of the column kernels: long columns on the large levels
template <typename T>
inline int cc_chunk(const CCLevelT<T>& L) {
    const long long work = (long long)L.nx * L.ny * L.nz / 300000;
    return (int)(work < 1 ? 1 : (work > 16 ? 16 : work));
}

template <typename T>
__global__ void k_cc_restrict(CCLevelT<T> F, CCLevelT<T> C) {
    const unsigned N = (unsigned)(C.nx * C.ny * C.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int i, j, k;
    split3(t, (unsigned)C.nx, (unsigned)C.ny, i, j, k);
    const T* r = F.res + ci3(F, 2 * i, 2 * j, 2 * k);
    const int sy = F.nx, sz = F.nx * F.ny;
    const T s = ((r[0] + r[1]) + (r[sy] + r[sy + 1])) + ((r[sz] + r[sz + 1]) + (r[sz + sy] + r[sz + sy + 1]));
    C.rhs[t] = T(0.125) * s;
    C.phi[t] = T(0);
}

template <typename T>
__global__ void k_cc_prolong(CCLevelT<T> F, CCLevelT<T> C) {
    const unsigned N = (unsigned)(F.nx * F.ny * F.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int i, j, k;
    split3(t, (unsigned)F.nx, (unsigned)F.ny, i, j, k);
    F.phi[t] += C.phi[ci3(C, i / 2, j / 2, k / 2)];
}

// The same pair between levels of a semicoarsened hierarchy: ratio rx, ry, rz
// (1 or 2 each) per direction, F.n = r C.n in every direction (checked where
// the hierarchy is built), w = 1 / (rx ry rz).  The fine cells of a coarse
// cell are summed z-, y-, x-outermost-first, as the oracle sums them.
template <typename T>
__global__ void k_cc_restrict_r(CCLevelT<T> F, CCLevelT<T> C, int rx, int ry, int rz, T w) {
    const unsigned N = (unsigned)(C.nx * C.ny * C.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int i, j, k;
    split3(t, (unsigned)C.nx, (unsigned)C.ny, i, j, k);
    T s = T(0);
    for (int c = 0; c < rz; ++c)
        for (int b = 0; b < ry; ++b)
            for (int a = 0; a < rx; ++a) s += F.res[ci3(F, rx * i + a, ry * j + b, rz * k + c)];
    C.rhs[t] = w * s;
    C.phi[t] = T(0);
}

template <typename T>
__global__ void k_cc_prolong_r(CCLevelT<T> F, CCLevelT<T> C, int rx, int ry, int rz) {
    const unsigned N = (unsigned)(F.nx * F.ny * F.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int i, j, k;
    split3(t, (unsigned)F.nx, (unsigned)F.ny, i, j, k);
    F.phi[t] += C.phi[ci3(C, i / rx, j / ry, k / rz)];
}

// Bottom solve: red-black sweeps by one CTA.  Levels of up to BOTTOM_SMEM
// points are staged in shared memory (phi and rhs), larger ones sweep in
// global memory.
constexpr int BOTTOM_SMEM = 2048;
template <typename T, bool SMEM>
__global__ void k_cc_bottom(CCLevelT<T> L, T beta, int sweeps) {
    const int N = L.nx * L.ny * L.nz;
    __shared__ T sp[SMEM ? BOTTOM_SMEM : 1], sr[SMEM ? BOTTOM_SMEM : 1];
    T* p = L.phi;
    const T* r = L.rhs;
    if (SMEM) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            sp[t] = L.phi[t];
            sr[t] = L.rhs[t];
        }
        __syncthreads();
        p = sp;
        r = sr;
    }
    for (int s = 0; s < sweeps; ++s)
        for (int color = 0; color < 2; ++color) {
            for (int t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                split3((unsigned)t, (unsigned)L.nx, (unsigned)L.ny, i, j, k);
                if (((i + j + k) & 1) != color) continue;
                p[t] = cc_gs_point(L, p, i, j, k, r[t]);
            }
            __syncthreads();
        }
    if (SMEM)
        for (int t = threadIdx.x; t < N; t += blockDim.x) L.phi[t] = sp[t];
}

// Direct bottom solve: phi = scale * Binv rhs, Binv the pinned inverse of the
// bottom level's operator (the solution with phi[0] = 0 of the singular
// system), one warp per row with the lanes over the columns.
template <typename T>
__global__ void k_bottom_direct(const T* __restrict__ binv, int n, const T* rhs, T* phi, T scale) {
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= n) return;  // whole warps
    const T* row = binv + (long long)r * n;
    T acc = T(0);
    for (int c = lane; c < n; c += 32) acc += row[c] * rhs[c];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) phi[r] = scale * acc;
}

// ---------------------------------------------------------------- nodal
template <typename T>
__device__ inline T nd_at(const NDLevelT<T>& L, const T* p, int i, int j, int k) {
    i = i < 0 ? i + L.nx : (i >= L.nx ? i - L.nx : i);
    j = j < 0 ? j + L.ny : (j >= L.ny ? j - L.ny : j);
    if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
    else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
    return p[(k * L.ny + j) * L.nx + i];
}

// sigma * (27-point Q1 stencil) at node (i,j,k); the weights are symmetric in
// each direction, so neighbours are summed by weight class first.
template <typename T>
__device__ inline T nd_ax(const NDLevelT<T>& L, const T* p, T sigma, int i, int j, int k) {
    const int im = i == 0 ? L.nx - 1 : i - 1, ip = i + 1 == L.nx ? 0 : i + 1;
    const int jm = j == 0 ? L.ny - 1 : j - 1, jp = j + 1 == L.ny ? 0 : j + 1;
    int km, kp;
    if (L.zper) {
        km = k == 0 ? L.nz - 1 : k - 1;
        kp = k + 1 == L.nz ? 0 : k + 1;
    } else {
        km = k == 0 ? 1 : k - 1;
        kp = k + 1 == L.nz ? L.nz - 2 : k + 1;
    }
    const int sy = L.nx, sz = L.nx * L.ny;
    const int rm = km * sz, r0 = k * sz, rp = kp * sz;
    const int cm = jm * sy, c0 = j * sy, cp = jp * sy;
    auto at = [&](int r, int c, int x) { return p[r + c + x]; };
    const T ctr = at(r0, c0, i);
    T fx = T(0), fy = T(0), fz = T(0);
    if (!L.faces_zero) {
        fx = at(r0, c0, im) + at(r0, c0, ip);
        fy = at(r0, cm, i) + at(r0, cp, i);
        fz = at(rm, c0, i) + at(rp, c0, i);
    }
    const T exy = at(r0, cm, im) + at(r0, cm, ip) + at(r0, cp, im) + at(r0, cp, ip);
    const T exz = at(rm, c0, im) + at(rm, c0, ip) + at(rp, c0, im) + at(rp, c0, ip);
    const T eyz = at(rm, cm, i) + at(rm, cp, i) + at(rp, cm, i) + at(rp, cp, i);
    const T cr = at(rm, cm, im) + at(rm, cm, ip) + at(rm, cp, im) + at(rm, cp, ip) + at(rp, cm, im) + at(rp, cm, ip) + at(rp, cp, im) +
                 at(rp, cp, ip);
    T s = L.W[13] * ctr + L.W[9] * exy + L.W[3] * exz + L.W[1] * eyz + L.W[0] * cr;
    if (!L.faces_zero) s += L.W[12] * fx + L.W[10] * fy + L.W[4] * fz;
    return sigma * s;
}

// sigma-scaled weight classes of the stencil (negated) and the Jacobi factor
// omega / (sigma W_centre), formed on the host once per launch
template <typename T>
struct NdCoef {
    T c13, c9, c3, c1, c0, c12, c10, c4, oinv;
};
template <typename T>
inline NdCoef<T> nd_coef(const NDLevelT<T>& L, double sigma, double omega) {
    NdCoef<T> c;
    c.c13 = T(-sigma * (double)L.W[13]);
    c.c9 = T(-sigma * (double)L.W[9]);
    c.c3 = T(-sigma * (double)L.W[3]);
    c.c1 = T(-sigma * (double)L.W[1]);
    c.c0 = T(-sigma * (double)L.W[0]);
    c.c12 = T(-sigma * (double)L.W[12]);
    c.c10 = T(-sigma * (double)L.W[10]);
    c.c4 = T(-sigma * (double)L.W[4]);
    c.oinv = T(omega * (double)L.inv_diag);
    return c;
}

// Column (z-marching) form of the same stencil for the sweeps over a whole
// level: each thread walks k through a chunk of one (i, j) column.  Per node
// plane it forms the in-plane corner sum P, the x- and y-neighbour sums Ex, Ey
// and the centre value C once; node k combines planes k-1, k, k+1:
//   A phi = W13 C0 + W9 P0 + W3 (Ex- + Ex+) + W1 (Ey- + Ey+) + W0 (P- + P+)
//           [+ W12 Ex0 + W10 Ey0 + W4 (C- + C+) when face weights are non-zero],
// about half the FP64 operations of the node-by-node sums; the residual is
// one FMA chain from rhs with the sigma-scaled weights.
// MODE 0: out = in + omega (rhs - A in) / diag.  MODE 1: the same plus block
// maxima of |rhs - A in|.  MODE 2: res = rhs - A phi plus block maxima.
template <typename T, int MODE>
__global__ void k_nd_col(NDLevelT<T> L, NdCoef<T> w, const T* in, T* out, int kc, double* parts, float* r32 = nullptr,
                         float* z32 = nullptr) {
    const int sz = L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    const unsigned M = (unsigned)(sz * nch);
    MaxAbs<T> mx;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        int i, j, ch;
        split3(t, (unsigned)L.nx, (unsigned)L.ny, i, j, ch);
        const int im = i == 0 ? L.nx - 1 : i - 1, ip = i + 1 == L.nx ? 0 : i + 1;
        const int cm = (j == 0 ? L.ny - 1 : j - 1) * L.nx, c0 = j * L.nx;
        const int cp = (j + 1 == L.ny ? 0 : j + 1) * L.nx;
        auto plane = [&](int k, T& P, T& Ex, T& Ey, T& C) {
            if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
            else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
            const T* q = in + k * sz;
            P = (q[cm + im] + q[cm + ip]) + (q[cp + im] + q[cp + ip]);
            Ex = q[c0 + im] + q[c0 + ip];
            Ey = q[cm + i] + q[cp + i];
            C = q[c0 + i];
        };
        const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
        T Pm, Exm, Eym, Cm, P0, Ex0, Ey0, C0;
        plane(k0 - 1, Pm, Exm, Eym, Cm);
        plane(k0, P0, Ex0, Ey0, C0);
        for (int k = k0; k < k1; ++k) {
            T Pp, Exp, Eyp, Cp;
            plane(k + 1, Pp, Exp, Eyp, Cp);
            const int idx = k * sz + c0 + i;
            T res = L.rhs[idx];
            res = w.c13 * C0 + res;
            res = w.c9 * P0 + res;
            res = w.c3 * (Exm + Exp) + res;
            res = w.c1 * (Eym + Eyp) + res;
            res = w.c0 * (Pm + Pp) + res;
            if (!L.faces_zero) {
                res = w.c12 * Ex0 + res;
                res = w.c10 * Ey0 + res;
                res = w.c4 * (Cm + Cp) + res;
            }
            if (MODE == 2) {
                if (r32) {  // residual to the FP32 cycle's right-hand side (as in k_cc_resid)
                    r32[idx] = (float)res;
                    z32[idx] = 0.0f;
                } else {
                    L.res[idx] = res;
                }
            } else {
                out[idx] = w.oinv * res + C0;
            }
            if (MODE >= 1) mx.add(res);
            Pm = P0;
            Exm = Ex0;
            Eym = Ey0;
            Cm = C0;
            P0 = Pp;
            Ex0 = Exp;
            Ey0 = Eyp;
            C0 = Cp;
        }
    }
    if (MODE >= 1) {
        const double m = bred<1>(mx.get());
        if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
    }
}

// FP32 form of k_nd_col for the sweeps (MODE 0) and residuals (MODE 2) of the
// mixed-precision cycles: two nodes per step of the column, so the loads of
// planes k + 1 and k + 2 are in flight together.  The FP32 sweep waits on
// memory latency rather than on issue (one plane of loads per step kept each
// warp idle for most of a DRAM round trip).
template <int MODE>
__global__ void __launch_bounds__(256, 4) k_nd_col2(NDLevelT<float> L, NdCoef<float> w, const float* in, float* out, int kc,
                                                    double* parts) {
    const int sz = L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    const unsigned M = (unsigned)(sz * nch);
    MaxAbs<float> mx;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        int i, j, ch;
        split3(t, (unsigned)L.nx, (unsigned)L.ny, i, j, ch);
        const int im = i == 0 ? L.nx - 1 : i - 1, ip = i + 1 == L.nx ? 0 : i + 1;
        const int cm = (j == 0 ? L.ny - 1 : j - 1) * L.nx, c0 = j * L.nx;
        const int cp = (j + 1 == L.ny ? 0 : j + 1) * L.nx;
        auto plane = [&](int k, float& P, float& Ex, float& Ey, float& C) {
            if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
            else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
            const float* q = in + k * sz;
            P = (q[cm + im] + q[cm + ip]) + (q[cp + im] + q[cp + ip]);
            Ex = q[c0 + im] + q[c0 + ip];
            Ey = q[cm + i] + q[cp + i];
            C = q[c0 + i];
        };
        auto node = [&](float res, float Pm, float Exm, float Eym, float Cm, float P0, float Ex0, float Ey0, float C0, float Pp, float Exp,
                        float Eyp, float Cp, int idx) {
            res = w.c13 * C0 + res;
            res = w.c9 * P0 + res;
            res = w.c3 * (Exm + Exp) + res;
            res = w.c1 * (Eym + Eyp) + res;
            res = w.c0 * (Pm + Pp) + res;
            if (!L.faces_zero) {
                res = w.c12 * Ex0 + res;
                res = w.c10 * Ey0 + res;
                res = w.c4 * (Cm + Cp) + res;
            }
            if (MODE == 2) L.res[idx] = res;
            else out[idx] = w.oinv * res + C0;
            if (MODE == 2) mx.add(res);
        };
        const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
        float Pm, Exm, Eym, Cm, P0, Ex0, Ey0, C0;
        plane(k0 - 1, Pm, Exm, Eym, Cm);
        plane(k0, P0, Ex0, Ey0, C0);
        for (int k = k0; k < k1; k += 2) {
            const bool two = k + 1 < k1;
            const int idx = k * sz + c0 + i;
            float Pp, Exp, Eyp, Cp, Pq = 0.0f, Exq = 0.0f, Eyq = 0.0f, Cq = 0.0f, r1 = 0.0f;
            plane(k + 1, Pp, Exp, Eyp, Cp);
            const float r0 = L.rhs[idx];
            if (two) {
                plane(k + 2, Pq, Exq, Eyq, Cq);
                r1 = L.rhs[idx + sz];
            }
            node(r0, Pm, Exm, Eym, Cm, P0, Ex0, Ey0, C0, Pp, Exp, Eyp, Cp, idx);
            if (two) {
                node(r1, P0, Ex0, Ey0, C0, Pp, Exp, Eyp, Cp, Pq, Exq, Eyq, Cq, idx + sz);
                Pm = Pp; Exm = Exp; Eym = Eyp; Cm = Cp;
                P0 = Pq; Ex0 = Exq; Ey0 = Eyq; C0 = Cq;
            } else {
                Pm = P0; Exm = Ex0; Eym = Ey0; Cm = C0;
                P0 = Pp; Ex0 = Exp; Ey0 = Eyp; C0 = Cp;
            }
        }
    }
    if (MODE == 2) {
        const double m = bred<1>(mx.get());
        if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
    }
}

// V consecutive nodes of a row as one vector access (the row offset is a
// multiple of V, the level's arrays V-element aligned: checked by the launchers)
template <int V, typename T>
__device__ inline void ldv(const T* p, T* v) {
    if constexpr (V == 4 && sizeof(T) == 4) {
        const float4 x = *reinterpret_cast<const float4*>(p);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else if constexpr (V == 2 && sizeof(T) == 8) {
        const double2 x = *reinterpret_cast<const double2*>(p);
        v[0] = x.x; v[1] = x.y;
    } else if constexpr (V == 2 && sizeof(T) == 4) {
        const float2 x = *reinterpret_cast<const float2*>(p);
        v[0] = x.x; v[1] = x.y;
    } else {
        for (int m = 0; m < V; ++m) v[m] = p[m];
    }
}
template <int V, typename T>
__device__ inline void stv(T* p, const T* v) {
    if constexpr (V == 4 && sizeof(T) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (V == 2 && sizeof(T) == 8) {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    } else if constexpr (V == 2 && sizeof(T) == 4) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else {
        for (int m = 0; m < V; ++m) p[m] = v[m];
    }
}

// FP32 column kernel over V = 4 nodes of a row per thread, for the sweeps
// (MODE 0) and residuals (MODE 2) of the mixed-precision cycles, which wait on
// load latency rather than on arithmetic.  A node plane's row j and its
// neighbour rows j -+ 1 are read as one vector each plus the two x-edge
// values (3 vector + 6 scalar loads per 4 nodes, where k_nd_col2 issues 9
// scalar loads per node), and adjacent nodes share their x sums:
//   Ey_m = a_m + c_m (rows j - 1, j + 1),  P_m = Ey_{m-1} + Ey_{m+1},
//   Ex_m = b_{m-1} + b_{m+1} (row j),      C_m = b_m.
// Each plane is reduced once to the terms a node takes from it as a z
// neighbour, Q = c3 Ex + c1 Ey + c0 P [+ c4 C], and as the centre plane,
// R = c13 C + c9 P [+ c12 Ex + c10 Ey], so that node k's residual is
//   rhs + R_k + (Q_{k-1} + Q_{k+1})
// (the sigma-scaled weights negated; the brackets when the face weights are
// non-zero).  FP64 keeps k_nd_col: it is bound by the FP64 pipe, and with
// equal spacings (face weights zero) the plane terms save no FP64 operation
// over its per-node chain once the planes above and below a column chunk
// are counted.  The template stays general in T and V (ldv / stv).
template <typename T, int V, int MODE>
__global__ void __launch_bounds__(256) k_nd_xv(NDLevelT<T> L, NdCoef<T> w, const T* in, T* out, int kc, double* parts) {
    const int nq = L.nx / V, sz = L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    const unsigned M = (unsigned)(nq * L.ny * nch);
    MaxAbs<T> mx;
    struct Pl {
        T Q[V], R[V], C[V];
    };
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        int q, j, ch;
        split3(t, (unsigned)nq, (unsigned)L.ny, q, j, ch);
        const int i0 = V * q;
        const int im = i0 == 0 ? L.nx - 1 : i0 - 1, ip = i0 + V == L.nx ? 0 : i0 + V;
        const int cm = (j == 0 ? L.ny - 1 : j - 1) * L.nx, c0 = j * L.nx;
        const int cp = (j + 1 == L.ny ? 0 : j + 1) * L.nx;
        auto plane = [&](int k, Pl& o) {
            if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
            else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
            const T* p = in + k * sz;
            T a[V + 2], b[V + 2], c[V + 2];
            ldv<V>(p + cm + i0, a + 1);
            ldv<V>(p + c0 + i0, b + 1);
            ldv<V>(p + cp + i0, c + 1);
            a[0] = p[cm + im]; a[V + 1] = p[cm + ip];
            b[0] = p[c0 + im]; b[V + 1] = p[c0 + ip];
            c[0] = p[cp + im]; c[V + 1] = p[cp + ip];
            T ey[V + 2];
            for (int m = 0; m < V + 2; ++m) ey[m] = a[m] + c[m];
            for (int m = 0; m < V; ++m) {
                const T P = ey[m] + ey[m + 2], Ex = b[m] + b[m + 2], Ey = ey[m + 1], C = b[m + 1];
                T Qv = w.c0 * P;
                Qv = w.c1 * Ey + Qv;
                Qv = w.c3 * Ex + Qv;
                T Rv = w.c13 * C;
                Rv = w.c9 * P + Rv;
                if (!L.faces_zero) {
                    Qv = w.c4 * C + Qv;
                    Rv = w.c12 * Ex + Rv;
                    Rv = w.c10 * Ey + Rv;
                }
                o.Q[m] = Qv;
                o.R[m] = Rv;
                o.C[m] = C;
            }
        };
        const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
        Pl pm, p0, pp;
        plane(k0 - 1, pm);
        plane(k0, p0);
        for (int k = k0; k < k1; ++k) {
            plane(k + 1, pp);
            const int idx = k * sz + c0 + i0;
            T r[V];
            ldv<V>(L.rhs + idx, r);
            for (int m = 0; m < V; ++m) {
                const T res = (r[m] + p0.R[m]) + (pm.Q[m] + pp.Q[m]);
                if (MODE >= 1) mx.add(res);
                r[m] = MODE == 2 ? res : w.oinv * res + p0.C[m];
            }
            stv<V>((MODE == 2 ? L.res : out) + idx, r);
            pm = p0;
            p0 = pp;
        }
    }
    if (MODE >= 1) {
        const double m = bred<1>(mx.get());
        if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
    }
}

// FP32 forms of k_cc_gsrb and k_cc_resid over 4 cells of a row per thread
// (the mixed-precision cycles on the large levels).  A layer's row j and its
// neighbour rows j -+ 1 and the right-hand side are read as one vector each,
// and the row j vectors of layers k -+ 1 are the ones the column step before
// and after reads as its centre, so that a layer costs 4 vector loads and one
// or two edge values where the scalar kernels issue 7 loads per cell.  Every
// cell is evaluated with the scalar kernels' expression (bitwise the same
// result).  In the half-sweep the thread updates the 2 cells of the colour,
// at offsets o and o + 2 (o = (j + k + colour) & 1); the values it keeps from
// one layer to the next are read only where they are of the other colour,
// which the half-sweep does not write.
__device__ inline float sel2(const float v[4], int o, int m) { return o ? v[m + 1] : v[m]; }

__global__ void __launch_bounds__(128) k_cc_gsrb4(CCLevelT<float> L, CCCoef<float> w, int color, int kc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (L.nx >> 2)) return;
    const int j = blockIdx.y;
    const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, L.nz);
    const int sy = L.nx, sz = L.nx * L.ny, i0 = 4 * q;
    const int dyp = (j + 1 == L.ny ? -j : 1) * sy, dym = (j == 0 ? L.ny - 1 : -1) * sy;
    const int el = i0 == 0 ? L.nx - 1 : -1, er = i0 + 4 == L.nx ? -i0 : 4;  // edge cells, from the quad's first
    float* p = L.phi;
    auto row = [&](int k, float v[4]) {
        if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
        if (k < 0 || k >= L.nz) {
            v[0] = v[1] = v[2] = v[3] = 0.0f;
            return;
        }
        ldv<4>(p + k * sz + j * sy + i0, v);
    };
    struct Ld {
        float ym[4], yp[4], r[4], up[4], e;
    };
    auto fetch = [&](int k, Ld& u) {
        const int b = k * sz + j * sy + i0;
        ldv<4>(p + b + dym, u.ym);
        ldv<4>(p + b + dyp, u.yp);
        ldv<4>(L.rhs + b, u.r);
        row(k + 1, u.up);
        u.e = p[b + (((j + k + color) & 1) ? er : el)];
    };
    float dn[4], cur[4];
    row(k0 - 1, dn);
    row(k0, cur);
    Ld a, nx;
    fetch(k0, a);
    for (int k = k0; k < k1; ++k) {
        if (k + 1 < k1) fetch(k + 1, nx);
        const int o = (j + k + color) & 1;
        float gx = w.gx0, gy = w.gy0, gz = w.gz0, iv = w.iv0;
        if (!L.zper && (k == 0 || k + 1 == L.nz)) {
            const bool one = L.nz == 1;
            gx = one ? w.gx2 : w.gx1;
            gy = one ? w.gy2 : w.gy1;
            gz = one ? w.gz2 : w.gz1;
            iv = one ? w.iv2 : w.iv1;
        }
        // x neighbours of the cells at o and o + 2: (edge, 1), (1, 3) or (0, 2), (2, edge)
        const float sx0 = o ? cur[0] + cur[2] : cur[1] + a.e, sx1 = o ? a.e + cur[2] : cur[3] + cur[1];
        const float sy0 = sel2(a.yp, o, 0) + sel2(a.ym, o, 0), sy1 = sel2(a.yp, o, 2) + sel2(a.ym, o, 2);
        const float sz0 = sel2(dn, o, 0) + sel2(a.up, o, 0), sz1 = sel2(dn, o, 2) + sel2(a.up, o, 2);
        const int b = k * sz + j * sy + i0 + o;
        p[b] = iv * sel2(a.r, o, 0) + (gx * sx0 + gy * sy0 + gz * sz0);
        p[b + 2] = iv * sel2(a.r, o, 2) + (gx * sx1 + gy * sy1 + gz * sz1);
        for (int m = 0; m < 4; ++m) {
            dn[m] = cur[m];
            cur[m] = a.up[m];
        }
        a = nx;
    }
}

__global__ void __launch_bounds__(256) k_cc_resid4(CCLevelT<float> L, CCCoef<float> w, int kc, double* parts) {
    const int nq = L.nx >> 2, sy = L.nx, sz = L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    const unsigned M = (unsigned)(nq * L.ny * nch);
    MaxAbs<float> mx;
    const float* p = L.phi;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        int q, j, ch;
        split3(t, (unsigned)nq, (unsigned)L.ny, q, j, ch);
        const int i0 = 4 * q;
        const int dyp = (j + 1 == L.ny ? -j : 1) * sy, dym = (j == 0 ? L.ny - 1 : -1) * sy;
        const int el = i0 == 0 ? L.nx - 1 : -1, er = i0 + 4 == L.nx ? -i0 : 4;
        const int k0 = ch * kc, k1 = min(k0 + kc, L.nz);
        auto row = [&](int k, float v[4]) {
            if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
            if (k < 0 || k >= L.nz) {
                v[0] = v[1] = v[2] = v[3] = 0.0f;
                return;
            }
            ldv<4>(p + k * sz + j * sy + i0, v);
        };
        float dn[4], cur[4];
        row(k0 - 1, dn);
        row(k0, cur);
        for (int k = k0; k < k1; ++k) {
            const int b = k * sz + j * sy + i0;
            float ym[4], yp[4], r[4], up[4];
            ldv<4>(p + b + dym, ym);
            ldv<4>(p + b + dyp, yp);
            ldv<4>(L.rhs + b, r);
            row(k + 1, up);
            float x[6];  // row j with its two edge cells
            x[0] = p[b + el];
            x[5] = p[b + er];
            for (int m = 0; m < 4; ++m) x[m + 1] = cur[m];
            float gx = w.gx0, gy = w.gy0, gz = w.gz0, dg = w.dg0;
            if (!L.zper && (k == 0 || k + 1 == L.nz)) {
                const bool one = L.nz == 1;
                gx = one ? w.gx2 : w.gx1;
                gy = one ? w.gy2 : w.gy1;
                gz = one ? w.gz2 : w.gz1;
                dg = one ? w.dg2 : w.dg1;
            }
            float v[4];
            for (int m = 0; m < 4; ++m) {
                const float S = gx * (x[m + 2] + x[m]) + gy * (yp[m] + ym[m]) + gz * (up[m] + dn[m]);
                v[m] = r[m] - dg * (cur[m] - S);
                mx.add(v[m]);
            }
            stv<4>(L.res + b, v);
            for (int m = 0; m < 4; ++m) {
                dn[m] = cur[m];
                cur[m] = up[m];
            }
        }
    }
    const double m = bred<1>(mx.get());
    if (threadIdx.x == 0 && parts) parts[blockIdx.x] = m;
}

// planes per thread: long columns on the large levels, short ones on the
// coarse levels so that they still fill the GPU
template <typename T>
inline int nd_chunk(const NDLevelT<T>& L) {
    const long long work = (long long)L.nx * L.ny * L.nz / 300000;
    return (int)(work < 2 ? 2 : (work > 16 ? 16 : work));
}
// whether a launch uses k_nd_xv<float, 4>: levels of more than 2^18 nodes
// (on smaller ones a quarter of the threads leaves the GPU short of warps),
// the row length a multiple of 4 and every array it touches 16-byte aligned
inline bool nd_vec_ok(const NDLevelT<float>& L, const void* a, const void* b) {
    auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
    return (long long)L.nx * L.ny * L.nz > (1LL << 18) && L.nx % 4 == 0 && al(L.rhs) && al(a) && al(b);
}
template <typename T>
inline long long nd_cols(const NDLevelT<T>& L, int kc) {
    return (long long)L.nx * L.ny * ((L.nz + kc - 1) / kc);
}

// Full weighting (1/4, 1/2, 1/4 in each direction) of the fine residual at a
// coarse node, summed by weight class per fine layer; the wrapped / mirrored
// fine indices are formed once (3 per direction) rather than per load.
template <typename T>
__global__ void k_nd_restrict(NDLevelT<T> F, NDLevelT<T> C) {
    const unsigned N = (unsigned)(C.nx * C.ny * C.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int i, j, k;
    split3(t, (unsigned)C.nx, (unsigned)C.ny, i, j, k);
    const int fi = 2 * i, fj = 2 * j, fk = 2 * k;
    const int xm = fi == 0 ? F.nx - 1 : fi - 1, xp = fi + 1 == F.nx ? 0 : fi + 1;
    const int sy = F.nx, sz = F.nx * F.ny;
    const int ym = (fj == 0 ? F.ny - 1 : fj - 1) * sy, y0 = fj * sy, yp = (fj + 1 == F.ny ? 0 : fj + 1) * sy;
    int zl[3];
    for (int c = -1; c <= 1; ++c) {
        int kk = fk + c;
        if (F.zper) kk = kk < 0 ? kk + F.nz : (kk >= F.nz ? kk - F.nz : kk);
        else kk = kk < 0 ? -kk : (kk >= F.nz ? 2 * (F.nz - 1) - kk : kk);
        zl[c + 1] = kk * sz;
    }
    const T* r = F.res;
    T lay[3];
    for (int c = 0; c < 3; ++c) {
        const T* q = r + zl[c];
        const T e = q[y0 + fi];
        const T ex = q[y0 + xm] + q[y0 + xp];
        const T ey = q[ym + fi] + q[yp + fi];
        const T cr = (q[ym + xm] + q[ym + xp]) + (q[yp + xm] + q[yp + xp]);
        // in-plane weights 1/4 e + 1/8 (ex + ey) + 1/16 cr
        lay[c] = T(0.25) * e + (T(0.125) * (ex + ey) + T(0.0625) * cr);
    }
    C.rhs[t] = T(0.5) * lay[1] + T(0.25) * (lay[0] + lay[2]);
    C.phi[t] = T(0);
}

// Trilinear prolongation added to the fine level, one thread per coarse node:
// it reads the 8 coarse nodes of the cube above it once and writes the up to 8
// fine nodes it spans (the midpoints take the mean of 2, 4 or 8 coarse
// values), with the pair sums shared.  A fine node of a wall-bounded z level
// above the last coarse layer does not exist.
template <typename T>
__global__ void k_nd_prolong(NDLevelT<T> F, NDLevelT<T> C) {
    const unsigned N = (unsigned)(C.nx * C.ny * C.nz);
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    int ci, cj, ck;
    split3(t, (unsigned)C.nx, (unsigned)C.ny, ci, cj, ck);
    const int cip = ci + 1 == C.nx ? 0 : ci + 1, cjp = cj + 1 == C.ny ? 0 : cj + 1;
    const bool up = C.zper || ck + 1 < C.nz;  // the fine layer 2 ck + 1 exists
    const int ckp = ck + 1 == C.nz ? 0 : ck + 1;
    const int csy = C.nx, csz = C.nx * C.ny;
    const T* c = C.phi;
    const T c000 = c[ck * csz + cj * csy + ci], c100 = c[ck * csz + cj * csy + cip];
    const T c010 = c[ck * csz + cjp * csy + ci], c110 = c[ck * csz + cjp * csy + cip];
    const T x00 = c000 + c100, x10 = c010 + c110, y00 = c000 + c010;
    const int fsy = F.nx, fsz = F.nx * F.ny;
    T* f = F.phi + (2 * ck) * fsz + (2 * cj) * fsy + 2 * ci;
    f[0] += c000;
    f[1] += T(0.5) * x00;
    f[fsy] += T(0.5) * y00;
    f[fsy + 1] += T(0.25) * (x00 + x10);
    if (!up) return;
    const T c001 = c[ckp * csz + cj * csy + ci], c101 = c[ckp * csz + cj * csy + cip];
    const T c011 = c[ckp * csz + cjp * csy + ci], c111 = c[ckp * csz + cjp * csy + cip];
    const T x01 = c001 + c101, x11 = c011 + c111;
    f[fsz] += T(0.5) * (c000 + c001);
    f[fsz + 1] += T(0.25) * (x00 + x01);
    f[fsz + fsy] += T(0.25) * (y00 + (c001 + c011));
    f[fsz + fsy + 1] += T(0.125) * ((x00 + x10) + (x01 + x11));
}

// Bottom solve: weighted-Jacobi sweeps by one CTA, staged in shared memory
// (phi, rhs and the sweep's output) for levels of up to BOTTOM_SMEM nodes
template <typename T, bool SMEM>
__global__ void k_nd_bottom(NDLevelT<T> L, T sigma, T omega, int sweeps) {
    const int N = L.nx * L.ny * L.nz;
    __shared__ T sp[SMEM ? BOTTOM_SMEM : 1], sr[SMEM ? BOTTOM_SMEM : 1], st[SMEM ? BOTTOM_SMEM : 1];
    T* p = L.phi;
    const T* r = L.rhs;
    T* q = L.tmp;
    if (SMEM) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            sp[t] = L.phi[t];
            sr[t] = L.rhs[t];
        }
        __syncthreads();
        p = sp;
        r = sr;
        q = st;
    }
    for (int s = 0; s < sweeps; ++s) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            split3((unsigned)t, (unsigned)L.nx, (unsigned)L.ny, i, j, k);
            q[t] = p[t] + omega * (r[t] - nd_ax(L, p, sigma, i, j, k)) * L.inv_diag;
        }
        __syncthreads();
        T* x = p;
        p = q;
        q = x;
    }
    // p holds the last sweep's output
    for (int t = threadIdx.x; t < N; t += blockDim.x) L.phi[t] = p[t];
}

// defect correction: phi64 += phi32
// First residual of a solve that starts from phi = 0: it is the right-hand
// side itself (rhs - A 0 = rhs exactly), so no stencil is evaluated.  With out
// (FP64 cycles) it also writes the first Jacobi sweep, omega rhs / diag (the
// sweep of the zero iterate: the value k_nd_col<double, 1> writes); with r32 /
// z32 (mixed precision) the FP32 cycle's right-hand side and zero start.
// Block maxima of |rhs| as the residual kernels return them.
__global__ void k_nd_zero_start(const double* rhs, long long n, double oinv, double* out, float* r32, float* z32, double* parts) {
    MaxAbs<double> mx;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double r = rhs[t];
        mx.add(r);
        if (out) out[t] = oinv * r;
        if (r32) {
            r32[t] = (float)r;
            z32[t] = 0.0f;
        }
    }
    const double m = bred<1>(mx.get());
    if (threadIdx.x == 0) parts[blockIdx.x] = m;
}

__global__ void k_add_f32(double* phi, const float* e, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    phi[t] += (double)e[t];
}

}  // namespace


template <typename T>
inline double ncc(const CCLevelT<T>& L) {
    return (double)L.nx * L.ny * L.nz;
}
template <typename T>
inline double nnd(const NDLevelT<T>& L) {
    return (double)L.nx * L.ny * L.nz;
}

// whether a launch uses the 4-cell FP32 kernels: as nd_vec_ok
inline bool cc_vec_ok(const CCLevelT<float>& L) {
    auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
    return (long long)L.nx * L.ny * L.nz > (1LL << 18) && L.nx % 4 == 0 && al(L.phi) && al(L.rhs) && al(L.res);
}

template <typename T>
void launch_cc_gsrb(Ctx& c, const CCLevelT<T>& L, double beta, int color) {
    (void)beta;
    if constexpr (sizeof(T) == 4) {
        if (cc_vec_ok(L)) {
            const int nq = L.nx / 4;
            const long long work = (long long)nq * L.ny * L.nz / 150000;
            const int kc = (int)(work < 1 ? 1 : (work > 8 ? 8 : work));
            const int bx = nq >= 128 ? 128 : 32 * ((nq + 31) / 32);
            const dim3 grid((unsigned)((nq + bx - 1) / bx), (unsigned)L.ny, (unsigned)((L.nz + kc - 1) / kc));
            KS_LAUNCH(c, k_cc_gsrb4, grid, bx, 4.0 * 2.0 * ncc(L), L, cc_coef(L), color, kc);
            return;
        }
    }
    // z chunk: long columns on the large levels, one layer on the small ones
    const long long work = (long long)(L.nx / 2) * L.ny * L.nz / 150000;
    const int kc = (int)(work < 1 ? 1 : (work > 16 ? 16 : work));
    const int hx = L.nx / 2, bx = hx >= 128 ? 128 : 32 * ((hx + 31) / 32);
    const dim3 grid((unsigned)((hx + bx - 1) / bx), (unsigned)L.ny, (unsigned)((L.nz + kc - 1) / kc));
    KS_LAUNCH(c, k_cc_gsrb<T>, grid, bx, sizeof(T) * 2.0 * ncc(L), L, cc_coef(L), color, kc);
}
template <typename T>
void launch_cc_resid(Ctx& c, const CCLevelT<T>& L, double beta, double* parts, int* np, int zero_color) {
    (void)beta;
    const int kc = cc_chunk(L);
    if constexpr (sizeof(T) == 4) {
        if (cc_vec_ok(L)) {
            const int n = parts_for((long long)(L.nx / 4) * L.ny * ((L.nz + kc - 1) / kc));
            if (np) *np = n;
            KS_LAUNCH(c, k_cc_resid4, n, BS, 4.0 * 3.0 * ncc(L), L, cc_coef(L), kc, parts);
            return;
        }
    }
    if (L.nx % 2) zero_color = -1;  // the pair form needs an even row
    const int n = parts_for((long long)(zero_color >= 0 ? L.nx / 2 : L.nx) * L.ny * ((L.nz + kc - 1) / kc));
    if (np) *np = n;
    KS_LAUNCH(c, k_cc_resid<T>, n, BS, sizeof(T) * 3.0 * ncc(L), L, cc_coef(L), kc, parts, (float*)nullptr, (float*)nullptr, zero_color);
}
void launch_cc_resid32(Ctx& c, const CCLevelT<double>& L, double beta, float* r32, float* z32, double* parts, int* np) {
    (void)beta;
    const int kc = cc_chunk(L);
    const int n = parts_for((long long)L.nx * L.ny * ((L.nz + kc - 1) / kc));
    *np = n;
    KS_LAUNCH(c, k_cc_resid<double>, n, BS, 8.0 * 2.0 * ncc(L) + 8.0 * ncc(L), L, cc_coef(L), kc, parts, r32, z32, -1);
}
void launch_nd_resid32(Ctx& c, const NDLevelT<double>& L, double sigma, float* r32, float* z32, double* parts, int* np) {
    const int kc = nd_chunk(L);
    const int n = parts_for(nd_cols(L, kc));
    *np = n;
    KS_LAUNCH(c, (k_nd_col<double, 2>), n, BS, 8.0 * 2.0 * nnd(L) + 8.0 * nnd(L), L, nd_coef(L, sigma, 0.0), (const double*)L.phi,
              (double*)nullptr, kc, parts, r32, z32);
}
// full coarsening (2 in every direction) or a semicoarsened pair, whose
// ratios the hierarchy's construction has checked to be 1 or 2 with F.n = r C.n
template <typename T>
inline bool cc_full_ratio(const CCLevelT<T>& F, const CCLevelT<T>& C) {
    return F.nx == 2 * C.nx && F.ny == 2 * C.ny && F.nz == 2 * C.nz;
}
template <typename T>
void launch_cc_restrict(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C) {
    if (cc_full_ratio(F, C)) {
        KS_LAUNCH(c, k_cc_restrict<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (ncc(F) + 2.0 * ncc(C)), F, C);
        return;
    }
    const int rx = F.nx / C.nx, ry = F.ny / C.ny, rz = F.nz / C.nz;
    KS_LAUNCH(c, k_cc_restrict_r<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (ncc(F) + 2.0 * ncc(C)), F, C, rx, ry,
              rz, T(1.0 / (rx * ry * rz)));
}
template <typename T>
void launch_cc_prolong(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C) {
    if (cc_full_ratio(F, C)) {
        KS_LAUNCH(c, k_cc_prolong<T>, nblocks((long long)F.nx * F.ny * F.nz, BS), BS, sizeof(T) * (2.0 * ncc(F) + ncc(C)), F, C);
        return;
    }
    KS_LAUNCH(c, k_cc_prolong_r<T>, nblocks((long long)F.nx * F.ny * F.nz, BS), BS, sizeof(T) * (2.0 * ncc(F) + ncc(C)), F, C,
              F.nx / C.nx, F.ny / C.ny, F.nz / C.nz);
}
template <typename T>
void launch_cc_bottom(Ctx& c, const CCLevelT<T>& L, double beta, int sweeps) {
    const int n = L.nx * L.ny * L.nz;
    if (L.binv) {
        KS_LAUNCH(c, k_bottom_direct<T>, (unsigned)((n + 7) / 8), 256, sizeof(T) * ((double)n * n + 2.0 * n), L.binv, n, (const T*)L.rhs,
                  L.phi, T(-1.0 / beta));
        return;
    }
    if (ncc(L) <= BOTTOM_SMEM) KS_LAUNCH(c, (k_cc_bottom<T, true>), 1, 256, sizeof(T) * 3.0 * ncc(L), L, T(beta), sweeps);
    else KS_LAUNCH(c, (k_cc_bottom<T, false>), 1, 256, sizeof(T) * 3.0 * ncc(L), L, T(beta), sweeps);
}
template <typename T>
void launch_nd_jacobi(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, const T* in, T* out) {
    const int kc = nd_chunk(L);
    const double bytes = sizeof(T) * 3.0 * nnd(L);
    if constexpr (sizeof(T) == 4) {
        if (nd_vec_ok(L, in, out))
            KS_LAUNCH(c, (k_nd_xv<float, 4, 0>), nblocks(nd_cols(L, kc) / 4, BS), BS, bytes, L, nd_coef(L, sigma, omega), in, out, kc,
                      nullptr);
        else
            KS_LAUNCH(c, k_nd_col2<0>, nblocks(nd_cols(L, kc), BS), BS, bytes, L, nd_coef(L, sigma, omega), in, out, kc, nullptr);
    } else {
        KS_LAUNCH(c, (k_nd_col<T, 0>), nblocks(nd_cols(L, kc), BS), BS, bytes, L, nd_coef(L, sigma, omega), in, out, kc, nullptr);
    }
}
template <typename T>
void launch_nd_resid(Ctx& c, const NDLevelT<T>& L, double sigma, double* parts, int* np) {
    const int kc = nd_chunk(L);
    const double bytes = sizeof(T) * 3.0 * nnd(L);
    if constexpr (sizeof(T) == 4) {
        if (nd_vec_ok(L, L.phi, L.res)) {
            const int n = parts_for(nd_cols(L, kc) / 4);
            if (np) *np = n;
            KS_LAUNCH(c, (k_nd_xv<float, 4, 2>), n, BS, bytes, L, nd_coef(L, sigma, 0.0), (const float*)L.phi, (float*)nullptr, kc, parts);
            return;
        }
    }
    const int n = parts_for(nd_cols(L, kc));
    if (np) *np = n;
    if constexpr (sizeof(T) == 4)
        KS_LAUNCH(c, k_nd_col2<2>, n, BS, bytes, L, nd_coef(L, sigma, 0.0), (const T*)L.phi, (T*)nullptr, kc, parts);
    else
        KS_LAUNCH(c, (k_nd_col<T, 2>), n, BS, bytes, L, nd_coef(L, sigma, 0.0), (const T*)L.phi, (T*)nullptr, kc, parts);
}
template <typename T>
void launch_nd_restrict(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C) {
    KS_LAUNCH(c, k_nd_restrict<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (nnd(F) + 2.0 * nnd(C)), F, C);
}
template <typename T>
void launch_nd_prolong(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C) {
    KS_LAUNCH(c, k_nd_prolong<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (2.0 * nnd(F) + nnd(C)), F, C);
}
template <typename T>
void launch_nd_bottom(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, int sweeps) {
    const int n = L.nx * L.ny * L.nz;
    if (L.binv) {
        KS_LAUNCH(c, k_bottom_direct<T>, (unsigned)((n + 7) / 8), 256, sizeof(T) * ((double)n * n + 2.0 * n), L.binv, n, (const T*)L.rhs,
                  L.phi, T(1.0 / sigma));
        return;
    }
    if (nnd(L) <= BOTTOM_SMEM) KS_LAUNCH(c, (k_nd_bottom<T, true>), 1, 256, sizeof(T) * 4.0 * nnd(L), L, T(sigma), T(omega), sweeps);
    else KS_LAUNCH(c, (k_nd_bottom<T, false>), 1, 256, sizeof(T) * 4.0 * nnd(L), L, T(sigma), T(omega), sweeps);
}
void launch_nd_jacobi_norm(Ctx& c, const NDLevelT<double>& L, double sigma, double omega, const double* in, double* out, double* parts,
                           int* np) {
    const int kc = nd_chunk(L);
    const int n = parts_for(nd_cols(L, kc));
    *np = n;
    KS_LAUNCH(c, (k_nd_col<double, 1>), n, BS, 8.0 * 3.0 * nnd(L), L, nd_coef(L, sigma, omega), in, out, kc, parts);
}
void launch_nd_zero_start(Ctx& c, const NDLevelT<double>& L, double sigma, double omega, double* out, float* r32, float* z32, double* parts,
                          int* np) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    *np = parts_for(n);
    KS_LAUNCH(c, k_nd_zero_start, *np, BS, 8.0 * n * (1 + (out ? 1 : 0)) + 8.0 * n * (r32 ? 1 : 0), L.rhs, n,
              (double)nd_coef(L, sigma, omega).oinv, out, r32, z32, parts);
}
void launch_add_f32(Ctx& c, double* phi, const float* e, long long n) {
    KS_LAUNCH(c, k_add_f32, nblocks(n, BS), BS, 20.0 * n, phi, e, n);
}

#define KS_INST(T)                                                                                           \
    template void launch_cc_gsrb<T>(Ctx&, const CCLevelT<T>&, double, int);                                  \
    template void launch_cc_resid<T>(Ctx&, const CCLevelT<T>&, double, double*, int*, int);                  \
    template void launch_cc_restrict<T>(Ctx&, const CCLevelT<T>&, const CCLevelT<T>&);                       \
    template void launch_cc_prolong<T>(Ctx&, const CCLevelT<T>&, const CCLevelT<T>&);                        \
    template void launch_cc_bottom<T>(Ctx&, const CCLevelT<T>&, double, int);                                \
    template void launch_nd_jacobi<T>(Ctx&, const NDLevelT<T>&, double, double, const T*, T*);               \
    template void launch_nd_resid<T>(Ctx&, const NDLevelT<T>&, double, double*, int*);                       \
    template void launch_nd_restrict<T>(Ctx&, const NDLevelT<T>&, const NDLevelT<T>&);                       \
    template void launch_nd_prolong<T>(Ctx&, const NDLevelT<T>&, const NDLevelT<T>&);                        \
    template void launch_nd_bottom<T>(Ctx&, const NDLevelT<T>&, double, double, int);
KS_INST(double)
KS_INST(float)
#undef KS_INST

}  // namespace ks
