// Geometric multigrid kernels for the two Poisson problems of the step.
//
// MAC projection (cell-centred, 7-point, beta = 1/rho0): red-black
// Gauss-Seidel with the exact local solve at Neumann z walls, residual with a
// max-norm partial, 8-cell average restriction, piecewise-constant
// prolongation, single-CTA bottom sweeps.
//
// Nodal projection (node-centred, 27-point Q1 finite-element Laplacian times
// sigma = dt/rho0): weighted Jacobi, residual, full-weighting restriction
// (the transpose of trilinear prolongation over 8), trilinear prolongation,
// single-CTA bottom sweeps.  Wall-bounded z uses mirror images of the
// node values about the boundary node plane.
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

// ---------------------------------------------------------------- cell-centred
template <typename T>
__device__ inline long long ci3(const CCLevelT<T>& L, int i, int j, int k) { return ((long long)k * L.ny + j) * L.nx + i; }

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

template <typename T>
__global__ void k_cc_gsrb(CCLevelT<T> L, T beta, int color) {
    const long long half = (long long)L.nx * L.ny * L.nz / 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= half) return;
    const int hx = L.nx / 2;
    const int i2 = (int)(t % hx);
    const long long r = t / hx;
    const int j = (int)(r % L.ny), k = (int)(r / L.ny);
    const int i = 2 * i2 + ((j + k + color) & 1);
    const long long c = ci3(L, i, j, k);
    L.phi[c] = cc_gs_point(L, L.phi, i, j, k, L.rhs[c]);
    (void)beta;
}

template <typename T>
__global__ void k_cc_resid(CCLevelT<T> L, T beta, double* parts) {
    const long long N = (long long)L.nx * L.ny * L.nz;
    double mx = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % L.nx);
        const long long r = t / L.nx;
        const int j = (int)(r % L.ny), k = (int)(r / L.ny);
        int cls;
        const T S = cc_nsum(L, L.phi, i, j, k, cls);
        const T v = L.rhs[t] - L.dg[cls] * (L.phi[t] - S);
        L.res[t] = v;
        mx = nmax(mx, fabs((double)v));
    }
    mx = bred<1>(mx);
    if (threadIdx.x == 0 && parts) parts[blockIdx.x] = mx;
}

template <typename T>
__global__ void k_cc_restrict(CCLevelT<T> F, CCLevelT<T> C) {
    const long long N = (long long)C.nx * C.ny * C.nz;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % C.nx);
    const long long r = t / C.nx;
    const int j = (int)(r % C.ny), k = (int)(r / C.ny);
    T s = T(0);
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) s += F.res[ci3(F, 2 * i + a, 2 * j + b, 2 * k + c)];
    C.rhs[t] = T(0.125) * s;
    C.phi[t] = T(0);
}

template <typename T>
__global__ void k_cc_prolong(CCLevelT<T> F, CCLevelT<T> C) {
    const long long N = (long long)F.nx * F.ny * F.nz;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % F.nx);
    const long long r = t / F.nx;
    const int j = (int)(r % F.ny), k = (int)(r / F.ny);
    F.phi[t] += C.phi[ci3(C, i / 2, j / 2, k / 2)];
}

template <typename T>
__global__ void k_cc_bottom(CCLevelT<T> L, T beta, int sweeps) {
    const long long N = (long long)L.nx * L.ny * L.nz;
    for (int s = 0; s < sweeps; ++s)
        for (int color = 0; color < 2; ++color) {
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                const int i = (int)(t % L.nx);
                const long long r = t / L.nx;
                const int j = (int)(r % L.ny), k = (int)(r / L.ny);
                if (((i + j + k) & 1) != color) continue;
                L.phi[t] = cc_gs_point(L, L.phi, i, j, k, L.rhs[t]);
            }
            __syncthreads();
        }
}

// ---------------------------------------------------------------- nodal
template <typename T>
__device__ inline T nd_at(const NDLevelT<T>& L, const T* p, int i, int j, int k) {
    i = i < 0 ? i + L.nx : (i >= L.nx ? i - L.nx : i);
    j = j < 0 ? j + L.ny : (j >= L.ny ? j - L.ny : j);
    if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
    else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
    return p[((long long)k * L.ny + j) * L.nx + i];
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
    const long long sx = 1, sy = L.nx, sz = (long long)L.nx * L.ny;
    (void)sx;
    const long long rm = km * sz, r0 = k * sz, rp = kp * sz;
    const long long cm = jm * sy, c0 = j * sy, cp = jp * sy;
    auto at = [&](long long r, long long c, int x) { return p[r + c + x]; };
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

// Column (z-marching) form of the same stencil for the sweeps over a whole
// level: each thread walks k through a chunk of one (i, j) column.  Per node
// plane it forms the in-plane corner sum P, the x- and y-neighbour sums Ex, Ey
// and the centre value C once; node k combines planes k-1, k, k+1:
//   A phi = W13 C0 + W9 P0 + W3 (Ex- + Ex+) + W1 (Ey- + Ey+) + W0 (P- + P+)
//           [+ W12 Ex0 + W10 Ey0 + W4 (C- + C+) when face weights are non-zero],
// about half the FP64 operations of the node-by-node sums.
// MODE 0: out = in + omega (rhs - A in) / diag.  MODE 1: the same plus block
// maxima of |rhs - A in|.  MODE 2: res = rhs - A phi plus block maxima.
template <typename T, int MODE>
__global__ void k_nd_col(NDLevelT<T> L, T sigma, T omega, const T* in, T* out, int kc, double* parts) {
    const long long sz = (long long)L.nx * L.ny;
    const int nch = (L.nz + kc - 1) / kc;
    const long long M = sz * nch;
    double mx = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % L.nx);
        const long long r = t / L.nx;
        const int j = (int)(r % L.ny), ch = (int)(r / L.ny);
        const int im = i == 0 ? L.nx - 1 : i - 1, ip = i + 1 == L.nx ? 0 : i + 1;
        const long long cm = (long long)(j == 0 ? L.ny - 1 : j - 1) * L.nx, c0 = (long long)j * L.nx;
        const long long cp = (long long)(j + 1 == L.ny ? 0 : j + 1) * L.nx;
        auto plane = [&](int k, T& P, T& Ex, T& Ey, T& C) {
            if (L.zper) k = k < 0 ? k + L.nz : (k >= L.nz ? k - L.nz : k);
            else k = k < 0 ? -k : (k >= L.nz ? 2 * (L.nz - 1) - k : k);
            const T* q = in + (long long)k * sz;
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
            T s = L.W[13] * C0 + L.W[9] * P0 + L.W[3] * (Exm + Exp) + L.W[1] * (Eym + Eyp) + L.W[0] * (Pm + Pp);
            if (!L.faces_zero) s += L.W[12] * Ex0 + L.W[10] * Ey0 + L.W[4] * (Cm + Cp);
            const long long idx = (long long)k * sz + c0 + i;
            const T res = L.rhs[idx] - sigma * s;
            if (MODE == 2) L.res[idx] = res;
            else out[idx] = C0 + omega * res * L.inv_diag;
            if (MODE >= 1) mx = nmax(mx, fabs((double)res));
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
        mx = bred<1>(mx);
        if (threadIdx.x == 0 && parts) parts[blockIdx.x] = mx;
    }
}

// planes per thread: long columns on the large levels, short ones on the
// coarse levels so that they still fill the GPU
template <typename T>
inline int nd_chunk(const NDLevelT<T>& L) {
    const long long work = (long long)L.nx * L.ny * L.nz / 300000;
    return (int)(work < 2 ? 2 : (work > 16 ? 16 : work));
}
template <typename T>
inline long long nd_cols(const NDLevelT<T>& L, int kc) {
    return (long long)L.nx * L.ny * ((L.nz + kc - 1) / kc);
}

template <typename T>
__global__ void k_nd_restrict(NDLevelT<T> F, NDLevelT<T> C) {
    const long long N = (long long)C.nx * C.ny * C.nz;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % C.nx);
    const long long r = t / C.nx;
    const int j = (int)(r % C.ny), k = (int)(r / C.ny);
    const T w1[3] = {T(0.25), T(0.5), T(0.25)};
    T s = T(0);
    for (int c = -1; c <= 1; ++c)
        for (int b = -1; b <= 1; ++b)
            for (int a = -1; a <= 1; ++a) s += w1[a + 1] * w1[b + 1] * w1[c + 1] * nd_at(F, F.res, 2 * i + a, 2 * j + b, 2 * k + c);
    C.rhs[t] = s;
    C.phi[t] = T(0);
}

template <typename T>
__global__ void k_nd_prolong(NDLevelT<T> F, NDLevelT<T> C) {
    const long long N = (long long)F.nx * F.ny * F.nz;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % F.nx);
    const long long r = t / F.nx;
    const int j = (int)(r % F.ny), k = (int)(r / F.ny);
    const int ci = i >> 1, cj = j >> 1, ck = k >> 1, oi = i & 1, oj = j & 1, ok = k & 1;
    T s = T(0);
    for (int c = 0; c <= ok; ++c)
        for (int b = 0; b <= oj; ++b)
            for (int a = 0; a <= oi; ++a) s += nd_at(C, C.phi, ci + a, cj + b, ck + c);
    const int cnt = (1 + oi) * (1 + oj) * (1 + ok);
    F.phi[t] += (cnt == 1) ? s : (cnt == 2 ? T(0.5) * s : (cnt == 4 ? T(0.25) * s : T(0.125) * s));
}

template <typename T>
__global__ void k_nd_bottom(NDLevelT<T> L, T sigma, T omega, int sweeps) {
    const long long N = (long long)L.nx * L.ny * L.nz;
    for (int s = 0; s < sweeps; ++s) {
        for (long long t = threadIdx.x; t < N; t += blockDim.x) {
            const int i = (int)(t % L.nx);
            const long long r = t / L.nx;
            const int j = (int)(r % L.ny), k = (int)(r / L.ny);
            L.tmp[t] = L.phi[t] + omega * (L.rhs[t] - nd_ax(L, L.phi, sigma, i, j, k)) * L.inv_diag;
        }
        __syncthreads();
        for (long long t = threadIdx.x; t < N; t += blockDim.x) L.phi[t] = L.tmp[t];
        __syncthreads();
    }
}

// defect correction helpers: rhs32 = (float) r64, phi32 = 0 ; phi64 += phi32
__global__ void k_to_f32(const double* r, float* rhs, float* phi, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    rhs[t] = (float)r[t];
    phi[t] = 0.0f;
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

template <typename T>
void launch_cc_gsrb(Ctx& c, const CCLevelT<T>& L, double beta, int color) {
    KS_LAUNCH(c, k_cc_gsrb<T>, nblocks((long long)L.nx * L.ny * L.nz / 2, BS), BS, sizeof(T) * 2.0 * ncc(L), L, T(beta), color);
}
template <typename T>
void launch_cc_resid(Ctx& c, const CCLevelT<T>& L, double beta, double* parts, int* np) {
    const int n = parts_for((long long)L.nx * L.ny * L.nz);
    if (np) *np = n;
    KS_LAUNCH(c, k_cc_resid<T>, n, BS, sizeof(T) * 3.0 * ncc(L), L, T(beta), parts);
}
template <typename T>
void launch_cc_restrict(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C) {
    KS_LAUNCH(c, k_cc_restrict<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (ncc(F) + 2.0 * ncc(C)), F, C);
}
template <typename T>
void launch_cc_prolong(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C) {
    KS_LAUNCH(c, k_cc_prolong<T>, nblocks((long long)F.nx * F.ny * F.nz, BS), BS, sizeof(T) * (2.0 * ncc(F) + ncc(C)), F, C);
}
template <typename T>
void launch_cc_bottom(Ctx& c, const CCLevelT<T>& L, double beta, int sweeps) {
    KS_LAUNCH(c, k_cc_bottom<T>, 1, 256, sizeof(T) * 3.0 * ncc(L), L, T(beta), sweeps);
}
template <typename T>
void launch_nd_jacobi(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, const T* in, T* out) {
    const int kc = nd_chunk(L);
    KS_LAUNCH(c, (k_nd_col<T, 0>), nblocks(nd_cols(L, kc), BS), BS, sizeof(T) * 3.0 * nnd(L), L, T(sigma), T(omega), in, out, kc, nullptr);
}
template <typename T>
void launch_nd_resid(Ctx& c, const NDLevelT<T>& L, double sigma, double* parts, int* np) {
    const int kc = nd_chunk(L);
    const int n = parts_for(nd_cols(L, kc));
    if (np) *np = n;
    KS_LAUNCH(c, (k_nd_col<T, 2>), n, BS, sizeof(T) * 3.0 * nnd(L), L, T(sigma), T(0), (const T*)L.phi, (T*)nullptr, kc, parts);
}
template <typename T>
void launch_nd_restrict(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C) {
    KS_LAUNCH(c, k_nd_restrict<T>, nblocks((long long)C.nx * C.ny * C.nz, BS), BS, sizeof(T) * (nnd(F) + 2.0 * nnd(C)), F, C);
}
template <typename T>
void launch_nd_prolong(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C) {
    KS_LAUNCH(c, k_nd_prolong<T>, nblocks((long long)F.nx * F.ny * F.nz, BS), BS, sizeof(T) * (2.0 * nnd(F) + nnd(C)), F, C);
}
template <typename T>
void launch_nd_bottom(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, int sweeps) {
    KS_LAUNCH(c, k_nd_bottom<T>, 1, 256, sizeof(T) * 4.0 * nnd(L), L, T(sigma), T(omega), sweeps);
}
void launch_nd_jacobi_norm(Ctx& c, const NDLevelT<double>& L, double sigma, double omega, const double* in, double* out, double* parts,
                           int* np) {
    const int kc = nd_chunk(L);
    const int n = parts_for(nd_cols(L, kc));
    *np = n;
    KS_LAUNCH(c, (k_nd_col<double, 1>), n, BS, 8.0 * 3.0 * nnd(L), L, sigma, omega, in, out, kc, parts);
}
void launch_to_f32(Ctx& c, const double* r, float* rhs, float* phi, long long n) {
    KS_LAUNCH(c, k_to_f32, nblocks(n, BS), BS, 16.0 * n, r, rhs, phi, n);
}
void launch_add_f32(Ctx& c, double* phi, const float* e, long long n) {
    KS_LAUNCH(c, k_add_f32, nblocks(n, BS), BS, 20.0 * n, phi, e, n);
}

#define KS_INST(T)                                                                                           \
    template void launch_cc_gsrb<T>(Ctx&, const CCLevelT<T>&, double, int);                                  \
    template void launch_cc_resid<T>(Ctx&, const CCLevelT<T>&, double, double*, int*);                       \
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
