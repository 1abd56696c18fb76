// Pointwise and stencil passes of the advance: initial fields, Smagorinsky,
// momentum sources, wall model, tensor diffusion (+ RK2 correction), RHS
// assembly, projection updates, CFL / norm reductions and the actuator-disk
// sampling and Gaussian spreading.  One thread per output point; periodic
// wrap and wall boundary conditions are applied inside the kernels (no ghost
// cells are stored).
#include <cmath>

#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;
constexpr int MAXPARTS = 1216;  // 152 SMs x 8

// cell index -> (i, j, k) in 32-bit arithmetic (grids hold fewer than 2^31
// cells; a 64-bit division costs as much issue as tens of FP64 operations)
__device__ inline void cell_of(const Grid& g, long long t, int& i, int& j, int& k) {
    const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
    i = (int)(u - r * (unsigned)g.nx);
    k = (int)(r / (unsigned)g.ny);
    j = (int)(r - (unsigned)k * (unsigned)g.ny);
}

template <int OPMAX>
__device__ inline double block_reduce(double v) {
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

__device__ inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------- init
// TaylorGreenVortex::initialize_fields (src/physics/TaylorGreenVortex.cpp:22-54)
__global__ void k_init_tgv(Grid g, double* vel, double x0, double y0, double z0, double Lx, double Ly, double Lz) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const double tp = 6.283185307179586476925;
    const double x = x0 + (i + 0.5) * g.dx, y = y0 + (j + 0.5) * g.dy, z = z0 + (k + 0.5) * g.dz;
    vel[t] = sin(tp * x / Lx) * cos(tp * y / Ly) * cos(tp * z / Lz);
    vel[g.N + t] = -cos(tp * x / Lx) * sin(tp * y / Ly) * cos(tp * z / Lz);
    vel[2 * g.N + t] = 0.0;
}

// Synthetic ABL / free-stream start: log-law or uniform mean plus uniform
// noise of amplitude amp below zmax, SplitMix64 keyed on (seed, comp, k, j, i).
__global__ void k_init_abl(Grid g, double* vel, int loglaw, double U0, double U1, double U2, double ut_k, double z0, double amp,
                           double zmax_rel, unsigned long long seed) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const double z = (k + 0.5) * g.dz;
    const double U[3] = {U0, U1, U2};
    for (int n = 0; n < 3; ++n) {
        double val = U[n];
        if (loglaw) val = (n == 0) ? ut_k * log(z / z0) : 0.0;
        if (amp > 0.0 && z < zmax_rel) {
            const uint64_t idx = (uint64_t)n * (uint64_t)g.N + (uint64_t)t;
            const uint64_t r = splitmix64(seed * 0x100000001b3ULL ^ idx);
            const double u01 = (double)(r >> 11) * (1.0 / 9007199254740992.0);
            val += amp * (2.0 * u01 - 1.0);
        }
        vel[n * g.N + t] = val;
    }
}

__global__ void k_fill(double* p, double v, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}
__global__ void k_copy(double* d, const double* s, long long n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) d[t] = s[t];
}

// ---------------------------------------------------------------- Smagorinsky
// mu_eff = mu + rho Cs^2 Delta^2 |S| (src/turbulence/LES/Smagorinsky.cpp:22-62,
// strain rate src/fvm/strainrate.H:24-86, one-sided z stencils at walls
// src/fvm/stencils.H:166-330).
// alpha_eff = mu / Pr + mu_t / Pr_t (TurbModelBase.H:28-35) when alpha is set
// T is the arithmetic type: double, or float in the mixed-precision form (the
// strain rate of the FP64 velocity read once per cell and rounded; mu_eff is
// stored in FP64).
template <typename T>
__global__ void k_smag(Grid g, const double* vel, double* mueff, double mu, double rho, double fac, int smag, double* alpha, double mu_pr,
                       double iprt) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    if (!smag) {
        mueff[t] = mu;
        if (alpha) alpha[t] = mu_pr;
        return;
    }
    int i, j, k;
    cell_of(g, t, i, j, k);
    VelFPT<T, double> V{vel, g, T(1)};
    const T hx = T(0.5 * g.idx), hy = T(0.5 * g.idy);
    T gx[3], gy[3], gz[3];
    for (int n = 0; n < 3; ++n) {
        gx[n] = hx * (V(n, i + 1, j, k) - V(n, i - 1, j, k));
        gy[n] = hy * (V(n, i, j + 1, k) - V(n, i, j - 1, k));
    }
    if (!g.zper && (k == 0 || k == g.nz - 1)) {  // one-sided through the wall (ghost) value
        T a = T(1.0 / 3.0), b = T(1), c = T(-4.0 / 3.0);
        if (k == g.nz - 1) { a = T(4.0 / 3.0); b = T(-1); c = T(-1.0 / 3.0); }
        const T iz = T(g.idz);
        for (int n = 0; n < 3; ++n) gz[n] = (a * V(n, i, j, k + 1) + b * V(n, i, j, k) + c * V(n, i, j, k - 1)) * iz;
    } else {
        const T hz = T(0.5 * g.idz);
        for (int n = 0; n < 3; ++n) gz[n] = hz * (V(n, i, j, k + 1) - V(n, i, j, k - 1));
    }
    const T sxy = gy[0] + gx[1], syz = gz[1] + gy[2], szx = gx[2] + gz[0];
    const T s = sqrt(T(2) * (gx[0] * gx[0] + gy[1] * gy[1] + gz[2] * gz[2]) + (sxy * sxy + syz * syz + szx * szx));
    const double mut = (rho * fac) * (double)s;
    mueff[t] = mu + mut;
    if (alpha) alpha[t] = mu_pr + iprt * mut;
}

// Mixed-precision form: the same FP32 strain rate from a shared-memory tile of
// 32 x 4 x 4 cells whose one-cell halo (fill-patch ghosts included) is staged
// once, so each velocity value is loaded and rounded about 2.4 times per cell
// instead of the 18 reads of the thread-per-cell form.
constexpr int SMX = 32, SMY = 4, SMZ = 4;
constexpr int SMHX = SMX + 2, SMHY = SMY + 2, SMHZ = SMZ + 2, SMNH = SMHX * SMHY * SMHZ;
__global__ void __launch_bounds__(SMX* SMY* SMZ) k_smag_tile(Grid g, const double* vel, double* mueff, double mu, double rho, double fac,
                                                            double* alpha, double mu_pr, double iprt) {
    __shared__ float sV[3 * SMNH];
    const int i0 = blockIdx.x * SMX, j0 = blockIdx.y * SMY, k0 = blockIdx.z * SMZ;
    const int tid = threadIdx.x, nthr = SMX * SMY * SMZ;
    const VelFPT<float, double> V{vel, g, 1.0f};
    for (int h = tid; h < SMNH; h += nthr) {
        const int hx = h % SMHX, hy = (h / SMHX) % SMHY, hz = h / (SMHX * SMHY);
        // a tile may be wider than the grid: wrap x, y (and periodic z) fully
        const int gi = ((i0 + hx - 1) % g.nx + g.nx) % g.nx, gj = ((j0 + hy - 1) % g.ny + g.ny) % g.ny;
        int gk = k0 + hz - 1;
        if (g.zper) gk = (gk % g.nz + g.nz) % g.nz;
        for (int n = 0; n < 3; ++n) sV[n * SMNH + h] = V(n, gi, gj, gk);
    }
    __syncthreads();
    const int tx = tid % SMX, ty = (tid / SMX) % SMY, tz = tid / (SMX * SMY);
    const int i = i0 + tx, j = j0 + ty, k = k0 + tz;
    if (i >= g.nx || j >= g.ny || k >= g.nz) return;
    const int c = ((tz + 1) * SMHY + ty + 1) * SMHX + tx + 1;
    const float hx = float(0.5 * g.idx), hy = float(0.5 * g.idy);
    float gx[3], gy[3], gz[3];
    for (int n = 0; n < 3; ++n) {
        const float* v = sV + n * SMNH + c;
        gx[n] = hx * (v[1] - v[-1]);
        gy[n] = hy * (v[SMHX] - v[-SMHX]);
    }
    if (!g.zper && (k == 0 || k == g.nz - 1)) {  // one-sided through the wall (ghost) value
        float a = 1.0f / 3.0f, b = 1.0f, cc = -4.0f / 3.0f;
        if (k == g.nz - 1) { a = 4.0f / 3.0f; b = -1.0f; cc = -1.0f / 3.0f; }
        const float iz = float(g.idz);
        for (int n = 0; n < 3; ++n) {
            const float* v = sV + n * SMNH + c;
            gz[n] = (a * v[SMHX * SMHY] + b * v[0] + cc * v[-SMHX * SMHY]) * iz;
        }
    } else {
        const float hz = float(0.5 * g.idz);
        for (int n = 0; n < 3; ++n) {
            const float* v = sV + n * SMNH + c;
            gz[n] = hz * (v[SMHX * SMHY] - v[-SMHX * SMHY]);
        }
    }
    const float sxy = gy[0] + gx[1], syz = gz[1] + gy[2], szx = gx[2] + gz[0];
    const float s = sqrtf(2.0f * (gx[0] * gx[0] + gy[1] * gy[1] + gz[2] * gz[2]) + (sxy * sxy + syz * syz + szx * szx));
    const double mut = (rho * fac) * (double)s;
    const long long t = cidx(g, i, j, k);
    mueff[t] = mu + mut;
    if (alpha) alpha[t] = mu_pr + iprt * mut;
}

// ---------------------------------------------------------------- sources
// src = rho (-gp/rho + geostrophic + Coriolis(u_old) + body + actuator)
// (icns_ops.H:78-124, PDEOps.H:94-145, GeostrophicForcing.cpp:103-,
// CoriolisForcing.cpp:60-108, BodyForce.cpp:117-169, ActuatorForcing.cpp:19-29)
// The sources are affine in the Old velocity, so the launcher folds them on
// the host: src_n = (c_n - gp_n) + sum_m M_nm u_m + rho act_n + rho g_n beta (T0 - theta),
// with c = rho (geostrophic + body + ABLForcing) and M = rho x the Coriolis
// map.  About 12 FP64 instructions per cell where the term-by-term form took 45.
struct SrcCoef {
    double c[3];
    double M[3][3];
    double rho, bous_g[3], T_ref;
    int cor, act, bous;
};
__global__ void k_sources(Grid g, const double* vel, const double* gp, const double* act, double* src, SrcCoef s, const double* theta) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const long long N = g.N;
    double f[3];
    for (int n = 0; n < 3; ++n) f[n] = s.c[n] - gp[n * N + t];
    if (s.cor) {
        const double u0 = vel[t], u1 = vel[N + t], u2 = vel[2 * N + t];
        for (int n = 0; n < 3; ++n) f[n] += s.M[n][0] * u0 + s.M[n][1] * u1 + s.M[n][2] * u2;
    }
    if (s.act)
        for (int n = 0; n < 3; ++n) f[n] += s.rho * act[n * N + t];
    if (s.bous) {  // BoussinesqBuoyancy.cpp:22-50: rho g beta (T0 - theta)
        const double dT = s.T_ref - theta[t];
        for (int n = 0; n < 3; ++n) f[n] += s.bous_g[n] * dT;
    }
    for (int n = 0; n < 3; ++n) src[n * N + t] = f[n];
}

// ---------------------------------------------------------------- ABL wall
// plane sums over the first cell layer: u, v, |u_h|
__global__ void k_plane_sums(Grid g, const double* vel, double* parts, int np) {
    double su = 0, sv = 0, sm = 0;
    const long long M = (long long)g.nx * g.ny;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const double u = vel[t], v = vel[g.N + t];
        su += u; sv += v; sm += sqrt(u * u + v * v);
    }
    su = block_reduce<0>(su);
    sv = block_reduce<0>(sv);
    sm = block_reduce<0>(sm);
    if (threadIdx.x == 0) { parts[blockIdx.x] = su; parts[np + blockIdx.x] = sv; parts[2 * np + blockIdx.x] = sm; }
}

// wall-normal gradient of the tangential velocity at z-lo: tau rho / mu_eff
// (ABLWallFunction.cpp:236-347, ShearStress.H:22-167), Old velocity.
__global__ void k_wall_grad(Grid g, const double* vel, const double* mueff, double* wg, int type, double ut2, double um0, double um1,
                            double vm, double rho) {
    const long long M = (long long)g.nx * g.ny;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    const double u = vel[t], v = vel[g.N + t];
    const double ws = sqrt(u * u + v * v);
    double tx, ty;
    if (type == 0) {  // moeng
        tx = ((u - um0) * vm + ws * um0) / (vm * vm) * ut2;
        ty = ((v - um1) * vm + ws * um1) / (vm * vm) * ut2;
    } else if (type == 1) {  // constant
        tx = um0 / vm * ut2;
        ty = um1 / vm * ut2;
    } else if (type == 2) {  // local
        tx = u / fmax(ws, 1.0e-6) * ut2;
        ty = v / fmax(ws, 1.0e-6) * ut2;
    } else {  // schumann
        tx = u / vm * ut2;
        ty = v / vm * ut2;
    }
    const double m = mueff[t];
    wg[t] = tx * rho / m;
    wg[M + t] = ty * rho / m;
}

// ---------------------------------------------------------------- diffusion
// Velocity seen by the tensor operator: periodic wrap; across a z wall the
// normal component is odd-reflected (Dirichlet 0), the tangential ones are
// even-reflected (Neumann) or shifted so that the face gradient equals the
// wall-model gradient (inhomogeneous Neumann).
struct VelDiff {
    const double* v;
    const double* wg;
    Grid g;
    __device__ inline double operator()(int n, int i, int j, int k) const {
        i = wrapn(i, g.nx);
        j = wrapn(j, g.ny);
        const double* c = v + n * g.N;
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
};

// Flux of mu (grad u + grad u^T) - 2/3 mu div(u) I through the d-face at the
// low side of cell (i,j,k).
__device__ inline void tensor_flux(const Grid& g, const VelDiff& V, const double* mu, int d, int i, int j, int k, double F[3]) {
    int e[3] = {0, 0, 0};
    e[d] = 1;
    const int im = i - e[0], jm = j - e[1], km = k - e[2];
    // face viscosity
    double mf;
    const long long cc = cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), g.zper ? wrapn(k, g.nz) : (k < g.nz ? k : g.nz - 1));
    if (d == 2 && !g.zper && k == 0) mf = mu[cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), 0)];
    else if (d == 2 && !g.zper && k == g.nz) mf = mu[cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), g.nz - 1)];
    else {
        const long long cm = cidx(g, wrapn(im, g.nx), wrapn(jm, g.ny), g.zper ? wrapn(km, g.nz) : km);
        mf = 0.5 * (mu[cm] + mu[cc]);
    }
    const double ih[3] = {g.idx, g.idy, g.idz};
    double gr[3][3];  // gr[m][n] = d u_n / d x_m on the face
    for (int n = 0; n < 3; ++n) {
        for (int m = 0; m < 3; ++m) {
            if (m == d) {
                gr[m][n] = (V(n, i, j, k) - V(n, im, jm, km)) * ih[m];
            } else {
                int f[3] = {0, 0, 0};
                f[m] = 1;
                gr[m][n] = 0.25 *
                           (V(n, i + f[0], j + f[1], k + f[2]) + V(n, im + f[0], jm + f[1], km + f[2]) - V(n, i - f[0], j - f[1], k - f[2]) -
                            V(n, im - f[0], jm - f[1], km - f[2])) *
                           ih[m];
            }
        }
    }
    const double dv = gr[0][0] + gr[1][1] + gr[2][2];
    for (int n = 0; n < 3; ++n) {
        if (n == d) F[n] = mf * (2.0 * gr[d][d] - (2.0 / 3.0) * dv);
        else F[n] = mf * (gr[d][n] + gr[n][d]);
    }
}

// Tensor fluxes on the d-faces, all three components, computed once per face.
__global__ void k_tau_flux(Grid g, int d, const double* vel, const double* mueff, const double* wg, double* F0, double* F1, double* F2) {
    const int nzl = (d == 2) ? nzfaces(g) : g.nz;
    const long long M = (long long)g.nx * g.ny * nzl;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    VelDiff V{vel, wg, g};
    double F[3];
    tensor_flux(g, V, mueff, d, i, j, k, F);
    const long long f = fidx(g, d, i, j, k);
    F0[f] = F[0];
    F1[f] = F[1];
    F2[f] = F[2];
}

struct Flux9 {
    const double* p[9];
};

// divtau = sum_d (F_d(c + e_d) - F_d(c)) / h_d ; mode 0: store; mode 1: also
// forces = (src + divtau)/rho; mode 2: out = base + 0.5 dt (divtau - dold)/rho
__global__ void k_tau_div(Grid g, Flux9 F, double* out, int mode, const double* src, double* forces, const double* base,
                          const double* dold, double dt, double rho) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const double ih[3] = {g.idx, g.idy, g.idz};
    const double irho = 1.0 / rho;  // once per thread
    double acc[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) {
        const long long lo = fidx(g, d, i, j, k), hi = fidx(g, d, i + (d == 0), j + (d == 1), k + (d == 2));
        for (int n = 0; n < 3; ++n) acc[n] += (F.p[3 * d + n][hi] - F.p[3 * d + n][lo]) * ih[d];
    }
    const long long N = g.N;
    if (mode == 0) {
        for (int n = 0; n < 3; ++n) out[n * N + t] = acc[n];
    } else if (mode == 1) {
        for (int n = 0; n < 3; ++n) {
            out[n * N + t] = acc[n];
            forces[n * N + t] = (src[n * N + t] + acc[n]) * irho;
        }
    } else {
        for (int n = 0; n < 3; ++n) out[n * N + t] = base[n * N + t] + 0.5 * dt * (acc[n] - dold[n * N + t]) * irho;
    }
}

// ---- fused tiled form of k_tau_flux + k_tau_div.  A block owns a
// TX x TY x TZ tile of cells; it stages the velocity seen by the flux stencil
// (VelDiff, ghosts included) and mu_eff for the tile plus a one-cell halo in
// shared memory, computes every face flux the tile needs once (the same
// arithmetic as tensor_flux) into shared memory, then forms the divergence
// and the mode epilogue of k_tau_div for its cells.  No face arrays touch HBM.
constexpr int TTX = 32, TTY = 4, TTZ = 4;
constexpr int THX = TTX + 2, THY = TTY + 2, THZ = TTZ + 2;
constexpr int TNH = THX * THY * THZ;
constexpr int TNFX = (TTX + 1) * TTY * TTZ, TNFY = TTX * (TTY + 1) * TTZ, TNFZ = TTX * TTY * (TTZ + 1);
// dynamic shared memory of the tile kernel staging and computing in type T
template <typename T>
constexpr size_t tau_smem() { return sizeof(T) * (4 * (size_t)TNH + 3 * ((size_t)TNFX + TNFY + TNFZ)); }

// Epilogue of the tiled tensor-diffusion kernel (acc = divtau(vel) of a cell):
//   0: out = acc
//   1: out = acc, forces = (src + acc) / rho
//   2: out = base + 0.5 dt (acc - dold) / rho                        (explicit RK2 correction)
//   3: out = (rho base + dt (0.5 (conv_o + conv_n) + 0.5 (dold + acc) + src)) / rho  (MOL corrector_rhs)
//   7: out = x + omega dinv (base - rho x + dt acc), x = vel           (Jacobi sweep of rho x - dt divtau x = base)
//   8: out = base - rho x + dt acc                                    (its residual)
// Modes 7 and 8 write block maxima of the residual's magnitude to parts when it is set.
struct TauEpi {
    int mode;
    const double *src, *base, *dold, *conv_o, *conv_n, *dinv;
    double* forces;
    double* parts;
    double dt, rho, omega;
    double irho;  // 1 / rho, formed on the host
};

// T: type of the staged values, the face fluxes and their arithmetic (double;
// float for the mixed-precision form, modes 0-2 only).  The inputs are FP64
// and rounded once when staged; the epilogue runs in FP64.
template <typename T>
__global__ void __launch_bounds__(TTX* TTY* TTZ) k_divtau_tile(Grid g, const double* vel, const double* mueff, const double* wg, double* out,
                                                               TauEpi E) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T* sm = reinterpret_cast<T*>(sm_raw);
    T* sV = sm;                // [3][THZ][THY][THX]
    T* sM = sm + 3 * TNH;      // [THZ][THY][THX]
    T* sFx = sm + 4 * TNH;     // [3][TTZ][TTY][TTX + 1]
    T* sFy = sFx + 3 * TNFX;   // [3][TTZ][TTY + 1][TTX]
    T* sFz = sFy + 3 * TNFY;   // [3][TTZ + 1][TTY][TTX]
    const int i0 = blockIdx.x * TTX, j0 = blockIdx.y * TTY, k0 = blockIdx.z * TTZ;
    const int tid = threadIdx.x;
    const int nthr = TTX * TTY * TTZ;
    const VelDiff V{vel, wg, g};
    auto hidx = [](int hx, int hy, int hz) { return (hz * THY + hy) * THX + hx; };
    for (int h = tid; h < TNH; h += nthr) {
        const int hx = h % THX, hy = (h / THX) % THY, hz = h / (THX * THY);
        // a tile may be wider than the grid (nx < TTX): wrap x, y (and periodic z) fully
        const int gi = ((i0 + hx - 1) % g.nx + g.nx) % g.nx, gj = ((j0 + hy - 1) % g.ny + g.ny) % g.ny;
        int gk = k0 + hz - 1;
        if (g.zper) gk = (gk % g.nz + g.nz) % g.nz;
        for (int n = 0; n < 3; ++n) sV[n * TNH + h] = (T)V(n, gi, gj, gk);
        const int kk = g.zper ? gk : (gk < 0 ? 0 : (gk >= g.nz ? g.nz - 1 : gk));
        sM[h] = (T)mueff[cidx(g, gi, gj, kk)];
    }
    __syncthreads();
    const T ih[3] = {(T)g.idx, (T)g.idy, (T)g.idz};
    const T qh[3] = {T(0.25 * g.idx), T(0.25 * g.idy), T(0.25 * g.idz)};
    // flux through the d-face at the low side of halo cell (hx, hy, hz)
    auto flux = [&](int d, int hx, int hy, int hz, int gk, T F[3]) {
        const int e0 = (d == 0), e1 = (d == 1), e2 = (d == 2);
        const int mx = hx - e0, my = hy - e1, mz = hz - e2;
        T mf;
        if (d == 2 && !g.zper && gk == 0) mf = sM[hidx(hx, hy, hz)];
        else if (d == 2 && !g.zper && gk == g.nz) mf = sM[hidx(mx, my, mz)];
        else mf = T(0.5) * (sM[hidx(mx, my, mz)] + sM[hidx(hx, hy, hz)]);
        T gr[3][3];
        const int hc = hidx(hx, hy, hz), hm = hidx(mx, my, mz);
        for (int n = 0; n < 3; ++n) {
            const T* v = sV + n * TNH;
            for (int m = 0; m < 3; ++m) {
                if (m == d) {
                    gr[m][n] = (v[hc] - v[hm]) * ih[m];
                } else {  // mean of the two cells' central differences along m
                    const int f = m == 0 ? 1 : (m == 1 ? THX : THX * THY);
                    gr[m][n] = qh[m] * ((v[hc + f] + v[hm + f]) - (v[hc - f] + v[hm - f]));
                }
            }
        }
        const T dv = gr[0][0] + gr[1][1] + gr[2][2];
        for (int n = 0; n < 3; ++n) {
            if (n == d) F[n] = mf * (T(2) * gr[d][d] - T(2.0 / 3.0) * dv);
            else F[n] = mf * (gr[d][n] + gr[n][d]);
        }
    };
    for (int f = tid; f < TNFX + TNFY + TNFZ; f += nthr) {
        T F[3];
        if (f < TNFX) {
            const int fx = f % (TTX + 1), fy = (f / (TTX + 1)) % TTY, fz = f / ((TTX + 1) * TTY);
            flux(0, fx + 1, fy + 1, fz + 1, k0 + fz, F);
            for (int n = 0; n < 3; ++n) sFx[n * TNFX + f] = F[n];
        } else if (f < TNFX + TNFY) {
            const int q = f - TNFX;
            const int fx = q % TTX, fy = (q / TTX) % (TTY + 1), fz = q / (TTX * (TTY + 1));
            flux(1, fx + 1, fy + 1, fz + 1, k0 + fz, F);
            for (int n = 0; n < 3; ++n) sFy[n * TNFY + q] = F[n];
        } else {
            const int q = f - TNFX - TNFY;
            const int fx = q % TTX, fy = (q / TTX) % TTY, fz = q / (TTX * TTY);
            flux(2, fx + 1, fy + 1, fz + 1, k0 + fz, F);
            for (int n = 0; n < 3; ++n) sFz[n * TNFZ + q] = F[n];
        }
    }
    __syncthreads();
    const int tx = tid % TTX, ty = (tid / TTX) % TTY, tz = tid / (TTX * TTY);
    const int i = i0 + tx, j = j0 + ty, k = k0 + tz;
    const bool live = i < g.nx && j < g.ny && k < g.nz;
    const double rho = E.rho, dt = E.dt, irho = E.irho;
    const long long N = g.N, t = live ? cidx(g, i, j, k) : 0;
    double rmax = 0.0;
    for (int n = 0; n < 3 && live; ++n) {
        const int ax = (tz * TTY + ty) * (TTX + 1) + tx;
        const int ay = (tz * (TTY + 1) + ty) * TTX + tx;
        const int az = (tz * TTY + ty) * TTX + tx;
        T acc_t = (sFx[n * TNFX + ax + 1] - sFx[n * TNFX + ax]) * ih[0];
        acc_t += (sFy[n * TNFY + ay + TTX] - sFy[n * TNFY + ay]) * ih[1];
        acc_t += (sFz[n * TNFZ + az + TTX * TTY] - sFz[n * TNFZ + az]) * ih[2];
        const double acc = (double)acc_t;
        const long long m = n * N + t;
        if (E.mode == 0) {
            out[m] = acc;
        } else if (E.mode == 1) {
            out[m] = acc;
            E.forces[m] = (E.src[m] + acc) * irho;
        } else if (E.mode == 2) {
            out[m] = E.base[m] + 0.5 * dt * (acc - E.dold[m]) * irho;
        } else if (E.mode == 3) {
            out[m] = (rho * E.base[m] + dt * (0.5 * (E.conv_o[m] + E.conv_n[m]) + 0.5 * E.dold[m] + 0.5 * acc + E.src[m])) * irho;
        } else {
            const double x = (double)sV[n * TNH + hidx(tx + 1, ty + 1, tz + 1)];
            const double r = E.base[m] - rho * x + dt * acc;
            rmax = nmax(rmax, fabs(r));
            out[m] = E.mode == 7 ? x + E.omega * E.dinv[m] * r : r;
        }
    }
    if (!E.parts) return;  // uniform over the block
    for (int o = 16; o > 0; o >>= 1) rmax = nmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    __shared__ double wmax[TTX * TTY * TTZ / 32];
    if ((tid & 31) == 0) wmax[tid >> 5] = rmax;
    __syncthreads();
    if (tid == 0) {
        double b = 0.0;
        for (int w = 0; w < TTX * TTY * TTZ / 32; ++w) b = nmax(b, wmax[w]);
        E.parts[(blockIdx.z * (long long)gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = b;
    }
}

// predictor_rhs (src/equation_systems/CompRHSOps.H:32-141); fac = 1 explicit,
// 1/2 Crank-Nicolson, 0 implicit
__global__ void k_pred_rhs(long long N3, const double* vo, const double* conv, const double* src, const double* dt_, double* vel, double dt,
                           double rho, double irho, double fac) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N3) return;
    vel[t] = (rho * vo[t] + dt * (conv[t] + src[t] + fac * dt_[t])) * irho;
}

// ---------------------------------------------------------------- projection
__global__ void k_proj_pre(long long N3, double* vel, const double* vo, const double* gp, double sr, int add_gp, int sub_old) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= N3) return;
    double v = vel[t];
    if (add_gp) v += gp[t] * sr;  // sr = scaling / rho, formed on the host
    if (sub_old) v -= vo[t];
    vel[t] = v;
}

// Nodal divergence of the cell velocity at node t (the MLNodeLaplacian
// right-hand side).  The cell velocity is seen with periodic wrap and mirror
// images across z walls (normal component odd, tangential even; the sign flip
// is taken on the bits).  Each direction's four edge differences are summed
// before its one scale q = dx^-1 / 4.
__device__ inline double nodal_div_at(const Grid& g, const double* vel, unsigned t, int& k, double qx, double qy, double qz) {
    const unsigned r = t / (unsigned)g.nx;
    const int i = (int)(t - r * (unsigned)g.nx);
    k = (int)(r / (unsigned)g.ny);
    const int j = (int)(r - (unsigned)k * (unsigned)g.ny);
    const int im = i == 0 ? g.nx - 1 : i - 1, jm = j == 0 ? g.ny - 1 : j - 1;
    // cell layers k - 1 and k as seen from the node (mirrored at walls)
    int kk[2];
    bool flip[2];
    for (int c = 0; c < 2; ++c) {
        int q = k - c;
        flip[c] = false;
        if (g.zper) q = q < 0 ? q + g.nz : (q >= g.nz ? q - g.nz : q);
        else if (q < 0) { q = -1 - q; flip[c] = true; }
        else if (q >= g.nz) { q = 2 * g.nz - 1 - q; flip[c] = true; }
        kk[c] = q;
    }
    const long long N = g.N;
    // the 8 cells around the node: layers k-1 (c = 1) and k (c = 0), columns (i, j), (i-1, j), (i, j-1), (i-1, j-1)
    double u[2][4], v[2][4], w[2][4];
    for (int c = 0; c < 2; ++c) {
        const long long r0 = (long long)kk[c] * g.ny;
        const long long o[4] = {(r0 + j) * g.nx + i, (r0 + j) * g.nx + im, (r0 + jm) * g.nx + i, (r0 + jm) * g.nx + im};
        for (int q = 0; q < 4; ++q) {
            u[c][q] = vel[o[q]];
            v[c][q] = vel[N + o[q]];
            const double z = vel[2 * N + o[q]];
            w[c][q] = flip[c] ? bitsd(dbits(z) ^ ~kMag) : z;
        }
    }
    double dx = 0, dy = 0, dz = 0;
    for (int c = 0; c < 2; ++c) {
        dx += (u[c][0] - u[c][1]) + (u[c][2] - u[c][3]);
        dy += (v[c][0] - v[c][2]) + (v[c][1] - v[c][3]);
    }
    // z: differences of w between the layers k and k - 1 over the four cells
    dz = ((w[0][0] - w[1][0]) + (w[0][1] - w[1][1])) + ((w[0][2] - w[1][2]) + (w[0][3] - w[1][3]));
    return qx * dx + (qy * dy + qz * dz);
}

// Nodal divergence into the right-hand side, with weighted partial sums
// (boundary nodes carry half weight) for the solvability shift.  A thread
// walks a chunk of the node column (i, j); the four cells around the column
// in cell layer c (mirrored at walls as in nodal_div_at) give
//   X(c) = (u(i,j) - u(i-1,j)) + (u(i,j-1) - u(i-1,j-1)),
//   Y(c) = (v(i,j) - v(i,j-1)) + (v(i-1,j) - v(i-1,j-1))
// and their four w values, and node k combines layers k and k - 1 in
// nodal_div_at's order (the same result): each cell layer is loaded and
// differenced once for the two nodes it borders, 20 FP64 operations per node
// where nodal_div_at spends 28.
__global__ void k_nodal_rhs(Grid g, const double* vel, double* rhs, double* parts, int np, double qx, double qy, double qz, int kc) {
    const int nzn = g.zper ? g.nz : g.nz + 1;
    const int nch = (nzn + kc - 1) / kc;
    const unsigned M = (unsigned)(g.nx * g.ny * nch);
    const long long N = g.N;
    double ws = 0, wt = 0;
    struct Lay {
        double X, Y, w[4];
    };
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const unsigned r = t / (unsigned)g.nx;
        const int i = (int)(t - r * (unsigned)g.nx);
        const int ch = (int)(r / (unsigned)g.ny);
        const int j = (int)(r - (unsigned)ch * (unsigned)g.ny);
        const int im = i == 0 ? g.nx - 1 : i - 1, jm = j == 0 ? g.ny - 1 : j - 1;
        auto layer = [&](int q, Lay& L) {
            bool flip = false;
            if (g.zper) q = q < 0 ? q + g.nz : (q >= g.nz ? q - g.nz : q);
            else if (q < 0) { q = -1 - q; flip = true; }
            else if (q >= g.nz) { q = 2 * g.nz - 1 - q; flip = true; }
            const long long r0 = (long long)q * g.ny;
            const long long o[4] = {(r0 + j) * g.nx + i, (r0 + j) * g.nx + im, (r0 + jm) * g.nx + i, (r0 + jm) * g.nx + im};
            double u[4], v[4];
            for (int m = 0; m < 4; ++m) {
                u[m] = vel[o[m]];
                v[m] = vel[N + o[m]];
                const double z = vel[2 * N + o[m]];
                L.w[m] = flip ? bitsd(dbits(z) ^ ~kMag) : z;
            }
            L.X = (u[0] - u[1]) + (u[2] - u[3]);
            L.Y = (v[0] - v[2]) + (v[1] - v[3]);
        };
        const int k0 = ch * kc, k1 = min(k0 + kc, nzn);
        Lay lo, hi;  // cell layers k - 1 and k
        layer(k0 - 1, lo);
        for (int k = k0; k < k1; ++k) {
            layer(k, hi);
            const double dx = hi.X + lo.X, dy = hi.Y + lo.Y;
            const double dz = ((hi.w[0] - lo.w[0]) + (hi.w[1] - lo.w[1])) + ((hi.w[2] - lo.w[2]) + (hi.w[3] - lo.w[3]));
            const double dv = qx * dx + (qy * dy + qz * dz);
            rhs[((long long)k * g.ny + j) * g.nx + i] = dv;
            const double wgt = (!g.zper && (k == 0 || k == nzn - 1)) ? 0.5 : 1.0;
            ws += wgt * dv;
            wt += wgt;
            lo = hi;
        }
    }
    ws = block_reduce<0>(ws);
    wt = block_reduce<0>(wt);
    if (threadIdx.x == 0) { parts[blockIdx.x] = ws; parts[np + blockIdx.x] = wt; }
}

// Post-projection diagnostic: per-block max-norm of the nodal divergence of
// the velocity (the operator the projection drives to zero) and of |u|.
// Both maxima are kept as bits, so a NaN survives to the host.
__global__ void k_nodal_divmax(Grid g, const double* vel, double* parts, int np, double qx, double qy, double qz) {
    const int nzn = g.zper ? g.nz : g.nz + 1;
    const unsigned M = (unsigned)(g.nx * g.ny * nzn);
    const unsigned stride = gridDim.x * blockDim.x;
    long long md = 0, mu = 0;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += stride) {
        int k;
        md = imax_abs(md, nodal_div_at(g, vel, t, k, qx, qy, qz));
    }
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < (unsigned)(3 * g.N); t += stride) mu = imax_abs(mu, vel[t]);
    const double a = block_reduce<1>(bitsd(md)), b = block_reduce<1>(bitsd(mu));
    if (threadIdx.x == 0) { parts[blockIdx.x] = a; parts[np + blockIdx.x] = b; }
}

// u -= sigma G phi ; gp = (or +=) G phi ; optional add-back of u_old.  G is the
// cell gradient of the nodal phi (the mean of the four edge differences in
// each direction), formed from the cell's 8 corner nodes with shared pair sums;
// q = dx^-1 / 4 and sigma q are folded on the host.
__global__ void k_nodal_post_cells(Grid g, const double* phi, double* vel, const double* vo, double* gp, double qx, double qy, double qz,
                                   double sqx, double sqy, double sqz, int add_old, int incr) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const int ip = i + 1 == g.nx ? 0 : i + 1, jp = j + 1 == g.ny ? 0 : j + 1;
    const int kp = (g.zper && k + 1 == g.nz) ? 0 : k + 1;  // nodes 0..nz at walls
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long r0 = k * sz, r1 = kp * sz, c0 = j * sy, c1 = jp * sy;
    const double n000 = phi[r0 + c0 + i], n100 = phi[r0 + c0 + ip], n010 = phi[r0 + c1 + i], n110 = phi[r0 + c1 + ip];
    const double n001 = phi[r1 + c0 + i], n101 = phi[r1 + c0 + ip], n011 = phi[r1 + c1 + i], n111 = phi[r1 + c1 + ip];
    const double za = n000 + n001, zb = n100 + n101, zc = n010 + n011, zd = n110 + n111;
    const double gx = (zb + zd) - (za + zc), gy = (zc + zd) - (za + zb);
    const double gz = ((n001 + n101) + (n011 + n111)) - ((n000 + n100) + (n010 + n110));
    const double Gv[3] = {gx, gy, gz}, q[3] = {qx, qy, qz}, sq[3] = {sqx, sqy, sqz};
    const long long N = g.N;
    for (int n = 0; n < 3; ++n) {
        double v = vel[n * N + t] - sq[n] * Gv[n];
        if (add_old) v += vo[n * N + t];
        vel[n * N + t] = v;
        const double G = q[n] * Gv[n];
        if (incr) gp[n * N + t] += G;
        else gp[n * N + t] = G;
    }
}

__global__ void k_nodal_post_nodes(long long M, const double* phi, double* p, int incr) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    if (incr) p[t] += phi[t];
    else p[t] = phi[t];
}

// MAC divergence + partial sums
__global__ void k_mac_rhs(Grid g, const double* um, const double* vm, const double* wm, double* rhs, double* parts, int np) {
    double s = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const double r = (um[fidx(g, 0, i + 1, j, k)] - um[t]) * g.idx + (vm[fidx(g, 1, i, j + 1, k)] - vm[t]) * g.idy +
                         (wm[fidx(g, 2, i, j, k + 1)] - wm[fidx(g, 2, i, j, k)]) * g.idz;
        rhs[t] = r;
        s += r;
    }
    s = block_reduce<0>(s);
    if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// Post-projection diagnostic: per-block maxima of |div u_mac| (the MAC
// projection's exact discrete divergence) and of the face speeds, as bits.
__global__ void k_mac_divmax(Grid g, const double* um, const double* vm, const double* wm, double* parts, int np) {
    long long md = 0, mu = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(g, t, i, j, k);
        const double r = (um[fidx(g, 0, i + 1, j, k)] - um[t]) * g.idx + (vm[fidx(g, 1, i, j + 1, k)] - vm[t]) * g.idy +
                         (wm[fidx(g, 2, i, j, k + 1)] - wm[fidx(g, 2, i, j, k)]) * g.idz;
        md = imax_abs(md, r);
        mu = imax_abs(imax_abs(imax_abs(mu, um[t]), vm[t]), wm[fidx(g, 2, i, j, k)]);
    }
    const double a = block_reduce<1>(bitsd(md)), b = block_reduce<1>(bitsd(mu));
    if (threadIdx.x == 0) { parts[blockIdx.x] = a; parts[np + blockIdx.x] = b; }
}

__global__ void k_mac_correct(Grid g, const double* phi, double* um, double* vm, double* wm, double beta) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    int i, j, k;
    cell_of(g, t, i, j, k);
    const double p0 = phi[t];
    um[t] -= beta * (p0 - phi[cidx(g, wrapn(i - 1, g.nx), j, k)]) * g.idx;
    vm[t] -= beta * (p0 - phi[cidx(g, i, wrapn(j - 1, g.ny), k)]) * g.idy;
    if (g.zper) wm[t] -= beta * (p0 - phi[cidx(g, i, j, wrapn(k - 1, g.nz))]) * g.idz;
    else if (k > 0) wm[t] -= beta * (p0 - phi[cidx(g, i, j, k - 1)]) * g.idz;
}

// ---------------------------------------------------------------- reductions
__global__ void k_cfl(Grid g, const double* vel, const double* src, const double* mu, double rho, double* parts, int np) {
    // The maxima of |u_n|, |src_n| and mu are taken on the integer pipe and
    // scaled once per thread: rounding is monotone, so max(|u|) / dx equals
    // max(|u| / dx) exactly, and no FP64 instruction runs per cell.
    const double dxi[3] = {g.idx, g.idy, g.idz};
    const double irho = 1.0 / rho;
    const double dxinv2 = 2.0 * (dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2]);
    long long um[3] = {0, 0, 0}, sm[3] = {0, 0, 0}, mm = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x) {
        for (int n = 0; n < 3; ++n) {
            um[n] = imax_abs(um[n], vel[n * g.N + t]);
            sm[n] = imax_abs(sm[n], src[n * g.N + t]);
        }
        mm = imax_abs(mm, mu[t]);  // mu_eff >= 0
    }
    double c = 0, d = 0, f = 0;
    for (int n = 0; n < 3; ++n) {
        c = nmax(c, bitsd(um[n]) * dxi[n]);
        f = nmax(f, bitsd(sm[n]) * dxi[n] * irho);
    }
    d = bitsd(mm) * dxinv2 * irho;
    c = block_reduce<1>(c);
    d = block_reduce<1>(d);
    f = block_reduce<1>(f);
    if (threadIdx.x == 0) { parts[blockIdx.x] = c; parts[np + blockIdx.x] = d; parts[2 * np + blockIdx.x] = f; }
}

__global__ void k_ke(Grid g, const double* vel, double rho, double* parts) {
    double s = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.N; t += (long long)gridDim.x * blockDim.x)
        for (int n = 0; n < 3; ++n) {
            const double v = vel[n * g.N + t];
            s += 0.5 * rho * v * v;
        }
    s = block_reduce<0>(s);
    if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

__global__ void k_reduce(const double* parts, int np, int op_max, double* out) {
    const int comp = blockIdx.x;
    double v = op_max ? -1.0e300 : 0.0;
    for (int m = threadIdx.x; m < np; m += blockDim.x) {
        const double x = parts[comp * np + m];
        v = op_max ? nmax(v, x) : v + x;
    }
    v = op_max ? block_reduce<1>(v) : block_reduce<0>(v);
    if (threadIdx.x == 0) out[comp] = v;
}

// a -= s[0] / den (den > 0) or a -= s[0] / s[1]; with parts, block maxima of
// |a| after the shift.  Grid-stride, so the FP64 division is formed once per
// thread rather than once per element.
__global__ void k_sub_ratio(double* a, long long n, const double* s, double den, double* parts) {
    const double r = s[0] / (den > 0.0 ? den : s[1]);
    long long mb = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double v = a[t] - r;
        a[t] = v;
        mb = imax_abs(mb, v);
    }
    if (!parts) return;
    const double m = block_reduce<1>(bitsd(mb));
    if (threadIdx.x == 0) parts[blockIdx.x] = m;
}

// ---------------------------------------------------------------- actuator
// Trilinear sampling of the velocity at disk points
// (ActuatorContainer.cpp:284-360); ghosts follow the fill-patch rules.
__global__ void k_act_sample(Grid g, const double* vel, const double* pts, int npts, double x0, double y0, double z0, double* out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    VelFP V{vel, g, 1.0};
    const double fx = (pts[3 * p] - x0 - 0.5 * g.dx) / g.dx;
    const double fy = (pts[3 * p + 1] - y0 - 0.5 * g.dy) / g.dy;
    const double fz = (pts[3 * p + 2] - z0 - 0.5 * g.dz) / g.dz;
    const int i = (int)floor(fx), j = (int)floor(fy), k = (int)floor(fz);
    const double wx = fx - i, wy = fy - j, wz = fz - k;
    for (int n = 0; n < 3; ++n) {
        double s = 0;
        for (int c = 0; c < 2; ++c)
            for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                    const double w = (a ? wx : 1 - wx) * (b ? wy : 1 - wy) * (c ? wz : 1 - wz);
                    s += w * V(n, i + a, j + b, k + c);
                }
        out[3 * p + n] = s;
    }
}

// Gaussian spreading of ring-point forces (disk_spreading.H:45-105,
// actuator_utils.H:45-60) over the cells of the cut-off box of one disk.
__global__ void k_act_spread(Grid g, double* act, const double* pts, int npts, double ax0, double ax1, double ax2, double eps,
                             double x0, double y0, double z0, int lo0, int lo1, int lo2, int n0, int n1, int n2) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long M = (long long)n0 * n1 * n2;
    if (t >= M) return;
    const int a = (int)(t % n0);
    const long long r = t / n0;
    const int b = (int)(r % n1), c = (int)(r / n1);
    const int i = lo0 + a, j = lo1 + b, k = lo2 + c;
    if (k < 0 || k >= g.nz) return;
    // cell centre of the unwrapped index; stored at the wrapped cell
    const double x = x0 + (i + 0.5) * g.dx, y = y0 + (j + 0.5) * g.dy, z = z0 + (k + 0.5) * g.dz;
    const double gfac = 0.17958712212516656 / (eps * eps * eps);
    double s = 0;
    for (int m = 0; m < npts; ++m) {
        const double rx = (pts[4 * m] - x) / eps, ry = (pts[4 * m + 1] - y) / eps, rz = (pts[4 * m + 2] - z) / eps;
        const double r2 = rx * rx + ry * ry + rz * rz;
        if (r2 < 16.0) s += gfac * exp(-rx * rx - ry * ry - rz * rz) * pts[4 * m + 3];
    }
    if (s == 0.0) return;
    const long long cc = cidx(g, wrapn(i, g.nx), wrapn(j, g.ny), k);
    act[cc] += s * ax0;
    act[g.N + cc] += s * ax1;
    act[2 * g.N + cc] += s * ax2;
}

}  // namespace

// ---------------------------------------------------------------- launchers

constexpr double B8 = 8.0;  // bytes per FP64 value

void launch_init_tgv(Ctx& c, const Grid& g, double* vel, const double plo[3], const double L[3]) {
    KS_LAUNCH(c, k_init_tgv, nblocks(g.N, BS), BS, B8 * 3 * g.N, g, vel, plo[0], plo[1], plo[2], L[0], L[1], L[2]);
}
void launch_init_abl(Ctx& c, const Grid& g, double* vel, int loglaw, const double U[3], double ut_k, double z0, double amp,
                     double zmax_rel, unsigned long long seed) {
    KS_LAUNCH(c, k_init_abl, nblocks(g.N, BS), BS, B8 * 3 * g.N, g, vel, loglaw, U[0], U[1], U[2], ut_k, z0, amp, zmax_rel, seed);
}
void launch_fill(Ctx& c, double* p, double v, long long n) { KS_LAUNCH(c, k_fill, nblocks(n, BS), BS, B8 * n, p, v, n); }
void launch_copy(Ctx& c, double* d, const double* s, long long n) { KS_LAUNCH(c, k_copy, nblocks(n, BS), BS, B8 * 2 * n, d, s, n); }
void launch_smagorinsky(Ctx& c, const Grid& g, const double* vel, double* mueff, const Scalars& s, double* alpha, int fp32) {
    if (!s.temp) alpha = nullptr;
    const double bytes = B8 * ((s.smag ? 4 : 1) + (alpha ? 1 : 0)) * g.N;
    if (fp32 && s.smag) {
        const dim3 grid((g.nx + SMX - 1) / SMX, (g.ny + SMY - 1) / SMY, (g.nz + SMZ - 1) / SMZ);
        KS_LAUNCH(c, k_smag_tile, grid, SMX * SMY * SMZ, bytes, g, vel, mueff, s.mu, s.rho, s.smag_fac, alpha, s.mu_pr, s.iprt);
    } else if (fp32)
        KS_LAUNCH(c, k_smag<float>, nblocks(g.N, BS), BS, bytes, g, vel, mueff, s.mu, s.rho, s.smag_fac, s.smag, alpha, s.mu_pr, s.iprt);
    else
        KS_LAUNCH(c, k_smag<double>, nblocks(g.N, BS), BS, bytes, g, vel, mueff, s.mu, s.rho, s.smag_fac, s.smag, alpha, s.mu_pr, s.iprt);
}
// src = rho (-gp/rho + geostrophic + Coriolis(u_old) + body + actuator + Boussinesq + ABLForcing)
// (icns_ops.H:78-124, PDEOps.H:94-145, GeostrophicForcing.cpp:103-, CoriolisForcing.cpp:60-108,
// BodyForce.cpp:117-169, ActuatorForcing.cpp:19-29): the Coriolis acceleration
//   ae e + an n + au u,  ae = f (un sin - h uu cos), an = -f ue sin, au = h f ue cos
// (e, n, u the east / north / up unit vectors, ue = e.u etc., f = corfac, h = hfac) is the linear map
//   M = f sin (e n^T - n e^T) + f h cos (u e^T - e u^T).
void launch_sources(Ctx& c, const Grid& g, const double* vel_old, const double* gp, const double* act, double* src, const Scalars& s,
                    const double* theta) {
    SrcCoef k{};
    k.rho = s.rho;
    k.cor = s.cor;
    k.act = s.act;
    k.bous = s.bous;
    k.T_ref = s.T_ref;
    for (int n = 0; n < 3; ++n) {
        double a = 0.0;
        if (s.geo) a += (n == 2 ? s.hfac : 1.0) * s.gf[n];
        if (s.body) a += (s.body_osc ? std::cos(s.body_omega * s.t_nph) : 1.0) * s.body_force[n];
        if (s.ablf && n < 2) a += s.ablf_force[n];
        k.c[n] = s.rho * a;
        k.bous_g[n] = s.rho * s.grav[n] * s.beta_T;
        for (int m = 0; m < 3; ++m)
            k.M[n][m] = s.rho * s.corfac *
                        (s.sinphi * (s.east[n] * s.north[m] - s.north[n] * s.east[m]) + s.hfac * s.cosphi * (s.up[n] * s.east[m] - s.east[n] * s.up[m]));
    }
    KS_LAUNCH(c, k_sources, nblocks(g.N, BS), BS, B8 * (6 + 3 * s.cor + 3 * s.act + s.bous) * g.N, g, vel_old, gp, act, src, k, theta);
}
void launch_plane_sums(Ctx& c, const Grid& g, const double* vel, double* parts, int* np) {
    *np = parts_for((long long)g.nx * g.ny);
    KS_LAUNCH(c, k_plane_sums, *np, BS, B8 * 2 * g.nx * g.ny, g, vel, parts, *np);
}
void launch_wall_grad(Ctx& c, const Grid& g, const double* vel_old, const double* mueff, double* wg, int type, double ut2, double um0,
                      double um1, double vm, double rho) {
    KS_LAUNCH(c, k_wall_grad, nblocks((long long)g.nx * g.ny, BS), BS, B8 * 5 * g.nx * g.ny, g, vel_old, mueff, wg, type, ut2, um0,
              um1, vm, rho);
}
void launch_divtau_faces(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, int mode,
                         const double* src, double* forces, const double* base, const double* dold, double dt, double rho,
                         double* const fl[9]) {
    for (int d = 0; d < 3; ++d) {
        const long long M = (long long)g.nx * g.ny * (d == 2 ? nzfaces(g) : g.nz);
        KS_LAUNCH(c, k_tau_flux, nblocks(M, BS), BS, B8 * (4.0 * g.N + 3.0 * M), g, d, vel, mueff, wg, fl[3 * d], fl[3 * d + 1],
                  fl[3 * d + 2]);
    }
    Flux9 F;
    for (int m = 0; m < 9; ++m) F.p[m] = fl[m];
    const double per_cell = 9 + 3 + (mode == 1 ? 6 : 0) + (mode == 2 ? 6 : 0);
    KS_LAUNCH(c, k_tau_div, nblocks(g.N, BS), BS, B8 * per_cell * g.N, g, F, out, mode, src, forces, base, dold, dt, rho);
}

void launch_divtau(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, int mode,
                   const double* src, double* forces, const double* base, const double* dold, double dt, double rho, double* const fl[9],
                   int fp32) {
    (void)fl;  // the tiled kernel keeps its face fluxes in shared memory
    const dim3 grid((g.nx + TTX - 1) / TTX, (g.ny + TTY - 1) / TTY, (g.nz + TTZ - 1) / TTZ);
    const double per_cell = 4 + 3 + (mode == 1 ? 6 : 0) + (mode == 2 ? 6 : 0);
    TauEpi E{mode, src, base, dold, nullptr, nullptr, nullptr, forces, nullptr, dt, rho, 0.0, 1.0 / rho};
    if (fp32) {
        cudaFuncSetAttribute(k_divtau_tile<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tau_smem<float>());
        KS_LAUNCH_SMEM(c, k_divtau_tile<float>, grid, TTX * TTY * TTZ, tau_smem<float>(), B8 * per_cell * g.N, g, vel, mueff, wg, out, E);
    } else {
        cudaFuncSetAttribute(k_divtau_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tau_smem<double>());
        KS_LAUNCH_SMEM(c, k_divtau_tile<double>, grid, TTX * TTY * TTZ, tau_smem<double>(), B8 * per_cell * g.N, g, vel, mueff, wg, out, E);
    }
}
void launch_divtau_corrector(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, const double* vel_old,
                             const double* conv_old, const double* conv_new, const double* dold, const double* src, double dt, double rho) {
    cudaFuncSetAttribute(k_divtau_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tau_smem<double>());
    const dim3 grid((g.nx + TTX - 1) / TTX, (g.ny + TTY - 1) / TTY, (g.nz + TTZ - 1) / TTZ);
    TauEpi E{3, src, vel_old, dold, conv_old, conv_new, nullptr, nullptr, nullptr, dt, rho, 0.0, 1.0 / rho};
    KS_LAUNCH_SMEM(c, k_divtau_tile<double>, grid, TTX * TTY * TTZ, tau_smem<double>(), B8 * 22.0 * g.N, g, vel, mueff, wg, out, E);
}
int divtau_tile_blocks(const Grid& g) { return ((g.nx + TTX - 1) / TTX) * ((g.ny + TTY - 1) / TTY) * ((g.nz + TTZ - 1) / TTZ); }
void launch_divtau_jacobi(Ctx& c, const Grid& g, const double* x, const double* mueff, const double* wg, const double* b, const double* dinv,
                          double* out, double rho, double dtd, double omega, double* parts) {
    cudaFuncSetAttribute(k_divtau_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tau_smem<double>());
    const dim3 grid((g.nx + TTX - 1) / TTX, (g.ny + TTY - 1) / TTY, (g.nz + TTZ - 1) / TTZ);
    TauEpi E{omega > 0.0 ? 7 : 8, nullptr, b, nullptr, nullptr, nullptr, dinv, nullptr, parts, dtd, rho, omega, 1.0 / rho};
    KS_LAUNCH_SMEM(c, k_divtau_tile<double>, grid, TTX * TTY * TTZ, tau_smem<double>(), B8 * ((omega > 0.0 ? 13.0 : 10.0) * g.N), g, x, mueff, wg, out, E);
}
void launch_predictor_rhs(Ctx& c, const Grid& g, const double* vo, const double* conv, const double* src, const double* dtau, double* vel,
                          double dt, double rho, double fac) {
    KS_LAUNCH(c, k_pred_rhs, nblocks(3 * g.N, BS), BS, B8 * 15 * g.N, 3 * g.N, vo, conv, src, dtau, vel, dt, rho, 1.0 / rho, fac);
}
void launch_proj_pre(Ctx& c, const Grid& g, double* vel, const double* vo, const double* gp, double scaling, double rho, int add_gp,
                     int sub_old) {
    KS_LAUNCH(c, k_proj_pre, nblocks(3 * g.N, BS), BS, B8 * 3 * (2 + add_gp + sub_old) * g.N, 3 * g.N, vel, vo, gp, scaling / rho, add_gp, sub_old);
}
void launch_nodal_rhs(Ctx& c, const Grid& g, const double* vel, double* rhs, double* parts, int* np) {
    const int nzn = g.zper ? g.nz : g.nz + 1;
    const long long M = (long long)g.nx * g.ny * nzn;
    const long long work = M / 300000;  // node layers per thread: long columns on large grids
    const int kc = (int)(work < 2 ? 2 : (work > 16 ? 16 : work));
    *np = parts_for((long long)g.nx * g.ny * ((nzn + kc - 1) / kc));
    KS_LAUNCH(c, k_nodal_rhs, *np, BS, B8 * (3 * g.N + M), g, vel, rhs, parts, *np, 0.25 * g.idx, 0.25 * g.idy, 0.25 * g.idz, kc);
}
void launch_nodal_divmax(Ctx& c, const Grid& g, const double* vel, double* parts, int* np) {
    const long long M = (long long)g.nx * g.ny * (g.zper ? g.nz : g.nz + 1);
    *np = parts_for(M);
    KS_LAUNCH(c, k_nodal_divmax, *np, BS, B8 * 3 * g.N, g, vel, parts, *np, 0.25 * g.idx, 0.25 * g.idy, 0.25 * g.idz);
}
void launch_nodal_post(Ctx& c, const Grid& g, const double* phi, double* vel, const double* vo, double* gp, double* p, double sigma,
                       int add_old, int incr) {
    const long long M = (long long)g.nx * g.ny * (g.zper ? g.nz : g.nz + 1);
    const double qx = 0.25 * g.idx, qy = 0.25 * g.idy, qz = 0.25 * g.idz;
    KS_LAUNCH(c, k_nodal_post_cells, nblocks(g.N, BS), BS, B8 * (M + (9 + 3 * add_old + 3 * incr) * g.N), g, phi, vel, vo, gp, qx, qy, qz,
              sigma * qx, sigma * qy, sigma * qz, add_old, incr);
    KS_LAUNCH(c, k_nodal_post_nodes, nblocks(M, BS), BS, B8 * (2 + incr) * M, M, phi, p, incr);
}
void launch_mac_rhs(Ctx& c, const Grid& g, const double* um, const double* vm, const double* wm, double* rhs, double* parts, int* np) {
    *np = parts_for(g.N);
    KS_LAUNCH(c, k_mac_rhs, *np, BS, B8 * (3 * g.N + g.NFz), g, um, vm, wm, rhs, parts, *np);
}
void launch_mac_divmax(Ctx& c, const Grid& g, const double* um, const double* vm, const double* wm, double* parts, int* np) {
    *np = parts_for(g.N);
    KS_LAUNCH(c, k_mac_divmax, *np, BS, B8 * (2 * g.N + g.NFz), g, um, vm, wm, parts, *np);
}
void launch_mac_correct(Ctx& c, const Grid& g, const double* phi, double* um, double* vm, double* wm, double beta) {
    KS_LAUNCH(c, k_mac_correct, nblocks(g.N, BS), BS, B8 * 7 * g.N, g, phi, um, vm, wm, beta);
}
void launch_cfl(Ctx& c, const Grid& g, const double* vel, const double* src, const double* mu, double rho, double* parts, int* np) {
    *np = parts_for(g.N);
    KS_LAUNCH(c, k_cfl, *np, BS, B8 * 7 * g.N, g, vel, src, mu, rho, parts, *np);
}
void launch_ke(Ctx& c, const Grid& g, const double* vel, double rho, double* parts, int* np) {
    *np = parts_for(g.N);
    KS_LAUNCH(c, k_ke, *np, BS, B8 * 3 * g.N, g, vel, rho, parts);
}
void launch_reduce(Ctx& c, const double* parts, int np, int ncomp, int op_max, double* out) {
    KS_LAUNCH(c, k_reduce, ncomp, 256, B8 * (np + 1) * ncomp, parts, np, op_max, out);
}
void launch_sub_ratio(Ctx& c, double* a, long long n, const double* s, double den, double* parts, int* np) {
    const int nb = parts_for(n);
    if (np) *np = nb;
    KS_LAUNCH(c, k_sub_ratio, nb, BS, B8 * 2 * n, a, n, s, den, parts);
}
void launch_act_sample(Ctx& c, const Grid& g, const double* vel, const double* pts, int npts, const double plo[3], double* out) {
    KS_LAUNCH(c, k_act_sample, nblocks(npts, 64), 64, B8 * 6 * npts, g, vel, pts, npts, plo[0], plo[1], plo[2], out);
}
void launch_act_spread(Ctx& c, const Grid& g, double* act, const double* pts, int npts, const double ax[3], double eps, const double plo[3],
                       const int lo[3], const int hi[3]) {
    const int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
    if (n0 <= 0 || n1 <= 0 || n2 <= 0) return;
    const long long M = (long long)n0 * n1 * n2;
    KS_LAUNCH(c, k_act_spread, nblocks(M, BS), BS, B8 * 6 * M, g, act, pts, npts, ax[0], ax[1], ax[2], eps, plo[0], plo[1], plo[2], lo[0],
              lo[1], lo[2], n0, n1, n2);
}

}  // namespace ks
