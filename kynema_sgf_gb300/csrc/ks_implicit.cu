// Pointwise and transfer passes of the implicit / Crank-Nicolson tensor
// diffusion solve, rho u - dtd divtau(u) = rho u_rhs
// (DiffSolverIface::linsys_solve, src/equation_systems/DiffusionOps.cpp:114-159,
// MLTensorOp with alpha 1, a = rho, beta = dtd).  The sweeps and residuals run
// in the tiled tensor-diffusion kernel (launch_divtau_jacobi); this file holds
// the Jacobi diagonal and the cell-centred restriction and prolongation of the
// multigrid cycle.
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

// block maximum (NaN-propagating) written by thread 0 to out
__device__ inline void block_max_to(double v, double* out) {
    __shared__ double w[BS / 32];
    for (int o = 16; o > 0; o >>= 1) v = nmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = w[0];
        for (int k = 1; k < BS / 32; ++k) m = nmax(m, w[k]);
        *out = m;
    }
}

// Diagonal of rho - dtd divtau: the own component's normal-derivative
// coefficient is 4/3 along its own direction and 1 across, times the face
// viscosity (mean of the two cells, the cell value on a z wall).  On a z wall
// the normal component's face gradient is 2 q0 / dz (odd reflection) and the
// tangential components' is fixed (Neumann data), so they carry weight 2 and 0.
// Also the block maxima of s = 1 - rho / D (off-diagonal weight of a row: the
// Jacobi iteration contracts by about s per sweep).
__global__ void k_diff_dinv(Grid g, const double* mu, double rho, double dtd, double* dinv, double* parts) {
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t0 < g.N;
    const long long t = live ? t0 : 0;
    const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
    const int i = (int)(u - r * (unsigned)g.nx);
    const int k = (int)(r / (unsigned)g.ny), j = (int)(r - (unsigned)k * (unsigned)g.ny);
    const double c0 = mu[t];
    const double mx = 0.5 * (mu[cidx(g, wrapn(i - 1, g.nx), j, k)] + c0) + 0.5 * (mu[cidx(g, wrapn(i + 1, g.nx), j, k)] + c0);
    const double my = 0.5 * (mu[cidx(g, i, wrapn(j - 1, g.ny), k)] + c0) + 0.5 * (mu[cidx(g, i, wrapn(j + 1, g.ny), k)] + c0);
    const bool wlo = !g.zper && k == 0, whi = !g.zper && k == g.nz - 1;
    const double zlo = wlo ? c0 : 0.5 * (mu[cidx(g, i, j, g.zper ? wrapn(k - 1, g.nz) : k - 1)] + c0);
    const double zhi = whi ? c0 : 0.5 * (mu[cidx(g, i, j, g.zper ? wrapn(k + 1, g.nz) : k + 1)] + c0);
    const double ix2 = g.idx * g.idx, iy2 = g.idy * g.idy, iz2 = g.idz * g.idz;
    double smax = 0.0;
    for (int n = 0; n < 3 && live; ++n) {
        const double w = n == 2 ? 2.0 : 0.0;
        const double sz = (wlo ? w * zlo : zlo) + (whi ? w * zhi : zhi);
        const double s = (n == 0 ? 4.0 / 3.0 : 1.0) * mx * ix2 + (n == 1 ? 4.0 / 3.0 : 1.0) * my * iy2 + (n == 2 ? 4.0 / 3.0 : 1.0) * sz * iz2;
        const double d = 1.0 / (rho + dtd * s);
        dinv[n * g.N + t] = d;
        smax = nmax(smax, 1.0 - rho * d);
    }
    if (parts) block_max_to(smax, parts + blockIdx.x);
}

__global__ void k_avg8(Grid f, Grid c, const double* fv, double* cv, int ncomp) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= c.N) return;
    const int i = (int)(t % c.nx);
    const long long r = t / c.nx;
    const int j = (int)(r % c.ny), k = (int)(r / c.ny);
    for (int n = 0; n < ncomp; ++n) {
        const double* q = fv + n * f.N;
        double s = 0.0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) s += q[cidx(f, 2 * i + di, 2 * j + dj, 2 * k + dk)];
        cv[n * c.N + t] = 0.125 * s;
    }
}

__global__ void k_prolong_add(Grid f, Grid c, const double* cv, double* fv) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= f.N) return;
    const int i = (int)(t % f.nx);
    const long long r = t / f.nx;
    const int j = (int)(r % f.ny), k = (int)(r / f.ny);
    const long long p = cidx(c, i / 2, j / 2, k / 2);
    for (int n = 0; n < 3; ++n) fv[n * f.N + t] += cv[n * c.N + p];
}

// b = rho u (3 components) with the block maxima of |b|
__global__ void k_rhs_b(Grid g, const double* u, double rho, double* b, double* parts) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double m = 0.0;
    if (t < g.N)
        for (int n = 0; n < 3; ++n) {
            const double v = rho * u[n * g.N + t];
            b[n * g.N + t] = v;
            m = nmax(m, fabs(v));
        }
    block_max_to(m, parts + blockIdx.x);
}

}  // namespace

int diff_cell_blocks(const Grid& g) { return (int)nblocks(g.N, BS); }
void launch_diff_dinv(Ctx& c, const Grid& g, const double* mueff, double rho, double dtd, double* dinv, double* parts) {
    KS_LAUNCH(c, k_diff_dinv, nblocks(g.N, BS), BS, 8.0 * 4.0 * g.N, g, mueff, rho, dtd, dinv, parts);
}
void launch_avg8(Ctx& c, const Grid& fine, const Grid& coarse, const double* f, double* cr, int ncomp) {
    KS_LAUNCH(c, k_avg8, nblocks(coarse.N, BS), BS, 8.0 * ncomp * (fine.N + coarse.N), fine, coarse, f, cr, ncomp);
}
void launch_prolong_add(Ctx& c, const Grid& fine, const Grid& coarse, const double* cr, double* f) {
    KS_LAUNCH(c, k_prolong_add, nblocks(fine.N, BS), BS, 8.0 * 3.0 * (2.0 * fine.N + coarse.N), fine, coarse, cr, f);
}
void launch_rhs_b(Ctx& c, const Grid& g, const double* u, double rho, double* b, double* parts) {
    KS_LAUNCH(c, k_rhs_b, nblocks(g.N, BS), BS, 8.0 * 6.0 * g.N, g, u, rho, b, parts);
}

}  // namespace ks
