// Temperature transport of the ABL physics (the Temperature PDE registered by
// src/wind_energy/ABL.cpp:27-28): initial fields (ABLFieldInit.cpp:215-372),
// layer averages (FieldPlaneAveraging.cpp:191-260) for the wall model and
// ABLForcing, the wall heat flux (ABLWallFunction.cpp:392-480), and the scalar
// diffusion operator of MLABecLaplacian (alpha 0, beta -1 for the apply;
// alpha 1, a = rho, beta = dt_diff for the solve, DiffusionOps.cpp:114-159)
// with its boundary data (incflo_diffusion.cpp:71-104).  The Godunov fluxes
// of rho theta are the scalar instantiation in ks_godunov.cu.
#include "ks_launch.hpp"

namespace ks {

namespace {

constexpr int BS = 256;

__device__ inline void block_max(double v, double* out) {
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

__global__ void k_init_abl_ref(Grid g, double* vel, double x0, double y0, double z0, double U0, double U1, double U2, int pert, double aval,
                               double bval, double ufac, double vfac, double refh, double ibh) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    double u = U0, v = U1;
    if (pert) {
        const double x = x0 + (i + 0.5) * g.dx, y = y0 + (j + 0.5) * g.dy;
        const double z = fmax(z0 + (k + 0.5) * g.dz - ibh, 0.0);
        const double zl = z / refh, damp = exp(-0.5 * zl * zl);
        u += ufac * damp * z * cos(aval * (y - y0));
        v += vfac * damp * z * cos(bval * (x - x0));
    }
    vel[t] = u;
    vel[g.N + t] = v;
    vel[2 * g.N + t] = U2;
}

// tv[0] outside the segments, linear inside (z in (h_m, h_m+1])
__global__ void k_theta_profile(Grid g, double* theta, double zlo, const double* h, const double* v, int n) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= g.N) return;
    const int k = (int)(t / ((long long)g.nx * g.ny));
    const double z = zlo + (k + 0.5) * g.dz;
    double th = v[0];
    for (int m = 0; m + 1 < n; ++m)
        if (z > h[m] && z <= h[m + 1]) th = v[m] + (z - h[m]) * ((v[m + 1] - v[m]) / (h[m + 1] - h[m]));
    theta[t] = 0.0 + th;
}

__global__ void k_layer_sums(Grid g, const double* f, double* out) {
    const int k = blockIdx.x;
    const long long M = (long long)g.nx * g.ny;
    const double* p = f + (long long)k * M;
    double s = 0.0;
    for (long long m = threadIdx.x; m < M; m += blockDim.x) s += p[m];
    __shared__ double w[BS / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < BS / 32; ++q) a += w[q];
        out[k] = a;
    }
}

// ShearStress.H heat fluxes with the surface temperature equal to theta_mean
// (neutral, surface_temp_flux = 0): Moeng (type 0), constant (1), local /
// Schumann (2, 3); gradient = rho q / alpha_eff of the first cell
__global__ void k_theta_wall_grad(Grid g, const double* vel, const double* theta, const double* alpha, double* gz, int type, double utau,
                                  double kappa, double phi_h, double vm, double tm, double rho) {
    const long long M = (long long)g.nx * g.ny;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M) return;
    const double u = vel[t], v = vel[g.N + t];
    const double wspd = sqrt(u * u + v * v);
    const double th = theta[t], ts = tm;
    double q;
    if (type == 0) {
        const double term1 = utau * kappa / (vm * phi_h);
        q = term1 * ((th - tm) * vm + (tm - ts) * wspd);
    } else if (type == 1) {
        q = utau * kappa / phi_h * (tm - ts);
    } else {
        q = utau * kappa / phi_h * (th - ts);
    }
    gz[t] = rho * q / alpha[t];
}

struct TdiffArgs {
    ScalarBC bc;
    int mode;
    const double *base, *dold, *b, *dinv;
    double* parts;
    double dt, rho, omega;
};

// face diffusivity: mean of the two cells, the cell value on a z wall
__global__ void k_tdiff(Grid g, const double* th, const double* al, double* out, TdiffArgs A) {
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t0 < g.N;
    const long long t = live ? t0 : 0;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const double q0 = th[t], a0 = al[t];
    const long long xm = cidx(g, wrapn(i - 1, g.nx), j, k), xp = cidx(g, wrapn(i + 1, g.nx), j, k);
    const long long ym = cidx(g, i, wrapn(j - 1, g.ny), k), yp = cidx(g, i, wrapn(j + 1, g.ny), k);
    const double fxl = 0.5 * (al[xm] + a0) * (q0 - th[xm]) * g.idx, fxh = 0.5 * (a0 + al[xp]) * (th[xp] - q0) * g.idx;
    const double fyl = 0.5 * (al[ym] + a0) * (q0 - th[ym]) * g.idy, fyh = 0.5 * (a0 + al[yp]) * (th[yp] - q0) * g.idy;
    double fzl, fzh;
    if (g.zper) {
        const long long zm = cidx(g, i, j, wrapn(k - 1, g.nz)), zp = cidx(g, i, j, wrapn(k + 1, g.nz));
        fzl = 0.5 * (al[zm] + a0) * (q0 - th[zm]) * g.idz;
        fzh = 0.5 * (a0 + al[zp]) * (th[zp] - q0) * g.idz;
    } else {
        if (k == 0) {
            const double gw = A.bc.zlo == 1 ? A.bc.gz[(long long)j * g.nx + i] : 0.0;
            const double ghost = q0 - gw * g.dz;
            fzl = a0 * (q0 - ghost) * g.idz;
        } else {
            const long long zm = cidx(g, i, j, k - 1);
            fzl = 0.5 * (al[zm] + a0) * (q0 - th[zm]) * g.idz;
        }
        if (k == g.nz - 1) {
            const double ghost = q0 + (A.bc.zhi == 2 ? A.bc.gtop : 0.0) * g.dz;
            fzh = a0 * (ghost - q0) * g.idz;
        } else {
            const long long zp = cidx(g, i, j, k + 1);
            fzh = 0.5 * (a0 + al[zp]) * (th[zp] - q0) * g.idz;
        }
    }
    const double acc = (fxh - fxl) * g.idx + (fyh - fyl) * g.idy + (fzh - fzl) * g.idz;
    double rmax = 0.0;
    if (live) {
        if (A.mode == 0) {
            out[t] = acc;
        } else if (A.mode == 2) {
            out[t] = A.base[t] + 0.5 * A.dt * (acc - A.dold[t]) / A.rho;
        } else {
            const double res = A.b[t] - A.rho * q0 + A.dt * acc;
            rmax = fabs(res);
            out[t] = A.mode == 7 ? q0 + A.omega * A.dinv[t] * res : res;
        }
    }
    if (A.parts) block_max(rmax, A.parts + blockIdx.x);
}

__global__ void k_tdiff_dinv(Grid g, const double* al, double rho, double dtd, double* dinv, double* parts) {
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t0 < g.N;
    const long long t = live ? t0 : 0;
    const int i = (int)(t % g.nx);
    const long long r = t / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const double a0 = al[t];
    double s = (0.5 * (al[cidx(g, wrapn(i - 1, g.nx), j, k)] + a0) + 0.5 * (al[cidx(g, wrapn(i + 1, g.nx), j, k)] + a0)) * g.idx * g.idx +
               (0.5 * (al[cidx(g, i, wrapn(j - 1, g.ny), k)] + a0) + 0.5 * (al[cidx(g, i, wrapn(j + 1, g.ny), k)] + a0)) * g.idy * g.idy;
    double zl, zh;
    if (g.zper) {
        zl = 0.5 * (al[cidx(g, i, j, wrapn(k - 1, g.nz))] + a0);
        zh = 0.5 * (al[cidx(g, i, j, wrapn(k + 1, g.nz))] + a0);
    } else {  // the wall faces' gradients are boundary data: no diagonal weight
        zl = k == 0 ? 0.0 : 0.5 * (al[cidx(g, i, j, k - 1)] + a0);
        zh = k == g.nz - 1 ? 0.0 : 0.5 * (al[cidx(g, i, j, k + 1)] + a0);
    }
    s += (zl + zh) * g.idz * g.idz;
    const double d = 1.0 / (rho + dtd * s);
    if (live) dinv[t] = d;
    if (parts) block_max(live ? 1.0 - rho * d : 0.0, parts + blockIdx.x);
}

__global__ void k_scalar_rhs(Grid g, const double* th, double rho, double* b, double* parts) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double m = 0.0;
    if (t < g.N) {
        b[t] = rho * th[t];
        m = fabs(b[t]);
    }
    block_max(m, parts + blockIdx.x);
}

// predictor_rhs of a scalar without sources: (rho s_old + dt (conv + 0 + fac dold)) / rho
__global__ void k_scalar_pred(long long n, const double* so, const double* conv, const double* dold, double* out, double dt, double rho,
                              double fac, double irho) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) out[t] = (rho * so[t] + dt * (conv[t] + 0.0 + fac * dold[t])) * irho;
}

__global__ void k_scalar_corr(long long n, const double* so, const double* co, const double* cn, const double* dold, const double* dnew,
                              double* out, double dt, double rho, double ofac, double nfac, double irho) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double dn = dnew ? nfac * dnew[t] : 0.0;
    out[t] = (rho * so[t] + dt * (0.5 * (co[t] + cn[t]) + ofac * dold[t] + dn + 0.0)) * irho;
}

__global__ void k_lincomb(long long n, double a, const double* x, double b, const double* y, double* out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) out[t] = a * x[t] + b * y[t];
}

}  // namespace

void launch_init_abl_ref(Ctx& c, const Grid& g, double* vel, const double plo[3], const double U[3], int pert, double aval, double bval,
                         double ufac, double vfac, double ref_height, double ib_height) {
    KS_LAUNCH(c, k_init_abl_ref, nblocks(g.N, BS), BS, 8.0 * 3 * g.N, g, vel, plo[0], plo[1], plo[2], U[0], U[1], U[2], pert, aval, bval, ufac,
              vfac, ref_height, ib_height);
}
void launch_theta_profile(Ctx& c, const Grid& g, double* theta, double zlo, const double* heights, const double* values, int n) {
    KS_LAUNCH(c, k_theta_profile, nblocks(g.N, BS), BS, 8.0 * g.N, g, theta, zlo, heights, values, n);
}
void launch_layer_sums(Ctx& c, const Grid& g, const double* f, double* out) {
    KS_LAUNCH(c, k_layer_sums, g.nz, BS, 8.0 * (g.N + g.nz), g, f, out);
}
void launch_theta_wall_grad(Ctx& c, const Grid& g, const double* vel_old, const double* theta_old, const double* alpha, double* gz, int type,
                            double utau, double kappa, double phi_h, double vmag_mean, double theta_mean, double rho) {
    const long long M = (long long)g.nx * g.ny;
    KS_LAUNCH(c, k_theta_wall_grad, nblocks(M, BS), BS, 8.0 * 5.0 * M, g, vel_old, theta_old, alpha, gz, type, utau, kappa, phi_h, vmag_mean,
              theta_mean, rho);
}
int tdiff_blocks(const Grid& g) { return (int)nblocks(g.N, BS); }
void launch_tdiff(Ctx& c, const Grid& g, const double* th, const double* alpha, const ScalarBC& bc, double* out, int mode, const double* base,
                  const double* dold, const double* b, const double* dinv, double* parts, double dt, double rho, double omega) {
    TdiffArgs A{bc, mode, base, dold, b, dinv, parts, dt, rho, omega};
    const double per = 3.0 + (mode == 2 ? 2.0 : 0.0) + (mode >= 7 ? 1.0 + (mode == 7 ? 1.0 : 0.0) : 0.0);
    KS_LAUNCH(c, k_tdiff, nblocks(g.N, BS), BS, 8.0 * per * g.N, g, th, alpha, out, A);
}
void launch_tdiff_dinv(Ctx& c, const Grid& g, const double* alpha, const ScalarBC& bc, double rho, double dtd, double* dinv, double* parts) {
    (void)bc;
    KS_LAUNCH(c, k_tdiff_dinv, nblocks(g.N, BS), BS, 8.0 * 2.0 * g.N, g, alpha, rho, dtd, dinv, parts);
}
void launch_scalar_rhs(Ctx& c, const Grid& g, const double* th, double rho, double* b, double* parts) {
    KS_LAUNCH(c, k_scalar_rhs, nblocks(g.N, BS), BS, 8.0 * 2.0 * g.N, g, th, rho, b, parts);
}
void launch_scalar_pred(Ctx& c, long long n, const double* so, const double* conv, const double* dold, double* out, double dt, double rho,
                        double fac) {
    KS_LAUNCH(c, k_scalar_pred, nblocks(n, BS), BS, 8.0 * 4.0 * n, n, so, conv, dold, out, dt, rho, fac, 1.0 / rho);
}
void launch_scalar_corr(Ctx& c, long long n, const double* s_old, const double* conv_old, const double* conv, const double* dold,
                        const double* dnew, double* out, double dt, double rho, double ofac, double nfac) {
    KS_LAUNCH(c, k_scalar_corr, nblocks(n, BS), BS, 8.0 * (6.0 + (dnew ? 1.0 : 0.0)) * n, n, s_old, conv_old, conv, dold, dnew, out, dt, rho,
              ofac, nfac, 1.0 / rho);
}
void launch_lincomb(Ctx& c, long long n, double a, const double* x, double b, const double* y, double* out) {
    KS_LAUNCH(c, k_lincomb, nblocks(n, BS), BS, 8.0 * 3.0 * n, n, a, x, b, y, out);
}

}  // namespace ks
