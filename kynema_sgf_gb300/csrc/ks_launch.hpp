// Host-side declarations of the kernel launchers (one per device pass).
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "ks_common.cuh"

namespace ks {

// Launch context: the stream every kernel of a handle runs on, a launch
// counter, and optional CUDA-event timing of selected kernels (by kernel
// name, or "*" for all) recorded on that same stream.
struct Ctx {
    cudaStream_t stream = nullptr;
    long long launches = 0;
    bool capturing = false;  // recording a CUDA graph: no per-launch profiling events
    std::string prof;
    struct Open {
        std::string name;
        cudaEvent_t a, b;
        double bytes;
    };
    struct Acc {
        long long launches = 0;
        double ms = 0.0, bytes = 0.0;
    };
    std::vector<Open> open;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, Acc> acc;  // kernel name -> totals

    // names compare without spaces (the report prints them without, e.g. "(k_nd_col<T,0>)")
    bool prof_match(const char* name) const {
        if (prof.empty() || capturing) return false;
        if (prof == "*") return true;
        size_t q = 0;
        for (const char* c = name; *c; ++c) {
            if (*c == ' ') continue;
            if (q >= prof.size() || prof[q] != *c) return false;
            ++q;
        }
        return q == prof.size();
    }
    cudaEvent_t ev() {
        cudaEvent_t e;
        if (!pool.empty()) {
            e = pool.back();
            pool.pop_back();
        } else {
            cudaEventCreate(&e);
        }
        return e;
    }
    void prof_begin(const char* name, double bytes) {
        open.push_back({name, ev(), ev(), bytes});
        cudaEventRecord(open.back().a, stream);
    }
    void prof_end() { cudaEventRecord(open.back().b, stream); }
    // fold recorded launches into acc (call after the stream is synchronised)
    void prof_collect() {
        for (auto& o : open) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, o.a, o.b);
            auto& a = acc[o.name];
            a.launches += 1;
            a.ms += ms;
            a.bytes += o.bytes;
            pool.push_back(o.a);
            pool.push_back(o.b);
        }
        open.clear();
    }
    ~Ctx() {
        for (auto& o : open) {
            cudaEventDestroy(o.a);
            cudaEventDestroy(o.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

// Launch on the context's stream.  `bytes` is the algorithmic HBM traffic of
// the launch: every distinct array the kernel reads or writes, counted once,
// times its element size (stencil neighbours are not counted again).
#define KS_LAUNCH(c, kern, grid, block, bytes, ...)            \
    do {                                                       \
        const bool ks_p_ = (c).prof_match(#kern);              \
        if (ks_p_) (c).prof_begin(#kern, (double)(bytes));     \
        kern<<<(grid), (block), 0, (c).stream>>>(__VA_ARGS__); \
        if (ks_p_) (c).prof_end();                             \
        ++(c).launches;                                        \
    } while (0)

// the same under a given profiling name (a kernel template launched for several ops)
#define KS_LAUNCH_NAMED(c, name, kern, grid, block, bytes, ...) \
    do {                                                        \
        const bool ks_p_ = (c).prof_match(name);                \
        if (ks_p_) (c).prof_begin(name, (double)(bytes));       \
        kern<<<(grid), (block), 0, (c).stream>>>(__VA_ARGS__);  \
        if (ks_p_) (c).prof_end();                              \
        ++(c).launches;                                         \
    } while (0)

// the same with dynamic shared memory
#define KS_LAUNCH_SMEM(c, kern, grid, block, smem, bytes, ...)        \
    do {                                                               \
        const bool ks_p_ = (c).prof_match(#kern);                      \
        if (ks_p_) (c).prof_begin(#kern, (double)(bytes));             \
        kern<<<(grid), (block), (smem), (c).stream>>>(__VA_ARGS__);    \
        if (ks_p_) (c).prof_end();                                     \
        ++(c).launches;                                                \
    } while (0)

struct Scalars {  // values fed to the pointwise kernels
    double rho, irho, mu, smag_fac;
    int smag;
    int geo, cor, body, act;
    double gf[3];
    double east[3], north[3], up[3];
    double corfac, sinphi, cosphi, hfac;
    double body_force[3];
    // BodyForce type oscillatory: body_force * cos(body_omega t_nph), t_nph the
    // mid-step time (BodyForce.cpp:145-160); body_osc = 0: uniform_constant
    int body_osc;
    double body_omega, t_nph;
    // temperature: alpha_eff = mu / Pr + mu_t / Pr_t; BoussinesqBuoyancy g beta (T0 - T); ABLForcing
    int temp, bous, ablf;
    double mu_pr, iprt;
    double grav[3], beta_T, T_ref;
    double ablf_force[2];
};

// ---- pointwise / stencil passes (ks_kernels.cu)
void launch_init_tgv(Ctx& c, const Grid& g, double* vel, const double plo[3], const double L[3]);
void launch_init_abl(Ctx& c, const Grid& g, double* vel, int loglaw, const double U[3], double ut_over_kappa, double z0,
                     double amp, double zmax_rel, unsigned long long seed);
// mu_eff (and alpha_eff when s.temp is set and alpha is not null)
// fp32 = 1: strain rate in FP32 arithmetic (mixed-precision form), mu_eff stored in FP64
void launch_smagorinsky(Ctx& c, const Grid& g, const double* vel, double* mueff, const Scalars& s, double* alpha = nullptr, int fp32 = 0);
void launch_fill(Ctx& c, double* p, double v, long long n);
void launch_copy(Ctx& c, double* dst, const double* src, long long n);
// src = rho (-gp / rho + sources); theta: the temperature state BoussinesqBuoyancy reads
void launch_sources(Ctx& c, const Grid& g, const double* vel_old, const double* gp, const double* act, double* src, const Scalars& s,
                    const double* theta = nullptr);
void launch_plane_sums(Ctx& c, const Grid& g, const double* vel, double* partials, int* nparts);
void launch_wall_grad(Ctx& c, const Grid& g, const double* vel_old, const double* mueff, double* wg, int shear_type, double ut2,
                      double um0, double um1, double vmag, double rho);
// out = divtau(vel) ; mode 0: plain, mode 1: forces = (src + divtau)/rho also written,
// mode 2: out = base + 0.5*dt*(divtau(vel) - dold)/rho (RK2 correction into out).
// Fused shared-memory tiles; face_scratch is not used.
// fp32 = 1 (modes 0-2): staging, face fluxes and divergence in FP32 (mixed-precision form), epilogue in FP64
void launch_divtau(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, int mode,
                   const double* src, double* forces, const double* base, const double* dold, double dt, double rho,
                   double* const face_scratch[9], int fp32 = 0);
// the same result through face-flux arrays in caller-provided scratch (9 arrays:
// N cells for x and y faces, nx*ny*(nz+1) for z faces) and a divergence pass
void launch_divtau_faces(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, int mode,
                         const double* src, double* forces, const double* base, const double* dold, double dt, double rho,
                         double* const face_scratch[9]);
// MOL corrector_rhs (explicit) fused into the tiled divtau of vel:
// out = (rho u_old + dt (0.5 (conv_old + conv_new) + 0.5 (dold + divtau(vel)) + src)) / rho
void launch_divtau_corrector(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, double* out, const double* vel_old,
                             const double* conv_old, const double* conv_new, const double* dold, const double* src, double dt, double rho);
// Tensor-diffusion solve passes on any level grid g: out = x + omega dinv (b - rho x + dtd divtau(x))
// (omega > 0, a Jacobi sweep) or out = b - rho x + dtd divtau(x) (omega = 0, the residual), with
// block maxima of the residual's magnitude in parts (divtau_tile_blocks(g) entries) when parts is set.
int divtau_tile_blocks(const Grid& g);
void launch_divtau_jacobi(Ctx& c, const Grid& g, const double* x, const double* mueff, const double* wg, const double* b, const double* dinv,
                          double* out, double rho, double dtd, double omega, double* parts);
// predictor_rhs: vel = (rho vel_old + dt (conv + src + fac divtau)) / rho
void launch_predictor_rhs(Ctx& c, const Grid& g, const double* vel_old, const double* conv, const double* src, const double* divtau,
                          double* vel, double dt, double rho, double fac);
void launch_proj_pre(Ctx& c, const Grid& g, double* vel, const double* vel_old, const double* gp, double scaling, double rho,
                     int add_gp, int sub_old);
void launch_nodal_rhs(Ctx& c, const Grid& g, const double* vel, double* rhs, double* partials, int* nparts);
// per-block maxima of |nodal divergence of vel| (parts[0..np)) and |vel| (parts[np..2np))
void launch_nodal_divmax(Ctx& c, const Grid& g, const double* vel, double* partials, int* nparts);
void launch_nodal_post(Ctx& c, const Grid& g, const double* phi, double* vel, const double* vel_old, double* gp, double* p,
                       double sigma, int add_old, int incremental);
void launch_mac_rhs(Ctx& c, const Grid& g, const double* um, const double* vm, const double* wm, double* rhs, double* partials,
                    int* nparts);
// per-block maxima of |div u_mac| (parts[0..np)) and of the face speeds (parts[np..2np))
void launch_mac_divmax(Ctx& c, const Grid& g, const double* um, const double* vm, const double* wm, double* partials, int* nparts);
void launch_mac_correct(Ctx& c, const Grid& g, const double* phi, double* um, double* vm, double* wm, double beta);
void launch_cfl(Ctx& c, const Grid& g, const double* vel, const double* src, const double* mueff, double rho, double* partials,
                int* nparts);
void launch_ke(Ctx& c, const Grid& g, const double* vel, double rho, double* partials, int* nparts);
// a -= s[0] / den (or s[0] / s[1] when den <= 0); with parts, block maxima of the shifted |a| (count in *np)
void launch_sub_ratio(Ctx& c, double* a, long long n, const double* s, double den, double* parts = nullptr, int* np = nullptr);
void launch_reduce(Ctx& c, const double* partials, int nparts, int ncomp, int op_max, double* out);
void launch_act_sample(Ctx& c, const Grid& g, const double* vel, const double* pts, int npts, const double plo[3], double* out);
void launch_act_spread(Ctx& c, const Grid& g, double* act, const double* pts, int npts, const double ax[3], double eps,
                       const double plo[3], const int lo[3], const int hi[3]);

// ---- Godunov (ks_godunov.cu)
// Godunov face scratch; each array holds FP64 or FP32 values (fp32 flag of
// the launchers), sized for FP64.
struct GodunovBufs {
    void* ad[3];        // pre-MAC advective velocities on d-faces
    void* edge[3][3];   // unlimited PPM edge values edge[d][n] on d-faces
    void* pm[3][3];     // limited PPM parabola (sm, sp) of every cell along d, component n (pre-MAC pass)
    void* pp[3][3];
    void* lo[3][3];     // left states lo[d][n]
    void* hi[3][3];     // right states hi[d][n]
    void* tedge[3][3];  // upwinded states tedge[d][n]
    void* tr[3][3][3];  // transverse-corrected states tr[a][b][n]
    void* flux[3][3];   // fluxes flux[d][n]
};
// FP32 copies of the advection inputs for the mixed-precision form: launch_premac fills vel and
// forces, launch_advection (same step) the MAC velocities
struct GodunovIn32 {
    float* vel;     // 3 N
    float* forces;  // 3 N
    float* mac[3];  // face arrays
};
void launch_premac(Ctx& c, const Grid& g, const double* vel_old, const double* forces, double dt, GodunovBufs& B, double* mac[3],
                   int fp32, GodunovIn32* in32);
void launch_advection(Ctx& c, const Grid& g, const double* vel_old, const double* forces, const double* mac[3], double dt, double rho,
                      GodunovBufs& B, double* conv, int fp32, GodunovIn32* in32);
// Godunov fluxes and conv = -div(flux) of rho s for a cell scalar s with forces fs = src + diff (FP64);
// B: component-0 face slots reused as scratch
void launch_scalar_advection(Ctx& c, const Grid& g, const double* s, const double* fs, const double* const mac[3], double dt, double rho,
                             GodunovBufs& B, double* conv);

// ---- temperature transport (ks_temperature.cu), FP64
// ABLFieldInit uniform-wind branch: velocity = U + sinusoidal perturbation (pert != 0)
void launch_init_abl_ref(Ctx& c, const Grid& g, double* vel, const double plo[3], const double U[3], int pert, double aval, double bval,
                         double ufac, double vfac, double ref_height, double ib_height);
// piecewise-linear temperature profile from (heights, values) in device memory (n points)
void launch_theta_profile(Ctx& c, const Grid& g, double* theta, double zlo, const double* heights, const double* values, int n);
// per-layer sums of f over x and y: out[k], k < nz (one block per layer)
void launch_layer_sums(Ctx& c, const Grid& g, const double* f, double* out);
// wall-normal temperature gradient at z-lo, rho q / alpha (nx ny values): type as the shear stress type,
// phi_h = ln(z_ref / z0t), neutral surface (surface temperature = theta_mean)
void launch_theta_wall_grad(Ctx& c, const Grid& g, const double* vel_old, const double* theta_old, const double* alpha, double* gz, int type,
                            double utau, double kappa, double phi_h, double vmag_mean, double theta_mean, double rho);
// scalar diffusion div(alpha grad theta) with z data: tzlo/tzhi 0 Neumann 0, 1 wall-model gradient gz, 2 fixed gradient gtop.
// mode 0: out = acc; 2: out = base + 0.5 dt (acc - dold) / rho; 7: Jacobi sweep out = th + omega dinv (b - rho th + dt acc);
// 8: residual out = b - rho th + dt acc.  Modes 7 / 8 write block maxima of the residual to parts when set.
struct ScalarBC {
    int zlo, zhi;
    const double* gz;
    double gtop;
};
int tdiff_blocks(const Grid& g);
void launch_tdiff(Ctx& c, const Grid& g, const double* th, const double* alpha, const ScalarBC& bc, double* out, int mode, const double* base,
                  const double* dold, const double* b, const double* dinv, double* parts, double dt, double rho, double omega);
// 1 / diagonal of rho - dtd div(alpha grad), with block maxima of 1 - rho / D in parts
void launch_tdiff_dinv(Ctx& c, const Grid& g, const double* alpha, const ScalarBC& bc, double rho, double dtd, double* dinv, double* parts);
// b = rho theta with block maxima of |b| in parts (tdiff_blocks(g) entries)
void launch_scalar_rhs(Ctx& c, const Grid& g, const double* th, double rho, double* b, double* parts);
// predictor_rhs of a scalar without sources: out = (rho s_old + dt (conv + fac dold)) / rho
void launch_scalar_pred(Ctx& c, long long n, const double* s_old, const double* conv, const double* dold, double* out, double dt, double rho,
                        double fac);
// corrector_rhs of a scalar without sources:
// out = (rho s_old + dt (0.5 (conv_old + conv) + ofac dold + nfac dnew)) / rho (dnew may be null when nfac = 0)
void launch_scalar_corr(Ctx& c, long long n, const double* s_old, const double* conv_old, const double* conv, const double* dold,
                        const double* dnew, double* out, double dt, double rho, double ofac, double nfac);
// out = a x + b y (n values)
void launch_lincomb(Ctx& c, long long n, double a, const double* x, double b, const double* y, double* out);

// ---- MOL advection (ks_mol.cu), FP64
// face-normal velocities extrapolated from vel (before the MAC projection)
void launch_mol_extrap(Ctx& c, const Grid& g, const double* vel, double* const mac[3]);
// conv = -div(u_mac (rho u)_face) through the nine face-flux arrays fl; mode 1
// also writes vel_out = (rho vel_old + dt (conv + src + fac dold)) / rho (predictor_rhs),
// mode 2 vel_out = (rho vel_old + dt (0.5 (conv_old + conv) + fac dold + src)) / rho
// (corrector_rhs of Crank-Nicolson / implicit diffusion)
void launch_mol_advection(Ctx& c, const Grid& g, const double* vel, const double* const mac[3], double rho, double* const fl[9],
                          double* conv, int mode, const double* vel_old, const double* src, const double* dold, const double* conv_old,
                          double* vel_out, double dt, double fac);

// conv = -div(u_mac (rho s)_face) of a cell scalar s (hoextrap at z walls) through three face arrays
void launch_mol_scalar_advection(Ctx& c, const Grid& g, const double* s, const double* const mac[3], double rho, double* const fl[3],
                                 double* conv);

// ---- implicit / Crank-Nicolson tensor diffusion solve (ks_implicit.cu)
// 1 / diagonal of rho - dtd divtau per cell and component (3 N_g values); parts, when
// set, receives diff_cell_blocks(g) block maxima of 1 - rho / diagonal
int diff_cell_blocks(const Grid& g);
void launch_diff_dinv(Ctx& c, const Grid& g, const double* mueff, double rho, double dtd, double* dinv, double* parts);
// coarse = mean of the 8 fine cells below each coarse cell, ncomp components
void launch_avg8(Ctx& c, const Grid& fine, const Grid& coarse, const double* f, double* cr, int ncomp);
// fine += coarse value of the parent cell (piecewise-constant prolongation), 3 components
void launch_prolong_add(Ctx& c, const Grid& fine, const Grid& coarse, const double* cr, double* f);
// b = rho u with diff_cell_blocks(g) block maxima of |b| in parts
void launch_rhs_b(Ctx& c, const Grid& g, const double* u, double rho, double* b, double* parts);

// ---- reverse mode of the Godunov passes (ks_adjoint.cu), FP64, periodic.
// Adjoints of the GodunovBufs arrays (same shapes) plus those of the MAC
// velocities, of the cell velocity (u: the input of both passes, 3N) and of
// the forces (3N).  Kernels accumulate into these arrays.
struct AdjBufs {
    double* ad[3];
    double* edge[3][3];
    double* lo[3][3];
    double* hi[3][3];
    double* tedge[3][3];
    double* tr[3][3][3];
    double* flux[3][3];
    double* umac[3];
    double* u;
    double* forces;
};
// fp32: the forward intermediates in B are FP32 (mixed-precision Godunov passes);
// the reverse arithmetic is FP64 either way
void launch_adj_edges(Ctx& c, const Grid& g, int d, const double* u, double* const Eb[3], double* ub, int fp32);
// scratch: 8N doubles for the gather form (null: the scatter form)
void launch_adj_faces(Ctx& c, const Grid& g, int d, int mode, const double* u, const GodunovBufs& B, const AdjBufs& A, double dt, double rho,
                      const double* umac_d, double* scratch, int fp32);
void launch_adj_pm_trans(Ctx& c, const Grid& g, int a, int b, int n, double dt, const GodunovBufs& B, const AdjBufs& A, int fp32);
void launch_adj_pm_final(Ctx& c, const Grid& g, int d, double dt, const GodunovBufs& B, const double* forces, const AdjBufs& A, int fp32);
// reverse of the post-MAC stages 2 (both transverse directions of the a-faces)
// and 3 (d-faces), gather form; CB: 6N doubles of scratch (the per-cell
// correction adjoints)
void launch_adj_adv_trans(Ctx& c, const Grid& g, int a, const double* u, double rho, double dt, const double* const mac[3],
                          const GodunovBufs& B, const AdjBufs& A, double* CB, int fp32);
void launch_adj_adv_flux(Ctx& c, const Grid& g, int d, const double* u, const double* forces, double rho, double dt, const double* const mac[3],
                         const GodunovBufs& B, const AdjBufs& A, double* CB, int fp32);
void launch_adj_div(Ctx& c, const Grid& g, const double* convb, const AdjBufs& A);
// reverse of divtau(vel; mueff, wg) for the adjoint s * divtau_b: accumulates the
// velocity (ub), cell viscosity (mub, may be null) and wall-gradient (wgb, may be null) adjoints
void launch_adj_tau(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wg, const double* divtau_b, double s, double* ub,
                    double* mub, double* wgb, int fp32 = 0);
// scratch: 9N doubles for the gather form (null: the scatter form)
void launch_adj_smag(Ctx& c, const Grid& g, const double* vel, const double* mub, const Scalars& s, double* ub, double* scratch, int fp32 = 0);
void launch_adj_wall_local(Ctx& c, const Grid& g, const double* vel, const double* mueff, const double* wgb, double ut2, double um0, double um1,
                           double vm, double rho, double* ub, double* mub, double* parts, int* np);
void launch_adj_wall_global(Ctx& c, const Grid& g, const double* vel, double bu, double bv, double bm, double* ub);
void launch_adj_coriolis(Ctx& c, const Grid& g, const double* srcb, const Scalars& s, double* ub);
void launch_adj_nodal_post(Ctx& c, const Grid& g, const double* psi, const double* ub, double* out);
void launch_axpby(Ctx& c, long long n, double a, const double* x, double b, const double* y, double* out);
void launch_objective(Ctx& c, const Grid& g, const double* u, const int lo[3], const int hi[3], double invM, double* ub, double* parts, int* np);
void launch_act_adj_dot(Ctx& c, const Grid& g, const double* actb, const double* pts, int npts, const double ax[3], double eps, const double plo[3],
                        const int lo[3], const int hi[3], double* parts, int* np);
void launch_act_sample_adj(Ctx& c, const Grid& g, const double* pts, const double* wb, int npts, const double plo[3], double* ub);

// ---- multigrid (ks_mg.cu); T = double (FP64 path) or float (cycles of the
// mixed-precision defect correction)
template <typename T>
struct CCLevelT {
    int nx, ny, nz, zper;
    T ix2, iy2, iz2;
    T inv_diag[3];  // 1/(-beta d): interior, wall-adjacent, single layer
    T gs[3][3];     // Gauss-Seidel neighbour weights w_m / d per class (x, y, z)
    T dg[3];        // diagonal -beta d per class
    T *phi, *rhs, *res;
    const T* binv;  // bottom level: pinned inverse of d p - sum w p (row-major), or null
};
template <typename T>
struct NDLevelT {
    int nx, ny, nz;  // nodes
    int zper;
    T W[27];
    T inv_diag;      // 1/(sigma W_centre)
    int faces_zero;  // face-neighbour weights vanish (equal spacings): skipped
    T *phi, *rhs, *res, *tmp;
    const T* binv;  // bottom level: pinned inverse of the unscaled stencil (row-major), or null
};
using CCLevelDev = CCLevelT<double>;
using NDLevelDev = NDLevelT<double>;
template <typename T>
void launch_cc_gsrb(Ctx& c, const CCLevelT<T>& L, double beta, int color);
template <typename T>
// zero_color 0 / 1: the cells of that colour were the last red-black half-sweep's (their
// residual is zero to rounding and is written as 0 without evaluation); -1: none
void launch_cc_resid(Ctx& c, const CCLevelT<T>& L, double beta, double* partials, int* nparts, int zero_color = -1);
// FP64 residuals of the mixed-precision defect correction, written as the FP32 cycle's
// right-hand side r32 with its solution z32 zeroed (L.res untouched)
void launch_cc_resid32(Ctx& c, const CCLevelT<double>& L, double beta, float* r32, float* z32, double* partials, int* nparts);
void launch_nd_resid32(Ctx& c, const NDLevelT<double>& L, double sigma, float* r32, float* z32, double* partials, int* nparts);
// first residual of a nodal solve from phi = 0 (the right-hand side): with out, also the
// first Jacobi sweep of the zero iterate; with r32 / z32, the FP32 cycle's right-hand side
void launch_nd_zero_start(Ctx& c, const NDLevelT<double>& L, double sigma, double omega, double* out, float* r32, float* z32,
                          double* partials, int* nparts);
template <typename T>
void launch_cc_restrict(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C);
template <typename T>
void launch_cc_prolong(Ctx& c, const CCLevelT<T>& F, const CCLevelT<T>& C);
template <typename T>
void launch_cc_bottom(Ctx& c, const CCLevelT<T>& L, double beta, int sweeps);
template <typename T>
void launch_nd_jacobi(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, const T* in, T* out);
template <typename T>
void launch_nd_resid(Ctx& c, const NDLevelT<T>& L, double sigma, double* partials, int* nparts);
// Jacobi sweep that also writes block maxima of |rhs - A in| (the residual of
// the input iterate) for the convergence test
void launch_nd_jacobi_norm(Ctx& c, const NDLevelT<double>& L, double sigma, double omega, const double* in, double* out,
                           double* partials, int* nparts);
template <typename T>
void launch_nd_restrict(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C);
template <typename T>
void launch_nd_prolong(Ctx& c, const NDLevelT<T>& F, const NDLevelT<T>& C);
template <typename T>
void launch_nd_bottom(Ctx& c, const NDLevelT<T>& L, double sigma, double omega, int sweeps);
void launch_add_f32(Ctx& c, double* phi, const float* e, long long n);

}  // namespace ks
