// Reverse mode of the advance: one-step vector-Jacobian products and the
// binomial (revolve-type) checkpointed reverse sweep over many steps.
//
// The reference has no adjoint; this is the differentiated form of the same
// single-level step (incflo::advance, src/incflo_advance.cpp:63-438) for a
// fixed dt: every pass of the path (periodic or wall-bounded z, laminar or
// Smagorinsky viscosity, Moeng wall model, geostrophic / Coriolis / body /
// actuator sources, UniformCtDisk actuators with a single thrust coefficient).
//
// Step n maps (u, gp) -> (u', gp'):
//   mu    = mu0 + rho Cs^2 D^2 |S(u)|;  wg = W(u_1, <u_1>, u_tau(<|u_1|>), mu)
//   act   = sum_d 0.5 ct_d (s_d . a_d)^2 B_d a_d,  s_d = sum_p w_p u(x_p)
//   src   = -gp + rho (C u + act + const);  dold = L(u; mu, wg)
//   forces = (src + dold)/rho
//   mac   = P_mac PREMAC(u, forces);  conv = ADV(u, mac, forces)
//   v*    = u + dt/rho (conv + src + dold)
//   v**   = v* + dt/(2 rho) (L(v*; mu, wg) - dold)
//   v     = v** + sigma gp,  sigma = dt/rho
//   phi   = (sigma A)^-1 Dn v;  u' = v - sigma Gn phi;  gp' = Gn phi
// P_mac is symmetric on the faces it changes; Gn^T = -Dn for the nodal pair
// (the wall rows of both carry the same half weight), so the nodal adjoint is
// one more solve with A: sigma A psi = Dn(gp_bar - sigma u_bar),
// v_bar = u_bar + Gn psi.  The other passes are reversed by the kernels of
// ks_adjoint.cu at the forward linearisation point, recomputed from the
// checkpointed (u, gp) in FP64.
#include "ks_sim.hpp"

namespace ks {

void Sim::adj_check() const {
    if (!godunov_) throw KsError(KS_ERR_UNSUPPORTED, "the reverse mode differentiates the Godunov scheme (incflo.use_godunov = 1)");
    if (diff_type_ != 0) throw KsError(KS_ERR_UNSUPPORTED, "the reverse mode differentiates explicit diffusion (incflo.diffusion_type = 0)");
    if (temp_ || S_.bous || S_.ablf) throw KsError(KS_ERR_UNSUPPORTED, "the reverse mode has no temperature, BoussinesqBuoyancy or ABLForcing");
    if (t_.adaptive) throw KsError(KS_ERR_UNSUPPORTED, "the adjoint needs a fixed time step (time.fixed_dt > 0)");
    if (wallmodel_ && shear_ != 0) throw KsError(KS_ERR_UNSUPPORTED, "the adjoint's wall model is ABL.wall_shear_stress_type = moeng");
    for (auto& d : disks_)
        if (d.ct.size() != 1) throw KsError(KS_ERR_UNSUPPORTED, "the adjoint needs a single thrust_coeff value per disk");
}

void Sim::adj_alloc() {
    adj_check();
    // The recomputation from checkpoints must repeat each forward step bit for
    // bit, so the Poisson solves start from zero (a warm start would carry
    // state the checkpoints do not hold).
    mg_warm_ = 0;
    mac_prev_ok_ = false;
    if (adj_) return;
    auto S = std::make_unique<AdjState>();
    const size_t N = (size_t)g_.N, NF = (size_t)g_.NFz, N3 = 3 * N;
    const size_t fsz[3] = {N, N, NF};
    size_t total = 0;
    for (int d = 0; d < 3; ++d) total += fsz[d] * 16;
    for (int a = 0; a < 3; ++a) total += 2 * 3 * fsz[a];
    S->gbuf.alloc(total);
    double* q = S->gbuf.p;
    AdjBufs& A = S->A;
    for (int d = 0; d < 3; ++d) {
        A.ad[d] = q; q += fsz[d];
        for (int n = 0; n < 3; ++n) { A.edge[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { A.lo[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { A.hi[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { A.tedge[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { A.flux[d][n] = q; q += fsz[d]; }
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            for (int n = 0; n < 3; ++n) A.tr[a][b][n] = nullptr;
            if (a == b) continue;
            for (int n = 0; n < 3; ++n) { A.tr[a][b][n] = q; q += fsz[a]; }
        }
    for (int d = 0; d < 3; ++d) {
        S->umacb[d].alloc(fsz[d]);
        A.umac[d] = S->umacb[d].p;
    }
    S->forcesb.alloc(N3);
    A.forces = S->forcesb.p;
    S->ub.alloc(N3);
    S->gpb.alloc(N3);
    A.u = S->ub.p;
    for (auto* b : {&S->w, &S->t1, &S->t2, &S->srcb, &S->doldb, &S->su, &S->sgp}) b->alloc(N3);
    S->sp.alloc(p_.n);
    S->mub.alloc(N);
    S->cbuf.alloc(9 * N);  // scratch of the gather-form reverse passes
    S->wgb.alloc(2 * (size_t)g_.nx * g_.ny);
    // post-MAC intermediates of the recompute: lo, hi, tedge, flux per direction and tr
    size_t total2 = 0;
    for (int d = 0; d < 3; ++d) total2 += fsz[d] * 12 + 2 * 3 * fsz[d];
    S->gbuf2.alloc(total2);
    GodunovBufs& G2 = S->gb2;
    q = S->gbuf2.p;
    for (int d = 0; d < 3; ++d) {
        G2.ad[d] = gb_.ad[d];
        for (int n = 0; n < 3; ++n) {
            G2.edge[d][n] = gb_.edge[d][n];  // the unlimited edges and limited parabolas are shared by both passes
            G2.pm[d][n] = gb_.pm[d][n];
            G2.pp[d][n] = gb_.pp[d][n];
            G2.lo[d][n] = q; q += fsz[d];
            G2.hi[d][n] = q; q += fsz[d];
            G2.tedge[d][n] = q; q += fsz[d];
            G2.flux[d][n] = q; q += fsz[d];
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int n = 0; n < 3; ++n) {
                G2.tr[a][b][n] = nullptr;
                if (a != b) { G2.tr[a][b][n] = q; q += fsz[a]; }
            }
    size_t maxpts = 1;
    for (auto& d : disks_) maxpts = std::max(maxpts, (size_t)d.nr * d.nt);
    S->pts.alloc(4 * maxpts);
    S->wb.alloc(3 * maxpts);
    ct_grad_.assign(disks_.size(), 0.0);
    adj_ = std::move(S);
}

void Sim::adjoint_reset() {
    adj_alloc();
    launch_fill(ctx_, adj_->ub.p, 0.0, 3 * g_.N);
    launch_fill(ctx_, adj_->gpb.p, 0.0, 3 * g_.N);
    ct_grad_.assign(disks_.size(), 0.0);
    sync();
}

void Sim::set_disk_ct(const double* ct, int n) {
    if (n != (int)disks_.size()) throw KsError(KS_ERR_ARG, "set_disk_ct: count differs from the number of disks");
    for (int m = 0; m < n; ++m) {
        if (disks_[m].ct.size() != 1) throw KsError(KS_ERR_UNSUPPORTED, "set_disk_ct needs a single thrust_coeff value per disk");
        disks_[m].ct[0] = ct[m];
        disks_[m].ct_now = ct[m];
    }
}

// Objective box: the cells whose centres lie in [lo, hi] (physical units).
void Sim::set_objective_box(const double lo[3], const double hi[3]) {
    adj_alloc();
    AdjState& S = *adj_;
    const double h[3] = {g_.dx, g_.dy, g_.dz};
    const int nn[3] = {g_.nx, g_.ny, g_.nz};
    for (int m = 0; m < 3; ++m) {
        const int a = (int)std::ceil((lo[m] - plo_[m]) / h[m] - 0.5);
        const int b = (int)std::floor((hi[m] - plo_[m]) / h[m] - 0.5);
        S.box_lo[m] = std::max(0, a);
        S.box_hi[m] = std::min(nn[m] - 1, b);
        if (S.box_hi[m] < S.box_lo[m]) throw KsError(KS_ERR_ARG, "objective box contains no cell centre");
    }
    S.box_set = true;
}

// J = mean over the box cells of 0.5 |u|^2 at the current state.  seed:
// velocity_adjoint = dJ/du, gp_adjoint = 0.
double Sim::objective(bool seed) {
    adj_alloc();
    AdjState& S = *adj_;
    if (!S.box_set) throw KsError(KS_ERR_ARG, "objective box not set");
    const double M = (double)(S.box_hi[0] - S.box_lo[0] + 1) * (S.box_hi[1] - S.box_lo[1] + 1) * (S.box_hi[2] - S.box_lo[2] + 1);
    int np = 0;
    launch_objective(ctx_, g_, vel_.p, S.box_lo, S.box_hi, 1.0 / M, seed ? S.ub.p : nullptr, parts_.p, &np);
    if (seed) launch_fill(ctx_, S.gpb.p, 0.0, 3 * g_.N);
    S.J = reduce(np, 1, 0, nullptr);
    return S.J;
}

// One forward step from the current state with the step's dt, without the
// clock (dt is fixed in the differentiable configuration).
void Sim::forward_core() {
    pre_advance();
    prepare_time_step();
    apply_predictor(false);
}

// Reverse of the actuator forcing.  srcb = adjoint of src; the actuator field
// enters src as rho * act.
void Sim::adjoint_disks(const double* srcb) {
    if (!S_.act) return;
    AdjState& S = *adj_;
    const double pi = 3.14159265358979323846;
    for (size_t di = 0; di < disks_.size(); ++di) {
        const Disk& d = disks_[di];
        const double* ax = d.normal;
        std::vector<double> hp, rpos;
        disk_points(d, hp, rpos);
        // q = sum_x actb(x) . a  B(x), B with the per-point weights pi (r+^2 - r-^2) / nt
        std::vector<double> ring;
        double bmin[3] = {1e300, 1e300, 1e300}, bmax[3] = {-1e300, -1e300, -1e300};
        for (int ip = 0; ip < d.nr; ++ip) {
            const double r = (ip + 0.5) * d.dr, rp = r + 0.5 * d.dr, rmn = r - 0.5 * d.dr;
            const double wgt = pi * (rp * rp - rmn * rmn) / d.nt;
            for (int it = 0; it < d.nt; ++it) {
                const double* o = &rpos[3 * (ip * d.nt + it)];
                for (int m = 0; m < 3; ++m) {
                    ring.push_back(o[m]);
                    bmin[m] = std::min(bmin[m], o[m]);
                    bmax[m] = std::max(bmax[m], o[m]);
                }
                ring.push_back(wgt);
            }
        }
        const int nring = (int)ring.size() / 4;
        int lo[3], hi[3];
        const double h[3] = {g_.dx, g_.dy, g_.dz};
        const int nn[3] = {g_.nx, g_.ny, g_.nz};
        for (int m = 0; m < 3; ++m) {
            lo[m] = std::max(0, (int)std::floor((bmin[m] - 4.0 * d.eps - plo_[m]) / h[m]) - 1);
            hi[m] = std::min(nn[m] - 1, (int)std::floor((bmax[m] + 4.0 * d.eps - plo_[m]) / h[m]) + 1);
        }
        if (hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2]) continue;
        ck(cudaMemcpyAsync(S.pts.p, ring.data(), ring.size() * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "H2D");
        int np = 0;
        launch_act_adj_dot(ctx_, g_, srcb, S.pts.p, nring, ax, d.eps, plo_, lo, hi, parts_.p, &np);
        const double q = rho_ * reduce(np, 1, 0, nullptr);
        // act = 0.5 ct un^2 B a:  dJ/dct += 0.5 un^2 q ;  un_bar = ct un q
        const double un = d.ref[0] * ax[0] + d.ref[1] * ax[1] + d.ref[2] * ax[2];
        ct_grad_[di] += 0.5 * un * un * q;
        const double unb = d.ct_now * un * q;
        // un = a . sum_p w_p u(x_p): scatter w_p unb a to the sampling stencils
        const int npts = d.nr * d.nt;
        std::vector<double> wb(3 * (size_t)npts);
        for (int ir = 0; ir < d.nr; ++ir) {
            const double w = ((ir + 1.0) * (ir + 1.0) - (double)ir * ir) / ((double)d.nr * d.nr * d.nt);
            for (int it = 0; it < d.nt; ++it)
                for (int m = 0; m < 3; ++m) wb[3 * (ir * d.nt + it) + m] = w * unb * ax[m];
        }
        ck(cudaMemcpyAsync(S.pts.p, hp.data(), hp.size() * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "H2D");
        ck(cudaMemcpyAsync(S.wb.p, wb.data(), wb.size() * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "H2D");
        launch_act_sample_adj(ctx_, g_, S.pts.p, S.wb.p, npts, plo_, S.ub.p);
        sync();  // host vectors and S.pts are reused by the next disk
    }
}

// Reverse of one step at the current state x^n = (velocity, gp).  On entry
// the adjoint fields hold the adjoint of x^{n+1} (or, with seed, they are set
// to dJ/dx^{n+1} from the recomputed x^{n+1}); on return they hold the
// adjoint of x^n, the disk thrust gradients are accumulated, and the forward
// state is x^n again.
void Sim::adjoint_step_impl(bool seed) {
    AdjState& S = *adj_;
    AdjBufs& A = S.A;
    const long long N3 = 3 * g_.N;
    const double dt = t_.dt[0], sigma = dt / rho_, dr = dt / rho_;
    struct Restore {  // post-MAC buffers and clock, also when a solve throws
        Sim& s;
        Clock clock;
        ~Restore() {
            s.adv_bufs_ = nullptr;
            s.t_ = clock;
        }
    } restore{*this, t_};
    // The linearisation point is the handle's own forward step, recomputed
    // at its precision: a mixed-precision handle's reverse kernels read the
    // FP32 Godunov intermediates its forward used (and accumulate in FP64);
    // its multigrid keeps FP32 cycles under the FP64 defect correction, here
    // and in the two reverse solves.  The post-MAC pass writes its own
    // buffers so that the pre-MAC intermediates survive for the reverse.
    adv_bufs_ = &S.gb2;
    const int fp32 = mixed_;
    launch_copy(ctx_, S.su.p, vel_.p, N3);
    launch_copy(ctx_, S.sgp.p, gp_.p, N3);
    launch_copy(ctx_, S.sp.p, p_.p, (long long)p_.n);
    forward_core();
    if (seed) {
        objective(true);
        if (!S.fu.p) {
            S.fu.alloc(N3);
            S.fgp.alloc(N3);
            S.fp.alloc(p_.n);
        }
        launch_copy(ctx_, S.fu.p, vel_.p, N3);
        launch_copy(ctx_, S.fgp.p, gp_.p, N3);
        launch_copy(ctx_, S.fp.p, p_.p, (long long)p_.n);
    }
    double* ub = S.ub.p;
    double* gpb = S.gpb.p;

    double* mub = S_.smag ? S.mub.p : nullptr;
    double* wgb = wallmodel_ ? S.wgb.p : nullptr;
    launch_fill(ctx_, S.mub.p, 0.0, g_.N);
    launch_fill(ctx_, S.wgb.p, 0.0, 2LL * g_.nx * g_.ny);
    // ---- nodal projection: sigma A psi = Dn(gp_bar - sigma u_bar); v_bar = u_bar + Gn psi
    launch_axpby(ctx_, N3, 1.0, gpb, -sigma, ub, S.w.p);
    nd_rhs(S.w.p);
    nd_solve(sigma);
    launch_adj_nodal_post(ctx_, g_, nd_[0].phi, ub, S.t1.p);  // t1 = v_bar = adjoint of v**
    // ---- v** = v* + dt/(2 rho) (L(v*) - dold); vel_tmp_ still holds v*
    launch_copy(ctx_, ub, S.t1.p, N3);
    launch_adj_tau(ctx_, g_, vel_tmp_.p, mueff_.p, wg_.p, S.t1.p, 0.5 * dr, ub, mub, wgb, fp32);  // ub = v*_bar
    launch_axpby(ctx_, N3, -0.5 * dr, S.t1.p, dr, ub, S.doldb.p);         // dold_bar
    launch_axpby(ctx_, N3, sigma, S.t1.p, 0.0, S.t1.p, gpb);              // gp_bar = sigma v_bar (v = v** + sigma gp)
    launch_axpby(ctx_, N3, dr, ub, 0.0, ub, S.srcb.p);                    // src_bar = conv_bar = dt/rho v*_bar
    // ---- advection (post-MAC pass) at the forward intermediates
    ck(cudaMemsetAsync(S.gbuf.p, 0, S.gbuf.n * sizeof(double), ctx_.stream), "memset");
    for (int d = 0; d < 3; ++d) ck(cudaMemsetAsync(A.umac[d], 0, S.umacb[d].n * sizeof(double), ctx_.stream), "memset");
    launch_fill(ctx_, A.forces, 0.0, N3);
    const double* mac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_adj_div(ctx_, g_, S.srcb.p, A);
    // stage 3 first: it accumulates the adjoints of the stage-2 outputs
    for (int d = 0; d < 3; ++d) launch_adj_adv_flux(ctx_, g_, d, vel_old_.p, forces_.p, rho_, dt, mac, S.gb2, A, S.cbuf.p, fp32);
    for (int a = 0; a < 3; ++a) launch_adj_adv_trans(ctx_, g_, a, vel_old_.p, rho_, dt, mac, S.gb2, A, S.cbuf.p, fp32);
    for (int a = 0; a < 3; ++a) launch_adj_faces(ctx_, g_, a, 1, vel_old_.p, S.gb2, A, dt, rho_, umac_[a].p, S.cbuf.p, fp32);
    // ---- MAC projection (symmetric on the faces it changes): the pre-MAC
    // output on wall faces is 0 whatever the input, so their adjoint is dropped
    if (!g_.zper) {
        const size_t layer = (size_t)g_.nx * g_.ny;
        ck(cudaMemsetAsync(A.umac[2], 0, layer * sizeof(double), ctx_.stream), "memset");
        ck(cudaMemsetAsync(A.umac[2] + (size_t)g_.nz * layer, 0, layer * sizeof(double), ctx_.stream), "memset");
    }
    {
        struct Swap {  // the MAC solver works on umac_; swap back even if it throws
            DevBuf<double>* f;
            double** b;
            Swap(DevBuf<double>* f_, double** b_) : f(f_), b(b_) {
                for (int d = 0; d < 3; ++d) std::swap(f[d].p, b[d]);
            }
            ~Swap() {
                for (int d = 0; d < 3; ++d) std::swap(f[d].p, b[d]);
            }
        } swap(umac_, A.umac);
        mac_project();
    }
    // ---- pre-MAC pass (its intermediates are in gb_)
    const size_t fsz[3] = {(size_t)g_.N, (size_t)g_.N, (size_t)g_.NFz};
    for (int d = 0; d < 3; ++d) {
        ck(cudaMemsetAsync(A.ad[d], 0, fsz[d] * sizeof(double), ctx_.stream), "memset");
        for (int n = 0; n < 3; ++n) {
            ck(cudaMemsetAsync(A.lo[d][n], 0, fsz[d] * sizeof(double), ctx_.stream), "memset");
            ck(cudaMemsetAsync(A.hi[d][n], 0, fsz[d] * sizeof(double), ctx_.stream), "memset");
            ck(cudaMemsetAsync(A.tedge[d][n], 0, fsz[d] * sizeof(double), ctx_.stream), "memset");
        }
        for (int b = 0; b < 3; ++b)
            if (b != d) ck(cudaMemsetAsync(A.tr[d][b][0], 0, fsz[d] * sizeof(double), ctx_.stream), "memset");
    }
    for (int d = 0; d < 3; ++d) launch_adj_pm_final(ctx_, g_, d, dt, gb_, forces_.p, A, fp32);
    const int tpl[6][3] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    for (auto& t : tpl) launch_adj_pm_trans(ctx_, g_, t[0], t[1], t[2], dt, gb_, A, fp32);
    for (int d = 0; d < 3; ++d) launch_adj_faces(ctx_, g_, d, 0, vel_old_.p, gb_, A, dt, 1.0, nullptr, S.cbuf.p, fp32);
    // ---- unlimited edges (shared by both passes)
    for (int d = 0; d < 3; ++d) launch_adj_edges(ctx_, g_, d, vel_old_.p, A.edge[d], ub, fp32);
    // ---- forces = (src + dold)/rho
    launch_axpby(ctx_, N3, 1.0, S.srcb.p, 1.0 / rho_, A.forces, S.srcb.p);
    launch_axpby(ctx_, N3, 1.0, S.doldb.p, 1.0 / rho_, A.forces, S.doldb.p);
    // ---- dold = L(u; mu_eff, wg)
    launch_adj_tau(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, S.doldb.p, 1.0, ub, mub, wgb, fp32);
    // ---- src = -gp + rho (Coriolis(u) + act + const)
    launch_axpby(ctx_, N3, 1.0, gpb, -1.0, S.srcb.p, gpb);
    if (S_.cor) launch_adj_coriolis(ctx_, g_, S.srcb.p, S_, ub);
    adjoint_disks(S.srcb.p);
    // ---- wall model: wg(u first layer, plane means, u_tau, mu_eff)
    if (wallmodel_) {
        int np = 0;
        launch_adj_wall_local(ctx_, g_, vel_old_.p, mueff_.p, S.wgb.p, utau_ * utau_, um_[0], um_[1], vmag_, rho_, ub, S.mub.p, parts_.p, &np);
        double b[4];
        reduce(np, 4, 0, b);
        const double M = (double)g_.nx * g_.ny;
        const double vmb = b[2] + b[3] * 2.0 * utau_ * utau_ / vmag_;  // u_tau^2 = (kappa vm / ln(zref/z0))^2
        launch_adj_wall_global(ctx_, g_, vel_old_.p, b[0] / M, b[1] / M, vmb / M, ub);
    }
    // ---- Smagorinsky: mu_eff(u)
    if (S_.smag) launch_adj_smag(ctx_, g_, vel_old_.p, S.mub.p, S_, ub, S.cbuf.p, fp32);
    // ---- back to x^n
    launch_copy(ctx_, vel_.p, S.su.p, N3);
    launch_copy(ctx_, gp_.p, S.sgp.p, N3);
    launch_copy(ctx_, p_.p, S.sp.p, (long long)p_.n);
    ++S.adj_steps;
}

void Sim::adjoint_step() {
    adj_alloc();
    adjoint_step_impl(false);
    sync();
}

// Binomial checkpointing.  cost(n, s) = fewest forward steps (beyond those
// inside the reverse steps) that reverse n steps when the first state is
// stored and s more slots are free:  cost(1, s) = 0,  cost(n, 0) =
// n (n - 1) / 2,  cost(n, s) = min_j [ j + cost(n - j, s - 1) + cost(j, s) ].
// The minimum equals the revolve bound (Griewank and Walther, ACM TOMS 26
// (2000) 19-45) for c = s + 1 checkpoints: t n - C(c + t, t - 1), t the least
// integer with C(c + t, t) >= n.
static void schedule_tables(int n, int s, std::vector<std::vector<long long>>& cost, std::vector<std::vector<int>>& split) {
    cost.assign(n + 1, std::vector<long long>(s + 1, 0));
    split.assign(n + 1, std::vector<int>(s + 1, 0));
    for (int m = 1; m <= n; ++m) cost[m][0] = (long long)m * (m - 1) / 2;
    for (int k = 1; k <= s; ++k)
        for (int m = 2; m <= n; ++m) {
            long long best = -1;
            int bj = 1;
            for (int j = 1; j < m; ++j) {
                const long long c = j + cost[m - j][k - 1] + cost[j][k];
                if (best < 0 || c < best) {
                    best = c;
                    bj = j;
                }
            }
            cost[m][k] = best;
            split[m][k] = bj;
        }
}

long long checkpoint_cost(int n, int snapshots) {
    const int s = std::max(0, std::min(snapshots, n) - 1);
    std::vector<std::vector<long long>> cost;
    std::vector<std::vector<int>> split;
    schedule_tables(n, s, cost, split);
    return cost[n][s];
}

// Reverse steps [a, b): x^a is in slot `slot`; `free_slots` slots above it
// are free.  The adjoint of x^b is in the adjoint fields (or is seeded when b
// is the last step).
void Sim::adj_reverse(int a, int b, int slot, int free_slots) {
    AdjState& S = *adj_;
    const long long N3 = 3 * g_.N;
    auto restore = [&](int sl) {
        launch_copy(ctx_, vel_.p, S.snaps.p + (size_t)sl * 2 * N3, N3);
        launch_copy(ctx_, gp_.p, S.snaps.p + (size_t)sl * 2 * N3 + N3, N3);
    };
    auto store = [&](int sl) {
        launch_copy(ctx_, S.snaps.p + (size_t)sl * 2 * N3, vel_.p, N3);
        launch_copy(ctx_, S.snaps.p + (size_t)sl * 2 * N3 + N3, gp_.p, N3);
    };
    const int n = b - a;
    if (n == 1) {
        restore(slot);
        adjoint_step_impl(b == S.nsteps);
        return;
    }
    if (free_slots == 0) {
        for (int k = b - 1; k >= a; --k) {
            restore(slot);
            for (int m = a; m < k; ++m, ++S.fwd_advances) forward_core();
            adjoint_step_impl(k + 1 == S.nsteps);
        }
        return;
    }
    const int j = S.split[n][free_slots];
    restore(slot);
    for (int m = 0; m < j; ++m, ++S.fwd_advances) forward_core();
    store(slot + 1);
    adj_reverse(a + j, b, slot + 1, free_slots - 1);
    adj_reverse(a, a + j, slot, free_slots);
}

// Forward nsteps from the current state with binomial checkpoints in HBM
// (`snapshots` slots of (velocity, gp), including the initial state), the
// objective at the final state, and the reverse sweep.  Returns J.  On return
// the forward state is the final state with the clock advanced by nsteps, the
// adjoint fields hold dJ/d(velocity, gp) of the initial state, and the disk
// thrust gradients are dJ/dct.
double Sim::adjoint_run(int nsteps, int snapshots) {
    adj_alloc();
    AdjState& S = *adj_;
    if (nsteps < 1) throw KsError(KS_ERR_ARG, "adjoint_run needs nsteps >= 1");
    if (snapshots < 1) throw KsError(KS_ERR_ARG, "adjoint_run needs at least one snapshot slot");
    if (!S.box_set) throw KsError(KS_ERR_ARG, "objective box not set");
    Clock c = t_;
    for (int m = 0; m < nsteps; ++m)
        if (!c.new_step()) throw KsError(KS_ERR_ARG, "nsteps runs past time.max_step / time.stop_time");
    const int slots = std::min(snapshots, nsteps);
    const long long N3 = 3 * g_.N;
    if (S.nslots < slots) {
        S.snaps.alloc((size_t)slots * 2 * N3);
        S.nslots = slots;
    }
    std::vector<std::vector<long long>> cost;
    schedule_tables(nsteps, slots - 1, cost, S.split);
    S.nsteps = nsteps;
    S.fwd_advances = 0;
    S.adj_steps = 0;
    ct_grad_.assign(disks_.size(), 0.0);
    const Clock clock = t_;
    launch_copy(ctx_, S.snaps.p, vel_.p, N3);
    launch_copy(ctx_, S.snaps.p + N3, gp_.p, N3);
    adj_reverse(0, nsteps, 0, slots - 1);
    // forward state: x^nsteps, as after nsteps Evolve steps
    launch_copy(ctx_, vel_.p, S.fu.p, N3);
    launch_copy(ctx_, gp_.p, S.fgp.p, N3);
    launch_copy(ctx_, p_.p, S.fp.p, (long long)p_.n);
    t_ = clock;
    for (int m = 0; m < nsteps; ++m) {
        t_.new_step();
        t_.next = t_.cur + t_.dt[0];
    }
    sync();
    return S.J;
}

double Sim::adjoint_stat(const std::string& n) const {
    if (!adj_) return 0.0;
    if (n == "adj_forward_steps") return (double)adj_->fwd_advances;
    if (n == "adj_reverse_steps") return (double)adj_->adj_steps;
    if (n == "adj_slots") return (double)adj_->nslots;
    if (n == "objective") return adj_->J;
    return 0.0;
}

}  // namespace ks
