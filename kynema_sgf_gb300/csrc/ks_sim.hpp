// Host-side state of one handle: deck, SimTime, actuator disks, device
// fields and the Sim class that sequences the device passes.  Shared by the
// forward driver (ks_host.cpp) and the reverse-mode driver (ks_adjoint_host.cpp).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ks.h"
#include "ks_launch.hpp"

namespace ks {

struct KsError : std::runtime_error {
    int code;
    KsError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        const int code = (e == cudaErrorMemoryAllocation) ? KS_ERR_OOM : KS_ERR_CUDA;
        throw KsError(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

inline std::string lc(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

// ---------------------------------------------------------------- deck
// ParmParse-style input: "prefix.key = v1 v2 ...", '#' starts a comment.
class Deck {
   public:
    explicit Deck(const std::string& text) {
        std::istringstream in(text);
        std::string ln;
        while (std::getline(in, ln)) {
            const auto hash = ln.find('#');
            if (hash != std::string::npos) ln.resize(hash);
            const auto eq = ln.find('=');
            if (eq == std::string::npos) continue;
            std::string k = trim(ln.substr(0, eq));
            std::istringstream vs(ln.substr(eq + 1));
            std::vector<std::string> v;
            for (std::string w; vs >> w;) {
                if (w.size() >= 2 && (w[0] == '"' || w[0] == '\'')) w = w.substr(1, w.size() - 2);
                v.push_back(w);
            }
            if (!k.empty()) kv_[k] = v;
        }
    }
    bool has(const std::string& k) const { return kv_.count(k) > 0; }
    bool has_prefix(const std::string& p) const {
        auto it = kv_.lower_bound(p);
        return it != kv_.end() && it->first.compare(0, p.size(), p) == 0;
    }
    std::vector<std::string> strs(const std::string& k) const {
        auto it = kv_.find(k);
        return it == kv_.end() ? std::vector<std::string>{} : it->second;
    }
    std::string str(const std::string& k, const std::string& def) const {
        auto v = strs(k);
        return v.empty() ? def : v[0];
    }
    double num(const std::string& k, double def) const {
        auto v = strs(k);
        return v.empty() ? def : std::stod(v[0]);
    }
    int flag(const std::string& k, int def) const {
        auto v = strs(k);
        if (v.empty()) return def;
        if (v[0] == "true") return 1;
        if (v[0] == "false") return 0;
        return std::stoi(v[0]);
    }
    std::vector<double> nums(const std::string& k) const {
        auto it = kv_.find(k);
        if (it == kv_.end()) throw KsError(KS_ERR_DECK, "missing deck key " + k);
        std::vector<double> r;
        for (auto& s : it->second) r.push_back(std::stod(s));
        return r;
    }

   private:
    static std::string trim(std::string s) {
        const auto a = s.find_first_not_of(" \t\r");
        if (a == std::string::npos) return "";
        const auto b = s.find_last_not_of(" \t\r");
        return s.substr(a, b - a + 1);
    }
    std::map<std::string, std::vector<std::string>> kv_;
};

// ---------------------------------------------------------------- SimTime
// src/core/SimTime.cpp:11-324 semantics for the keys on this path.
struct Clock {
    double cur = 0, next = 0, dt[3] = {0, 0, 0};  // SimTime::m_dt starts at 0 (SimTime.H:194-195)
    double cfl = 1, fixed_dt = -1, init_dt = -1, max_dt = -1, min_dt = -1, shrink = 0.1, growth = 0.1, stop = -1;
    int max_step = -1, step = 0;
    bool adaptive = false, init = true, force_cfl = true;
    double cur_cfl = 0, conv_cfl = 0, diff_cfl = 0, src_cfl = 0;

    void set_cfl(double conv, double diff, double src) {
        const double eps = 2.220446049250313e-16;
        const double cd = conv + diff;
        const double unit = cd + std::sqrt(cd * cd + 4.0 * src);
        bool use_init = false;
        if (adaptive && !init && unit < eps) {
            if (cur < eps && init_dt > 0) use_init = true;
            else throw KsError(KS_ERR_NONFINITE, "CFL is below machine epsilon and the time step is adaptive");
        }
        double d = use_init ? init_dt : 2.0 * cfl / std::max(unit, eps);
        if (init) d *= shrink;
        if (dt[0] > 0 && adaptive) d = std::min(d, (1.0 + growth) * dt[0]);
        if (adaptive) {
            if (max_dt > 0) d = std::min(d, max_dt);
            if (min_dt > 0 && d < min_dt) throw KsError(KS_ERR_NONFINITE, "adaptive dt fell below time.min_dt");
            if (stop > 0 && cur + d > stop) d = stop - cur;
            if (init && init_dt > 0) d = std::min(d, init_dt);
            dt[0] = d;
        } else {
            dt[0] = fixed_dt;
        }
        cur_cfl = 0.5 * unit * dt[0];
        conv_cfl = conv * dt[0];
        diff_cfl = diff * dt[0];
        src_cfl = std::sqrt(src) * dt[0];
    }
    bool keep_going() const {
        if (max_step >= 0 && step >= max_step) return false;
        if (stop > 0 && next >= stop - 2.220446049250313e-12) return false;
        return true;
    }
    bool new_step() {
        const bool go = keep_going();
        init = false;
        if (go) {
            dt[2] = dt[1];
            dt[1] = dt[0];
            ++step;
            cur = next;
        }
        return go;
    }
};

struct Disk {
    double center[3], normal[3], cvec[3];
    double sample[3];  // axis of the upstream sampling disk (sample_vec)
    double D, eps, to_sample, dr;
    std::vector<double> ct, ws;
    int nr, nt;
    bool about_center;
    double ct_now = 0, uinf2 = 0, ref[3] = {0, 0, 0};
};

struct MGParams {
    double rtol = 1.0e5 * 2.220446049250313e-16, atol = 1.0e2 * 2.220446049250313e-16;
    int maxiter = 200, nu1 = 2, nu2 = 2, bottom = 100;
    int fixed_iters = 1;  // MLMGOptions do_fixed_iters: stop at maxiter without an error
    int semi = 0;         // MLMGOptions do_semicoarsening (honoured by the MAC solve)
    int max_semi = 1 << 30;  // max_semicoarsening_level: coarsenings that may be partial
    double omega = 0.9;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        reset();
        n = count;
        ck(cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)), "cudaMalloc");
        ck(cudaMemset(p, 0, std::max<size_t>(1, count) * sizeof(T)), "cudaMemset");
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// ---------------------------------------------------------------- reverse mode
// Device state of the reverse sweep, allocated on the first adjoint call.
struct AdjState {
    DevBuf<double> gbuf;            // adjoints of the Godunov face arrays (AdjBufs)
    AdjBufs A{};
    DevBuf<double> ub, gpb;         // adjoints of (velocity, gp) at the current time level
    DevBuf<double> w, t1, t2, srcb, doldb, forcesb;  // 3N scratch
    DevBuf<double> mub, wgb;        // adjoints of mu_eff (N) and of the wall-model gradient (2 nx ny)
    DevBuf<double> cbuf;            // 9N scratch of the gather-form reverse passes
    DevBuf<double> umacb[3];        // adjoint of the MAC velocities
    DevBuf<double> gbuf2;           // post-MAC intermediates of the recompute (the pre-MAC ones stay in gb_)
    GodunovBufs gb2{};
    DevBuf<double> su, sgp, sp;     // forward state saved across a reverse step
    DevBuf<double> fu, fgp, fp;     // forward state at the end of an adjoint run
    DevBuf<double> snaps;           // binomial checkpoints, 6N values per slot
    int nslots = 0;
    DevBuf<double> pts, wb;         // disk points / sample adjoints
    int box_lo[3] = {0, 0, 0}, box_hi[3] = {-1, -1, -1};
    bool box_set = false;
    double J = 0.0;
    int nsteps = 0;
    long long fwd_advances = 0, adj_steps = 0;
    std::vector<std::vector<int>> split;  // optimal first split per (steps, free slots)
};

// An AMReX plot file (single level, one box) from host data: nvars = names.size()
// cell fields of n[0] n[1] n[2] values each, component-major, x fastest.
void write_plotfile_host(const std::string& dir, const std::vector<std::string>& names, const int n[3], const double plo[3], const double phi[3],
                         double time, int step, const double* data, const std::string& info);

// Fewest forward steps (beyond the one inside each reverse step) that reverse
// n steps with `snapshots` checkpoint slots, the first holding the initial state.
long long checkpoint_cost(int n, int snapshots);

// ---------------------------------------------------------------- simulation
class Sim {
   public:
    explicit Sim(const std::string& text);
    ~Sim();

    void init_data();
    void sources(const double* vel, const double* theta);
    void compute_dt();
    void pre_advance();
    void prepare_time_step();
    // ApplyPredictor of the deck's scheme (Godunov: the whole advance; MOL: its
    // predictor), ApplyCorrector (MOL only)
    void apply_predictor(bool incremental);
    void apply_corrector();
    void apply_projection(double time, double scaling, bool incremental);
    int step();
    bool godunov() const { return godunov_; }

    double scalar(const std::string& name);
    void layout(const std::string& name, ks_layout& L);
    void get(const std::string& name, void* dst, int where);
    void set(const std::string& name, const void* src, int where);
    void sync() { ck(cudaStreamSynchronize(ctx_.stream), "stream synchronize"); }

    // ---- reverse mode (ks_adjoint_host.cpp)
    void set_objective_box(const double lo[3], const double hi[3]);
    double objective(bool seed);
    void adjoint_step();
    double adjoint_run(int nsteps, int snapshots);
    void adjoint_reset();
    void set_disk_ct(const double* ct, int n);
    const std::vector<double>& ct_gradient() const { return ct_grad_; }
    int ndisks() const { return (int)disks_.size(); }
    double adjoint_stat(const std::string& name) const;

    // ---- plot files, checkpoints and restart (ks_io.cpp)
    void write_plotfile(const std::string& dir);
    void write_checkpoint(const std::string& dir);
    void read_checkpoint(const std::string& dir);
    // the plot / checkpoint files due at the current step (SimTime::write_plot_file,
    // write_checkpoint; last = the end-of-run rules write_last_plot_file / _checkpoint)
    void write_outputs(bool last);

    Ctx ctx_;
    Grid g_{};
    Clock t_;
    int mac_it_ = 0, nod_it_ = 0, dif_it_ = 0;
    double dif_r0_ = 0, dif_r_ = 0, dif_b_ = 0;
    int mixed_ = 0;  // 1: FP32 advection and multigrid cycles with FP64 defect correction
    GodunovBufs* adv_bufs_ = nullptr;  // post-MAC pass scratch when not gb_ (reverse-step recompute keeps both passes)
    double mac_r0_ = 0, mac_r_ = 0, nod_r0_ = 0, nod_r_ = 0;
    double mac_tgt_ = 0, nod_tgt_ = 0;  // stopping thresholds max(atol, rtol max(|rhs|, r0)) of the last solves
    std::string err_;

   private:
    void setup(const Deck& D);
    void alloc();
    void init_fields(const Deck& D);
    void abl_update();
    void actuator_update();
    void mac_project();
    double reduce(int np, int ncomp, int op_max, double* host);
    template <typename T>
    void cc_vcycle(std::vector<CCLevelT<T>>& Ls, size_t l, double beta, bool in_graph = false);
    template <typename T>
    void nd_vcycle(std::vector<NDLevelT<T>>& Ls, size_t l, double sigma, int skip_sweeps = 0, bool in_graph = false);
    // The launch-bound coarse tail of a V-cycle (levels >= glev_) recorded once
    // as a CUDA graph and replayed; re-recorded when its scalar key changes.
    struct MGGraph {
        cudaGraphExec_t exec = nullptr;
        long long nodes = 0;
        double key = 0.0;
    };
    MGGraph gcc_[2], gnd_[2];  // [FP64, FP32] MAC and nodal tails
    size_t glev_ = 0;          // first graphed level (0: none)
    int mg_graphs_ = 1;        // ks.mg_graphs
    int mg_inner_ = 2;         // ks.mixed_inner_cycles (MAC)
    int mg_inner_nd_ = 4;      // ks.mixed_inner_cycles_nodal (at most; see nd_solve)
    double nod_rho_ = 0.0;     // last measured FP32 nodal V-cycle contraction (0: none yet)
    bool nod_zero_ = false;    // nd_rhs zero-filled the finest nodal phi for the next solve
    template <typename F>
    void mg_graph_run(MGGraph& G, double key, F&& body);
   public:
    void set_mixed(int on);

   private:
    double* field(const std::string& name, int& ncomp, int& kind);
    void nd_rhs(const double* cell_field, bool from_pressure = false);
    void nd_solve(double sigma);
    void mol_predictor(bool incremental);
    void diff_alloc();
    void diffuse_solve(double dtd);
    void diff_vcycle(size_t l, double dtd);
    void temperature_predictor(double dt);
    void temperature_mol(bool corrector, double dt);
    void tdiffuse_solve(double dtd);
    void abl_forcing_update();
    ScalarBC tbc() const { return ScalarBC{tzlo_, tzhi_, tgz_.p, tgtop_}; }
    std::vector<std::pair<std::string, int>> plot_fields() const;
    std::vector<double> host_field(const std::string& name, int nc);
    std::string info_text() const;
    std::string deck_text_, restart_file_, plt_prefix_ = "plt", chk_prefix_ = "chk";
    int plot_interval_ = -1, chk_interval_ = -1, plot_start_ = 0, chk_start_ = 0;
    double diff_fac() const { return diff_type_ == 0 ? 1.0 : (diff_type_ == 1 ? 0.5 : 0.0); }
    void disk_points(const Disk& d, std::vector<double>& sample, std::vector<double>& ring) const;
    // reverse mode
    void adj_check() const;
    void adj_alloc();
    void forward_core();
    void adjoint_step_impl(bool seed);
    void adjoint_disks(const double* srcb);
    void adj_reverse(int a, int b, int slot, int free_slots);
    std::unique_ptr<AdjState> adj_;
    std::vector<double> ct_grad_;

    double plo_[3], phi_[3];
    double rho_ = 1, mu_ = 0;
    Scalars S_{};
    bool wallmodel_ = false;
    int shear_ = 0;
    double kappa_ = 0.41, z0_ = 0.1, zref_ = 0, utau_ = 0, um_[2] = {0, 0}, vmag_ = 0;
    std::vector<Disk> disks_;
    MGParams mac_, nod_;
    int initial_proj_ = 1, initial_iters_ = 3;
    bool godunov_ = true;  // incflo.use_godunov; false: MOL predictor-corrector
    int diff_type_ = 1;    // incflo.diffusion_type: 0 explicit, 1 Crank-Nicolson, 2 implicit
    MGParams dif_;         // tensor diffusion solve (prefixes diffusion, velocity_diffusion)
    // one level of the diffusion solve's multigrid: grid, iterate, right-hand
    // side, residual, sweep target, cell viscosity, inverse diagonal
    struct DiffLevel {
        Grid g;
        double *x, *b, *r, *t, *mu, *dinv;
        double omega;  // Jacobi weight of the level's sweeps
    };
    std::vector<DiffLevel> dl_;
    DevBuf<double> dbuf_, dtmp_, dparts_;

    DevBuf<double> vel_, vel_old_, vel_tmp_, gp_, p_, src_, forces_, mueff_, divtau_, conv_, act_, wg_;
    DevBuf<double> conv_old_;  // MOL: conv_term(Old) of the predictor
    // temperature transport (ABL physics with a temperature profile)
    bool temp_ = false;
    int tzlo_ = 0, tzhi_ = 0;  // 0 Neumann 0, 1 wall-model heat flux, 2 fixed gradient
    double tgtop_ = 0.0, z0t_ = 0.1, theta_mean_ = 0.0;
    double ablf_h_ = 0.0, ablf_target_[2] = {0.0, 0.0};
    int tdif_it_ = 0;
    MGParams tdif_;
    DevBuf<double> theta_, theta_old_, theta_nph_, alpha_, tdiff_, tconv_, ttmp_, tb_, tdinv_, tgz_, tprof_, layer_, tparts_;
    DevBuf<double> tconv_old_;  // MOL: the scalar's conv_term(Old)
    DevBuf<double> umac_[3];
    DevBuf<double> gbuf_;
    GodunovBufs gb_{};
    std::vector<CCLevelDev> cc_;
    std::vector<NDLevelDev> nd_;
    std::vector<CCLevelT<float>> cc32_;  // mixed precision: FP32 cycle levels
    std::vector<NDLevelT<float>> nd32_;
    DevBuf<double> mgbuf_;
    DevBuf<float> mgbuf32_;
    // direct bottom solves: pinned inverses of the coarsest MAC and nodal operators
    std::vector<double> binv_cc_h_, binv_nd_h_;
    DevBuf<double> binv_;
    DevBuf<float> binv32_;
    DevBuf<float> g32_;  // mixed precision: FP32 copies of the advection inputs
    GodunovIn32 in32_{};
    void bottom_setup();
    // MAC semicoarsening (mac_proj.do_semicoarsening): the MAC solve's own
    // hierarchy, used in place of cc_ / cc32_ when some coarsening is partial.
    // Its level 0 shares cc_[0]'s (and cc32_[0]'s) arrays; cc_ keeps the full
    // coarsening the diffusion solve and the nodal sizes follow.
    void mac_semi_setup();
    void mac_semi_mixed();
    bool mac_semi_ = false;
    size_t glev_s_ = 0;  // first graphed level of ccs_ (0: none)
    std::vector<CCLevelDev> ccs_;
    std::vector<CCLevelT<float>> ccs32_;
    std::vector<double> binv_ccs_h_;
    DevBuf<double> mgbufs_, binvs_;
    DevBuf<float> mgbufs32_, binvs32_;
    int mg_warm_ = 1;          // ks.mg_warm_start
    bool mac_prev_ok_ = false; // mac_phi_prev_ holds the last MAC potential
    DevBuf<double> mac_phi_prev_;
    double nod_bnorm_ = 0.0;   // |rhs| of a warm-started nodal solve (0: zero start)
    DevBuf<double> parts_, red_;
    DevBuf<double> pts_, samp_;
    double* hred_ = nullptr;  // pinned
};

}  // namespace ks
