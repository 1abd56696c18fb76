/*
 * ks_oracle.cpp -- CPU oracle (TEST INFRASTRUCTURE, never shipped, never
 * called by the product library).
 *
 * A plain C++/OpenMP FP64 restatement of Kynema-SGF's single-level
 * incompressible advance on a uniform single-box grid:
 *   incflo::advance -> ApplyPredictor (Godunov, explicit diffusion) ->
 *   ApplyProjection, preceded by compute_dt and the ABL / actuator
 *   pre-advance work, and InitData's initial projection and pressure
 *   iterations.
 *
 * The code is written AMReX-style on purpose (arrays with ghost cells, a
 * fill-patch step before each stencil pass, one loop nest per pass) so that it
 * stays structurally independent of the CUDA product, which keeps no ghost
 * cells and applies boundary conditions inside its kernels.
 *
 * Parity status: partially pinned.  The pieces that live in Kynema-SGF's own
 * sources (strain rate, Smagorinsky, sources, RHS assembly, RK2 correction,
 * CFL / SimTime, wall model, actuator disk) follow the cited files and are
 * checked against the known answers of the reference's unit tests.  The pieces
 * that live in the absent AMReX / AMReX-Hydro submodules (PPM Godunov, MAC and
 * nodal projectors, tensor operator, multigrid) are restatements of the
 * published methods (Colella & Woodward 1984 PPM; Almgren, Bell & Szymczak
 * unsplit Godunov with corner transport; Q1 finite-element nodal projection;
 * cell-centred and nodal geometric multigrid) -- parity unpinned there.
 *
 * Reference files cited below are paths inside the Kynema-SGF repository.
 */
#include "ks_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace kso {

constexpr double kPi = 3.14159265358979323846;
constexpr double kSmallVel = 1.0e-8;  // AMReX-Hydro small_vel
constexpr double kEps = 2.220446049250313e-16;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
enum { OK = 0, ERR_DECK = 1, ERR_UNSUPPORTED = 2, ERR_NOT_CONVERGED = 3,
       ERR_NONFINITE = 4, ERR_ARG = 6, DONE = 7 };

// ---------------------------------------------------------------- deck
// ParmParse-style "prefix.key = v1 v2 ..." lines, '#' comments.
struct Deck {
    std::map<std::string, std::vector<std::string>> kv;
    void parse(const std::string& text) {
        std::istringstream is(text);
        std::string line;
        while (std::getline(is, line)) {
            auto h = line.find('#');
            if (h != std::string::npos) line = line.substr(0, h);
            auto e = line.find('=');
            if (e == std::string::npos) continue;
            std::string key = line.substr(0, e);
            key.erase(0, key.find_first_not_of(" \t\r"));
            key.erase(key.find_last_not_of(" \t\r") + 1);
            std::istringstream vs(line.substr(e + 1));
            std::vector<std::string> vals;
            std::string v;
            while (vs >> v) {
                if (v.size() >= 2 && (v.front() == '"' || v.front() == '\'')) v = v.substr(1, v.size() - 2);
                vals.push_back(v);
            }
            if (!key.empty()) kv[key] = vals;
        }
    }
    bool has(const std::string& k) const { return kv.count(k) != 0; }
    bool has_prefix(const std::string& p) const {
        auto it = kv.lower_bound(p);
        return it != kv.end() && it->first.compare(0, p.size(), p) == 0;
    }
    const std::vector<std::string>& raw(const std::string& k) const {
        auto it = kv.find(k);
        if (it == kv.end()) throw Error(ERR_DECK, "missing deck key " + k);
        return it->second;
    }
    double d(const std::string& k, double def) const {
        return has(k) ? std::stod(raw(k).at(0)) : def;
    }
    int i(const std::string& k, int def) const {
        if (!has(k)) return def;
        const std::string& s = raw(k).at(0);
        if (s == "true") return 1;
        if (s == "false") return 0;
        return std::stoi(s);
    }
    std::string s(const std::string& k, const std::string& def) const {
        return has(k) && !raw(k).empty() ? raw(k)[0] : def;
    }
    std::vector<double> v(const std::string& k) const {
        std::vector<double> r;
        for (auto& x : raw(k)) r.push_back(std::stod(x));
        return r;
    }
    std::vector<std::string> sv(const std::string& k) const {
        return has(k) ? raw(k) : std::vector<std::string>{};
    }
};

static std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

// ---------------------------------------------------------------- arrays
// A box-indexed multi-component array (AMReX Array4 order: x fastest).
struct Arr {
    int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1}, nc = 0;
    long sy = 0, sz = 0, sc = 0;
    std::vector<double> d;
    void define(int l0, int l1, int l2, int h0, int h1, int h2, int ncomp) {
        lo[0] = l0; lo[1] = l1; lo[2] = l2; hi[0] = h0; hi[1] = h1; hi[2] = h2; nc = ncomp;
        sy = h0 - l0 + 1; sz = sy * (h1 - l1 + 1); sc = sz * (h2 - l2 + 1);
        d.assign((size_t)(sc * nc), 0.0);
    }
    inline double& operator()(int i, int j, int k, int n = 0) {
        return d[(size_t)(n * sc + (k - lo[2]) * sz + (j - lo[1]) * sy + (i - lo[0]))];
    }
    inline double operator()(int i, int j, int k, int n = 0) const {
        return d[(size_t)(n * sc + (k - lo[2]) * sz + (j - lo[1]) * sy + (i - lo[0]))];
    }
    void setval(double v) { std::fill(d.begin(), d.end(), v); }
};

enum ZBC { ZPER = 0, SLIP = 1, WALLMODEL = 2 };

struct Geo {
    int n[3];
    double plo[3], phi[3], dx[3];
    bool per[3];
    int zlo, zhi;
};

// Cell-centred array on [0,n-1] grown by ng.
static void def_cc(Arr& a, const Geo& g, int ng, int nc) {
    a.define(-ng, -ng, -ng, g.n[0] - 1 + ng, g.n[1] - 1 + ng, g.n[2] - 1 + ng, nc);
}

// Periodic wrap of every ghost point in the periodic directions.  Points whose
// non-periodic coordinate lies outside the valid range keep their value, so the
// caller fills non-periodic ghosts first over the valid (x,y) range.
// nodal[d] = 1 if the array is node/face-centred in direction d.
static void fill_periodic(Arr& a, const Geo& g, const int nodal[3]) {
    const int nvalid[3] = {g.n[0] + (g.per[0] ? 0 : nodal[0]), g.n[1] + (g.per[1] ? 0 : nodal[1]),
                           g.n[2] + (g.per[2] ? 0 : nodal[2])};
    for (int n = 0; n < a.nc; ++n)
#pragma omp parallel for collapse(2)
        for (int k = a.lo[2]; k <= a.hi[2]; ++k)
            for (int j = a.lo[1]; j <= a.hi[1]; ++j)
                for (int i = a.lo[0]; i <= a.hi[0]; ++i) {
                    int c[3] = {i, j, k};
                    bool ghost = false;
                    for (int d = 0; d < 3; ++d) {
                        if (!g.per[d]) continue;
                        int hiv = g.n[d] - 1 + nodal[d];
                        if (c[d] < 0 || c[d] > hiv) {
                            ghost = true;
                            c[d] = ((c[d] % g.n[d]) + g.n[d]) % g.n[d];
                        }
                    }
                    (void)nvalid;
                    if (ghost) a(i, j, k, n) = a(c[0], c[1], c[2], n);
                }
}

// ---------------------------------------------------------------- params
struct DiskParams {
    std::string label;
    double center[3] = {0, 0, 0}, normal[3] = {0, 1, 0}, sample[3] = {0, 1, 0};
    double diameter = 0, epsilon = 0, diameters_to_sample = 0;
    std::vector<double> ct, wind_speed;
    int nr = 1, nt = 1;
    bool about_center = false;
    // derived / state
    double cvec[3] = {0, 0, 0}, dr = 0;
    double current_ct = 0, uinf_sqr = 0, ref_vel[3] = {0, 0, 0};
};

struct MGOpts {
    double rtol = 1.0e5 * kEps, atol = 1.0e2 * kEps;
    int maxiter = 200, nu1 = 2, nu2 = 2, bottom = 100;
    double omega = 0.9;  // nodal Jacobi weight
    int fixed_iters = 1;  // MLMGOptions do_fixed_iters: stop at maxiter without an error
    int semicoarsening = 0, max_semi = 1 << 30;  // do_semicoarsening, max_semicoarsening_level
};

struct SimTime {
    double cur = 0, newt = 0, dt[3] = {0, 0, 0};  // SimTime::m_dt starts at 0 (SimTime.H:194-195)
    double max_cfl = 1, fixed_dt = -1, init_dt = -1, max_dt = -1, min_dt = -1;
    double init_shrink = 0.1, growth = 0.1, stop_time = -1, dt_calc = 0;
    int max_step = -1, step = 0;
    bool adaptive = false, is_init = true, use_force_cfl = true;
    double conv_cfl = 0, diff_cfl = 0, src_cfl = 0, cur_cfl = 0;

    // src/core/SimTime.cpp:162-291
    void set_current_cfl(double conv, double diff, double src) {
        bool use_init_dt = false;
        const double cd = conv + diff;
        const double cfl_unit = cd + std::sqrt(cd * cd + 4.0 * src);
        if (adaptive && !is_init && cfl_unit < kEps) {
            if (cur < kEps && init_dt > 0) use_init_dt = true;
            else throw Error(ERR_ARG, "CFL below machine epsilon with adaptive dt");
        }
        double dtn = use_init_dt ? init_dt : 2.0 * max_cfl / std::max(cfl_unit, kEps);
        if (is_init) dtn *= init_shrink;
        if (dt[0] > 0 && adaptive) dtn = std::min(dtn, (1.0 + growth) * dt[0]);
        if (adaptive) {
            if (max_dt > 0) dtn = std::min(dtn, max_dt);
            if (min_dt > 0 && dtn < min_dt) throw Error(ERR_NONFINITE, "dt below min_dt");
            if (stop_time > 0 && cur + dtn > stop_time) dtn = stop_time - cur;
            if (is_init && init_dt > 0) dtn = std::min(dtn, init_dt);
            dt[0] = dtn;
        } else {
            dt[0] = fixed_dt;
        }
        cur_cfl = 0.5 * cfl_unit * dt[0];
        conv_cfl = conv * dt[0];
        diff_cfl = diff * dt[0];
        src_cfl = std::sqrt(src) * dt[0];
        dt_calc = dtn;
    }
    void advance_time() { newt = cur + dt[0]; }
    bool continue_sim() const {
        const double eps = kEps * 1.0e4;
        if (max_step >= 0 && step >= max_step) return false;
        if (stop_time > 0 && newt >= stop_time - eps) return false;
        return true;
    }
    bool new_timestep() {
        bool c = continue_sim();
        is_init = false;
        if (c) {
            dt[2] = dt[1];
            dt[1] = dt[0];
            ++step;
            cur = newt;
        }
        return c;
    }
};

// ---------------------------------------------------------------- simulation
struct Sim {
    Deck deck;
    Geo g;
    double rho = 1.0, mu = 0.0;
    bool smag = false;
    double Cs = 0.135;
    std::string physics;
    bool src_geo = false, src_cor = false, src_body = false, src_act = false;
    // temperature transport (ABL physics with a temperature profile)
    bool has_temp = false, src_bous = false, src_ablf = false;
    double gravity[3] = {0.0, 0.0, -9.81};
    double Pr = 1.0, Prt = 1.0, T_ref = -1.0, beta_T = 0.0;
    double z0t = 0.1, theta_mean = 0.0;
    int tzlo = 0, tzhi = 0;     // temperature z BCs: 0 Neumann 0, 1 wall model heat flux, 2 fixed gradient
    double tgrad_hi = 0.0;      // fixed gradient at zhi
    double ablf_height = 0.0, ablf_target[2] = {0.0, 0.0}, ablf_force[2] = {0.0, 0.0};
    double lat = 90.0, rot_period = 86164.091;
    double east[3] = {1, 0, 0}, north[3] = {0, 1, 0}, up[3] = {0, 0, 1};
    bool cor_horizontal = false;
    double geo_wind[3] = {0, 0, 0}, body_force[3] = {0, 0, 0};
    bool body_osc = false;
    double body_omega = 0;
    double kappa = 0.41, z0 = 0.1;
    std::string shear_type = "moeng";
    double utau = 0, umean[2] = {0, 0}, vmag_mean = 0, zref = 0;
    std::vector<DiskParams> disks;
    MGOpts mac, nod, dif;  // dif: the tensor diffusion solve (prefixes diffusion, velocity_diffusion)
    MGOpts tdif;           // the temperature diffusion solve (prefixes diffusion, temperature_diffusion)
    int tdiff_iters = 0;
    int do_initial_proj = 1, initial_iterations = 3;
    bool godunov = true;  // incflo.use_godunov; false selects the MOL predictor-corrector
    int diff_type = 1;    // incflo.diffusion_type: 0 explicit, 1 Crank-Nicolson, 2 implicit
    SimTime t;
    std::string err;

    // fields
    Arr vel, vel_old, gp, p, src, forces, mueff, divtau, divtau_new, conv, conv_old, act_src;
    Arr theta, theta_old, theta_nph, alpha, tsrc, tdiff, tdiff_new, tconv, tconv_old;
    Arr umac, vmac, wmac;
    int mac_iters = 0, nodal_iters = 0;
    std::vector<std::array<int, 3>> mac_dims;  // cells per level of the last MAC hierarchy
    double mac_res0 = 0, mac_res = 0, nodal_res0 = 0, nodal_res = 0;
    int diff_iters = 0;
    double diff_res0 = 0, diff_res = 0, diff_bnorm = 0;

    void setup(const std::string& text);
    void init_fields();
    // passes
    void fill_vel(Arr& v) const;
    void fill_cc_foextrap(Arr& a) const;
    void update_mueff(Arr& v);
    void compute_sources(const Arr& v, const Arr* th = nullptr);
    void fill_scalar(Arr& a) const;
    void theta_wall_gradient(std::vector<double>& gz) const;
    void tdiff_op(const Arr& th_in, Arr& out);
    void temperature_predictor(double dt);
    void tdiffuse_solve(double dtd);
    void abl_forcing_update();
    void wall_gradient(std::vector<double>& gx, std::vector<double>& gy) const;
    void divtau_op(const Arr& v_in, Arr& out);
    void premac(double dt);
    void mac_project();
    void advection(double dt);
    void advect_field(const Arr& q, const Arr& fq, int normal, double dt, Arr& out);
    void nodal_project(double time, double scaling, bool incremental);
    void compute_dt();
    void abl_update_umean();
    void actuator_update();
    void apply_predictor(bool incremental);
    void mol_extrap(Arr& v);
    void mol_conv(Arr& v, Arr& out);
    void mol_conv_field(const Arr& q, int normal, Arr& out);
    void temperature_mol(bool corrector, double dt);
    void mol_predictor(bool incremental);
    void mol_corrector();
    void diffuse_solve(double dtd);
    void init_data();
    int step_once();
    double ke() const;
    double divu(double* umax) const;
    void predictor_rhs(double dt, double fac);
    void explicit_rk2_post_hoc(double dt, const Arr& d);
    double mac_divu(double* umax) const;
};

// ---- setup -----------------------------------------------------------------
void Sim::setup(const std::string& text) {
    deck.parse(text);
    const Deck& D = deck;
    auto nc = D.v("amr.n_cell");
    auto plo = D.v("geometry.prob_lo");
    auto phi = D.v("geometry.prob_hi");
    auto per = D.v("geometry.is_periodic");
    if (D.i("amr.max_level", 0) != 0) throw Error(ERR_UNSUPPORTED, "only amr.max_level = 0");
    for (int d = 0; d < 3; ++d) {
        g.n[d] = (int)nc.at(d);
        g.plo[d] = plo.at(d);
        g.phi[d] = phi.at(d);
        g.dx[d] = (g.phi[d] - g.plo[d]) / g.n[d];
        g.per[d] = per.at(d) != 0;
    }
    if (!g.per[0] || !g.per[1]) throw Error(ERR_UNSUPPORTED, "x and y must be periodic");
    g.zlo = g.zhi = ZPER;
    if (!g.per[2]) {
        auto bt = [&](const std::string& k) {
            std::string s = lower(D.s(k, ""));
            if (s == "slip_wall") return (int)SLIP;
            if (s == "wall_model") return (int)WALLMODEL;
            throw Error(ERR_UNSUPPORTED, "unsupported " + k + " = " + s);
        };
        g.zlo = bt("zlo.type");
        g.zhi = bt("zhi.type");
        if (g.zhi == WALLMODEL) throw Error(ERR_DECK, "ABL wall models are not applicable to a zhi BC");
        if (g.n[2] < 4) throw Error(ERR_UNSUPPORTED, "wall-bounded z needs >= 4 cells");
    }
    for (int d = 0; d < 3; ++d)
        if (g.n[d] % 2 != 0 || g.n[d] < 4) throw Error(ERR_UNSUPPORTED, "cell counts must be even and at least 4");

    rho = D.d("incflo.density", 1.0);
    mu = D.d("transport.viscosity", 0.0);
    godunov = D.i("incflo.use_godunov", 1) != 0;
    if (godunov) {
        std::string gt = lower(D.s("incflo.godunov_type", "weno_z"));
        if (gt != "ppm") throw Error(ERR_UNSUPPORTED, "only incflo.godunov_type = ppm");
        if (D.i("incflo.godunov_use_forces_in_trans", 0) != 0) throw Error(ERR_UNSUPPORTED, "forces_in_trans");
    }
    // src/setup/init.cpp:60-76 (the default is Crank-Nicolson)
    diff_type = D.i("incflo.diffusion_type", 1);
    if (diff_type < 0 || diff_type > 2)
        throw Error(ERR_DECK, "We currently require diffusion_type = 0 for explicit, 1 for Crank-Nicolson or 2 for implicit");
    if (D.i("incflo.icns_conserv", 1) != 1) throw Error(ERR_UNSUPPORTED, "icns_conserv = 0");
    do_initial_proj = D.i("incflo.do_initial_proj", 1);
    initial_iterations = D.i("incflo.initial_iterations", 3);
    physics = D.s("incflo.physics", "");
    std::string tm = lower(D.s("turbulence.model", "laminar"));
    if (tm == "smagorinsky") smag = true;
    else if (tm != "laminar") throw Error(ERR_UNSUPPORTED, "turbulence.model " + tm);
    Cs = D.d("Smagorinsky_coeffs.Cs", 0.135);

    for (auto& s : D.sv("ICNS.source_terms")) {
        if (s == "GeostrophicForcing") src_geo = true;
        else if (s == "CoriolisForcing") src_cor = true;
        else if (s == "BodyForce") src_body = true;
        else if (s == "ActuatorForcing") src_act = true;
        else if (s == "BoussinesqBuoyancy") src_bous = true;
        else if (s == "ABLForcing") src_ablf = true;
        else throw Error(ERR_UNSUPPORTED, "source term " + s);
    }
    rot_period = D.d("CoriolisForcing.rotational_time_period", 86164.091);
    if (src_geo || src_cor) lat = D.v("CoriolisForcing.latitude").at(0);
    if (D.has("CoriolisForcing.east_vector")) { auto e = D.v("CoriolisForcing.east_vector"); for (int d = 0; d < 3; ++d) east[d] = e.at(d); }
    if (D.has("CoriolisForcing.north_vector")) { auto e = D.v("CoriolisForcing.north_vector"); for (int d = 0; d < 3; ++d) north[d] = e.at(d); }
    auto nrm = [](double* v) { double m = std::sqrt(v[0]*v[0]+v[1]*v[1]+v[2]*v[2]); for (int d = 0; d < 3; ++d) v[d] /= m; };
    nrm(east); nrm(north);
    up[0] = east[1]*north[2]-east[2]*north[1]; up[1] = east[2]*north[0]-east[0]*north[2]; up[2] = east[0]*north[1]-east[1]*north[0];
    cor_horizontal = D.i("CoriolisForcing.is_horizontal", 0) != 0;
    if (src_geo) { auto w = D.v("GeostrophicForcing.geostrophic_wind"); for (int d = 0; d < 3; ++d) geo_wind[d] = w.at(d); }
    if (src_body) {
        // BodyForce::BodyForce (src/equation_systems/icns/source_terms/BodyForce.cpp:20-58):
        // uniform_constant (default) or oscillatory with angular_frequency
        const std::string bt = lower(D.s("BodyForce.type", "uniform_constant"));
        if (bt == "height_varying" || bt == "height-varying" || bt == "uniform_timetable" || D.has("BodyForce.uniform_timetable_file"))
            throw Error(ERR_UNSUPPORTED, "BodyForce.type " + bt);
        if (bt != "uniform_constant" && bt != "oscillatory") throw Error(ERR_DECK, "BodyForce.type " + bt);
        auto m = D.v("BodyForce.magnitude"); for (int d = 0; d < 3; ++d) body_force[d] = m.at(d);
        body_osc = bt == "oscillatory";
        if (body_osc) body_omega = D.v("BodyForce.angular_frequency").at(0);
    }
    kappa = D.d("ABL.kappa", 0.41);
    z0 = D.d("ABL.surface_roughness_z0", 0.1);
    shear_type = lower(D.s("ABL.wall_shear_stress_type", "moeng"));
    if (shear_type != "moeng" && shear_type != "constant" && shear_type != "local" && shear_type != "schumann")
        throw Error(ERR_UNSUPPORTED, "ABL.wall_shear_stress_type " + shear_type);
    zref = D.has("ABL.log_law_height") ? D.d("ABL.log_law_height", 0) : 0.5 * g.dx[2];
    if (std::fabs(zref - 0.5 * g.dx[2]) > 1e-12 * g.dx[2] && g.zlo == WALLMODEL)
        throw Error(ERR_UNSUPPORTED, "ABL.log_law_height other than the first cell centre");

    // Temperature transport: the ABL physics registers the Temperature PDE
    // (src/wind_energy/ABL.cpp:27-28); here it is advanced when the deck gives the
    // initial profile (ABL.temperature_heights, required by ABLFieldInit.cpp:96-99).
    has_temp = physics == "ABL" && D.has("ABL.temperature_heights");
    if (D.has("incflo.gravity")) { auto gv = D.v("incflo.gravity"); for (int d = 0; d < 3; ++d) gravity[d] = gv.at(d); }
    Pr = D.d("transport.laminar_prandtl", 1.0);   // ConstTransport.H:20-95
    Prt = D.d("transport.turbulent_prandtl", 1.0);
    T_ref = D.d("transport.reference_temperature", -1.0);
    if (src_bous) {
        if (!has_temp) throw Error(ERR_DECK, "BoussinesqBuoyancy needs the temperature field (ABL.temperature_heights)");
        beta_T = D.has("transport.thermal_expansion_coefficient") ? D.d("transport.thermal_expansion_coefficient", 0.0) : 1.0 / T_ref;
        if (T_ref < 0.0) throw Error(ERR_DECK, "Reference temperature was not set");
    }
    if (src_ablf) {  // ABLForcing.cpp:13-60
        if (physics != "ABL") throw Error(ERR_DECK, "ABLForcing needs the ABL physics");
        ablf_height = D.v("ABLForcing.abl_forcing_height").at(0);
        if (D.has("ABLForcing.velocity_timetable")) throw Error(ERR_UNSUPPORTED, "ABLForcing.velocity_timetable");
        auto tv = D.v("incflo.velocity");
        ablf_target[0] = tv.at(0);
        ablf_target[1] = tv.at(1);
    }
    if (has_temp) {
        if (D.has("ABL.surface_temp_rate") || D.has("ABL.surface_temp_timetable") ||
            std::fabs(D.d("ABL.surface_temp_flux", 0.0)) > 0.0)
            throw Error(ERR_UNSUPPORTED, "non-neutral surface temperature forcing (only ABL.surface_temp_flux = 0)");
        if (D.i("ABL.perturb_temperature", 0)) throw Error(ERR_UNSUPPORTED, "ABL.perturb_temperature (random perturbations)");
        z0t = D.d("ABL.surface_roughness_z0t", z0);
        // temperature BCs (BCInterface.cpp:289-350, incflo_diffusion.cpp:71-104): a face's
        // <face>.temperature_type overrides its velocity BC type
        auto tbc = [&](const char* face, int zbc) {
            const std::string key = std::string(face) + ".temperature_type";
            std::string t = lower(D.s(key, zbc == WALLMODEL ? "wall_model" : "slip_wall"));
            if (t == "wall_model") return 1;
            if (t == "fixed_gradient") return 2;
            if (t == "slip_wall" || t == "zero_gradient" || t == "symmetric_wall") return 0;
            throw Error(ERR_UNSUPPORTED, key + " = " + t);
        };
        if (!g.per[2]) {
            tzlo = tbc("zlo", g.zlo);
            tzhi = tbc("zhi", g.zhi);
            if (tzhi == 1) throw Error(ERR_DECK, "ABL wall models are not applicable to a zhi BC");
            if (tzlo == 1 && g.zlo != WALLMODEL) throw Error(ERR_UNSUPPORTED, "temperature wall model without the velocity wall model");
            if (tzlo == 2) throw Error(ERR_UNSUPPORTED, "zlo fixed_gradient temperature");
            if (tzhi == 2) tgrad_hi = D.v("zhi.temperature").at(0);
        }
    }

    auto rd = [&](MGOpts& o, const std::string& pfx) {
        o.rtol = D.d(pfx + ".mg_rtol", o.rtol);
        o.atol = D.d(pfx + ".mg_atol", o.atol);
        o.maxiter = D.i(pfx + ".maxiter", o.maxiter);
        o.nu1 = D.i(pfx + ".num_pre_smooth", o.nu1);
        o.nu2 = D.i(pfx + ".num_post_smooth", o.nu2);
        o.fixed_iters = D.i(pfx + ".do_fixed_iters", o.fixed_iters);
        o.semicoarsening = D.i(pfx + ".do_semicoarsening", o.semicoarsening);
        o.max_semi = D.i(pfx + ".max_semicoarsening_level", o.max_semi);
    };
    rd(mac, "mac_proj");
    rd(nod, "nodal_proj");
    rd(dif, "diffusion");  // MLMGOptions(default prefix, custom prefix), MLMGOptions.cpp:8-13
    rd(dif, "velocity_diffusion");
    rd(tdif, "diffusion");
    rd(tdif, "temperature_diffusion");

    t.stop_time = D.d("time.stop_time", -1);
    t.max_step = D.i("time.max_step", -1);
    t.fixed_dt = D.d("time.fixed_dt", -1);
    t.init_dt = D.d("time.initial_dt", -1);
    t.max_dt = D.d("time.max_dt", -1);
    t.min_dt = D.d("time.min_dt", -1);
    t.init_shrink = D.d("time.init_shrink", 0.1);
    t.growth = D.d("time.max_dt_growth", 0.1);
    t.max_cfl = D.d("time.cfl", 1.0);
    t.use_force_cfl = D.i("time.use_force_cfl", 1) != 0;
    if (t.fixed_dt > 0) t.dt[0] = t.fixed_dt; else t.adaptive = true;
    // src/setup/init.cpp:78-88
    if (!godunov && t.max_cfl > 0.5) throw Error(ERR_DECK, "We currently require cfl <= 0.5 when using the MOL advection scheme");
    if (godunov && t.max_cfl > 1.0) throw Error(ERR_DECK, "We currently require cfl <= 1.0 when using the Godunov advection scheme");

    // actuators: src/wind_energy/actuator/disk/disk_ops.cpp:182-276
    if (src_act) {
        for (auto& lab : D.sv("Actuator.labels")) {
            DiskParams dp;
            dp.label = lab;
            std::string type = D.s("Actuator." + lab + ".type", D.s("Actuator.type", ""));
            if (type != "UniformCtDisk") throw Error(ERR_UNSUPPORTED, "actuator type " + type);
            auto key = [&](const std::string& k) {
                std::string a = "Actuator." + lab + "." + k;
                return D.has(a) ? a : "Actuator." + type + "." + k;
            };
            dp.diameter = D.d(key("rotor_diameter"), 0);
            dp.epsilon = D.d(key("epsilon"), 0);
            dp.ct = D.v(key("thrust_coeff"));
            if (D.has(key("wind_speed"))) dp.wind_speed = D.v(key("wind_speed"));
            if (dp.ct.size() == 1) dp.wind_speed = {1.0};
            if (dp.wind_speed.size() != dp.ct.size()) throw Error(ERR_DECK, "wind_speed / thrust_coeff sizes");
            dp.nr = D.i(key("num_points_r"), 1);
            dp.nt = D.i(key("num_points_t"), 1);
            if (lower(D.s(key("spreading_type"), "LinearBasis")) != "uniformgaussian")
                throw Error(ERR_UNSUPPORTED, "only spreading_type = UniformGaussian");
            // ops::base::check_for_parse_conflicts (disk_ops.cpp:278-300)
            const char* pairs[6][2] = {{"disk_normal", "yaw"}, {"disk_normal", "tilt"}, {"sample_normal", "sample_yaw"},
                                       {"sample_normal", "sample_tilt"}, {"disk_center", "base_position"}, {"disk_center", "hub_height"}};
            for (auto& pr : pairs)
                if (D.has(key(pr[0])) && D.has(key(pr[1]))) throw Error(ERR_DECK, std::string("ActuatorDisk Conflict: ") + pr[0] + " and " + pr[1]);
            if (D.has(key("base_position")) != D.has(key("hub_height"))) throw Error(ERR_DECK, "base_position requires hub_height");
            if (D.has(key("disk_center"))) { auto c = D.v(key("disk_center")); for (int d = 0; d < 3; ++d) dp.center[d] = c.at(d); }
            else if (D.has(key("base_position"))) {
                auto b = D.v(key("base_position")); double hh = D.v(key("hub_height")).at(0);
                for (int d = 0; d < 3; ++d) dp.center[d] = b.at(d);
                dp.center[2] += hh;
            }
            // ops::base::optional_parameters (disk_ops.cpp:182-264): reference
            // vectors from the "Coriolis" (then "Coriolis.Forcing") parameters;
            // normal = R_z(-yaw) R_east(-tilt) normal0, with the rotation tensors
            // (vs::zrot, vs::quaternion) applied as v & T = T^T v
            double dn[3] = {0, 1, 0}, de[3] = {1, 0, 0};
            for (const char* pre : {"Coriolis.Forcing.", "Coriolis."}) {
                if (D.has(std::string(pre) + "north_vector")) { auto v = D.v(std::string(pre) + "north_vector"); for (int d = 0; d < 3; ++d) dn[d] = v.at(d); }
                if (D.has(std::string(pre) + "east_vector")) { auto v = D.v(std::string(pre) + "east_vector"); for (int d = 0; d < 3; ++d) de[d] = v.at(d); }
            }
            for (int d = 0; d < 3; ++d) { dp.normal[d] = dn[d]; dp.sample[d] = dn[d]; }
            if (D.has(key("disk_normal"))) { auto nn = D.v(key("disk_normal")); for (int d = 0; d < 3; ++d) dp.normal[d] = nn.at(d); }
            if (D.has(key("sample_normal"))) { auto nn = D.v(key("sample_normal")); for (int d = 0; d < 3; ++d) dp.sample[d] = nn.at(d); }
            auto apply = [&](double* v, const char* tilt_key, const char* yaw_key) {
                double T[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
                auto mul = [&](const double* B) {  // T = T B
                    double R[9];
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) R[3 * a + b] = T[3 * a] * B[b] + T[3 * a + 1] * B[3 + b] + T[3 * a + 2] * B[6 + b];
                    for (int q = 0; q < 9; ++q) T[q] = R[q];
                };
                if (D.has(key(tilt_key))) {  // vs::quaternion(east, -tilt)
                    const double ang = -(-D.v(key(tilt_key)).at(0)) * kPi / 180.0;
                    const double am = std::sqrt(de[0] * de[0] + de[1] * de[1] + de[2] * de[2]);
                    const double q0 = std::cos(0.5 * ang), sv = std::sin(0.5 * ang);
                    const double q1 = sv * de[0] / am, q2 = sv * de[1] / am, q3 = sv * de[2] / am;
                    const double Q[9] = {q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2 * (q1 * q2 - q0 * q3), 2 * (q0 * q2 + q1 * q3),
                                         2 * (q1 * q2 + q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2 * (q2 * q3 - q0 * q1),
                                         2 * (q1 * q3 - q0 * q2), 2 * (q0 * q1 + q2 * q3), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3};
                    mul(Q);
                }
                if (D.has(key(yaw_key))) {  // vs::zrot(-yaw)
                    const double ang = -D.v(key(yaw_key)).at(0) * kPi / 180.0, c = std::cos(ang), sn = std::sin(ang);
                    const double Z[9] = {c, sn, 0, -sn, c, 0, 0, 0, 1};
                    mul(Z);
                }
                const double o[3] = {T[0] * v[0] + T[3] * v[1] + T[6] * v[2], T[1] * v[0] + T[4] * v[1] + T[7] * v[2],
                                     T[2] * v[0] + T[5] * v[1] + T[8] * v[2]};
                for (int d = 0; d < 3; ++d) v[d] = o[d];
            };
            apply(dp.normal, "tilt", "yaw");
            apply(dp.sample, "sample_tilt", "sample_yaw");
            if (!D.has(key("sample_normal")) && !D.has(key("sample_tilt")) && !D.has(key("sample_yaw")))
                for (int d = 0; d < 3; ++d) dp.sample[d] = dp.normal[d];
            nrm(dp.normal);
            nrm(dp.sample);
            if (dp.normal[0] * dp.normal[0] + dp.normal[1] * dp.normal[1] <= 2.220446049250313e-16)
                throw Error(ERR_DECK, "A constant Ct disk normal is too close to vertical.");
            dp.diameters_to_sample = D.d(key("diameters_to_sample"), 0.0);
            dp.about_center = D.i(key("ks_spread_about_center"), 0) != 0;
            // coplanar vector k x n (disk_ops.cpp:278-282)
            double* n = dp.normal;
            dp.cvec[0] = -n[1]; dp.cvec[1] = n[0]; dp.cvec[2] = 0;
            nrm(dp.cvec);
            dp.dr = 0.5 * dp.diameter / dp.nr;
            dp.current_ct = dp.ct[0];
            disks.push_back(dp);
        }
    }

    def_cc(vel, g, 3, 3); def_cc(vel_old, g, 3, 3);
    def_cc(gp, g, 1, 3); def_cc(src, g, 1, 3); def_cc(forces, g, 1, 3);
    def_cc(mueff, g, 1, 1); def_cc(divtau, g, 0, 3); def_cc(divtau_new, g, 0, 3);
    def_cc(conv, g, 0, 3); def_cc(act_src, g, 0, 3);
    if (!godunov) def_cc(conv_old, g, 0, 3);
    if (has_temp) {
        def_cc(theta, g, 3, 1); def_cc(theta_old, g, 3, 1); def_cc(theta_nph, g, 0, 1);
        def_cc(alpha, g, 1, 1); def_cc(tsrc, g, 1, 1); def_cc(tdiff, g, 0, 1);
        def_cc(tdiff_new, g, 0, 1); def_cc(tconv, g, 0, 1); def_cc(tconv_old, g, 0, 1);
    }
    const int nzn = g.n[2] + (g.per[2] ? 0 : 1);
    p.define(-1, -1, -1, g.n[0], g.n[1], nzn, 1);
    umac.define(-1, -1, -1, g.n[0] + 1, g.n[1], g.n[2], 1);
    vmac.define(-1, -1, -1, g.n[0], g.n[1] + 1, g.n[2], 1);
    wmac.define(-1, -1, -1, g.n[0], g.n[1], g.n[2] + 1, 1);
    mueff.setval(mu);
    init_fields();
}

// ---- initial conditions ------------------------------------------------------
static uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

void Sim::init_fields() {
    const Deck& D = deck;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    if (physics == "TaylorGreenVortex") {
        // src/physics/TaylorGreenVortex.cpp:22-54
        rho = D.d("TGV.density", rho);
        const double Lx = g.phi[0] - g.plo[0], Ly = g.phi[1] - g.plo[1], Lz = g.phi[2] - g.plo[2];
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    double x = g.plo[0] + (i + 0.5) * g.dx[0], y = g.plo[1] + (j + 0.5) * g.dx[1], z = g.plo[2] + (k + 0.5) * g.dx[2];
                    vel(i, j, k, 0) = std::sin(2 * kPi * x / Lx) * std::cos(2 * kPi * y / Ly) * std::cos(2 * kPi * z / Lz);
                    vel(i, j, k, 1) = -std::cos(2 * kPi * x / Lx) * std::sin(2 * kPi * y / Ly) * std::cos(2 * kPi * z / Lz);
                    vel(i, j, k, 2) = 0.0;
                }
    } else if (physics == "ABL" && !D.has_prefix("ks_init.")) {
        // ABLFieldInit (src/wind_energy/ABLFieldInit.cpp:215-372), uniform-wind
        // branch: incflo.velocity plus the sinusoidal perturbation (perturb_velocity,
        // default on) damped by exp(-z^2 / (2 ref_height^2))
        auto u = D.v("incflo.velocity");
        const bool pert = D.i("ABL.perturb_velocity", 1) != 0;
        const double refh = D.d("ABL.perturb_ref_height", 50.0), ibh = D.d("ABL.ib_height", 0.0);
        const double Up = D.d("ABL.Uperiods", 4.0), Vp = D.d("ABL.Vperiods", 4.0);
        const double dU = D.d("ABL.deltaU", 1.0), dV = D.d("ABL.deltaV", 1.0);
        if (D.i("ABL.linear_profile", 0)) throw Error(ERR_UNSUPPORTED, "ABL.linear_profile");
        const double aval = Up * 2.0 * kPi / (g.phi[1] - g.plo[1]);
        const double bval = Vp * 2.0 * kPi / (g.phi[0] - g.plo[0]);
        const double ufac = dU * std::exp(0.5) / refh, vfac = dV * std::exp(0.5) / refh;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    vel(i, j, k, 0) = u.at(0);
                    vel(i, j, k, 1) = u.at(1);
                    vel(i, j, k, 2) = u.at(2);
                    if (!pert) continue;
                    const double x = g.plo[0] + (i + 0.5) * g.dx[0], y = g.plo[1] + (j + 0.5) * g.dx[1];
                    const double z = std::max(g.plo[2] + (k + 0.5) * g.dx[2] - ibh, 0.0);
                    const double zl = z / refh, damp = std::exp(-0.5 * zl * zl);
                    vel(i, j, k, 0) += ufac * damp * z * std::cos(aval * (y - g.plo[1]));
                    vel(i, j, k, 1) += vfac * damp * z * std::cos(bval * (x - g.plo[0]));
                }
    } else if (physics == "ABL" || physics == "FreeStream") {
        // Synthetic initial fields (not a reference feature): log-law or
        // uniform mean plus seeded uniform noise from SplitMix64 keyed on
        // (seed, comp, k, j, i).
        std::string prof = lower(D.s("ks_init.profile", physics == "ABL" ? "loglaw" : "uniform"));
        double U[3] = {0, 0, 0};
        if (D.has("incflo.velocity")) { auto u = D.v("incflo.velocity"); for (int d = 0; d < 3; ++d) U[d] = u.at(d); }
        const double utop = D.d("ks_init.loglaw_utop", 8.0);
        const double H = g.phi[2] - g.plo[2];
        const double ut = utop * kappa / std::log(H / z0);
        const double amp = D.d("ks_init.noise_amplitude", 0.0);
        const double zmax = D.d("ks_init.noise_zmax", 1e300);
        const uint64_t seed = (uint64_t)D.i("ks_init.noise_seed", 0);
        for (int n = 0; n < 3; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const double z = (k + 0.5) * g.dx[2];
                        double val = U[n];
                        if (prof == "loglaw") val = (n == 0) ? ut / kappa * std::log(z / z0) : 0.0;
                        if (amp > 0 && g.plo[2] + z < zmax) {
                            uint64_t idx = (((uint64_t)n * nz + k) * ny + j) * nx + i;
                            uint64_t r = splitmix64(seed * 0x100000001b3ULL ^ idx);
                            double u01 = (double)(r >> 11) * (1.0 / 9007199254740992.0);
                            val += amp * (2.0 * u01 - 1.0);
                        }
                        vel(i, j, k, n) = val;
                    }
    } else if (!physics.empty()) {
        throw Error(ERR_UNSUPPORTED, "incflo.physics " + physics);
    }
    if (has_temp) {  // piecewise-linear profile, tv[0] outside the segments (ABLFieldInit.cpp:318-327)
        auto th = D.v("ABL.temperature_heights"), tv = D.v("ABL.temperature_values");
        if (th.size() != tv.size() || th.empty()) throw Error(ERR_DECK, "ABL.temperature_heights and temperature_values differ in length");
        for (int k = 0; k < nz; ++k) {
            const double z = g.plo[2] + (k + 0.5) * g.dx[2];
            double t = tv[0];
            for (size_t m = 0; m + 1 < th.size(); ++m)
                if (z > th[m] && z <= th[m + 1]) t = tv[m] + (z - th[m]) * ((tv[m + 1] - tv[m]) / (th[m + 1] - th[m]));
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) theta(i, j, k) = 0.0 + t;
        }
    }
}

// ---- fill patch ----------------------------------------------------------------
// Velocity ghosts (src/boundary_conditions/BCInterface.cpp:169-260): periodic
// wrap; at slip_wall / wall_model z faces the tangential components use
// high-order extrapolation to the face, (15 q0 - 10 q1 + 3 q2)/8, repeated in
// every ghost layer, and the normal component is Dirichlet 0.
void Sim::fill_vel(Arr& v) const {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const int ng = -v.lo[2];
    if (!g.per[2]) {
        for (int n = 0; n < 3; ++n)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    double lo = (n == 2) ? 0.0 : 0.125 * (15 * v(i, j, 0, n) - 10 * v(i, j, 1, n) + 3 * v(i, j, 2, n));
                    double hi = (n == 2) ? 0.0 : 0.125 * (15 * v(i, j, nz - 1, n) - 10 * v(i, j, nz - 2, n) + 3 * v(i, j, nz - 3, n));
                    for (int m = 1; m <= ng; ++m) {
                        v(i, j, -m, n) = lo;
                        v(i, j, nz - 1 + m, n) = hi;
                    }
                }
    }
    const int cc[3] = {0, 0, 0};
    fill_periodic(v, g, cc);
}

// First-order extrapolation ghosts in z (src_term, viscosity fill-patch).
void Sim::fill_cc_foextrap(Arr& a) const {
    const int nz = g.n[2];
    const int ng = -a.lo[2];
    if (!g.per[2] && ng > 0)
        for (int n = 0; n < a.nc; ++n)
            for (int j = 0; j < g.n[1]; ++j)
                for (int i = 0; i < g.n[0]; ++i)
                    for (int m = 1; m <= ng; ++m) {
                        a(i, j, -m, n) = a(i, j, 0, n);
                        a(i, j, nz - 1 + m, n) = a(i, j, nz - 1, n);
                    }
    const int cc[3] = {0, 0, 0};
    fill_periodic(a, g, cc);
}

// ---- Smagorinsky ---------------------------------------------------------------
// src/turbulence/LES/Smagorinsky.cpp:22-62, src/fvm/strainrate.H:24-86,
// one-sided stencils src/fvm/stencils.H:166-330 at non-periodic z faces.
void Sim::update_mueff(Arr& v) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    // alpha_eff = mu / Pr + mu_t / Pr_t (TurbModelBase.H:28-35, LaminarModel.cpp:90-94)
    if (!smag) {
        mueff.setval(mu);
        if (has_temp) alpha.setval(mu / Pr);
        return;
    }
    fill_vel(v);
    const double idx = 1.0 / g.dx[0], idy = 1.0 / g.dx[1], idz = 1.0 / g.dx[2];
    const double ds = std::cbrt(g.dx[0] * g.dx[1] * g.dx[2]);
    const double fac = Cs * Cs * ds * ds;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double c20 = 0.5, c21 = 0.0, c22 = -0.5;
                if (!g.per[2] && k == 0) { c20 = 1.0 / 3.0; c21 = 1.0; c22 = -4.0 / 3.0; }
                if (!g.per[2] && k == nz - 1) { c20 = 4.0 / 3.0; c21 = -1.0; c22 = -1.0 / 3.0; }
                double gx[3], gy[3], gz[3];
                for (int n = 0; n < 3; ++n) {
                    gx[n] = 0.5 * (v(i + 1, j, k, n) - v(i - 1, j, k, n)) * idx;
                    gy[n] = 0.5 * (v(i, j + 1, k, n) - v(i, j - 1, k, n)) * idy;
                    gz[n] = (c20 * v(i, j, k + 1, n) + c21 * v(i, j, k, n) + c22 * v(i, j, k - 1, n)) * idz;
                }
                const double sr = std::sqrt(2 * gx[0] * gx[0] + 2 * gy[1] * gy[1] + 2 * gz[2] * gz[2] +
                                            (gy[0] + gx[1]) * (gy[0] + gx[1]) + (gz[1] + gy[2]) * (gz[1] + gy[2]) +
                                            (gx[2] + gz[0]) * (gx[2] + gz[0]));
                const double mut = rho * fac * sr;
                mueff(i, j, k) = mu + mut;
                if (has_temp) alpha(i, j, k) = mu / Pr + (1.0 / Prt) * mut;
            }
}

// ---- momentum sources ------------------------------------------------------------
// src/equation_systems/icns/icns_ops.H:78-124 and PDEOps.H:94-145:
// src = rho * (-gp/rho + sum of sources); the Coriolis term reads the velocity
// state v (Old for the predictor's Old and NPH states, New for the corrector:
// field_impl::dof_state, src/core/FieldUtils.H:110-113).
void Sim::compute_sources(const Arr& v, const Arr* th) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const double omega = 2 * kPi / rot_period;
    const double latr = lat * kPi / 180.0;
    const double sinphi = std::sin(latr), cosphi = std::cos(latr);
    const double geo_cf = 2 * omega * sinphi;  // GeostrophicForcing.cpp:28-77
    const double gf[3] = {-geo_cf * geo_wind[1], geo_cf * geo_wind[0], 0.0};
    const double hfac = cor_horizontal ? 0.0 : 1.0;
    const double corfac = 2 * omega;
    // BodyForce::operator() (BodyForce.cpp:117-169): the oscillatory type scales
    // the magnitude by cos(omega t) at t = (current + new time) / 2
    const double bcoef = body_osc ? std::cos(body_omega * 0.5 * (t.cur + t.newt)) : 1.0;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double s[3];
                for (int n = 0; n < 3; ++n) s[n] = -gp(i, j, k, n) / rho;
                if (src_geo)
                    for (int n = 0; n < 3; ++n) s[n] += (n == 2 ? hfac : 1.0) * gf[n];
                if (src_cor) {  // CoriolisForcing.cpp:60-108
                    const double u0 = v(i, j, k, 0), u1 = v(i, j, k, 1), u2 = v(i, j, k, 2);
                    const double ue = east[0] * u0 + east[1] * u1 + east[2] * u2;
                    const double un = north[0] * u0 + north[1] * u1 + north[2] * u2;
                    const double uu = up[0] * u0 + up[1] * u1 + up[2] * u2;
                    const double ae = corfac * (un * sinphi - hfac * uu * cosphi);
                    const double an = -corfac * ue * sinphi;
                    const double au = hfac * corfac * ue * cosphi;
                    for (int n = 0; n < 3; ++n) s[n] += ae * east[n] + an * north[n] + au * up[n];
                }
                if (src_body)
                    for (int n = 0; n < 3; ++n) s[n] += bcoef * body_force[n];
                if (src_act)
                    for (int n = 0; n < 3; ++n) s[n] += act_src(i, j, k, n);
                if (src_bous) {  // BoussinesqBuoyancy.cpp:22-50: g beta (T0 - T)
                    const double fac = beta_T * (T_ref - (*th)(i, j, k));
                    for (int n = 0; n < 3; ++n) s[n] += gravity[n] * fac;
                }
                if (src_ablf) {  // ABLForcing.cpp:97-139: horizontal components
                    s[0] += ablf_force[0];
                    s[1] += ablf_force[1];
                }
                for (int n = 0; n < 3; ++n) src(i, j, k, n) = rho * s[n];
            }
}

// ---- ABL wall model ----------------------------------------------------------------
// src/wind_energy/ABLWallFunction.cpp:164-347, ShearStress.H:22-167,
// MOData.cpp:52-103 (neutral: utau = kappa U / ln(zref/z0)).
void Sim::abl_update_umean() {
    if (g.zlo != WALLMODEL) return;
    const int nx = g.n[0], ny = g.n[1];
    double su = 0, sv = 0, sm = 0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double u = vel(i, j, 0, 0), v = vel(i, j, 0, 1);
            su += u; sv += v; sm += std::sqrt(u * u + v * v);
        }
    umean[0] = su / (nx * ny);
    umean[1] = sv / (nx * ny);
    vmag_mean = sm / (nx * ny);
    utau = kappa * vmag_mean / std::log(zref / z0);
    if (has_temp) {  // theta_mean at z_ref for the heat flux (ABLWallFunction.cpp:206-207)
        double st = 0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) st += theta(i, j, 0);
        theta_mean = st / (nx * ny);
    }
}

// ABL::pre_advance_work -> ABLForcing::set_mean_velocities (ABL.cpp:176-205,
// ABLForcing.H:37-64): plane averages of u and v interpolated to the forcing
// height (FieldPlaneAveraging.cpp:78-96,151-164), force = (target - mean) / dt.
void Sim::abl_forcing_update() {
    if (!src_ablf) return;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    std::vector<double> ua(nz), va(nz);
    for (int k = 0; k < nz; ++k) {
        double su = 0, sv = 0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) { su += vel(i, j, k, 0); sv += vel(i, j, k, 1); }
        ua[k] = su / (nx * ny);
        va[k] = sv / (nx * ny);
    }
    int ind = 0;
    double c = 0.0;
    const double x = ablf_height, xlo = g.plo[2], dz = g.dx[2];
    if (x > xlo + 0.5 * dz) {
        ind = (int)std::floor((x - xlo) / dz - 0.5);
        c = (x - (xlo + (ind + 0.5) * dz)) / dz;
    }
    if (ind + 1 >= nz) { ind = nz - 2; c = 1.0; }
    const double mu0 = ua[ind] * (1.0 - c) + ua[ind + 1] * c, mv0 = va[ind] * (1.0 - c) + va[ind + 1] * c;
    ablf_force[0] = (ablf_target[0] - mu0) / t.dt[0];
    ablf_force[1] = (ablf_target[1] - mv0) / t.dt[0];
}

// Wall-normal velocity gradient imposed at z-lo for the tangential components:
// tau * rho / mu_eff evaluated with the Old velocity of the first cell.
void Sim::wall_gradient(std::vector<double>& gx, std::vector<double>& gy) const {
    const int nx = g.n[0], ny = g.n[1];
    gx.assign((size_t)nx * ny, 0.0);
    gy.assign((size_t)nx * ny, 0.0);
    if (g.zlo != WALLMODEL) return;
    const double ut2 = utau * utau;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double u = vel_old(i, j, 0, 0), v = vel_old(i, j, 0, 1);
            const double wspd = std::sqrt(u * u + v * v);
            double tx, ty;
            if (shear_type == "moeng") {
                tx = ((u - umean[0]) * vmag_mean + wspd * umean[0]) / (vmag_mean * vmag_mean) * ut2;
                ty = ((v - umean[1]) * vmag_mean + wspd * umean[1]) / (vmag_mean * vmag_mean) * ut2;
            } else if (shear_type == "constant") {
                tx = umean[0] / vmag_mean * ut2;
                ty = umean[1] / vmag_mean * ut2;
            } else if (shear_type == "local") {
                tx = u / std::max(wspd, 1.0e-6) * ut2;
                ty = v / std::max(wspd, 1.0e-6) * ut2;
            } else {  // schumann
                tx = u / vmag_mean * ut2;
                ty = v / vmag_mean * ut2;
            }
            const double m = mueff(i, j, 0);
            gx[(size_t)j * nx + i] = tx * rho / m;
            gy[(size_t)j * nx + i] = ty * rho / m;
        }
}

// ---- tensor diffusion operator -----------------------------------------------------
// div( mu (grad u + grad u^T) - 2/3 mu (div u) I ): MLTensorOp apply with
// alpha = 0, beta = -1 (icns_diffusion.H:37-48).  Face viscosity is the
// arithmetic mean of the two cells, the cell value on domain faces
// (incflo_diffusion.cpp:108-206).  Boundary conditions come from
// get_diffuse_tensor_bc (incflo_diffusion.cpp:11-69) and are imposed through
// one ghost layer: Dirichlet-0 normal component -> odd reflection, Neumann
// tangential -> even reflection, inhomogeneous Neumann (wall model) -> ghost =
// q0 - g dz so that the face gradient equals g.
void Sim::divtau_op(const Arr& v_in, Arr& out) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    Arr v;
    def_cc(v, g, 1, 3);
    for (int n = 0; n < 3; ++n)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) v(i, j, k, n) = v_in(i, j, k, n);
    std::vector<double> gxw, gyw;
    wall_gradient(gxw, gyw);
    if (!g.per[2]) {
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                for (int n = 0; n < 3; ++n) {
                    const double q0 = v(i, j, 0, n), qn = v(i, j, nz - 1, n);
                    if (n == 2) { v(i, j, -1, n) = -q0; v(i, j, nz, n) = -qn; continue; }
                    double glo = 0.0;
                    if (g.zlo == WALLMODEL) glo = (n == 0 ? gxw : gyw)[(size_t)j * nx + i];
                    v(i, j, -1, n) = q0 - glo * g.dx[2];
                    v(i, j, nz, n) = qn;
                }
            }
    }
    const int cc[3] = {0, 0, 0};
    fill_periodic(v, g, cc);
    Arr m;
    def_cc(m, g, 1, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) m(i, j, k) = mueff(i, j, k);
    fill_cc_foextrap(m);
    const double dx = g.dx[0], dy = g.dx[1], dz = g.dx[2];
    Arr fx, fy, fz;
    fx.define(0, 0, 0, nx, ny - 1, nz - 1, 3);
    fy.define(0, 0, 0, nx - 1, ny, nz - 1, 3);
    fz.define(0, 0, 0, nx - 1, ny - 1, nz, 3);
    // x faces
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const double mf = 0.5 * (m(i - 1, j, k) + m(i, j, k));
                double dqx[3], dqy[3], dqz[3];
                for (int n = 0; n < 3; ++n) {
                    dqx[n] = (v(i, j, k, n) - v(i - 1, j, k, n)) / dx;
                    dqy[n] = 0.25 * (v(i, j + 1, k, n) + v(i - 1, j + 1, k, n) - v(i, j - 1, k, n) - v(i - 1, j - 1, k, n)) / dy;
                    dqz[n] = 0.25 * (v(i, j, k + 1, n) + v(i - 1, j, k + 1, n) - v(i, j, k - 1, n) - v(i - 1, j, k - 1, n)) / dz;
                }
                const double dv = dqx[0] + dqy[1] + dqz[2];
                fx(i, j, k, 0) = mf * (2 * dqx[0] - (2.0 / 3.0) * dv);
                fx(i, j, k, 1) = mf * (dqx[1] + dqy[0]);
                fx(i, j, k, 2) = mf * (dqx[2] + dqz[0]);
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double mf = 0.5 * (m(i, j - 1, k) + m(i, j, k));
                double dqx[3], dqy[3], dqz[3];
                for (int n = 0; n < 3; ++n) {
                    dqy[n] = (v(i, j, k, n) - v(i, j - 1, k, n)) / dy;
                    dqx[n] = 0.25 * (v(i + 1, j, k, n) + v(i + 1, j - 1, k, n) - v(i - 1, j, k, n) - v(i - 1, j - 1, k, n)) / dx;
                    dqz[n] = 0.25 * (v(i, j, k + 1, n) + v(i, j - 1, k + 1, n) - v(i, j, k - 1, n) - v(i, j - 1, k - 1, n)) / dz;
                }
                const double dv = dqx[0] + dqy[1] + dqz[2];
                fy(i, j, k, 0) = mf * (dqy[0] + dqx[1]);
                fy(i, j, k, 1) = mf * (2 * dqy[1] - (2.0 / 3.0) * dv);
                fy(i, j, k, 2) = mf * (dqy[2] + dqz[1]);
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double mf;
                if (!g.per[2] && k == 0) mf = m(i, j, 0);
                else if (!g.per[2] && k == nz) mf = m(i, j, nz - 1);
                else mf = 0.5 * (m(i, j, k - 1) + m(i, j, k));
                double dqx[3], dqy[3], dqz[3];
                for (int n = 0; n < 3; ++n) {
                    dqz[n] = (v(i, j, k, n) - v(i, j, k - 1, n)) / dz;
                    dqx[n] = 0.25 * (v(i + 1, j, k, n) + v(i + 1, j, k - 1, n) - v(i - 1, j, k, n) - v(i - 1, j, k - 1, n)) / dx;
                    dqy[n] = 0.25 * (v(i, j + 1, k, n) + v(i, j + 1, k - 1, n) - v(i, j - 1, k, n) - v(i, j - 1, k - 1, n)) / dy;
                }
                const double dv = dqx[0] + dqy[1] + dqz[2];
                fz(i, j, k, 0) = mf * (dqz[0] + dqx[2]);
                fz(i, j, k, 1) = mf * (dqz[1] + dqy[2]);
                fz(i, j, k, 2) = mf * (2 * dqz[2] - (2.0 / 3.0) * dv);
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int n = 0; n < 3; ++n)
                    out(i, j, k, n) = (fx(i + 1, j, k, n) - fx(i, j, k, n)) / dx + (fy(i, j + 1, k, n) - fy(i, j, k, n)) / dy +
                                      (fz(i, j, k + 1, n) - fz(i, j, k, n)) / dz;
}

// ---- PPM (Colella & Woodward 1984, van Leer limited edges) -------------------------------
struct PPM {
    static double vl(double a, double b, double c) {
        const double dsc = 0.5 * (c - a), dsl = 2 * (b - a), dsr = 2 * (c - b);
        if (dsl * dsr > 0) return std::copysign(std::min(std::fabs(dsc), std::min(std::fabs(dsl), std::fabs(dsr))), dsc);
        return 0.0;
    }
    static double clip(double e, double a, double b) {
        e = std::max(e, std::min(a, b));
        return std::min(e, std::max(a, b));
    }
    // Limited parabola edges (sm, sp) of cell c from q[-2..2] (q points at
    // cell c).  zw >= 0 marks a line along a wall-bounded z direction with zw
    // cells; c is then the cell index.  Faces on the walls take the boundary
    // value held in the first ghost cell; the faces one cell inside use the
    // one-sided fourth-order edge formula, clipped to the adjacent cells.
    static void edges(const double* q, int c, int zw, double& sm, double& sp) {
        auto std_edge = [&](int f) {  // face between cells f-1 and f (relative)
            const double e = 0.5 * (q[f - 1] + q[f]) - (1.0 / 6.0) * (vl(q[f - 1], q[f], q[f + 1]) - vl(q[f - 2], q[f - 1], q[f]));
            return clip(e, q[f - 1], q[f]);
        };
        if (zw >= 0 && c == 0) sm = q[-1];
        else if (zw >= 0 && c == 1) sm = clip(-0.2 * q[-2] + 0.75 * q[-1] + 0.5 * q[0] - 0.05 * q[1], q[-1], q[0]);
        else if (zw >= 0 && c == zw - 1) sm = clip(-0.2 * q[1] + 0.75 * q[0] + 0.5 * q[-1] - 0.05 * q[-2], q[0], q[-1]);
        else sm = std_edge(0);
        if (zw >= 0 && c == zw - 1) sp = q[1];
        else if (zw >= 0 && c == zw - 2) sp = clip(-0.2 * q[2] + 0.75 * q[1] + 0.5 * q[0] - 0.05 * q[-1], q[1], q[0]);
        else if (zw >= 0 && c == 0) sp = clip(-0.2 * q[-1] + 0.75 * q[0] + 0.5 * q[1] - 0.05 * q[2], q[0], q[1]);
        else sp = std_edge(1);
        const double s0 = q[0];
        if ((sp - s0) * (s0 - sm) <= 0.0) { sp = s0; sm = s0; }
        else if (std::fabs(sp - s0) >= 2.0 * std::fabs(sm - s0)) sp = 3.0 * s0 - 2.0 * sm;
        else if (std::fabs(sm - s0) >= 2.0 * std::fabs(sp - s0)) sm = 3.0 * s0 - 2.0 * sp;
    }
};

// Gather the 5-point line through (i,j,k) along direction d for component n.
static int line(const Arr& a, const Geo& g, int d, int i, int j, int k, int n, double* q) {
    for (int m = -2; m <= 2; ++m) {
        int c[3] = {i, j, k};
        c[d] += m;
        if (d == 2 && !g.per[2]) c[2] = std::max(-1, std::min(g.n[2], c[2]));
        q[m + 2] = a(c[0], c[1], c[2], n);
    }
    return (d == 2 && !g.per[2]) ? g.n[2] : -1;
}

// SetXEdgeBCs restricted to z walls: tangential components (and hoextrap
// scalars) take the interior state, the normal component is Dirichlet 0 on
// both sides.
static void zedge_bc(const Geo& g, int k, bool normal, double& lo, double& hi) {
    if (g.per[2]) return;
    if (k == 0) {
        if (normal) { lo = 0.0; hi = 0.0; } else lo = hi;
    } else if (k == g.n[2]) {
        if (normal) { lo = 0.0; hi = 0.0; } else hi = lo;
    }
}

static inline double upwind(double vel, double lo, double hi) {
    const double st = (vel >= 0.0) ? lo : hi;
    const double fu = (std::fabs(vel) < kSmallVel) ? 0.0 : 1.0;
    return fu * st + (1.0 - fu) * 0.5 * (lo + hi);
}

static inline double riemann(double lo, double hi) {
    const double st = (lo + hi >= 0.0) ? lo : hi;
    const bool ltm = (lo <= 0.0 && hi >= 0.0) || (std::fabs(lo + hi) < kSmallVel);
    return ltm ? 0.0 : st;
}

// Godunov traces of every component in every direction, on cells [-1, n]
// (z restricted to the valid range for walls).  mode 0: cell velocity as the
// characteristic speed (PredictVelOnXFace); mode 1: face velocities
// (PredictStateOnXFace).
struct Traces {
    Arr Im[3], Ip[3];
};

static void compute_traces(const Arr& q, const Geo& g, double dt, int mode, const Arr* vcell, const Arr* fv[3], Traces& T) {
    const int nz = g.n[2];
    const int klo = g.per[2] ? -1 : 0, khi = g.per[2] ? nz : nz - 1;
    for (int d = 0; d < 3; ++d) {
        T.Im[d].define(-1, -1, klo, g.n[0], g.n[1], khi, q.nc);
        T.Ip[d].define(-1, -1, klo, g.n[0], g.n[1], khi, q.nc);
        const double dtdx = dt / g.dx[d];
        for (int n = 0; n < q.nc; ++n)
#pragma omp parallel for collapse(2)
            for (int k = klo; k <= khi; ++k)
                for (int j = -1; j <= g.n[1]; ++j)
                    for (int i = -1; i <= g.n[0]; ++i) {
                        double L[5];
                        const int zw = line(q, g, d, i, j, k, n, L);
                        double sm, sp;
                        PPM::edges(L + 2, (d == 0 ? i : d == 1 ? j : k), zw, sm, sp);
                        const double s0 = L[2];
                        const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
                        double im = s0, ip = s0;
                        if (mode == 0) {
                            const double u = (*vcell)(i, j, k, d);
                            const double sig = std::fabs(u) * dtdx;
                            if (u > kSmallVel) ip = sp - 0.5 * sig * ((sp - sm) - (1.0 - 2.0 / 3.0 * sig) * s6);
                            else if (u < -kSmallVel) im = sm + 0.5 * sig * ((sp - sm) + (1.0 - 2.0 / 3.0 * sig) * s6);
                        } else {
                            int c[3] = {i, j, k};
                            const double um = (*fv[d])(c[0], c[1], c[2]);
                            c[d] += 1;
                            const double up = (*fv[d])(c[0], c[1], c[2]);
                            const double sigp = std::fabs(up) * dtdx, sigm = std::fabs(um) * dtdx;
                            if (up > kSmallVel) ip = sp - 0.5 * sigp * ((sp - sm) - (1.0 - 2.0 / 3.0 * sigp) * s6);
                            if (um < -kSmallVel) im = sm + 0.5 * sigm * ((sp - sm) + (1.0 - 2.0 / 3.0 * sigm) * s6);
                        }
                        T.Im[d](i, j, k, n) = im;
                        T.Ip[d](i, j, k, n) = ip;
                    }
    }
}

// Transverse-state array on a-faces corrected along b: faces [0, n_a] in a,
// cells [0, n_b - 1] in b, cells grown by one in the third direction (not in a
// wall-bounded z).
static void def_trans(Arr& a, const Geo& g, int fa, int fb, int nc) {
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        if (d == fa) { lo[d] = 0; hi[d] = g.n[d]; }
        else if (d == fb) { lo[d] = 0; hi[d] = g.n[d] - 1; }
        else if (d == 2 && !g.per[2]) { lo[d] = 0; hi[d] = g.n[d] - 1; }
        else { lo[d] = -1; hi[d] = g.n[d]; }
    }
    a.define(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], nc);
}

// Face-centred arrays over faces [0, n] in their normal direction and grown
// by one in the two transverse directions.
static void def_face(Arr& a, const Geo& g, int d, int nc) {
    const int klo = g.per[2] ? -1 : 0;
    const int khi_c = g.per[2] ? g.n[2] : g.n[2] - 1;
    if (d == 0) a.define(0, -1, klo, g.n[0], g.n[1], khi_c, nc);
    if (d == 1) a.define(-1, 0, klo, g.n[0], g.n[1], khi_c, nc);
    if (d == 2) a.define(-1, -1, 0, g.n[0], g.n[1], g.n[2], nc);
}

// ---- pre-MAC velocity extrapolation ------------------------------------------------------------
// HydroUtils::ExtrapVelToFaces (called at icns_advection.H:211-216): PPM traces
// with the cell velocity, Riemann-solved advective velocities, upwinded
// transverse states, 3-D corner-transport corrections (dt/6 terms), then the
// final Riemann solve with the forces added at the end.
void Sim::premac(double dt) {
    const Geo& G = g;
    Arr& q = vel_old;
    fill_vel(q);
    fill_cc_foextrap(forces);
    Traces T;
    compute_traces(q, G, dt, 0, &q, nullptr, T);
    const int nz = G.n[2];
    Arr ad[3], lo[3], hi[3], edge[3];
    for (int d = 0; d < 3; ++d) {
        def_face(ad[d], G, d, 1);
        def_face(lo[d], G, d, 3);
        def_face(hi[d], G, d, 3);
        def_face(edge[d], G, d, 3);
        Arr& A = ad[d];
        for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
            for (int k = A.lo[2]; k <= A.hi[2]; ++k)
                for (int j = A.lo[1]; j <= A.hi[1]; ++j)
                    for (int i = A.lo[0]; i <= A.hi[0]; ++i) {
                        int c[3] = {i, j, k};
                        const bool wall = (d == 2 && !G.per[2] && (k == 0 || k == nz));
                        double l = 0, h = 0;
                        c[d] -= 1;
                        if (!(wall && k == 0)) l = T.Ip[d](c[0], c[1], c[2], n);
                        c[d] += 1;
                        if (!(wall && k == nz)) h = T.Im[d](c[0], c[1], c[2], n);
                        if (d == 2) zedge_bc(G, k, n == 2, l, h);
                        lo[d](i, j, k, n) = l;
                        hi[d](i, j, k, n) = h;
                        if (n == d) A(i, j, k) = riemann(l, h);
                    }
        for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
            for (int k = A.lo[2]; k <= A.hi[2]; ++k)
                for (int j = A.lo[1]; j <= A.hi[1]; ++j)
                    for (int i = A.lo[0]; i <= A.hi[0]; ++i)
                        edge[d](i, j, k, n) = upwind(A(i, j, k), lo[d](i, j, k, n), hi[d](i, j, k, n));
    }
    const double dx = G.dx[0], dy = G.dx[1], dz = G.dx[2];
    // transverse-corrected states: T2[a][b] = states on a-faces of the
    // component normal to the remaining direction, corrected by direction b.
    // needed: (y,z)->comp0, (z,y)->comp0, (x,z)->comp1, (z,x)->comp1,
    // (x,y)->comp2, (y,x)->comp2
    struct TP { int a, b, n; };
    const TP tps[6] = {{1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {2, 0, 1}, {0, 1, 2}, {1, 0, 2}};
    Arr tr[6];
    for (int t = 0; t < 6; ++t) {
        const int a = tps[t].a, b = tps[t].b, n = tps[t].n;
        def_trans(tr[t], G, a, b, 1);
        Arr& R = tr[t];
        const double cb = dt / (6.0 * G.dx[b]);
#pragma omp parallel for collapse(2)
        for (int k = R.lo[2]; k <= R.hi[2]; ++k)
            for (int j = R.lo[1]; j <= R.hi[1]; ++j)
                for (int i = R.lo[0]; i <= R.hi[0]; ++i) {
                    const bool wall = (a == 2 && !G.per[2] && (k == 0 || k == nz));
                    double l = lo[a](i, j, k, n), h = hi[a](i, j, k, n);
                    // lo side: cell (face - e_a); hi side: cell at the face index
                    int c[3] = {i, j, k};
                    if (!(wall && k == nz)) {
                        int cp[3] = {c[0], c[1], c[2]};
                        cp[b] += 1;
                        h -= cb * (ad[b](cp[0], cp[1], cp[2]) + ad[b](c[0], c[1], c[2])) *
                             (edge[b](cp[0], cp[1], cp[2], n) - edge[b](c[0], c[1], c[2], n));
                    }
                    if (!(wall && k == 0)) {
                        int cl[3] = {c[0], c[1], c[2]};
                        cl[a] -= 1;
                        int cq[3] = {cl[0], cl[1], cl[2]};
                        cq[b] += 1;
                        l -= cb * (ad[b](cq[0], cq[1], cq[2]) + ad[b](cl[0], cl[1], cl[2])) *
                             (edge[b](cq[0], cq[1], cq[2], n) - edge[b](cl[0], cl[1], cl[2], n));
                    }
                    if (a == 2) zedge_bc(G, k, n == 2, l, h);
                    R(i, j, k) = upwind(ad[a](i, j, k), l, h);
                }
    }
    // final normal velocities.  For face direction d, the transverse
    // directions b1 < b2 use tr of (b, other) with comp d.
    auto tr_of = [&](int a, int b) -> Arr& {
        for (int t = 0; t < 6; ++t)
            if (tps[t].a == a && tps[t].b == b) return tr[t];
        throw Error(ERR_ARG, "internal");
    };
    Arr* mac[3] = {&umac, &vmac, &wmac};
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        Arr& T1 = tr_of(b1, b2);  // b1-faces corrected by b2
        Arr& T2 = tr_of(b2, b1);
        const double c1 = dt / (4.0 * G.dx[b1]), c2 = dt / (4.0 * G.dx[b2]);
        const int nd = G.n[d];
        const int kmax = (d == 2) ? nz : nz - 1;
#pragma omp parallel for collapse(2)
        for (int k = 0; k <= kmax; ++k)
            for (int j = 0; j <= (d == 1 ? G.n[1] : G.n[1] - 1); ++j)
                for (int i = 0; i <= (d == 0 ? G.n[0] : G.n[0] - 1); ++i) {
                    const bool wall = (d == 2 && !G.per[2] && (k == 0 || k == nz));
                    int c[3] = {i, j, k};
                    auto side = [&](int* cell, double base) {
                        int p1[3] = {cell[0], cell[1], cell[2]};
                        p1[b1] += 1;
                        int p2[3] = {cell[0], cell[1], cell[2]};
                        p2[b2] += 1;
                        double s = base;
                        s -= c1 * (ad[b1](p1[0], p1[1], p1[2]) + ad[b1](cell[0], cell[1], cell[2])) *
                             (T1(p1[0], p1[1], p1[2]) - T1(cell[0], cell[1], cell[2]));
                        s -= c2 * (ad[b2](p2[0], p2[1], p2[2]) + ad[b2](cell[0], cell[1], cell[2])) *
                             (T2(p2[0], p2[1], p2[2]) - T2(cell[0], cell[1], cell[2]));
                        s += 0.5 * dt * forces(cell[0], cell[1], cell[2], d);
                        return s;
                    };
                    double stl = 0, sth = 0;
                    int cl[3] = {c[0], c[1], c[2]};
                    cl[d] -= 1;
                    if (!(wall && k == 0)) stl = side(cl, lo[d](i, j, k, d));
                    if (!(wall && k == nz)) sth = side(c, hi[d](i, j, k, d));
                    if (d == 2) zedge_bc(G, k, d == 2, stl, sth);
                    (*mac[d])(i, j, k) = riemann(stl, sth);
                    (void)nd;
                }
    }
}

// ---- multigrid: cell-centred 7-point Poisson -----------------------------------------------------
// Coarsening ratio of one level to the next (1 or 2 per direction).  Full
// coarsening needs every count divisible by 4 (the coarse count stays even).
// Semicoarsening (MLMGOptions do_semicoarsening, src/core/MLMGOptions.cpp:24-28)
// halves only the directions of smallest spacing while the spacings differ,
// each of them divisible by 4; with equal spacings, or when one of them is not
// divisible, the level coarsens fully or not at all as without it.
static void semi_ratio(const int n[3], const double h[3], bool semi, int r[3]) {
    const double hmin = std::min(h[0], std::min(h[1], h[2])), hmax = std::max(h[0], std::max(h[1], h[2]));
    bool full = true;
    for (int d = 0; d < 3; ++d) full = full && (n[d] % 4 == 0);
    if (semi && hmax > 1.0000001 * hmin) {
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
            r[d] = (h[d] <= 1.0000001 * hmin) ? 2 : 1;
            if (r[d] == 2 && n[d] % 4 != 0) ok = false;
        }
        if (ok) return;
    }
    for (int d = 0; d < 3; ++d) r[d] = full ? 2 : 1;
}

struct CCLevel {
    int n[3];
    double h[3];
    int r[3] = {2, 2, 2};  // coarsening ratio to the next level
    Arr phi, rhs, res;
};

static void cc_fill(Arr& a, const int n[3], bool zper) {
    // periodic x, y (and z), Neumann mirror in z
    const int nx = n[0], ny = n[1], nz = n[2];
    for (int k = -1; k <= nz; ++k)
        for (int j = -1; j <= ny; ++j)
            for (int i = -1; i <= nx; ++i) {
                if (i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz) continue;
                int ii = (i + nx) % nx, jj = (j + ny) % ny, kk;
                if (zper) kk = (k + nz) % nz;
                else kk = std::max(0, std::min(nz - 1, k));
                a(i, j, k) = a(ii, jj, kk);
            }
}

// A phi = beta * laplacian(phi); at Neumann z walls the wall-side term drops
// out (ghost equals the cell value).
static void cc_apply(const CCLevel& L, double beta, bool zper, int i, int j, int k, double& Ax, double& diag) {
    const Arr& p = L.phi;
    const double ix2 = 1.0 / (L.h[0] * L.h[0]), iy2 = 1.0 / (L.h[1] * L.h[1]), iz2 = 1.0 / (L.h[2] * L.h[2]);
    double s = ix2 * (p(i + 1, j, k) + p(i - 1, j, k)) + iy2 * (p(i, j + 1, k) + p(i, j - 1, k));
    double dg = 2 * ix2 + 2 * iy2;
    if (zper || k > 0) { s += iz2 * p(i, j, k - 1); dg += iz2; }
    if (zper || k < L.n[2] - 1) { s += iz2 * p(i, j, k + 1); dg += iz2; }
    Ax = beta * (s - dg * p(i, j, k));
    diag = -beta * dg;
}

static void cc_smooth(CCLevel& L, double beta, bool zper, int sweeps) {
    for (int s = 0; s < sweeps; ++s)
        for (int color = 0; color < 2; ++color) {
            cc_fill(L.phi, L.n, zper);
#pragma omp parallel for collapse(2)
            for (int k = 0; k < L.n[2]; ++k)
                for (int j = 0; j < L.n[1]; ++j)
                    for (int i = 0; i < L.n[0]; ++i) {
                        if (((i + j + k) & 1) != color) continue;
                        double Ax, dg;
                        cc_apply(L, beta, zper, i, j, k, Ax, dg);
                        L.phi(i, j, k) += (L.rhs(i, j, k) - Ax) / dg;
                    }
        }
}

static double cc_residual(CCLevel& L, double beta, bool zper) {
    cc_fill(L.phi, L.n, zper);
    double mx = 0;
#pragma omp parallel for collapse(2) reduction(max : mx)
    for (int k = 0; k < L.n[2]; ++k)
        for (int j = 0; j < L.n[1]; ++j)
            for (int i = 0; i < L.n[0]; ++i) {
                double Ax, dg;
                cc_apply(L, beta, zper, i, j, k, Ax, dg);
                L.res(i, j, k) = L.rhs(i, j, k) - Ax;
                mx = std::max(mx, std::fabs(L.res(i, j, k)));
            }
    return mx;
}

static void cc_vcycle(std::vector<CCLevel>& Ls, size_t l, double beta, bool zper, const MGOpts& o) {
    CCLevel& L = Ls[l];
    if (l + 1 == Ls.size()) {
        cc_smooth(L, beta, zper, o.bottom);
        return;
    }
    cc_smooth(L, beta, zper, o.nu1);
    cc_residual(L, beta, zper);
    CCLevel& C = Ls[l + 1];
    const int rx = L.r[0], ry = L.r[1], rz = L.r[2];
    const double w = 1.0 / (rx * ry * rz);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < C.n[2]; ++k)
        for (int j = 0; j < C.n[1]; ++j)
            for (int i = 0; i < C.n[0]; ++i) {
                double s = 0;
                for (int c = 0; c < rz; ++c)
                    for (int b = 0; b < ry; ++b)
                        for (int a = 0; a < rx; ++a) s += L.res(rx * i + a, ry * j + b, rz * k + c);
                C.rhs(i, j, k) = w * s;
                C.phi(i, j, k) = 0.0;
            }
    cc_vcycle(Ls, l + 1, beta, zper, o);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < L.n[2]; ++k)
        for (int j = 0; j < L.n[1]; ++j)
            for (int i = 0; i < L.n[0]; ++i) L.phi(i, j, k) += C.phi(i / rx, j / ry, k / rz);
    cc_smooth(L, beta, zper, o.nu2);
}

static std::vector<CCLevel> cc_levels(const Geo& g, const MGOpts& o) {
    std::vector<CCLevel> Ls;
    int n[3] = {g.n[0], g.n[1], g.n[2]};
    double h[3] = {g.dx[0], g.dx[1], g.dx[2]};
    while (true) {
        CCLevel L;
        for (int d = 0; d < 3; ++d) { L.n[d] = n[d]; L.h[d] = h[d]; }
        L.phi.define(-1, -1, -1, n[0], n[1], n[2], 1);
        L.rhs.define(0, 0, 0, n[0] - 1, n[1] - 1, n[2] - 1, 1);
        L.res.define(0, 0, 0, n[0] - 1, n[1] - 1, n[2] - 1, 1);
        semi_ratio(n, h, o.semicoarsening && (int)Ls.size() < o.max_semi, L.r);
        const bool can = L.r[0] + L.r[1] + L.r[2] > 3;
        Ls.push_back(std::move(L));
        if (!can) break;
        for (int d = 0; d < 3; ++d) { n[d] /= Ls.back().r[d]; h[d] *= Ls.back().r[d]; }
    }
    return Ls;
}

// MAC projection (icns_advection.cpp:206-375): beta = 1/rho0, Neumann at walls,
// u_mac -= beta grad(phi).
void Sim::mac_project() {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const bool zper = g.per[2];
    const double beta = 1.0 / rho;
    std::vector<CCLevel> Ls = cc_levels(g, mac);
    mac_dims.clear();
    for (const CCLevel& C : Ls) mac_dims.push_back({C.n[0], C.n[1], C.n[2]});
    CCLevel& L = Ls[0];
    double sum = 0;
#pragma omp parallel for collapse(2) reduction(+ : sum)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double r = (umac(i + 1, j, k) - umac(i, j, k)) / g.dx[0] + (vmac(i, j + 1, k) - vmac(i, j, k)) / g.dx[1] +
                                 (wmac(i, j, k + 1) - wmac(i, j, k)) / g.dx[2];
                L.rhs(i, j, k) = r;
                sum += r;
            }
    const double mean = sum / ((double)nx * ny * nz);
    for (auto& x : L.rhs.d) x -= mean;
    double r0 = cc_residual(L, beta, zper);
    mac_res0 = r0;
    const double target = std::max(mac.atol, mac.rtol * r0);
    int it = 0;
    double rn = r0;
    while (rn > target && it < mac.maxiter) {
        cc_vcycle(Ls, 0, beta, zper, mac);
        rn = cc_residual(L, beta, zper);
        ++it;
        if (!std::isfinite(rn)) throw Error(ERR_NONFINITE, "MAC projection diverged");
        if (rn > 1e20 * r0) throw Error(ERR_NOT_CONVERGED, "MAC projection diverged (residual above 1e20 times the initial one)");
    }
    // fixed-iteration mode is the MLMGOptions default (MLMGOptions.H:126-128): no abort at maxiter
    if (rn > target && !mac.fixed_iters) throw Error(ERR_NOT_CONVERGED, "MAC projection did not converge in mac_proj.maxiter V-cycles");
    mac_iters = it;
    mac_res = rn;
    cc_fill(L.phi, L.n, zper);
    Arr& f = L.phi;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                umac(i, j, k) -= beta * (f(i, j, k) - f(i - 1, j, k)) / g.dx[0];
                vmac(i, j, k) -= beta * (f(i, j, k) - f(i, j - 1, k)) / g.dx[1];
                if (zper || k > 0) wmac(i, j, k) -= beta * (f(i, j, k) - f(i, j, k - 1)) / g.dx[2];
            }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) umac(nx, j, k) = umac(0, j, k);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) vmac(i, ny, k) = vmac(i, 0, k);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) wmac(i, j, nz) = zper ? wmac(i, j, 0) : 0.0;
    const int fx[3] = {1, 0, 0}, fy[3] = {0, 1, 0}, fz[3] = {0, 0, 1};
    fill_periodic(umac, g, fx);
    fill_periodic(vmac, g, fy);
    fill_periodic(wmac, g, fz);
}

// ---- temperature transport (Godunov; src/incflo_advance.cpp:296-341) -----------------------------
// hoextrap ghosts at z walls (BCScalar::set_bcrec, BCInterface.cpp:289-350), periodic wrap
void Sim::fill_scalar(Arr& a) const {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const int ng = -a.lo[2];
    if (!g.per[2])
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double lo = 0.125 * (15 * a(i, j, 0) - 10 * a(i, j, 1) + 3 * a(i, j, 2));
                const double hi = 0.125 * (15 * a(i, j, nz - 1) - 10 * a(i, j, nz - 2) + 3 * a(i, j, nz - 3));
                for (int m = 1; m <= ng; ++m) { a(i, j, -m) = lo; a(i, j, nz - 1 + m) = hi; }
            }
    const int cc[3] = {0, 0, 0};
    fill_periodic(a, g, cc);
}

// Wall-normal temperature gradient at z-lo, rho q / alpha_eff (ABLTempWallFunc,
// ABLWallFunction.cpp:392-480) with the heat flux q of the shear-stress model
// (ShearStress.H:22-167); neutral surface (surface_temp_flux = 0): the surface
// temperature equals theta_mean (MOData.cpp:66-71) and phi_h = ln(z_ref / z0t).
void Sim::theta_wall_gradient(std::vector<double>& gz) const {
    const int nx = g.n[0], ny = g.n[1];
    gz.assign((size_t)nx * ny, 0.0);
    if (tzlo != 1) return;
    const double phi_h = std::log(zref / z0t);
    const double ts = theta_mean;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double u = vel_old(i, j, 0, 0), v = vel_old(i, j, 0, 1);
            const double wspd = std::sqrt(u * u + v * v);
            const double th = theta_old(i, j, 0);
            double q;
            if (shear_type == "moeng") {
                const double term1 = utau * kappa / (vmag_mean * phi_h);
                q = term1 * ((th - theta_mean) * vmag_mean + (theta_mean - ts) * wspd);
            } else if (shear_type == "constant") {
                q = utau * kappa / phi_h * (theta_mean - ts);
            } else {  // local, schumann
                q = utau * kappa / phi_h * (th - ts);
            }
            gz[(size_t)j * nx + i] = rho * q / alpha(i, j, 0);
        }
}

// div(alpha grad theta): MLABecLaplacian apply with alpha 0, beta -1, face
// diffusivity the mean of the two cells (the cell value on domain faces), z
// boundaries through one ghost layer: Neumann 0 (slip wall), the wall-model
// gradient at z-lo, the fixed gradient at z-hi (incflo_diffusion.cpp:71-104).
void Sim::tdiff_op(const Arr& th_in, Arr& out) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    Arr q;
    def_cc(q, g, 1, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) q(i, j, k) = th_in(i, j, k);
    std::vector<double> gz;
    theta_wall_gradient(gz);
    if (!g.per[2])
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                q(i, j, -1) = q(i, j, 0) - (tzlo == 1 ? gz[(size_t)j * nx + i] : 0.0) * g.dx[2];
                q(i, j, nz) = q(i, j, nz - 1) + (tzhi == 2 ? tgrad_hi : 0.0) * g.dx[2];
            }
    const int cc[3] = {0, 0, 0};
    fill_periodic(q, g, cc);
    Arr a;
    def_cc(a, g, 1, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) a(i, j, k) = alpha(i, j, k);
    fill_cc_foextrap(a);
    const double dx = g.dx[0], dy = g.dx[1], dz = g.dx[2];
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                auto fx = [&](int ii) { return 0.5 * (a(ii - 1, j, k) + a(ii, j, k)) * (q(ii, j, k) - q(ii - 1, j, k)) / dx; };
                auto fy = [&](int jj) { return 0.5 * (a(i, jj - 1, k) + a(i, jj, k)) * (q(i, jj, k) - q(i, jj - 1, k)) / dy; };
                auto fz = [&](int kk) {
                    double af;
                    if (!g.per[2] && kk == 0) af = a(i, j, 0);
                    else if (!g.per[2] && kk == nz) af = a(i, j, nz - 1);
                    else af = 0.5 * (a(i, j, kk - 1) + a(i, j, kk));
                    return af * (q(i, j, kk) - q(i, j, kk - 1)) / dz;
                };
                out(i, j, k) = (fx(i + 1) - fx(i)) / dx + (fy(j + 1) - fy(j)) / dy + (fz(k + 1) - fz(k)) / dz;
            }
}

// rho theta - dtd div(alpha grad theta) = rho theta_rhs (DiffSolverIface::linsys_solve
// with MLABecLaplacian), solved by Jacobi iterations to MLMG's target
void Sim::tdiffuse_solve(double dtd) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    Arr b, L, R, Dg;
    def_cc(b, g, 0, 1); def_cc(L, g, 0, 1); def_cc(R, g, 0, 1); def_cc(Dg, g, 0, 1);
    Arr a;
    def_cc(a, g, 1, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) a(i, j, k) = alpha(i, j, k);
    fill_cc_foextrap(a);
    const double ih2[3] = {1.0 / (g.dx[0] * g.dx[0]), 1.0 / (g.dx[1] * g.dx[1]), 1.0 / (g.dx[2] * g.dx[2])};
    double bnorm = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double c0 = a(i, j, k);
                double s = (0.5 * (a(i - 1, j, k) + c0) + 0.5 * (a(i + 1, j, k) + c0)) * ih2[0] +
                           (0.5 * (a(i, j - 1, k) + c0) + 0.5 * (a(i, j + 1, k) + c0)) * ih2[1];
                const double zlo = (!g.per[2] && k == 0) ? 0.0 : 0.5 * (a(i, j, k - 1) + c0);
                const double zhi = (!g.per[2] && k == nz - 1) ? 0.0 : 0.5 * (a(i, j, k + 1) + c0);
                s += (zlo + zhi) * ih2[2];
                Dg(i, j, k) = rho + dtd * s;
                b(i, j, k) = rho * theta(i, j, k);
                bnorm = std::max(bnorm, std::fabs(b(i, j, k)));
            }
    auto residual = [&]() {
        tdiff_op(theta, L);
        double rn = 0;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double r = b(i, j, k) - rho * theta(i, j, k) + dtd * L(i, j, k);
                    R(i, j, k) = r;
                    rn = std::max(rn, std::fabs(r));
                }
        if (!std::isfinite(rn)) throw Error(ERR_NONFINITE, "temperature diffusion solve diverged");
        return rn;
    };
    double rn = residual();
    const double target = std::max(tdif.atol, tdif.rtol * std::max(bnorm, rn));
    int it = 0;
    while (rn > target) {
        if (++it > 200000) throw Error(ERR_NOT_CONVERGED, "oracle Jacobi iterations of the temperature solve did not converge");
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) theta(i, j, k) += R(i, j, k) / Dg(i, j, k);
        rn = residual();
    }
    tdiff_iters = it;
}

// The scalar part of ApplyPredictor (incflo_advance.cpp:296-341) after the MAC
// projection: Godunov fluxes of rho theta with the forces src + diff
// (AdvOp_Godunov.H:114-329), sources at NPH (none), predictor_rhs, explicit RK2
// correction or the diffusion solve, theta_nph = (theta_old + theta) / 2.
// diff_term(Old) (tdiff) and alpha_eff are formed before the MAC projection.
void Sim::temperature_predictor(double dt) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    Arr q, fq;
    def_cc(q, g, 3, 1);
    def_cc(fq, g, 1, 1);
    fill_scalar(theta_old);
    for (size_t m = 0; m < q.d.size(); ++m) q.d[m] = rho * theta_old.d[m];
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) fq(i, j, k) = tsrc(i, j, k) + tdiff(i, j, k);
    fill_cc_foextrap(fq);
    advect_field(q, fq, -1, dt, tconv);
    tsrc.setval(0.0);  // compute_source_term(NPH): the deck has no temperature sources
    const double fac = diff_type == 0 ? 1.0 : (diff_type == 1 ? 0.5 : 0.0);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                theta(i, j, k) = (rho * theta_old(i, j, k) + dt * (tconv(i, j, k) + tsrc(i, j, k) + fac * tdiff(i, j, k))) / rho;
    if (diff_type == 0) {
        tdiff_op(theta, tdiff_new);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) theta(i, j, k) += 0.5 * dt * (tdiff_new(i, j, k) - tdiff(i, j, k)) / rho;
    } else {
        tdiffuse_solve(diff_type == 2 ? dt : 0.5 * dt);
    }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) theta_nph(i, j, k) = 0.5 * theta_old(i, j, k) + 0.5 * theta(i, j, k);
}

// ---- post-MAC advective fluxes ----------------------------------------------------------------------
// HydroUtils::ComputeFluxesOnBoxFromState + ComputeDivergence
// (icns_advection.H:250-442 for q = rho u; AdvOp_Godunov.H:114-329 for
// q = rho theta of a scalar) with conservative transverse terms (dt/3 corner
// corrections), forces added at the end, flux = u_mac * q_edge, conv =
// -div(flux).  q and fq carry three ghost layers and one; component `normal`
// (2 for the velocity, -1 for a scalar) is the Dirichlet-0 one at z walls.
void Sim::advection(double dt) {
    Arr q, fq;
    def_cc(q, g, 3, 3);
    def_cc(fq, g, 1, 3);
    fill_vel(vel_old);
    for (size_t m = 0; m < q.d.size(); ++m) q.d[m] = rho * vel_old.d[m];
    fill_cc_foextrap(forces);
    for (size_t m = 0; m < fq.d.size(); ++m) fq.d[m] = rho * forces.d[m];
    advect_field(q, fq, 2, dt, conv);
}

void Sim::advect_field(const Arr& q, const Arr& fq, int normal, double dt, Arr& out) {
    const Geo& G = g;
    const int nx = G.n[0], ny = G.n[1], nz = G.n[2];
    const int nc = q.nc;
    const Arr* fv[3] = {&umac, &vmac, &wmac};
    Traces T;
    compute_traces(q, G, dt, 1, nullptr, fv, T);
    Arr lo[3], hi[3], edge[3];
    for (int d = 0; d < 3; ++d) {
        def_face(lo[d], G, d, nc);
        def_face(hi[d], G, d, nc);
        def_face(edge[d], G, d, nc);
        Arr& A = lo[d];
        for (int n = 0; n < nc; ++n)
#pragma omp parallel for collapse(2)
            for (int k = A.lo[2]; k <= A.hi[2]; ++k)
                for (int j = A.lo[1]; j <= A.hi[1]; ++j)
                    for (int i = A.lo[0]; i <= A.hi[0]; ++i) {
                        int c[3] = {i, j, k};
                        const bool wall = (d == 2 && !G.per[2] && (k == 0 || k == nz));
                        double l = 0, h = 0;
                        c[d] -= 1;
                        if (!(wall && k == 0)) l = T.Ip[d](c[0], c[1], c[2], n);
                        c[d] += 1;
                        if (!(wall && k == nz)) h = T.Im[d](c[0], c[1], c[2], n);
                        if (d == 2) zedge_bc(G, k, n == normal, l, h);
                        lo[d](i, j, k, n) = l;
                        hi[d](i, j, k, n) = h;
                        edge[d](i, j, k, n) = upwind((*fv[d])(i, j, k), l, h);
                    }
    }
    // transverse states for all components: tr[a][b] on a-faces corrected by b
    Arr tr[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            def_trans(tr[a][b], G, a, b, nc);
            Arr& R = tr[a][b];
            const double cb = dt / (3.0 * G.dx[b]);
            for (int n = 0; n < nc; ++n)
#pragma omp parallel for collapse(2)
                for (int k = R.lo[2]; k <= R.hi[2]; ++k)
                    for (int j = R.lo[1]; j <= R.hi[1]; ++j)
                        for (int i = R.lo[0]; i <= R.hi[0]; ++i) {
                            const bool wall = (a == 2 && !G.per[2] && (k == 0 || k == nz));
                            double l = lo[a](i, j, k, n), h = hi[a](i, j, k, n);
                            auto corr = [&](int* cell) {
                                int p[3] = {cell[0], cell[1], cell[2]};
                                p[b] += 1;
                                const double vp = (*fv[b])(p[0], p[1], p[2]), vm = (*fv[b])(cell[0], cell[1], cell[2]);
                                return -cb * (vp * edge[b](p[0], p[1], p[2], n) - vm * edge[b](cell[0], cell[1], cell[2], n)) +
                                       cb * q(cell[0], cell[1], cell[2], n) * (vp - vm);
                            };
                            int c[3] = {i, j, k};
                            if (!(wall && k == nz)) h += corr(c);
                            int cl[3] = {i, j, k};
                            cl[a] -= 1;
                            if (!(wall && k == 0)) l += corr(cl);
                            if (a == 2) zedge_bc(G, k, n == normal, l, h);
                            R(i, j, k, n) = upwind((*fv[a])(i, j, k), l, h);
                        }
        }
    // final states and fluxes
    Arr F[3];
    F[0].define(0, 0, 0, nx, ny - 1, nz - 1, nc);
    F[1].define(0, 0, 0, nx - 1, ny, nz - 1, nc);
    F[2].define(0, 0, 0, nx - 1, ny - 1, nz, nc);
    for (int d = 0; d < 3; ++d) {
        const int b1 = (d + 1) % 3, b2 = (d + 2) % 3;
        const double c1 = dt / (2.0 * G.dx[b1]), c2 = dt / (2.0 * G.dx[b2]);
        Arr& R = F[d];
        for (int n = 0; n < nc; ++n)
#pragma omp parallel for collapse(2)
            for (int k = 0; k <= R.hi[2]; ++k)
                for (int j = 0; j <= R.hi[1]; ++j)
                    for (int i = 0; i <= R.hi[0]; ++i) {
                        const bool wall = (d == 2 && !G.per[2] && (k == 0 || k == nz));
                        auto side = [&](int* cell, double base) {
                            int p1[3] = {cell[0], cell[1], cell[2]};
                            p1[b1] += 1;
                            int p2[3] = {cell[0], cell[1], cell[2]};
                            p2[b2] += 1;
                            const double v1p = (*fv[b1])(p1[0], p1[1], p1[2]), v1m = (*fv[b1])(cell[0], cell[1], cell[2]);
                            const double v2p = (*fv[b2])(p2[0], p2[1], p2[2]), v2m = (*fv[b2])(cell[0], cell[1], cell[2]);
                            double s = base;
                            s -= c1 * (tr[b1][b2](p1[0], p1[1], p1[2], n) * v1p - tr[b1][b2](cell[0], cell[1], cell[2], n) * v1m);
                            s -= c2 * (tr[b2][b1](p2[0], p2[1], p2[2], n) * v2p - tr[b2][b1](cell[0], cell[1], cell[2], n) * v2m);
                            s += c1 * q(cell[0], cell[1], cell[2], n) * (v1p - v1m);
                            s += c2 * q(cell[0], cell[1], cell[2], n) * (v2p - v2m);
                            s += 0.5 * dt * fq(cell[0], cell[1], cell[2], n);
                            return s;
                        };
                        int c[3] = {i, j, k};
                        int cl[3] = {i, j, k};
                        cl[d] -= 1;
                        double stl = 0, sth = 0;
                        if (!(wall && k == 0)) stl = side(cl, lo[d](i, j, k, n));
                        if (!(wall && k == nz)) sth = side(c, hi[d](i, j, k, n));
                        if (d == 2) zedge_bc(G, k, n == normal, stl, sth);
                        const double um = (*fv[d])(i, j, k);
                        double st = (um >= 0.0) ? stl : sth;
                        if (std::fabs(um) < kSmallVel) st = 0.5 * (stl + sth);
                        R(i, j, k, n) = um * st;
                    }
    }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int n = 0; n < nc; ++n)
                    out(i, j, k, n) = -((F[0](i + 1, j, k, n) - F[0](i, j, k, n)) / G.dx[0] +
                                         (F[1](i, j + 1, k, n) - F[1](i, j, k, n)) / G.dx[1] +
                                         (F[2](i, j, k + 1, n) - F[2](i, j, k, n)) / G.dx[2]);
}

// ---- nodal projection ---------------------------------------------------------------------------------
// Q1 finite-element nodal Laplacian (the MLNodeLaplacian discretisation),
// nodal divergence of the cell velocity, cell-averaged nodal gradient.
struct NDLevel {
    int n[3];   // cells
    int nn[3];  // nodes
    double h[3];
    Arr phi, rhs, res, tmp;
    double w[3][3];  // 27-point weights W[a+1][b+1][c+1] are built below
    double W[27];
};

static void nd_weights(NDLevel& L) {
    double sg[3][3], mu[3] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0};
    for (int d = 0; d < 3; ++d) {
        const double i2 = 1.0 / (L.h[d] * L.h[d]);
        sg[d][0] = -i2; sg[d][1] = 2 * i2; sg[d][2] = -i2;
    }
    for (int c = 0; c < 3; ++c)
        for (int b = 0; b < 3; ++b)
            for (int a = 0; a < 3; ++a)
                L.W[(c * 3 + b) * 3 + a] = -(sg[0][a] * mu[b] * mu[c] + mu[a] * sg[1][b] * mu[c] + mu[a] * mu[b] * sg[2][c]);
}

static void nd_fill(Arr& a, const NDLevel& L, bool zper) {
    const int nx = L.nn[0], ny = L.nn[1], nz = L.nn[2];
    for (int k = -1; k <= nz; ++k)
        for (int j = -1; j <= ny; ++j)
            for (int i = -1; i <= nx; ++i) {
                if (i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz) continue;
                int ii = (i + nx) % nx, jj = (j + ny) % ny, kk;
                if (zper) kk = (k + nz) % nz;
                else kk = (k < 0) ? -k : (k >= nz ? 2 * (nz - 1) - k : k);
                a(i, j, k) = a(ii, jj, kk);
            }
}

static double nd_apply(const NDLevel& L, double sigma, int i, int j, int k) {
    double s = 0;
    for (int c = -1; c <= 1; ++c)
        for (int b = -1; b <= 1; ++b)
            for (int a = -1; a <= 1; ++a) s += L.W[((c + 1) * 3 + b + 1) * 3 + a + 1] * L.phi(i + a, j + b, k + c);
    return sigma * s;
}

static void nd_smooth(NDLevel& L, double sigma, bool zper, int sweeps, double omega) {
    const double diag = sigma * L.W[13];
    for (int s = 0; s < sweeps; ++s) {
        nd_fill(L.phi, L, zper);
#pragma omp parallel for collapse(2)
        for (int k = 0; k < L.nn[2]; ++k)
            for (int j = 0; j < L.nn[1]; ++j)
                for (int i = 0; i < L.nn[0]; ++i)
                    L.tmp(i, j, k) = L.phi(i, j, k) + omega * (L.rhs(i, j, k) - nd_apply(L, sigma, i, j, k)) / diag;
#pragma omp parallel for collapse(2)
        for (int k = 0; k < L.nn[2]; ++k)
            for (int j = 0; j < L.nn[1]; ++j)
                for (int i = 0; i < L.nn[0]; ++i) L.phi(i, j, k) = L.tmp(i, j, k);
    }
}

static double nd_residual(NDLevel& L, double sigma, bool zper) {
    nd_fill(L.phi, L, zper);
    double mx = 0;
#pragma omp parallel for collapse(2) reduction(max : mx)
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                L.res(i, j, k) = L.rhs(i, j, k) - nd_apply(L, sigma, i, j, k);
                mx = std::max(mx, std::fabs(L.res(i, j, k)));
            }
    return mx;
}

static void nd_vcycle(std::vector<NDLevel>& Ls, size_t l, double sigma, bool zper, const MGOpts& o) {
    NDLevel& L = Ls[l];
    if (l + 1 == Ls.size()) {
        nd_smooth(L, sigma, zper, o.bottom, o.omega);
        return;
    }
    nd_smooth(L, sigma, zper, o.nu1, o.omega);
    nd_residual(L, sigma, zper);
    nd_fill(L.res, L, zper);
    NDLevel& C = Ls[l + 1];
    const double w1[3] = {0.25, 0.5, 0.25};
#pragma omp parallel for collapse(2)
    for (int k = 0; k < C.nn[2]; ++k)
        for (int j = 0; j < C.nn[1]; ++j)
            for (int i = 0; i < C.nn[0]; ++i) {
                double s = 0;
                for (int c = -1; c <= 1; ++c)
                    for (int b = -1; b <= 1; ++b)
                        for (int a = -1; a <= 1; ++a) s += w1[a + 1] * w1[b + 1] * w1[c + 1] * L.res(2 * i + a, 2 * j + b, 2 * k + c);
                C.rhs(i, j, k) = s;
                C.phi(i, j, k) = 0.0;
            }
    nd_vcycle(Ls, l + 1, sigma, zper, o);
    nd_fill(C.phi, C, zper);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int ci = i / 2, cj = j / 2, ck = k / 2;
                const int oi = i & 1, oj = j & 1, ok = k & 1;
                double s = 0;
                for (int c = 0; c <= ok; ++c)
                    for (int b = 0; b <= oj; ++b)
                        for (int a = 0; a <= oi; ++a) s += C.phi(ci + a, cj + b, ck + c);
                L.phi(i, j, k) += s / (double)((1 + oi) * (1 + oj) * (1 + ok));
            }
    nd_smooth(L, sigma, zper, o.nu2, o.omega);
}

// Weighted-Jacobi weight of the nodal smoother.  The largest eigenvalue of
// D^-1 A for the Q1 stencil lies at a corner of the frequency cube; it is 1.5
// on isotropic cells (omega 0.9 gives omega * lambda_max = 1.35) and grows with
// the cell aspect ratio (3.0 at dz = dx / 2, where omega = 0.9 diverges).  The
// weight is reduced so that omega * lambda_max stays at 1.35.
static double nodal_jacobi_weight(const double* W, double omega) {
    double lmax = 0.0;
    for (int m = 1; m < 8; ++m) {
        double A = 0.0;
        for (int c = 0; c < 3; ++c)
            for (int b = 0; b < 3; ++b)
                for (int a = 0; a < 3; ++a) {
                    double f = 1.0;
                    if ((m & 1) && a != 1) f = -f;
                    if ((m & 2) && b != 1) f = -f;
                    if ((m & 4) && c != 1) f = -f;
                    A += W[(c * 3 + b) * 3 + a] * f;
                }
        lmax = std::max(lmax, A / W[13]);
    }
    if (omega * lmax > 1.35 * (1.0 + 1e-9)) omega = 1.35 / lmax;
    return omega;
}

static std::vector<NDLevel> nd_levels(const Geo& g) {
    std::vector<NDLevel> Ls;
    int n[3] = {g.n[0], g.n[1], g.n[2]};
    double h[3] = {g.dx[0], g.dx[1], g.dx[2]};
    while (true) {
        NDLevel L;
        for (int d = 0; d < 3; ++d) {
            L.n[d] = n[d];
            L.h[d] = h[d];
            L.nn[d] = n[d] + ((d == 2 && !g.per[2]) ? 1 : 0);
        }
        L.phi.define(-1, -1, -1, L.nn[0], L.nn[1], L.nn[2], 1);
        L.res.define(-1, -1, -1, L.nn[0], L.nn[1], L.nn[2], 1);
        L.rhs.define(0, 0, 0, L.nn[0] - 1, L.nn[1] - 1, L.nn[2] - 1, 1);
        L.tmp.define(0, 0, 0, L.nn[0] - 1, L.nn[1] - 1, L.nn[2] - 1, 1);
        nd_weights(L);
        Ls.push_back(std::move(L));
        bool can = true;
        for (int d = 0; d < 3; ++d) can = can && (n[d] % 4 == 0);
        if (!can) break;
        for (int d = 0; d < 3; ++d) { n[d] /= 2; h[d] *= 2; }
    }
    return Ls;
}

// Nodal divergence of a cell velocity (NodalProjector::computeRHS, the
// MLNodeLaplacian right-hand side, absent AMReX submodule; call site
// src/projection/incflo_apply_nodal_projection.cpp:344-355): at each node the
// mean over the four surrounding cell edges of each direction's difference,
// with the velocity zero outside a wall (setBndry(0)) and periodic wrap; wall
// nodes see half the support and are scaled by 2.  out: nodes (nx, ny, nzn).
static void nodal_divergence(const Geo& g, const Arr& vel, Arr& out) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const bool zper = g.per[2];
    Arr v;
    def_cc(v, g, 1, 3);
    for (int n = 0; n < 3; ++n)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) v(i, j, k, n) = vel(i, j, k, n);
    const int cc[3] = {0, 0, 0};
    fill_periodic(v, g, cc);
    const int nzn = nz + (zper ? 0 : 1);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nzn; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double dv = 0;
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b) {
                        dv += 0.25 / g.dx[0] * (v(i, j - b, k - c, 0) - v(i - 1, j - b, k - c, 0));
                        dv += 0.25 / g.dx[1] * (v(i - b, j, k - c, 1) - v(i - b, j - 1, k - c, 1));
                        dv += 0.25 / g.dx[2] * (v(i - b, j - c, k, 2) - v(i - b, j - c, k - 1, 2));
                    }
                if (!zper && (k == 0 || k == nzn - 1)) dv *= 2.0;
                out(i, j, k) = dv;
            }
}

// Post-projection diagnostic: max-norm of the divergence of the MAC face
// velocities (1/s; the MAC projection is exact, so this is its residual);
// umax receives the largest face speed.
double Sim::mac_divu(double* umax) const {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    double m = 0, mu = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double r = (umac(i + 1, j, k) - umac(i, j, k)) / g.dx[0] + (vmac(i, j + 1, k) - vmac(i, j, k)) / g.dx[1] +
                                 (wmac(i, j, k + 1) - wmac(i, j, k)) / g.dx[2];
                m = std::max(m, std::fabs(r));
                mu = std::max(mu, std::max(std::fabs(umac(i, j, k)), std::max(std::fabs(vmac(i, j, k)), std::fabs(wmac(i, j, k)))));
            }
    if (umax) *umax = mu;
    return m;
}

// Post-projection diagnostic: max-norm of the nodal divergence of the current
// velocity (1/s; the nodal projection is approximate, so this is
// truncation-sized); umax receives max |u| over all components.
double Sim::divu(double* umax) const {
    const int nzn = g.n[2] + (g.per[2] ? 0 : 1);
    Arr d;
    d.define(0, 0, 0, g.n[0] - 1, g.n[1] - 1, nzn - 1, 1);
    nodal_divergence(g, vel, d);
    double m = 0, mu = 0;
    for (double x : d.d) m = std::max(m, std::fabs(x));
    for (int n = 0; n < 3; ++n)
        for (int k = 0; k < g.n[2]; ++k)
            for (int j = 0; j < g.n[1]; ++j)
                for (int i = 0; i < g.n[0]; ++i) mu = std::max(mu, std::fabs(vel(i, j, k, n)));
    if (umax) *umax = mu;
    return m;
}

// incflo::ApplyProjection (src/projection/incflo_apply_nodal_projection.cpp:149-465)
void Sim::nodal_project(double time, double scaling, bool incremental) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const bool zper = g.per[2];
    const bool small_dt = (time > 0.0 && t.dt[0] < 0.1 * t.dt[1]);
    if (!incremental)
        for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) vel(i, j, k, n) += gp(i, j, k, n) * scaling / rho;
    if (small_dt || incremental)
        for (int n = 0; n < 3; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) vel(i, j, k, n) -= vel_old(i, j, k, n);
    const double sigma = scaling / rho;
    std::vector<NDLevel> Ls = nd_levels(g);
    NDLevel& L = Ls[0];
    nodal_divergence(g, vel, L.rhs);
    const int nzn = L.nn[2];
    double wsum = 0, wtot = 0;
#pragma omp parallel for collapse(2) reduction(+ : wsum, wtot)
    for (int k = 0; k < nzn; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double w = (!zper && (k == 0 || k == nzn - 1)) ? 0.5 : 1.0;
                wsum += w * L.rhs(i, j, k);
                wtot += w;
            }
    const double mean = wsum / wtot;
    for (auto& x : L.rhs.d) x -= mean;
    double r0 = nd_residual(L, sigma, zper);
    nodal_res0 = r0;
    const double target = std::max(nod.atol, nod.rtol * r0);
    int it = 0;
    double rn = r0;
    MGOpts o = nod;
    o.omega = nodal_jacobi_weight(L.W, nod.omega);
    while (rn > target && it < nod.maxiter) {
        nd_vcycle(Ls, 0, sigma, zper, o);
        rn = nd_residual(L, sigma, zper);
        ++it;
        if (!std::isfinite(rn)) throw Error(ERR_NONFINITE, "nodal projection diverged");
        if (rn > 1e20 * r0) throw Error(ERR_NOT_CONVERGED, "nodal projection diverged (residual above 1e20 times the initial one)");
    }
    if (rn > target && !nod.fixed_iters) throw Error(ERR_NOT_CONVERGED, "nodal projection did not converge in nodal_proj.maxiter V-cycles");
    nodal_iters = it;
    nodal_res = rn;
    nd_fill(L.phi, L, zper);
    Arr& f = L.phi;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double gx = 0, gy = 0, gz = 0;
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b) {
                        gx += f(i + 1, j + b, k + c) - f(i, j + b, k + c);
                        gy += f(i + b, j + 1, k + c) - f(i + b, j, k + c);
                        gz += f(i + b, j + c, k + 1) - f(i + b, j + c, k);
                    }
                const double G[3] = {0.25 * gx / g.dx[0], 0.25 * gy / g.dx[1], 0.25 * gz / g.dx[2]};
                for (int n = 0; n < 3; ++n) {
                    vel(i, j, k, n) -= sigma * G[n];
                    if (small_dt || incremental) vel(i, j, k, n) += vel_old(i, j, k, n);
                    if (incremental) gp(i, j, k, n) += G[n];
                    else gp(i, j, k, n) = G[n];
                }
            }
    for (int k = 0; k < nzn; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                if (incremental) p(i, j, k) += f(i, j, k);
                else p(i, j, k) = f(i, j, k);
            }
}

// ---- compute_dt (src/incflo_compute_dt.cpp:33-221) ------------------------------------------
void Sim::compute_dt() {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    double conv = 0, diff = 0, frc = 0;
    const double dxi[3] = {1 / g.dx[0], 1 / g.dx[1], 1 / g.dx[2]};
    const double dxinv2 = 2.0 * (dxi[0] * dxi[0] + dxi[1] * dxi[1] + dxi[2] * dxi[2]);
#pragma omp parallel for collapse(2) reduction(max : conv, diff, frc)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                for (int n = 0; n < 3; ++n) {
                    conv = std::max(conv, std::fabs(vel(i, j, k, n)) * dxi[n]);
                    frc = std::max(frc, std::fabs(src(i, j, k, n)) * dxi[n] / rho);
                }
                diff = std::max(diff, mueff(i, j, k) * dxinv2 / rho);
            }
    if (!t.use_force_cfl) frc = 0;
    if (diff_type != 0) diff = 0;  // incflo_compute_dt.cpp:37,140-145,211-214: explicit diffusion only
    t.set_current_cfl(conv, diff, frc);
}

// ---- actuator disks -------------------------------------------------------------------------------------
static void rotate(const double* ax, double ang, const double* v, double* out) {
    const double c = std::cos(ang), s = std::sin(ang);
    const double d = ax[0] * v[0] + ax[1] * v[1] + ax[2] * v[2];
    const double cr[3] = {ax[1] * v[2] - ax[2] * v[1], ax[2] * v[0] - ax[0] * v[2], ax[0] * v[1] - ax[1] * v[0]};
    for (int m = 0; m < 3; ++m) out[m] = v[m] * c + cr[m] * s + ax[m] * d * (1 - c);
}

// Sampling points of a disk and their area weights (ops::base::compute_disk_points,
// src/wind_energy/actuator/disk/disk_ops.cpp:373-412, with the sampling vector as the
// cylinder axis and diameters_to_sample as the offset; AreaComputer::weight,
// disk_ops.cpp:105-123): the reference vector khat x axis (compute_coplanar_vector,
// disk_ops.cpp:322-326) is rotated about the axis by 2 pi j / nt at radius
// dr (i + 1/2) (dr i for a single radial point), radius-major; the weight of ring i is
// ((i + 1)^2 - i^2) / (nr^2 nt).
static void sample_points(const DiskParams& dp, std::vector<double>& x, std::vector<double>& w) {
    const double* ax = dp.sample;
    double refv[3] = {-ax[1], ax[0], 0.0};
    {
        double m = std::sqrt(refv[0] * refv[0] + refv[1] * refv[1]);
        refv[0] /= m; refv[1] /= m;
    }
    const double drs = 0.5 * dp.diameter / dp.nr;
    const double shift = dp.nr == 1 ? 0.0 : 0.5;
    x.assign(3 * (size_t)dp.nr * dp.nt, 0.0);
    w.assign((size_t)dp.nr * dp.nt, 0.0);
    for (int ir = 0; ir < dp.nr; ++ir)
        for (int it = 0; it < dp.nt; ++it) {
            const size_t p = (size_t)ir * dp.nt + it;
            double rp[3];
            rotate(ax, 2 * kPi / dp.nt * it, refv, rp);
            for (int m = 0; m < 3; ++m) x[3 * p + m] = dp.center[m] + dp.diameters_to_sample * dp.diameter * ax[m] + drs * (ir + shift) * rp[m];
            w[p] = ((ir + 1.0) * (ir + 1.0) - (double)ir * ir) / ((double)dp.nr * dp.nr * dp.nt);
        }
}

// Actuator::pre_advance_work (src/wind_energy/actuator/Actuator.cpp:148-158):
// trilinear sampling (ActuatorContainer.cpp:284-360), area-weighted average
// (disk_ops.H:144-169), Ct table (disk_ops.H:128-134), uniform-Ct force
// (uniform_ct_ops.H:71-97), Gaussian spreading (disk_spreading.H:45-105,
// actuator_utils.H:45-60).
void Sim::actuator_update() {
    if (!src_act) return;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    fill_vel(vel);
    act_src.setval(0.0);
    for (auto& dp : disks) {
        const double R = 0.5 * dp.diameter;
        // sampling points on the upstream (sample) disk
        double ref[3] = {0, 0, 0};
        std::vector<double> xs, ws;
        sample_points(dp, xs, ws);
        for (int ir = 0; ir < dp.nr; ++ir) {
            for (int it = 0; it < dp.nt; ++it) {
                const size_t p = (size_t)ir * dp.nt + it;
                const double wgt = ws[p];
                const double* x = &xs[3 * p];
                const double fx = (x[0] - g.plo[0] - 0.5 * g.dx[0]) / g.dx[0];
                const double fy = (x[1] - g.plo[1] - 0.5 * g.dx[1]) / g.dx[1];
                const double fz = (x[2] - g.plo[2] - 0.5 * g.dx[2]) / g.dx[2];
                const int i = (int)std::floor(fx), j = (int)std::floor(fy), k = (int)std::floor(fz);
                const double wx = fx - i, wy = fy - j, wz = fz - k;
                if (k < -1 || k + 1 > nz || i < -1 || i + 1 > nx || j < -1 || j + 1 > ny)
                    throw Error(ERR_DECK, "actuator sample outside domain");
                for (int n = 0; n < 3; ++n) {
                    double s = 0;
                    for (int c = 0; c < 2; ++c)
                        for (int b = 0; b < 2; ++b)
                            for (int a = 0; a < 2; ++a) {
                                const int ii = ((i + a) % nx + nx) % nx, jj = ((j + b) % ny + ny) % ny;
                                const double w = (a ? wx : 1 - wx) * (b ? wy : 1 - wy) * (c ? wz : 1 - wz);
                                s += w * vel(ii, jj, k + c, n);
                            }
                    ref[n] += s * wgt;
                }
            }
        }
        for (int n = 0; n < 3; ++n) dp.ref_vel[n] = ref[n];
        const double* ax = dp.normal;  // U_inf is the sampled velocity along the disk normal; the force ring lies in the disk plane
        const double un = ref[0] * ax[0] + ref[1] * ax[1] + ref[2] * ax[2];
        dp.uinf_sqr = un * un;
        // linear table with end clamping
        const double umag = std::sqrt(dp.uinf_sqr);
        const auto& X = dp.wind_speed;
        const auto& Y = dp.ct;
        if (X.size() == 1 || umag <= X.front()) dp.current_ct = Y.front();
        else if (umag >= X.back()) dp.current_ct = Y.back();
        else {
            size_t m = 0;
            while (m + 1 < X.size() && X[m + 1] < umag) ++m;
            dp.current_ct = Y[m] + (Y[m + 1] - Y[m]) * (umag - X[m]) / (X[m + 1] - X[m]);
        }
        const double aero = 0.5 * dp.uinf_sqr * dp.current_ct;
        std::vector<double> fmag(dp.nr);
        for (int ip = 0; ip < dp.nr; ++ip) {
            const double r = (ip + 0.5) * dp.dr, rp = r + 0.5 * dp.dr, rm = r - 0.5 * dp.dr;
            fmag[ip] = aero * kPi * (rp * rp - rm * rm);
        }
        // ring points (rotated force points)
        std::vector<double> pts;
        for (int ip = 0; ip < dp.nr; ++ip) {
            double pos[3];
            for (int m = 0; m < 3; ++m) pos[m] = dp.center[m] + (ip + 0.5) * dp.dr * dp.cvec[m];
            for (int it = 0; it < dp.nt; ++it) {
                const double ang = 2 * kPi / dp.nt * it;
                double out[3];
                if (dp.about_center) {
                    double rel[3] = {pos[0] - dp.center[0], pos[1] - dp.center[1], pos[2] - dp.center[2]};
                    rotate(ax, ang, rel, out);
                    for (int m = 0; m < 3; ++m) out[m] += dp.center[m];
                } else {
                    rotate(ax, ang, pos, out);  // disk_spreading.H:85-86 rotates the absolute position
                }
                pts.push_back(out[0]); pts.push_back(out[1]); pts.push_back(out[2]);
                pts.push_back(fmag[ip] / dp.nt);
            }
        }
        const double eps = dp.epsilon;
        const double gfac = 0.17958712212516656 / (eps * eps * eps);
        const int np = (int)pts.size() / 4;
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double x = g.plo[0] + (i + 0.5) * g.dx[0], y = g.plo[1] + (j + 0.5) * g.dx[1], z = g.plo[2] + (k + 0.5) * g.dx[2];
                    double s = 0;
                    for (int m = 0; m < np; ++m) {
                        const double rx = (pts[4 * m] - x) / eps, ry = (pts[4 * m + 1] - y) / eps, rz = (pts[4 * m + 2] - z) / eps;
                        const double r2 = rx * rx + ry * ry + rz * rz;
                        if (r2 < 16.0) s += gfac * std::exp(-rx * rx - ry * ry - rz * rz) * pts[4 * m + 3];
                    }
                    for (int n = 0; n < 3; ++n) act_src(i, j, k, n) += s * ax[n];
                }
    }
}

// ---- ApplyPredictor (src/incflo_advance.cpp:186-438), Godunov + explicit --------------------
void Sim::apply_predictor(bool incremental) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const double dt = t.dt[0];
    update_mueff(vel_old);
    const Arr* th_old = has_temp ? &theta_old : nullptr;
    compute_sources(vel_old, th_old);  // BoussinesqBuoyancy reads theta at Old (phi_state)
    divtau_op(vel_old, divtau);  // divtau with u = Old (copied into New)
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) forces(i, j, k, n) = (src(i, j, k, n) + divtau(i, j, k, n)) / rho;
    if (has_temp) {  // temperature sources at Old (none) and diff_term(Old)
        tsrc.setval(0.0);
        tdiff_op(theta_old, tdiff);
    }
    premac(dt);
    mac_project();
    if (has_temp) temperature_predictor(dt);
    advection(dt);
    // compute_source_term(NPH): Coriolis reads the Old velocity, BoussinesqBuoyancy
    // theta at n+1/2; compute_diffusion_term(Old) reproduces divtau.
    compute_sources(vel_old, has_temp ? &theta_nph : nullptr);
    // predictor_rhs (CompRHSOps.H:32-141): diffusion factor 1 explicit, 1/2 Crank-Nicolson, 0 implicit
    predictor_rhs(dt, diff_type == 0 ? 1.0 : (diff_type == 1 ? 0.5 : 0.0));
    if (diff_type != 0) {  // icns().solve(dt_diff), incflo_advance.cpp:376-386
        diffuse_solve(diff_type == 2 ? dt : 0.5 * dt);
        nodal_project(t.newt, dt, incremental);
        return;
    }
    // explicit RK2 correction (incflo_advance.cpp:388-400): divtau(New) - divtau(Old), then
    // improve_explicit_diffusion
    divtau_op(vel, divtau_new);
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) divtau_new(i, j, k, n) = divtau_new(i, j, k, n) - divtau(i, j, k, n);
    explicit_rk2_post_hoc(dt, divtau_new);
    nodal_project(incremental ? t.newt : t.newt, dt, incremental);
}

// ComputeRHSOp::predictor_rhs (src/equation_systems/CompRHSOps.H:32-141) for
// the explicit / Crank-Nicolson / implicit diffusion factor fac (1, 1/2, 0),
// constant density: u = (rho u_old + dt (conv + src + fac divtau)) / rho.
void Sim::predictor_rhs(double dt, double fac) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    vel(i, j, k, n) = (rho * vel_old(i, j, k, n) + dt * (conv(i, j, k, n) + src(i, j, k, n) + fac * divtau(i, j, k, n))) / rho;
}

// ComputeRHSOp::explicit_rk2_post_hoc (src/equation_systems/CompRHSOps.H:267-300):
// d holds divtau(New) - divtau(Old); u += 1/2 dt d / rho.
void Sim::explicit_rk2_post_hoc(double dt, const Arr& d) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) vel(i, j, k, n) += 0.5 * dt * d(i, j, k, n) / rho;
}

// ---- MOL scheme -------------------------------------------------------------------------------
// Monotonized-central slope of order 2 (AMReX's amrex_calc_{x,y,z}slope and
// their _extdir forms, AMReX_Slopes_K.H in the AMReX submodule): the minmod of
// the doubled one-sided differences and the central difference.  In the cell
// next to an ext_dir / hoextrap domain face (edge -1 low side, +1 high side)
// the central difference becomes the one-sided quadratic through the face value
// held in the ghost cell: (q+ + 3 q0 - 4 qb)/3 and (4 qb - 3 q0 - q-)/3.
static double mc_slope(double qm, double q0, double qp, int edge) {
    const double dl = 2.0 * (q0 - qm), dr = 2.0 * (qp - q0);
    double dc = 0.5 * (qp - qm);
    if (edge < 0) dc = (qp + 3.0 * q0 - 4.0 * qm) / 3.0;
    else if (edge > 0) dc = (4.0 * qp - 3.0 * q0 - qm) / 3.0;
    double s = std::min(std::fabs(dl), std::min(std::fabs(dc), std::fabs(dr)));
    if (!(dr * dl > 0.0)) s = 0.0;
    return dc > 0.0 ? s : -s;
}

// Slope along d of component n at cell (i, j, k) of a ghost-filled array.  Every
// velocity component is ext_dir (normal) or hoextrap (tangential) at a z wall,
// so the one-sided form applies at k = 0 and k = nz - 1 when z is bounded.
static double mol_slope(const Arr& a, const Geo& g, int d, int i, int j, int k, int n) {
    int c[3] = {i, j, k};
    c[d] -= 1;
    const double qm = a(c[0], c[1], c[2], n);
    c[d] += 2;
    const double qp = a(c[0], c[1], c[2], n);
    int edge = 0;
    if (d == 2 && !g.per[2]) edge = (k == 0) ? -1 : (k == g.n[2] - 1 ? 1 : 0);
    return mc_slope(qm, a(i, j, k, n), qp, edge);
}

// MOL::ExtrapVelToFaces (AMReX-Hydro's MOL velocity extrapolation, called from
// icns_advection.H:501-527 before the MAC projection): the normal velocity on
// each face from the MC-limited states of its two cells, zero where they
// diverge (umns < 0 < upls) or where their mean is below small_vel = 1e-10,
// else the upwind state.  A face on an ext_dir boundary (the normal component
// at a z wall) takes the ghost value, which is the wall velocity 0.
void Sim::mol_extrap(Arr& v) {
    fill_vel(v);
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const double small_vel = 1.0e-10;
    auto pick = [&](double umns, double upls) {
        if (umns < 0.0 && upls > 0.0) return 0.0;
        const double avg = 0.5 * (upls + umns);
        if (std::fabs(avg) < small_vel) return 0.0;
        return avg >= 0.0 ? umns : upls;
    };
    Arr* mac[3] = {&umac, &vmac, &wmac};
    for (int d = 0; d < 3; ++d) {
        const int hi[3] = {nx - 1 + (d == 0), ny - 1 + (d == 1), nz - 1 + (d == 2)};
        Arr& M = *mac[d];
#pragma omp parallel for collapse(2)
        for (int k = 0; k <= hi[2]; ++k)
            for (int j = 0; j <= hi[1]; ++j)
                for (int i = 0; i <= hi[0]; ++i) {
                    if (d == 2 && !g.per[2] && (k == 0 || k == nz)) { M(i, j, k) = 0.0; continue; }
                    int c[3] = {i, j, k};
                    c[d] -= 1;
                    const double umns = v(c[0], c[1], c[2], d) + 0.5 * mol_slope(v, g, d, c[0], c[1], c[2], d);
                    const double upls = v(i, j, k, d) - 0.5 * mol_slope(v, g, d, i, j, k, d);
                    M(i, j, k) = pick(umns, upls);
                }
    }
    const int fx[3] = {1, 0, 0}, fy[3] = {0, 1, 0}, fz[3] = {0, 0, 1};
    fill_periodic(umac, g, fx);
    fill_periodic(vmac, g, fy);
    fill_periodic(wmac, g, fz);
}

// MOL convective term (icns_advection.H:531-594: q = rho u,
// mol::compute_convective_fluxes and mol::compute_convective_rate,
// src/convection/incflo_mol_fluxes.cpp:9-268): the face state is the
// MC-limited extrapolation upwinded with the MAC velocity, the mean of both
// states where |u_mac| <= small_vel = FLT_EPSILON, and the ghost value on an
// ext_dir face; flux = q_face u_mac; conv = sum_d dxinv_d (F_lo - F_hi).
void Sim::mol_conv(Arr& v, Arr& out) {
    fill_vel(v);
    Arr q;
    def_cc(q, g, 3, 3);
    for (size_t m = 0; m < q.d.size(); ++m) q.d[m] = rho * v.d[m];
    mol_conv_field(q, 2, out);
}

// The same for a ghost-filled field q of any component count; component
// `normal` (2 for the velocity, -1 for a scalar) is ext_dir at z walls.
// Scalars are hoextrap there, so their wall faces take the slope branch
// (AdvOp_MOL.H:38-118 with the scalar's BCRec).
void Sim::mol_conv_field(const Arr& q, int normal, Arr& out) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const int nc = q.nc;
    const double small_vel = (double)std::numeric_limits<float>::epsilon();
    const Arr* mac[3] = {&umac, &vmac, &wmac};
    Arr F[3];
    F[0].define(0, 0, 0, nx, ny - 1, nz - 1, nc);
    F[1].define(0, 0, 0, nx - 1, ny, nz - 1, nc);
    F[2].define(0, 0, 0, nx - 1, ny - 1, nz, nc);
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < nc; ++n)
#pragma omp parallel for collapse(2)
            for (int k = 0; k <= F[d].hi[2]; ++k)
                for (int j = 0; j <= F[d].hi[1]; ++j)
                    for (int i = 0; i <= F[d].hi[0]; ++i) {
                        const double um = (*mac[d])(i, j, k);
                        double qs;
                        if (d == 2 && !g.per[2] && n == normal && (k == 0 || k == nz)) {
                            qs = q(i, j, k == 0 ? -1 : nz, n);  // ext_dir: the boundary value in the ghost cell
                        } else {
                            int c[3] = {i, j, k};
                            c[d] -= 1;
                            const double qmns = q(c[0], c[1], c[2], n) + 0.5 * mol_slope(q, g, d, c[0], c[1], c[2], n);
                            const double qpls = q(i, j, k, n) - 0.5 * mol_slope(q, g, d, i, j, k, n);
                            if (um > small_vel) qs = qmns;
                            else if (um < -small_vel) qs = qpls;
                            else qs = 0.5 * (qmns + qpls);
                        }
                        F[d](i, j, k, n) = qs * um;
                    }
    const double dxi[3] = {1.0 / g.dx[0], 1.0 / g.dx[1], 1.0 / g.dx[2]};
    for (int n = 0; n < nc; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    out(i, j, k, n) = (dxi[0] * (F[0](i, j, k, n) - F[0](i + 1, j, k, n))) +
                                      (dxi[1] * (F[1](i, j, k, n) - F[1](i, j + 1, k, n))) +
                                      (dxi[2] * (F[2](i, j, k, n) - F[2](i, j, k + 1, n)));
}

// The scalar parts of the MOL ApplyPredictor / ApplyCorrector
// (incflo_advance.cpp:296-341, 555-600): predictor — conv_term(Old) of rho
// theta from the MAC velocities of the Old state, predictor_rhs with the
// factor of the diffusion type, the solve (Crank-Nicolson / implicit);
// corrector — conv_term(New) (formed by the caller before mu_eff is updated),
// diff_term(New) for explicit diffusion, corrector_rhs (1/2, 1/2 explicit; 1/2,
// 0 Crank-Nicolson; 0, 0 implicit), the solve.  Both end with theta_nph =
// (theta_old + theta) / 2 for the buoyancy; no temperature sources.
void Sim::temperature_mol(bool corrector, double dt) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    if (!corrector) {
        Arr q;
        def_cc(q, g, 3, 1);
        fill_scalar(theta_old);
        for (size_t m = 0; m < q.d.size(); ++m) q.d[m] = rho * theta_old.d[m];
        mol_conv_field(q, -1, tconv_old);
        const double fac = diff_type == 0 ? 1.0 : (diff_type == 1 ? 0.5 : 0.0);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    theta(i, j, k) = (rho * theta_old(i, j, k) + dt * (tconv_old(i, j, k) + 0.0 + fac * tdiff(i, j, k))) / rho;
    } else {
        const double ofac = diff_type == 2 ? 0.0 : 0.5, nfac = diff_type == 0 ? 0.5 : 0.0;
        if (diff_type == 0) tdiff_op(theta, tdiff_new);  // wall data: Old theta and velocity, the new alpha_eff
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double dn = diff_type == 0 ? nfac * tdiff_new(i, j, k) : 0.0;
                    theta(i, j, k) = (rho * theta_old(i, j, k) +
                                      dt * (0.5 * (tconv_old(i, j, k) + tconv(i, j, k)) + ofac * tdiff(i, j, k) + dn + 0.0)) /
                                     rho;
                }
    }
    if (diff_type != 0) tdiffuse_solve(diff_type == 2 ? dt : 0.5 * dt);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) theta_nph(i, j, k) = 0.5 * theta_old(i, j, k) + 0.5 * theta(i, j, k);
}

// ApplyPredictor for MOL with explicit diffusion (src/incflo_advance.cpp:186-438):
// mu_eff and diff_term(Old) from the Old velocity, face velocities extrapolated
// from Old and MAC-projected, conv_term(Old), sources at NPH (Old velocity),
// predictor_rhs with fstate Old (CompRHSOps.H:32-141), nodal projection.
void Sim::mol_predictor(bool incremental) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const double dt = t.dt[0];
    update_mueff(vel_old);
    divtau_op(vel_old, divtau);
    if (has_temp && diff_type != 2) tdiff_op(theta_old, tdiff);  // need_divtau(): not for implicit MOL
    mol_extrap(vel_old);
    mac_project();
    if (has_temp) temperature_mol(false, dt);
    mol_conv(vel_old, conv_old);
    compute_sources(vel_old, has_temp ? &theta_nph : nullptr);
    const double fac = diff_type == 0 ? 1.0 : (diff_type == 1 ? 0.5 : 0.0);
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    vel(i, j, k, n) =
                        (rho * vel_old(i, j, k, n) + dt * (conv_old(i, j, k, n) + src(i, j, k, n) + fac * divtau(i, j, k, n))) / rho;
    if (diff_type != 0) diffuse_solve(diff_type == 2 ? dt : 0.5 * dt);
    nodal_project(t.newt, dt, incremental);
}

// ApplyCorrector (src/incflo_advance.cpp:528-652): face velocities from the
// predicted velocity and MAC projection, conv_term(New), mu_eff(New),
// diff_term(New) (the wall-model gradient keeps the Old velocity and takes the
// new mu_eff, ABLWallFunction.cpp:236-300), sources at New, corrector_rhs
// with the explicit factors 1/2, 1/2 (CompRHSOps.H:160-250) and a
// non-incremental nodal projection.
void Sim::mol_corrector() {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const double dt = t.dt[0];
    mol_extrap(vel);
    mac_project();
    Arr th_star;
    if (has_temp) {  // conv_term(New) of the scalar, from the predicted temperature
        th_star = theta;
        Arr q;
        def_cc(q, g, 3, 1);
        fill_scalar(th_star);
        for (size_t m = 0; m < q.d.size(); ++m) q.d[m] = rho * th_star.d[m];
        mol_conv_field(q, -1, tconv);
    }
    mol_conv(vel, conv);
    update_mueff(vel);
    if (has_temp) temperature_mol(true, dt);
    if (diff_type != 0) {  // corrector_rhs with ofac 1/2 (Crank-Nicolson) or 0 (implicit), nfac 0, then the solve
        compute_sources(vel, has_temp ? &theta_nph : nullptr);
        const double ofac = diff_type == 1 ? 0.5 : 0.0;
        for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i)
                        vel(i, j, k, n) = (rho * vel_old(i, j, k, n) +
                                           dt * (0.5 * (conv_old(i, j, k, n) + conv(i, j, k, n)) + ofac * divtau(i, j, k, n) + src(i, j, k, n))) /
                                          rho;
        diffuse_solve(diff_type == 2 ? dt : 0.5 * dt);
        nodal_project(t.newt, dt, false);
        return;
    }
    divtau_op(vel, divtau_new);
    compute_sources(vel, has_temp ? &theta_nph : nullptr);
    for (int n = 0; n < 3; ++n)
#pragma omp parallel for collapse(2)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i)
                    vel(i, j, k, n) = (rho * vel_old(i, j, k, n) +
                                       dt * (0.5 * (conv_old(i, j, k, n) + conv(i, j, k, n)) + 0.5 * divtau(i, j, k, n) +
                                             0.5 * divtau_new(i, j, k, n) + src(i, j, k, n))) /
                                      rho;
    nodal_project(t.newt, dt, false);
}

// ---- implicit / Crank-Nicolson tensor diffusion solve -------------------------------------
// DiffSolverIface::linsys_solve (src/equation_systems/DiffusionOps.cpp:114-159):
// MLTensorOp with alpha 1, a = rho, beta = dtd and the face viscosity of the
// current mu_eff: rho u - dtd divtau(u) = rho u_rhs, u_rhs the current velocity
// (also the initial guess), divtau the operator of divtau_op with its wall-model
// data (Old velocity, current mu_eff).  MLMG stops when the max-norm residual
// is below max(atol, rtol * max(|rhs|, initial residual)) (MLMGOptions
// defaults, prefixes diffusion and velocity_diffusion).  The oracle reaches that point by Jacobi
// iterations, a different solver from the CUDA path's, so that parity
// checks the discrete solution rather than a shared iteration.
void Sim::diffuse_solve(double dtd) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    Arr b, L, R, Dg;
    def_cc(b, g, 0, 3);
    def_cc(L, g, 0, 3);
    def_cc(R, g, 0, 3);
    def_cc(Dg, g, 0, 3);
    Arr m;
    def_cc(m, g, 1, 1);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) m(i, j, k) = mueff(i, j, k);
    fill_cc_foextrap(m);
    const double ih2[3] = {1.0 / (g.dx[0] * g.dx[0]), 1.0 / (g.dx[1] * g.dx[1]), 1.0 / (g.dx[2] * g.dx[2])};
    // diagonal of rho - dtd divtau: the normal-derivative coefficient of the
    // own component is 4/3 along its own direction and 1 across; at a z wall the
    // normal component's face gradient is 2 q0 / dz and the tangential ones' is fixed
    for (int n = 0; n < 3; ++n)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double c0 = m(i, j, k);
                    double s = 0;
                    const double cx = n == 0 ? 4.0 / 3.0 : 1.0, cy = n == 1 ? 4.0 / 3.0 : 1.0, cz = n == 2 ? 4.0 / 3.0 : 1.0;
                    s += cx * (0.5 * (m(i - 1, j, k) + c0) + 0.5 * (m(i + 1, j, k) + c0)) * ih2[0];
                    s += cy * (0.5 * (m(i, j - 1, k) + c0) + 0.5 * (m(i, j + 1, k) + c0)) * ih2[1];
                    const double wall_w = n == 2 ? 2.0 : 0.0;
                    const double zlo = (!g.per[2] && k == 0) ? wall_w * c0 : 0.5 * (m(i, j, k - 1) + c0);
                    const double zhi = (!g.per[2] && k == nz - 1) ? wall_w * c0 : 0.5 * (m(i, j, k + 1) + c0);
                    s += cz * (zlo + zhi) * ih2[2];
                    Dg(i, j, k, n) = rho + dtd * s;
                    b(i, j, k, n) = rho * vel(i, j, k, n);
                }
    auto residual = [&]() {
        divtau_op(vel, L);
        double rn = 0;
        for (int n = 0; n < 3; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const double r = b(i, j, k, n) - rho * vel(i, j, k, n) + dtd * L(i, j, k, n);
                        R(i, j, k, n) = r;
                        rn = std::max(rn, std::fabs(r));
                    }
        if (!std::isfinite(rn)) throw Error(ERR_NONFINITE, "diffusion solve diverged");
        return rn;
    };
    double rn = residual();
    diff_res0 = rn;
    double bnorm = 0;
    for (double v : b.d) bnorm = std::max(bnorm, std::fabs(v));
    // MLMG measures against the larger of |rhs| and the initial residual ("bnorm" / "resid0")
    const double target = std::max(dif.atol, dif.rtol * std::max(bnorm, rn));
    int it = 0;
    while (rn > target) {
        if (++it > 200000) throw Error(ERR_NOT_CONVERGED, "oracle Jacobi iterations of the diffusion solve did not converge");
        for (int n = 0; n < 3; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) vel(i, j, k, n) += R(i, j, k, n) / Dg(i, j, k, n);
        rn = residual();
    }
    diff_iters = it;
    diff_res = rn;
    diff_bnorm = bnorm;
}

// ---- InitData (src/setup/init.cpp:104-225) -------------------------------------------------------
void Sim::init_data() {
    abl_update_umean();  // ABL::post_init_actions
    if (do_initial_proj) {
        nodal_project(t.cur, 1.0, false);
        p.setval(0.0);
        gp.setval(0.0);
    }
    if (initial_iterations > 0) {
        compute_dt();
        vel_old = vel;
        if (has_temp) theta_old = theta;
        for (int it = 0; it < initial_iterations; ++it) {
            if (godunov) apply_predictor(true);
            else mol_predictor(true);  // init.cpp:153-159: ApplyPredictor only, for both schemes
            vel = vel_old;
            if (has_temp) theta = theta_old;
        }
    }
}

int Sim::step_once() {
    if (!t.new_timestep()) return DONE;
    compute_dt();
    t.advance_time();
    abl_update_umean();    // ABL::pre_advance_work
    abl_forcing_update();
    actuator_update();     // Actuator::pre_advance_work
    vel_old = vel;         // prepare_time_step / advance_states
    if (has_temp) theta_old = theta;
    if (godunov) {
        apply_predictor(false);
    } else {  // incflo::advance (src/incflo_advance.cpp:63-79)
        mol_predictor(false);
        mol_corrector();
    }
    return OK;
}

double Sim::ke() const {
    double s = 0;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    for (int n = 0; n < 3; ++n)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) s += 0.5 * rho * vel(i, j, k, n) * vel(i, j, k, n);
    return s / ((double)nx * ny * nz);
}

}  // namespace kso

using kso::Sim;

struct KsoHandle {
    Sim sim;
    std::string err;
};

template <typename F>
static int guard(void* h, F&& f) {
    auto* H = static_cast<KsoHandle*>(h);
    if (!H) return kso::ERR_ARG;
    try {
        return f(H->sim);
    } catch (const kso::Error& e) {
        H->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        H->err = e.what();
        return kso::ERR_DECK;
    }
}

static kso::Arr* field_ptr(Sim& s, const std::string& name, int& nodal_z, int& fdir) {
    nodal_z = 0;
    fdir = -1;
    if (name == "velocity") return &s.vel;
    if (name == "velocity_old") return &s.vel_old;
    if (name == "gp") return &s.gp;
    if (name == "p") { nodal_z = 1; return &s.p; }
    if (name == "src_term") return &s.src;
    if (name == "forces") return &s.forces;
    if (name == "velocity_mueff") return &s.mueff;
    if (name == "diff_term") return &s.divtau;
    if (name == "diff_term_new") return &s.divtau_new;
    if (name == "conv_term") return &s.conv;
    if (name == "conv_term_old") return s.godunov ? nullptr : &s.conv_old;
    if (s.has_temp) {
        if (name == "temperature") return &s.theta;
        if (name == "temperature_old") return &s.theta_old;
        if (name == "temperature_mueff") return &s.alpha;
        if (name == "temperature_conv_term") return &s.tconv;
        if (name == "temperature_diff_term") return &s.tdiff;
    }
    if (name == "actuator_src_term") return &s.act_src;
    if (name == "u_mac") { fdir = 0; return &s.umac; }
    if (name == "v_mac") { fdir = 1; return &s.vmac; }
    if (name == "w_mac") { fdir = 2; return &s.wmac; }
    return nullptr;
}

extern "C" {

int kso_create(const char* deck_text, void** out) {
    if (!deck_text || !out) return kso::ERR_ARG;
    auto* H = new KsoHandle();
    *out = H;
    return guard(H, [&](Sim& s) { s.setup(deck_text); return 0; });
}

void kso_destroy(void* h) { delete static_cast<KsoHandle*>(h); }

const char* kso_last_error(void* h) { return h ? static_cast<KsoHandle*>(h)->err.c_str() : "null handle"; }

int kso_init_data(void* h) { return guard(h, [](Sim& s) { s.init_data(); return 0; }); }

int kso_step(void* h) { return guard(h, [](Sim& s) { return s.step_once(); }); }

int kso_evolve(void* h, int nsteps) {
    return guard(h, [&](Sim& s) {
        for (int m = 0; m < nsteps; ++m)
            if (s.step_once() == kso::DONE) break;
        return 0;
    });
}

int kso_compute_dt(void* h, double* dt) {
    return guard(h, [&](Sim& s) { s.compute_dt(); if (dt) *dt = s.t.dt[0]; return 0; });
}

int kso_pre_advance(void* h) {
    return guard(h, [](Sim& s) {
        s.t.advance_time();
        s.abl_update_umean();
        s.abl_forcing_update();
        s.actuator_update();
        return 0;
    });
}

int kso_prepare_time_step(void* h) {
    return guard(h, [](Sim& s) {
        s.vel_old = s.vel;
        if (s.has_temp) s.theta_old = s.theta;
        return 0;
    });
}

int kso_apply_predictor(void* h, int incremental, int fpi) {
    return guard(h, [&](Sim& s) {
        if (fpi != 0) throw kso::Error(kso::ERR_UNSUPPORTED, "fixed-point iterations");
        if (s.godunov) s.apply_predictor(incremental != 0);
        else s.mol_predictor(incremental != 0);
        return 0;
    });
}

int kso_apply_corrector(void* h) {
    return guard(h, [](Sim& s) {
        if (s.godunov) throw kso::Error(kso::ERR_UNSUPPORTED, "ApplyCorrector belongs to the MOL scheme");
        s.mol_corrector();
        return 0;
    });
}

int kso_apply_projection(void* h, double time, double scaling, int incremental) {
    return guard(h, [&](Sim& s) { s.nodal_project(time, scaling, incremental != 0); return 0; });
}

int kso_update_mueff(void* h) { return guard(h, [](Sim& s) { s.update_mueff(s.vel_old); return 0; }); }

int kso_compute_divtau(void* h, int use_new) {
    return guard(h, [&](Sim& s) {
        if (use_new) s.divtau_op(s.vel, s.divtau_new);
        else s.divtau_op(s.vel_old, s.divtau);
        return 0;
    });
}

int kso_compute_sources(void* h) { return guard(h, [](Sim& s) { s.compute_sources(s.vel_old); return 0; }); }

int kso_predictor_rhs(void* h, double fac) { return guard(h, [&](Sim& s) { s.predictor_rhs(s.t.dt[0], fac); return 0; }); }

int kso_improve_explicit_diffusion(void* h) {
    return guard(h, [](Sim& s) { s.explicit_rk2_post_hoc(s.t.dt[0], s.divtau); return 0; });
}

int kso_field_shape(void* h, const char* name, int* nc, int* nx, int* ny, int* nz) {
    return guard(h, [&](Sim& s) {
        int ndz, fd;
        kso::Arr* a = field_ptr(s, name, ndz, fd);
        if (!a) throw kso::Error(kso::ERR_ARG, std::string("unknown field ") + name);
        *nc = a->nc;
        *nx = s.g.n[0] + (fd == 0 ? 1 : 0);
        *ny = s.g.n[1] + (fd == 1 ? 1 : 0);
        *nz = s.g.n[2] + (fd == 2 ? 1 : 0) + ((ndz && !s.g.per[2]) ? 1 : 0);
        return 0;
    });
}

static int xfer(void* h, const char* name, double* out, const double* in) {
    return guard(h, [&](Sim& s) {
        int ndz, fd;
        kso::Arr* a = field_ptr(s, name, ndz, fd);
        if (!a) throw kso::Error(kso::ERR_ARG, std::string("unknown field ") + name);
        const int nx = s.g.n[0] + (fd == 0 ? 1 : 0), ny = s.g.n[1] + (fd == 1 ? 1 : 0);
        const int nz = s.g.n[2] + (fd == 2 ? 1 : 0) + ((ndz && !s.g.per[2]) ? 1 : 0);
        size_t m = 0;
        for (int n = 0; n < a->nc; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i, ++m) {
                        if (out) out[m] = (*a)(i, j, k, n);
                        else (*a)(i, j, k, n) = in[m];
                    }
        return 0;
    });
}

int kso_get_field(void* h, const char* name, double* out) { return xfer(h, name, out, nullptr); }
int kso_set_field(void* h, const char* name, const double* in) { return xfer(h, name, nullptr, in); }

double kso_get_scalar(void* h, const char* name) {
    auto* H = static_cast<KsoHandle*>(h);
    if (!H) return NAN;
    Sim& s = H->sim;
    std::string n = name;
    if (n == "time") return s.t.cur;
    if (n == "new_time") return s.t.newt;
    if (n == "dt") return s.t.dt[0];
    if (n == "dt_nm1") return s.t.dt[1];
    if (n == "step") return s.t.step;
    if (n == "mac_iters") return s.mac_iters;
    if (n == "mac_levels") return (double)s.mac_dims.size();
    if (n.rfind("mac_level:", 0) == 0) {  // mac_level:l:d, cells of MAC level l in direction d
        const size_t c = n.find(':', 10);
        if (c == std::string::npos) throw kso::Error(kso::ERR_ARG, "scalar " + n);
        return s.mac_dims.at((size_t)std::stoul(n.substr(10, c - 10))).at((size_t)std::stoul(n.substr(c + 1)));
    }
    if (n == "nodal_iters") return s.nodal_iters;
    if (n == "mac_res0") return s.mac_res0;
    if (n == "mac_res") return s.mac_res;
    if (n == "nodal_res0") return s.nodal_res0;
    if (n == "nodal_res") return s.nodal_res;
    if (n == "diff_iters") return s.diff_iters;
    if (n == "diff_res0") return s.diff_res0;
    if (n == "diff_res") return s.diff_res;
    if (n == "diff_rhs_norm") return s.diff_bnorm;
    if (n == "temperature_diff_iters") return s.tdiff_iters;
    if (n == "theta_mean") return s.theta_mean;
    if (n == "abl_forcing_x") return s.ablf_force[0];
    if (n == "abl_forcing_y") return s.ablf_force[1];
    if (n == "utau") return s.utau;
    if (n == "ke") return s.ke();
    if (n == "divu") return s.divu(nullptr);
    if (n == "mac_divu") return s.mac_divu(nullptr);
    if (n == "divu_rel" || n == "mac_divu_rel") {
        double um = 0;
        const double d = n[0] == 'm' ? s.mac_divu(&um) : s.divu(&um);
        const double hmin = std::min(s.g.dx[0], std::min(s.g.dx[1], s.g.dx[2]));
        return um > 0.0 ? d * hmin / um : d;
    }
    if (n == "cfl") return s.t.cur_cfl;
    if (n == "conv_cfl") return s.t.conv_cfl;
    if (n == "diff_cfl") return s.t.diff_cfl;
    if (n == "src_cfl") return s.t.src_cfl;
    if (n == "density") return s.rho;
    if (n.rfind("disk_ct:", 0) == 0) return s.disks.at(std::stoi(n.substr(8))).current_ct;
    if (n.rfind("disk_uinf2:", 0) == 0) return s.disks.at(std::stoi(n.substr(11))).uinf_sqr;
    if (n.rfind("disk_normal:", 0) == 0 || n.rfind("disk_sample:", 0) == 0) {
        const size_t c = n.find(':', 12);
        const auto& dp = s.disks.at(std::stoi(n.substr(12, c - 12)));
        const int m = std::stoi(n.substr(c + 1));
        return n[5] == 'n' ? dp.normal[m] : dp.sample[m];
    }
    // "disk_point:k:p:m" / "disk_weight:k:p": sampling point p of disk k and its area weight
    if (n.rfind("disk_point:", 0) == 0 || n.rfind("disk_weight:", 0) == 0) {
        const bool pt = n[5] == 'p';
        const size_t a = pt ? 11 : 12, b = n.find(':', a);
        const auto& dp = s.disks.at(std::stoi(n.substr(a, b - a)));
        std::vector<double> xs, ws;
        sample_points(dp, xs, ws);
        if (!pt) return ws.at(std::stoi(n.substr(b + 1)));
        const size_t c = n.find(':', b + 1);
        return xs.at(3 * std::stoul(n.substr(b + 1, c - b - 1)) + std::stoi(n.substr(c + 1)));
    }
    return NAN;
}

int kso_set_scalar(void* h, const char* name, double v) {
    return guard(h, [&](Sim& s) {
        std::string n = name;
        if (n == "dt") s.t.dt[0] = v;
        else if (n == "dt_nm1") s.t.dt[1] = v;
        else if (n == "time") s.t.cur = v;
        else if (n == "new_time") s.t.newt = v;
        else if (n == "utau") s.utau = v;
        else if (n == "nodal_omega") s.nod.omega = v;
        else throw kso::Error(kso::ERR_ARG, "unknown scalar " + n);
        return 0;
    });
}

}  // extern "C"
