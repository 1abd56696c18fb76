// Host driver of the GB300-native advance and its C ABI (include/ks.h).
//
// Owns the deck, SimTime, the device fields of one single-box grid and one
// CUDA stream; sequences the device passes in the order of the reference's
// incflo::advance (src/incflo_advance.cpp:63-438) and ApplyProjection
// (src/projection/incflo_apply_nodal_projection.cpp:149-465).  Every device
// pass is a hand-written kernel in ks_kernels.cu, ks_godunov.cu or ks_mg.cu;
// the host only computes scalars (dt, u_tau, disk forces) and launches.
#include <cuda_runtime.h>
#include "ks_sim.hpp"

namespace ks {

Sim::Sim(const std::string& text) {
    Deck D(text);
    deck_text_ = text;
    setup(D);
    ck(cudaStreamCreateWithFlags(&ctx_.stream, cudaStreamNonBlocking), "stream create");
    ck(cudaMallocHost(&hred_, 64 * sizeof(double)), "pinned alloc");
    alloc();
    init_fields(D);
    const std::string prec = lc(D.str("ks.precision", "fp64"));
    if (prec == "mixed") set_mixed(1);
    else if (prec != "fp64") throw KsError(KS_ERR_DECK, "ks.precision must be fp64 or mixed");
    sync();
}

Sim::~Sim() {
    if (ctx_.stream) cudaStreamSynchronize(ctx_.stream);
    for (MGGraph* G : {&gcc_[0], &gcc_[1], &gnd_[0], &gnd_[1]})
        if (G->exec) cudaGraphExecDestroy(G->exec);
    if (hred_) cudaFreeHost(hred_);
    if (ctx_.stream) cudaStreamDestroy(ctx_.stream);
}

void Sim::setup(const Deck& D) {
    std::vector<double> nc, lo, hi, per;
    nc = D.nums("amr.n_cell");
    lo = D.nums("geometry.prob_lo");
    hi = D.nums("geometry.prob_hi");
    per = D.nums("geometry.is_periodic");
    if (nc.size() < 3 || lo.size() < 3 || hi.size() < 3 || per.size() < 3) throw KsError(KS_ERR_DECK, "geometry needs 3 values");
    if (D.flag("amr.max_level", 0) != 0) throw KsError(KS_ERR_UNSUPPORTED, "single level only (amr.max_level = 0)");
    for (int d = 0; d < 3; ++d) {
        plo_[d] = lo[d];
        phi_[d] = hi[d];
    }
    g_.nx = (int)nc[0];
    g_.ny = (int)nc[1];
    g_.nz = (int)nc[2];
    g_.dx = (hi[0] - lo[0]) / g_.nx;
    g_.dy = (hi[1] - lo[1]) / g_.ny;
    g_.dz = (hi[2] - lo[2]) / g_.nz;
    if (per[0] == 0 || per[1] == 0) throw KsError(KS_ERR_UNSUPPORTED, "x and y must be periodic");
    g_.zper = per[2] != 0;
    g_.zlo = g_.zhi = ZPER;
    if (!g_.zper) {
        auto bc = [&](const char* key) {
            const std::string s = lc(D.str(key, ""));
            if (s == "slip_wall") return (int)ZSLIP;
            if (s == "wall_model") return (int)ZWALLMODEL;
            throw KsError(KS_ERR_UNSUPPORTED, std::string(key) + " = " + s + " is outside this path");
        };
        g_.zlo = bc("zlo.type");
        g_.zhi = bc("zhi.type");
        if (g_.zhi == ZWALLMODEL) throw KsError(KS_ERR_DECK, "ABL wall models are not applicable to a zhi BC");
        if (g_.nz < 4) throw KsError(KS_ERR_UNSUPPORTED, "wall-bounded z needs at least 4 cells");
    }
    if (g_.nx % 2 || g_.ny % 2 || g_.nz % 2 || g_.nx < 4 || g_.ny < 4 || g_.nz < 4)
        throw KsError(KS_ERR_UNSUPPORTED, "cell counts must be even and at least 4");
    g_.idx = 1.0 / g_.dx;
    g_.idy = 1.0 / g_.dy;
    g_.idz = 1.0 / g_.dz;
    g_.N = (long long)g_.nx * g_.ny * g_.nz;
    g_.NFz = (long long)g_.nx * g_.ny * (g_.nz + 1);
    wallmodel_ = (g_.zlo == ZWALLMODEL);

    rho_ = D.num("incflo.density", 1.0);
    mu_ = D.num("transport.viscosity", 0.0);
    godunov_ = D.flag("incflo.use_godunov", 1) != 0;
    if (godunov_) {
        if (lc(D.str("incflo.godunov_type", "weno_z")) != "ppm") throw KsError(KS_ERR_UNSUPPORTED, "incflo.godunov_type must be ppm");
        if (D.flag("incflo.godunov_use_forces_in_trans", 0) != 0) throw KsError(KS_ERR_UNSUPPORTED, "godunov_use_forces_in_trans");
    }
    // src/setup/init.cpp:60-76 (the default is Crank-Nicolson)
    diff_type_ = D.flag("incflo.diffusion_type", 1);
    if (diff_type_ < 0 || diff_type_ > 2)
        throw KsError(KS_ERR_DECK, "We currently require diffusion_type = 0 for explicit, 1 for Crank-Nicolson or 2 for implicit");
    if (D.flag("incflo.icns_conserv", 1) != 1) throw KsError(KS_ERR_UNSUPPORTED, "non-conservative momentum form");
    initial_proj_ = D.flag("incflo.do_initial_proj", 1);
    initial_iters_ = D.flag("incflo.initial_iterations", 3);
    const std::string tm = lc(D.str("turbulence.model", "laminar"));
    if (tm != "laminar" && tm != "smagorinsky") throw KsError(KS_ERR_UNSUPPORTED, "turbulence.model = " + tm);
    S_.rho = rho_;
    S_.irho = 1.0 / rho_;
    S_.mu = mu_;
    S_.smag = tm == "smagorinsky";
    const double Cs = D.num("Smagorinsky_coeffs.Cs", 0.135);
    const double ds = std::cbrt(g_.dx * g_.dy * g_.dz);
    S_.smag_fac = Cs * Cs * ds * ds;

    for (auto& s : D.strs("ICNS.source_terms")) {
        if (s == "GeostrophicForcing") S_.geo = 1;
        else if (s == "CoriolisForcing") S_.cor = 1;
        else if (s == "BodyForce") S_.body = 1;
        else if (s == "ActuatorForcing") S_.act = 1;
        else if (s == "BoussinesqBuoyancy") S_.bous = 1;
        else if (s == "ABLForcing") S_.ablf = 1;
        else throw KsError(KS_ERR_UNSUPPORTED, "momentum source " + s);
    }
    const double pi = 3.14159265358979323846;
    const double period = D.num("CoriolisForcing.rotational_time_period", 86164.091);
    const double lat = (S_.geo || S_.cor) ? D.nums("CoriolisForcing.latitude").at(0) * pi / 180.0 : 0.5 * pi;
    const double omega = 2 * pi / period;
    S_.sinphi = std::sin(lat);
    S_.cosphi = std::cos(lat);
    S_.corfac = 2 * omega;
    S_.hfac = D.flag("CoriolisForcing.is_horizontal", 0) ? 0.0 : 1.0;
    double e[3] = {1, 0, 0}, n[3] = {0, 1, 0};
    if (D.has("CoriolisForcing.east_vector")) { auto v = D.nums("CoriolisForcing.east_vector"); for (int d = 0; d < 3; ++d) e[d] = v.at(d); }
    if (D.has("CoriolisForcing.north_vector")) { auto v = D.nums("CoriolisForcing.north_vector"); for (int d = 0; d < 3; ++d) n[d] = v.at(d); }
    auto unit = [](double* v) { const double m = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); for (int d = 0; d < 3; ++d) v[d] /= m; };
    unit(e);
    unit(n);
    for (int d = 0; d < 3; ++d) { S_.east[d] = e[d]; S_.north[d] = n[d]; }
    S_.up[0] = e[1] * n[2] - e[2] * n[1];
    S_.up[1] = e[2] * n[0] - e[0] * n[2];
    S_.up[2] = e[0] * n[1] - e[1] * n[0];
    if (S_.geo) {
        auto w = D.nums("GeostrophicForcing.geostrophic_wind");
        const double cf = 2 * omega * S_.sinphi;
        S_.gf[0] = -cf * w.at(1);
        S_.gf[1] = cf * w.at(0);
        S_.gf[2] = 0.0;
    }
    if (S_.body) {
        // BodyForce::BodyForce (BodyForce.cpp:20-58): uniform_constant (default) or
        // oscillatory with angular_frequency; the file-driven types are not built
        const std::string bt = lc(D.str("BodyForce.type", "uniform_constant"));
        if (bt == "height_varying" || bt == "height-varying" || bt == "uniform_timetable" || D.has("BodyForce.uniform_timetable_file"))
            throw KsError(KS_ERR_UNSUPPORTED, "BodyForce.type " + bt + " (file-driven forcing)");
        if (bt != "uniform_constant" && bt != "oscillatory") throw KsError(KS_ERR_DECK, "BodyForce.type " + bt);
        auto m = D.nums("BodyForce.magnitude");
        for (int d = 0; d < 3; ++d) S_.body_force[d] = m.at(d);
        S_.body_osc = bt == "oscillatory";
        if (S_.body_osc) S_.body_omega = D.nums("BodyForce.angular_frequency").at(0);
    }
    kappa_ = D.num("ABL.kappa", 0.41);
    z0_ = D.num("ABL.surface_roughness_z0", 0.1);
    const std::string st = lc(D.str("ABL.wall_shear_stress_type", "moeng"));
    if (st == "moeng") shear_ = 0;
    else if (st == "constant") shear_ = 1;
    else if (st == "local") shear_ = 2;
    else if (st == "schumann") shear_ = 3;
    else throw KsError(KS_ERR_UNSUPPORTED, "ABL.wall_shear_stress_type = " + st);
    zref_ = D.has("ABL.log_law_height") ? D.num("ABL.log_law_height", 0) : 0.5 * g_.dz;
    if (wallmodel_ && std::fabs(zref_ - 0.5 * g_.dz) > 1e-12 * g_.dz)
        throw KsError(KS_ERR_UNSUPPORTED, "ABL.log_law_height other than the first cell centre");

    // Temperature transport: the ABL physics registers the Temperature PDE
    // (src/wind_energy/ABL.cpp:27-28); it is advanced when the deck gives the
    // initial profile (ABL.temperature_heights, required by ABLFieldInit.cpp:96-99).
    const std::string phys = D.str("incflo.physics", "");
    temp_ = phys == "ABL" && D.has("ABL.temperature_heights");
    S_.temp = temp_ ? 1 : 0;
    S_.grav[0] = 0.0; S_.grav[1] = 0.0; S_.grav[2] = -9.81;
    if (D.has("incflo.gravity")) { auto gv = D.nums("incflo.gravity"); for (int d = 0; d < 3; ++d) S_.grav[d] = gv.at(d); }
    const double Pr = D.num("transport.laminar_prandtl", 1.0), Prt = D.num("transport.turbulent_prandtl", 1.0);  // ConstTransport.H:20-95
    S_.mu_pr = mu_ / Pr;
    S_.iprt = 1.0 / Prt;
    S_.T_ref = D.num("transport.reference_temperature", -1.0);
    if (S_.bous) {  // BoussinesqBuoyancy.cpp:10-17, ConstTransport.H:32-95,184-200
        if (!temp_) throw KsError(KS_ERR_DECK, "BoussinesqBuoyancy needs the temperature field (ABL.temperature_heights)");
        if (S_.T_ref < 0.0) throw KsError(KS_ERR_DECK, "Reference temperature was not set");
        S_.beta_T = D.has("transport.thermal_expansion_coefficient") ? D.num("transport.thermal_expansion_coefficient", 0.0) : 1.0 / S_.T_ref;
    }
    if (S_.ablf) {  // ABLForcing.cpp:13-60
        if (phys != "ABL") throw KsError(KS_ERR_DECK, "ABLForcing needs the ABL physics");
        if (D.has("ABLForcing.velocity_timetable")) throw KsError(KS_ERR_UNSUPPORTED, "ABLForcing.velocity_timetable");
        ablf_h_ = D.nums("ABLForcing.abl_forcing_height").at(0);
        auto tv = D.nums("incflo.velocity");
        ablf_target_[0] = tv.at(0);
        ablf_target_[1] = tv.at(1);
    }
    if (temp_) {
        if (D.has("ABL.surface_temp_rate") || D.has("ABL.surface_temp_timetable") || std::fabs(D.num("ABL.surface_temp_flux", 0.0)) > 0.0)
            throw KsError(KS_ERR_UNSUPPORTED, "non-neutral surface temperature forcing (only ABL.surface_temp_flux = 0)");
        if (D.flag("ABL.perturb_temperature", 0)) throw KsError(KS_ERR_UNSUPPORTED, "ABL.perturb_temperature (random perturbations)");
        z0t_ = D.num("ABL.surface_roughness_z0t", z0_);
        // temperature BCs (BCInterface.cpp:289-350, incflo_diffusion.cpp:71-104);
        // <face>.temperature_type overrides the face's velocity BC type
        auto tbc = [&](const char* face, int zbc) {
            const std::string key = std::string(face) + ".temperature_type";
            const std::string t = lc(D.str(key, zbc == ZWALLMODEL ? "wall_model" : "slip_wall"));
            if (t == "wall_model") return 1;
            if (t == "fixed_gradient") return 2;
            if (t == "slip_wall" || t == "zero_gradient" || t == "symmetric_wall") return 0;
            throw KsError(KS_ERR_UNSUPPORTED, key + " = " + t);
        };
        if (!g_.zper) {
            tzlo_ = tbc("zlo", g_.zlo);
            tzhi_ = tbc("zhi", g_.zhi);
            if (tzhi_ == 1) throw KsError(KS_ERR_DECK, "ABL wall models are not applicable to a zhi BC");
            if (tzlo_ == 1 && g_.zlo != ZWALLMODEL) throw KsError(KS_ERR_UNSUPPORTED, "temperature wall model without the velocity wall model");
            if (tzlo_ == 2) throw KsError(KS_ERR_UNSUPPORTED, "zlo fixed_gradient temperature");
            if (tzhi_ == 2) tgtop_ = D.nums("zhi.temperature").at(0);
        }
    }

    auto mg = [&](MGParams& m, const std::string& p) {
        m.rtol = D.num(p + ".mg_rtol", m.rtol);
        m.atol = D.num(p + ".mg_atol", m.atol);
        m.maxiter = D.flag(p + ".maxiter", m.maxiter);
        m.nu1 = D.flag(p + ".num_pre_smooth", m.nu1);
        m.nu2 = D.flag(p + ".num_post_smooth", m.nu2);
        m.fixed_iters = D.flag(p + ".do_fixed_iters", m.fixed_iters);
        m.semi = D.flag(p + ".do_semicoarsening", m.semi);
        m.max_semi = D.flag(p + ".max_semicoarsening_level", m.max_semi);
    };
    mg(mac_, "mac_proj");
    mg(nod_, "nodal_proj");
    mg(dif_, "diffusion");  // MLMGOptions(default prefix, custom prefix), src/core/MLMGOptions.cpp:8-13
    mg(dif_, "velocity_diffusion");
    mg(tdif_, "diffusion");
    mg(tdif_, "temperature_diffusion");
    // I/O (IOManager::initialize_io, SimTime::parse_parameters)
    // Warm start of the Poisson solves (not a reference key): the nodal projection starts
    // from the current pressure, the MAC projection from the previous MAC potential.  The
    // stopping test stays MLMG's: max-norm residual <= max(atol, rtol * max(|rhs|, initial
    // residual)), so a solve ends at the same tolerance as one from zero, in fewer V-cycles.
    mg_warm_ = D.flag("ks.mg_warm_start", 1);
    mg_graphs_ = D.flag("ks.mg_graphs", 1);  // coarse V-cycle levels as CUDA graphs (not a reference key)
    // mixed precision: FP32 V-cycles per FP64 defect-correction residual (not a reference key)
    mg_inner_ = D.flag("ks.mixed_inner_cycles", 2);
    mg_inner_nd_ = D.flag("ks.mixed_inner_cycles_nodal", 4);
    if (mg_inner_ < 1 || mg_inner_nd_ < 1) throw KsError(KS_ERR_DECK, "ks.mixed_inner_cycles(_nodal) must be >= 1");
    restart_file_ = D.str("io.restart_file", "");
    plt_prefix_ = D.str("io.plot_file", "plt");
    chk_prefix_ = D.str("io.check_file", "chk");
    plot_interval_ = D.flag("time.plot_interval", -1);
    chk_interval_ = D.flag("time.checkpoint_interval", -1);

    t_.stop = D.num("time.stop_time", -1);
    t_.max_step = D.flag("time.max_step", -1);
    t_.fixed_dt = D.num("time.fixed_dt", -1);
    t_.init_dt = D.num("time.initial_dt", -1);
    t_.max_dt = D.num("time.max_dt", -1);
    t_.min_dt = D.num("time.min_dt", -1);
    t_.shrink = D.num("time.init_shrink", 0.1);
    t_.growth = D.num("time.max_dt_growth", 0.1);
    t_.cfl = D.num("time.cfl", 1.0);
    t_.force_cfl = D.flag("time.use_force_cfl", 1) != 0;
    if (t_.fixed_dt > 0) t_.dt[0] = t_.fixed_dt;
    else t_.adaptive = true;
    // src/setup/init.cpp:78-88
    if (!godunov_ && t_.cfl > 0.5) throw KsError(KS_ERR_DECK, "We currently require cfl <= 0.5 when using the MOL advection scheme");
    if (godunov_ && t_.cfl > 1.0) throw KsError(KS_ERR_DECK, "We currently require cfl <= 1.0 when using the Godunov advection scheme");

    // Actuator disks (src/wind_energy/actuator/disk/disk_ops.cpp:182-276,
    // uniform_ct_ops.cpp:53-88)
    if (S_.act) {
        // Disk orientation (disk_ops.cpp:125-147, 182-264): the reference vectors
        // come from the "Coriolis" / "Coriolis.Forcing" parameters (defaults
        // north = y, east = x); tilt turns the normal by -tilt degrees about east,
        // then yaw by -yaw degrees about z (clockwise seen from above).
        auto orient = [&](const std::string& k, const double* def, double* out) {
            const std::string a = "Coriolis." + k, b = "Coriolis.Forcing." + k;
            const std::string key = D.has(a) ? a : (D.has(b) ? b : std::string());
            for (int m = 0; m < 3; ++m) out[m] = key.empty() ? def[m] : D.nums(key).at(m);
        };
        const double jhat[3] = {0.0, 1.0, 0.0}, ihat[3] = {1.0, 0.0, 0.0}, khat[3] = {0.0, 0.0, 1.0};
        double dnorth[3], deast[3];
        orient("north_vector", jhat, dnorth);
        orient("east_vector", ihat, deast);
        auto turn = [](const double* axis, double deg, double* v) {  // v rotated by deg about axis (right-handed)
            const double am = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
            const double a[3] = {axis[0] / am, axis[1] / am, axis[2] / am};
            const double th = deg * 3.14159265358979323846 / 180.0, c = std::cos(th), sn = std::sin(th);
            const double dd = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
            const double x[3] = {a[1] * v[2] - a[2] * v[1], a[2] * v[0] - a[0] * v[2], a[0] * v[1] - a[1] * v[0]};
            double o[3];
            for (int m = 0; m < 3; ++m) o[m] = v[m] * c + x[m] * sn + a[m] * dd * (1.0 - c);
            for (int m = 0; m < 3; ++m) v[m] = o[m];
        };
        for (auto& lab : D.strs("Actuator.labels")) {
            const std::string type = D.str("Actuator." + lab + ".type", D.str("Actuator.type", ""));
            if (type != "UniformCtDisk") throw KsError(KS_ERR_UNSUPPORTED, "actuator type " + type);
            auto key = [&](const std::string& k) {
                const std::string a = "Actuator." + lab + "." + k;
                return D.has(a) ? a : "Actuator." + type + "." + k;
            };
            Disk d{};
            d.D = D.num(key("rotor_diameter"), 0);
            d.eps = D.num(key("epsilon"), 0);
            if (d.D <= 0 || d.eps <= 0) throw KsError(KS_ERR_DECK, "actuator rotor_diameter and epsilon are required");
            d.ct = D.nums(key("thrust_coeff"));
            if (D.has(key("wind_speed"))) d.ws = D.nums(key("wind_speed"));
            if (d.ct.size() == 1) d.ws = {1.0};
            if (d.ws.size() != d.ct.size()) throw KsError(KS_ERR_DECK, "wind_speed and thrust_coeff must have the same number of values");
            d.nr = D.flag(key("num_points_r"), 1);
            d.nt = D.flag(key("num_points_t"), 1);
            if (d.nr < 1 || d.nt < 1) throw KsError(KS_ERR_DECK, "num_points_r and num_points_t must both be >=1");
            if (lc(D.str(key("spreading_type"), "LinearBasis")) != "uniformgaussian")
                throw KsError(KS_ERR_UNSUPPORTED, "only spreading_type = UniformGaussian");
            // check_for_parse_conflicts (disk_ops.cpp:278-300)
            auto conflict = [&](const char* a, const char* b) {
                if (D.has(key(a)) && D.has(key(b)))
                    throw KsError(KS_ERR_DECK, std::string("ActuatorDisk Conflict: ") + a + " and " + b);
            };
            conflict("disk_normal", "yaw");
            conflict("disk_normal", "tilt");
            conflict("sample_normal", "sample_yaw");
            conflict("sample_normal", "sample_tilt");
            conflict("disk_center", "base_position");
            conflict("disk_center", "hub_height");
            if (D.has(key("base_position")) != D.has(key("hub_height")))
                throw KsError(KS_ERR_DECK, "ActuatorDisk Dependency Missing: base_position and hub_height go together");
            for (int m = 0; m < 3; ++m) { d.center[m] = 0; d.normal[m] = dnorth[m]; d.sample[m] = dnorth[m]; }
            if (D.has(key("disk_center"))) {
                auto c = D.nums(key("disk_center"));
                for (int m = 0; m < 3; ++m) d.center[m] = c.at(m);
            } else if (D.has(key("base_position"))) {
                auto b = D.nums(key("base_position"));
                for (int m = 0; m < 3; ++m) d.center[m] = b.at(m);
                d.center[2] += D.nums(key("hub_height")).at(0);
            }
            if (D.has(key("disk_normal"))) {
                auto v = D.nums(key("disk_normal"));
                for (int m = 0; m < 3; ++m) d.normal[m] = v.at(m);
            }
            if (D.has(key("tilt"))) turn(deast, -D.nums(key("tilt")).at(0), d.normal);
            if (D.has(key("yaw"))) turn(khat, -D.nums(key("yaw")).at(0), d.normal);
            const bool own_sample = D.has(key("sample_normal")) || D.has(key("sample_yaw")) || D.has(key("sample_tilt"));
            if (D.has(key("sample_normal"))) {
                auto v = D.nums(key("sample_normal"));
                for (int m = 0; m < 3; ++m) d.sample[m] = v.at(m);
            }
            if (D.has(key("sample_tilt"))) turn(deast, -D.nums(key("sample_tilt")).at(0), d.sample);
            if (D.has(key("sample_yaw"))) turn(khat, -D.nums(key("sample_yaw")).at(0), d.sample);
            if (!own_sample)
                for (int m = 0; m < 3; ++m) d.sample[m] = d.normal[m];
            unit(d.normal);
            unit(d.sample);
            if (d.normal[0] * d.normal[0] + d.normal[1] * d.normal[1] <= 2.220446049250313e-16)  // |k x n|^2 <= eps (disk_ops.cpp:335-337)
                throw KsError(KS_ERR_DECK, "A constant Ct disk normal is too close to vertical.");
            d.cvec[0] = -d.normal[1];
            d.cvec[1] = d.normal[0];
            d.cvec[2] = 0.0;
            unit(d.cvec);
            d.to_sample = D.num(key("diameters_to_sample"), 0.0);
            d.about_center = D.flag(key("ks_spread_about_center"), 0) != 0;
            d.dr = 0.5 * d.D / d.nr;
            d.ct_now = d.ct[0];
            disks_.push_back(d);
        }
    }
}

// Weighted-Jacobi weight of the nodal smoother.  The largest eigenvalue of
// D^-1 A for the Q1 stencil lies at a corner of the frequency cube; it is 1.5
// on isotropic cells (omega 0.9 gives omega * lambda_max = 1.35) and grows with
// the cell aspect ratio (3.0 at dz = dx / 2, where omega = 0.9 diverges).  The
// weight is reduced so that omega * lambda_max stays at 1.35.  All levels have
// the same aspect ratio, so the finest level's stencil decides.
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

// Inverse of the singular operator A (n x n, row-major, null space the
// constants) restricted to the unknowns 1..n-1: the returned n x n matrix maps
// a compatible right-hand side to the solution with x[0] = 0 (row and column 0
// are zero).  Gauss-Jordan with partial pivoting; false when a pivot is below
// 1e-12 of the largest entry (no direct bottom solve).
constexpr int kDirectBottom = 512;

static bool pinned_inverse(const std::vector<double>& A, int n, std::vector<double>& inv) {
    const int m = n - 1;
    if (m < 1) return false;
    std::vector<double> a((size_t)m * 2 * m, 0.0);
    double amax = 0.0;
    for (int r = 0; r < m; ++r)
        for (int c = 0; c < m; ++c) {
            a[(size_t)r * 2 * m + c] = A[(size_t)(r + 1) * n + (c + 1)];
            amax = std::max(amax, std::fabs(A[(size_t)(r + 1) * n + (c + 1)]));
        }
    for (int r = 0; r < m; ++r) a[(size_t)r * 2 * m + m + r] = 1.0;
    for (int c = 0; c < m; ++c) {
        int piv = c;
        for (int r = c + 1; r < m; ++r)
            if (std::fabs(a[(size_t)r * 2 * m + c]) > std::fabs(a[(size_t)piv * 2 * m + c])) piv = r;
        if (!(std::fabs(a[(size_t)piv * 2 * m + c]) > 1e-12 * amax)) return false;
        if (piv != c)
            for (int q = 0; q < 2 * m; ++q) std::swap(a[(size_t)c * 2 * m + q], a[(size_t)piv * 2 * m + q]);
        const double d = 1.0 / a[(size_t)c * 2 * m + c];
        for (int q = 0; q < 2 * m; ++q) a[(size_t)c * 2 * m + q] *= d;
        for (int r = 0; r < m; ++r) {
            if (r == c) continue;
            const double f = a[(size_t)r * 2 * m + c];
            if (f == 0.0) continue;
            for (int q = 0; q < 2 * m; ++q) a[(size_t)r * 2 * m + q] -= f * a[(size_t)c * 2 * m + q];
        }
    }
    inv.assign((size_t)n * n, 0.0);
    for (int r = 0; r < m; ++r)
        for (int c = 0; c < m; ++c) inv[(size_t)(r + 1) * n + (c + 1)] = a[(size_t)r * 2 * m + m + c];
    return true;
}

// The coarsest MAC operator d p - sum w p of level C, assembled and inverted
// with one unknown pinned (pinned_inverse); inv is left empty if that fails.
static void cc_direct_inverse(const CCLevelDev& C, std::vector<double>& inv) {
    const int nc = C.nx * C.ny * C.nz;
    std::vector<double> A((size_t)nc * nc, 0.0);
    const double d0 = 2.0 * C.ix2 + 2.0 * C.iy2;
    auto at = [&](int ii, int jj, int kk) { return (kk * C.ny + jj) * C.nx + ii; };
    for (int k = 0; k < C.nz; ++k)
        for (int j = 0; j < C.ny; ++j)
            for (int i = 0; i < C.nx; ++i) {
                const int r = at(i, j, k);
                const int ip = (i + 1) % C.nx, im = (i + C.nx - 1) % C.nx, jp = (j + 1) % C.ny, jm = (j + C.ny - 1) % C.ny;
                double d = d0;
                A[(size_t)r * nc + at(ip, j, k)] -= C.ix2;
                A[(size_t)r * nc + at(im, j, k)] -= C.ix2;
                A[(size_t)r * nc + at(i, jp, k)] -= C.iy2;
                A[(size_t)r * nc + at(i, jm, k)] -= C.iy2;
                if (C.zper) {
                    d += 2.0 * C.iz2;
                    A[(size_t)r * nc + at(i, j, (k + 1) % C.nz)] -= C.iz2;
                    A[(size_t)r * nc + at(i, j, (k + C.nz - 1) % C.nz)] -= C.iz2;
                } else {
                    if (k > 0) { d += C.iz2; A[(size_t)r * nc + at(i, j, k - 1)] -= C.iz2; }
                    if (k < C.nz - 1) { d += C.iz2; A[(size_t)r * nc + at(i, j, k + 1)] -= C.iz2; }
                }
                A[(size_t)r * nc + r] += d;
            }
    if (!pinned_inverse(A, nc, inv)) inv.clear();
}

// Bottom levels of up to kDirectBottom points are solved exactly: the coarsest MAC
// operator d p - sum w p (scaled by -beta in the solve) and the coarsest nodal
// stencil (scaled by sigma) are assembled on the host, their pinned inverses
// uploaded once.  A bottom solve is then one small matrix-vector product in
// place of relaxation sweeps, whose FP64 dependency chains on one SM cost
// about 0.1 ms per solve on this GPU.
void Sim::bottom_setup() {
    constexpr int kMaxDirect = kDirectBottom;
    binv_cc_h_.clear();
    binv_nd_h_.clear();
    CCLevelDev& C = cc_.back();
    NDLevelDev& D = nd_.back();
    const int nc = C.nx * C.ny * C.nz, nn = D.nx * D.ny * D.nz;
    if (nc <= kMaxDirect && cc_.size() > 1) cc_direct_inverse(C, binv_cc_h_);
    if (nn <= kMaxDirect && nd_.size() > 1) {
        std::vector<double> A((size_t)nn * nn, 0.0);
        for (int k = 0; k < D.nz; ++k)
            for (int j = 0; j < D.ny; ++j)
                for (int i = 0; i < D.nx; ++i) {
                    const int r = (k * D.ny + j) * D.nx + i;
                    for (int c = 0; c < 3; ++c)
                        for (int b = 0; b < 3; ++b)
                            for (int a = 0; a < 3; ++a) {
                                const int w = (c * 3 + b) * 3 + a;
                                if (D.faces_zero && (w == 4 || w == 10 || w == 12 || w == 14 || w == 16 || w == 22)) continue;
                                const int ii = (i + a - 1 + D.nx) % D.nx, jj = (j + b - 1 + D.ny) % D.ny;
                                int kk = k + c - 1;
                                if (D.zper) kk = (kk + D.nz) % D.nz;
                                else kk = kk < 0 ? -kk : (kk >= D.nz ? 2 * (D.nz - 1) - kk : kk);
                                A[(size_t)r * nn + (kk * D.ny + jj) * D.nx + ii] += D.W[w];
                            }
                }
        if (!pinned_inverse(A, nn, binv_nd_h_)) binv_nd_h_.clear();
    }
    binv_.alloc(std::max<size_t>(1, binv_cc_h_.size() + binv_nd_h_.size()));
    if (!binv_cc_h_.empty())
        ck(cudaMemcpy(binv_.p, binv_cc_h_.data(), binv_cc_h_.size() * sizeof(double), cudaMemcpyHostToDevice), "H2D bottom inverse");
    if (!binv_nd_h_.empty())
        ck(cudaMemcpy(binv_.p + binv_cc_h_.size(), binv_nd_h_.data(), binv_nd_h_.size() * sizeof(double), cudaMemcpyHostToDevice),
           "H2D bottom inverse");
    C.binv = binv_cc_h_.empty() ? nullptr : binv_.p;
    D.binv = binv_nd_h_.empty() ? nullptr : binv_.p + binv_cc_h_.size();
}

// Coarsening ratio (1 or 2 per direction) from a level of n cells of spacing
// h to the next.  Full coarsening needs every count divisible by 4 (the
// coarse count stays even for the red-black sweeps).  Semicoarsening
// (MLMGOptions do_semicoarsening, src/core/MLMGOptions.cpp:24-28) halves only
// the directions of smallest spacing while the spacings differ, each of them
// divisible by 4; otherwise the level coarsens fully or not at all.  The
// oracle's semi_ratio is the same rule.
static void mg_ratio(const int n[3], const double h[3], bool semi, int r[3]) {
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

// The MAC hierarchy under mac_proj.do_semicoarsening: levels coarsened by
// mg_ratio until one cannot coarsen or a level below the finest holds at most
// kDirectBottom cells (solved exactly, as in cc_).  When every coarsening is
// full the hierarchy equals cc_ and nothing is built.
void Sim::mac_semi_setup() {
    std::vector<std::array<int, 3>> dims;
    int n3[3] = {g_.nx, g_.ny, g_.nz};
    double h[3] = {g_.dx, g_.dy, g_.dz};
    bool partial = false;
    while (true) {
        dims.push_back({n3[0], n3[1], n3[2]});
        int r[3];
        mg_ratio(n3, h, (long long)dims.size() - 1 < (long long)mac_.max_semi, r);
        if (r[0] * r[1] * r[2] == 1) break;
        if (dims.size() > 1 && (long long)n3[0] * n3[1] * n3[2] <= kDirectBottom) break;
        for (int d = 0; d < 3; ++d) {
            if (r[d] != 1 && r[d] != 2) throw KsError(KS_ERR_UNSUPPORTED, "MAC semicoarsening ratio");
            n3[d] /= r[d];
            h[d] *= r[d];
        }
        if (r[0] * r[1] * r[2] != 8) partial = true;
    }
    if (!partial) return;
    size_t tot = 0;
    for (size_t l = 1; l < dims.size(); ++l) tot += 3 * (size_t)dims[l][0] * dims[l][1] * dims[l][2];
    mgbufs_.alloc(tot);
    double* q = mgbufs_.p;
    ccs_.clear();
    ccs_.push_back(cc_[0]);
    ccs_[0].binv = nullptr;
    double hl[3] = {g_.dx, g_.dy, g_.dz};
    for (size_t l = 1; l < dims.size(); ++l) {
        const CCLevelDev& F = ccs_.back();
        CCLevelDev C{};
        C.nx = dims[l][0]; C.ny = dims[l][1]; C.nz = dims[l][2]; C.zper = g_.zper;
        // the restriction and prolongation kernels index F = r C, r in {1, 2}
        const int fn[3] = {F.nx, F.ny, F.nz}, cn[3] = {C.nx, C.ny, C.nz};
        for (int d = 0; d < 3; ++d) {
            if (fn[d] != cn[d] && fn[d] != 2 * cn[d]) throw KsError(KS_ERR_UNSUPPORTED, "MAC semicoarsening level sizes");
            hl[d] *= fn[d] / cn[d];
        }
        C.ix2 = 1.0 / (hl[0] * hl[0]); C.iy2 = 1.0 / (hl[1] * hl[1]); C.iz2 = 1.0 / (hl[2] * hl[2]);
        const size_t nc = (size_t)C.nx * C.ny * C.nz;
        C.phi = q; q += nc; C.rhs = q; q += nc; C.res = q; q += nc;
        ccs_.push_back(C);
    }
    binv_ccs_h_.clear();
    CCLevelDev& B = ccs_.back();
    if (ccs_.size() > 1 && (long long)B.nx * B.ny * B.nz <= kDirectBottom) cc_direct_inverse(B, binv_ccs_h_);
    binvs_.alloc(std::max<size_t>(1, binv_ccs_h_.size()));
    if (!binv_ccs_h_.empty())
        ck(cudaMemcpy(binvs_.p, binv_ccs_h_.data(), binv_ccs_h_.size() * sizeof(double), cudaMemcpyHostToDevice), "H2D bottom inverse");
    B.binv = binv_ccs_h_.empty() ? nullptr : binvs_.p;
    glev_s_ = 0;
    for (size_t l = 1; l + 1 < ccs_.size(); ++l)
        if ((long long)ccs_[l].nx * ccs_[l].ny * ccs_[l].nz <= (1LL << 18)) {
            glev_s_ = l;
            break;
        }
    mac_semi_ = true;
}

// FP32 copies of the semicoarsened MAC levels (mixed precision); level 0 is
// cc32_[0].
void Sim::mac_semi_mixed() {
    size_t tot = 0;
    for (size_t l = 1; l < ccs_.size(); ++l) tot += 3 * (size_t)ccs_[l].nx * ccs_[l].ny * ccs_[l].nz;
    mgbufs32_.alloc(tot);
    float* q = mgbufs32_.p;
    ccs32_.clear();
    ccs32_.push_back(cc32_[0]);
    ccs32_[0].binv = nullptr;
    for (size_t l = 1; l < ccs_.size(); ++l) {
        CCLevelT<float> C{};
        C.nx = ccs_[l].nx; C.ny = ccs_[l].ny; C.nz = ccs_[l].nz; C.zper = ccs_[l].zper;
        C.ix2 = (float)ccs_[l].ix2; C.iy2 = (float)ccs_[l].iy2; C.iz2 = (float)ccs_[l].iz2;
        const size_t nc = (size_t)C.nx * C.ny * C.nz;
        C.phi = q; q += nc; C.rhs = q; q += nc; C.res = q; q += nc;
        ccs32_.push_back(C);
    }
    std::vector<float> b32(binv_ccs_h_.size());
    for (size_t m = 0; m < binv_ccs_h_.size(); ++m) b32[m] = (float)binv_ccs_h_[m];
    binvs32_.alloc(std::max<size_t>(1, b32.size()));
    if (!b32.empty()) ck(cudaMemcpy(binvs32_.p, b32.data(), b32.size() * sizeof(float), cudaMemcpyHostToDevice), "H2D bottom inverse");
    ccs32_.back().binv = b32.empty() ? nullptr : binvs32_.p;
}

// ---------------------------------------------------------------- allocation
void Sim::alloc() {
    const size_t N = (size_t)g_.N, NF = (size_t)g_.NFz;
    vel_.alloc(3 * N);
    vel_old_.alloc(3 * N);
    vel_tmp_.alloc(3 * N);
    gp_.alloc(3 * N);
    p_.alloc((size_t)g_.nx * g_.ny * (g_.zper ? g_.nz : g_.nz + 1));
    src_.alloc(3 * N);
    forces_.alloc(3 * N);
    mueff_.alloc(N);
    divtau_.alloc(3 * N);
    conv_.alloc(3 * N);
    act_.alloc(S_.act ? 3 * N : 3);
    wg_.alloc(2 * (size_t)g_.nx * g_.ny);
    umac_[0].alloc(N);
    umac_[1].alloc(N);
    umac_[2].alloc(NF);
    // Godunov scratch: per face direction ad, edge[3], lo[3], hi[3], tedge[3],
    // flux[3]; tr[a][b][3] for the six (a, b) pairs.  MOL needs the fluxes only.
    const size_t fsz[3] = {N, N, NF};
    size_t total = 0;
    for (int d = 0; d < 3; ++d) total += fsz[d] * (godunov_ ? 16 : 3);
    if (godunov_)
        for (int a = 0; a < 3; ++a) total += 2 * 3 * fsz[a] + 2 * 3 * N;
    gbuf_.alloc(total);
    double* q = gbuf_.p;
    if (!godunov_) {
        conv_old_.alloc(3 * N);
        for (int d = 0; d < 3; ++d)
            for (int n = 0; n < 3; ++n) { gb_.flux[d][n] = q; q += fsz[d]; }
    }
    for (int d = 0; d < 3 && godunov_; ++d) {
        gb_.ad[d] = q; q += fsz[d];
        for (int n = 0; n < 3; ++n) { gb_.edge[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { gb_.lo[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { gb_.hi[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { gb_.tedge[d][n] = q; q += fsz[d]; }
        for (int n = 0; n < 3; ++n) { gb_.flux[d][n] = q; q += fsz[d]; }
    }
    for (int a = 0; a < 3 && godunov_; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            for (int n = 0; n < 3; ++n) { gb_.tr[a][b][n] = q; q += fsz[a]; }
        }
    for (int d = 0; d < 3 && godunov_; ++d)
        for (int n = 0; n < 3; ++n) {
            gb_.pm[d][n] = q; q += N;
            gb_.pp[d][n] = q; q += N;
        }
    // multigrid hierarchies
    std::vector<std::array<int, 3>> dims;
    int n3[3] = {g_.nx, g_.ny, g_.nz};
    while (true) {
        dims.push_back({n3[0], n3[1], n3[2]});
        bool can = true;
        for (int d = 0; d < 3; ++d) can = can && (n3[d] % 4 == 0);
        if (!can) break;
        // a level of at most kDirectBottom cells and nodes is solved exactly
        // (bottom_setup), cheaper than the launch-bound levels below it
        const long long ncl = (long long)n3[0] * n3[1] * n3[2], nnl = (long long)n3[0] * n3[1] * (n3[2] + (g_.zper ? 0 : 1));
        if (dims.size() > 1 && ncl <= kDirectBottom && nnl <= kDirectBottom) break;
        for (int d = 0; d < 3; ++d) n3[d] /= 2;
    }
    size_t mgtot = 0;
    for (auto& dm : dims) {
        const size_t nc = (size_t)dm[0] * dm[1] * dm[2];
        const size_t nn = (size_t)dm[0] * dm[1] * (dm[2] + (g_.zper ? 0 : 1));
        mgtot += 3 * nc + 4 * nn;
    }
    // the multigrid and face kernels index a level with 32-bit integers and put
    // y (and z chunks) on the second grid dimension of their launches
    if ((long long)g_.nx * g_.ny * (g_.nz + 1) >= (1LL << 31)) throw KsError(KS_ERR_UNSUPPORTED, "grid of 2^31 or more nodes");
    auto chunks = [](long long n) { return (n + 31) / 32; };
    if (g_.ny > 65535 || g_.nz > 65535 || g_.ny * chunks(g_.nz + 1) > 65535 || g_.nz * chunks(g_.ny) > 65535)
        throw KsError(KS_ERR_UNSUPPORTED, "amr.n_cell too large in y or z for the column launches");
    mgbuf_.alloc(mgtot);
    q = mgbuf_.p;
    double h[3] = {g_.dx, g_.dy, g_.dz};
    for (auto& dm : dims) {
        CCLevelDev C{};
        C.nx = dm[0]; C.ny = dm[1]; C.nz = dm[2]; C.zper = g_.zper;
        C.ix2 = 1.0 / (h[0] * h[0]); C.iy2 = 1.0 / (h[1] * h[1]); C.iz2 = 1.0 / (h[2] * h[2]);
        const size_t nc = (size_t)dm[0] * dm[1] * dm[2];
        C.phi = q; q += nc; C.rhs = q; q += nc; C.res = q; q += nc;
        cc_.push_back(C);
        NDLevelDev Nd{};
        Nd.nx = dm[0]; Nd.ny = dm[1]; Nd.nz = dm[2] + (g_.zper ? 0 : 1); Nd.zper = g_.zper;
        const double mu1[3] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0};
        double sg[3][3];
        for (int d = 0; d < 3; ++d) {
            const double i2 = 1.0 / (h[d] * h[d]);
            sg[d][0] = -i2; sg[d][1] = 2.0 * i2; sg[d][2] = -i2;
        }
        for (int c = 0; c < 3; ++c)
            for (int b = 0; b < 3; ++b)
                for (int a = 0; a < 3; ++a)
                    Nd.W[(c * 3 + b) * 3 + a] = -(sg[0][a] * mu1[b] * mu1[c] + mu1[a] * sg[1][b] * mu1[c] + mu1[a] * mu1[b] * sg[2][c]);
        const double wf = std::max(std::fabs(Nd.W[12]), std::max(std::fabs(Nd.W[10]), std::fabs(Nd.W[4])));
        Nd.faces_zero = wf <= 1e-13 * std::fabs(Nd.W[13]);
        const size_t nn = (size_t)Nd.nx * Nd.ny * Nd.nz;
        Nd.phi = q; q += nn; Nd.rhs = q; q += nn; Nd.res = q; q += nn; Nd.tmp = q; q += nn;
        nd_.push_back(Nd);
        for (int d = 0; d < 3; ++d) h[d] *= 2;
    }
    nod_.omega = nodal_jacobi_weight(nd_[0].W, nod_.omega);
    bottom_setup();
    // graphed tail: from the first level below level 0 of at most 2^18 cells
    // (its kernels fill a fraction of the GPU and are bound by launch latency)
    glev_ = 0;
    for (size_t l = 1; l + 1 < cc_.size(); ++l)
        if ((long long)cc_[l].nx * cc_[l].ny * cc_[l].nz <= (1LL << 18)) {
            glev_ = l;
            break;
        }
    if (mac_.semi) mac_semi_setup();
    parts_.alloc(4 * 1216);
    red_.alloc(8);
    if (temp_ || S_.ablf) layer_.alloc(3 * (size_t)g_.nz);
    if (temp_) {
        for (DevBuf<double>* b : {&theta_, &theta_old_, &theta_nph_, &alpha_, &tdiff_, &tconv_, &ttmp_, &tb_, &tdinv_}) b->alloc(N);
        tgz_.alloc((size_t)g_.nx * g_.ny);
        tparts_.alloc((size_t)tdiff_blocks(g_));
        if (!godunov_) tconv_old_.alloc(N);
        if (gb_.flux[0][0] == nullptr) throw KsError(KS_ERR_UNSUPPORTED, "temperature transport needs the face scratch");
    }
    size_t maxpts = 1;
    for (auto& d : disks_) maxpts = std::max(maxpts, (size_t)d.nr * d.nt);
    pts_.alloc(4 * maxpts);
    samp_.alloc(3 * maxpts);
    launch_fill(ctx_, mueff_.p, mu_, g_.N);
}

void Sim::init_fields(const Deck& D) {
    const std::string phys = D.str("incflo.physics", "");
    if (phys == "TaylorGreenVortex") {
        rho_ = D.num("TGV.density", rho_);
        S_.rho = rho_;
        S_.irho = 1.0 / rho_;
        const double L[3] = {phi_[0] - plo_[0], phi_[1] - plo_[1], phi_[2] - plo_[2]};
        launch_init_tgv(ctx_, g_, vel_.p, plo_, L);
    } else if (phys == "ABL" && !D.has_prefix("ks_init.")) {
        // ABLFieldInit (src/wind_energy/ABLFieldInit.cpp:215-372), uniform-wind branch:
        // incflo.velocity plus the sinusoidal perturbation (perturb_velocity, default on)
        auto u = D.nums("incflo.velocity");
        const double U[3] = {u.at(0), u.at(1), u.at(2)};
        if (D.flag("ABL.linear_profile", 0)) throw KsError(KS_ERR_UNSUPPORTED, "ABL.linear_profile");
        const double pi = 3.14159265358979323846;
        const double refh = D.num("ABL.perturb_ref_height", 50.0), ibh = D.num("ABL.ib_height", 0.0);
        const double aval = D.num("ABL.Uperiods", 4.0) * 2.0 * pi / (phi_[1] - plo_[1]);
        const double bval = D.num("ABL.Vperiods", 4.0) * 2.0 * pi / (phi_[0] - plo_[0]);
        const double ufac = D.num("ABL.deltaU", 1.0) * std::exp(0.5) / refh, vfac = D.num("ABL.deltaV", 1.0) * std::exp(0.5) / refh;
        launch_init_abl_ref(ctx_, g_, vel_.p, plo_, U, D.flag("ABL.perturb_velocity", 1), aval, bval, ufac, vfac, refh, ibh);
    } else if (phys == "ABL" || phys == "FreeStream") {
        const std::string prof = lc(D.str("ks_init.profile", phys == "ABL" ? "loglaw" : "uniform"));
        double U[3] = {0, 0, 0};
        if (D.has("incflo.velocity")) { auto u = D.nums("incflo.velocity"); for (int d = 0; d < 3; ++d) U[d] = u.at(d); }
        const double utop = D.num("ks_init.loglaw_utop", 8.0);
        const double H = phi_[2] - plo_[2];
        const double ut = utop * kappa_ / std::log(H / z0_);
        const double amp = D.num("ks_init.noise_amplitude", 0.0);
        const double zmax = D.num("ks_init.noise_zmax", 1e300);
        const unsigned long long seed = (unsigned long long)D.flag("ks_init.noise_seed", 0);
        launch_init_abl(ctx_, g_, vel_.p, prof == "loglaw", U, ut / kappa_, z0_, amp, zmax - plo_[2], seed);
    } else if (!phys.empty()) {
        throw KsError(KS_ERR_UNSUPPORTED, "incflo.physics = " + phys);
    }
    if (temp_) {  // piecewise-linear temperature profile (ABLFieldInit.cpp:318-327)
        auto th = D.nums("ABL.temperature_heights"), tv = D.nums("ABL.temperature_values");
        if (th.size() != tv.size() || th.empty()) throw KsError(KS_ERR_DECK, "ABL.temperature_heights and temperature_values differ in length");
        std::vector<double> hv(th);
        hv.insert(hv.end(), tv.begin(), tv.end());
        tprof_.alloc(hv.size());
        ck(cudaMemcpy(tprof_.p, hv.data(), hv.size() * sizeof(double), cudaMemcpyHostToDevice), "H2D");
        launch_theta_profile(ctx_, g_, theta_.p, plo_[2], tprof_.p, tprof_.p + th.size(), (int)th.size());
    }
}

// ---------------------------------------------------------------- reductions
double Sim::reduce(int np, int ncomp, int op_max, double* host) {
    launch_reduce(ctx_, parts_.p, np, ncomp, op_max, red_.p);
    ck(cudaMemcpyAsync(hred_, red_.p, ncomp * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
    sync();
    if (host)
        for (int c = 0; c < ncomp; ++c) host[c] = hred_[c];
    return hred_[0];
}

// ---------------------------------------------------------------- compute_dt
void Sim::compute_dt() {
    int np = 0;
    launch_cfl(ctx_, g_, vel_.p, src_.p, mueff_.p, rho_, parts_.p, &np);
    double m[3];
    reduce(np, 3, 1, m);
    if (!std::isfinite(m[0]) || !std::isfinite(m[1]) || !std::isfinite(m[2])) throw KsError(KS_ERR_NONFINITE, "non-finite CFL");
    // the diffusion CFL counts for explicit diffusion only (incflo_compute_dt.cpp:37,140-145,211-214)
    t_.set_cfl(m[0], diff_type_ == 0 ? m[1] : 0.0, t_.force_cfl ? m[2] : 0.0);
}

// SrcTermOp<ICNS> (icns_ops.H:78-124) at the clock's current step: the
// oscillatory BodyForce takes its factor at the mid-step time (BodyForce.cpp:145-160)
void Sim::sources(const double* vel, const double* theta) {
    S_.t_nph = 0.5 * (t_.cur + t_.next);
    launch_sources(ctx_, g_, vel, gp_.p, act_.p, src_.p, S_, theta);
}

// ---------------------------------------------------------------- ABL
void Sim::abl_update() {
    if (!wallmodel_) return;
    int np = 0;
    launch_plane_sums(ctx_, g_, vel_.p, parts_.p, &np);
    double s[3];
    reduce(np, 3, 0, s);
    const double M = (double)g_.nx * g_.ny;
    um_[0] = s[0] / M;
    um_[1] = s[1] / M;
    vmag_ = s[2] / M;
    utau_ = kappa_ * vmag_ / std::log(zref_ / z0_);
    if (temp_) {  // theta_mean at z_ref for the heat flux (ABLWallFunction.cpp:206-207)
        launch_layer_sums(ctx_, g_, theta_.p, layer_.p);
        ck(cudaMemcpyAsync(hred_, layer_.p, sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
        sync();
        theta_mean_ = hred_[0] / M;
    }
}

// ABL::pre_advance_work -> ABLForcing::set_mean_velocities (ABL.cpp:176-205,
// ABLForcing.H:37-64): layer averages of u and v interpolated to the forcing
// height as FieldPlaneAveraging does (FieldPlaneAveraging.cpp:78-96,151-164),
// force = (target - mean) / dt.
void Sim::abl_forcing_update() {
    if (!S_.ablf) return;
    const int nz = g_.nz;
    launch_layer_sums(ctx_, g_, vel_.p, layer_.p);
    launch_layer_sums(ctx_, g_, vel_.p + g_.N, layer_.p + nz);
    std::vector<double> h(2 * (size_t)nz);
    ck(cudaMemcpyAsync(h.data(), layer_.p, 2 * nz * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
    sync();
    const double M = (double)g_.nx * g_.ny;
    int ind = 0;
    double c = 0.0;
    const double x = ablf_h_, xlo = plo_[2], dz = g_.dz;
    if (x > xlo + 0.5 * dz) {
        ind = (int)std::floor((x - xlo) / dz - 0.5);
        c = (x - (xlo + (ind + 0.5) * dz)) / dz;
    }
    if (ind + 1 >= nz) {
        ind = nz - 2;
        c = 1.0;
    }
    const double mu0 = (h[ind] / M) * (1.0 - c) + (h[ind + 1] / M) * c;
    const double mv0 = (h[nz + ind] / M) * (1.0 - c) + (h[nz + ind + 1] / M) * c;
    S_.ablf_force[0] = (ablf_target_[0] - mu0) / t_.dt[0];
    S_.ablf_force[1] = (ablf_target_[1] - mv0) / t_.dt[0];
}

// ---------------------------------------------------------------- actuators
static void rot(const double* a, double ang, const double* v, double* o) {
    const double c = std::cos(ang), s = std::sin(ang);
    const double dd = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
    const double x[3] = {a[1] * v[2] - a[2] * v[1], a[2] * v[0] - a[0] * v[2], a[0] * v[1] - a[1] * v[0]};
    for (int m = 0; m < 3; ++m) o[m] = v[m] * c + x[m] * s + a[m] * dd * (1 - c);
}

// Sampling points (disk_ops.cpp:378-412) and force ring points
// (disk_spreading.H:45-105) of one disk, x/y/z per point, ordered radius-major.
void Sim::disk_points(const Disk& d, std::vector<double>& sample, std::vector<double>& ring) const {
    const double pi = 3.14159265358979323846;
    const double* ax = d.sample;  // the sampling disk's axis (compute_disk_points with sample_vec)
    double rv[3] = {-ax[1], ax[0], 0.0};
    const double rm = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1]);
    rv[0] /= rm;
    rv[1] /= rm;
    const double drs = 0.5 * d.D / d.nr;
    const double shift = d.nr == 1 ? 0.0 : 0.5;
    const int np = d.nr * d.nt;
    sample.assign(3 * (size_t)np, 0.0);
    for (int ir = 0; ir < d.nr; ++ir)
        for (int it = 0; it < d.nt; ++it) {
            double r[3];
            rot(ax, 2 * pi / d.nt * it, rv, r);
            for (int m = 0; m < 3; ++m) sample[3 * (ir * d.nt + it) + m] = d.center[m] + d.to_sample * d.D * ax[m] + drs * (ir + shift) * r[m];
        }
    ring.assign(3 * (size_t)np, 0.0);
    ax = d.normal;  // the force ring lies in the disk plane
    for (int ip = 0; ip < d.nr; ++ip) {
        double pos[3];
        for (int m = 0; m < 3; ++m) pos[m] = d.center[m] + (ip + 0.5) * d.dr * d.cvec[m];
        for (int it = 0; it < d.nt; ++it) {
            const double ang = 2 * pi / d.nt * it;
            double* o = &ring[3 * (ip * d.nt + it)];
            if (d.about_center) {
                const double rel[3] = {pos[0] - d.center[0], pos[1] - d.center[1], pos[2] - d.center[2]};
                rot(ax, ang, rel, o);
                for (int m = 0; m < 3; ++m) o[m] += d.center[m];
            } else {
                rot(ax, ang, pos, o);  // the reference rotates the absolute position (disk_spreading.H:85-86)
            }
        }
    }
}

void Sim::actuator_update() {
    if (!S_.act) return;
    const double pi = 3.14159265358979323846;
    launch_fill(ctx_, act_.p, 0.0, 3 * g_.N);
    for (auto& d : disks_) {
        // sample points on the sampling disk (disk_ops.cpp:378-412)
        const double* ax = d.normal;
        const int np = d.nr * d.nt;
        std::vector<double> hp, rpos;
        disk_points(d, hp, rpos);
        for (int p = 0; p < np; ++p) {
            const double hh[3] = {g_.dx, g_.dy, g_.dz};
            const int nn[3] = {g_.nx, g_.ny, g_.nz};
            for (int m = 0; m < 3; ++m) {
                const int c = (int)std::floor((hp[3 * p + m] - plo_[m] - 0.5 * hh[m]) / hh[m]);
                if (c < -1 || c + 1 > nn[m]) throw KsError(KS_ERR_DECK, "actuator sample point outside the domain");
            }
        }
        ck(cudaMemcpyAsync(pts_.p, hp.data(), hp.size() * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "H2D");
        launch_act_sample(ctx_, g_, vel_.p, pts_.p, np, plo_, samp_.p);
        std::vector<double> sv(3 * (size_t)np);
        ck(cudaMemcpyAsync(sv.data(), samp_.p, sv.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
        sync();
        double ref[3] = {0, 0, 0};
        for (int ir = 0; ir < d.nr; ++ir) {
            const double w = ((ir + 1.0) * (ir + 1.0) - (double)ir * ir) / ((double)d.nr * d.nr * d.nt);
            for (int it = 0; it < d.nt; ++it)
                for (int m = 0; m < 3; ++m) ref[m] += sv[3 * (ir * d.nt + it) + m] * w;
        }
        for (int m = 0; m < 3; ++m) d.ref[m] = ref[m];
        const double un = ref[0] * ax[0] + ref[1] * ax[1] + ref[2] * ax[2];
        d.uinf2 = un * un;
        const double umag = std::sqrt(d.uinf2);
        if (d.ws.size() == 1 || umag <= d.ws.front()) d.ct_now = d.ct.front();
        else if (umag >= d.ws.back()) d.ct_now = d.ct.back();
        else {
            size_t m = 0;
            while (m + 1 < d.ws.size() && d.ws[m + 1] < umag) ++m;
            d.ct_now = d.ct[m] + (d.ct[m + 1] - d.ct[m]) * (umag - d.ws[m]) / (d.ws[m + 1] - d.ws[m]);
        }
        const double aero = 0.5 * d.uinf2 * d.ct_now;
        // ring points with per-point force magnitude
        std::vector<double> ring;
        double bmin[3] = {1e300, 1e300, 1e300}, bmax[3] = {-1e300, -1e300, -1e300};
        for (int ip = 0; ip < d.nr; ++ip) {
            const double r = (ip + 0.5) * d.dr, rp = r + 0.5 * d.dr, rmn = r - 0.5 * d.dr;
            const double f = aero * pi * (rp * rp - rmn * rmn);
            for (int it = 0; it < d.nt; ++it) {
                const double* o = &rpos[3 * (ip * d.nt + it)];
                for (int m = 0; m < 3; ++m) {
                    ring.push_back(o[m]);
                    bmin[m] = std::min(bmin[m], o[m]);
                    bmax[m] = std::max(bmax[m], o[m]);
                }
                ring.push_back(f / d.nt);
            }
        }
        const int nring = (int)ring.size() / 4;
        ck(cudaMemcpyAsync(pts_.p, ring.data(), ring.size() * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "H2D");
        // cells within 4 eps of any ring point, clamped to the domain
        int lo[3], hi[3];
        const double h[3] = {g_.dx, g_.dy, g_.dz};
        const int nn[3] = {g_.nx, g_.ny, g_.nz};
        for (int m = 0; m < 3; ++m) {
            lo[m] = std::max(0, (int)std::floor((bmin[m] - 4.0 * d.eps - plo_[m]) / h[m]) - 1);
            hi[m] = std::min(nn[m] - 1, (int)std::floor((bmax[m] + 4.0 * d.eps - plo_[m]) / h[m]) + 1);
        }
        launch_act_spread(ctx_, g_, act_.p, pts_.p, nring, ax, d.eps, plo_, lo, hi);
        sync();  // pts_ is reused by the next disk
    }
}

// ---------------------------------------------------------------- MAC projection
template <typename F>
void Sim::mg_graph_run(MGGraph& G, double key, F&& body) {
    if (!G.exec || G.key != key) {
        cudaGraph_t graph = nullptr;
        const long long l0 = ctx_.launches;
        ck(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        ctx_.capturing = true;
        body();
        ctx_.capturing = false;
        ck(cudaStreamEndCapture(ctx_.stream, &graph), "graph capture");
        G.nodes = ctx_.launches - l0;
        ctx_.launches = l0;
        if (G.exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(G.exec, graph, &info) != cudaSuccess) {
                (void)cudaGetLastError();
                cudaGraphExecDestroy(G.exec);
                G.exec = nullptr;
            }
        }
        if (!G.exec) ck(cudaGraphInstantiate(&G.exec, graph, 0), "graph instantiate");
        cudaGraphDestroy(graph);
        G.key = key;
    }
    const bool p = ctx_.prof_match("(mg_coarse_graph)");
    if (p) ctx_.prof_begin("(mg_coarse_graph)", 0.0);
    ck(cudaGraphLaunch(G.exec, ctx_.stream), "graph launch");
    if (p) ctx_.prof_end();
    ctx_.launches += G.nodes;
}

template <typename T>
void Sim::cc_vcycle(std::vector<CCLevelT<T>>& Ls, size_t l, double beta, bool in_graph) {
    CCLevelT<T>& L = Ls[l];
    const size_t gl = mac_semi_ ? glev_s_ : glev_;  // the MAC solve uses one hierarchy for the life of the handle
    if (!in_graph && mg_graphs_ && gl > 0 && l == gl) {
        mg_graph_run(gcc_[sizeof(T) == 4 ? 1 : 0], beta, [&]() { cc_vcycle(Ls, l, beta, true); });
        return;
    }
    if (l + 1 == Ls.size()) {
        launch_cc_bottom(ctx_, L, beta, mac_.bottom);
        return;
    }
    for (int s = 0; s < mac_.nu1; ++s) {
        launch_cc_gsrb(ctx_, L, beta, 0);
        launch_cc_gsrb(ctx_, L, beta, 1);
    }
    launch_cc_resid(ctx_, L, beta, nullptr, nullptr, mac_.nu1 > 0 ? 1 : -1);  // after the colour-1 half-sweep
    launch_cc_restrict(ctx_, L, Ls[l + 1]);
    cc_vcycle(Ls, l + 1, beta, in_graph);
    launch_cc_prolong(ctx_, L, Ls[l + 1]);
    for (int s = 0; s < mac_.nu2; ++s) {
        launch_cc_gsrb(ctx_, L, beta, 0);
        launch_cc_gsrb(ctx_, L, beta, 1);
    }
}

// Mixed precision: FP32 copies of the multigrid hierarchies.  The FP64
// residual, right-hand side and solution of the finest level stay in the
// FP64 levels; each outer (defect-correction) iteration solves the FP64
// residual equation with one FP32 V-cycle and adds the correction in FP64.
void Sim::set_mixed(int on) {
    mixed_ = on ? 1 : 0;
    if (!mixed_ || !cc32_.empty()) return;
    size_t tot = 0;
    for (size_t l = 0; l < cc_.size(); ++l) {
        tot += 3 * (size_t)cc_[l].nx * cc_[l].ny * cc_[l].nz;
        tot += 4 * (size_t)nd_[l].nx * nd_[l].ny * nd_[l].nz;
    }
    mgbuf32_.alloc(tot);
    float* q = mgbuf32_.p;
    for (size_t l = 0; l < cc_.size(); ++l) {
        CCLevelT<float> C{};
        C.nx = cc_[l].nx; C.ny = cc_[l].ny; C.nz = cc_[l].nz; C.zper = cc_[l].zper;
        C.ix2 = (float)cc_[l].ix2; C.iy2 = (float)cc_[l].iy2; C.iz2 = (float)cc_[l].iz2;
        const size_t nc = (size_t)C.nx * C.ny * C.nz;
        C.phi = q; q += nc; C.rhs = q; q += nc; C.res = q; q += nc;
        cc32_.push_back(C);
        NDLevelT<float> Nd{};
        Nd.nx = nd_[l].nx; Nd.ny = nd_[l].ny; Nd.nz = nd_[l].nz; Nd.zper = nd_[l].zper;
        for (int m = 0; m < 27; ++m) Nd.W[m] = (float)nd_[l].W[m];
        Nd.faces_zero = nd_[l].faces_zero;
        const size_t nn = (size_t)Nd.nx * Nd.ny * Nd.nz;
        Nd.phi = q; q += nn; Nd.rhs = q; q += nn; Nd.res = q; q += nn; Nd.tmp = q; q += nn;
        nd32_.push_back(Nd);
    }
    // FP32 copies of the advection inputs
    {
        const size_t N = (size_t)g_.N;
        g32_.alloc(6 * N + 2 * N + (size_t)g_.NFz);
        float* f = g32_.p;
        in32_.vel = f; f += 3 * N;
        in32_.forces = f; f += 3 * N;
        in32_.mac[0] = f; f += N;
        in32_.mac[1] = f; f += N;
        in32_.mac[2] = f;
    }
    // FP32 copies of the bottom inverses
    std::vector<float> b32(binv_cc_h_.size() + binv_nd_h_.size());
    for (size_t m = 0; m < binv_cc_h_.size(); ++m) b32[m] = (float)binv_cc_h_[m];
    for (size_t m = 0; m < binv_nd_h_.size(); ++m) b32[binv_cc_h_.size() + m] = (float)binv_nd_h_[m];
    binv32_.alloc(std::max<size_t>(1, b32.size()));
    if (!b32.empty()) ck(cudaMemcpy(binv32_.p, b32.data(), b32.size() * sizeof(float), cudaMemcpyHostToDevice), "H2D bottom inverse");
    cc32_.back().binv = binv_cc_h_.empty() ? nullptr : binv32_.p;
    nd32_.back().binv = binv_nd_h_.empty() ? nullptr : binv32_.p + binv_cc_h_.size();
    if (mac_semi_) mac_semi_mixed();
}

void Sim::mac_project() {
    const double beta = 1.0 / rho_;
    std::vector<CCLevelDev>& M = mac_semi_ ? ccs_ : cc_;
    std::vector<CCLevelT<float>>& M32 = mac_semi_ ? ccs32_ : cc32_;
    for (auto& L : M) {
        const double d0 = 2.0 * L.ix2 + 2.0 * L.iy2;
        L.inv_diag[0] = 1.0 / (-beta * (d0 + 2.0 * L.iz2));
        L.inv_diag[1] = 1.0 / (-beta * (d0 + L.iz2));
        L.inv_diag[2] = 1.0 / (-beta * d0);
        const double dc[3] = {d0 + 2.0 * L.iz2, d0 + L.iz2, d0};
        for (int m = 0; m < 3; ++m) {
            L.dg[m] = -beta * dc[m];
            L.gs[m][0] = L.ix2 / dc[m];
            L.gs[m][1] = L.iy2 / dc[m];
            L.gs[m][2] = L.iz2 / dc[m];
        }
    }
    for (size_t l = 0; l < M32.size(); ++l)
        for (int m = 0; m < 3; ++m) {
            M32[l].inv_diag[m] = (float)M[l].inv_diag[m];
            M32[l].dg[m] = (float)M[l].dg[m];
            for (int q = 0; q < 3; ++q) M32[l].gs[m][q] = (float)M[l].gs[m][q];
        }
    CCLevelDev& L = M[0];
    int np = 0;
    launch_mac_rhs(ctx_, g_, umac_[0].p, umac_[1].p, umac_[2].p, L.rhs, parts_.p, &np);
    launch_reduce(ctx_, parts_.p, np, 1, 0, red_.p);
    const bool warm = mg_warm_ && mac_prev_ok_;
    launch_sub_ratio(ctx_, L.rhs, g_.N, red_.p, (double)g_.N, warm ? parts_.p : nullptr, &np);
    double bnorm = 0.0;  // |rhs|, the initial residual of a zero start
    if (warm) {
        bnorm = reduce(np, 1, 1, nullptr);
        ck(cudaMemcpyAsync(L.phi, mac_phi_prev_.p, sizeof(double) * g_.N, cudaMemcpyDeviceToDevice, ctx_.stream), "D2D");
    } else {
        launch_fill(ctx_, L.phi, 0.0, g_.N);
    }
    // mixed precision: each FP64 residual is the next FP32 cycle's right-hand side
    int zc = -1;  // the colour whose residual is zero (none for the starting iterate)
    auto resid = [&]() {
        if (mixed_) launch_cc_resid32(ctx_, L, beta, M32[0].rhs, M32[0].phi, parts_.p, &np);
        else launch_cc_resid(ctx_, L, beta, parts_.p, &np, zc);
    };
    resid();
    // after a V-cycle the last half-sweep was colour 1's (post-smoothing on a level above the bottom)
    if (mac_.nu2 > 0 && M.size() > 1) zc = 1;
    const double r0 = reduce(np, 1, 1, nullptr);
    mac_r0_ = r0;
    const double target = std::max(mac_.atol, mac_.rtol * std::max(bnorm, r0));
    mac_tgt_ = target;
    int it = 0;
    double rn = r0;
    while (rn > target && it < mac_.maxiter) {
        int inner = 1;
        if (mixed_) {  // up to mg_inner_ FP32 V-cycles on the correction equation (as the nodal solve)
            inner = std::min(mg_inner_, mac_.maxiter - it);
            for (int c = 0; c < inner; ++c) cc_vcycle(M32, 0, beta);
            launch_add_f32(ctx_, L.phi, M32[0].phi, g_.N);
        } else {
            cc_vcycle(M, 0, beta);
        }
        resid();
        rn = reduce(np, 1, 1, nullptr);
        it += inner;
        if (!std::isfinite(rn)) throw KsError(KS_ERR_NONFINITE, "MAC projection diverged");
        if (rn > 1e20 * r0) throw KsError(KS_ERR_NOT_CONVERGED, "MAC projection diverged (residual above 1e20 times the initial one)");
    }
    // MLMGOptions sets fixed-iteration mode by default (src/core/MLMGOptions.H:126-128,
    // MLMGOptions.cpp:65-66): MLMG then stops at maxiter without aborting;
    // with do_fixed_iters = 0 it aborts
    if (rn > target && !mac_.fixed_iters) throw KsError(KS_ERR_NOT_CONVERGED, "MAC projection did not converge in mac_proj.maxiter V-cycles");
    mac_it_ = it;
    mac_r_ = rn;
    launch_mac_correct(ctx_, g_, L.phi, umac_[0].p, umac_[1].p, umac_[2].p, beta);
    if (mg_warm_) {
        if (mac_phi_prev_.n != (size_t)g_.N) mac_phi_prev_.alloc(g_.N);
        ck(cudaMemcpyAsync(mac_phi_prev_.p, L.phi, sizeof(double) * g_.N, cudaMemcpyDeviceToDevice, ctx_.stream), "D2D");
        mac_prev_ok_ = true;
    }
}

// ---------------------------------------------------------------- nodal projection
template <typename T>
void Sim::nd_vcycle(std::vector<NDLevelT<T>>& Ls, size_t l, double sigma, int skip_sweeps, bool in_graph) {
    NDLevelT<T>& L = Ls[l];
    // a replay must leave the host's phi / tmp pointers as the recording did:
    // an even number of Jacobi swaps per level returns them to their start
    if (!in_graph && mg_graphs_ && glev_ > 0 && l == glev_ && (nod_.nu1 + nod_.nu2) % 2 == 0) {
        mg_graph_run(gnd_[sizeof(T) == 4 ? 1 : 0], sigma, [&]() { nd_vcycle(Ls, l, sigma, 0, true); });
        return;
    }
    if (l + 1 == Ls.size()) {
        launch_nd_bottom(ctx_, L, sigma, nod_.omega, nod_.bottom);
        return;
    }
    for (int s = skip_sweeps; s < nod_.nu1; ++s) {
        launch_nd_jacobi(ctx_, L, sigma, nod_.omega, L.phi, L.tmp);
        std::swap(L.phi, L.tmp);
    }
    launch_nd_resid(ctx_, L, sigma, nullptr, nullptr);
    launch_nd_restrict(ctx_, L, Ls[l + 1]);
    nd_vcycle(Ls, l + 1, sigma, 0, in_graph);
    launch_nd_prolong(ctx_, L, Ls[l + 1]);
    for (int s = 0; s < nod_.nu2; ++s) {
        launch_nd_jacobi(ctx_, L, sigma, nod_.omega, L.phi, L.tmp);
        std::swap(L.phi, L.tmp);
    }
}

// Nodal divergence of a cell field into the finest level's right-hand side,
// made solvable (weighted mean removed); the initial guess is zero.
void Sim::nd_rhs(const double* cell_field, bool from_pressure) {
    NDLevelDev& L = nd_[0];
    const long long M = (long long)L.nx * L.ny * L.nz;
    int np = 0;
    launch_nodal_rhs(ctx_, g_, cell_field, L.rhs, parts_.p, &np);
    launch_reduce(ctx_, parts_.p, np, 2, 0, red_.p);
    launch_sub_ratio(ctx_, L.rhs, M, red_.p, 0.0, from_pressure ? parts_.p : nullptr, &np);
    nod_bnorm_ = 0.0;
    if (from_pressure) {  // the pressure is the unknown of a non-incremental projection
        nod_bnorm_ = reduce(np, 1, 1, nullptr);
        ck(cudaMemcpyAsync(L.phi, p_.p, sizeof(double) * M, cudaMemcpyDeviceToDevice, ctx_.stream), "D2D");
        nod_zero_ = false;
    } else {
        launch_fill(ctx_, L.phi, 0.0, M);
        nod_zero_ = true;
    }
}

// Solve sigma A phi = rhs on the finest nodal level to the relative /
// absolute tolerance of nodal_proj (solution in nd_[0].phi).
void Sim::nd_solve(double sigma) {
    NDLevelDev& L = nd_[0];
    const long long M = (long long)L.nx * L.ny * L.nz;
    int np = 0;
    for (auto& Lv : nd_) Lv.inv_diag = 1.0 / (sigma * Lv.W[13]);
    for (size_t l = 0; l < nd32_.size(); ++l) nd32_[l].inv_diag = (float)nd_[l].inv_diag;
    int it = 0;
    double rn = 0.0, target = 0.0;
    // a solve from zero (set up by nd_rhs) takes its first residual from the
    // right-hand side without a stencil pass
    const bool zero = nod_zero_;
    nod_zero_ = false;
    if (mixed_) {  // each FP64 residual is the next FP32 cycle's right-hand side
        if (zero) launch_nd_zero_start(ctx_, L, sigma, nod_.omega, nullptr, nd32_[0].rhs, nd32_[0].phi, parts_.p, &np);
        else launch_nd_resid32(ctx_, L, sigma, nd32_[0].rhs, nd32_[0].phi, parts_.p, &np);
        const double r0 = reduce(np, 1, 1, nullptr);
        nod_r0_ = r0;
        target = std::max(nod_.atol, nod_.rtol * std::max(nod_bnorm_, r0));
        nod_tgt_ = target;
        rn = r0;
        while (rn > target && it < nod_.maxiter) {
            // The correction equation gets as many FP32 V-cycles (each
            // continuing from the last) as the contraction seen so far says
            // are still needed, at most mg_inner_nd_: FP32 holds the correction
            // to ~1e-7 of the FP64 residual, and 4 nodal cycles reduce it by
            // ~1e-4.  An FP64 residual costs about one FP32 cycle, so checking
            // only where convergence is expected saves residuals without
            // adding cycles.  Early cycles contract faster than later ones,
            // so the prediction gets half a cycle of margin.
            int inner = mg_inner_nd_;
            if (nod_rho_ > 0.0 && nod_rho_ < 1.0) {
                const double need = std::ceil(std::log(target / rn) / std::log(nod_rho_) + 0.5);
                inner = (int)std::max(1.0, std::min((double)mg_inner_nd_, need));
            }
            inner = std::min(inner, nod_.maxiter - it);
            for (int c = 0; c < inner; ++c) nd_vcycle(nd32_, 0, sigma);
            launch_add_f32(ctx_, L.phi, nd32_[0].phi, M);
            launch_nd_resid32(ctx_, L, sigma, nd32_[0].rhs, nd32_[0].phi, parts_.p, &np);
            const double rprev = rn;
            rn = reduce(np, 1, 1, nullptr);
            if (rn > 0.0 && rn < rprev) nod_rho_ = std::max(1e-3, std::pow(rn / rprev, 1.0 / inner));
            it += inner;
            if (!std::isfinite(rn)) throw KsError(KS_ERR_NONFINITE, "nodal projection diverged");
            if (rn > 1e20 * r0) throw KsError(KS_ERR_NOT_CONVERGED, "nodal projection diverged (residual above 1e20 times the initial one)");
        }
    } else {
        // The first pre-smoothing sweep of each V-cycle evaluates the residual
        // of the current iterate; its max-norm is the convergence test.  When
        // the test passes, that sweep's output is discarded.
        while (true) {
            if (it == 0 && zero) launch_nd_zero_start(ctx_, L, sigma, nod_.omega, nod_.nu1 > 0 ? L.tmp : nullptr, nullptr, nullptr, parts_.p, &np);
            else if (nod_.nu1 > 0) launch_nd_jacobi_norm(ctx_, L, sigma, nod_.omega, L.phi, L.tmp, parts_.p, &np);
            else launch_nd_resid(ctx_, L, sigma, parts_.p, &np);
            rn = reduce(np, 1, 1, nullptr);
            if (!std::isfinite(rn)) throw KsError(KS_ERR_NONFINITE, "nodal projection diverged");
            if (it == 0) {
                nod_r0_ = rn;
                target = std::max(nod_.atol, nod_.rtol * std::max(nod_bnorm_, rn));
                nod_tgt_ = target;
            }
            if (rn > 1e20 * nod_r0_) throw KsError(KS_ERR_NOT_CONVERGED, "nodal projection diverged (residual above 1e20 times the initial one)");
            if (rn <= target || it >= nod_.maxiter) break;
            if (nod_.nu1 > 0) std::swap(L.phi, L.tmp);
            nd_vcycle(nd_, 0, sigma, nod_.nu1 > 0 ? 1 : 0);
            ++it;
        }
    }
    if (rn > target && !nod_.fixed_iters) throw KsError(KS_ERR_NOT_CONVERGED, "nodal projection did not converge in nodal_proj.maxiter V-cycles");
    nod_it_ = it;
    nod_r_ = rn;
}

// ---------------------------------------------------------------- diffusion solve
// rho u - dtd divtau(u) = rho u_rhs (DiffSolverIface::linsys_solve,
// src/equation_systems/DiffusionOps.cpp:114-159: MLTensorOp, alpha 1, a = rho,
// beta = dtd, face viscosity of the current mu_eff, wall-model data from the Old
// velocity), u_rhs the current velocity and initial guess.  The stopping test
// is MLMG's: max-norm residual <= max(atol, rtol * max(|rhs|, initial
// residual)), or maxiter iterations.
//
// Every iteration is built from weighted-Jacobi sweeps of the full tensor
// operator, each one tiled divtau pass with the update fused in; the first
// sweep of an iteration also returns the max-norm residual of the incoming
// iterate.  With s = max(1 - rho / D) over the rows (D the diagonal), the
// eigenvalues of D^-1 A lie in [1 - s, 1 + s], so an unweighted sweep
// contracts the error by s.  When s < 0.1 (every LES and laminar case whose
// diffusion number dt nu / h^2 is small) an iteration is that one sweep.
// Otherwise it is a V-cycle on the MAC hierarchy's levels: weight 0.8 where
// s_l >= 0.5 (smoothing of the 1 + s end), 1 below, 8-cell averaging
// restriction, piecewise-constant prolongation, viscosity averaged to the
// coarse cells and homogeneous boundary data below the finest level.
constexpr int kDiffBottom = 24;  // sweeps on the coarsest level

void Sim::diff_alloc() {
    if (!dl_.empty()) return;
    size_t tot = 0;
    for (size_t l = 0; l < cc_.size(); ++l) {
        const size_t n = (size_t)cc_[l].nx * cc_[l].ny * cc_[l].nz;
        tot += l == 0 ? 6 * n : 16 * n;  // level 0: r, dinv; coarser: x, b, r, t, dinv (3 each) + mu
    }
    dbuf_.alloc(tot);
    dtmp_.alloc(3 * (size_t)g_.N);
    dparts_.alloc((size_t)std::max(divtau_tile_blocks(g_), 2 * diff_cell_blocks(g_)));
    double* q = dbuf_.p;
    for (size_t l = 0; l < cc_.size(); ++l) {
        DiffLevel L{};
        L.g = g_;
        L.g.nx = cc_[l].nx;
        L.g.ny = cc_[l].ny;
        L.g.nz = cc_[l].nz;
        const double f = (double)(1 << l);
        L.g.dx = g_.dx * f;
        L.g.dy = g_.dy * f;
        L.g.dz = g_.dz * f;
        L.g.idx = 1.0 / L.g.dx;
        L.g.idy = 1.0 / L.g.dy;
        L.g.idz = 1.0 / L.g.dz;
        L.g.N = (long long)L.g.nx * L.g.ny * L.g.nz;
        L.g.NFz = (long long)L.g.nx * L.g.ny * (L.g.nz + 1);
        if (l > 0 && L.g.zlo == ZWALLMODEL) L.g.zlo = ZSLIP;  // the correction equation has zero Neumann data
        const size_t n = (size_t)L.g.N;
        if (l == 0) {
            L.r = q; q += 3 * n;
            L.dinv = q; q += 3 * n;
            L.mu = mueff_.p;
        } else {
            L.x = q; q += 3 * n;
            L.b = q; q += 3 * n;
            L.r = q; q += 3 * n;
            L.t = q; q += 3 * n;
            L.dinv = q; q += 3 * n;
            L.mu = q; q += n;
        }
        dl_.push_back(L);
    }
}

void Sim::diff_vcycle(size_t l, double dtd) {
    DiffLevel& L = dl_[l];
    auto sweep = [&]() {
        launch_divtau_jacobi(ctx_, L.g, L.x, L.mu, nullptr, L.b, L.dinv, L.t, rho_, dtd, L.omega, nullptr);
        std::swap(L.x, L.t);
    };
    if (l + 1 == dl_.size()) {
        for (int s = 0; s < kDiffBottom; ++s) sweep();
        return;
    }
    for (int s = 0; s < dif_.nu1; ++s) sweep();
    launch_divtau_jacobi(ctx_, L.g, L.x, L.mu, nullptr, L.b, nullptr, L.r, rho_, dtd, 0.0, nullptr);
    DiffLevel& C = dl_[l + 1];
    launch_avg8(ctx_, L.g, C.g, L.r, C.b, 3);
    launch_fill(ctx_, C.x, 0.0, 3 * C.g.N);
    diff_vcycle(l + 1, dtd);
    launch_prolong_add(ctx_, L.g, C.g, C.x, L.x);
    for (int s = 0; s < dif_.nu2; ++s) sweep();
}

void Sim::diffuse_solve(double dtd) {
    diff_alloc();
    DiffLevel& L0 = dl_[0];
    L0.mu = mueff_.p;
    const int nc = diff_cell_blocks(g_);
    launch_rhs_b(ctx_, g_, vel_.p, rho_, vel_tmp_.p, dparts_.p);  // b = rho u_rhs, |b| maxima
    launch_diff_dinv(ctx_, g_, mueff_.p, rho_, dtd, L0.dinv, dparts_.p + nc);
    launch_reduce(ctx_, dparts_.p, nc, 2, 1, red_.p);
    ck(cudaMemcpyAsync(hred_, red_.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
    sync();
    const double bnorm = hred_[0], s0 = hred_[1];
    if (!std::isfinite(bnorm) || !std::isfinite(s0)) throw KsError(KS_ERR_NONFINITE, "non-finite diffusion right-hand side or coefficients");
    const bool cycles = s0 >= 0.1 && dl_.size() > 1;
    for (size_t l = 0; l < dl_.size(); ++l) dl_[l].omega = s0 / (double)(1u << (2 * l)) < 0.5 ? 1.0 : 0.8;
    if (cycles)
        for (size_t l = 1; l < dl_.size(); ++l) {
            launch_avg8(ctx_, dl_[l - 1].g, dl_[l].g, dl_[l - 1].mu, dl_[l].mu, 1);
            launch_diff_dinv(ctx_, dl_[l].g, dl_[l].mu, rho_, dtd, dl_[l].dinv, nullptr);
        }
    auto sweep0 = [&](double* parts) {
        launch_divtau_jacobi(ctx_, g_, vel_.p, mueff_.p, wg_.p, vel_tmp_.p, L0.dinv, dtmp_.p, rho_, dtd, L0.omega, parts);
        std::swap(vel_.p, dtmp_.p);
    };
    const int np = divtau_tile_blocks(g_);
    int it = 0;
    double r0 = 0.0, rn = 0.0, target = 0.0;
    while (true) {
        sweep0(dparts_.p);
        launch_reduce(ctx_, dparts_.p, np, 1, 1, red_.p);
        ck(cudaMemcpyAsync(hred_, red_.p, sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
        sync();
        rn = hred_[0];
        if (it == 0) {
            r0 = rn;
            target = std::max(dif_.atol, dif_.rtol * std::max(bnorm, r0));
        }
        if (!std::isfinite(rn)) throw KsError(KS_ERR_NONFINITE, "diffusion solve diverged");
        if (rn > 1e20 * std::max(r0, 1e-300)) throw KsError(KS_ERR_NOT_CONVERGED, "diffusion solve diverged (residual above 1e20 times the initial one)");
        if (rn <= target || it >= dif_.maxiter) break;
        ++it;
        if (!cycles) continue;
        // the rest of a V-cycle on the finest level (its first sweep is the one above)
        for (int s = 1; s < dif_.nu1; ++s) sweep0(nullptr);
        launch_divtau_jacobi(ctx_, g_, vel_.p, mueff_.p, wg_.p, vel_tmp_.p, nullptr, L0.r, rho_, dtd, 0.0, nullptr);
        DiffLevel& C = dl_[1];
        launch_avg8(ctx_, g_, C.g, L0.r, C.b, 3);
        launch_fill(ctx_, C.x, 0.0, 3 * C.g.N);
        diff_vcycle(1, dtd);
        launch_prolong_add(ctx_, g_, C.g, C.x, vel_.p);
        for (int s = 0; s < dif_.nu2; ++s) sweep0(nullptr);
    }
    if (rn > target && !dif_.fixed_iters) throw KsError(KS_ERR_NOT_CONVERGED, "diffusion solve did not converge in diffusion.maxiter iterations");
    dif_it_ = it;
    dif_r0_ = r0;
    dif_r_ = rn;
    dif_b_ = bnorm;
}

void Sim::apply_projection(double time, double scaling, bool incremental) {
    const bool small_dt = (time > 0.0 && t_.dt[0] < 0.1 * t_.dt[1]);
    const bool sub_old = small_dt || incremental;
    launch_proj_pre(ctx_, g_, vel_.p, vel_old_.p, gp_.p, scaling, rho_, incremental ? 0 : 1, sub_old ? 1 : 0);
    nd_rhs(vel_.p, mg_warm_ && !incremental);
    const double sigma = scaling / rho_;
    nd_solve(sigma);
    launch_nodal_post(ctx_, g_, nd_[0].phi, vel_.p, vel_old_.p, gp_.p, p_.p, sigma, sub_old ? 1 : 0, incremental ? 1 : 0);
}

// ---------------------------------------------------------------- ApplyPredictor
void Sim::apply_predictor(bool incremental) {
    if (!godunov_) {
        mol_predictor(incremental);
        return;
    }
    const double dt = t_.dt[0];
    launch_smagorinsky(ctx_, g_, vel_old_.p, mueff_.p, S_, alpha_.p, mixed_);
    sources(vel_old_.p, theta_old_.p);  // BoussinesqBuoyancy: theta at Old
    if (wallmodel_) launch_wall_grad(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, shear_, utau_ * utau_, um_[0], um_[1], vmag_, rho_);
    double* fl[9];
    for (int m = 0; m < 9; ++m) fl[m] = static_cast<double*>(gb_.flux[m / 3][m % 3]);
    launch_divtau(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, divtau_.p, 1, src_.p, forces_.p, nullptr, nullptr, dt, rho_, fl, mixed_);
    if (temp_) {  // the temperature's diff_term(Old) (no temperature sources)
        if (tzlo_ == 1)
            launch_theta_wall_grad(ctx_, g_, vel_old_.p, theta_old_.p, alpha_.p, tgz_.p, shear_, utau_, kappa_, std::log(zref_ / z0t_), vmag_,
                                   theta_mean_, rho_);
        launch_tdiff(ctx_, g_, theta_old_.p, alpha_.p, tbc(), tdiff_.p, 0, nullptr, nullptr, nullptr, nullptr, nullptr, dt, rho_, 0.0);
    }
    double* mac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_premac(ctx_, g_, vel_old_.p, forces_.p, dt, gb_, mac, mixed_, mixed_ ? &in32_ : nullptr);
    mac_project();
    if (temp_) temperature_predictor(dt);
    const double* cmac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_advection(ctx_, g_, vel_old_.p, forces_.p, cmac, dt, rho_, adv_bufs_ ? *adv_bufs_ : gb_, conv_.p, mixed_, mixed_ ? &in32_ : nullptr);
    // compute_source_term(NPH): Coriolis reads the Old velocity and gp is
    // unchanged, so only BoussinesqBuoyancy (theta at n+1/2) changes src;
    // compute_diffusion_term(Old) reproduces divtau.
    if (S_.bous) sources(vel_old_.p, theta_nph_.p);
    launch_predictor_rhs(ctx_, g_, vel_old_.p, conv_.p, src_.p, divtau_.p, vel_.p, dt, rho_, diff_fac());
    if (diff_type_ == 0) {  // explicit RK2 correction (incflo_advance.cpp:388-400)
        launch_divtau(ctx_, g_, vel_.p, mueff_.p, wg_.p, vel_tmp_.p, 2, nullptr, nullptr, vel_.p, divtau_.p, dt, rho_, fl, mixed_);
        std::swap(vel_.p, vel_tmp_.p);
    } else {  // icns().solve(dt_diff) (incflo_advance.cpp:376-386)
        diffuse_solve(diff_type_ == 2 ? dt : 0.5 * dt);
    }
    apply_projection(t_.next, dt, incremental);
}

// ---------------------------------------------------------------- MOL
// ApplyPredictor for MOL with explicit diffusion (src/incflo_advance.cpp:186-438):
// mu_eff, wall gradient and diff_term(Old) from the Old velocity, sources at
// NPH (the Coriolis term reads Old), face velocities extrapolated from Old and
// MAC-projected, conv_term(Old) with predictor_rhs (fstate Old,
// CompRHSOps.H:32-141) fused into its divergence pass, nodal projection.
void Sim::mol_predictor(bool incremental) {
    const double dt = t_.dt[0];
    launch_smagorinsky(ctx_, g_, vel_old_.p, mueff_.p, S_, alpha_.p);
    if (wallmodel_) launch_wall_grad(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, shear_, utau_ * utau_, um_[0], um_[1], vmag_, rho_);
    double* fl[9];
    for (int m = 0; m < 9; ++m) fl[m] = static_cast<double*>(gb_.flux[m / 3][m % 3]);
    // diff_term(Old) enters predictor_rhs with factor 1 / 0.5 / 0 (implicit: not formed)
    const double fac = diff_fac();
    if (fac != 0.0) launch_divtau(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, divtau_.p, 0, nullptr, nullptr, nullptr, nullptr, dt, rho_, fl);
    if (temp_) {
        if (tzlo_ == 1)
            launch_theta_wall_grad(ctx_, g_, vel_old_.p, theta_old_.p, alpha_.p, tgz_.p, shear_, utau_, kappa_, std::log(zref_ / z0t_), vmag_,
                                   theta_mean_, rho_);
        if (fac != 0.0)
            launch_tdiff(ctx_, g_, theta_old_.p, alpha_.p, tbc(), tdiff_.p, 0, nullptr, nullptr, nullptr, nullptr, nullptr, dt, rho_, 0.0);
    }
    double* mac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_mol_extrap(ctx_, g_, vel_old_.p, mac);
    mac_project();
    const double* cmac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    if (temp_) temperature_mol(false, dt);
    // sources at NPH: the Coriolis term reads Old, BoussinesqBuoyancy theta at n+1/2
    sources(vel_old_.p, temp_ ? theta_nph_.p : nullptr);
    launch_mol_advection(ctx_, g_, vel_old_.p, cmac, rho_, fl, conv_old_.p, 1, vel_old_.p, src_.p, divtau_.p, nullptr, vel_.p, dt, fac);
    if (diff_type_ != 0) diffuse_solve(diff_type_ == 2 ? dt : 0.5 * dt);
    apply_projection(t_.next, dt, incremental);
}

// ApplyCorrector (src/incflo_advance.cpp:528-652): face velocities from the
// predicted velocity and MAC projection, conv_term(New), mu_eff(New), the
// wall-model gradient (Old velocity, new mu_eff: ABLWallFunction.cpp:236-300),
// sources at New, diff_term(New) fused with corrector_rhs (explicit factors
// 1/2, 1/2: CompRHSOps.H:160-250), non-incremental nodal projection.
void Sim::apply_corrector() {
    if (godunov_) throw KsError(KS_ERR_UNSUPPORTED, "ApplyCorrector is the MOL corrector; the Godunov path completes in ApplyPredictor");
    const double dt = t_.dt[0];
    double* fl[9];
    for (int m = 0; m < 9; ++m) fl[m] = static_cast<double*>(gb_.flux[m / 3][m % 3]);
    double* mac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_mol_extrap(ctx_, g_, vel_.p, mac);
    mac_project();
    const double* cmac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    if (temp_) {  // conv_term(New) of the scalar from the predicted temperature
        double* tfl[3] = {fl[0], fl[3], fl[6]};
        launch_mol_scalar_advection(ctx_, g_, theta_.p, cmac, rho_, tfl, tconv_.p);
    }
    // mu_eff(New) and the wall data from the predicted velocity (it is read before the corrector overwrites it)
    launch_smagorinsky(ctx_, g_, vel_.p, mueff_.p, S_, alpha_.p);
    if (wallmodel_) launch_wall_grad(ctx_, g_, vel_old_.p, mueff_.p, wg_.p, shear_, utau_ * utau_, um_[0], um_[1], vmag_, rho_);
    if (temp_) temperature_mol(true, dt);
    // sources at New: the Coriolis term reads the predicted velocity, BoussinesqBuoyancy theta at n+1/2
    sources(vel_.p, temp_ ? theta_nph_.p : nullptr);
    if (diff_type_ != 0) {
        // corrector_rhs with ofac 1/2 (Crank-Nicolson) or 0 (implicit) and nfac 0, fused into the
        // divergence of the fluxes, then the solve with mu_eff(New) (incflo_advance.cpp:620-640)
        launch_mol_advection(ctx_, g_, vel_.p, cmac, rho_, fl, conv_.p, 2, vel_old_.p, src_.p, divtau_.p, conv_old_.p, vel_tmp_.p, dt,
                             diff_type_ == 1 ? 0.5 : 0.0);
        std::swap(vel_.p, vel_tmp_.p);
        diffuse_solve(diff_type_ == 2 ? dt : 0.5 * dt);
        apply_projection(t_.next, dt, false);
        return;
    }
    launch_mol_advection(ctx_, g_, vel_.p, cmac, rho_, fl, conv_.p, 0, nullptr, nullptr, nullptr, nullptr, nullptr, dt, 0.0);
    launch_divtau_corrector(ctx_, g_, vel_.p, mueff_.p, wg_.p, vel_tmp_.p, vel_old_.p, conv_old_.p, conv_.p, divtau_.p, src_.p, dt, rho_);
    std::swap(vel_.p, vel_tmp_.p);
    apply_projection(t_.next, dt, false);
}

void Sim::prepare_time_step() {
    launch_copy(ctx_, vel_old_.p, vel_.p, 3 * g_.N);
    if (temp_) launch_copy(ctx_, theta_old_.p, theta_.p, g_.N);
}

void Sim::pre_advance() {
    t_.next = t_.cur + t_.dt[0];
    abl_update();
    abl_forcing_update();
    actuator_update();
}

// ---------------------------------------------------------------- temperature
// The scalar part of ApplyPredictor (incflo_advance.cpp:296-341) after the MAC
// projection: Godunov fluxes of rho theta with the forces src + diff (no
// temperature sources), predictor_rhs, the explicit RK2 correction or the
// diffusion solve, theta_nph = (theta_old + theta) / 2 for the buoyancy.
void Sim::temperature_predictor(double dt) {
    const long long N = g_.N;
    const double* cmac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    launch_scalar_advection(ctx_, g_, theta_old_.p, tdiff_.p, cmac, dt, rho_, gb_, tconv_.p);
    launch_scalar_pred(ctx_, N, theta_old_.p, tconv_.p, tdiff_.p, theta_.p, dt, rho_, diff_fac());
    if (diff_type_ == 0) {  // explicit RK2 correction with the same wall data
        launch_tdiff(ctx_, g_, theta_.p, alpha_.p, tbc(), ttmp_.p, 2, theta_.p, tdiff_.p, nullptr, nullptr, nullptr, dt, rho_, 0.0);
        std::swap(theta_.p, ttmp_.p);
    } else {
        tdiffuse_solve(diff_type_ == 2 ? dt : 0.5 * dt);
    }
    launch_lincomb(ctx_, N, 0.5, theta_old_.p, 0.5, theta_.p, theta_nph_.p);
}

// The scalar parts of the MOL ApplyPredictor / ApplyCorrector
// (incflo_advance.cpp:296-341, 555-600): predictor — conv_term(Old) of rho theta
// and predictor_rhs with the diffusion factor; corrector — conv_term(New)
// (formed by the caller), diff_term(New) for explicit diffusion (wall data from
// the Old state and the new alpha_eff), corrector_rhs (1/2, 1/2 explicit; 1/2, 0
// Crank-Nicolson; 0, 0 implicit); then the solve and theta_nph.
void Sim::temperature_mol(bool corrector, double dt) {
    const long long N = g_.N;
    double* fl[3] = {static_cast<double*>(gb_.flux[0][0]), static_cast<double*>(gb_.flux[1][0]), static_cast<double*>(gb_.flux[2][0])};
    const double* cmac[3] = {umac_[0].p, umac_[1].p, umac_[2].p};
    if (!corrector) {
        launch_mol_scalar_advection(ctx_, g_, theta_old_.p, cmac, rho_, fl, tconv_old_.p);
        launch_scalar_pred(ctx_, N, theta_old_.p, tconv_old_.p, tdiff_.p, theta_.p, dt, rho_, diff_fac());
    } else {
        const double ofac = diff_type_ == 2 ? 0.0 : 0.5;
        const double* dnew = nullptr;
        if (tzlo_ == 1)  // the new alpha_eff enters the wall gradient
            launch_theta_wall_grad(ctx_, g_, vel_old_.p, theta_old_.p, alpha_.p, tgz_.p, shear_, utau_, kappa_, std::log(zref_ / z0t_), vmag_,
                                   theta_mean_, rho_);
        if (diff_type_ == 0) {
            launch_tdiff(ctx_, g_, theta_.p, alpha_.p, tbc(), ttmp_.p, 0, nullptr, nullptr, nullptr, nullptr, nullptr, dt, rho_, 0.0);
            dnew = ttmp_.p;
        }
        launch_scalar_corr(ctx_, N, theta_old_.p, tconv_old_.p, tconv_.p, tdiff_.p, dnew, tb_.p, dt, rho_, ofac, diff_type_ == 0 ? 0.5 : 0.0);
        std::swap(theta_.p, tb_.p);
    }
    if (diff_type_ != 0) tdiffuse_solve(diff_type_ == 2 ? dt : 0.5 * dt);
    launch_lincomb(ctx_, N, 0.5, theta_old_.p, 0.5, theta_.p, theta_nph_.p);
}

// rho theta - dtd div(alpha grad theta) = rho theta_rhs (MLABecLaplacian solve,
// DiffusionOps.cpp:114-159) by unweighted Jacobi sweeps, one scalar stencil pass
// each with the residual of the incoming iterate; D^-1 A has its spectrum in
// [1 - s, 1 + s], s = max(1 - rho / D) < 1, so every sweep contracts the error
// by s.  MLMG's stopping target on max(|rhs|, initial residual).
void Sim::tdiffuse_solve(double dtd) {
    const int np = tdiff_blocks(g_);
    launch_scalar_rhs(ctx_, g_, theta_.p, rho_, tb_.p, tparts_.p);
    launch_reduce(ctx_, tparts_.p, np, 1, 1, red_.p);
    launch_tdiff_dinv(ctx_, g_, alpha_.p, tbc(), rho_, dtd, tdinv_.p, nullptr);
    ck(cudaMemcpyAsync(hred_, red_.p, sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
    sync();
    const double bnorm = hred_[0];
    int it = 0;
    double r0 = 0.0, rn = 0.0, target = 0.0;
    while (true) {
        launch_tdiff(ctx_, g_, theta_.p, alpha_.p, tbc(), ttmp_.p, 7, nullptr, nullptr, tb_.p, tdinv_.p, tparts_.p, dtd, rho_, 1.0);
        std::swap(theta_.p, ttmp_.p);
        launch_reduce(ctx_, tparts_.p, np, 1, 1, red_.p);
        ck(cudaMemcpyAsync(hred_, red_.p, sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "D2H");
        sync();
        rn = hred_[0];
        if (it == 0) {
            r0 = rn;
            target = std::max(tdif_.atol, tdif_.rtol * std::max(bnorm, r0));
        }
        if (!std::isfinite(rn)) throw KsError(KS_ERR_NONFINITE, "temperature diffusion solve diverged");
        if (rn <= target || it >= tdif_.maxiter) break;
        ++it;
    }
    if (rn > target && !tdif_.fixed_iters) throw KsError(KS_ERR_NOT_CONVERGED, "temperature diffusion solve did not converge");
    tdif_it_ = it;
}

void Sim::init_data() {
    mac_prev_ok_ = false;
    if (!restart_file_.empty()) {  // restart: fields from the checkpoint, no initial projection or iterations
        read_checkpoint(restart_file_);
        plot_start_ = chk_start_ = t_.step;  // SimTime::set_restart_time
        abl_update();
        sync();
        return;
    }
    abl_update();
    if (initial_proj_) {
        apply_projection(t_.cur, 1.0, false);
        launch_fill(ctx_, p_.p, 0.0, (long long)p_.n);
        launch_fill(ctx_, gp_.p, 0.0, 3 * g_.N);
    }
    if (initial_iters_ > 0) {
        compute_dt();
        prepare_time_step();
        for (int it = 0; it < initial_iters_; ++it) {
            apply_predictor(true);
            launch_copy(ctx_, vel_.p, vel_old_.p, 3 * g_.N);
            if (temp_) launch_copy(ctx_, theta_.p, theta_old_.p, g_.N);
        }
    }
    sync();
}

int Sim::step() {
    if (!t_.new_step()) return KS_DONE;
    compute_dt();
    pre_advance();
    prepare_time_step();
    apply_predictor(false);
    if (!godunov_) apply_corrector();  // incflo::advance (src/incflo_advance.cpp:63-79)
    return KS_OK;
}

// ---------------------------------------------------------------- field access
// kind: 0 cell, 1 node, 2/3/4 x/y/z face, 5 bottom-wall plane (nx x ny)
double* Sim::field(const std::string& name, int& nc, int& kind) {
    kind = 0;
    nc = 3;
    if (name == "wall_grad") {  // wall-model gradient of u, v at z-lo (read-only)
        if (!wallmodel_) throw KsError(KS_ERR_ARG, "wall_grad needs zlo.type = wall_model");
        nc = 2;
        kind = 5;
        return wg_.p;
    }
    if (name == "velocity") return vel_.p;
    if (name == "velocity_old") return vel_old_.p;
    if (name == "gp") return gp_.p;
    if (name == "src_term") return src_.p;
    if (name == "forces") return forces_.p;
    if (name == "diff_term") return divtau_.p;
    if (name == "conv_term") return conv_.p;
    if (name == "conv_term_old" && !godunov_) return conv_old_.p;
    if (temp_ && name.rfind("temperature", 0) == 0) {
        nc = 1;
        if (name == "temperature") return theta_.p;
        if (name == "temperature_old") return theta_old_.p;
        if (name == "temperature_mueff") return alpha_.p;
        if (name == "temperature_conv_term") return tconv_.p;
        if (name == "temperature_diff_term") return tdiff_.p;
    }
    if (name == "velocity_adjoint" || name == "gp_adjoint") {
        adj_alloc();
        return name == "velocity_adjoint" ? adj_->ub.p : adj_->gpb.p;
    }
    if (name == "actuator_src_term") { if (!S_.act) throw KsError(KS_ERR_ARG, "no actuator source"); return act_.p; }
    nc = 1;
    if (name == "velocity_mueff") return mueff_.p;
    if (name == "p") { kind = 1; return p_.p; }
    if (name == "u_mac") { kind = 2; return umac_[0].p; }
    if (name == "v_mac") { kind = 3; return umac_[1].p; }
    if (name == "w_mac") { kind = 4; return umac_[2].p; }
    throw KsError(KS_ERR_ARG, "unknown field " + name);
}

void Sim::layout(const std::string& name, ks_layout& L) {
    int nc, kind;
    field(name, nc, kind);
    L.ncomp = nc;
    L.nx = g_.nx + (kind == 2);
    L.ny = g_.ny + (kind == 3);
    L.nz = kind == 5 ? 1 : g_.nz + (kind == 4) + ((kind == 1 && !g_.zper) ? 1 : 0);
}

void Sim::get(const std::string& name, void* dst, int where) {
    int nc, kind;
    double* f = field(name, nc, kind);
    ks_layout L;
    layout(name, L);
    const size_t out = (size_t)L.ncomp * L.nx * L.ny * L.nz;
    if (kind < 2 || kind == 5) {
        ck(cudaMemcpyAsync(dst, f, out * sizeof(double), where == KS_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx_.stream),
           "get_field");
        sync();
        return;
    }
    // face fields: expand the periodic storage with the duplicate last face
    const size_t stored = (kind == 4) ? (size_t)g_.NFz : (size_t)g_.N;
    std::vector<double> h(stored), o(out);
    ck(cudaMemcpyAsync(h.data(), f, stored * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream), "get_field");
    sync();
    const int d = kind - 2;
    for (int k = 0; k < L.nz; ++k)
        for (int j = 0; j < L.ny; ++j)
            for (int i = 0; i < L.nx; ++i) {
                int a = i % g_.nx, b = j % g_.ny, c = k;
                if (d != 2 || g_.zper) c = k % g_.nz;
                o[((size_t)k * L.ny + j) * L.nx + i] = h[((size_t)c * g_.ny + b) * g_.nx + a];
            }
    if (where == KS_DEVICE) {
        ck(cudaMemcpyAsync(dst, o.data(), out * sizeof(double), cudaMemcpyHostToDevice, ctx_.stream), "get_field");
        sync();
    } else {
        std::memcpy(dst, o.data(), out * sizeof(double));
    }
}

void Sim::set(const std::string& name, const void* src, int where) {
    int nc, kind;
    double* f = field(name, nc, kind);
    if (kind >= 2) throw KsError(KS_ERR_ARG, "face fields and the wall gradient are derived and cannot be set");
    ks_layout L;
    layout(name, L);
    const size_t n = (size_t)L.ncomp * L.nx * L.ny * L.nz;
    ck(cudaMemcpyAsync(f, src, n * sizeof(double), where == KS_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx_.stream),
       "set_field");
    sync();
}

double Sim::scalar(const std::string& n) {
    if (n == "time") return t_.cur;
    if (n == "new_time") return t_.next;
    if (n == "dt") return t_.dt[0];
    if (n == "dt_nm1") return t_.dt[1];
    if (n == "step") return t_.step;
    if (n == "mac_iters") return mac_it_;
    if (n == "nodal_iters") return nod_it_;
    if (n == "mac_levels") return (double)(mac_semi_ ? ccs_ : cc_).size();
    if (n.rfind("mac_level:", 0) == 0) {  // mac_level:l:d, cells of MAC level l in direction d
        const std::vector<CCLevelDev>& M = mac_semi_ ? ccs_ : cc_;
        const size_t c = n.find(':', 10);
        if (c == std::string::npos) throw KsError(KS_ERR_ARG, "scalar " + n);
        const size_t l = (size_t)std::stoul(n.substr(10, c - 10));
        const int d = std::stoi(n.substr(c + 1));
        if (l >= M.size() || d < 0 || d > 2) throw KsError(KS_ERR_ARG, "scalar " + n);
        return d == 0 ? M[l].nx : (d == 1 ? M[l].ny : M[l].nz);
    }
    if (n == "diff_iters") return dif_it_;
    if (n == "diff_res0") return dif_r0_;
    if (n == "diff_res") return dif_r_;
    if (n == "diff_rhs_norm") return dif_b_;
    if (n == "temperature_diff_iters") return tdif_it_;
    if (n == "theta_mean") return theta_mean_;
    if (n == "abl_forcing_x") return S_.ablf_force[0];
    if (n == "abl_forcing_y") return S_.ablf_force[1];
    if (n == "mac_res0") return mac_r0_;
    if (n == "mac_target") return mac_tgt_;    // the last solve's stopping threshold
    if (n == "nodal_target") return nod_tgt_;
    if (n == "mac_res") return mac_r_;
    if (n == "nodal_res0") return nod_r0_;
    if (n == "nodal_res") return nod_r_;
    if (n == "utau") return utau_;
    if (n == "cfl") return t_.cur_cfl;
    if (n == "conv_cfl") return t_.conv_cfl;
    if (n == "diff_cfl") return t_.diff_cfl;
    if (n == "src_cfl") return t_.src_cfl;
    if (n == "density") return rho_;
    if (n == "ncells") return (double)g_.N;
    if (n == "precision") return (double)mixed_;
    if (n == "ke") {
        int np = 0;
        launch_ke(ctx_, g_, vel_.p, rho_, parts_.p, &np);
        return reduce(np, 1, 0, nullptr) / (double)g_.N;
    }
    if (n == "divu" || n == "divu_rel" || n == "mac_divu" || n == "mac_divu_rel") {
        // Post-projection divergence, max-norm (1/s): "divu" is the nodal
        // divergence of the cell velocity (the right-hand side operator of the
        // nodal projection, which is an approximate projection: this is
        // truncation-sized, not zero); "mac_divu" is the divergence of the MAC
        // face velocities (an exact projection: it is the MAC solve's residual).
        // The _rel forms scale by max|u| / min(dx, dy, dz).
        int np = 0;
        if (n[0] == 'm') launch_mac_divmax(ctx_, g_, umac_[0].p, umac_[1].p, umac_[2].p, parts_.p, &np);
        else launch_nodal_divmax(ctx_, g_, vel_.p, parts_.p, &np);
        double m[2];
        reduce(np, 2, 1, m);
        if (n.back() != 'l') return m[0];
        const double hmin = std::min(g_.dx, std::min(g_.dy, g_.dz));
        return m[1] > 0.0 ? m[0] * hmin / m[1] : m[0];
    }
    if (n == "ndisks") return (double)disks_.size();
    if (n == "nodal_omega") return nod_.omega;
    if (n.rfind("adj_", 0) == 0 || n == "objective") return adjoint_stat(n);
    if (n.rfind("disk_ct:", 0) == 0) return disks_.at(std::stoul(n.substr(8))).ct_now;
    if (n.rfind("disk_uinf2:", 0) == 0) return disks_.at(std::stoul(n.substr(11))).uinf2;
    if (n.rfind("disk_normal:", 0) == 0 || n.rfind("disk_sample:", 0) == 0) {  // disk_normal:<disk>:<component>
        const size_t c = n.find(':', 12);
        if (c == std::string::npos) throw KsError(KS_ERR_ARG, "unknown scalar " + n);
        const Disk& d = disks_.at(std::stoul(n.substr(12, c - 12)));
        const int m = std::stoi(n.substr(c + 1));
        if (m < 0 || m > 2) throw KsError(KS_ERR_ARG, "unknown scalar " + n);
        return n[5] == 'n' ? d.normal[m] : d.sample[m];
    }
    throw KsError(KS_ERR_ARG, "unknown scalar " + n);
}

}  // namespace ks

// ---------------------------------------------------------------- C ABI
struct ks_handle {
    std::unique_ptr<ks::Sim> sim;
    std::string err;
};

template <typename F>
static int guarded(ks_handle* h, F&& f) {
    if (!h || !h->sim) return KS_ERR_ARG;
    try {
        const int rc = f(*h->sim);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            h->err = std::string("CUDA: ") + cudaGetErrorString(e);
            return KS_ERR_CUDA;
        }
        return rc;
    } catch (const ks::KsError& e) {
        h->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        h->err = e.what();
        return KS_ERR_DECK;
    }
}

extern "C" {

int ks_create(const char* deck_text, ks_handle** out) {
    if (!deck_text || !out) return KS_ERR_ARG;
    *out = nullptr;
    auto* h = new ks_handle();
    *out = h;
    try {
        h->sim = std::make_unique<ks::Sim>(deck_text);
    } catch (const ks::KsError& e) {
        h->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        h->err = e.what();
        return KS_ERR_DECK;
    }
    return KS_OK;
}

void ks_destroy(ks_handle* h) { delete h; }

const char* ks_last_error(const ks_handle* h) { return h ? h->err.c_str() : "null handle"; }

int ks_init_data(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.init_data(); return 0; }); }

int ks_compute_dt(ks_handle* h, double* dt) {
    return guarded(h, [&](ks::Sim& s) {
        s.compute_dt();
        if (dt) *dt = s.t_.dt[0];
        return 0;
    });
}

int ks_pre_advance(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.pre_advance(); return 0; }); }

int ks_prepare_time_step(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.prepare_time_step(); s.sync(); return 0; }); }

int ks_advance(ks_handle* h, int fpi) {
    return guarded(h, [&](ks::Sim& s) {
        if (fpi != 0) throw ks::KsError(KS_ERR_UNSUPPORTED, "fixed-point iterations > 0");
        s.prepare_time_step();
        s.apply_predictor(false);
        if (!s.godunov()) s.apply_corrector();
        s.sync();
        return 0;
    });
}

int ks_apply_predictor(ks_handle* h, int incremental, int fpi) {
    return guarded(h, [&](ks::Sim& s) {
        if (fpi != 0) throw ks::KsError(KS_ERR_UNSUPPORTED, "fixed-point iterations > 0");
        s.apply_predictor(incremental != 0);
        s.sync();
        return 0;
    });
}

int ks_apply_corrector(ks_handle* h) {
    return guarded(h, [](ks::Sim& s) {
        s.apply_corrector();
        s.sync();
        return 0;
    });
}

int ks_apply_projection(ks_handle* h, double time, double scaling, int incremental) {
    return guarded(h, [&](ks::Sim& s) {
        s.apply_projection(time, scaling, incremental != 0);
        s.sync();
        return 0;
    });
}

int ks_step(ks_handle* h) {
    return guarded(h, [](ks::Sim& s) {
        const int rc = s.step();
        s.sync();
        return rc;
    });
}

int ks_evolve(ks_handle* h, int nsteps) {
    return guarded(h, [&](ks::Sim& s) {
        for (int m = 0; m < nsteps; ++m)
            if (s.step() == KS_DONE) break;
        s.sync();
        return 0;
    });
}

int ks_field_layout(ks_handle* h, const char* name, ks_layout* L) {
    if (!name || !L) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.layout(name, *L); return 0; });
}

int ks_get_field(ks_handle* h, const char* name, void* dst, ks_memory where) {
    if (!name || !dst) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.get(name, dst, (int)where); return 0; });
}

int ks_set_field(ks_handle* h, const char* name, const void* src, ks_memory where) {
    if (!name || !src) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.set(name, src, (int)where); return 0; });
}

int ks_get_scalar(ks_handle* h, const char* name, double* v) {
    if (!name || !v) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { *v = s.scalar(name); return 0; });
}

int ks_last_solver_stats(const ks_handle* h, ks_mg_stats* st) {
    if (!h || !h->sim || !st) return KS_ERR_ARG;
    const ks::Sim& s = *h->sim;
    st->mac_iterations = s.mac_it_;
    st->mac_initial_residual = s.mac_r0_;
    st->mac_final_residual = s.mac_r_;
    st->nodal_iterations = s.nod_it_;
    st->nodal_initial_residual = s.nod_r0_;
    st->nodal_final_residual = s.nod_r_;
    return KS_OK;
}

int ks_set_precision(ks_handle* h, int precision) {
    if (precision != KS_FP64 && precision != KS_MIXED) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) {
        s.set_mixed(precision == KS_MIXED);
        return 0;
    });
}

int ks_synchronize(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.sync(); return 0; }); }

int ks_get_stream(ks_handle* h, void** stream) {
    if (!h || !h->sim || !stream) return KS_ERR_ARG;
    *stream = (void*)h->sim->ctx_.stream;
    return KS_OK;
}

int ks_profile_kernels(ks_handle* h, const char* kernel) {
    return guarded(h, [&](ks::Sim& s) {
        s.sync();
        s.ctx_.prof_collect();
        s.ctx_.acc.clear();
        s.ctx_.prof = kernel ? kernel : "";
        return 0;
    });
}

long long ks_profile_report(ks_handle* h, char* buf, long long len) {
    if (!h || !h->sim) return -KS_ERR_ARG;
    ks::Sim& s = *h->sim;
    try {
        s.sync();
    } catch (const std::exception& e) {
        h->err = e.what();
        return -KS_ERR_CUDA;
    }
    s.ctx_.prof_collect();
    std::string out;
    char line[256];
    for (auto& kv : s.ctx_.acc) {
        std::string name;
        for (char ch : kv.first)
            if (ch != ' ') name += ch;
        std::snprintf(line, sizeof(line), "%s %lld %.6f %.0f\n", name.c_str(), kv.second.launches, kv.second.ms, kv.second.bytes);
        out += line;
    }
    const long long need = (long long)out.size() + 1;
    if (buf && len >= need) {
        std::memcpy(buf, out.c_str(), (size_t)need);
        s.ctx_.acc.clear();
    }
    return need;
}

int ks_set_objective_box(ks_handle* h, const double lo[3], const double hi[3]) {
    if (!lo || !hi) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.set_objective_box(lo, hi); return 0; });
}

int ks_objective(ks_handle* h, int seed, double* J) {
    return guarded(h, [&](ks::Sim& s) {
        const double v = s.objective(seed != 0);
        if (J) *J = v;
        return 0;
    });
}

int ks_adjoint_step(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.adjoint_step(); return 0; }); }

int ks_adjoint_run(ks_handle* h, int nsteps, int snapshots, double* J) {
    return guarded(h, [&](ks::Sim& s) {
        const double v = s.adjoint_run(nsteps, snapshots);
        if (J) *J = v;
        return 0;
    });
}

int ks_get_ct_gradient(ks_handle* h, double* grad, int n) {
    if (!grad) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) {
        if (n != s.ndisks()) throw ks::KsError(KS_ERR_ARG, "ks_get_ct_gradient: n differs from the number of disks");
        const auto& g = s.ct_gradient();
        for (int m = 0; m < n; ++m) grad[m] = m < (int)g.size() ? g[m] : 0.0;
        return 0;
    });
}

int ks_adjoint_reset(ks_handle* h) { return guarded(h, [](ks::Sim& s) { s.adjoint_reset(); return 0; }); }

int ks_set_disk_ct(ks_handle* h, const double* ct, int n) {
    if (!ct) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.set_disk_ct(ct, n); return 0; });
}

int ks_checkpoint_cost(int nsteps, int snapshots, long long* forward_steps) {
    if (!forward_steps || nsteps < 1 || snapshots < 1 || nsteps > 100000) return KS_ERR_ARG;
    try {
        *forward_steps = ks::checkpoint_cost(nsteps, snapshots);
    } catch (const std::exception&) {
        return KS_ERR_OOM;
    }
    return KS_OK;
}

int ks_write_plotfile(ks_handle* h, const char* path) {
    if (!path) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.write_plotfile(path); return 0; });
}

int ks_write_checkpoint(ks_handle* h, const char* path) {
    if (!path) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.write_checkpoint(path); return 0; });
}

int ks_read_checkpoint(ks_handle* h, const char* path) {
    if (!path) return KS_ERR_ARG;
    return guarded(h, [&](ks::Sim& s) { s.read_checkpoint(path); return 0; });
}

int ks_write_outputs(ks_handle* h, int last) {
    return guarded(h, [&](ks::Sim& s) { s.write_outputs(last != 0); return 0; });
}

int ks_plotfile_write_host(const char* path, int nvars, const char* const* names, const int n[3], const double prob_lo[3],
                           const double prob_hi[3], double time, int step, const double* data) {
    if (!path || nvars < 1 || !names || !n || !prob_lo || !prob_hi || !data) return KS_ERR_ARG;
    try {
        std::vector<std::string> nm(names, names + nvars);
        ks::write_plotfile_host(path, nm, n, prob_lo, prob_hi, time, step, data, "");
        return KS_OK;
    } catch (const ks::KsError& e) {
        return e.code;
    } catch (const std::exception&) {
        return KS_ERR_ARG;
    }
}

int ks_kernel_launches(const ks_handle* h, long long* count) {
    if (!h || !h->sim || !count) return KS_ERR_ARG;
    *count = h->sim->ctx_.launches;
    return KS_OK;
}

}  // extern "C"
