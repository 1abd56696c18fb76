// AMReX-format plot files and the checkpoint / restart files of the reference
// (src/utilities/IOManager.cpp:34-330, src/utilities/io.cpp:11-220): host code
// over device-to-host copies of the handle's fields.
//
// Plot file (amrex::WriteMultiLevelPlotfile, single level, one box): the
// directory holds Header (HyperCLaw-V1.1 text header), kynema_sgf_info and
// Level_0/Cell_H (the VisMF header) with Level_0/Cell_D_00000 (one FAB: a
// text line naming the IEEE-754 little-endian double layout and the box,
// then the values component by component, x fastest).  Checkpoint: Header
// (version line, finest level, step, time, dt, dt_nm1, dt_nm2, prob_lo,
// prob_hi, the BoxArray) and one VisMF MultiFab per restart field with the
// reference's ghost widths.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

#include "ks_sim.hpp"

namespace ks {

namespace {

void make_dir(const std::string& d) {
    if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) throw KsError(KS_ERR_ARG, "cannot create directory " + d);
}

std::string box_str(const int lo[3], const int hi[3], int type) {
    std::ostringstream o;
    o << "((" << lo[0] << ',' << lo[1] << ',' << lo[2] << ") (" << hi[0] << ',' << hi[1] << ',' << hi[2] << ") (" << type << ',' << type << ','
      << type << "))";
    return o.str();
}

// IEEE double, little-endian byte order (amrex::FPC descriptor of x86-64 and aarch64)
const char* kRealDesc = "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))";

// One VisMF MultiFab of a single FAB: <prefix>_H and <prefix>_D_00000.  `data`
// covers the grown box [lo - ngrow, hi + ngrow] (hi already nodal when type
// is 1), component-major, x fastest; min / max are taken over the valid box.
void write_vismf(const std::string& prefix, int ncomp, int ngrow, int type, const int hi[3], const std::vector<double>& data) {
    const int lo[3] = {0, 0, 0};
    const int glo[3] = {-ngrow, -ngrow, -ngrow}, ghi[3] = {hi[0] + ngrow, hi[1] + ngrow, hi[2] + ngrow};
    const long long gx = ghi[0] - glo[0] + 1, gy = ghi[1] - glo[1] + 1, gz = ghi[2] - glo[2] + 1, gn = gx * gy * gz;
    const std::string base = prefix.substr(prefix.find_last_of('/') + 1);
    std::ofstream d(prefix + "_D_00000", std::ios::binary | std::ios::trunc);
    if (!d) throw KsError(KS_ERR_ARG, "cannot write " + prefix + "_D_00000");
    d << "FAB " << kRealDesc << box_str(glo, ghi, type) << ' ' << ncomp << '\n';
    d.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)(data.size() * sizeof(double)));
    if (!d) throw KsError(KS_ERR_ARG, "write failed: " + prefix + "_D_00000");
    std::vector<double> mn(ncomp), mx(ncomp);
    for (int n = 0; n < ncomp; ++n) {
        double a = 1e300, b = -1e300;
        for (int k = 0; k <= hi[2]; ++k)
            for (int j = 0; j <= hi[1]; ++j)
                for (int i = 0; i <= hi[0]; ++i) {
                    const double v = data[(size_t)(n * gn + ((k + ngrow) * gy + (j + ngrow)) * gx + (i + ngrow))];
                    a = std::min(a, v);
                    b = std::max(b, v);
                }
        mn[n] = a;
        mx[n] = b;
    }
    std::ofstream h(prefix + "_H", std::ios::trunc);
    if (!h) throw KsError(KS_ERR_ARG, "cannot write " + prefix + "_H");
    h << std::setprecision(17);
    h << 1 << '\n' << 1 << '\n' << ncomp << '\n' << ngrow << '\n';
    h << "(1 0\n" << box_str(lo, hi, type) << "\n)\n";
    h << 1 << '\n' << "FabOnDisk: " << base << "_D_00000 0\n\n";
    h << 1 << ',' << ncomp << '\n';
    for (int n = 0; n < ncomp; ++n) h << mn[n] << ',';
    h << "\n\n" << 1 << ',' << ncomp << '\n';
    for (int n = 0; n < ncomp; ++n) h << mx[n] << ',';
    h << "\n";
}

// Valid region [0, n) of a VisMF MultiFab written by write_vismf (or by
// AMReX with one FAB): reads the grown FAB and returns the valid values.
std::vector<double> read_vismf(const std::string& prefix, int ncomp_expect, const int n[3]) {
    std::ifstream h(prefix + "_H");
    if (!h) throw KsError(KS_ERR_ARG, "missing " + prefix + "_H");
    int vers = 0, how = 0, ncomp = 0, ngrow = 0;
    h >> vers >> how >> ncomp >> ngrow;
    if (ncomp != ncomp_expect) throw KsError(KS_ERR_DECK, prefix + ": component count differs");
    std::ifstream d(prefix + "_D_00000", std::ios::binary);
    if (!d) throw KsError(KS_ERR_ARG, "missing " + prefix + "_D_00000");
    std::string line;
    std::getline(d, line);
    if (line.compare(0, 4, "FAB ") != 0 || line.find("(8 7 6 5 4 3 2 1)") == std::string::npos)
        throw KsError(KS_ERR_DECK, prefix + ": not a little-endian FP64 FAB");
    // box of the FAB: the second parenthesised triple list after the descriptor
    const size_t bpos = line.find(")))") + 3;
    int lo[3], hi[3], ty[3], nc2;
    if (std::sscanf(line.c_str() + bpos, "((%d,%d,%d) (%d,%d,%d) (%d,%d,%d)) %d", &lo[0], &lo[1], &lo[2], &hi[0], &hi[1], &hi[2], &ty[0], &ty[1],
                    &ty[2], &nc2) != 10 || nc2 != ncomp)
        throw KsError(KS_ERR_DECK, prefix + ": FAB header");
    const long long gx = hi[0] - lo[0] + 1, gy = hi[1] - lo[1] + 1, gz = hi[2] - lo[2] + 1;
    std::vector<double> all((size_t)(gx * gy * gz * ncomp));
    d.read(reinterpret_cast<char*>(all.data()), (std::streamsize)(all.size() * sizeof(double)));
    if (!d) throw KsError(KS_ERR_DECK, prefix + ": short FAB");
    std::vector<double> out((size_t)n[0] * n[1] * n[2] * ncomp);
    for (int c = 0; c < ncomp; ++c)
        for (int k = 0; k < n[2]; ++k)
            for (int j = 0; j < n[1]; ++j)
                for (int i = 0; i < n[0]; ++i) {
                    const long long src = c * gx * gy * gz + ((k - lo[2]) * gy + (j - lo[1])) * gx + (i - lo[0]);
                    out[(size_t)(((c * (long long)n[2] + k) * n[1] + j) * n[0] + i)] = all[(size_t)src];
                }
    return out;
}

// grown copy of a valid-region field (ncomp, dims n) with ghosts filled by
// periodic wrap or, across a bounded z, the nearest valid layer
std::vector<double> grown(const std::vector<double>& v, int ncomp, const int n[3], int ngrow, bool zper) {
    const long long gx = n[0] + 2 * ngrow, gy = n[1] + 2 * ngrow, gz = n[2] + 2 * ngrow;
    std::vector<double> g((size_t)(gx * gy * gz * ncomp));
    auto wrap = [](int i, int m) { return ((i % m) + m) % m; };
    for (int c = 0; c < ncomp; ++c)
        for (long long k = 0; k < gz; ++k)
            for (long long j = 0; j < gy; ++j)
                for (long long i = 0; i < gx; ++i) {
                    const int ii = wrap((int)i - ngrow, n[0]), jj = wrap((int)j - ngrow, n[1]);
                    int kk = (int)k - ngrow;
                    kk = zper ? wrap(kk, n[2]) : std::max(0, std::min(n[2] - 1, kk));
                    g[(size_t)(((c * gz + k) * gy + j) * gx + i)] = v[(size_t)(((c * (long long)n[2] + kk) * n[1] + jj) * n[0] + ii)];
                }
    return g;
}

}  // namespace

void write_plotfile_host(const std::string& dir, const std::vector<std::string>& names, const int n[3], const double plo[3], const double phi[3],
                         double time, int step, const double* data, const std::string& info) {
    const int nv = (int)names.size();
    make_dir(dir);
    make_dir(dir + "/Level_0");
    std::ofstream hd(dir + "/Header", std::ios::trunc);
    if (!hd) throw KsError(KS_ERR_ARG, "cannot write " + dir + "/Header");
    hd << std::setprecision(17);
    hd << "HyperCLaw-V1.1\n" << nv << '\n';
    for (auto& s : names) hd << s << '\n';
    hd << 3 << '\n' << time << '\n' << 0 << '\n';
    for (int d = 0; d < 3; ++d) hd << plo[d] << ' ';
    hd << '\n';
    for (int d = 0; d < 3; ++d) hd << phi[d] << ' ';
    hd << "\n\n";
    const int lo[3] = {0, 0, 0}, hi[3] = {n[0] - 1, n[1] - 1, n[2] - 1};
    hd << box_str(lo, hi, 0) << " \n" << step << " \n";
    for (int d = 0; d < 3; ++d) hd << (phi[d] - plo[d]) / n[d] << ' ';
    hd << '\n' << 0 << '\n' << 0 << '\n';
    hd << 0 << ' ' << 1 << ' ' << time << '\n' << step << '\n';
    for (int d = 0; d < 3; ++d) hd << plo[d] << ' ' << phi[d] << '\n';
    hd << "Level_0/Cell\n";
    const size_t N = (size_t)n[0] * n[1] * n[2];
    write_vismf(dir + "/Level_0/Cell", nv, 0, 0, hi, std::vector<double>(data, data + N * nv));
    std::ofstream in(dir + "/kynema_sgf_info", std::ios::trunc);
    in << info;
}

// ---------------------------------------------------------------- Sim
// Default output variables of the reference (IOManager::initialize_io with the
// fields registered by icns_ops.H:62-68, TurbModelBase.H:95-110, PDEOps.H:52):
// a sorted set of field names, expanded to <name>x/y/z for three components.
std::vector<std::pair<std::string, int>> Sim::plot_fields() const {
    std::vector<std::pair<std::string, int>> f = {{"density", 1}, {"gp", 3}, {"p", 1}, {"velocity", 3}};
    if (S_.smag) {
        f.push_back({"mu_turb", 1});
        f.push_back({"velocity_mueff", 1});
        if (temp_) f.push_back({"temperature_mueff", 1});
    }
    if (temp_) f.push_back({"temperature", 1});
    std::sort(f.begin(), f.end());
    return f;
}

// valid-region host copy of a named output field (cell layout; p takes the
// node at each cell's low corner, as MultiFab::Copy into the cell-centred
// plot MultiFab does)
std::vector<double> Sim::host_field(const std::string& name, int nc) {
    const size_t N = (size_t)g_.N;
    std::vector<double> h(N * nc);
    if (name == "density") {
        std::fill(h.begin(), h.end(), rho_);
    } else if (name == "p") {
        ks_layout L;
        layout("p", L);
        std::vector<double> pn((size_t)L.nx * L.ny * L.nz);
        get("p", pn.data(), 0);
        for (int k = 0; k < g_.nz; ++k)
            for (int j = 0; j < g_.ny; ++j)
                for (int i = 0; i < g_.nx; ++i) h[((size_t)k * g_.ny + j) * g_.nx + i] = pn[((size_t)k * L.ny + j) * L.nx + i];
    } else if (name == "mu_turb") {
        get("velocity_mueff", h.data(), 0);
        for (auto& v : h) v -= mu_;
    } else {
        get(name, h.data(), 0);
    }
    return h;
}

std::string Sim::info_text() const {
    std::ostringstream o;
    o << "Kynema-SGF single-level advance, GB300 (sm_103a)\n" << std::string(78, '-') << "\nGrid information: \n";
    o << "  Level: 0\n    num. boxes = 1\n    maximum zones = " << g_.nx << ' ' << g_.ny << ' ' << g_.nz << '\n';
    o << std::string(78, '-') << "\nInput file parameters: \n" << deck_text_;
    return o.str();
}

void Sim::write_plotfile(const std::string& dir) {
    std::vector<std::string> names;
    std::vector<double> all;
    const char* comp[3] = {"x", "y", "z"};
    for (auto& f : plot_fields()) {
        auto h = host_field(f.first, f.second);
        all.insert(all.end(), h.begin(), h.end());
        if (f.second == 1) names.push_back(f.first);
        else
            for (int c = 0; c < 3; ++c) names.push_back(f.first + comp[c]);
    }
    const int n[3] = {g_.nx, g_.ny, g_.nz};
    write_plotfile_host(dir, names, n, plo_, phi_, t_.next > t_.cur ? t_.next : t_.cur, t_.step, all.data(), info_text());
}

// Checkpoint (IOManager::write_checkpoint_file / write_header): the restart
// fields with their ghost widths (velocity, density, temperature 3; p nodal 3;
// gp 0; mu_turb, velocity_mueff 1).
void Sim::write_checkpoint(const std::string& dir) {
    make_dir(dir);
    make_dir(dir + "/Level_0");
    {
        std::ofstream hd(dir + "/Header", std::ios::trunc);
        if (!hd) throw KsError(KS_ERR_ARG, "cannot write " + dir + "/Header");
        hd << std::setprecision(17);
        hd << "Checkpoint version: 1\n" << 0 << '\n' << t_.step << '\n' << (t_.next > t_.cur ? t_.next : t_.cur) << '\n' << t_.dt[0] << '\n'
           << t_.dt[1] << '\n' << t_.dt[2] << '\n';
        for (int d = 0; d < 3; ++d) hd << plo_[d] << ' ';
        hd << '\n';
        for (int d = 0; d < 3; ++d) hd << phi_[d] << ' ';
        hd << '\n';
        const int lo[3] = {0, 0, 0}, hi[3] = {g_.nx - 1, g_.ny - 1, g_.nz - 1};
        hd << "(1 0\n" << box_str(lo, hi, 0) << "\n)\n";
    }
    const int n[3] = {g_.nx, g_.ny, g_.nz};
    const int hi[3] = {g_.nx - 1, g_.ny - 1, g_.nz - 1};
    auto cell = [&](const std::string& name, int nc, int ng) {
        auto h = host_field(name, nc);
        write_vismf(dir + "/Level_0/" + name, nc, ng, 0, hi, grown(h, nc, n, ng, g_.zper));
    };
    cell("density", 1, 3);
    cell("gp", 3, 0);
    cell("velocity", 3, 3);
    if (S_.smag) {
        cell("mu_turb", 1, 1);
        cell("velocity_mueff", 1, 1);
    }
    if (temp_) cell("temperature", 1, 3);
    if (mg_warm_ && mac_prev_ok_) {  // the MAC projection's warm start: a restart continues bit for bit
        std::vector<double> h((size_t)g_.N);
        sync();
        ck(cudaMemcpy(h.data(), mac_phi_prev_.p, sizeof(double) * g_.N, cudaMemcpyDeviceToHost), "D2H");
        write_vismf(dir + "/Level_0/mac_phi", 1, 0, 0, hi, grown(h, 1, n, 0, g_.zper));
    }
    {  // nodal p on the nodes 0..n in every direction (periodic duplicates wrapped)
        ks_layout L;
        layout("p", L);
        std::vector<double> pn((size_t)L.nx * L.ny * L.nz);
        get("p", pn.data(), 0);
        const int ng = 3;
        const int nn[3] = {g_.nx + 1, g_.ny + 1, g_.nz + 1};
        const long long gx = nn[0] + 2 * ng, gy = nn[1] + 2 * ng, gz = nn[2] + 2 * ng;
        std::vector<double> g((size_t)(gx * gy * gz));
        auto wrap = [](int i, int m) { return ((i % m) + m) % m; };
        for (long long k = 0; k < gz; ++k)
            for (long long j = 0; j < gy; ++j)
                for (long long i = 0; i < gx; ++i) {
                    const int ii = wrap((int)i - ng, g_.nx), jj = wrap((int)j - ng, g_.ny);
                    int kk = (int)k - ng;
                    kk = g_.zper ? wrap(kk, g_.nz) : std::max(0, std::min(L.nz - 1, kk));
                    g[(size_t)((k * gy + j) * gx + i)] = pn[((size_t)kk * L.ny + jj) * L.nx + ii];
                }
        const int phi_n[3] = {g_.nx, g_.ny, g_.nz};
        write_vismf(dir + "/Level_0/p", 1, ng, 1, phi_n, g);
    }
    std::ofstream in(dir + "/kynema_sgf_info", std::ios::trunc);
    in << info_text();
}

// Restart (incflo::ReadCheckpointFile, io.cpp:11-220, and
// IOManager::read_checkpoint_fields): step, time and dt history from the
// header; the fields from their MultiFabs; a domain that is an integer multiple
// of the checkpoint's replicates it.
void Sim::read_checkpoint(const std::string& dir) {
    std::ifstream hd(dir + "/Header");
    if (!hd) throw KsError(KS_ERR_ARG, "cannot read " + dir + "/Header");
    std::string line;
    std::getline(hd, line);
    int finest = 0, step = 0;
    double time = 0, dt0 = 0, dt1 = 0, dt2 = 0, lo[3], hi[3];
    hd >> finest >> step >> time >> dt0 >> dt1 >> dt2 >> lo[0] >> lo[1] >> lo[2] >> hi[0] >> hi[1] >> hi[2];
    if (!hd || finest != 0) throw KsError(KS_ERR_DECK, "checkpoint header: single-level checkpoints only");
    std::getline(hd, line);
    std::getline(hd, line);  // "(1 0"
    std::getline(hd, line);  // the box
    int b0[3], b1[3], ty[3];
    if (std::sscanf(line.c_str(), "((%d,%d,%d) (%d,%d,%d) (%d,%d,%d))", &b0[0], &b0[1], &b0[2], &b1[0], &b1[1], &b1[2], &ty[0], &ty[1], &ty[2]) != 9)
        throw KsError(KS_ERR_DECK, "checkpoint header: box");
    const int cn[3] = {b1[0] - b0[0] + 1, b1[1] - b0[1] + 1, b1[2] - b0[2] + 1};
    const int n[3] = {g_.nx, g_.ny, g_.nz};
    int rep[3];
    for (int d = 0; d < 3; ++d) {
        const double ratio = (phi_[d] - plo_[d]) / (hi[d] - lo[d]);
        rep[d] = (int)ratio;
        if (std::fabs(rep[d] - ratio) > 1e-6 || rep[d] < 1 || cn[d] * rep[d] != n[d])
            throw KsError(KS_ERR_DECK, "checkpoint domain does not tile the deck's domain (amr.n_cell, geometry.prob_lo/hi)");
    }
    if (rep[2] != 1 && !g_.zper) throw KsError(KS_ERR_DECK, "replication along a bounded z");
    // a cell field of the checkpoint tiled over the deck's domain (empty: absent)
    auto tiled = [&](const std::string& name, int nc, bool required) {
        std::vector<double> full;
        std::ifstream probe(dir + "/Level_0/" + name + "_H");
        if (!probe) {
            if (required) throw KsError(KS_ERR_ARG, "checkpoint lacks " + name);
            return full;
        }
        auto v = read_vismf(dir + "/Level_0/" + name, nc, cn);
        full.resize((size_t)g_.N * nc);
        for (int c = 0; c < nc; ++c)
            for (int k = 0; k < n[2]; ++k)
                for (int j = 0; j < n[1]; ++j)
                    for (int i = 0; i < n[0]; ++i)
                        full[(((size_t)c * n[2] + k) * n[1] + j) * n[0] + i] =
                            v[(((size_t)c * cn[2] + k % cn[2]) * cn[1] + j % cn[1]) * cn[0] + i % cn[0]];
        return full;
    };
    auto load = [&](const std::string& name, int nc) { set(name, tiled(name, nc, true).data(), 0); };
    load("velocity", 3);
    load("gp", 3);
    if (temp_) load("temperature", 1);
    // the MAC projection's warm start (written by this implementation only)
    mac_prev_ok_ = false;
    if (mg_warm_) {
        auto m = tiled("mac_phi", 1, false);
        if (!m.empty()) {
            if (mac_phi_prev_.n != (size_t)g_.N) mac_phi_prev_.alloc(g_.N);
            ck(cudaMemcpy(mac_phi_prev_.p, m.data(), sizeof(double) * g_.N, cudaMemcpyHostToDevice), "H2D");
            mac_prev_ok_ = true;
        }
    }
    {  // nodal p: nodes 0..n of the checkpoint, stored without periodic duplicates
        const int nn[3] = {cn[0] + 1, cn[1] + 1, cn[2] + 1};
        auto pv = read_vismf(dir + "/Level_0/p", 1, nn);
        ks_layout L;
        layout("p", L);
        std::vector<double> pn((size_t)L.nx * L.ny * L.nz);
        for (int k = 0; k < L.nz; ++k)
            for (int j = 0; j < L.ny; ++j)
                for (int i = 0; i < L.nx; ++i) {
                    const int kk = (g_.zper ? k % cn[2] : k);
                    pn[((size_t)k * L.ny + j) * L.nx + i] = pv[((size_t)kk * nn[1] + j % cn[1]) * nn[0] + i % cn[0]];
                }
        set("p", pn.data(), 0);
    }
    t_.step = step;
    t_.cur = time;
    t_.next = time;
    (void)dt0;  // read but not applied, as in the reference: the next compute_dt starts afresh
    t_.dt[1] = dt1;
    t_.dt[2] = dt2;
    sync();
}

static std::string concat(const std::string& root, int num) {  // amrex::Concatenate, 5 digits
    std::ostringstream o;
    o << root << std::setfill('0') << std::setw(5) << num;
    return o.str();
}

void Sim::write_outputs(bool last) {
    auto due = [&](int interval, int start) {
        if (interval <= 0) return false;
        const int r = (t_.step - start) % interval;
        return last ? r != 0 : r == 0;
    };
    if (due(plot_interval_, plot_start_)) write_plotfile(concat(plt_prefix_, t_.step));
    if (due(chk_interval_, chk_start_)) write_checkpoint(concat(chk_prefix_, t_.step));
}

}  // namespace ks
