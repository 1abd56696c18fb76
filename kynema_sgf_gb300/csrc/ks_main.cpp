// Deck-compatible driver executable over the C ABI (the counterpart of the
// reference's src/main.cpp: `exe <input_file> [key=value ...]`, InitData, then
// the Evolve loop with its per-step console lines and the plot / checkpoint
// files of time.plot_interval / time.checkpoint_interval; io.restart_file
// restarts from a checkpoint).  Command-line key=value
// pairs override the input file, as ParmParse does.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/ks.h"

namespace {

void usage(FILE* f, const char* exe) {
    std::fprintf(f,
                 "Usage: %s <input_file> [param=value] [param=value] ...\n\n"
                 "  Runs the single-level incompressible advance of the input deck on the\n"
                 "  current CUDA device: InitData, then Evolve until time.max_step or\n"
                 "  time.stop_time.  param=value pairs override the deck.\n\n"
                 "Optional arguments:\n"
                 "  -h, --help   print this message and exit\n",
                 exe);
}

void solver_table(const ks_mg_stats& s) {
    std::printf("  %-26s%6s%22s%22s\n", "Solver", "Iters", "Initial residual", "Final residual");
    std::printf("  ----------------------------------------------------------------------------\n");
    std::printf("  %-26s%6d%22.6e%22.6e\n", "MAC_projection", s.mac_iterations, s.mac_initial_residual, s.mac_final_residual);
    std::printf("  %-26s%6d%22.6e%22.6e\n", "Nodal_projection", s.nodal_iterations, s.nodal_initial_residual, s.nodal_final_residual);
}

int fail(ks_handle* h, int rc) {
    std::fprintf(stderr, "ERROR: status %d: %s\n", rc, ks_last_error(h));
    ks_destroy(h);
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        usage(stdout, argv[0]);
        std::fprintf(stderr, "ERROR: No input file provided. Exiting!!\n");
        return 1;
    }
    for (int i = 1; i < argc; ++i)
        if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) {
            usage(stdout, argv[0]);
            return 0;
        }
    std::ifstream in(argv[1]);
    if (!in) {
        usage(stdout, argv[0]);
        std::fprintf(stderr, "ERROR: Input file does not exist = %s. Exiting!!\n", argv[1]);
        return 1;
    }
    std::stringstream deck;
    deck << in.rdbuf() << "\n";
    for (int i = 2; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) {
            std::fprintf(stderr, "ERROR: argument '%s' is not param=value\n", argv[i]);
            return 1;
        }
        deck << std::string(argv[i], eq - argv[i]) << " = " << (eq + 1) << "\n";
    }

    ks_handle* h = nullptr;
    int rc = ks_create(deck.str().c_str(), &h);
    if (rc != KS_OK) return fail(h, rc);
    rc = ks_init_data(h);
    if (rc != KS_OK) return fail(h, rc);
    rc = ks_write_outputs(h, 0);  // plot / checkpoint files of step 0 (incflo.cpp:203-208)
    if (rc != KS_OK) return fail(h, rc);
    double ncells = 0.0;
    ks_get_scalar(h, "ncells", &ncells);
    std::printf("\nBegin simulation: %.0f cells\n", ncells);
    std::printf("==============================================================================\n");
    while (true) {
        rc = ks_step(h);
        if (rc == KS_DONE) break;
        if (rc != KS_OK) return fail(h, rc);
        double step = 0, dt = 0, t0 = 0, t1 = 0, cfl = 0, conv = 0, diff = 0, src = 0;
        ks_get_scalar(h, "step", &step);
        ks_get_scalar(h, "dt", &dt);
        ks_get_scalar(h, "time", &t0);
        ks_get_scalar(h, "new_time", &t1);
        ks_get_scalar(h, "cfl", &cfl);
        ks_get_scalar(h, "conv_cfl", &conv);
        ks_get_scalar(h, "diff_cfl", &diff);
        ks_get_scalar(h, "src_cfl", &src);
        std::printf("\nStep: %.0f dt: %.6g Time: %.6g to %.6g\n", step, dt, t0, t1);
        std::printf("CFL: %.6g (conv: %.6g diff: %.6g src: %.6g )\n", cfl, conv, diff, src);
        ks_mg_stats st{};
        ks_last_solver_stats(h, &st);
        solver_table(st);
        rc = ks_write_outputs(h, 0);  // post_advance_work (incflo.cpp:321-327)
        if (rc != KS_OK) return fail(h, rc);
    }
    rc = ks_write_outputs(h, 1);  // write_last_plot_file / write_last_checkpoint (incflo.cpp:404-409)
    if (rc != KS_OK) return fail(h, rc);
    std::printf("\n==============================================================================\n");
    std::printf("Time stepping finished.\n");
    ks_destroy(h);
    return 0;
}
