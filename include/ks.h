/*
 * ks.h -- C ABI of the GB300-native single-level incompressible advance.
 *
 * One handle owns one uniform single-box grid, its device fields and one CUDA
 * stream.  Calls on a handle are single-threaded (the handle is not
 * re-entrant); different handles are independent.  No C++ exception crosses
 * this boundary: every entry point returns a ks_status (0 on success).
 *
 * Each entry point replaces one member of the reference's incflo operator
 * surface (paths inside the Kynema-SGF repository):
 *   ks_create / ks_destroy     incflo::incflo(), ReadParameters, init_mesh     src/incflo.cpp:43-61, src/setup/init.cpp:48-96
 *   ks_init_data               incflo::InitData (initial projection + pressure iterations)  src/incflo.cpp:218-228, src/setup/init.cpp:104-225
 *   ks_compute_dt              incflo::compute_dt + SimTime::set_current_cfl  src/incflo_compute_dt.cpp:33-221, src/core/SimTime.cpp:162-291
 *   ks_pre_advance             pre_advance_stage1 + pre_advance_stage2 (ABL, actuators)  src/incflo_advance.cpp:15-32
 *   ks_prepare_time_step       incflo::prepare_time_step (New -> Old)          src/incflo_advance.cpp:34-44
 *   ks_advance                 incflo::advance(fixed_point_iteration)          src/incflo_advance.cpp:63-79
 *   ks_apply_predictor         incflo::ApplyPredictor                          src/incflo_advance.cpp:186-438
 *   ks_apply_corrector         incflo::ApplyCorrector (MOL: incflo.use_godunov = false)  src/incflo_advance.cpp:528-652
 *   ks_apply_projection        incflo::ApplyProjection                         src/projection/incflo_apply_nodal_projection.cpp:149-465
 *   ks_evolve                  incflo::Evolve time loop                        src/incflo.cpp:338-411
 *   ks_set_field / ks_get_field  FieldRepo field access by name              src/core/FieldRepo.H:139-173
 *   ks_last_solver_stats       io::print_mlmg_info                            src/utilities/console_io.cpp:178-186
 *   ks_write_plotfile / ks_write_checkpoint / ks_write_outputs  IOManager      src/utilities/IOManager.cpp:135-330
 *   ks_read_checkpoint         incflo::ReadCheckpointFile                      src/utilities/io.cpp:11-220
 *
 * Deck: ParmParse text ("prefix.key = values" lines), the reference's keys.
 * Field exchange: valid region only, structure of arrays, x fastest, then y,
 * then z, then component (AMReX Array4 order, no ghost cells).  Cell fields
 * hold nx*ny*nz points per component; the node field "p" has one more point
 * along a wall-bounded z; face fields u_mac/v_mac/w_mac have one more point
 * along their normal direction.
 */
#ifndef KS_H
#define KS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ks_status {
    KS_OK = 0,
    KS_ERR_DECK = 1,            /* invalid or missing deck value */
    KS_ERR_UNSUPPORTED = 2,     /* valid reference option outside this path */
    KS_ERR_NOT_CONVERGED = 3,   /* multigrid hit maxiter (only when abort-on-fail is on) */
    KS_ERR_NONFINITE = 4,       /* NaN/Inf detected, or dt below time.min_dt */
    KS_ERR_OOM = 5,             /* device allocation failed */
    KS_ERR_ARG = 6,             /* bad handle, name, pointer or size */
    KS_DONE = 7,                /* time loop finished (max_step / stop_time) */
    KS_ERR_CUDA = 8             /* CUDA runtime error */
} ks_status;

typedef enum ks_precision { KS_FP64 = 0, KS_MIXED = 1 } ks_precision;

typedef enum ks_memory { KS_HOST = 0, KS_DEVICE = 1 } ks_memory;

typedef struct ks_handle ks_handle;

typedef struct ks_mg_stats {
    int mac_iterations;
    double mac_initial_residual;
    double mac_final_residual;
    int nodal_iterations;
    double nodal_initial_residual;
    double nodal_final_residual;
} ks_mg_stats;

typedef struct ks_layout {
    int ncomp;
    int nx, ny, nz;   /* points per component along x, y, z */
} ks_layout;

int ks_create(const char* deck_text, ks_handle** out);
void ks_destroy(ks_handle* h);
const char* ks_last_error(const ks_handle* h);

int ks_init_data(ks_handle* h);
int ks_compute_dt(ks_handle* h, double* dt);
int ks_pre_advance(ks_handle* h);
int ks_prepare_time_step(ks_handle* h);
int ks_advance(ks_handle* h, int fixed_point_iteration);
int ks_apply_predictor(ks_handle* h, int incremental_projection, int fixed_point_iteration);
int ks_apply_corrector(ks_handle* h);
int ks_apply_projection(ks_handle* h, double time, double scaling_factor, int incremental);
int ks_evolve(ks_handle* h, int nsteps);
int ks_step(ks_handle* h);

int ks_field_layout(ks_handle* h, const char* name, ks_layout* layout);
int ks_get_field(ks_handle* h, const char* name, void* dst, ks_memory where);
int ks_set_field(ks_handle* h, const char* name, const void* src, ks_memory where);
int ks_get_scalar(ks_handle* h, const char* name, double* value);
int ks_last_solver_stats(const ks_handle* h, ks_mg_stats* stats);
int ks_set_precision(ks_handle* h, int precision);
int ks_synchronize(ks_handle* h);
int ks_kernel_launches(const ks_handle* h, long long* count);

/* Plot files, checkpoints and restart (IOManager, src/utilities/IOManager.cpp:34-330;
 * incflo::ReadCheckpointFile, src/utilities/io.cpp:11-220).
 * ks_write_plotfile: an AMReX plot file directory (HyperCLaw-V1.1 Header,
 * Level_0/Cell_H + Cell_D_00000) with the reference's default variables
 * (density, gp, p, velocity; mu_turb, velocity_mueff with Smagorinsky;
 * temperature [+ temperature_mueff]) at the current step and time.
 * ks_write_checkpoint / ks_read_checkpoint: the reference's checkpoint layout
 * (Header + one VisMF MultiFab per restart field); reading restores the step,
 * the time, dt_nm1 / dt_nm2 and the fields; a domain that is an integer
 * multiple of the checkpoint's replicates it.  The deck key io.restart_file
 * makes ks_init_data restart instead of initialising.
 * ks_write_outputs: the files due at the current step under time.plot_interval
 * and time.checkpoint_interval (prefixes io.plot_file, io.check_file; last != 0:
 * the end-of-run rules), as incflo::Evolve writes them.
 * ks_plotfile_write_host: the plot file writer on host data only (no device):
 * nvars cell fields of n[0]*n[1]*n[2] values each, component-major, x fastest. */
int ks_write_plotfile(ks_handle* h, const char* path);
int ks_write_checkpoint(ks_handle* h, const char* path);
int ks_read_checkpoint(ks_handle* h, const char* path);
int ks_write_outputs(ks_handle* h, int last);
int ks_plotfile_write_host(const char* path, int nvars, const char* const* names, const int n[3], const double prob_lo[3],
                           const double prob_hi[3], double time, int step, const double* data);

/* Reverse mode of the advance (no counterpart in the reference: the adjoint
 * entry points ks_adjoint_step / ks_set_objective_box / ks_get_ct_gradient
 * extend the operator surface of src/incflo.H:51-233).
 *
 * Differentiable configuration: the Godunov scheme (incflo.use_godunov = 1),
 * time.fixed_dt > 0, periodic z or slip / wall-model walls (wall model with
 * ABL.wall_shear_stress_type = moeng), laminar or Smagorinsky viscosity,
 * momentum sources among ActuatorForcing, BodyForce, CoriolisForcing and
 * GeostrophicForcing, UniformCtDisk actuators with one thrust_coeff value
 * each.  Other decks return KS_ERR_UNSUPPORTED from every call below.
 * The objective J is the mean of 0.5 |u|^2 over the cells whose centres lie in
 * the box [lo, hi] (physical units).  The adjoint state is held in the fields
 * "velocity_adjoint" and "gp_adjoint" (layouts of "velocity" and "gp"; get and
 * set them with ks_get_field / ks_set_field).  Limiter, Riemann and upwind
 * branches are frozen at the forward state; projections are reversed with
 * solves of the same self-adjoint operators at the forward tolerances. */
int ks_set_objective_box(ks_handle* h, const double lo[3], const double hi[3]);
/* J at the current state; seed != 0 also sets the adjoint fields to dJ/du
 * and 0 (the terminal condition of a reverse sweep). */
int ks_objective(ks_handle* h, int seed, double* J);
/* One reverse step at the current state x^n = (velocity, gp): the adjoint
 * fields go from the adjoint of x^{n+1} to that of x^n and dJ/dct
 * accumulates; the forward state and the clock are left at x^n.  The step is
 * recomputed from x^n at the handle's precision (ks_set_precision) and
 * linearised there; the reverse arithmetic is FP64. */
int ks_adjoint_step(ks_handle* h);
/* nsteps forward steps from the current state with binomial checkpointing in
 * device memory (`snapshots` slots of (velocity, gp), the first holding the
 * initial state; snapshots >= nsteps stores every state), J at the final
 * state, and the reverse sweep.  On return: *J set, the forward state and the
 * clock are those after nsteps steps, the adjoint fields hold dJ/d(velocity,
 * gp) of the initial state, and ks_get_ct_gradient returns dJ/dct. */
int ks_adjoint_run(ks_handle* h, int nsteps, int snapshots, double* J);
/* Accumulated dJ/dct per disk (deck order, n = number of disks). */
int ks_get_ct_gradient(ks_handle* h, double* grad, int n);
/* Zero the adjoint fields and the accumulated dJ/dct. */
int ks_adjoint_reset(ks_handle* h);
/* Thrust coefficient of every disk (deck order, n = number of disks). */
int ks_set_disk_ct(ks_handle* h, const double* ct, int n);
/* Forward steps beyond the reverse steps' own that a binomial schedule needs
 * to reverse nsteps steps with `snapshots` slots (host only, no device). */
int ks_checkpoint_cost(int nsteps, int snapshots, long long* forward_steps);

/* Instrumentation (no counterpart in the reference): the CUDA stream all
 * kernels of the handle run on, and CUDA-event timing of kernels whose name
 * matches `kernel` ("*" = every kernel, NULL or "" = off).  The report is
 * "name launches total_ms algorithmic_bytes" lines (bytes: every distinct array
 * each launch reads or writes, counted once); it returns the bytes needed (including the
 * terminating zero) and clears the accumulated totals. */
int ks_get_stream(ks_handle* h, void** stream);
int ks_profile_kernels(ks_handle* h, const char* kernel);
long long ks_profile_report(ks_handle* h, char* buf, long long len);

/* Compute-roofline probe (no counterpart in the reference): FMA throughput
 * in GFLOP/s of the current device for FP64 (fp64 = 1) or FP32 (fp64 = 0),
 * measured with independent in-register FMA chains. */
int ks_fma_peak(int fp64, double* gflops);

/* Allocation-free tensor diffusion term (no counterpart in the reference).
 *
 * For callers that cannot call cudaMalloc where they need the viscous term:
 * hosts whose device memory is reserved up front by another allocator,
 * plug-in code inside an application that owns every device allocation,
 * latency-critical loops that must not trigger an allocation.  Computes divtau = div(mu (grad u + grad u^T) - 2/3 mu div(u) I)
 * for a caller-owned device velocity (3 components, SoA, x fastest), cell
 * viscosity mueff and output divtau (3 components), on stream `stream` (NULL =
 * legacy default stream), with the boundary treatment of the advance: x and y
 * periodic; z periodic or slip walls, or a wall-model bottom whose wall-normal
 * tangential-velocity gradient is given in wall_grad (2 x nx*ny, device).
 * Its face-flux scratch lives in a static device array sized for at most
 * KS_NOALLOC_MAX_CELLS cells (about 24 MB, held by every GPU that loads the
 * library until exit); larger grids are rejected with KS_ERR_ARG.  The first
 * call on a device looks up that array's address with that device current;
 * make that first call before any stream capture.  All calls share the
 * array: calls whose kernels overlap on the GPU race, order them.  A CUDA
 * error already pending on the calling thread is left in place and the call
 * returns KS_ERR_CUDA without launching; calls after cudaDeviceReset are not
 * supported. */
#define KS_NOALLOC_MAX_CELLS 262144
int ks_divtau_noalloc(const double* vel, const double* mueff, const double* wall_grad, double* divtau, int nx, int ny, int nz,
                      double dx, double dy, double dz, int z_periodic, int zlo_wall_model, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* KS_H */
