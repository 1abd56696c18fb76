/*
 * CPU oracle for the single-level incompressible advance (test infrastructure).
 *
 * This header declares the C entry points of the FP64 CPU restatement of
 * Kynema-SGF's Godunov and MOL explicit-diffusion steps (oracle/ks_oracle.cpp).  It is
 * used ONLY by tests/, the package smoke check and the CPU-baseline leg of
 * bench.py, as the checker and as the timed CPU baseline.  The product library
 * (include/ks.h) never links, loads or calls it.
 *
 * Field exchange: every field is copied as its valid region, structure of
 * arrays, x fastest, then y, then z, then component (AMReX Array4 order without
 * ghost cells).  Node-centred fields have one more point along each
 * non-periodic direction; face fields have one more point along their normal
 * direction.
 */
#ifndef KS_ORACLE_H
#define KS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

int kso_create(const char* deck_text, void** out);
void kso_destroy(void* h);
const char* kso_last_error(void* h);

int kso_init_data(void* h);
int kso_evolve(void* h, int nsteps);
int kso_step(void* h);
int kso_compute_dt(void* h, double* dt);
int kso_pre_advance(void* h);
int kso_prepare_time_step(void* h);
int kso_apply_predictor(void* h, int incremental, int fixed_point_iteration);
int kso_apply_corrector(void* h);
int kso_apply_projection(void* h, double time, double scaling, int incremental);

int kso_field_shape(void* h, const char* name, int* ncomp, int* nx, int* ny, int* nz);
int kso_get_field(void* h, const char* name, double* out);
int kso_set_field(void* h, const char* name, const double* in);
double kso_get_scalar(void* h, const char* name);
int kso_set_scalar(void* h, const char* name, double value);

/* Operator-level entry points used by the known-answer tests. */
int kso_update_mueff(void* h);
int kso_compute_divtau(void* h, int use_new_state);
int kso_compute_sources(void* h);
/* predictor_rhs with diffusion factor fac and dt = the clock's dt (velocity
 * from velocity_old, conv_term, src_term, diff_term). */
int kso_predictor_rhs(void* h, double fac);
/* explicit_rk2_post_hoc: velocity += dt/2 diff_term / rho, diff_term holding
 * divtau(New) - divtau(Old) (the caller sets it). */
int kso_improve_explicit_diffusion(void* h);

#ifdef __cplusplus
}
#endif

#endif
