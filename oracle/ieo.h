/*
 * ieo.h -- CPU oracle for the InflationEasy lattice hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA engine
 * is compared against; it is never linked into, loaded by, or called from the
 * product (libiegpu / ie_gpu_main).  Only tests/, __graft_entry__.smoke() and
 * the cpu_baseline / --impl reference legs of bench.py may use it.
 *
 * It restates, in plain C with explicit state (no globals), the algorithm of
 * caravangelo/inflation-easy for the leapfrog evolution path, keeping every
 * floating-point operation in the reference's order so that results are
 * bit-identical to the reference built from source (see oracle/build_ref.py and
 * tests/test_oracle_pin.py).  Each function cites the reference file:line it
 * follows.  Parity status: pinned (bit-exact against the reference program at
 * N=16/32, hilltop and tabulated potentials, SIGW on/off, deltaN on).
 *
 * Lattice layout: flat index (i*N + j)*N + k, k fastest (src/main.h:34-38).
 * N is a run-time value here (the reference fixes it at compile time).
 */
#ifndef IEO_H
#define IEO_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Run-time parameters, one field per params.txt key of
 * src/runtime_parameters.cpp:17-112 plus the compile-time switches of
 * src/parameters.h:22-66 (here run-time). */
typedef struct {
    int N;
    int numerical_potential;   /* 0: hilltop (src/potential.cpp:77-83), 1: table */
    int perform_deltaN;
    int calculate_SIGW;
    int criterion;             /* +1 monotonic, -1 antimonotonic, 0 generic (src/parameters.h:60-66) */
    int seed;
    double rescale_s, af, V0, rescale_B, ns;
    double initial_field, initial_derivative, L, dt;
    int output_freq, output_infrequent_freq;
    double dN, Nend;
    int use_phiref_manual;
    double phiref_manual_value;
    double high_cutoff_index, low_cutoff_index;
    int forcing_cutoff;
    int output_spectra, output_histogram, output_energy, output_box3D, output_box2D;
    int screen_updates, nbins, int_err, int_errN;
    double dx;
    /* post-inflation phase (src/parameters.h:31 switch, src/runtime_parameters.cpp:48-52, 295-299) */
    int post_inflation, af_post_given;
    double horizon_factor, omega, dt_post_inflation, af_post_inflation;
    /* integrators, src/runtime_parameters.cpp:141-166: 0 leapfrog, 1 rk4, 2 rk45 */
    int inflation_integrator, pad_;
    int post_inflation_integrator, deltaN_integrator;
    /* RK45 controls, src/runtime_parameters.cpp:82-86, 184-192, 351-353 */
    double rk45_abs_tol, rk45_rel_tol, rk45_min_dt, rk45_max_dt, rk45_safety;
    int rk45_min_given, rk45_max_given;
} ieo_params;

typedef struct ieo_state ieo_state;

/* Defaults of src/runtime_parameters.cpp:17-112 for a given N and potential. */
void ieo_params_defaults(ieo_params* p, int N, int numerical_potential);
/* params.txt parser following src/runtime_parameters.cpp:195-365 (plus the
 * keys N, numerical_potential, perform_deltaN, calculate_SIGW, which the
 * reference fixes at compile time).  Returns 0, or -1 if the file is missing. */
int ieo_params_load(ieo_params* p, const char* path);
/* Derived quantities (rescale_B default, af default, dx):
 * src/runtime_parameters.cpp:342-354. */
void ieo_params_finalize(ieo_params* p, int rescale_B_given, int af_given);

ieo_state* ieo_create(const ieo_params* p);
void ieo_destroy(ieo_state* S);
void ieo_set_threads(int n);
const ieo_params* ieo_get_params(const ieo_state* S);

/* Tabulated potential: phi must be sorted descending (src/potential.cpp:18). */
int ieo_set_table(ieo_state* S, const double* phi, const double* V, const double* dV, int n);

/* Field access (pointers into the state; N^3 elements). */
double* ieo_f(ieo_state* S);
double* ieo_fd(ieo_state* S);
double* ieo_deltaN(ieo_state* S);
double* ieo_fnyquist(ieo_state* S);   /* N x 2N */
double* ieo_fdnyquist(ieo_state* S);
float*  ieo_h(ieo_state* S, int c);
float*  ieo_hd(ieo_state* S, int c);

typedef struct { double t, a, ad, ad2, astep, Ne, phiref, hubble_init; } ieo_scalars;
void ieo_get_scalars(const ieo_state* S, ieo_scalars* out);
void ieo_set_scalars(ieo_state* S, const ieo_scalars* in);

/* Error reporting: the reference prints and exit(1)s; the oracle records the
 * message and returns nonzero from the calling function. */
const char* ieo_last_error(const ieo_state* S);

/* ---- RNG + initial conditions: src/initialize.cpp:18-232 ---- */
double ieo_rand_uniform(ieo_state* S);
int ieo_initialize(ieo_state* S);      /* src/initialize.cpp:93-114 */
int ieo_initializef(ieo_state* S);     /* src/initialize.cpp:118-214 */
void ieo_initializeGW(ieo_state* S);   /* src/initialize.cpp:236-243 */

/* ---- potential: src/potential.cpp ---- */
double ieo_potential(ieo_state* S, double v);
double ieo_potential_energy(ieo_state* S);

/* ---- engine-arithmetic mode ----
 * The GPU engine forms the Friedmann update's lattice sums exactly (the
 * correctly rounded exact sum of exact products f lapl(f), in any order),
 * sums the exact f^2 (hilltop) or the slope form of V (table) for the
 * potential, and evaluates pow(a, y) as
 * exact products and quotients for y = 0, 1, 2, -1.  With the mode on, the
 * oracle's leapfrog does the same, so the engine can be compared with it bit
 * for bit; with it off (the default) the oracle is the reference: serial sums
 * in loop order and libm pow.  The two modes differ only by rounding, which
 * measures the reference's own floor. */
void ieo_set_engine_arith(ieo_state* S, int on);
/* The mode of states created from now on (ieo_create, ieo_run_program). */
void ieo_set_engine_arith_default(int on);
/* Correctly rounded exact sum of n doubles, and of the exact products
 * x[i] y[i] (the mode's summations). */
double ieo_exact_sum(const double* x, size_t n);
double ieo_exact_dot(const double* x, const double* y, size_t n);

/* ---- leapfrog: src/evolution.cpp ---- */
double ieo_gradient_energy(ieo_state* S);
double ieo_kin_energy(ieo_state* S);
int ieo_evolve_derivs(ieo_state* S, double d);
void ieo_evolve_fields(ieo_state* S, double d);
double ieo_rescaled_step(const ieo_state* S, double astep);
/* Runs `nsteps` iterations of the leapfrog loop body of
 * src/evolution.cpp:937-945 without output; stops early once a > af.
 * Returns the number of steps taken (or -1 on error). */
int ieo_leapfrog_steps(ieo_state* S, int nsteps);

/* ---- RK4 inflation step: rk4_step_inflation(h), src/evolution.cpp:760-779, with
 * compute_inflation_rhs (:418-512); the RHS sums are serial in loop order, which is
 * what the reference's OpenMP reduction gives with one thread. ---- */
int ieo_rk4_step_inflation(ieo_state* S, double h);
/* RK45 (Dormand-Prince 5(4)): one attempt, the clamp and hmax helpers and the
 * accept/reject driver of src/evolution.cpp:326-363, 781-904 */
int ieo_rk45_step_inflation(ieo_state* S, double h, double hmax, double* h_next, int* accepted);
int ieo_rk45_accept(ieo_state* S, double* h, double hmax);
double ieo_rk45_clamp(const ieo_state* S, double h, double hmax);
double ieo_rk45_hmax(const ieo_state* S, double base_step);
/* the deltaN loop's RK4 step, RK45 attempt and accept driver, src/evolution.cpp:1063-1267, 1338-1366 */
int ieo_rk4_step_deltaN(ieo_state* S, double h);
int ieo_rk45_step_deltaN(ieo_state* S, double h, double hmax, double* h_next, int* accepted);
int ieo_rk45_accept_deltaN(ieo_state* S, double* h, double hmax);
/* selects the post-inflation right-hand side for the RK steps */
void ieo_set_rk_post(ieo_state* S, int post);

/* ---- post-inflation phase: src/initialize.cpp:245-290, src/evolution.cpp:1378-1653 ---- */
void ieo_initialize_post_inflation(ieo_state* S);
void ieo_evolve_derivs_post_inflation(ieo_state* S, double d);

/* ---- FFT: src/ffteasy.hpp ---- */
void ieo_fftrn_d(double* f, double* fny, int N, int forward);
void ieo_fftrn_f(float* f, float* fny, int N, int forward);
void ieo_fftc1_d(double* f, int n, int skip, int forward);

/* ---- spectra: src/output.cpp:63-151 (without printing) ---- */
int ieo_numbins(int N);
/* Bins an r2c field already in k-space; f2 holds the raw sums (before /count). */
void ieo_bin_spectrum(int N, const double* field_fft, const double* nyq, int* counts, double* f2);
/* spectraf(): forward FFT of f, bin, inverse FFT (f is modified in place at
 * round-off level, as in the reference). */
void ieo_spectrum_f(ieo_state* S, int* counts, double* f2);
/* The same with the forcing cutoff (src/output.cpp:330-401) applied to f and
 * fd between the binning and the inverse FFT when high > 0: modes with
 * |p| > high or |p| < low are zeroed. */
void ieo_spectrum_f_cut(ieo_state* S, int* counts, double* f2, double high, double low);
/* The cutoff alone, with f in k-space (fd is transformed forward and back). */
void ieo_forcing_cutoff(ieo_state* S, double high, double low);
/* GW TT spectrum, src/output.cpp:466-625.  mode: 0 = h, 1 = hd (DoubleThenFloat
 * scaling with to_phys).  f2_float gets the reference's float accumulators;
 * f2_double (may be NULL) gets the same per-mode float values summed in double. */
void ieo_gw_spectrum(ieo_state* S, int which, double to_phys, int* counts, float* f2_float, double* f2_double);

/* ---- deltaN: src/evolution.cpp:1004-1375, src/initialize.cpp:219-232 ---- */
int ieo_initializeN(ieo_state* S);
int ieo_evolve_derivsN(ieo_state* S, double d);
void ieo_evolve_fieldsN(ieo_state* S, double d);
double ieo_get_phiref(ieo_state* S);
/* Loop of src/evolution.cpp:1321-1329 (no output).  Returns steps taken. */
int ieo_deltaN_steps(ieo_state* S, int max_steps);
/* saveN float-accumulator mean, src/output.cpp:1527-1537. */
float ieo_saveN_mean(const ieo_state* S, double cutoff);

/* Whole program, src/main.cpp:103-146, writing the reference's results/ .dat
 * files into results_dir (inputs_dir holds field_values.dat, potential.dat,
 * potential_derivative.dat when numerical_potential = 1). */
int ieo_run_program(const ieo_params* p, const char* results_dir, const char* inputs_dir);
/* Same, also writing trace.txt and state.bin into dump_dir (NULL: none). */
int ieo_run_program_dump(const ieo_params* p, const char* results_dir, const char* inputs_dir, const char* dump_dir);

#ifdef __cplusplus
}
#endif
#endif
