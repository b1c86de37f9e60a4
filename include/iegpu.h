/*
 * iegpu.h -- C ABI of the GB300 (sm_103a) InflationEasy evolution engine.
 *
 * The reference program (caravangelo/inflation-easy) reaches its physics
 * through free functions over global state (src/main.h:137-205).  This header
 * is the drop-in boundary for that hot path: each entry point names the
 * reference function it replaces.  The host keeps the reference's driver,
 * params.txt handling and output formats; the lattice state lives on the GPU
 * inside an opaque context.
 *
 * Conventions
 *  - Every call returns an int status (IEGPU_OK = 0).  Nothing exits or
 *    throws across the ABI; iegpu_last_error() gives the message the
 *    reference would have printed before exit(1).
 *  - Host arrays use the reference layout: N^3 values, flat index
 *    (i*N + j)*N + k, k fastest (src/main.h:34-38); Nyquist planes are N x 2N
 *    (src/main.cpp:27-29).  Arrays are copied; no pointer is retained.
 *  - Background scalars (t, a, ad, ad2, astep) travel in iegpu_bg and the
 *    host copy is authoritative between calls.
 *  - One context = one lattice = one CUDA stream; a context is not
 *    re-entrant.  Calls are stream-ordered and synchronise before returning
 *    results to the host.
 */
#ifndef IEGPU_ABI_H
#define IEGPU_ABI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct iegpu_ctx iegpu_ctx;

/* ---- status codes ---------------------------------------------------- */
#define IEGPU_OK            0
#define IEGPU_EINVAL        1  /* bad argument or configuration */
#define IEGPU_ECUDA         2  /* CUDA runtime error */
#define IEGPU_ERANGE        3  /* field outside the potential table, src/potential.cpp:19-27 */
#define IEGPU_ENAN          4  /* non-finite field mean, src/output.cpp:251-258 */
#define IEGPU_ECOURANT      5  /* dt > dx/sqrt(3), src/initialize.cpp:94-97 */
#define IEGPU_ENOMEM        6  /* device allocation failed */
#define IEGPU_ETABLE        7  /* repeated table nodes, src/potential.cpp:62-65 */
#define IEGPU_EUNSUPPORTED  8  /* feature not available in this form */
#define IEGPU_ETIMEOUT      9  /* a bounded device wait gave up */
#define IEGPU_ETOOBIG      10  /* size above a fixed, documented limit */
#define IEGPU_ECONVERGE    11  /* RK45 step control gave up, src/evolution.cpp:974-979, 1629-1634 */

/* ---- configuration --------------------------------------------------- */
#define IEGPU_POT_HILLTOP   0  /* analytic hilltop, src/potential.cpp:77-83 */
#define IEGPU_POT_TABLE     1  /* tabulated V, V' (numerical_potential = 1) */

#define IEGPU_FORM_FP64     0  /* plain FP64: per-site arithmetic in the reference's order */
#define IEGPU_FORM_SPLIT    1  /* FP32 perturbations about an FP64 background */
#define IEGPU_FORM_SPLIT_COMP 2 /* the split form with compensated (Kahan) steps:
                                   FP32 perturbations plus bf16 residuals;
                                   N = 128, 256 or 512 */

#define IEGPU_CRIT_GENERIC        0  /* evolve while V(phi) > V(phiref) */
#define IEGPU_CRIT_MONOTONIC      1  /* evolve while |phi| > |phiref| */
#define IEGPU_CRIT_ANTIMONOTONIC (-1) /* evolve while |phi| < |phiref| */

typedef struct {
    int N;            /* points per side: power of two, 8 <= N <= 1024 (src/parameters.h:42-44) */
    int potential;    /* IEGPU_POT_*            (src/parameters.h:26)  */
    int sigw;         /* evolve h_ij            (calculate_SIGW)        */
    int form;         /* IEGPU_FORM_*                                    */
    int criterion;    /* IEGPU_CRIT_*           (src/parameters.h:60-66) */
    double L;         /* comoving box size                               */
    double dt;        /* base time step                                  */
    double rescale_s; /* field-rescaling exponent                        */
    double rescale_B; /* time rescaling B                                */
    double V0, ns;    /* hilltop parameters                              */
} iegpu_config;

/* Background scalars of src/main.cpp:31-33. */
typedef struct {
    double t, a, ad, ad2, astep;
} iegpu_bg;

/* RK45 controls, src/runtime_parameters.cpp:82-86 (keys rk45_abs_tol,
 * rk45_rel_tol, rk45_min_dt, rk45_max_dt, rk45_safety).  The library applies
 * sanitize_rk45_controls (:184-192) to a copy: min_dt <= 0 means 1e-6 |dt|,
 * max_dt <= 0 means |dt|, and out-of-range tolerances or safety take the
 * defaults 1e-8, 1e-6, 0.9. */
typedef struct {
    double abs_tol, rel_tol, min_dt, max_dt, safety;
} iegpu_rk45_controls;
/* The controls the RK45 entry points use for base step dt: *out = the
 * sanitised copy of *in described above.  Needs no context or device. */
int  iegpu_rk45_effective(const iegpu_rk45_controls* in, double dt, iegpu_rk45_controls* out);

/* Field selectors for upload/download/FFT/spectra. */
#define IEGPU_F       0   /* phi             (f)        */
#define IEGPU_FD      1   /* phi'            (fd)       */
#define IEGPU_DELTAN  2   /* deltaN map      (deltaN)   */
#define IEGPU_H(c)   (8 + (c))   /* h_ij packed component c = 0..5 (xx,yy,zz,xy,xz,yz) */
#define IEGPU_HD(c)  (16 + (c))  /* h_ij' */

/* ---- context ---------------------------------------------------------- */
int  iegpu_version(void);
const char* iegpu_strerror(int code);
/* Allocates the device state for one lattice.  Replaces the global vectors
 * of src/main.cpp:16-29 and the sizing in src/initialize.cpp:118-120. */
int  iegpu_create(const iegpu_config* cfg, struct iegpu_ctx** out);
int  iegpu_destroy(struct iegpu_ctx* ctx);
const char* iegpu_last_error(const struct iegpu_ctx* ctx);
/* The CUDA stream (cudaStream_t) the context launches on. */
void* iegpu_stream(struct iegpu_ctx* ctx);
/* Number of kernels this context has launched so far. */
long long iegpu_launch_count(const struct iegpu_ctx* ctx);

/* Tabulated potential (inputs/field_values.dat, potential.dat,
 * potential_derivative.dat; src/main.cpp:46-50).  phi sorted descending. */
int  iegpu_set_table(struct iegpu_ctx* ctx, const double* phi, const double* V, const double* dV, int n);

/* ---- state transfer --------------------------------------------------- */
/* field: IEGPU_F, IEGPU_FD, IEGPU_DELTAN (double), IEGPU_H(c), IEGPU_HD(c)
 * (float).  nyquist (N x 2N, same type) may be NULL. */
int  iegpu_upload(struct iegpu_ctx* ctx, int field, const void* host, const void* nyquist);
int  iegpu_download(struct iegpu_ctx* ctx, int field, void* host, void* nyquist);
/* x += value at every site (initializef background add, src/initialize.cpp:197-200). */
int  iegpu_add(struct iegpu_ctx* ctx, int field, double value);

/* ---- initial conditions (src/initialize.cpp) -------------------------- */
/* initialize() + initializef(), src/initialize.cpp:93-214, on the device:
 * Bunch-Davies modes with the reference's Park-Miller stream (seed; seed < 1
 * gives the reference's constant 0.33 draws), the zero mode removed, the
 * inverse r2c FFT, and the homogeneous values phi0, dphi0 added.  The mode
 * cutoff of set_mode applies when high_cutoff_index > 0.  *hubble_init
 * receives sqrt((kinetic + potential + gradient)/3) of the new lattice at
 * a = 1 (src/initialize.cpp:202-212).  Fails with IEGPU_ECOURANT when
 * dt > dx/sqrt(3). */
int  iegpu_bunch_davies(struct iegpu_ctx* ctx, int seed, double phi0, double dphi0,
                        double high_cutoff_index, double low_cutoff_index, double* hubble_init);

/* ---- leapfrog (src/evolution.cpp) ------------------------------------- */
/* evolve_fields(d), src/evolution.cpp:260-284: t += d; f += d fd; h += d hd; a += d ad. */
int  iegpu_evolve_fields(struct iegpu_ctx* ctx, double d, iegpu_bg* bg);
/* evolve_derivs(d), src/evolution.cpp:150-257: Friedmann half-kicks of ad
 * around the kick of fd (and hd when SIGW is on). */
int  iegpu_evolve_derivs(struct iegpu_ctx* ctx, double d, iegpu_bg* bg);
/* The leapfrog branch of run_evolution_loop, src/evolution.cpp:937-945:
 *   while (a <= af && steps < max_steps) {
 *       d = dt*astep^(s-1); evolve_derivs(d); evolve_fields(d); astep = a; }
 * runs entirely on the device (CUDA graph).  *steps_taken receives the number
 * of steps; a_trace (may be NULL) receives a after each step, as written to
 * results/output.txt by report_step (src/evolution.cpp:926-927).  The final
 * "astep = a" of the last step taken is left to the caller, who runs its
 * report/save first (save() drifts with the old astep, src/output.cpp:1472)
 * and then sets bg->astep = bg->a before the next call. */
int  iegpu_leapfrog(struct iegpu_ctx* ctx, double af, int max_steps, iegpu_bg* bg,
                    int* steps_taken, double* a_trace);
/* rk4_step_inflation(h), src/evolution.cpp:760-779 (inflation_integrator =
 * rk4; plain FP64 form): four evaluations of compute_inflation_rhs
 * (:418-512) on the stage states of :641-690, then the weighted update of
 * f, fd (h, hd with SIGW) and of a, ad (:717-758), and t += h.  ad2 is not
 * touched.  The stage's lattice sums are combined on the device in a fixed
 * order, so a, ad agree with the reference to rounding of those sums; every
 * per-site expression is the reference's. */
int  iegpu_rk4_step_inflation(struct iegpu_ctx* ctx, double h, iegpu_bg* bg);
/* The RK4 branch of run_evolution_loop, src/evolution.cpp:948-956: as
 * iegpu_leapfrog (same stepping, a_trace and "astep = a" contract), with
 * rk4_step_inflation(dt*astep^(s-1)) as the step.  No half drift precedes
 * or follows the loop for this integrator. */
int  iegpu_rk4(struct iegpu_ctx* ctx, double af, int max_steps, iegpu_bg* bg,
               int* steps_taken, double* a_trace);
/* rk45_step_inflation(h, hmax, h_next), src/evolution.cpp:781-904
 * (inflation_integrator = rk45; plain FP64 form): one Dormand-Prince 5(4)
 * attempt of step h.  The weighted-RMS error over f, fd (h, hd) and a, ad
 * decides acceptance: *accepted = 1 and bg takes the 5th-order state, or
 * *accepted = 0 and the state is kept.  *h_next is the step the reference's
 * controller proposes (clamped to hmax). */
int  iegpu_rk45_step_inflation(struct iegpu_ctx* ctx, const iegpu_rk45_controls* ctl, double h, double hmax,
                               double* h_next, int* accepted, iegpu_bg* bg);
/* The RK45 branch of run_evolution_loop, src/evolution.cpp:958-985: while
 * a <= af, hmax = min(max_dt, max(min_dt, 2 dt astep^(s-1))), *h clamped to
 * it, attempts until one is accepted (rk45_accept_step, :345-363), then
 * "astep = a" (left to the caller after the last step, as iegpu_leapfrog).
 * *h carries the proposed step between steps and calls; the first call takes
 * dt astep^(s-1) (:959).  After 25 rejections, or at the minimum step, it
 * returns IEGPU_ECONVERGE with the reference's message. */
int  iegpu_rk45(struct iegpu_ctx* ctx, const iegpu_rk45_controls* ctl, double af, int max_steps, double* h,
                iegpu_bg* bg, int* steps_taken, double* a_trace);
/* kin_energy(), gradient_energy(), potential_energy():
 * src/evolution.cpp:130-145, src/potential.cpp:151-171.  out[3] = {kin, grad, pot}. */
int  iegpu_energies(struct iegpu_ctx* ctx, const iegpu_bg* bg, double out[3]);

/* ---- measurement ------------------------------------------------------ */
/* CUDA events recorded on the context's stream: start, then stop returns the
 * elapsed device time in milliseconds (synchronising on the stop event). */
int  iegpu_timer_start(struct iegpu_ctx* ctx);
int  iegpu_timer_stop(struct iegpu_ctx* ctx, float* ms);
/* Like iegpu_leapfrog, but each kernel is launched on its own with a pair of
 * CUDA events around it.  FP64 form: ms_out[0] accumulates the reduction
 * kernel's device time, ms_out[1] the kick/drift kernel's.  Split form:
 * ms_out[0] is the priming reduction, ms_out[1] the fused step kernels'
 * total.  For profiling only. */
int  iegpu_profile_leapfrog(struct iegpu_ctx* ctx, double af, int nsteps, iegpu_bg* bg, double* ms_out, int nk);
/* No counterpart in the reference: a throughput probe of the current device's
 * FP64 pipe (op 0: DFMA, 1: DADD, 2: DMUL), in thread instructions per second,
 * the denominator of the plain FP64 form's roofline.  Needs no context. */
int  iegpu_measure_fp64_rate(int op, double* inst_per_s);

/* Split form: run the launch-shape autotuner now (it otherwise runs on the
 * first iegpu_leapfrog call) and report the chosen shape of the step kernel:
 * rows per tile, planes prefetched, plane chunks.  The lattice state is left
 * unchanged. */
int  iegpu_autotune(struct iegpu_ctx* ctx, const iegpu_bg* bg, int* rows, int* prefetch, int* chunks);
/* Split form, 32 <= N <= 512: fix the step kernel's launch shape instead of
 * tuning it: rows per tile 4 or 8 with 1 or 2 planes prefetched (rows 4 at
 * N >= 128 also 3 or 4), rows 16 at 128 <= N <= 256 with 1 to 3, or rows = N
 * for whole planes (N = 32, 64) with 2 or 4; 1 <= chunks <= N/8 plane
 * chunks, or chunks = 0 (N >= 128) for one wave
 * of CTAs that each take an equal share of the lattice.  prefetch + 10 stages
 * the planes by bulk (TMA) copies instead (N >= 128: rows 8 with 2 planes
 * ahead, rows 16 at N <= 256 with 1 to 3); iegpu_autotune reports that
 * encoding too. */
int  iegpu_set_shape(struct iegpu_ctx* ctx, int rows, int prefetch, int chunks);
/* Split form, 128 <= N <= 256 without SIGW: iegpu_leapfrog runs the step kernel for
 * up to 64 steps per cooperative launch (on = 1, the default), each step's
 * first copies overlapping the scalar update of the step before, or one
 * launch per step in CUDA graphs (on = 0).  Both give the same bits.  No
 * counterpart in the reference (its loop is serial host code). */
int  iegpu_set_persistent(struct iegpu_ctx* ctx, int on);
/* No counterpart in the reference: the bounds of the split form's device-side
 * waits (the persistent step barrier and the bulk-copy barriers), which end
 * a call with IEGPU_ETIMEOUT instead of hanging when a wait cannot finish.
 * polls: poll limit of each wait (0: the default, 2^20, about half a second).
 * unreachable != 0 makes the persistent step barrier wait for a count that no
 * launch reaches, so that it gives up: a hook for failure-path tests (the
 * context stays usable; the next call starts from the host's background).
 * Persistent launches run at 128 <= N <= 256 without SIGW. */
int  iegpu_set_wait_limit(struct iegpu_ctx* ctx, unsigned polls, int unreachable);

/* ---- post-inflation phase (plain FP64 form, SIGW on) ------------------- */
/* initialize_post_inflation(), src/initialize.cpp:245-290, without its save:
 * f = Phi (deltaN - <deltaN>) with Phi = 3(1+omega)/(5+3 omega) (from_deltaN
 * = 1), or Phi (f - <f>) / (<fd> a^(s-1) / (ad a^(s-2))) otherwise, the means
 * summed serially in the reference's loop order; fd is kept; h and h' are
 * zeroed; bg gets t = 0, a = 1, ad = horizon_factor N 2 pi / L (ad2 and astep
 * are kept, as in the reference). */
int  iegpu_initialize_post_inflation(struct iegpu_ctx* ctx, double horizon_factor, double omega, int from_deltaN,
                                     iegpu_bg* bg);
/* evolve_derivs_post_inflation(d), src/evolution.cpp:1436-1555: ad2 and the
 * half kicks of ad on the host, the radiation-era kick of fd and the tensor
 * kick with the Hessian source (build_deriv_pack, :1398-1418) on the device. */
int  iegpu_evolve_derivs_post_inflation(struct iegpu_ctx* ctx, double d, double omega, iegpu_bg* bg);
/* The leapfrog loop body of run_post_inflation_loop, src/evolution.cpp:1589-1597:
 * while bg->a <= af_post, evolve_derivs_post_inflation(dt_post) then
 * evolve_fields(dt_post), at most max_steps times; *steps = steps taken.  The
 * half drift before the loop and the saves are the caller's, as in the
 * reference.  The steps are enqueued without synchronisation.  a_trace (may
 * be null, else max_steps entries) receives a after each step taken. */
int  iegpu_post_inflation_leapfrog(struct iegpu_ctx* ctx, double af_post, double dt_post, double omega, int max_steps,
                                   iegpu_bg* bg, int* steps, double* a_trace);
/* The RK4 and RK45 branches of run_post_inflation_loop,
 * src/evolution.cpp:1606-1641: the post-inflation equations of
 * compute_inflation_rhs (:515-598) in rk4_step_inflation with step dt_post,
 * or in the RK45 step control with hmax from dt_post (*h as in iegpu_rk45,
 * the first call taking dt_post), while bg->a <= af_post, at most max_steps
 * steps.  No half drift precedes the loop for these integrators, and the
 * saves do not re-synchronise. */
int  iegpu_post_inflation_rk4(struct iegpu_ctx* ctx, double af_post, double dt_post, double omega, int max_steps,
                              iegpu_bg* bg, int* steps, double* a_trace);
int  iegpu_post_inflation_rk45(struct iegpu_ctx* ctx, const iegpu_rk45_controls* ctl, double af_post, double dt_post,
                               double omega, int max_steps, double* h, iegpu_bg* bg, int* steps, double* a_trace);

/* ---- diagnostics (src/output.cpp) ------------------------------------- */
/* Sums of meansvars(), src/output.cpp:235-240: out[3] = {sum f, sum fd, sum f^2}. */
int  iegpu_means(struct iegpu_ctx* ctx, double out[3]);
/* histograms()/histogramsN(), src/output.cpp:1070-1135/1220-1277.
 * freq[nbins] = counts / numpts; *bmin, *df as printed to histogramtimes.
 * 1 <= nbins <= 8192. */
int  iegpu_histogram(struct iegpu_ctx* ctx, int field, int nbins, double* bmin, double* df, double* freq);
/* fftrnd / fftrnf of src/ffteasy.hpp:127-190 in place on a device field and
 * its Nyquist plane (forward = +1 or -1). */
int  iegpu_fft(struct iegpu_ctx* ctx, int field, int forward);
/* Number of spectrum bins: (int)(1.73205*(N/2)) + 1, src/output.cpp:69. */
int  iegpu_numbins(int N);
/* spectraf() / spectraN() core, src/output.cpp:297-406, 1140-1169: forward
 * FFT, isotropic binning (write_isotropic_spectrum_from_fft_r2c,
 * src/output.cpp:63-151), inverse FFT.  counts[nbins] (exact integers) and
 * f2[nbins] = sum of weighted |X_k|^2 per bin (before /count and norm1). */
int  iegpu_spectrum(struct iegpu_ctx* ctx, int field, int* counts, double* f2, int nbins);
/* spectraf() with its forcing cutoff, src/output.cpp:297-406 (and
 * spectraf_post_inflation, :1667-1770): forward FFT of f, the binning of
 * iegpu_spectrum, then, when high_cutoff_index > 0, the k-space filter of
 * :330-401 -- every mode of f and fd with |p| > high_cutoff_index or
 * |p| < low_cutoff_index is zeroed (p the integer lattice momentum; fd is
 * transformed forward and back; a low cutoff > 0 zeroes the k = 0 mode too)
 * -- and the inverse FFT of f.  With high_cutoff_index <= 0 it is
 * iegpu_spectrum(ctx, IEGPU_F, ...).  The reference runs it when
 * forcing_cutoff is set.  Plain FP64 form only (IEGPU_EUNSUPPORTED on the
 * split forms). */
int  iegpu_spectrum_cutoff(struct iegpu_ctx* ctx, int* counts, double* f2, int nbins, double high_cutoff_index,
                           double low_cutoff_index);
/* spectraGW()/spectraGWdot() core, src/output.cpp:466-648: forward FFT of
 * the six h (which = 0) or h' (which = 1, scaled by to_phys), TT projection
 * per mode in float as the reference, binning (bins < floor(0.8*numbins)),
 * inverse FFT.  f2 accumulates the per-mode float values in double. */
int  iegpu_gw_spectrum(struct iegpu_ctx* ctx, int which, double to_phys, int* counts, double* f2, int nbins);
/* The same spectrum with the reference's own accumulators: f2[nbins] (float)
 * is write_gw_spectrum_impl's f2 (src/output.cpp:478-612) before the
 * division by the counts, i.e. the per-mode float values (2 fp2 for
 * 0 < kz < N/2, fp2 on the kz = 0 and kz = N/2 planes) added in float in the
 * reference's loop order (i, j, then kz); f2_sum (may be NULL) receives the
 * same values added in double (in another order).  Given the same h, f2 is
 * the reference's bit for bit. */
int  iegpu_gw_spectrum_ref(struct iegpu_ctx* ctx, int which, double to_phys, int* counts, float* f2, double* f2_sum,
                           int nbins);

/* Allocation-free variant of the shell binning inside iegpu_spectrum, for
 * callers that cannot allocate device memory: a plugin whose host framework
 * owns all device memory through its own caching allocator and forbids
 * direct cudaMalloc, or a process whose fixed memory budget is already spent
 * on the lattice, and which has no iegpu context (creating one allocates).
 * It has no counterpart in the reference.
 * modes: the r2c field after the forward FFT (N^3 doubles, the layout
 * iegpu_fft produces); nyquist: its N x 2N Nyquist plane; counts[nbins] and
 * f2[nbins] (nbins = iegpu_numbins(N)) receive the same values as
 * iegpu_spectrum's.  All five pointers are device memory; the work is
 * enqueued on `stream` (a cudaStream_t, 0 for the default stream) and the
 * call returns without synchronising.
 * Nothing is allocated: the partial sums live in one fixed 681,984-byte
 * array inside the library, which every GPU that loads it holds until exit.
 * Limit: N <= 512 (larger N returns IEGPU_ETOOBIG).  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress), so
 * make it before any stream capture.  All calls share the array: calls that
 * overlap on the GPU (on different streams, or from different threads)
 * race; order them on one stream. */
int  iegpu_shell_spectrum_noalloc(const double* modes, const double* nyquist, int N, int* counts,
                                  double* f2, void* stream);

/* ---- deltaN (src/evolution.cpp:1004-1375) ----------------------------- */
/* initializeN(), src/initialize.cpp:219-232: fd <- fd*a^(s-1)/sqrt(V/3), deltaN = 0. */
int  iegpu_initializeN(struct iegpu_ctx* ctx, double a);
/* get_phiref(), src/evolution.cpp:1271-1288 (first extremal site in loop order). */
int  iegpu_get_phiref(struct iegpu_ctx* ctx, double* phiref);
/* evolve_fieldsN(d) (src/evolution.cpp:1015-1037) on the lattice; the scalar
 * updates t += d, a += d*ad are left to the caller. */
int  iegpu_evolve_fieldsN(struct iegpu_ctx* ctx, double d, double phiref);
/* evolve_derivsN(d), src/evolution.cpp:1004-1012. */
int  iegpu_evolve_derivsN(struct iegpu_ctx* ctx, double d);
/* nsteps iterations of { evolve_derivsN(dN); evolve_fieldsN(dN); } with each
 * site's state held in registers for the whole run. */
int  iegpu_deltaN_steps(struct iegpu_ctx* ctx, double dN, int nsteps, double phiref);
/* nsteps of rk4_step_deltaN(dN) (deltaN_integrator = rk4,
 * src/evolution.cpp:1176-1188, 1324-1332): per site, four evaluations of
 * compute_deltaN_rhs (:1063-1113) held in registers, then the weighted
 * update of f, fd and deltaN; bg->a (with its constant derivative ad) and
 * bg->t advance as apply_deltaN_weighted_update advances them.  Ne is the
 * caller's (Ne += dN per step).  No half drift precedes or follows the loop
 * for this integrator. */
int  iegpu_deltaN_rk4_steps(struct iegpu_ctx* ctx, double dN, int nsteps, double phiref, iegpu_bg* bg);
/* The RK45 branch of run_deltaN_loop, src/evolution.cpp:1334-1367: while
 * *Ne <= Nend (at most max_steps steps), hmax from dN, *h clamped to it,
 * rk45_step_deltaN attempts (:1190-1267) until one is accepted, then
 * *Ne += *h with the step proposed for the next iteration, as the reference
 * adds it.  *h carries that step between calls; the first call takes dN.
 * Ne_trace (may be NULL, else max_steps entries) receives Ne after each step.
 * After 25 rejections, or at the minimum step, it returns IEGPU_ECONVERGE
 * with the reference's message. */
int  iegpu_deltaN_rk45(struct iegpu_ctx* ctx, const iegpu_rk45_controls* ctl, double dN, double Nend, int max_steps,
                       double phiref, double* h, double* Ne, iegpu_bg* bg, int* steps, double* Ne_trace);
/* saveN() mean, src/output.cpp:1527-1537: sequential float accumulation of
 * deltaN over sites with deltaN <= cutoff, divided by N^3 in float. */
int  iegpu_saveN_mean(struct iegpu_ctx* ctx, double cutoff, float* nmean);
/* deltaN -= value (src/output.cpp:1539-1542, 161-163). */
int  iegpu_shift(struct iegpu_ctx* ctx, int field, double value);
/* x = (x > threshold) ? 0 : x  (src/output.cpp:1549-1553). */
int  iegpu_zero_above(struct iegpu_ctx* ctx, int field, double threshold);
/* Sum of a field over the lattice (build_deltaN_linear mean, src/output.cpp:156-164). */
int  iegpu_sum(struct iegpu_ctx* ctx, int field, double* sum);

/* ---- ensembles ---------------------------------------------------------
 * The reference evolves one lattice per process; these entry points evolve
 * many independent lattices (seeds, sizes) in one set of device buffers, in
 * the split form: per leapfrog step one kernel launch for all the lattices of
 * one size, the sizes side by side as parallel branches of a CUDA graph of
 * 16 steps.  Every lattice b follows the
 * reference's program with its own a(t), H and stop condition a > af[b]:
 * initial conditions (src/initialize.cpp:93-214), the leapfrog loop
 * (src/evolution.cpp:934-945), the deltaN stage (src/evolution.cpp:1291-1375)
 * and saveN's zeta (src/output.cpp:1522-1560).  Arrays of `count` entries
 * are indexed by lattice.  N in {32, 64, 128, 256}. */
typedef struct iegpu_ens iegpu_ens;
/* cfg: everything but N is shared; form must be IEGPU_FORM_SPLIT, sigw 0. */
int  iegpu_ens_create(const iegpu_config* cfg, const int* Ns, int count, struct iegpu_ens** out);
int  iegpu_ens_destroy(struct iegpu_ens* ens);
const char* iegpu_ens_last_error(const struct iegpu_ens* ens);
long long iegpu_ens_launch_count(const struct iegpu_ens* ens);
void* iegpu_ens_stream(struct iegpu_ens* ens);
int  iegpu_ens_set_table(struct iegpu_ens* ens, const double* phi, const double* V, const double* dV, int n);
/* iegpu_bunch_davies for every lattice with seeds[b]: lattice b gets the same
 * fields as a single lattice of its size and seed; hubble_init[count]. */
int  iegpu_ens_bunch_davies(struct iegpu_ens* ens, const int* seeds, double phi0, double dphi0,
                            double high_cutoff_index, double low_cutoff_index, double* hubble_init);
/* evolve_fields(d[b]) of every lattice (src/evolution.cpp:260-284). */
int  iegpu_ens_evolve_fields(struct iegpu_ens* ens, const double* d, iegpu_bg* bg);
/* iegpu_leapfrog for every lattice at once: lattice b stops after max_steps
 * or once a > af[b]; steps[count] (may be NULL) receives the steps taken.  As
 * there, the final "astep = a" is left to the caller. */
int  iegpu_ens_leapfrog(struct iegpu_ens* ens, const double* af, int max_steps, iegpu_bg* bg, int* steps);
/* nsteps steps launched one by one between CUDA events: *ms_prime = the
 * priming reduction, *ms_steps = the step kernels' total device time. */
int  iegpu_ens_profile(struct iegpu_ens* ens, int nsteps, iegpu_bg* bg, double* ms_prime, double* ms_steps);
/* Times candidate launch shapes of every lattice size on the live state
 * (restored afterwards) and keeps the fastest; rows, prefetch and chunks
 * (arrays of count, may be NULL) receive each lattice's shape. */
int  iegpu_ens_autotune(struct iegpu_ens* ens, const iegpu_bg* bg, int* rows, int* prefetch, int* chunks);
/* Sets the launch shape of the lattices of size N, as iegpu_set_shape. */
int  iegpu_ens_set_shape(struct iegpu_ens* ens, int N, int rows, int prefetch, int chunks);
/* The current launch shape of each lattice (arrays of count, may be NULL),
 * as iegpu_ens_autotune reports it, without tuning. */
int  iegpu_ens_shapes(struct iegpu_ens* ens, int* rows, int* prefetch, int* chunks);
/* No counterpart in the reference (it runs one lattice per process).  on = 1:
 * iegpu_ens_leapfrog advances every lattice in cooperative launches of up to
 * 64 steps each, the CTAs pulling (lattice, row tile, step) items of every
 * size from one queue, the largest lattices first; an item waits only for its
 * own lattice's update of the step before (bounded: IEGPU_ETIMEOUT).  Every
 * lattice uses 8-row tiles with 2 planes ahead and 32 planes per item.
 * on = 0: one kernel per lattice size and step, the sizes as parallel
 * branches of a CUDA graph (the default).  N in {32, 64, 128} for on = 1. */
int  iegpu_ens_set_persistent(struct iegpu_ens* ens, int on);
int  iegpu_ens_timer_start(struct iegpu_ens* ens);
int  iegpu_ens_timer_stop(struct iegpu_ens* ens, float* ms);
/* N_b^3 doubles of lattice b: IEGPU_F / IEGPU_FD (phibar + dphi, pibar + dpi,
 * or the FP64 fields once the deltaN stage has begun), IEGPU_DELTAN. */
int  iegpu_ens_download(struct iegpu_ens* ens, int lattice, int field, double* host);
/* The deltaN stage of every lattice, run_deltaN_loop (src/evolution.cpp:1291-1375)
 * with the leapfrog integrator, then saveN's Nmean and deltaN -= Nmean
 * (src/output.cpp:1522-1542): afterwards IEGPU_DELTAN holds zeta.
 * phiref[count] and nmean[count] may be NULL.  A site stops being integrated
 * once it has reached the end surface, so fd there is not advanced further. */
int  iegpu_ens_deltaN(struct iegpu_ens* ens, iegpu_bg* bg, double dN, double Nend, int use_phiref_manual,
                      double phiref_manual, double* phiref, float* nmean);
/* spectraN of every lattice (src/output.cpp:1140-1170): counts/f2 hold
 * lattice b's iegpu_numbins(N_b) bins after those of lattices 0 .. b-1. */
int  iegpu_ens_zeta_spectra(struct iegpu_ens* ens, int* counts, double* f2);
/* Pooled one-point histogram of zeta over the lattices of size N (0: all):
 * nbins bins over [-nsigma*sigma, +nsigma*sigma], sigma the pooled standard
 * deviation; outside[0], outside[1]: values below and above the range. */
int  iegpu_ens_zeta_histogram(struct iegpu_ens* ens, int N, int nbins, double nsigma, double* sigma, double* lo,
                              double* width, long long* counts, long long* outside);

#ifdef __cplusplus
}
#endif
#endif
