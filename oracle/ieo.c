/*
 * ieo.c -- CPU oracle for the InflationEasy lattice hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see ieo.h).  This is a restatement of the
 * algorithm of caravangelo/inflation-easy, written from its behaviour, in C
 * with an explicit state struct.  Floating-point expressions are evaluated in
 * exactly the order the reference evaluates them, and reductions run serially
 * in the reference's loop order, because the oracle is pinned bit-for-bit
 * against the reference program built from source (oracle/build_ref.py).
 * Compile with -ffp-contract=off: fused multiply-adds would change results.
 *
 * Parity: pinned (tests/test_oracle_pin.py compares the full results/ .dat
 * output and full-precision field dumps with the reference program).
 */
#include "ieo.h"

#include <errno.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx_d;
typedef struct { float re, im; } cplx_f;

struct ieo_state {
    ieo_params p;
    size_t gs;                 /* N^3 */
    double pi;                 /* 2*asin(1), src/main.h:26 */
    /* fields, src/main.cpp:16-29 */
    double *f, *fd, *deltaN, *fny, *fdny;
    float *h[6], *hd[6], *hny[6], *hdny[6];
    /* scalars, src/main.cpp:31-35 */
    double t, t0, a, ad, ad2, astep, Ne, phiref, hubble_init;
    /* table, src/main.cpp:38-43 */
    int ntab;
    double *tphi, *tV, *tdV;
    int *lstart;
    /* rand_uniform statics, src/initialize.cpp:18-31 */
    int rng_started, rng_next;
    /* set_mode statics, src/initialize.cpp:56-59 */
    int sm_started;
    double sm_norm, sm_hbterm;
    int err;
    char errmsg[512];
    /* RK scratch (allocated on first use), src/evolution.cpp:288-321 */
    double *ftmp, *fdtmp, *kf[7], *kfd[7];
    float *htmp[6], *hdtmp[6], *kh[7][6], *khd[7][6];
    double *dntmp, *kdn[7];   /* deltaN RK scratch (DeltaNRKScratch, src/evolution.cpp:1040-1059) */
    int rk_post;        /* post-inflation right-hand side (g_use_post_inflation_rhs) */
    double rk45_err;    /* error norm of the last RK45 attempt */
    int engine_arith;   /* the GPU engine's lattice-sum arithmetic (see ieo_set_engine_arith) */
};

static inline double pw2(double x) { return x * x; }

static void set_err(ieo_state* S, const char* fmt, ...) {
    if (S->err) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(S->errmsg, sizeof(S->errmsg), fmt, ap);
    va_end(ap);
    S->err = 1;
}

/* ------------------------------------------------------------------------- */
/* parameters                                                                */
/* ------------------------------------------------------------------------- */

/* src/runtime_parameters.cpp:17-112 */
void ieo_params_defaults(ieo_params* p, int N, int numerical) {
    memset(p, 0, sizeof(*p));
    p->N = N;
    p->numerical_potential = numerical;
    p->perform_deltaN = 1;
    p->calculate_SIGW = 0;
    p->criterion = numerical ? 1 : -1;
    p->seed = 8;
    p->rescale_s = 0.0;
    p->af = 2.0 * N;
    p->V0 = numerical ? 3e-9 : 3.338e-13;
    p->rescale_B = sqrt(p->V0);
    p->ns = 0.97;
    if (numerical) {
        p->initial_field = 2.9181235049318586;
        p->initial_derivative = -0.06727651095116181;
        p->L = 10.0;
        p->dt = 0.001;
        p->output_freq = 500;
        p->output_infrequent_freq = 500;
        p->dN = 0.0001;
        p->Nend = 5.0;
    } else {
        p->initial_field = 0.0935;
        p->initial_derivative = 0.000796;
        p->L = 10.0;
        p->dt = 0.0005;
        p->output_freq = 200;
        p->output_infrequent_freq = 200;
        p->dN = 0.0000001;
        p->Nend = 0.001;
    }
    p->use_phiref_manual = 0;
    p->phiref_manual_value = 0.0;
    /* post-inflation controls, src/runtime_parameters.cpp:48-52 (off here:
     * the reference switches the phase on at compile time) */
    p->post_inflation = 0;
    p->horizon_factor = 1.0;
    p->omega = 1.0 / 3.0;
    p->dt_post_inflation = 0.001;
    p->af_post_inflation = 2.0 * N;
    p->af_post_given = 0;
    p->inflation_integrator = 0;
    p->post_inflation_integrator = 0;
    p->deltaN_integrator = 0;
    p->rk45_abs_tol = 1e-8;
    p->rk45_rel_tol = 1e-6;
    p->rk45_min_dt = -1.0;
    p->rk45_max_dt = -1.0;
    p->rk45_safety = 0.9;
    p->rk45_min_given = 0;
    p->rk45_max_given = 0;
    p->high_cutoff_index = 0.0;
    p->low_cutoff_index = 0.0;
    p->forcing_cutoff = 0;
    p->output_spectra = 1;
    p->output_histogram = 1;
    p->output_energy = 1;
    p->output_box3D = 0;
    p->output_box2D = 0;
    p->screen_updates = 1;
    p->nbins = 256;
    p->int_err = 5;
    p->int_errN = 5;
    p->dx = p->L / (double)N;
}

/* src/runtime_parameters.cpp:342-354 */
void ieo_params_finalize(ieo_params* p, int rescale_B_given, int af_given) {
    if (!rescale_B_given) p->rescale_B = sqrt(p->V0);
    if (!af_given) p->af = 2.0 * p->N;
    if (!p->af_post_given) p->af_post_inflation = 2.0 * p->N;
    p->dx = p->L / (double)p->N;
    /* src/runtime_parameters.cpp:351-353 and sanitize_rk45_controls (:184-192) */
    if (!p->rk45_min_given || p->rk45_min_dt <= 0.0) p->rk45_min_dt = fabs(p->dt) * 1e-6;
    if (!p->rk45_max_given || p->rk45_max_dt <= 0.0) p->rk45_max_dt = fabs(p->dt);
    if (!(p->rk45_min_dt > 0.0)) p->rk45_min_dt = fabs(p->dt) * 1e-6;
    if (!(p->rk45_max_dt > 0.0)) p->rk45_max_dt = fabs(p->dt);
    if (p->rk45_min_dt <= 0.0) p->rk45_min_dt = 1e-16;
    if (p->rk45_max_dt < p->rk45_min_dt) p->rk45_max_dt = p->rk45_min_dt;
    if (!(p->rk45_abs_tol > 0.0)) p->rk45_abs_tol = 1e-8;
    if (!(p->rk45_rel_tol > 0.0)) p->rk45_rel_tol = 1e-6;
    if (!(p->rk45_safety > 0.0 && p->rk45_safety < 1.0)) p->rk45_safety = 0.9;
}

/* parse_integrator, src/runtime_parameters.cpp:141-166 */
static int parse_integrator(const char* val, int* out) {
    char lw[64];
    size_t q = 0;
    for (; val[q] && q < sizeof lw - 1; ++q) lw[q] = (char)((val[q] >= 'A' && val[q] <= 'Z') ? val[q] + 32 : val[q]);
    lw[q] = 0;
    if (!strcmp(lw, "leapfrog") || !strcmp(lw, "lf")) { *out = 0; return 1; }
    if (!strcmp(lw, "rk4")) { *out = 1; return 1; }
    if (!strcmp(lw, "rk45") || !strcmp(lw, "rkf45") || !strcmp(lw, "dopri5")) { *out = 2; return 1; }
    char* end;
    const long v = strtol(val, &end, 10);
    if (end != val && !*end && v >= 0 && v <= 2) { *out = (int)v; return 1; }
    return 0;
}

static char* trim(char* s) {
    while (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\n' || *s == '\f' || *s == '\v') ++s;
    char* e = s + strlen(s);
    while (e > s && (e[-1] == ' ' || e[-1] == '\t' || e[-1] == '\r' || e[-1] == '\n' || e[-1] == '\f' || e[-1] == '\v')) --e;
    *e = 0;
    return s;
}

static int parse_d(const char* v, double* out) {
    char* end;
    errno = 0;
    double x = strtod(v, &end);
    if (end == v || errno) return 0;
    while (*end == ' ' || *end == '\t') ++end;
    if (*end) return 0;
    *out = x;
    return 1;
}

static int parse_i(const char* v, int* out) {
    char* end;
    errno = 0;
    long x = strtol(v, &end, 10);
    if (end == v || errno) return 0;
    while (*end == ' ' || *end == '\t') ++end;
    if (*end) return 0;
    *out = (int)x;
    return 1;
}

/* src/runtime_parameters.cpp:195-365.  N and the feature switches are accepted
 * as keys here because the oracle takes them at run time. */
int ieo_params_load(ieo_params* p, const char* path) {
    FILE* fp = fopen(path, "r");
    if (!fp) {
        ieo_params_finalize(p, 0, 0);
        return -1;
    }
    int B_given = 0, af_given = 0;
    char buf[4096];
    while (fgets(buf, sizeof buf, fp)) {
        char* hash = strchr(buf, '#');
        if (hash) *hash = 0;
        char* line = trim(buf);
        if (!*line) continue;
        char* eq = strchr(line, '=');
        if (!eq) continue;
        *eq = 0;
        char* key = trim(line);
        char* val = trim(eq + 1);
        double d; int i;
#define KD(name, field) else if (!strcmp(key, name) && parse_d(val, &d)) p->field = d;
#define KI(name, field) else if (!strcmp(key, name) && parse_i(val, &i)) p->field = i;
#define KB(name, field) else if (!strcmp(key, name) && parse_i(val, &i)) p->field = (i != 0);
        if (0) {}
        KI("seed", seed)
        KD("rescale_s", rescale_s)
        else if (!strcmp(key, "af") && parse_d(val, &d)) { p->af = d; af_given = 1; }
        KD("V0", V0)
        else if (!strcmp(key, "rescale_B") && parse_d(val, &d)) { p->rescale_B = d; B_given = 1; }
        KD("ns", ns)
        KD("initial_field", initial_field)
        KD("initial_derivative", initial_derivative)
        KD("L", L)
        KD("dt", dt)
        KI("output_freq", output_freq)
        KI("output_infrequent_freq", output_infrequent_freq)
        KD("dN", dN)
        KD("Nend", Nend)
        KB("use_phiref_manual", use_phiref_manual)
        KD("phiref_manual_value", phiref_manual_value)
        KD("high_cutoff_index", high_cutoff_index)
        KD("low_cutoff_index", low_cutoff_index)
        KB("forcing_cutoff", forcing_cutoff)
        KB("output_spectra", output_spectra)
        KB("output_histogram", output_histogram)
        KB("output_energy", output_energy)
        KB("output_box3D", output_box3D)
        KB("output_box2D", output_box2D)
        KB("screen_updates", screen_updates)
        KI("nbins", nbins)
        else if (!strcmp(key, "int_err") && parse_i(val, &i)) p->int_err = i < 1 ? 1 : i;
        else if (!strcmp(key, "int_errN") && parse_i(val, &i)) p->int_errN = i < 1 ? 1 : i;
        KI("N", N)
        KB("numerical_potential", numerical_potential)
        KB("perform_deltaN", perform_deltaN)
        KB("calculate_SIGW", calculate_SIGW)
        KI("criterion", criterion)
        KB("post_inflation", post_inflation)
        KD("horizon_factor", horizon_factor)
        KD("omega", omega)
        KD("dt_post_inflation", dt_post_inflation)
        else if (!strcmp(key, "af_post_inflation") && parse_d(val, &d)) { p->af_post_inflation = d; p->af_post_given = 1; }
        else if (!strcmp(key, "inflation_integrator")) parse_integrator(val, &p->inflation_integrator);
        else if (!strcmp(key, "post_inflation_integrator")) parse_integrator(val, &p->post_inflation_integrator);
        else if (!strcmp(key, "deltaN_integrator")) parse_integrator(val, &p->deltaN_integrator);
        KD("rk45_abs_tol", rk45_abs_tol)
        KD("rk45_rel_tol", rk45_rel_tol)
        else if (!strcmp(key, "rk45_min_dt") && parse_d(val, &d)) { p->rk45_min_dt = d; p->rk45_min_given = 1; }
        else if (!strcmp(key, "rk45_max_dt") && parse_d(val, &d)) { p->rk45_max_dt = d; p->rk45_max_given = 1; }
        KD("rk45_safety", rk45_safety)
#undef KD
#undef KI
#undef KB
    }
    fclose(fp);
    ieo_params_finalize(p, B_given, af_given);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* state                                                                     */
/* ------------------------------------------------------------------------- */

void ieo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static int g_engine_arith_default = 0;

void ieo_set_engine_arith_default(int on) { g_engine_arith_default = on != 0; }

ieo_state* ieo_create(const ieo_params* p) {
    ieo_state* S = (ieo_state*)calloc(1, sizeof(ieo_state));
    if (!S) return NULL;
    S->engine_arith = g_engine_arith_default;
    S->p = *p;
    S->p.dx = p->L / (double)p->N;
    const size_t N = (size_t)p->N;
    S->gs = N * N * N;
    S->pi = 2.0 * asin(1.0);
    S->f = (double*)calloc(S->gs, sizeof(double));
    S->fd = (double*)calloc(S->gs, sizeof(double));
    S->deltaN = (double*)calloc(S->gs, sizeof(double));
    S->fny = (double*)calloc(N * 2 * N, sizeof(double));
    S->fdny = (double*)calloc(N * 2 * N, sizeof(double));
    if (p->calculate_SIGW) {
        for (int c = 0; c < 6; ++c) {
            S->h[c] = (float*)calloc(S->gs, sizeof(float));
            S->hd[c] = (float*)calloc(S->gs, sizeof(float));
            S->hny[c] = (float*)calloc(N * 2 * N, sizeof(float));
            S->hdny[c] = (float*)calloc(N * 2 * N, sizeof(float));
        }
    }
    S->lstart = (int*)calloc(S->gs, sizeof(int));
    S->astep = 1.0; S->a = 1.0; S->ad = 0.0; S->ad2 = 0.0; S->Ne = 0.0;
    S->t = 0.0; S->t0 = 0.0; S->phiref = 0.0; S->hubble_init = 0.0;
    return S;
}

void ieo_destroy(ieo_state* S) {
    if (!S) return;
    free(S->f); free(S->fd); free(S->deltaN); free(S->fny); free(S->fdny);
    for (int c = 0; c < 6; ++c) { free(S->h[c]); free(S->hd[c]); free(S->hny[c]); free(S->hdny[c]); }
    free(S->tphi); free(S->tV); free(S->tdV); free(S->lstart);
    free(S->ftmp); free(S->fdtmp);
    for (int q = 0; q < 7; ++q) { free(S->kf[q]); free(S->kfd[q]); free(S->kdn[q]); }
    free(S->dntmp);
    for (int c = 0; c < 6; ++c) {
        free(S->htmp[c]); free(S->hdtmp[c]);
        for (int q = 0; q < 7; ++q) { free(S->kh[q][c]); free(S->khd[q][c]); }
    }
    free(S);
}

const ieo_params* ieo_get_params(const ieo_state* S) { return &S->p; }
double* ieo_f(ieo_state* S) { return S->f; }
double* ieo_fd(ieo_state* S) { return S->fd; }
double* ieo_deltaN(ieo_state* S) { return S->deltaN; }
double* ieo_fnyquist(ieo_state* S) { return S->fny; }
double* ieo_fdnyquist(ieo_state* S) { return S->fdny; }
float* ieo_h(ieo_state* S, int c) { return S->h[c]; }
float* ieo_hd(ieo_state* S, int c) { return S->hd[c]; }
const char* ieo_last_error(const ieo_state* S) { return S->err ? S->errmsg : ""; }

void ieo_get_scalars(const ieo_state* S, ieo_scalars* o) {
    o->t = S->t; o->a = S->a; o->ad = S->ad; o->ad2 = S->ad2; o->astep = S->astep;
    o->Ne = S->Ne; o->phiref = S->phiref; o->hubble_init = S->hubble_init;
}
void ieo_set_scalars(ieo_state* S, const ieo_scalars* i) {
    S->t = i->t; S->a = i->a; S->ad = i->ad; S->ad2 = i->ad2; S->astep = i->astep;
    S->Ne = i->Ne; S->phiref = i->phiref; S->hubble_init = i->hubble_init;
}

int ieo_set_table(ieo_state* S, const double* phi, const double* V, const double* dV, int n) {
    free(S->tphi); free(S->tV); free(S->tdV);
    S->tphi = (double*)malloc(sizeof(double) * n);
    S->tV = (double*)malloc(sizeof(double) * n);
    S->tdV = (double*)malloc(sizeof(double) * n);
    memcpy(S->tphi, phi, sizeof(double) * n);
    memcpy(S->tV, V, sizeof(double) * n);
    memcpy(S->tdV, dV, sizeof(double) * n);
    S->ntab = n;
    return 0;
}

static inline size_t IDX(int N, int i, int j, int k) {
    return ((size_t)i * N + (size_t)j) * N + (size_t)k;
}

/* ------------------------------------------------------------------------- */
/* potential, src/potential.cpp                                              */
/* ------------------------------------------------------------------------- */

/* find_bracketing_index, src/potential.cpp:11-50.  Returns -1 on error. */
static int bracket(ieo_state* S, double v, int start) {
    const int n = S->ntab;
    const double* x = S->tphi;
    if (n < 2) { set_err(S, "Numerical potential table must contain at least two points.\n"); return -1; }
    if (v > x[0] || v < x[n - 1]) {
        set_err(S, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v, x[n - 1], x[0]);
        return -1;
    }
    if (start <= 1) {
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
            const int mid = lo + (hi - lo) / 2;
            if (x[mid] >= v) lo = mid; else hi = mid;
        }
        return hi;
    }
    int l = start < 1 ? 1 : (start > n - 1 ? n - 1 : start);
    while (l < n && x[l] >= v) ++l;
    while (l > 1 && x[l - 1] < v) --l;
    if (l <= 0 || l >= n) { set_err(S, "Interpolation index out of bounds for field value %.17g.\n", v); return -1; }
    return l;
}

/* interpolate_from_table, src/potential.cpp:52-68 */
static double interp(ieo_state* S, double v, int l, const double* y) {
    const double x0 = S->tphi[l - 1], x1 = S->tphi[l];
    const double y0 = y[l - 1], y1 = y[l];
    if (x0 == x1) { set_err(S, "Interpolation failed due to repeated field grid points.\n"); return 0.0; }
    return y1 + (v - x1) * (y0 - y1) / (x0 - x1);
}

/* analytic hilltop, src/potential.cpp:77-83 */
static inline double hill_V(const ieo_params* p, double v) {
    return p->V0 * (1.0 - (1.0 - p->ns) / 4.0 * pw2(v)) / pw2(p->rescale_B);
}
static inline double hill_dV(const ieo_params* p, double v) {
    return -p->V0 * (1.0 - p->ns) / 2.0 * v / pw2(p->rescale_B);
}

/* potential(), src/potential.cpp:91-98 */
double ieo_potential(ieo_state* S, double v) {
    if (S->p.numerical_potential) {
        const int l = bracket(S, v, 1);
        if (l < 0) return 0.0;
        return interp(S, v, l, S->tV) / pw2(S->p.rescale_B);
    }
    return hill_V(&S->p, v);
}


/* ------------------------------------------------------------------------- */
/* exact sums (engine-arithmetic mode)                                       */
/* ------------------------------------------------------------------------- */

/* A fixed-point accumulator over the whole double range and the range of
 * products of two doubles (a "long accumulator", Kulisch): 32-bit chunks
 * held in signed 64-bit limbs, least significant bit 2^-2150, so every finite
 * double and every exact product of two finite doubles is added without
 * error.  The total is rounded once to the nearest double, ties to even
 * (subnormal results at 2^-1074).  This is an independent restatement of what
 * the GPU engine's exact sums compute (the correctly rounded exact sum);
 * Python's math.fsum gives the same value for sums of doubles. */
#define XS_LIMBS 136   /* up to 2^(4352 - 2150): every product of two finite doubles */
#define XS_SUBNORMAL_LSB 1076   /* bit position of 2^-1074 */
typedef struct { int64_t l[XS_LIMBS]; long count; int nonfinite; } xsum_t;

static void xs_init(xsum_t* X) { memset(X, 0, sizeof *X); }

static void xs_norm(xsum_t* X) {
    int64_t carry = 0;
    for (int k = 0; k < XS_LIMBS; ++k) {
        const int64_t v = X->l[k] + carry;
        const int64_t lo = v & 0xFFFFFFFFLL;
        carry = (v - lo) / 4294967296LL;   /* exact: v - lo is a multiple of 2^32 */
        X->l[k] = lo;
    }
    X->l[XS_LIMBS - 1] += carry * 4294967296LL;
    X->count = 0;
}

/* adds (negative ? -1 : 1) * v * 2^(pos - 2150) for v < 2^107 */
static void xs_add_bits(xsum_t* X, unsigned __int128 v, int pos, int negative) {
    const int k = pos >> 5, r = pos & 31;
    unsigned __int128 w = v;
    int64_t c[5];
    /* chunks of v << r: at most 107 + 31 = 138 bits, five 32-bit chunks */
    c[0] = (int64_t)(uint64_t)((w << r) & 0xFFFFFFFFu);
    w >>= (32 - r);
    for (int q = 1; q < 5; ++q) {
        c[q] = (int64_t)(uint64_t)(w & 0xFFFFFFFFu);
        w >>= 32;
    }
    for (int q = 0; q < 5; ++q) {
        if (negative) X->l[k + q] -= c[q];
        else X->l[k + q] += c[q];
    }
    if (++X->count >= (1L << 29)) xs_norm(X);
}

static void xs_add(xsum_t* X, double t) {
    uint64_t b;
    memcpy(&b, &t, sizeof b);
    int e = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0x000FFFFFFFFFFFFFULL;
    if (e == 0x7FF) { X->nonfinite = 1; return; }
    if (e == 0) { if (!m) return; e = 1; } else m |= 1ULL << 52;
    xs_add_bits(X, (unsigned __int128)m, e + 1075, (int)(b >> 63));
}

/* adds the exact product x y */
static void xs_add_product(xsum_t* X, double x, double y) {
    uint64_t bx, by;
    memcpy(&bx, &x, sizeof bx);
    memcpy(&by, &y, sizeof by);
    int ex = (int)((bx >> 52) & 0x7FF), ey = (int)((by >> 52) & 0x7FF);
    if (ex == 0x7FF || ey == 0x7FF) { X->nonfinite = 1; return; }
    uint64_t mx = bx & 0x000FFFFFFFFFFFFFULL, my = by & 0x000FFFFFFFFFFFFFULL;
    if (ex) mx |= 1ULL << 52; else ex = 1;
    if (ey) my |= 1ULL << 52; else ey = 1;
    if (!mx || !my) return;
    xs_add_bits(X, (unsigned __int128)mx * my, ex + ey, (int)((bx ^ by) >> 63));
}

static void xs_merge(xsum_t* X, const xsum_t* Y) {
    for (int k = 0; k < XS_LIMBS; ++k) X->l[k] += Y->l[k];
    X->nonfinite |= Y->nonfinite;
    X->count += Y->count;
    if (X->count >= (1L << 29)) xs_norm(X);
}

static double xs_round(xsum_t* X) {
    if (X->nonfinite) return NAN;
    xs_norm(X);
    int neg = X->l[XS_LIMBS - 1] < 0;
    uint32_t w[XS_LIMBS];
    if (neg) {   /* magnitude of the two's-complement value in 32-bit chunks */
        int64_t borrow = 0;
        for (int k = 0; k < XS_LIMBS; ++k) {
            int64_t v = -X->l[k] - borrow;
            borrow = 0;
            while (v < 0) { v += 4294967296LL; ++borrow; }
            w[k] = (uint32_t)v;
        }
    } else {
        for (int k = 0; k < XS_LIMBS; ++k) w[k] = (uint32_t)X->l[k];
    }
    int top = -1;
    for (int k = XS_LIMBS - 1; k >= 0 && top < 0; --k)
        if (w[k]) { int q = 31; while (!((w[k] >> q) & 1u)) --q; top = 32 * k + q; }
    if (top < 0) return 0.0;
#define XS_BIT(p) ((p) < 0 ? 0u : ((w[(p) >> 5] >> ((p) & 31)) & 1u))
    int lsb = top - 52;
    if (lsb < XS_SUBNORMAL_LSB) lsb = XS_SUBNORMAL_LSB;   /* subnormal results: 2^-1074 steps */
    uint64_t M = 0;
    for (int p = top; p >= lsb; --p) M = (M << 1) | XS_BIT(p);
    const unsigned rb = XS_BIT(lsb - 1);
    int sticky = 0;
    for (int p = lsb - 2; p >= 0 && !sticky; --p) sticky = XS_BIT(p) != 0;
    if (rb && (sticky || (M & 1u))) {
        M += 1;
        if (M >> 53) { M >>= 1; lsb += 1; }
    }
#undef XS_BIT
    const double v = ldexp((double)M, lsb - 2150);
    return neg ? -v : v;
}

/* The correctly rounded exact sum of x[0..n). */
double ieo_exact_sum(const double* x, size_t n) {
    xsum_t X;
    xs_init(&X);
    for (size_t i = 0; i < n; ++i) xs_add(&X, x[i]);
    return xs_round(&X);
}

/* The correctly rounded exact sum of the exact products x[i] y[i]. */
double ieo_exact_dot(const double* x, const double* y, size_t n) {
    xsum_t X;
    xs_init(&X);
    for (size_t i = 0; i < n; ++i) xs_add_product(&X, x[i], y[i]);
    return xs_round(&X);
}

void ieo_set_engine_arith(ieo_state* S, int on) { S->engine_arith = on != 0; }

/* pow(x, y) as the engine evaluates the Friedmann update's powers: exact
 * products and quotients for y = 0, 1, 2, -1, libm pow otherwise. */
static double eng_pow(const ieo_state* S, double x, double y) {
    if (!S->engine_arith) return pow(x, y);
    if (y == 0.0) return 1.0;
    if (y == 1.0) return x;
    if (y == 2.0) return x * x;
    if (y == -1.0) return 1.0 / x;
    return pow(x, y);
}

/* potential_derivative(i,j,k), src/potential.cpp:103-112 */
static inline double pot_deriv_site(ieo_state* S, size_t id) {
    if (S->p.numerical_potential) {
        const int l = bracket(S, S->f[id], S->lstart[id]);
        if (l < 0) return 0.0;
        S->lstart[id] = (l - S->p.int_err) > 1 ? (l - S->p.int_err) : 1;
        return interp(S, S->f[id], l, S->tdV) / pw2(S->p.rescale_B);
    }
    return hill_dV(&S->p, S->f[id]);
}

/* The engine's potential sum: exact sum f^2 (hilltop, then
 * V0 (N^3 - c1 sum) / B^2 / N^3) or exact sum of V + (v - x_l) slope_l
 * (table, then sum / B^2 / N^3), slope_l = (V_{l-1} - V_l)/(x_{l-1} - x_l). */
static double potential_energy_engine(ieo_state* S) {
    const size_t gs = S->gs;
    const long n = (long)gs;
    const double* f = S->f;
    xsum_t tot;
    xs_init(&tot);
    int bad = 0;
    #pragma omp parallel
    {
        xsum_t X;
        xs_init(&X);
        #pragma omp for schedule(static) reduction(|:bad)
        for (long id = 0; id < n; ++id) {
            const double v = f[id];
            if (S->p.numerical_potential) {
                const int l = bracket(S, v, 1);
                if (l < 0) { bad = 1; continue; }
                const double slope = (S->tV[l - 1] - S->tV[l]) / (S->tphi[l - 1] - S->tphi[l]);
                xs_add(&X, S->tV[l] + (v - S->tphi[l]) * slope);
            } else {
                xs_add_product(&X, v, v);
            }
        }
        #pragma omp critical
        xs_merge(&tot, &X);
    }
    if (bad) return 0.0;
    const double Pn = xs_round(&tot);
    const double g = (double)gs, B2 = pw2(S->p.rescale_B);
    if (S->p.numerical_potential) return (Pn / B2) / g;
    const double c1 = (1.0 - S->p.ns) / 4.0;
    return (S->p.V0 * (g - c1 * Pn) / B2) / g;
}

/* potential_energy(), src/potential.cpp:151-171 (serial) */
double ieo_potential_energy(ieo_state* S) {
    if (S->engine_arith) return potential_energy_engine(S);
    double pot = 0.0;
    const size_t gs = S->gs;
    if (S->p.numerical_potential) {
        for (size_t id = 0; id < gs; ++id) {
            const int l = bracket(S, S->f[id], S->lstart[id]);
            if (l < 0) return 0.0;
            pot += interp(S, S->f[id], l, S->tV) / pw2(S->p.rescale_B);
            S->lstart[id] = (l - S->p.int_err) > 1 ? (l - S->p.int_err) : 1;
        }
    } else {
        for (size_t id = 0; id < gs; ++id) pot += ieo_potential(S, S->f[id]);
    }
    pot /= (double)gs;
    return pot;
}

/* pot_ratio(i,j,k), src/potential.cpp:177-192 */
static inline double pot_ratio_site(ieo_state* S, size_t id) {
    double pot, der;
    if (S->p.numerical_potential) {
        const int l = bracket(S, S->f[id], S->lstart[id]);
        if (l < 0) return 0.0;
        pot = interp(S, S->f[id], l, S->tV);
        der = interp(S, S->f[id], l, S->tdV);
        S->lstart[id] = (l - S->p.int_errN) > 1 ? (l - S->p.int_errN) : 1;
    } else {
        pot = hill_V(&S->p, S->f[id]);
        der = hill_dV(&S->p, S->f[id]);
    }
    return der / pot;
}

/* ------------------------------------------------------------------------- */
/* RNG and initial conditions, src/initialize.cpp                            */
/* ------------------------------------------------------------------------- */

/* Park-Miller minimal standard generator with Schrage's factorisation and a
 * 99-call warm-up, src/initialize.cpp:13-31. */
static void rng_advance(ieo_state* S) {
    S->rng_next = 16807 * (S->rng_next % 127773) - 2836 * (S->rng_next / 127773);
    if (S->rng_next < 0) S->rng_next += 2147483647;
}

double ieo_rand_uniform(ieo_state* S) {
    if (S->p.seed < 1) return 0.33;
    if (!S->rng_started) {
        S->rng_next = S->p.seed;
    }
    if (!(S->rng_next > 0)) {
        printf("Invalid seed used in random number function. Using seed=1\n");
        S->rng_next = 1;
    }
    if (!S->rng_started) {
        S->rng_started = 1;
        for (int w = 1; w < 100; ++w) rng_advance(S);
    }
    rng_advance(S);
    return (double)S->rng_next / (double)2147483647;
}

/* set_mode, src/initialize.cpp:53-89 (its statics live in the state) */
static void set_mode(ieo_state* S, double p2, double p2lat, double m2, double* field, double* deriv, int real) {
    double phase, amplitude, rms_amplitude, omega;
    double re_f_left, im_f_left;
    const ieo_params* p = &S->p;
    if (!S->sm_started) {
        S->sm_norm = p->rescale_B * pow(p->L / pw2(p->dx), 1.5);
        S->sm_hbterm = -S->hubble_init;
        S->sm_started = 1;
    }
    const double ii = p->L / (2.0 * S->pi) * sqrt(p2lat);
    omega = (p2 + m2 > 0.0) ? sqrt(p2 + m2) : sqrt(p2);
    rms_amplitude = (omega > 0.0) ? S->sm_norm / sqrt(2.0 * omega) : 0.0;
    if (p->high_cutoff_index > 0 && (ii > p->high_cutoff_index || ii < p->low_cutoff_index)) rms_amplitude = 0.0;
    amplitude = rms_amplitude * sqrt(log(1.0 / ieo_rand_uniform(S)));
    phase = 2.0 * S->pi * ieo_rand_uniform(S);
    re_f_left = amplitude * cos(phase);
    im_f_left = amplitude * sin(phase);
    field[0] = re_f_left;
    field[1] = im_f_left;
    deriv[0] = omega * im_f_left + S->sm_hbterm * field[0];
    deriv[1] = -omega * re_f_left + S->sm_hbterm * field[1];
    if (real == 1) { field[1] = 0.0; deriv[1] = 0.0; }
}

/* initialize(), src/initialize.cpp:93-114 */
int ieo_initialize(ieo_state* S) {
    const ieo_params* p = &S->p;
    if (p->dt > p->dx / sqrt(3.0)) {
        set_err(S, "Time step too large. Courant condition violated: dt/dx = %f\n", p->dt / p->dx);
        return 1;
    }
    S->t0 = 0.0;
    S->hubble_init = sqrt(ieo_potential(S, p->initial_field) / 3.0);
    if (S->err) return 1;
    S->ad = S->hubble_init;
    memset(S->lstart, 0, sizeof(int) * S->gs);
    return 0;
}

/* initializef(), src/initialize.cpp:118-214 */
int ieo_initializef(ieo_state* S) {
    const ieo_params* p = &S->p;
    const int N = p->N;
    const double pi = S->pi;
    double* f = S->f;
    double* fd = S->fd;
    double p2, p2lat, mass_sq = 0.0;
    const double dp2 = pw2(2.0 * pi / p->L);
    int i, j, k, iconj, jconj;
    double px, py, pz;

    if (p->dt > p->dx / sqrt(3.0)) {
        set_err(S, "Time step too large. Courant condition violated: dt/dx = %f\n", p->dt / p->dx);
        return 1;
    }
    memset(f, 0, sizeof(double) * S->gs);
    memset(fd, 0, sizeof(double) * S->gs);
    S->hubble_init = sqrt((0.5 * pw2(p->initial_derivative) + ieo_potential(S, p->initial_field)) / 3.0);
    if (S->err) return 1;
    S->ad = S->hubble_init;

    double (*fny)[2] = (double (*)[2])S->fny;      /* element [i*N + j] = fny[i][2j..2j+1] */
    double (*fdny)[2] = (double (*)[2])S->fdny;
    const double NL = (double)N / p->L;
    for (i = 0; i < N; i++) {
        px = (i <= N / 2 ? i : i - N);
        iconj = (i == 0 ? 0 : N - i);
        for (j = 0; j < N; j++) {
            py = (j <= N / 2 ? j : j - N);
            for (k = 1; k < N / 2; k++) {
                pz = k;
                p2lat = dp2 * (pw2(px) + pw2(py) + pw2(pz));
                p2 = 4.0 * pw2(NL) * (pw2(sin(px * pi / N)) + pw2(sin(py * pi / N)) + pw2(sin(pz * pi / N)));
                set_mode(S, p2, p2lat, mass_sq, &f[IDX(N, i, j, 2 * k)], &fd[IDX(N, i, j, 2 * k)], 0);
            }
            if (j > N / 2 || (i > N / 2 && (j == 0 || j == N / 2))) {
                jconj = (j == 0 ? 0 : N - j);
                p2lat = dp2 * (pw2(px) + pw2(py));
                p2 = 4.0 * pw2(NL) * (pw2(sin(px * pi / N)) + pw2(sin(py * pi / N)));
                set_mode(S, p2, p2lat, mass_sq, &f[IDX(N, i, j, 0)], &fd[IDX(N, i, j, 0)], 0);
                f[IDX(N, iconj, jconj, 0)] = f[IDX(N, i, j, 0)];
                f[IDX(N, iconj, jconj, 1)] = -f[IDX(N, i, j, 1)];
                fd[IDX(N, iconj, jconj, 0)] = fd[IDX(N, i, j, 0)];
                fd[IDX(N, iconj, jconj, 1)] = -fd[IDX(N, i, j, 1)];
                p2lat = dp2 * (pw2(px) + pw2(py) + pw2(N / 2));
                p2 = 4.0 * pw2(NL) * (pw2(sin(px * pi / N)) + pw2(sin(py * pi / N)) + 1.0);
                set_mode(S, p2, p2lat, mass_sq, fny[(size_t)i * N + j], fdny[(size_t)i * N + j], 0);
                fny[(size_t)iconj * N + jconj][0] = fny[(size_t)i * N + j][0];
                fny[(size_t)iconj * N + jconj][1] = -fny[(size_t)i * N + j][1];
                fdny[(size_t)iconj * N + jconj][0] = fdny[(size_t)i * N + j][0];
                fdny[(size_t)iconj * N + jconj][1] = -fdny[(size_t)i * N + j][1];
            } else if ((i == 0 || i == N / 2) && (j == 0 || j == N / 2)) {
                p2lat = dp2 * (pw2(px) + pw2(py));
                p2 = 4.0 * pw2(NL) * (pw2(sin(px * pi / N)) + pw2(sin(py * pi / N)));
                if (p2 > 0.0) set_mode(S, p2, p2lat, mass_sq, &f[IDX(N, i, j, 0)], &fd[IDX(N, i, j, 0)], 1);
                p2lat = dp2 * (pw2(px) + pw2(py) + pw2(N / 2));
                p2 = 4.0 * pw2(NL) * (pw2(sin(px * pi / N)) + pw2(sin(py * pi / N)) + 1.0);
                set_mode(S, p2, p2lat, mass_sq, fny[(size_t)i * N + j], fdny[(size_t)i * N + j], 1);
            }
        }
    }
    f[0] = 0.0; f[1] = 0.0; fd[0] = 0.0; fd[1] = 0.0;

    ieo_fftrn_d(f, S->fny, N, -1);
    ieo_fftrn_d(fd, S->fdny, N, -1);

    for (size_t id = 0; id < S->gs; ++id) {
        f[id] += p->initial_field;
        fd[id] += p->initial_derivative;
    }
    double vard = 0.0;
    for (size_t id = 0; id < S->gs; ++id) vard += pw2(fd[id]);
    const double deriv_energy_in = 0.5 * vard / (double)S->gs;
    const double pe = ieo_potential_energy(S);
    if (S->err) return 1;
    const double ge = ieo_gradient_energy(S);
    S->hubble_init = sqrt((deriv_energy_in + pe + ge) / 3.0);
    S->ad = S->hubble_init;
    return 0;
}

/* initializeGW(), src/initialize.cpp:236-243 */
void ieo_initializeGW(ieo_state* S) {
    if (!S->p.calculate_SIGW) return;
    for (int c = 0; c < 6; ++c) {
        memset(S->h[c], 0, sizeof(float) * S->gs);
        memset(S->hd[c], 0, sizeof(float) * S->gs);
    }
}

/* ------------------------------------------------------------------------- */
/* leapfrog, src/evolution.cpp                                               */
/* ------------------------------------------------------------------------- */

/* lapl<double>, src/evolution.cpp:34-51: (k+1)+(k-1)+(j+1)+(j-1)+(i+1)+(i-1)-6f */
#define LAPL_AT(T, F, N, i, j, k, ip, im, jp, jm, kp, km)                    \
    ((F)[IDX(N, i, j, kp)] + (F)[IDX(N, i, j, km)] + (F)[IDX(N, i, jp, k)] +  \
     (F)[IDX(N, i, jm, k)] + (F)[IDX(N, ip, j, k)] + (F)[IDX(N, im, j, k)] -   \
     (T)6 * (F)[IDX(N, i, j, k)])

/* The engine's gradient sum: G = exact sum f lapl(f), gradient = -G. */
static double gradient_energy_engine(ieo_state* S) {
    const int N = S->p.N;
    const double* f = S->f;
    xsum_t tot;
    xs_init(&tot);
    #pragma omp parallel
    {
        xsum_t X;
        xs_init(&X);
        #pragma omp for schedule(static)
        for (int i = 0; i < N; ++i) {
            const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
            for (int j = 0; j < N; ++j) {
                const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
                for (int k = 0; k < N; ++k) {
                    const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                    xs_add_product(&X, f[IDX(N, i, j, k)], LAPL_AT(double, f, N, i, j, k, ip, im, jp, jm, kp, km));
                }
            }
        }
        #pragma omp critical
        xs_merge(&tot, &X);
    }
    const double gradient = -xs_round(&tot);
    const double norm = pw2(1.0 / (S->a * S->p.dx));
    return 0.5 * gradient * norm / (double)S->gs;
}

/* gradient_energy(), src/evolution.cpp:130-136 (serial) */
double ieo_gradient_energy(ieo_state* S) {
    if (S->engine_arith) return gradient_energy_engine(S);
    const int N = S->p.N;
    const double* f = S->f;
    double gradient = 0.0;
    const double norm = pw2(1.0 / (S->a * S->p.dx));
    for (int i = 0; i < N; ++i) {
        const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
        for (int j = 0; j < N; ++j) {
            const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
            for (int k = 0; k < N; ++k) {
                const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                gradient -= f[IDX(N, i, j, k)] * LAPL_AT(double, f, N, i, j, k, ip, im, jp, jm, kp, km);
            }
        }
    }
    return 0.5 * gradient * norm / (double)S->gs;
}

/* kin_energy(), src/evolution.cpp:139-145 */
double ieo_kin_energy(ieo_state* S) {
    double e = 0.0;
    if (S->engine_arith) {
        xsum_t X;
        xs_init(&X);
        for (size_t id = 0; id < S->gs; ++id) xs_add_product(&X, S->fd[id], S->fd[id]);
        e = xs_round(&X);
    } else {
        for (size_t id = 0; id < S->gs; ++id) e += pw2(S->fd[id]);
    }
    e /= (double)S->gs;
    return 0.5 * pow(S->a, 2.0 * S->p.rescale_s - 2.0) * e;
}

/* evolve_derivs(d), src/evolution.cpp:150-257 */
int ieo_evolve_derivs(ieo_state* S, double d) {
    const ieo_params* p = &S->p;
    const int N = p->N;
    const double s = p->rescale_s;
    const double laplnorm = eng_pow(S, S->a, -2.0 * s) / pw2(p->dx);
    const double sfev1 = s + 1.0;
    const double sfev2 = -2.0 * s + 2.0;

    const double ge = ieo_gradient_energy(S);
    const double pe = ieo_potential_energy(S);
    if (S->err) return 1;
    S->ad2 = (-2.0 * S->ad - 2.0 * S->a / d / sfev1 * (
        1.0 - sqrt(1.0 + 2.0 * d * sfev1 * S->ad / S->a +
        pw2(d) * sfev1 * eng_pow(S, S->a, sfev2) * (2.0 * ge / 3.0 + pe)))) / d;
    S->ad += 0.5 * d * S->ad2;

    const double friction = (2.0 + s) * S->ad / S->a;
    const double potnorm = eng_pow(S, S->a, 2.0 - 2.0 * s);
    double* f = S->f;
    double* fd = S->fd;

    #pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
        for (int j = 0; j < N; ++j) {
            const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
            for (int k = 0; k < N; ++k) {
                const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                const size_t id = IDX(N, i, j, k);
                fd[id] += d * (laplnorm * LAPL_AT(double, f, N, i, j, k, ip, im, jp, jm, kp, km)
                               - friction * fd[id]
                               - potnorm * pot_deriv_site(S, id));
            }
        }
    }
    if (S->err) return 1;

    if (p->calculate_SIGW) {
        const double srcAmp = 2.0 * eng_pow(S, S->a, -2.0 * s);
        const double half_over_dx = 0.5 / p->dx;
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
            for (int j = 0; j < N; ++j) {
                const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
                for (int k = 0; k < N; ++k) {
                    const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                    const size_t id = IDX(N, i, j, k);
                    /* dfdx<double>, src/evolution.cpp:55-77 */
                    const double gx = (f[IDX(N, ip, j, k)] - f[IDX(N, im, j, k)]) * half_over_dx;
                    const double gy = (f[IDX(N, i, jp, k)] - f[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gz = (f[IDX(N, i, j, kp)] - f[IDX(N, i, j, km)]) * half_over_dx;
                    const double T[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
                    for (int c = 0; c < 6; ++c) {
                        const float* h = S->h[c];
                        const float lapf = LAPL_AT(float, h, N, i, j, k, ip, im, jp, jm, kp, km);
                        const double lap_h = (double)lapf;
                        const double rhs = d * (laplnorm * lap_h - friction * (double)S->hd[c][id] + srcAmp * T[c]);
                        S->hd[c][id] += (float)rhs;
                    }
                }
            }
        }
    }
    S->ad += 0.5 * d * S->ad2;
    return 0;
}

/* evolve_fields(d), src/evolution.cpp:260-284 */
void ieo_evolve_fields(ieo_state* S, double d) {
    S->t += d;
    double* f = S->f;
    const double* fd = S->fd;
    const long gs = (long)S->gs;
    #pragma omp parallel for schedule(static)
    for (long id = 0; id < gs; ++id) f[id] += d * fd[id];
    if (S->p.calculate_SIGW) {
        for (int c = 0; c < 6; ++c) {
            float* h = S->h[c];
            const float* hd = S->hd[c];
            #pragma omp parallel for schedule(static)
            for (long id = 0; id < gs; ++id) h[id] += (float)(d * hd[id]);
        }
    }
    S->a += d * S->ad;
}

/* initialize_post_inflation(), src/initialize.cpp:245-290, without the
 * save_post_inflation(1) it ends with (the program driver makes it).  With
 * deltaN, f becomes Phi_from_zeta (deltaN - <deltaN>); fd keeps its value (the
 * reference only resizes it); h and h' are zeroed; ad2 and astep are left as
 * they are. */
void ieo_initialize_post_inflation(ieo_state* S) {
    const ieo_params* p = &S->p;
    const size_t gs = S->gs;
    S->t0 = 0.0;
    S->t = 0.0;
    for (int c = 0; c < 6; ++c) {
        memset(S->h[c], 0, sizeof(float) * gs);
        memset(S->hd[c], 0, sizeof(float) * gs);
    }
    const double Phi_from_zeta = 3.0 * (1.0 + p->omega) / (5.0 + 3.0 * p->omega);
    if (p->perform_deltaN) {
        double Nmean = 0.;
        for (size_t id = 0; id < gs; ++id) Nmean += S->deltaN[id];
        Nmean = Nmean / (double)gs;
        for (size_t id = 0; id < gs; ++id) S->f[id] = Phi_from_zeta * (S->deltaN[id] - Nmean);
    } else {
        double fmean = 0.0, fdmean = 0.0;
        for (size_t id = 0; id < gs; ++id) {
            fmean += S->f[id];
            fdmean += S->fd[id];
        }
        fmean = fmean / (double)gs;
        fdmean = fdmean / (double)gs;
        const double s = p->rescale_s;
        for (size_t id = 0; id < gs; ++id)
            S->f[id] = Phi_from_zeta * (S->f[id] - fmean) /
                       (fdmean * pow(S->a, s - 1.0) / (S->ad * pow(S->a, s - 2.0)));
    }
    S->a = 1.0;
    S->ad = p->horizon_factor * p->N * 2.0 * S->pi / p->L;
}

/* d2_cross_state, src/evolution.cpp:93-106: the neighbours are chosen per
 * index from whether d1 or d2 names it, and the four corners are
 * (ip, jp, kp), (ip, jm, km), (im, jp, kp), (im, jm, km).  For (d1, d2) =
 * (1, 2) the i index does not move, so fpp = fmp and fpm = fmm and the value
 * is the rounding residue of (fpp - fpm - fmp + fmm): kept as it is. */
static inline double d2_cross_at(const double* f, int N, int d1, int d2, int i, int j, int k, double den) {
    const int iu = (d1 == 0 || d2 == 0), ju = (d1 == 1 || d2 == 1), ku = (d1 == 2 || d2 == 2);
    const int ip = iu ? (i == N - 1 ? 0 : i + 1) : i, im = iu ? (i == 0 ? N - 1 : i - 1) : i;
    const int jp = ju ? (j == N - 1 ? 0 : j + 1) : j, jm = ju ? (j == 0 ? N - 1 : j - 1) : j;
    const int kp = ku ? (k == N - 1 ? 0 : k + 1) : k, km = ku ? (k == 0 ? N - 1 : k - 1) : k;
    const double fpp = f[IDX(N, ip, jp, kp)];
    const double fpm = f[IDX(N, ip, jm, km)];
    const double fmp = f[IDX(N, im, jp, kp)];
    const double fmm = f[IDX(N, im, jm, km)];
    return (fpp - fpm - fmp + fmm) / den;
}

/* evolve_derivs_post_inflation(d), src/evolution.cpp:1436-1555: radiation-era
 * kick of fd and, with SIGW, of the six h' with the Hessian-based source
 * (build_deriv_pack, src/evolution.cpp:1398-1418); the tensor source reads
 * the fd just kicked.  ad2 depends on ad and a only. */
void ieo_evolve_derivs_post_inflation(ieo_state* S, double d) {
    const ieo_params* p = &S->p;
    const int N = p->N;
    const double s = p->rescale_s, omega = p->omega, dx = p->dx;
    const double laplnorm = pow(S->a, -2.0 * s) / pw2(dx);
    S->ad2 = -(s - 0.5 * (1.0 - 3.0 * omega)) * pw2(S->ad) / S->a;
    S->ad += 0.5 * d * S->ad2;
    const double a = S->a, ad = S->ad;
    double* f = S->f;
    double* fd = S->fd;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
        for (int j = 0; j < N; ++j) {
            const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
            for (int k = 0; k < N; ++k) {
                const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                const size_t id = IDX(N, i, j, k);
                fd[id] += d * (omega * laplnorm * LAPL_AT(double, f, N, i, j, k, ip, im, jp, jm, kp, km)
                               - (3.0 * (1.0 + omega) + s) * ad * fd[id] / a);
            }
        }
    }
    if (p->calculate_SIGW) {
        const double Htilde = ad / a;
        const double invH = 1.0 / Htilde;
        const double coeffU = 4.0 / (3.0 * (1.0 + omega));
        const double srcAmp = 2.0 * pow(a, -2.0 * s);
        const double half_over_dx = 0.5 / dx;
        const double inv_dx2 = 1.0 / (dx * dx);
        const double den = 4.0 * dx * dx;
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < N; ++i) {
            const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
            for (int j = 0; j < N; ++j) {
                const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
                for (int k = 0; k < N; ++k) {
                    const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                    const size_t id = IDX(N, i, j, k);
                    /* dfdx<double> of f and of the kicked fd, src/evolution.cpp:55-77 */
                    const double gx = (f[IDX(N, ip, j, k)] - f[IDX(N, im, j, k)]) * half_over_dx;
                    const double gy = (f[IDX(N, i, jp, k)] - f[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gz = (f[IDX(N, i, j, kp)] - f[IDX(N, i, j, km)]) * half_over_dx;
                    const double gdx = (fd[IDX(N, ip, j, k)] - fd[IDX(N, im, j, k)]) * half_over_dx;
                    const double gdy = (fd[IDX(N, i, jp, k)] - fd[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gdz = (fd[IDX(N, i, j, kp)] - fd[IDX(N, i, j, km)]) * half_over_dx;
                    /* d2_same_state, src/evolution.cpp:79-91 */
                    const double Hxx = (f[IDX(N, ip, j, k)] - 2.0 * f[id] + f[IDX(N, im, j, k)]) * inv_dx2;
                    const double Hyy = (f[IDX(N, i, jp, k)] - 2.0 * f[id] + f[IDX(N, i, jm, k)]) * inv_dx2;
                    const double Hzz = (f[IDX(N, i, j, kp)] - 2.0 * f[id] + f[IDX(N, i, j, km)]) * inv_dx2;
                    const double Hxy = d2_cross_at(f, N, 0, 1, i, j, k, den);
                    const double Hxz = d2_cross_at(f, N, 0, 2, i, j, k, den);
                    const double Hyz = d2_cross_at(f, N, 1, 2, i, j, k, den);
                    const double Phi = f[id];
                    const double dux = gdx * invH + gx;
                    const double duy = gdy * invH + gy;
                    const double duz = gdz * invH + gz;
                    const double Sc[6] = {
                        4.0 * Phi * Hxx + 2.0 * gx * gx - coeffU * (dux * dux),
                        4.0 * Phi * Hyy + 2.0 * gy * gy - coeffU * (duy * duy),
                        4.0 * Phi * Hzz + 2.0 * gz * gz - coeffU * (duz * duz),
                        4.0 * Phi * Hxy + 2.0 * gx * gy - coeffU * (dux * duy),
                        4.0 * Phi * Hxz + 2.0 * gx * gz - coeffU * (dux * duz),
                        4.0 * Phi * Hyz + 2.0 * gy * gz - coeffU * (duy * duz)};
                    for (int c = 0; c < 6; ++c) {
                        const float* h = S->h[c];
                        const float lapf = LAPL_AT(float, h, N, i, j, k, ip, im, jp, jm, kp, km);
                        const double lap_h = (double)lapf;
                        const double rhs = d * (laplnorm * lap_h - (2.0 + s) * ad * (double)S->hd[c][id] / a +
                                                srcAmp * Sc[c]);
                        S->hd[c][id] += (float)rhs;
                    }
                }
            }
        }
    }
    S->ad += 0.5 * d * S->ad2;
}

/* compute_inflation_rhs, src/evolution.cpp:418-599: the time derivatives of a
 * stage state (fs, fds; hs, hds with SIGW) into kf, kfd (kh, khd), and dadt,
 * daddt.  S->rk_post selects the post-inflation equations (the reference's
 * g_use_post_inflation_rhs, set for the RK branches of
 * run_post_inflation_loop).  Inflation: the sums run serially in loop order
 * (the reference's OpenMP reduction with one thread); the table lookup keeps
 * the per-site hint (evaluate_potential_from_value, src/potential.cpp:123-146).
 * Post-inflation: no lattice sums; the tensor source is the Hessian form of
 * build_deriv_pack with the stage's fd (src/evolution.cpp:532-595). */
static int rk_rhs(ieo_state* S, const double* fs, const double* fds, float* const* hs, float* const* hds, double* kf,
                  double* kfd, float* const* kh, float* const* khd, double a_st, double ad_st, double* dadt,
                  double* daddt) {
    const ieo_params* p = &S->p;
    const int N = p->N;
    const double s = p->rescale_s, dx = p->dx, B2 = pw2(p->rescale_B);
    const double laplnorm = pow(a_st, -2.0 * s) / pw2(dx);
    const double srcAmp = 2.0 * pow(a_st, -2.0 * s);
    const double half_over_dx = 0.5 / dx;
    if (S->rk_post) {
        const double omega = p->omega;
        const double scalar_friction = (3.0 * (1.0 + omega) + s) * ad_st / a_st;
        const double tensor_friction = (2.0 + s) * ad_st / a_st;
        const double Htilde = ad_st / a_st;
        const double invH = 1.0 / Htilde;
        const double coeffU = 4.0 / (3.0 * (1.0 + omega));
        const double inv_dx2 = 1.0 / (dx * dx);
        const double den = 4.0 * dx * dx;
        for (int i = 0; i < N; ++i) {
            const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
            for (int j = 0; j < N; ++j) {
                const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
                for (int k = 0; k < N; ++k) {
                    const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                    const size_t id = IDX(N, i, j, k);
                    const double lap = LAPL_AT(double, fs, N, i, j, k, ip, im, jp, jm, kp, km);
                    kf[id] = fds[id];
                    kfd[id] = omega * laplnorm * lap - scalar_friction * fds[id];
                    if (!p->calculate_SIGW) continue;
                    const double gx = (fs[IDX(N, ip, j, k)] - fs[IDX(N, im, j, k)]) * half_over_dx;
                    const double gy = (fs[IDX(N, i, jp, k)] - fs[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gz = (fs[IDX(N, i, j, kp)] - fs[IDX(N, i, j, km)]) * half_over_dx;
                    const double gdx = (fds[IDX(N, ip, j, k)] - fds[IDX(N, im, j, k)]) * half_over_dx;
                    const double gdy = (fds[IDX(N, i, jp, k)] - fds[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gdz = (fds[IDX(N, i, j, kp)] - fds[IDX(N, i, j, km)]) * half_over_dx;
                    const double Hxx = (fs[IDX(N, ip, j, k)] - 2.0 * fs[id] + fs[IDX(N, im, j, k)]) * inv_dx2;
                    const double Hyy = (fs[IDX(N, i, jp, k)] - 2.0 * fs[id] + fs[IDX(N, i, jm, k)]) * inv_dx2;
                    const double Hzz = (fs[IDX(N, i, j, kp)] - 2.0 * fs[id] + fs[IDX(N, i, j, km)]) * inv_dx2;
                    const double Hxy = d2_cross_at(fs, N, 0, 1, i, j, k, den);
                    const double Hxz = d2_cross_at(fs, N, 0, 2, i, j, k, den);
                    const double Hyz = d2_cross_at(fs, N, 1, 2, i, j, k, den);
                    const double dux = gdx * invH + gx;
                    const double duy = gdy * invH + gy;
                    const double duz = gdz * invH + gz;
                    const double Phi = fs[id];
                    const double Sc[6] = {
                        4.0 * Phi * Hxx + 2.0 * gx * gx - coeffU * (dux * dux),
                        4.0 * Phi * Hyy + 2.0 * gy * gy - coeffU * (duy * duy),
                        4.0 * Phi * Hzz + 2.0 * gz * gz - coeffU * (duz * duz),
                        4.0 * Phi * Hxy + 2.0 * gx * gy - coeffU * (dux * duy),
                        4.0 * Phi * Hxz + 2.0 * gx * gz - coeffU * (dux * duz),
                        4.0 * Phi * Hyz + 2.0 * gy * gz - coeffU * (duy * duz)};
                    for (int c = 0; c < 6; ++c) {
                        const float lapf = LAPL_AT(float, hs[c], N, i, j, k, ip, im, jp, jm, kp, km);
                        kh[c][id] = hds[c][id];
                        khd[c][id] = (float)(laplnorm * (double)lapf - tensor_friction * (double)hds[c][id] +
                                             srcAmp * Sc[c]);
                    }
                }
            }
        }
        *dadt = ad_st;
        *daddt = -(s - 0.5 * (1.0 - 3.0 * omega)) * pw2(ad_st) / a_st;
        return 0;
    }
    const double friction = (2.0 + s) * ad_st / a_st;
    const double potnorm = pow(a_st, 2.0 - 2.0 * s);
    double gradient_sum = 0.0, potential_sum = 0.0;
    for (int i = 0; i < N; ++i) {
        const int ip = (i == N - 1) ? 0 : i + 1, im = (i == 0) ? N - 1 : i - 1;
        for (int j = 0; j < N; ++j) {
            const int jp = (j == N - 1) ? 0 : j + 1, jm = (j == 0) ? N - 1 : j - 1;
            for (int k = 0; k < N; ++k) {
                const int kp = (k == N - 1) ? 0 : k + 1, km = (k == 0) ? N - 1 : k - 1;
                const size_t id = IDX(N, i, j, k);
                const double field = fs[id];
                const double lap = LAPL_AT(double, fs, N, i, j, k, ip, im, jp, jm, kp, km);
                double pot, dpot;
                if (p->numerical_potential) {
                    const int l = bracket(S, field, S->lstart[id]);
                    if (l < 0) return 1;
                    pot = interp(S, field, l, S->tV) / B2;
                    dpot = interp(S, field, l, S->tdV) / B2;
                    const int back = p->int_err > 1 ? p->int_err : 1;
                    S->lstart[id] = (l - back) > 1 ? (l - back) : 1;
                } else {
                    pot = hill_V(p, field);
                    dpot = hill_dV(p, field);
                }
                kf[id] = fds[id];
                kfd[id] = laplnorm * lap - friction * fds[id] - potnorm * dpot;
                gradient_sum -= field * lap;
                potential_sum += pot;
                if (p->calculate_SIGW) {
                    const double gx = (fs[IDX(N, ip, j, k)] - fs[IDX(N, im, j, k)]) * half_over_dx;
                    const double gy = (fs[IDX(N, i, jp, k)] - fs[IDX(N, i, jm, k)]) * half_over_dx;
                    const double gz = (fs[IDX(N, i, j, kp)] - fs[IDX(N, i, j, km)]) * half_over_dx;
                    const double T[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
                    for (int c = 0; c < 6; ++c) {
                        const float lapf = LAPL_AT(float, hs[c], N, i, j, k, ip, im, jp, jm, kp, km);
                        kh[c][id] = hds[c][id];
                        khd[c][id] = (float)(laplnorm * (double)lapf - friction * (double)hds[c][id] + srcAmp * T[c]);
                    }
                }
            }
        }
    }
    const double gradient = 0.5 * gradient_sum * pw2(1.0 / (a_st * dx)) / (double)S->gs;
    const double potential_avg = potential_sum / (double)S->gs;
    const double source = 2.0 * gradient / 3.0 + potential_avg;
    *dadt = ad_st;
    *daddt = pow(a_st, 3.0 - 2.0 * s) * source - (s + 1.0) * pw2(ad_st) / a_st;
    return 0;
}

/* RK4_A, RK4_B and the Dormand-Prince 5(4) tableau (DormandPrince45Coefficients,
 * src/evolution.cpp:366-414, 601-637): the published coefficients; e = b - b*. */
static const double RK4_A[7][7] = {{0.0}, {0.5}, {0.0, 0.5}, {0.0, 0.0, 1.0}};
static const double RK4_B[7] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
#define DP_B1 (35.0 / 384.0)
#define DP_B3 (500.0 / 1113.0)
#define DP_B4 (125.0 / 192.0)
#define DP_B5 (-2187.0 / 6784.0)
#define DP_B6 (11.0 / 84.0)
static const double DP_A[7][7] = {
    {0.0},
    {1.0 / 5.0},
    {3.0 / 40.0, 9.0 / 40.0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0},
    {DP_B1, 0.0, DP_B3, DP_B4, DP_B5, DP_B6}};
static const double DP_B[7] = {DP_B1, 0.0, DP_B3, DP_B4, DP_B5, DP_B6, 0.0};
static const double DP_E[7] = {DP_B1 - 5179.0 / 57600.0, 0.0, DP_B3 - 7571.0 / 16695.0, DP_B4 - 393.0 / 640.0,
                               DP_B5 - -92097.0 / 339200.0, DP_B6 - 187.0 / 2100.0, -(1.0 / 40.0)};

static void rk_scratch(ieo_state* S) {
    if (S->ftmp) return;
    const size_t gs = S->gs;
    S->ftmp = (double*)calloc(gs, sizeof(double));
    S->fdtmp = (double*)calloc(gs, sizeof(double));
    for (int q = 0; q < 7; ++q) {
        S->kf[q] = (double*)calloc(gs, sizeof(double));
        S->kfd[q] = (double*)calloc(gs, sizeof(double));
    }
    if (S->p.calculate_SIGW)
        for (int c = 0; c < 6; ++c) {
            S->htmp[c] = (float*)calloc(gs, sizeof(float));
            S->hdtmp[c] = (float*)calloc(gs, sizeof(float));
            for (int q = 0; q < 7; ++q) {
                S->kh[q][c] = (float*)calloc(gs, sizeof(float));
                S->khd[q][c] = (float*)calloc(gs, sizeof(float));
            }
        }
}

/* evaluate_inflation_stage, src/evolution.cpp:692-715: the stage state of
 * prepare_inflation_stage_state (:639-671), the background stage of
 * prepare_inflation_background_state (:673-690) and the stage's derivatives. */
static int rk_stage(ieo_state* S, double h, int stage, const double (*A)[7], double* ka, double* kad) {
    const size_t gs = S->gs;
    for (size_t id = 0; id < gs; ++id) {
        double sum_f = 0.0, sum_fd = 0.0;
        for (int q = 0; q < stage; ++q) {
            const double c = A[stage][q];
            if (c == 0.0) continue;
            sum_f += c * S->kf[q][id];
            sum_fd += c * S->kfd[q][id];
        }
        S->ftmp[id] = S->f[id] + h * sum_f;
        S->fdtmp[id] = S->fd[id] + h * sum_fd;
    }
    if (S->p.calculate_SIGW)
        for (int c = 0; c < 6; ++c)
            for (size_t id = 0; id < gs; ++id) {
                double sum_h = 0.0, sum_hd = 0.0;
                for (int q = 0; q < stage; ++q) {
                    const double cs = A[stage][q];
                    if (cs == 0.0) continue;
                    sum_h += cs * (double)S->kh[q][c][id];
                    sum_hd += cs * (double)S->khd[q][c][id];
                }
                S->htmp[c][id] = (float)((double)S->h[c][id] + h * sum_h);
                S->hdtmp[c][id] = (float)((double)S->hd[c][id] + h * sum_hd);
            }
    double a_st = S->a, ad_st = S->ad;
    for (int q = 0; q < stage; ++q) {
        const double c = A[stage][q];
        if (c == 0.0) continue;
        a_st += h * c * ka[q];
        ad_st += h * c * kad[q];
    }
    return rk_rhs(S, S->ftmp, S->fdtmp, S->htmp, S->hdtmp, S->kf[stage], S->kfd[stage], S->kh[stage], S->khd[stage],
                  a_st, ad_st, &ka[stage], &kad[stage]);
}

/* rk4_step_inflation(h), src/evolution.cpp:760-779, with the weighted update
 * of apply_inflation_weighted_update (:717-758).  ad2 is not touched. */
int ieo_rk4_step_inflation(ieo_state* S, double h) {
    rk_scratch(S);
    const size_t gs = S->gs;
    const int sigw = S->p.calculate_SIGW;
    double ka[7] = {0.0}, kad[7] = {0.0};
    if (rk_rhs(S, S->f, S->fd, S->h, S->hd, S->kf[0], S->kfd[0], S->kh[0], S->khd[0], S->a, S->ad, &ka[0], &kad[0]))
        return 1;
    for (int stage = 1; stage < 4; ++stage)
        if (rk_stage(S, h, stage, RK4_A, ka, kad)) return 1;
    for (size_t id = 0; id < gs; ++id) {
        double sum_f = 0.0, sum_fd = 0.0;
        for (int q = 0; q < 4; ++q) {
            const double bs = RK4_B[q];
            if (bs == 0.0) continue;
            sum_f += bs * S->kf[q][id];
            sum_fd += bs * S->kfd[q][id];
        }
        S->f[id] += h * sum_f;
        S->fd[id] += h * sum_fd;
    }
    if (sigw)
        for (int c = 0; c < 6; ++c)
            for (size_t id = 0; id < gs; ++id) {
                double sum_h = 0.0, sum_hd = 0.0;
                for (int q = 0; q < 4; ++q) {
                    const double bs = RK4_B[q];
                    if (bs == 0.0) continue;
                    sum_h += bs * (double)S->kh[q][c][id];
                    sum_hd += bs * (double)S->khd[q][c][id];
                }
                S->h[c][id] = (float)((double)S->h[c][id] + h * sum_h);
                S->hd[c][id] = (float)((double)S->hd[c][id] + h * sum_hd);
            }
    for (int q = 0; q < 4; ++q) {
        const double bs = RK4_B[q];
        if (bs == 0.0) continue;
        S->a += h * bs * ka[q];
        S->ad += h * bs * kad[q];
    }
    S->t += h;
    return 0;
}

/* std::max / std::min / std::clamp as the reference calls them */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

/* clamp_rk45_step, src/evolution.cpp:326-332 */
double ieo_rk45_clamp(const ieo_state* S, double h, double hmax) {
    const double hmin = smax(1e-16, S->p.rk45_min_dt);
    const double hhi = smax(hmin, hmax);
    if (h < hmin) return hmin;
    if (h > hhi) return hhi;
    return h;
}

/* rk45_hmax_from_base_step, src/evolution.cpp:341-343 */
double ieo_rk45_hmax(const ieo_state* S, double base_step) {
    return smin(S->p.rk45_max_dt, smax(S->p.rk45_min_dt, 2.0 * base_step));
}

/* rk45_step_inflation(h, hmax, h_next), src/evolution.cpp:781-904: one
 * Dormand-Prince 5(4) attempt; on acceptance the 5th-order state is taken
 * and *accepted = 1.  The error norm is the weighted RMS over f, fd (and the
 * twelve tensor arrays) and a, ad, summed in the reference's order. */
int ieo_rk45_step_inflation(ieo_state* S, double h, double hmax, double* h_next, int* accepted) {
    rk_scratch(S);
    const ieo_params* p = &S->p;
    const size_t gs = S->gs;
    const double atol = p->rk45_abs_tol, rtol = p->rk45_rel_tol;
    double ka[7] = {0.0}, kad[7] = {0.0};
    if (rk_rhs(S, S->f, S->fd, S->h, S->hd, S->kf[0], S->kfd[0], S->kh[0], S->khd[0], S->a, S->ad, &ka[0], &kad[0]))
        return 1;
    for (int stage = 1; stage < 7; ++stage)
        if (rk_stage(S, h, stage, DP_A, ka, kad)) return 1;
    double a5 = S->a, ad5 = S->ad, erra = 0.0, errad = 0.0;
    for (int q = 0; q < 7; ++q) {
        const double bs = DP_B[q], es = DP_E[q];
        if (bs != 0.0) {
            a5 += h * bs * ka[q];
            ad5 += h * bs * kad[q];
        }
        if (es != 0.0) {
            erra += h * es * ka[q];
            errad += h * es * kad[q];
        }
    }
    double err_acc = 0.0;
    size_t nvars = 2 * gs + 2;
    for (size_t id = 0; id < gs; ++id) {
        double y5f = S->f[id], y5fd = S->fd[id], errf = 0.0, errfd = 0.0;
        for (int q = 0; q < 7; ++q) {
            const double bs = DP_B[q], es = DP_E[q];
            if (bs != 0.0) {
                y5f += h * bs * S->kf[q][id];
                y5fd += h * bs * S->kfd[q][id];
            }
            if (es != 0.0) {
                errf += h * es * S->kf[q][id];
                errfd += h * es * S->kfd[q][id];
            }
        }
        S->ftmp[id] = y5f;
        S->fdtmp[id] = y5fd;
        const double sf = atol + rtol * smax(fabs(S->f[id]), fabs(y5f));
        const double sfd = atol + rtol * smax(fabs(S->fd[id]), fabs(y5fd));
        err_acc += pw2(errf / sf) + pw2(errfd / sfd);
    }
    if (p->calculate_SIGW) {
        nvars += 12 * gs;
        for (int c = 0; c < 6; ++c)
            for (size_t id = 0; id < gs; ++id) {
                double y5h = (double)S->h[c][id], y5hd = (double)S->hd[c][id], errh = 0.0, errhd = 0.0;
                for (int q = 0; q < 7; ++q) {
                    const double bs = DP_B[q], es = DP_E[q];
                    if (bs != 0.0) {
                        y5h += h * bs * (double)S->kh[q][c][id];
                        y5hd += h * bs * (double)S->khd[q][c][id];
                    }
                    if (es != 0.0) {
                        errh += h * es * (double)S->kh[q][c][id];
                        errhd += h * es * (double)S->khd[q][c][id];
                    }
                }
                S->htmp[c][id] = (float)y5h;
                S->hdtmp[c][id] = (float)y5hd;
                const double sh = atol + rtol * smax(fabs((double)S->h[c][id]), fabs(y5h));
                const double shd = atol + rtol * smax(fabs((double)S->hd[c][id]), fabs(y5hd));
                err_acc += pw2(errh / sh) + pw2(errhd / shd);
            }
    }
    const double sa = atol + rtol * smax(fabs(S->a), fabs(a5));
    const double sad = atol + rtol * smax(fabs(S->ad), fabs(ad5));
    err_acc += pw2(erra / sa) + pw2(errad / sad);
    const double err_norm = sqrt(err_acc / (double)nvars);
    const double safe_err = smax(err_norm, 1e-16);
    double factor = p->rk45_safety * pow(safe_err, -0.2);
    factor = (factor < 0.1) ? 0.1 : (5.0 < factor) ? 5.0 : factor;
    S->rk45_err = err_norm;
    if (err_norm <= 1.0) {
        double* t;
        t = S->f; S->f = S->ftmp; S->ftmp = t;
        t = S->fd; S->fd = S->fdtmp; S->fdtmp = t;
        if (p->calculate_SIGW)
            for (int c = 0; c < 6; ++c) {
                float* u = S->h[c]; S->h[c] = S->htmp[c]; S->htmp[c] = u;
                u = S->hd[c]; S->hd[c] = S->hdtmp[c]; S->hdtmp[c] = u;
            }
        S->a = a5;
        S->ad = ad5;
        S->t += h;
        *h_next = ieo_rk45_clamp(S, h * factor, hmax);
        *accepted = 1;
        return 0;
    }
    *h_next = ieo_rk45_clamp(S, h * smax(0.1, smin(0.5, factor)), hmax);
    *accepted = 0;
    return 0;
}

/* rk45_accept_step, src/evolution.cpp:345-363: attempts until one is
 * accepted; fails after 25 rejections or at the minimum step.  Returns the
 * step proposed for the next call in *h. */
int ieo_rk45_accept(ieo_state* S, double* h, double hmax) {
    int accepted = 0, attempts = 0;
    while (!accepted) {
        double hs = *h;
        if (ieo_rk45_step_inflation(S, *h, hmax, &hs, &accepted)) return 1;
        *h = hs;
        ++attempts;
        if (!accepted && (attempts > 25 || *h <= S->p.rk45_min_dt * (1.0 + 1e-12))) {
            if (S->rk_post)
                set_err(S, "RK45 failed to converge in post-inflation at a=%e, t=%e (attempts=%d, h=%e)\n", S->a, S->t,
                        attempts, *h);
            else
                set_err(S, "RK45 failed to converge at a=%e, t=%e (attempts=%d, h=%e)\n", S->a, S->t, attempts, *h);
            return 1;
        }
    }
    return 0;
}

void ieo_set_rk_post(ieo_state* S, int post) { S->rk_post = post != 0; }

/* inflation_rescaled_step, src/evolution.cpp:338-340 */
double ieo_rescaled_step(const ieo_state* S, double astep) {
    return S->p.dt * eng_pow(S, astep, S->p.rescale_s - 1.0);
}

int ieo_leapfrog_steps(ieo_state* S, int nsteps) {
    int n = 0;
    while (n < nsteps && S->a <= S->p.af) {
        const double d = ieo_rescaled_step(S, S->astep);
        if (ieo_evolve_derivs(S, d)) return -1;
        ieo_evolve_fields(S, d);
        ++n;
        S->astep = S->a;
    }
    return n;
}

/* ------------------------------------------------------------------------- */
/* FFT: radix-2 FFTEASY variant of src/ffteasy.hpp                           */
/* ------------------------------------------------------------------------- */

/* One macro body per precision keeps the two instantiations identical. */
#define DEFINE_FFT(T, CPLX, SFX, SIN, COS, ASIN)                                                      \
static void fftc1_##SFX(T* fr, int n, int skip, int forward) {                                        \
    int b, index1, index2, trans_size, trans;                                                          \
    const T pi2 = (T)4 * ASIN((T)1);                                                                   \
    T pi2n, cospi2n, sinpi2n;                                                                          \
    CPLX wb, temp1, temp2;                                                                             \
    CPLX* c = (CPLX*)fr;                                                                               \
    for (index1 = 1, index2 = 0; index1 < n; ++index1) {                                               \
        for (b = n / 2; index2 >= b; b >>= 1) index2 -= b;                                             \
        index2 += b;                                                                                   \
        if (index2 > index1) {                                                                         \
            temp1 = c[(size_t)index2 * skip];                                                          \
            c[(size_t)index2 * skip] = c[(size_t)index1 * skip];                                       \
            c[(size_t)index1 * skip] = temp1;                                                          \
        }                                                                                              \
    }                                                                                                  \
    for (trans_size = 2; trans_size <= n; trans_size <<= 1) {                                          \
        pi2n = (T)forward * pi2 / (T)trans_size;                                                       \
        cospi2n = COS(pi2n);                                                                           \
        sinpi2n = SIN(pi2n);                                                                           \
        wb.re = (T)1; wb.im = (T)0;                                                                    \
        for (b = 0; b < trans_size / 2; ++b) {                                                         \
            for (trans = 0; trans < n / trans_size; ++trans) {                                         \
                size_t i1 = (size_t)(trans * trans_size + b) * skip;                                   \
                size_t i2 = i1 + (size_t)(trans_size / 2) * skip;                                      \
                temp1 = c[i1];                                                                         \
                temp2 = c[i2];                                                                         \
                c[i1].re = temp1.re + wb.re * temp2.re - wb.im * temp2.im;                             \
                c[i1].im = temp1.im + wb.re * temp2.im + wb.im * temp2.re;                             \
                c[i2].re = temp1.re - wb.re * temp2.re + wb.im * temp2.im;                             \
                c[i2].im = temp1.im - wb.re * temp2.im - wb.im * temp2.re;                             \
            }                                                                                          \
            temp1 = wb;                                                                                \
            wb.re = cospi2n * temp1.re - sinpi2n * temp1.im;                                           \
            wb.im = cospi2n * temp1.im + sinpi2n * temp1.re;                                           \
        }                                                                                              \
    }                                                                                                  \
    if (forward < 0) {                                                                                 \
        for (size_t q = 0; q < (size_t)skip * n; q += skip) {                                          \
            c[q].re /= (T)n;                                                                           \
            c[q].im /= (T)n;                                                                           \
        }                                                                                              \
    }                                                                                                  \
}                                                                                                      \
static void fftcn_##SFX(T* fr, int ndims, const int* size, int forward) {                             \
    size_t planesize = 1, skip = 1, totalsize = 1;                                                     \
    for (int dim = 0; dim < ndims; ++dim) totalsize *= size[dim];                                      \
    for (int dim = ndims - 1; dim >= 0; --dim) {                                                       \
        planesize *= size[dim];                                                                        \
        for (size_t i = 0; i < totalsize; i += planesize)                                              \
            for (size_t j = 0; j < skip; ++j)                                                          \
                fftc1_##SFX(fr + 2 * (i + j), size[dim], (int)skip, forward);                          \
        skip *= size[dim];                                                                             \
    }                                                                                                  \
}                                                                                                      \
static void fftrn3_##SFX(T* fr, T* fnyq, int N, int forward) {                                        \
    int size[3] = {N, N, N / 2};                                                                       \
    const T pi2n = ((T)4 * ASIN((T)1)) / (T)N;                                                         \
    const T cospi2n = COS(pi2n);                                                                       \
    const T sinpi2n = SIN(pi2n);                                                                       \
    CPLX wb, temp1, temp2;                                                                             \
    CPLX* c = (CPLX*)fr;                                                                               \
    CPLX* cny = (CPLX*)fnyq;                                                                           \
    const size_t rowlen = (size_t)(N / 2);                                                             \
    const size_t totalsize = (size_t)N * N * rowlen;                                                   \
    const T fw = (T)forward;                                                                           \
    if (forward == 1) {                                                                                \
        fftcn_##SFX(fr, 3, size, 1);                                                                   \
        for (size_t r = 0; r < totalsize / rowlen; ++r) cny[r] = c[r * rowlen];                        \
    }                                                                                                  \
    int ii = 0, jj = 0;                                                                                \
    for (size_t index = 0; index < totalsize; index += rowlen) {                                       \
        const int in_ = (ii == 0) ? 0 : N - ii, jn_ = (jj == 0) ? 0 : N - jj;                          \
        const size_t rneg = (size_t)in_ * N + (size_t)jn_;                                             \
        const size_t indexneg = rneg * rowlen;                                                         \
        wb.re = (T)1; wb.im = (T)0;                                                                    \
        for (int b = 1; b < N / 4; ++b) {                                                              \
            temp1 = wb;                                                                                \
            wb.re = cospi2n * temp1.re - sinpi2n * temp1.im;                                           \
            wb.im = cospi2n * temp1.im + sinpi2n * temp1.re;                                           \
            temp1 = c[index + b];                                                                      \
            temp2 = c[indexneg + N / 2 - b];                                                           \
            c[index + b].re = (T)0.5 * (temp1.re + temp2.re + fw * wb.re * (temp1.im + temp2.im) + wb.im * (temp1.re - temp2.re)); \
            c[index + b].im = (T)0.5 * (temp1.im - temp2.im - fw * wb.re * (temp1.re - temp2.re) + wb.im * (temp1.im + temp2.im)); \
            c[indexneg + N / 2 - b].re = (T)0.5 * (temp1.re + temp2.re - fw * wb.re * (temp1.im + temp2.im) - wb.im * (temp1.re - temp2.re)); \
            c[indexneg + N / 2 - b].im = (T)0.5 * (-temp1.im + temp2.im - fw * wb.re * (temp1.re - temp2.re) + wb.im * (temp1.im + temp2.im)); \
        }                                                                                              \
        temp1 = c[index];                                                                              \
        temp2 = cny[rneg];                                                                             \
        c[index].re = (T)0.5 * (temp1.re + temp2.re + fw * (temp1.im + temp2.im));                     \
        c[index].im = (T)0.5 * (temp1.im - temp2.im - fw * (temp1.re - temp2.re));                     \
        cny[rneg].re = (T)0.5 * (temp1.re + temp2.re - fw * (temp1.im + temp2.im));                    \
        cny[rneg].im = (T)0.5 * (-temp1.im + temp2.im - fw * (temp1.re - temp2.re));                   \
        if (++jj == N) { jj = 0; ++ii; }                                                               \
    }                                                                                                  \
    if (forward == -1) fftcn_##SFX(fr, 3, size, -1);                                                   \
}

DEFINE_FFT(double, cplx_d, d, sin, cos, asin)
DEFINE_FFT(float, cplx_f, f, sinf, cosf, asinf)

void ieo_fftrn_d(double* f, double* fny, int N, int forward) { fftrn3_d(f, fny, N, forward); }
void ieo_fftrn_f(float* f, float* fny, int N, int forward) { fftrn3_f(f, fny, N, forward); }
void ieo_fftc1_d(double* f, int n, int skip, int forward) { fftc1_d(f, n, skip, forward); }

/* ------------------------------------------------------------------------- */
/* spectra, src/output.cpp:63-151 and 466-625                                */
/* ------------------------------------------------------------------------- */

int ieo_numbins(int N) { return (int)(1.73205 * (N / 2)) + 1; }

/* write_isotropic_spectrum_from_fft_r2c binning, src/output.cpp:63-151.
 * Serial in the reference's (i, j, k) order. */
void ieo_bin_spectrum(int N, const double* ff, const double* nyq, int* counts, double* f2) {
    const int numbins = ieo_numbins(N);
    for (int b = 0; b < numbins; ++b) { counts[b] = 0; f2[b] = 0.0; }
    for (int i = 0; i < N; i++) {
        const int px = (i <= N / 2 ? i : i - N);
        for (int j = 0; j < N; j++) {
            const int py = (j <= N / 2 ? j : j - N);
            for (int k = 1; k < N / 2; k++) {
                const int pz = k;
                const double pm = sqrt(pw2((double)px) + pw2((double)py) + pw2((double)pz));
                const int bin = (int)lround(pm);
                if (bin < 0 || bin >= numbins) continue;
                const double re = ff[IDX(N, i, j, 2 * k)];
                const double im = ff[IDX(N, i, j, 2 * k + 1)];
                const double fp2 = re * re + im * im;
                counts[bin] += 2;
                f2[bin] += 2.0 * fp2;
            }
            for (int k = 0; k <= N / 2; k += N / 2) {
                const int pz = k;
                const double pm = sqrt(pw2((double)px) + pw2((double)py) + pw2((double)pz));
                const int bin = (int)lround(pm);
                if (bin < 0 || bin >= numbins) continue;
                double fp2;
                if (k == 0) {
                    const double re = ff[IDX(N, i, j, 0)], im = ff[IDX(N, i, j, 1)];
                    fp2 = re * re + im * im;
                } else {
                    const double re = nyq[(size_t)i * 2 * N + 2 * j], im = nyq[(size_t)i * 2 * N + 2 * j + 1];
                    fp2 = re * re + im * im;
                }
                counts[bin] += 1;
                f2[bin] += fp2;
            }
        }
    }
}

/* Whether the mode of lattice momentum p (s = |p|^2, an exact integer in
 * double) is outside [low, high]: sqrt(s) > high || sqrt(s) < low, the test
 * of src/output.cpp:352-353. */
static int mode_cut(double s, double high, double low) {
    const double pd = sqrt(s);
    return pd > high || pd < low;
}

static void zero_pair(double* a, double* b) { a[0] = 0.; a[1] = 0.; b[0] = 0.; b[1] = 0.; }

/* The forcing cutoff of spectraf(), src/output.cpp:330-401 (the same block
 * closes spectraf_post_inflation, :1700-1765), applied with f already in
 * k-space: fd is transformed forward, every mode outside [low, high] is
 * zeroed in f and fd, and fd is transformed back; f stays in k-space for the
 * caller's inverse transform.  Modes 0 < kz < N/2 are tested one by one.  On
 * the kz = 0 plane (f[(i N + j) N + 0, 1]) and the Nyquist plane (fny[i][2j,
 * 2j + 1]) the reference walks one member of each conjugate pair (j > N/2,
 * or i > N/2 on the rows j = 0 and j = N/2): it zeroes that member and writes
 * its partner (N - i, N - j) as the conjugate, i.e. (+0, -0).  The four
 * self-conjugate points (i, j in {0, N/2}) are zeroed alone.  The partner is
 * never tested itself; its |p| is the walked member's. */
void ieo_forcing_cutoff(ieo_state* S, double high, double low) {
    const int N = S->p.N, h = N / 2;
    double* f = S->f;
    double* fd = S->fd;
    double* fny = S->fny;
    double* fdny = S->fdny;
    ieo_fftrn_d(fd, fdny, N, 1);
    for (int i = 0; i < N; ++i) {
        const double px = (double)(i <= h ? i : i - N);
        const int ic = i == 0 ? 0 : N - i;
        for (int j = 0; j < N; ++j) {
            const double py = (double)(j <= h ? j : j - N);
            const size_t row = ((size_t)i * N + j) * N;
            for (int k = 1; k < h; ++k)
                if (mode_cut(px * px + py * py + (double)k * k, high, low))
                    zero_pair(f + row + 2 * k, fd + row + 2 * k);
            const int walked = j > h || (i > h && (j == 0 || j == h));
            const int self = (i == 0 || i == h) && (j == 0 || j == h);
            if (!walked && !self) continue;
            const int jc = j == 0 ? 0 : N - j;
            const size_t rowc = ((size_t)ic * N + jc) * N;
            if (mode_cut(px * px + py * py, high, low)) {
                zero_pair(f + row, fd + row);
                if (walked) {
                    f[rowc] = f[row]; f[rowc + 1] = -f[row + 1];
                    fd[rowc] = fd[row]; fd[rowc + 1] = -fd[row + 1];
                }
            }
            if (mode_cut(px * px + py * py + (double)h * h, high, low)) {
                const size_t q = (size_t)i * 2 * N + 2 * j, qc = (size_t)ic * 2 * N + 2 * jc;
                zero_pair(fny + q, fdny + q);
                if (walked) {
                    fny[qc] = fny[q]; fny[qc + 1] = -fny[q + 1];
                    fdny[qc] = fdny[q]; fdny[qc + 1] = -fdny[q + 1];
                }
            }
        }
    }
    ieo_fftrn_d(fd, fdny, N, -1);
}

/* spectraf() without printing, src/output.cpp:297-406: forward FFT of f,
 * bin, the forcing cutoff when high > 0, inverse FFT of f. */
void ieo_spectrum_f_cut(ieo_state* S, int* counts, double* f2, double high, double low) {
    const int N = S->p.N;
    ieo_fftrn_d(S->f, S->fny, N, 1);
    ieo_bin_spectrum(N, S->f, S->fny, counts, f2);
    if (high > 0) ieo_forcing_cutoff(S, high, low);
    ieo_fftrn_d(S->f, S->fny, N, -1);
}

void ieo_spectrum_f(ieo_state* S, int* counts, double* f2) { ieo_spectrum_f_cut(S, counts, f2, 0.0, 0.0); }

/* write_gw_spectrum_impl, src/output.cpp:466-625 (float arithmetic) */
void ieo_gw_spectrum(ieo_state* S, int which, double to_phys, int* counts, float* f2, double* f2d) {
    const int N = S->p.N;
    const double dx = S->p.dx;
    const double pi = S->pi;
    const int numbins = (int)(sqrt(3.0) * (N / 2)) + 1;
    const int i_max_out = (int)floor(0.80 * numbins);
    float** H = which ? S->hd : S->h;
    float** HN = which ? S->hdny : S->hny;
    static const int comp_of[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    for (int b = 0; b < numbins; ++b) { counts[b] = 0; f2[b] = 0.f; if (f2d) f2d[b] = 0.0; }
    for (int c = 0; c < 6; ++c) ieo_fftrn_f(H[c], HN[c], N, 1);

    for (int i = 0; i < N; ++i) {
        const int px = (i <= N / 2 ? i : i - N);
        for (int j = 0; j < N; ++j) {
            const int py = (j <= N / 2 ? j : j - N);
            /* interior modes, src/output.cpp:490-547 */
            for (int k = 1; k < N / 2; ++k) {
                const int pz = k;
                const float kx = (2.f / (float)dx) * sinf((float)pi * px / (float)N);
                const float ky = (2.f / (float)dx) * sinf((float)pi * py / (float)N);
                const float kz = (2.f / (float)dx) * sinf((float)pi * pz / (float)N);
                const float kt2 = kx * kx + ky * ky + kz * kz;
                if (kt2 == 0.f) continue;
                const int bin = (int)lroundf(sqrtf((float)(px * px + py * py + pz * pz)));
                if (bin >= i_max_out) continue;
                const size_t im_ = IDX(N, i, j, 2 * k);
                float Cr[3][3], Ci[3][3];
                for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) {
                    const int cc = comp_of[l][m];
                    float re = H[cc][im_], imv = H[cc][im_ + 1];
                    if (which) { re = (float)((double)re * to_phys); imv = (float)((double)imv * to_phys); }
                    Cr[l][m] = re; Ci[l][m] = imv;
                }
                const float inv = 1.0f / sqrtf(kt2);
                const float kh[3] = {kx * inv, ky * inv, kz * inv};
                float P[3][3];
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.f : 0.f) - kh[a] * kh[b];
                float Ar[3][3], Ai[3][3], Tr = 0.f, Ti = 0.f;
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
                    float r = 0.f, q = 0.f;
                    for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) {
                        const float pal = P[a][l], pbm = P[b][m];
                        r += pal * Cr[l][m] * pbm;
                        q += pal * Ci[l][m] * pbm;
                    }
                    Ar[a][b] = r; Ai[a][b] = q;
                }
                for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) { Tr += P[l][m] * Cr[l][m]; Ti += P[l][m] * Ci[l][m]; }
                float fp2 = 0.f;
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
                    const float Xr = Ar[a][b] - 0.5f * P[a][b] * Tr;
                    const float Xi = Ai[a][b] - 0.5f * P[a][b] * Ti;
                    fp2 += Xr * Xr + Xi * Xi;
                }
                counts[bin] += 2;
                f2[bin] += 2.f * fp2;
                if (f2d) f2d[bin] += (double)(2.f * fp2);
            }
            /* special planes k = 0 and k = N/2, src/output.cpp:550-612 */
            for (int q2 = 0; q2 <= 1; ++q2) {
                const int k = q2 * (N / 2);
                const int pz = k;
                const float kx = (2.f / (float)dx) * sinf((float)pi * px / (float)N);
                const float ky = (2.f / (float)dx) * sinf((float)pi * py / (float)N);
                const float kz = (2.f / (float)dx) * sinf((float)pi * pz / (float)N);
                const float kt2 = kx * kx + ky * ky + kz * kz;
                if (kt2 == 0.f) continue;
                const int bin = (int)lroundf(sqrtf((float)(px * px + py * py + pz * pz)));
                if (bin >= i_max_out) continue;
                float Cr[3][3], Ci[3][3];
                for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) {
                    const int cc = comp_of[l][m];
                    float re, imv;
                    if (k == 0) { re = H[cc][IDX(N, i, j, 0)]; imv = H[cc][IDX(N, i, j, 0) + 1]; }
                    else { re = HN[cc][(size_t)i * 2 * N + 2 * j]; imv = HN[cc][(size_t)i * 2 * N + 2 * j + 1]; }
                    if (which) { re = (float)((double)re * to_phys); imv = (float)((double)imv * to_phys); }
                    Cr[l][m] = re; Ci[l][m] = imv;
                }
                const float inv = 1.0f / sqrtf(kt2);
                const float kh[3] = {kx * inv, ky * inv, kz * inv};
                float P[3][3];
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.f : 0.f) - kh[a] * kh[b];
                float Ar[3][3], Ai[3][3], Tr = 0.f, Ti = 0.f;
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
                    float r = 0.f, q = 0.f;
                    for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) {
                        const float pal = P[a][l], pbm = P[b][m];
                        r += pal * Cr[l][m] * pbm;
                        q += pal * Ci[l][m] * pbm;
                    }
                    Ar[a][b] = r; Ai[a][b] = q;
                }
                for (int l = 0; l < 3; ++l) for (int m = 0; m < 3; ++m) { Tr += P[l][m] * Cr[l][m]; Ti += P[l][m] * Ci[l][m]; }
                float fp2 = 0.f;
                for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
                    const float Xr = Ar[a][b] - 0.5f * P[a][b] * Tr;
                    const float Xi = Ai[a][b] - 0.5f * P[a][b] * Ti;
                    fp2 += Xr * Xr + Xi * Xi;
                }
                counts[bin] += 1;
                f2[bin] += fp2;
                if (f2d) f2d[bin] += (double)fp2;
            }
        }
    }
    for (int c = 0; c < 6; ++c) ieo_fftrn_f(H[c], HN[c], N, -1);
}

/* ------------------------------------------------------------------------- */
/* deltaN, src/evolution.cpp:1004-1375                                       */
/* ------------------------------------------------------------------------- */

/* initializeN(), src/initialize.cpp:219-232 */
int ieo_initializeN(ieo_state* S) {
    const double s = S->p.rescale_s;
    for (size_t id = 0; id < S->gs; ++id) {
        if (S->p.numerical_potential) S->lstart[id] -= 100;
        const double H_lat = sqrt(ieo_potential(S, S->f[id]) / 3.0);
        S->fd[id] = S->fd[id] * pow(S->a, s - 1.0) / H_lat;
        S->deltaN[id] = 0.0;
    }
    return S->err;
}

/* evolve_derivsN(d), src/evolution.cpp:1004-1012 */
int ieo_evolve_derivsN(ieo_state* S, double d) {
    double* fd = S->fd;
    const long gs = (long)S->gs;
    #pragma omp parallel for schedule(static)
    for (long id = 0; id < gs; ++id) {
        fd[id] += d * (-(3.0 - 0.5 * pw2(fd[id])) * (fd[id] + pot_ratio_site(S, (size_t)id)));
    }
    return S->err;
}

static inline int dn_active(ieo_state* S, double v) {
    if (S->p.criterion > 0) return fabs(v) > fabs(S->phiref);
    if (S->p.criterion < 0) return fabs(v) < fabs(S->phiref);
    return ieo_potential(S, v) > ieo_potential(S, S->phiref);
}

/* evolve_fieldsN(d), src/evolution.cpp:1015-1037 */
void ieo_evolve_fieldsN(ieo_state* S, double d) {
    S->t += d;
    double* f = S->f;
    const double* fd = S->fd;
    double* dn = S->deltaN;
    const long gs = (long)S->gs;
    #pragma omp parallel for schedule(static)
    for (long id = 0; id < gs; ++id) {
        if (dn_active(S, f[id])) {
            dn[id] += d;
            f[id] += d * fd[id];
        }
    }
    S->a += d * S->ad;
}

/* get_phiref(), src/evolution.cpp:1271-1288 */
double ieo_get_phiref(ieo_state* S) {
    double fref = S->f[0];
    for (size_t id = 0; id < S->gs; ++id) {
        const double v = S->f[id];
        int take;
        if (S->p.criterion > 0) take = fabs(v) < fabs(fref);
        else if (S->p.criterion < 0) take = fabs(v) > fabs(fref);
        else take = ieo_potential(S, v) < ieo_potential(S, fref);
        if (take) fref = v;
    }
    return fref;
}

/* compute_deltaN_rhs, src/evolution.cpp:1063-1113: per site, in e-fold time,
 * k_f = fd and k_dn = 1 at active sites (0 and 0 where the site has crossed
 * the end surface), k_fd = -(3 - fd^2/2)(fd + V'/V) with V, V' as
 * evaluate_potential_from_value gives them (divided by B^2 each, the hint
 * stepped back by int_errN).  dadt = ad. */
static int rkN_rhs(ieo_state* S, const double* fs, const double* fds, double* kf, double* kfd, double* kdn) {
    const ieo_params* p = &S->p;
    const double B2 = pw2(p->rescale_B);
    const double Vref = ieo_potential(S, S->phiref);
    for (size_t id = 0; id < S->gs; ++id) {
        const double field = fs[id], deriv = fds[id];
        double pot, dpot;
        if (p->numerical_potential) {
            const int l = bracket(S, field, S->lstart[id]);
            if (l < 0) return 1;
            pot = interp(S, field, l, S->tV) / B2;
            dpot = interp(S, field, l, S->tdV) / B2;
            const int back = p->int_errN > 1 ? p->int_errN : 1;
            S->lstart[id] = (l - back) > 1 ? (l - back) : 1;
        } else {
            pot = hill_V(p, field);
            dpot = hill_dV(p, field);
        }
        const double ratio = dpot / pot;
        int active;
        if (p->criterion > 0) active = fabs(field) > fabs(S->phiref);
        else if (p->criterion < 0) active = fabs(field) < fabs(S->phiref);
        else active = pot > Vref;
        kfd[id] = -(3.0 - 0.5 * pw2(deriv)) * (deriv + ratio);
        kf[id] = active ? deriv : 0.0;
        kdn[id] = active ? 1.0 : 0.0;
    }
    return 0;
}

static void rkN_scratch(ieo_state* S) {
    rk_scratch(S);
    if (S->dntmp) return;
    S->dntmp = (double*)calloc(S->gs, sizeof(double));
    for (int q = 0; q < 7; ++q) S->kdn[q] = (double*)calloc(S->gs, sizeof(double));
}

/* evaluate_deltaN_stage with prepare_deltaN_stage_state, src/evolution.cpp:1115-1145 */
static int rkN_stage(ieo_state* S, double h, int stage, const double (*A)[7]) {
    for (size_t id = 0; id < S->gs; ++id) {
        double sum_f = 0.0, sum_fd = 0.0, sum_dn = 0.0;
        for (int q = 0; q < stage; ++q) {
            const double c = A[stage][q];
            if (c == 0.0) continue;
            sum_f += c * S->kf[q][id];
            sum_fd += c * S->kfd[q][id];
            sum_dn += c * S->kdn[q][id];
        }
        S->ftmp[id] = S->f[id] + h * sum_f;
        S->fdtmp[id] = S->fd[id] + h * sum_fd;
        S->dntmp[id] = S->deltaN[id] + h * sum_dn;
    }
    return rkN_rhs(S, S->ftmp, S->fdtmp, S->kf[stage], S->kfd[stage], S->kdn[stage]);
}

/* rk4_step_deltaN(h), src/evolution.cpp:1176-1188, with
 * apply_deltaN_weighted_update (:1147-1174): a moves with its constant
 * derivative ad, t += h. */
int ieo_rk4_step_deltaN(ieo_state* S, double h) {
    rkN_scratch(S);
    if (rkN_rhs(S, S->f, S->fd, S->kf[0], S->kfd[0], S->kdn[0])) return 1;
    for (int stage = 1; stage < 4; ++stage)
        if (rkN_stage(S, h, stage, RK4_A)) return 1;
    for (size_t id = 0; id < S->gs; ++id) {
        double sum_f = 0.0, sum_fd = 0.0, sum_dn = 0.0;
        for (int q = 0; q < 4; ++q) {
            const double bs = RK4_B[q];
            if (bs == 0.0) continue;
            sum_f += bs * S->kf[q][id];
            sum_fd += bs * S->kfd[q][id];
            sum_dn += bs * S->kdn[q][id];
        }
        S->f[id] += h * sum_f;
        S->fd[id] += h * sum_fd;
        S->deltaN[id] += h * sum_dn;
    }
    for (int q = 0; q < 4; ++q) {
        const double bs = RK4_B[q];
        if (bs == 0.0) continue;
        S->a += h * bs * S->ad;
    }
    S->t += h;
    return 0;
}

/* rk45_step_deltaN(h, hmax, h_next), src/evolution.cpp:1190-1267 */
int ieo_rk45_step_deltaN(ieo_state* S, double h, double hmax, double* h_next, int* accepted) {
    rkN_scratch(S);
    const ieo_params* p = &S->p;
    const double atol = p->rk45_abs_tol, rtol = p->rk45_rel_tol;
    if (rkN_rhs(S, S->f, S->fd, S->kf[0], S->kfd[0], S->kdn[0])) return 1;
    for (int stage = 1; stage < 7; ++stage)
        if (rkN_stage(S, h, stage, DP_A)) return 1;
    double a5 = S->a, erra = 0.0;
    for (int q = 0; q < 7; ++q) {
        if (DP_B[q] != 0.0) a5 += h * DP_B[q] * S->ad;
        if (DP_E[q] != 0.0) erra += h * DP_E[q] * S->ad;
    }
    double err_acc = 0.0;
    const size_t nvars = 3 * S->gs + 1;
    for (size_t id = 0; id < S->gs; ++id) {
        double y5f = S->f[id], y5fd = S->fd[id], y5dn = S->deltaN[id];
        double errf = 0.0, errfd = 0.0, errdn = 0.0;
        for (int q = 0; q < 7; ++q) {
            const double bs = DP_B[q], es = DP_E[q];
            if (bs != 0.0) {
                y5f += h * bs * S->kf[q][id];
                y5fd += h * bs * S->kfd[q][id];
                y5dn += h * bs * S->kdn[q][id];
            }
            if (es != 0.0) {
                errf += h * es * S->kf[q][id];
                errfd += h * es * S->kfd[q][id];
                errdn += h * es * S->kdn[q][id];
            }
        }
        S->ftmp[id] = y5f;
        S->fdtmp[id] = y5fd;
        S->dntmp[id] = y5dn;
        const double sf = atol + rtol * smax(fabs(S->f[id]), fabs(y5f));
        const double sfd = atol + rtol * smax(fabs(S->fd[id]), fabs(y5fd));
        const double sdn = atol + rtol * smax(fabs(S->deltaN[id]), fabs(y5dn));
        err_acc += pw2(errf / sf) + pw2(errfd / sfd) + pw2(errdn / sdn);
    }
    const double sa = atol + rtol * smax(fabs(S->a), fabs(a5));
    err_acc += pw2(erra / sa);
    const double err_norm = sqrt(err_acc / (double)nvars);
    const double safe_err = smax(err_norm, 1e-16);
    double factor = p->rk45_safety * pow(safe_err, -0.2);
    factor = (factor < 0.1) ? 0.1 : (5.0 < factor) ? 5.0 : factor;
    S->rk45_err = err_norm;
    if (err_norm <= 1.0) {
        double* t;
        t = S->f; S->f = S->ftmp; S->ftmp = t;
        t = S->fd; S->fd = S->fdtmp; S->fdtmp = t;
        t = S->deltaN; S->deltaN = S->dntmp; S->dntmp = t;
        S->a = a5;
        S->t += h;
        *h_next = ieo_rk45_clamp(S, h * factor, hmax);
        *accepted = 1;
        return 0;
    }
    *h_next = ieo_rk45_clamp(S, h * smax(0.1, smin(0.5, factor)), hmax);
    *accepted = 0;
    return 0;
}

/* rk45_accept_step around rk45_step_deltaN, src/evolution.cpp:1338-1366 */
int ieo_rk45_accept_deltaN(ieo_state* S, double* h, double hmax) {
    int accepted = 0, attempts = 0;
    while (!accepted) {
        double hs = *h;
        if (ieo_rk45_step_deltaN(S, *h, hmax, &hs, &accepted)) return 1;
        *h = hs;
        ++attempts;
        if (!accepted && (attempts > 25 || *h <= S->p.rk45_min_dt * (1.0 + 1e-12))) {
            set_err(S, "RK45 failed to converge in deltaN loop at N=%e, t=%e (attempts=%d, h=%e)\n", S->Ne, S->t,
                    attempts, *h);
            return 1;
        }
    }
    return 0;
}

int ieo_deltaN_steps(ieo_state* S, int max_steps) {
    int n = 0;
    while (n < max_steps && S->Ne <= S->p.Nend) {
        if (ieo_evolve_derivsN(S, S->p.dN)) return -1;
        ieo_evolve_fieldsN(S, S->p.dN);
        S->Ne += S->p.dN;
        ++n;
    }
    return n;
}

/* saveN() float accumulator, src/output.cpp:1527-1537 */
float ieo_saveN_mean(const ieo_state* S, double cutoff) {
    float Nmean = 0.f;
    for (size_t id = 0; id < S->gs; ++id)
        if (S->deltaN[id] <= cutoff) Nmean = (float)((double)Nmean + S->deltaN[id]);
    Nmean = Nmean / (float)S->gs;
    return Nmean;
}

/* ------------------------------------------------------------------------- */
/* program, src/main.cpp:103-146 and src/output.cpp                          */
/* ------------------------------------------------------------------------- */

/* trace of the background scalars at each save, and full-precision copies of
 * the printed means and spectra (program runner only) */
static FILE* g_trace;
static FILE* g_prec;

static void prec_line(const char* tag, const double* v, int n) {
    if (!g_prec) return;
    fprintf(g_prec, "%s", tag);
    for (int i = 0; i < n; ++i) fprintf(g_prec, " %.17g", v[i]);
    fprintf(g_prec, "\n");
}

typedef struct {
    char dir[1024];
    FILE *output, *means, *vars, *velocity, *sf, *energy, *conservation, *spectra, *spectratimes,
         *histogram, *histogramtimes, *spectraGW, *spectraGWdot, *modes, *spectraN, *histogramN,
         *histogramtimesN, *box2d_phi, *box2d_phidot, *box2d_deltaN, *box3d, *info;
    /* results/post_inflation/, src/output.cpp:1573-1867 */
    FILE *pmeans, *pvars, *pvelocity, *psf, *pspectra, *pspectratimes, *pspectraGW, *pspectraGWdot, *phistogram,
         *phistogramtimes;
    time_t tstart;
} outfiles;

static FILE* open_out(ieo_state* S, outfiles* O, FILE** slot, const char* name) {
    if (*slot) return *slot;
    char path[1200];
    snprintf(path, sizeof path, "%s/%s.dat", O->dir, name);
    *slot = fopen(path, "w");
    if (!*slot) set_err(S, "Failed to open output file: %s\n", path);
    return *slot;
}

/* write_isotropic_spectrum_from_fft_r2c printing, src/output.cpp:143-150 */
static void print_spectrum(FILE* out, int N, double L, const int* counts, double* f2, double norm1, const char* tag) {
    const int numbins = ieo_numbins(N);
    const double dp = 2.0 * (2.0 * asin(1.0)) / L;
    double* pv = (double*)malloc(sizeof(double) * numbins);
    for (int i = 0; i < numbins; i++) {
        const double pi_ = dp * i;
        if (counts[i] > 0) f2[i] /= (double)counts[i];
        fprintf(out, "%e %d %e\n", pi_, counts[i], norm1 * f2[i]);
        pv[i] = norm1 * f2[i];
    }
    prec_line(tag, pv, numbins);
    free(pv);
    fprintf(out, "\n");
    fflush(out);
}

/* meansvars, src/output.cpp:204-269; post: meansvars_post_inflation,
 * src/output.cpp:1576-1639 (same columns, results/post_inflation/) */
static int out_meansvars(ieo_state* S, outfiles* O, int post) {
    FILE* m = post ? open_out(S, O, &O->pmeans, "post_inflation/means") : open_out(S, O, &O->means, "means");
    FILE* v = post ? open_out(S, O, &O->pvars, "post_inflation/variance") : open_out(S, O, &O->vars, "variance");
    FILE* ve = post ? open_out(S, O, &O->pvelocity, "post_inflation/velocity")
                    : open_out(S, O, &O->velocity, "velocity");
    if (S->err) return 1;
    fprintf(m, "%f", S->t); fprintf(m, " %e", S->a);
    fprintf(ve, "%f", S->t); fprintf(ve, " %e", S->a);
    fprintf(v, "%f", S->t); fprintf(v, " %e", S->a);
    double av = 0., vel = 0., var = 0.;
    for (size_t id = 0; id < S->gs; ++id) { av += S->f[id]; vel += S->fd[id]; var += pw2(S->f[id]); }
    av = av / (double)S->gs;
    vel = vel / (double)S->gs;
    vel = vel * pow(S->a, S->p.rescale_s - 1.0) * S->p.rescale_B;
    fprintf(m, " %e", av); fprintf(ve, " %e", vel); fprintf(v, " %e", var - pw2(av));
    {
        const double q[5] = {S->t, S->a, av, vel, S->ad * S->p.rescale_B * pow(S->a, S->p.rescale_s - 2.0)};
        prec_line(post ? "post_means" : "means", q, 5);
    }
    if (av + DBL_MAX == av || (av != 0. && av / av != 1.)) {
        set_err(S, "Unstable solution developed. Scalar field not numerical at t=%f\n", S->t);
        fflush(m); fflush(v);
        return 1;
    }
    fprintf(m, "\n"); fprintf(v, "\n"); fprintf(ve, "\n");
    fflush(m); fflush(v); fflush(ve);
    return 0;
}

/* scale, src/output.cpp:272-293; post: scale_post_inflation, src/output.cpp:1642-1662 */
static void out_scale(ieo_state* S, outfiles* O, int post) {
    FILE* fp = post ? open_out(S, O, &O->psf, "post_inflation/sf") : open_out(S, O, &O->sf, "sf");
    if (!fp) return;
    const double s = S->p.rescale_s, B = S->p.rescale_B, a = S->a;
    fprintf(fp, "%f %f %e %e\n", S->t, a, S->ad * B * pow(a, s - 2.0),
            pw2(B) * pow(a, 2.0 * s - 2.0) * (S->ad2 + (s - 1.0) * pw2(S->ad) / a));
    fflush(fp);
}

/* energy, src/output.cpp:983-1026 */
static int out_energy(ieo_state* S, outfiles* O) {
    FILE* e = open_out(S, O, &O->energy, "energy");
    FILE* c = open_out(S, O, &O->conservation, "conservation");
    if (S->err) return 1;
    const double B = S->p.rescale_B;
    double totalE = 0.;
    fprintf(e, "%f", S->t); fprintf(e, " %e", S->a);
    const double de = ieo_kin_energy(S); totalE += de; fprintf(e, " %e", de * B);
    const double ge = ieo_gradient_energy(S); totalE += ge; fprintf(e, " %e", ge * B);
    const double pe = ieo_potential_energy(S); totalE += pe; fprintf(e, " %e", pe * B);
    fprintf(e, "\n"); fflush(e);
    fprintf(c, "%e %e %e\n", S->t, S->a, 3.0 * pow(S->a, 2.0 * S->p.rescale_s - 4.0) * pw2(S->ad) / (totalE));
    fflush(c);
    return S->err;
}

/* histograms / histogramsN, src/output.cpp:1070-1135 and 1220-1277 */
static void out_histogram(ieo_state* S, const double* x, FILE* hist, FILE* times, int deltaN_style) {
    const int nbins = S->p.nbins;
    if (deltaN_style) fprintf(times, "%f %e", S->t, S->a);
    else { fprintf(times, "%f", S->t); fprintf(times, " %e", S->a); }
    double bmin = x[0], bmax = bmin;
    for (size_t id = 0; id < S->gs; ++id) {
        bmin = (x[id] < bmin ? x[id] : bmin);
        bmax = (x[id] > bmax ? x[id] : bmax);
    }
    double df = (bmax - bmin) / (double)nbins;
    if (!isfinite(df) || df <= 0.0) df = 1.0;
    double* binfreq = (double*)calloc(nbins > 0 ? nbins : 1, sizeof(double));
    int numpts = 0;
    for (size_t id = 0; id < S->gs; ++id) {
        int binnum = (int)((x[id] - bmin) / df);
        if (x[id] == bmax) binnum = nbins - 1;
        if (binnum >= 0 && binnum < nbins) { binfreq[binnum]++; numpts++; }
    }
    if (numpts == 0) numpts = 1;
    for (int i = 0; i < nbins; i++) fprintf(hist, "%e\n", binfreq[i] / (double)numpts);
    fprintf(hist, "\n");
    fflush(hist);
    if (deltaN_style) fprintf(times, " %e %e\n", bmin, df);
    else { fprintf(times, " %e %e", bmin, df); fprintf(times, "\n"); }
    fflush(times);
    free(binfreq);
}

static void out_box2d(ieo_state* S, FILE* fp, const double* x, double scale, int scaled) {
    const int N = S->p.N;
    const int i = (N < 64) ? 5 : 50;
    for (int j = 0; j < N; j++) for (int k = 0; k < N; k++) {
        if (scaled) fprintf(fp, "%.17g\n", x[IDX(N, i, j, k)] * scale);
        else fprintf(fp, "%.17g\n", x[IDX(N, i, j, k)]);
    }
    fprintf(fp, "\n");
    fflush(fp);
}

/* spectraGW / spectraGWdot printing, src/output.cpp:618-624.  Post:
 * spectraGW_post_inflation / spectraGWdot_post_inflation, src/output.cpp:652-669;
 * the latter scales h' in float by (float)(B a^(s-1)), which gives the same
 * bits as rounding (double)h' * (double)(float)(B a^(s-1)) to float (the
 * double product of two floats is exact). */
static void out_gw(ieo_state* S, outfiles* O, int which, int post) {
    FILE* fp = post ? (which ? open_out(S, O, &O->pspectraGWdot, "post_inflation/spectraGWdot")
                             : open_out(S, O, &O->pspectraGW, "post_inflation/spectraGW"))
                    : (which ? open_out(S, O, &O->spectraGWdot, "spectraGWdot")
                             : open_out(S, O, &O->spectraGW, "spectraGW"));
    if (!fp) return;
    const int N = S->p.N;
    const int numbins = (int)(sqrt(3.0) * (N / 2)) + 1;
    int* counts = (int*)calloc(numbins, sizeof(int));
    float* f2 = (float*)calloc(numbins, sizeof(float));
    double to_phys = which ? S->p.rescale_B * pow(S->a, S->p.rescale_s - 1.0) : 1.0;
    if (post && which) to_phys = (double)(float)to_phys;
    double* f2d = (double*)calloc(numbins, sizeof(double));
    ieo_gw_spectrum(S, which, to_phys, counts, f2, f2d);
    if (g_prec) {
        const double n1 = 0.5 * pow(S->p.L / S->p.rescale_B, 3) / pow((double)N, 6);
        for (int i = 0; i < numbins; ++i) f2d[i] = counts[i] > 0 ? n1 * f2d[i] / counts[i] : 0.0;
        prec_line(which ? (post ? "post_spectrumGWdot" : "spectrumGWdot") : (post ? "post_spectrumGW" : "spectrumGW"),
                  f2d, numbins);
    }
    free(f2d);
    const float dp = 2.f * (float)S->pi / (float)S->p.L;
    const float norm1 = 0.5f * pow(S->p.L / S->p.rescale_B, 3) / pow((double)(float)N, 6);
    for (int i = 0; i < numbins; ++i) {
        const float pi_ = dp * i;
        if (counts[i] > 0) f2[i] /= (float)counts[i];
        fprintf(fp, "%e %d %e\n", pi_, counts[i], norm1 * f2[i]);
    }
    fprintf(fp, "\n");
    fflush(fp);
    free(counts); free(f2);
}

/* save(), src/output.cpp:1469-1503 */
static int out_save(ieo_state* S, outfiles* O, int infrequent) {
    const ieo_params* p = &S->p;
    if (g_trace)
        fprintf(g_trace, "save %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, S->t, S->a, S->ad, S->ad2, S->astep);
    /* the half-step sync is the leapfrog's (inflation_uses_staggered_derivatives, src/main.h:184-186) */
    const int stag = p->inflation_integrator == 0;
    if (stag && S->t > 0.) ieo_evolve_fields(S, -.5 * p->dt * pow(S->astep, p->rescale_s - 1));
    if (out_meansvars(S, O, 0)) return 1;
    out_scale(S, O, 0);
    if (infrequent) {
        if (p->output_box3D) {
            FILE* fp = open_out(S, O, &O->box3d, "box");
            for (size_t id = 0; id < S->gs; ++id) fprintf(fp, "%.17g\n", S->f[id]);
            fprintf(fp, "\n");
        }
        if (p->output_box2D) {
            out_box2d(S, open_out(S, O, &O->box2d_phi, "snapshots_2d_phi"), S->f, 0, 0);
            out_box2d(S, open_out(S, O, &O->box2d_phidot, "snapshots_2d_phidot"), S->fd, p->rescale_B, 1);
        }
        if (p->output_energy && out_energy(S, O)) return 1;
        if (p->output_spectra) {
            FILE* sp = open_out(S, O, &O->spectra, "spectra");
            FILE* st = open_out(S, O, &O->spectratimes, "spectratimes");
            if (S->err) return 1;
            const int nb = ieo_numbins(p->N);
            int* counts = (int*)calloc(nb, sizeof(int));
            double* f2 = (double*)calloc(nb, sizeof(double));
            const double norm1 = pow(p->L / p->rescale_B, 3) / pow((double)p->N, 6);
            ieo_fftrn_d(S->f, S->fny, p->N, 1);
            ieo_bin_spectrum(p->N, S->f, S->fny, counts, f2);
            print_spectrum(sp, p->N, p->L, counts, f2, norm1, "spectrum");
            fprintf(st, "%f %e\n", S->t, S->a);
            fflush(st);
            if (p->high_cutoff_index > 0 && p->forcing_cutoff)
                ieo_forcing_cutoff(S, p->high_cutoff_index, p->low_cutoff_index);
            ieo_fftrn_d(S->f, S->fny, p->N, -1);
            free(counts); free(f2);
            if (p->calculate_SIGW) { out_gw(S, O, 0, 0); out_gw(S, O, 1, 0); }
        }
        if (p->output_histogram)
            out_histogram(S, S->f, open_out(S, O, &O->histogram, "histogram"),
                          open_out(S, O, &O->histogramtimes, "histogramtimes"), 0);
    }
    if (stag && S->t > 0.) ieo_evolve_fields(S, .5 * p->dt * pow(S->astep, p->rescale_s - 1));
    return S->err;
}

/* save_post_inflation(), src/output.cpp:1840-1865 (leapfrog: staggered) */
static int out_save_post(ieo_state* S, outfiles* O, int infrequent) {
    const ieo_params* p = &S->p;
    if (g_trace)
        fprintf(g_trace, "savep %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, S->t, S->a, S->ad, S->ad2, S->astep);
    /* the sync is the leapfrog's (post_inflation_uses_staggered_derivatives, src/main.h:193-195) */
    const int stag = p->post_inflation_integrator == 0;
    if (stag && S->t > 0.) ieo_evolve_fields(S, -.5 * p->dt_post_inflation);
    if (out_meansvars(S, O, 1)) return 1;
    out_scale(S, O, 1);
    if (infrequent) {
        if (p->output_spectra) {
            /* spectraf_post_inflation(), src/output.cpp:1667-1770 */
            FILE* sp = open_out(S, O, &O->pspectra, "post_inflation/spectra");
            FILE* st = open_out(S, O, &O->pspectratimes, "post_inflation/spectratimes");
            if (S->err) return 1;
            const int nb = ieo_numbins(p->N);
            int* counts = (int*)calloc(nb, sizeof(int));
            double* f2 = (double*)calloc(nb, sizeof(double));
            const double norm1 = pow(p->L / p->rescale_B, 3) / pow((double)p->N, 6);
            ieo_fftrn_d(S->f, S->fny, p->N, 1);
            ieo_bin_spectrum(p->N, S->f, S->fny, counts, f2);
            print_spectrum(sp, p->N, p->L, counts, f2, norm1, "post_spectrum");
            fprintf(st, "%f %e\n", S->t, S->a);
            fflush(st);
            if (p->high_cutoff_index > 0 && p->forcing_cutoff)
                ieo_forcing_cutoff(S, p->high_cutoff_index, p->low_cutoff_index);
            ieo_fftrn_d(S->f, S->fny, p->N, -1);
            free(counts); free(f2);
            out_gw(S, O, 0, 1);
            out_gw(S, O, 1, 1);
        }
        if (p->output_histogram)
            out_histogram(S, S->f, open_out(S, O, &O->phistogram, "post_inflation/histogram"),
                          open_out(S, O, &O->phistogramtimes, "post_inflation/histogramtimes"), 0);
    }
    if (stag && S->t > 0.) ieo_evolve_fields(S, .5 * p->dt_post_inflation);
    return S->err;
}

/* get_modes, src/output.cpp:674-738 */
static void out_modes(ieo_state* S, outfiles* O) {
    FILE* fp = open_out(S, O, &O->modes, "modes");
    if (!fp) return;
    const int N = S->p.N;
    const double L = S->p.L, pi = S->pi;
    const int numbins = (int)(sqrt(3.0) * (N / 2)) + 1;
    int* np = (int*)calloc(numbins + 1, sizeof(int));
    double* pp = (double*)calloc(numbins + 1, sizeof(double));
    for (int i = 0; i < N; i++) {
        const int px = (i <= N / 2 ? i : i - N);
        for (int j = 0; j < N; j++) {
            const int py = (j <= N / 2 ? j : j - N);
            for (int k = 1; k < N / 2; k++) {
                const int pz = k;
                const double pm = sqrt(pw2((double)px) + pw2((double)py) + pw2((double)pz));
                const double pph = sqrt(4.0 * pw2((double)N / (double)L) * (pw2(sin((double)px * pi / N)) + pw2(sin((double)py * pi / N)) + pw2(sin((double)pz * pi / N))));
                np[(int)pm] += 2;
                pp[(int)pm] += 2.0 * pph;
            }
            for (int k = 0; k <= N / 2; k += N / 2) {
                const int pz = k;
                const double pm = sqrt(pw2((double)px) + pw2((double)py) + pw2((double)pz));
                const double pph = sqrt(4.0 * pw2((double)N / (double)L) * (pw2(sin((double)px * pi / N)) + pw2(sin((double)py * pi / N)) + pw2(sin((double)pz * pi / N))));
                np[(int)pm]++;
                pp[(int)pm] += pph;
            }
        }
    }
    for (int i = 0; i < numbins; i++) {
        if (np[i] > 0) pp[i] = pp[i] / np[i];
        fprintf(fp, "%e\n", S->p.rescale_B * pp[i]);
    }
    fprintf(fp, "\n");
    fflush(fp);
    free(np); free(pp);
}

/* saveN(), src/output.cpp:1522-1560, with spectraN() of :1140-1169 */
static int out_saveN(ieo_state* S, outfiles* O) {
    const ieo_params* p = &S->p;
    if (g_trace) fprintf(g_trace, "saveN %.17g %.17g %.17g %.17g\n", S->t, S->a, S->Ne, S->phiref);
    /* the sync and the dN below Nend are the leapfrog's (deltaN_uses_staggered_derivatives, src/output.cpp:1523-1527) */
    const int stag = p->deltaN_integrator == 0;
    if (stag && S->t > 0.) ieo_evolve_fieldsN(S, -.5 * p->dN);
    const double cutoff = p->Nend - (stag ? p->dN : 0.0);
    const float Nmean = ieo_saveN_mean(S, cutoff);
    for (size_t id = 0; id < S->gs; ++id) S->deltaN[id] -= Nmean;
    out_histogram(S, S->deltaN, open_out(S, O, &O->histogramN, "histogramN"),
                  open_out(S, O, &O->histogramtimesN, "histogramtimesN"), 1);
    if (p->output_box2D) out_box2d(S, open_out(S, O, &O->box2d_deltaN, "snapshots_2d_deltaN"), S->deltaN, 0, 0);
    for (size_t id = 0; id < S->gs; ++id)
        if (S->deltaN[id] > (cutoff - Nmean)) S->deltaN[id] = 0;
    if (p->output_spectra) {
        FILE* sp = open_out(S, O, &O->spectraN, "spectraN");
        if (!sp) return 1;
        double m = 0.0;
        for (size_t id = 0; id < S->gs; ++id) m += S->deltaN[id];
        m /= (double)S->gs;
        for (size_t id = 0; id < S->gs; ++id) S->deltaN[id] -= m;
        const int nb = ieo_numbins(p->N);
        int* counts = (int*)calloc(nb, sizeof(int));
        double* f2 = (double*)calloc(nb, sizeof(double));
        const double norm1 = pow(p->L / p->rescale_B, 3) / pow((double)p->N, 6);
        ieo_fftrn_d(S->deltaN, S->fny, p->N, 1);
        ieo_bin_spectrum(p->N, S->deltaN, S->fny, counts, f2);
        print_spectrum(sp, p->N, p->L, counts, f2, norm1, "spectrumN");
        ieo_fftrn_d(S->deltaN, S->fny, p->N, -1);
        free(counts); free(f2);
    }
    if (stag && S->t > 0.) ieo_evolve_fieldsN(S, .5 * p->dN);
    return S->err;
}

static int load_table_file(const char* path, double** out, int* n) {
    FILE* fp = fopen(path, "r");
    if (!fp) return -1;
    int cap = 2048, m = 0;
    double* v = (double*)malloc(sizeof(double) * cap);
    double x;
    while (fscanf(fp, "%lf", &x) == 1) {
        if (m == cap) { cap *= 2; v = (double*)realloc(v, sizeof(double) * cap); }
        v[m++] = x;
    }
    fclose(fp);
    if (m == 0) { free(v); return -2; }
    *out = v;
    *n = m;
    return 0;
}

static void close_all(outfiles* O) {
    FILE** all[] = {&O->output, &O->means, &O->vars, &O->velocity, &O->sf, &O->energy, &O->conservation,
                    &O->spectra, &O->spectratimes, &O->histogram, &O->histogramtimes, &O->spectraGW,
                    &O->spectraGWdot, &O->modes, &O->spectraN, &O->histogramN, &O->histogramtimesN,
                    &O->box2d_phi, &O->box2d_phidot, &O->box2d_deltaN, &O->box3d, &O->info,
                    &O->pmeans, &O->pvars, &O->pvelocity, &O->psf, &O->pspectra, &O->pspectratimes,
                    &O->pspectraGW, &O->pspectraGWdot, &O->phistogram, &O->phistogramtimes};
    for (size_t q = 0; q < sizeof(all) / sizeof(all[0]); ++q)
        if (*all[q]) { fclose(*all[q]); *all[q] = NULL; }
}

static void write_state(ieo_state* S, const char* path) {
    FILE* fp = fopen(path, "wb");
    if (!fp) return;
    const double scal[8] = {S->t, S->a, S->ad, S->ad2, S->astep, S->Ne, S->phiref, S->hubble_init};
    const int hdr[4] = {S->p.N, S->p.perform_deltaN, S->p.calculate_SIGW, S->p.numerical_potential};
    fwrite(hdr, sizeof(int), 4, fp);
    fwrite(scal, sizeof(double), 8, fp);
    fwrite(S->f, sizeof(double), S->gs, fp);
    fwrite(S->fd, sizeof(double), S->gs, fp);
    if (S->p.perform_deltaN) fwrite(S->deltaN, sizeof(double), S->gs, fp);
    if (S->p.calculate_SIGW) {
        for (int c = 0; c < 6; ++c) fwrite(S->h[c], sizeof(float), S->gs, fp);
        for (int c = 0; c < 6; ++c) fwrite(S->hd[c], sizeof(float), S->gs, fp);
    }
    fclose(fp);
}

int ieo_run_program(const ieo_params* p, const char* results_dir, const char* inputs_dir) {
    return ieo_run_program_dump(p, results_dir, inputs_dir, NULL);
}

/* As ieo_run_program; when dump_dir is given, also writes trace.txt (the
 * background scalars at every save) and state.bin (the final state) there,
 * in the format of oracle/ref_driver.cpp. */
int ieo_run_program_dump(const ieo_params* p, const char* results_dir, const char* inputs_dir, const char* dump_dir) {
    outfiles O;
    memset(&O, 0, sizeof O);
    snprintf(O.dir, sizeof O.dir, "%s", results_dir);
    mkdir(results_dir, 0777);
    ieo_state* S = ieo_create(p);
    if (!S) return 1;
    int rc = 1;
    char path[1200];
    snprintf(path, sizeof path, "%s/output.txt", results_dir);
    O.output = fopen(path, "w");
    if (dump_dir) {
        snprintf(path, sizeof path, "%s/trace.txt", dump_dir);
        g_trace = fopen(path, "w");
        snprintf(path, sizeof path, "%s/precise.txt", dump_dir);
        g_prec = fopen(path, "w");
    }
    if (!O.output) goto done;
    if (p->numerical_potential) {
        double *x = NULL, *V = NULL, *dV = NULL;
        int n1, n2, n3;
        char q[1200];
        snprintf(q, sizeof q, "%s/field_values.dat", inputs_dir);
        if (load_table_file(q, &x, &n1)) goto done;
        snprintf(q, sizeof q, "%s/potential.dat", inputs_dir);
        if (load_table_file(q, &V, &n2)) goto done;
        snprintf(q, sizeof q, "%s/potential_derivative.dat", inputs_dir);
        if (load_table_file(q, &dV, &n3)) goto done;
        ieo_set_table(S, x, V, dV, n1);
        free(x); free(V); free(dV);
    }
    /* initialize_simulation(), src/initialize.cpp:40-48 */
    if (ieo_initialize(S)) goto done;
    if (ieo_initializef(S)) goto done;
    ieo_initializeGW(S);
    {
        FILE* info = open_out(S, &O, &O.info, "info");
        time(&O.tstart);
        if (info) { fprintf(info, "Grid size=%d^%d\nL=%f\n", p->N, 3, p->L); fflush(info); }
    }
    if (out_save(S, &O, 1)) goto done;
    S->t = S->t0;

    /* run_evolution_loop(), src/evolution.cpp:909-997 */
    {
        int numsteps = 0;
        const int leap = p->inflation_integrator == 0;
        /* RK45: the first h, src/evolution.cpp:959 */
        double h45 = ieo_rk45_clamp(S, ieo_rescaled_step(S, S->astep), p->rk45_max_dt);
        if (leap) ieo_evolve_fields(S, 0.5 * p->dt);
        while (S->a <= p->af) {
            const double d = ieo_rescaled_step(S, S->astep);
            if (leap) {
                if (ieo_evolve_derivs(S, d)) goto done;
                ieo_evolve_fields(S, d);
            } else if (p->inflation_integrator == 1) {
                if (ieo_rk4_step_inflation(S, d)) goto done;
            } else {
                const double hmax = ieo_rk45_hmax(S, d);
                h45 = ieo_rk45_clamp(S, h45, hmax);
                if (ieo_rk45_accept(S, &h45, hmax)) goto done;
            }
            numsteps++;
            if (numsteps % p->output_freq == 0 && S->a < p->af)
                if (out_save(S, &O, (numsteps % p->output_infrequent_freq == 0) ? 1 : 0)) goto done;
            fprintf(O.output, "scale factor a = %f\n", S->a);
            fprintf(O.output, "numsteps %i\n\n", numsteps);
            if (numsteps % p->output_freq == 0) fflush(O.output);
            S->astep = S->a;
        }
        fflush(O.output);
        if (out_save(S, &O, 1)) goto done;
        if (leap) ieo_evolve_fields(S, -0.5 * ieo_rescaled_step(S, S->astep));
        out_modes(S, &O);
    }

    /* run_deltaN_loop(), leapfrog, RK4 and RK45 branches, src/evolution.cpp:1291-1375 */
    if (p->perform_deltaN) {
        fprintf(O.output, "Starting deltaN calculation\n");
        int numsteps = 0;
        const int nint = p->deltaN_integrator;
        S->Ne = 0.0;
        if (ieo_initializeN(S)) goto done;
        if (nint == 0) ieo_evolve_fieldsN(S, 0.5 * p->dN);
        S->phiref = p->use_phiref_manual ? p->phiref_manual_value : ieo_get_phiref(S);
        double hN = ieo_rk45_clamp(S, p->dN, p->rk45_max_dt);
        while (S->Ne <= p->Nend) {
            if (nint == 0) {
                if (ieo_evolve_derivsN(S, p->dN)) goto done;
                ieo_evolve_fieldsN(S, p->dN);
                S->Ne += p->dN;
            } else if (nint == 1) {
                if (ieo_rk4_step_deltaN(S, p->dN)) goto done;
                S->Ne += p->dN;
            } else {
                const double hmax = ieo_rk45_hmax(S, p->dN);
                hN = ieo_rk45_clamp(S, hN, hmax);
                if (ieo_rk45_accept_deltaN(S, &hN, hmax)) goto done;
                S->Ne += hN;   /* the step proposed for the next iteration, as the reference adds it */
            }
            numsteps++;
            fprintf(O.output, "N = %f\n\n", S->Ne);
            if (numsteps % p->output_freq == 0) fflush(O.output);
        }
        if (out_saveN(S, &O)) goto done;
        fflush(O.output);
        if (nint == 0) ieo_evolve_fieldsN(S, -0.5 * p->dN);
    }
    /* run_post_inflation_loop(), leapfrog, RK4 and RK45 branches, src/evolution.cpp:1561-1653 */
    if (p->post_inflation) {
        if (!p->calculate_SIGW) {
            set_err(S, "post_inflation requires calculate_SIGW = 1\n");
            goto done;
        }
        snprintf(path, sizeof path, "%s/post_inflation", results_dir);
        mkdir(path, 0777);
        ieo_initialize_post_inflation(S);
        if (out_save_post(S, &O, 1)) goto done;
        int numsteps = 0;
        const int pint = p->post_inflation_integrator;
        /* RK branches: the post-inflation right-hand side (ScopedPostInflationRhsMode) */
        S->rk_post = pint != 0;
        double h45 = ieo_rk45_clamp(S, p->dt_post_inflation, p->rk45_max_dt);
        if (pint == 0) ieo_evolve_fields(S, 0.5 * p->dt_post_inflation);
        while (S->a <= p->af_post_inflation) {
            if (pint == 0) {
                ieo_evolve_derivs_post_inflation(S, p->dt_post_inflation);
                ieo_evolve_fields(S, p->dt_post_inflation);
            } else if (pint == 1) {
                if (ieo_rk4_step_inflation(S, p->dt_post_inflation)) goto done;
            } else {
                const double hmax = ieo_rk45_hmax(S, p->dt_post_inflation);
                h45 = ieo_rk45_clamp(S, h45, hmax);
                if (ieo_rk45_accept(S, &h45, hmax)) goto done;
            }
            numsteps++;
            if (numsteps % p->output_freq == 0)
                if (out_save_post(S, &O, (numsteps % p->output_infrequent_freq == 0) ? 1 : 0)) goto done;
            fprintf(O.output, "scale factor a = %f\n", S->a);
            fprintf(O.output, "numsteps %i\n\n", numsteps);
            if (numsteps % p->output_freq == 0) fflush(O.output);
        }
        fflush(O.output);
        if (out_save_post(S, &O, 1)) goto done;
    }
    fprintf(O.output, "InflationEasy program finished\n");
    if (dump_dir) {
        snprintf(path, sizeof path, "%s/state.bin", dump_dir);
        write_state(S, path);
    }
    rc = 0;
done:
    if (g_trace) { fclose(g_trace); g_trace = NULL; }
    if (g_prec) { fclose(g_prec); g_prec = NULL; }
    if (rc && S->err) {
        fprintf(stderr, "%s", S->errmsg);
    }
    close_all(&O);
    ieo_destroy(S);
    return rc;
}
