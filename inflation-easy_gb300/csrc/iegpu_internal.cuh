// iegpu_internal.cuh -- shared definitions of the GB300 InflationEasy engine.
//
// Device layout (one context = one N^3 lattice, all in HBM):
//   plain FP64 form:  f[2] (ping-pong, N^3 double), fd (N^3 double, updated in
//                     place), deltaN (N^3 double), Nyquist planes (N x 2N).
//   SIGW:             h[2][6] (ping-pong, N^3 float each), hd[6] (N^3 float).
// Index (i*N + j)*N + k with k fastest, the reference's layout
// (src/main.h:34-38), so uploads and downloads are plain copies.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/iegpu.h"
#include "exact.cuh"

namespace iegpu {

constexpr int kThreads = 256;

// Background scalars and per-step coefficients, resident on the device so the
// leapfrog loop never returns to the host between steps.
struct DevBg {
    double t, a, ad, ad2, astep;
};

struct DevStep {
    double d;          // rescaled step dt*astep^(s-1)       (src/evolution.cpp:938)
    double laplnorm;   // a^(-2s)/dx^2                       (src/evolution.cpp:153)
    double friction;   // (2+s) ad/a after the first half-kick (src/evolution.cpp:167)
    double potnorm;    // a^(2-2s)                           (src/evolution.cpp:168)
    double srcAmp;     // 2 a^(-2s)                          (src/evolution.cpp:185)
    int active;        // 0 once the loop has ended
    int pad;
};

struct DevCtl {
    DevBg bg;
    DevStep st;
    double af;
    double d_given;     // kick-only mode (evolve_derivs) step size
    int steps_done;
    int steps_limit;
    int done;
    int mode;           // kModeLeapfrog or kModeKick
    int error;          // first device-side error code
    unsigned sumflags;  // exact lattice sums: bit q set, sum q met a non-finite term
    double errval;      // offending value for IEGPU_ERANGE
};

constexpr int kModeLeapfrog = 0;
constexpr int kModeKick = 1;

// Potential description passed by value to kernels.
struct PotDev {
    int table;          // 0 hilltop, 1 tabulated
    int n;              // table length
    double V0, c1, c2, B2;  // hilltop: V = V0(1 - c1 v^2)/B2, V' = (c2 v)/B2
    DivConst divB2;         // x / B2, correctly rounded, on the integer pipes
    const double* x;        // table nodes (descending)
    const long long* key;   // monotone integer keys of x
    const double* V;        // V at nodes
    const double* dV;       // V' at nodes
    const double* dxl;      // x[l-1] - x[l]
    const double* dyV;      // V[l-1] - V[l]
    const double* dydV;     // dV[l-1] - dV[l]
    const double* slopeV;   // dyV/dxl
    const double* slopedV;  // dydV/dxl
    const DivConst* ddx;    // x / dxl[l], correctly rounded, on the integer pipes
};

// Split form (FP32 perturbations about an FP64 background).
constexpr int kWin = 24;  // table brackets per window

// Window of table brackets around a background value phibar: brackets
// l0 .. l0+n-1, node offsets u[q] = x[l0-1+q] - phibar (descending), and per
// bracket the line A[q] + s[q]*dphi = F(phibar + dphi) - F(phibar).  phibar
// and Fbar = F(phibar) let a site beyond the window form its bracket's line
// from the whole table (far_line).
struct SplitWin {
    double phibar, Fbar;
    int l0, n, ok, pad;
    float u[kWin + 1];
    float A[kWin];
    float s[kWin];
};

// The part of the scalar update that does not depend on the step's lattice
// sums, formed during the step by the first CTA to finish its tile:
//   E = c0 + cS0 S0 + cS1 S1 + cS2 S2      (2 grad/3 + pot)
//   x = cx0 + cx1 E,  ad2 = ca0 + ca1 sqrt(1 + x),  adh = ad + hd ad2
//   friction = cf adh,  pibar' = cb0 + cb1 friction
//
// With `fast` set (hilltop potential, vector row kernel), the coefficients of
// the friction's chain are also held as double-float pairs (hi[q] + lo[q],
// q = kPreC0 .. kPreCf), so the last CTA of the step forms the friction on
// the FP32 pipes and leaves the FP64 update of a, ad, t, phibar and pibar to
// the next step (`deferred` in SplitCtl).
enum { kPreC0, kPreS0, kPreS1, kPreS2, kPreX0, kPreX1, kPreA0, kPreA1, kPreAd, kPreHd, kPreCf, kPreN };
struct SplitPre {
    int ok, fast;
    double d, astep, hd;
    double c0, cS0, cS1, cS2, cx0, cx1, ca0, ca1, cf, cb0, cb1;
    float lapl, pn, kv, srcAmp, d32, pad;
    float hi[kPreN], lo[kPreN];
};

struct SplitCtl {
    DevBg bg;
    double phibar, pibar;   // FP64 background
    double af, d_given, errval, dd;
    int steps_done, steps_limit, done, mode, error, active;
    // coefficients of the coming step, in FP32 for the lattice
    float d, lapl, fric, pn, kv, srcAmp;
    SplitWin wk;   // V' window around phibar of the coming step (kick)
    SplitWin wv;   // V window around phibar after it (sums of the new dphi)
    double sums[3];
    int pre_claim, pad2;
    SplitPre pre;
    // A scalar update whose FP64 part is still to be applied: the step's sums
    // as double-float pairs and the index of its a_trace entry.
    int deferred, def_step;
    float dsum_hi[3], dsum_lo[3];
    // bounded device waits: poll limit (0: the default) and, for tests, a
    // bias added to the persistent step barrier's target so that it is never
    // reached
    unsigned spin_polls, spin_bias;
};

// Per-lattice constants of the split step: base step, rescaling exponent,
// lattice spacing, number of sites, and the reciprocals the per-step scalar
// update multiplies by (1/dt, 1/dx, 1/dx^2, 1/N^3, 1/(s+1), 1/B^2).
struct SplitConst {
    double dt, s, dx, gs;
    double idt, idx, idx2, igs, isfev1, iB2;
};

inline SplitConst make_split_const(double dt, double s, double dx, double gs, double B2) {
    SplitConst K;
    K.dt = dt;
    K.s = s;
    K.dx = dx;
    K.gs = gs;
    K.idt = 1.0 / dt;
    K.idx = 1.0 / dx;
    K.idx2 = 1.0 / (dx * dx);
    K.igs = 1.0 / gs;
    K.isfev1 = 1.0 / (s + 1.0);
    K.iB2 = 1.0 / B2;
    return K;
}

// Launch shape of the split row kernel (chosen by the autotuner).
struct RowCfg {
    int TJ = 0;       // rows per tile (0: untuned default)
    int PF = 2;       // planes prefetched
    int chunks = 1;   // plane ranges along i
    int tma = 0;      // planes staged by bulk (TMA) copies instead of cp.async
};

struct SigwSplit {
    const float* hs[6];
    float* hdst[6];
    float* hd[6];
};

struct FftTw {
    // complex-pass twiddles for line length M, per direction, stage-major
    // (stage s uses entries [2^(s-1)-1, 2^s-1)), computed on the host with the
    // reference's recurrence; unpack twiddles for b = 1..N/4-1.
    double2* c_fwd_d[2];   // [0]: length N, [1]: length N/2
    double2* c_inv_d[2];
    double2* unpack_d;
    float2* c_fwd_f[2];
    float2* c_inv_f[2];
    float2* unpack_f;
};

}  // namespace iegpu

struct iegpu_ctx {
    iegpu_config cfg;
    int N = 0, lg = 0;
    size_t gs = 0;          // N^3
    int sms = 0;
    int persist = 1;   // split form, vector row kernel: many steps per cooperative launch
    cudaStream_t stream = nullptr;
    std::string err;
    long long launches = 0;

    // plain FP64 state
    double* f[2] = {nullptr, nullptr};
    int cur = 0;
    double* fd = nullptr;
    double* dn = nullptr;
    double* fny = nullptr;
    double* fdny = nullptr;
    double* lap = nullptr;      // lapl(f) of the current step (leapfrog), allocated on first use
    // SIGW state
    float* h[2][6] = {};
    float* hd[6] = {};
    float* hny[6] = {};
    float* hdny[6] = {};
    // RK4 scratch, allocated on the first RK4 step: stage f, fd, k_fd
    // (doubles) and stage h, hd, k_hd (floats, SIGW)
    double* rk_d = nullptr;
    float* rk_h = nullptr;
    int rk_nst = 0;   // stages the scratch is laid out for
    double* dn_y5 = nullptr;   // deltaN RK45 candidate (f, fd, deltaN), allocated on first use

    // table (device copies, plus the host copy for scalar evaluations)
    std::vector<double> htab_x, htab_V, htab_dV;
    int ntab = 0;
    double* tab = nullptr;      // packed arrays, see iegpu_set_table
    long long* tkey = nullptr;
    iegpu::DivConst* tdiv = nullptr;   // per-bracket divisors of the interpolation
    iegpu::PotDev pot{};

    // control and scratch
    iegpu::DevCtl* ctl = nullptr;      // device
    iegpu::DevCtl* ctl_h = nullptr;    // pinned host mirror
    double* part = nullptr;            // per-CTA reduction partials
    unsigned* counter = nullptr;       // last-CTA detection
    int red_grid = 0;
    double* a_trace = nullptr;
    int a_trace_cap = 0;
    double* spec_part = nullptr;       // spectrum partials [blocks][nbins]
    // GW spectra in the reference's float accumulation order (built on first use)
    int* gw_pos = nullptr;             // per mode slot: its place in the bin-major list, or -1
    int* gw_start = nullptr;           // [nbins + 1] list offsets per bin
    float* gw_vals = nullptr;          // per-mode values, bin-major, loop order within a bin
    float* gw_f2f = nullptr;           // [nbins] float sums
    double* gw_f2d = nullptr;          // [nbins] double sums
    std::vector<int> gw_counts;        // the reference's numpoints per bin
    int* spec_cnt = nullptr;
    int spec_blocks = 0;
    double* misc = nullptr;            // small device scratch (sums, min/max)
    double* misc_h = nullptr;          // pinned mirror
    iegpu::FftTw tw{};

    // split form state
    float* sp[2] = {nullptr, nullptr};    // dphi (ping-pong)
    float* spi[2] = {nullptr, nullptr};   // dpi  (ping-pong)
    // compensated split form: Kahan residuals of dphi and dpi (bf16 bits,
    // ping-pong with sp / spi; the value is x - residual)
    unsigned short* sxl[2] = {nullptr, nullptr};
    unsigned short* spl[2] = {nullptr, nullptr};
    int comp = 0;
    iegpu::SplitCtl* sctl = nullptr;      // device
    iegpu::SplitCtl* sctl_h = nullptr;    // pinned host mirror
    cudaGraphExec_t sp_exec[2] = {nullptr, nullptr};
    int sp_steps = 0;
    int split_mat = 0;                    // FP64 buffers hold the field (deltaN stage)
    iegpu::RowCfg row_cfg;                // split row-kernel launch shape
    int tuned = 0;
    int tuning = 0;                       // the autotuner is timing shapes: no tensor kernel
    int part_cap = 0;
    unsigned wait_polls = 0;              // bounded device waits: poll limit (0: default)
    unsigned wait_bias = 0;               // test hook: persistent barrier target never reached

    // timing events
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

    // leapfrog graphs: [parity of the current buffer]
    cudaGraphExec_t lf_exec[2] = {nullptr, nullptr};
    int lf_steps = 0;
};

namespace iegpu {

int set_error(iegpu_ctx* c, int code, const char* fmt, ...);
// Opts kernel `fn` in to `bytes` of dynamic shared memory on the current
// device.  The opt-in is a per-device function attribute: it is made once per
// (kernel, device, size) under a mutex, and its status is returned.
cudaError_t smem_optin(const void* fn, size_t bytes);
int check_cuda(iegpu_ctx* c, cudaError_t e, const char* what);
int sync_and_check(iegpu_ctx* c, const char* what);
bool is_double_field(int field);
double* dfield(iegpu_ctx* c, int field);
float* ffield(iegpu_ctx* c, int field);
double* dnyq(iegpu_ctx* c, int field);
float* fnyq(iegpu_ctx* c, int field);
int valid_field(iegpu_ctx* c, int field);
// potential(v) of src/potential.cpp:91-98 evaluated on the host.
double host_potential(const iegpu_ctx* c, double v);

// pow(x, y) for the exponents the leapfrog uses with rescale_s = 0; exact
// products and quotients there, CUDA pow otherwise.
__host__ __device__ inline double pow_exp(double x, double y) {
    if (y == 0.0) return 1.0;
    if (y == 1.0) return x;
    if (y == 2.0) return x * x;
    if (y == -1.0) return 1.0 / x;
    return pow(x, y);
}

// saveN's float accumulator, src/output.cpp:1527-1537: over the sites with
// x <= cutoff, in site order, Nmean += x with a float Nmean and a double x
// (the sum formed in double, then rounded to float), and Nmean / gridsize in
// float.  The recurrence is serial by definition.  On GB300 each step of a
// device replay is a chain of dependent FP64 operations (about 150 ns a
// site); the host runs it at a few ns a site, so the map is copied down and
// replayed here.
inline float float_mean_serial(const double* x, long long n, double cutoff) {
    float m = 0.f;
    for (long long i = 0; i < n; ++i)
        if (x[i] <= cutoff) m = (float)((double)m + x[i]);
    return m / (float)n;
}

// --- launchers implemented in the .cu files ---------------------------------
// leapfrog_fp64.cu
int fp64_leapfrog(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace);
int fp64_evolve_derivs(iegpu_ctx* c, double d, iegpu_bg* bg);
int fp64_evolve_fields(iegpu_ctx* c, double d, iegpu_bg* bg);
int fp64_post_init(iegpu_ctx* c, double horizon_factor, double omega, int from_deltaN, iegpu_bg* bg);
int fp64_rk4_step(iegpu_ctx* c, double h, iegpu_bg* bg);
int fp64_rk4(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace);
int fp64_rk45_step(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double h, double hmax, double* h_next, int* accepted,
                   iegpu_bg* bg);
int fp64_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af, int max_steps, double* h, iegpu_bg* bg,
              int* steps, double* a_trace);
// RK45 controls and step clamps shared by the lattice and deltaN integrators
iegpu_rk45_controls rk45_sanitized(const iegpu_ctx* c, const iegpu_rk45_controls* in);
iegpu_rk45_controls rk45_sanitized_dt(const iegpu_rk45_controls* in, double dt);
double rk45_clamp(const iegpu_rk45_controls& K, double h, double hmax);
double rk45_hmax(const iegpu_rk45_controls& K, double base_step);
int deltaN_rk4(iegpu_ctx* c, double h, int nsteps, double phiref, iegpu_bg* bg);
int deltaN_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double dN, double Nend, int max_steps, double phiref,
                double* h, double* Ne, iegpu_bg* bg, int* steps, double* Ne_trace);
int fp64_post_rk4(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps, iegpu_bg* bg, int* steps,
                  double* a_trace);
int fp64_post_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af_post, double dt_post, double omega,
                   int max_steps, double* h, iegpu_bg* bg, int* steps, double* a_trace);
int fp64_post_derivs(iegpu_ctx* c, double d, double omega, iegpu_bg* bg);
int fp64_post_leapfrog(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps, iegpu_bg* bg,
                       int* steps, double* a_trace);
int fp64_energies(iegpu_ctx* c, const iegpu_bg* bg, double out[3]);
int fp64_profile(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms, int nk);
void fp64_destroy_graphs(iegpu_ctx* c);
// fft.cu
int fft_init(iegpu_ctx* c);
void fft_free(iegpu_ctx* c);
int fft_d(iegpu_ctx* c, double* f, double* fny, int forward);
int fft_f(iegpu_ctx* c, float* f, float* fny, int forward);
// spectra.cu
int spectrum_bin_d(iegpu_ctx* c, const double* f, const double* fny, int* counts, double* f2, int nbins);
int gw_bin(iegpu_ctx* c, int which, double to_phys, int* counts, double* f2, int nbins);
// the same binning with the reference's float accumulators (and the same values summed in double)
int gw_bin_ref(iegpu_ctx* c, int which, double to_phys, int* counts, float* f2, double* f2d, int nbins);
// zeroes f's and fd's modes outside [low, high] (both in k-space), spectraf()'s forcing cutoff
int forcing_cutoff(iegpu_ctx* c, double* f, double* fny, double* fd, double* fdny, double high, double low);
// reduce.cu
int field_means(iegpu_ctx* c, double out[3]);
int field_sum(iegpu_ctx* c, int field, double* out);
int field_histogram(iegpu_ctx* c, int field, int nbins, double* bmin, double* df, double* freq);
int field_add(iegpu_ctx* c, int field, double v);
int field_zero_above(iegpu_ctx* c, int field, double thr);
int saveN_mean(iegpu_ctx* c, double cutoff, float* out);
int get_phiref(iegpu_ctx* c, double* out);
// split_fp32.cu
int split_leapfrog(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace);
int split_evolve_derivs(iegpu_ctx* c, double d, iegpu_bg* bg);
int split_profile(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms, int nk);
int split_autotune(iegpu_ctx* c, const iegpu_bg* bg);
int split_set_shape(iegpu_ctx* c, int rows, int prefetch, int chunks);
int split_evolve_fields(iegpu_ctx* c, double d, iegpu_bg* bg);
int split_sums(iegpu_ctx* c, double out[6]);
int split_materialize(iegpu_ctx* c, int which, double* out);
int split_to_double(iegpu_ctx* c, int which, double* out);
int split_absorb(iegpu_ctx* c, int which, const double* in, double mean);
void split_destroy_graphs(iegpu_ctx* c);
// ic.cu
int bunch_davies(iegpu_ctx* c, int seed, double phi0, double dphi0, double hubble, double hi_cut, double lo_cut);
// deltaN.cu
int deltaN_init(iegpu_ctx* c, double a);
int deltaN_steps(iegpu_ctx* c, double dN, int nsteps, double phiref, int do_derivs, int do_fields);

}  // namespace iegpu
