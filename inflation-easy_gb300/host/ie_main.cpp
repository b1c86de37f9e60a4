// ie_main.cpp -- host program of the GB300 InflationEasy engine.
//
// The reference's driver (src/main.cpp:103-146), leapfrog loops
// (src/evolution.cpp:909-997, 1291-1375, 1561-1653), the RK4 and RK45
// branches of the inflation, deltaN and post-inflation loops, initial conditions
// (src/initialize.cpp) and output routines (src/output.cpp), with every
// lattice operation sent through the C ABI of include/iegpu.h.  It reads
// params.txt from the working directory and writes results/ in the
// reference's file formats.  Background scalars (t, a, ad, ad2, astep, Ne)
// are advanced here with the reference's own expressions, except inside
// iegpu_leapfrog, where the device advances them between host visits.
//
// Usage: ie_gpu_main [params.txt] [results_dir] [dump_dir]
//        ie_gpu_main --check-params [params.txt]   (resolved parameters; no device)
// dump_dir (optional) receives trace.txt (background scalars at each save),
// precise.txt (printed means and spectra at full precision) and state.bin.
#include <sys/stat.h>

#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "ie_params.h"
#include "iegpu.h"

namespace {

IeParams P;
iegpu_ctx* G = nullptr;
iegpu_bg bg = {0.0, 1.0, 0.0, 0.0, 1.0};  // t, a, ad, ad2, astep (src/main.cpp:31-32)
double t0 = 0.0, Ne = 0.0, phiref = 0.0, hubble_init = 0.0;
FILE* output_ = nullptr;
std::string RES = "results";
const double pi = 2.0 * std::asin(1.0);
std::vector<double> tab_x, tab_V, tab_dV;
// optional full-precision diagnostics (third command-line argument)
FILE* g_trace = nullptr;
FILE* g_prec = nullptr;

void prec_line(const char* tag, const double* v, int n) {
    if (!g_prec) return;
    std::fprintf(g_prec, "%s", tag);
    for (int i = 0; i < n; ++i) std::fprintf(g_prec, " %.17g", v[i]);
    std::fprintf(g_prec, "\n");
}

inline double pw2(double x) { return x * x; }
inline size_t idx(int i, int j, int k) { return ((size_t)i * P.N + (size_t)j) * P.N + (size_t)k; }

[[noreturn]] void fatal(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(stderr, fmt, ap);
    va_end(ap);
    std::exit(1);
}

// Status of an engine call: the engine's message is the reference's message.
void ck(int rc) {
    if (rc == IEGPU_OK) return;
    const char* m = G ? iegpu_last_error(G) : iegpu_strerror(rc);
    std::fprintf(stderr, "%s", m);
    if (m[0] && m[std::strlen(m) - 1] != '\n') std::fprintf(stderr, "\n");
    std::exit(1);
}

FILE* open_or_die(const std::string& name, const char* mode = "w") {
    const std::string path = RES + "/" + name + ".dat";
    FILE* fp = std::fopen(path.c_str(), mode);
    if (!fp) fatal("Failed to open output file: %s\n", path.c_str());
    return fp;
}

// The output files of the inflation phase (post = 0) or of the post-inflation
// phase (post = 1, results/post_inflation/, src/output.cpp:1573-1867), opened
// on first use and kept open, as the reference's static FILE pointers.
FILE* out_file(const char* name, int post) {
    static std::vector<std::pair<std::string, FILE*>> files;
    const std::string key = std::string(post ? "post_inflation/" : "") + name;
    for (auto& e : files)
        if (e.first == key) return e.second;
    FILE* fp = open_or_die(key);
    files.emplace_back(key, fp);
    return fp;
}

// ---- potential on the host (src/potential.cpp:11-98) -----------------------

int find_bracket(double v) {
    const int n = (int)tab_x.size();
    if (n < 2) fatal("Numerical potential table must contain at least two points.\n");
    if (v > tab_x.front() || v < tab_x.back())
        fatal("Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v, tab_x.back(), tab_x.front());
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (tab_x[mid] >= v) lo = mid; else hi = mid;
    }
    return hi;
}

double potential(double v) {
    if (P.numerical_potential) {
        const int l = find_bracket(v);
        const double x0 = tab_x[l - 1], x1 = tab_x[l], y0 = tab_V[l - 1], y1 = tab_V[l];
        if (x0 == x1) fatal("Interpolation failed due to repeated field grid points.\n");
        return (y1 + (v - x1) * (y0 - y1) / (x0 - x1)) / pw2(P.rescale_B);
    }
    return P.V0 * (1.0 - (1.0 - P.ns) / 4.0 * pw2(v)) / pw2(P.rescale_B);
}

void load_vector(const std::string& filename, std::vector<double>& vec) {
    std::ifstream in(filename);
    if (!in) fatal("Could not open file: %s\n", filename.c_str());
    double v;
    while (in >> v) vec.push_back(v);
    if (vec.empty()) fatal("File appears to be empty or malformed: %s\n", filename.c_str());
}

// ---- scalar evolution pieces ------------------------------------------------

double rescaled_step(double astep) { return P.dt * std::pow(astep, P.rescale_s - 1.0); }

iegpu_rk45_controls rk45_controls() {
    return {P.rk45_abs_tol, P.rk45_rel_tol, P.rk45_min_dt, P.rk45_max_dt, P.rk45_safety};
}

void evolve_fields(double d) { ck(iegpu_evolve_fields(G, d, &bg)); }

// evolve_fieldsN(d), src/evolution.cpp:1015-1037: lattice part on the device,
// t and a here.
void evolve_fieldsN(double d) {
    bg.t += d;
    ck(iegpu_evolve_fieldsN(G, d, phiref));
    bg.a += d * bg.ad;
}

// ---- initial conditions (src/initialize.cpp) --------------------------------

int rng_next = 0, rng_started = 0;

double rand_uniform() {
    if (P.seed < 1) return 0.33;
    if (!rng_started) rng_next = P.seed;
    if (!(rng_next > 0)) {
        std::printf("Invalid seed used in random number function. Using seed=1\n");
        rng_next = 1;
    }
    auto advance = [] {
        rng_next = 16807 * (rng_next % 127773) - 2836 * (rng_next / 127773);
        if (rng_next < 0) rng_next += 2147483647;
    };
    if (!rng_started) {
        rng_started = 1;
        for (int w = 1; w < 100; ++w) advance();
    }
    advance();
    return (double)rng_next / (double)2147483647;
}

bool sm_started = false;
double sm_norm = 0.0, sm_hbterm = 0.0;

void set_mode(double p2, double p2lat, double m2, double* field, double* deriv, int real) {
    if (!sm_started) {
        sm_norm = P.rescale_B * std::pow(P.L / pw2(P.dx), 1.5);
        sm_hbterm = -hubble_init;
        sm_started = true;
    }
    static int tachyonic = 0;
    const double ii = P.L / (2.0 * pi) * std::sqrt(p2lat);
    const double omega = (p2 + m2 > 0.0) ? std::sqrt(p2 + m2) : std::sqrt(p2);
    if (p2 + m2 <= 0.0 && tachyonic == 0) {
        std::printf("Warning: Tachyonic mode(s) may be initialized inaccurately\n");
        tachyonic = 1;
    }
    double rms = (omega > 0.0) ? sm_norm / std::sqrt(2.0 * omega) : 0.0;
    if (P.high_cutoff_index > 0 && (ii > P.high_cutoff_index || ii < P.low_cutoff_index)) rms = 0.0;
    const double amplitude = rms * std::sqrt(std::log(1.0 / rand_uniform()));
    const double phase = 2.0 * pi * rand_uniform();
    const double re = amplitude * std::cos(phase), im = amplitude * std::sin(phase);
    field[0] = re;
    field[1] = im;
    deriv[0] = omega * im + sm_hbterm * field[0];
    deriv[1] = -omega * re + sm_hbterm * field[1];
    if (real == 1) { field[1] = 0.0; deriv[1] = 0.0; }
}

// initialize() + initializef(), src/initialize.cpp:93-214: the Bunch-Davies
// modes are drawn on the host in the reference's order, the inverse r2c FFT
// and the background add run on the device.  Selected by ic_on_host = 1; the
// default draws the modes on the device (iegpu_bunch_davies).
void initialize_fields_host() {
    if (P.dt > P.dx / std::sqrt(3.0)) {
        std::printf("Time step too large. Courant condition violated: dt/dx = %f\n", P.dt / P.dx);
        std::exit(1);
    }
    std::printf("Generating initial conditions for new run at t = 0\n");
    t0 = 0.0;
    hubble_init = std::sqrt(potential(P.initial_field) / 3.0);
    bg.ad = hubble_init;
    const int N = P.N;
    const size_t gs = (size_t)N * N * N;
    std::vector<double> f(gs, 0.0), fd(gs, 0.0), fny((size_t)N * 2 * N, 0.0), fdny((size_t)N * 2 * N, 0.0);
    hubble_init = std::sqrt((0.5 * pw2(P.initial_derivative) + potential(P.initial_field)) / 3.0);
    bg.ad = hubble_init;
    const double dp2 = pw2(2.0 * pi / P.L);
    const double m2 = 0.0;
    auto ny = [&](std::vector<double>& a, int i, int j) { return &a[(size_t)i * 2 * N + 2 * j]; };
    for (int i = 0; i < N; i++) {
        const double px = (i <= N / 2 ? i : i - N);
        const int iconj = (i == 0 ? 0 : N - i);
        for (int j = 0; j < N; j++) {
            const double py = (j <= N / 2 ? j : j - N);
            for (int k = 1; k < N / 2; k++) {
                const double pz = k;
                const double p2lat = dp2 * (pw2(px) + pw2(py) + pw2(pz));
                const double p2 = 4.0 * pw2(N / P.L) * (pw2(std::sin(px * pi / N)) + pw2(std::sin(py * pi / N)) + pw2(std::sin(pz * pi / N)));
                set_mode(p2, p2lat, m2, &f[idx(i, j, 2 * k)], &fd[idx(i, j, 2 * k)], 0);
            }
            if (j > N / 2 || (i > N / 2 && (j == 0 || j == N / 2))) {
                const int jconj = (j == 0 ? 0 : N - j);
                double p2lat = dp2 * (pw2(px) + pw2(py));
                double p2 = 4.0 * pw2(N / P.L) * (pw2(std::sin(px * pi / N)) + pw2(std::sin(py * pi / N)));
                set_mode(p2, p2lat, m2, &f[idx(i, j, 0)], &fd[idx(i, j, 0)], 0);
                f[idx(iconj, jconj, 0)] = f[idx(i, j, 0)];
                f[idx(iconj, jconj, 1)] = -f[idx(i, j, 1)];
                fd[idx(iconj, jconj, 0)] = fd[idx(i, j, 0)];
                fd[idx(iconj, jconj, 1)] = -fd[idx(i, j, 1)];
                p2lat = dp2 * (pw2(px) + pw2(py) + pw2(N / 2));
                p2 = 4.0 * pw2(N / P.L) * (pw2(std::sin(px * pi / N)) + pw2(std::sin(py * pi / N)) + 1.0);
                set_mode(p2, p2lat, m2, ny(fny, i, j), ny(fdny, i, j), 0);
                ny(fny, iconj, jconj)[0] = ny(fny, i, j)[0];
                ny(fny, iconj, jconj)[1] = -ny(fny, i, j)[1];
                ny(fdny, iconj, jconj)[0] = ny(fdny, i, j)[0];
                ny(fdny, iconj, jconj)[1] = -ny(fdny, i, j)[1];
            } else if ((i == 0 || i == N / 2) && (j == 0 || j == N / 2)) {
                double p2lat = dp2 * (pw2(px) + pw2(py));
                double p2 = 4.0 * pw2(N / P.L) * (pw2(std::sin(px * pi / N)) + pw2(std::sin(py * pi / N)));
                if (p2 > 0.0) set_mode(p2, p2lat, m2, &f[idx(i, j, 0)], &fd[idx(i, j, 0)], 1);
                p2lat = dp2 * (pw2(px) + pw2(py) + pw2(N / 2));
                p2 = 4.0 * pw2(N / P.L) * (pw2(std::sin(px * pi / N)) + pw2(std::sin(py * pi / N)) + 1.0);
                set_mode(p2, p2lat, m2, ny(fny, i, j), ny(fdny, i, j), 1);
            }
        }
    }
    f[0] = f[1] = fd[0] = fd[1] = 0.0;
    ck(iegpu_upload(G, IEGPU_F, f.data(), fny.data()));
    ck(iegpu_upload(G, IEGPU_FD, fd.data(), fdny.data()));
    ck(iegpu_fft(G, IEGPU_F, -1));
    ck(iegpu_fft(G, IEGPU_FD, -1));
    ck(iegpu_add(G, IEGPU_F, P.initial_field));
    ck(iegpu_add(G, IEGPU_FD, P.initial_derivative));
    double e[3];
    iegpu_bg b1 = bg;
    b1.a = 1.0;
    ck(iegpu_energies(G, &b1, e));
    hubble_init = std::sqrt((e[0] + e[2] + e[1]) / 3.0);
    bg.ad = hubble_init;
    std::printf("Finished initial conditions\n");
}

void initialize_fields() {
    if (P.ic_on_host && P.form != 0)
        std::fprintf(stderr, "ic_on_host applies to the FP64 form; the split forms draw their modes on the device.\n");
    if (P.ic_on_host && P.form == 0) {
        initialize_fields_host();
        return;
    }
    std::printf("Generating initial conditions for new run at t = 0\n");
    t0 = 0.0;
    (void)potential(P.initial_field);  // the reference's range check, src/initialize.cpp:101
    ck(iegpu_bunch_davies(G, P.seed, P.initial_field, P.initial_derivative, P.high_cutoff_index, P.low_cutoff_index,
                          &hubble_init));
    bg.ad = hubble_init;
    std::printf("Finished initial conditions\n");
}

// ---- output (src/output.cpp) ------------------------------------------------

void print_spectrum(FILE* out, const std::vector<int>& counts, std::vector<double>& f2, double norm1, const char* tag) {
    const double dp = 2.0 * pi / P.L;
    std::vector<double> pv(counts.size());
    for (size_t i = 0; i < counts.size(); i++) {
        if (counts[i] > 0) f2[i] /= (double)counts[i];
        std::fprintf(out, "%e %d %e\n", dp * (double)i, counts[i], norm1 * f2[i]);
        pv[i] = norm1 * f2[i];
    }
    prec_line(tag, pv.data(), (int)pv.size());
    std::fprintf(out, "\n");
    std::fflush(out);
}

// meansvars(), src/output.cpp:204-269; post: meansvars_post_inflation, :1576-1639
void meansvars(int post = 0) {
    FILE* m = out_file("means", post);
    FILE* v = out_file("variance", post);
    FILE* ve = out_file("velocity", post);
    std::fprintf(m, "%f", bg.t); std::fprintf(m, " %e", bg.a);
    std::fprintf(ve, "%f", bg.t); std::fprintf(ve, " %e", bg.a);
    std::fprintf(v, "%f", bg.t); std::fprintf(v, " %e", bg.a);
    double s[3];
    ck(iegpu_means(G, s));
    const double gs = (double)P.N * P.N * P.N;
    const double av = s[0] / gs;
    double vel = s[1] / gs;
    vel = vel * std::pow(bg.a, P.rescale_s - 1.0) * P.rescale_B;
    std::fprintf(m, " %e", av);
    std::fprintf(ve, " %e", vel);
    std::fprintf(v, " %e", s[2] - pw2(av));
    {
        const double q[5] = {bg.t, bg.a, av, vel, bg.ad * P.rescale_B * std::pow(bg.a, P.rescale_s - 2.0)};
        prec_line(post ? "post_means" : "means", q, 5);
    }
    if (av + DBL_MAX == av || (av != 0. && av / av != 1.)) {
        std::printf("Unstable solution developed. Scalar field not numerical at t=%f\n", bg.t);
        std::fflush(m); std::fflush(v);
        std::exit(1);
    }
    std::fprintf(m, "\n"); std::fprintf(v, "\n"); std::fprintf(ve, "\n");
    std::fflush(m); std::fflush(v); std::fflush(ve);
}

// scale(), src/output.cpp:272-293; post: scale_post_inflation, :1642-1662
void scale(int post = 0) {
    FILE* sf = out_file("sf", post);
    const double B = P.rescale_B, s = P.rescale_s, a = bg.a;
    std::fprintf(sf, "%f %f %e %e\n", bg.t, a, bg.ad * B * std::pow(a, s - 2.0),
                 pw2(B) * std::pow(a, 2.0 * s - 2.0) * (bg.ad2 + (s - 1.0) * pw2(bg.ad) / a));
    std::fflush(sf);
}

void energy() {
    static FILE *e = nullptr, *c = nullptr;
    if (!e) { e = open_or_die("energy"); c = open_or_die("conservation"); }
    double en[3];
    ck(iegpu_energies(G, &bg, en));
    const double B = P.rescale_B;
    double totalE = 0.0;
    std::fprintf(e, "%f", bg.t); std::fprintf(e, " %e", bg.a);
    totalE += en[0]; std::fprintf(e, " %e", en[0] * B);
    totalE += en[1]; std::fprintf(e, " %e", en[1] * B);
    totalE += en[2]; std::fprintf(e, " %e", en[2] * B);
    std::fprintf(e, "\n"); std::fflush(e);
    std::fprintf(c, "%e %e %e\n", bg.t, bg.a, 3.0 * std::pow(bg.a, 2.0 * P.rescale_s - 4.0) * pw2(bg.ad) / totalE);
    std::fflush(c);
}

// spectraf(), src/output.cpp:297-406; post: spectraf_post_inflation, :1667-1770
void spectraf(int post = 0) {
    FILE* sp = out_file("spectra", post);
    FILE* st = out_file("spectratimes", post);
    const int nb = iegpu_numbins(P.N);
    std::vector<int> counts(nb);
    std::vector<double> f2(nb);
    const double norm1 = std::pow(P.L / P.rescale_B, 3) / std::pow((double)P.N, 6);
    // with forcing_cutoff, f's and fd's modes outside [low, high] are zeroed
    // after the binning (src/output.cpp:330-401)
    if (P.forcing_cutoff && P.high_cutoff_index > 0)
        ck(iegpu_spectrum_cutoff(G, counts.data(), f2.data(), nb, P.high_cutoff_index, P.low_cutoff_index));
    else
        ck(iegpu_spectrum(G, IEGPU_F, counts.data(), f2.data(), nb));
    print_spectrum(sp, counts, f2, norm1, post ? "post_spectrum" : "spectrum");
    std::fprintf(st, "%f %e\n", bg.t, bg.a);
    std::fflush(st);
}

// spectraGW / spectraGWdot, src/output.cpp:618-648: the per-bin sums come
// back as the reference's own float accumulators (its loop order, bit for bit
// given the same h); division and normalisation are the reference's float
// ones.
// Post (src/output.cpp:652-669): spectraGWdot_post_inflation multiplies h' in
// float by (float)(B a^(s-1)); rounding (double)h' * (double)(float)(B a^(s-1))
// to float gives the same bits, the double product of two floats being exact.
void spectra_gw(int which, int post = 0) {
    FILE* fp = out_file(which ? "spectraGWdot" : "spectraGW", post);
    const int nb = iegpu_numbins(P.N);
    std::vector<int> counts(nb);
    std::vector<float> f2f(nb);   // the reference's float accumulators, its loop order
    std::vector<double> f2(nb);   // the same values summed in double (full-precision dump)
    double to_phys = which ? P.rescale_B * std::pow(bg.a, P.rescale_s - 1.0) : 1.0;
    if (post && which) to_phys = (double)(float)to_phys;
    ck(iegpu_gw_spectrum_ref(G, which, to_phys, counts.data(), f2f.data(), f2.data(), nb));
    const int numbins = (int)(std::sqrt(3.0) * (P.N / 2)) + 1;
    if (g_prec) {
        const double n1 = 0.5 * std::pow(P.L / P.rescale_B, 3) / std::pow((double)P.N, 6);
        std::vector<double> pv((size_t)numbins);
        for (int i = 0; i < numbins; ++i) pv[(size_t)i] = counts[i] > 0 ? n1 * f2[i] / counts[i] : 0.0;
        prec_line(which ? (post ? "post_spectrumGWdot" : "spectrumGWdot") : (post ? "post_spectrumGW" : "spectrumGW"),
                  pv.data(), numbins);
    }
    const float dp = 2.f * (float)pi / (float)P.L;
    const float norm1 = 0.5f * std::pow(P.L / P.rescale_B, 3) / std::pow((float)P.N, 6);
    for (int i = 0; i < numbins; ++i) {
        float v = f2f[i];
        if (counts[i] > 0) v /= (float)counts[i];
        std::fprintf(fp, "%e %d %e\n", dp * i, counts[i], norm1 * v);
    }
    std::fprintf(fp, "\n");
    std::fflush(fp);
}

void histogram_out(int field, FILE* hist, FILE* times, bool deltaN_style) {
    if (deltaN_style) std::fprintf(times, "%f %e", bg.t, bg.a);
    else { std::fprintf(times, "%f", bg.t); std::fprintf(times, " %e", bg.a); }
    double bmin, df;
    std::vector<double> freq(P.nbins);
    ck(iegpu_histogram(G, field, P.nbins, &bmin, &df, freq.data()));
    for (int i = 0; i < P.nbins; i++) std::fprintf(hist, "%e\n", freq[i]);
    std::fprintf(hist, "\n");
    std::fflush(hist);
    if (deltaN_style) std::fprintf(times, " %e %e\n", bmin, df);
    else { std::fprintf(times, " %e %e", bmin, df); std::fprintf(times, "\n"); }
    std::fflush(times);
}

void box2d(FILE* fp, int field, double scale, bool scaled) {
    const int N = P.N;
    const int i = (N < 64) ? 5 : 50;
    std::vector<double> x((size_t)N * N * N);
    ck(iegpu_download(G, field, x.data(), nullptr));
    for (int j = 0; j < N; j++)
        for (int k = 0; k < N; k++) {
            if (scaled) std::fprintf(fp, "%.17g\n", x[idx(i, j, k)] * scale);
            else std::fprintf(fp, "%.17g\n", x[idx(i, j, k)]);
        }
    std::fprintf(fp, "\n");
    std::fflush(fp);
}

// save(), src/output.cpp:1469-1503
void save(int infrequent) {
    if (g_trace)
        std::fprintf(g_trace, "save %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, bg.t, bg.a, bg.ad, bg.ad2, bg.astep);
    // the staggered (leapfrog) state is synchronised around the outputs
    // (src/output.cpp:1471-1472, 1501-1502); RK4 states need no sync
    const bool sync = P.inflation_integrator == IE_LEAPFROG && bg.t > 0.;
    if (sync) evolve_fields(-.5 * P.dt * std::pow(bg.astep, P.rescale_s - 1));
    meansvars();
    scale();
    if (infrequent) {
        if (P.output_box3D) {
            static FILE* bx = open_or_die("box");
            std::vector<double> x((size_t)P.N * P.N * P.N);
            ck(iegpu_download(G, IEGPU_F, x.data(), nullptr));
            for (double v : x) std::fprintf(bx, "%.17g\n", v);
            std::fprintf(bx, "\n");
            std::fflush(bx);
        }
        if (P.output_box2D) {
            static FILE* b1 = open_or_die("snapshots_2d_phi");
            static FILE* b2 = open_or_die("snapshots_2d_phidot");
            box2d(b1, IEGPU_F, 0.0, false);
            box2d(b2, IEGPU_FD, P.rescale_B, true);
        }
        if (P.output_energy) energy();
        if (P.output_spectra) {
            spectraf();
            if (P.calculate_SIGW) { spectra_gw(0); spectra_gw(1); }
        }
        if (P.output_histogram) {
            static FILE* h = open_or_die("histogram");
            static FILE* ht = open_or_die("histogramtimes");
            histogram_out(IEGPU_F, h, ht, false);
        }
    }
    if (sync) evolve_fields(.5 * P.dt * std::pow(bg.astep, P.rescale_s - 1));
}

// get_modes, src/output.cpp:674-738
void get_modes() {
    FILE* fp = open_or_die("modes");
    const int N = P.N;
    const int numbins = (int)(std::sqrt(3.0) * (N / 2)) + 1;
    std::vector<int> np(numbins + 1, 0);
    std::vector<double> pp(numbins + 1, 0.0);
    for (int i = 0; i < N; i++) {
        const int px = (i <= N / 2 ? i : i - N);
        for (int j = 0; j < N; j++) {
            const int py = (j <= N / 2 ? j : j - N);
            auto add = [&](int pz, int w) {
                const double pm = std::sqrt(pw2((double)px) + pw2((double)py) + pw2((double)pz));
                const double pph = std::sqrt(4.0 * pw2((double)N / (double)P.L) *
                                             (pw2(std::sin((double)px * pi / N)) + pw2(std::sin((double)py * pi / N)) +
                                              pw2(std::sin((double)pz * pi / N))));
                np[(int)pm] += w;
                pp[(int)pm] += w == 2 ? 2.0 * pph : pph;
            };
            for (int k = 1; k < N / 2; k++) add(k, 2);
            for (int k = 0; k <= N / 2; k += N / 2) add(k, 1);
        }
    }
    for (int i = 0; i < numbins; i++) {
        if (np[i] > 0) pp[i] = pp[i] / np[i];
        std::fprintf(fp, "%e\n", P.rescale_B * pp[i]);
    }
    std::fprintf(fp, "\n");
    std::fclose(fp);
}

void output_parameters(bool first) {
    static FILE* info = nullptr;
    static time_t tstart;
    if (first) {
        info = open_or_die("info");
        std::fprintf(info, "--------------------------\nGeneral Program Information\n-----------------------------\n");
        std::fprintf(info, "Grid size=%d^%d\n", P.N, 3);
        std::fprintf(info, "L=%f\nf0=%f\nfd0=%f\n", P.L, P.initial_field, P.initial_derivative);
        std::fprintf(info, "dt=%f, dt/dx=%f\n", P.dt, P.dt / P.dx);
        std::fprintf(info, "inflation_integrator=%s\n", ie_integrator_name(P.inflation_integrator));
        if (P.perform_deltaN) std::fprintf(info, "deltaN_integrator=%s\n", ie_integrator_name(P.deltaN_integrator));
        if (P.post_inflation)
            std::fprintf(info, "post_inflation_integrator=%s\n", ie_integrator_name(P.post_inflation_integrator));
        const bool rk45 = P.inflation_integrator == IE_RK45 ||
                          (P.perform_deltaN && P.deltaN_integrator == IE_RK45) ||
                          (P.post_inflation && P.post_inflation_integrator == IE_RK45);
        if (rk45) {
            // the controls in effect (src/output.cpp:1435-1448)
            const iegpu_rk45_controls raw = rk45_controls();
            iegpu_rk45_controls k;
            iegpu_rk45_effective(&raw, P.dt, &k);
            std::fprintf(info, "rk45_abs_tol=%e\nrk45_rel_tol=%e\nrk45_min_dt=%e\nrk45_max_dt=%e\nrk45_safety=%e\n",
                         k.abs_tol, k.rel_tol, k.min_dt, k.max_dt, k.safety);
        }
        std::fprintf(info, "rescale_s=%f\nrescale_B=%e\n", P.rescale_s, P.rescale_B);
        std::fprintf(info, "engine=iegpu %d (GB300, %s)\n", iegpu_version(), P.form == 2 ? "compensated split FP32" : P.form ? "split FP32" : "plain FP64");
        time(&tstart);
        std::fprintf(info, "\nRun began at %s", ctime(&tstart));
    } else if (info) {
        time_t tf;
        time(&tf);
        std::fprintf(info, "Run ended at %s", ctime(&tf));
        std::fprintf(info, "\nRun from t=%f to t=%f took %d seconds\n", t0, bg.t, (int)(tf - tstart));
    }
    if (info) std::fflush(info);
}

// ---- loops ------------------------------------------------------------------

// run_evolution_loop, leapfrog and RK4 branches (src/evolution.cpp:909-997).
// The device runs the steps between two outputs in one call.  Only the
// leapfrog has the half drifts before and after the loop; RK45 carries its
// proposed step h from one call to the next.
void run_evolution_loop() {
    int numsteps = 0;
    const bool leap = P.inflation_integrator == IE_LEAPFROG;
    if (leap) evolve_fields(0.5 * P.dt);
    const iegpu_rk45_controls ctl = rk45_controls();
    double h45 = rescaled_step(bg.astep);   // clamped by the library, src/evolution.cpp:959
    std::vector<double> trace;
    while (bg.a <= P.af) {
        const int chunk = P.output_freq - numsteps % P.output_freq;
        trace.assign((size_t)chunk, 0.0);
        int taken = 0;
        if (leap) ck(iegpu_leapfrog(G, P.af, chunk, &bg, &taken, trace.data()));
        else if (P.inflation_integrator == IE_RK4) ck(iegpu_rk4(G, P.af, chunk, &bg, &taken, trace.data()));
        else ck(iegpu_rk45(G, &ctl, P.af, chunk, &h45, &bg, &taken, trace.data()));
        for (int s = 0; s < taken; ++s) {
            numsteps++;
            double a_now = trace[(size_t)s];
            const bool last = (s == taken - 1);
            if (last && numsteps % P.output_freq == 0 && bg.a < P.af) {
                save((numsteps % P.output_infrequent_freq == 0) ? 1 : 0);
                a_now = bg.a;
            }
            if (P.screen_updates && numsteps % P.output_freq == 0) {
                std::printf("scale factor a = %f\n", a_now);
                std::printf("numsteps %i\n\n", numsteps);
            }
            std::fprintf(output_, "scale factor a = %f\n", a_now);
            std::fprintf(output_, "numsteps %i\n\n", numsteps);
            if (numsteps % P.output_freq == 0) std::fflush(output_);
        }
        bg.astep = bg.a;
        if (taken == 0) break;
    }
    std::printf("Saving final inflaton data\n");
    std::fflush(output_);
    save(1);
    if (leap) evolve_fields(-0.5 * rescaled_step(bg.astep));
    get_modes();
}

// saveN(), src/output.cpp:1522-1560
void saveN() {
    if (g_trace) std::fprintf(g_trace, "saveN %.17g %.17g %.17g %.17g\n", bg.t, bg.a, Ne, phiref);
    // the sync and the dN below Nend are the leapfrog's
    // (deltaN_uses_staggered_derivatives, src/output.cpp:1523-1527)
    const bool stag = P.deltaN_integrator == IE_LEAPFROG;
    if (stag && bg.t > 0.) evolve_fieldsN(-.5 * P.dN);
    const double cutoff = P.Nend - (stag ? P.dN : 0.0);
    float Nmean = 0.f;
    ck(iegpu_saveN_mean(G, cutoff, &Nmean));
    ck(iegpu_shift(G, IEGPU_DELTAN, (double)Nmean));
    {
        FILE* h = open_or_die("histogramN");
        FILE* ht = open_or_die("histogramtimesN");
        histogram_out(IEGPU_DELTAN, h, ht, true);
        std::fclose(h);
        std::fclose(ht);
    }
    if (P.output_box2D) {
        FILE* b = open_or_die("snapshots_2d_deltaN");
        box2d(b, IEGPU_DELTAN, 0.0, false);
        std::fclose(b);
    }
    ck(iegpu_zero_above(G, IEGPU_DELTAN, cutoff - Nmean));
    if (P.output_spectra) {
        FILE* sp = open_or_die("spectraN");
        double sum = 0.0;
        ck(iegpu_sum(G, IEGPU_DELTAN, &sum));
        const double mean = sum / ((double)P.N * P.N * P.N);
        ck(iegpu_shift(G, IEGPU_DELTAN, mean));
        const int nb = iegpu_numbins(P.N);
        std::vector<int> counts(nb);
        std::vector<double> f2(nb);
        const double norm1 = std::pow(P.L / P.rescale_B, 3) / std::pow((double)P.N, 6);
        ck(iegpu_spectrum(G, IEGPU_DELTAN, counts.data(), f2.data(), nb));
        print_spectrum(sp, counts, f2, norm1, "spectrumN");
        std::fclose(sp);
    }
    if (stag && bg.t > 0.) evolve_fieldsN(.5 * P.dN);
}

// run_deltaN_loop, leapfrog, RK4 and RK45 branches (src/evolution.cpp:1291-1375).
// All sites are integrated on the device in one call per output interval.
// The leapfrog's scalar recurrences (t, a, Ne) are replayed here; the RK
// calls advance t and a themselves, and RK45 also advances Ne.
void run_deltaN_loop() {
    std::printf("Starting deltaN calculation\n");
    std::fprintf(output_, "Starting deltaN calculation\n");
    int numsteps = 0;
    Ne = 0.0;
    ck(iegpu_initializeN(G, bg.a));
    const int integ = P.deltaN_integrator;
    if (integ == IE_LEAPFROG) evolve_fieldsN(0.5 * P.dN);
    if (P.use_phiref_manual) phiref = P.phiref_manual_value;
    else ck(iegpu_get_phiref(G, &phiref));
    if (P.criterion == 0) (void)potential(phiref);  // range check, src/evolution.cpp:1305
    if (integ == IE_RK45) {
        // src/evolution.cpp:1334-1367: Ne advances by the step proposed for
        // the next iteration; the library returns Ne after every step
        const iegpu_rk45_controls ctl = rk45_controls();
        double h45 = P.dN;
        std::vector<double> ne_trace;
        while (Ne <= P.Nend) {
            const int limit = P.output_freq - numsteps % P.output_freq;
            ne_trace.assign((size_t)limit, 0.0);
            int taken = 0;
            ck(iegpu_deltaN_rk45(G, &ctl, P.dN, P.Nend, limit, phiref, &h45, &Ne, &bg, &taken, ne_trace.data()));
            for (int s = 0; s < taken; ++s) {
                numsteps++;
                if (P.screen_updates && numsteps % P.output_freq == 0) std::printf("N = %f\n\n", ne_trace[(size_t)s]);
                std::fprintf(output_, "N = %f\n\n", ne_trace[(size_t)s]);
                if (numsteps % P.output_freq == 0) std::fflush(output_);
            }
            if (taken == 0) break;
        }
    }
    while (integ != IE_RK45 && Ne <= P.Nend) {
        // steps until the next flush point, or until Ne passes Nend
        int n = 0;
        double Ne_try = Ne;
        const int limit = P.output_freq - numsteps % P.output_freq;
        while (Ne_try <= P.Nend && n < limit) { Ne_try += P.dN; ++n; }
        if (integ == IE_LEAPFROG) ck(iegpu_deltaN_steps(G, P.dN, n, phiref));
        else ck(iegpu_deltaN_rk4_steps(G, P.dN, n, phiref, &bg));
        for (int s = 0; s < n; ++s) {
            if (integ == IE_LEAPFROG) {
                bg.t += P.dN;
                bg.a += P.dN * bg.ad;
            }
            Ne += P.dN;
            numsteps++;
            if (P.screen_updates && numsteps % P.output_freq == 0) std::printf("N = %f\n\n", Ne);
            std::fprintf(output_, "N = %f\n\n", Ne);
            if (numsteps % P.output_freq == 0) std::fflush(output_);
        }
    }
    saveN();
    std::fflush(output_);
    if (integ == IE_LEAPFROG) evolve_fieldsN(-0.5 * P.dN);
}

// save_post_inflation(), src/output.cpp:1840-1865 (the sync is the
// leapfrog's: post_inflation_uses_staggered_derivatives, src/main.h:193-195)
void save_post(int infrequent) {
    if (g_trace)
        std::fprintf(g_trace, "savep %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, bg.t, bg.a, bg.ad, bg.ad2, bg.astep);
    const bool sync = P.post_inflation_integrator == IE_LEAPFROG && bg.t > 0.;
    if (sync) evolve_fields(-.5 * P.dt_post_inflation);
    meansvars(1);
    scale(1);
    if (infrequent) {
        if (P.output_spectra) {
            spectraf(1);
            spectra_gw(0, 1);
            spectra_gw(1, 1);
        }
        if (P.output_histogram) histogram_out(IEGPU_F, out_file("histogram", 1), out_file("histogramtimes", 1), false);
    }
    if (sync) evolve_fields(.5 * P.dt_post_inflation);
}


// run_post_inflation_loop, leapfrog, RK4 and RK45 branches (src/evolution.cpp:1561-1653),
// with initialize_post_inflation (src/initialize.cpp:245-290).  The device
// runs the steps between two outputs in one call.
void run_post_inflation_loop() {
    const std::string dir = RES + "/post_inflation";
    struct stat st;
    if (stat(dir.c_str(), &st) != 0 && mkdir(dir.c_str(), 0777) != 0)
        fatal("Failed to create '%s' directory.\n", dir.c_str());
    t0 = 0.0;
    ck(iegpu_initialize_post_inflation(G, P.horizon_factor, P.omega, P.perform_deltaN, &bg));
    save_post(1);
    int numsteps = 0;
    const int integ = P.post_inflation_integrator;
    if (integ == IE_LEAPFROG) evolve_fields(0.5 * P.dt_post_inflation);
    const iegpu_rk45_controls ctl = rk45_controls();
    double h45 = P.dt_post_inflation;   // clamped by the library, src/evolution.cpp:1617
    std::vector<double> trace;
    while (bg.a <= P.af_post_inflation) {
        const int chunk = P.output_freq - numsteps % P.output_freq;
        trace.assign((size_t)chunk, 0.0);
        int taken = 0;
        if (integ == IE_LEAPFROG)
            ck(iegpu_post_inflation_leapfrog(G, P.af_post_inflation, P.dt_post_inflation, P.omega, chunk, &bg, &taken,
                                             trace.data()));
        else if (integ == IE_RK4)
            ck(iegpu_post_inflation_rk4(G, P.af_post_inflation, P.dt_post_inflation, P.omega, chunk, &bg, &taken,
                                        trace.data()));
        else
            ck(iegpu_post_inflation_rk45(G, &ctl, P.af_post_inflation, P.dt_post_inflation, P.omega, chunk, &h45, &bg,
                                         &taken, trace.data()));
        for (int s = 0; s < taken; ++s) {
            numsteps++;
            double a_now = trace[(size_t)s];
            if (s == taken - 1 && numsteps % P.output_freq == 0) {
                save_post((numsteps % P.output_infrequent_freq == 0) ? 1 : 0);
                a_now = bg.a;
            }
            if (P.screen_updates && numsteps % P.output_freq == 0) {
                std::printf("scale factor a = %f\n", a_now);
                std::printf("numsteps %i\n\n", numsteps);
            }
            std::fprintf(output_, "scale factor a = %f\n", a_now);
            std::fprintf(output_, "numsteps %i\n\n", numsteps);
            if (numsteps % P.output_freq == 0) std::fflush(output_);
        }
        if (taken == 0) break;
    }
    std::printf("Saving final inflaton data\n");
    std::fflush(output_);
    save_post(1);
}

// Final state in the binary layout of the oracle's state.bin.
void write_state(const std::string& path) {
    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) fatal("Failed to open %s\n", path.c_str());
    const size_t gs = (size_t)P.N * P.N * P.N;
    const int hdr[4] = {P.N, P.perform_deltaN, P.calculate_SIGW, P.numerical_potential};
    const double scal[8] = {bg.t, bg.a, bg.ad, bg.ad2, bg.astep, Ne, phiref, hubble_init};
    std::fwrite(hdr, sizeof(int), 4, fp);
    std::fwrite(scal, sizeof(double), 8, fp);
    std::vector<double> x(gs);
    const int dfields[3] = {IEGPU_F, IEGPU_FD, IEGPU_DELTAN};
    for (int q = 0; q < (P.perform_deltaN ? 3 : 2); ++q) {
        ck(iegpu_download(G, dfields[q], x.data(), nullptr));
        std::fwrite(x.data(), sizeof(double), gs, fp);
    }
    if (P.calculate_SIGW) {
        std::vector<float> h(gs);
        for (int q = 0; q < 12; ++q) {
            ck(iegpu_download(G, q < 6 ? IEGPU_H(q) : IEGPU_HD(q - 6), h.data(), nullptr));
            std::fwrite(h.data(), sizeof(float), gs, fp);
        }
    }
    std::fclose(fp);
}

}  // namespace

// --check-params: the run-time parameters after params.txt, the reference's
// defaults and derived values, and the RK45 controls the library will use,
// one "key value" line each (%.17g).  Touches no device.
int check_params(const char* path) {
    ie_params_load(P, path);
    const iegpu_rk45_controls raw = rk45_controls();
    iegpu_rk45_controls eff;
    if (iegpu_rk45_effective(&raw, P.dt, &eff) != IEGPU_OK) return 1;
    const std::pair<const char*, double> kv[] = {
        {"N", P.N}, {"numerical_potential", P.numerical_potential}, {"perform_deltaN", P.perform_deltaN},
        {"calculate_SIGW", P.calculate_SIGW}, {"criterion", P.criterion}, {"seed", P.seed},
        {"rescale_s", P.rescale_s}, {"af", P.af}, {"V0", P.V0}, {"rescale_B", P.rescale_B}, {"ns", P.ns},
        {"initial_field", P.initial_field}, {"initial_derivative", P.initial_derivative}, {"L", P.L},
        {"dt", P.dt}, {"dx", P.dx}, {"output_freq", P.output_freq},
        {"output_infrequent_freq", P.output_infrequent_freq}, {"dN", P.dN}, {"Nend", P.Nend},
        {"post_inflation", P.post_inflation}, {"horizon_factor", P.horizon_factor}, {"omega", P.omega},
        {"dt_post_inflation", P.dt_post_inflation}, {"af_post_inflation", P.af_post_inflation},
        {"inflation_integrator", P.inflation_integrator}, {"deltaN_integrator", P.deltaN_integrator},
        {"post_inflation_integrator", P.post_inflation_integrator}, {"rk45_abs_tol", eff.abs_tol},
        {"rk45_rel_tol", eff.rel_tol}, {"rk45_min_dt", eff.min_dt}, {"rk45_max_dt", eff.max_dt},
        {"rk45_safety", eff.safety}};
    for (const auto& e : kv) std::printf("%s %.17g\n", e.first, e.second);
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::string(argv[1]) == "--check-params") return check_params(argc > 2 ? argv[2] : "params.txt");
    const char* params_path = argc > 1 ? argv[1] : "params.txt";
    if (argc > 2) RES = argv[2];
    std::string dump_dir = argc > 3 ? argv[3] : "";
    if (!dump_dir.empty()) {
        g_trace = std::fopen((dump_dir + "/trace.txt").c_str(), "w");
        g_prec = std::fopen((dump_dir + "/precise.txt").c_str(), "w");
    }
    ie_params_load(P, params_path);
    if (P.seed < 1)
        std::printf("Warning: The parameter seed has been set to %d, which will result in incorrect output.\n", P.seed);
    if (P.inflation_integrator != IE_LEAPFROG && P.form != 0)
        fatal("the %s inflation integrator runs on the plain FP64 form (form = fp64)\n",
              ie_integrator_name(P.inflation_integrator));
    if (P.forcing_cutoff && P.high_cutoff_index > 0 && P.form != 0)
        fatal("forcing_cutoff runs on the plain FP64 form (form = fp64)\n");
    if (P.post_inflation && !P.calculate_SIGW) fatal("post_inflation requires calculate_SIGW = 1\n");
    if (P.post_inflation && P.form != 0) fatal("the post-inflation phase runs on the plain FP64 form (form = fp64)\n");
    if (P.output_bispectrum || P.output_LOG)
        std::fprintf(stderr, "Ignoring output_bispectrum / output_LOG: not provided by this engine.\n");
    struct stat st;
    if (stat(RES.c_str(), &st) != 0) {
        if (mkdir(RES.c_str(), 0777) != 0) fatal("Failed to create '%s' directory.\n", RES.c_str());
    } else if (!(st.st_mode & S_IFDIR)) {
        fatal("'%s' exists but is not a directory.\n", RES.c_str());
    }
    output_ = std::fopen((RES + "/output.txt").c_str(), "w");
    if (!output_) fatal("Failed to open output file.\n");
    if (P.numerical_potential) {
        load_vector("inputs/field_values.dat", tab_x);
        load_vector("inputs/potential.dat", tab_V);
        load_vector("inputs/potential_derivative.dat", tab_dV);
    }
    iegpu_config cfg{};
    cfg.N = P.N;
    cfg.potential = P.numerical_potential ? IEGPU_POT_TABLE : IEGPU_POT_HILLTOP;
    cfg.sigw = P.calculate_SIGW;
    cfg.form = P.form;
    cfg.criterion = P.criterion;
    cfg.L = P.L;
    cfg.dt = P.dt;
    cfg.rescale_s = P.rescale_s;
    cfg.rescale_B = P.rescale_B;
    cfg.V0 = P.V0;
    cfg.ns = P.ns;
    const int rc = iegpu_create(&cfg, &G);
    if (rc) fatal("iegpu_create failed: %s\n", iegpu_strerror(rc));
    if (P.numerical_potential) ck(iegpu_set_table(G, tab_x.data(), tab_V.data(), tab_dV.data(), (int)tab_x.size()));

    // initialize_simulation(), src/initialize.cpp:40-48
    initialize_fields();
    output_parameters(true);
    save(1);
    bg.t = t0;

    run_evolution_loop();
    if (P.perform_deltaN) run_deltaN_loop();
    if (P.post_inflation) run_post_inflation_loop();

    output_parameters(false);
    if (!dump_dir.empty()) {
        write_state(dump_dir + "/state.bin");
        std::fclose(g_trace);
        std::fclose(g_prec);
    }
    std::fprintf(output_, "InflationEasy program finished\n");
    std::printf("InflationEasy program finished\n");
    std::fclose(output_);
    iegpu_destroy(G);
    return 0;
}
