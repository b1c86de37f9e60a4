// ie_params.cpp -- params.txt parser of the host program.
// Key set, defaults and derived values follow src/runtime_parameters.cpp.
#include "ie_params.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>

void ie_params_defaults(IeParams& p, int N, int numerical) {
    p = IeParams();
    p.N = N;
    p.numerical_potential = numerical;
    p.af = 2.0 * N;
    if (numerical) {
        p.V0 = 3e-9;
        p.initial_field = 2.9181235049318586;
        p.initial_derivative = -0.06727651095116181;
        p.dt = 0.001;
        p.output_freq = p.output_infrequent_freq = 500;
        p.dN = 0.0001;
        p.Nend = 5.0;
    } else {
        p.V0 = 3.338e-13;
        p.initial_field = 0.0935;
        p.initial_derivative = 0.000796;
        p.dt = 0.0005;
        p.output_freq = p.output_infrequent_freq = 200;
        p.dN = 0.0000001;
        p.Nend = 0.001;
    }
    p.rescale_B = std::sqrt(p.V0);
    p.dx = p.L / (double)N;
}

static std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}

static bool to_double(const std::string& v, double& out) {
    if (v.empty()) return false;
    char* end = nullptr;
    errno = 0;
    const double x = std::strtod(v.c_str(), &end);
    if (errno || end == v.c_str() || *end) return false;
    out = x;
    return true;
}

static bool to_int(const std::string& v, int& out) {
    if (v.empty()) return false;
    char* end = nullptr;
    errno = 0;
    const long x = std::strtol(v.c_str(), &end, 10);
    if (errno || end == v.c_str() || *end) return false;
    out = (int)x;
    return true;
}

// parse_integrator, src/runtime_parameters.cpp:141-166: the names (any case)
// leapfrog/lf, rk4, rk45/rkf45/dopri5, or the integer code 0-2.
static bool parse_integrator(const std::string& raw, int& out) {
    std::string s = raw;
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    if (s == "leapfrog" || s == "lf") { out = IE_LEAPFROG; return true; }
    if (s == "rk4") { out = IE_RK4; return true; }
    if (s == "rk45" || s == "rkf45" || s == "dopri5") { out = IE_RK45; return true; }
    int iv = 0;
    if (to_int(s, iv) && iv >= IE_LEAPFROG && iv <= IE_RK45) { out = iv; return true; }
    return false;
}

// integrator_name, src/runtime_parameters.cpp:367-374
const char* ie_integrator_name(int integrator) {
    switch (integrator) {
        case IE_LEAPFROG: return "leapfrog";
        case IE_RK4: return "rk4";
        case IE_RK45: return "rk45";
        default: return "unknown";
    }
}

bool ie_params_load(IeParams& p, const char* path) {
    std::ifstream in(path);
    std::map<std::string, std::string> kv;
    std::map<std::string, int> line_of;
    if (in.good()) {
        std::string line;
        int lineno = 0;
        while (std::getline(in, line)) {
            ++lineno;
            const auto hash = line.find('#');
            if (hash != std::string::npos) line.erase(hash);
            line = trim(line);
            if (line.empty()) continue;
            const auto eq = line.find('=');
            if (eq == std::string::npos) {
                std::fprintf(stderr, "Ignoring malformed line %d in %s: %s\n", lineno, path, line.c_str());
                continue;
            }
            const std::string k = trim(line.substr(0, eq));
            kv[k] = trim(line.substr(eq + 1));
            line_of[k] = lineno;
        }
    }
    // the switches decide the defaults, then every key overrides
    int N = p.N, numerical = p.numerical_potential;
    if (kv.count("N")) to_int(kv["N"], N);
    if (kv.count("numerical_potential")) to_int(kv["numerical_potential"], numerical);
    ie_params_defaults(p, N, numerical != 0);
    bool B_given = false, af_given = false, af_post_given = false;
    for (const auto& [k, v] : kv) {
        double d;
        int i;
        bool ok = true;
        if (k == "N" || k == "numerical_potential") continue;
        else if (k == "perform_deltaN" && to_int(v, i)) p.perform_deltaN = (i != 0);
        else if (k == "calculate_SIGW" && to_int(v, i)) p.calculate_SIGW = (i != 0);
        else if (k == "criterion" && to_int(v, i)) p.criterion = i;
        else if (k == "form") p.form = (v == "split" || v == "1") ? 1 : (v == "split_comp" || v == "2") ? 2 : 0;
        else if (k == "ic_on_host" && to_int(v, i)) p.ic_on_host = (i != 0);
        else if (k == "seed" && to_int(v, i)) p.seed = i;
        else if (k == "rescale_s" && to_double(v, d)) p.rescale_s = d;
        else if (k == "af" && to_double(v, d)) { p.af = d; af_given = true; }
        else if (k == "V0" && to_double(v, d)) p.V0 = d;
        else if (k == "rescale_B" && to_double(v, d)) { p.rescale_B = d; B_given = true; }
        else if (k == "ns" && to_double(v, d)) p.ns = d;
        else if (k == "initial_field" && to_double(v, d)) p.initial_field = d;
        else if (k == "initial_derivative" && to_double(v, d)) p.initial_derivative = d;
        else if (k == "L" && to_double(v, d)) p.L = d;
        else if (k == "dt" && to_double(v, d)) p.dt = d;
        else if (k == "inflation_integrator") {
            if (!parse_integrator(v, p.inflation_integrator))
                std::fprintf(stderr, "Ignoring invalid inflation_integrator '%s' on line %d.\n", v.c_str(), line_of[k]);
        }
        else if (k == "deltaN_integrator") {
            if (!parse_integrator(v, p.deltaN_integrator))
                std::fprintf(stderr, "Ignoring invalid deltaN_integrator '%s' on line %d.\n", v.c_str(), line_of[k]);
        }
        else if (k == "post_inflation" && to_int(v, i)) p.post_inflation = (i != 0);
        else if (k == "horizon_factor" && to_double(v, d)) p.horizon_factor = d;
        else if (k == "omega" && to_double(v, d)) p.omega = d;
        else if (k == "dt_post_inflation" && to_double(v, d)) p.dt_post_inflation = d;
        else if (k == "af_post_inflation" && to_double(v, d)) { p.af_post_inflation = d; af_post_given = true; }
        else if (k == "post_inflation_integrator") {
            if (!parse_integrator(v, p.post_inflation_integrator))
                std::fprintf(stderr, "Ignoring invalid post_inflation_integrator '%s' on line %d.\n", v.c_str(), line_of[k]);
        }
        else if (k == "rk45_abs_tol" && to_double(v, d)) p.rk45_abs_tol = d;
        else if (k == "rk45_rel_tol" && to_double(v, d)) p.rk45_rel_tol = d;
        else if (k == "rk45_min_dt" && to_double(v, d)) p.rk45_min_dt = d;
        else if (k == "rk45_max_dt" && to_double(v, d)) p.rk45_max_dt = d;
        else if (k == "rk45_safety" && to_double(v, d)) p.rk45_safety = d;
        else if (k == "output_freq" && to_int(v, i)) p.output_freq = i;
        else if (k == "output_infrequent_freq" && to_int(v, i)) p.output_infrequent_freq = i;
        else if (k == "dN" && to_double(v, d)) p.dN = d;
        else if (k == "Nend" && to_double(v, d)) p.Nend = d;
        else if (k == "use_phiref_manual" && to_int(v, i)) p.use_phiref_manual = (i != 0);
        else if (k == "phiref_manual_value" && to_double(v, d)) p.phiref_manual_value = d;
        else if (k == "high_cutoff_index" && to_double(v, d)) p.high_cutoff_index = d;
        else if (k == "low_cutoff_index" && to_double(v, d)) p.low_cutoff_index = d;
        else if (k == "forcing_cutoff" && to_int(v, i)) p.forcing_cutoff = (i != 0);
        else if (k == "output_spectra" && to_int(v, i)) p.output_spectra = (i != 0);
        else if (k == "output_histogram" && to_int(v, i)) p.output_histogram = (i != 0);
        else if (k == "output_energy" && to_int(v, i)) p.output_energy = (i != 0);
        else if (k == "output_box3D" && to_int(v, i)) p.output_box3D = (i != 0);
        else if (k == "output_box2D" && to_int(v, i)) p.output_box2D = (i != 0);
        else if (k == "output_bispectrum" && to_int(v, i)) p.output_bispectrum = (i != 0);
        else if (k == "output_LOG" && to_int(v, i)) p.output_LOG = (i != 0);
        else if (k == "eta_log") {}
        else if (k == "screen_updates" && to_int(v, i)) p.screen_updates = (i != 0);
        else if (k == "nbins" && to_int(v, i)) p.nbins = i;
        else if (k == "int_err" && to_int(v, i)) p.int_err = i < 1 ? 1 : i;
        else if (k == "int_errN" && to_int(v, i)) p.int_errN = i < 1 ? 1 : i;
        else ok = false;
        if (!ok) std::fprintf(stderr, "Ignoring unknown or invalid parameter '%s' on line %d.\n", k.c_str(), line_of[k]);
    }
    if (!B_given) p.rescale_B = std::sqrt(p.V0);
    if (!af_given) p.af = 2.0 * p.N;
    if (!af_post_given) p.af_post_inflation = 2.0 * p.N;
    p.dx = p.L / (double)p.N;
    if (p.criterion == 99) p.criterion = p.numerical_potential ? 1 : -1;
    return true;
}
