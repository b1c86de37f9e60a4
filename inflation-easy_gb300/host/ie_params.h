// ie_params.h -- run-time parameters of the host program.
//
// The keys, defaults and derived values of the reference's params.txt handling
// (src/runtime_parameters.cpp:17-112, 195-365).  The switches the reference
// fixes at compile time in src/parameters.h (N, numerical_potential,
// perform_deltaN, calculate_SIGW, post_inflation, the deltaN criterion) are
// run-time keys here, plus `form` (fp64 | split | split_comp) for the engine's
// arithmetic form.
#pragma once

#include <string>

// Integrators of src/parameters.h (INTEGRATOR_LEAPFROG, _RK4, _RK45).
enum { IE_LEAPFROG = 0, IE_RK4 = 1, IE_RK45 = 2 };
const char* ie_integrator_name(int integrator);

struct IeParams {
    // compile-time switches of the reference, run-time here
    int N = 128;
    int numerical_potential = 1;
    int perform_deltaN = 1;
    int calculate_SIGW = 0;
    int criterion = 99;          // 99: derive from numerical_potential (src/parameters.h:65-71)
    int form = 0;                // 0 fp64, 1 split, 2 compensated split
    int ic_on_host = 0;          // 1: draw the initial modes on the host (bit-identical to the reference)
    // src/runtime_parameters.cpp:17-112
    int seed = 8;
    double rescale_s = 0.0;
    double af = 256.0;
    double V0 = 3e-9;
    double rescale_B = 0.0;
    double ns = 0.97;
    double initial_field = 2.9181235049318586;
    double initial_derivative = -0.06727651095116181;
    double L = 10.0;
    double dt = 0.001;
    int output_freq = 500;
    int output_infrequent_freq = 500;
    double dN = 0.0001;
    double Nend = 5.0;
    int use_phiref_manual = 0;
    double phiref_manual_value = 0.0;
    double high_cutoff_index = 0.0;
    double low_cutoff_index = 0.0;
    int forcing_cutoff = 0;
    int output_spectra = 1;
    int output_histogram = 1;
    int output_energy = 1;
    int output_box3D = 0;
    int output_box2D = 0;
    int output_bispectrum = 0;
    int output_LOG = 0;
    int screen_updates = 1;
    int nbins = 256;
    int int_err = 5;
    int int_errN = 5;
    double dx = 0.0;
    int inflation_integrator = IE_LEAPFROG;
    int deltaN_integrator = IE_LEAPFROG;
    // post-inflation phase (src/parameters.h:31 switch, run-time here and off
    // by default; src/runtime_parameters.cpp:48-52, 295-299)
    int post_inflation = 0;
    double horizon_factor = 1.0;
    double omega = 1.0 / 3.0;
    double dt_post_inflation = 0.001;
    double af_post_inflation = 0.0;   // 2N unless given
    int post_inflation_integrator = IE_LEAPFROG;
    // RK45 controls (src/runtime_parameters.cpp:82-86); non-positive steps
    // mean the reference's defaults, applied by the library
    double rk45_abs_tol = 1e-8;
    double rk45_rel_tol = 1e-6;
    double rk45_min_dt = -1.0;
    double rk45_max_dt = -1.0;
    double rk45_safety = 0.9;
};

// Defaults of the reference for the given potential kind and N.
void ie_params_defaults(IeParams& p, int N, int numerical);
// Reads params.txt (missing file keeps the defaults); warns on unknown keys
// as src/runtime_parameters.cpp:333-339 does.  Returns false on a fatal error.
bool ie_params_load(IeParams& p, const char* path);
