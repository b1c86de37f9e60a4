// ref_driver.cpp -- full-precision dump driver for the reference program.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles the unmodified
// reference sources (src/*.cpp of caravangelo/inflation-easy, with only the
// compile-time lines of src/parameters.h set per configuration) together with
// this file.  The reference's main() (src/main.cpp:103-146) is compiled as
// ie_ref_main() and run unchanged; this driver only observes it:
//   * the linker wraps save(int), saveN() and, with the post-inflation phase,
//     save_post_inflation(int) (--wrap) so the background scalars are traced
//     at full precision each time the reference saves;
//   * after the run the final lattice state is written in binary.
// Usage: ie_ref <workdir>   (workdir holds params.txt and inputs/)
//
// A second mode runs the reference's spectraf() (src/output.cpp:297-406) once
// on given fields, with the forcing cutoff on, to pin the mode filter of
// :330-401 for any cutoffs (a low cutoff also zeroes the k = 0 mode, so a
// whole run with one is no useful case):
//   ie_ref --spectraf <workdir>
// reads workdir/cut_in.bin (f, fd: N^3 doubles each; then high_cutoff_index,
// low_cutoff_index), writes f and fd after the call to workdir/cut_out.bin;
// the spectrum goes to workdir/results/spectra.dat as in a run.
#include "main.h"

#include <cstdio>
#include <cstring>
#include <unistd.h>

int ie_ref_main();

static FILE* g_trace = nullptr;

extern "C" void __real__Z4savei(int);
extern "C" void __wrap__Z4savei(int infrequent) {
    if (g_trace)
        std::fprintf(g_trace, "save %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, t, a, ad, ad2, astep);
    __real__Z4savei(infrequent);
}

#if perform_deltaN
extern "C" void __real__Z5saveNv();
extern "C" void __wrap__Z5saveNv() {
    if (g_trace) std::fprintf(g_trace, "saveN %.17g %.17g %.17g %.17g\n", t, a, Ne, phiref);
    __real__Z5saveNv();
}
#endif

#if post_inflation
extern "C" void __real__Z19save_post_inflationi(int);
extern "C" void __wrap__Z19save_post_inflationi(int infrequent) {
    if (g_trace)
        std::fprintf(g_trace, "savep %d %.17g %.17g %.17g %.17g %.17g\n", infrequent, t, a, ad, ad2, astep);
    __real__Z19save_post_inflationi(infrequent);
}
#endif

template <typename T>
static void dump(FILE* fp, const std::vector<T>& v) {
    std::fwrite(v.data(), sizeof(T), v.size(), fp);
}

void spectraf();   // src/output.cpp:297 (not declared in src/main.h)

static int run_spectraf() {
    const size_t gs = (size_t)N * N * N;
    f.assign(gs, 0.0);
    fd.assign(gs, 0.0);
    double cut[2];
    FILE* in = std::fopen("cut_in.bin", "rb");
    if (!in) return 2;
    const bool ok = std::fread(f.data(), sizeof(double), gs, in) == gs &&
                    std::fread(fd.data(), sizeof(double), gs, in) == gs && std::fread(cut, sizeof(double), 2, in) == 2;
    std::fclose(in);
    if (!ok) return 2;
    high_cutoff_index = cut[0];
    low_cutoff_index = cut[1];
    forcing_cutoff = 1;
    spectraf();
    FILE* out = std::fopen("cut_out.bin", "wb");
    dump(out, f);
    dump(out, fd);
    std::fclose(out);
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 3 && std::strcmp(argv[1], "--spectraf") == 0) {
        if (chdir(argv[2]) != 0) return 2;
        return run_spectraf();
    }
    if (argc < 2 || chdir(argv[1]) != 0) {
        std::fprintf(stderr, "usage: ie_ref <workdir>\n");
        return 2;
    }
    g_trace = std::fopen("trace.txt", "w");
    const int rc = ie_ref_main();
    std::fclose(g_trace);
    g_trace = nullptr;
    FILE* fp = std::fopen("state.bin", "wb");
    const double scal[8] = {t, a, ad, ad2, astep, Ne, phiref, hubble_init};
    const int hdr[4] = {N, perform_deltaN, calculate_SIGW, numerical_potential};
    std::fwrite(hdr, sizeof(int), 4, fp);
    std::fwrite(scal, sizeof(double), 8, fp);
    dump(fp, f);
    dump(fp, fd);
#if perform_deltaN
    dump(fp, deltaN);
#endif
#if calculate_SIGW
    for (int c = 0; c < 6; ++c) dump(fp, hij[c]);
    for (int c = 0; c < 6; ++c) dump(fp, hijd[c]);
#endif
    std::fclose(fp);
    return rc;
}
