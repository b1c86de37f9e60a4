// Host-side check of the split step's window lookups (inflation-easy_gb300/
// csrc/split_window.cuh), built with nvcc and run on the CPU by
// tests/test_window_cache.py:
//   window_cache_check SEED WINDOWS
// For WINDOWS random windows (1 .. kWin brackets of random widths around a
// background at 0, random lines) and many values around the background
// (random spreads of up to several brackets, the nodes themselves and their
// float neighbours), every lookup is compared with a search over the whole
// window: window_find and window_lift give the value's bracket (or -1 outside
// the window); the three-bracket cache answers exactly for the background's
// bracket and its neighbours, the five-bracket cache for two brackets either
// side, each with that bracket's own line, bit for bit.  Prints the number of
// mismatches.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "split_window.cuh"

using namespace iegpu;

static unsigned long long splitmix(unsigned long long& s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unit(unsigned long long& s) { return (double)(splitmix(s) >> 11) * 0x1.0p-53; }

static bool same(float a, float b) { return std::memcmp(&a, &b, sizeof a) == 0; }

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: window_cache_check SEED WINDOWS\n");
        return 2;
    }
    unsigned long long seed = std::strtoull(argv[1], nullptr, 10);
    const long windows = std::strtol(argv[2], nullptr, 10);
    long checks = 0, bad = 0;
    std::vector<float> w(3 * kWin + 1);
    for (long t = 0; t < windows; ++t) {
        const int n = 1 + (int)(splitmix(seed) % kWin);
        // nodes u[0] > ... > u[n] with 0 in (u[n], u[0]]: widths from 1e-6 to 1e-2
        std::vector<double> width(n);
        double total = 0;
        for (int q = 0; q < n; ++q) total += width[q] = std::exp(std::log(1e-6) + unit(seed) * std::log(1e4));
        const double top = total * unit(seed);
        double u = top;
        for (int q = 0; q <= n; ++q) {
            w[q] = (float)u;
            if (q < n) u -= width[q];
        }
        if (!(w[0] >= 0.f && 0.f > w[n])) continue;   // rounding put the background on an edge: skip
        bool strict = true;
        for (int q = 0; q < n; ++q) strict = strict && w[q] > w[q + 1];
        if (!strict) continue;
        for (int q = 0; q < kWin; ++q) {
            w[kWin + 1 + q] = (float)(unit(seed) * 2 - 1);
            w[2 * kWin + 1 + q] = (float)(unit(seed) * 2 - 1);
        }
        const WinCache c3 = win_cache<true, false>(w.data(), n);
        const WinCache c5 = win_cache<true, true>(w.data(), n);
        const int qc = window_find(w.data(), n, 0.f);
        std::vector<float> xs;
        for (int q = 0; q <= n; ++q) {
            xs.push_back(w[q]);
            xs.push_back(std::nextafter(w[q], 1.f));
            xs.push_back(std::nextafter(w[q], -1.f));
        }
        const double spread = width[qc] * (0.5 + 4 * unit(seed));
        for (int k = 0; k < 400; ++k) xs.push_back((float)((unit(seed) * 2 - 1) * spread));
        for (float x : xs) {
            int b = -1;   // the whole window's bracket: u[b] >= x > u[b+1]
            for (int q = 0; q < n; ++q)
                if (x <= w[q] && x > w[q + 1]) b = q;
            ++checks;
            if (window_find(w.data(), n, x) != b) ++bad;
            if (window_lift(w.data(), n, x) != b) ++bad;
            for (int wide = 0; wide < 2; ++wide) {
                float A = 0.f, s = 0.f;
                const bool hit = wide ? cache_line<true>(c5, x, A, s) : cache_line<false>(c3, x, A, s);
                const int reach = wide ? 2 : 1;
                const bool want = b >= 0 && b >= qc - reach && b <= qc + reach;
                if (hit != want) {
                    ++bad;
                    continue;
                }
                if (hit && (!same(A, w[kWin + 1 + b]) || !same(s, w[2 * kWin + 1 + b]))) ++bad;
            }
        }
    }
    std::printf("checks %ld mismatches %ld\n", checks, bad);
    return 0;
}
