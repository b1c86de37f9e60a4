// Host-side check of the engine's exact arithmetic (inflation-easy_gb300/
// csrc/exact.cuh), built with nvcc and run on the CPU by
// tests/test_exact_arith.py:
//   div SEED COUNT   the exact division by a fixed divisor against IEEE
//                    division for COUNT random dividends per divisor; prints
//                    the number of mismatching results
//   sum FILE         the exact sum of the doubles in FILE (raw little-endian
//                    binary); prints its bits in hex and the flags
//   sumprod FILE     the exact sum of the products of the pairs of doubles in
//                    FILE (x0 y0 x1 y1 ...); prints its bits and the flags
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "exact.cuh"

using namespace iegpu;

static unsigned long long splitmix(unsigned long long& s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static int check_div(unsigned long long seed, long count) {
    std::vector<double> ys = {3.338e-13, 3e-9, 3.0, 0.1, 1.0 / 3.0, 7.0, 1.5, 1.0, 0.25, 6.02e23, 1e-300};
    ys[0] = 5.777542733278901e-07 * 5.777542733278901e-07;   // B^2 of the hilltop preset
    ys[1] = 5.477225575051661e-05 * 5.477225575051661e-05;   // B^2 of the USR preset
    for (int q = 0; q < 16; ++q) {
        const unsigned long long b = (splitmix(seed) & 0x000FFFFFFFFFFFFFull) |
                                     ((unsigned long long)(1 + splitmix(seed) % 2046) << 52);
        ys.push_back(bitsd(b));
    }
    long bad = 0, n = 0;
    for (double y : ys) {
        const DivConst D = make_div_const(y);
        for (long i = 0; i < count; ++i) {
            double x;
            const unsigned long long r = splitmix(seed);
            switch (i & 3) {
                case 0: x = bitsd(r); break;                                   // any bit pattern
                case 1: x = bitsd((r & 0x800FFFFFFFFFFFFFull) | (dbits(y) & 0x7FF0000000000000ull)); break;  // quotient near 1
                case 2: x = y * (double)(r >> 11) * 0x1p-40; break;            // near multiples of y
                default: x = bitsd((r & 0x800FFFFFFFFFFFFFull) | ((unsigned long long)(r % 2047) << 52)); break;
            }
            const double a = div_exact(x, D), b = x / y;
            const unsigned long long ba = dbits(a), bb = dbits(b);
            const bool both_nan = (a != a) && (b != b);
            if (ba != bb && !both_nan) {
                if (bad < 10) std::printf("mismatch y=%a x=%a got %a want %a\n", y, x, a, b);
                ++bad;
            }
            ++n;
        }
    }
    std::printf("checked %ld mismatches %ld\n", n, bad);
    return bad ? 1 : 0;
}

static int check_sum(const char* path) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return 2;
    std::vector<double> x;
    double v;
    while (std::fread(&v, sizeof v, 1, fp) == 1) x.push_back(v);
    std::fclose(fp);
    Acc4 A;
    acc_zero(A);
    unsigned flags = 0;
    for (double t : x) acc_add_term(A, t, flags);
    const double s = acc_to_double(A);
    std::printf("%016llx %u\n", dbits(s), flags);
    return 0;
}

static int check_sumprod(const char* path) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return 2;
    std::vector<double> x;
    double v;
    while (std::fread(&v, sizeof v, 1, fp) == 1) x.push_back(v);
    std::fclose(fp);
    Acc4 A;
    acc_zero(A);
    unsigned flags = 0;
    for (size_t i = 0; i + 1 < x.size(); i += 2) acc_add_product(A, x[i], x[i + 1], flags);
    std::printf("%016llx %u\n", dbits(acc_to_double(A)), flags);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 4 && !std::strcmp(argv[1], "div")) return check_div(std::strtoull(argv[2], 0, 10), std::atol(argv[3]));
    if (argc >= 3 && !std::strcmp(argv[1], "sum")) return check_sum(argv[2]);
    if (argc >= 3 && !std::strcmp(argv[1], "sumprod")) return check_sumprod(argv[2]);
    std::fprintf(stderr, "usage: %s div SEED COUNT | sum FILE | sumprod FILE\n", argv[0]);
    return 2;
}
