// ic.cu -- Bunch-Davies initial conditions on the device
// (initializef, src/initialize.cpp:118-214).
//
// The reference draws two uniforms per mode from one Park-Miller stream
// (src/initialize.cpp:18-31, 99 warm-up calls) while it walks the half-space
// of modes in (i, j, k) order.  Here one thread owns one (i, j) row: the host
// counts the set_mode calls that precede each row in that walk, and the thread
// jumps the stream there (x_q = seed * 16807^(100+q) mod 2^31-1, by
// square-and-multiply), so every mode gets exactly the reference's uniforms.
// The mode amplitudes use the reference's expressions; the lattice
// dispersion sin^2 table is computed on the host with the reference's own
// expression, so p2, omega and the rms amplitude are bit-identical, and only
// log/cos/sin come from the device maths library.  The inverse r2c FFT
// (fft.cu) and the background add then complete initializef.
#include <cmath>
#include <vector>

#include "iegpu_internal.cuh"

namespace iegpu {

struct IcArgs {
    double* f;
    double* fd;
    double* fny;
    double* fdny;
    const double* s2;           // sin^2(pi p / N) at [p + N/2], p = -N/2..N/2
    const long long* row_draw;  // index of the first uniform drawn for row (i, j)
    int lg;
    int seed;
    double norm, hbterm, dp2, four_NL2, L_over_2pi, hi_cut, lo_cut;
};

constexpr unsigned long long kM31 = 2147483647ULL;

__device__ __forceinline__ unsigned long long mulmod31(unsigned long long a, unsigned long long b) {
    return (a * b) % kM31;
}

struct Stream {
    unsigned long long x;
    int constant;
    __device__ double next() {
        if (constant) return 0.33;
        const double v = (double)x / (double)2147483647;
        x = mulmod31(x, 16807ULL);
        return v;
    }
};

__device__ void set_mode_dev(const IcArgs& A, Stream& rng, double p2, double p2lat, double* field, double* deriv,
                             int real) {
    const double ii = A.L_over_2pi * sqrt(p2lat);
    const double omega = sqrt(p2);
    double rms = (omega > 0.0) ? A.norm / sqrt(2.0 * omega) : 0.0;
    if (A.hi_cut > 0 && (ii > A.hi_cut || ii < A.lo_cut)) rms = 0.0;
    const double amplitude = rms * sqrt(log(1.0 / rng.next()));
    const double phase = 2.0 * 3.14159265358979311600 * rng.next();
    double sp, cp;
    sincos(phase, &sp, &cp);
    const double re = amplitude * cp, im = amplitude * sp;
    field[0] = re;
    field[1] = im;
    deriv[0] = omega * im + A.hbterm * field[0];
    deriv[1] = -omega * re + A.hbterm * field[1];
    if (real == 1) { field[1] = 0.0; deriv[1] = 0.0; }
}

__global__ void k_bunch_davies(IcArgs A) {
    const int N = 1 << A.lg, h = N >> 1;
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (long long)N * N) return;
    const int i = (int)(r >> A.lg), j = (int)(r & (N - 1));
    Stream rng;
    rng.constant = A.seed < 1;
    {
        // x = seed * 16807^(100 + q) mod (2^31 - 1)
        unsigned long long e = 100ULL + (unsigned long long)A.row_draw[r], base = 16807ULL, acc = 1ULL;
        while (e) {
            if (e & 1ULL) acc = mulmod31(acc, base);
            base = mulmod31(base, base);
            e >>= 1;
        }
        rng.x = mulmod31(acc, (unsigned long long)(A.seed < 1 ? 1 : A.seed));
    }
    const int px = (i <= h ? i : i - N), py = (j <= h ? j : j - N);
    const int iconj = (i == 0 ? 0 : N - i);
    const double s2x = A.s2[px + h], s2y = A.s2[py + h];
    const double dpx = px, dpy = py;
    auto at = [&](int ii, int jj, int kk) { return ((long long)ii * N + jj) * N + kk; };
    for (int k = 1; k < h; k++) {
        const double pz = k;
        const double p2lat = A.dp2 * ((dpx * dpx) + (dpy * dpy) + (pz * pz));
        const double p2 = A.four_NL2 * (s2x + s2y + A.s2[k + h]);
        set_mode_dev(A, rng, p2, p2lat, &A.f[at(i, j, 2 * k)], &A.fd[at(i, j, 2 * k)], 0);
    }
    double* ny = A.fny + (long long)i * 2 * N + 2 * j;
    double* dny = A.fdny + (long long)i * 2 * N + 2 * j;
    const double hh = (double)(h * h);
    if (j > h || (i > h && (j == 0 || j == h))) {
        const int jconj = (j == 0 ? 0 : N - j);
        double p2lat = A.dp2 * ((dpx * dpx) + (dpy * dpy));
        double p2 = A.four_NL2 * (s2x + s2y);
        set_mode_dev(A, rng, p2, p2lat, &A.f[at(i, j, 0)], &A.fd[at(i, j, 0)], 0);
        A.f[at(iconj, jconj, 0)] = A.f[at(i, j, 0)];
        A.f[at(iconj, jconj, 1)] = -A.f[at(i, j, 1)];
        A.fd[at(iconj, jconj, 0)] = A.fd[at(i, j, 0)];
        A.fd[at(iconj, jconj, 1)] = -A.fd[at(i, j, 1)];
        p2lat = A.dp2 * ((dpx * dpx) + (dpy * dpy) + hh);
        p2 = A.four_NL2 * (s2x + s2y + 1.0);
        set_mode_dev(A, rng, p2, p2lat, ny, dny, 0);
        double* cny = A.fny + (long long)iconj * 2 * N + 2 * jconj;
        double* cdny = A.fdny + (long long)iconj * 2 * N + 2 * jconj;
        cny[0] = ny[0];
        cny[1] = -ny[1];
        cdny[0] = dny[0];
        cdny[1] = -dny[1];
    } else if ((i == 0 || i == h) && (j == 0 || j == h)) {
        double p2lat = A.dp2 * ((dpx * dpx) + (dpy * dpy));
        double p2 = A.four_NL2 * (s2x + s2y);
        if (p2 > 0.0) set_mode_dev(A, rng, p2, p2lat, &A.f[at(i, j, 0)], &A.fd[at(i, j, 0)], 1);
        p2lat = A.dp2 * ((dpx * dpx) + (dpy * dpy) + hh);
        p2 = A.four_NL2 * (s2x + s2y + 1.0);
        set_mode_dev(A, rng, p2, p2lat, ny, dny, 1);
    }
    if (r == 0) {
        // the zero mode is removed (src/initialize.cpp:188-191)
        A.f[0] = 0.0;
        A.f[1] = 0.0;
        A.fd[0] = 0.0;
        A.fd[1] = 0.0;
    }
}

// Number of set_mode calls the reference makes for row (i, j) before k
// reaches the special planes: N/2-1 interior modes plus 0, 1 or 2 specials.
static int row_calls(int N, int i, int j) {
    const int h = N / 2;
    int n = h - 1;
    if (j > h || (i > h && (j == 0 || j == h))) n += 2;
    else if ((i == 0 || i == h) && (j == 0 || j == h)) n += (i == 0 && j == 0) ? 1 : 2;
    return n;
}

int bunch_davies(iegpu_ctx* c, int seed, double phi0, double dphi0, double hubble, double hi_cut, double lo_cut) {
    const int N = c->N, h = N / 2;
    const double pi = 2.0 * std::asin(1.0);
    const double L = c->cfg.L, dx = L / (double)N;
    std::vector<long long> draws((size_t)N * N);
    long long q = 0;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            draws[(size_t)i * N + j] = 2 * q;
            q += row_calls(N, i, j);
        }
    std::vector<double> s2((size_t)N + 1);
    for (int p = -h; p <= h; ++p) {
        const double sp = std::sin((double)p * pi / N);
        s2[(size_t)(p + h)] = sp * sp;
    }
    long long* d_draws = nullptr;
    double* d_s2 = nullptr;
    if (check_cuda(c, cudaMalloc(&d_draws, sizeof(long long) * draws.size()), "ic alloc")) return IEGPU_ENOMEM;
    if (check_cuda(c, cudaMalloc(&d_s2, sizeof(double) * s2.size()), "ic alloc")) { cudaFree(d_draws); return IEGPU_ENOMEM; }
    int rc = check_cuda(c, cudaMemcpyAsync(d_draws, draws.data(), sizeof(long long) * draws.size(), cudaMemcpyHostToDevice, c->stream), "ic upload");
    if (!rc) rc = check_cuda(c, cudaMemcpyAsync(d_s2, s2.data(), sizeof(double) * s2.size(), cudaMemcpyHostToDevice, c->stream), "ic upload");
    double* f = c->f[c->cur];
    if (!rc) {
        cudaMemsetAsync(f, 0, sizeof(double) * c->gs, c->stream);
        cudaMemsetAsync(c->fd, 0, sizeof(double) * c->gs, c->stream);
        cudaMemsetAsync(c->fny, 0, sizeof(double) * N * 2 * N, c->stream);
        cudaMemsetAsync(c->fdny, 0, sizeof(double) * N * 2 * N, c->stream);
        IcArgs A;
        A.f = f;
        A.fd = c->fd;
        A.fny = c->fny;
        A.fdny = c->fdny;
        A.s2 = d_s2;
        A.row_draw = d_draws;
        A.lg = c->lg;
        A.seed = seed;
        A.norm = c->cfg.rescale_B * std::pow(L / (dx * dx), 1.5);
        A.hbterm = -hubble;
        A.dp2 = (2.0 * pi / L) * (2.0 * pi / L);
        A.four_NL2 = 4.0 * ((N / L) * (N / L));
        A.L_over_2pi = L / (2.0 * pi);
        A.hi_cut = hi_cut;
        A.lo_cut = lo_cut;
        const long long rows = (long long)N * N;
        k_bunch_davies<<<(unsigned)((rows + 127) / 128), 128, 0, c->stream>>>(A);
        c->launches++;
        rc = check_cuda(c, cudaGetLastError(), "ic launch");
    }
    if (!rc) rc = fft_d(c, f, c->fny, -1);
    if (!rc) rc = fft_d(c, c->fd, c->fdny, -1);
    if (!rc) rc = sync_and_check(c, "initial conditions");
    cudaFree(d_draws);
    cudaFree(d_s2);
    if (!rc) rc = field_add(c, IEGPU_F, phi0);
    if (!rc) rc = field_add(c, IEGPU_FD, dphi0);
    return rc;
}

}  // namespace iegpu
