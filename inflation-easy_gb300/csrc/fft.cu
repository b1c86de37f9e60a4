// fft.cu -- in-place real 3D FFT with a separate Nyquist plane, computing
// exactly what fftrnd / fftrnf of src/ffteasy.hpp:127-190 compute.
//
// The reference transform is: a complex 3D FFT of the N x N x N/2 complex
// view (radix-2, bit-reversal then Danielson-Lanczos stages, one 1D pass per
// dimension, k first, src/ffteasy.hpp:21-88), then a per-row unpacking that
// pairs row (i,j) with row (-i,-j) and moves the k = 0 column against the
// Nyquist plane (src/ffteasy.hpp:146-184).  The inverse runs the unpacking
// first and normalises each 1D pass by its length.
//
// Here every 1D pass is a shared-memory kernel working on a tile of lines
// (coalesced along k for the strided j and i passes).  The butterflies use the
// reference's twiddle values (generated on the host with the reference's own
// cos/sin recurrence) and the reference's expression order, and this file is
// compiled with -fmad=false, so the output is bit-identical to the reference
// transform.  Butterflies of one stage are independent, and each unpacking
// pair is touched by exactly one thread, so the parallel order cannot change
// any result.
#include <cmath>
#include <cstdio>
#include <vector>

#include "iegpu_internal.cuh"

namespace iegpu {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

// Pass geometry: element e of line l lives at base(l) + e*stride.
//   kind 0 (k lines): base = l*M, stride 1
//   kind 1 (j lines): base = (l / M2)*N*M2 + (l % M2), stride M2
//   kind 2 (i lines): base = l, stride N*M2
struct PassGeom {
    int kind;
    int M;        // line length
    int lgM;
    int N;
    int M2;       // N/2 (complex row length)
    long long stride;
};

__device__ __forceinline__ long long line_base(const PassGeom& g, long long l) {
    if (g.kind == 0) return l * g.M;
    if (g.kind == 1) return (l / g.M2) * (long long)g.N * g.M2 + (l % g.M2);
    return l;
}

__device__ __forceinline__ int bitrev(int x, int lg) { return (int)(__brev((unsigned)x) >> (32 - lg)); }

// One Danielson-Lanczos butterfly, src/ffteasy.hpp:46-58, in the reference's
// expression order (this file is compiled with -fmad=false).
template <typename C2>
__device__ __forceinline__ void butterfly(C2& t1, C2& t2, C2 wb) {
    C2 o1, o2;
    o1.x = t1.x + wb.x * t2.x - wb.y * t2.y;
    o1.y = t1.y + wb.x * t2.y + wb.y * t2.x;
    o2.x = t1.x - wb.x * t2.x + wb.y * t2.y;
    o2.y = t1.y - wb.x * t2.y - wb.y * t2.x;
    t1 = o1;
    t2 = o2;
}

// One 1D complex FFT pass over LPB lines per CTA (fftc1, src/ffteasy.hpp:21-70).
template <typename T>
__global__ void __launch_bounds__(256) k_fft_pass(typename Cplx<T>::type* __restrict__ data,
                                                  const typename Cplx<T>::type* __restrict__ tw, PassGeom g,
                                                  int LPB, int inverse) {
    using C2 = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2* sm = reinterpret_cast<C2*>(smem_raw);
    const int M = g.M, lgM = g.lgM;
    const int ld = M + 1;  // padded line length in shared memory
    const long long l0 = (long long)blockIdx.x * LPB;
    const int total = LPB * M;
    // load, scattering each line into bit-reversed order
    if (g.kind == 0) {
        const long long base = l0 * M;
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            const int ll = q / M, e = q - ll * M;
            sm[ll * ld + bitrev(e, lgM)] = data[base + q];
        }
    } else {
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            const int e = q / LPB, ll = q - e * LPB;
            sm[ll * ld + bitrev(e, lgM)] = data[line_base(g, l0 + ll) + (long long)e * g.stride];
        }
    }
    __syncthreads();
    // Danielson-Lanczos stages, two per pass through shared memory: stages s
    // and s + 1 (half h = 2^(s-1)) touch the elements e, e + h, e + 2h, e + 3h
    // of a block of 4h only among themselves, so one thread runs the four
    // butterflies of such a group in registers (stage s: (e, e+h) and
    // (e+2h, e+3h) with w_s[b]; stage s + 1: (e, e+2h) with w_{s+1}[b] and
    // (e+h, e+3h) with w_{s+1}[b+h]).  Each butterfly is the reference's, on the
    // same operands, so the bits do not change; an odd last stage runs alone.
    const int half_lines = M >> 1, quarter_lines = M >> 2;
    int s = 1;
    for (; s + 1 <= lgM; s += 2) {
        const int h = 1 << (s - 1);
        const C2* w1 = tw + (h - 1);
        const C2* w2 = tw + (2 * h - 1);
        for (int q = threadIdx.x; q < LPB * quarter_lines; q += blockDim.x) {
            const int ll = q / quarter_lines, r = q - ll * quarter_lines;
            const int blk = r >> (s - 1), b = r & (h - 1);
            const int e = blk * (h << 2) + b;
            C2* line = sm + ll * ld;
            C2 x0 = line[e], x1 = line[e + h], x2 = line[e + 2 * h], x3 = line[e + 3 * h];
            butterfly(x0, x1, w1[b]);
            butterfly(x2, x3, w1[b]);
            butterfly(x0, x2, w2[b]);
            butterfly(x1, x3, w2[b + h]);
            line[e] = x0;
            line[e + h] = x1;
            line[e + 2 * h] = x2;
            line[e + 3 * h] = x3;
        }
        __syncthreads();
    }
    if (s == lgM) {
        const int half = 1 << (s - 1);
        const C2* w = tw + (half - 1);
        for (int q = threadIdx.x; q < LPB * half_lines; q += blockDim.x) {
            const int ll = q / half_lines, r = q - ll * half_lines;
            const int trans = r >> (s - 1), b = r & (half - 1);
            const int i1 = trans * (half << 1) + b, i2 = i1 + half;
            C2* line = sm + ll * ld;
            C2 t1 = line[i1], t2 = line[i2];
            butterfly(t1, t2, w[b]);
            line[i1] = t1;
            line[i2] = t2;
        }
        __syncthreads();
    }
    // store (inverse: divide by the line length, src/ffteasy.hpp:64-69).  M is
    // a power of two, so x / M and x * (1/M) are the same exact real number and
    // both IEEE operations round it identically (subnormal results included):
    // the multiplication by the exact reciprocal gives the division's bits
    // without the division's FP64 iteration.
    const T rinv = (T)1 / (T)M;
    if (g.kind == 0) {
        const long long base = l0 * M;
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            const int ll = q / M, e = q - ll * M;
            C2 v = sm[ll * ld + e];
            if (inverse) { v.x *= rinv; v.y *= rinv; }
            data[base + q] = v;
        }
    } else {
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            const int e = q / LPB, ll = q - e * LPB;
            C2 v = sm[ll * ld + e];
            if (inverse) { v.x *= rinv; v.y *= rinv; }
            data[line_base(g, l0 + ll) + (long long)e * g.stride] = v;
        }
    }
}

// cnyquist[r] = c[r*M2] before the forward unpacking (src/ffteasy.hpp:146-150).
template <typename T>
__global__ void k_fft_nyq_copy(const typename Cplx<T>::type* __restrict__ c, typename Cplx<T>::type* __restrict__ ny,
                               int rows, int M2) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) ny[r] = c[(long long)r * M2];
}

// Row unpacking of src/ffteasy.hpp:152-184.  Thread (r, b): b >= 1 updates the
// pair (row r, b) / (row -r, M2-b); b == 0 updates (row r, 0) / Nyquist[-r].
template <typename T>
__global__ void k_fft_unpack(typename Cplx<T>::type* __restrict__ c, typename Cplx<T>::type* __restrict__ ny,
                             const typename Cplx<T>::type* __restrict__ uw, int lgN, int forward) {
    using C2 = typename Cplx<T>::type;
    const int N = 1 << lgN, M2 = N >> 1, Q = N >> 2;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)N * N;
    if (q >= rows * Q) return;
    const int b = (int)(q % Q);
    const long long r = q / Q;
    const int i = (int)(r >> lgN), j = (int)(r & (N - 1));
    const long long rneg = (long long)((N - i) & (N - 1)) * N + ((N - j) & (N - 1));
    const T fw = (T)forward, h = (T)0.5;
    if (b == 0) {
        const C2 t1 = c[r * M2], t2 = ny[rneg];
        C2 a, z;
        a.x = h * (t1.x + t2.x + fw * (t1.y + t2.y));
        a.y = h * (t1.y - t2.y - fw * (t1.x - t2.x));
        z.x = h * (t1.x + t2.x - fw * (t1.y + t2.y));
        z.y = h * (-t1.y + t2.y - fw * (t1.x - t2.x));
        c[r * M2] = a;
        ny[rneg] = z;
    } else {
        const C2 wb = uw[b];
        const long long p1 = r * M2 + b, p2 = rneg * M2 + (M2 - b);
        const C2 t1 = c[p1], t2 = c[p2];
        C2 a, z;
        a.x = h * (t1.x + t2.x + fw * wb.x * (t1.y + t2.y) + wb.y * (t1.x - t2.x));
        a.y = h * (t1.y - t2.y - fw * wb.x * (t1.x - t2.x) + wb.y * (t1.y + t2.y));
        z.x = h * (t1.x + t2.x - fw * wb.x * (t1.y + t2.y) - wb.y * (t1.x - t2.x));
        z.y = h * (-t1.y + t2.y - fw * wb.x * (t1.x - t2.x) + wb.y * (t1.y + t2.y));
        c[p1] = a;
        c[p2] = z;
    }
}

// ---------------------------------------------------------------------------
// host side: twiddle tables with the reference's recurrence
// ---------------------------------------------------------------------------

template <typename T> static T host_cos(T x);
template <typename T> static T host_sin(T x);
template <typename T> static T host_asin(T x);
template <> double host_cos<double>(double x) { return std::cos(x); }
template <> double host_sin<double>(double x) { return std::sin(x); }
template <> double host_asin<double>(double x) { return std::asin(x); }
template <> float host_cos<float>(float x) { return std::cos(x); }
template <> float host_sin<float>(float x) { return std::sin(x); }
template <> float host_asin<float>(float x) { return std::asin(x); }

// Stage twiddles of fftc1 (src/ffteasy.hpp:40-60) for a line of length M.
template <typename T, typename C2>
static std::vector<C2> stage_twiddles(int M, int forward) {
    std::vector<C2> out((size_t)(M > 1 ? M - 1 : 1));
    const T pi2 = T(4) * host_asin<T>(T(1));
    for (int ts = 2; ts <= M; ts <<= 1) {
        const T pi2n = T(forward) * pi2 / T(ts);
        const T cs = host_cos<T>(pi2n), sn = host_sin<T>(pi2n);
        T wr = T(1), wi = T(0);
        for (int b = 0; b < ts / 2; ++b) {
            out[(size_t)(ts / 2 - 1 + b)] = C2{wr, wi};
            const T tr = wr, ti = wi;
            wr = cs * tr - sn * ti;
            wi = cs * ti + sn * tr;
        }
    }
    return out;
}

// Unpacking twiddles of fftrn (src/ffteasy.hpp:132-157), b = 1..N/4-1.
template <typename T, typename C2>
static std::vector<C2> unpack_twiddles(int N) {
    std::vector<C2> out((size_t)(N / 4 > 1 ? N / 4 : 1), C2{T(0), T(0)});
    const T pi2n = (T(4) * host_asin<T>(T(1))) / T(N);
    const T cs = host_cos<T>(pi2n), sn = host_sin<T>(pi2n);
    T wr = T(1), wi = T(0);
    for (int b = 1; b < N / 4; ++b) {
        const T tr = wr, ti = wi;
        wr = cs * tr - sn * ti;
        wi = cs * ti + sn * tr;
        out[(size_t)b] = C2{wr, wi};
    }
    return out;
}

template <typename C2>
static int upload_vec(iegpu_ctx* c, C2** dst, const std::vector<C2>& v) {
    if (check_cuda(c, cudaMalloc(dst, sizeof(C2) * v.size()), "twiddle alloc")) return IEGPU_ENOMEM;
    return check_cuda(c, cudaMemcpy(*dst, v.data(), sizeof(C2) * v.size(), cudaMemcpyHostToDevice), "twiddle upload");
}

int fft_init(iegpu_ctx* c) {
    const int N = c->N;
    const int lens[2] = {N, N / 2};
    for (int q = 0; q < 2; ++q) {
        if (upload_vec(c, &c->tw.c_fwd_d[q], stage_twiddles<double, double2>(lens[q], 1))) return IEGPU_ECUDA;
        if (upload_vec(c, &c->tw.c_inv_d[q], stage_twiddles<double, double2>(lens[q], -1))) return IEGPU_ECUDA;
        if (upload_vec(c, &c->tw.c_fwd_f[q], stage_twiddles<float, float2>(lens[q], 1))) return IEGPU_ECUDA;
        if (upload_vec(c, &c->tw.c_inv_f[q], stage_twiddles<float, float2>(lens[q], -1))) return IEGPU_ECUDA;
    }
    if (upload_vec(c, &c->tw.unpack_d, unpack_twiddles<double, double2>(N))) return IEGPU_ECUDA;
    if (upload_vec(c, &c->tw.unpack_f, unpack_twiddles<float, float2>(N))) return IEGPU_ECUDA;
    return IEGPU_OK;
}

void fft_free(iegpu_ctx* c) {
    for (int q = 0; q < 2; ++q) {
        cudaFree(c->tw.c_fwd_d[q]); cudaFree(c->tw.c_inv_d[q]);
        cudaFree(c->tw.c_fwd_f[q]); cudaFree(c->tw.c_inv_f[q]);
    }
    cudaFree(c->tw.unpack_d);
    cudaFree(c->tw.unpack_f);
    c->tw = FftTw{};
}

static int ilog2(int x) { int l = 0; while ((1 << l) < x) ++l; return l; }

template <typename T>
static void run_pass(iegpu_ctx* c, typename Cplx<T>::type* data, int kind, int forward) {
    using C2 = typename Cplx<T>::type;
    const int N = c->N, M2 = N / 2;
    PassGeom g;
    g.kind = kind;
    g.N = N;
    g.M2 = M2;
    g.M = (kind == 0) ? M2 : N;
    g.lgM = ilog2(g.M);
    g.stride = (kind == 0) ? 1 : (kind == 1 ? M2 : (long long)N * M2);
    const long long lines = (kind == 0) ? (long long)N * N : (long long)N * M2;
    // lines per CTA: about 64 KB of shared memory, at least 8 lines when the
    // pass is strided so that each row load is a 128-byte segment or more
    int LPB = (int)(65536 / ((long long)(g.M + 1) * sizeof(C2)));
    if (LPB < 1) LPB = 1;
    if (LPB > 32) LPB = 32;
    while (lines % LPB) --LPB;
    const size_t smem = (size_t)LPB * (g.M + 1) * sizeof(C2);
    const C2* tw;
    const int q = (g.M == N) ? 0 : 1;
    if (sizeof(T) == 8) tw = (const C2*)(forward > 0 ? (const void*)c->tw.c_fwd_d[q] : (const void*)c->tw.c_inv_d[q]);
    else tw = (const C2*)(forward > 0 ? (const void*)c->tw.c_fwd_f[q] : (const void*)c->tw.c_inv_f[q]);
    if (smem_optin((const void*)k_fft_pass<T>, 200 * 1024) != cudaSuccess) {
        set_error(c, IEGPU_ECUDA, "shared memory opt-in of the FFT pass failed");   // the launch then fails
    }
    k_fft_pass<T><<<(unsigned)(lines / LPB), 256, smem, c->stream>>>(data, tw, g, LPB, forward < 0 ? 1 : 0);
    c->launches++;
}

template <typename T>
static int fft_impl(iegpu_ctx* c, T* f, T* fny, int forward) {
    using C2 = typename Cplx<T>::type;
    C2* data = reinterpret_cast<C2*>(f);
    C2* ny = reinterpret_cast<C2*>(fny);
    const int N = c->N;
    const long long rows = (long long)N * N;
    const long long nunp = rows * (N / 4);
    const C2* uw = (const C2*)(sizeof(T) == 8 ? (const void*)c->tw.unpack_d : (const void*)c->tw.unpack_f);
    if (forward == 1) {
        for (int kind = 0; kind < 3; ++kind) run_pass<T>(c, data, kind, 1);
        k_fft_nyq_copy<T><<<(unsigned)((rows + 255) / 256), 256, 0, c->stream>>>(data, ny, (int)rows, N / 2);
        k_fft_unpack<T><<<(unsigned)((nunp + 255) / 256), 256, 0, c->stream>>>(data, ny, uw, c->lg, 1);
        c->launches += 2;
    } else {
        k_fft_unpack<T><<<(unsigned)((nunp + 255) / 256), 256, 0, c->stream>>>(data, ny, uw, c->lg, -1);
        c->launches++;
        for (int kind = 0; kind < 3; ++kind) run_pass<T>(c, data, kind, -1);
    }
    return check_cuda(c, cudaGetLastError(), "fft launch");
}

int fft_d(iegpu_ctx* c, double* f, double* fny, int forward) { return fft_impl<double>(c, f, fny, forward); }
int fft_f(iegpu_ctx* c, float* f, float* fny, int forward) { return fft_impl<float>(c, f, fny, forward); }

}  // namespace iegpu
