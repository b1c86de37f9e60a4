// spectra.cu -- isotropic shell binning of r2c spectra.
//
// Scalar spectra follow write_isotropic_spectrum_from_fft_r2c
// (src/output.cpp:63-151): the bin of mode (px, py, pz) is
// lround(sqrt(px^2+py^2+pz^2)); interior modes 1 <= k < N/2 carry weight 2,
// the k = 0 column and the Nyquist plane weight 1.  Tensor spectra follow
// write_gw_spectrum_impl (src/output.cpp:466-625): per mode, the lattice
// momentum k_i = (2/dx) sin(pi p_i/N), the projector P = 1 - khat khat and the
// TT part Lambda = P C P - P tr(PC)/2 of the 3x3 complex matrix C of the six
// h components, all in float with the reference's operation order (the
// sin table is computed on the host with the reference's float expression);
// bins stop below floor(0.8*numbins).
//
// Binning is deterministic: along k the bin index is non-decreasing, so each
// warp takes 32 consecutive k of one (i, j) row, combines equal bins with a
// segmented shuffle scan, and the segment tails add into that warp's own
// shared-memory histogram.  Warps, then CTAs, are combined in index order.
// Compiled with -fmad=false.
#include <cmath>
#include <mutex>
#include <vector>

#include "iegpu_internal.cuh"

namespace iegpu {

constexpr int kSpecWarps = 4;
constexpr int kSpecThreads = kSpecWarps * 32;

__device__ __forceinline__ int round_sqrt_int(int n) {
    // lround(sqrt(n)) for integer n >= 0 (never a tie)
    int b = (int)(sqrtf((float)n) + 0.5f);
    while (b * b + b < n) ++b;
    while (b > 0 && b * b - b >= n) --b;
    return b;
}

// Adds (key, value, count) from all lanes into the warp's histogram; keys are
// non-decreasing across valid lanes, invalid lanes carry unique negative keys.
__device__ __forceinline__ void warp_segment_add(int key, double v, int cnt, double* wbin, int* wcnt) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double ov = __shfl_up_sync(0xffffffffu, v, o);
        const int oc = __shfl_up_sync(0xffffffffu, cnt, o);
        const int ok = __shfl_up_sync(0xffffffffu, key, o);
        if (lane >= o && ok == key) { v += ov; cnt += oc; }
    }
    const int nk = __shfl_down_sync(0xffffffffu, key, 1);
    const bool tail = (lane == 31) || (nk != key);
    if (key >= 0 && tail) {
        wbin[key] += v;
        wcnt[key] += cnt;
    }
    __syncwarp();
}

template <typename C2>
__device__ __forceinline__ double mag2(C2 z) { return (double)z.x * (double)z.x + (double)z.y * (double)z.y; }

__global__ void __launch_bounds__(kSpecThreads) k_bin_scalar(const double2* __restrict__ c, const double2* __restrict__ ny,
                                                             int lgN, int nbins, double* part, int* cpart) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* wb = reinterpret_cast<double*>(smem_raw);
    int* wc = reinterpret_cast<int*>(wb + kSpecWarps * nbins);
    const int N = 1 << lgN, M2 = N >> 1;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = threadIdx.x; q < kSpecWarps * nbins; q += blockDim.x) { wb[q] = 0.0; wc[q] = 0; }
    __syncthreads();
    double* mybin = wb + w * nbins;
    int* mycnt = wc + w * nbins;
    const long long rows = (long long)N * N;
    for (long long r = (long long)blockIdx.x * kSpecWarps + w; r < rows; r += (long long)gridDim.x * kSpecWarps) {
        const int i = (int)(r >> lgN), j = (int)(r & (N - 1));
        const int px = (i <= M2 ? i : i - N), py = (j <= M2 ? j : j - N);
        const int pxy = px * px + py * py;
        for (int k0 = 1; k0 < M2; k0 += 32) {
            const int k = k0 + lane;
            int key = -1 - lane;
            double v = 0.0;
            if (k < M2) {
                const int bin = round_sqrt_int(pxy + k * k);
                if (bin < nbins) {
                    const double2 z = c[r * M2 + k];
                    const double fp2 = z.x * z.x + z.y * z.y;
                    v = 2.0 * fp2;
                    key = bin;
                }
            }
            warp_segment_add(key, v, key >= 0 ? 2 : 0, mybin, mycnt);
        }
        if (lane == 0) {
            const int b0 = round_sqrt_int(pxy);
            if (b0 < nbins) {
                const double2 z = c[r * M2];
                mybin[b0] += z.x * z.x + z.y * z.y;
                mycnt[b0] += 1;
            }
            const int b1 = round_sqrt_int(pxy + M2 * M2);
            if (b1 < nbins) {
                const double2 z = ny[r];
                mybin[b1] += z.x * z.x + z.y * z.y;
                mycnt[b1] += 1;
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        double s = 0.0;
        int n = 0;
        for (int q = 0; q < kSpecWarps; ++q) { s += wb[q * nbins + b]; n += wc[q * nbins + b]; }
        part[(long long)blockIdx.x * nbins + b] = s;
        cpart[(long long)blockIdx.x * nbins + b] = n;
    }
}

__global__ void k_bin_combine(const double* part, const int* cpart, int nblocks, int nbins, double* out, int* cout) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    double s = 0.0;
    int n = 0;
    for (int q = 0; q < nblocks; ++q) { s += part[(long long)q * nbins + b]; n += cpart[(long long)q * nbins + b]; }
    out[b] = s;
    cout[b] = n;
}

// ---- tensor (GW) spectrum -------------------------------------------------

struct GwArgs {
    const float2* c[6];
    const float2* ny[6];
    const float* ksin;   // (2/dx) sin(pi p/N), p = -N/2..N/2 stored at [p + N/2]
    double to_phys_d;
    int scale;           // 0: none, 1: (float)((double)x * to_phys)
    int imax;            // bins >= imax are dropped
};

__device__ __forceinline__ float gw_tt(const float (&Cr)[3][3], const float (&Ci)[3][3], float kx, float ky, float kz,
                                       float kt2) {
    const float inv = 1.0f / sqrtf(kt2);
    const float kh[3] = {kx * inv, ky * inv, kz * inv};
    float P[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.f : 0.f) - kh[a] * kh[b];
    float Ar[3][3], Ai[3][3], Tr = 0.f, Ti = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float r = 0.f, q = 0.f;
#pragma unroll
            for (int l = 0; l < 3; ++l)
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    const float pal = P[a][l], pbm = P[b][m];
                    r += pal * Cr[l][m] * pbm;
                    q += pal * Ci[l][m] * pbm;
                }
            Ar[a][b] = r;
            Ai[a][b] = q;
        }
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            Tr += P[l][m] * Cr[l][m];
            Ti += P[l][m] * Ci[l][m];
        }
    float fp2 = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float Xr = Ar[a][b] - 0.5f * P[a][b] * Tr;
            const float Xi = Ai[a][b] - 0.5f * P[a][b] * Ti;
            fp2 += Xr * Xr + Xi * Xi;
        }
    return fp2;
}

__device__ __forceinline__ void gw_load(const GwArgs& A, bool nyq, long long idx, float (&Cr)[3][3], float (&Ci)[3][3]) {
    // packed components: 0 xx, 1 yy, 2 zz, 3 xy, 4 xz, 5 yz (src/main.h:42-64)
    const int comp[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const float2 z = nyq ? A.ny[comp[l][m]][idx] : A.c[comp[l][m]][idx];
            float re = z.x, im = z.y;
            if (A.scale) {
                re = (float)((double)re * A.to_phys_d);
                im = (float)((double)im * A.to_phys_d);
            }
            Cr[l][m] = re;
            Ci[l][m] = im;
        }
}

__global__ void __launch_bounds__(kSpecThreads) k_bin_gw(GwArgs A, int lgN, int nbins, double* part, int* cpart) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* wb = reinterpret_cast<double*>(smem_raw);
    int* wc = reinterpret_cast<int*>(wb + kSpecWarps * nbins);
    const int N = 1 << lgN, M2 = N >> 1;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = threadIdx.x; q < kSpecWarps * nbins; q += blockDim.x) { wb[q] = 0.0; wc[q] = 0; }
    __syncthreads();
    double* mybin = wb + w * nbins;
    int* mycnt = wc + w * nbins;
    const long long rows = (long long)N * N;
    const float* ks = A.ksin + M2;  // ks[p] for p in [-M2+1, M2]
    for (long long r = (long long)blockIdx.x * kSpecWarps + w; r < rows; r += (long long)gridDim.x * kSpecWarps) {
        const int i = (int)(r >> lgN), j = (int)(r & (N - 1));
        const int px = (i <= M2 ? i : i - N), py = (j <= M2 ? j : j - N);
        const int pxy = px * px + py * py;
        const float kx = ks[px], ky = ks[py];
        for (int k0 = 1; k0 < M2; k0 += 32) {
            const int k = k0 + lane;
            int key = -1 - lane;
            double v = 0.0;
            if (k < M2) {
                const float kz = ks[k];
                const float kt2 = kx * kx + ky * ky + kz * kz;
                const int bin = (int)roundf(sqrtf((float)(pxy + k * k)));
                if (kt2 != 0.f && bin < A.imax) {
                    float Cr[3][3], Ci[3][3];
                    gw_load(A, false, r * M2 + k, Cr, Ci);
                    const float fp2 = gw_tt(Cr, Ci, kx, ky, kz, kt2);
                    v = (double)(2.f * fp2);
                    key = bin;
                }
            }
            warp_segment_add(key, v, key >= 0 ? 2 : 0, mybin, mycnt);
        }
        if (lane < 2) {
            // k = 0 (lane 0) and k = N/2 (lane 1); bins differ, lanes write in turn
            for (int t = 0; t < 2; ++t) {
                if (lane == t) {
                    const int pz = t ? M2 : 0;
                    const float kz = ks[pz];
                    const float kt2 = kx * kx + ky * ky + kz * kz;
                    const int bin = (int)roundf(sqrtf((float)(pxy + pz * pz)));
                    if (kt2 != 0.f && bin < A.imax) {
                        float Cr[3][3], Ci[3][3];
                        gw_load(A, t == 1, t ? r : r * M2, Cr, Ci);
                        const float fp2 = gw_tt(Cr, Ci, kx, ky, kz, kt2);
                        mybin[bin] += (double)fp2;
                        mycnt[bin] += 1;
                    }
                }
                __syncwarp(0x3u);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        double s = 0.0;
        int n = 0;
        for (int q = 0; q < kSpecWarps; ++q) { s += wb[q * nbins + b]; n += wc[q * nbins + b]; }
        part[(long long)blockIdx.x * nbins + b] = s;
        cpart[(long long)blockIdx.x * nbins + b] = n;
    }
}

// ---------------------------------------------------------------------------

static int finish_bins(iegpu_ctx* c, int nbins, int* counts, double* f2) {
    double* out = c->misc;
    int* cout = reinterpret_cast<int*>(c->misc + nbins);
    k_bin_combine<<<(nbins + 127) / 128, 128, 0, c->stream>>>(c->spec_part, c->spec_cnt, c->spec_blocks, nbins, out, cout);
    c->launches++;
    if (check_cuda(c, cudaMemcpyAsync(c->misc_h, c->misc, sizeof(double) * nbins + sizeof(int) * nbins,
                                      cudaMemcpyDeviceToHost, c->stream), "spectrum download"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "spectrum")) return IEGPU_ECUDA;
    const int* ch = reinterpret_cast<const int*>(c->misc_h + nbins);
    for (int b = 0; b < nbins; ++b) { f2[b] = c->misc_h[b]; counts[b] = ch[b]; }
    return IEGPU_OK;
}

int spectrum_bin_d(iegpu_ctx* c, const double* f, const double* fny, int* counts, double* f2, int nbins) {
    const size_t smem = (size_t)kSpecWarps * nbins * (sizeof(double) + sizeof(int));
    k_bin_scalar<<<c->spec_blocks, kSpecThreads, smem, c->stream>>>(reinterpret_cast<const double2*>(f),
                                                                     reinterpret_cast<const double2*>(fny), c->lg, nbins,
                                                                     c->spec_part, c->spec_cnt);
    c->launches++;
    return finish_bins(c, nbins, counts, f2);
}

// ---------------------------------------------------------------------------
// The forcing cutoff of spectraf(), src/output.cpp:330-401 (the same block
// closes spectraf_post_inflation, :1700-1765), on f and fd in k-space: every
// mode whose lattice momentum has |p| = sqrt(px^2 + py^2 + pz^2) (exact
// integers in double; IEEE square root) above high or below low is zeroed.
// One thread per complex element (i, j, kz), kz = 0 .. N/2 (kz = N/2 is the
// Nyquist plane ny[i][j]); each element is written by its own thread only.
// Interior modes 0 < kz < N/2 are zeroed as (+0, +0).  On the kz = 0 and
// Nyquist planes the reference walks one member of each conjugate pair
// ((i, j) with j > N/2, or i > N/2 on the rows j = 0, N/2), zeroes it and
// writes its partner (N - i, N - j) as the conjugate, so the partner holds
// (+0, -0); the four self-conjugate points (i, j in {0, N/2}) are zeroed as
// (+0, +0).  The partner's |p| equals the walked member's, so its thread
// decides alone.  Nothing is read: the kernel writes the zeroed modes only.
__global__ void k_forcing_cutoff(double2* __restrict__ f, double2* __restrict__ fny, double2* __restrict__ fd,
                                 double2* __restrict__ fdny, int N, double high, double low) {
    const int h = N >> 1;
    const size_t n = (size_t)N * N * (h + 1);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int kz = (int)(t % (size_t)(h + 1));
        const size_t ij = t / (size_t)(h + 1);
        const int j = (int)(ij % (size_t)N), i = (int)(ij / (size_t)N);
        const int px = i <= h ? i : i - N, py = j <= h ? j : j - N;
        const double pd = sqrt((double)(px * px + py * py + kz * kz));
        if (!(pd > high || pd < low)) continue;
        const bool plane = kz == 0 || kz == h;
        const bool walked = j > h || (i > h && (j == 0 || j == h));
        const bool self = (i == 0 || i == h) && (j == 0 || j == h);
        const double2 z = make_double2(0.0, (plane && !walked && !self) ? -0.0 : 0.0);
        if (kz == h) {
            fny[ij] = z;
            fdny[ij] = z;
        } else {
            const size_t e = ij * (size_t)h + kz;
            f[e] = z;
            fd[e] = z;
        }
    }
}

int forcing_cutoff(iegpu_ctx* c, double* f, double* fny, double* fd, double* fdny, double high, double low) {
    const int N = c->N;
    const size_t n = (size_t)N * N * (N / 2 + 1);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_forcing_cutoff<<<blocks, 256, 0, c->stream>>>(reinterpret_cast<double2*>(f), reinterpret_cast<double2*>(fny),
                                                    reinterpret_cast<double2*>(fd), reinterpret_cast<double2*>(fdny),
                                                    N, high, low);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "forcing cutoff") ? IEGPU_ECUDA : IEGPU_OK;
}

int gw_bin(iegpu_ctx* c, int which, double to_phys, int* counts, double* f2, int nbins) {
    const int N = c->N, M2 = N / 2;
    // kx table with the reference's float expression, src/output.cpp:493-495
    const float pi_f = (float)(2.0 * std::asin(1.0));
    const float dx_f = (float)(c->cfg.L / (double)N);
    std::vector<float> ks((size_t)N + 1);
    for (int p = -M2; p <= M2; ++p) ks[(size_t)(p + M2)] = (2.f / dx_f) * std::sin(pi_f * p / (float)N);
    // device copy lives in misc scratch after the bin outputs
    float* dks = reinterpret_cast<float*>(c->misc + 2 * (size_t)nbins + 8);
    if (check_cuda(c, cudaMemcpyAsync(dks, ks.data(), sizeof(float) * ks.size(), cudaMemcpyHostToDevice, c->stream), "ksin"))
        return IEGPU_ECUDA;
    GwArgs A{};
    for (int q = 0; q < 6; ++q) {
        A.c[q] = reinterpret_cast<const float2*>(which ? c->hd[q] : c->h[c->cur][q]);
        A.ny[q] = reinterpret_cast<const float2*>(which ? c->hdny[q] : c->hny[q]);
    }
    A.ksin = dks;
    A.to_phys_d = to_phys;
    A.scale = which ? 1 : 0;
    const int numbins = (int)(std::sqrt(3.0) * (N / 2)) + 1;
    A.imax = (int)std::floor(0.80 * numbins);
    const size_t smem = (size_t)kSpecWarps * nbins * (sizeof(double) + sizeof(int));
    k_bin_gw<<<c->spec_blocks, kSpecThreads, smem, c->stream>>>(A, c->lg, nbins, c->spec_part, c->spec_cnt);
    c->launches++;
    return finish_bins(c, nbins, counts, f2);
}

// ---------------------------------------------------------------------------
// GW spectra with the reference's float accumulators
// ---------------------------------------------------------------------------
//
// write_gw_spectrum_impl (src/output.cpp:478-612) adds each mode's float value
// to a float accumulator of its bin, in its loop order: rows (i, j) in order,
// in each row kz = 1 .. N/2-1 (2 fp2 each), then kz = 0 and kz = N/2 (fp2).
// Mode slot (i N + j)(N/2 + 1) + t holds kz = t + 1 for t < N/2 - 1, kz = 0 for
// t = N/2 - 1 and kz = N/2 for t = N/2.  The slots of each bin, in slot order,
// form one list (a stable counting sort on the host, once per context):
// k_gw_vals writes every mode's value to its place in its bin's list, and
// k_gw_serial adds each list in order, one warp per bin, in float as the
// reference does (and in double beside it, in another order).  Given the same
// h, the float sums are the reference's bit for bit.

__global__ void __launch_bounds__(kSpecThreads) k_gw_vals(GwArgs A, const int* __restrict__ pos,
                                                         float* __restrict__ vals, int lgN) {
    const int N = 1 << lgN, M2 = N >> 1, W = M2 + 1;
    const long long S = (long long)N * N * W;
    const float* ks = A.ksin + M2;
    for (long long sl = (long long)blockIdx.x * blockDim.x + threadIdx.x; sl < S;
         sl += (long long)gridDim.x * blockDim.x) {
        const int at = pos[sl];
        if (at < 0) continue;
        const long long r = sl / W;
        const int t = (int)(sl - r * W);
        const int i = (int)(r >> lgN), j = (int)(r & (N - 1));
        const int px = (i <= M2 ? i : i - N), py = (j <= M2 ? j : j - N);
        const float kx = ks[px], ky = ks[py];
        const bool interior = t < M2 - 1;
        const int pz = interior ? t + 1 : (t == M2 - 1 ? 0 : M2);
        const float kz = ks[pz];
        const float kt2 = kx * kx + ky * ky + kz * kz;
        float Cr[3][3], Ci[3][3];
        if (interior) gw_load(A, false, r * M2 + pz, Cr, Ci);
        else gw_load(A, pz != 0, pz ? r : r * M2, Cr, Ci);
        const float fp2 = gw_tt(Cr, Ci, kx, ky, kz, kt2);
        vals[at] = interior ? 2.f * fp2 : fp2;
    }
}

// One warp per bin: the lanes load 128 values at a time (the next 128 while
// the current ones are added), and every lane adds them in list order (the
// shuffles broadcast them), so the float sum is one chain in the reference's
// order.  The double sum (for full-precision output) is formed per chunk
// across the lanes and off that chain: the same values, another order.
__global__ void __launch_bounds__(32) k_gw_serial(const float* __restrict__ vals, const int* __restrict__ start,
                                                  float* __restrict__ f2f, double* __restrict__ f2d) {
    const int b = blockIdx.x, lane = threadIdx.x;
    const int t0 = start[b], t1 = start[b + 1];
    float sf = 0.f;
    double sd = 0.0;
    float v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int t = t0 + 4 * lane + q;
        v[q] = t < t1 ? vals[t] : 0.f;
    }
    for (int base = t0; base < t1; base += 128) {
        float vn[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int t = base + 128 + 4 * lane + q;
            vn[q] = t < t1 ? vals[t] : 0.f;
        }
        const int n = t1 - base < 128 ? t1 - base : 128;
        if (n == 128) {
#pragma unroll
            for (int l = 0; l < 32; ++l)
#pragma unroll
                for (int q = 0; q < 4; ++q) sf = __fadd_rn(sf, __shfl_sync(0xffffffffu, v[q], l));
        } else {
            for (int l = 0; l < 32; ++l)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float x = __shfl_sync(0xffffffffu, v[q], l);
                    if (4 * l + q < n) sf = __fadd_rn(sf, x);
                }
        }
        // lanes past the list hold 0, which adds nothing to the double sum
        double d = ((double)v[0] + (double)v[1]) + ((double)v[2] + (double)v[3]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        sd += d;
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = vn[q];
    }
    if (lane == 0) {
        f2f[b] = sf;
        f2d[b] = sd;
    }
}

// The bin lists of the reference's loop order for this lattice size.
static int gw_order_init(iegpu_ctx* c, int nbins) {
    if (c->gw_pos) return IEGPU_OK;
    const int N = c->N, M2 = N / 2, W = M2 + 1;
    const int imax = (int)std::floor(0.80 * nbins);
    const size_t S = (size_t)N * N * W;
    std::vector<int> bin(S), cnt((size_t)nbins + 1, 0);
    c->gw_counts.assign((size_t)nbins, 0);
    for (int i = 0; i < N; ++i) {
        const int px = i <= M2 ? i : i - N;
        for (int j = 0; j < N; ++j) {
            const int py = j <= M2 ? j : j - N;
            const size_t row = ((size_t)i * N + j) * W;
            for (int t = 0; t < W; ++t) {
                const int pz = t < M2 - 1 ? t + 1 : (t == M2 - 1 ? 0 : M2);
                const int sq = px * px + py * py + pz * pz;
                // kt2 = 0 only at the k = 0 mode, which the reference skips
                int b = sq == 0 ? -1 : (int)lroundf(std::sqrt((float)sq));
                if (b >= imax) b = -1;
                bin[row + t] = b;
                if (b >= 0) {
                    ++cnt[(size_t)b + 1];
                    c->gw_counts[(size_t)b] += t < M2 - 1 ? 2 : 1;
                }
            }
        }
    }
    for (int b = 0; b < nbins; ++b) cnt[(size_t)b + 1] += cnt[(size_t)b];
    const std::vector<int> start(cnt);
    std::vector<int> pos(S);
    for (size_t sl = 0; sl < S; ++sl) pos[sl] = bin[sl] < 0 ? -1 : cnt[(size_t)bin[sl]]++;
    const size_t total = (size_t)start[(size_t)nbins];
    // published only when every buffer is in place (a failed call leaves none behind)
    int *dpos = nullptr, *dstart = nullptr;
    float *dvals = nullptr, *df2f = nullptr;
    double* df2d = nullptr;
    if (check_cuda(c, cudaMalloc(&dpos, sizeof(int) * S), "gw order") ||
        check_cuda(c, cudaMalloc(&dstart, sizeof(int) * start.size()), "gw order") ||
        check_cuda(c, cudaMalloc(&dvals, sizeof(float) * (total > 0 ? total : 1)), "gw order") ||
        check_cuda(c, cudaMalloc(&df2f, sizeof(float) * nbins), "gw order") ||
        check_cuda(c, cudaMalloc(&df2d, sizeof(double) * nbins), "gw order") ||
        check_cuda(c, cudaMemcpy(dpos, pos.data(), sizeof(int) * S, cudaMemcpyHostToDevice), "gw order") ||
        check_cuda(c, cudaMemcpy(dstart, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice),
                   "gw order")) {
        cudaFree(dpos);
        cudaFree(dstart);
        cudaFree(dvals);
        cudaFree(df2f);
        cudaFree(df2d);
        c->gw_counts.clear();
        return IEGPU_ENOMEM;
    }
    c->gw_pos = dpos;
    c->gw_start = dstart;
    c->gw_vals = dvals;
    c->gw_f2f = df2f;
    c->gw_f2d = df2d;
    return IEGPU_OK;
}

int gw_bin_ref(iegpu_ctx* c, int which, double to_phys, int* counts, float* f2, double* f2d, int nbins) {
    const int N = c->N, M2 = N / 2;
    if (int rc = gw_order_init(c, nbins)) return rc;
    const float pi_f = (float)(2.0 * std::asin(1.0));
    const float dx_f = (float)(c->cfg.L / (double)N);
    std::vector<float> ks((size_t)N + 1);
    for (int p = -M2; p <= M2; ++p) ks[(size_t)(p + M2)] = (2.f / dx_f) * std::sin(pi_f * p / (float)N);
    float* dks = reinterpret_cast<float*>(c->misc + 2 * (size_t)nbins + 8);
    if (check_cuda(c, cudaMemcpyAsync(dks, ks.data(), sizeof(float) * ks.size(), cudaMemcpyHostToDevice, c->stream), "ksin"))
        return IEGPU_ECUDA;
    GwArgs A{};
    for (int q = 0; q < 6; ++q) {
        A.c[q] = reinterpret_cast<const float2*>(which ? c->hd[q] : c->h[c->cur][q]);
        A.ny[q] = reinterpret_cast<const float2*>(which ? c->hdny[q] : c->hny[q]);
    }
    A.ksin = dks;
    A.to_phys_d = to_phys;
    A.scale = which ? 1 : 0;
    A.imax = (int)std::floor(0.80 * nbins);
    k_gw_vals<<<c->sms * 8, kSpecThreads, 0, c->stream>>>(A, c->gw_pos, c->gw_vals, c->lg);
    k_gw_serial<<<nbins, 32, 0, c->stream>>>(c->gw_vals, c->gw_start, c->gw_f2f, c->gw_f2d);
    c->launches += 2;
    std::vector<double> hd((size_t)nbins);
    if (check_cuda(c, cudaMemcpyAsync(f2, c->gw_f2f, sizeof(float) * nbins, cudaMemcpyDeviceToHost, c->stream),
                   "gw spectrum download") ||
        check_cuda(c, cudaMemcpyAsync(hd.data(), c->gw_f2d, sizeof(double) * nbins, cudaMemcpyDeviceToHost, c->stream),
                   "gw spectrum download"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "gw spectrum")) return IEGPU_ECUDA;
    for (int b = 0; b < nbins; ++b) {
        counts[b] = c->gw_counts[(size_t)b];
        if (f2d) f2d[b] = hd[(size_t)b];
    }
    return IEGPU_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free shell binning
// ---------------------------------------------------------------------------
//
// For callers that cannot allocate device memory, themselves or through
// this library: a plugin whose host framework owns all device memory through
// its own caching allocator and forbids direct cudaMalloc, or a process whose
// fixed memory budget is already spent on the lattice.  The per-CTA partial
// sums live in one fixed file-scope array instead of context scratch.  The array is sized for N <= kNoAllocMaxN and a grid of
// kNoAllocBlocks CTAs: kNoAllocBlocks * kNoAllocMaxBins * (8 + 4) bytes
// = 681,984 bytes, held by every GPU that loads the library until exit.

constexpr int kNoAllocBlocks = 128;
constexpr int kNoAllocMaxN = 512;
constexpr int kNoAllocMaxBins = (int)(1.73205 * (kNoAllocMaxN / 2)) + 1;
constexpr size_t kNoAllocF2Bytes = sizeof(double) * kNoAllocBlocks * kNoAllocMaxBins;
constexpr size_t kNoAllocBytes = kNoAllocF2Bytes + sizeof(int) * kNoAllocBlocks * kNoAllocMaxBins;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol is only a stand-in, so the address is fetched once per device
// with that device current and cached.
static int noalloc_scratch(unsigned char** out) {
    static std::mutex mu;
    static unsigned char* addr[128] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
        cudaGetLastError();
        return IEGPU_ECUDA;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return IEGPU_ECUDA;
        }
        addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = addr[dev];
    return IEGPU_OK;
}

}  // namespace iegpu

extern "C" int iegpu_shell_spectrum_noalloc(const double* modes, const double* nyquist, int N, int* counts,
                                            double* f2, void* stream) {
    using namespace iegpu;
    if (!modes || !nyquist || !counts || !f2) return IEGPU_EINVAL;
    if (N < 8 || (N & (N - 1))) return IEGPU_EINVAL;
    if (N > kNoAllocMaxN) return IEGPU_ETOOBIG;
    unsigned char* scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    const int nbins = iegpu_numbins(N);
    double* part = reinterpret_cast<double*>(scratch);
    int* cpart = reinterpret_cast<int*>(scratch + kNoAllocF2Bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every launch rewrites all nbins partials of each of its CTAs, so the
    // contents left by an earlier call are never read
    const size_t smem = (size_t)kSpecWarps * nbins * (sizeof(double) + sizeof(int));
    k_bin_scalar<<<kNoAllocBlocks, kSpecThreads, smem, st>>>(reinterpret_cast<const double2*>(modes),
                                                             reinterpret_cast<const double2*>(nyquist), lg, nbins,
                                                             part, cpart);
    k_bin_combine<<<(nbins + 127) / 128, 128, 0, st>>>(part, cpart, kNoAllocBlocks, nbins, f2, counts);
    return cudaGetLastError() == cudaSuccess ? IEGPU_OK : IEGPU_ECUDA;
}
