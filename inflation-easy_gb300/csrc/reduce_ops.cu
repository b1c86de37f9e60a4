// reduce_ops.cu -- lattice reductions and element-wise updates used by the
// diagnostics and deltaN output of src/output.cpp.
//
//   field_means        meansvars sums (src/output.cpp:235-240)
//   field_sum          build_deltaN_linear mean (src/output.cpp:156-164)
//   field_histogram    histograms / histogramsN (src/output.cpp:1070-1277):
//                      exact min/max, then integer bin counts
//   get_phiref         first extremal site in loop order (src/evolution.cpp:1271-1288)
//   saveN_mean         the float accumulator of saveN (src/output.cpp:1527-1537),
//                      a serial recurrence, replayed on the host in site order
//                      (float_mean_serial)
//   field_add / field_zero_above   element-wise updates
// Sums are formed in a fixed order (block trees, then CTA partials summed on
// the host in CTA order).  Compiled with -fmad=false.
#include <cfloat>
#include <cmath>
#include <vector>

#include "iegpu_internal.cuh"
#include "pot.cuh"
#include "reduce.cuh"

namespace iegpu {

__global__ void __launch_bounds__(kThreads) k_means(const double* __restrict__ f, const double* __restrict__ fd,
                                                    long long gs, double* part) {
    double v[3] = {0.0, 0.0, 0.0};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const double x = f[id];
        v[0] += x;
        v[1] += fd[id];
        v[2] += x * x;
    }
    block_sum<3>(v);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = v[0];
        part[3 * blockIdx.x + 1] = v[1];
        part[3 * blockIdx.x + 2] = v[2];
    }
}

__global__ void __launch_bounds__(kThreads) k_sum(const double* __restrict__ x, long long gs, double* part) {
    double v[1] = {0.0};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads)
        v[0] += x[id];
    block_sum<1>(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
}

__global__ void __launch_bounds__(kThreads) k_minmax(const double* __restrict__ x, long long gs, double* part) {
    __shared__ double smin[kThreads], smax[kThreads];
    double mn = x[0], mx = x[0];
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const double v = x[id];
        mn = (v < mn ? v : mn);
        mx = (v > mx ? v : mx);
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double a = smin[threadIdx.x + o], b = smax[threadIdx.x + o];
            if (a < smin[threadIdx.x]) smin[threadIdx.x] = a;
            if (b > smax[threadIdx.x]) smax[threadIdx.x] = b;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = smin[0];
        part[2 * blockIdx.x + 1] = smax[0];
    }
}

// binnum = (int)((x - bmin)/df); the maximum goes to the top bin
__global__ void __launch_bounds__(kThreads) k_hist(const double* __restrict__ x, long long gs, double bmin, double bmax,
                                                   double df, int nbins, unsigned long long* counts) {
    extern __shared__ unsigned int sh_cnt[];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh_cnt[b] = 0;
    __syncthreads();
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const double v = x[id];
        int bin = (int)((v - bmin) / df);
        if (v == bmax) bin = nbins - 1;
        if (bin >= 0 && bin < nbins) atomicAdd(&sh_cnt[bin], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
        if (sh_cnt[b]) atomicAdd(&counts[b], (unsigned long long)sh_cnt[b]);
}

// Extremal site: crit > 0 smallest |f|, crit < 0 largest |f|, crit == 0
// smallest V(f); ties go to the lowest index (the reference keeps the first).
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_phiref(const double* __restrict__ f, long long gs, int crit, PotDev P,
                                                     double* pval, long long* pidx) {
    __shared__ double sv[kThreads];
    __shared__ long long si[kThreads];
    double best = 0.0;
    long long bi = -1;
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const double x = f[id];
        double key;
        if (crit > 0) key = fabs(x);
        else if (crit < 0) key = -fabs(x);
        else {
            bool o;
            key = V_exact<TABLE>(P, x, &o);
        }
        if (bi < 0 || key < best) { best = key; bi = id; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const long long j = si[threadIdx.x + o];
            const double v = sv[threadIdx.x + o];
            const long long i0 = si[threadIdx.x];
            if (j >= 0 && (i0 < 0 || v < sv[threadIdx.x] || (v == sv[threadIdx.x] && j < i0))) {
                sv[threadIdx.x] = v;
                si[threadIdx.x] = j;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pval[blockIdx.x] = sv[0];
        pidx[blockIdx.x] = si[0];
    }
}

__global__ void k_add(double* x, long long gs, double v) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < gs) x[id] = x[id] + v;
}

__global__ void k_zero_above(double* x, long long gs, double thr) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < gs && x[id] > thr) x[id] = 0;
}

// ---------------------------------------------------------------------------

static int fetch(iegpu_ctx* c, void* dst, const void* src, size_t bytes, const char* what) {
    if (check_cuda(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream), what)) return IEGPU_ECUDA;
    return sync_and_check(c, what);
}

int field_means(iegpu_ctx* c, double out[3]) {
    const int g = c->red_grid;
    k_means<<<g, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, (long long)c->gs, c->part);
    c->launches++;
    std::vector<double> h((size_t)g * 3);
    if (fetch(c, h.data(), c->part, sizeof(double) * h.size(), "means")) return IEGPU_ECUDA;
    out[0] = out[1] = out[2] = 0.0;
    for (int b = 0; b < g; ++b) { out[0] += h[3 * b]; out[1] += h[3 * b + 1]; out[2] += h[3 * b + 2]; }
    return IEGPU_OK;
}

int field_sum(iegpu_ctx* c, int field, double* out) {
    double* x = dfield(c, field);
    if (!x) return set_error(c, IEGPU_EINVAL, "field %d cannot be summed", field);
    const int g = c->red_grid;
    k_sum<<<g, kThreads, 0, c->stream>>>(x, (long long)c->gs, c->part);
    c->launches++;
    std::vector<double> h((size_t)g);
    if (fetch(c, h.data(), c->part, sizeof(double) * h.size(), "sum")) return IEGPU_ECUDA;
    double s = 0.0;
    for (int b = 0; b < g; ++b) s += h[b];
    *out = s;
    return IEGPU_OK;
}

int field_histogram(iegpu_ctx* c, int field, int nbins, double* bmin_out, double* df_out, double* freq) {
    double* x = dfield(c, field);
    if (!x || nbins <= 0) return set_error(c, IEGPU_EINVAL, "bad histogram request (field %d, nbins %d)", field, nbins);
    const int g = c->red_grid;
    k_minmax<<<g, kThreads, 0, c->stream>>>(x, (long long)c->gs, c->part);
    c->launches++;
    std::vector<double> h((size_t)g * 2);
    if (fetch(c, h.data(), c->part, sizeof(double) * h.size(), "minmax")) return IEGPU_ECUDA;
    double bmin = h[0], bmax = h[1];
    for (int b = 0; b < g; ++b) {
        bmin = (h[2 * b] < bmin ? h[2 * b] : bmin);
        bmax = (h[2 * b + 1] > bmax ? h[2 * b + 1] : bmax);
    }
    double df = (bmax - bmin) / (double)nbins;
    if (!std::isfinite(df) || df <= 0.0) df = 1.0;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c->spec_part);
    if (check_cuda(c, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * nbins, c->stream), "hist memset")) return IEGPU_ECUDA;
    k_hist<<<g, kThreads, sizeof(unsigned) * nbins, c->stream>>>(x, (long long)c->gs, bmin, bmax, df, nbins, cnt);
    c->launches++;
    std::vector<unsigned long long> hc((size_t)nbins);
    if (fetch(c, hc.data(), cnt, sizeof(unsigned long long) * nbins, "histogram")) return IEGPU_ECUDA;
    unsigned long long numpts = 0;
    for (int b = 0; b < nbins; ++b) numpts += hc[b];
    const int np = numpts == 0 ? 1 : (int)numpts;
    for (int b = 0; b < nbins; ++b) freq[b] = (double)hc[b] / (double)np;
    *bmin_out = bmin;
    *df_out = df;
    return IEGPU_OK;
}

int get_phiref(iegpu_ctx* c, double* out) {
    const int g = c->red_grid;
    double* pval = c->part;
    long long* pidx = reinterpret_cast<long long*>(c->part + g);
    if (c->pot.table) k_phiref<true><<<g, kThreads, 0, c->stream>>>(c->f[c->cur], (long long)c->gs, c->cfg.criterion, c->pot, pval, pidx);
    else k_phiref<false><<<g, kThreads, 0, c->stream>>>(c->f[c->cur], (long long)c->gs, c->cfg.criterion, c->pot, pval, pidx);
    c->launches++;
    std::vector<double> hv((size_t)g);
    std::vector<long long> hi((size_t)g);
    if (fetch(c, hv.data(), pval, sizeof(double) * g, "phiref")) return IEGPU_ECUDA;
    if (fetch(c, hi.data(), pidx, sizeof(long long) * g, "phiref")) return IEGPU_ECUDA;
    double best = 0.0;
    long long bi = -1;
    for (int b = 0; b < g; ++b) {
        if (hi[b] < 0) continue;
        if (bi < 0 || hv[b] < best || (hv[b] == best && hi[b] < bi)) { best = hv[b]; bi = hi[b]; }
    }
    double v;
    if (fetch(c, &v, c->f[c->cur] + bi, sizeof(double), "phiref value")) return IEGPU_ECUDA;
    *out = v;
    return IEGPU_OK;
}

int saveN_mean(iegpu_ctx* c, double cutoff, float* out) {
    std::vector<double> x(c->gs);
    if (fetch(c, x.data(), c->dn, sizeof(double) * c->gs, "saveN mean")) return IEGPU_ECUDA;
    *out = float_mean_serial(x.data(), (long long)c->gs, cutoff);
    return IEGPU_OK;
}

int field_add(iegpu_ctx* c, int field, double v) {
    double* x = dfield(c, field);
    if (!x) return set_error(c, IEGPU_EINVAL, "field %d cannot be shifted", field);
    k_add<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(x, (long long)c->gs, v);
    c->launches++;
    return sync_and_check(c, "add");
}

int field_zero_above(iegpu_ctx* c, int field, double thr) {
    double* x = dfield(c, field);
    if (!x) return set_error(c, IEGPU_EINVAL, "field %d cannot be clipped", field);
    k_zero_above<<<(unsigned)((c->gs + 255) / 256), 256, 0, c->stream>>>(x, (long long)c->gs, thr);
    c->launches++;
    return sync_and_check(c, "zero_above");
}

}  // namespace iegpu
