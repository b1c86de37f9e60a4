// ensemble_dn.cu -- the deltaN stage of an ensemble and its zeta statistics.
//
// Per site, the same FP64 arithmetic as the one-lattice deltaN stage
// (src/evolution.cpp:1004-1037, src/initialize.cpp:219-232, compiled with
// -fmad=false), over the concatenated lattices with per-lattice a, phiref and
// V(phiref).  One difference, for speed: a site whose field has reached the
// end surface (the criterion is false) no longer changes f or deltaN, so the
// integration of that site stops there and its fd is left as it was at that
// step (the reference keeps integrating fd, which no output of saveN reads).
// Results per lattice follow saveN (src/output.cpp:1522-1560): the float mean
// Nmean of the deltaN <= Nend - dN sites and zeta = deltaN - Nmean.
//
// Ensemble statistics: the pooled one-point zeta histogram of the lattices of
// one size, over +-nsigma pooled standard deviations, and per-lattice zeta
// power spectra (spectraN) formed on the one-lattice contexts of each size.
#include <cmath>
#include <vector>

#include <thread>

#include "ensemble.cuh"
#include "pot.cuh"
#include "reduce.cuh"

namespace iegpu {

struct EnsDn {
    const EnsLat* lat;
    int count;
    double* f;
    double* fd;
    double* dn;
    PotDev P;
    DevCtl* err;
};

__device__ __forceinline__ int block_lattice(const EnsLat* lat, int count) {
    __shared__ int b_s;
    if (threadIdx.x == 0) b_s = ens_lattice_of(lat, count, (long long)blockIdx.x * 256);
    __syncthreads();
    return b_s;
}

// phi = phibar + dphi, phi' = pibar + dpi (as k_split_materialize)
__global__ void __launch_bounds__(256) k_ens_materialize(const float* __restrict__ x0, const float* __restrict__ x1,
                                                         const float* __restrict__ p0, const float* __restrict__ p1,
                                                         const int* __restrict__ cur, const SplitCtl* __restrict__ ctl,
                                                         EnsDn A) {
    const int b = block_lattice(A.lat, A.count);
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    const int c = cur[b] & 1;
    A.f[id] = ctl[b].phibar + (double)(c ? x1 : x0)[id];
    A.fd[id] = ctl[b].pibar + (double)(c ? p1 : p0)[id];
}

// initializeN(), src/initialize.cpp:219-232, apow[b] = a_b^(s-1)
template <bool TABLE>
__global__ void __launch_bounds__(256) k_ens_initN(EnsDn A, const double* __restrict__ apow) {
    const int b = block_lattice(A.lat, A.count);
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    bool oor;
    const double H_lat = sqrt(V_exact<TABLE>(A.P, A.f[id], &oor) / 3.0);
    if (TABLE && oor) flag_error(A.err, IEGPU_ERANGE, A.f[id]);
    A.fd[id] = A.fd[id] * apow[b] / H_lat;
    A.dn[id] = 0.0;
}

// evolve_derivsN + evolve_fieldsN for nsteps (src/evolution.cpp:1004-1037),
// per lattice phiref[b] and Vref[b]; stops at a site once it has ended.
template <bool TABLE, int CRIT>
__global__ void __launch_bounds__(256) k_ens_deltaN(EnsDn A, const double* __restrict__ phiref,
                                                    const double* __restrict__ Vref, double d, int nsteps,
                                                    int do_derivs, int do_fields) {
    const int b = block_lattice(A.lat, A.count);
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    double x = A.f[id], v = A.fd[id], n = A.dn[id];
    const double aref = fabs(phiref[b]), vref = Vref[b];
    bool oor = false, bad = false;
    auto active = [&](double y) {
        if (CRIT > 0) return fabs(y) > aref;
        if (CRIT < 0) return fabs(y) < aref;
        bool o2;
        const bool r = V_exact<TABLE>(A.P, y, &o2) > vref;
        bad |= o2;
        return r;
    };
    // an ended site changes neither f nor deltaN again
    if (do_fields && do_derivs && !active(x)) {
        if (bad) flag_error(A.err, IEGPU_ERANGE, x);
        return;
    }
    int l = 1;
    if (TABLE) {
        l = table_bracket(A.P, x, &oor);
        bad |= oor;
    }
    for (int s = 0; s < nsteps; ++s) {
        if (do_derivs) {
            double ratio;
            if (TABLE) {
                l = table_walk(A.P, x, l, &oor);
                bad |= oor;
                const double pot = table_interp(A.P, A.P.V, A.P.dyV, x, l);
                const double der = table_interp(A.P, A.P.dV, A.P.dydV, x, l);
                ratio = der / pot;
            } else {
                const double pot = div_exact(A.P.V0 * (1.0 - A.P.c1 * (x * x)), A.P.divB2);
                const double der = div_exact(A.P.c2 * x, A.P.divB2);
                ratio = der / pot;
            }
            v = v + d * (-(3.0 - 0.5 * (v * v)) * (v + ratio));
        }
        if (do_fields) {
            if (active(x)) {
                n = n + d;
                x = x + d * v;
            } else if (do_derivs) {
                break;
            }
        }
    }
    if (bad) flag_error(A.err, IEGPU_ERANGE, x);
    A.f[id] = x;
    A.fd[id] = v;
    A.dn[id] = n;
}

// get_phiref per lattice (src/evolution.cpp:1271-1288): the first site in
// loop order with the smallest key; slot s of S CTAs per lattice.
template <bool TABLE>
__global__ void __launch_bounds__(256) k_ens_phiref(EnsDn A, int crit, int S, double* pval, long long* pidx) {
    __shared__ double sv[256];
    __shared__ long long si[256];
    const int b = blockIdx.x / S, s = blockIdx.x - b * S;
    const EnsLat& L = A.lat[b];
    const long long gs = 1LL << (3 * L.lg);
    const double* f = A.f + L.off;
    double best = 0.0;
    long long bi = -1;
    for (long long id = (long long)s * 256 + threadIdx.x; id < gs; id += (long long)S * 256) {
        const double x = f[id];
        double key;
        if (crit > 0) key = fabs(x);
        else if (crit < 0) key = -fabs(x);
        else {
            bool o;
            key = V_exact<TABLE>(A.P, x, &o);
        }
        if (bi < 0 || key < best) { best = key; bi = id; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
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

// Combines the S slots of each lattice (ties to the lowest index) and reads
// the field value there.
__global__ void k_ens_phiref_pick(EnsDn A, int S, const double* pval, const long long* pidx, double* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= A.count) return;
    double best = 0.0;
    long long bi = -1;
    for (int s = 0; s < S; ++s) {
        const long long j = pidx[b * S + s];
        const double v = pval[b * S + s];
        if (j < 0) continue;
        if (bi < 0 || v < best || (v == best && j < bi)) { best = v; bi = j; }
    }
    out[b] = A.f[A.lat[b].off + bi];
}

// zeta = deltaN - Nmean (deltaN[idx] -= Nmean, a float promoted to double)
__global__ void __launch_bounds__(256) k_ens_shift(EnsDn A, const float* __restrict__ nmean) {
    const int b = block_lattice(A.lat, A.count);
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    A.dn[id] = A.dn[id] + (-(double)nmean[b]);
}

// Block sums of zeta and zeta^2 over the lattices of size N (N = 0: all);
// one partial pair per block, zero for blocks of other sizes.
__global__ void __launch_bounds__(256) k_ens_zeta_moments(EnsDn A, int lgsel, double* part) {
    const int b = block_lattice(A.lat, A.count);
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (lgsel == 0 || A.lat[b].lg == lgsel) {
        const double z = A.dn[id];
        v[0] = z;
        v[1] = z * z;
    }
    block_sum<2>(v);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = v[0];
        part[2 * blockIdx.x + 1] = v[1];
    }
}

// bin = floor((zeta - lo) / width); below and above the range counted apart
__global__ void __launch_bounds__(256) k_ens_zeta_hist(EnsDn A, int lgsel, double lo, double width, int nbins,
                                                       unsigned long long* counts) {
    extern __shared__ unsigned int sh[];
    for (int q = threadIdx.x; q < nbins + 2; q += blockDim.x) sh[q] = 0;
    const int b = block_lattice(A.lat, A.count);   // synchronises the block
    const long long id = (long long)blockIdx.x * 256 + threadIdx.x;
    if (lgsel == 0 || A.lat[b].lg == lgsel) {
        const double u = (A.dn[id] - lo) / width;
        int q;
        if (!(u >= 0.0)) q = nbins;                 // below (or NaN)
        else if (u >= (double)nbins) q = nbins + 1; // above
        else q = (int)u;
        atomicAdd(&sh[q], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nbins + 2; q += blockDim.x)
        if (sh[q]) atomicAdd(&counts[q], (unsigned long long)sh[q]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static EnsDn ens_dn(const iegpu_ens* e) {
    EnsDn A;
    A.lat = e->lat;
    A.count = e->count;
    A.f = e->f;
    A.fd = e->fd;
    A.dn = e->dn;
    A.P = e->helper[0]->pot;
    A.err = e->dctl;
    return A;
}

static unsigned ens_blocks(const iegpu_ens* e) { return (unsigned)(e->total / 256); }

static int ens_dsync(iegpu_ens* e, const char* what) {
    if (int rc = ens_cuda(e, cudaGetLastError(), what)) return rc;
    return ens_cuda(e, cudaStreamSynchronize(e->stream), what);
}

static int ens_put(iegpu_ens* e, double* dst, const double* src_h, size_t n, const char* what) {
    for (size_t q = 0; q < n; ++q) e->dscr_h[q] = src_h[q];
    return ens_cuda(e, cudaMemcpyAsync(dst, e->dscr_h, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream), what);
}

static int ens_check_error(iegpu_ens* e) {
    DevCtl h;
    if (int rc = ens_cuda(e, cudaMemcpyAsync(&h, e->dctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, e->stream), "error word"))
        return rc;
    if (int rc = ens_dsync(e, "deltaN")) return rc;
    if (h.error == IEGPU_ERANGE) {
        const iegpu_ctx* c = e->helper[0];
        return ens_error(e, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n",
                         h.errval, c->htab_x.empty() ? 0.0 : c->htab_x.back(), c->htab_x.empty() ? 0.0 : c->htab_x.front());
    }
    return IEGPU_OK;
}

int ens_materialize(iegpu_ens* e) {
    k_ens_materialize<<<ens_blocks(e), 256, 0, e->stream>>>(e->x[0], e->x[1], e->p[0], e->p[1], e->cur, e->ctl, ens_dn(e));
    e->launches++;
    return ens_cuda(e, cudaGetLastError(), "materialize");
}

int ens_initN(iegpu_ens* e, const double* apow_h) {
    if (int rc = ens_put(e, e->dscr, apow_h, (size_t)e->count, "initializeN")) return rc;
    const EnsDn A = ens_dn(e);
    if (A.P.table) k_ens_initN<true><<<ens_blocks(e), 256, 0, e->stream>>>(A, e->dscr);
    else k_ens_initN<false><<<ens_blocks(e), 256, 0, e->stream>>>(A, e->dscr);
    e->launches++;
    return ens_dsync(e, "initializeN");   // the scalar buffer is reused by the next call
}

int ens_deltaN_steps(iegpu_ens* e, double d, int nsteps, const double* phiref_h, int do_derivs, int do_fields) {
    if (nsteps <= 0) return IEGPU_OK;
    const int n = e->count;
    std::vector<double> vals(2 * (size_t)n);
    for (int b = 0; b < n; ++b) {
        vals[(size_t)b] = phiref_h[b];
        // potential(phiref) for the generic criterion, src/evolution.cpp:1028
        vals[(size_t)(n + b)] = e->cfg.criterion == 0 ? host_potential(e->helper[0], phiref_h[b]) : 0.0;
    }
    if (int rc = ens_put(e, e->dscr, vals.data(), vals.size(), "deltaN")) return rc;
    const EnsDn A = ens_dn(e);
    const int crit = e->cfg.criterion;
    const int chunk = 2000;   // keeps each launch short
    for (int s0 = 0; s0 < nsteps; s0 += chunk) {
        const int ns = (nsteps - s0) < chunk ? (nsteps - s0) : chunk;
#define IEGPU_ENS_DN(TAB, CR) \
    k_ens_deltaN<TAB, CR><<<ens_blocks(e), 256, 0, e->stream>>>(A, e->dscr, e->dscr + n, d, ns, do_derivs, do_fields)
        if (A.P.table) {
            if (crit > 0) IEGPU_ENS_DN(true, 1); else if (crit < 0) IEGPU_ENS_DN(true, -1); else IEGPU_ENS_DN(true, 0);
        } else {
            if (crit > 0) IEGPU_ENS_DN(false, 1); else if (crit < 0) IEGPU_ENS_DN(false, -1); else IEGPU_ENS_DN(false, 0);
        }
#undef IEGPU_ENS_DN
        e->launches++;
    }
    return ens_dsync(e, "deltaN steps");
}

int ens_phiref(iegpu_ens* e, double* phiref_h) {
    int S = 64;
    for (int b = 0; b < e->count; ++b) {
        const long long gs = (long long)e->N[(size_t)b] * e->N[(size_t)b] * e->N[(size_t)b];
        if (gs / 256 < S) S = (int)(gs / 256);
    }
    const size_t need = (size_t)e->count * S * 2 + (size_t)e->count;
    if (need > e->red_cap) {
        if (int rc = ens_dsync(e, "phiref")) return rc;
        if (e->red) cudaFree(e->red);
        e->red = nullptr;
        e->red_cap = 0;
        if (int rc = ens_cuda(e, cudaMalloc(&e->red, sizeof(double) * need), "phiref scratch")) return rc;
        e->red_cap = need;
    }
    double* pval = e->red;
    long long* pidx = reinterpret_cast<long long*>(e->red + (size_t)e->count * S);
    double* out = e->red + (size_t)e->count * S * 2;
    const EnsDn A = ens_dn(e);
    if (A.P.table) k_ens_phiref<true><<<e->count * S, 256, 0, e->stream>>>(A, e->cfg.criterion, S, pval, pidx);
    else k_ens_phiref<false><<<e->count * S, 256, 0, e->stream>>>(A, e->cfg.criterion, S, pval, pidx);
    k_ens_phiref_pick<<<(e->count + 127) / 128, 128, 0, e->stream>>>(A, S, pval, pidx, out);
    e->launches += 2;
    if (int rc = ens_cuda(e, cudaMemcpyAsync(e->dscr_h, out, sizeof(double) * (size_t)e->count, cudaMemcpyDeviceToHost,
                                             e->stream), "phiref"))
        return rc;
    if (int rc = ens_dsync(e, "phiref")) return rc;
    for (int b = 0; b < e->count; ++b) phiref_h[b] = e->dscr_h[b];
    return IEGPU_OK;
}

// saveN's float accumulator of every lattice (float_mean_serial): the maps
// are copied down and the lattices' recurrences run on host threads.
int ens_saveN_mean(iegpu_ens* e, double cutoff, float* nmean_h) {
    const long long total = e->lat_h.back().off + (1LL << (3 * e->lat_h.back().lg));
    std::vector<double> x((size_t)total);
    if (int rc = ens_cuda(e, cudaMemcpyAsync(x.data(), e->dn, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost,
                                             e->stream), "saveN mean"))
        return rc;
    if (int rc = ens_dsync(e, "saveN mean")) return rc;
    const int count = e->count;
    unsigned nt = std::thread::hardware_concurrency();
    if (nt < 1) nt = 1;
    if (nt > 16) nt = 16;
    if ((int)nt > count) nt = (unsigned)count;
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
            for (int b = (int)t; b < count; b += (int)nt) {
                const EnsLat& L = e->lat_h[(size_t)b];
                nmean_h[b] = float_mean_serial(x.data() + L.off, 1LL << (3 * L.lg), cutoff);
            }
        });
    for (auto& th : pool) th.join();
    return IEGPU_OK;
}

int ens_shift(iegpu_ens* e, const float* nmean_h) {
    float* d = reinterpret_cast<float*>(e->iscr);
    if (int rc = ens_cuda(e, cudaMemcpyAsync(d, nmean_h, sizeof(float) * (size_t)e->count, cudaMemcpyHostToDevice,
                                             e->stream), "shift"))
        return rc;
    k_ens_shift<<<ens_blocks(e), 256, 0, e->stream>>>(ens_dn(e), d);
    e->launches++;
    return ens_dsync(e, "shift");
}

static int lg_of(int N) {
    int l = 0;
    while ((1 << l) < N) ++l;
    return N > 0 ? l : 0;
}

int ens_zeta_moments(iegpu_ens* e, int N, double* sum, double* sumsq, long long* n) {
    const unsigned nb = ens_blocks(e);
    double* part = nullptr;
    if (int rc = ens_cuda(e, cudaMalloc(&part, sizeof(double) * 2 * nb), "moments scratch")) return rc;
    k_ens_zeta_moments<<<nb, 256, 0, e->stream>>>(ens_dn(e), lg_of(N), part);
    e->launches++;
    std::vector<double> h(2 * (size_t)nb);
    int rc = ens_cuda(e, cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e->stream),
                      "moments");
    if (!rc) rc = ens_dsync(e, "moments");
    cudaFree(part);
    if (rc) return rc;
    double s = 0.0, s2 = 0.0;
    for (unsigned q = 0; q < nb; ++q) { s += h[2 * q]; s2 += h[2 * q + 1]; }
    long long cnt = 0;
    for (int b = 0; b < e->count; ++b)
        if (N == 0 || e->N[(size_t)b] == N) cnt += (long long)e->N[(size_t)b] * e->N[(size_t)b] * e->N[(size_t)b];
    *sum = s;
    *sumsq = s2;
    *n = cnt;
    return IEGPU_OK;
}

int ens_zeta_hist(iegpu_ens* e, int N, double lo, double width, int nbins, long long* counts, long long* outside) {
    unsigned long long* d = nullptr;
    if (int rc = ens_cuda(e, cudaMalloc(&d, sizeof(unsigned long long) * (nbins + 2)), "histogram scratch")) return rc;
    int rc = ens_cuda(e, cudaMemsetAsync(d, 0, sizeof(unsigned long long) * (nbins + 2), e->stream), "histogram");
    if (!rc) {
        k_ens_zeta_hist<<<ens_blocks(e), 256, sizeof(unsigned) * (nbins + 2), e->stream>>>(ens_dn(e), lg_of(N), lo, width,
                                                                                           nbins, d);
        e->launches++;
    }
    std::vector<unsigned long long> h((size_t)nbins + 2);
    if (!rc) rc = ens_cuda(e, cudaMemcpyAsync(h.data(), d, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                                              e->stream), "histogram");
    if (!rc) rc = ens_dsync(e, "histogram");
    cudaFree(d);
    if (rc) return rc;
    for (int q = 0; q < nbins; ++q) counts[q] = (long long)h[(size_t)q];
    outside[0] = (long long)h[(size_t)nbins];
    outside[1] = (long long)h[(size_t)nbins + 1];
    return IEGPU_OK;
}

}  // namespace iegpu

using namespace iegpu;

extern "C" {

// The deltaN stage of every lattice: run_deltaN_loop (src/evolution.cpp:1291-1375)
// up to saveN's Nmean and shift (src/output.cpp:1522-1531).
int iegpu_ens_deltaN(iegpu_ens* e, iegpu_bg* bg, double dN, double Nend, int use_phiref_manual, double phiref_manual,
                     double* phiref, float* nmean) {
    if (!e || !bg || !(dN > 0)) return IEGPU_EINVAL;
    const int n = e->count;
    if (cudaMemsetAsync(e->dctl, 0, sizeof(DevCtl), e->stream) != cudaSuccess) return ens_cuda(e, cudaGetLastError(), "memset");
    if (int rc = ens_materialize(e)) return rc;
    e->mat = 1;
    e->zeta_ready = 0;
    std::vector<double> v((size_t)n), ref((size_t)n, 0.0);
    for (int b = 0; b < n; ++b) v[(size_t)b] = std::pow(bg[b].a, e->cfg.rescale_s - 1.0);
    if (int rc = ens_initN(e, v.data())) return rc;
    if (int rc = ens_check_error(e)) return rc;
    // evolve_fieldsN(0.5 dN) with the initial global phiref = 0 (src/evolution.cpp:1300-1302)
    for (int b = 0; b < n; ++b) bg[b].t += 0.5 * dN;
    if (int rc = ens_deltaN_steps(e, 0.5 * dN, 1, ref.data(), 0, 1)) return rc;
    for (int b = 0; b < n; ++b) bg[b].a += 0.5 * dN * bg[b].ad;
    if (use_phiref_manual) {
        for (int b = 0; b < n; ++b) ref[(size_t)b] = phiref_manual;
    } else if (int rc = ens_phiref(e, ref.data())) {
        return rc;
    }
    // the loop: while (Ne <= Nend) { evolve_derivsN(dN); evolve_fieldsN(dN); Ne += dN; }
    double Ne = 0.0;
    int steps = 0;
    while (Ne <= Nend) {
        Ne += dN;
        ++steps;
    }
    if (int rc = ens_deltaN_steps(e, dN, steps, ref.data(), 1, 1)) return rc;
    for (int s = 0; s < steps; ++s)
        for (int b = 0; b < n; ++b) {
            bg[b].t += dN;
            bg[b].a += dN * bg[b].ad;
        }
    // saveN: evolve_fieldsN(-0.5 dN) when t > 0, Nmean, deltaN -= Nmean
    bool back = false;
    for (int b = 0; b < n; ++b) back |= bg[b].t > 0.0;
    if (back) {
        for (int b = 0; b < n; ++b) bg[b].t += -0.5 * dN;
        if (int rc = ens_deltaN_steps(e, -0.5 * dN, 1, ref.data(), 0, 1)) return rc;
        for (int b = 0; b < n; ++b) bg[b].a += -0.5 * dN * bg[b].ad;
    }
    if (int rc = ens_check_error(e)) return rc;
    const double cutoff = Nend - dN;
    e->nmean.assign((size_t)n, 0.f);
    if (int rc = ens_saveN_mean(e, cutoff, e->nmean.data())) return rc;
    if (int rc = ens_shift(e, e->nmean.data())) return rc;
    e->phiref = ref;
    e->zeta_cutoff = cutoff;
    e->zeta_ready = 1;
    for (int b = 0; b < n; ++b) {
        if (phiref) phiref[b] = ref[(size_t)b];
        if (nmean) nmean[b] = e->nmean[(size_t)b];
    }
    return IEGPU_OK;
}

// spectraN of every lattice (src/output.cpp:1140-1170 after saveN's zeroing):
// zeta above cutoff - Nmean set to 0, the lattice mean removed, FFT, shell
// sums.  counts/f2 hold lattice b's iegpu_numbins(N_b) bins after those of
// lattices 0..b-1.  The ensemble's zeta map is left unchanged.
int iegpu_ens_zeta_spectra(iegpu_ens* e, int* counts, double* f2) {
    if (!e || !counts || !f2) return IEGPU_EINVAL;
    if (!e->zeta_ready) return ens_error(e, IEGPU_EINVAL, "run iegpu_ens_deltaN first");
    if (int rc = ens_dsync(e, "spectra")) return rc;
    size_t at = 0;
    for (int b = 0; b < e->count; ++b) {
        const int N = e->N[(size_t)b];
        iegpu_ctx* h = nullptr;
        for (size_t q = 0; q < e->sizes.size(); ++q)
            if (e->sizes[q] == N) h = e->helper[q];
        const size_t gs = (size_t)N * N * N;
        if (int rc = ens_cuda(e, cudaMemcpyAsync(h->dn, e->dn + e->off[(size_t)b], sizeof(double) * gs,
                                                 cudaMemcpyDeviceToDevice, h->stream), "zeta copy"))
            return rc;
        int rc = iegpu_zero_above(h, IEGPU_DELTAN, e->zeta_cutoff - (double)e->nmean[(size_t)b]);
        double sum = 0.0;
        if (!rc) rc = iegpu_sum(h, IEGPU_DELTAN, &sum);
        if (!rc) rc = iegpu_shift(h, IEGPU_DELTAN, sum / (double)gs);
        const int nb = iegpu_numbins(N);
        if (!rc) rc = iegpu_spectrum(h, IEGPU_DELTAN, counts + at, f2 + at, nb);
        if (rc) return ens_error(e, rc, "lattice %d: %s", b, iegpu_last_error(h));
        at += (size_t)nb;
    }
    return IEGPU_OK;
}

// Pooled one-point histogram of zeta over the lattices of size N (0: all):
// nbins equal bins over [-nsigma sigma, +nsigma sigma], sigma the pooled
// standard deviation of zeta about its pooled mean.
int iegpu_ens_zeta_histogram(iegpu_ens* e, int N, int nbins, double nsigma, double* sigma, double* lo, double* width,
                             long long* counts, long long* outside) {
    if (!e || nbins <= 0 || nbins > 4096 || !(nsigma > 0) || !sigma || !lo || !width || !counts || !outside)
        return IEGPU_EINVAL;
    if (!e->zeta_ready) return ens_error(e, IEGPU_EINVAL, "run iegpu_ens_deltaN first");
    double s = 0.0, s2 = 0.0;
    long long n = 0;
    if (int rc = ens_zeta_moments(e, N, &s, &s2, &n)) return rc;
    if (n == 0) return ens_error(e, IEGPU_EINVAL, "no lattice of size %d", N);
    const double mean = s / (double)n;
    const double var = s2 / (double)n - mean * mean;
    *sigma = var > 0.0 ? std::sqrt(var) : 0.0;
    if (!(*sigma > 0.0)) return ens_error(e, IEGPU_EINVAL, "zeta has no spread");
    *lo = -nsigma * *sigma;
    *width = 2.0 * nsigma * *sigma / (double)nbins;
    return ens_zeta_hist(e, N, *lo, *width, nbins, counts, outside);
}

}  // extern "C"
