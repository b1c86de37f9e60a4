// ctx.cu -- C ABI entry points (include/iegpu.h): context lifetime, state
// transfer, and dispatch to the kernels of the other translation units.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include <map>
#include <mutex>
#include <utility>

#include "iegpu_internal.cuh"
#include "pot.cuh"

#define IEGPU_VERSION 1

namespace iegpu {

int set_error(iegpu_ctx* c, int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

int check_cuda(iegpu_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return IEGPU_OK;
    return set_error(c, IEGPU_ECUDA, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

int sync_and_check(iegpu_ctx* c, const char* what) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    return check_cuda(c, e, what);
}

bool is_double_field(int field) { return field == IEGPU_F || field == IEGPU_FD || field == IEGPU_DELTAN; }

double* dfield(iegpu_ctx* c, int field) {
    if (field == IEGPU_F) return c->f[c->cur];
    if (field == IEGPU_FD) return c->fd;
    if (field == IEGPU_DELTAN) return c->dn;
    return nullptr;
}

double* dnyq(iegpu_ctx* c, int field) {
    if (field == IEGPU_F) return c->fny;
    if (field == IEGPU_FD) return c->fdny;
    if (field == IEGPU_DELTAN) return c->fny;  // spectraN reuses the f Nyquist plane (src/output.cpp:1161)
    return nullptr;
}

float* ffield(iegpu_ctx* c, int field) {
    if (!c->cfg.sigw) return nullptr;
    if (field >= 8 && field < 14) return c->h[c->cur][field - 8];
    if (field >= 16 && field < 22) return c->hd[field - 16];
    return nullptr;
}

float* fnyq(iegpu_ctx* c, int field) {
    if (!c->cfg.sigw) return nullptr;
    if (field >= 8 && field < 14) return c->hny[field - 8];
    if (field >= 16 && field < 22) return c->hdny[field - 16];
    return nullptr;
}

int valid_field(iegpu_ctx* c, int field) {
    if (is_double_field(field)) return 1;
    return ffield(c, field) != nullptr;
}

// potential(v), src/potential.cpp:91-98, on the host (binary search + interp).
double host_potential(const iegpu_ctx* c, double v) {
    const PotDev& P = c->pot;
    if (!P.table) return (P.V0 * (1.0 - P.c1 * (v * v))) / P.B2;
    const std::vector<double>& x = c->htab_x;
    const int n = (int)x.size();
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (x[mid] >= v) lo = mid; else hi = mid;
    }
    const int l = hi;
    const double x0 = x[l - 1], x1 = x[l], y0 = c->htab_V[l - 1], y1 = c->htab_V[l];
    return (y1 + (v - x1) * (y0 - y1) / (x0 - x1)) / P.B2;
}

template <typename T>
static int dalloc(iegpu_ctx* c, T** p, size_t n) {
    if (cudaMalloc(p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, IEGPU_ENOMEM, "device allocation of %zu bytes failed", sizeof(T) * n);
    }
    return IEGPU_OK;
}

static void free_all(iegpu_ctx* c) {
    fp64_destroy_graphs(c);
    split_destroy_graphs(c);
    for (int q = 0; q < 2; ++q) {
        cudaFree(c->sp[q]);
        cudaFree(c->spi[q]);
        cudaFree(c->sxl[q]);
        cudaFree(c->spl[q]);
    }
    cudaFree(c->sctl);
    if (c->sctl_h) cudaFreeHost(c->sctl_h);
    fft_free(c);
    for (int q = 0; q < 2; ++q) cudaFree(c->f[q]);
    cudaFree(c->fd); cudaFree(c->dn); cudaFree(c->fny); cudaFree(c->fdny); cudaFree(c->lap);
    for (int q = 0; q < 6; ++q) {
        cudaFree(c->h[0][q]); cudaFree(c->h[1][q]); cudaFree(c->hd[q]); cudaFree(c->hny[q]); cudaFree(c->hdny[q]);
    }
    cudaFree(c->rk_d); cudaFree(c->rk_h); cudaFree(c->dn_y5);
    cudaFree(c->tab); cudaFree(c->tkey); cudaFree(c->tdiv);
    cudaFree(c->ctl); cudaFree(c->part); cudaFree(c->counter); cudaFree(c->a_trace);
    cudaFree(c->spec_part); cudaFree(c->spec_cnt); cudaFree(c->misc);
    cudaFree(c->gw_pos); cudaFree(c->gw_start); cudaFree(c->gw_vals); cudaFree(c->gw_f2f); cudaFree(c->gw_f2d);
    if (c->ctl_h) cudaFreeHost(c->ctl_h);
    if (c->misc_h) cudaFreeHost(c->misc_h);
    for (int q = 0; q < 4; ++q)
        if (c->ev[q]) cudaEventDestroy(c->ev[q]);
    if (c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace iegpu

namespace iegpu {

cudaError_t smem_optin(const void* fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> done;
    int dev = 0;
    const cudaError_t ge = cudaGetDevice(&dev);
    if (ge != cudaSuccess) return ge;
    std::lock_guard<std::mutex> lock(mu);
    size_t& have = done[std::make_pair(fn, dev)];
    if (have >= bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}

}  // namespace iegpu

using namespace iegpu;

extern "C" {

int iegpu_version(void) { return IEGPU_VERSION; }

const char* iegpu_strerror(int code) {
    switch (code) {
        case IEGPU_OK: return "ok";
        case IEGPU_EINVAL: return "invalid argument";
        case IEGPU_ECUDA: return "CUDA error";
        case IEGPU_ERANGE: return "field value outside the numerical potential range";
        case IEGPU_ENAN: return "unstable solution (non-finite mean)";
        case IEGPU_ECOURANT: return "Courant condition violated";
        case IEGPU_ENOMEM: return "device out of memory";
        case IEGPU_ETABLE: return "invalid potential table";
        case IEGPU_EUNSUPPORTED: return "unsupported in this form";
        case IEGPU_ETIMEOUT: return "device wait timed out";
        case IEGPU_ETOOBIG: return "size above the fixed limit of this entry point";
        case IEGPU_ECONVERGE: return "RK45 step control failed to converge";
        default: return "unknown error";
    }
}

int iegpu_create(const iegpu_config* cfg, iegpu_ctx** out) {
    if (!cfg || !out) return IEGPU_EINVAL;
    *out = nullptr;
    const int N = cfg->N;
    if (N < 8 || N > 1024 || (N & (N - 1))) return IEGPU_EINVAL;
    if (cfg->form != IEGPU_FORM_FP64 && cfg->form != IEGPU_FORM_SPLIT && cfg->form != IEGPU_FORM_SPLIT_COMP)
        return IEGPU_EINVAL;
    // the compensated steps live in the row-tile kernel of 128 <= N <= 512
    if (cfg->form == IEGPU_FORM_SPLIT_COMP && (N < 128 || N > 512)) return IEGPU_EUNSUPPORTED;
    if (!(cfg->L > 0) || !(cfg->dt > 0) || !(cfg->rescale_B > 0)) return IEGPU_EINVAL;
    iegpu_ctx* c = new (std::nothrow) iegpu_ctx();
    if (!c) return IEGPU_ENOMEM;
    c->cfg = *cfg;
    c->N = N;
    while ((1 << c->lg) < N) ++c->lg;
    c->gs = (size_t)N * N * N;
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return IEGPU_ECUDA;
    }
    c->sms = prop.multiProcessorCount;
    int rc = IEGPU_OK;
    if (check_cuda(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream create")) rc = IEGPU_ECUDA;
    const size_t gs = c->gs, ny = (size_t)N * 2 * N;
    if (!rc) rc = dalloc(c, &c->f[0], gs);
    if (!rc) rc = dalloc(c, &c->f[1], gs);
    if (!rc) rc = dalloc(c, &c->fd, gs);
    if (!rc) rc = dalloc(c, &c->dn, gs);
    if (!rc) rc = dalloc(c, &c->fny, ny);
    if (!rc) rc = dalloc(c, &c->fdny, ny);
    if (!rc && cfg->sigw) {
        for (int q = 0; q < 6 && !rc; ++q) {
            rc = dalloc(c, &c->h[0][q], gs);
            if (!rc) rc = dalloc(c, &c->h[1][q], gs);
            if (!rc) rc = dalloc(c, &c->hd[q], gs);
            if (!rc) rc = dalloc(c, &c->hny[q], ny);
            if (!rc) rc = dalloc(c, &c->hdny[q], ny);
        }
    }
    c->red_grid = c->sms * 4;
    const long long sites = (long long)gs;
    if (c->red_grid * 256LL > sites) c->red_grid = (int)((sites + 255) / 256);
    c->spec_blocks = c->sms * 2;
    const int nb = iegpu_numbins(N) + 1;
    // partial sums: up to 12 words (three exact sums) per reduction CTA, or 3
    // per CTA of the split step kernel
    // (at most max(8 per SM, number of 8x32 tiles))
    const long long tiles = (long long)(N / (N >= 32 ? 8 : (N >= 16 ? 16 : 8))) * (N / (N >= 32 ? 32 : N));
    const long long step_ctas = tiles > 8LL * c->sms ? tiles : 8LL * c->sms;
    c->part_cap = (int)(12 * c->red_grid + 3 * step_ctas + 64);
    if (!rc) rc = dalloc(c, &c->ctl, 1);
    if (!rc) rc = dalloc(c, &c->part, (size_t)c->part_cap);
    c->comp = cfg->form == IEGPU_FORM_SPLIT_COMP;
    if (!rc && cfg->form != IEGPU_FORM_FP64) {
        for (int q = 0; q < 2 && !rc; ++q) {
            rc = dalloc(c, &c->sp[q], gs);
            if (!rc) rc = dalloc(c, &c->spi[q], gs);
            if (!rc && c->comp) rc = dalloc(c, &c->sxl[q], gs);
            if (!rc && c->comp) rc = dalloc(c, &c->spl[q], gs);
        }
        if (!rc) rc = dalloc(c, &c->sctl, 1);
        if (!rc && check_cuda(c, cudaMallocHost(&c->sctl_h, sizeof(SplitCtl)), "pinned alloc")) rc = IEGPU_ENOMEM;
        if (!rc) {
            memset(c->sctl_h, 0, sizeof(SplitCtl));
            cudaMemsetAsync(c->sctl, 0, sizeof(SplitCtl), c->stream);
            for (int q = 0; q < 2; ++q) {
                cudaMemsetAsync(c->sp[q], 0, sizeof(float) * gs, c->stream);
                cudaMemsetAsync(c->spi[q], 0, sizeof(float) * gs, c->stream);
                if (c->comp) {
                    cudaMemsetAsync(c->sxl[q], 0, sizeof(unsigned short) * gs, c->stream);
                    cudaMemsetAsync(c->spl[q], 0, sizeof(unsigned short) * gs, c->stream);
                }
            }
        }
    }
    if (!rc) rc = dalloc(c, &c->counter, 4);   // [0] last-CTA detection, [2..3] persistent step sync
    if (!rc) rc = dalloc(c, &c->spec_part, (size_t)c->spec_blocks * nb + 65536);
    if (!rc) rc = dalloc(c, &c->spec_cnt, (size_t)c->spec_blocks * nb);
    if (!rc) rc = dalloc(c, &c->misc, (size_t)4 * nb + N + 64);
    if (!rc && check_cuda(c, cudaMallocHost(&c->ctl_h, sizeof(DevCtl)), "pinned alloc")) rc = IEGPU_ENOMEM;
    if (!rc && check_cuda(c, cudaMallocHost(&c->misc_h, sizeof(double) * ((size_t)4 * nb + N + 64)), "pinned alloc")) rc = IEGPU_ENOMEM;
    if (!rc) {
        // zero-initialised state, as the reference's vectors (src/initialize.cpp:119-120)
        cudaMemsetAsync(c->f[0], 0, sizeof(double) * gs, c->stream);
        cudaMemsetAsync(c->f[1], 0, sizeof(double) * gs, c->stream);
        cudaMemsetAsync(c->fd, 0, sizeof(double) * gs, c->stream);
        cudaMemsetAsync(c->dn, 0, sizeof(double) * gs, c->stream);
        cudaMemsetAsync(c->fny, 0, sizeof(double) * ny, c->stream);
        cudaMemsetAsync(c->fdny, 0, sizeof(double) * ny, c->stream);
        for (int q = 0; q < 6 && cfg->sigw; ++q) {
            cudaMemsetAsync(c->h[0][q], 0, sizeof(float) * gs, c->stream);
            cudaMemsetAsync(c->h[1][q], 0, sizeof(float) * gs, c->stream);
            cudaMemsetAsync(c->hd[q], 0, sizeof(float) * gs, c->stream);
            cudaMemsetAsync(c->hny[q], 0, sizeof(float) * ny, c->stream);
            cudaMemsetAsync(c->hdny[q], 0, sizeof(float) * ny, c->stream);
        }
        cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), c->stream);
        cudaMemsetAsync(c->counter, 0, 4 * sizeof(unsigned), c->stream);
        rc = sync_and_check(c, "create");
    }
    // hilltop constants with the reference's evaluation order (src/potential.cpp:77-83)
    PotDev& P = c->pot;
    P.table = cfg->potential == IEGPU_POT_TABLE;
    P.V0 = cfg->V0;
    P.c1 = (1.0 - cfg->ns) / 4.0;
    P.c2 = -cfg->V0 * (1.0 - cfg->ns) / 2.0;
    P.B2 = cfg->rescale_B * cfg->rescale_B;
    P.divB2 = make_div_const(P.B2);
    for (int q = 0; q < 4 && !rc; ++q)
        if (check_cuda(c, cudaEventCreate(&c->ev[q]), "event create")) rc = IEGPU_ECUDA;
    if (!rc) rc = fft_init(c);
    if (rc) {
        const int code = rc;
        free_all(c);
        delete c;
        return code;
    }
    *out = c;
    return IEGPU_OK;
}

int iegpu_destroy(iegpu_ctx* c) {
    if (!c) return IEGPU_EINVAL;
    cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return IEGPU_OK;
}

const char* iegpu_last_error(const iegpu_ctx* c) { return c ? c->err.c_str() : "null context"; }
void* iegpu_stream(iegpu_ctx* c) { return c ? (void*)c->stream : nullptr; }
long long iegpu_launch_count(const iegpu_ctx* c) { return c ? c->launches : 0; }

int iegpu_set_table(iegpu_ctx* c, const double* phi, const double* V, const double* dV, int n) {
    if (!c || !phi || !V || !dV || n < 2) return c ? set_error(c, IEGPU_ETABLE, "Numerical potential table must contain at least two points.\n") : IEGPU_EINVAL;
    for (int l = 1; l < n; ++l) {
        if (phi[l - 1] == phi[l]) return set_error(c, IEGPU_ETABLE, "Interpolation failed due to repeated field grid points.\n");
        if (!(phi[l - 1] > phi[l])) return set_error(c, IEGPU_ETABLE, "field table must be sorted in descending order");
    }
    // packed: x, V, dV, dxl, dyV, dydV, slopeV, slopedV (n each) + keys
    std::vector<double> h((size_t)8 * n, 0.0);
    std::vector<long long> k((size_t)n);
    for (int l = 0; l < n; ++l) {
        h[l] = phi[l];
        h[n + l] = V[l];
        h[2 * n + l] = dV[l];
        k[l] = order_key(phi[l]);
        if (l >= 1) {
            h[3 * n + l] = phi[l - 1] - phi[l];
            h[4 * n + l] = V[l - 1] - V[l];
            h[5 * n + l] = dV[l - 1] - dV[l];
            h[6 * n + l] = (V[l - 1] - V[l]) / (phi[l - 1] - phi[l]);
            h[7 * n + l] = (dV[l - 1] - dV[l]) / (phi[l - 1] - phi[l]);
        }
    }
    std::vector<DivConst> dv((size_t)n);
    for (int l = 1; l < n; ++l) dv[l] = make_div_const(h[3 * n + l]);
    dv[0] = make_div_const(1.0);
    cudaFree(c->tab);
    cudaFree(c->tkey);
    cudaFree(c->tdiv);
    c->tab = nullptr;
    c->tkey = nullptr;
    c->tdiv = nullptr;
    if (dalloc(c, &c->tab, h.size()) || dalloc(c, &c->tkey, k.size()) || dalloc(c, &c->tdiv, dv.size())) return IEGPU_ENOMEM;
    if (check_cuda(c, cudaMemcpy(c->tab, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice), "table upload") ||
        check_cuda(c, cudaMemcpy(c->tkey, k.data(), sizeof(long long) * k.size(), cudaMemcpyHostToDevice), "table upload") ||
        check_cuda(c, cudaMemcpy(c->tdiv, dv.data(), sizeof(DivConst) * dv.size(), cudaMemcpyHostToDevice), "table upload"))
        return IEGPU_ECUDA;
    c->htab_x.assign(phi, phi + n);
    c->htab_V.assign(V, V + n);
    c->htab_dV.assign(dV, dV + n);
    c->ntab = n;
    PotDev& P = c->pot;
    P.n = n;
    P.x = c->tab;
    P.V = c->tab + n;
    P.dV = c->tab + 2 * n;
    P.dxl = c->tab + 3 * n;
    P.dyV = c->tab + 4 * n;
    P.dydV = c->tab + 5 * n;
    P.slopeV = c->tab + 6 * n;
    P.slopedV = c->tab + 7 * n;
    P.key = c->tkey;
    P.ddx = c->tdiv;
    fp64_destroy_graphs(c);  // graphs hold the potential by value
    split_destroy_graphs(c);
    return IEGPU_OK;
}

static bool is_split(const iegpu_ctx* c) { return c->cfg.form != IEGPU_FORM_FP64; }
// F or FD held in the split representation (not the FP64 buffers)
static bool split_field(const iegpu_ctx* c, int field) {
    return is_split(c) && !c->split_mat && (field == IEGPU_F || field == IEGPU_FD);
}

// Split form: bring F and FD into the FP64 buffers (deltaN stage and FP64-only
// diagnostics).
static int split_materialize_both(iegpu_ctx* c) {
    int rc = split_materialize(c, 0, c->f[c->cur]);
    if (!rc) rc = split_materialize(c, 1, c->fd);
    return rc;
}

// Split form: the FP64 field buffer -> background (its mean) + perturbation.
static int split_absorb_field(iegpu_ctx* c, int field) {
    double* x = field == IEGPU_F ? c->f[c->cur] : c->fd;
    double sum = 0.0;
    int rc = field_sum(c, field, &sum);
    if (rc) return rc;
    (void)x;
    return split_absorb(c, field == IEGPU_F ? 0 : 1, x, sum / (double)c->gs);
}

static int need_table(iegpu_ctx* c) {
    if (c->pot.table && c->ntab < 2) return set_error(c, IEGPU_ETABLE, "numerical potential selected but no table was set");
    return IEGPU_OK;
}

int iegpu_upload(iegpu_ctx* c, int field, const void* host, const void* nyquist) {
    if (!c || !host) return IEGPU_EINVAL;
    if (!valid_field(c, field)) return set_error(c, IEGPU_EINVAL, "unknown field %d", field);
    const size_t ny = (size_t)c->N * 2 * c->N;
    if (is_double_field(field)) {
        if (check_cuda(c, cudaMemcpy(dfield(c, field), host, sizeof(double) * c->gs, cudaMemcpyHostToDevice), "upload")) return IEGPU_ECUDA;
        if (nyquist && check_cuda(c, cudaMemcpy(dnyq(c, field), nyquist, sizeof(double) * ny, cudaMemcpyHostToDevice), "upload")) return IEGPU_ECUDA;
        if (is_split(c) && (field == IEGPU_F || field == IEGPU_FD)) {
            c->split_mat = 0;
            if (int rc = split_absorb_field(c, field)) return rc;
            return sync_and_check(c, "upload");
        }
    } else {
        if (check_cuda(c, cudaMemcpy(ffield(c, field), host, sizeof(float) * c->gs, cudaMemcpyHostToDevice), "upload")) return IEGPU_ECUDA;
        if (nyquist && check_cuda(c, cudaMemcpy(fnyq(c, field), nyquist, sizeof(float) * ny, cudaMemcpyHostToDevice), "upload")) return IEGPU_ECUDA;
    }
    return IEGPU_OK;
}

int iegpu_download(iegpu_ctx* c, int field, void* host, void* nyquist) {
    if (!c || !host) return IEGPU_EINVAL;
    if (!valid_field(c, field)) return set_error(c, IEGPU_EINVAL, "unknown field %d", field);
    if (sync_and_check(c, "download")) return IEGPU_ECUDA;
    const size_t ny = (size_t)c->N * 2 * c->N;
    if (split_field(c, field)) {
        if (int rc = split_materialize(c, field == IEGPU_F ? 0 : 1, dfield(c, field))) return rc;
        if (sync_and_check(c, "download")) return IEGPU_ECUDA;
    }
    if (is_double_field(field)) {
        if (check_cuda(c, cudaMemcpy(host, dfield(c, field), sizeof(double) * c->gs, cudaMemcpyDeviceToHost), "download")) return IEGPU_ECUDA;
        if (nyquist && check_cuda(c, cudaMemcpy(nyquist, dnyq(c, field), sizeof(double) * ny, cudaMemcpyDeviceToHost), "download")) return IEGPU_ECUDA;
    } else {
        if (check_cuda(c, cudaMemcpy(host, ffield(c, field), sizeof(float) * c->gs, cudaMemcpyDeviceToHost), "download")) return IEGPU_ECUDA;
        if (nyquist && check_cuda(c, cudaMemcpy(nyquist, fnyq(c, field), sizeof(float) * ny, cudaMemcpyDeviceToHost), "download")) return IEGPU_ECUDA;
    }
    return IEGPU_OK;
}

int iegpu_add(iegpu_ctx* c, int field, double value) {
    if (!c) return IEGPU_EINVAL;
    if (split_field(c, field)) {
        // a constant shifts the FP64 background only
        if (check_cuda(c, cudaMemcpy(c->sctl_h, c->sctl, sizeof(SplitCtl), cudaMemcpyDeviceToHost), "ctl")) return IEGPU_ECUDA;
        if (field == IEGPU_F) c->sctl_h->phibar += value;
        else c->sctl_h->pibar += value;
        return check_cuda(c, cudaMemcpy(c->sctl, c->sctl_h, sizeof(SplitCtl), cudaMemcpyHostToDevice), "ctl");
    }
    return field_add(c, field, value);
}

int iegpu_shift(iegpu_ctx* c, int field, double value) {
    if (!c) return IEGPU_EINVAL;
    return field_add(c, field, -value);
}

int iegpu_zero_above(iegpu_ctx* c, int field, double threshold) {
    if (!c) return IEGPU_EINVAL;
    return field_zero_above(c, field, threshold);
}

int iegpu_sum(iegpu_ctx* c, int field, double* sum) {
    if (!c || !sum) return IEGPU_EINVAL;
    if (split_field(c, field)) {
        double v[6];
        if (int rc = split_sums(c, v)) return rc;
        *sum = (double)c->gs * (field == IEGPU_F ? c->sctl_h->phibar : c->sctl_h->pibar) + (field == IEGPU_F ? v[0] : v[2]);
        return IEGPU_OK;
    }
    return field_sum(c, field, sum);
}

static int split_running(iegpu_ctx* c) {
    if (c->split_mat) return set_error(c, IEGPU_EUNSUPPORTED, "the split-form lattice was handed to the deltaN stage; upload F and FD to evolve it again");
    return IEGPU_OK;
}

int iegpu_evolve_fields(iegpu_ctx* c, double d, iegpu_bg* bg) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (is_split(c)) {
        if (int rc = split_running(c)) return rc;
        return split_evolve_fields(c, d, bg);
    }
    return fp64_evolve_fields(c, d, bg);
}

int iegpu_evolve_derivs(iegpu_ctx* c, double d, iegpu_bg* bg) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    if (is_split(c)) {
        if (int rc = split_running(c)) return rc;
        return split_evolve_derivs(c, d, bg);
    }
    return fp64_evolve_derivs(c, d, bg);
}

int iegpu_leapfrog(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps_taken, double* a_trace) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    if (is_split(c)) {
        if (int rc = split_running(c)) return rc;
        return split_leapfrog(c, af, max_steps, bg, steps_taken, a_trace);
    }
    return fp64_leapfrog(c, af, max_steps, bg, steps_taken, a_trace);
}

int iegpu_energies(iegpu_ctx* c, const iegpu_bg* bg, double out[3]) {
    if (!c || !bg || !out) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    if (is_split(c) && !c->split_mat) {
        double v[6];
        if (int rc = split_sums(c, v)) return rc;
        const double gs = (double)c->gs, a = bg->a, s = c->cfg.rescale_s, dx = c->cfg.L / (double)c->N;
        const double pb = c->sctl_h->phibar, qb = c->sctl_h->pibar;
        const PotDev& P = c->pot;
        // <fd^2> = pibar^2 + 2 pibar <dpi> + <dpi^2>
        const double fd2 = qb * qb + 2.0 * qb * (v[2] / gs) + v[3] / gs;
        out[0] = 0.5 * pow(a, 2.0 * s - 2.0) * fd2;
        out[1] = 0.5 * v[4] * ((1.0 / (a * dx)) * (1.0 / (a * dx))) / gs;
        const double Vbar = host_potential(c, pb);
        if (P.table) out[2] = Vbar + (v[5] / P.B2) / gs;
        else out[2] = Vbar - (P.V0 * P.c1 / P.B2) * (2.0 * pb * v[0] + v[1]) / gs;
        return IEGPU_OK;
    }
    return fp64_energies(c, bg, out);
}

int iegpu_bunch_davies(iegpu_ctx* c, int seed, double phi0, double dphi0, double hi_cut, double lo_cut,
                       double* hubble_init) {
    if (!c || !hubble_init) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    const double dx = c->cfg.L / (double)c->N;
    if (c->cfg.dt > dx / std::sqrt(3.0))
        return set_error(c, IEGPU_ECOURANT, "Time step too large. Courant condition violated: dt/dx = %f\n", c->cfg.dt / dx);
    if (c->pot.table && (phi0 > c->htab_x.front() || phi0 < c->htab_x.back()))
        return set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n",
                         phi0, c->htab_x.back(), c->htab_x.front());
    // hubble_init before the modes are drawn (src/initialize.cpp:125-131): set_mode's hbterm
    const double h0 = std::sqrt((0.5 * dphi0 * dphi0 + host_potential(c, phi0)) / 3.0);
    int rc = bunch_davies(c, seed, phi0, dphi0, h0, hi_cut, lo_cut);
    if (rc) return rc;
    iegpu_bg b{0.0, 1.0, 0.0, 0.0, 1.0};
    double e[3];
    rc = fp64_energies(c, &b, e);
    if (rc) return rc;
    *hubble_init = std::sqrt((e[0] + e[2] + e[1]) / 3.0);
    if (is_split(c)) {
        // split form: the FP64 fields become background + FP32 perturbation
        c->split_mat = 0;
        rc = split_absorb_field(c, IEGPU_F);
        if (!rc) rc = split_absorb_field(c, IEGPU_FD);
        if (!rc) rc = sync_and_check(c, "split initial conditions");
    }
    return rc;
}

int iegpu_timer_start(iegpu_ctx* c) {
    if (!c) return IEGPU_EINVAL;
    return check_cuda(c, cudaEventRecord(c->ev[3], c->stream), "timer start");
}

int iegpu_timer_stop(iegpu_ctx* c, float* ms) {
    if (!c || !ms) return IEGPU_EINVAL;
    if (check_cuda(c, cudaEventRecord(c->ev[0], c->stream), "timer stop")) return IEGPU_ECUDA;
    if (check_cuda(c, cudaEventSynchronize(c->ev[0]), "timer sync")) return IEGPU_ECUDA;
    return check_cuda(c, cudaEventElapsedTime(ms, c->ev[3], c->ev[0]), "timer elapsed");
}

int iegpu_profile_leapfrog(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms_out, int nk) {
    if (!c || !bg || !ms_out || nsteps < 0) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    if (is_split(c)) {
        if (int rc = split_running(c)) return rc;
        return split_profile(c, af, nsteps, bg, ms_out, nk);
    }
    return fp64_profile(c, af, nsteps, bg, ms_out, nk);
}

int iegpu_autotune(iegpu_ctx* c, const iegpu_bg* bg, int* rows, int* prefetch, int* chunks) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (is_split(c) && !c->split_mat) {
        if (int rc = need_table(c)) return rc;
        if (int rc = split_autotune(c, bg)) return rc;
    }
    if (rows) *rows = c->row_cfg.TJ;
    if (prefetch) *prefetch = c->row_cfg.PF + (c->row_cfg.tma ? 10 : 0);
    if (chunks) *chunks = c->row_cfg.chunks;
    return IEGPU_OK;
}

int iegpu_set_shape(iegpu_ctx* c, int rows, int prefetch, int chunks) {
    if (!c) return IEGPU_EINVAL;
    if (!is_split(c)) return set_error(c, IEGPU_EUNSUPPORTED, "the launch shape belongs to the split form");
    return split_set_shape(c, rows, prefetch, chunks);
}

// The RK4 integrator runs on the plain FP64 state (the split form's step is
// the leapfrog).
static int rk_ok(iegpu_ctx* c) {
    if (is_split(c)) return set_error(c, IEGPU_EUNSUPPORTED, "the rk4 integrator runs on the plain FP64 form");
    return need_table(c);
}

int iegpu_rk4_step_inflation(iegpu_ctx* c, double h, iegpu_bg* bg) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (int rc = rk_ok(c)) return rc;
    return fp64_rk4_step(c, h, bg);
}

int iegpu_rk4(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps_taken, double* a_trace) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (steps_taken) *steps_taken = 0;
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (int rc = rk_ok(c)) return rc;
    return fp64_rk4(c, af, max_steps, bg, steps_taken, a_trace);
}

int iegpu_rk45_effective(const iegpu_rk45_controls* in, double dt, iegpu_rk45_controls* out) {
    if (!in || !out) return IEGPU_EINVAL;
    *out = rk45_sanitized_dt(in, dt);
    return IEGPU_OK;
}

int iegpu_rk45_step_inflation(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double h, double hmax, double* h_next,
                              int* accepted, iegpu_bg* bg) {
    if (!c || !bg || !ctl || !h_next || !accepted) return IEGPU_EINVAL;
    if (int rc = rk_ok(c)) return rc;
    return fp64_rk45_step(c, ctl, h, hmax, h_next, accepted, bg);
}

int iegpu_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af, int max_steps, double* h, iegpu_bg* bg,
               int* steps_taken, double* a_trace) {
    if (!c || !bg || !ctl || !h) return IEGPU_EINVAL;
    if (steps_taken) *steps_taken = 0;
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (int rc = rk_ok(c)) return rc;
    return fp64_rk45(c, ctl, af, max_steps, h, bg, steps_taken, a_trace);
}

// The post-inflation phase runs on the plain FP64 state with SIGW on, as
// the reference requires (src/parameters.h:33-35).
static int post_ok(iegpu_ctx* c) {
    if (is_split(c)) return set_error(c, IEGPU_EUNSUPPORTED, "the post-inflation phase runs on the plain FP64 form");
    if (!c->cfg.sigw) return set_error(c, IEGPU_EUNSUPPORTED, "post_inflation requires calculate_SIGW = 1");
    return IEGPU_OK;
}

int iegpu_initialize_post_inflation(iegpu_ctx* c, double horizon_factor, double omega, int from_deltaN, iegpu_bg* bg) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (int rc = post_ok(c)) return rc;
    return fp64_post_init(c, horizon_factor, omega, from_deltaN != 0, bg);
}

int iegpu_evolve_derivs_post_inflation(iegpu_ctx* c, double d, double omega, iegpu_bg* bg) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (int rc = post_ok(c)) return rc;
    return fp64_post_derivs(c, d, omega, bg);
}

int iegpu_post_inflation_leapfrog(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps,
                                  iegpu_bg* bg, int* steps, double* a_trace) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (steps) *steps = 0;
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (int rc = post_ok(c)) return rc;
    return fp64_post_leapfrog(c, af_post, dt_post, omega, max_steps, bg, steps, a_trace);
}

int iegpu_post_inflation_rk4(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps, iegpu_bg* bg,
                             int* steps, double* a_trace) {
    if (!c || !bg) return IEGPU_EINVAL;
    if (steps) *steps = 0;
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (int rc = post_ok(c)) return rc;
    return fp64_post_rk4(c, af_post, dt_post, omega, max_steps, bg, steps, a_trace);
}

int iegpu_post_inflation_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af_post, double dt_post,
                              double omega, int max_steps, double* h, iegpu_bg* bg, int* steps, double* a_trace) {
    if (!c || !bg || !ctl || !h) return IEGPU_EINVAL;
    if (steps) *steps = 0;
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (int rc = post_ok(c)) return rc;
    return fp64_post_rk45(c, ctl, af_post, dt_post, omega, max_steps, h, bg, steps, a_trace);
}

int iegpu_set_persistent(iegpu_ctx* c, int on) {
    if (!c) return IEGPU_EINVAL;
    if (!is_split(c)) return set_error(c, IEGPU_EUNSUPPORTED, "persistent launches belong to the split form");
    c->persist = on != 0;
    return IEGPU_OK;
}

int iegpu_set_wait_limit(iegpu_ctx* c, unsigned polls, int unreachable) {
    if (!c) return IEGPU_EINVAL;
    if (!is_split(c)) return set_error(c, IEGPU_EUNSUPPORTED, "bounded device waits belong to the split form");
    c->wait_polls = polls;
    c->wait_bias = unreachable ? 0x40000000u : 0u;
    return IEGPU_OK;
}

int iegpu_means(iegpu_ctx* c, double out[3]) {
    if (!c || !out) return IEGPU_EINVAL;
    if (is_split(c) && !c->split_mat) {
        double v[6];
        if (int rc = split_sums(c, v)) return rc;
        const double gs = (double)c->gs, pb = c->sctl_h->phibar, qb = c->sctl_h->pibar;
        out[0] = gs * pb + v[0];
        out[1] = gs * qb + v[2];
        out[2] = gs * pb * pb + 2.0 * pb * v[0] + v[1];
        return IEGPU_OK;
    }
    return field_means(c, out);
}

int iegpu_histogram(iegpu_ctx* c, int field, int nbins, double* bmin, double* df, double* freq) {
    if (c && split_field(c, field) && is_double_field(field)) {
        if (int rc = split_materialize(c, field == IEGPU_F ? 0 : 1, dfield(c, field))) return rc;
    }
    // bin counters live in shared memory: at most 8192 bins
    if (!c || !bmin || !df || !freq || nbins <= 0 || nbins > 8192) return c ? set_error(c, IEGPU_EINVAL, "bad histogram arguments (1 <= nbins <= 8192)") : IEGPU_EINVAL;
    return field_histogram(c, field, nbins, bmin, df, freq);
}

int iegpu_fft(iegpu_ctx* c, int field, int forward) {
    if (!c || (forward != 1 && forward != -1)) return IEGPU_EINVAL;
    if (!valid_field(c, field)) return set_error(c, IEGPU_EINVAL, "unknown field %d", field);
    if (split_field(c, field))
        return set_error(c, IEGPU_EUNSUPPORTED, "in-place FFT of f/fd is provided by the FP64 form; the split form uses iegpu_bunch_davies and iegpu_spectrum");
    int rc;
    if (is_double_field(field)) rc = fft_d(c, dfield(c, field), dnyq(c, field), forward);
    else rc = fft_f(c, ffield(c, field), fnyq(c, field), forward);
    if (rc) return rc;
    return sync_and_check(c, "fft");
}

int iegpu_numbins(int N) { return (int)(1.73205 * (N / 2)) + 1; }

int iegpu_spectrum(iegpu_ctx* c, int field, int* counts, double* f2, int nbins) {
    if (!c || !counts || !f2) return IEGPU_EINVAL;
    if (!is_double_field(field)) return set_error(c, IEGPU_EINVAL, "spectra are defined for f, fd and deltaN");
    if (nbins != iegpu_numbins(c->N)) return set_error(c, IEGPU_EINVAL, "nbins must be %d", iegpu_numbins(c->N));
    double* x = dfield(c, field);
    double* ny = dnyq(c, field);
    if (split_field(c, field)) {
        // spectrum of the FP32 perturbation, taken in FP64; the k = 0 mode
        // (bin 0, count 1) is the lattice sum of background + perturbation
        double v[6];
        int rc = split_sums(c, v);
        if (!rc) rc = split_to_double(c, field == IEGPU_F ? 0 : 1, x);
        if (!rc) rc = fft_d(c, x, ny, 1);
        if (!rc) rc = spectrum_bin_d(c, x, ny, counts, f2, nbins);
        if (rc) return rc;
        const double k0 = (double)c->gs * (field == IEGPU_F ? c->sctl_h->phibar : c->sctl_h->pibar) +
                          (field == IEGPU_F ? v[0] : v[2]);
        f2[0] = k0 * k0;
        return IEGPU_OK;
    }
    int rc = fft_d(c, x, ny, 1);
    if (!rc) rc = spectrum_bin_d(c, x, ny, counts, f2, nbins);
    if (!rc) rc = fft_d(c, x, ny, -1);
    if (!rc) rc = sync_and_check(c, "spectrum");
    return rc;
}

int iegpu_spectrum_cutoff(iegpu_ctx* c, int* counts, double* f2, int nbins, double high_cutoff_index,
                          double low_cutoff_index) {
    if (!c || !counts || !f2) return IEGPU_EINVAL;
    if (!(high_cutoff_index > 0)) return iegpu_spectrum(c, IEGPU_F, counts, f2, nbins);
    if (is_split(c))
        return set_error(c, IEGPU_EUNSUPPORTED, "the forcing cutoff is provided by the plain FP64 form");
    if (nbins != iegpu_numbins(c->N)) return set_error(c, IEGPU_EINVAL, "nbins must be %d", iegpu_numbins(c->N));
    double* x = dfield(c, IEGPU_F);
    double* ny = dnyq(c, IEGPU_F);
    double* xd = dfield(c, IEGPU_FD);
    double* nyd = dnyq(c, IEGPU_FD);
    int rc = fft_d(c, x, ny, 1);
    if (!rc) rc = spectrum_bin_d(c, x, ny, counts, f2, nbins);
    if (!rc) rc = fft_d(c, xd, nyd, 1);
    if (!rc) rc = forcing_cutoff(c, x, ny, xd, nyd, high_cutoff_index, low_cutoff_index);
    if (!rc) rc = fft_d(c, xd, nyd, -1);
    if (!rc) rc = fft_d(c, x, ny, -1);
    if (!rc) rc = sync_and_check(c, "spectrum with forcing cutoff");
    return rc;
}

int iegpu_gw_spectrum_ref(iegpu_ctx* c, int which, double to_phys, int* counts, float* f2, double* f2_sum,
                          int nbins) {
    if (!c || !counts || !f2 || (which != 0 && which != 1)) return IEGPU_EINVAL;
    if (!c->cfg.sigw) return set_error(c, IEGPU_EUNSUPPORTED, "context was created without SIGW");
    if (nbins != iegpu_numbins(c->N)) return set_error(c, IEGPU_EINVAL, "nbins must be %d", iegpu_numbins(c->N));
    for (int q = 0; q < 6; ++q) {
        float* x = which ? c->hd[q] : c->h[c->cur][q];
        float* ny = which ? c->hdny[q] : c->hny[q];
        if (int rc = fft_f(c, x, ny, 1)) return rc;
    }
    int rc = gw_bin_ref(c, which, to_phys, counts, f2, f2_sum, nbins);
    for (int q = 0; q < 6 && !rc; ++q) {
        float* x = which ? c->hd[q] : c->h[c->cur][q];
        float* ny = which ? c->hdny[q] : c->hny[q];
        rc = fft_f(c, x, ny, -1);
    }
    if (!rc) rc = sync_and_check(c, "gw spectrum");
    return rc;
}

int iegpu_gw_spectrum(iegpu_ctx* c, int which, double to_phys, int* counts, double* f2, int nbins) {
    if (!c || !counts || !f2 || (which != 0 && which != 1)) return IEGPU_EINVAL;
    if (!c->cfg.sigw) return set_error(c, IEGPU_EUNSUPPORTED, "context was created without SIGW");
    if (nbins != iegpu_numbins(c->N)) return set_error(c, IEGPU_EINVAL, "nbins must be %d", iegpu_numbins(c->N));
    for (int q = 0; q < 6; ++q) {
        float* x = which ? c->hd[q] : c->h[c->cur][q];
        float* ny = which ? c->hdny[q] : c->hny[q];
        if (int rc = fft_f(c, x, ny, 1)) return rc;
    }
    int rc = gw_bin(c, which, to_phys, counts, f2, nbins);
    for (int q = 0; q < 6 && !rc; ++q) {
        float* x = which ? c->hd[q] : c->h[c->cur][q];
        float* ny = which ? c->hdny[q] : c->hny[q];
        rc = fft_f(c, x, ny, -1);
    }
    if (!rc) rc = sync_and_check(c, "gw spectrum");
    return rc;
}

int iegpu_initializeN(iegpu_ctx* c, double a) {
    if (!c) return IEGPU_EINVAL;
    if (int rc = need_table(c)) return rc;
    if (is_split(c) && !c->split_mat) {
        // the deltaN integration is FP64: hand over phibar + dphi, pibar + dpi
        if (int rc = split_materialize_both(c)) return rc;
        c->split_mat = 1;
    }
    int rc = deltaN_init(c, a);
    if (!rc) rc = sync_and_check(c, "initializeN");
    if (!rc) {
        int e = 0;
        cudaMemcpy(&e, &c->ctl->error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e) {
            double v = 0;
            cudaMemcpy(&v, &c->ctl->errval, sizeof(double), cudaMemcpyDeviceToHost);
            rc = set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v,
                           c->htab_x.back(), c->htab_x.front());
        }
    }
    return rc;
}

int iegpu_get_phiref(iegpu_ctx* c, double* phiref) {
    if (!c || !phiref) return IEGPU_EINVAL;
    if (split_field(c, IEGPU_F)) {
        if (int rc = split_materialize(c, 0, c->f[c->cur])) return rc;
    }
    return get_phiref(c, phiref);
}

static int deltaN_run(iegpu_ctx* c, double d, int nsteps, double phiref, int dd, int df) {
    if (int rc = need_table(c)) return rc;
    if (is_split(c) && !c->split_mat)
        return set_error(c, IEGPU_EINVAL, "call iegpu_initializeN before the deltaN steps");
    if (check_cuda(c, cudaMemsetAsync(&c->ctl->error, 0, sizeof(int), c->stream), "memset")) return IEGPU_ECUDA;
    int rc = deltaN_steps(c, d, nsteps, phiref, dd, df);
    if (!rc) rc = sync_and_check(c, "deltaN");
    if (!rc) {
        int e = 0;
        cudaMemcpy(&e, &c->ctl->error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e) {
            double v = 0;
            cudaMemcpy(&v, &c->ctl->errval, sizeof(double), cudaMemcpyDeviceToHost);
            rc = set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v,
                           c->htab_x.back(), c->htab_x.front());
        }
    }
    return rc;
}

int iegpu_evolve_fieldsN(iegpu_ctx* c, double d, double phiref) {
    if (!c) return IEGPU_EINVAL;
    return deltaN_run(c, d, 1, phiref, 0, 1);
}

int iegpu_evolve_derivsN(iegpu_ctx* c, double d) {
    if (!c) return IEGPU_EINVAL;
    return deltaN_run(c, d, 1, 0.0, 1, 0);
}

int iegpu_deltaN_steps(iegpu_ctx* c, double dN, int nsteps, double phiref) {
    if (!c || nsteps < 0) return IEGPU_EINVAL;
    if (nsteps == 0) return IEGPU_OK;
    return deltaN_run(c, dN, nsteps, phiref, 1, 1);
}

static int deltaN_ready(iegpu_ctx* c) {
    if (int rc = need_table(c)) return rc;
    if (is_split(c) && !c->split_mat)
        return set_error(c, IEGPU_EINVAL, "call iegpu_initializeN before the deltaN steps");
    if (check_cuda(c, cudaMemsetAsync(&c->ctl->error, 0, sizeof(int), c->stream), "memset")) return IEGPU_ECUDA;
    return IEGPU_OK;
}

static int deltaN_range_status(iegpu_ctx* c, int rc) {
    if (!rc) rc = sync_and_check(c, "deltaN");
    if (!rc) {
        int e = 0;
        cudaMemcpy(&e, &c->ctl->error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e) {
            double v = 0;
            cudaMemcpy(&v, &c->ctl->errval, sizeof(double), cudaMemcpyDeviceToHost);
            rc = set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v,
                           c->htab_x.back(), c->htab_x.front());
        }
    }
    return rc;
}

int iegpu_deltaN_rk4_steps(iegpu_ctx* c, double dN, int nsteps, double phiref, iegpu_bg* bg) {
    if (!c || !bg || nsteps < 0) return IEGPU_EINVAL;
    if (nsteps == 0) return IEGPU_OK;
    if (int rc = deltaN_ready(c)) return rc;
    return deltaN_range_status(c, deltaN_rk4(c, dN, nsteps, phiref, bg));
}

int iegpu_deltaN_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double dN, double Nend, int max_steps,
                      double phiref, double* h, double* Ne, iegpu_bg* bg, int* steps, double* Ne_trace) {
    if (!c || !ctl || !h || !Ne || !bg || max_steps < 0) return IEGPU_EINVAL;
    if (steps) *steps = 0;
    if (int rc = deltaN_ready(c)) return rc;
    const int rc = deltaN_rk45(c, ctl, dN, Nend, max_steps, phiref, h, Ne, bg, steps, Ne_trace);
    if (rc) return rc;
    return deltaN_range_status(c, rc);
}

int iegpu_saveN_mean(iegpu_ctx* c, double cutoff, float* nmean) {
    if (!c || !nmean) return IEGPU_EINVAL;
    return saveN_mean(c, cutoff, nmean);
}

}  // extern "C"
