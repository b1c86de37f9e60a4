// leapfrog_fp64.cu -- plain FP64 leapfrog of src/evolution.cpp:150-284, and the
// other integrators of the plain FP64 state.
//
// Compiled with -fmad=false: every per-site expression is evaluated with the
// reference's operation order and rounding (no contraction), so a site given
// the same inputs produces the same bits as the reference CPU code.
//
// One leapfrog step is two kernels, captured in a CUDA graph:
//   k_lsum    reads f (7-point stencil), stores lapl(f) for the kick and adds
//             f*lapl(f) and the potential term of every site exactly
//             (gradient_energy / potential_energy, src/evolution.cpp:130-136,
//             src/potential.cpp:151-171; exact sums, exact.cuh); the last CTA
//             to finish rounds the two sums and runs the Friedmann update of
//             src/evolution.cpp:153-168 on the device.
//   k_kick    kick of fd (and hd) with the stored Laplacian and V', then the
//             drift f += d fd into the other f buffer (ping-pong), and
//             h += (float)(d hd) (src/evolution.cpp:170-281).
// GB300's FP64 pipe, not HBM, bounds this form: the Laplacian is formed once
// per step (the reference forms it twice, in the sum and in the kick), the
// sums' additions and the division by B^2 run on the integer pipes, so a
// site costs 19 FP64 operations (hilltop).  Algorithmic HBM traffic per
// site-update: 32 B of state (read f, fd; write f, fd); the stored Laplacian
// adds 16 B and the second read of f 8 B.
//
// The same unit holds the other integrators of the plain FP64 state, with the
// same per-site rules: the post-inflation leapfrog (src/evolution.cpp:1378-1653)
// and the Runge-Kutta steps (RK4, RK45) of the inflation and post-inflation
// loops (src/evolution.cpp:286-905).
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "iegpu_internal.cuh"
#include "pot.cuh"
#include "reduce.cuh"
#include "rk_tableau.cuh"

namespace iegpu {

struct SigwPtrs {
    const float* hs[6];
    float* hdst[6];
    float* hd[6];
};

struct StepConst {
    double dt, s, dx, gs, half_over_dx;
};

struct Nbr {
    long long c, kp, km, jp, jm, ip, im;
};

__device__ __forceinline__ Nbr neighbours(long long id, int lg) {
    const int m = (1 << lg) - 1;
    const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
    Nbr n;
    n.c = id;
    n.kp = id - k + ((k + 1) & m);
    n.km = id - k + ((k - 1) & m);
    n.jp = id + ((long long)(((j + 1) & m) - j) << lg);
    n.jm = id + ((long long)(((j - 1) & m) - j) << lg);
    n.ip = id + ((long long)(((i + 1) & m) - i) << (2 * lg));
    n.im = id + ((long long)(((i - 1) & m) - i) << (2 * lg));
    return n;
}

// lapl<T>, src/evolution.cpp:34-51: (k+1)+(k-1)+(j+1)+(j-1)+(i+1)+(i-1)-6f
template <typename T>
__device__ __forceinline__ T lapl7(const T* __restrict__ f, const Nbr& n, T fc) {
    return __ldg(&f[n.kp]) + __ldg(&f[n.km]) + __ldg(&f[n.jp]) + __ldg(&f[n.jm]) + __ldg(&f[n.ip]) +
           __ldg(&f[n.im]) - T(6) * fc;
}

// Friedmann update and step coefficients (src/evolution.cpp:153-168, 256,
// 283, 938, 944).  Runs in one thread.  G = sum f*lapl(f), Pn = potential sum
// (hilltop: sum f^2; table: sum V*B^2).
__device__ void step_scalars(DevCtl* ctl, const PotDev& P, const StepConst& K, double G, double Pn,
                             double* a_trace) {
    DevCtl& C = *ctl;
    double d;
    if (C.mode == kModeLeapfrog) {
        // loop body of src/evolution.cpp:937-945; "astep = a" closes an
        // iteration after its report, so the last step of a call leaves it
        // to the caller (the reference's save() still sees the old astep).
        if (C.steps_done >= C.steps_limit) {
            C.st.active = 0;
            C.done = 1;
            return;
        }
        if (C.steps_done > 0) C.bg.astep = C.bg.a;
        if (!(C.bg.a <= C.af)) {
            C.st.active = 0;
            C.done = 1;
            return;
        }
        d = K.dt * pow_exp(C.bg.astep, K.s - 1.0);
    } else {
        d = C.d_given;
    }
    const double a = C.bg.a;
    double ad = C.bg.ad;
    const double s = K.s;
    const double laplnorm = pow_exp(a, -2.0 * s) / (K.dx * K.dx);
    const double sfev1 = s + 1.0;
    const double sfev2 = -2.0 * s + 2.0;
    const double gradient = -G;
    const double grad = 0.5 * gradient * ((1.0 / (a * K.dx)) * (1.0 / (a * K.dx))) / K.gs;
    double pot;
    if (P.table) pot = (Pn / P.B2) / K.gs;
    else pot = (P.V0 * (K.gs - P.c1 * Pn) / P.B2) / K.gs;
    const double ad2 = (-2.0 * ad - 2.0 * a / d / sfev1 *
                        (1.0 - sqrt(1.0 + 2.0 * d * sfev1 * ad / a +
                                    (d * d) * sfev1 * pow_exp(a, sfev2) * (2.0 * grad / 3.0 + pot)))) / d;
    ad += 0.5 * d * ad2;
    C.st.d = d;
    C.st.laplnorm = laplnorm;
    C.st.friction = (2.0 + s) * ad / a;
    C.st.potnorm = pow_exp(a, 2.0 - 2.0 * s);
    C.st.srcAmp = 2.0 * pow_exp(a, -2.0 * s);
    C.st.active = 1;
    ad += 0.5 * d * ad2;
    C.bg.ad = ad;
    C.bg.ad2 = ad2;
    if (C.mode == kModeLeapfrog) {
        C.bg.t += d;
        C.bg.a = a + d * ad;
        if (a_trace) a_trace[C.steps_done] = C.bg.a;
        C.steps_done += 1;
    }
}

// Block combine of NV exact sums: the block's total is left in thread 0.
template <int NV>
__device__ __forceinline__ void acc_block_sum(Acc4 (&v)[NV]) {
    __shared__ Acc4 sh[NV][kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) acc_warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q][w] = v[q];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            if (lane < kThreads / 32) v[q] = sh[q][lane];
            else acc_zero(v[q]);
            acc_warp_sum(v[q]);
        }
    }
}

// Exact block partials: NV words of 4 limbs per CTA.
template <int NV>
__device__ __forceinline__ void acc_store_partial(unsigned long long* part, const Acc4 (&v)[NV]) {
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int l = 0; l < 4; ++l) part[((size_t)blockIdx.x * NV + q) * 4 + l] = v[q].w[l];
    }
}

// Sum of the CTAs' exact partials by warp 0; the rounded totals are valid in
// lane 0.  Integer sums: the order of the CTAs does not matter.
template <int NV>
__device__ __forceinline__ void acc_sum_partials(const unsigned long long* part, int nb, double (&out)[NV]) {
    const int lane = threadIdx.x & 31;
    Acc4 s[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc_zero(s[q]);
    for (int b = lane; b < nb; b += 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const unsigned long long* p = part + ((size_t)b * NV + q) * 4;
            acc_add4(s[q], __ldcg(p), __ldcg(p + 1), __ldcg(p + 2), __ldcg(p + 3));
        }
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        acc_warp_sum(s[q]);
        out[q] = lane == 0 ? acc_to_double(s[q]) : 0.0;
    }
}

// Flags of the exact sums from every thread of the CTA into ctl->sumflags:
// bit q: sum q met a non-finite term; a finite term of magnitude >= 2^30
// (beyond the accumulator) raises IEGPU_ETOOBIG.
template <int NV>
__device__ __forceinline__ void acc_publish_flags(DevCtl* ctl, const unsigned (&fl)[NV]) {
    unsigned nonfinite = 0, big = 0;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        nonfinite |= (fl[q] & 1u) << q;
        big |= fl[q] & 2u;
    }
    nonfinite = __reduce_or_sync(0xffffffffu, nonfinite);
    big = __reduce_or_sync(0xffffffffu, big);
    if ((threadIdx.x & 31) == 0) {
        if (nonfinite) atomicOr(&ctl->sumflags, nonfinite);
        if (big) flag_error(ctl, IEGPU_ETOOBIG, 0.0);
    }
}

// Pass 1 of a leapfrog step: lapl(f) of every site stored for the kick, and
// the two lattice sums of the Friedmann update, exact: G = sum f lapl(f) and
// Pn = sum f^2 (hilltop) or sum V B^2 (table).  The last CTA rounds them and
// runs the scalar update.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_lsum(const double* __restrict__ f, double* __restrict__ lap, PotDev P,
                                                   DevCtl* ctl, unsigned long long* part, unsigned* counter,
                                                   double* a_trace, int lg, StepConst K) {
    if (ctl->mode == kModeLeapfrog && ctl->done) return;
    const long long gs = 1LL << (3 * lg);
    Acc4 v[2];
    acc_zero(v[0]);
    acc_zero(v[1]);
    unsigned fl[2] = {0u, 0u};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const Nbr n = neighbours(id, lg);
        const double fc = __ldg(&f[id]);
        const double L = lapl7(f, n, fc);
        lap[id] = L;
        acc_add_product(v[0], fc, L, fl[0]);
        if (TABLE) {
            bool oor;
            acc_add_term(v[1], V_table_sum_term(P, fc, &oor), fl[1]);
            if (oor) flag_error(ctl, IEGPU_ERANGE, fc);
        } else {
            acc_add_product(v[1], fc, fc, fl[1]);
        }
    }
    acc_publish_flags<2>(ctl, fl);
    acc_block_sum<2>(v);
    acc_store_partial<2>(part, v);
    if (!arrive_last(counter)) return;
    if (threadIdx.x < 32) {
        double tot[2];
        acc_sum_partials<2>(part, gridDim.x, tot);
        if (threadIdx.x == 0) {
            *counter = 0;
            const unsigned nf = ctl->sumflags;
            ctl->sumflags = 0;
            if (nf & 1u) tot[0] = __longlong_as_double(0x7FF8000000000000LL);
            if (nf & 2u) tot[1] = __longlong_as_double(0x7FF8000000000000LL);
            if (ctl->error) {
                ctl->st.active = 0;
                ctl->done = 1;
            } else {
                step_scalars(ctl, P, K, tot[0], tot[1], a_trace);
            }
        }
    }
}

// Pass 2: kick of fd with the stored Laplacian, src/evolution.cpp:170-180,
// and the drift into the other f buffer; with SIGW the tensor kick and drift
// of src/evolution.cpp:183-254, 272-281.
template <bool TABLE, bool SIGW, int MODE>
__global__ void __launch_bounds__(kThreads) k_kick(const double* __restrict__ fs, const double* __restrict__ lap,
                                                   double* __restrict__ fdst, double* __restrict__ fd, SigwPtrs sg,
                                                   PotDev P, DevCtl* ctl, int lg, double half_over_dx) {
    const DevStep st = ctl->st;
    if (!st.active) return;
    // two consecutive sites per thread: 16-byte loads and stores, and the step
    // coefficients read once for both
    const long long id0 = 2 * ((long long)blockIdx.x * kThreads + threadIdx.x);
    const double2 fc2 = __ldg(reinterpret_cast<const double2*>(fs + id0));
    const double2 L2 = __ldg(reinterpret_cast<const double2*>(lap + id0));
    const double2 fdo2 = *reinterpret_cast<const double2*>(fd + id0);
    const double fcv[2] = {fc2.x, fc2.y}, Lv[2] = {L2.x, L2.y}, fdov[2] = {fdo2.x, fdo2.y};
    double fdn[2], fnew[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        bool oor;
        const double dv = dV_exact<TABLE>(P, fcv[e], &oor);
        if (TABLE && oor) flag_error(ctl, IEGPU_ERANGE, fcv[e]);
        fdn[e] = fdov[e] + st.d * (st.laplnorm * Lv[e] - st.friction * fdov[e] - st.potnorm * dv);
        fnew[e] = fcv[e] + st.d * fdn[e];
    }
    *reinterpret_cast<double2*>(fd + id0) = make_double2(fdn[0], fdn[1]);
    if (MODE == kModeLeapfrog) *reinterpret_cast<double2*>(fdst + id0) = make_double2(fnew[0], fnew[1]);
    if (SIGW) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            // dfdx<double>, src/evolution.cpp:55-77, and the six tensor updates
            // of src/evolution.cpp:183-254 (float storage, double right-hand side).
            const long long id = id0 + e;
            const Nbr n = neighbours(id, lg);
            const double gx = (__ldg(&fs[n.ip]) - __ldg(&fs[n.im])) * half_over_dx;
            const double gy = (__ldg(&fs[n.jp]) - __ldg(&fs[n.jm])) * half_over_dx;
            const double gz = (__ldg(&fs[n.kp]) - __ldg(&fs[n.km])) * half_over_dx;
            const double T[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const float* h = sg.hs[c];
                const float hc = __ldg(&h[id]);
                const float lf = lapl7(h, n, hc);
                const float hdo = sg.hd[c][id];
                const double rhs = st.d * (st.laplnorm * (double)lf - st.friction * (double)hdo + st.srcAmp * T[c]);
                const float hdn = hdo + (float)rhs;
                sg.hd[c][id] = hdn;
                if (MODE == kModeLeapfrog) sg.hdst[c][id] = hc + (float)(st.d * (double)hdn);
            }
        }
    }
}

// evolve_fields drift, src/evolution.cpp:265-281 (in place).
template <bool SIGW>
__global__ void __launch_bounds__(kThreads) k_drift(double* __restrict__ f, const double* __restrict__ fd,
                                                    SigwPtrs sg, long long gs, double d) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (id >= gs) return;
    f[id] = f[id] + d * fd[id];
    if (SIGW) {
#pragma unroll
        for (int c = 0; c < 6; ++c) sg.hdst[c][id] = sg.hdst[c][id] + (float)(d * (double)sg.hd[c][id]);
    }
}

// Lattice sums for kin_energy / gradient_energy / potential_energy, exact
// (as the leapfrog's): sum f lapl(f), the potential sum and sum fd^2.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads) k_energy_sums(const double* __restrict__ f, const double* __restrict__ fd,
                                                          PotDev P, DevCtl* ctl, unsigned long long* part, int lg) {
    const long long gs = 1LL << (3 * lg);
    Acc4 v[3];
    acc_zero(v[0]);
    acc_zero(v[1]);
    acc_zero(v[2]);
    unsigned fl[3] = {0u, 0u, 0u};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const Nbr n = neighbours(id, lg);
        const double fc = __ldg(&f[id]);
        acc_add_product(v[0], fc, lapl7(f, n, fc), fl[0]);
        if (TABLE) {
            bool oor;
            acc_add_term(v[1], V_table_sum_term(P, fc, &oor), fl[1]);
            if (oor) flag_error(ctl, IEGPU_ERANGE, fc);
        } else {
            acc_add_product(v[1], fc, fc, fl[1]);
        }
        const double q = __ldg(&fd[id]);
        acc_add_product(v[2], q, q, fl[2]);
    }
    acc_publish_flags<3>(ctl, fl);
    acc_block_sum<3>(v);
    acc_store_partial<3>(part, v);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static StepConst step_const(const iegpu_ctx* c) {
    StepConst K;
    K.dt = c->cfg.dt;
    K.s = c->cfg.rescale_s;
    K.dx = c->cfg.L / (double)c->N;
    K.gs = (double)c->gs;
    K.half_over_dx = 0.5 / K.dx;
    return K;
}

static SigwPtrs sigw_ptrs(iegpu_ctx* c, int src) {
    SigwPtrs s{};
    if (!c->cfg.sigw) return s;
    for (int q = 0; q < 6; ++q) {
        s.hs[q] = c->h[src][q];
        s.hdst[q] = c->h[src ^ 1][q];
        s.hd[q] = c->hd[q];
    }
    return s;
}

// The stored Laplacian of the leapfrog (N^3 doubles), allocated on first use.
static int ensure_lap(iegpu_ctx* c) {
    if (c->lap) return IEGPU_OK;
    if (check_cuda(c, cudaMalloc(&c->lap, sizeof(double) * c->gs), "Laplacian buffer")) return IEGPU_ENOMEM;
    return IEGPU_OK;
}

static void launch_reduce(iegpu_ctx* c, int src) {
    const StepConst K = step_const(c);
    unsigned long long* part = reinterpret_cast<unsigned long long*>(c->part);
    if (c->pot.table)
        k_lsum<true><<<c->red_grid, kThreads, 0, c->stream>>>(c->f[src], c->lap, c->pot, c->ctl, part, c->counter, c->a_trace, c->lg, K);
    else
        k_lsum<false><<<c->red_grid, kThreads, 0, c->stream>>>(c->f[src], c->lap, c->pot, c->ctl, part, c->counter, c->a_trace, c->lg, K);
    c->launches++;
}

template <int MODE>
static void launch_kick(iegpu_ctx* c, int src) {
    const unsigned grid = (unsigned)(c->gs / (2 * kThreads));   // two sites per thread (gs >= 8^3)
    const SigwPtrs sg = sigw_ptrs(c, src);
    const double hodx = 0.5 / (c->cfg.L / (double)c->N);
    double* fdst = c->f[src ^ 1];
    const double* L = c->lap;
    const bool tab = c->pot.table != 0, sig = c->cfg.sigw != 0;
    if (tab && sig) k_kick<true, true, MODE><<<grid, kThreads, 0, c->stream>>>(c->f[src], L, fdst, c->fd, sg, c->pot, c->ctl, c->lg, hodx);
    else if (tab) k_kick<true, false, MODE><<<grid, kThreads, 0, c->stream>>>(c->f[src], L, fdst, c->fd, sg, c->pot, c->ctl, c->lg, hodx);
    else if (sig) k_kick<false, true, MODE><<<grid, kThreads, 0, c->stream>>>(c->f[src], L, fdst, c->fd, sg, c->pot, c->ctl, c->lg, hodx);
    else k_kick<false, false, MODE><<<grid, kThreads, 0, c->stream>>>(c->f[src], L, fdst, c->fd, sg, c->pot, c->ctl, c->lg, hodx);
    c->launches++;
}

void fp64_destroy_graphs(iegpu_ctx* c) {
    for (int p = 0; p < 2; ++p) {
        if (c->lf_exec[p]) cudaGraphExecDestroy(c->lf_exec[p]);
        c->lf_exec[p] = nullptr;
    }
}

// Steps per graph launch; even, so a full graph returns to its start buffer.
static int graph_steps(const iegpu_ctx* c) { return c->N <= 64 ? 32 : 8; }

static int build_graphs(iegpu_ctx* c) {
    const int L = graph_steps(c);
    for (int p = 0; p < 2; ++p) {
        cudaGraph_t g;
        if (check_cuda(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture")) return IEGPU_ECUDA;
        const long long before = c->launches;
        for (int s = 0; s < L; ++s) {
            const int src = (p + s) & 1;
            launch_reduce(c, src);
            launch_kick<kModeLeapfrog>(c, src);
        }
        c->launches = before;
        if (check_cuda(c, cudaStreamEndCapture(c->stream, &g), "graph capture end")) return IEGPU_ECUDA;
        cudaError_t e = cudaGraphInstantiate(&c->lf_exec[p], g, 0);
        cudaGraphDestroy(g);
        if (check_cuda(c, e, "graph instantiate")) return IEGPU_ECUDA;
    }
    c->lf_steps = L;
    return IEGPU_OK;
}

static int upload_ctl(iegpu_ctx* c) {
    return check_cuda(c, cudaMemcpyAsync(c->ctl, c->ctl_h, sizeof(DevCtl), cudaMemcpyHostToDevice, c->stream), "control upload");
}

static int read_ctl(iegpu_ctx* c) {
    if (check_cuda(c, cudaMemcpyAsync(c->ctl_h, c->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, c->stream), "control download"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "leapfrog")) return IEGPU_ECUDA;
    if (c->ctl_h->error == IEGPU_ERANGE) {
        const double v = c->ctl_h->errval;
        return set_error(c, IEGPU_ERANGE, "Field value %.17g is outside the numerical potential range [%.17g, %.17g].\n", v,
                         c->htab_x.empty() ? 0.0 : c->htab_x.back(), c->htab_x.empty() ? 0.0 : c->htab_x.front());
    }
    if (c->ctl_h->error == IEGPU_ETOOBIG)
        return set_error(c, IEGPU_ETOOBIG, "a lattice-sum term of magnitude >= 2^30 is beyond the exact accumulator\n");
    return IEGPU_OK;
}

static void fill_ctl(iegpu_ctx* c, const iegpu_bg* bg, int mode) {
    DevCtl& C = *c->ctl_h;
    memset(&C, 0, sizeof C);
    C.bg.t = bg->t;
    C.bg.a = bg->a;
    C.bg.ad = bg->ad;
    C.bg.ad2 = bg->ad2;
    C.bg.astep = bg->astep;
    C.mode = mode;
}

static void copy_bg(const iegpu_ctx* c, iegpu_bg* bg) {
    const DevBg& B = c->ctl_h->bg;
    bg->t = B.t;
    bg->a = B.a;
    bg->ad = B.ad;
    bg->ad2 = B.ad2;
    bg->astep = B.astep;
}

int fp64_leapfrog(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace) {
    if (max_steps < 0) return set_error(c, IEGPU_EINVAL, "max_steps must be >= 0");
    if (steps) *steps = 0;
    if (max_steps == 0) return IEGPU_OK;
    if (max_steps > c->a_trace_cap) {
        if (c->a_trace) cudaFree(c->a_trace);
        c->a_trace = nullptr;
        c->a_trace_cap = 0;
        const int cap = max_steps < 1024 ? 1024 : max_steps;
        if (check_cuda(c, cudaMalloc(&c->a_trace, sizeof(double) * (size_t)cap), "a_trace alloc")) return IEGPU_ENOMEM;
        c->a_trace_cap = cap;
        fp64_destroy_graphs(c);  // graphs captured the old pointer
    }
    if (ensure_lap(c)) return IEGPU_ENOMEM;
    if (!c->lf_exec[0]) {
        int rc = build_graphs(c);
        if (rc) return rc;
    }
    fill_ctl(c, bg, kModeLeapfrog);
    c->ctl_h->af = af;
    c->ctl_h->steps_limit = max_steps;
    if (upload_ctl(c)) return IEGPU_ECUDA;
    const int L = c->lf_steps;
    const int launches = (max_steps + L - 1) / L;
    const int start = c->cur;
    for (int q = 0; q < launches; ++q) {
        // a full graph of L (even) steps returns to the start buffer
        if (check_cuda(c, cudaGraphLaunch(c->lf_exec[start], c->stream), "graph launch")) return IEGPU_ECUDA;
        c->launches += 2LL * L;
    }
    int rc = read_ctl(c);
    const int taken = c->ctl_h->steps_done;
    // kernels after the last active step exit at once; the buffer holding the
    // newest f is decided by how many steps ran.
    c->cur = (start + taken) & 1;
    if (rc) return rc;
    copy_bg(c, bg);
    if (steps) *steps = taken;
    if (a_trace && taken > 0) {
        if (check_cuda(c, cudaMemcpy(a_trace, c->a_trace, sizeof(double) * taken, cudaMemcpyDeviceToHost), "a_trace download"))
            return IEGPU_ECUDA;
    }
    return IEGPU_OK;
}

int fp64_profile(iegpu_ctx* c, double af, int nsteps, iegpu_bg* bg, double* ms, int nk) {
    for (int q = 0; q < nk; ++q) ms[q] = 0.0;
    if (ensure_lap(c)) return IEGPU_ENOMEM;
    fill_ctl(c, bg, kModeLeapfrog);
    c->ctl_h->af = af;
    c->ctl_h->steps_limit = nsteps;
    if (upload_ctl(c)) return IEGPU_ECUDA;
    const int start = c->cur;
    for (int s = 0; s < nsteps; ++s) {
        const int src = (start + s) & 1;
        float t0 = 0.f, t1 = 0.f;
        cudaEventRecord(c->ev[0], c->stream);
        launch_reduce(c, src);
        cudaEventRecord(c->ev[1], c->stream);
        launch_kick<kModeLeapfrog>(c, src);
        cudaEventRecord(c->ev[2], c->stream);
        if (check_cuda(c, cudaEventSynchronize(c->ev[2]), "profile")) return IEGPU_ECUDA;
        cudaEventElapsedTime(&t0, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&t1, c->ev[1], c->ev[2]);
        if (nk > 0) ms[0] += t0;
        if (nk > 1) ms[1] += t1;
    }
    int rc = read_ctl(c);
    const int taken = c->ctl_h->steps_done;
    c->cur = (start + taken) & 1;
    if (rc) return rc;
    copy_bg(c, bg);
    return IEGPU_OK;
}

int fp64_evolve_derivs(iegpu_ctx* c, double d, iegpu_bg* bg) {
    if (ensure_lap(c)) return IEGPU_ENOMEM;
    fill_ctl(c, bg, kModeKick);
    c->ctl_h->d_given = d;
    if (upload_ctl(c)) return IEGPU_ECUDA;
    launch_reduce(c, c->cur);
    launch_kick<kModeKick>(c, c->cur);
    int rc = read_ctl(c);
    if (rc) return rc;
    copy_bg(c, bg);
    return IEGPU_OK;
}

int fp64_evolve_fields(iegpu_ctx* c, double d, iegpu_bg* bg) {
    // scalar part on the host, exactly as src/evolution.cpp:262,283
    bg->t += d;
    const unsigned grid = (unsigned)((c->gs + kThreads - 1) / kThreads);
    SigwPtrs sg{};
    if (c->cfg.sigw)
        for (int q = 0; q < 6; ++q) { sg.hdst[q] = c->h[c->cur][q]; sg.hd[q] = c->hd[q]; }
    if (c->cfg.sigw) k_drift<true><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, sg, (long long)c->gs, d);
    else k_drift<false><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, sg, (long long)c->gs, d);
    c->launches++;
    bg->a += d * bg->ad;
    return sync_and_check(c, "evolve_fields");
}

int fp64_energies(iegpu_ctx* c, const iegpu_bg* bg, double out[3]) {
    const int grid = c->red_grid;
    c->ctl_h->error = 0;
    // error and sumflags are adjacent ints of the control block
    if (check_cuda(c, cudaMemsetAsync(&c->ctl->error, 0, 2 * sizeof(int), c->stream), "memset")) return IEGPU_ECUDA;
    unsigned long long* part = reinterpret_cast<unsigned long long*>(c->part);
    if (c->pot.table) k_energy_sums<true><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, c->pot, c->ctl, part, c->lg);
    else k_energy_sums<false><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, c->pot, c->ctl, part, c->lg);
    c->launches++;
    std::vector<unsigned long long> h((size_t)grid * 12);
    if (check_cuda(c, cudaMemcpyAsync(h.data(), part, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost, c->stream),
                   "energy partials"))
        return IEGPU_ECUDA;
    int rc = read_ctl(c);
    if (rc) return rc;
    double tot[3];
    for (int q = 0; q < 3; ++q) {
        unsigned long long w[4] = {0, 0, 0, 0};
        for (int b = 0; b < grid; ++b) {
            unsigned carry = 0;
            for (int l = 0; l < 4; ++l) {
                const unsigned long long x = h[((size_t)b * 3 + q) * 4 + l];
                const unsigned long long t = w[l] + x;
                const unsigned c1 = t < x;
                w[l] = t + carry;
                carry = c1 | (w[l] < t);
            }
        }
        Acc4 A;
        for (int l = 0; l < 4; ++l) A.w[l] = w[l];
        tot[q] = (c->ctl_h->sumflags >> q) & 1u ? __builtin_nan("") : acc_to_double(A);
    }
    const double G = tot[0], Pn = tot[1], K2 = tot[2];
    const double gs = (double)c->gs, a = bg->a, s = c->cfg.rescale_s, dx = c->cfg.L / (double)c->N;
    const double B2 = c->pot.B2;
    // kin_energy, src/evolution.cpp:139-145
    out[0] = 0.5 * pow(a, 2.0 * s - 2.0) * (K2 / gs);
    // gradient_energy, src/evolution.cpp:130-136
    const double norm = (1.0 / (a * dx)) * (1.0 / (a * dx));
    out[1] = 0.5 * (-G) * norm / gs;
    // potential_energy, src/potential.cpp:151-171
    if (c->pot.table) out[2] = (Pn / B2) / gs;
    else out[2] = (c->pot.V0 * (gs - c->pot.c1 * Pn) / B2) / gs;
    return IEGPU_OK;
}

}  // namespace iegpu

namespace iegpu {

// ---------------------------------------------------------------------------
// post-inflation phase: src/initialize.cpp:245-290, src/evolution.cpp:1378-1653
// ---------------------------------------------------------------------------
//
// The background has no lattice sums in this phase (a'' = -(s - (1 - 3w)/2)
// a'^2 / a), so every scalar is formed on the host with the reference's
// expressions, and the kernels take the step's coefficients as arguments: a
// run of steps is enqueued with no synchronisation.  Per-site expressions are
// the reference's, in its order (this unit is compiled with -fmad=false).

// initialize_post_inflation's field, src/initialize.cpp:258-283:
// f = Phi (x - mean), or Phi (x - mean) / den without deltaN.
__global__ void __launch_bounds__(kThreads) k_post_field(double* __restrict__ f, const double* x, long long gs,
                                                         double Phi, double mean, double den, int divide) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (id >= gs) return;
    const double v = x[id];
    f[id] = divide ? Phi * (v - mean) / den : Phi * (v - mean);
}

// fd kick of evolve_derivs_post_inflation, src/evolution.cpp:1448-1457:
// fd += d (w laplnorm lapl(f) - (3 (1 + w) + s) ad fd / a), with
// c_lap = w laplnorm and c_fr = (3 (1 + w) + s) ad formed on the host.
// The divisions by a and by 4 dx^2 (ten per site with SIGW) are exact
// divisions by fixed divisors on the integer pipes (div_exact, exact.cuh).
__global__ void __launch_bounds__(kThreads) k_post_kick(const double* __restrict__ f, double* __restrict__ fd, int lg,
                                                        double d, double c_lap, double c_fr, DivConst Da) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    const Nbr n = neighbours(id, lg);
    const double lap = lapl7(f, n, __ldg(&f[id]));
    const double fdo = fd[id];
    fd[id] = fdo + d * (c_lap * lap - div_exact(c_fr * fdo, Da));
}

struct PostSigwK {
    double d, laplnorm, c_hf, invH, coeffU, srcAmp, half_over_dx, inv_dx2;
    DivConst Da, Dden;   // a and 4 dx^2
};

// (fpp - fpm - fmp + fmm) / den of d2_cross_state, src/evolution.cpp:93-106
__device__ __forceinline__ double cross4(const double* __restrict__ f, long long pp, long long pm, long long mp,
                                         long long mm, const DivConst& den) {
    return div_exact(__ldg(&f[pp]) - __ldg(&f[pm]) - __ldg(&f[mp]) + __ldg(&f[mm]), den);
}

// Tensor kick of evolve_derivs_post_inflation, src/evolution.cpp:1459-1551,
// with the derivative pack of build_deriv_pack (:1398-1418): central first
// derivatives of f and of the fd just kicked, the Hessian of f (d2_same_state
// :79-91; d2_cross_state :93-106, whose neighbours are chosen per index from
// whether d1 or d2 names it: for (y, z) the i index does not move, so the
// corners pair up and the value is the rounding residue the reference gets).
__global__ void __launch_bounds__(kThreads) k_post_sigw(const double* __restrict__ f, const double* __restrict__ fd,
                                                        SigwPtrs sg, int lg, PostSigwK K) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    const Nbr n = neighbours(id, lg);
    const long long dip = n.ip - id, dim = n.im - id, djp = n.jp - id, djm = n.jm - id, dkp = n.kp - id,
                    dkm = n.km - id;
    const double fc = __ldg(&f[id]);
    const double gx = (__ldg(&f[n.ip]) - __ldg(&f[n.im])) * K.half_over_dx;
    const double gy = (__ldg(&f[n.jp]) - __ldg(&f[n.jm])) * K.half_over_dx;
    const double gz = (__ldg(&f[n.kp]) - __ldg(&f[n.km])) * K.half_over_dx;
    const double gdx = (__ldg(&fd[n.ip]) - __ldg(&fd[n.im])) * K.half_over_dx;
    const double gdy = (__ldg(&fd[n.jp]) - __ldg(&fd[n.jm])) * K.half_over_dx;
    const double gdz = (__ldg(&fd[n.kp]) - __ldg(&fd[n.km])) * K.half_over_dx;
    const double Hxx = (__ldg(&f[n.ip]) - 2.0 * fc + __ldg(&f[n.im])) * K.inv_dx2;
    const double Hyy = (__ldg(&f[n.jp]) - 2.0 * fc + __ldg(&f[n.jm])) * K.inv_dx2;
    const double Hzz = (__ldg(&f[n.kp]) - 2.0 * fc + __ldg(&f[n.km])) * K.inv_dx2;
    // corners (ip, jp, kp), (ip, jm, km), (im, jp, kp), (im, jm, km) with the
    // indices d1, d2 do not name left in place
    const double Hxy = cross4(f, id + dip + djp, id + dip + djm, id + dim + djp, id + dim + djm, K.Dden);
    const double Hxz = cross4(f, id + dip + dkp, id + dip + dkm, id + dim + dkp, id + dim + dkm, K.Dden);
    const double Hyz = cross4(f, id + djp + dkp, id + djm + dkm, id + djp + dkp, id + djm + dkm, K.Dden);
    const double dux = gdx * K.invH + gx;
    const double duy = gdy * K.invH + gy;
    const double duz = gdz * K.invH + gz;
    const double S[6] = {4.0 * fc * Hxx + 2.0 * gx * gx - K.coeffU * (dux * dux),
                         4.0 * fc * Hyy + 2.0 * gy * gy - K.coeffU * (duy * duy),
                         4.0 * fc * Hzz + 2.0 * gz * gz - K.coeffU * (duz * duz),
                         4.0 * fc * Hxy + 2.0 * gx * gy - K.coeffU * (dux * duy),
                         4.0 * fc * Hxz + 2.0 * gx * gz - K.coeffU * (dux * duz),
                         4.0 * fc * Hyz + 2.0 * gy * gz - K.coeffU * (duy * duz)};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float* h = sg.hs[c];
        const float lf = lapl7(h, n, __ldg(&h[id]));
        const float hdo = sg.hd[c][id];
        const double rhs = K.d * (K.laplnorm * (double)lf - div_exact(K.c_hf * (double)hdo, K.Da) + K.srcAmp * S[c]);
        sg.hd[c][id] = hdo + (float)rhs;
    }
}

// initialize_post_inflation(), src/initialize.cpp:245-290 (without its save):
// the means are serial sums over the downloaded field in the reference's
// loop order, so that f is the reference's bit for bit.
int fp64_post_init(iegpu_ctx* c, double horizon_factor, double omega, int from_deltaN, iegpu_bg* bg) {
    const size_t gs = c->gs;
    double* f = c->f[c->cur];
    std::vector<double> x(gs);
    const double* src = from_deltaN ? c->dn : f;
    if (check_cuda(c, cudaMemcpyAsync(x.data(), src, sizeof(double) * gs, cudaMemcpyDeviceToHost, c->stream), "post init"))
        return IEGPU_ECUDA;
    std::vector<double> y;
    if (!from_deltaN) {
        y.resize(gs);
        if (check_cuda(c, cudaMemcpyAsync(y.data(), c->fd, sizeof(double) * gs, cudaMemcpyDeviceToHost, c->stream), "post init"))
            return IEGPU_ECUDA;
    }
    if (sync_and_check(c, "post init")) return IEGPU_ECUDA;
    const double Phi_from_zeta = 3.0 * (1.0 + omega) / (5.0 + 3.0 * omega);
    double mean = 0.0, den = 1.0;
    if (from_deltaN) {
        for (size_t id = 0; id < gs; ++id) mean += x[id];
        mean = mean / (double)gs;
    } else {
        double fdmean = 0.0;
        for (size_t id = 0; id < gs; ++id) {
            mean += x[id];
            fdmean += y[id];
        }
        mean = mean / (double)gs;
        fdmean = fdmean / (double)gs;
        const double s = c->cfg.rescale_s;
        den = fdmean * pow(bg->a, s - 1.0) / (bg->ad * pow(bg->a, s - 2.0));
    }
    const unsigned grid = (unsigned)((gs + kThreads - 1) / kThreads);
    k_post_field<<<grid, kThreads, 0, c->stream>>>(f, src, (long long)gs, Phi_from_zeta, mean, den, !from_deltaN);
    c->launches++;
    for (int q = 0; q < 6 && c->cfg.sigw; ++q) {
        cudaMemsetAsync(c->h[c->cur][q], 0, sizeof(float) * gs, c->stream);
        cudaMemsetAsync(c->hd[q], 0, sizeof(float) * gs, c->stream);
    }
    const double pi = 2.0 * asin(1.0);
    bg->t = 0.0;
    bg->a = 1.0;
    bg->ad = horizon_factor * c->N * 2.0 * pi / c->cfg.L;
    return sync_and_check(c, "post init");
}

// evolve_derivs_post_inflation(d), src/evolution.cpp:1436-1555, enqueued.
static void post_kick(iegpu_ctx* c, double d, double omega, iegpu_bg* bg) {
    const double s = c->cfg.rescale_s, dx = c->cfg.L / (double)c->N;
    const double a = bg->a;
    const double laplnorm = pow(a, -2.0 * s) / (dx * dx);
    bg->ad2 = -(s - 0.5 * (1.0 - 3.0 * omega)) * (bg->ad * bg->ad) / a;
    bg->ad += 0.5 * d * bg->ad2;
    const double ad = bg->ad;
    const unsigned grid = (unsigned)(c->gs / kThreads);
    double* f = c->f[c->cur];
    const DivConst Da = make_div_const(a);
    k_post_kick<<<grid, kThreads, 0, c->stream>>>(f, c->fd, c->lg, d, omega * laplnorm, (3.0 * (1.0 + omega) + s) * ad, Da);
    c->launches++;
    if (c->cfg.sigw) {
        SigwPtrs sg{};
        for (int q = 0; q < 6; ++q) { sg.hs[q] = c->h[c->cur][q]; sg.hd[q] = c->hd[q]; }
        const double Htilde = ad / a;
        PostSigwK K;
        K.d = d;
        K.laplnorm = laplnorm;
        K.c_hf = (2.0 + s) * ad;
        K.Da = Da;
        K.invH = 1.0 / Htilde;
        K.coeffU = 4.0 / (3.0 * (1.0 + omega));
        K.srcAmp = 2.0 * pow(a, -2.0 * s);
        K.half_over_dx = 0.5 / dx;
        K.inv_dx2 = 1.0 / (dx * dx);
        K.Dden = make_div_const(4.0 * dx * dx);
        k_post_sigw<<<grid, kThreads, 0, c->stream>>>(f, c->fd, sg, c->lg, K);
        c->launches++;
    }
    bg->ad += 0.5 * d * bg->ad2;
}

// evolve_fields(d), src/evolution.cpp:260-284, enqueued.
static void post_drift(iegpu_ctx* c, double d, iegpu_bg* bg) {
    bg->t += d;
    const unsigned grid = (unsigned)((c->gs + kThreads - 1) / kThreads);
    SigwPtrs sg{};
    if (c->cfg.sigw)
        for (int q = 0; q < 6; ++q) { sg.hdst[q] = c->h[c->cur][q]; sg.hd[q] = c->hd[q]; }
    if (c->cfg.sigw) k_drift<true><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, sg, (long long)c->gs, d);
    else k_drift<false><<<grid, kThreads, 0, c->stream>>>(c->f[c->cur], c->fd, sg, (long long)c->gs, d);
    c->launches++;
    bg->a += d * bg->ad;
}

int fp64_post_derivs(iegpu_ctx* c, double d, double omega, iegpu_bg* bg) {
    post_kick(c, d, omega, bg);
    return sync_and_check(c, "post-inflation kick");
}

// The leapfrog loop body of run_post_inflation_loop, src/evolution.cpp:1589-1597:
// while a <= af_post: kick, drift; at most max_steps steps.
int fp64_post_leapfrog(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps, iegpu_bg* bg,
                       int* steps, double* a_trace) {
    int n = 0;
    while (n < max_steps && bg->a <= af_post) {
        post_kick(c, dt_post, omega, bg);
        post_drift(c, dt_post, bg);
        if (a_trace) a_trace[n] = bg->a;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "post-inflation leapfrog");
}

}  // namespace iegpu

namespace iegpu {

// ---------------------------------------------------------------------------
// Runge-Kutta integrators (inflation_integrator / post_inflation_integrator =
// rk4 | rk45): rk4_step_inflation and rk45_step_inflation,
// src/evolution.cpp:760-904, with compute_inflation_rhs (:418-599: the
// inflation equations, or the post-inflation ones that the RK branches of
// run_post_inflation_loop select), the stage states of
// prepare_inflation_stage_state (:639-671), the background stages of
// prepare_inflation_background_state (:673-690), the weighted update of
// apply_inflation_weighted_update (:717-758) and the step control of
// :326-363.
// ---------------------------------------------------------------------------
//
// A stage's derivatives are k_f = fd and k_fd (k_h = hd and k_hd with SIGW).
// k_f of a stage is that stage's fd, so it is read from the stage state
// instead of being stored.  Scratch per site for an s-stage method, in
// doubles: f of the current stage, fd of stages 1..s-1, k_fd of stages
// 0..s-1 and the RK45 candidate fd (2s + 1); with SIGW, in floats: h of the
// current stage, hd of stages 1..s-1, k_hd of stages 0..s-1 and the candidate
// hd (6 (2s + 1)).  The RK45 candidate f and h go to the stage f and h
// buffers.  The background stages of the inflation equations need each
// stage's two lattice sums, so they are formed on the host with the
// reference's expressions from a 16-byte read-back per stage; the
// post-inflation equations have no lattice sums.  So does the RK45 error
// norm: its lattice part is summed on the device, the rest is the
// reference's host arithmetic.

struct RkSigw {
    const float* hs[6];
    const float* hds[6];
    float* khd[6];
};

struct RkCoef {
    double laplnorm, friction, potnorm, srcAmp, half_over_dx;
};

// compute_inflation_rhs on one stage state, inflation equations: k_fd (and
// k_hd) per site, and the sums of f lapl(f) and V(f); the last CTA combines
// the block partials in a fixed order into sums[0..1].
template <bool TABLE, bool SIGW>
__global__ void __launch_bounds__(kThreads) k_rk_rhs(const double* __restrict__ fs, const double* __restrict__ fds,
                                                     double* __restrict__ kfd, RkSigw sg, PotDev P, DevCtl* ctl,
                                                     double* part, unsigned* counter, double* sums, int lg, RkCoef K) {
    const long long gs = 1LL << (3 * lg);
    double v[2] = {0.0, 0.0};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const Nbr n = neighbours(id, lg);
        const double field = __ldg(&fs[id]);
        const double lap = lapl7(fs, n, field);
        double pot, dpot;
        if (TABLE) {
            bool oor;
            const int l = table_bracket(P, field, &oor);
            if (oor) flag_error(ctl, IEGPU_ERANGE, field);
            pot = div_exact(table_interp(P, P.V, P.dyV, field, l), P.divB2);
            dpot = div_exact(table_interp(P, P.dV, P.dydV, field, l), P.divB2);
        } else {
            bool oor;
            pot = V_exact<false>(P, field, &oor);
            dpot = dV_exact<false>(P, field, &oor);
        }
        kfd[id] = K.laplnorm * lap - K.friction * __ldg(&fds[id]) - K.potnorm * dpot;
        v[0] += field * lap;
        v[1] += pot;
        if (SIGW) {
            const double gx = (__ldg(&fs[n.ip]) - __ldg(&fs[n.im])) * K.half_over_dx;
            const double gy = (__ldg(&fs[n.jp]) - __ldg(&fs[n.jm])) * K.half_over_dx;
            const double gz = (__ldg(&fs[n.kp]) - __ldg(&fs[n.km])) * K.half_over_dx;
            const double T[6] = {gx * gx, gy * gy, gz * gz, gx * gy, gx * gz, gy * gz};
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const float* h = sg.hs[c];
                const float lf = lapl7(h, n, __ldg(&h[id]));
                sg.khd[c][id] = (float)(K.laplnorm * (double)lf - K.friction * (double)__ldg(&sg.hds[c][id]) +
                                        K.srcAmp * T[c]);
            }
        }
    }
    block_sum<2>(v);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = v[0];
        part[2 * blockIdx.x + 1] = v[1];
    }
    if (!arrive_last(counter)) return;
    if (threadIdx.x < 32) {
        double tot[2];
        sum_partials<2>(part, gridDim.x, tot);
        if (threadIdx.x == 0) {
            *counter = 0;
            sums[0] = tot[0];
            sums[1] = tot[1];
        }
    }
}

struct RkPostCoef {
    double omega, laplnorm, scalar_friction, tensor_friction, invH, coeffU, srcAmp, half_over_dx, inv_dx2;
    DivConst Dden;   // 4 dx^2
};

// compute_inflation_rhs, post-inflation equations (src/evolution.cpp:515-598):
// k_fd = omega laplnorm lapl(f) - scalar_friction fd; the tensor source is
// the Hessian form with the gradients of the stage's f and fd (the pack of
// k_post_sigw, here without the kick).
template <bool SIGW>
__global__ void __launch_bounds__(kThreads) k_rk_rhs_post(const double* __restrict__ fs,
                                                          const double* __restrict__ fds, double* __restrict__ kfd,
                                                          RkSigw sg, int lg, RkPostCoef K) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    const Nbr n = neighbours(id, lg);
    const double fc = __ldg(&fs[id]);
    const double lap = lapl7(fs, n, fc);
    kfd[id] = K.omega * K.laplnorm * lap - K.scalar_friction * __ldg(&fds[id]);
    if (SIGW) {
        const long long dip = n.ip - id, dim = n.im - id, djp = n.jp - id, djm = n.jm - id, dkp = n.kp - id,
                        dkm = n.km - id;
        const double gx = (__ldg(&fs[n.ip]) - __ldg(&fs[n.im])) * K.half_over_dx;
        const double gy = (__ldg(&fs[n.jp]) - __ldg(&fs[n.jm])) * K.half_over_dx;
        const double gz = (__ldg(&fs[n.kp]) - __ldg(&fs[n.km])) * K.half_over_dx;
        const double gdx = (__ldg(&fds[n.ip]) - __ldg(&fds[n.im])) * K.half_over_dx;
        const double gdy = (__ldg(&fds[n.jp]) - __ldg(&fds[n.jm])) * K.half_over_dx;
        const double gdz = (__ldg(&fds[n.kp]) - __ldg(&fds[n.km])) * K.half_over_dx;
        const double Hxx = (__ldg(&fs[n.ip]) - 2.0 * fc + __ldg(&fs[n.im])) * K.inv_dx2;
        const double Hyy = (__ldg(&fs[n.jp]) - 2.0 * fc + __ldg(&fs[n.jm])) * K.inv_dx2;
        const double Hzz = (__ldg(&fs[n.kp]) - 2.0 * fc + __ldg(&fs[n.km])) * K.inv_dx2;
        const double Hxy = cross4(fs, id + dip + djp, id + dip + djm, id + dim + djp, id + dim + djm, K.Dden);
        const double Hxz = cross4(fs, id + dip + dkp, id + dip + dkm, id + dim + dkp, id + dim + dkm, K.Dden);
        const double Hyz = cross4(fs, id + djp + dkp, id + djm + dkm, id + djp + dkp, id + djm + dkm, K.Dden);
        const double dux = gdx * K.invH + gx;
        const double duy = gdy * K.invH + gy;
        const double duz = gdz * K.invH + gz;
        const double S[6] = {4.0 * fc * Hxx + 2.0 * gx * gx - K.coeffU * (dux * dux),
                             4.0 * fc * Hyy + 2.0 * gy * gy - K.coeffU * (duy * duy),
                             4.0 * fc * Hzz + 2.0 * gz * gz - K.coeffU * (duz * duz),
                             4.0 * fc * Hxy + 2.0 * gx * gy - K.coeffU * (dux * duy),
                             4.0 * fc * Hxz + 2.0 * gx * gz - K.coeffU * (dux * duz),
                             4.0 * fc * Hyz + 2.0 * gy * gz - K.coeffU * (duy * duz)};
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const float* h = sg.hs[c];
            const float lf = lapl7(h, n, __ldg(&h[id]));
            sg.khd[c][id] = (float)(K.laplnorm * (double)lf - K.tensor_friction * (double)__ldg(&sg.hds[c][id]) +
                                    K.srcAmp * S[c]);
        }
    }
}

constexpr int kRkMax = IE_RK_STAGES;

// One row of a tableau: out = base + h sum_q c_q k_q over the nonzero c_q,
// the sum started from 0.0 in q order (prepare_inflation_stage_state and
// apply_inflation_weighted_update).  out may alias base.
struct RkRow {
    const double* kf[kRkMax];
    const double* kfd[kRkMax];
    const float* kh[kRkMax][6];
    const float* khd[kRkMax][6];
    double c[kRkMax];
    int nq;
};

struct RkH {
    const float* hb[6];
    const float* hdb[6];
    float* ho[6];
    float* hdo[6];
};

// y_out = y + h * sum_t c_t k_t over the NT nonzero coefficients of a stage
// row, in stage order (the host drops the zero ones, which the reference's
// loop skips too), each sum formed from 0.0 term by term as the reference
// forms it.  Every load of a site is issued before its arithmetic; plain
// loads throughout: the RK4 update writes f, fd, h and hd in place, and k_f,
// k_h of stage 0 are fd, hd themselves (each site is read by its own thread
// before that thread writes it).
template <int NT, bool SIGW>
__global__ void __launch_bounds__(kThreads) k_rk_combine(const double* f, const double* fd, double* fout,
                                                         double* fdout, RkRow R, RkH H, double h) {
    const long long id = (long long)blockIdx.x * kThreads + threadIdx.x;
    double kf[NT > 0 ? NT : 1], kfd[NT > 0 ? NT : 1];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        kf[t] = R.kf[t][id];
        kfd[t] = R.kfd[t][id];
    }
    const double f0 = f[id], fd0 = fd[id];
    double sum_f = 0.0, sum_fd = 0.0;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        sum_f += R.c[t] * kf[t];
        sum_fd += R.c[t] * kfd[t];
    }
    fout[id] = f0 + h * sum_f;
    fdout[id] = fd0 + h * sum_fd;
    if (SIGW) {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float kh[NT > 0 ? NT : 1], khd[NT > 0 ? NT : 1];
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                kh[t] = R.kh[t][c][id];
                khd[t] = R.khd[t][c][id];
            }
            const double hb = (double)H.hb[c][id], hdb = (double)H.hdb[c][id];
            double sum_h = 0.0, sum_hd = 0.0;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                sum_h += R.c[t] * (double)kh[t];
                sum_hd += R.c[t] * (double)khd[t];
            }
            H.ho[c][id] = (float)(hb + h * sum_h);
            H.hdo[c][id] = (float)(hdb + h * sum_hd);
        }
    }
}

// std::max / std::min as the reference calls them
__host__ __device__ __forceinline__ double ref_max(double a, double b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ double ref_min(double a, double b) { return (b < a) ? b : a; }

struct Rk45Fin {
    const double* kf[kRkMax];
    const double* kfd[kRkMax];
    const float* kh[kRkMax][6];
    const float* khd[kRkMax][6];
    const float* hs[6];
    const float* hds[6];
    double* y5f;
    double* y5fd;
    float* y5h[6];
    float* y5hd[6];
    double b[kRkMax], e[kRkMax];
    double h, atol, rtol;
};

// The lattice part of rk45_step_inflation (src/evolution.cpp:826-874): the
// 5th-order candidate y5 = y + sum_q h b_q k_q and the embedded error
// sum_q h e_q k_q per variable, each term added in q order, and the sum over
// variables of (err / (atol + rtol max(|y|, |y5|)))^2, combined by the last
// CTA in a fixed order into sums[0].
template <bool SIGW>
__global__ void __launch_bounds__(kThreads) k_rk45_final(const double* f, const double* fd, Rk45Fin F, double* part,
                                                         unsigned* counter, double* sums, long long gs) {
    double v[1] = {0.0};
    for (long long id = (long long)blockIdx.x * kThreads + threadIdx.x; id < gs; id += (long long)gridDim.x * kThreads) {
        const double f0 = f[id], fd0 = fd[id];
        double y5f = f0, y5fd = fd0, errf = 0.0, errfd = 0.0;
#pragma unroll
        for (int q = 0; q < kRkMax; ++q) {
            const double bs = F.b[q], es = F.e[q];
            if (bs != 0.0) {
                y5f += F.h * bs * F.kf[q][id];
                y5fd += F.h * bs * F.kfd[q][id];
            }
            if (es != 0.0) {
                errf += F.h * es * F.kf[q][id];
                errfd += F.h * es * F.kfd[q][id];
            }
        }
        F.y5f[id] = y5f;
        F.y5fd[id] = y5fd;
        const double sf = F.atol + F.rtol * ref_max(fabs(f0), fabs(y5f));
        const double sfd = F.atol + F.rtol * ref_max(fabs(fd0), fabs(y5fd));
        const double qf = errf / sf, qfd = errfd / sfd;
        v[0] += qf * qf + qfd * qfd;
        if (SIGW) {
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const double h0 = (double)F.hs[c][id], hd0 = (double)F.hds[c][id];
                double y5h = h0, y5hd = hd0, errh = 0.0, errhd = 0.0;
#pragma unroll
                for (int q = 0; q < kRkMax; ++q) {
                    const double bs = F.b[q], es = F.e[q];
                    if (bs != 0.0) {
                        y5h += F.h * bs * (double)F.kh[q][c][id];
                        y5hd += F.h * bs * (double)F.khd[q][c][id];
                    }
                    if (es != 0.0) {
                        errh += F.h * es * (double)F.kh[q][c][id];
                        errhd += F.h * es * (double)F.khd[q][c][id];
                    }
                }
                F.y5h[c][id] = (float)y5h;
                F.y5hd[c][id] = (float)y5hd;
                const double sh = F.atol + F.rtol * ref_max(fabs(h0), fabs(y5h));
                const double shd = F.atol + F.rtol * ref_max(fabs(hd0), fabs(y5hd));
                const double qh = errh / sh, qhd = errhd / shd;
                v[0] += qh * qh + qhd * qhd;
            }
        }
    }
    block_sum<1>(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v[0];
    if (!arrive_last(counter)) return;
    if (threadIdx.x < 32) {
        double tot[1];
        sum_partials<1>(part, gridDim.x, tot);
        if (threadIdx.x == 0) {
            *counter = 0;
            sums[0] = tot[0];
        }
    }
}

static const double kRk4A[kRkMax][kRkMax] = IE_RK4_A_INIT;
static const double kRk4B[kRkMax] = IE_RK4_B_INIT;
static const double kDpA[kRkMax][kRkMax] = IE_DP_A_INIT;
static const double kDpB[kRkMax] = IE_DP_B_INIT;
static const double kDpE[kRkMax] = IE_DP_E_INIT;

struct RkBufs {
    double* f;                 // stage f; the RK45 candidate f
    double* fd[kRkMax];        // stage fd: [0] is the state's own fd
    double* kfd[kRkMax];
    double* y5fd;              // RK45 candidate fd
    float* h[6];               // stage h; the RK45 candidate h
    float* hd[kRkMax][6];      // stage hd: [0] is the state's own hd
    float* khd[kRkMax][6];
    float* y5hd[6];
};

// Which equations the stages use: inflation, or post-inflation with omega.
struct RkEq {
    bool post;
    double omega;
};

static int rk_bufs(iegpu_ctx* c, int nst, RkBufs& B) {
    const size_t gs = c->gs;
    const size_t nd = 2 * (size_t)nst + 1, nf = 6 * nd;
    if (c->rk_nst < nst) {
        cudaFree(c->rk_d);
        cudaFree(c->rk_h);
        c->rk_d = nullptr;
        c->rk_h = nullptr;
        c->rk_nst = 0;
        if (cudaMalloc(&c->rk_d, sizeof(double) * nd * gs) != cudaSuccess) {
            cudaGetLastError();
            c->rk_d = nullptr;
            return set_error(c, IEGPU_ENOMEM, "device allocation of the RK scratch (%zu bytes) failed", sizeof(double) * nd * gs);
        }
        if (c->cfg.sigw && cudaMalloc(&c->rk_h, sizeof(float) * nf * gs) != cudaSuccess) {
            cudaGetLastError();
            c->rk_h = nullptr;
            return set_error(c, IEGPU_ENOMEM, "device allocation of the RK tensor scratch (%zu bytes) failed", sizeof(float) * nf * gs);
        }
        c->rk_nst = nst;
    }
    memset(&B, 0, sizeof B);
    B.f = c->rk_d;
    B.fd[0] = c->fd;
    for (int q = 1; q < nst; ++q) B.fd[q] = c->rk_d + q * gs;
    for (int q = 0; q < nst; ++q) B.kfd[q] = c->rk_d + (nst + q) * gs;
    B.y5fd = c->rk_d + 2 * (size_t)nst * gs;
    for (int k = 0; k < 6 && c->cfg.sigw; ++k) {
        float* const base = c->rk_h;
        B.h[k] = base + k * gs;
        B.hd[0][k] = c->hd[k];
        for (int q = 1; q < nst; ++q) B.hd[q][k] = base + (6 * (size_t)q + k) * gs;
        for (int q = 0; q < nst; ++q) B.khd[q][k] = base + (6 * ((size_t)nst + q) + k) * gs;
        B.y5hd[k] = base + (12 * (size_t)nst + k) * gs;
    }
    return IEGPU_OK;
}

// compute_inflation_rhs for one stage.  Inflation equations: launches the
// kernel, reads the two sums back and forms dadt, daddt on the host
// (src/evolution.cpp:500-511).  Post-inflation equations: enqueued; a'' from
// a, a' (:596-597).
static int rk_rhs(iegpu_ctx* c, const RkEq& E, const double* fs, const double* fds, const float* const* hs,
                  const float* const* hds, double* kfd, float* const* khd, double a_st, double ad_st, double* dadt,
                  double* daddt) {
    const double s = c->cfg.rescale_s, dx = c->cfg.L / (double)c->N;
    const bool sig = c->cfg.sigw != 0;
    RkSigw sg{};
    for (int k = 0; k < 6 && sig; ++k) {
        sg.hs[k] = hs[k];
        sg.hds[k] = hds[k];
        sg.khd[k] = khd[k];
    }
    if (E.post) {
        const double omega = E.omega;
        RkPostCoef K;
        K.omega = omega;
        K.laplnorm = pow(a_st, -2.0 * s) / (dx * dx);
        K.scalar_friction = (3.0 * (1.0 + omega) + s) * ad_st / a_st;
        K.tensor_friction = (2.0 + s) * ad_st / a_st;
        const double Htilde = ad_st / a_st;
        K.invH = 1.0 / Htilde;
        K.coeffU = 4.0 / (3.0 * (1.0 + omega));
        K.srcAmp = 2.0 * pow(a_st, -2.0 * s);
        K.half_over_dx = 0.5 / dx;
        K.inv_dx2 = 1.0 / (dx * dx);
        K.Dden = make_div_const(4.0 * dx * dx);
        const unsigned grid = (unsigned)(c->gs / kThreads);
        if (sig) k_rk_rhs_post<true><<<grid, kThreads, 0, c->stream>>>(fs, fds, kfd, sg, c->lg, K);
        else k_rk_rhs_post<false><<<grid, kThreads, 0, c->stream>>>(fs, fds, kfd, sg, c->lg, K);
        c->launches++;
        *dadt = ad_st;
        *daddt = -(s - 0.5 * (1.0 - 3.0 * omega)) * (ad_st * ad_st) / a_st;
        return IEGPU_OK;
    }
    RkCoef K;
    K.laplnorm = pow(a_st, -2.0 * s) / (dx * dx);
    K.friction = (2.0 + s) * ad_st / a_st;
    K.potnorm = pow(a_st, 2.0 - 2.0 * s);
    K.srcAmp = 2.0 * pow(a_st, -2.0 * s);
    K.half_over_dx = 0.5 / dx;
    const bool tab = c->pot.table != 0;
    const dim3 g(c->red_grid), b(kThreads);
    if (tab && sig) k_rk_rhs<true, true><<<g, b, 0, c->stream>>>(fs, fds, kfd, sg, c->pot, c->ctl, c->part, c->counter, c->misc, c->lg, K);
    else if (tab) k_rk_rhs<true, false><<<g, b, 0, c->stream>>>(fs, fds, kfd, sg, c->pot, c->ctl, c->part, c->counter, c->misc, c->lg, K);
    else if (sig) k_rk_rhs<false, true><<<g, b, 0, c->stream>>>(fs, fds, kfd, sg, c->pot, c->ctl, c->part, c->counter, c->misc, c->lg, K);
    else k_rk_rhs<false, false><<<g, b, 0, c->stream>>>(fs, fds, kfd, sg, c->pot, c->ctl, c->part, c->counter, c->misc, c->lg, K);
    c->launches++;
    if (check_cuda(c, cudaMemcpyAsync(c->misc_h, c->misc, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "RK sums"))
        return IEGPU_ECUDA;
    if (check_cuda(c, cudaMemcpyAsync(&c->ctl_h->error, &c->ctl->error, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "RK status"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "RK stage")) return IEGPU_ECUDA;
    if (c->ctl_h->error) return read_ctl(c);
    const double gradient_sum = -c->misc_h[0];
    const double potential_sum = c->misc_h[1];
    const double gsd = (double)c->gs;
    const double gradient = 0.5 * gradient_sum * ((1.0 / (a_st * dx)) * (1.0 / (a_st * dx))) / gsd;
    const double potential_avg = potential_sum / gsd;
    const double source = 2.0 * gradient / 3.0 + potential_avg;
    *dadt = ad_st;
    *daddt = pow(a_st, 3.0 - 2.0 * s) * source - (s + 1.0) * (ad_st * ad_st) / a_st;
    return IEGPU_OK;
}

template <int NT>
static void rk_combine_launch(iegpu_ctx* c, unsigned grid, const double* f, const double* fd, double* fout,
                              double* fdout, const RkRow& R, const RkH& H, double h) {
    if (c->cfg.sigw) k_rk_combine<NT, true><<<grid, kThreads, 0, c->stream>>>(f, fd, fout, fdout, R, H, h);
    else k_rk_combine<NT, false><<<grid, kThreads, 0, c->stream>>>(f, fd, fout, fdout, R, H, h);
}

static void rk_combine(iegpu_ctx* c, const RkBufs& B, const double* coef, int nq, const double* f, const double* fd,
                       double* fout, double* fdout, const float* const* hb, const float* const* hdb, float* const* hout,
                       float* const* hdout, double h) {
    // the nonzero terms of the row, in stage order
    RkRow R{};
    int nt = 0;
    for (int q = 0; q < nq; ++q) {
        if (coef[q] == 0.0) continue;
        R.kf[nt] = B.fd[q];
        R.kfd[nt] = B.kfd[q];
        for (int k = 0; k < 6; ++k) {
            R.kh[nt][k] = B.hd[q][k];
            R.khd[nt][k] = B.khd[q][k];
        }
        R.c[nt] = coef[q];
        ++nt;
    }
    R.nq = nt;
    RkH H{};
    for (int k = 0; k < 6 && c->cfg.sigw; ++k) {
        H.hb[k] = hb[k];
        H.hdb[k] = hdb[k];
        H.ho[k] = hout[k];
        H.hdo[k] = hdout[k];
    }
    const unsigned grid = (unsigned)(c->gs / kThreads);
    static_assert(kRkMax == 7, "one instance per term count 0..kRkMax");
    switch (nt) {
        case 0: rk_combine_launch<0>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 1: rk_combine_launch<1>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 2: rk_combine_launch<2>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 3: rk_combine_launch<3>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 4: rk_combine_launch<4>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 5: rk_combine_launch<5>(c, grid, f, fd, fout, fdout, R, H, h); break;
        case 6: rk_combine_launch<6>(c, grid, f, fd, fout, fdout, R, H, h); break;
        default: rk_combine_launch<7>(c, grid, f, fd, fout, fdout, R, H, h); break;
    }
    c->launches++;
}

struct RkState {
    double* f;
    float* h[6];
};

static RkState rk_state(iegpu_ctx* c) {
    RkState S{};
    S.f = c->f[c->cur];
    for (int k = 0; k < 6 && c->cfg.sigw; ++k) S.h[k] = c->h[c->cur][k];
    return S;
}

// The stages 1..nst-1 of a tableau after the stage-0 derivatives
// (evaluate_inflation_stage, src/evolution.cpp:692-715).
static int rk_stages(iegpu_ctx* c, const RkEq& E, const RkBufs& B, const double (*A)[kRkMax], int nst, double h,
                     const iegpu_bg* bg, double* ka, double* kad) {
    const RkState S = rk_state(c);
    for (int stage = 1; stage < nst; ++stage) {
        rk_combine(c, B, A[stage], stage, S.f, c->fd, B.f, B.fd[stage], S.h, c->hd, B.h, B.hd[stage], h);
        double a_st = bg->a, ad_st = bg->ad;
        for (int q = 0; q < stage; ++q) {
            const double cq = A[stage][q];
            if (cq == 0.0) continue;
            a_st += h * cq * ka[q];
            ad_st += h * cq * kad[q];
        }
        if (int rc = rk_rhs(c, E, B.f, B.fd[stage], B.h, B.hd[stage], B.kfd[stage], B.khd[stage], a_st, ad_st,
                            &ka[stage], &kad[stage]))
            return rc;
    }
    return IEGPU_OK;
}

// rk4_step_inflation(h): four right-hand sides, three stage states, the
// weighted update of the lattice and of (a, ad), then t += h.  ad2 is not
// touched.
static int rk4_step(iegpu_ctx* c, const RkEq& E, const RkBufs& B, double h, iegpu_bg* bg) {
    const RkState S = rk_state(c);
    double ka[kRkMax] = {0.0}, kad[kRkMax] = {0.0};
    if (int rc = rk_rhs(c, E, S.f, B.fd[0], S.h, B.hd[0], B.kfd[0], B.khd[0], bg->a, bg->ad, &ka[0], &kad[0])) return rc;
    if (int rc = rk_stages(c, E, B, kRk4A, 4, h, bg, ka, kad)) return rc;
    rk_combine(c, B, kRk4B, 4, S.f, c->fd, S.f, c->fd, S.h, c->hd, S.h, c->hd, h);
    for (int q = 0; q < 4; ++q) {
        const double bq = kRk4B[q];
        if (bq == 0.0) continue;
        bg->a += h * bq * ka[q];
        bg->ad += h * bq * kad[q];
    }
    bg->t += h;
    return IEGPU_OK;
}

// sanitize_rk45_controls, src/runtime_parameters.cpp:184-192
iegpu_rk45_controls rk45_sanitized(const iegpu_ctx* c, const iegpu_rk45_controls* in) {
    return rk45_sanitized_dt(in, c->cfg.dt);
}

iegpu_rk45_controls rk45_sanitized_dt(const iegpu_rk45_controls* in, double dt_in) {
    iegpu_rk45_controls K = *in;
    const double dt = fabs(dt_in);
    if (!(K.min_dt > 0.0)) K.min_dt = dt * 1e-6;
    if (!(K.max_dt > 0.0)) K.max_dt = dt;
    if (K.min_dt <= 0.0) K.min_dt = 1e-16;
    if (K.max_dt < K.min_dt) K.max_dt = K.min_dt;
    if (!(K.abs_tol > 0.0)) K.abs_tol = 1e-8;
    if (!(K.rel_tol > 0.0)) K.rel_tol = 1e-6;
    if (!(K.safety > 0.0 && K.safety < 1.0)) K.safety = 0.9;
    return K;
}

// clamp_rk45_step, src/evolution.cpp:326-332
double rk45_clamp(const iegpu_rk45_controls& K, double h, double hmax) {
    const double hmin = ref_max(1e-16, K.min_dt);
    const double hhi = ref_max(hmin, hmax);
    if (h < hmin) return hmin;
    if (h > hhi) return hhi;
    return h;
}

// rk45_hmax_from_base_step, src/evolution.cpp:341-343
double rk45_hmax(const iegpu_rk45_controls& K, double base_step) {
    return ref_min(K.max_dt, ref_max(K.min_dt, 2.0 * base_step));
}

// rk45_step_inflation(h, hmax, h_next), src/evolution.cpp:781-904: seven
// right-hand sides, the candidate and its error norm; on acceptance the
// candidate becomes the state.
static int rk45_attempt(iegpu_ctx* c, const RkEq& E, const RkBufs& B, const iegpu_rk45_controls& K, double h,
                        double hmax, double* h_next, int* accepted, iegpu_bg* bg) {
    const RkState S = rk_state(c);
    const bool sig = c->cfg.sigw != 0;
    double ka[kRkMax] = {0.0}, kad[kRkMax] = {0.0};
    if (int rc = rk_rhs(c, E, S.f, B.fd[0], S.h, B.hd[0], B.kfd[0], B.khd[0], bg->a, bg->ad, &ka[0], &kad[0])) return rc;
    if (int rc = rk_stages(c, E, B, kDpA, kRkMax, h, bg, ka, kad)) return rc;
    double a5 = bg->a, ad5 = bg->ad, erra = 0.0, errad = 0.0;
    for (int q = 0; q < kRkMax; ++q) {
        const double bs = kDpB[q], es = kDpE[q];
        if (bs != 0.0) {
            a5 += h * bs * ka[q];
            ad5 += h * bs * kad[q];
        }
        if (es != 0.0) {
            erra += h * es * ka[q];
            errad += h * es * kad[q];
        }
    }
    Rk45Fin F{};
    for (int q = 0; q < kRkMax; ++q) {
        F.kf[q] = B.fd[q];
        F.kfd[q] = B.kfd[q];
        for (int k = 0; k < 6 && sig; ++k) {
            F.kh[q][k] = B.hd[q][k];
            F.khd[q][k] = B.khd[q][k];
        }
        F.b[q] = kDpB[q];
        F.e[q] = kDpE[q];
    }
    for (int k = 0; k < 6 && sig; ++k) {
        F.hs[k] = S.h[k];
        F.hds[k] = c->hd[k];
        F.y5h[k] = B.h[k];
        F.y5hd[k] = B.y5hd[k];
    }
    F.y5f = B.f;
    F.y5fd = B.y5fd;
    F.h = h;
    F.atol = K.abs_tol;
    F.rtol = K.rel_tol;
    if (sig) k_rk45_final<true><<<c->red_grid, kThreads, 0, c->stream>>>(S.f, c->fd, F, c->part, c->counter, c->misc, (long long)c->gs);
    else k_rk45_final<false><<<c->red_grid, kThreads, 0, c->stream>>>(S.f, c->fd, F, c->part, c->counter, c->misc, (long long)c->gs);
    c->launches++;
    if (check_cuda(c, cudaMemcpyAsync(c->misc_h, c->misc, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "RK45 error"))
        return IEGPU_ECUDA;
    if (sync_and_check(c, "RK45 error")) return IEGPU_ECUDA;
    double err_acc = c->misc_h[0];
    size_t nvars = 2 * c->gs + 2;
    if (sig) nvars += 12 * c->gs;
    const double sa = K.abs_tol + K.rel_tol * ref_max(fabs(bg->a), fabs(a5));
    const double sad = K.abs_tol + K.rel_tol * ref_max(fabs(bg->ad), fabs(ad5));
    err_acc += (erra / sa) * (erra / sa) + (errad / sad) * (errad / sad);
    const double err_norm = sqrt(err_acc / (double)nvars);
    const double safe_err = ref_max(err_norm, 1e-16);
    double factor = K.safety * pow(safe_err, -0.2);
    factor = (factor < 0.1) ? 0.1 : (5.0 < factor) ? 5.0 : factor;
    if (err_norm <= 1.0) {
        const size_t bytes = sizeof(double) * c->gs;
        cudaError_t e = cudaMemcpyAsync(S.f, B.f, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->fd, B.y5fd, bytes, cudaMemcpyDeviceToDevice, c->stream);
        for (int k = 0; k < 6 && sig && e == cudaSuccess; ++k) {
            e = cudaMemcpyAsync(S.h[k], B.h[k], bytes / 2, cudaMemcpyDeviceToDevice, c->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(c->hd[k], B.y5hd[k], bytes / 2, cudaMemcpyDeviceToDevice, c->stream);
        }
        if (check_cuda(c, e, "RK45 accept")) return IEGPU_ECUDA;
        bg->a = a5;
        bg->ad = ad5;
        bg->t += h;
        *h_next = rk45_clamp(K, h * factor, hmax);
        *accepted = 1;
        return IEGPU_OK;
    }
    *h_next = rk45_clamp(K, h * ref_max(0.1, ref_min(0.5, factor)), hmax);
    *accepted = 0;
    return IEGPU_OK;
}

// rk45_accept_step, src/evolution.cpp:345-363: attempts until one is
// accepted; fails after 25 rejections or at the minimum step, with the
// reference's message.  *h: in, the step to try; out, the step proposed for
// the next one.
static int rk45_accept(iegpu_ctx* c, const RkEq& E, const RkBufs& B, const iegpu_rk45_controls& K, double* h,
                       double hmax, iegpu_bg* bg) {
    int accepted = 0, attempts = 0;
    while (!accepted) {
        double hs = *h;
        if (int rc = rk45_attempt(c, E, B, K, *h, hmax, &hs, &accepted, bg)) return rc;
        *h = hs;
        ++attempts;
        if (!accepted && (attempts > 25 || *h <= K.min_dt * (1.0 + 1e-12))) {
            if (E.post)
                return set_error(c, IEGPU_ECONVERGE, "RK45 failed to converge in post-inflation at a=%e, t=%e (attempts=%d, h=%e)\n",
                                 bg->a, bg->t, attempts, *h);
            return set_error(c, IEGPU_ECONVERGE, "RK45 failed to converge at a=%e, t=%e (attempts=%d, h=%e)\n", bg->a,
                             bg->t, attempts, *h);
        }
    }
    return IEGPU_OK;
}

static int rk_begin(iegpu_ctx* c, const iegpu_bg* bg, int nst, RkBufs& B) {
    if (int rc = rk_bufs(c, nst, B)) return rc;
    fill_ctl(c, bg, kModeLeapfrog);
    c->ctl_h->st.active = 0;
    c->ctl_h->done = 1;
    return upload_ctl(c);
}

int fp64_rk4_step(iegpu_ctx* c, double h, iegpu_bg* bg) {
    RkBufs B;
    if (int rc = rk_begin(c, bg, 4, B)) return rc;
    if (int rc = rk4_step(c, RkEq{false, 0.0}, B, h, bg)) return rc;
    return sync_and_check(c, "RK4 step");
}

// The RK4 branch of run_evolution_loop, src/evolution.cpp:948-956: while
// a <= af, one step of d = dt astep^(s-1), then "astep = a".  As in
// fp64_leapfrog, the "astep = a" after the last step of a call is left to the
// caller, who reports that step first.
int fp64_rk4(iegpu_ctx* c, double af, int max_steps, iegpu_bg* bg, int* steps, double* a_trace) {
    if (steps) *steps = 0;
    RkBufs B;
    if (int rc = rk_begin(c, bg, 4, B)) return rc;
    const double s = c->cfg.rescale_s;
    int n = 0;
    while (n < max_steps) {
        if (n > 0) bg->astep = bg->a;
        if (!(bg->a <= af)) break;
        const double d = c->cfg.dt * pow(bg->astep, s - 1.0);
        if (int rc = rk4_step(c, RkEq{false, 0.0}, B, d, bg)) {
            if (steps) *steps = n;
            return rc;
        }
        if (a_trace) a_trace[n] = bg->a;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "RK4");
}

int fp64_rk45_step(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double h, double hmax, double* h_next, int* accepted,
                   iegpu_bg* bg) {
    RkBufs B;
    if (int rc = rk_begin(c, bg, kRkMax, B)) return rc;
    const iegpu_rk45_controls K = rk45_sanitized(c, ctl);
    if (int rc = rk45_attempt(c, RkEq{false, 0.0}, B, K, h, hmax, h_next, accepted, bg)) return rc;
    return sync_and_check(c, "RK45 step");
}

// The RK45 branch of run_evolution_loop, src/evolution.cpp:958-985: while
// a <= af, hmax from dt astep^(s-1), h clamped to it, then accepted attempts
// (rk45_accept_step) and "astep = a".  *h carries the proposed step from one
// step (and call) to the next.
int fp64_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af, int max_steps, double* h, iegpu_bg* bg,
              int* steps, double* a_trace) {
    if (steps) *steps = 0;
    RkBufs B;
    if (int rc = rk_begin(c, bg, kRkMax, B)) return rc;
    const iegpu_rk45_controls K = rk45_sanitized(c, ctl);
    const double s = c->cfg.rescale_s;
    int n = 0;
    while (n < max_steps) {
        if (n > 0) bg->astep = bg->a;
        if (!(bg->a <= af)) break;
        const double hmax = rk45_hmax(K, c->cfg.dt * pow(bg->astep, s - 1.0));
        *h = rk45_clamp(K, *h, hmax);
        if (int rc = rk45_accept(c, RkEq{false, 0.0}, B, K, h, hmax, bg)) {
            if (steps) *steps = n;
            return rc;
        }
        if (a_trace) a_trace[n] = bg->a;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "RK45");
}

// The RK4 and RK45 branches of run_post_inflation_loop,
// src/evolution.cpp:1606-1641: the post-inflation equations, steps of
// dt_post (RK4) or adaptive steps with hmax from dt_post (RK45) while
// a <= af_post.
int fp64_post_rk4(iegpu_ctx* c, double af_post, double dt_post, double omega, int max_steps, iegpu_bg* bg, int* steps,
                  double* a_trace) {
    if (steps) *steps = 0;
    RkBufs B;
    if (int rc = rk_begin(c, bg, 4, B)) return rc;
    int n = 0;
    while (n < max_steps && bg->a <= af_post) {
        if (int rc = rk4_step(c, RkEq{true, omega}, B, dt_post, bg)) {
            if (steps) *steps = n;
            return rc;
        }
        if (a_trace) a_trace[n] = bg->a;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "post-inflation RK4");
}

int fp64_post_rk45(iegpu_ctx* c, const iegpu_rk45_controls* ctl, double af_post, double dt_post, double omega,
                   int max_steps, double* h, iegpu_bg* bg, int* steps, double* a_trace) {
    if (steps) *steps = 0;
    RkBufs B;
    if (int rc = rk_begin(c, bg, kRkMax, B)) return rc;
    const iegpu_rk45_controls K = rk45_sanitized(c, ctl);
    int n = 0;
    while (n < max_steps && bg->a <= af_post) {
        const double hmax = rk45_hmax(K, dt_post);
        *h = rk45_clamp(K, *h, hmax);
        if (int rc = rk45_accept(c, RkEq{true, omega}, B, K, h, hmax, bg)) {
            if (steps) *steps = n;
            return rc;
        }
        if (a_trace) a_trace[n] = bg->a;
        ++n;
    }
    if (steps) *steps = n;
    return sync_and_check(c, "post-inflation RK45");
}

}  // namespace iegpu
