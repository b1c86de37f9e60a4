// split_kernels.cuh -- device building blocks of the split-precision step,
// shared by the one-lattice form and the ensemble form.
//
// The field is stored as phi = phibar(t) + dphi(x), phi' = pibar(t) + dpi(x)
// (background in FP64, perturbations in FP32).  Everything here works on one
// lattice: a step CTA owns a tile of rows and a chunk of planes, writes its
// block sums to a partial slot, and the last CTA of the lattice to arrive
// runs the FP64 Friedmann and background update of that lattice.
#pragma once
#include <cmath>
#include <cstddef>

#include "iegpu_internal.cuh"
#include "pot.cuh"
#include "reduce.cuh"
#include "split_window.cuh"

namespace iegpu {

// The line A + s x of a site beyond the window, from the whole table: its
// bracket l (x[l-1] >= phibar + x > x[l]) by bisection, and the bracket's line
// formed in FP64 as build_window_warp forms the window's lines, so that a
// bracket the window also holds gives the same float coefficients.  wb =
// {phibar, Fbar} of the window; y, slope: the tabulated function and its
// bracket slopes.  On a coarsely tabulated stretch a perturbation is a small
// fraction of a bracket and this path is rare; where the table is dense
// (the USR plateau of inputs/*.dat has brackets of 2.7e-6) the perturbations
// span many brackets and more sites take it.  bad: beyond the table.
// The out-of-line part takes plain pointers and returns its range flag, so
// that a step loop calling it keeps the table descriptor and the flag in
// registers (no address of either is taken).
struct FarLine {
    float v;
    int oor;
};

static __device__ __noinline__ FarLine far_line_at(const long long* key, const double* xs, int n, const double* y,
                                                   const double* slope, double phibar, double Fbar, float x) {
    bool oor;
    const int l = table_bracket_keys(key, n, phibar + (double)x, &oor);
    if (oor) return FarLine{0.f, 1};
    const double s = __ldg(&slope[l]);
    const float A = (float)((__ldg(&y[l]) + (phibar - __ldg(&xs[l])) * s) - Fbar);
    return FarLine{A + (float)s * x, 0};
}

__device__ __forceinline__ float far_line(const PotDev& P, const double* y, const double* slope, const double* wb,
                                          float x, bool& bad) {
    const FarLine r = far_line_at(P.key, P.x, P.n, y, slope, wb[0], wb[1], x);
    bad = bad || r.oor != 0;
    return r.v;
}

// potnorm [V'(phibar + x) - V'(phibar)] / B^2 (table) or kv x (hilltop).
// wb: {phibar, Fbar} of the kick window, for sites beyond it.
// LIFT: a site beyond the three brackets searches the window branch-free
// (window_lift), else by a walk (window_find).
template <bool TABLE, bool LIFT = false, bool WIDE = false>
__device__ __forceinline__ float split_dv(float x, const float* wk, int nk, const WinCache& c, float pn, float kv,
                                          bool& bad, const PotDev& P, const double* wb) {
    if (TABLE) {
        float A, sl;
        // the background's bracket or a neighbour, chosen without a branch
        if (cache_line<WIDE>(c, x, A, sl)) return pn * (A + sl * x);
        const int q = LIFT ? window_lift(wk, nk, x) : window_find(wk, nk, x);
        if (q < 0) return pn * far_line(P, P.dV, P.slopedV, wb, x, bad);
        return pn * (wk[kWin + 1 + q] + wk[2 * kWin + 1 + q] * x);
    }
    return kv * x;
}

// V(phibar + x) - V(phibar) in table units (table) or x^2 (hilltop).
// wb: {phibar, Fbar} of the potential window, for sites beyond it.
template <bool TABLE, bool LIFT = false, bool WIDE = false>
__device__ __forceinline__ float split_v(float x, const float* wv, int nv, const WinCache& c, bool& bad,
                                         const PotDev& P, const double* wb) {
    if (TABLE) {
        float A, sl;
        if (cache_line<WIDE>(c, x, A, sl)) return A + sl * x;
        const int q = LIFT ? window_lift(wv, nv, x) : window_find(wv, nv, x);
        if (q < 0) return far_line(P, P.V, P.slopeV, wb, x, bad);
        return wv[kWin + 1 + q] + wv[2 * kWin + 1 + q] * x;
    }
    return x * x;
}

// {phibar, Fbar} of the kick window (wb[0..1]) and of the potential window
// (wb[2..3]) into shared memory, by thread 0; CG: read through L2 (the
// control block of a persistent launch, written during the launch).
template <bool CG>
__device__ __forceinline__ void load_win_centres(double* wb, const SplitCtl* ctl) {
    if (threadIdx.x == 0) {
        wb[0] = CG ? __ldcg(&ctl->wk.phibar) : ctl->wk.phibar;
        wb[1] = CG ? __ldcg(&ctl->wk.Fbar) : ctl->wk.Fbar;
        wb[2] = CG ? __ldcg(&ctl->wv.phibar) : ctl->wv.phibar;
        wb[3] = CG ? __ldcg(&ctl->wv.Fbar) : ctl->wv.Fbar;
    }
}

// ---------------------------------------------------------------------------
// Kahan accumulator
// ---------------------------------------------------------------------------

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
    __device__ __forceinline__ struct df64 df() const;
};

// ---------------------------------------------------------------------------
// double-float arithmetic
// ---------------------------------------------------------------------------
//
// A value hi + lo held in two floats (about 44 significant bits), added with
// the error-free sum of Knuth and Dekker on FP32 adds.  GB300's FP64
// operations have hundreds of cycles of latency; these run on the FP32 pipes.
// The _rn intrinsics keep the compiler from reassociating the error terms.
struct df64 {
    float hi, lo;
};

__device__ __forceinline__ df64 df_quick(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return df64{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return df64{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
    const df64 s = df_two_sum(a.hi, b.hi);
    const df64 t = df_two_sum(a.lo, b.lo);
    const df64 u = df_quick(s.hi, __fadd_rn(s.lo, t.hi));
    return df_quick(u.hi, __fadd_rn(u.lo, t.lo));
}

__device__ __forceinline__ double df_to(df64 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df64 df_from(double x) {
    const float h = (float)x;
    return df64{h, (float)(x - (double)h)};
}

// Product with the exact error of hi*hi from an FMA (Dekker's product).
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return df_quick(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}

// Square root of a > 0: the FP32 root r corrected by one Newton step,
// r + (a - r^2) / (2r), with r^2 formed exactly by an FMA.
__device__ __forceinline__ df64 df_sqrt(df64 a) {
    const float r = sqrtf(a.hi);
    const float p = __fmul_rn(r, r);
    const float e = __fmaf_rn(r, r, -p);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
    return df_quick(r, __fmul_rn(res, __frcp_rn(__fadd_rn(r, r))));
}

__device__ __forceinline__ df64 df_shfl_down(df64 v, int o) {
    return df64{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

__device__ __forceinline__ df64 Kahan::df() const { return df_two_sum(s, -c); }

// Sum over the block of NV df64 values per thread in a fixed order (lane
// trees, then warps in index order); the result is valid in lane 0 of warp
// `leader`.  The one barrier is the last the other warps take part in.
template <int NV>
__device__ __forceinline__ void block_sum_df(df64 (&v)[NV], int leader) {
    __shared__ df64 sh[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] = df_add(v[q], df_shfl_down(v[q], o));
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q][w] = v[q];
    }
    __syncthreads();
    if (w == leader) {
        const int nw = (int)(blockDim.x >> 5);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            v[q] = lane < nw ? sh[q][lane] : df64{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[q] = df_add(v[q], df_shfl_down(v[q], o));
        }
    }
}

// Sum of the df64 partials p[b*NV + q], b < nb, by one warp in a fixed order
// (lane l adds slots l, l+32, ... in turn, then a lane tree); result valid in
// lane 0.  The loads of up to 32*kBatch slots are all issued before the adds,
// so the sum waits for about one L2 round trip per batch.
template <int NV>
__device__ __forceinline__ void sum_partials_df(const df64* p, int nb, df64 (&out)[NV]) {
    constexpr int kBatch = 8;
    const int lane = threadIdx.x & 31;
    const float2* src = reinterpret_cast<const float2*>(p);
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = df64{0.f, 0.f};
    for (int b0 = 0; b0 < nb; b0 += 32 * kBatch) {
        float2 x[kBatch][NV];
#pragma unroll
        for (int i = 0; i < kBatch; ++i) {
            const int b = b0 + lane + 32 * i;
#pragma unroll
            for (int q = 0; q < NV; ++q)
                x[i][q] = b < nb ? __ldcg(src + (size_t)b * NV + q) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int i = 0; i < kBatch; ++i) {
            if (b0 + lane + 32 * i >= nb) break;
#pragma unroll
            for (int q = 0; q < NV; ++q) out[q] = df_add(out[q], df64{x[i][q].x, x[i][q].y});
        }
    }
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) out[q] = df_add(out[q], df_shfl_down(out[q], o));
}

// ---------------------------------------------------------------------------
// scalar update (one warp): Friedmann, background, coefficients, windows
// ---------------------------------------------------------------------------
//
// Every lane evaluates the FP64 scalar recurrences (identical values); the
// table searches and the window nodes are shared out over the lanes, so the
// update costs a few dependent loads instead of a hundred, and lane 0 writes
// the results.

// The bracket of v, as table_bracket: the count of nodes with key >= key(v),
// clamped to [1, n-1] (the nodes descend strictly), counted by the warp.
// hint: a bracket near v (the last step's, from its window), or < 0.  The
// warp first looks at the 32 nodes around it: when v lies among them the
// count is their offset plus one ballot, one load per lane; otherwise it
// counts over the whole table.
__device__ __forceinline__ int warp_bracket(const PotDev& P, double v, int hint = -1) {
    const long long kv = order_key(v);
    if (hint >= 0 && P.n >= 32) {
        int base = hint - 16;
        base = base < 0 ? 0 : (base > P.n - 32 ? P.n - 32 : base);
        const bool ge = __ldg(&P.key[base + (threadIdx.x & 31)]) >= kv;
        const unsigned m = __ballot_sync(0xffffffffu, ge);
        // nodes before base are all >= kv when node base is (or base = 0),
        // nodes after base + 31 all < kv when that one is (or it is the last)
        const bool lo_ok = base == 0 || (m & 1u);
        const bool hi_ok = base + 32 == P.n || !(m >> 31);
        if (lo_ok && hi_ok) {
            const int cnt = base + __popc(m);
            return cnt < 1 ? 1 : (cnt > P.n - 1 ? P.n - 1 : cnt);
        }
    }
    int cnt = 0;
    for (int i = threadIdx.x & 31; i < P.n; i += 32) cnt += (__ldg(&P.key[i]) >= kv) ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    return cnt < 1 ? 1 : (cnt > P.n - 1 ? P.n - 1 : cnt);
}

__device__ __forceinline__ bool table_out_of_range(const PotDev& P, double v) {
    const long long kv = order_key(v);
    return !is_nan_bits(v) && (kv > __ldg(&P.key[0]) || kv < __ldg(&P.key[P.n - 1]));
}

// build_window by a warp: lane q writes node q and bracket q.  slope[l] =
// dy[l] / dxl[l], precomputed on the host (the same IEEE quotient).
__device__ __forceinline__ void build_window_warp(SplitWin& W, const PotDev& P, const double* y,
                                                  const double* slope, double phibar, int* err) {
    const int lane = threadIdx.x & 31;
    // the window being replaced holds last step's bracket (ok = 0: none yet)
    const int hint = W.ok ? W.l0 + kWin / 2 : -1;
    __syncwarp();
    if (lane == 0) W.ok = 0;
    if (!P.table) return;
    if (table_out_of_range(P, phibar)) {
        *err = 1;
        return;
    }
    const int lb = warp_bracket(P, phibar, hint);
    int l0 = lb - kWin / 2;
    if (l0 < 1) l0 = 1;
    int n = kWin;
    if (l0 + n - 1 > P.n - 1) n = P.n - 1 - l0 + 1;
    // value of the tabulated function at phibar (its own bracket)
    const double Fbar = y[lb] + (phibar - P.x[lb]) * slope[lb];
    if (lane <= n) W.u[lane] = (float)(P.x[l0 - 1 + lane] - phibar);
    if (lane < n) {
        const int l = l0 + lane;
        const double s = slope[l];
        W.s[lane] = (float)s;
        W.A[lane] = (float)((y[l] + (phibar - P.x[l]) * s) - Fbar);
    }
    if (lane == 0) {
        W.phibar = phibar;
        W.Fbar = Fbar;
        W.l0 = l0;
        W.n = n;
        W.ok = 1;
    }
}

// V(phibar) and V'(phibar) times B^2 (src/potential.cpp:77-98) for the
// bracket l of phibar (table) or the hilltop formula.
__device__ __forceinline__ void bar_potential_at(const PotDev& P, double phibar, int l, double* V, double* dV) {
    if (P.table) {
        const double u = phibar - P.x[l];
        *V = P.V[l] + u * P.slopeV[l];
        *dV = P.dV[l] + u * P.slopedV[l];
    } else {
        *V = P.V0 * (1.0 - P.c1 * (phibar * phibar));
        *dV = P.c2 * phibar;
    }
}

// sums: [0] sum of squared forward differences of dphi, [1] sum dphi,
// [2] hilltop: sum dphi^2 / table: sum of V differences (table units).
// Called by the 32 lanes of one warp with the same sums.  GB300's FP64 pipe
// is narrow and a dependent FP64 operation takes hundreds of cycles, so the
// recurrences run on lane 0 alone and multiply by precomputed reciprocals:
// one division (1/a, beside d) and one square root lie on the path from the
// sums to the next step's coefficients.  The table searches and window nodes
// are shared out over the lanes.
static __device__ __noinline__ void split_scalars_warp(SplitCtl& C, const PotDev& P, const SplitConst& K,
                                                       const double* sums, double* a_trace) {
    const bool w0 = (threadIdx.x & 31) == 0;
    const int mode = C.mode, steps_done = C.steps_done, steps_limit = C.steps_limit, error0 = C.error;
    const double phibar0 = C.phibar;
    __syncwarp();   // every lane has read the control block before lane 0 writes it
    if (mode == kModeLeapfrog) {
        // the stop checks read the same values in every lane
        if (steps_done >= steps_limit) {
            if (w0) { C.active = 0; C.done = 1; }
            return;
        }
        const double a0 = C.bg.a, af = C.af;
        if (!(a0 <= af)) {
            if (w0) {
                if (steps_done > 0) C.bg.astep = a0;
                C.active = 0;
                C.done = 1;
            }
            return;
        }
    }
    const int lbar = P.table ? warp_bracket(P, phibar0, C.wk.ok ? C.wk.l0 + kWin / 2 : -1) : 0;
    double phibar_new = phibar0;
    if (w0) {
        double t = C.bg.t, a = C.bg.a, ad = C.bg.ad, astep = C.bg.astep;
        double phibar = phibar0, pibar = C.pibar;
        const double s = K.s;
        double d, rd;
        if (mode == kModeLeapfrog) {
            if (steps_done > 0) astep = a;
            // d = dt astep^(s-1), 1/d = astep^(1-s) / dt
            if (s == 0.0) {
                d = K.dt / astep;
                rd = astep * K.idt;
            } else {
                d = K.dt * pow_exp(astep, s - 1.0);
                rd = pow_exp(astep, 1.0 - s) * K.idt;
            }
        } else {
            d = C.d_given;
            rd = 1.0 / d;
        }
        const double ra = 1.0 / a;
        const double g1 = ra * K.idx;
        const double grad = 0.5 * sums[0] * (g1 * g1) * K.igs;
        double Vb, dVb;   // times B^2
        bar_potential_at(P, phibar, lbar, &Vb, &dVb);
        double pot;
        if (P.table) pot = (Vb + sums[2] * K.igs) * K.iB2;
        else pot = (Vb - P.V0 * P.c1 * (2.0 * phibar * sums[1] + sums[2]) * K.igs) * K.iB2;
        const double sfev1 = s + 1.0, sfev2 = -2.0 * s + 2.0;
        const double a_sfev2 = (s == 0.0) ? a * a : pow_exp(a, sfev2);
        const double x = 2.0 * d * sfev1 * ad * ra + (d * d) * sfev1 * a_sfev2 * (2.0 * grad * (1.0 / 3.0) + pot);
        const double ad2 = (-2.0 * ad - 2.0 * a * rd * K.isfev1 * (1.0 - sqrt(1.0 + x))) * rd;
        ad += 0.5 * d * ad2;
        const double a_m2s = (s == 0.0) ? 1.0 : pow_exp(a, -2.0 * s);
        const double laplnorm = a_m2s * K.idx2;
        const double friction = (2.0 + s) * ad * ra;
        const double potnorm = (s == 0.0) ? a * a : pow_exp(a, 2.0 - 2.0 * s);
        const double srcAmp = 2.0 * a_m2s;
        ad += 0.5 * d * ad2;
        // background kick (homogeneous mode of the lattice kick)
        pibar = pibar + d * (-friction * pibar - potnorm * (dVb * K.iB2));
        C.d = (float)d;
        C.lapl = (float)laplnorm;
        C.fric = (float)friction;
        C.pn = (float)(potnorm * K.iB2);
        C.kv = (float)(potnorm * P.c2 * K.iB2);
        C.srcAmp = (float)srcAmp;
        C.dd = d;
        C.bg.astep = astep;
        C.bg.ad = ad;
        C.bg.ad2 = ad2;
        C.pibar = pibar;
        C.active = 1;
        if (mode == kModeLeapfrog) {
            phibar = phibar + d * pibar;
            t += d;
            C.phibar = phibar;
            C.bg.t = t;
            C.bg.a = a + d * ad;
            if (a_trace) a_trace[steps_done] = C.bg.a;
            C.steps_done = steps_done + 1;
        }
        phibar_new = phibar;
    }
    phibar_new = __shfl_sync(0xffffffffu, phibar_new, 0);
    int err = 0;
    build_window_warp(C.wk, P, P.dV, P.slopedV, phibar0, &err);
    build_window_warp(C.wv, P, P.V, P.slopeV, phibar_new, &err);
    if (err && !error0 && w0) { C.error = IEGPU_ERANGE; C.errval = phibar_new; C.active = 0; C.done = 1; }
}

// The sum-independent part of the coming scalar update (leapfrog mode),
// formed by one warp of the first CTA of a step to finish its tile: the FP64
// latency is spent while the other CTAs still stream, and the last CTA only
// runs the short chain from the sums (split_scalars_warp).  Same arithmetic
// as the full update, regrouped into coefficients of S0, S1, S2.
static __device__ __noinline__ void split_precompute(SplitCtl& C, const PotDev& P, const SplitConst& K,
                                                     bool allow_fast) {
    const bool w0 = (threadIdx.x & 31) == 0;
    const int mode = C.mode, steps_done = C.steps_done, steps_limit = C.steps_limit;
    const double phibar = C.phibar;
    if (mode != kModeLeapfrog || steps_done >= steps_limit || !(C.bg.a <= C.af)) return;
    const int lbar = P.table ? warp_bracket(P, phibar, C.wk.ok ? C.wk.l0 + kWin / 2 : -1) : 0;
    if (!w0) return;
    const double a = C.bg.a, ad = C.bg.ad, pibar = C.pibar, s = K.s;
    const double astep = steps_done > 0 ? a : C.bg.astep;
    double d, rd;
    if (s == 0.0) {
        d = K.dt / astep;
        rd = astep * K.idt;
    } else {
        d = K.dt * pow_exp(astep, s - 1.0);
        rd = pow_exp(astep, 1.0 - s) * K.idt;
    }
    const double ra = 1.0 / a;
    const double g1 = ra * K.idx;
    const double cgrad = 0.5 * (g1 * g1) * K.igs;
    double Vb, dVb;   // times B^2
    bar_potential_at(P, phibar, lbar, &Vb, &dVb);
    SplitPre& Q = C.pre;
    Q.d = d;
    Q.astep = astep;
    Q.hd = 0.5 * d;
    Q.c0 = Vb * K.iB2;
    Q.cS0 = cgrad * (2.0 / 3.0);
    if (P.table) {
        Q.cS1 = 0.0;
        Q.cS2 = K.igs * K.iB2;
    } else {
        const double h = -P.V0 * P.c1 * K.igs * K.iB2;
        Q.cS1 = 2.0 * phibar * h;
        Q.cS2 = h;
    }
    const double sfev1 = s + 1.0, sfev2 = -2.0 * s + 2.0;
    const double a_sfev2 = (s == 0.0) ? a * a : pow_exp(a, sfev2);
    Q.cx0 = 2.0 * d * sfev1 * ad * ra;
    Q.cx1 = (d * d) * sfev1 * a_sfev2;
    // ad2 = (-2ad - K (1 - sq)) rd, K = 2a rd / (s+1)
    const double Kc = 2.0 * a * rd * K.isfev1;
    Q.ca0 = (-2.0 * ad - Kc) * rd;
    Q.ca1 = Kc * rd;
    Q.cf = (2.0 + s) * ra;
    const double a_m2s = (s == 0.0) ? 1.0 : pow_exp(a, -2.0 * s);
    const double potnorm = (s == 0.0) ? a * a : pow_exp(a, 2.0 - 2.0 * s);
    Q.cb0 = pibar - d * (potnorm * (dVb * K.iB2));
    Q.cb1 = -d * pibar;
    Q.lapl = (float)(a_m2s * K.idx2);
    Q.pn = (float)(potnorm * K.iB2);
    Q.kv = (float)(potnorm * P.c2 * K.iB2);
    Q.srcAmp = (float)(2.0 * a_m2s);
    Q.d32 = (float)d;
    Q.fast = allow_fast && !P.table;
    if (Q.fast) {
        const double v[kPreN] = {Q.c0, Q.cS0, Q.cS1, Q.cS2, Q.cx0, Q.cx1, Q.ca0, Q.ca1, ad, Q.hd, Q.cf};
#pragma unroll
        for (int q = 0; q < kPreN; ++q) {
            const df64 f = df_from(v[q]);
            Q.hi[q] = f.hi;
            Q.lo[q] = f.lo;
        }
    }
    Q.ok = 1;
}

// FP64 part of the precomputed update (lane 0): a, ad, ad2, t, astep, phibar
// and pibar after the step with lattice sums `sums`, the a_trace entry
// `step`; returns the friction and the new phibar.
static __device__ __forceinline__ void pre_state_update(SplitCtl& C, const double* sums, double* a_trace, int step,
                                                        double& friction, double& phibar_new) {
    const SplitPre& Q = C.pre;
    const double d = Q.d, a = C.bg.a, ad = C.bg.ad;
    const double E = Q.c0 + Q.cS0 * sums[0] + Q.cS1 * sums[1] + Q.cS2 * sums[2];
    const double x = Q.cx0 + Q.cx1 * E;
    const double ad2 = Q.ca0 + Q.ca1 * sqrt(1.0 + x);
    const double adh = ad + Q.hd * ad2;
    friction = Q.cf * adh;
    const double pibar = Q.cb0 + Q.cb1 * friction;
    const double adn = adh + Q.hd * ad2;
    C.dd = d;
    C.bg.astep = Q.astep;
    C.bg.ad = adn;
    C.bg.ad2 = ad2;
    C.pibar = pibar;
    phibar_new = C.phibar + d * pibar;
    C.phibar = phibar_new;
    C.bg.t = C.bg.t + d;
    C.bg.a = a + d * adn;
    if (a_trace) a_trace[step] = C.bg.a;
}

// The last CTA's update when a precomputed part is there (leapfrog mode,
// the stop checks already passed in split_precompute).
static __device__ __noinline__ void split_scalars_pre(SplitCtl& C, const PotDev& P, const double* sums,
                                                      double* a_trace) {
    const bool w0 = (threadIdx.x & 31) == 0;
    const int steps_done = C.steps_done, error0 = C.error;
    const double phibar0 = C.phibar;
    __syncwarp();
    double phibar_new = phibar0;
    if (w0) {
        const SplitPre& Q = C.pre;
        double friction;
        pre_state_update(C, sums, a_trace, steps_done, friction, phibar_new);
        C.fric = (float)friction;
        C.d = Q.d32;
        C.lapl = Q.lapl;
        C.pn = Q.pn;
        C.kv = Q.kv;
        C.srcAmp = Q.srcAmp;
        C.active = 1;
        C.steps_done = steps_done + 1;
    }
    phibar_new = __shfl_sync(0xffffffffu, phibar_new, 0);
    int err = 0;
    build_window_warp(C.wk, P, P.dV, P.slopedV, phibar0, &err);
    build_window_warp(C.wv, P, P.V, P.slopeV, phibar_new, &err);
    if (err && !error0 && w0) { C.error = IEGPU_ERANGE; C.errval = phibar_new; C.active = 0; C.done = 1; }
}

// The last CTA's update on the fast path (lane 0): the friction of the coming
// step from the double-float sums and coefficients; the FP64 update is left
// to split_apply_deferred.  Hilltop only: its kernels need no window.
static __device__ __forceinline__ void split_scalars_fast(SplitCtl& C, const df64 (&S)[3]) {
    const SplitPre& Q = C.pre;
    df64 f[kPreN];
#pragma unroll
    for (int q = 0; q < kPreN; ++q) f[q] = df64{Q.hi[q], Q.lo[q]};
    const int steps_done = C.steps_done;
    df64 E = df_add(f[kPreC0], df_mul(f[kPreS0], S[0]));
    E = df_add(E, df_mul(f[kPreS1], S[1]));
    E = df_add(E, df_mul(f[kPreS2], S[2]));
    const df64 x = df_add(f[kPreX0], df_mul(f[kPreX1], E));
    const df64 ad2 = df_add(f[kPreA0], df_mul(f[kPreA1], df_sqrt(df_add(df64{1.f, 0.f}, x))));
    const df64 adh = df_add(f[kPreAd], df_mul(f[kPreHd], ad2));
    const df64 fr = df_mul(f[kPreCf], adh);
    C.fric = __fadd_rn(fr.hi, fr.lo);
    C.d = Q.d32;
    C.lapl = Q.lapl;
    C.pn = Q.pn;
    C.kv = Q.kv;
    C.srcAmp = Q.srcAmp;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        C.dsum_hi[q] = S[q].hi;
        C.dsum_lo[q] = S[q].lo;
    }
    C.def_step = steps_done;
    C.deferred = 1;
    C.active = 1;
    C.steps_done = steps_done + 1;
}

// The FP64 part of a fast-path update, by lane 0 of the calling warp: the
// same arithmetic as split_scalars_pre, from the sums the fast path saved.
static __device__ __noinline__ void split_apply_deferred(SplitCtl& C, double* a_trace) {
    if ((threadIdx.x & 31) != 0 || !C.deferred) return;
    double sums[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        sums[q] = df_to(df64{C.dsum_hi[q], C.dsum_lo[q]});
        C.sums[q] = sums[q];
    }
    double friction, phibar_new;
    pre_state_update(C, sums, a_trace, C.def_step, friction, phibar_new);
    C.deferred = 0;
}

// After its tile, the first CTA of the step to get here forms the
// precomputed part (warp 0); the others go on at once.
__device__ __forceinline__ void maybe_precompute(SplitCtl* ctl, const PotDev& P, const SplitConst& K) {
    __shared__ int claimed;
    if (threadIdx.x == 0) claimed = atomicCAS(&ctl->pre_claim, 0, 1) == 0;
    __syncthreads();
    if (claimed && threadIdx.x < 32) {
        split_apply_deferred(*ctl, nullptr);
        split_precompute(*ctl, P, K, false);
    }
}

// One lane, for the diagnostics that build a window outside the step.
static __device__ __noinline__ void build_window(SplitWin& W, const PotDev& P, const double* y, const double* dy,
                                                 double phibar, int* err) {
    W.ok = 0;
    if (!P.table) return;
    bool oor;
    const int lb = table_bracket(P, phibar, &oor);
    if (oor) { *err = 1; return; }
    int l0 = lb - kWin / 2;
    if (l0 < 1) l0 = 1;
    int n = kWin;
    if (l0 + n - 1 > P.n - 1) n = P.n - 1 - l0 + 1;
    W.l0 = l0;
    W.n = n;
    const double Fbar = y[lb] + (phibar - P.x[lb]) * (dy[lb] / P.dxl[lb]);
    W.phibar = phibar;
    W.Fbar = Fbar;
    for (int q = 0; q <= n; ++q) W.u[q] = (float)(P.x[l0 - 1 + q] - phibar);
    for (int q = 0; q < n; ++q) {
        const int l = l0 + q;
        const double s = dy[l] / P.dxl[l];
        W.s[q] = (float)s;
        W.A[q] = (float)((y[l] + (phibar - P.x[l]) * s) - Fbar);
    }
    W.ok = 1;
}

// Publication of a step's scalar update to the other CTAs of a persistent
// launch: `seq` is set to `val` after the update's writes.
struct StepSeq {
    unsigned* seq = nullptr;   // null: one step per kernel
    unsigned base = 0;         // arrivals of the launch's earlier steps
    unsigned val = 0;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Block sums into partial slot `slot` of `nslots`; the last of the nslots CTAs
// to arrive adds the partials in slot order and runs the scalar update.
// Warp `leader` publishes the CTA's partials and, in the last CTA, runs the
// update; the other warps are done after the block sum.  The CTA barrier in
// the block sum orders every thread's field stores before the leader's fence
// and arrival, which a persistent launch relies on (the next step of a
// one-step kernel reads them after this grid has completed).  `state` (may be
// null) is the ensemble form's per-lattice word: that CTA toggles its bit 0
// (the ping-pong half) after a step (`toggle`), and sets bit 1 once the
// lattice has stopped.  With `sq.seq`, arrivals count on from `sq.base`
// without a reset and the last CTA sets *sq.seq = sq.val after the update.
__device__ __forceinline__ void finish_sums_slot(df64 (&v)[3], SplitCtl* ctl, const PotDev& P, const SplitConst& K,
                                                 double* part, unsigned* counter, double* a_trace, int slot,
                                                 int nslots, int* state, bool toggle, int leader = 0,
                                                 StepSeq sq = StepSeq()) {
    block_sum_df<3>(v, leader);
    if ((int)(threadIdx.x >> 5) != leader) return;
    const int lane = threadIdx.x & 31;
    df64* pd = reinterpret_cast<df64*>(part);   // one df64 per double slot
    int last = 0;
    if (lane == 0) {
        pd[3 * slot] = v[0];
        pd[3 * slot + 1] = v[1];
        pd[3 * slot + 2] = v[2];
        __threadfence();
        last = (atomicAdd(counter, 1u) == sq.base + (unsigned)nslots - 1);
        // in a persistent launch this SM may have read earlier steps' partials:
        // the fence orders the reads below after the other CTAs' writes
        if (last && sq.seq) __threadfence();
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    df64 tot[3];
    sum_partials_df<3>(pd, nslots, tot);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        tot[q].hi = __shfl_sync(0xffffffffu, tot[q].hi, 0);
        tot[q].lo = __shfl_sync(0xffffffffu, tot[q].lo, 0);
    }
    SplitCtl& C = *ctl;
    int error = 0;
    if (lane == 0) {
        if (!sq.seq) *counter = 0;
        if (state && toggle) *state ^= 1;
        error = C.error;
    }
    error = __shfl_sync(0xffffffffu, error, 0);
    const int pre = C.pre_claim && C.pre.ok;
    const int fast = pre && C.pre.fast;
    __syncwarp();
    if (lane == 0) {
        C.pre_claim = 0;
        C.pre.ok = 0;
    }
    if (fast && !error) {
        if (lane == 0) split_scalars_fast(C, tot);
    } else {
        // an update still deferred (only when no CTA of this step claimed the precompute)
        split_apply_deferred(C, a_trace);
        __syncwarp();
        const double sums[3] = {df_to(tot[0]), df_to(tot[1]), df_to(tot[2])};
        if (lane == 0) {
            C.sums[0] = sums[0];
            C.sums[1] = sums[1];
            C.sums[2] = sums[2];
        }
        if (error) {
            if (lane == 0) { C.active = 0; C.done = 1; }
        } else if (pre) {
            split_scalars_pre(C, P, sums, a_trace);
        } else {
            split_scalars_warp(C, P, K, sums, a_trace);
        }
    }
    __syncwarp();
    if (lane == 0 && state && C.done) *state |= 2;
    if (lane == 0 && sq.seq) {
        __threadfence();
        st_release(sq.seq, sq.val);
    }
}

__device__ __forceinline__ void finish_sums(df64 (&v)[3], SplitCtl* ctl, const PotDev& P, const SplitConst& K,
                                            double* part, unsigned* counter, double* a_trace) {
    finish_sums_slot(v, ctl, P, K, part, counter, a_trace, blockIdx.x + gridDim.x * blockIdx.y, gridDim.x * gridDim.y,
                     nullptr, false);
}

// Sums of the current dphi (start of a leapfrog call), thread per site:
// One CTA's share (slot of nslots, grid-stride over the sites) of the sums.
template <bool TABLE>
__device__ __forceinline__ void prime_body(const float* __restrict__ x, SplitCtl* ctl, const PotDev& P,
                                           const SplitConst& K, double* part, unsigned* counter, double* a_trace,
                                           int lg, int slot, int nslots, int* state) {
    __shared__ float su[kWin + 1], sA[kWin], ss[kWin];
    __shared__ int sn;
    __shared__ SplitWin W;
    if (threadIdx.x == 0) sn = 0;
    if (TABLE && threadIdx.x < 32) {
        // every CTA forms the window around the current phibar itself
        int err = 0;
        build_window_warp(W, P, P.V, P.slopeV, ctl->phibar, &err);
        __syncwarp();
        if (threadIdx.x == 0) sn = err ? -1 : W.n;
        if (!err) {
            if (threadIdx.x <= W.n) su[threadIdx.x] = W.u[threadIdx.x];
            if (threadIdx.x < W.n) { sA[threadIdx.x] = W.A[threadIdx.x]; ss[threadIdx.x] = W.s[threadIdx.x]; }
        }
    }
    __syncthreads();
    const long long gs = 1LL << (3 * lg);
    const int m = (1 << lg) - 1;
    Kahan g, s1, s2;
    bool bad = TABLE && sn < 0;
    for (long long id = (long long)slot * kThreads + threadIdx.x; id < gs; id += (long long)nslots * kThreads) {
        const int k = (int)(id & m), j = (int)((id >> lg) & m), i = (int)(id >> (2 * lg));
        const float xc = x[id];
        const float xk = x[id - k + ((k + 1) & m)];
        const float xj = x[id + ((long long)(((j + 1) & m) - j) << lg)];
        const float xi = x[id + ((long long)(((i + 1) & m) - i) << (2 * lg))];
        const float dk = xk - xc, dj = xj - xc, di = xi - xc;
        g.add(dk * dk + dj * dj + di * di);
        s1.add(xc);
        if (TABLE) {
            if (sn < 0) {
                bad = true;
            } else {
                const int q = window_find(su, sn, xc);
                s2.add(q >= 0 ? sA[q] + ss[q] * xc : far_line(P, P.V, P.slopeV, &W.phibar, xc, bad));
            }
        } else {
            s2.add(xc * xc);
        }
    }
    if (bad) {
        if (atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = ctl->phibar;
    }
    df64 v[3] = {g.df(), s1.df(), s2.df()};
    finish_sums_slot(v, ctl, P, K, part, counter, a_trace, slot, nslots, state, false);
}

struct SplitBufs {
    const float* xs;   // dphi (step n)
    float* xd;         // dphi (step n+1)
    const float* ps;   // dpi  (n-1/2)
    float* pd;         // dpi  (n+1/2)
    // compensated form: the Kahan residuals of dphi and dpi (bf16; the value
    // is x - residual), read for step n and written for step n+1
    const unsigned short* xls = nullptr;
    unsigned short* xld = nullptr;
    const unsigned short* pls = nullptr;
    unsigned short* pld = nullptr;
};

// Compensated form: v + inc with Kahan's compensated summation (the value is
// v - c); returns the new v and updates c.  Over a run's ~10^4 steps the
// rounding of a plain FP32 update accumulates as a random walk; with the
// residual carried from step to step the state keeps the precision of one
// rounding (Kahan, CACM 8 (1965) 40).
__device__ __forceinline__ float kahan_add(float v, float inc, float& c) {
    const float y = inc - c;
    const float t = v + y;
    c = (t - v) - y;
    return t;
}

// Four bf16 residuals <-> float4 (round to nearest even), through L2: in a
// persistent launch the residuals a step reads were written by other CTAs
// during the launch.
__device__ __forceinline__ uint2 ld_res4(const unsigned short* p) {
    uint2 u;
    asm volatile("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(u.x), "=r"(u.y) : "l"(p));
    return u;
}

__device__ __forceinline__ float4 unpack_res4(uint2 u) {
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u), __uint_as_float(u.y << 16),
                       __uint_as_float(u.y & 0xFFFF0000u));
}

__device__ __forceinline__ unsigned bf16x2_rn(float lo, float hi) {
    unsigned r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void st_res4(unsigned short* p, float4 v) {
    const uint2 u = make_uint2(bf16x2_rn(v.x, v.y), bf16x2_rn(v.z, v.w));
    *reinterpret_cast<uint2*>(p) = u;
}

// Asynchronous global -> shared copies (cp.async), so the planes a CTA will
// need next are in flight while it works on the current one.
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

// Programmatic dependent launch: a step kernel lets the next one be launched
// at once (its CTAs take SM slots as this kernel's CTAs exit) and waits for
// the previous kernel to complete before it reads anything that kernel
// wrote.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
template <int n>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(n) : "memory"); }
// Barrier 1 over the first NT threads of the block (the warps that march).
template <int NT>
__device__ __forceinline__ void march_sync() { asm volatile("bar.sync 1, %0;\n" ::"n"(NT) : "memory"); }

// Bulk asynchronous copies (TMA engine) into shared memory with mbarrier
// completion: one instruction moves a whole row, and the threads only wait on
// the barrier of the group.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase of the given parity, at most `limit` polls; false if
// it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned limit) {
    for (unsigned t = 0; t < limit; ++t)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Orders this thread's earlier shared-memory accesses before later bulk
// copies into the same memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

constexpr unsigned kMbarPolls = 1u << 20;   // far beyond any copy's latency (about a second at most)

// Poll limit of the step kernels' bounded waits: the control block's value
// (set through iegpu_set_wait_limit), or the default.
__device__ __forceinline__ unsigned wait_limit(const SplitCtl* ctl) {
    const unsigned v = __ldcg(&ctl->spin_polls);
    return v ? v : kMbarPolls;
}

constexpr int kPrefetch = 3;   // planes in flight ahead of the one being computed
constexpr int kPhiSlots = 6;   // three stencil planes + kPrefetch
constexpr int kPiSlots = 4;    // one plane in use + kPrefetch
constexpr int kColOff = 4;     // shared-memory column of k = 0 (16-byte aligned rows)

// Shared-memory floats of the step kernel for tile TJ x TK.
__host__ __device__ inline int split_step_smem_floats(int TJ, int TK) {
    const int RS = TK + 8;
    return kPhiSlots * (TJ + 3) * RS + kPiSlots * (TJ + 1) * RS + 2 * (TJ + 1) * (TK + 1) + 2 * (3 * kWin + 1);
}


// Full-row variant of the step for 32 <= N <= 512: a tile is TJ rows of
// complete k lines, so the k direction is periodic inside shared memory and
// needs no halo.  Warp w computes row j0+w for w = 0..TJ (row TJ is the +j
// halo row whose new values only feed the j differences of row TJ-1); lane l
// handles k = l + 32c, c < C = N/32.  The planes come in through a cp.async
// ring kRowPrefetch planes ahead.  Row partial sums are added per plane into
// Kahan-compensated per-thread accumulators.
__host__ __device__ inline int split_row_smem_floats(int TJ, int N, int PF) {
    return (3 + PF) * (TJ + 3) * N + (1 + PF) * (TJ + 1) * N + (TJ + 1) * N + 2 * (3 * kWin + 1);
}

// PF = planes prefetched ahead; the i range [0, N) is cut into `chunks`
// nearly equal plane ranges (any count, so the grid can match the SMs).
// One CTA: rows j0 .. j0+TJ-1, planes i0 .. i0+CH-1; its sums go to partial
// slot `slot` of `nslots`.
// sq: the publication of the step's update (persistent ensemble launch).
template <bool TABLE, int C, int TJ, int PF>
__device__ __forceinline__ void rows_body(const SplitBufs& B, SplitCtl* ctl, const PotDev& P, const SplitConst& K,
                                          double* part, unsigned* counter, double* a_trace, int j0, int i0, int CH,
                                          int slot, int nslots, int* state, StepSeq sq = StepSeq()) {
    constexpr int kRowPrefetch = PF, kRowPhiSlots = 3 + PF, kRowPiSlots = 1 + PF;
    constexpr int N = 32 * C, m = N - 1;
    constexpr int lgN = (C == 1) ? 5 : (C == 2) ? 6 : (C == 4) ? 7 : (C == 8) ? 8 : 9;
    constexpr int RP = (TJ + 3) * N, PP = (TJ + 1) * N, NTH = (TJ + 1) * 32;
    extern __shared__ __align__(16) float smem[];
    float* ring = smem;
    float* pis = ring + kRowPhiSlots * RP;
    float* nb = pis + kRowPiSlots * PP;
    float* wk = nb + (TJ + 1) * N;
    float* wv = wk + 3 * kWin + 1;
    __shared__ int nk_s, nv_s, active_s;
    __shared__ double wbar[4];
    __shared__ float cf[6];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // the control block is read through L2: in a persistent ensemble launch
    // another CTA wrote it during the launch
    if (tid == 0) {
        const SplitCtl& Cc = *ctl;
        active_s = __ldcg(&Cc.active);
        cf[0] = __ldcg(&Cc.d); cf[1] = __ldcg(&Cc.lapl); cf[2] = __ldcg(&Cc.fric); cf[3] = __ldcg(&Cc.pn);
        cf[4] = __ldcg(&Cc.kv);
        nk_s = __ldcg(&Cc.wk.n);
        nv_s = __ldcg(&Cc.wv.n);
    }
    if (TABLE) {
        for (int q = tid; q <= kWin; q += NTH) { wk[q] = __ldcg(&ctl->wk.u[q]); wv[q] = __ldcg(&ctl->wv.u[q]); }
        for (int q = tid; q < kWin; q += NTH) {
            wk[kWin + 1 + q] = __ldcg(&ctl->wk.A[q]); wk[2 * kWin + 1 + q] = __ldcg(&ctl->wk.s[q]);
            wv[kWin + 1 + q] = __ldcg(&ctl->wv.A[q]); wv[2 * kWin + 1 + q] = __ldcg(&ctl->wv.s[q]);
        }
        load_win_centres<true>(wbar, ctl);
    }
    __syncthreads();
    if (!active_s) return;
    const float d = cf[0], lap_n = cf[1], fric = cf[2], pn = cf[3], kv = cf[4];
    const WinCache ck = win_cache<TABLE>(wk, nk_s), cv = win_cache<TABLE>(wv, nv_s);

    auto issue_phi = [&](int i) {
        float* dst = ring + ((i - i0 + 1) % kRowPhiSlots) * RP;
        const float* src = B.xs + ((long long)(i & m) << (2 * lgN));
        constexpr int ops = (TJ + 3) * (N / 4);
        for (int o = tid; o < ops; o += NTH) {
            const int r = o / (N / 4), q = o - r * (N / 4);
            cp_async16(dst + r * N + 4 * q, src + ((long long)((j0 + r - 1) & m) << lgN) + 4 * q);
        }
    };
    auto issue_pi = [&](int i) {
        float* dst = pis + ((i - i0) % kRowPiSlots) * PP;
        const float* src = B.ps + ((long long)(i & m) << (2 * lgN));
        constexpr int ops = (TJ + 1) * (N / 4);
        for (int o = tid; o < ops; o += NTH) {
            const int r = o / (N / 4), q = o - r * (N / 4);
            cp_async16(dst + r * N + 4 * q, src + ((long long)((j0 + r) & m) << lgN) + 4 * q);
        }
    };

    Kahan g, s1, s2;
    bool bad = false;
    float xprev[C];
    issue_phi(i0 - 1);
    issue_phi(i0);
    cp_commit();
    for (int q = 0; q < kRowPrefetch; ++q) {
        if (q + 1 <= CH + 1) issue_phi(i0 + 1 + q);
        if (q <= CH) issue_pi(i0 + q);
        cp_commit();
    }
    const int jl = w;              // row of this warp (TJ: halo row)
    const bool interior = jl < TJ;
    for (int p = 0; p <= CH; ++p) {
        const int i = i0 + p;
        cp_wait<kRowPrefetch - 1>();
        __syncthreads();
        const float* pc = ring + ((p + 1) % kRowPhiSlots) * RP + (jl + 1) * N;
        const float* pu = ring + ((p + 2) % kRowPhiSlots) * RP + (jl + 1) * N;
        const float* pl = ring + (p % kRowPhiSlots) * RP + (jl + 1) * N;
        const float* pp = pis + (p % kRowPiSlots) * PP + jl * N;
        float xnew[C];
        float rs1 = 0.f, rs2 = 0.f;
        const bool store = interior && p < CH;
        const long long gb = ((long long)(i & m) << (2 * lgN)) + ((long long)(j0 + jl) << lgN);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int k = lane + 32 * c;
            const float x = pc[k];
            const float lap = pc[(k + 1) & m] + pc[(k - 1) & m] + pc[k + N] + pc[k - N] + pu[k] + pl[k] - 6.f * x;
            const float pi0 = pp[k];
            const float dv = split_dv<TABLE>(x, wk, nk_s, ck, pn, kv, bad, P, wbar);
            const float pin = pi0 + d * (lap_n * lap - fric * pi0 - dv);
            const float xn = x + d * pin;
            xnew[c] = xn;
            nb[jl * N + k] = xn;
            if (store) {
                B.xd[gb + k] = xn;
                B.pd[gb + k] = pin;
                rs1 += xn;
                rs2 += split_v<TABLE>(xn, wv, nv_s, cv, bad, P, wbar + 2);
            }
        }
        __syncthreads();
        // planes kRowPrefetch ahead go into the slots no longer needed
        if (p + kRowPrefetch + 1 <= CH + 1) issue_phi(i + 1 + kRowPrefetch);
        if (p + kRowPrefetch <= CH) issue_pi(i + kRowPrefetch);
        cp_commit();
        if (interior) {
            float rg = 0.f;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int k = lane + 32 * c;
                if (p < CH) {
                    const float dk = nb[jl * N + ((k + 1) & m)] - xnew[c];
                    const float dj = nb[(jl + 1) * N + k] - xnew[c];
                    rg += dk * dk + dj * dj;
                }
                if (p >= 1) {
                    const float di = xnew[c] - xprev[c];
                    rg += di * di;
                }
                xprev[c] = xnew[c];
            }
            g.add(rg);
            if (store) { s1.add(rs1); s2.add(rs2); }
        }
    }
    cp_wait<0>();
    if (bad) {
        if (atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = ctl->phibar;
    }
    // a lattice stepped by one CTA runs its update straight after its tile:
    // there is nothing for a precomputed part to overlap with
    if (nslots > 1) maybe_precompute(ctl, P, K);
    df64 v[3] = {g.df(), s1.df(), s2.df()};
    finish_sums_slot(v, ctl, P, K, part, counter, a_trace, slot, nslots, state, true, 0, sq);
}

// Vector variant of the row kernel for N >= 128: lane l owns the four
// consecutive sites k = 4(l + 32v) .. +3, v < C4 = N/128, so plane rows move
// with 128-bit shared and global accesses and the k +- 1 neighbours across
// lanes come by warp shuffles.  The new planes are double-buffered, which
// leaves one barrier per plane: iteration p finishes the differences of plane
// p-1 and computes plane p.  A block is TJ + 2 warps: TJ + 1 march (rows
// j0 .. j0+TJ), the last forms the precomputed part of the scalar update.
__host__ __device__ inline int row4_threads(int TJ) { return (TJ + 2) * 32; }
__host__ __device__ inline int split_row4_smem_floats(int TJ, int N, int PF) {
    return (3 + PF) * (TJ + 3) * N + (1 + PF) * (TJ + 1) * N + 2 * (TJ + 1) * N + 2 * (3 * kWin + 1);
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Geometry of one march of the vector row kernel: the units [s, e) of one
// row tile that a march over a CTA's range [u0, u1) covers next, from the
// running unit u (moved past them); planes i0 .. i0+CH-1 of rows j0 .. j0+TJ-1.
struct Row4March {
    long long s, e;
    int j0, i0, CH;
    bool rev;
    __device__ __forceinline__ int plane(int q) const { return rev ? i0 + CH - 1 - q : i0 + q; }
};
template <int N, int TJ>
__device__ __forceinline__ Row4March row4_march(long long& u, long long u0, long long u1, bool rev) {
    Row4March M;
    if (rev) {
        M.e = u;
        M.s = ((M.e - 1) / N) * N;
        if (M.s < u0) M.s = u0;
        u = M.s;
    } else {
        M.s = u;
        M.e = (M.s / N + 1) * N;
        if (M.e > u1) M.e = u1;
        u = M.e;
    }
    M.j0 = (int)(M.s / N) * TJ;
    M.i0 = (int)(M.s % N);
    M.CH = (int)(M.e - M.s);
    M.rev = rev;
    return M;
}

// cp.async copies of march position q into its ring slots, by the NTH march
// threads: dphi rows j0-1 .. j0+TJ+1 (slot (q+1) mod PHS), dpi rows j0 ..
// j0+TJ (slot q mod PIS).
template <int C4, int TJ, int PF>
__device__ __forceinline__ void row4_issue_phi(float* ring, const float* xs, const Row4March& M, int q) {
    constexpr int N = 128 * C4, m = N - 1, lgN = (C4 == 1) ? 7 : (C4 == 2) ? 8 : 9;
    constexpr int RP = (TJ + 3) * N, NTH = (TJ + 1) * 32, PHS = 3 + PF;
    float* dst = ring + ((q + 1) % PHS) * RP;
    const float* src = xs + ((long long)(M.plane(q) & m) << (2 * lgN));
    constexpr int ops = (TJ + 3) * (N / 4);
    for (int o = threadIdx.x; o < ops; o += NTH) {
        const int r = o / (N / 4), c = o - r * (N / 4);
        cp_async16(dst + r * N + 4 * c, src + ((long long)((M.j0 + r - 1) & m) << lgN) + 4 * c);
    }
}
template <int C4, int TJ, int PF>
__device__ __forceinline__ void row4_issue_pi(float* pis, const float* ps, const Row4March& M, int q) {
    constexpr int N = 128 * C4, m = N - 1, lgN = (C4 == 1) ? 7 : (C4 == 2) ? 8 : 9;
    constexpr int PP = (TJ + 1) * N, NTH = (TJ + 1) * 32, PIS = 1 + PF;
    float* dst = pis + (q % PIS) * PP;
    const float* src = ps + ((long long)(M.plane(q) & m) << (2 * lgN));
    constexpr int ops = (TJ + 1) * (N / 4);
    for (int o = threadIdx.x; o < ops; o += NTH) {
        const int r = o / (N / 4), c = o - r * (N / 4);
        cp_async16(dst + r * N + 4 * c, src + ((long long)((M.j0 + r) & m) << lgN) + 4 * c);
    }
}
// The copies a march starts with: dphi positions -1 and 0 (one group), then
// PF groups of dphi position q+1 and dpi position q.
template <int C4, int TJ, int PF>
__device__ __forceinline__ void row4_issue_start(float* ring, float* pis, const SplitBufs& B, const Row4March& M) {
    row4_issue_phi<C4, TJ, PF>(ring, B.xs, M, -1);
    row4_issue_phi<C4, TJ, PF>(ring, B.xs, M, 0);
    cp_commit();
    for (int q = 0; q < PF; ++q) {
        if (q + 1 <= M.CH + 1) row4_issue_phi<C4, TJ, PF>(ring, B.xs, M, 1 + q);
        if (q <= M.CH) row4_issue_pi<C4, TJ, PF>(pis, B.ps, M, q);
        cp_commit();
    }
}

template <bool TABLE, int C4, int TJ, int PF, bool TMA = false, bool COMP = false>
__device__ __forceinline__ bool rows4_body(const SplitBufs& B, SplitCtl* ctl, const PotDev& P, const SplitConst& K,
                                           double* part, unsigned* counter, double* a_trace, long long u0,
                                           long long u1, int slot, int nslots, int* state, bool rev,
                                           bool preissued = false, StepSeq sq = StepSeq()) {
    constexpr int N = 128 * C4, m = N - 1;
    constexpr bool kLift = C4 >= 4;   // 512^3: the branch-free window search
    constexpr bool kWide = C4 >= 4;   // 512^3: five cached brackets
    constexpr int lgN = (C4 == 1) ? 7 : (C4 == 2) ? 8 : 9;
    constexpr int RP = (TJ + 3) * N, PP = (TJ + 1) * N, NBP = (TJ + 1) * N, NTH = (TJ + 1) * 32;
    constexpr int PHS = 3 + PF, PIS = 1 + PF;
    extern __shared__ __align__(16) float smem[];
    float* ring = smem;
    float* pis = ring + PHS * RP;
    float* nb = pis + PIS * PP;
    float* wk = nb + 2 * NBP;
    float* wv = wk + 3 * kWin + 1;
    __shared__ int nk_s, nv_s, active_s;
    __shared__ double wbar[4];
    __shared__ float cf[6];
    __shared__ unsigned tma_fail_g, tma_issued, mbar_limit;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // the control block is read through L2: in a persistent launch the last
    // CTA of the step before wrote it during this kernel
    if (tid == 0) {
        const SplitCtl& Cc = *ctl;
        // a step that a failed wait of this call has marked is not taken
        active_s = __ldcg(&Cc.active) && !__ldcg(&Cc.error);
        tma_fail_g = 0xFFFFFFFFu;
        tma_issued = 0u;
        mbar_limit = wait_limit(ctl);
        cf[0] = __ldcg(&Cc.d); cf[1] = __ldcg(&Cc.lapl); cf[2] = __ldcg(&Cc.fric);
        cf[3] = __ldcg(&Cc.pn); cf[4] = __ldcg(&Cc.kv);
        nk_s = __ldcg(&Cc.wk.n);
        nv_s = __ldcg(&Cc.wv.n);
    }
    if (TABLE) {
        for (int q = tid; q <= kWin; q += NTH) { wk[q] = __ldcg(&ctl->wk.u[q]); wv[q] = __ldcg(&ctl->wv.u[q]); }
        for (int q = tid; q < kWin; q += NTH) {
            wk[kWin + 1 + q] = __ldcg(&ctl->wk.A[q]); wk[2 * kWin + 1 + q] = __ldcg(&ctl->wk.s[q]);
            wv[kWin + 1 + q] = __ldcg(&ctl->wv.A[q]); wv[2 * kWin + 1 + q] = __ldcg(&ctl->wv.s[q]);
        }
        load_win_centres<true>(wbar, ctl);
    }
    __syncthreads();
    if (!active_s) {
        if (!TMA) cp_wait<0>();   // copies a persistent launch issued ahead
        return false;
    }
    const float d = cf[0], lap_n = cf[1], fric = cf[2], pn = cf[3], kv = cf[4];
    const int nk = nk_s, nv = nv_s;
    const WinCache ck = win_cache<TABLE, kWide>(wk, nk), cv = win_cache<TABLE, kWide>(wv, nv);

    Kahan g, s1, s2;
    bool bad = false;
    const int jl = w;
    const bool interior = jl < TJ;
    // TMA: group g of a march (g = -1: dphi planes i0-1, i0; g >= 0: dphi plane
    // i0+g+1 and dpi plane i0+g; g > CH: empty) completes barrier G % NB,
    // G = the CTA's running group count.
    constexpr int NB = PF + 2;
    __shared__ __align__(8) unsigned long long bars[TMA ? NB : 1];
    unsigned G0 = 0;
    bool aborted = false;   // a bulk-copy wait gave up: no more copies are issued
    if (TMA) {
        if (tid == 0) {
            for (int q = 0; q < NB; ++q) mbar_init(&bars[q], 1);
            mbar_init_fence();
        }
        __syncthreads();
    }
    // rev: march backwards (units from u1-1 down, planes from high i to low),
    // so that a step first reads what the step before, marching the other
    // way, wrote last, while part of it is still in L2.
    // Units u0 .. u1-1, unit u = (row tile u / N, plane u mod N): one march
    // along i per row tile the range touches.
    // The warp after the march warps forms the sum-independent part of this
    // step's scalar update (split_precompute) in the first CTA to claim it,
    // while the march warps stream; the march warps meet on barrier 1.
    if (w == TJ + 1) {
        int claimed = 0;
        if (lane == 0) claimed = atomicCAS(&ctl->pre_claim, 0, 1) == 0;
        claimed = __shfl_sync(0xffffffffu, claimed, 0);
        if (claimed) {
            // the FP64 part of the update that started this step, then the
            // sum-independent part of the one that ends it
            split_apply_deferred(*ctl, a_trace);
            split_precompute(*ctl, P, K, true);
            __threadfence();
        }
    }
    const bool marcher = w <= TJ;
    bool first = true;
    for (long long u = rev ? u1 : u0; marcher && !aborted && (rev ? u > u0 : u < u1);) {
        // this march covers units [s, e) of one row tile
        const Row4March M = row4_march<N, TJ>(u, u0, u1, rev);
        const int j0 = M.j0, CH = M.CH;
        // march position q -> plane; q = -1 and q = CH are the halo planes
        auto plane = [&](int q) { return M.plane(q); };
        auto issue_phi = [&](int q) { row4_issue_phi<C4, TJ, PF>(ring, B.xs, M, q); };
        auto issue_pi = [&](int q) { row4_issue_pi<C4, TJ, PF>(pis, B.ps, M, q); };
        // TMA group g, issued by warp 0 (lane 0 arms the barrier first)
        auto issue_group = [&](int gi) {
            unsigned long long* bar = &bars[(G0 + (unsigned)(gi + 1)) % NB];
            if (lane == 0) tma_issued = G0 + (unsigned)(gi + 2);   // groups issued so far
            const int nphi = gi < 0 ? 2 * (TJ + 3) : (gi <= CH ? TJ + 3 : 0);
            const int npi = (gi >= 0 && gi <= CH) ? TJ + 1 : 0;
            if (lane == 0) mbar_expect_tx(bar, (unsigned)((nphi + npi) * N * 4));
            __syncwarp();
            for (int r = lane; r < nphi + npi; r += 32) {
                if (r < nphi) {
                    const int q = gi < 0 ? (r < TJ + 3 ? -1 : 0) : gi + 1;
                    const int rr = gi < 0 ? r % (TJ + 3) : r;
                    float* dst = ring + ((q + 1) % PHS) * RP + rr * N;
                    const float* src = B.xs + ((long long)(plane(q) & m) << (2 * lgN)) + ((long long)((j0 + rr - 1) & m) << lgN);
                    bulk_g2s(dst, src, N * 4, bar);
                } else {
                    const int rr = r - nphi, q = gi;
                    float* dst = pis + (q % PIS) * PP + rr * N;
                    const float* src = B.ps + ((long long)(plane(q) & m) << (2 * lgN)) + ((long long)((j0 + rr) & m) << lgN);
                    bulk_g2s(dst, src, N * 4, bar);
                }
            }
        };
        auto wait_group = [&](int gi) {
            // a wait that gives up records its group; after the next march
            // barrier every marcher stops and warp 0 issues nothing more
            const unsigned Gq = G0 + (unsigned)(gi + 1);
            if (!mbar_wait(&bars[Gq % NB], (Gq / NB) & 1u, mbar_limit)) atomicMin(&tma_fail_g, Gq);
        };
        float4 xp1[C4], xp2[C4];   // new values of this row: plane p-1 and p-2
        uint2 rxn[C4], rpn[C4];    // compensated form: residuals of the next plane
        if (TMA) {
            if (w == 0) {
                fence_proxy_async();
                issue_group(-1);
                for (int q = 0; q < PF; ++q) issue_group(q);
            }
        } else if (!(first && preissued)) {
            row4_issue_start<C4, TJ, PF>(ring, pis, B, M);
        }
        first = false;
        // differences of plane p-1 (k and j) and of the pair (p-2, p-1) (i)
        auto diffs = [&](int p, bool kj) {
            const float* nr = nb + ((p - 1) & 1) * NBP;
            float rg = 0.f;
    #pragma unroll
            for (int v = 0; v < C4; ++v) {
                const int k = 4 * (lane + 32 * v);
                const float4 xc = xp1[v];
                if (kj) {
                    // x(k+4): lane+1's first element, or the next vector's lane 0 (periodic)
                    const float nxt_same = __shfl_down_sync(0xffffffffu, xc.x, 1);
                    const float nxt_wrap = __shfl_sync(0xffffffffu, xp1[(v + 1) % C4].x, 0);
                    const float x4 = lane == 31 ? nxt_wrap : nxt_same;
                    const float4 up = ld4(nr + (jl + 1) * N + k);
                    const float a0 = xc.y - xc.x, a1 = xc.z - xc.y, a2 = xc.w - xc.z, a3 = x4 - xc.w;
                    const float b0 = up.x - xc.x, b1 = up.y - xc.y, b2 = up.z - xc.z, b3 = up.w - xc.w;
                    rg += a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + b0 * b0 + b1 * b1 + b2 * b2 + b3 * b3;
                }
                if (p >= 2) {
                    const float4 xo = xp2[v];
                    const float c0 = xc.x - xo.x, c1 = xc.y - xo.y, c2 = xc.z - xo.z, c3 = xc.w - xo.w;
                    rg += c0 * c0 + c1 * c1 + c2 * c2 + c3 * c3;
                }
            }
            g.add(rg);
        };
        for (int p = 0; p <= CH; ++p) {
            const int i = plane(p);
            if (TMA) {
                if (p == 0) wait_group(-1);
                wait_group(p);
            } else {
                cp_wait<PF - 1>();
            }
            march_sync<NTH>();
            if (TMA && *(volatile unsigned*)&tma_fail_g != 0xFFFFFFFFu) {
                aborted = true;
                break;
            }
            // planes PF ahead go into the slots of planes no longer read
            if (TMA) {
                if (w == 0) {
                    fence_proxy_async();
                    issue_group(p + PF);
                }
            } else {
                if (p + PF + 1 <= CH + 1) issue_phi(p + 1 + PF);
                if (p + PF <= CH) issue_pi(p + PF);
                cp_commit();
            }
            if (interior && p >= 1) diffs(p, true);
            const float* pc = ring + ((p + 1) % PHS) * RP + (jl + 1) * N;
            const float* pu = ring + ((p + 2) % PHS) * RP + (jl + 1) * N;
            const float* pl = ring + (p % PHS) * RP + (jl + 1) * N;
            const float* pp = pis + (p % PIS) * PP + jl * N;
            float* nw = nb + (p & 1) * NBP + jl * N;
            const bool store = interior && p < CH;
            // (j0 + jl) & m: the halo row of the last tile wraps (its values
            // are computed here, as its owner computes them, but not stored)
            const long long gb = ((long long)(i & m) << (2 * lgN)) + ((long long)((j0 + jl) & m) << lgN);
            float4 xs[C4];
            // compensated form: this plane's residuals (loaded one plane
            // ahead), and the loads of the next plane's
            uint2 rx[C4], rp[C4];
            if (COMP) {
    #pragma unroll
                for (int v = 0; v < C4; ++v) {
                    rx[v] = p == 0 ? ld_res4(B.xls + gb + 4 * (lane + 32 * v)) : rxn[v];
                    rp[v] = p == 0 ? ld_res4(B.pls + gb + 4 * (lane + 32 * v)) : rpn[v];
                }
                if (p < CH) {
                    const long long gn = ((long long)(plane(p + 1) & m) << (2 * lgN)) + ((long long)((j0 + jl) & m) << lgN);
    #pragma unroll
                    for (int v = 0; v < C4; ++v) {
                        rxn[v] = ld_res4(B.xls + gn + 4 * (lane + 32 * v));
                        rpn[v] = ld_res4(B.pls + gn + 4 * (lane + 32 * v));
                    }
                }
            }
    #pragma unroll
            for (int v = 0; v < C4; ++v) xs[v] = ld4(pc + 4 * (lane + 32 * v));
            float rs1 = 0.f, rs2 = 0.f;
    #pragma unroll
            for (int v = 0; v < C4; ++v) {
                const int k = 4 * (lane + 32 * v);
                const float4 x = xs[v];
                // k-1 and k+4 with periodic wrap across vectors and the row
                const float lft_same = __shfl_up_sync(0xffffffffu, x.w, 1);
                const float lft_wrap = __shfl_sync(0xffffffffu, xs[(v + C4 - 1) % C4].w, 31);
                const float rgt_same = __shfl_down_sync(0xffffffffu, x.x, 1);
                const float rgt_wrap = __shfl_sync(0xffffffffu, xs[(v + 1) % C4].x, 0);
                const float xl = lane == 0 ? lft_wrap : lft_same;
                const float xr = lane == 31 ? rgt_wrap : rgt_same;
                const float4 up = ld4(pc + k + N), dn = ld4(pc + k - N), iu = ld4(pu + k), il = ld4(pl + k);
                const float4 pi = ld4(pp + k);
                float4 lap;
                lap.x = (x.y + xl) + (up.x + dn.x) + (iu.x + il.x) - 6.f * x.x;
                lap.y = (x.z + x.x) + (up.y + dn.y) + (iu.y + il.y) - 6.f * x.y;
                lap.z = (x.w + x.y) + (up.z + dn.z) + (iu.z + il.z) - 6.f * x.z;
                lap.w = (xr + x.z) + (up.w + dn.w) + (iu.w + il.w) - 6.f * x.w;
                float4 pin, xn;
                if (COMP) {
                    float4 cx = unpack_res4(rx[v]), cp = unpack_res4(rp[v]);
                    pin.x = kahan_add(pi.x, d * (lap_n * lap.x - fric * pi.x - split_dv<TABLE, kLift, kWide>(x.x, wk, nk, ck, pn, kv, bad, P, wbar)), cp.x);
                    pin.y = kahan_add(pi.y, d * (lap_n * lap.y - fric * pi.y - split_dv<TABLE, kLift, kWide>(x.y, wk, nk, ck, pn, kv, bad, P, wbar)), cp.y);
                    pin.z = kahan_add(pi.z, d * (lap_n * lap.z - fric * pi.z - split_dv<TABLE, kLift, kWide>(x.z, wk, nk, ck, pn, kv, bad, P, wbar)), cp.z);
                    pin.w = kahan_add(pi.w, d * (lap_n * lap.w - fric * pi.w - split_dv<TABLE, kLift, kWide>(x.w, wk, nk, ck, pn, kv, bad, P, wbar)), cp.w);
                    xn.x = kahan_add(x.x, d * pin.x, cx.x);
                    xn.y = kahan_add(x.y, d * pin.y, cx.y);
                    xn.z = kahan_add(x.z, d * pin.z, cx.z);
                    xn.w = kahan_add(x.w, d * pin.w, cx.w);
                    if (store) {
                        st_res4(B.xld + gb + k, cx);
                        st_res4(B.pld + gb + k, cp);
                    }
                } else {
                    pin.x = pi.x + d * (lap_n * lap.x - fric * pi.x - split_dv<TABLE, kLift, kWide>(x.x, wk, nk, ck, pn, kv, bad, P, wbar));
                    pin.y = pi.y + d * (lap_n * lap.y - fric * pi.y - split_dv<TABLE, kLift, kWide>(x.y, wk, nk, ck, pn, kv, bad, P, wbar));
                    pin.z = pi.z + d * (lap_n * lap.z - fric * pi.z - split_dv<TABLE, kLift, kWide>(x.z, wk, nk, ck, pn, kv, bad, P, wbar));
                    pin.w = pi.w + d * (lap_n * lap.w - fric * pi.w - split_dv<TABLE, kLift, kWide>(x.w, wk, nk, ck, pn, kv, bad, P, wbar));
                    xn.x = x.x + d * pin.x;
                    xn.y = x.y + d * pin.y;
                    xn.z = x.z + d * pin.z;
                    xn.w = x.w + d * pin.w;
                }
                st4(nw + k, xn);
                if (store) {
                    st4(B.xd + gb + k, xn);
                    st4(B.pd + gb + k, pin);
                    rs1 += (xn.x + xn.y) + (xn.z + xn.w);
                    rs2 += (split_v<TABLE, kLift, kWide>(xn.x, wv, nv, cv, bad, P, wbar + 2) + split_v<TABLE, kLift, kWide>(xn.y, wv, nv, cv, bad, P, wbar + 2)) +
                           (split_v<TABLE, kLift, kWide>(xn.z, wv, nv, cv, bad, P, wbar + 2) + split_v<TABLE, kLift, kWide>(xn.w, wv, nv, cv, bad, P, wbar + 2));
                }
                xp2[v] = xp1[v];
                xp1[v] = xn;
            }
            if (store) { s1.add(rs1); s2.add(rs2); }
        }
        // the last pair (CH-1, CH) along i
        if (interior) {
            float rg = 0.f;
    #pragma unroll
            for (int v = 0; v < C4; ++v) {
                const float4 xc = xp1[v], xo = xp2[v];
                const float c0 = xc.x - xo.x, c1 = xc.y - xo.y, c2 = xc.z - xo.z, c3 = xc.w - xo.w;
                rg += c0 * c0 + c1 * c1 + c2 * c2 + c3 * c3;
            }
            g.add(rg);
        }
        if (!TMA) cp_wait<0>();
        G0 += (unsigned)(CH + PF + 2);
        march_sync<NTH>();   // the ring is refilled by the next march
    }
    if (TMA && marcher) {
        // a wait gave up: drain the groups still in flight (bounded waits, in
        // issue order, at most NB of them) before the CTA leaves, so no bulk
        // copy lands in shared memory after it has exited
        march_sync<NTH>();
        const unsigned fg = *(volatile unsigned*)&tma_fail_g;
        if (fg != 0xFFFFFFFFu) {
            if (tid == 0) {
                const unsigned last = *(volatile unsigned*)&tma_issued;
                for (unsigned Gq = fg; Gq < last; ++Gq) mbar_wait(&bars[Gq % NB], (Gq / NB) & 1u, kMbarPolls);
                if (atomicCAS(&ctl->error, 0, IEGPU_ETIMEOUT) == 0) ctl->errval = 0.0;
            }
            march_sync<NTH>();
        }
    }
    cp_wait<0>();
    if (bad) {
        if (atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = ctl->phibar;
    }
    df64 v3[3] = {g.df(), s1.df(), s2.df()};
    finish_sums_slot(v3, ctl, P, K, part, counter, a_trace, slot, nslots, state, true, TJ + 1, sq);
    return true;
}

// Whole-plane variant of the step for small lattices (N = 32, 64): a CTA owns
// complete (j, k) planes of its chunk of i, so j and k are periodic inside
// shared memory and no halo rows are recomputed.  Thread t owns the float4
// vectors q = t + v*NT (v < V) of every plane: row j = q / (N/4), sites
// k = 4(q mod N/4) .. +3; the N/4 lanes of a row are adjacent in a warp, so
// the k +- 1 neighbours come by shuffles.  A plane of dphi and of dpi arrives
// as one contiguous N^2-float cp.async copy, PF planes ahead; the new planes
// are double-buffered (one barrier per plane), as in the vector row kernel.
// Threads of a whole-plane CTA and the CTAs per SM its registers are sized
// for: at N = 32, 128 threads with two vectors of each plane apiece and five
// CTAs per SM (about 100 registers, so the window caches and sums stay in
// registers); at N = 64, 512 threads and one CTA.
__host__ __device__ constexpr int plane_nt(int N) { return N == 32 ? 128 : 512; }
__host__ __device__ constexpr int plane_min_ctas(int N) { return N == 32 ? 5 : 1; }

__host__ __device__ inline int split_plane_smem_floats(int N, int PF) {
    return ((3 + PF) + (1 + PF) + 2) * N * N + 2 * (3 * kWin + 1);
}

template <bool TABLE, int N, int NT, int PF>
__device__ __forceinline__ void plane_body(const SplitBufs& B, SplitCtl* ctl, const PotDev& P, const SplitConst& K,
                                           double* part, unsigned* counter, double* a_trace, int i0, int CH,
                                           int slot, int nslots, int* state) {
    constexpr int m = N - 1, NN = N * N, Q = NN / 4, V = Q / NT, W = N / 4;
    constexpr int lgN = (N == 32) ? 5 : 6;
    constexpr int PHS = 3 + PF, PIS = 1 + PF;
    static_assert(V * NT == Q && (N == 32 || N == 64), "plane tiling");
    extern __shared__ __align__(16) float smem[];
    float* ring = smem;
    float* pis = ring + PHS * NN;
    float* nb = pis + PIS * NN;
    float* wk = nb + 2 * NN;
    float* wv = wk + 3 * kWin + 1;
    __shared__ int nk_s, nv_s, active_s;
    __shared__ double wbar[4];
    __shared__ float cf[6];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) {
        const SplitCtl& Cc = *ctl;
        active_s = Cc.active;
        cf[0] = Cc.d; cf[1] = Cc.lapl; cf[2] = Cc.fric; cf[3] = Cc.pn; cf[4] = Cc.kv;
        nk_s = Cc.wk.n;
        nv_s = Cc.wv.n;
    }
    if (TABLE) {
        for (int q = tid; q <= kWin; q += NT) { wk[q] = ctl->wk.u[q]; wv[q] = ctl->wv.u[q]; }
        for (int q = tid; q < kWin; q += NT) {
            wk[kWin + 1 + q] = ctl->wk.A[q]; wk[2 * kWin + 1 + q] = ctl->wk.s[q];
            wv[kWin + 1 + q] = ctl->wv.A[q]; wv[2 * kWin + 1 + q] = ctl->wv.s[q];
        }
        load_win_centres<false>(wbar, ctl);
    }
    __syncthreads();
    if (!active_s) return;
    const float d = cf[0], lap_n = cf[1], fric = cf[2], pn = cf[3], kv = cf[4];
    const int nk = nk_s, nv = nv_s;
    const WinCache ck = win_cache<TABLE>(wk, nk), cv = win_cache<TABLE>(wv, nv);
    // lanes of the same row: the previous and next vector (periodic in k)
    const int rowbase = lane & ~(W - 1);
    const int lprev = rowbase | ((lane + W - 1) & (W - 1));
    const int lnext = rowbase | ((lane + 1) & (W - 1));

    auto issue_phi = [&](int i) {
        float* dst = ring + ((i - i0 + 1) % PHS) * NN;
        const float* src = B.xs + ((long long)(i & m) << (2 * lgN));
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int q = tid + v * NT;
            cp_async16(dst + 4 * q, src + 4 * q);
        }
    };
    auto issue_pi = [&](int i) {
        float* dst = pis + ((i - i0) % PIS) * NN;
        const float* src = B.ps + ((long long)(i & m) << (2 * lgN));
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int q = tid + v * NT;
            cp_async16(dst + 4 * q, src + 4 * q);
        }
    };

    Kahan g, s1, s2;
    bool bad = false;
    float4 xp1[V], xp2[V];   // new values of this thread's vectors: plane p-1 and p-2
    issue_phi(i0 - 1);
    issue_phi(i0);
    cp_commit();
    for (int q = 0; q < PF; ++q) {
        if (q + 1 <= CH + 1) issue_phi(i0 + 1 + q);
        if (q <= CH) issue_pi(i0 + q);
        cp_commit();
    }
    // differences of plane p-1 (k and j) and of the pair (p-2, p-1) (i)
    auto diffs = [&](int p) {
        const float* nr = nb + ((p - 1) & 1) * NN;
        float rg = 0.f;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int q = tid + v * NT;
            const int j = q / W, k = 4 * (q % W);
            const float4 xc = xp1[v];
            const float x4 = __shfl_sync(0xffffffffu, xc.x, lnext);
            const float4 up = ld4(nr + ((j + 1) & m) * N + k);
            const float a0 = xc.y - xc.x, a1 = xc.z - xc.y, a2 = xc.w - xc.z, a3 = x4 - xc.w;
            const float b0 = up.x - xc.x, b1 = up.y - xc.y, b2 = up.z - xc.z, b3 = up.w - xc.w;
            rg += a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + b0 * b0 + b1 * b1 + b2 * b2 + b3 * b3;
            if (p >= 2) {
                const float4 xo = xp2[v];
                const float c0 = xc.x - xo.x, c1 = xc.y - xo.y, c2 = xc.z - xo.z, c3 = xc.w - xo.w;
                rg += c0 * c0 + c1 * c1 + c2 * c2 + c3 * c3;
            }
        }
        g.add(rg);
    };
    for (int p = 0; p <= CH; ++p) {
        const int i = i0 + p;
        cp_wait<PF - 1>();
        __syncthreads();
        // planes PF ahead go into the slots of planes no longer read
        if (p + PF + 1 <= CH + 1) issue_phi(i + 1 + PF);
        if (p + PF <= CH) issue_pi(i + PF);
        cp_commit();
        if (p >= 1) diffs(p);
        const float* pc = ring + ((p + 1) % PHS) * NN;
        const float* pu = ring + ((p + 2) % PHS) * NN;
        const float* pl = ring + (p % PHS) * NN;
        const float* pp = pis + (p % PIS) * NN;
        float* nw = nb + (p & 1) * NN;
        const bool store = p < CH;
        const long long gb = (long long)(i & m) << (2 * lgN);
        float rs1 = 0.f, rs2 = 0.f;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int q = tid + v * NT;
            const int j = q / W, k = 4 * (q % W), o = j * N + k;
            const float4 x = ld4(pc + o);
            const float xl = __shfl_sync(0xffffffffu, x.w, lprev);
            const float xr = __shfl_sync(0xffffffffu, x.x, lnext);
            const float4 up = ld4(pc + ((j + 1) & m) * N + k), dn = ld4(pc + ((j - 1) & m) * N + k);
            const float4 iu = ld4(pu + o), il = ld4(pl + o);
            const float4 pi = ld4(pp + o);
            float4 lap;
            lap.x = (x.y + xl) + (up.x + dn.x) + (iu.x + il.x) - 6.f * x.x;
            lap.y = (x.z + x.x) + (up.y + dn.y) + (iu.y + il.y) - 6.f * x.y;
            lap.z = (x.w + x.y) + (up.z + dn.z) + (iu.z + il.z) - 6.f * x.z;
            lap.w = (xr + x.z) + (up.w + dn.w) + (iu.w + il.w) - 6.f * x.w;
            float4 pin, xn;
            pin.x = pi.x + d * (lap_n * lap.x - fric * pi.x - split_dv<TABLE>(x.x, wk, nk, ck, pn, kv, bad, P, wbar));
            pin.y = pi.y + d * (lap_n * lap.y - fric * pi.y - split_dv<TABLE>(x.y, wk, nk, ck, pn, kv, bad, P, wbar));
            pin.z = pi.z + d * (lap_n * lap.z - fric * pi.z - split_dv<TABLE>(x.z, wk, nk, ck, pn, kv, bad, P, wbar));
            pin.w = pi.w + d * (lap_n * lap.w - fric * pi.w - split_dv<TABLE>(x.w, wk, nk, ck, pn, kv, bad, P, wbar));
            xn.x = x.x + d * pin.x;
            xn.y = x.y + d * pin.y;
            xn.z = x.z + d * pin.z;
            xn.w = x.w + d * pin.w;
            st4(nw + o, xn);
            if (store) {
                st4(B.xd + gb + o, xn);
                st4(B.pd + gb + o, pin);
                rs1 += (xn.x + xn.y) + (xn.z + xn.w);
                rs2 += (split_v<TABLE>(xn.x, wv, nv, cv, bad, P, wbar + 2) + split_v<TABLE>(xn.y, wv, nv, cv, bad, P, wbar + 2)) +
                       (split_v<TABLE>(xn.z, wv, nv, cv, bad, P, wbar + 2) + split_v<TABLE>(xn.w, wv, nv, cv, bad, P, wbar + 2));
            }
            xp2[v] = xp1[v];
            xp1[v] = xn;
        }
        if (store) { s1.add(rs1); s2.add(rs2); }
    }
    // the last pair (CH-1, CH) along i
    {
        float rg = 0.f;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float4 xc = xp1[v], xo = xp2[v];
            const float c0 = xc.x - xo.x, c1 = xc.y - xo.y, c2 = xc.z - xo.z, c3 = xc.w - xo.w;
            rg += c0 * c0 + c1 * c1 + c2 * c2 + c3 * c3;
        }
        g.add(rg);
    }
    cp_wait<0>();
    if (bad) {
        if (atomicCAS(&ctl->error, 0, IEGPU_ERANGE) == 0) ctl->errval = ctl->phibar;
    }
    if (nslots > 1) maybe_precompute(ctl, P, K);   // as in rows_body
    df64 v3[3] = {g.df(), s1.df(), s2.df()};
    finish_sums_slot(v3, ctl, P, K, part, counter, a_trace, slot, nslots, state, true);
}

}  // namespace iegpu
